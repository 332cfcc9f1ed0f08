"""Edge cases of the CUDA path: empty batches, the largest degree the
reference's example transforms (N = 2^20, examples/ntt.cpp:22-23), odd batch
sizes in place, 1-limb and 9-limb moduli, and argument errors returned as
status codes with the context still usable afterwards."""
import ctypes

import numpy as np
import pytest

from hmpc_gb300 import _lib
from hmpc_gb300.comp import Queue, Tensor

pytestmark = pytest.mark.gpu

KEY = [3, 1, 4, 1, 5, 9, 2, 6]
Q_NTT = 0x18F25CD9A75CCBD9C146D4ABAEC00001  # examples/ntt.cpp:22, L=4
Q_256 = 0xCFF479B9B12CCF05AF55BCA0D7AE005D53E20D920B577D2785F3A1F156740001  # L=8
Q_279 = 0x591F5B834C0D961F67343BCC8902BDEDA2771F54306FF151162FF8D2B40F4194DC0001  # L=9
Q_32 = 0xFFF00001  # one limb, 2^20 | Q - 1
P_64 = 0x8822D80623320001  # L=2


@pytest.fixture(scope="module")
def queue():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    q = Queue(key=KEY)
    yield q
    q.close()


def test_empty_batches_launch_nothing(queue):
    gm = queue.modulus(Q_256)
    gm.prepare(1024)
    before = queue.launches
    nonce = queue.nonce
    x = Tensor(gm, (0,), 1024)
    queue.ntt(x)
    queue.intt(x)
    queue.ntt_centered_binomial(gm, 1024, (0,), 20)
    queue.ntt_uniform(gm, 1024, (0,))
    queue.fma(x, x, x)
    queue.uniform(gm, (0,))
    queue.centered_binomial(gm, (0,), 20)
    queue.cast(x, queue.modulus(P_64))
    assert queue.launches == before
    assert queue.nonce == nonce


def test_degree_2_to_the_20(queue, oracle, cpu_threads):
    """examples/ntt.cpp:23 transforms degree-2^20 polynomials mod a 125-bit Q"""
    n = 1 << 20
    gm = queue.modulus(Q_NTT)
    om = oracle.Modulus(Q_NTT)
    queue.nonce = [0, 0, 0]
    x = queue.uniform(gm, (1,), n)
    y = queue.ntt(x)
    assert np.array_equal(y.numpy(), oracle.ntt(om, n, 1, src=x.numpy(), threads=cpu_threads))
    assert (queue.intt(y).data == x.data).all().item()


@pytest.mark.parametrize("batch", [1, 3, 7, 17])
def test_odd_batches_in_place(queue, oracle, batch):
    n = 1 << 13
    gm = queue.modulus(Q_256)
    om = oracle.Modulus(Q_256)
    x = queue.uniform(gm, (batch,), n)
    ref = oracle.ntt(om, n, batch, src=x.numpy())
    y = Tensor(gm, (batch,), n, x.data.clone())
    queue.ntt(y, out=y)
    assert np.array_equal(y.numpy(), ref)
    queue.intt(y, out=y)
    assert (y.data == x.data).all().item()


@pytest.mark.parametrize("q", [Q_32, Q_279])
@pytest.mark.parametrize("n", [4, 64, 1 << 12])
def test_narrowest_and_widest_moduli(queue, oracle, q, n):
    """one-limb and nine-limb moduli through the fused sampler transform"""
    gm = queue.modulus(q)
    om = oracle.Modulus(q)
    queue.nonce = [1, 0, 0]
    y = queue.ntt_centered_binomial(gm, n, (2,), 20)
    ref = oracle.ntt(om, n, 2, sampler="cbd", variance_x2=20, key=KEY, nonce=[1, 0, 0])
    assert np.array_equal(y.numpy(), ref)
    assert np.array_equal(queue.intt(y).numpy(), oracle.ntt(om, n, 2, inverse=True, src=ref))


def test_errors_are_status_codes(queue):
    lib = _lib.load()
    gm = queue.modulus(Q_256)
    out = Tensor(gm, (1,), 16)
    optr = out.ptr()
    no_src = _lib.Producer(_lib.PRODUCER_TENSOR, None, 0, 0)
    assert lib.hmpc_ntt_forward(queue.handle, gm.handle, 16, 1, ctypes.byref(no_src), optr) == 1
    src = _lib.Producer(_lib.PRODUCER_TENSOR, out.ptr(), 0, 0)
    assert lib.hmpc_ntt_forward(queue.handle, gm.handle, 24, 1, ctypes.byref(src), optr) == 1
    assert lib.hmpc_ntt_forward(queue.handle, gm.handle, 2, 1, ctypes.byref(src), optr) == 1
    wide_cbd = _lib.Producer(_lib.PRODUCER_CBD, None, 65, 0)
    assert lib.hmpc_ntt_forward(queue.handle, gm.handle, 16, 1, ctypes.byref(wide_cbd), optr) == 2
    assert lib.hmpc_sample_uniform(queue.handle, gm.handle, 16, 128, optr) == 2
    # the broadcast operands' sizes must divide the result size
    assert lib.hmpc_binary(queue.handle, gm.handle, 0, 16, optr, 3, optr, 16, optr) == 1
    handle = ctypes.c_void_p()
    even = (ctypes.c_uint32 * 1)(10)
    assert lib.hmpc_modulus_create(queue.handle, even, 1, ctypes.byref(handle)) == 1
    wide = (ctypes.c_uint32 * 10)(*([0xFFFFFFFF] * 10))
    assert lib.hmpc_modulus_create(queue.handle, wide, 10, ctypes.byref(handle)) == 2
    assert lib.hmpc_last_error()
    # the context stays usable
    x = queue.uniform(gm, (1,), 16)
    assert (queue.intt(queue.ntt(x)).data == x.data).all().item()


def test_rate_probes_are_plausible(queue):
    """The live denominators of the integer rooflines: 32-bit multiplies and
    ChaCha20 blocks per second, both well inside what 152 SMs at up to about
    2 GHz can issue."""
    import bench

    rates = bench.rate_probes()
    mul, blocks = rates["int_multiply_rate"], rates["chacha_rate"]
    assert 1e12 < mul < 1e14
    # about a thousand integer operations per block
    assert 1e9 < blocks < 1e12
