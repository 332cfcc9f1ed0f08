"""Parity of the tensor-core transform engine (tile shape radix bits 0) with
the CPU oracle for moduli of 2 to 8 limbs: bit-exact forward and inverse transforms, fused CBD(V)
samplers, the uniform sampler's transform, ragged batches, in-place calls, and
the fallback to the CUDA-core tiles for calls the engine does not cover."""
import numpy as np
import pytest

from hmpc_gb300 import _lib
from hmpc_gb300.comp import Queue, Tensor

pytestmark = pytest.mark.gpu

KEY = [0x9E3779B9, 0x7F4A7C15, 0xF39CC060, 0x5CEDC834, 0x1082276B, 0xF3A27251, 0xF86C6A11, 0x4D2A8E5B]
Q_256 = 0xCFF479B9B12CCF05AF55BCA0D7AE005D53E20D920B577D2785F3A1F156740001  # L=8
Q_128 = 0xE78EC7A9E37BEFBFF59DF3057EBC0001  # L=4
Q_NTT = 0x18F25CD9A75CCBD9C146D4ABAEC00001  # examples/ntt.cpp:22, L=4, 125 bits
P_64 = 0x8822D80623320001  # tests/expr/crypto/lhe/enc.cpp:16, L=2
Q_96 = 0x800000000000000002060001  # L=3
Q_160 = 0x92155E09E949EDD961C374C93DE4B90B9F220001  # L=5
Q_192 = 0x8605423C957246B58997DEC24F688AB3DD46CB31C5700001  # L=6
Q_224 = 0xE9E9C9C7700173EE913AE1871AE48451A42CE7E731BC0F8A00C20001  # L=7
Q_288 = (1 << 287) + 0x5E0001  # an odd 9-limb modulus: not covered by the engine


@pytest.fixture(scope="module")
def queue():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    q = Queue(key=KEY)
    yield q
    q.close()


def groups(n):
    return (n.bit_length() - 1 + 2) // 3


def random_residues(oracle, mod, count, seed):
    rng = np.random.default_rng(seed)
    words = rng.integers(0, 2**32, size=(mod.limbs, count), dtype=np.uint64).astype(np.uint32)
    words[mod.limbs - 1] &= np.uint32((1 << (mod.bits % 32 or 32)) - 1)
    vals = [v % mod.value for v in oracle.unplanar(words)]
    return oracle.from_uint(mod, oracle.planar(vals, mod.limbs))


def tensor_plan(gm, n, batch, inverse=False):
    gm.set_plan(n, batch, inverse, radix_bits=0)
    assert gm.plan(n, batch, inverse)["radix_bits"] == 0


@pytest.mark.parametrize("q", [Q_256, Q_128, Q_NTT, P_64, Q_96, Q_160, Q_192, Q_224])
@pytest.mark.parametrize("n,batch", [(16, 3), (32, 1), (64, 5), (1 << 10, 2), (1 << 12, 130), (1 << 13, 3)])
def test_forward_and_inverse_match_oracle(queue, oracle, q, n, batch, cpu_threads):
    om = oracle.Modulus(q)
    gm = queue.modulus(q)
    tensor_plan(gm, n, batch)
    tensor_plan(gm, n, batch, inverse=True)
    x = random_residues(oracle, om, n * batch, n + batch)
    dx = Tensor.from_numpy(gm, x, (batch,), n)
    before = queue.launches
    y = queue.ntt(dx)
    assert queue.launches - before == groups(n)
    ref = oracle.ntt(om, n, batch, src=x, threads=cpu_threads)
    assert np.array_equal(y.numpy(), ref)
    z = queue.intt(y)
    assert np.array_equal(z.numpy(), x)
    assert _lib.call("hmpc_context_synchronize", queue.handle) == 0


@pytest.mark.parametrize("q", [Q_256, Q_128, P_64, Q_96, Q_160, Q_192, Q_224])
@pytest.mark.parametrize("vx2", [1, 7, 20, 64])
def test_fused_cbd_matches_oracle(queue, oracle, q, vx2, cpu_threads):
    om = oracle.Modulus(q)
    gm = queue.modulus(q)
    n, batch = 1 << 11, 5
    tensor_plan(gm, n, batch)
    nonce = [0xFFFFFFF0, 7, 1]
    queue.nonce = nonce
    y = queue.ntt_centered_binomial(gm, n, (batch,), vx2)
    assert queue.nonce == oracle.nonce_add(nonce, n * batch)
    ref = oracle.ntt(om, n, batch, sampler="cbd", variance_x2=vx2, key=KEY, nonce=nonce, threads=cpu_threads)
    assert np.array_equal(y.numpy(), ref)


@pytest.mark.parametrize("q", [Q_256, Q_128, Q_192])
@pytest.mark.parametrize("n,batch", [(1 << 10, 1), (1 << 10, 3), (1 << 16, 1), (1 << 16, 2)])
@pytest.mark.parametrize("vx2", [1, 64])
def test_wide_first_group_edges(queue, oracle, q, n, batch, vx2, cpu_threads):
    """the first six stages as one group: the smallest and largest degrees it
    covers (four groups at 2^10, the wide one then 3 + 1 stages; 2^16), a
    single polynomial (fewer rows than one 128-row tile), both ends of 2V"""
    om, gm = oracle.Modulus(q), queue.modulus(q)
    tensor_plan(gm, n, batch)
    nonce = [0x7FFFFFFF, 0xFFFFFFFF, 2]
    queue.nonce = nonce
    before = queue.launches
    y = queue.ntt_centered_binomial(gm, n, (batch,), vx2)
    assert queue.launches - before == groups(n) - 1  # the wide group replaces the first two
    assert queue.nonce == oracle.nonce_add(nonce, n * batch)
    ref = oracle.ntt(om, n, batch, sampler="cbd", variance_x2=vx2, key=KEY, nonce=nonce, threads=cpu_threads)
    assert np.array_equal(y.numpy(), ref)


def test_full_size_bgv_transform(queue, oracle, cpu_threads):
    """the bench's transform shape: 2^15 coefficients, q 256-bit, a batch
    spanning several 128-row tiles per constant matrix"""
    om = oracle.Modulus(Q_256)
    gm = queue.modulus(Q_256)
    n, batch = 1 << 15, 260
    tensor_plan(gm, n, batch)
    tensor_plan(gm, n, batch, inverse=True)
    queue.nonce = [5, 0, 0]
    y = queue.ntt_centered_binomial(gm, n, (batch,), 20)
    # spot-check the first and the last polynomials against the oracle
    ref = oracle.ntt(om, n, batch, sampler="cbd", variance_x2=20, key=KEY, nonce=[5, 0, 0], threads=cpu_threads)
    got = y.numpy()
    assert np.array_equal(got, ref)
    x = random_residues(oracle, om, n * 2, 77)
    big = Tensor(gm, (batch,), n)
    big.data.zero_()
    big.data[:, : 2 * n] = Tensor.from_numpy(gm, x, (2,), n).data
    z = queue.intt(queue.ntt(big))
    assert (z.data == big.data).all().item()


@pytest.mark.parametrize("q", [Q_256, P_64, Q_192, Q_224])
@pytest.mark.parametrize("n,batch", [(64, 5), (1 << 12, 130)])
def test_unsplit_contiguous_group(queue, oracle, q, n, batch, cpu_threads):
    """the forward transform's last group and the inverse's first with one
    constant image per block (local bits 1) instead of two"""
    om = oracle.Modulus(q)
    gm = queue.modulus(q)
    for inverse in (False, True):
        gm.set_plan(n, batch, inverse, radix_bits=0, local_bits=1)
        assert gm.plan(n, batch, inverse) == {"radix_bits": 0, "local_bits": 1, "col_bits": 4}
    x = random_residues(oracle, om, n * batch, 3 * n + batch)
    y = queue.ntt(Tensor.from_numpy(gm, x, (batch,), n))
    assert np.array_equal(y.numpy(), oracle.ntt(om, n, batch, src=x, threads=cpu_threads))
    assert np.array_equal(queue.intt(y).numpy(), x)
    with pytest.raises(_lib.HmpcError):
        gm.set_plan(n, batch, False, radix_bits=0, local_bits=3)


def test_in_place_and_zero(queue, oracle):
    om = oracle.Modulus(Q_256)
    gm = queue.modulus(Q_256)
    n, batch = 1 << 12, 3
    tensor_plan(gm, n, batch)
    x = random_residues(oracle, om, n * batch, 9)
    dx = Tensor.from_numpy(gm, x, (batch,), n)
    queue.ntt(dx, out=dx)
    assert np.array_equal(dx.numpy(), oracle.ntt(om, n, batch, src=x))
    zero = Tensor.from_numpy(gm, np.zeros_like(x), (batch,), n)
    assert not queue.ntt(zero).numpy().any()


@pytest.mark.parametrize("q", [Q_256, Q_128, Q_192, P_64, Q_96])
@pytest.mark.parametrize("n,batch", [(16, 3), (1 << 10, 2), (1 << 12, 130)])
def test_uniform_producer_on_the_engine(queue, oracle, q, n, batch, cpu_threads):
    """the uniform sampler's transform: one launch draws the stage-0 pairs'
    values (the generator of pair (j, j + n/2) at counter j, u before v)
    into the output, then the engine's groups run in place"""
    om, gm = oracle.Modulus(q), queue.modulus(q)
    tensor_plan(gm, n, batch)
    nonce = [0xFFFFFFF8, 3, 9]
    queue.nonce = nonce
    before = queue.launches
    y = queue.ntt_uniform(gm, n, (batch,))
    assert queue.launches - before == 1 + groups(n)
    assert queue.nonce == oracle.nonce_add(nonce, n * batch)
    ref = oracle.ntt(om, n, batch, sampler="uniform", key=KEY, nonce=nonce, threads=cpu_threads)
    assert np.array_equal(y.numpy(), ref)


def test_uncovered_calls_fall_back(queue, oracle):
    """degrees below 16 and unsupported moduli run the CUDA-core tiles"""
    gm = queue.modulus(Q_256)
    om = oracle.Modulus(Q_256)
    n, batch = 1 << 10, 2
    g288 = queue.modulus(Q_288)
    with pytest.raises(_lib.HmpcError):
        g288.set_plan(n, batch, False, radix_bits=0)
    small = Tensor.from_numpy(gm, random_residues(oracle, om, 8 * 2, 3), (2,), 8)
    gm.set_plan(8, 2, False, radix_bits=0)
    assert np.array_equal(queue.ntt(small).numpy(), oracle.ntt(om, 8, 2, src=small.numpy()))


def test_tuner_considers_the_engine(queue):
    gm = queue.modulus(Q_256)
    n, batch = 1 << 12, 64
    ms = gm.tune(n, batch)
    assert ms > 0
    assert gm.plan(n, batch)["radix_bits"] in (0, 2, 3)
