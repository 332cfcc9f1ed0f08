"""The cluster transform (tile shape radix bits 1): one thread-block cluster
of 8 CTAs per polynomial, the polynomial in distributed shared memory, one
launch per transform -- bit-exact with the oracle (the reference's stage
formulas, hmpc/expr/number_theoretic_transform.hpp:90-197) for degrees
2^10..2^14 and 1 to 9 limbs, in place and out of place; calls it does not
cover run the default tiles with the same results."""
import numpy as np
import pytest

from hmpc_gb300.comp import Queue, Tensor

pytestmark = pytest.mark.gpu

KEY = [0xC1, 0xC2, 0xC3, 0xC4, 0xC5, 0xC6, 0xC7, 0xC8]
MODULI = [
    0xFFF00001,  # 1 limb
    0x8822D80623320001,  # 2 limbs (tests/expr/crypto/lhe/enc.cpp:16)
    0x18F25CD9A75CCBD9C146D4ABAEC00001,  # 4 limbs (examples/ntt.cpp:22)
    0x8605423C957246B58997DEC24F688AB3DD46CB31C5700001,  # 6 limbs
    0xCFF479B9B12CCF05AF55BCA0D7AE005D53E20D920B577D2785F3A1F156740001,  # 8 limbs
]


@pytest.fixture(scope="module")
def queue():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    q = Queue(key=KEY)
    yield q
    q.close()


def cluster_plan(gm, n, batch):
    for inverse in (False, True):
        gm.set_plan(n, batch, inverse, radix_bits=1)
        assert gm.plan(n, batch, inverse)["radix_bits"] == 1


@pytest.mark.parametrize("q", MODULI)
@pytest.mark.parametrize("log_n", [10, 11, 12, 13, 14])
@pytest.mark.parametrize("batch", [1, 3])
def test_cluster_transform_matches_oracle(queue, oracle, q, log_n, batch, cpu_threads):
    n = 1 << log_n
    om, gm = oracle.Modulus(q), queue.modulus(q)
    cluster_plan(gm, n, batch)
    x = queue.uniform(gm, (batch,), n)
    before = queue.launches
    y = queue.ntt(x)
    assert queue.launches - before == 1
    ref = oracle.ntt(om, n, batch, src=x.numpy(), threads=cpu_threads)
    assert np.array_equal(y.numpy(), ref)
    z = queue.intt(y)
    assert np.array_equal(z.numpy(), x.numpy())
    # the inverse on arbitrary input against the oracle's inverse
    w = queue.intt(x)
    assert np.array_equal(w.numpy(), oracle.ntt(om, n, batch, src=x.numpy(), inverse=True, threads=cpu_threads))


def test_cluster_transform_in_place(queue, oracle, cpu_threads):
    q = MODULI[2]
    n, batch = 1 << 12, 2
    om, gm = oracle.Modulus(q), queue.modulus(q)
    cluster_plan(gm, n, batch)
    x = queue.uniform(gm, (batch,), n)
    keep = x.numpy().copy()
    queue.ntt(x, out=x)
    assert np.array_equal(x.numpy(), oracle.ntt(om, n, batch, src=keep, threads=cpu_threads))
    queue.intt(x, out=x)
    assert np.array_equal(x.numpy(), keep)


def test_uncovered_calls_run_the_default_tiles(queue, oracle, cpu_threads):
    """degrees outside 2^10..2^14 and sampler producers under a cluster plan"""
    q = MODULI[2]
    om, gm = oracle.Modulus(q), queue.modulus(q)
    for n in (1 << 9, 1 << 15):
        cluster_plan(gm, n, 1)
        x = queue.uniform(gm, (1,), n)
        assert np.array_equal(queue.ntt(x).numpy(), oracle.ntt(om, n, 1, src=x.numpy(), threads=cpu_threads))
    n = 1 << 12
    cluster_plan(gm, n, 2)
    nonce = queue.nonce
    y = queue.ntt_centered_binomial(gm, n, (2,), 20)
    assert np.array_equal(y.numpy(), oracle.ntt(om, n, 2, sampler="cbd", variance_x2=20, key=KEY, nonce=nonce,
                                                threads=cpu_threads))


def test_tuner_considers_the_cluster_engine(queue):
    gm = queue.modulus(MODULI[2])
    n = 1 << 12
    assert gm.tune(n, 1) > 0
    assert gm.plan(n, 1)["radix_bits"] in (1, 2, 3)
