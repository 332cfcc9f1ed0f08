"""Linear BGV on the GPU against the oracle: key generation, encryption and
decryption bit-exact on the same key and nonces, and the round trip of the
reference's own test (tests/expr/crypto/lhe/enc.cpp)."""
import numpy as np
import pytest

from hmpc_gb300 import lhe
from hmpc_gb300.comp import Queue, Tensor

pytestmark = pytest.mark.gpu

KEY = [0x9E3779B9 * (i + 1) & 0xFFFFFFFF for i in range(8)]
P_64 = 0x8822D80623320001
Q_256 = 0xCFF479B9B12CCF05AF55BCA0D7AE005D53E20D920B577D2785F3A1F156740001
Q_279 = 0x591F5B834C0D961F67343BCC8902BDEDA2771F54306FF151162FF8D2B40F4194DC0001


@pytest.fixture(scope="module")
def queue():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    q = Queue(key=KEY)
    yield q
    q.close()


@pytest.mark.parametrize("n,batch", [(1 << 10, 3), (1 << 12, 2)])
def test_keygen_enc_dec_match_oracle(queue, oracle, n, batch, cpu_threads):
    om_q, om_p = oracle.Modulus(Q_256), oracle.Modulus(P_64)
    gq, gp = queue.modulus(Q_256), queue.modulus(P_64)
    queue.nonce = [0, 0, 0]
    s, key = lhe.keygen(queue, gq, gp, n)
    s_ref, a_ref, b_ref, nonce = oracle.lhe_keygen(om_q, om_p, n, KEY, [0, 0, 0], threads=cpu_threads)
    assert queue.nonce == nonce
    assert np.array_equal(s.numpy(), s_ref)
    assert np.array_equal(key.b.numpy(), b_ref)
    assert np.array_equal(key.a.numpy(), a_ref)

    msgs = queue.uniform(gp, (batch,), n)
    msgs_ref = oracle.sample_uniform(om_p, n * batch, KEY, nonce)
    assert np.array_equal(msgs.numpy(), msgs_ref)
    nonce = queue.nonce
    ct = lhe.enc(queue, key, msgs, gq)
    c0, c1, nonce_ref = oracle.lhe_enc(om_q, om_p, n, batch, a_ref, b_ref, msgs_ref, False, KEY, nonce,
                                       threads=cpu_threads)
    assert queue.nonce == nonce_ref
    assert np.array_equal(ct.c0.numpy(), c0)
    assert np.array_equal(ct.c1.numpy(), c1)
    y = lhe.dec(queue, s, ct, gp)
    assert np.array_equal(y.numpy(), msgs_ref)


def test_reference_round_trip(queue, oracle):
    """tests/expr/crypto/lhe/enc.cpp: a = b = raw representative i, s = one,
    plaintext in NTT form mod p with raw representative i, shape {4, 2},
    N = 2^16, q 279-bit."""
    n, shape = 1 << 16, (4, 2)
    gq, gp = queue.modulus(Q_279), queue.modulus(P_64)
    ramp = np.arange(n, dtype=np.uint64)
    a = np.zeros((gq.limbs, n), dtype=np.uint32)
    a[0] = ramp.astype(np.uint32)
    s = oracle.planar([gq.one] * n, gq.limbs)
    x = np.zeros((gp.limbs, 8 * n), dtype=np.uint32)
    x[0] = np.arange(8 * n, dtype=np.uint64).astype(np.uint32)
    ka = Tensor.from_numpy(gq, a, (), n)
    key = lhe.Key(ka, ka)
    dx = Tensor.from_numpy(gp, x, shape, n)
    queue.nonce = [0, 0, 0]
    ct = lhe.enc(queue, key, dx, gq, plaintext_ntt=True)
    assert queue.nonce == [3 * 8 * n, 0, 0]
    y = lhe.dec(queue, Tensor.from_numpy(gq, s, (), n), ct, gp, plaintext_ntt=True)
    assert np.array_equal(y.numpy(), x)
    # homomorphic: ct + ct decrypts to 2x, ct - ct to 0
    d = lhe.add(queue, ct, ct)
    y2 = lhe.dec(queue, Tensor.from_numpy(gq, s, (), n), d, gp, plaintext_ntt=True)
    om_p = oracle.Modulus(P_64)
    assert np.array_equal(y2.numpy(), oracle.binary(om_p, oracle.OP_ADD, x, x))
    z = lhe.dec(queue, Tensor.from_numpy(gq, s, (), n), lhe.sub(queue, ct, ct), gp, plaintext_ntt=True)
    assert not z.numpy().any()


def test_bgv_full_size_round_trip(queue):
    """keygen + encryption of 256 messages at N = 2^15, q ~ 2^256: decryption
    returns every message (size-independent property at the bench size)."""
    n, batch = 1 << 15, 256
    gq, gp = queue.modulus(Q_256), queue.modulus(P_64)
    queue.nonce = [0, 0, 0]
    s, key = lhe.keygen(queue, gq, gp, n)
    msgs = queue.uniform(gp, (batch,), n)
    ct = lhe.enc(queue, key, msgs, gq)
    y = lhe.dec(queue, s, ct, gp)
    assert (y.data == msgs.data).all().item()


def test_ciphertext_product_decrypts_to_plaintext_product(queue, oracle, cpu_threads):
    """ct x ct (not in the reference): dec2(enc(m1) * enc(m2)) is the negacyclic
    product m1*m2 mod p, and each product component matches the oracle."""
    n, batch = 1 << 12, 2
    om_q, om_p = oracle.Modulus(Q_256), oracle.Modulus(P_64)
    gq, gp = queue.modulus(Q_256), queue.modulus(P_64)
    queue.nonce = [7, 0, 0]
    s, key = lhe.keygen(queue, gq, gp, n)
    m1 = queue.uniform(gp, (batch,), n)
    m2 = queue.uniform(gp, (batch,), n)
    x = lhe.enc(queue, key, m1, gq)
    y = lhe.enc(queue, key, m2, gq)
    prod = lhe.mul(queue, x, y)
    a0, a1, b0, b1 = (t.numpy() for t in (x.c0, x.c1, y.c0, y.c1))
    mul = lambda u, v: oracle.binary(om_q, oracle.OP_MUL, u, v)  # noqa: E731
    assert np.array_equal(prod.c0.numpy(), mul(a0, b0))
    assert np.array_equal(prod.c1.numpy(), oracle.binary(om_q, oracle.OP_ADD, mul(a0, b1), mul(a1, b0)))
    assert np.array_equal(prod.c2.numpy(), mul(a1, b1))
    got = lhe.dec2(queue, s, prod, gp)
    f1 = oracle.ntt(om_p, n, batch, src=m1.numpy(), threads=cpu_threads)
    f2 = oracle.ntt(om_p, n, batch, src=m2.numpy(), threads=cpu_threads)
    expect = oracle.ntt(om_p, n, batch, src=oracle.binary(om_p, oracle.OP_MUL, f1, f2), inverse=True,
                        threads=cpu_threads)
    assert np.array_equal(got.numpy(), expect)
