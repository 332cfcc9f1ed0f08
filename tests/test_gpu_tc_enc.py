"""BGV encryption with the tensor-core plan on q: p*v and the lifted
plaintext enter one transform and p*w another (the NTT is linear), and the
three transforms run stacked (shared groups over 3 * batch polynomials) -- the
ciphertexts must still equal the oracle's (the reference's four-transform
plan) bit for bit."""
import numpy as np
import pytest

from hmpc_gb300 import lhe
from hmpc_gb300.comp import Queue

pytestmark = pytest.mark.gpu

KEY = [0x0BADC0DE ^ (i * 0x01000193) for i in range(8)]
P_64 = 0x8822D80623320001  # tests/expr/crypto/lhe/enc.cpp:16, L=2
Q_256 = 0xCFF479B9B12CCF05AF55BCA0D7AE005D53E20D920B577D2785F3A1F156740001
Q_128 = 0xE78EC7A9E37BEFBFF59DF3057EBC0001
P_32 = 0xFFF00001  # one-limb plaintext modulus


@pytest.fixture(scope="module")
def queue():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    q = Queue(key=KEY)
    yield q
    q.close()


Q_192 = 0x8605423C957246B58997DEC24F688AB3DD46CB31C5700001
Q_224 = 0xE9E9C9C7700173EE913AE1871AE48451A42CE7E731BC0F8A00C20001


@pytest.mark.parametrize("qv,pv", [(Q_256, P_64), (Q_128, P_64), (Q_256, P_32), (Q_192, P_64), (Q_224, P_32)])
@pytest.mark.parametrize("n,batch", [(1 << 12, 3), (64, 5), (32, 2), (1 << 10, 130), (1 << 16, 1)])
@pytest.mark.parametrize("plaintext_ntt", [False, True])
def test_three_transform_encryption_matches_oracle(queue, oracle, qv, pv, n, batch, plaintext_ntt, cpu_threads):
    om_q, om_p = oracle.Modulus(qv), oracle.Modulus(pv)
    gq, gp = queue.modulus(qv), queue.modulus(pv)
    queue.nonce = [7, 0, 0]
    s, key = lhe.keygen(queue, gq, gp, n)
    s_ref, a_ref, b_ref, nonce = oracle.lhe_keygen(om_q, om_p, n, KEY, [7, 0, 0], threads=cpu_threads)
    assert np.array_equal(key.a.numpy(), a_ref)
    gq.set_plan(n, batch, False, radix_bits=0)
    msgs = queue.uniform(gp, (batch,), n)
    msgs_ref = oracle.sample_uniform(om_p, n * batch, KEY, nonce)
    nonce = queue.nonce
    before = queue.launches
    ct = lhe.enc(queue, key, msgs, gq, plaintext_ntt=plaintext_ntt)
    groups = (n.bit_length() - 1 + 2) // 3
    # u, p*v + lift(m) and p*w stacked on the tensor cores (three first-group
    # launches, then one launch per remaining group), one combine writing c0
    # and c1, and the INTT mod p when the plaintext is in NTT form
    launched = queue.launches - before
    if plaintext_ntt:
        assert launched > 3 + (groups - 1) + 1
    else:
        assert launched == 3 + (groups - 1) + 1
    c0, c1, nonce_ref = oracle.lhe_enc(om_q, om_p, n, batch, a_ref, b_ref, msgs_ref, plaintext_ntt, KEY, nonce,
                                       threads=cpu_threads)
    assert queue.nonce == nonce_ref
    assert np.array_equal(ct.c0.numpy(), c0)
    assert np.array_equal(ct.c1.numpy(), c1)
    y = lhe.dec(queue, s, ct, gp, plaintext_ntt=plaintext_ntt)
    assert np.array_equal(y.numpy(), msgs_ref)


def test_bench_shape(queue, oracle, cpu_threads):
    """256 x 2^15, q 256-bit, p 64-bit: the shape bench.py measures"""
    n, batch = 1 << 15, 256
    om_q, om_p = oracle.Modulus(Q_256), oracle.Modulus(P_64)
    gq, gp = queue.modulus(Q_256), queue.modulus(P_64)
    queue.nonce = [0, 0, 0]
    s, key = lhe.keygen(queue, gq, gp, n)
    _, a_ref, b_ref, nonce = oracle.lhe_keygen(om_q, om_p, n, KEY, [0, 0, 0], threads=cpu_threads)
    gq.set_plan(n, batch, False, radix_bits=0)
    msgs = queue.uniform(gp, (batch,), n)
    msgs_ref = oracle.sample_uniform(om_p, n * batch, KEY, nonce)
    nonce = queue.nonce
    ct = lhe.enc(queue, key, msgs, gq)
    c0, c1, _ = oracle.lhe_enc(om_q, om_p, n, batch, a_ref, b_ref, msgs_ref, False, KEY, nonce, threads=cpu_threads)
    assert np.array_equal(ct.c0.numpy(), c0)
    assert np.array_equal(ct.c1.numpy(), c1)
    assert (lhe.dec(queue, s, ct, gp).data == msgs.data).all().item()
