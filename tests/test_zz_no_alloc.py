"""The allocation-free BGV encryption (hmpc_lhe_enc_noalloc) against the
regular one (hmpc_lhe_enc), called through the C ABI.

hmpc_lhe_enc_noalloc exists for callers that cannot allocate device memory
(a serving process whose memory is reserved up front by its own pool, or a
latency-critical loop that must not pay the synchronisation of
cudaMalloc/cudaFree).  Its intermediates live in a fixed 32 MiB array inside
the library, shared by every call on the device, so this file is collected
last and checks two calls in a row: the second must not see stale state from
the first.  Results are integers, compared bit for bit.
"""
import ctypes

import numpy as np
import pytest

from hmpc_gb300 import _lib
from hmpc_gb300.comp import Queue, Tensor

pytestmark = pytest.mark.gpu

KEY = [0x0BADF00D, 1, 2, 3, 4, 5, 6, 0xFFFFFFFF]
Q_256 = 0xCFF479B9B12CCF05AF55BCA0D7AE005D53E20D920B577D2785F3A1F156740001
P_64 = 0x8822D80623320001


@pytest.fixture(scope="module")
def queue():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    q = Queue(key=KEY)
    yield q
    q.close()


def encrypt(queue, name, q, p, n, batch, key_a, key_b, plaintext, plaintext_ntt):
    c0 = Tensor(q, (batch,), n)
    c1 = Tensor(q, (batch,), n)
    _lib.call(name, queue.handle, q.handle, p.handle, n, batch, key_a.ptr(), key_b.ptr(), plaintext.ptr(),
              int(plaintext_ntt), c0.ptr(), c1.ptr())
    queue.wait()
    return c0.numpy(), c1.numpy()


@pytest.mark.parametrize("n,batch,plaintext_ntt", [(1 << 12, 4, False), (1 << 11, 3, True)])
def test_noalloc_matches_regular_encryption_twice(queue, n, batch, plaintext_ntt):
    q, p = queue.modulus(Q_256), queue.modulus(P_64)
    q.prepare(n)
    p.prepare(n)
    queue.nonce = [0, 0, 0]
    key_a = queue.uniform(q, (), n)
    key_b = queue.uniform(q, (), n)
    messages = [queue.uniform(p, (batch,), n) for _ in range(2)]
    start = queue.nonce
    regular, nonces = [], []
    for m in messages:
        regular.append(encrypt(queue, "hmpc_lhe_enc", q, p, n, batch, key_a, key_b, m, plaintext_ntt))
        nonces.append(queue.nonce)
    queue.nonce = start
    for i, m in enumerate(messages):
        got = encrypt(queue, "hmpc_lhe_enc_noalloc", q, p, n, batch, key_a, key_b, m, plaintext_ntt)
        assert queue.nonce == nonces[i]
        assert np.array_equal(got[0], regular[i][0]), f"c0 differs on call {i + 1}"
        assert np.array_equal(got[1], regular[i][1]), f"c1 differs on call {i + 1}"


def test_noalloc_rejects_oversized_batches_and_missing_tables(queue):
    q, p = queue.modulus(Q_256), queue.modulus(P_64)
    n = 1 << 15
    q.prepare(n)
    big = 11  # 3 * 11 * 2^15 * 8 words > 8 Mi words
    a = Tensor(q, (), n)
    x = Tensor(p, (big,), n)
    c = Tensor(q, (big,), n)
    rc = _lib.load().hmpc_lhe_enc_noalloc(queue.handle, q.handle, p.handle, n, big, a.ptr(), a.ptr(), x.ptr(), 0,
                                          c.ptr(), c.ptr())
    assert rc == 1
    assert b"at most" in _lib.load().hmpc_last_error()
    m = 1 << 4  # no tables built for this degree
    rc = _lib.load().hmpc_lhe_enc_noalloc(queue.handle, q.handle, p.handle, m, 1, a.ptr(), a.ptr(), x.ptr(), 0,
                                          c.ptr(), c.ptr())
    assert rc == 1
    assert b"hmpc_modulus_prepare" in _lib.load().hmpc_last_error()


def test_noalloc_matches_the_oracle_and_a_tensor_core_plan(queue, oracle, cpu_threads):
    """the allocation-free path (CUDA-core tiles, four transforms) against the
    oracle directly, and against hmpc_lhe_enc with q's transforms on the
    tensor-core engine (three stacked transforms): the same bits"""
    n, batch = 1 << 11, 5
    q, p = queue.modulus(Q_256), queue.modulus(P_64)
    om_q, om_p = oracle.Modulus(Q_256), oracle.Modulus(P_64)
    q.prepare(n)
    p.prepare(n)
    queue.nonce = [11, 0, 0]
    key_a = queue.uniform(q, (), n)
    key_b = queue.uniform(q, (), n)
    msgs = queue.uniform(p, (batch,), n)
    start = queue.nonce
    got = encrypt(queue, "hmpc_lhe_enc_noalloc", q, p, n, batch, key_a, key_b, msgs, False)
    c0, c1, _ = oracle.lhe_enc(om_q, om_p, n, batch, key_a.numpy(), key_b.numpy(), msgs.numpy(), False, KEY, start,
                               threads=cpu_threads)
    assert np.array_equal(got[0], c0) and np.array_equal(got[1], c1)
    q.set_plan(n, batch, False, radix_bits=0)
    queue.nonce = start
    tc = encrypt(queue, "hmpc_lhe_enc", q, p, n, batch, key_a, key_b, msgs, False)
    assert np.array_equal(tc[0], c0) and np.array_equal(tc[1], c1)
    queue.nonce = start
    again = encrypt(queue, "hmpc_lhe_enc_noalloc", q, p, n, batch, key_a, key_b, msgs, False)
    assert np.array_equal(again[0], c0) and np.array_equal(again[1], c1)


def test_noalloc_takes_no_device_memory(queue):
    """On a fresh context whose tables are prepared, the first calls allocate
    nothing: the device's free memory is the same before and after (the
    library's fixed array is loaded by a call on another context first)."""
    import torch

    n, batch = 1 << 12, 6
    q0, p0 = queue.modulus(Q_256), queue.modulus(P_64)
    q0.prepare(n)
    p0.prepare(n)
    a0 = queue.uniform(q0, (), n)
    m0 = queue.uniform(p0, (batch,), n)
    encrypt(queue, "hmpc_lhe_enc_noalloc", q0, p0, n, batch, a0, a0, m0, False)
    fresh = Queue(key=KEY)
    q, p = fresh.modulus(Q_256), fresh.modulus(P_64)
    q.prepare(n)
    p.prepare(n)
    key_a = fresh.uniform(q, (), n)
    key_b = fresh.uniform(q, (), n)
    msgs = fresh.uniform(p, (batch,), n)
    c0, c1 = Tensor(q, (batch,), n), Tensor(q, (batch,), n)
    fresh.wait()
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    for _ in range(2):
        _lib.call("hmpc_lhe_enc_noalloc", fresh.handle, q.handle, p.handle, n, batch, key_a.ptr(), key_b.ptr(),
                  msgs.ptr(), 0, c0.ptr(), c1.ptr())
    fresh.wait()
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before
    # the regular entry point on the same context grows its workspace
    _lib.call("hmpc_lhe_enc", fresh.handle, q.handle, p.handle, n, batch, key_a.ptr(), key_b.ptr(), msgs.ptr(), 0,
              c0.ptr(), c1.ptr())
    fresh.wait()
    assert torch.cuda.mem_get_info()[0] < free_before
    fresh.close()
