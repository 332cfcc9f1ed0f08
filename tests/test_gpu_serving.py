"""The serving loop: every request's result is the same alone and in the
mix (bit-exact), encryptions equal hmpc_lhe_enc with the request's nonce,
admission rejects what cannot fit and serialises what fits one at a time."""
import numpy as np
import pytest

from hmpc_gb300 import lhe
from hmpc_gb300.comp import Queue, Tensor
from hmpc_gb300.serving import REQUEST_CT_MUL, REQUEST_ENCRYPT, REQUEST_NTT, Server, poisson_stream
from hmpc_gb300.moduli import MODULI

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def queue():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    q = Queue(key=[0x13579BDF] * 8)
    yield q
    q.close()


def build_requests(queue, arrivals, p):
    keys, reqs = {}, []
    for a in arrivals:
        n = 1 << a.log_n
        q = queue.modulus(MODULI[a.q])
        q.prepare(n)
        p.prepare(n)
        if a.kind == REQUEST_NTT:
            reqs.append((a, (queue.uniform(q, (a.count,), n),)))
        elif a.kind == REQUEST_ENCRYPT:
            if (a.q, n) not in keys:
                keys[(a.q, n)] = lhe.keygen(queue, q, p, n)[1]
            reqs.append((a, (queue.uniform(p, (a.count,), n),)))
        else:
            reqs.append((a, tuple(queue.uniform(q, (a.count,), n) for _ in range(4))))
    return keys, reqs


def run(queue, server, keys, reqs, p):
    ids = {k: server.add_key(queue.modulus(MODULI[k[0]]), p, v) for k, v in keys.items()}
    outs, tickets = [], []
    for a, ins in reqs:
        n = 1 << a.log_n
        q = queue.modulus(MODULI[a.q])
        if a.kind == REQUEST_NTT:
            o = (Tensor(q, (a.count,), n),)
            tickets.append(server.submit_ntt(q, ins[0], o[0]))
        elif a.kind == REQUEST_ENCRYPT:
            o = (Tensor(q, (a.count,), n), Tensor(q, (a.count,), n))
            tickets.append(server.submit_encrypt(ids[(a.q, n)], q, ins[0], o[0], o[1], [a.index, 7, 0]))
        else:
            o = tuple(Tensor(q, (a.count,), n) for _ in range(3))
            tickets.append(server.submit_ct_mul(q, *ins, *o))
        outs.append(o)
    server.drain()
    assert all(server.poll(t)[0] == 2 for t in tickets)
    return [[t.numpy() for t in o] for o in outs]


def test_same_result_alone_and_in_the_mix(queue, oracle):
    p = queue.modulus(MODULI["p64"])
    arrivals = poisson_stream(40, seed=3, log_n=(10, 12), counts=(1, 3))
    assert {a.kind for a in arrivals} == {0, 1, 2}
    keys, reqs = build_requests(queue, arrivals, p)
    alone = Server(queue, memory_budget=1 << 28, lanes=1, max_batch=1)
    solo = run(queue, alone, keys, reqs, p)
    alone.close()
    mixed = Server(queue, memory_budget=1 << 28, lanes=4, max_batch=8)
    mix = run(queue, mixed, keys, reqs, p)
    stats = mixed.stats()
    mixed.close()
    for x, y in zip(solo, mix):
        for u, v in zip(x, y):
            assert np.array_equal(u, v)
    assert stats["completed"] == len(reqs) and stats["failed"] == 0
    # encryptions equal the library's encryption with the request's nonce,
    # transforms and products equal the oracle
    for (a, ins), out in zip(reqs, mix):
        n = 1 << a.log_n
        q = queue.modulus(MODULI[a.q])
        if a.kind == REQUEST_ENCRYPT:
            queue.nonce = [a.index, 7, 0]
            ct = lhe.enc(queue, keys[(a.q, n)], ins[0], q)
            assert np.array_equal(ct.c0.numpy(), out[0]) and np.array_equal(ct.c1.numpy(), out[1])
        elif a.kind == REQUEST_NTT:
            om = oracle.Modulus(MODULI[a.q])
            assert np.array_equal(out[0], oracle.ntt(om, n, a.count, src=ins[0].numpy()))
        else:
            om = oracle.Modulus(MODULI[a.q])
            a0, a1, b0, b1 = (t.numpy() for t in ins)
            assert np.array_equal(out[0], oracle.binary(om, oracle.OP_MUL, a0, b0))
            cross = oracle.binary(om, oracle.OP_ADD, oracle.binary(om, oracle.OP_MUL, a0, b1),
                                  oracle.binary(om, oracle.OP_MUL, a1, b0))
            assert np.array_equal(out[1], cross)
            assert np.array_equal(out[2], oracle.binary(om, oracle.OP_MUL, a1, b1))


def test_admission_by_memory(queue):
    p = queue.modulus(MODULI["p64"])
    q = queue.modulus(MODULI["q256"])
    n = 1 << 12
    q.prepare(n)
    _, key = lhe.keygen(queue, q, p, n)
    # one 2-plaintext encryption needs 3 * 2 * n * 8 words = 768 KiB of scratch
    server = Server(queue, memory_budget=800 * 1024, lanes=4, max_batch=8)
    kid = server.add_key(q, p, key)
    msgs = [queue.uniform(p, (2,), n) for _ in range(6)]
    outs = [(Tensor(q, (2,), n), Tensor(q, (2,), n)) for _ in range(6)]
    tickets = [server.submit_encrypt(kid, q, m, o[0], o[1], [i, 0, 0]) for i, (m, o) in enumerate(zip(msgs, outs))]
    big = queue.uniform(p, (4,), n)
    assert server.submit_encrypt(kid, q, big, Tensor(q, (4,), n), Tensor(q, (4,), n), [9, 0, 0]) is None
    server.drain()
    st = server.stats()
    assert st["completed"] == 6 and st["rejected"] == 1 and st["mean_batch"] == 1.0
    for i, (m, o) in enumerate(zip(msgs, outs)):
        queue.nonce = [i, 0, 0]
        ct = lhe.enc(queue, key, m, q)
        assert (ct.c0.data == o[0].data).all().item() and (ct.c1.data == o[1].data).all().item()
    server.close()


def test_batching_window_groups_compatible_requests(queue):
    """With a window, compatible requests submitted close together share
    dispatches (mean batch above one) and each result still equals the
    request's encryption alone."""
    p = queue.modulus(MODULI["p64"])
    q = queue.modulus(MODULI["q256"])
    n = 1 << 11
    q.prepare(n)
    p.prepare(n)
    _, key = lhe.keygen(queue, q, p, n)
    server = Server(queue, memory_budget=1 << 28, lanes=2, max_batch=8, batch_window_us=20000)
    kid = server.add_key(q, p, key)
    msgs = [queue.uniform(p, (1,), n) for _ in range(16)]
    outs = [(Tensor(q, (1,), n), Tensor(q, (1,), n)) for _ in range(16)]
    queue.wait()
    tickets = [server.submit_encrypt(kid, q, m, o[0], o[1], [100 + i, 0, 0]) for i, (m, o) in enumerate(zip(msgs, outs))]
    server.drain()
    st = server.stats()
    server.close()
    assert st["completed"] == 16 and st["mean_batch"] > 1.0
    for i, (m, o) in enumerate(zip(msgs, outs)):
        queue.nonce = [100 + i, 0, 0]
        ct = lhe.enc(queue, key, m, q)
        assert (ct.c0.data == o[0].data).all().item() and (ct.c1.data == o[1].data).all().item()
    assert all(t is not None for t in tickets)


def test_tensor_core_plans_inside_the_loop(queue, oracle):
    """A modulus whose plan for a dispatch's shape is the tensor-core engine
    runs that dispatch's transforms on it -- a transform request's and the
    plaintext transform of an encryption -- with the digit buffers taken from
    the server's pool; results equal the oracle and the library's encryption."""
    import torch

    p = queue.modulus(MODULI["p64"])
    q = queue.modulus(MODULI["q256"])
    om = oracle.Modulus(MODULI["q256"])
    n, count = 1 << 12, 3
    q.prepare(n)
    p.prepare(n)
    _, key = lhe.keygen(queue, q, p, n)
    q.set_plan(n, count, False, radix_bits=0)
    x = queue.uniform(q, (count,), n)
    y = Tensor(q, (count,), n)
    msgs = queue.uniform(p, (count,), n)
    c0, c1 = Tensor(q, (count,), n), Tensor(q, (count,), n)
    server = Server(queue, memory_budget=1 << 26, lanes=1, max_batch=1)
    kid = server.add_key(q, p, key)
    # warm the lane (tensor-core constants, error word), then count
    server.submit_ntt(q, x, y)
    server.drain()
    queue.wait()
    free_before = torch.cuda.mem_get_info()[0]
    launches = server.stats()["launches"]
    t = server.submit_ntt(q, x, y)
    server.drain()
    groups = (n.bit_length() - 1 + 2) // 3
    assert server.stats()["launches"] - launches == groups
    assert server.poll(t)[0] == 2
    assert np.array_equal(y.numpy(), oracle.ntt(om, n, count, src=x.numpy()))
    t = server.submit_encrypt(kid, q, msgs, c0, c1, [21, 0, 0])
    server.drain()
    assert server.poll(t)[0] == 2
    assert torch.cuda.mem_get_info()[0] == free_before  # digit buffers from the pool
    server.close()
    queue.nonce = [21, 0, 0]
    ct = lhe.enc(queue, key, msgs, q)
    assert (ct.c0.data == c0.data).all().item() and (ct.c1.data == c1.data).all().item()
