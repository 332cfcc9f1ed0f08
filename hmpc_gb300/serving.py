"""Client side of the serving loop (hmpc_server_* in the C ABI): request
submission, a seeded Poisson request stream mixing transforms, encryptions
and ciphertext products of mixed degree and limb count, and a replay driver
that reports throughput and p50/p99 latency."""
import ctypes
import math
import time
from dataclasses import dataclass, field

from . import _lib, lhe
from .comp import Tensor
from .moduli import MODULI, chacha20_words

REQUEST_NTT, REQUEST_ENCRYPT, REQUEST_CT_MUL = 0, 1, 2
QUEUED, RUNNING, DONE, FAILED = 0, 1, 2, -2


class ServerConfig(ctypes.Structure):
    _fields_ = [("memory_budget_bytes", ctypes.c_uint64), ("lanes", ctypes.c_uint32),
                ("max_batch", ctypes.c_uint32), ("max_batch_polynomials", ctypes.c_uint32),
                ("batch_window_us", ctypes.c_uint32)]


class Request(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("key_id", ctypes.c_uint32), ("q", ctypes.c_void_p),
                ("n", ctypes.c_uint64), ("count", ctypes.c_uint64),
                ("in0", ctypes.c_void_p), ("in1", ctypes.c_void_p), ("in2", ctypes.c_void_p),
                ("in3", ctypes.c_void_p), ("out0", ctypes.c_void_p), ("out1", ctypes.c_void_p),
                ("out2", ctypes.c_void_p), ("nonce", ctypes.c_uint32 * 3)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_uint64), ("completed", ctypes.c_uint64), ("rejected", ctypes.c_uint64),
                ("failed", ctypes.c_uint64), ("dispatches", ctypes.c_uint64), ("launches", ctypes.c_uint64),
                ("mean_batch", ctypes.c_double), ("p50_us", ctypes.c_double), ("p99_us", ctypes.c_double),
                ("mean_us", ctypes.c_double)]


_SIGS = {
    "hmpc_server_create": ([ctypes.c_void_p, ctypes.POINTER(ServerConfig), ctypes.POINTER(ctypes.c_void_p)],
                           ctypes.c_int),
    "hmpc_server_add_key": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p,
                             ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint32)], ctypes.c_int),
    "hmpc_server_submit": ([ctypes.c_void_p, ctypes.POINTER(Request), ctypes.POINTER(ctypes.c_uint64)],
                           ctypes.c_int),
    "hmpc_server_poll": ([ctypes.c_void_p, ctypes.c_uint64, ctypes.POINTER(ctypes.c_int),
                          ctypes.POINTER(ctypes.c_double)], ctypes.c_int),
    "hmpc_server_drain": ([ctypes.c_void_p, ctypes.c_uint32], ctypes.c_int),
    "hmpc_server_get_stats": ([ctypes.c_void_p, ctypes.POINTER(ServerStats)], ctypes.c_int),
    "hmpc_server_destroy": ([ctypes.c_void_p], ctypes.c_int),
}


def _bind():
    lib = _lib.load()
    for name, (args, res) in _SIGS.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    return lib


class Server:
    """A serving loop on the queue's device.  max_batch=1, lanes=1 gives plain
    per-request launches (every request alone, one after the other)."""

    def __init__(self, queue, memory_budget=1 << 30, lanes=4, max_batch=16, max_batch_polynomials=0,
                 batch_window_us=0):
        self.lib = _bind()
        self.queue = queue
        cfg = ServerConfig(memory_budget, lanes, max_batch, max_batch_polynomials, batch_window_us)
        handle = ctypes.c_void_p()
        _lib.check(self.lib.hmpc_server_create(queue.handle, ctypes.byref(cfg), ctypes.byref(handle)))
        self.handle = handle

    def add_key(self, q, p, key):
        kid = ctypes.c_uint32()
        n = key.a.n
        _lib.check(self.lib.hmpc_server_add_key(self.handle, q.handle, p.handle, n, key.a.data.data_ptr(),
                                                key.b.data.data_ptr(), ctypes.byref(kid)))
        return kid.value

    def submit(self, req):
        ticket = ctypes.c_uint64()
        rc = self.lib.hmpc_server_submit(self.handle, ctypes.byref(req), ctypes.byref(ticket))
        if rc == 7:  # rejected by admission
            return None
        _lib.check(rc)
        return ticket.value

    def submit_ntt(self, q, x, out):
        r = Request(REQUEST_NTT, 0, q.handle.value, x.n, x.batch, x.data.data_ptr(), None, None, None,
                    out.data.data_ptr(), None, None)
        return self.submit(r)

    def submit_encrypt(self, key_id, q, plaintext, c0, c1, nonce):
        r = Request(REQUEST_ENCRYPT, key_id, q.handle.value, plaintext.n, plaintext.batch, plaintext.data.data_ptr(),
                    None, None, None, c0.data.data_ptr(), c1.data.data_ptr(), None)
        for i in range(3):
            r.nonce[i] = nonce[i]
        return self.submit(r)

    def submit_ct_mul(self, q, a0, a1, b0, b1, d0, d1, d2):
        r = Request(REQUEST_CT_MUL, 0, q.handle.value, a0.n, a0.batch, a0.data.data_ptr(), a1.data.data_ptr(),
                    b0.data.data_ptr(), b1.data.data_ptr(), d0.data.data_ptr(), d1.data.data_ptr(),
                    d2.data.data_ptr())
        return self.submit(r)

    def poll(self, ticket):
        state, lat = ctypes.c_int(), ctypes.c_double()
        _lib.check(self.lib.hmpc_server_poll(self.handle, ticket, ctypes.byref(state), ctypes.byref(lat)))
        return state.value, lat.value

    def drain(self, timeout_ms=120000):
        _lib.check(self.lib.hmpc_server_drain(self.handle, timeout_ms))

    def stats(self):
        st = ServerStats()
        _lib.check(self.lib.hmpc_server_get_stats(self.handle, ctypes.byref(st)))
        return {name: getattr(st, name) for name, _ in ServerStats._fields_}

    def close(self):
        if self.handle:
            _lib.check(self.lib.hmpc_server_destroy(self.handle))
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class Arrival:
    t: float          # seconds after the start
    kind: int
    log_n: int
    q: str
    count: int
    index: int = 0


SERVING_MODULI = ["q128", "q160", "q192", "q224", "q256"]  # 4..8 limbs


def poisson_stream(count, rate=2000.0, seed=1, log_n=(12, 16), counts=(1, 4), moduli=SERVING_MODULI,
                   kinds=(REQUEST_NTT, REQUEST_ENCRYPT, REQUEST_CT_MUL)):
    """Seeded request stream: exponential inter-arrival times (mean 1/rate),
    kind uniform over `kinds` (NTT, encrypt, ct x ct), degree uniform over
    {2^log_n[0]..2^log_n[1]}, modulus uniform over `moduli` (4..8 limbs),
    polynomial count uniform over counts (all from one ChaCha20 stream)."""
    words = chacha20_words([0x5E5E0000 + seed] + [0] * 7, 5 * count)
    out, t = [], 0.0
    for i in range(count):
        w = words[5 * i:5 * i + 5]
        u = (w[0] + 0.5) / 2.0 ** 32
        t += -math.log(u) / rate
        out.append(Arrival(t, kinds[w[1] % len(kinds)], log_n[0] + w[2] % (log_n[1] - log_n[0] + 1),
                           moduli[w[3] % len(moduli)],
                           counts[0] + w[4] % (counts[1] - counts[0] + 1), i))
    return out


@dataclass
class Buffers:
    """Device buffers reused by requests of one (kind, degree, modulus) shape."""
    inputs: list = field(default_factory=list)
    outputs: list = field(default_factory=list)


def prepare(queue, arrivals, slots=8, p_name="p64"):
    """Resident keys (one per (q, N)), plaintexts and ciphertext operands, and
    a ring of output buffers per request shape."""
    p = queue.modulus(MODULI[p_name])
    shapes = {}
    keys = {}
    for a in arrivals:
        n = 1 << a.log_n
        q = queue.modulus(MODULI[a.q])
        q.prepare(n)
        p.prepare(n)
        if a.kind == REQUEST_ENCRYPT and (a.q, n) not in keys:
            keys[(a.q, n)] = lhe.keygen(queue, q, p, n)
        key = (a.kind, a.log_n, a.q, a.count)
        if key in shapes:
            continue
        b = Buffers()
        for _ in range(slots):
            if a.kind == REQUEST_NTT:
                b.inputs.append((queue.uniform(q, (a.count,), n),))
                b.outputs.append((Tensor(q, (a.count,), n),))
            elif a.kind == REQUEST_ENCRYPT:
                b.inputs.append((queue.uniform(p, (a.count,), n),))
                b.outputs.append((Tensor(q, (a.count,), n), Tensor(q, (a.count,), n)))
            else:
                b.inputs.append(tuple(queue.uniform(q, (a.count,), n) for _ in range(4)))
                b.outputs.append(tuple(Tensor(q, (a.count,), n) for _ in range(3)))
        shapes[key] = b
    queue.wait()
    return p, keys, shapes


def replay(queue, server, arrivals, p, keys, shapes, real_time=True):
    """Submit the stream (at its arrival times when real_time) and wait for it;
    returns (tickets, wall seconds, server stats)."""
    key_ids = {k: server.add_key(queue.modulus(MODULI[k[0]]), p, v[1]) for k, v in keys.items()}
    slot = {}
    tickets = []
    start = time.perf_counter()
    for a in arrivals:
        if real_time:
            while time.perf_counter() - start < a.t:
                pass
        n = 1 << a.log_n
        q = queue.modulus(MODULI[a.q])
        shape = (a.kind, a.log_n, a.q, a.count)
        i = slot.get(shape, 0)
        slot[shape] = i + 1
        b = shapes[shape]
        ins, outs = b.inputs[i % len(b.inputs)], b.outputs[i % len(b.outputs)]
        if a.kind == REQUEST_NTT:
            t = server.submit_ntt(q, ins[0], outs[0])
        elif a.kind == REQUEST_ENCRYPT:
            t = server.submit_encrypt(key_ids[(a.q, n)], q, ins[0], outs[0], outs[1], [a.index, 0xC0FFEE, 1])
        else:
            t = server.submit_ct_mul(q, *ins, *outs)
        tickets.append(t)
    server.drain()
    wall = time.perf_counter() - start
    return tickets, wall, server.stats()
