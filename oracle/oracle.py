"""ctypes front end of the C oracle (oracle/hmpc_oracle.c).

TEST INFRASTRUCTURE ONLY.  Imported by tests/, by __graft_entry__.smoke() as
the checker, and by bench.py's CPU-baseline leg; the product never imports it.

Tensors are numpy uint32 arrays in the reference's limb-planar layout
[limbs][elements] (hmpc/comp/tensor.hpp:21,25-29).
"""
import ctypes
import os
import pathlib
import subprocess

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "libhmpc_oracle.so"
MAX_LIMBS = 16

PRODUCER_TENSOR = 0
PRODUCER_CBD = 1
PRODUCER_UNIFORM = 2
PRODUCER_CAST = 3

OP_ADD, OP_SUB, OP_MUL = 0, 1, 2


def build(force=False):
    """Compile the oracle with its Makefile (gcc + OpenMP)."""
    src = HERE / "hmpc_oracle.c"
    if force or not LIB_PATH.exists() or LIB_PATH.stat().st_mtime < src.stat().st_mtime:
        subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB_PATH


class _Modulus(ctypes.Structure):
    _fields_ = [
        ("limbs", ctypes.c_int),
        ("bits", ctypes.c_int),
        ("ninv", ctypes.c_uint32),
        ("q", ctypes.c_uint32 * MAX_LIMBS),
        ("half", ctypes.c_uint32 * MAX_LIMBS),
        ("one", ctypes.c_uint32 * MAX_LIMBS),
        ("r2", ctypes.c_uint32 * MAX_LIMBS),
    ]


class _Producer(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int),
        ("src", ctypes.c_void_p),
        ("src_modulus", ctypes.POINTER(_Modulus)),
        ("variance_x2", ctypes.c_int),
        ("security", ctypes.c_int),
        ("key", ctypes.c_uint32 * 8),
        ("nonce", ctypes.c_uint32 * 3),
    ]


class _Generator(ctypes.Structure):
    _fields_ = [
        ("key", ctypes.c_uint32 * 8),
        ("nonce", ctypes.c_uint32 * 3),
        ("counter", ctypes.c_uint32),
        ("block", ctypes.c_uint32 * 16),
        ("index", ctypes.c_int),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(str(LIB_PATH))
        u32p = ctypes.POINTER(ctypes.c_uint32)
        mp = ctypes.POINTER(_Modulus)
        _lib.orc_modulus_init.argtypes = [mp, u32p, ctypes.c_int]
        _lib.orc_sample_cbd.restype = ctypes.c_int64
        _lib.orc_generator_next.restype = ctypes.c_uint32
        _lib.orc_ntt.argtypes = [mp, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int, ctypes.POINTER(_Producer),
                                 ctypes.c_void_p, ctypes.c_int]
        _lib.orc_fma.argtypes = [mp, ctypes.c_uint64] + [ctypes.c_void_p] * 4 + [ctypes.c_int]
        _lib.orc_binary.argtypes = [mp, ctypes.c_int, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_uint64,
                                    ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_int]
        _lib.orc_sample_uniform_tensor.argtypes = [mp, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p,
                                                   ctypes.c_int, ctypes.c_void_p, ctypes.c_int]
        _lib.orc_sample_cbd_tensor.argtypes = [mp, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p,
                                               ctypes.c_int, ctypes.c_void_p, ctypes.c_int]
        _lib.orc_cast_tensor.argtypes = [mp, mp, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        _lib.orc_to_uint_tensor.argtypes = [mp, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        _lib.orc_from_uint_tensor.argtypes = [mp, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        _lib.orc_lhe_enc.argtypes = [mp, mp, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p,
                                     ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                     ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        _lib.orc_lhe_dec.argtypes = [mp, mp, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p,
                                     ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int]
        _lib.orc_lhe_keygen.argtypes = [mp, mp, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        _lib.orc_matvec.argtypes = [mp] + [ctypes.c_uint64] * 4 + [ctypes.c_void_p, ctypes.c_uint64,
                                                                    ctypes.c_void_p, ctypes.c_uint64,
                                                                    ctypes.c_void_p, ctypes.c_int]
        _lib.orc_matvec_monomial.argtypes = [mp] + [ctypes.c_uint64] * 4 + [ctypes.c_void_p, ctypes.c_uint64,
                                                                             ctypes.c_void_p, ctypes.c_uint64,
                                                                             ctypes.c_void_p, ctypes.c_int]
        _lib.orc_reduce_mod.argtypes = [mp, ctypes.c_int, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p]
        _lib.orc_reduce_uint.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_uint64, ctypes.c_void_p,
                                         ctypes.c_void_p]
        _lib.orc_equal.argtypes = [ctypes.c_int, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p,
                                   ctypes.c_void_p]
    return _lib


def to_limbs(value, n):
    return [(value >> (32 * i)) & 0xFFFFFFFF for i in range(n)]


def from_limbs(words):
    return sum(int(w) << (32 * i) for i, w in enumerate(words))


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _u32(values):
    arr = (ctypes.c_uint32 * len(values))(*values)
    return arr


class Modulus:
    """A modulus Q with the reference's Montgomery constants (mod.hpp:73-127)."""

    def __init__(self, q):
        self.value = int(q)
        words = max(1, (self.value.bit_length() + 31) // 32)
        self._m = _Modulus()
        rc = lib().orc_modulus_init(ctypes.byref(self._m), _u32(to_limbs(self.value, words)), words)
        if rc:
            raise ValueError(f"unsupported modulus {q:#x} (rc={rc})")
        self.limbs = self._m.limbs
        self.bits = self._m.bits

    @property
    def ref(self):
        return ctypes.byref(self._m)

    @property
    def one(self):
        return from_limbs(self._m.one[: self.limbs])

    @property
    def r2(self):
        return from_limbs(self._m.r2[: self.limbs])

    # scalar helpers (values as Python ints holding the raw limbs)
    def _call2(self, fn, a, b):
        out = (ctypes.c_uint32 * MAX_LIMBS)()
        fn(self.ref, out, _u32(to_limbs(a, self.limbs)), _u32(to_limbs(b, self.limbs)))
        return from_limbs(out[: self.limbs])

    def mul(self, a, b):
        return self._call2(lib().orc_mul, a, b)

    def add(self, a, b):
        return self._call2(lib().orc_add, a, b)

    def sub(self, a, b):
        return self._call2(lib().orc_sub, a, b)

    def from_uint(self, v):
        n = max(1, (int(v).bit_length() + 31) // 32)
        out = (ctypes.c_uint32 * MAX_LIMBS)()
        lib().orc_from_uint(self.ref, out, _u32(to_limbs(int(v), n)), n)
        return from_limbs(out[: self.limbs])

    def from_int(self, v):
        out = (ctypes.c_uint32 * MAX_LIMBS)()
        lib().orc_from_int64(self.ref, out, ctypes.c_int64(int(v)))
        return from_limbs(out[: self.limbs])

    def to_uint(self, x):
        out = (ctypes.c_uint32 * MAX_LIMBS)()
        lib().orc_to_uint(self.ref, out, _u32(to_limbs(x, self.limbs)))
        return from_limbs(out[: self.limbs])

    def cast_from(self, src, x):
        out = (ctypes.c_uint32 * MAX_LIMBS)()
        lib().orc_cast(self.ref, src.ref, out, _u32(to_limbs(x, src.limbs)))
        return from_limbs(out[: self.limbs])

    def root_of_unity(self, degree):
        out = (ctypes.c_uint32 * MAX_LIMBS)()
        rc = lib().orc_root_of_unity(self.ref, ctypes.c_uint64(degree), out)
        if rc:
            raise ValueError(f"no root of unity of degree {degree} (rc={rc})")
        return from_limbs(out[: self.limbs])

    def twiddles(self, n, inverse=False):
        table = np.zeros(n * self.limbs, dtype=np.uint32)
        rc = lib().orc_twiddles(self.ref, ctypes.c_uint64(n), int(inverse), _ptr(table))
        if rc:
            raise ValueError(f"twiddles failed (rc={rc})")
        return table.reshape(n, self.limbs)


def chacha20_block(key, counter, nonce):
    out = (ctypes.c_uint32 * 16)()
    lib().orc_chacha20_block(_u32(key), ctypes.c_uint32(counter), _u32(nonce), out)
    return list(out)


def quarter_round(a, b, c, d):
    v = [ctypes.c_uint32(x) for x in (a, b, c, d)]
    lib().orc_chacha_quarter_round(*[ctypes.byref(x) for x in v])
    return [x.value for x in v]


class Generator:
    def __init__(self, key, nonce, counter):
        self._g = _Generator()
        lib().orc_generator_init(ctypes.byref(self._g), _u32(key), _u32(nonce), ctypes.c_uint32(counter))

    def next(self):
        return lib().orc_generator_next(ctypes.byref(self._g))

    def cbd(self, variance_x2):
        return lib().orc_sample_cbd(ctypes.byref(self._g), variance_x2)


def nonce_add(nonce, v):
    arr = _u32(list(nonce))
    lib().orc_nonce_add(arr, ctypes.c_uint64(v))
    return list(arr)


def planar(values, limbs):
    """list of ints -> limb-planar uint32 array [limbs][len(values)]"""
    arr = np.zeros((limbs, len(values)), dtype=np.uint32)
    for e, v in enumerate(values):
        for j in range(limbs):
            arr[j, e] = (int(v) >> (32 * j)) & 0xFFFFFFFF
    return arr


def unplanar(arr):
    """limb-planar array -> list of ints"""
    arr = np.asarray(arr, dtype=np.uint64)
    out = np.zeros(arr.shape[1], dtype=object)
    for j in range(arr.shape[0]):
        out = out + (arr[j].astype(object) << (32 * j))
    return [int(x) for x in out]


def _producer(kind, src=None, src_modulus=None, variance_x2=0, security=80, key=(0,) * 8, nonce=(0, 0, 0)):
    pr = _Producer()
    pr.kind = kind
    pr.src = None if src is None else src.ctypes.data
    if src_modulus is not None:
        pr.src_modulus = ctypes.pointer(src_modulus._m)
    pr.variance_x2 = variance_x2
    pr.security = security
    for i in range(8):
        pr.key[i] = key[i]
    for i in range(3):
        pr.nonce[i] = nonce[i]
    return pr


def ntt(m, n, batch, *, inverse=False, src=None, src_modulus=None, sampler=None, variance_x2=0, key=(0,) * 8,
        nonce=(0, 0, 0), security=80, threads=0):
    """Batched NTT/INTT with a stage-0 producer; returns limb-planar output."""
    if sampler == "cbd":
        pr = _producer(PRODUCER_CBD, variance_x2=variance_x2, key=key, nonce=nonce)
    elif sampler == "uniform":
        pr = _producer(PRODUCER_UNIFORM, security=security, key=key, nonce=nonce)
    elif src_modulus is not None:
        src = np.ascontiguousarray(src, dtype=np.uint32)
        pr = _producer(PRODUCER_CAST, src=src, src_modulus=src_modulus)
    else:
        src = np.ascontiguousarray(src, dtype=np.uint32)
        pr = _producer(PRODUCER_TENSOR, src=src)
    out = np.zeros((m.limbs, n * batch), dtype=np.uint32)
    rc = lib().orc_ntt(m.ref, n, batch, int(inverse), ctypes.byref(pr), _ptr(out), threads)
    if rc:
        raise ValueError(f"orc_ntt failed (rc={rc})")
    return out


def fma(m, a, b, c, threads=0):
    a, b, c = (np.ascontiguousarray(x, dtype=np.uint32) for x in (a, b, c))
    d = np.zeros_like(a)
    lib().orc_fma(m.ref, a.shape[1], _ptr(a), _ptr(b), _ptr(c), _ptr(d), threads)
    return d


def binary(m, op, a, b, elements=None, threads=0):
    a = np.ascontiguousarray(a, dtype=np.uint32)
    b = np.ascontiguousarray(b, dtype=np.uint32)
    elements = elements or max(a.shape[1], b.shape[1])
    out = np.zeros((m.limbs, elements), dtype=np.uint32)
    lib().orc_binary(m.ref, op, elements, _ptr(a), a.shape[1], _ptr(b), b.shape[1], _ptr(out), threads)
    return out


def sample_uniform(m, elements, key, nonce, security=80, threads=0):
    out = np.zeros((m.limbs, elements), dtype=np.uint32)
    lib().orc_sample_uniform_tensor(m.ref, elements, _u32(key), _u32(nonce), security, _ptr(out), threads)
    return out


def sample_cbd(m, elements, key, nonce, variance_x2, threads=0):
    out = np.zeros((m.limbs, elements), dtype=np.uint32)
    lib().orc_sample_cbd_tensor(m.ref, elements, _u32(key), _u32(nonce), variance_x2, _ptr(out), threads)
    return out


def cast(dst, src, x, threads=0):
    x = np.ascontiguousarray(x, dtype=np.uint32)
    out = np.zeros((dst.limbs, x.shape[1]), dtype=np.uint32)
    lib().orc_cast_tensor(dst.ref, src.ref, x.shape[1], _ptr(x), _ptr(out), threads)
    return out


def to_uint(m, x, threads=0):
    x = np.ascontiguousarray(x, dtype=np.uint32)
    out = np.zeros_like(x)
    lib().orc_to_uint_tensor(m.ref, x.shape[1], _ptr(x), _ptr(out), threads)
    return out


def from_uint(m, x, threads=0):
    x = np.ascontiguousarray(x, dtype=np.uint32)
    out = np.zeros_like(x)
    lib().orc_from_uint_tensor(m.ref, x.shape[1], _ptr(x), _ptr(out), threads)
    return out


def lhe_keygen(q, p, n, key, nonce, threads=0):
    """returns (s, a, b, new_nonce)"""
    s = np.zeros((q.limbs, n), dtype=np.uint32)
    a = np.zeros_like(s)
    b = np.zeros_like(s)
    nn = _u32(list(nonce))
    rc = lib().orc_lhe_keygen(q.ref, p.ref, n, _u32(key), nn, _ptr(s), _ptr(a), _ptr(b), threads)
    if rc:
        raise ValueError(f"keygen failed (rc={rc})")
    return s, a, b, list(nn)


def lhe_enc(q, p, n, batch, key_a, key_b, plaintext, plaintext_ntt, key, nonce, threads=0):
    """returns (c0, c1, new_nonce)"""
    key_a, key_b, plaintext = (np.ascontiguousarray(x, dtype=np.uint32) for x in (key_a, key_b, plaintext))
    c0 = np.zeros((q.limbs, n * batch), dtype=np.uint32)
    c1 = np.zeros_like(c0)
    nn = _u32(list(nonce))
    rc = lib().orc_lhe_enc(q.ref, p.ref, n, batch, _ptr(key_a), _ptr(key_b), _ptr(plaintext), int(plaintext_ntt),
                           _u32(key), nn, _ptr(c0), _ptr(c1), threads)
    if rc:
        raise ValueError(f"enc failed (rc={rc})")
    return c0, c1, list(nn)


def lhe_dec(q, p, n, batch, s, c0, c1, plaintext_ntt, threads=0):
    s, c0, c1 = (np.ascontiguousarray(x, dtype=np.uint32) for x in (s, c0, c1))
    out = np.zeros((p.limbs, n * batch), dtype=np.uint32)
    rc = lib().orc_lhe_dec(q.ref, p.ref, n, batch, _ptr(s), _ptr(c0), _ptr(c1), int(plaintext_ntt), _ptr(out),
                           threads)
    if rc:
        raise ValueError(f"dec failed (rc={rc})")
    return out


def cipher_enc(key, nonce, planar):
    planar = np.ascontiguousarray(planar, dtype=np.uint32)
    limbs, elements = planar.shape
    out = np.zeros(limbs * elements, dtype=np.uint32)
    lib().orc_cipher_enc(_u32(key), _u32(nonce), ctypes.c_uint64(elements), limbs, _ptr(planar), _ptr(out))
    return out


def cipher_dec(key, nonce, flat, limbs):
    flat = np.ascontiguousarray(flat, dtype=np.uint32)
    elements = flat.size // limbs
    out = np.zeros((limbs, elements), dtype=np.uint32)
    lib().orc_cipher_dec(_u32(key), _u32(nonce), ctypes.c_uint64(elements), limbs, _ptr(flat), _ptr(out))
    return out


REDUCE_OPS = {"add": 0, "multiply": 1, "bit_and": 2, "bit_or": 3, "bit_xor": 4, "min": 5, "max": 6}


def matvec(m, batch, rows, cols, coeffs, mat, x, threads=0):
    """z[b][i][c] = sum_k mat[b][i][k][c] * x[b][k][c] mod Q; mat and x are
    limb-planar with a batch of `batch` or 1 (broadcast)."""
    mat = np.ascontiguousarray(mat, dtype=np.uint32)
    x = np.ascontiguousarray(x, dtype=np.uint32)
    m_batch = mat.shape[1] // (rows * cols * coeffs)
    x_batch = x.shape[1] // (cols * coeffs)
    z = np.zeros((m.limbs, batch * rows * coeffs), dtype=np.uint32)
    lib().orc_matvec(m.ref, batch, rows, cols, coeffs, _ptr(mat), m_batch, _ptr(x), x_batch, _ptr(z), threads)
    return z


def matvec_monomial(m, n, batch, rows, cols, degrees, x, threads=0):
    """z[b][i] = sum_k X^degrees[b][i][k] * x[b][k] in Z_Q[X]/(X^n + 1),
    coefficient form; a negative degree is no monomial."""
    degrees = np.ascontiguousarray(degrees, dtype=np.int64).reshape(-1)
    x = np.ascontiguousarray(x, dtype=np.uint32)
    d_batch = degrees.size // (rows * cols)
    x_batch = x.shape[1] // (cols * n)
    z = np.zeros((m.limbs, batch * rows * n), dtype=np.uint32)
    lib().orc_matvec_monomial(m.ref, n, batch, rows, cols, _ptr(degrees), d_batch, _ptr(x), x_batch, _ptr(z),
                              threads)
    return z


def reduce_mod(m, op, x):
    x = np.ascontiguousarray(x, dtype=np.uint32)
    out = np.zeros(m.limbs, dtype=np.uint32)
    if lib().orc_reduce_mod(m.ref, REDUCE_OPS.get(op, op), x.shape[1], _ptr(x), _ptr(out)):
        raise ValueError(f"bad reduction {op}")
    return out


def reduce_uint(op, bits, x):
    x = np.ascontiguousarray(x, dtype=np.uint32)
    out = np.zeros((bits + 31) // 32, dtype=np.uint32)
    if lib().orc_reduce_uint(REDUCE_OPS.get(op, op), bits, x.shape[1], _ptr(x), _ptr(out)):
        raise ValueError(f"bad reduction {op} over {bits} bits")
    return out


def equal(a, b):
    a = np.ascontiguousarray(a, dtype=np.uint32)
    b = np.ascontiguousarray(b, dtype=np.uint32)
    out = np.zeros(a.shape[1], dtype=np.uint32)
    lib().orc_equal(a.shape[0], a.shape[1], _ptr(a), _ptr(b), _ptr(out))
    return out


def cpu_threads():
    return len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()
