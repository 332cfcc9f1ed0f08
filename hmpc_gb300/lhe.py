"""Linear BGV (hmpc/expr/crypto/lhe, hmpc/comp/crypto/lhe): keys, ciphertexts,
encryption and decryption on the GPU through the C ABI."""
import ctypes
from dataclasses import dataclass

from . import _lib
from .comp import Tensor, make_tensor


@dataclass
class Key:
    """comp::crypto::lhe::key{a, b} (comp/crypto/lhe/key.hpp:7-12): one
    polynomial each, NTT representation mod q."""
    a: Tensor
    b: Tensor


@dataclass
class Ciphertext:
    """comp::crypto::lhe::ciphertext{c0, c1} (comp/crypto/lhe/ciphertext.hpp:8-32)"""
    c0: Tensor
    c1: Tensor


def keygen(queue, q, p, n):
    """Secret s and public key (a, b) with a = b*s + p*e (no counterpart in
    the reference, whose keys are given tensors).  Returns (s, Key)."""
    s = make_tensor(q, (), n)
    a = make_tensor(q, (), n)
    b = make_tensor(q, (), n)
    _lib.call("hmpc_lhe_keygen", queue.handle, q.handle, p.handle, n, s.ptr(), a.ptr(), b.ptr())
    return s, Key(a, b)


def enc(queue, key, plaintext, q, plaintext_ntt=False, out=None):
    """enc(key, tensor(x), randomness<Rq>(shape)) (expr/crypto/lhe/enc.hpp:19-69)"""
    n = plaintext.n
    if out is None:
        out = Ciphertext(make_tensor(q, plaintext.shape, n), make_tensor(q, plaintext.shape, n))
    _lib.call("hmpc_lhe_enc", queue.handle, q.handle, plaintext.modulus.handle, n, plaintext.batch, key.a.ptr(),
              key.b.ptr(), plaintext.ptr(), int(plaintext_ntt), out.c0.ptr(), out.c1.ptr())
    return out


def dec(queue, s, ct, p, plaintext_ntt=False, out=None):
    """dec<Plaintext>(s, ct) (expr/crypto/lhe/dec.hpp:13-45)"""
    c0 = ct.c0
    out = out or make_tensor(p, c0.shape, c0.n)
    _lib.call("hmpc_lhe_dec", queue.handle, c0.modulus.handle, p.handle, c0.n, c0.batch, s.ptr(), c0.ptr(),
              ct.c1.ptr(), int(plaintext_ntt), out.ptr())
    return out


@dataclass
class Ciphertext2:
    """degree-2 ciphertext (c0, c1, c2): the product of two ciphertexts"""
    c0: Tensor
    c1: Tensor
    c2: Tensor


def mul(queue, x, y):
    """ciphertext x ciphertext: the NTT-domain tensor product (no counterpart in
    the reference, whose ciphertexts are linear only)"""
    a0 = x.c0
    out = Ciphertext2(*(make_tensor(a0.modulus, a0.shape, a0.n) for _ in range(3)))
    _lib.call("hmpc_lhe_ct_mul", queue.handle, a0.modulus.handle, a0.elements, x.c0.ptr(), x.c1.ptr(), y.c0.ptr(),
              y.c1.ptr(), out.c0.ptr(), out.c1.ptr(), out.c2.ptr())
    return out


def dec2(queue, s, ct, p, plaintext_ntt=False, out=None):
    """decryption of a degree-2 ciphertext: c0 - s*c1 + s^2*c2"""
    c0 = ct.c0
    out = out or make_tensor(p, c0.shape, c0.n)
    _lib.call("hmpc_lhe_dec2", queue.handle, c0.modulus.handle, p.handle, c0.n, c0.batch, s.ptr(), c0.ptr(),
              ct.c1.ptr(), ct.c2.ptr(), int(plaintext_ntt), out.ptr())
    return out


def add(queue, x, y):
    """ciphertext + ciphertext (expr/crypto/lhe/ciphertext.hpp:49-53)"""
    return Ciphertext(queue.add(x.c0, y.c0), queue.add(x.c1, y.c1))


def sub(queue, x, y):
    """ciphertext - ciphertext (ciphertext.hpp:56-60)"""
    return Ciphertext(queue.sub(x.c0, y.c0), queue.sub(x.c1, y.c1))


def mul_plain(queue, x, m):
    """ciphertext * plaintext (NTT form mod q, broadcast allowed) (ciphertext.hpp:69-81)"""
    return Ciphertext(queue.mul(x.c0, m), queue.mul(x.c1, m))
