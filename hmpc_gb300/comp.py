"""Device-side objects that mirror hmpc::comp: the queue (one GPU, its stream
and the RNG capability), moduli, and limb-planar tensors.

Reference interfaces: hmpc/comp/queue.hpp:163-599 (queue), hmpc/comp/tensor.hpp
:9-90 (tensor, make_tensor), hmpc/ints/mod.hpp:73-193 (mod<Q>).  Every
operation runs through the C ABI of libhmpc_gb300.so; PyTorch only provides
device memory and the stream.
"""
import ctypes
import os

import numpy as np
import torch

from . import _lib


def _words(value, n=None):
    value = int(value)
    n = n or max(1, (value.bit_length() + 31) // 32)
    return [(value >> (32 * i)) & 0xFFFFFFFF for i in range(n)]


def _u32_array(values):
    return (ctypes.c_uint32 * len(values))(*values)


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)


class Modulus:
    """mod<Q> registered on a queue: L, bit width and Montgomery one
    (hmpc/ints/mod.hpp:90-127).  Twiddle tables per ring degree are cached on
    the device (hmpc/comp/queue.hpp:364-381)."""

    def __init__(self, queue, q):
        self.queue = queue
        self.value = int(q)
        handle = ctypes.c_void_p()
        words = _words(self.value)
        _lib.call("hmpc_modulus_create", queue.handle, _u32_array(words), len(words), ctypes.byref(handle))
        self.handle = handle
        limbs, bits = ctypes.c_int(), ctypes.c_int()
        one = (ctypes.c_uint32 * 16)()
        _lib.call("hmpc_modulus_info", handle, ctypes.byref(limbs), ctypes.byref(bits), one)
        self.limbs = limbs.value
        self.bits = bits.value
        self.one = sum(int(one[i]) << (32 * i) for i in range(self.limbs))

    def prepare(self, n):
        _lib.call("hmpc_modulus_prepare", self.handle, n)

    def set_plan(self, n, batch, inverse=False, radix_bits=3, local_bits=0, col_bits=4):
        _lib.call("hmpc_modulus_set_plan", self.handle, n, batch, int(inverse), radix_bits, local_bits, col_bits)

    def tune(self, n, batch, inverse=False):
        """time the tile shapes for this (degree, batch, direction); returns ms"""
        ms = ctypes.c_float()
        _lib.call("hmpc_modulus_tune", self.handle, n, batch, int(inverse), ctypes.byref(ms))
        return ms.value

    def plan(self, n, batch, inverse=False):
        """the tile shape (radix_bits, local_bits, col_bits) these transforms run with"""
        r, lb, cb = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _lib.call("hmpc_modulus_get_plan", self.handle, n, batch, int(inverse), ctypes.byref(r), ctypes.byref(lb),
                  ctypes.byref(cb))
        return {"radix_bits": r.value, "local_bits": lb.value, "col_bits": cb.value}

    def tc_column_max(self, n, inverse=False, splits=1):
        """largest column sum of |digit| of the tensor-core constants of (n, direction, splits)"""
        out = ctypes.c_uint32()
        _lib.call("hmpc_modulus_tc_column_max", self.handle, n, int(inverse), splits, ctypes.byref(out))
        return out.value

    def tc_cost(self, n, batch, inverse=False, producer=_lib.PRODUCER_TENSOR, splits=1):
        """launches, algorithmic DRAM bytes and MMA flops of one tensor-core transform"""
        out = _lib.TcCost()
        _lib.call("hmpc_modulus_tc_cost", self.handle, n, batch, int(inverse), producer, splits, ctypes.byref(out))
        return {"launches": out.launches, "bytes": out.bytes, "flops": out.flops}

    def root(self, n, inverse=False):
        out = (ctypes.c_uint32 * 16)()
        _lib.call("hmpc_modulus_root", self.handle, n, int(inverse), out)
        return sum(int(out[i]) << (32 * i) for i in range(self.limbs))

    def twiddles(self, n, inverse=False):
        table = np.zeros(n * self.limbs, dtype=np.uint32)
        _lib.call("hmpc_modulus_twiddles", self.handle, n, int(inverse),
                  table.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)))
        return table.reshape(n, self.limbs)

    def __repr__(self):
        return f"Modulus({self.value:#x}, limbs={self.limbs})"


class Tensor:
    """comp::tensor<T, Dimensions...>: limb-planar device storage
    [limbs][elements] (hmpc/comp/tensor.hpp:21,25-29).  `shape` is the batch
    shape and `n` the polynomial degree (1 for plain residues), so elements =
    prod(shape) * n in (batch..., coefficient) row-major order."""

    def __init__(self, modulus, shape, n=1, data=None):
        self.modulus = modulus
        self.shape = tuple(int(s) for s in shape)
        self.n = int(n)
        self.elements = int(np.prod(self.shape, dtype=np.int64)) * self.n
        if data is None:
            data = torch.empty((modulus.limbs, self.elements), dtype=torch.int32, device=modulus.queue.device)
        assert data.dtype == torch.int32 and data.shape == (modulus.limbs, self.elements) and data.is_contiguous()
        self.data = data

    @property
    def batch(self):
        return int(np.prod(self.shape, dtype=np.int64))

    def numpy(self):
        return self.data.cpu().numpy().view(np.uint32)

    @classmethod
    def from_numpy(cls, modulus, array, shape, n=1):
        array = np.ascontiguousarray(array, dtype=np.uint32)
        data = torch.from_numpy(array.view(np.int32)).to(modulus.queue.device)
        return cls(modulus, shape, n, data.contiguous())

    def ptr(self):
        return _ptr(self.data)


def make_tensor(modulus, shape, n=1):
    """hmpc::comp::make_tensor<T>(shape) (hmpc/comp/tensor.hpp:86-90)"""
    return Tensor(modulus, shape, n)


class Queue:
    """hmpc::comp::queue on one GPU: the stream, the 8-word ChaCha20 key and
    the 96-bit nonce of the RNG capability (hmpc/comp/queue.hpp:175-253)."""

    def __init__(self, key=None, device=0, stream=None):
        self.device = torch.device("cuda", device)
        if key is None:
            key = list(np.frombuffer(os.urandom(32), dtype=np.uint32))  # queue.hpp:229-233
        self.key = [int(k) & 0xFFFFFFFF for k in key]
        self.stream = stream if stream is not None else torch.cuda.current_stream(self.device)
        handle = ctypes.c_void_p()
        _lib.call("hmpc_context_create", device, _u32_array(self.key), ctypes.c_void_p(self.stream.cuda_stream),
                  ctypes.byref(handle))
        self.handle = handle
        self._moduli = {}

    def close(self):
        if self.handle:
            _lib.call("hmpc_context_destroy", self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream):
        self.stream = stream
        _lib.call("hmpc_context_set_stream", self.handle, ctypes.c_void_p(stream.cuda_stream))

    @property
    def nonce(self):
        out = (ctypes.c_uint32 * 3)()
        _lib.call("hmpc_context_get_nonce", self.handle, out)
        return [int(x) for x in out]

    @nonce.setter
    def nonce(self, value):
        _lib.call("hmpc_context_set_nonce", self.handle, _u32_array([int(v) & 0xFFFFFFFF for v in value]))

    @property
    def launches(self):
        """kernels launched through this queue so far"""
        out = ctypes.c_uint64()
        _lib.call("hmpc_context_launch_count", self.handle, ctypes.byref(out))
        return out.value

    def set_tc_column_bound(self, bound):
        """lower the tensor-core engine's column bound for constants built afterwards"""
        _lib.call("hmpc_context_set_tc_column_bound", self.handle, int(bound))

    def wait(self):
        """queue.wait() (hmpc/comp/queue.hpp:531-534)"""
        _lib.call("hmpc_context_synchronize", self.handle)

    def modulus(self, q):
        q = int(q)
        if q not in self._moduli:
            self._moduli[q] = Modulus(self, q)
        return self._moduli[q]

    # ------------------------------------------------------------ transforms
    def ntt(self, x, out=None):
        """number_theoretic_transform(tensor(x))"""
        out = out or make_tensor(x.modulus, x.shape, x.n)
        prod = _lib.Producer(_lib.PRODUCER_TENSOR, x.data.data_ptr(), 0, 0)
        _lib.call("hmpc_ntt_forward", self.handle, x.modulus.handle, x.n, x.batch, ctypes.byref(prod), out.ptr())
        return out

    def intt(self, x, out=None):
        """inverse_number_theoretic_transform(tensor(x))"""
        out = out or make_tensor(x.modulus, x.shape, x.n)
        _lib.call("hmpc_ntt_inverse", self.handle, x.modulus.handle, x.n, x.batch, x.ptr(), out.ptr())
        return out

    def ntt_centered_binomial(self, modulus, n, shape, variance_x2, out=None):
        """number_theoretic_transform(centered_binomial<R>(shape, V)), 2V = variance_x2;
        the sampler runs inside the transform's first pass."""
        out = out or make_tensor(modulus, shape, n)
        prod = _lib.Producer(_lib.PRODUCER_CBD, None, variance_x2, 0)
        _lib.call("hmpc_ntt_forward", self.handle, modulus.handle, n, out.batch, ctypes.byref(prod), out.ptr())
        return out

    def ntt_uniform(self, modulus, n, shape, security=80, out=None):
        """number_theoretic_transform(uniform<R>(shape))"""
        out = out or make_tensor(modulus, shape, n)
        prod = _lib.Producer(_lib.PRODUCER_UNIFORM, None, 0, security)
        _lib.call("hmpc_ntt_forward", self.handle, modulus.handle, n, out.batch, ctypes.byref(prod), out.ptr())
        return out

    def ntt_plain(self, x, out=None, inverse=False):
        """the per-stage comparator transform (one launch per stage)"""
        out = out or make_tensor(x.modulus, x.shape, x.n)
        if inverse:
            _lib.call("hmpc_ntt_inverse_plain", self.handle, x.modulus.handle, x.n, x.batch, x.ptr(), out.ptr())
        else:
            prod = _lib.Producer(_lib.PRODUCER_TENSOR, x.data.data_ptr(), 0, 0)
            _lib.call("hmpc_ntt_forward_plain", self.handle, x.modulus.handle, x.n, x.batch, ctypes.byref(prod),
                      out.ptr())
        return out

    def ntt_plain_centered_binomial(self, modulus, n, shape, variance_x2, out=None):
        out = out or make_tensor(modulus, shape, n)
        prod = _lib.Producer(_lib.PRODUCER_CBD, None, variance_x2, 0)
        _lib.call("hmpc_ntt_forward_plain", self.handle, modulus.handle, n, out.batch, ctypes.byref(prod),
                  out.ptr())
        return out

    # ----------------------------------------------------------- elementwise
    def fma(self, a, b, c, out=None):
        out = out or make_tensor(a.modulus, a.shape, a.n)
        _lib.call("hmpc_fma", self.handle, a.modulus.handle, a.elements, a.ptr(), b.ptr(), c.ptr(), out.ptr())
        return out

    def binary(self, op, a, b, out=None):
        big = a if a.elements >= b.elements else b
        out = out or make_tensor(big.modulus, big.shape, big.n)
        _lib.call("hmpc_binary", self.handle, big.modulus.handle, op, out.elements, a.ptr(), a.elements, b.ptr(),
                  b.elements, out.ptr())
        return out

    def add(self, a, b, out=None):
        return self.binary(_lib.OP_ADD, a, b, out)

    def sub(self, a, b, out=None):
        return self.binary(_lib.OP_SUB, a, b, out)

    def mul(self, a, b, out=None):
        return self.binary(_lib.OP_MUL, a, b, out)

    def uniform(self, modulus, shape, n=1, security=80, out=None):
        """uniform<T>(shape) evaluated elementwise (expr/random/uniform.hpp:11-46)"""
        out = out or make_tensor(modulus, shape, n)
        _lib.call("hmpc_sample_uniform", self.handle, modulus.handle, out.elements, security, out.ptr())
        return out

    def centered_binomial(self, modulus, shape, variance_x2, n=1, out=None):
        out = out or make_tensor(modulus, shape, n)
        _lib.call("hmpc_sample_cbd", self.handle, modulus.handle, out.elements, variance_x2, out.ptr())
        return out

    def cast(self, x, modulus, out=None):
        """cast<mod<Q'>>(x): centred lift (hmpc/ints/mod.hpp:259-307)"""
        out = out or make_tensor(modulus, x.shape, x.n)
        _lib.call("hmpc_cast", self.handle, modulus.handle, x.modulus.handle, x.elements, x.ptr(), out.ptr())
        return out

    def cipher_enc(self, key, nonce, x):
        """enc(cipher(key, nonce), tensor(x)): element-major int32 words
        (expr/crypto/cipher.hpp:59-173)"""
        out = torch.empty(x.elements * x.modulus.limbs, dtype=torch.int32, device=self.device)
        _lib.call("hmpc_cipher_enc", self.handle, _u32_array(key), _u32_array(nonce), x.elements, x.modulus.limbs,
                  x.ptr(), _ptr(out))
        return out

    def cipher_dec(self, key, nonce, words, modulus, shape, n=1):
        """dec<T>(cipher(key, nonce), y) back to a limb-planar tensor"""
        out = make_tensor(modulus, shape, n)
        _lib.call("hmpc_cipher_dec", self.handle, _u32_array(key), _u32_array(nonce), out.elements, modulus.limbs,
                  _ptr(words), out.ptr())
        return out

    def to_montgomery(self, x, out=None):
        out = out or make_tensor(x.modulus, x.shape, x.n)
        _lib.call("hmpc_to_montgomery", self.handle, x.modulus.handle, x.elements, x.ptr(), out.ptr())
        return out

    def from_montgomery(self, x, out=None):
        out = out or make_tensor(x.modulus, x.shape, x.n)
        _lib.call("hmpc_from_montgomery", self.handle, x.modulus.handle, x.elements, x.ptr(), out.ptr())
        return out

    # ------------------------------------------- matrix products, reductions
    def matrix_vector_product(self, m, x, out=None):
        """hmpc::expr::matrix_vector_product(m, x) of residue tensors
        (hmpc/expr/matrix_vector_product.hpp:88-140): m has shape
        (batch or 1, rows, cols), x shape (batch or 1, cols), both with the
        same n (coefficients of NTT-form polynomials, whose ring product is
        elementwise; 1 for plain residues); the result has shape (batch, rows)."""
        mb, rows, cols = m.shape
        xb, xcols = x.shape
        if xcols != cols or m.n != x.n:
            raise ValueError("matrix columns and vector length differ")
        batch = max(mb, xb)
        out = out or make_tensor(m.modulus, (batch, rows), m.n)
        _lib.call("hmpc_matvec", self.handle, m.modulus.handle, batch, rows, cols, m.n, m.ptr(), mb, x.ptr(), xb,
                  out.ptr())
        return out

    def monomial_matrix_vector_product(self, degrees, x, out=None):
        """matrix_vector_product(bit_monomial<n>(degrees), x)
        (hmpc/expr/bit_monomial.hpp:18-165): degrees is an int64 device
        tensor of shape (batch or 1, rows, cols), -1 for std::nullopt; x holds
        coefficient-form polynomials of shape (batch or 1, cols)."""
        db, rows, cols = degrees.shape
        xb, xcols = x.shape
        if xcols != cols or degrees.dtype != torch.int64 or not degrees.is_contiguous():
            raise ValueError("degrees must be a contiguous int64 tensor matching the vector length")
        batch = max(db, xb)
        out = out or make_tensor(x.modulus, (batch, rows), x.n)
        _lib.call("hmpc_matvec_monomial", self.handle, x.modulus.handle, x.n, batch, rows, cols, _ptr(degrees), db,
                  x.ptr(), xb, out.ptr())
        return out

    def reduce(self, x, op):
        """hmpc::expr::reduce(x, op) of a residue tensor to one value
        (hmpc/expr/reduce.hpp:206-277): op "add" or "multiply"."""
        out = make_tensor(x.modulus, ())
        _lib.call("hmpc_reduce", self.handle, x.modulus.handle, _lib.REDUCE_OPS[op], x.elements, x.ptr(), out.ptr())
        return out

    def sum(self, x):
        return self.reduce(x, "add")

    def product(self, x):
        return self.reduce(x, "multiply")

    def reduce_uint(self, data, bits, op):
        """reduce over uint<bits> values held limb-planar in an int32 device
        tensor of shape (ceil(bits / 32), elements); returns the (limbs,) value"""
        limbs = (bits + 31) // 32
        if data.dim() != 2 or data.shape[0] != limbs or data.dtype != torch.int32 or not data.is_contiguous():
            raise ValueError("uint tensors are contiguous int32 [limbs][elements]")
        out = torch.empty(limbs, dtype=torch.int32, device=self.device)
        _lib.call("hmpc_reduce_uint", self.handle, _lib.REDUCE_OPS[op], bits, data.shape[1], _ptr(data), _ptr(out))
        return out

    def equal(self, a, b):
        """the hmpc::bit tensor of a == b (one int32 0/1 per element) for two
        limb-planar int32 tensors of the same shape"""
        if a.shape != b.shape or a.dim() != 2:
            raise ValueError("operands differ in shape")
        out = torch.empty(a.shape[1], dtype=torch.int32, device=self.device)
        _lib.call("hmpc_equal", self.handle, a.shape[0], a.shape[1], _ptr(a), _ptr(b), _ptr(out))
        return out

    def all(self, bits):
        """hmpc::expr::all of a bit tensor (one int32 0/1 per element)"""
        return bool(self.reduce_uint(bits.reshape(1, -1), 1, "bit_and").item())

    def any(self, bits):
        """hmpc::expr::any of a bit tensor"""
        return bool(self.reduce_uint(bits.reshape(1, -1), 1, "bit_or").item())
