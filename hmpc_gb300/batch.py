"""Batched transforms of polynomials of uneven degree (one persistent kernel
launch from a captured CUDA graph, autotuned tile shape)."""
import ctypes

import numpy as np

from . import _lib
from .comp import Tensor


class NttBatch:
    """A planned batch: `degrees[i]` is the ring degree of polynomial i."""

    def __init__(self, queue, modulus, degrees, inverse=False, autotune=True, tensor_cores=False):
        """autotune: time the CUDA-core tile shapes and the tensor-core engine
        and keep the fastest; tensor_cores: the tensor-core engine (one
        transform per degree over the polynomials' own buffers)"""
        self.queue = queue
        self.modulus = modulus
        self.degrees = [int(d) for d in degrees]
        handle = ctypes.c_void_p()
        arr = (ctypes.c_uint64 * len(self.degrees))(*self.degrees)
        mode = _lib.BATCH_TENSOR_CORES if tensor_cores else (_lib.BATCH_AUTOTUNE if autotune else _lib.BATCH_DEFAULT)
        _lib.call("hmpc_ntt_batch_create", queue.handle, modulus.handle, len(self.degrees), arr, int(inverse),
                  mode, ctypes.byref(handle))
        self.handle = handle

    def info(self):
        r, lb, cb = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        items, ms = ctypes.c_uint32(), ctypes.c_float()
        _lib.call("hmpc_ntt_batch_info", self.handle, ctypes.byref(r), ctypes.byref(lb), ctypes.byref(cb),
                  ctypes.byref(items), ctypes.byref(ms))
        return {"engine": "tensor" if r.value == 0 else "cuda", "radix": 1 << r.value, "local_bits": lb.value,
                "col_bits": cb.value, "items": items.value, "tuned_ms": ms.value}

    def run(self, inputs, outputs=None):
        """inputs / outputs: lists of Tensors (one polynomial each)"""
        if outputs is None:
            outputs = [Tensor(self.modulus, (), d) for d in self.degrees]
        ins = (ctypes.c_void_p * len(inputs))(*[t.data.data_ptr() for t in inputs])
        outs = (ctypes.c_void_p * len(outputs))(*[t.data.data_ptr() for t in outputs])
        _lib.call("hmpc_ntt_batch_run", self.handle, ins, outs)
        return outputs

    def status(self):
        failed = ctypes.c_uint32()
        _lib.call("hmpc_ntt_batch_status", self.handle, ctypes.byref(failed))
        return failed.value

    def close(self):
        if self.handle:
            _lib.call("hmpc_ntt_batch_destroy", self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def uneven_degrees(count, log_min=12, log_max=16, seed=0):
    """Degrees drawn uniformly from {2^log_min..2^log_max} by a seeded ChaCha20
    stream (one word per polynomial, reduced modulo the number of choices)."""
    import struct

    from .moduli import chacha20_words

    words = chacha20_words([seed] + [0] * 7, count)
    choices = log_max - log_min + 1
    return [1 << (log_min + (w % choices)) for w in words]
