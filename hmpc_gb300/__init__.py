"""hmpc_gb300: GB300-native (sm_103a) implementation of hmpc's data-parallel
hot path -- multi-limb Montgomery NTT/INTT, modular FMA, ChaCha20 samplers
and linear BGV -- behind a C ABI (include/hmpc_gb300.h)."""
from . import _lib
from .comp import Modulus, Queue, Tensor, make_tensor

__all__ = ["Modulus", "Queue", "Tensor", "make_tensor", "build", "library_path"]


def build(verbose=False):
    from .build import build as _build

    return _build(verbose=verbose)


def library_path():
    return _lib.LIB_PATH
