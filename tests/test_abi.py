"""The C-ABI library loads and exports every entry point that
include/hmpc_gb300.h declares (no device needed: nothing is called)."""
import ctypes

from hmpc_gb300 import _lib


def test_library_exports_declared_symbols():
    lib = ctypes.CDLL(str(_lib.LIB_PATH))
    declared = _lib.declared_symbols()
    assert len(declared) >= 30
    missing = [name for name in declared if not hasattr(lib, name)]
    assert not missing
    assert set(_lib.SIGNATURES) <= set(declared)


def test_last_error_without_device_calls():
    lib = _lib.load()
    major, minor = ctypes.c_int(), ctypes.c_int()
    assert lib.hmpc_version(ctypes.byref(major), ctypes.byref(minor)) == 0
    assert lib.hmpc_last_error() == b""
    # argument validation happens before any CUDA call
    assert lib.hmpc_context_create(0, None, None, None) == 1
    assert b"null" in lib.hmpc_last_error()


def test_rate_probe_library_is_separate():
    """the benchmark's rate probes live in their own library, outside the
    product's ABI"""
    import importlib

    _build = importlib.import_module("hmpc_gb300.build")

    probes = ctypes.CDLL(str(_build.PROBES))
    assert hasattr(probes, "hmpc_bench_int_multiply_rate") and hasattr(probes, "hmpc_bench_chacha_rate")
    assert not any("probe" in name for name in _lib.declared_symbols())
