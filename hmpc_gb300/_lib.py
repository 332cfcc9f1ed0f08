"""ctypes binding of libhmpc_gb300.so (the C ABI declared in
include/hmpc_gb300.h).  Loading fails loudly when the library has not been
built: there is no CPU fallback."""
import ctypes
import pathlib

HERE = pathlib.Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "libhmpc_gb300.so"
HEADER = HERE.parent / "include" / "hmpc_gb300.h"

HMPC_OK = 0
ERRORS = {
    1: "invalid argument",
    2: "unsupported",
    3: "CUDA error",
    4: "out of memory",
    5: "no root of unity",
    6: "timeout",
    7: "rejected",
}

PRODUCER_TENSOR = 0
PRODUCER_CBD = 1
PRODUCER_UNIFORM = 2
BATCH_DEFAULT, BATCH_AUTOTUNE, BATCH_TENSOR_CORES = 0, 1, 2
OP_ADD, OP_SUB, OP_MUL = 0, 1, 2
REDUCE_OPS = {"add": 0, "multiply": 1, "bit_and": 2, "bit_or": 3, "bit_xor": 4, "min": 5, "max": 6}


class HmpcError(RuntimeError):
    def __init__(self, code, message):
        super().__init__(f"{ERRORS.get(code, code)}: {message}")
        self.code = code


class TcCost(ctypes.Structure):
    _fields_ = [("launches", ctypes.c_uint32), ("bytes", ctypes.c_double), ("flops", ctypes.c_double)]


class WireMessage(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_uint8),
        ("datatype", ctypes.c_uint8),
        ("sender", ctypes.c_uint16),
        ("receiver", ctypes.c_uint16),
        ("id", ctypes.c_uint64),
        ("payload", ctypes.c_void_p),
        ("bytes", ctypes.c_uint64),
        ("planes", ctypes.c_uint32),
        ("plane_stride", ctypes.c_uint64),
    ]


class Producer(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int),
        ("src", ctypes.c_void_p),
        ("variance_x2", ctypes.c_uint32),
        ("security", ctypes.c_uint32),
    ]


_vp = ctypes.c_void_p
_u64 = ctypes.c_uint64
_int = ctypes.c_int
_u32p = ctypes.POINTER(ctypes.c_uint32)

SIGNATURES = {
    "hmpc_last_error": ([], ctypes.c_char_p),
    "hmpc_version": ([ctypes.POINTER(_int), ctypes.POINTER(_int)], _int),
    "hmpc_context_create": ([_int, _u32p, _vp, ctypes.POINTER(_vp)], _int),
    "hmpc_context_destroy": ([_vp], _int),
    "hmpc_context_set_stream": ([_vp, _vp], _int),
    "hmpc_context_get_nonce": ([_vp, _u32p], _int),
    "hmpc_context_set_nonce": ([_vp, _u32p], _int),
    "hmpc_context_synchronize": ([_vp], _int),
    "hmpc_context_launch_count": ([_vp, ctypes.POINTER(_u64)], _int),
    "hmpc_modulus_create": ([_vp, _u32p, _int, ctypes.POINTER(_vp)], _int),
    "hmpc_modulus_destroy": ([_vp], _int),
    "hmpc_modulus_info": ([_vp, ctypes.POINTER(_int), ctypes.POINTER(_int), _u32p], _int),
    "hmpc_modulus_prepare": ([_vp, _u64], _int),
    "hmpc_modulus_root": ([_vp, _u64, _int, _u32p], _int),
    "hmpc_modulus_set_plan": ([_vp, _u64, _u64, _int, _int, _int, _int], _int),
    "hmpc_modulus_get_plan": ([_vp, _u64, _u64, _int] + [ctypes.POINTER(_int)] * 3, _int),
    "hmpc_modulus_tc_cost": ([_vp, _u64, _u64, _int, _int, _int, ctypes.POINTER(TcCost)], _int),
    "hmpc_modulus_tc_column_max": ([_vp, _u64, _int, _int, _u32p], _int),
    "hmpc_context_set_tc_column_bound": ([_vp, ctypes.c_uint32], _int),
    "hmpc_wire_layout": ([ctypes.POINTER(WireMessage), _u64, ctypes.c_uint8, ctypes.POINTER(_u64),
                          ctypes.POINTER(_u64)], _int),
    "hmpc_wire_pack": ([_vp, ctypes.POINTER(WireMessage), _u64, ctypes.c_uint8, ctypes.c_char_p,
                        ctypes.POINTER(_u64), _vp], _int),
    "hmpc_wire_unpack": ([_vp, _vp, ctypes.POINTER(_u64), ctypes.POINTER(_u64), _u64, ctypes.c_uint8,
                          ctypes.c_char_p, ctypes.POINTER(WireMessage), ctypes.POINTER(_vp), _vp], _int),
    "hmpc_wire_message_id": ([ctypes.c_uint8, ctypes.c_uint8, ctypes.POINTER(ctypes.c_uint16), _int,
                              ctypes.POINTER(ctypes.c_uint16), _int, ctypes.POINTER(ctypes.c_uint16), _int, _u64,
                              ctypes.POINTER(_u64)], _int),
    "hmpc_wire_sha256": ([ctypes.c_char_p, _u64, ctypes.c_char_p], _int),
    "hmpc_modulus_tune": ([_vp, _u64, _u64, _int, ctypes.POINTER(ctypes.c_float)], _int),
    "hmpc_modulus_twiddles": ([_vp, _u64, _int, _u32p], _int),
    "hmpc_tensor_alloc": ([_vp, _u64, ctypes.POINTER(_vp)], _int),
    "hmpc_tensor_free": ([_vp, _vp], _int),
    "hmpc_tensor_upload": ([_vp, _vp, _vp, _u64], _int),
    "hmpc_tensor_download": ([_vp, _vp, _vp, _u64], _int),
    "hmpc_ntt_forward": ([_vp, _vp, _u64, _u64, ctypes.POINTER(Producer), _vp], _int),
    "hmpc_ntt_inverse": ([_vp, _vp, _u64, _u64, _vp, _vp], _int),
    "hmpc_ntt_forward_plain": ([_vp, _vp, _u64, _u64, ctypes.POINTER(Producer), _vp], _int),
    "hmpc_ntt_inverse_plain": ([_vp, _vp, _u64, _u64, _vp, _vp], _int),
    "hmpc_lhe_dec2": ([_vp, _vp, _vp, _u64, _u64, _vp, _vp, _vp, _vp, _int, _vp], _int),
    "hmpc_lhe_ct_mul": ([_vp, _vp, _u64, _vp, _vp, _vp, _vp, _vp, _vp, _vp], _int),
    "hmpc_ntt_batch_create": ([_vp, _vp, _u64, ctypes.POINTER(_u64), _int, _int, ctypes.POINTER(_vp)], _int),
    "hmpc_ntt_batch_run": ([_vp, ctypes.POINTER(_vp), ctypes.POINTER(_vp)], _int),
    "hmpc_ntt_batch_info": ([_vp, ctypes.POINTER(_int), ctypes.POINTER(_int), ctypes.POINTER(_int),
                             ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_float)], _int),
    "hmpc_ntt_batch_status": ([_vp, ctypes.POINTER(ctypes.c_uint32)], _int),
    "hmpc_ntt_batch_destroy": ([_vp], _int),
    "hmpc_ntt_batch_set_test_wait": ([_vp, ctypes.c_uint32, ctypes.c_uint32], _int),
    "hmpc_context_set_test_wait": ([_vp, ctypes.c_uint32, _int], _int),
    "hmpc_cipher_enc": ([_vp, _u32p, _u32p, _u64, _int, _vp, _vp], _int),
    "hmpc_cipher_dec": ([_vp, _u32p, _u32p, _u64, _int, _vp, _vp], _int),
    "hmpc_fma": ([_vp, _vp, _u64, _vp, _vp, _vp, _vp], _int),
    "hmpc_binary": ([_vp, _vp, _int, _u64, _vp, _u64, _vp, _u64, _vp], _int),
    "hmpc_sample_uniform": ([_vp, _vp, _u64, ctypes.c_uint32, _vp], _int),
    "hmpc_sample_cbd": ([_vp, _vp, _u64, ctypes.c_uint32, _vp], _int),
    "hmpc_cast": ([_vp, _vp, _vp, _u64, _vp, _vp], _int),
    "hmpc_to_montgomery": ([_vp, _vp, _u64, _vp, _vp], _int),
    "hmpc_from_montgomery": ([_vp, _vp, _u64, _vp, _vp], _int),
    "hmpc_lhe_enc": ([_vp, _vp, _vp, _u64, _u64, _vp, _vp, _vp, _int, _vp, _vp], _int),
    "hmpc_lhe_enc_noalloc": ([_vp, _vp, _vp, _u64, _u64, _vp, _vp, _vp, _int, _vp, _vp], _int),
    "hmpc_lhe_dec": ([_vp, _vp, _vp, _u64, _u64, _vp, _vp, _vp, _int, _vp], _int),
    "hmpc_lhe_keygen": ([_vp, _vp, _vp, _u64, _vp, _vp, _vp], _int),
    "hmpc_matvec": ([_vp, _vp, _u64, _u64, _u64, _u64, _vp, _u64, _vp, _u64, _vp], _int),
    "hmpc_matvec_monomial": ([_vp, _vp, _u64, _u64, _u64, _u64, _vp, _u64, _vp, _u64, _vp], _int),
    "hmpc_reduce": ([_vp, _vp, _int, _u64, _vp, _vp], _int),
    "hmpc_reduce_uint": ([_vp, _int, _int, _u64, _vp, _vp], _int),
    "hmpc_equal": ([_vp, _int, _u64, _vp, _vp, _vp], _int),
}

_lib = None


def load():
    """Load the library (building is a separate step: hmpc_gb300.build)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(
                f"{LIB_PATH} is missing: build the CUDA extension first "
                "(python -c 'import __graft_entry__ as g; g.build()')")
        lib = ctypes.CDLL(str(LIB_PATH))
        for name, (args, res) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = res
        _lib = lib
    return _lib


def check(rc):
    if rc != HMPC_OK:
        msg = load().hmpc_last_error()
        raise HmpcError(rc, msg.decode() if msg else "")
    return rc


def call(name, *args):
    return check(getattr(load(), name)(*args))


def declared_symbols():
    """Entry points declared in include/hmpc_gb300.h."""
    import re

    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:const char\*|int)\s+(hmpc_\w+)\(", text, re.M)))
