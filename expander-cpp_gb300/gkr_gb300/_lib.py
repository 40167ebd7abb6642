"""ctypes binding of libgkrgpu.so (include/gkrgpu.h).

The library is built in-tree by gkr_gb300.build; loading fails loudly when it is missing
(there is no CPU fallback for the prove path).
"""
import ctypes
import os

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libgkrgpu.so")

OK, ERR_INVALID, ERR_CUDA, ERR_NOMEM, ERR_CAPACITY, ERR_TIMEOUT, ERR_STATE, ERR_IO = range(8)

# Field_type numbering of include/configuration/config.hpp:12-16 (GKRGPU_FIELD_*).
FIELDS = {"M31": 0, "BabyBear": 1, "BN254": 2}
# FiatShamir_hash_type numbering (include/configuration/config.hpp:18-24)
FS_HASHES = {"SHA256": 0, "Keccak256": 1}


class GkrGpuError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"gkrgpu error {code}: {msg}")
        self.code = code


class MulGate(ctypes.Structure):
    _fields_ = [("o_id", ctypes.c_uint32), ("i0", ctypes.c_uint32), ("i1", ctypes.c_uint32), ("coef", ctypes.c_uint32)]


class AddGate(ctypes.Structure):
    _fields_ = [("o_id", ctypes.c_uint32), ("i0", ctypes.c_uint32), ("coef", ctypes.c_uint32)]


class LayerDesc(ctypes.Structure):
    _fields_ = [("nb_output_vars", ctypes.c_uint32), ("nb_input_vars", ctypes.c_uint32),
                ("n_mul", ctypes.c_uint64), ("n_add", ctypes.c_uint64),
                ("mul", ctypes.c_void_p), ("add", ctypes.c_void_p)]


class TileChoice(ctypes.Structure):
    _fields_ = [("threads_per_row", ctypes.c_uint32), ("ctas", ctypes.c_uint32), ("ms", ctypes.c_double)]


class KernelStat(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char_p), ("launches", ctypes.c_uint64), ("total_ms", ctypes.c_double),
                ("algorithmic_bytes", ctypes.c_double)]


# Every entry point include/gkrgpu.h declares: (name, restype, argtypes).
_P, _U32, _U64, _I = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int
SIGNATURES = [
    ("gkrgpu_last_error", ctypes.c_char_p, []),
    ("gkrgpu_version", ctypes.c_char_p, []),
    ("gkrgpu_num_repetitions", _I, [_I]),
    ("gkrgpu_num_repetitions_field", _I, [_I, _I]),
    ("gkrgpu_field_bytes", _U32, [_I]),
    ("gkrgpu_create", _I, [_I, ctypes.POINTER(_P)]),
    ("gkrgpu_destroy", None, [_P]),
    ("gkrgpu_circuit_load", _I, [_P, _P, _I, ctypes.POINTER(_P)]),
    ("gkrgpu_circuit_load_field", _I, [_P, _P, _I, _I, ctypes.POINTER(_P)]),
    ("gkrgpu_circuit_field", _I, [_P]),
    ("gkrgpu_circuit2_parse", _I, [_P, _U64, ctypes.POINTER(_P)]),
    ("gkrgpu_extracted_parse", _I, [_P, _U64, _P, _U64, ctypes.POINTER(_P)]),
    ("gkrgpu_parsed_layers", _I, [_P]),
    ("gkrgpu_parsed_layer", _I, [_P, _I, _P]),
    ("gkrgpu_parsed_free", None, [_P]),
    ("gkrgpu_circuit_free", None, [_P]),
    ("gkrgpu_proof_size", _U64, [_P, _U32, _I]),
    ("gkrgpu_value_rows", _U64, [_P, _I]),
    ("gkrgpu_evaluate", _I, [_P, _P, _U32, _P, _P, _I]),
    ("gkrgpu_prove", _I, [_P, _P, _U32, _I, _P, _P, _U64, ctypes.POINTER(_U64), _P]),
    ("gkrgpu_prove_device", _I, [_P, _P, _U32, _I, _P, _P, _U64, ctypes.POINTER(_U64), _P]),
    ("gkrgpu_prove_submit", _I, [_P, _P, _U32, _I, _P, _I, _P, _U64, _P, _I, ctypes.POINTER(_P)]),
    ("gkrgpu_prove_wait", _I, [_P, ctypes.POINTER(_U64)]),
    ("gkrgpu_prove_submit_resident", _I, [_P, _P, _U32, _I, _P, _P, _P, _U64, _P, _I, ctypes.POINTER(_P)]),
    ("gkrgpu_verify", _I, [_P, _P, _U32, _I, _P, _U64, _P, ctypes.POINTER(_I)]),
    ("gkrgpu_set_fs_hash", _I, [_P, _I]),
    ("gkrgpu_keccak256", None, [_P, _U64, _P]),
    ("gkrgpu_sha3_256", None, [_P, _U64, _P]),
    ("gkrgpu_set_concurrency", _I, [_P, _I, _U64]),
    ("gkrgpu_set_host_threads", _I, [_P, _I]),
    ("gkrgpu_workspace_bytes", _U64, [_P, _U32, _I, _I]),
    ("gkrgpu_memory_stats", _I, [_P, ctypes.POINTER(_U64), ctypes.POINTER(_U64), ctypes.POINTER(_U64)]),
    ("gkrgpu_eval_multilinear", _I, [_P, _P, _U32, _U32, _P, _I, _P]),
    ("gkrgpu_eval_multilinear_noalloc", _I, [_P, _U32, _U32, _P, _I, _P, _P]),
    ("gkrgpu_set_round_tail", _I, [_P, _I]),
    ("gkrgpu_check_device_wait", _I, [_P, _U32, ctypes.POINTER(_I), ctypes.POINTER(_I)]),
    ("gkrgpu_device_alloc", _I, [_P, _U64, ctypes.POINTER(_P)]),
    ("gkrgpu_device_free", _I, [_P, _P]),
    ("gkrgpu_host_alloc", _I, [_U64, ctypes.POINTER(_P)]),
    ("gkrgpu_host_free", _I, [_P]),
    ("gkrgpu_memcpy_h2d", _I, [_P, _P, _P, _U64]),
    ("gkrgpu_memcpy_d2h", _I, [_P, _P, _P, _U64]),
    ("gkrgpu_upload", _I, [_P, _P, _P, _U64]),
    ("gkrgpu_set_timing", _I, [_P, _I]),
    ("gkrgpu_reset_stats", _I, [_P]),
    ("gkrgpu_kernel_stats", _I, [_P, _P, _I]),
    ("gkrgpu_set_tile", _I, [_P, _U32, _U32, _U32]),
    ("gkrgpu_autotune", _I, [_P, _P, _U32, _I, _P, _I, _P, _I]),
    ("gkrgpu_mark", _I, [_P, _I]),
    ("gkrgpu_elapsed_ms", _I, [_P, _I, _I, ctypes.POINTER(ctypes.c_double)]),
    ("gkrgpu_transfer_stats", _I, [_P, ctypes.POINTER(_U64), ctypes.POINTER(_U64)]),
    ("gkrgpu_proof_write", _I, [ctypes.c_char_p, _P, _U64]),
    ("gkrgpu_proof_read", _I, [ctypes.c_char_p, _P, _U64, ctypes.POINTER(_U64)]),
]

_lib = None


def load():
    """Loads and types the library (once)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is not built; run __graft_entry__.build() (or gkr_gb300.build.build())")
    lib = ctypes.CDLL(LIB_PATH)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc):
    if rc != OK:
        msg = load().gkrgpu_last_error()
        raise GkrGpuError(rc, msg.decode() if msg else "")
    return rc


def _digest(fn, data: bytes) -> bytes:
    buf = (ctypes.c_uint8 * max(len(data), 1)).from_buffer_copy(data or b"\0")
    out = (ctypes.c_uint8 * 32)()
    fn(buf, len(data), out)
    return bytes(out)


def keccak256(data: bytes) -> bytes:
    """Keccak-256 as the transcript uses it (host-side, gkrgpu_keccak256)."""
    return _digest(load().gkrgpu_keccak256, bytes(data))


def sha3_256(data: bytes) -> bytes:
    """SHA3-256 over the same Keccak-f[1600] sponge (gkrgpu_sha3_256)."""
    return _digest(load().gkrgpu_sha3_256, bytes(data))
