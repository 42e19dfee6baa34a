"""ctypes loader for the in-tree CUDA library ``libnrldpc_gb300.so``.

There is no fallback: if the library is missing or cannot be loaded, every
GPU entry point raises.  Symbol list = the declarations of
include/nr_gpu_ldpc_gb300.h.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libnrldpc_gb300.so")

_lib = None


class NrLdpcError(RuntimeError):
    """A C-ABI call returned a negative nrldpc_status."""

    def __init__(self, fn: str, status: int, msg: str):
        super().__init__(f"{fn} failed: {msg} (status {status})")
        self.status = status


class LdpcParamsC(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("A", "bg_index", "Z", "K", "N", "H_rows", "H_cols",
                                       "n_nz_in_row", "n_nz_in_col", "n_iterations",
                                       "N_before_puncture", "i_ls", "C", "K_b")] + \
               [("rate", C.c_float)]


class ConfigC(C.Structure):
    _fields_ = [("bg", C.c_int), ("z", C.c_int), ("max_batch", C.c_int), ("alpha", C.c_float),
                ("device", C.c_int), ("cw_per_cta", C.c_int)]


class SegmentInfoC(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("B", "C", "L", "k_prime", "k", "zc", "kb", "filler", "bg")]


_vp, _i, _f, _u64 = C.c_void_p, C.c_int, C.c_float, C.c_uint64
_ip = C.POINTER(C.c_int)

SIGNATURES = {
    "nrldpc_setup_ldpc": (_i, [_i, _f, _i, C.POINTER(LdpcParamsC)]),
    "nrldpc_set_index": (_i, [_i]),
    "nrldpc_base_matrix": (_i, [_i, _i, _vp, _ip, _ip]),
    "nrldpc_init": (_i, [C.POINTER(ConfigC), C.POINTER(_vp)]),
    "nrldpc_init_custom": (_i, [_vp, _i, _i, C.POINTER(ConfigC), C.POINTER(_vp)]),
    "nrldpc_destroy": (_i, [_vp]),
    "nrldpc_geometry": (_i, [_vp, _ip, _ip, _ip, _ip, _ip, _ip]),
    "nrldpc_decode": (_i, [_vp, _vp, _vp, _i, _i, _i, _vp, _vp, _vp]),
    "nrldpc_decode_host_async": (_i, [_vp, _vp, _vp, _i, _i, _i, _vp]),
    "nrldpc_decode_host_async_q": (_i, [_vp, _vp, _i, _f, _vp, _i, _i, _i, _vp]),
    "nrldpc_set_schedule": (_i, [_vp, _i]),
    "nrldpc_set_host_transfer": (_i, [_vp, _i]),
    "nrldpc_set_weights": (_i, [_vp, _vp, _i]),
    "nrldpc_decode_weighted": (_i, [_vp, _vp, _vp, _i, _i, _i, _vp, _vp, _vp]),
    "nrldpc_wms_workspace_bytes": (_i, [_vp, _i, _i, C.POINTER(C.c_size_t)]),
    "nrldpc_wms_forward": (_i, [_vp, _vp, _vp, _i, _i, _vp, _vp, _f, _vp, _vp, _vp]),
    "nrldpc_wms_backward": (_i, [_vp, _i, _i, _vp, _vp, _vp, _vp]),
    "nrldpc_adam_step": (_i, [_i, _vp, _vp, _vp, _vp, _i, _f, _f, _f, _f, _f, _vp]),
    "nrldpc_gen_llr": (_i, [_vp, _u64, _u64, _i, _vp, _i, _vp, _vp, _vp]),
    "nrldpc_count_errors": (_i, [_vp, _vp, _vp, _i, _i, _vp, _vp]),
    "nrldpc_batch_create": (_i, [_i, _i, _f, C.POINTER(_vp)]),
    "nrldpc_batch_destroy": (_i, [_vp]),
    "nrldpc_batch_set_cw_per_cta": (_i, [_vp, _i, _i, _i]),
    "nrldpc_batch_get_cw_per_cta": (_i, [_vp, _i, _i, _ip]),
    "nrldpc_batch_set_sub_rows_per_thread": (_i, [_vp, _i, _i, _i]),
    "nrldpc_batch_get_sub_rows_per_thread": (_i, [_vp, _i, _i, _ip]),
    "nrldpc_batch_set_jobs": (_i, [_vp, _vp, _i]),
    "nrldpc_batch_gen": (_i, [_vp, _u64, _u64, _vp, _vp, _vp]),
    "nrldpc_batch_derate": (_i, [_vp, _vp, _vp, _vp]),
    "nrldpc_batch_decode": (_i, [_vp, _vp, _vp, _i, _i, _vp, _vp]),
    "nrldpc_batch_count_errors": (_i, [_vp, _vp, _vp, _vp, _vp]),
    "nrldpc_rm_k0": (_i, [_i, _i, _i]),
    "nrldpc_crc": (_i, [_vp, _i, _i, _i, _i, _vp, _vp]),
    "nrldpc_segment": (_i, [_i, _i, C.POINTER(SegmentInfoC)]),
    "nrldpc_cb_segment": (_i, [_vp, C.POINTER(SegmentInfoC), _vp, _i, _vp]),
    "nrldpc_cb_desegment": (_i, [_vp, _i, C.POINTER(SegmentInfoC), _vp, _vp, _vp]),
    "nrldpc_decode_noalloc": (_i, [_i, _i, _f, _vp, _vp, _i, _i, _i, _vp]),
    "nrldpc_device_error": (_i, [_vp]),
    "nrldpc_selftest_wait_timeout": (_i, [_vp, _vp, _vp, _i, _vp]),
    "nrldpc_noalloc_device_error": (_i, []),
    "nrldpc_selftest_noalloc_wait_timeout": (_i, [_i, _i, _vp, _vp, _i, _vp]),
    "nrldpc_status_string": (C.c_char_p, [_i]),
}


def load(build_if_missing: bool = True):
    """Load (building first if needed) the CUDA library; raises on failure."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise NrLdpcError("load", -8, f"{LIB_PATH} missing; run nr_gpu_ldpc_gb300.build.build()")
        from . import build as _build
        _build.build()
    try:
        lib = C.CDLL(LIB_PATH)
    except OSError as e:
        raise NrLdpcError("load", -8, f"cannot load {LIB_PATH}: {e}") from e
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(fn: str, status: int) -> None:
    if status < 0:
        msg = load().nrldpc_status_string(status).decode()
        raise NrLdpcError(fn, status, msg)
