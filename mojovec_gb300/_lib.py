"""ctypes binding of libmojovec_gpu.so (include/mojovec_gpu.h).

The library is built in-tree by mojovec_gb300/build.py. There is no CPU
fallback: if the shared library is missing or no GB300-class device is
present, load() raises.
"""

from __future__ import annotations

import ctypes as C
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmojovec_gpu.so")

MV_OK = 0
MV_ERR_ARG = -1
MV_ERR_OOM = -2
MV_ERR_CUDA = -3
MV_ERR_TIMEOUT = -4
MV_ERR_STATE = -5
MV_ERR_UNSUPPORTED = -6
MV_ERR_INTERNAL = -7

METRIC_L2 = 0
METRIC_IP = 1
FORM_PLAIN = 0
FORM_FAST = 1

STAGES = ("coarse", "select", "scan", "lut", "rerank", "flat", "encode", "append", "adc")

_ERR_NAMES = {
    MV_ERR_ARG: "MV_ERR_ARG",
    MV_ERR_OOM: "MV_ERR_OOM",
    MV_ERR_CUDA: "MV_ERR_CUDA",
    MV_ERR_TIMEOUT: "MV_ERR_TIMEOUT",
    MV_ERR_STATE: "MV_ERR_STATE",
    MV_ERR_UNSUPPORTED: "MV_ERR_UNSUPPORTED",
    MV_ERR_INTERNAL: "MV_ERR_INTERNAL",
}


class MojoVecGPUError(RuntimeError):
    """A non-zero status from the C ABI; .code holds the MV_ERR_* value."""

    def __init__(self, code: int, message: str):
        super().__init__(f"{message} ({_ERR_NAMES.get(code, code)})")
        self.code = code


class SearchParams(C.Structure):
    """mv_search_params."""

    _fields_ = [
        ("form", C.c_int32),
        ("nprobe", C.c_int32),
        ("rerank", C.c_int32),
        ("coarse_fp32", C.c_int32),
        ("lut_fp16", C.c_int32),
        ("coarse_path", C.c_int32),
        ("plain_scan", C.c_int32),
        ("flat_e4m3", C.c_int32),
        ("rerank_fp32", C.c_int32),
    ]


_vp = C.c_void_p
_i32 = C.c_int32
_i64 = C.c_int64
_f32 = C.c_float

# name -> (restype, argtypes); the exported C ABI.
SIGNATURES = {
    "mv_last_error": (_i32, [C.c_char_p, C.c_size_t]),
    "mv_version": (C.c_char_p, []),
    "mv_ctx_create": (_i32, [_i32, C.POINTER(_vp)]),
    "mv_ctx_certify_stats": (_i32, [_vp, _vp]),
    "mv_ctx_destroy": (_i32, [_vp]),
    "mv_ctx_synchronize": (_i32, [_vp]),
    "mv_ctx_kernel_launches": (_i64, [_vp]),
    "mv_ctx_set_wait_limit": (_i32, [_vp, _i64]),
    "mv_ctx_profile": (_i32, [_vp, _i32]),
    "mv_ctx_stage_times": (_i32, [_vp, _vp, _vp, _i32]),
    "mv_ivfpq_create": (_i32, [_vp, _i32, _i32, _i32, _i32, C.POINTER(_vp)]),
    "mv_ivfpq_destroy": (_i32, [_vp]),
    "mv_ivfpq_set_nprobe": (_i32, [_vp, _i32]),
    "mv_ivfpq_info": (_i32, [_vp, _vp]),
    "mv_ivfpq_set_codebooks": (_i32, [_vp, _vp, _vp]),
    "mv_ivfpq_get_codebooks": (_i32, [_vp, _vp, _vp]),
    "mv_ivfpq_train": (_i32, [_vp, _vp, _i64, _i32, _i32]),
    "mv_ivfpq_train_ex": (_i32, [_vp, _vp, _i64, _i32, _i32, _vp]),
    "mv_ivfpq_add": (_i32, [_vp, _vp, _i64]),
    "mv_ivfpq_add_with_ids": (_i32, [_vp, _vp, _vp, _i64]),
    "mv_ivfpq_get_lists": (_i32, [_vp, _vp, _vp, _vp]),
    "mv_ivfpq_set_lists": (_i32, [_vp, _vp, _vp, _vp]),
    "mv_ivfpq_load_snapshot": (_i32, [_vp, C.c_char_p, C.POINTER(_vp)]),
    "mv_ivfpq_save_snapshot": (_i32, [_vp, C.c_char_p, C.c_char_p, C.c_char_p, _vp, _i64]),
    "mv_ivfpq_snapshot_info": (_i32, [_vp, C.c_char_p, C.c_size_t, C.c_char_p, C.c_size_t, _vp, _vp]),
    "mv_snapshot_checksum": (C.c_uint64, [_vp, C.c_size_t]),
    "mv_ivfpq_search": (_i32, [_vp, _vp, _i64, _i32, _vp, _i64, _vp, _vp, _vp]),
    "mv_ivfpq_search_device": (_i32, [_vp, _vp, _i64, _i32, _vp, _i64, _vp, _vp, _vp, _vp]),
    "mv_ivfpq_search_noalloc": (_i32, [_vp, _vp, _i64, _i32, _i32, _vp, _vp, _vp]),
    "mv_flat_create": (_i32, [_vp, _i32, _i32, C.POINTER(_vp)]),
    "mv_flat_destroy": (_i32, [_vp]),
    "mv_flat_add": (_i32, [_vp, _vp, _i64]),
    "mv_flat_ntotal": (_i64, [_vp]),
    "mv_flat_search": (_i32, [_vp, _vp, _i64, _i32, _vp, _vp, _vp, _vp]),
    "mv_flat_rerank": (_i32, [_vp, _vp, _i64, _vp, _i32, _i32, _vp, _vp]),
    "mv_flat_rerank_device": (_i32, [_vp, _vp, _i64, _vp, _i32, _i32, _vp, _vp, _vp]),
    "mv_flat_search_device": (_i32, [_vp, _vp, _i64, _i32, _vp, _vp, _vp, _vp, _vp]),
    "mv_sq8_create": (_i32, [_vp, _i32, _i32, C.POINTER(_vp)]),
    "mv_sq8_destroy": (_i32, [_vp]),
    "mv_sq8_add": (_i32, [_vp, _vp, _i64]),
    "mv_sq8_params": (_i32, [_vp, _vp]),
    "mv_sq8_ntotal": (_i64, [_vp]),
    "mv_sq8_get_codes": (_i32, [_vp, _vp, _vp]),
    "mv_sq8_search": (_i32, [_vp, _vp, _i64, _i32, _vp, _vp, _vp]),
    "mv_sq8_search_rerank": (_i32, [_vp, _vp, _i64, _i32, _i32, _vp, _vp]),
    "mv_sq8_search_ex": (_i32, [_vp, _vp, _i64, _i32, _vp, _i32, _vp, _vp, _vp]),
    "mv_sq8_search_device": (_i32, [_vp, _vp, _i64, _i32, _vp, _i32, _vp, _vp, _vp, _vp]),
    "mv_kmeans_train": (_i32, [_vp, _vp, _i64, _i32, _i32, _i32, _vp, _vp]),
    "mv_ivfpq_search_batch": (_i32, [_vp, _vp, _i64, _vp, _vp, _i32, _vp, _vp, _vp]),
    "mv_ivfpq_plan_create": (_i32, [_vp, _i64, _i32, _i32, _vp, _vp]),
    "mv_ivfpq_plan_destroy": (_i32, [_vp]),
    "mv_ivfpq_plan_buffers": (_i32, [_vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "mv_ivfpq_plan_set_queries": (_i32, [_vp, _vp, _i64, _vp, _vp]),
    "mv_ivfpq_plan_tune": (_i32, [_vp, _i64, _vp, _vp]),
    "mv_ivfpq_plan_run": (_i32, [_vp, _i64, _i32, _vp]),
    "mv_ivfpq_plan_results": (_i32, [_vp, _i64, _vp, _vp]),
    "mv_ivfflat_create": (_i32, [_vp, _i32, _i32, _i32, _vp]),
    "mv_ivfflat_destroy": (_i32, [_vp]),
    "mv_ivfflat_set_nprobe": (_i32, [_vp, _i32]),
    "mv_ivfflat_ntotal": (_i64, [_vp]),
    "mv_ivfflat_train": (_i32, [_vp, _vp, _i64, _i32, _vp]),
    "mv_ivfflat_get_centroids": (_i32, [_vp, _vp]),
    "mv_ivfflat_add": (_i32, [_vp, _vp, _i64]),
    "mv_ivfflat_add_with_ids": (_i32, [_vp, _vp, _vp, _i64]),
    "mv_ivfflat_search": (_i32, [_vp, _vp, _i64, _i32, _vp, _vp, _vp]),
    "mv_ivfflat_search_device": (_i32, [_vp, _vp, _i64, _i32, _vp, _vp, _vp, _vp]),
    "mv_server_create": (_i32, [_vp, _i64, _i32, _i64, _vp]),
    "mv_server_destroy": (_i32, [_vp]),
    "mv_server_add_ivfpq": (_i32, [_vp, _vp, _vp, _vp]),
    "mv_server_add_flat": (_i32, [_vp, _vp, _vp, _vp]),
    "mv_server_add_sq8": (_i32, [_vp, _vp, _i32, _vp, _vp]),
    "mv_server_submit": (_i32, [_vp, _i32, _vp, _i64, _i32, _vp, _vp, _vp]),
    "mv_server_wait": (_i32, [_vp, _i64, _vp]),
    "mv_server_device_overlap": (_i32, [_vp, _vp]),
    "mv_server_stats": (_i32, [_vp, _vp]),
    "mv_kmeans_train_ex": (_i32, [_vp, _vp, _i64, _i32, _i32, _i32, _vp, _vp, _vp, _vp]),
    "mv_pq_train": (_i32, [_vp, _vp, _i64, _i32, _i32, _i32, _vp]),
    "mv_pq_encode": (_i32, [_vp, _vp, _i32, _i32, _vp, _i64, _vp]),
    "mv_pq_distance_tables": (_i32, [_vp, _vp, _i32, _i32, _vp, _i64, _i32, _vp]),
    "mv_sq8_encode": (_i32, [_vp, _vp, _i64, _i32, _f32, _f32, _i32, _vp, _vp]),
    "mv_normalize": (_i32, [_vp, _vp, _i64, _i32, _vp]),
    "mv_distance_matrix": (_i32, [_vp, _vp, _i64, _vp, _i64, _i32, _i32, _i32, _vp]),
}

_lib = None
_lock = threading.Lock()


def load(path: str = LIB_PATH):
    """Loads the CUDA library and declares every signature. Raises if it is
    missing: the product path has no fallback."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(path):
            raise ImportError(
                f"{path} not found: build it with mojovec_gb300/build.py "
                "(there is no CPU fallback)"
            )
        lib = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def last_error() -> str:
    buf = C.create_string_buffer(1024)
    load().mv_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(status: int):
    if status != MV_OK:
        raise MojoVecGPUError(status, last_error())
