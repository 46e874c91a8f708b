"""ctypes binding of ``libfiuncho_gpu.so`` (C ABI in include/fiuncho_gpu.h).

The library is built in-tree by ``fiuncho_gb300.build``.  Loading fails loudly
when it is missing: there is no CPU fallback for any entry point.
"""
from __future__ import annotations

import ctypes as C
import os
import re

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfiuncho_gpu.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "fiuncho_gpu.h")

FIU_OK, FIU_ERR_INVALID, FIU_ERR_NOMEM, FIU_ERR_CUDA, FIU_ERR_UNSUPPORTED, FIU_ERR_TIMEOUT, FIU_ERR_CANCELLED = \
    range(7)
FIU_MAX_ORDER = 8
KERNEL_AUTO, KERNEL_FULL, KERNEL_ELIDED_POPC, KERNEL_ELIDED_HS, KERNEL_TENSOR = 0, 1, 2, 3, 4
FIU_MAX_OUTPUTS = 7000
FIU_NOALLOC_MAX_SAMPLES = 65536

ERRORS = {FIU_ERR_INVALID: "invalid argument", FIU_ERR_NOMEM: "out of memory", FIU_ERR_CUDA: "CUDA error",
          FIU_ERR_UNSUPPORTED: "unsupported", FIU_ERR_TIMEOUT: "timeout", FIU_ERR_CANCELLED: "cancelled"}


class FiunchoError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (ERRORS.get(code, "error"), code, msg))
        self.code = code


class Dataset_t(C.Structure):
    _fields_ = [("data", C.POINTER(C.c_uint64)), ("snps", C.c_uint64), ("cases", C.c_uint64),
                ("ctrls", C.c_uint64), ("cases_words", C.c_uint64), ("ctrls_words", C.c_uint64)]


class Distribution_t(C.Structure):
    _fields_ = [("n", C.c_int32), ("k", C.c_int32), ("step", C.c_int32), ("offset", C.c_int32)]


class Scan_t(C.Structure):
    _fields_ = [("res", C.c_void_p), ("order", C.c_uint), ("distribution", Distribution_t), ("outputs", C.c_uint),
                ("out_combinations", C.POINTER(C.c_int32)), ("out_vals", C.POINTER(C.c_float)),
                ("out_vals64", C.POINTER(C.c_double)), ("out_count", C.c_uint), ("status", C.c_int),
                ("shard", C.c_uint), ("n_shards", C.c_uint)]


class ServerStats_t(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("failed", C.c_uint64), ("queued", C.c_uint64),
                ("active", C.c_uint64), ("rounds", C.c_uint64), ("bytes_in_use", C.c_uint64), ("p50_ms", C.c_double),
                ("p99_ms", C.c_double), ("mean_ms", C.c_double), ("max_ms", C.c_double),
                ("combos_samples", C.c_double), ("solo", C.c_uint64),
                ("overlapped", C.c_uint64), ("peak_bytes", C.c_uint64)]


_u64p = C.POINTER(C.c_uint64)
_u32p = C.POINTER(C.c_uint32)
_i32p = C.POINTER(C.c_int32)
_f32p = C.POINTER(C.c_float)
_f64p = C.POINTER(C.c_double)
_vp = C.c_void_p

_SIGS = {
    "fiu_create": (C.c_int, [C.c_int, C.POINTER(_vp)]),
    "fiu_destroy": (None, [_vp]),
    "fiu_last_error": (C.c_char_p, [_vp]),
    "fiu_launch_count": (C.c_uint64, [_vp]),
    "fiu_stream": (_vp, [_vp]),
    "fiu_set_kernel": (C.c_int, [_vp, C.c_int]),
    "fiu_set_autotune": (C.c_int, [_vp, C.c_int]),
    "fiu_last_tile": (C.c_int, [_vp, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "fiu_set_kernel_timing": (C.c_int, [_vp, C.c_int]),
    "fiu_kernel_timing": (C.c_int, [_vp, _f64p, _u64p, _u64p]),
    "fiu_probe_popc_rate": (C.c_int, [_vp, _f64p]),
    "fiu_probe_lg2_error": (C.c_int, [_vp, C.c_uint, _f64p]),
    "fiu_probe_wait_limit": (C.c_int, [_vp, C.c_uint, C.c_int, C.POINTER(C.c_int), _f64p]),
    "fiu_dataset_upload": (C.c_int, [_vp, C.POINTER(Dataset_t), C.POINTER(_vp)]),
    "fiu_dataset_free": (None, [_vp, _vp]),
    "fiu_dataset_is_one_hot": (C.c_int, [_vp]),
    "fiu_search": (C.c_int, [_vp, C.POINTER(Dataset_t), C.c_uint, C.POINTER(Distribution_t), C.c_uint, _i32p,
                             _f32p, C.POINTER(C.c_uint)]),
    "fiu_search_resident": (C.c_int, [_vp, _vp, C.c_uint, C.POINTER(Distribution_t), C.c_uint, _i32p, _f32p,
                                      C.POINTER(C.c_uint)]),
    "fiu_search_resident64": (C.c_int, [_vp, _vp, C.c_uint, C.POINTER(Distribution_t), C.c_uint, _i32p, _f32p,
                                        _f64p, C.POINTER(C.c_uint)]),
    "fiu_search_shard": (C.c_int, [_vp, C.POINTER(Dataset_t), C.c_uint, C.c_uint, C.c_uint, C.c_uint, _i32p, _f32p,
                                   C.POINTER(C.c_uint)]),
    "fiu_search_shard_resident64": (C.c_int, [_vp, _vp, C.c_uint, C.c_uint, C.c_uint, C.c_uint, _i32p, _f32p,
                                              _f64p, C.POINTER(C.c_uint)]),
    "fiu_combine": (C.c_int, [_vp, _u64p, C.c_uint, _u64p, C.c_uint64, C.c_uint64, _u64p]),
    "fiu_combine_and_popcnt": (C.c_int, [_vp, _u64p, C.c_uint, _u64p, C.c_uint64, C.c_uint64, _u32p, _u32p,
                                         C.c_uint]),
    "fiu_mi_compute": (C.c_int, [_vp, _u32p, _u32p, C.c_size_t, C.c_size_t, C.c_uint, C.c_uint, C.c_int, _f32p,
                                 _f64p]),
    "fiu_mi_compute_noalloc": (C.c_int, [_vp, _vp, C.c_size_t, C.c_size_t, C.c_uint, C.c_uint, _vp, _vp]),
    "fiu_search_batch": (C.c_int, [_vp, C.POINTER(Scan_t), C.c_uint, C.c_int]),
    "fiu_server_create": (C.c_int, [C.c_int, C.c_uint64, C.POINTER(_vp)]),
    "fiu_server_set_policy": (C.c_int, [_vp, C.c_int]),
    "fiu_server_submit": (C.c_int, [_vp, C.POINTER(Dataset_t), C.c_uint, C.c_uint, C.POINTER(C.c_uint64)]),
    "fiu_server_submit_shard": (C.c_int, [_vp, C.POINTER(Dataset_t), C.c_uint, C.c_uint, C.c_uint, C.c_uint,
                                          C.POINTER(C.c_uint64)]),
    "fiu_server_poll": (C.c_int, [_vp, C.c_uint64, C.c_int, _i32p, _f32p, _f64p, C.POINTER(C.c_uint),
                                  C.POINTER(C.c_double)]),
    "fiu_server_stats": (C.c_int, [_vp, C.POINTER(ServerStats_t)]),
    "fiu_server_destroy": (None, [_vp]),
    "fiu_tables": (C.c_int, [_vp, _vp, C.c_uint, _i32p, C.c_size_t, _u32p, _u32p]),
    "fiu_scan_tables": (C.c_int, [_vp, _vp, C.c_uint, C.POINTER(Distribution_t), C.c_int, _u32p, C.c_size_t]),
    "fiu_scan_digest": (C.c_int, [_vp, _vp, C.c_uint, C.POINTER(Distribution_t), C.c_int, _u64p, _u64p]),
    "fiu_read_genotypes": (C.c_int, [_vp, C.c_char_p, C.c_char_p, C.c_int, C.POINTER(_vp)]),
    "fiu_genotypes_info": (C.c_int, [_vp, _u64p, _u64p, C.POINTER(C.POINTER(C.c_uint8)),
                                     C.POINTER(C.POINTER(C.c_uint8))]),
    "fiu_genotypes_free": (None, [_vp]),
    "fiu_dataset_upload_genotypes": (C.c_int, [_vp, C.POINTER(C.c_uint8), C.POINTER(C.c_uint8), C.c_uint64,
                                               C.c_uint64, C.POINTER(_vp)]),
    "fiu_dataset_packed": (C.c_int, [_vp, _vp, C.POINTER(Dataset_t), _u64p]),
}

_lib = None


def header_symbols():
    """Function names declared in include/fiuncho_gpu.h."""
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(fiu_[a-z_0-9]+)\s*\(", txt, re.M)))


def load(path: str = LIB_PATH):
    """Loads the library (once).  Raises if it was not built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError("libfiuncho_gpu.so not built (run `python -c \"import __graft_entry__ as g; g.build()\"` "
                          "or `python -m fiuncho_gb300.build`); there is no CPU fallback")
    lib = C.CDLL(path)
    for name, (res, args) in _SIGS.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))
