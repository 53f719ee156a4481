"""ctypes binding of libgfpdb.so and the Arrow C Data Interface structures.

The library is the product; this module only loads it and declares its
entry points. Loading fails loudly when the shared library has not been
built: there is no Python or CPU fallback for any operator.
"""

from __future__ import annotations

import ctypes
import os
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libgfpdb.so"

GFPDB_OK = 0
GFPDB_EINVAL = 1
GFPDB_ECUDA = 2
GFPDB_EDEVICE = 3
GFPDB_ETIMEDOUT = 4
GFPDB_ENOMEM = 5
GFPDB_EUNSUPPORTED = 6

ARROW_DEVICE_CPU = 1
ARROW_DEVICE_CUDA = 2
ARROW_DEVICE_CUDA_HOST = 3


class ArrowSchema(ctypes.Structure):
    pass


SCHEMA_RELEASE = ctypes.CFUNCTYPE(None, ctypes.POINTER(ArrowSchema))
ArrowSchema._fields_ = [
    ("format", ctypes.c_char_p),
    ("name", ctypes.c_char_p),
    ("metadata", ctypes.c_char_p),
    ("flags", ctypes.c_int64),
    ("n_children", ctypes.c_int64),
    ("children", ctypes.POINTER(ctypes.POINTER(ArrowSchema))),
    ("dictionary", ctypes.POINTER(ArrowSchema)),
    ("release", SCHEMA_RELEASE),
    ("private_data", ctypes.c_void_p),
]


class ArrowArray(ctypes.Structure):
    pass


ARRAY_RELEASE = ctypes.CFUNCTYPE(None, ctypes.POINTER(ArrowArray))
ArrowArray._fields_ = [
    ("length", ctypes.c_int64),
    ("null_count", ctypes.c_int64),
    ("offset", ctypes.c_int64),
    ("n_buffers", ctypes.c_int64),
    ("n_children", ctypes.c_int64),
    ("buffers", ctypes.POINTER(ctypes.c_void_p)),
    ("children", ctypes.POINTER(ctypes.POINTER(ArrowArray))),
    ("dictionary", ctypes.POINTER(ArrowArray)),
    ("release", ARRAY_RELEASE),
    ("private_data", ctypes.c_void_p),
]


class ArrowDeviceArray(ctypes.Structure):
    _fields_ = [
        ("array", ArrowArray),
        ("device_id", ctypes.c_int64),
        ("device_type", ctypes.c_int32),
        ("sync_event", ctypes.c_void_p),
        ("reserved", ctypes.c_int64 * 3),
    ]


class ExecStats(ctypes.Structure):
    _fields_ = [
        ("elapsed_ns", ctypes.c_int64),
        ("kernel_launches", ctypes.c_int64),
        ("h2d_bytes", ctypes.c_int64),
        ("d2h_bytes", ctypes.c_int64),
        ("num_ops", ctypes.c_int64),
        ("messages", ctypes.c_int64),
        ("device_ns", ctypes.c_int64),
    ]


class RequestStats(ctypes.Structure):
    _fields_ = [
        ("status", ctypes.c_int32),
        ("batch_size", ctypes.c_int32),
        ("submit_ns", ctypes.c_int64),
        ("start_ns", ctypes.c_int64),
        ("end_ns", ctypes.c_int64),
        ("kernel_launches", ctypes.c_int64),
        ("cache_misses", ctypes.c_int64),
        ("worker", ctypes.c_int32),
        ("pad", ctypes.c_int32),
    ]


class ServerStats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int64) for n in (
        "submitted", "completed", "failed", "batches", "batched_requests", "cache_hits", "cache_misses",
        "cache_evictions", "cache_bytes", "cache_capacity", "reserved_bytes", "hbm_budget", "admission_waits")]


class GfpdbError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"gfpdb error {code}: {message}")
        self.code = code
        self.message = message


_P = ctypes.c_void_p
_S = ctypes.POINTER(ArrowSchema)
_A = ctypes.POINTER(ArrowDeviceArray)
_CP = ctypes.POINTER(ctypes.c_char_p)
_I32 = ctypes.c_int32
_I64 = ctypes.c_int64

# name -> (restype, argtypes); every symbol declared in include/gfpdb.h
SIGNATURES = {
    "gfpdb_last_error": (ctypes.c_char_p, []),
    "gfpdb_version": (_I32, []),
    "gfpdb_device_init": (_I32, [_I32]),
    "gfpdb_kernel_launch_count": (ctypes.c_uint64, []),
    "gfpdb_thread_device_alloc_bytes": (_I64, []),
    "gfpdb_memcpy": (_I32, [_P, _P, _I64, _I32, _P]),
    "gfpdb_result_layout": (_I32, [_S, _A, _I32, ctypes.POINTER(_I64), ctypes.POINTER(_I32), ctypes.POINTER(_I32),
                                   ctypes.c_char_p, _I64, ctypes.POINTER(_P), ctypes.POINTER(_P)]),
    "gfpdb_result_release": (None, [_S, _A]),
    "gfpdb_host_alloc": (_I32, [ctypes.POINTER(_P), _I64]),
    "gfpdb_host_free": (_I32, [_P]),
    "gfpdb_stream_synchronize": (_I32, [_P]),
    "gfpdb_profile_enable": (_I32, [_I32]),
    "gfpdb_profile_reset": (_I32, []),
    "gfpdb_profile_read": (_I32, [ctypes.c_char_p, ctypes.POINTER(_I64), ctypes.POINTER(ctypes.c_double),
                                  ctypes.POINTER(ctypes.c_double)]),
    "gfpdb_profile_kernels": (_I32, [ctypes.c_char_p, _I64]),
    "gfpdb_filter_compile": (_I32, [ctypes.c_char_p, _S, ctypes.POINTER(_P)]),
    "gfpdb_filter_evaluate": (_I32, [_P, _S, _A, _CP, _I32, _S, _A, _P]),
    "gfpdb_filter_free": (None, [_P]),
    "gfpdb_filter_evaluate_noalloc": (_I32, [_P, _S, _A, _CP, _I32, ctypes.POINTER(_P), ctypes.POINTER(_I64), _P]),
    "gfpdb_bloom_create": (_I32, [_S, ctypes.POINTER(_A), _I32, _CP, _I32, _I32, _I32, ctypes.POINTER(_P), _P]),
    "gfpdb_bloom_use": (_I32, [_P, _S, _A, _CP, _I32, _S, _A, _P]),
    "gfpdb_bloom_info": (
        _I32,
        [_P, ctypes.POINTER(_I64), ctypes.POINTER(_I64), ctypes.POINTER(_I32), ctypes.POINTER(_I32), ctypes.POINTER(_P)],
    ),
    "gfpdb_bloom_free": (None, [_P]),
    "gfpdb_shuffle": (_I32, [_S, _A, _CP, _I32, _I64, _S, _A, ctypes.POINTER(_I64), _P]),
    "gfpdb_select": (_I32, [_P, _I32, ctypes.POINTER(_P), _CP, _S, _A, _CP, _I32, _S, _A, _P]),
    "gfpdb_hashjoin_create": (_I32, [_I32, _CP, _CP, _I32, _CP, _I32, ctypes.c_double, ctypes.POINTER(_P)]),
    "gfpdb_hashjoin_put_build": (_I32, [_P, _S, _A, _P]),
    "gfpdb_hashjoin_finalize_build": (_I32, [_P, _P]),
    "gfpdb_hashjoin_probe": (_I32, [_P, _S, _A, _S, _A, _P]),
    "gfpdb_hashjoin_info": (_I32, [_P, ctypes.POINTER(_I64), ctypes.POINTER(_I64), ctypes.POINTER(_I64)]),
    "gfpdb_hashjoin_finish": (_I32, [_P, _S, _S, _A, _P]),
    "gfpdb_hashjoin_free": (None, [_P]),
    "gfpdb_group_create": (_I32, [ctypes.c_char_p, ctypes.POINTER(_P)]),
    "gfpdb_group_update": (_I32, [_P, _S, _A, _P]),
    "gfpdb_group_finalize": (_I32, [_P, _S, _A, _P]),
    "gfpdb_group_clear": (_I32, [_P]),
    "gfpdb_hashjoin_clear": (_I32, [_P]),
    "gfpdb_group_free": (None, [_P]),
    "gfpdb_parquet_read": (_I32, [_P, _I64, _CP, _I32, _I64, _I64, _S, _A, _P]),
    "gfpdb_parquet_read_file": (_I32, [ctypes.c_char_p, _CP, _I32, _I64, _I64, _S, _A, _P]),
    "gfpdb_csv_read": (_I32, [_P, _I64, _I32, ctypes.c_char, _I32, _S, _CP, _I32, _S, _A, _P]),
    "gfpdb_execute_plan": (
        _I32,
        [ctypes.c_char_p, _I32, _CP, ctypes.POINTER(_S), ctypes.POINTER(_A), _I32, _S, _A, ctypes.POINTER(ExecStats), _P],
    ),
    "gfpdb_plan_prepare": (_I32, [ctypes.c_char_p, _I32, _CP, ctypes.POINTER(_S), ctypes.POINTER(_A),
                                  ctypes.POINTER(_P)]),
    "gfpdb_prepared_run": (_I32, [_P, ctypes.POINTER(ExecStats), _P, ctypes.POINTER(_I64), ctypes.POINTER(_I64)]),
    "gfpdb_prepared_launch": (_I32, [_P, _P]),
    "gfpdb_prepared_wait": (_I32, [_P, ctypes.POINTER(ExecStats), ctypes.POINTER(_I64), ctypes.POINTER(_I64)]),
    "gfpdb_prepared_layout": (_I32, [_P, _I32, ctypes.POINTER(_I64), ctypes.POINTER(_I32), ctypes.c_char_p, _I64,
                                     ctypes.POINTER(_P), ctypes.POINTER(_P)]),
    "gfpdb_prepared_free": (None, [_P]),
    "gfpdb_plan_validate": (_I32, [ctypes.c_char_p]),
    "gfpdb_plan_predicate_transfer": (_I32, [ctypes.c_char_p, ctypes.c_char_p, _I64, ctypes.POINTER(_I64)]),
    "gfpdb_plan_fuse": (_I32, [ctypes.c_char_p, ctypes.c_char_p, _I64, ctypes.POINTER(_I64)]),
    "gfpdb_parquet_layout": (_I32, [_P, _I64, _CP, _I32, _I64, _I64, ctypes.c_char_p, _I64, ctypes.POINTER(_I64)]),
    "gfpdb_graph_cache_clear": (_I32, []),
    "gfpdb_server_create": (_I32, [ctypes.c_char_p, ctypes.POINTER(_P)]),
    "gfpdb_server_register_table": (_I32, [_P, ctypes.c_char_p, _S, _A]),
    "gfpdb_server_submit": (_I32, [_P, ctypes.c_char_p, ctypes.POINTER(ctypes.c_uint64)]),
    "gfpdb_server_wait": (_I32, [_P, ctypes.c_uint64, _I64, _S, _A, ctypes.POINTER(RequestStats)]),
    "gfpdb_server_get_stats": (_I32, [_P, ctypes.POINTER(ServerStats)]),
    "gfpdb_server_destroy": (_I32, [_P]),
    "gfpdb_batch_prepare": (_I32, [ctypes.c_char_p, _I32, _CP, ctypes.POINTER(_S), ctypes.POINTER(_A),
                                   ctypes.POINTER(_P)]),
    "gfpdb_batch_launch": (_I32, [_P, _P]),
    "gfpdb_batch_wait": (_I32, [_P, ctypes.POINTER(ExecStats), ctypes.POINTER(_I64)]),
    "gfpdb_batch_run": (_I32, [_P, ctypes.POINTER(ExecStats), _P, ctypes.POINTER(_I64)]),
    "gfpdb_batch_layout": (_I32, [_P, _I32, ctypes.POINTER(_I64), ctypes.POINTER(_I32), ctypes.c_char_p, _I64,
                                  ctypes.POINTER(_P)]),
    "gfpdb_batch_free": (None, [_P]),
    "gfpdb_star_batch": (
        _I32,
        [ctypes.c_char_p, _I32, _CP, ctypes.POINTER(_S), ctypes.POINTER(_A), _I32, _I32, _S, _A,
         ctypes.POINTER(ExecStats), _P],
    ),
}

_lib = None


def lib() -> ctypes.CDLL:
    """Load libgfpdb.so (built by flexpushdowndb_gb300.build)."""
    global _lib
    if _lib is None:
        path = os.environ.get("GFPDB_LIB", str(LIB_PATH))
        if not Path(path).exists():
            raise ImportError(
                f"{path} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
                "(the GPU path has no fallback)"
            )
        L = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(code: int) -> None:
    if code != GFPDB_OK:
        msg = lib().gfpdb_last_error().decode("utf-8", "replace")
        raise GfpdbError(code, msg)


def cstr_array(names):
    arr = (ctypes.c_char_p * max(1, len(names)))()
    for i, n in enumerate(names):
        arr[i] = n.encode()
    return arr
