"""ctypes binding of the C ABI in include/lbvh_gb300.h.

Loads the in-tree lbvh_gb300/liblbvh_gb300.so. There is no fallback: if the
library is missing or fails to load, every entry point raises.
"""
from __future__ import annotations

import ctypes
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liblbvh_gb300.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "lbvh_gb300.h")

LBVH_OK = 0
LBVH_ERR_INVALID_ARG = 1
LBVH_ERR_OOM = 2
LBVH_ERR_TIMEOUT = 3
LBVH_ERR_DEVICE = 4
LBVH_ERR_BAD_TOPOLOGY = 5
LBVH_ERR_NOT_RESIDENT = 6
LBVH_ERR_BUDGET = 7
LBVH_ERR_CANCELLED = 8
LBVH_ERR_EXPIRED = 9

REQ_BUILD, REQ_REFIT, REQ_TRACE = 0, 1, 2

NOALLOC_MAX_PRIMS = 65536
PARAM_TRACE_BLOCKS_PER_SM = 1
PARAM_TRACE_REFILL = 2
PARAM_BATCH_THREADS = 3
PARAM_TRACE_CHUNK = 4
PARAM_TRACE_IN_PLACE = 5
PARAM_LOOKBACK_SPIN_LIMIT = 6
PARAM_TEST_LOOKBACK_STALL = 7
PARAM_TRACE_LEAF_BATCH = 8
PARAM_BATCH_RADIX_BITS = 9
PARAM_BATCH_KEYS_PER_THREAD = 10
PARAM_SORT_TILE_KEYS = 11
PARAM_BUCKET_SORT_MIN = 12
PARAM_BOUNDS_BLOCKS_PER_SM = 13
PARAM_TREE_WALK_FUSED = 14
PARAM_TEST_TREE_MERGE_CAP = 15
PARAM_SMALL_BUILD_MAX = 16
PARAM_TRACE_RAY_ORDER = 17
LBVH_BUILD_SORTED_LEAVES = 0x1
LBVH_BUILD_KEEP_CURVE = 0x2
LEAF_BIT = 0x80000000
MISS = 0xFFFFFFFF

_P = ctypes.c_void_p
_S = ctypes.c_size_t
_U32 = ctypes.c_uint32
_I = ctypes.c_int
_PP = ctypes.POINTER(ctypes.c_void_p)

# name -> (restype, argtypes)
SIGNATURES = {
    "lbvh_version": (_I, []),
    "lbvh_status_string": (ctypes.c_char_p, [_I]),
    "lbvh_ctx_create": (_I, [_I, _P, _PP]),
    "lbvh_ctx_destroy": (_I, [_P]),
    "lbvh_ctx_synchronize": (_I, [_P]),
    "lbvh_ctx_last_error": (ctypes.c_char_p, [_P]),
    "lbvh_ctx_reserve": (_I, [_P, _S, _S]),
    "lbvh_ctx_set_param": (_I, [_P, _I, _I]),
    "lbvh_make_triangles": (_I, [_P, _P, _S, _P]),
    "lbvh_bvh_create": (_I, [_P, _PP]),
    "lbvh_bvh_destroy": (_I, [_P, _P]),
    "lbvh_build_triangles": (_I, [_P, _P, _S, _U32, _P]),
    "lbvh_build_boxes": (_I, [_P, _P, _S, _U32, _P]),
    "lbvh_refit_triangles": (_I, [_P, _P, _P]),
    "lbvh_refit_boxes": (_I, [_P, _P, _P]),
    "lbvh_bvh_import_triangles": (_I, [_P, _P, _S, _P, _P]),
    "lbvh_bvh_info": (_I, [_P, ctypes.POINTER(_S), ctypes.POINTER(_S), ctypes.POINTER(_U32)]),
    "lbvh_bvh_nodes": (_I, [_P, _P, _P]),
    "lbvh_bvh_primitives": (_I, [_P, _P, _P]),
    "lbvh_bvh_device_nodes": (_P, [_P]),
    "lbvh_bvh_curve": (_I, [_P, _P, _P, _P, _P, _P]),
    "lbvh_trace_triangles": (_I, [_P, _P, _P, _S, _P]),
    "lbvh_trace_spheres": (_I, [_P, _P, _P, _P, _S, _P]),
    "lbvh_trace_triangles_counts": (_I, [_P, _P, _P, _S, _P, _P, _P]),
    "lbvh_build_triangles_noalloc": (_I, [_P, _S, _P, _P, _P]),
    "lbvh_bvh_prepare_trace": (_I, [_P, _P]),
    "lbvh_batch_prepare_trace": (_I, [_P, _P]),
    "lbvh_batch_create": (_I, [_P, _PP]),
    "lbvh_batch_destroy": (_I, [_P, _P]),
    "lbvh_batch_build_triangles": (_I, [_P, _P, _S, _P, _S, _P]),
    "lbvh_batch_build": (_I, [_P, _P, _S, _P, _S, _U32, _P]),
    "lbvh_batch_info": (_I, [_P, ctypes.POINTER(_S), ctypes.POINTER(_S), ctypes.POINTER(_S)]),
    "lbvh_batch_nodes": (_I, [_P, _P, _P]),
    "lbvh_batch_trace_triangles": (_I, [_P, _P, _P, _P, _S, _P]),
    "lbvh_batch_mesh_nodes": (_I, [_P, _P, _S, _P]),
    "lbvh_server_create": (_I, [_P, _PP]),
    "lbvh_server_submit": (_I, [_P, _I, ctypes.c_int64, _P, _S, _P, ctypes.POINTER(ctypes.c_uint64)]),
    "lbvh_server_wait_any": (_I, [_P, _P, _S, ctypes.c_double, ctypes.POINTER(_S)]),
    "lbvh_server_drain": (_I, [_P]),
    "lbvh_server_cancel": (_I, [_P, ctypes.c_uint64]),
    "lbvh_server_inject_alloc_failures": (_I, [_P, _U32]),
    "lbvh_server_clock": (ctypes.c_double, [_P]),
    "lbvh_server_stats_get": (_I, [_P, _P]),
    "lbvh_server_resident": (_I, [_P, _P, _S, ctypes.POINTER(_S)]),
    "lbvh_server_destroy": (_I, [_P]),
}


class ServerConfig(ctypes.Structure):
    """lbvh_server_config"""
    _fields_ = [("device", _I), ("slots", _I), ("hbm_budget", _S), ("batch_max_tris", _S),
                ("batch_max_requests", _S), ("trace_batch_max_rays", _S), ("host_budget", _S),
                ("max_queue_s", ctypes.c_double)]


class RequestDone(ctypes.Structure):
    """lbvh_request_done"""
    _fields_ = [("ticket", ctypes.c_uint64), ("status", _I), ("kind", _I), ("scene", ctypes.c_int64),
                ("arrival", ctypes.c_double), ("start", ctypes.c_double), ("done", ctypes.c_double),
                ("message", ctypes.c_char * 160)]


class ServerStats(ctypes.Structure):
    """lbvh_server_stats"""
    _fields_ = [("submitted", ctypes.c_uint64), ("completed", ctypes.c_uint64),
                ("coalesced_requests", ctypes.c_uint64), ("evictions", ctypes.c_uint64),
                ("resident_scenes", ctypes.c_uint64), ("resident_bytes", ctypes.c_uint64),
                ("spills", ctypes.c_uint64), ("reloads", ctypes.c_uint64),
                ("spilled_scenes", ctypes.c_uint64), ("spilled_bytes", ctypes.c_uint64),
                ("cancelled", ctypes.c_uint64), ("expired", ctypes.c_uint64)]


class LbvhError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"lbvh status {status}: {msg}")
        self.status = status


_lib = None


def declared_symbols() -> list[str]:
    """Names of every function the public header declares."""
    with open(HEADER) as f:
        text = f.read()
    return re.findall(r"LBVH_API\s+[\w\s\*]+?\b(lbvh_\w+)\s*\(", text)


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
                "(the CUDA library has no CPU fallback)"
            )
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def status_string(st: int) -> str:
    return lib().lbvh_status_string(st).decode()
