"""ctypes binding of libadeco_gb300.so (the C ABI in include/adeco_deposit.h).

The library is the only compute path: if it is missing or fails to load the
import raises -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB_PATH = os.path.join(HERE, "libadeco_gb300.so")
HEADER = os.path.join(ROOT, "include", "adeco_deposit.h")

OK = 0
STATUS_NAMES = {0: "OK", 1: "ERR_ARGUMENT", 2: "ERR_OVERFLOW", 3: "ERR_DEVICE", 4: "ERR_CUDA", 5: "ERR_MEMORY",
                6: "ERR_INCONSISTENT", 7: "ERR_STATE", 8: "ERR_NOT_FOUND", 9: "ERR_LIMIT"}
ERR_ARGUMENT, ERR_MEMORY = 1, 5
PREC_MIXED, PREC_FP64 = 0, 1
ORDER_REF, ORDER_CONFORMING = 0, 1
FORMAT_SORTED_BY_ID, FORMAT_DARK_SKY = 0, 1
OCTREE_DEVICE, OCTREE_HOST = 0, 1
OUT_F32, OUT_F64 = 0, 1


class AdecoError(RuntimeError):
    """A non-zero adeco_status_code; `code` holds it."""

    def __init__(self, code, message):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {message}")
        self.code = code


class DepositArgs(C.Structure):
    _fields_ = [("use_specific_gpu", C.c_int), ("device_id", C.c_size_t), ("patch_offset", C.c_size_t),
                ("num_patches", C.c_size_t), ("positions", C.c_void_p), ("positions_size", C.c_size_t),
                ("meta_cells_per_patch", C.c_int), ("bbox", C.c_void_p), ("dims", C.c_int), ("data", C.c_void_p),
                ("out_type", C.c_int), ("precision", C.c_int), ("tet_order", C.c_int), ("tet_mass", C.c_double)]


class SessionConfig(C.Structure):
    _fields_ = [("device", C.c_int), ("tet_order", C.c_int), ("tet_mass", C.c_double), ("hbm_fraction", C.c_double),
                ("accumulate_fp64", C.c_int)]


class Node(C.Structure):
    _fields_ = [("min", C.c_float * 3), ("ext", C.c_float), ("level", C.c_int32), ("parent", C.c_int32),
                ("first_child", C.c_int32), ("n_meta", C.c_int32), ("estimate", C.c_uint64)]


class Timing(C.Structure):
    _fields_ = [("kernel_ms", C.c_double), ("total_ms", C.c_double), ("launches", C.c_uint64), ("tets", C.c_uint64),
                ("candidate_pairs", C.c_uint64), ("partial_pairs", C.c_uint64), ("cell_inside_pairs", C.c_uint64),
                ("tet_inside_pairs", C.c_uint64), ("fp64_pairs", C.c_uint64), ("items", C.c_uint64),
                ("routed_tets", C.c_uint64), ("serial_pieces", C.c_uint64)]

    def as_dict(self):
        return {n: (float(getattr(self, n)) if t is C.c_double else int(getattr(self, n))) for n, t in self._fields_}


class Tuning(C.Structure):
    _fields_ = [("zoom_tile", C.c_int), ("share_chunk", C.c_int), ("clip_batch", C.c_int), ("ctas_per_sm", C.c_int),
                ("route_capacity", C.c_uint64), ("item_pairs", C.c_uint32)]

    def as_dict(self):
        return {n: int(getattr(self, n)) for n, _ in self._fields_}


class ServingStats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("queued", C.c_uint64),
                ("admission_waits", C.c_uint64), ("running", C.c_uint32), ("max_running", C.c_uint32),
                ("arena_bytes", C.c_uint64), ("arena_budget", C.c_uint64)]

    def as_dict(self):
        return {n: int(getattr(self, n)) for n, _ in self._fields_}


class Request(C.Structure):
    _fields_ = [("center", C.c_float * 3), ("side", C.c_float), ("dims", C.c_int), ("precision", C.c_int)]


def declared_symbols():
    """Entry points declared in include/adeco_deposit.h."""
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w[\w\s\*]*?\b(adeco_\w+)\s*\(", text, re.M)))


_vp, _sz, _i, _d = C.c_void_p, C.c_size_t, C.c_int, C.c_double
_SIGS = {
    "adeco_last_error": ([], C.c_char_p),
    "adeco_abi_version": ([], _i),
    "adeco_deposit_tets": ([_i, _sz, _sz, _sz, _vp, _sz, _i, _vp, _i, _vp], _i),
    "adeco_deposit_tets_ex": ([C.POINTER(DepositArgs)], _i),
    "adeco_deposit_tets_device": ([_vp, _sz, _sz, _sz, _i, _vp, _i, _vp, _i, _i, _d, _vp], _i),
    "adeco_deposit_tets_device_noalloc": ([_vp, _sz, _sz, _sz, _i, _vp, _i, _vp, _i, _d, _vp], _i),
    "adeco_session_create": ([C.POINTER(SessionConfig), _vp, _i, _i, _i, C.POINTER(_vp)], _i),
    "adeco_session_destroy": ([_vp], _i),
    "adeco_session_create_from_file": ([C.POINTER(SessionConfig), C.c_char_p, _i, _i, _i, _vp, C.POINTER(_vp)], _i),
    "adeco_session_lattice_dims": ([_vp, _vp], _i),
    "adeco_session_positions": ([_vp, _vp, _sz], _i),
    "adeco_session_bbox": ([_vp, _vp], _i),
    "adeco_session_build_octree": ([_vp, _vp, _vp, C.c_uint64, _i, _i], _i),
    "adeco_session_set_octree_builder": ([_vp, _i], _i),
    "adeco_session_octree_size": ([_vp, C.POINTER(_i), C.POINTER(_i), C.POINTER(_i)], _i),
    "adeco_session_octree_nodes": ([_vp, C.POINTER(Node), _i], _i),
    "adeco_session_leaves": ([_vp, _vp, _i], _i),
    "adeco_session_leaf_meta": ([_vp, _i, _vp, _i, C.POINTER(_i)], _i),
    "adeco_session_deposit_leaves": ([_vp, _i, _vp, _i, C.POINTER(Timing)], _i),
    "adeco_session_leaf_grids_device": ([_vp, C.POINTER(_vp), C.POINTER(_sz)], _i),
    "adeco_session_replay_leaves": ([_vp, _i, C.POINTER(Timing)], _i),
    "adeco_session_submit": ([_vp, C.POINTER(Request), _i, C.POINTER(C.c_uint64)], _i),
    "adeco_session_poll": ([_vp, C.c_uint64, C.POINTER(_i)], _i),
    "adeco_session_wait": ([_vp, C.c_uint64, _d], _i),
    "adeco_session_result": ([_vp, C.c_uint64, _i, _vp, _sz], _i),
    "adeco_session_latency": ([_vp, C.c_uint64, _i, C.POINTER(_d)], _i),
    "adeco_session_batch_device_ms": ([_vp, C.c_uint64, C.POINTER(C.c_double)], _i),
    "adeco_session_release": ([_vp, C.c_uint64], _i),
    "adeco_session_get_tuning": ([_vp, C.POINTER(Tuning)], _i),
    "adeco_session_set_tuning": ([_vp, C.POINTER(Tuning)], _i),
    "adeco_session_serving_stats": ([_vp, C.POINTER(ServingStats)], _i),
    "adeco_debug_bounded_wait": ([C.c_uint], _i),
    "adeco_debug_tet_records": ([_vp, _sz, _i, _sz, _sz, _vp, _i, _i, _vp, _vp], _i),
    "adeco_probe_fp32_tflops": ([_i, C.POINTER(_d)], _i),
}

_lib = None


def load(build_if_missing: bool = True):
    """Load (building first if needed) the library; raises if that fails."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise ImportError(f"{LIB_PATH} is missing; run python -m adeco_gb300.build")
        from . import build
        build.build()
    lib = C.CDLL(LIB_PATH)
    for name, (args, res) in _SIGS.items():
        fn = getattr(lib, name, None)
        if fn is None:
            continue
        fn.argtypes, fn.restype = args, res
    _lib = lib
    return lib


def check(rc: int):
    if rc != OK:
        msg = _lib.adeco_last_error().decode(errors="replace") if _lib is not None else ""
        raise AdecoError(rc, msg)
    return rc
