"""ctypes bindings for the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline legs may
import this module: it is the checker and the timed CPU baseline, never the
product path.  ``liboracle.so`` is the C restatement of ADECO's CPU deposit
(oracle/adeco_oracle.c); ``_ref/libadeco_ref.so`` is the reference's own code
compiled from its sources (oracle/ref_harness.cpp), present only where the
reference tree was available at build time.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libadeco_ref.so")

NO_INTERSECTION, TET_INSIDE_CELL, CELL_INSIDE_TET, PARTIAL = 0, 1, 2, 3
ORDER_REF, ORDER_CONFORMING = 0, 1

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
_u64p = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")


class Stats(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in (
        "cubes", "padded_cubes", "tets_in_grid", "zero_volume", "candidate_pairs", "bbox_pairs",
        "no_pairs", "tet_inside_pairs", "cell_inside_pairs", "partial_pairs")]

    def as_dict(self):
        return {n: int(getattr(self, n)) for n, _ in self._fields_}


class Node(C.Structure):
    _fields_ = [("min", C.c_float * 3), ("ext", C.c_float), ("level", C.c_int32), ("parent", C.c_int32),
                ("first_child", C.c_int32), ("pad", C.c_int32), ("estimate", C.c_uint64)]


def build(ref: bool = True, ref_src: str | None = None) -> None:
    """Compile liboracle.so and, when `ref` is set and the reference's `src/`
    directory is given (`ref_src`, else the REF_SRC environment variable) and
    exists, the reference harness."""
    targets = ["all"]
    src = ref_src or os.environ.get("REF_SRC")
    extra = []
    if ref and src and os.path.isdir(src):
        targets.append("ref")
        extra.append(f"REF_SRC={src}")
    subprocess.run(["make", "-s", "-C", HERE] + targets + extra, check=True)


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build(ref=False)
        L = C.CDLL(LIB_PATH)
        vp = C.c_void_p
        for sfx, rp, rt in (("f", _f32p, C.c_float), ("d", _f64p, C.c_double)):
            fn = getattr(L, f"ora_clip_volume_{sfx}")
            fn.argtypes, fn.restype = [rp], rt
            fn = getattr(L, f"ora_classify_{sfx}")
            fn.argtypes, fn.restype = [rp], C.c_int
            fn = getattr(L, f"ora_deposit_patches_{sfx}")
            fn.argtypes = [C.c_size_t, C.c_size_t, _f32p, C.c_size_t, C.c_int, _f32p, C.c_int, C.c_int, rt, rp,
                           vp, vp]
            fn.restype = C.c_int
            fn = getattr(L, f"ora_deposit_patches_mt_{sfx}")
            fn.argtypes = [C.c_size_t, C.c_size_t, _f32p, C.c_size_t, C.c_int, _f32p, C.c_int, C.c_int, rt, rp,
                           C.c_int]
            fn.restype = C.c_int
            fn = getattr(L, f"ora_deposit_meta_{sfx}")
            fn.argtypes = [_f32p, C.c_int, C.c_int, C.c_int, _u64p, C.c_size_t, _f32p, C.c_int, C.c_int, rt, rp, vp]
            fn.restype = None
        L.ora_tet_records_f.argtypes = [C.c_size_t, C.c_size_t, _f32p, C.c_int, _f32p, C.c_int, C.c_int, _i32p]
        L.ora_tet_records_f.restype = None
        L.ora_flops_reset.argtypes, L.ora_flops_reset.restype = [], None
        L.ora_flops_get.argtypes, L.ora_flops_get.restype = [], C.c_uint64
        L.ora_meta_count.argtypes, L.ora_meta_count.restype = [C.c_int] * 3, C.c_size_t
        L.ora_meta_bboxes.argtypes, L.ora_meta_bboxes.restype = [_f32p, C.c_int, C.c_int, C.c_int, _f32p], None
        L.ora_generate_tree.argtypes = [_f32p, C.c_int, C.c_int, C.c_int, _f32p, _f32p, C.c_uint64, C.c_int,
                                        C.POINTER(Node), C.c_int, _i64p, _u64p, C.c_int64]
        L.ora_generate_tree.restype = C.c_int
        L.ora_leaf_order.argtypes = [C.POINTER(Node), C.c_int, _i32p]
        L.ora_leaf_order.restype = C.c_int
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_PATH)


def ref():
    """The reference's own code (built here from its sources); None if absent."""
    global _ref
    if _ref is None:
        if not ref_available():
            return None
        R = C.CDLL(REF_PATH)
        R.ref_deposit_patches_f32.argtypes = [C.c_size_t, C.c_size_t, _f32p, C.c_size_t, C.c_int, _f32p, C.c_int,
                                              _f32p]
        R.ref_deposit_patches_f32.restype = C.c_int
        R.ref_deposit_patches_f64.argtypes = [C.c_size_t, C.c_size_t, _f32p, C.c_int, _f32p, C.c_int, C.c_int,
                                              _f64p]
        R.ref_deposit_patches_f64.restype = C.c_int
        R.ref_clip_volume_f32.argtypes, R.ref_clip_volume_f32.restype = [_f32p], C.c_float
        R.ref_clip_volume_f64.argtypes, R.ref_clip_volume_f64.restype = [_f64p], C.c_double
        R.ref_classify_f32.argtypes, R.ref_classify_f32.restype = [_f32p], C.c_int
        R.ref_generate_tree.argtypes = [_f32p, C.c_int, C.c_int, C.c_int, _f32p, _f32p, C.c_uint64, C.c_int,
                                        _f32p, _i32p, _u64p, C.c_int, _i32p, _i32p, _i64p, _u64p, C.c_int64]
        R.ref_generate_tree.restype = C.c_int
        R.ref_deposit_leaf_f32.argtypes = [_f32p, C.c_int, C.c_int, C.c_int, _u64p, C.c_size_t, _f32p, C.c_int,
                                           _f32p]
        R.ref_deposit_leaf_f32.restype = C.c_int
        _ref = R
    return _ref


# --------------------------------------------------------------------------- helpers

def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def clip_volume(tet, fp64=True):
    t = np.ascontiguousarray(tet, dtype=np.float64 if fp64 else np.float32).reshape(12)
    return (lib().ora_clip_volume_d if fp64 else lib().ora_clip_volume_f)(t)


def classify(tet, fp64=False):
    t = np.ascontiguousarray(tet, dtype=np.float64 if fp64 else np.float32).reshape(12)
    return (lib().ora_classify_d if fp64 else lib().ora_classify_f)(t)


def deposit_patches(positions, m, bbox, dims, *, fp64=True, order=ORDER_REF, mass=1.0, patch_offset=0,
                    num_patches=None, grid=None, counts=False, stats=False, threads=1):
    """Reference-boundary deposit of (m+1)^3-vertex patches (ACCUMULATED into grid)."""
    pos = _f32(positions).reshape(-1)
    fpp = 3 * (m + 1) ** 3
    if num_patches is None:
        num_patches = pos.size // fpp - patch_offset
    dt = np.float64 if fp64 else np.float32
    if grid is None:
        grid = np.zeros(dims ** 3, dtype=dt)
    cand = np.zeros(dims ** 3, dtype=np.uint32) if counts else None
    st = Stats() if stats else None
    L = lib()
    if threads > 1:
        fn = L.ora_deposit_patches_mt_d if fp64 else L.ora_deposit_patches_mt_f
        rc = fn(patch_offset, num_patches, pos, pos.size, m, _f32(bbox), dims, order, mass, grid, threads)
    else:
        fn = L.ora_deposit_patches_d if fp64 else L.ora_deposit_patches_f
        rc = fn(patch_offset, num_patches, pos, pos.size, m, _f32(bbox), dims, order, mass, grid,
                cand.ctypes.data if counts else None, C.addressof(st) if stats else None)
    if rc != 0:
        raise ValueError(f"oracle deposit rejected its inputs (code {rc})")
    out = [grid]
    if counts:
        out.append(cand)
    if stats:
        out.append(st.as_dict())
    return out[0] if len(out) == 1 else tuple(out)


def tet_records(positions, m, bbox, dims, order=ORDER_REF):
    pos = _f32(positions).reshape(-1)
    ncubes = (pos.size // (3 * (m + 1) ** 3)) * m ** 3
    rec = np.zeros(ncubes * 6 * 13, dtype=np.int32)
    lib().ora_tet_records_f(0, ncubes, pos, m, _f32(bbox), dims, order, rec)
    return rec.reshape(ncubes * 6, 13)


def meta_bboxes(pos, dims3):
    nx, ny, nz = dims3
    n = lib().ora_meta_count(nx, ny, nz)
    out = np.zeros(6 * n, dtype=np.float32)
    lib().ora_meta_bboxes(_f32(pos).reshape(-1), nx, ny, nz, out)
    return out.reshape(n, 6)


def generate_tree(pos, dims3, box6, roi6, max_tets, max_level, max_nodes=1 << 20):
    """Octree: returns (nodes structured array, meta_off, meta_ids, leaf_order)."""
    nx, ny, nz = dims3
    nodes = (Node * max_nodes)()
    nmc = lib().ora_meta_count(nx, ny, nz)
    max_ids = max(16 * nmc, 1 << 16)
    off = np.zeros(max_nodes + 1, dtype=np.int64)
    ids = np.zeros(max_ids, dtype=np.uint64)
    nn = lib().ora_generate_tree(_f32(pos).reshape(-1), nx, ny, nz, _f32(box6), _f32(roi6), int(max_tets),
                                 int(max_level), nodes, max_nodes, off, ids, max_ids)
    if nn < 0:
        raise RuntimeError("oracle octree: output buffers too small")
    arr = np.ctypeslib.as_array(nodes)[:nn].copy()
    leaves = np.zeros(nn, dtype=np.int32)
    nl = lib().ora_leaf_order(nodes, nn, leaves)
    return arr, off[:nn + 1].copy(), ids[:off[nn]].copy(), leaves[:nl].copy()


def deposit_meta(pos, dims3, ids, bbox, dims, *, fp64=True, order=ORDER_REF, mass=1.0, stats=False):
    nx, ny, nz = dims3
    ids = np.ascontiguousarray(ids, dtype=np.uint64)
    dt = np.float64 if fp64 else np.float32
    grid = np.zeros(dims ** 3, dtype=dt)
    st = Stats() if stats else None
    fn = lib().ora_deposit_meta_d if fp64 else lib().ora_deposit_meta_f
    fn(_f32(pos).reshape(-1), nx, ny, nz, ids, ids.size, _f32(bbox), dims, order, mass, grid,
       C.addressof(st) if stats else None)
    return (grid, st.as_dict()) if stats else grid
