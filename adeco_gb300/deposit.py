"""Host-side mirror of ADECO's deposit interface over the C ABI.

* ``DepositWrapper.deposit_tets`` keeps the reference's signature and meaning
  (src/AdDeposit2Grid.h:82-91): positions in (m+1)^3-vertex patches, grid over
  bbox = (xmin,xmax,ymin,ymax,zmin,zmax), result ACCUMULATED into ``data``;
  errors raise ``AdRuntimeException`` as the reference throws
  ``AdRuntimeException`` (src/AdException.h).
* ``Session`` holds a resident particle lattice and its octree:
  ``build_octree`` is generate_tree (src/AdOctreeGeneration.h:76),
  ``deposit_leaves`` the single-rank leaf loop (src/AdDynamicLoadBalancing.h:983).
* ``deposit_workflow`` strings them together like deposit_workflow
  (src/AdDepositWorkFlow.h:60-237) for one rank, returning the leaf grids
  instead of writing files (``write_patch`` is ``write_leaf_files``).

All arithmetic runs in libadeco_gb300.so on the GPU.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

from . import _lib as L
from ._lib import AdecoError


class AdRuntimeException(AdecoError):
    """Raised where the reference throws AdRuntimeException."""


def _ptr(a):
    return C.c_void_p(a.ctypes.data) if a is not None else None


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _raise(rc):
    if rc != L.OK:
        raise AdRuntimeException(rc, L.load().adeco_last_error().decode(errors="replace"))


class DepositWrapper:
    """``AdaptiveMassDeposit::DepositWrapper`` (src/AdDeposit2Grid.h:59-93)."""

    h_grid_mass_type = np.float32
    vertex_type = np.float32
    mass_type = np.float32

    @staticmethod
    def deposit_tets(use_specific_gpu, device_id_to_use, tet_offset, num_tets_2_process, positions, positions_size,
                     meta_cells_per_patch, bbox, dims, data):
        """Deposit patches [tet_offset, tet_offset+num_tets_2_process) into ``data`` (+=)."""
        lib = L.load()
        pos = _f32(positions).reshape(-1)
        bb = _f32(bbox).reshape(6)
        if not (isinstance(data, np.ndarray) and data.dtype == np.float32 and data.flags.c_contiguous):
            raise AdRuntimeException(L.ERR_ARGUMENT if hasattr(L, "ERR_ARGUMENT") else 1,
                                     "data must be a C-contiguous float32 array")
        if data.size != dims ** 3:
            raise AdRuntimeException(1, f"data has {data.size} cells, expected dims^3 = {dims ** 3}")
        _raise(lib.adeco_deposit_tets(int(bool(use_specific_gpu)), int(device_id_to_use), int(tet_offset),
                                      int(num_tets_2_process), _ptr(pos), int(positions_size), int(meta_cells_per_patch),
                                      _ptr(bb), int(dims), _ptr(data)))


def deposit_tets_ex(positions, m, bbox, dims, *, data=None, patch_offset=0, num_patches=None, out_dtype=np.float64,
                    precision=L.PREC_MIXED, tet_order=L.ORDER_REF, tet_mass=1.0, device=None):
    """Extended boundary: FP64 or FP32 output, precision / tet-order / mass options."""
    lib = L.load()
    pos = _f32(positions).reshape(-1)
    bb = _f32(bbox).reshape(6)
    fpp = 3 * (m + 1) ** 3
    if num_patches is None:
        num_patches = pos.size // fpp - patch_offset
    if data is None:
        data = np.zeros(dims ** 3, dtype=out_dtype)
    a = L.DepositArgs()
    a.use_specific_gpu = int(device is not None)
    a.device_id = int(device or 0)
    a.patch_offset = int(patch_offset)
    a.num_patches = int(num_patches)
    a.positions = pos.ctypes.data
    a.positions_size = pos.size
    a.meta_cells_per_patch = int(m)
    a.bbox = bb.ctypes.data
    a.dims = int(dims)
    a.data = data.ctypes.data
    a.out_type = L.OUT_F64 if data.dtype == np.float64 else L.OUT_F32
    a.precision = int(precision)
    a.tet_order = int(tet_order)
    a.tet_mass = float(tet_mass)
    _raise(lib.adeco_deposit_tets_ex(C.byref(a)))
    return data


def tet_records(positions, m, bbox, dims, tet_order=L.ORDER_REF, counts=False):
    """Per-tet connectivity / candidate-range records computed on the GPU."""
    lib = L.load()
    pos = _f32(positions).reshape(-1)
    ncubes = (pos.size // (3 * (m + 1) ** 3)) * m ** 3
    rec = np.zeros(max(1, ncubes * 6 * 13), dtype=np.int32)
    cand = np.zeros(dims ** 3, dtype=np.uint32) if counts else None
    _raise(lib.adeco_debug_tet_records(_ptr(pos), pos.size, int(m), 0, ncubes, _ptr(_f32(bbox)), int(dims),
                                       int(tet_order), _ptr(rec), _ptr(cand)))
    rec = rec[:ncubes * 6 * 13].reshape(ncubes * 6, 13)
    return (rec, cand) if counts else rec


@dataclass
class OctreeInfo:
    nodes: np.ndarray      # structured: min(3), ext, level, parent, first_child, n_meta, estimate
    leaves: np.ndarray     # node ids, getLeafNodes order
    levels: int


class Session:
    """A resident particle lattice (+ octree) on one GPU."""

    def __init__(self, positions, *, device=0, tet_order=L.ORDER_REF, tet_mass=1.0, hbm_fraction=0.75,
                 accumulate_fp64=True):
        lib = L.load()
        pos = _f32(positions)
        if pos.ndim != 4 or pos.shape[-1] != 3:
            raise ValueError("positions must have shape (nz, ny, nx, 3) (x fastest)")
        self.shape = pos.shape[:3]
        nz, ny, nx = self.shape
        cfg = L.SessionConfig(device, tet_order, tet_mass, hbm_fraction, int(bool(accumulate_fp64)))
        h = C.c_void_p()
        _raise(lib.adeco_session_create(C.byref(cfg), _ptr(pos), nx, ny, nz, C.byref(h)))
        self._h = h
        self._lib = lib
        self.leaf_dims = None
        self.tet_mass = tet_mass

    @classmethod
    def from_file(cls, path, fmt="DARK_SKY", *, stride=1, periodic=True, device=0, tet_order=L.ORDER_REF,
                  tet_mass=1.0, hbm_fraction=0.75, accumulate_fp64=True):
        """A session whose lattice is read from a SORTED_BY_ID or DARK_SKY particle
        file (the reference's reader step); `read_bbox` holds the particles'
        bounding box before the periodic unwrap."""
        lib = L.load()
        code = {"SORTED_BY_ID": L.FORMAT_SORTED_BY_ID, "DARK_SKY": L.FORMAT_DARK_SKY}
        key = next((k for k in code if k in fmt), None)
        if key is None:
            raise AdRuntimeException(L.ERR_ARGUMENT, f"id_type {fmt} not supported")
        cfg = L.SessionConfig(device, tet_order, tet_mass, hbm_fraction, int(bool(accumulate_fp64)))
        bb = np.zeros(6, np.float32)
        h = C.c_void_p()
        _raise(lib.adeco_session_create_from_file(C.byref(cfg), os.fsencode(path), code[key], int(stride),
                                                  int(bool(periodic)), _ptr(bb), C.byref(h)))
        self = cls.__new__(cls)
        self._h, self._lib = h, lib
        dims = np.zeros(3, np.int32)
        _raise(lib.adeco_session_lattice_dims(h, _ptr(dims)))
        self.shape = (int(dims[2]), int(dims[1]), int(dims[0]))
        self.leaf_dims = None
        self.tet_mass = tet_mass
        self.read_bbox = bb
        return self

    def positions(self):
        """The resident lattice, (nz, ny, nx, 3) float32."""
        out = np.zeros(self.shape + (3,), np.float32)
        _raise(self._lib.adeco_session_positions(self._h, _ptr(out), out.size))
        return out

    def close(self):
        if getattr(self, "_h", None):
            self._lib.adeco_session_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def bbox(self):
        b = np.zeros(6, np.float32)
        _raise(self._lib.adeco_session_bbox(self._h, _ptr(b)))
        return b

    def build_octree(self, max_tets_per_node, max_level, leaf_dims=16, box6=None, roi6=None, builder="device"):
        """generate_tree over the resident lattice; `builder` "device" (default)
        or "host" says where the per-(node, meta-cell) work runs: both give the
        same tree."""
        b = None if box6 is None else _f32(box6)
        r = None if roi6 is None else _f32(roi6)
        which = {"device": L.OCTREE_DEVICE, "host": L.OCTREE_HOST}[builder]
        _raise(self._lib.adeco_session_set_octree_builder(self._h, which))
        _raise(self._lib.adeco_session_build_octree(self._h, _ptr(b), _ptr(r), int(max_tets_per_node),
                                                    int(max_level), int(leaf_dims)))
        self.leaf_dims = leaf_dims
        return self.octree()

    def octree(self) -> OctreeInfo:
        nn, nl, lv = C.c_int(), C.c_int(), C.c_int()
        _raise(self._lib.adeco_session_octree_size(self._h, C.byref(nn), C.byref(nl), C.byref(lv)))
        nodes = (L.Node * nn.value)()
        _raise(self._lib.adeco_session_octree_nodes(self._h, nodes, nn.value))
        leaves = np.zeros(nl.value, np.int32)
        _raise(self._lib.adeco_session_leaves(self._h, _ptr(leaves), nl.value))
        return OctreeInfo(np.ctypeslib.as_array(nodes).copy(), leaves, lv.value)

    def leaf_meta(self, leaf_index):
        cnt = C.c_int()
        _raise(self._lib.adeco_session_leaf_meta(self._h, int(leaf_index), None, 0, C.byref(cnt)))
        ids = np.zeros(max(1, cnt.value), np.uint64)
        _raise(self._lib.adeco_session_leaf_meta(self._h, int(leaf_index), _ptr(ids), cnt.value, C.byref(cnt)))
        return ids[:cnt.value]

    def deposit_leaves(self, precision=L.PREC_MIXED, fetch=True, stats=False):
        """Deposit all leaves; returns (grids (n_leaves, d, d, d) FP64 or None, timing dict)."""
        info = self.octree()
        d = self.leaf_dims
        out = np.zeros((len(info.leaves), d, d, d), np.float64) if fetch else None
        t = L.Timing()
        _raise(self._lib.adeco_session_deposit_leaves(self._h, int(precision), _ptr(out), int(bool(stats)),
                                                      C.byref(t)))
        return out, t.as_dict()

    def replay_leaves(self, reps):
        t = L.Timing()
        _raise(self._lib.adeco_session_replay_leaves(self._h, int(reps), C.byref(t)))
        return t.as_dict()

    def leaf_grids_device(self):
        p, n = C.c_void_p(), C.c_size_t()
        _raise(self._lib.adeco_session_leaf_grids_device(self._h, C.byref(p), C.byref(n)))
        return p.value, n.value

    # --- zoom requests / serving
    def submit(self, requests):
        """requests: iterable of (center(3), side, dims[, precision]) -> batch id."""
        reqs = list(requests)
        arr = (L.Request * len(reqs))()
        for i, r in enumerate(reqs):
            c, side, dims = r[0], r[1], r[2]
            prec = r[3] if len(r) > 3 else L.PREC_MIXED
            arr[i].center[0], arr[i].center[1], arr[i].center[2] = (float(c[0]), float(c[1]), float(c[2]))
            arr[i].side = float(side)
            arr[i].dims = int(dims)
            arr[i].precision = int(prec)
        bid = C.c_uint64()
        _raise(self._lib.adeco_session_submit(self._h, arr, len(reqs), C.byref(bid)))
        return bid.value

    def poll(self, batch):
        done = C.c_int()
        _raise(self._lib.adeco_session_poll(self._h, C.c_uint64(batch), C.byref(done)))
        return bool(done.value)

    def wait(self, batch, timeout_s=600.0):
        _raise(self._lib.adeco_session_wait(self._h, C.c_uint64(batch), float(timeout_s)))

    def result(self, batch, index, dims):
        out = np.zeros((dims, dims, dims), np.float64)
        _raise(self._lib.adeco_session_result(self._h, C.c_uint64(batch), int(index), _ptr(out), out.size))
        return out

    def latency_ms(self, batch, index):
        v = C.c_double()
        _raise(self._lib.adeco_session_latency(self._h, C.c_uint64(batch), int(index), C.byref(v)))
        return v.value

    def device_ms(self, batch):
        """Device time of the batch's deposit launch (waits for the batch)."""
        v = C.c_double()
        _raise(self._lib.adeco_session_batch_device_ms(self._h, C.c_uint64(batch), C.byref(v)))
        return v.value

    def release(self, batch):
        _raise(self._lib.adeco_session_release(self._h, C.c_uint64(batch)))

    def serving_stats(self):
        st = L.ServingStats()
        _raise(self._lib.adeco_session_serving_stats(self._h, C.byref(st)))
        return st.as_dict()

    # --- launch-shape / batching parameters (adeco_tuning)
    def get_tuning(self):
        t = L.Tuning()
        _raise(self._lib.adeco_session_get_tuning(self._h, C.byref(t)))
        return t.as_dict()

    def set_tuning(self, **fields):
        """Change the named adeco_tuning fields (zoom_tile, share_chunk, clip_batch,
        ctas_per_sm, route_capacity); returns the previous values."""
        t = L.Tuning()
        _raise(self._lib.adeco_session_get_tuning(self._h, C.byref(t)))
        old = t.as_dict()
        for k, v in fields.items():
            if k not in old:
                raise AdRuntimeException(L.ERR_ARGUMENT, f"unknown tuning field {k}")
            setattr(t, k, int(v))
        _raise(self._lib.adeco_session_set_tuning(self._h, C.byref(t)))
        return old


def leaf_bbox(node):
    """(xmin,xmax,ymin,ymax,zmin,zmax) of an octree node, as the leaf loop forms it."""
    mn, e = node["min"], node["ext"]
    return np.array([mn[0], np.float32(mn[0] + e), mn[1], np.float32(mn[1] + e), mn[2], np.float32(mn[2] + e)],
                    dtype=np.float32)


def leaf_file_name(info: OctreeInfo, q, leaf_dims):
    """``node_<level>_<ix>_<iy>_<iz>`` of leaf q: its origin in cells of its own
    level from the root's corner (src/AdOctreeGridWriter.h:104-123)."""
    root, nd = info.nodes[0], info.nodes[info.leaves[q]]
    cell = float(nd["ext"]) / leaf_dims
    io = [int(np.rint((float(nd["min"][a]) - float(root["min"][a])) / cell)) for a in range(3)]
    return f"node_{int(nd['level'])}_{io[0]}_{io[1]}_{io[2]}", io


def write_leaf_files(out_dir, info: OctreeInfo, grids, leaf_dims):
    """``write_patch`` (src/AdOctreeGridWriter.h:67-144): float32 density per leaf
    into ``node_<level>_<ix>_<iy>_<iz>``, then the index ``write_meta_data``
    would write.  Returns the total mass."""
    os.makedirs(out_dir, exist_ok=True)
    total = 0.0
    masses = []
    for q, nid in enumerate(info.leaves):
        nd = info.nodes[nid]
        cell = float(nd["ext"]) / leaf_dims
        inv_cell_vol = 1.0 / (cell * cell * cell)
        g = grids[q].reshape(-1)
        m = float(g.sum())
        masses.append(m)
        total += m
        name, _ = leaf_file_name(info, q, leaf_dims)
        (g * inv_cell_vol).astype(np.float32).tofile(os.path.join(out_dir, name))
    write_meta_data(out_dir, info, leaf_dims, masses)
    return total


def write_meta_data(out_dir, info: OctreeInfo, leaf_dims, masses=None, filename="octree_meta.json"):
    """The leaf index the reference declares but leaves empty (``write_meta_data``,
    src/AdOctreeGridWriter.h:58-64): the root box, the leaf resolution and, per
    leaf in getLeafNodes order, its file name, level, integer origin, FP32
    corner and extent and deposited mass.  JSON, so any reader can find a
    leaf's file and place its cells."""
    import json
    root = info.nodes[0]
    leaves = []
    for q, nid in enumerate(info.leaves):
        nd = info.nodes[nid]
        name, io = leaf_file_name(info, q, leaf_dims)
        leaves.append({"file": name, "node": int(nid), "level": int(nd["level"]), "origin_cells": io,
                       "min": [float(v) for v in nd["min"]], "ext": float(nd["ext"]),
                       "mass": None if masses is None else float(masses[q])})
    meta = {"format": "float32 density (mass / cell volume), x fastest", "leaf_dims": int(leaf_dims),
            "root_min": [float(v) for v in root["min"]], "root_ext": float(root["ext"]),
            "levels": int(info.levels), "leaves": leaves}
    with open(os.path.join(out_dir, filename), "w") as f:
        json.dump(meta, f, indent=1)


def deposit_workflow(positions, *, max_tets_per_octree_node, max_refinement_level, linear_patch_resolution=16,
                     region_of_interest=None, precision=L.PREC_MIXED, output_directory=None, device=0):
    """Single-rank deposit_workflow: octree over the particle AABB, every leaf
    deposited; returns (OctreeInfo, leaf grids (n_leaves, d, d, d), total mass)."""
    with Session(positions, device=device) as s:
        info = s.build_octree(max_tets_per_octree_node, max_refinement_level, linear_patch_resolution,
                              roi6=region_of_interest)
        grids, _ = s.deposit_leaves(precision=precision)
    total = float(grids.sum())
    if output_directory:
        write_leaf_files(output_directory, info, grids, linear_patch_resolution)
    return info, grids, total
