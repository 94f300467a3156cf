"""Generate the golden fixtures from the reference's own code.

Run here, where the reference tree exists (oracle/_ref/libadeco_ref.so is
built from it by ``make -C oracle ref``):

    python tests/golden/make_golden.py

Every array in the .npz files below is an output of the reference's code
(src/AdDeposit2Grid.cpp, src/AdDepositTets2Grid.h, src/AdTetIntersection.h,
src/AdOctreeGeneration.h) on seeded inputs that are stored beside it, so the
fixtures pin the oracle and the GPU path without the reference present.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from adeco_gb300.synthetic import zeldovich_lattice  # noqa: E402
from oracle import oracle as O  # noqa: E402


def cubic_box(pos, pad=0.0):
    p = pos.reshape(-1, 3)
    lo = float(p.min()) - pad
    hi = float(p.max()) + pad
    return np.array([lo, hi, lo, hi, lo, hi], dtype=np.float32)


def kat_tets():
    """Known-answer tets in cell-scaled coordinates (the unit cell is [0,1]^3)."""
    T = {}
    T["inside_one_cell"] = [[0.1, 0.1, 0.1], [0.6, 0.1, 0.1], [0.1, 0.6, 0.1], [0.1, 0.1, 0.6]]
    T["unit_corner_tet"] = [[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]]
    T["cell_inside_tet"] = [[-1, -1, -1], [5, -1, -1], [-1, 5, -1], [-1, -1, 5]]
    T["straddle_one_face"] = [[0.5, 0.2, 0.2], [1.5, 0.2, 0.3], [0.6, 0.7, 0.2], [0.6, 0.3, 0.8]]
    T["straddle_two_faces"] = [[0.7, 0.7, 0.2], [1.4, 0.6, 0.3], [0.6, 1.5, 0.2], [0.8, 0.8, 0.9]]
    T["straddle_three_faces"] = [[0.8, 0.8, 0.8], [1.6, 0.7, 0.7], [0.7, 1.6, 0.7], [0.7, 0.7, 1.6]]
    T["large_through"] = [[-2.3, -1.7, -2.1], [3.1, -0.4, -1.2], [0.2, 3.3, -0.7], [0.4, 0.6, 3.9]]
    T["near_degenerate"] = [[0.2, 0.3, 0.4], [1.3, 0.3, 0.4], [0.2, 1.3, 0.4], [0.75, 0.8, 0.4000001]]
    T["zero_volume"] = [[0.2, 0.3, 0.4], [1.3, 0.3, 0.4], [0.2, 1.3, 0.4], [0.5, 0.5, 0.4]]
    T["vertex_on_face"] = [[0.0, 0.3, 0.4], [0.9, 0.3, 0.4], [0.2, 0.9, 0.4], [0.3, 0.4, 1.0]]
    T["outside"] = [[1.5, 1.5, 1.5], [2.5, 1.5, 1.5], [1.5, 2.5, 1.5], [1.5, 1.5, 2.5]]
    names = sorted(T)
    tets = np.array([T[k] for k in names], dtype=np.float64)
    # positively orient (the clip routine's contract)
    for t in tets:
        v6 = np.linalg.det(np.array([t[0] - t[3], t[1] - t[3], t[2] - t[3]]))
        if v6 < 0:
            t[[0, 3]] = t[[3, 0]]
    return names, tets


def main():
    O.build(ref=True, ref_src=os.environ.get("REF_SRC") or "/root/reference/src")
    R = O.ref()
    if R is None:
        raise SystemExit("reference harness missing: run `make -C oracle ref` where the reference exists")

    # 1. known-answer tets
    names, tets = kat_tets()
    v32 = np.array([R.ref_clip_volume_f32(np.ascontiguousarray(t.astype(np.float32).reshape(12))) for t in tets],
                   dtype=np.float32)
    v64 = np.array([R.ref_clip_volume_f64(np.ascontiguousarray(t.reshape(12))) for t in tets])
    cls = np.array([R.ref_classify_f32(np.ascontiguousarray(t.astype(np.float32).reshape(12))) for t in tets],
                   dtype=np.int32)
    np.savez_compressed(os.path.join(HERE, "kat_tets.npz"), names=np.array(names), tets=tets, vol_f32=v32,
                        vol_f64=v64, class_f32=cls)

    # 2. one-patch lattice deposits (the reference boundary, m = n-1)
    cases = {}
    for tag, n, disp, dims, seed in (("lat9_d0.5", 9, 0.5, 12, 0), ("lat12_d3", 12, 3.0, 16, 1),
                                     ("lat8_d0", 8, 0.0, 14, 2)):
        pos = zeldovich_lattice(n, L=100.0 * n / 64.0, seed=seed, rms_disp=disp)
        flat = np.ascontiguousarray(pos.reshape(-1))
        bb = cubic_box(pos, pad=0.0)
        m = n - 1
        g32 = np.zeros(dims ** 3, np.float32)
        assert R.ref_deposit_patches_f32(0, 1, flat, flat.size, m, bb, dims, g32) == 0
        g64 = np.zeros(dims ** 3, np.float64)
        R.ref_deposit_patches_f64(0, 1, flat, m, bb, dims, 0, g64)
        c64 = np.zeros(dims ** 3, np.float64)
        R.ref_deposit_patches_f64(0, 1, flat, m, bb, dims, 1, c64)
        cases[tag] = dict(positions=flat, m=m, bbox=bb, dims=dims, grid_f32=g32, grid_f64=g64, conf_f64=c64)
    # a grid box that cuts the lattice (mass outside is dropped) and a shifted sub-box
    pos = zeldovich_lattice(10, L=15.0, seed=3, rms_disp=1.0)
    flat = np.ascontiguousarray(pos.reshape(-1))
    cb = cubic_box(pos)
    mid = 0.5 * (cb[0] + cb[1])
    sub = np.array([mid - 3.0, mid + 2.0, mid - 2.5, mid + 2.5, mid - 1.0, mid + 4.0], np.float32)
    g32 = np.zeros(20 ** 3, np.float32)
    assert R.ref_deposit_patches_f32(0, 1, flat, flat.size, 9, sub, 20, g32) == 0
    g64 = np.zeros(20 ** 3, np.float64)
    R.ref_deposit_patches_f64(0, 1, flat, 9, sub, 20, 0, g64)
    cases["subbox"] = dict(positions=flat, m=9, bbox=sub, dims=20, grid_f32=g32, grid_f64=g64,
                           conf_f64=np.zeros(0))
    for tag, c in cases.items():
        np.savez_compressed(os.path.join(HERE, f"lattice_{tag}.npz"), **c)

    # 3. multi-patch sequence with 666 padding + patch offset (the leaf-loop input form)
    n = 11
    pos = zeldovich_lattice(n, L=17.0, seed=4, rms_disp=1.0)
    flat = np.ascontiguousarray(pos.reshape(-1))
    mcb = O.meta_bboxes(flat, (n, n, n))
    nmc = mcb.shape[0]
    blocks = []
    for mc in range(nmc):
        cz, r = divmod(mc, 2 * 2)  # 2x2x2 meta-cells for n=11 (ceil(10/7)=2)
        cy, cx = divmod(r, 2)
        blk = np.full((8, 8, 8, 3), 666.0, np.float32)
        mn = [cx * 7, cy * 7, cz * 7]
        d = [(n - mn[a]) if (c + 1 == 2) else 8 for a, c in enumerate((cx, cy, cz))]
        blk[:d[2], :d[1], :d[0]] = pos[mn[2]:mn[2] + d[2], mn[1]:mn[1] + d[1], mn[0]:mn[0] + d[0]]
        blocks.append(blk.reshape(-1))
    patches = np.ascontiguousarray(np.concatenate(blocks))
    bb = cubic_box(pos, pad=0.5)
    g32 = np.zeros(18 ** 3, np.float32)
    assert R.ref_deposit_patches_f32(1, nmc - 2, patches, patches.size, 7, bb, 18, g32) == 0
    np.savez_compressed(os.path.join(HERE, "patches_padded.npz"), positions=patches, m=7, bbox=bb, dims=18,
                        patch_offset=1, num_patches=nmc - 2, grid_f32=g32)

    # 4. octree topology + one leaf deposit
    n = 20
    pos = zeldovich_lattice(n, L=30.0, seed=5, rms_disp=2.0)
    flat = np.ascontiguousarray(pos.reshape(-1))
    p = flat.reshape(-1, 3)
    box = np.array([*p.min(0), *p.max(0)], np.float32)
    roi = np.array([1, 1, 1, 0, 0, 0], np.float32)  # invalid ROI -> whole domain
    maxn, maxid = 1 << 15, 1 << 20
    nf = np.zeros(4 * maxn, np.float32)
    ni = np.zeros(3 * maxn, np.int32)
    ne = np.zeros(maxn, np.uint64)
    lid = np.zeros(maxn, np.int32)
    nl = np.zeros(1, np.int32)
    lo = np.zeros(maxn + 1, np.int64)
    lids = np.zeros(maxid, np.uint64)
    max_tets, max_level = 3000, 5
    nn = R.ref_generate_tree(flat, n, n, n, box, roi, max_tets, max_level, nf, ni, ne, maxn, lid, nl, lo, lids,
                             maxid)
    assert nn > 0
    nleaf = int(nl[0])
    leaf_grids = []
    leaf_dims = 8
    nodes_f = nf[:4 * nn].reshape(nn, 4)
    for q in range(min(nleaf, 6)):
        node = nodes_f[lid[q]]
        lb = np.array([node[0], node[0] + node[3], node[1], node[1] + node[3], node[2], node[2] + node[3]],
                      np.float32)
        ids = np.ascontiguousarray(lids[lo[q]:lo[q + 1]])
        g = np.zeros(leaf_dims ** 3, np.float32)
        R.ref_deposit_leaf_f32(flat, n, n, n, ids, ids.size, lb, leaf_dims, g)
        leaf_grids.append(g)
    np.savez_compressed(os.path.join(HERE, "octree.npz"), positions=flat, n=n, box=box, roi=roi,
                        max_tets=max_tets, max_level=max_level, node_f=nodes_f, node_i=ni[:3 * nn].reshape(nn, 3),
                        node_est=ne[:nn], leaf_ids=lid[:nleaf], leaf_meta_off=lo[:nleaf + 1],
                        leaf_meta_ids=lids[:lo[nleaf]], leaf_dims=leaf_dims, leaf_grids=np.array(leaf_grids))
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
