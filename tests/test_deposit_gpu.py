"""GPU parity: the CUDA path (through the C ABI) against the oracle and the
reference-made golden fixtures.

Bars:
* tet connectivity and per-tet candidate ranges / per-cell candidate counts:
  bit-exact;
* octree topology: bit-exact;
* cell masses: |gpu - fp64| <= REL * fp64 + ABS per cell, REL = 1e-5, with
  ABS = 1e-7 tet masses: FP32 clipping leaves an absolute error of a few
  1e-8 tet masses in the cells a tet only grazes, so the bar is relative for
  every cell holding more than 1e-2 of a tet's mass (all interior cells) and
  absolute for the near-empty cells at the edge of the particle distribution;
* total mass: within 1e-9 relative at workload scale (>= 10^6 tets, asserted
  in test_total_mass_workload_scale).  The mixed path's per-tet mass error is
  random with a standard deviation of about 1e-7 (FP32 clipping arithmetic),
  so on the few-thousand-tet golden lattices the total is checked against
  that statistical bound, 1e-9 * M + 3e-7 * sqrt(N_tets).
"""
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN, load_golden

pytestmark = pytest.mark.gpu

REL = 1e-5
ABS = 1e-7


@pytest.fixture(scope="module")
def adeco():
    from adeco_gb300 import build, deposit
    build.build()
    return deposit


def check_cells(got, ref, rel=REL, abs_=ABS, n_tets=0):
    got = np.asarray(got, np.float64).reshape(-1)
    ref = np.asarray(ref, np.float64).reshape(-1)
    bad = np.abs(got - ref) > rel * np.abs(ref) + abs_
    assert not bad.any(), (f"{bad.sum()} cells out of tolerance; worst abs {np.abs(got - ref).max():.3e}; "
                           f"e.g. got {got[bad][:3]} ref {ref[bad][:3]}")
    if ref.sum() > 0:
        assert abs(got.sum() - ref.sum()) <= 1e-9 * ref.sum() + 3e-7 * np.sqrt(n_tets) + 1e-12


LATTICES = sorted(glob.glob(os.path.join(GOLDEN, "lattice_*.npz")))


@pytest.mark.parametrize("path", LATTICES)
def test_tet_connectivity_and_ranges_bitexact(adeco, oracle, path):
    g = dict(np.load(path))
    m, dims = int(g["m"]), int(g["dims"])
    for order in (oracle.ORDER_REF, oracle.ORDER_CONFORMING):
        rec, cand = adeco.tet_records(g["positions"], m, g["bbox"], dims, tet_order=order, counts=True)
        ref = oracle.tet_records(g["positions"], m, g["bbox"], dims, order=order)
        assert np.array_equal(rec, ref)
        _, ocand = oracle.deposit_patches(g["positions"], m, g["bbox"], dims, fp64=False, order=order, counts=True)
        assert np.array_equal(cand, ocand)


@pytest.mark.parametrize("path", LATTICES)
@pytest.mark.parametrize("precision", [0, 1], ids=["mixed", "plain_fp64"])
def test_lattice_deposit_vs_reference_fp64(adeco, path, precision):
    g = dict(np.load(path))
    m, dims = int(g["m"]), int(g["dims"])
    nt = 6 * m ** 3 if precision == 0 else 0
    # plain FP64 clips in a different (cancellation-free) order than the
    # reference's FP64 instantiation: both exact to rounding, ~1e-12 apart
    tol = dict(rel=REL, abs_=ABS) if precision == 0 else dict(rel=1e-10, abs_=1e-12)
    got = adeco.deposit_tets_ex(g["positions"], m, g["bbox"], dims, precision=precision)
    check_cells(got, g["grid_f64"], n_tets=nt, **tol)
    if g["conf_f64"].size:
        got = adeco.deposit_tets_ex(g["positions"], m, g["bbox"], dims, precision=precision, tet_order=1)
        check_cells(got, g["conf_f64"], n_tets=nt, **tol)


def test_reference_boundary_accumulates_float(adeco):
    """DepositWrapper.deposit_tets: float grid, +=, same meaning as the reference."""
    g = load_golden("lattice_lat12_d3.npz")
    m, dims = int(g["m"]), int(g["dims"])
    data = np.zeros(dims ** 3, np.float32)
    adeco.DepositWrapper.deposit_tets(True, 0, 0, 1, g["positions"], g["positions"].size, m, g["bbox"], dims, data)
    check_cells(data, g["grid_f64"], rel=1e-6 + REL, abs_=1e-6, n_tets=6 * m ** 3)
    first = data.copy()
    adeco.DepositWrapper.deposit_tets(False, 0, 0, 1, g["positions"], g["positions"].size, m, g["bbox"], dims, data)
    assert np.allclose(data, 2 * first, rtol=1e-6, atol=1e-6)
    # against the reference's own FP32 result: its error vs FP64 is the bound
    ref32 = g["grid_f32"].astype(np.float64)
    err_ref = np.abs(ref32 - g["grid_f64"]).max()
    assert np.abs(first - g["grid_f64"]).max() <= err_ref + 1e-6


@pytest.mark.parametrize("precision", [0, 1], ids=["mixed", "plain_fp64"])
@pytest.mark.parametrize("out_dtype", [np.float64, np.float32], ids=["f64", "f32"])
def test_boundary_adds_only_the_vertex_box(adeco, oracle, precision, out_dtype):
    """A cubic grid larger than the lattice (the vertices fill part of it
    along each axis): the call brings back and adds only the cells of the
    vertices' box, so a pre-filled grid gains the fresh deposit there and
    keeps every other cell; the fresh deposit matches the FP64 oracle.  (The
    plain FP64 path sums with FP64 atomics, so two calls agree to rounding,
    not bit for bit.)"""
    g = load_golden("lattice_lat12_d3.npz")
    m = int(g["m"])
    bb = g["bbox"].astype(np.float64)
    ext = bb[1::2] - bb[0::2]
    below = np.array([1.5, 0.0, 0.7]) * ext  # the lattice in the upper part along x, the lower along y
    grid = np.empty(6, np.float32)
    grid[0::2] = bb[0::2] - below
    grid[1::2] = bb[0::2] - below + 2.5 * ext  # cubic cells: the same extent along every axis
    dims = 40
    fresh = adeco.deposit_tets_ex(g["positions"], m, grid, dims, precision=precision,
                                  data=np.zeros(dims ** 3, out_dtype))
    ref = oracle.deposit_patches(g["positions"], m, grid, dims, fp64=True)
    tol = dict(rel=REL, abs_=ABS) if precision == 0 else dict(rel=1e-10, abs_=1e-12)
    if out_dtype == np.float32:
        tol = dict(rel=1e-6 + REL, abs_=1e-6)
    nt = 6 * m ** 3 if (precision == 0 or out_dtype == np.float32) else 0
    check_cells(fresh.astype(np.float64), ref, n_tets=nt, **tol)
    assert np.count_nonzero(fresh) < dims ** 3 // 4
    pre = np.random.default_rng(3).uniform(0.5, 2.0, dims ** 3).astype(out_dtype)
    got = adeco.deposit_tets_ex(g["positions"], m, grid, dims, precision=precision, data=pre.copy())
    outside = fresh == 0
    assert np.array_equal(got[outside], pre[outside])
    if precision == 0:
        assert np.array_equal(got, pre + fresh)
    else:
        assert np.allclose(got, pre + fresh, rtol=1e-12 if out_dtype == np.float64 else 1e-6, atol=0)


def test_padded_patch_sequence(adeco, oracle):
    g = load_golden("patches_padded.npz")
    m, dims = int(g["m"]), int(g["dims"])
    kw = dict(patch_offset=int(g["patch_offset"]), num_patches=int(g["num_patches"]))
    ref = oracle.deposit_patches(g["positions"], m, g["bbox"], dims, fp64=True, **kw)
    got = adeco.deposit_tets_ex(g["positions"], m, g["bbox"], dims, **kw)
    check_cells(got, ref, n_tets=6 * m ** 3 * int(g["num_patches"]))
    assert np.abs(g["grid_f32"] - ref).max() < 1e-3  # the fixture is the reference's FP32 of the same call


def test_random_lattice_vs_oracle(adeco, oracle):
    from adeco_gb300.synthetic import zeldovich_lattice
    for seed, n, disp, dims in ((11, 20, 1.0, 24), (12, 16, 4.0, 40), (13, 14, 0.3, 7)):
        pos = zeldovich_lattice(n, L=30.0, seed=seed, rms_disp=disp)
        p = pos.reshape(-1, 3)
        lo, hi = float(p.min()) + 1.0, float(p.max()) - 2.0
        bb = np.array([lo, hi, lo, hi, lo, hi], np.float32)
        ref = oracle.deposit_patches(pos.reshape(-1), n - 1, bb, dims, fp64=True)
        got = adeco.deposit_tets_ex(pos.reshape(-1), n - 1, bb, dims)
        check_cells(got, ref, n_tets=6 * (n - 1) ** 3)


def test_deterministic_bitwise(adeco):
    g = load_golden("lattice_lat12_d3.npz")
    m, dims = int(g["m"]), int(g["dims"])
    a = adeco.deposit_tets_ex(g["positions"], m, g["bbox"], dims)
    b = adeco.deposit_tets_ex(g["positions"], m, g["bbox"], dims)
    assert np.array_equal(a.view(np.uint64), b.view(np.uint64))


def test_empty_input_is_a_no_op(adeco):
    data = np.ones(8, np.float32)
    adeco.DepositWrapper.deposit_tets(False, 0, 0, 0, np.zeros(0, np.float32), 0, 7,
                                      np.array([0, 1, 0, 1, 0, 1], np.float32), 2, data)
    assert np.all(data == 1)


def test_errors_raise_like_the_reference(adeco):
    g = load_golden("lattice_lat9_d0.5.npz")
    m, dims = int(g["m"]), int(g["dims"])
    data = np.zeros(dims ** 3, np.float32)
    pos = g["positions"]
    with pytest.raises(adeco.AdRuntimeException) as e:       # inconsistent offset
        adeco.DepositWrapper.deposit_tets(False, 0, 1, 1, pos, pos.size, m, g["bbox"], dims, data)
    assert e.value.code == 6
    with pytest.raises(adeco.AdRuntimeException) as e:       # invalid device id
        adeco.DepositWrapper.deposit_tets(True, 4096, 0, 1, pos, pos.size, m, g["bbox"], dims, data)
    assert e.value.code == 3
    with pytest.raises(adeco.AdRuntimeException) as e:       # positions not a whole number of patches
        adeco.DepositWrapper.deposit_tets(False, 0, 0, 1, pos[:-3], pos.size - 3, m, g["bbox"], dims, data)
    assert e.value.code == 1
    with pytest.raises(adeco.AdRuntimeException) as e:       # int overflow of the cube counter
        adeco.DepositWrapper.deposit_tets(False, 0, 0, 1 << 26, pos, pos.size, m, g["bbox"], dims, data)
    assert e.value.code == 2
    assert np.all(data == 0)


def test_octree_topology_and_leaves(adeco, oracle):
    g = load_golden("octree.npz")
    n = int(g["n"])
    pos = g["positions"].reshape(n, n, n, 3)
    d = int(g["leaf_dims"])
    with adeco.Session(pos) as s:
        box = g["box"]
        info = s.build_octree(int(g["max_tets"]), int(g["max_level"]), leaf_dims=d, box6=box, roi6=g["roi"])
        nodes = info.nodes
        assert len(nodes) == len(g["node_f"])
        assert np.array_equal(np.stack([nodes["min"][:, 0], nodes["min"][:, 1], nodes["min"][:, 2], nodes["ext"]], 1),
                              g["node_f"])
        assert np.array_equal(nodes["level"], g["node_i"][:, 0])
        assert np.array_equal(nodes["parent"], g["node_i"][:, 1])
        assert np.array_equal(nodes["first_child"], g["node_i"][:, 2])
        assert np.array_equal(nodes["estimate"], g["node_est"])
        assert np.array_equal(info.leaves, g["leaf_ids"])
        for q in range(len(info.leaves)):
            ref_ids = g["leaf_meta_ids"][g["leaf_meta_off"][q]:g["leaf_meta_off"][q + 1]]
            assert np.array_equal(s.leaf_meta(q), ref_ids)
        grids, _ = s.deposit_leaves()
        plain, _ = s.deposit_leaves(precision=1)
        for q, nid in enumerate(info.leaves):
            lb = adeco.leaf_bbox(nodes[nid])
            ref = oracle.deposit_meta(g["positions"], (n, n, n), s.leaf_meta(q), lb, d, fp64=True)
            check_cells(grids[q], ref, n_tets=2058 * len(s.leaf_meta(q)))
            check_cells(plain[q], ref, rel=1e-10, abs_=1e-12)
            if q < len(g["leaf_grids"]):  # the reference's own FP32 leaf deposit
                assert np.abs(g["leaf_grids"][q] - ref).max() < 1e-3
        # every tet lies in the root box and the leaves tile it; the leaves'
        # FP32 boxes (min + ext per axis, as the reference forms them) meet to
        # within an ulp, so the FP64 total is the tet count to ~1e-8
        total = 6 * (n - 1) ** 3
        assert abs(plain.sum() - total) <= 1e-7 * total
        assert abs(grids.sum() - plain.sum()) <= 1e-9 * total + 3e-7 * np.sqrt(total)


def test_clustered_leaves_vs_oracle_fp64(adeco, oracle):
    """The clustered regime: a 48^3 Zel'dovich lattice (rms 3 spacings) with 40
    spherical infall regions, where tets reach kappa = L^3/|6V| ~ 3e8 and a
    fifth of them take the barycentric route (kappa > 32).  Octree to depth
    10, 16^3 leaves; the densest leaves and a spread sample of the rest are
    checked against the FP64 oracle per cell at 1e-5 relative + 1e-7 tet
    masses, and the routed-tet count shows the route ran."""
    from concurrent.futures import ThreadPoolExecutor

    from adeco_gb300.synthetic import zeldovich_lattice
    n, d = 48, 16
    pos = zeldovich_lattice(n, L=100.0, seed=4, rms_disp=3.0, infall=40)
    flat = np.ascontiguousarray(pos.reshape(-1))
    with adeco.Session(pos) as s:
        info = s.build_octree(20000, 10, leaf_dims=d)
        grids, t = s.deposit_leaves(stats=True)
        metas = [s.leaf_meta(q) for q in range(len(info.leaves))]
    assert t["routed_tets"] > 10000, t
    est = info.nodes["estimate"][info.leaves]
    dense = list(np.argsort(-est.astype(np.float64))[:16])
    chosen = sorted(set(dense) | set(range(0, len(info.leaves), 6)))

    def ref(q):
        return oracle.deposit_meta(flat, (n, n, n), metas[q], adeco.leaf_bbox(info.nodes[info.leaves[q]]), d,
                                   fp64=True)

    with ThreadPoolExecutor(max_workers=os.cpu_count() or 1) as ex:
        refs = list(ex.map(ref, chosen))
    for q, r in zip(chosen, refs):
        check_cells(grids[q], r, n_tets=2058 * len(metas[q]))


def test_c1_periodic_uniform_grid_vs_oracle_fp64(adeco, oracle):
    """C1 at full size through the reference boundary: a periodic 64^3
    Zel'dovich lattice (rms 0.5 spacings, seed 0, L = 100) as 64^3 cubes =
    1,572,864 tets -- ghost vertex planes shifted by +L, cut into 64 patches
    of 16^3 cubes -- deposited onto a uniform 128^3 grid over the box; the
    periodic wrap is the sum over the box's 27 images (each call accumulates,
    as the reference's deposit_tets does).  Every cell against the FP64
    oracle (the same image sum) at 1e-5 relative + 1e-7 tet masses; the total
    is the tet count to 1e-9."""
    from adeco_gb300.synthetic import image_boxes, lattice_patches, periodic_ghost_lattice, zeldovich_lattice
    n, L, m, dims = 64, 100.0, 16, 128
    pos = zeldovich_lattice(n, L=L, seed=0, rms_disp=0.5)
    patches = lattice_patches(periodic_ghost_lattice(pos, L), m)
    box = np.array([0, L, 0, L, 0, L], np.float32)
    got = np.zeros(dims ** 3)
    ref = np.zeros(dims ** 3)
    for b in image_boxes(box, L):
        adeco.deposit_tets_ex(patches, m, b, dims, data=got)
        oracle.deposit_patches(patches, m, b, dims, fp64=True, grid=ref, threads=os.cpu_count() or 1)
    tets = 6 * n ** 3
    assert abs(ref.sum() - tets) <= 1e-9 * tets
    check_cells(got, ref, n_tets=tets)
    assert abs(got.sum() - tets) <= 1e-9 * tets, got.sum() - tets


def _tree(s, builder, max_tets, max_level, box6=None, roi6=None):
    info = s.build_octree(max_tets, max_level, leaf_dims=8, box6=box6, roi6=roi6, builder=builder)
    return info.nodes, info.leaves, [s.leaf_meta(q) for q in range(len(info.leaves))]


@pytest.mark.parametrize("case", ["zeldovich96", "clustered64", "roi_corner", "small_box", "root_leaf", "level0"])
def test_octree_device_equals_host(adeco, case):
    """The device octree builder gives the host builder's tree: every node
    (boxes, level, parent, first child, meta count, estimate), the leaf order
    and every leaf's meta-cell list, bit for bit."""
    from adeco_gb300.synthetic import zeldovich_lattice
    if case == "clustered64":
        pos = zeldovich_lattice(64, L=100.0, seed=4, rms_disp=3.0, infall=40)
    else:
        pos = zeldovich_lattice(96 if case == "zeldovich96" else 48, L=100.0, seed=0, rms_disp=3.0)
    n = pos.shape[0]
    p = pos.reshape(-1, 3)
    lo, hi = p.min(0), p.max(0)
    args = {"zeldovich96": (262144 // 8, 8, None, None),
            "clustered64": (2000, 10, None, None),
            "roi_corner": (3000, 9, None, np.array([*lo, *(lo + 0.3 * (hi - lo))], np.float32)),
            "small_box": (3000, 7, np.array([*(lo + 0.2 * (hi - lo)), *(hi - 0.1 * (hi - lo))], np.float32), None),
            "root_leaf": (6 * n ** 3, 8, None, None),
            "level0": (100, 0, None, None)}[case]
    with adeco.Session(pos) as s:
        nd, ld, md = _tree(s, "device", args[0], args[1], args[2], args[3])
        nh, lh, mh = _tree(s, "host", args[0], args[1], args[2], args[3])
    assert len(nd) == len(nh)
    for f in ("min", "ext", "level", "parent", "first_child", "n_meta", "estimate"):
        assert np.array_equal(nd[f], nh[f]), f
    assert np.array_equal(ld, lh)
    assert all(np.array_equal(a, b) for a, b in zip(md, mh))
    if case in ("zeldovich96", "clustered64"):
        assert len(nd) > 8 * 8 + 1  # more than two levels refined


def test_total_mass_workload_scale(adeco):
    """Total mass at workload scale: a 96^3 Zel'dovich lattice (5.1M tets).
    Octree leaves: the mixed total equals the plain FP64 total of the same
    leaves to 1e-9 (the leaves' FP32 boxes, formed as the reference forms
    them, meet only to an ulp, so the FP64 total itself is the tet count to
    ~1e-8).  Uniform 128^3 grid over a box holding every particle: the total
    equals the tet count to 1e-9."""
    from adeco_gb300.synthetic import zeldovich_lattice
    n = 96
    pos = zeldovich_lattice(n, L=100.0, seed=0, rms_disp=3.0)
    total = 6 * (n - 1) ** 3
    with adeco.Session(pos) as s:
        s.build_octree(262144 // 8, 8, leaf_dims=16)
        grids, t = s.deposit_leaves(stats=True)
        plain, _ = s.deposit_leaves(precision=1)
        # the mixed total against the FP64 total of the same leaves
        assert abs(grids.sum() - plain.sum()) <= 1e-9 * total, grids.sum() - plain.sum()
        # per cell: 1e-5 relative with a floor of only 1e-9 tet masses (pieces
        # are clipped in the cell's mirrored frame near upper faces, so thin
        # slices keep their precision)
        d = np.abs(grids - plain)
        assert np.all(d <= 1e-5 * plain + 1e-9), float((d - 1e-5 * plain).max())
        assert abs(plain.sum() - total) <= 1e-7 * total
        assert t["tets"] >= total
    p = pos.reshape(-1, 3)
    lo, hi = float(p.min()) - 0.5, float(p.max()) + 0.5
    bb = np.array([lo, hi, lo, hi, lo, hi], np.float32)
    got = adeco.deposit_tets_ex(pos.reshape(-1), n - 1, bb, 128)
    assert abs(got.sum() - total) <= 1e-9 * total, got.sum() - total


def test_graph_replay_matches_launch(adeco):
    g = load_golden("octree.npz")
    n = int(g["n"])
    pos = g["positions"].reshape(n, n, n, 3)
    with adeco.Session(pos) as s:
        s.build_octree(int(g["max_tets"]), int(g["max_level"]), leaf_dims=8)
        a, _ = s.deposit_leaves()
        s.replay_leaves(3)
        _, nvals = s.leaf_grids_device()
        b, _ = s.deposit_leaves()
        assert nvals == a.size
        assert np.array_equal(a, b)


def test_session_from_page_locked_positions(adeco):
    """Page-locked host positions (read by the conversion kernel directly) give
    the same lattice and the same leaf deposits as pageable ones (copied
    through a staging buffer)."""
    import torch
    g = load_golden("octree.npz")
    n = int(g["n"])
    pos = np.ascontiguousarray(g["positions"].reshape(n, n, n, 3), dtype=np.float32)
    pinned = torch.empty(pos.size, dtype=torch.float32, pin_memory=True)
    pinned.numpy()[:] = pos.reshape(-1)
    view = pinned.numpy().reshape(n, n, n, 3)
    out = []
    for src in (pos, view):
        with adeco.Session(src) as s:
            assert np.array_equal(s.positions(), pos)
            s.build_octree(int(g["max_tets"]), int(g["max_level"]), leaf_dims=8)
            out.append(s.deposit_leaves()[0])
    assert np.array_equal(out[0], out[1])


def test_zoom_batch_same_alone_and_in_mix(adeco):
    from adeco_gb300.synthetic import zeldovich_lattice
    pos = zeldovich_lattice(24, L=40.0, seed=7, rms_disp=2.0)
    reqs = [((20.0, 20.0, 20.0), 6.0, 16), ((10.0, 25.0, 18.0), 10.0, 24), ((30.0, 12.0, 22.0), 3.0, 32)]
    with adeco.Session(pos) as s:
        alone = []
        for r in reqs:
            b = s.submit([r])
            s.wait(b)
            alone.append(s.result(b, 0, r[2]))
            s.release(b)
        b1 = s.submit(reqs[:2])
        b2 = s.submit(reqs[2:])
        s.wait(b1)
        s.wait(b2)
        mixed = [s.result(b1, 0, reqs[0][2]), s.result(b1, 1, reqs[1][2]), s.result(b2, 0, reqs[2][2])]
        for a, m_ in zip(alone, mixed):
            assert np.array_equal(a, m_)
        assert s.latency_ms(b1, 0) > 0


def test_zoom_requests_vs_oracle(adeco, oracle):
    """Zoom boxes over a resident lattice against the FP64 oracle over the same
    meta-cells: per-cell bar and total mass, boxes inside, across and beyond
    the particle distribution, at resolutions from coarse (many tets per cell)
    to fine (many cells per tet), one grid split into several tiles."""
    from adeco_gb300.synthetic import zeldovich_lattice
    n = 22
    pos = zeldovich_lattice(n, L=40.0, seed=11, rms_disp=2.0)
    flat = np.ascontiguousarray(pos.reshape(-1))
    cd = -(-(n - 1) // 7)
    ids = np.arange(cd ** 3, dtype=np.uint64)
    reqs = [((20.0, 20.0, 20.0), 12.0, 8), ((8.0, 30.0, 15.0), 7.0, 24), ((38.0, 2.0, 20.0), 9.0, 16),
            ((21.3, 18.7, 25.1), 2.5, 40), ((19.0, 21.0, 20.5), 6.0, 80)]
    with adeco.Session(pos) as s:
        b = s.submit(reqs)
        s.wait(b)
        assert s.device_ms(b) > 0
        for k, (c, side, d) in enumerate(reqs):
            got = s.result(b, k, d).reshape(-1)
            h = np.float32(0.5) * np.float32(side)
            box = np.array([np.float32(c[0]) - h, np.float32(c[0]) + h, np.float32(c[1]) - h, np.float32(c[1]) + h,
                            np.float32(c[2]) - h, np.float32(c[2]) + h], np.float32)
            ref = oracle.deposit_meta(flat, (n, n, n), ids, box, d, fp64=True)
            bad = np.abs(got - ref) > REL * np.abs(ref) + ABS
            assert not bad.any(), (k, int(bad.sum()), float(np.abs(got - ref).max()))
            assert abs(got.sum() - ref.sum()) <= 1e-9 * ref.sum() + 3e-7 * np.sqrt(6 * (n - 1) ** 3) + 1e-12
        s.release(b)


@pytest.mark.parametrize("precision", [0, 1], ids=["mixed", "plain_fp64"])
def test_fine_grid_vs_oracle(adeco, oracle, precision):
    """Cells much smaller than the tets (tens of cells per tet edge): same
    masses as the oracle's cell-by-cell deposit on both paths."""
    from adeco_gb300.synthetic import zeldovich_lattice
    n = 8
    pos = zeldovich_lattice(n, L=16.0, seed=21, rms_disp=1.5)
    bb = np.array([5.0, 9.0, 5.0, 9.0, 5.0, 9.0], np.float32)
    dims = 72
    ref = oracle.deposit_patches(pos.reshape(-1), n - 1, bb, dims, fp64=True)
    got = adeco.deposit_tets_ex(pos.reshape(-1), n - 1, bb, dims, precision=precision)
    if precision == 1:
        assert np.allclose(got, ref, rtol=1e-10, atol=1e-12)
    else:
        check_cells(got, ref, n_tets=6 * (n - 1) ** 3)


def test_particle_readers_vs_reference_fixtures(adeco, tmp_path):
    """Sessions read from SORTED_BY_ID / DARK_SKY files: lattice positions and
    bounding box bit-exact against what the reference's own readers made from
    the same files (periodic unwrap on and off, stride 1, 2, 4), and the
    reference's error conditions."""
    import sys
    sys.path.insert(0, GOLDEN)
    from make_golden_readers import CASES, write_inputs
    g = load_golden("readers.npz")
    paths = write_inputs(g["lattice"], str(tmp_path))
    for k, (fmt, stride, periodic) in enumerate(CASES):
        with adeco.Session.from_file(paths[fmt], fmt, stride=stride, periodic=bool(periodic)) as s:
            assert np.array_equal(s.positions(), g[f"xyz_{k}"]), (fmt, stride, periodic)
            assert np.array_equal(s.read_bbox, g[f"bbox_{k}"])
    with pytest.raises(adeco.AdRuntimeException):
        adeco.Session.from_file(paths["DARK_SKY"], "DARK_SKY", stride=3)       # 16 not a multiple of 3
    bad = tmp_path / "short.bin"
    bad.write_bytes(b"\0" * (12 * 15))                                          # 15 particles: not a cube
    with pytest.raises(adeco.AdRuntimeException):
        adeco.Session.from_file(str(bad), "SORTED_BY_ID")
    with pytest.raises(adeco.AdRuntimeException):
        adeco.Session.from_file(str(tmp_path / "missing.sdf"), "DARK_SKY")


def test_clustered_zoom_requests_vs_oracle(adeco, oracle):
    """Zoom requests over a clustered lattice (30 infall regions, many tets
    with kappa > 32): the batch kernel's one-item CTAs and the barycentric
    route kernel of the serving path, against the FP64 oracle per cell; a
    request alone gives the same masses, bit for bit, as inside the batch."""
    from adeco_gb300.synthetic import zeldovich_lattice
    n = 40
    pos = zeldovich_lattice(n, L=100.0, seed=6, rms_disp=3.0, infall=30)
    flat = np.ascontiguousarray(pos.reshape(-1))
    cd = -(-(n - 1) // 7)
    ids = np.arange(cd ** 3, dtype=np.uint64)
    reqs = [((50.0, 50.0, 50.0), 80.0, 32), ((30.0, 60.0, 45.0), 40.0, 24), ((65.0, 40.0, 55.0), 20.0, 40)]
    with adeco.Session(pos) as s:
        s.build_octree(20000, 8, leaf_dims=16)
        _, t = s.deposit_leaves(stats=True, fetch=False)
        assert t["routed_tets"] > 1000, t  # the lattice has ill-conditioned tets
        b = s.submit(reqs)
        got = [s.result(b, k, r[2]).reshape(-1) for k, r in enumerate(reqs)]
        s.release(b)
        b1 = s.submit([reqs[2]])
        assert np.array_equal(s.result(b1, 0, reqs[2][2]).reshape(-1), got[2])
        s.release(b1)
    for k, (c, side, d) in enumerate(reqs):
        h = np.float32(0.5) * np.float32(side)
        box = np.array([np.float32(c[0]) - h, np.float32(c[0]) + h, np.float32(c[1]) - h, np.float32(c[1]) + h,
                        np.float32(c[2]) - h, np.float32(c[2]) + h], np.float32)
        ref = oracle.deposit_meta(flat, (n, n, n), ids, box, d, fp64=True)
        bad = np.abs(got[k] - ref) > REL * np.abs(ref) + ABS
        assert not bad.any(), (k, int(bad.sum()), float(np.abs(got[k] - ref).max()))
        assert abs(got[k].sum() - ref.sum()) <= 1e-9 * ref.sum() + 3e-7 * np.sqrt(6 * (n - 1) ** 3) + 1e-12
