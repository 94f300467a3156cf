"""The CPU oracle against the golden fixtures made by the reference's own code
(tests/golden/make_golden.py): FP32 bit-exact, FP64 bit-exact, octree topology
identical.  These pin the oracle that every GPU parity test relies on."""
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN, load_golden


def test_kat_clip_volumes(oracle):
    g = load_golden("kat_tets.npz")
    for name, tet, v32, v64, cls in zip(g["names"], g["tets"], g["vol_f32"], g["vol_f64"], g["class_f32"]):
        assert np.float32(oracle.clip_volume(tet.astype(np.float32), fp64=False)) == v32, name
        assert oracle.clip_volume(tet, fp64=True) == v64, name
        assert oracle.classify(tet.astype(np.float32)) == cls, name


def test_kat_known_volumes(oracle):
    """Analytic answers for the shapes whose volume is known in closed form."""
    g = load_golden("kat_tets.npz")
    vol = dict(zip(g["names"], g["vol_f64"]))
    assert vol["inside_one_cell"] == pytest.approx(0.5 ** 3 / 6, rel=1e-12)
    assert vol["unit_corner_tet"] == pytest.approx(1 / 6, rel=1e-12)
    assert vol["cell_inside_tet"] == pytest.approx(1.0, rel=1e-12)
    assert vol["outside"] == 0.0
    assert abs(vol["zero_volume"]) < 1e-12


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "lattice_*.npz"))))
def test_lattice_deposits_bitexact(oracle, path):
    g = dict(np.load(path))
    m, dims = int(g["m"]), int(g["dims"])
    f32 = oracle.deposit_patches(g["positions"], m, g["bbox"], dims, fp64=False)
    assert np.array_equal(f32.view(np.uint32), g["grid_f32"].view(np.uint32))
    f64 = oracle.deposit_patches(g["positions"], m, g["bbox"], dims, fp64=True)
    assert np.array_equal(f64, g["grid_f64"])
    if g["conf_f64"].size:
        c64 = oracle.deposit_patches(g["positions"], m, g["bbox"], dims, fp64=True, order=oracle.ORDER_CONFORMING)
        assert np.array_equal(c64, g["conf_f64"])


def test_padded_patch_sequence_bitexact(oracle):
    g = load_golden("patches_padded.npz")
    f32 = oracle.deposit_patches(g["positions"], int(g["m"]), g["bbox"], int(g["dims"]), fp64=False,
                                 patch_offset=int(g["patch_offset"]), num_patches=int(g["num_patches"]))
    assert np.array_equal(f32.view(np.uint32), g["grid_f32"].view(np.uint32))


def test_octree_topology_identical(oracle):
    g = load_golden("octree.npz")
    n = int(g["n"])
    nodes, off, ids, leaves = oracle.generate_tree(g["positions"], (n, n, n), g["box"], g["roi"],
                                                   int(g["max_tets"]), int(g["max_level"]))
    assert len(nodes) == len(g["node_f"])
    assert np.array_equal(np.stack([nodes["min"][:, 0], nodes["min"][:, 1], nodes["min"][:, 2], nodes["ext"]], 1),
                          g["node_f"])
    assert np.array_equal(nodes["level"], g["node_i"][:, 0])
    assert np.array_equal(nodes["parent"], g["node_i"][:, 1])
    assert np.array_equal(nodes["first_child"], g["node_i"][:, 2])
    assert np.array_equal(nodes["estimate"], g["node_est"])
    assert np.array_equal(leaves, g["leaf_ids"])
    for q, leaf in enumerate(leaves):
        assert np.array_equal(ids[off[leaf]:off[leaf + 1]], g["leaf_meta_ids"][g["leaf_meta_off"][q]:g["leaf_meta_off"][q + 1]])


def test_leaf_deposits_bitexact(oracle):
    g = load_golden("octree.npz")
    n = int(g["n"])
    nodes, off, ids, leaves = oracle.generate_tree(g["positions"], (n, n, n), g["box"], g["roi"],
                                                   int(g["max_tets"]), int(g["max_level"]))
    d = int(g["leaf_dims"])
    for q, ref in enumerate(g["leaf_grids"]):
        nd = nodes[leaves[q]]
        lb = np.array([nd["min"][0], nd["min"][0] + nd["ext"], nd["min"][1], nd["min"][1] + nd["ext"],
                       nd["min"][2], nd["min"][2] + nd["ext"]], np.float32)
        got = oracle.deposit_meta(g["positions"], (n, n, n), ids[off[leaves[q]]:off[leaves[q] + 1]], lb, d, fp64=False)
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))


def test_fp64_mass_conservation(oracle):
    """Each tet deposits exactly its mass when the (cubic) grid contains it."""
    g = load_golden("lattice_lat12_d3.npz")
    pos = g["positions"].reshape(-1, 3)
    lo, hi = float(pos.min()) - 1.0, float(pos.max()) + 1.0
    bb = np.array([lo, hi, lo, hi, lo, hi], np.float32)
    m = int(g["m"])
    for order in (oracle.ORDER_REF, oracle.ORDER_CONFORMING):
        grid = oracle.deposit_patches(g["positions"], m, bb, 16, fp64=True, order=order)
        assert grid.sum() == pytest.approx(6 * m ** 3, rel=1e-12)


def test_empty_input_is_a_no_op(oracle):
    grid = np.ones(8, np.float32)
    oracle.deposit_patches(np.zeros(0, np.float32), 7, np.array([0, 1, 0, 1, 0, 1], np.float32), 2,
                           fp64=False, grid=grid, num_patches=0)
    assert np.all(grid == 1)


def test_reader_restatement_matches_reference_fixtures(tmp_path):
    """oracle/readers.py against the lattices the reference's own readers made
    from the same SORTED_BY_ID / DARK_SKY files (bit-exact, bbox included)."""
    import sys
    from oracle import readers as R
    sys.path.insert(0, str(GOLDEN))
    from make_golden_readers import CASES, write_inputs
    g = load_golden("readers.npz")
    paths = write_inputs(g["lattice"], str(tmp_path))
    for k, (fmt, stride, periodic) in enumerate(CASES):
        xyz, bbox = R.read_particles(paths[fmt], fmt, stride, bool(periodic))
        assert np.array_equal(xyz, g[f"xyz_{k}"]), (fmt, stride, periodic)
        assert np.array_equal(bbox, g[f"bbox_{k}"])
    with pytest.raises(ValueError):
        R.read_particles(paths["DARK_SKY"], "DARK_SKY", 3, True)   # 16 is not a multiple of 3
