"""CPU-side checks of the drop-in boundary: the C-ABI library builds, loads
and exports every entry point include/adeco_deposit.h declares (no compute
calls without a GPU), and the C++ shim header compiles against it."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from adeco_gb300 import _lib as L

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from adeco_gb300 import build
    build.build()
    return L.load()


def test_header_declares_entry_points():
    names = L.declared_symbols()
    for expected in ("adeco_deposit_tets", "adeco_deposit_tets_ex", "adeco_session_create",
                     "adeco_session_build_octree", "adeco_session_deposit_leaves", "adeco_session_submit"):
        assert expected in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in L.declared_symbols() if not hasattr(lib, n)]
    assert not missing, f"declared but not exported: {missing}"


def test_bindings_cover_every_declared_symbol():
    assert set(L.declared_symbols()) <= set(L._SIGS), set(L.declared_symbols()) - set(L._SIGS)


def test_abi_version(lib):
    assert lib.adeco_abi_version() == 2


def test_last_error_is_empty_string_initially(lib):
    assert isinstance(lib.adeco_last_error(), bytes)


def test_boundary_argument_errors_on_the_host(lib):
    """The reference's AdRuntimeException cases (AdDeposit2Grid.cu:260-268,
    338-346; AdDeposit2Grid.cpp:95-98) and its silent return on empty input
    (AdDeposit2Grid.cpp:86-87) are decided on the host before any device call:
    the same status codes with or without a GPU, and the caller's grid is
    left untouched."""
    from adeco_gb300 import deposit as D
    from conftest import load_golden
    g = load_golden("lattice_lat9_d0.5.npz")
    m, dims = int(g["m"]), int(g["dims"])
    pos = np.ascontiguousarray(g["positions"], np.float32).reshape(-1)
    bbox = g["bbox"]
    data = np.full(dims ** 3, 7.0, np.float32)
    cases = [
        (dict(patch_offset=1, num_patches=1), 6),                                     # inconsistent offset
        (dict(patch_offset=0, num_patches=1, positions_size=pos.size - 3), 1),        # not a whole number of patches
        (dict(patch_offset=0, num_patches=1 << 26), 2),                               # int overflow of the cube counter
    ]
    for kw, code in cases:
        with pytest.raises(D.AdRuntimeException) as e:
            D.DepositWrapper.deposit_tets(False, 0, kw["patch_offset"], kw["num_patches"], pos,
                                          kw.get("positions_size", pos.size), m, bbox, dims, data)
        assert e.value.code == code, (kw, e.value)
    with pytest.raises(D.AdRuntimeException) as e:  # an empty bbox axis
        D.DepositWrapper.deposit_tets(False, 0, 0, 1, pos, pos.size, m, np.zeros(6, np.float32), dims, data)
    assert e.value.code == 1
    with pytest.raises(D.AdRuntimeException) as e:  # an unknown precision
        D.deposit_tets_ex(pos, m, bbox, dims, data=np.zeros(dims ** 3), precision=7)
    assert e.value.code == 1
    D.DepositWrapper.deposit_tets(False, 0, 0, 0, pos, pos.size, m, bbox, dims, data)  # empty: a no-op
    D.DepositWrapper.deposit_tets(False, 0, 0, 1, pos, 0, m, bbox, dims, data)
    assert np.all(data == 7.0)


def test_cpp_wrapper_header_compiles(tmp_path):
    src = tmp_path / "use_wrapper.cpp"
    src.write_text('#include "adeco_deposit_wrapper.hpp"\n'
                   'int main(){ float d[8]={0}; const float bb[6]={0,1,0,1,0,1};\n'
                   '  try { AdaptiveMassDeposit::DepositWrapper::deposit_tets(false,0,0,0,nullptr,0,7,bb,2,d); }\n'
                   '  catch (const AdaptiveMassDeposit::AdRuntimeException&) { return 1; }\n'
                   '  return 0; }\n')
    r = subprocess.run(["g++", "-std=c++11", "-fsyntax-only", "-I", os.path.join(ROOT, "include"), str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_leaf_writer_files_and_meta(tmp_path):
    """write_leaf_files: one float32 density file per leaf, named by level and
    integer origin as write_patch names them, plus the JSON leaf index."""
    import json
    import numpy as np
    from adeco_gb300.deposit import OctreeInfo, write_leaf_files
    dt = np.dtype([("min", "<f4", 3), ("ext", "<f4"), ("level", "<i4"), ("parent", "<i4"), ("first_child", "<i4"),
                   ("n_meta", "<i4"), ("estimate", "<u8")])
    nodes = np.zeros(9, dt)
    nodes[0] = ((0.0, 0.0, 0.0), 8.0, 0, -1, 1, 0, 0)
    for q in range(8):
        i, j, k = q & 1, (q >> 1) & 1, q >> 2
        nodes[1 + q] = ((4.0 * i, 4.0 * j, 4.0 * k), 4.0, 1, 0, -1, 0, 0)
    info = OctreeInfo(nodes=nodes, leaves=np.arange(8, 0, -1), levels=2)
    d = 4
    grids = np.arange(8 * d ** 3, dtype=np.float64).reshape(8, d, d, d)
    total = write_leaf_files(str(tmp_path), info, grids, d)
    assert total == grids.sum()
    meta = json.load(open(tmp_path / "octree_meta.json"))
    assert meta["leaf_dims"] == d and len(meta["leaves"]) == 8
    for q, leaf in enumerate(meta["leaves"]):
        nd = nodes[info.leaves[q]]
        expect = [int(nd["min"][a] / 1.0) for a in range(3)]        # cell = 4 / 4 = 1
        assert leaf["origin_cells"] == expect and leaf["file"] == "node_1_%d_%d_%d" % tuple(expect)
        data = np.fromfile(tmp_path / leaf["file"], np.float32)
        assert np.allclose(data, grids[q].reshape(-1) / 1.0)          # density = mass / 1^3
        assert leaf["mass"] == grids[q].sum()
