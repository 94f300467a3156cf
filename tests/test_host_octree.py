"""CPU check of the host octree builder (adeco_gb300/csrc/octree.cpp, the
builder adeco_session_set_octree_builder selects) against the golden tree the
reference's generate_tree made: every node, the leaf order and every leaf's
meta-cell list, bit for bit.  Compiled for the host with g++; no GPU."""
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

from conftest import load_golden

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _build(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path / "host_octree_check")
    cmd = [gxx, "-std=c++17", "-O2", "-ffp-contract=off", "-o", exe, os.path.join(HERE, "host_octree_check.cpp"),
           os.path.join(ROOT, "adeco_gb300", "csrc", "octree.cpp")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    return exe


def _run(exe, tmp_path, pos, n, box, roi, max_tets, max_level):
    src, dst = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(src, "wb") as f:
        f.write(struct.pack("<iiq", n, max_level, max_tets))
        f.write(np.asarray(box, np.float32).tobytes())
        f.write(np.asarray(roi, np.float32).tobytes())
        f.write(np.ascontiguousarray(pos, np.float32).tobytes())
    r = subprocess.run([exe, str(src), str(dst)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    b = dst.read_bytes()
    nn = struct.unpack_from("<i", b, 0)[0]
    node = np.dtype([("min", "<f4", 3), ("ext", "<f4"), ("level", "<i4"), ("parent", "<i4"),
                     ("first_child", "<i4"), ("estimate", "<u8")])
    o = 4
    nodes = np.frombuffer(b, node, nn, o)
    o += nn * node.itemsize
    nl = struct.unpack_from("<i", b, o)[0]
    o += 4
    leaves = np.frombuffer(b, "<i4", nl, o)
    o += 4 * nl
    off = np.frombuffer(b, "<i8", nl + 1, o)
    o += 8 * (nl + 1)
    ids = np.frombuffer(b, "<u8", int(off[-1]), o)
    return nodes, leaves, off, ids


def test_host_octree_matches_reference_golden(tmp_path):
    g = load_golden("octree.npz")
    n = int(g["n"])
    exe = _build(tmp_path)
    nodes, leaves, off, ids = _run(exe, tmp_path, g["positions"], n, g["box"], g["roi"], int(g["max_tets"]),
                                   int(g["max_level"]))
    assert len(nodes) == len(g["node_f"])
    assert np.array_equal(np.stack([nodes["min"][:, 0], nodes["min"][:, 1], nodes["min"][:, 2], nodes["ext"]], 1),
                          g["node_f"])
    assert np.array_equal(nodes["level"], g["node_i"][:, 0])
    assert np.array_equal(nodes["parent"], g["node_i"][:, 1])
    assert np.array_equal(nodes["first_child"], g["node_i"][:, 2])
    assert np.array_equal(nodes["estimate"], g["node_est"])
    assert np.array_equal(leaves, g["leaf_ids"])
    assert np.array_equal(off, g["leaf_meta_off"])
    assert np.array_equal(ids, g["leaf_meta_ids"])
