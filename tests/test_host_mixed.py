"""CPU checks of the mixed path's per-pair arithmetic against FP64 clipping,
compiled for the host from the CUDA headers (no GPU): setup_tet,
classify_pair, the one-face closed form and the clip engine's steps in the
cell frames the GPU engine uses, on seeded lattice-like tets; and the
barycentric clipping of flat tets (thickness 1e-2 .. 1e-4 of their extent)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def _run_check(tmp_path, name):
    nvcc = next((c for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc")
                 if c and os.path.exists(c)), None)
    if nvcc is None:
        pytest.skip("nvcc not available")
    exe = str(tmp_path / name)
    r = subprocess.run([nvcc, "-std=c++17", "-O2", "-Xcompiler", "-ffp-contract=off", "-o", exe,
                        os.path.join(HERE, name + ".cu")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr


def test_host_mixed_pairs_vs_fp64(tmp_path):
    _run_check(tmp_path, "host_mixed_check")


def test_host_barycentric_flat_tets_vs_fp64(tmp_path):
    _run_check(tmp_path, "host_bary_check")
