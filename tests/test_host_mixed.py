"""CPU check of the mixed path's per-pair arithmetic (setup_tet,
classify_pair, the one-face closed form, the clip engine's steps in the cell
frames the GPU engine uses) against FP64 clipping, on seeded random
lattice-like tets; compiled for the host from the CUDA headers, no GPU."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_host_mixed_pairs_vs_fp64(tmp_path):
    nvcc = next((c for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc")
                 if c and os.path.exists(c)), None)
    if nvcc is None:
        pytest.skip("nvcc not available")
    exe = str(tmp_path / "host_mixed_check")
    r = subprocess.run([nvcc, "-std=c++17", "-O2", "-Xcompiler", "-ffp-contract=off", "-o", exe,
                        os.path.join(HERE, "host_mixed_check.cu")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
