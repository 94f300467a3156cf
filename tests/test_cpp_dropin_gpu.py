"""The C++ drop-in on the GPU: a C++ caller written against ADECO's
DepositWrapper::deposit_tets (src/AdDeposit2Grid.h:82-91), compiled with
include/adeco_deposit_wrapper.hpp in place of AdDeposit2Grid.h and linked
against libadeco_gb300.so -- what an ADECO build switched to this library
does.  It deposits a reference-made golden lattice twice into one float grid
(the call accumulates) and calls once with a device id that does not exist,
which must throw AdRuntimeException as the reference does."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, load_golden

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CALLER = r'''
#include <cstdio>
#include <cstdlib>
#include <vector>
#include "adeco_deposit_wrapper.hpp"

using AdaptiveMassDeposit::AdRuntimeException;
using AdaptiveMassDeposit::DepositWrapper;

static std::vector<char> slurp(const char *path)
{
    std::vector<char> b;
    FILE *f = std::fopen(path, "rb");
    if (!f) return b;
    std::fseek(f, 0, SEEK_END);
    b.resize((size_t)std::ftell(f));
    std::fseek(f, 0, SEEK_SET);
    if (std::fread(b.data(), 1, b.size(), f) != b.size()) b.clear();
    std::fclose(f);
    return b;
}

int main(int argc, char **argv)
{
    if (argc != 6) return 2;
    const int m = std::atoi(argv[3]), dims = std::atoi(argv[4]);
    std::vector<char> pos = slurp(argv[1]), box = slurp(argv[2]);
    const float *p = reinterpret_cast<const float *>(pos.data());
    const size_t n = pos.size() / sizeof(float);
    const size_t fpp = 3 * (size_t)(m + 1) * (m + 1) * (m + 1);
    std::vector<DepositWrapper::h_grid_mass_type> grid((size_t)dims * dims * dims, 0.f);
    for (int k = 0; k < 2; ++k)
        DepositWrapper::deposit_tets(false, 0, 0, n / fpp, p, n, m, reinterpret_cast<const float *>(box.data()), dims,
                                     grid.data());
    int threw = 0;
    try {
        DepositWrapper::deposit_tets(true, 999, 0, n / fpp, p, n, m, reinterpret_cast<const float *>(box.data()), dims,
                                     grid.data());
    } catch (const AdRuntimeException &e) {
        threw = 1;
        std::printf("threw: %s\n", e.what());
    }
    FILE *f = std::fopen(argv[5], "wb");
    std::fwrite(grid.data(), sizeof(float), grid.size(), f);
    std::fclose(f);
    return threw ? 0 : 3;
}
'''


def test_cpp_caller_through_the_wrapper(tmp_path):
    from adeco_gb300 import build
    lib = build.build()
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    src = tmp_path / "caller.cpp"
    src.write_text(CALLER)
    exe = tmp_path / "caller"
    libdir = os.path.dirname(lib)
    r = subprocess.run([gxx, "-std=c++11", "-O1", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe),
                        "-L", libdir, "-ladeco_gb300", f"-Wl,-rpath,{libdir}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    g = load_golden("lattice_lat12_d3.npz")
    m, dims = int(g["m"]), int(g["dims"])
    np.ascontiguousarray(g["positions"], np.float32).tofile(tmp_path / "pos.bin")
    np.ascontiguousarray(g["bbox"], np.float32).tofile(tmp_path / "box.bin")
    out = tmp_path / "grid.bin"
    r = subprocess.run([str(exe), str(tmp_path / "pos.bin"), str(tmp_path / "box.bin"), str(m), str(dims), str(out)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "threw" in r.stdout
    got = np.fromfile(out, np.float32).astype(np.float64)
    want = 2.0 * g["grid_f64"]  # the reference's FP64 instantiation of the same call, accumulated twice
    assert np.all(np.abs(got - want) <= 1e-5 * np.abs(want) + 2e-7), float(np.abs(got - want).max())
    assert os.path.exists(os.path.join(GOLDEN, "lattice_lat12_d3.npz"))
