"""The no-allocation entry point, adeco_deposit_tets_device_noalloc.

It serves callers that must not allocate device memory while they deposit:
an application that gives all of the GPU's memory to its own pool at
start-up, or a latency-critical loop where cudaMalloc's unbounded time and
cudaFree's device-wide synchronisation are not allowed.  Its scratch is a
fixed device array compiled into the library.  These tests call it through
the C ABI and check its output against the allocating entry point
adeco_deposit_tets_device on the same inputs, within the per-cell tolerance
of the parity tests, on two calls in a row (the shared scratch must not
leak one call's sums into the next); on the golden patch fixture also
against the FP64 oracle, and on a seeded Zel'dovich patch set at its item
limit.  Its name makes pytest collect it last.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu

REL, ABS = 1e-5, 1e-7
ERR_LIMIT = 9
MAX_ITEMS = 4096  # the entry point's limit on patch sub-blocks per call


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from adeco_gb300 import _lib, build
    build.build()
    return torch, _lib.load()


def _call(fn, torch, d_pos, bbox, m, dims, patch_offset, num_patches, out):
    bbox = np.ascontiguousarray(bbox, dtype=np.float32)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    args = [C.c_void_p(d_pos.data_ptr()), d_pos.numel(), patch_offset, num_patches, m,
            C.c_void_p(bbox.ctypes.data), dims, C.c_void_p(out.data_ptr())]
    if fn.__name__.endswith("noalloc"):
        return fn(*args, 0, 1.0, stream)  # no precision argument: always the mixed path
    return fn(*args, 0, 0, 1.0, stream)  # mixed precision, reference tet order


def _both(torch, lib, d_pos, bbox, m, dims, p0, npat):
    """The allocating entry point's grid, then two no-alloc grids in a row."""
    ref = torch.zeros(dims ** 3, dtype=torch.float64, device="cuda")
    assert _call(lib.adeco_deposit_tets_device, torch, d_pos, bbox, m, dims, p0, npat, ref) == 0, \
        lib.adeco_last_error()
    want = ref.cpu().numpy()
    got = []
    for _ in range(2):
        out = torch.zeros(dims ** 3, dtype=torch.float64, device="cuda")
        rc = _call(lib.adeco_deposit_tets_device_noalloc, torch, d_pos, bbox, m, dims, p0, npat, out)
        assert rc == 0, lib.adeco_last_error()
        got.append(out.cpu().numpy())
    return want, got


def test_noalloc_matches_allocating_entry_point_twice(env, oracle):
    torch, lib = env
    g = load_golden("patches_padded.npz")
    m, dims = int(g["m"]), int(g["dims"])
    p0, npat = int(g["patch_offset"]), int(g["num_patches"])
    d_pos = torch.from_numpy(np.ascontiguousarray(g["positions"], dtype=np.float32)).cuda()
    want, got = _both(torch, lib, d_pos, g["bbox"], m, dims, p0, npat)
    assert want.sum() > 0
    fp64 = oracle.deposit_patches(g["positions"], m, g["bbox"], dims, fp64=True, patch_offset=p0,
                                  num_patches=npat)
    for grid in got:
        assert np.all(np.abs(grid - want) <= REL * np.abs(want) + ABS)
        assert np.all(np.abs(grid - fp64) <= REL * np.abs(fp64) + ABS)


def _patch_set(n_side, seed, disp):
    """n_side^3 patches of 7^3 cubes (8^3 vertices each, neighbours sharing a
    plane) cut from one seeded Zel'dovich lattice, x fastest."""
    from adeco_gb300.synthetic import zeldovich_lattice
    n = 7 * n_side + 1
    pos = zeldovich_lattice(n, L=100.0, seed=seed, rms_disp=disp)
    patches = np.empty((n_side, n_side, n_side, 8, 8, 8, 3), np.float32)
    for pz in range(n_side):
        for py in range(n_side):
            for px in range(n_side):
                patches[pz, py, px] = pos[7 * pz:7 * pz + 8, 7 * py:7 * py + 8, 7 * px:7 * px + 8]
    flat = patches.reshape(-1)
    p = pos.reshape(-1, 3)
    lo, hi = p.min(0) + 5.0, p.max(0) - 5.0
    bbox = np.array([lo[0], hi[0], lo[1], hi[1], lo[2], hi[2]], np.float32)
    return flat, bbox


def test_noalloc_at_its_item_limit(env):
    """4096 patches of 7^3 cubes (8.4M tets, the item limit) into 96^3 cells."""
    torch, lib = env
    flat, bbox = _patch_set(16, seed=21, disp=3.0)
    d_pos = torch.from_numpy(flat).cuda()
    want, got = _both(torch, lib, d_pos, bbox, 7, 96, 0, MAX_ITEMS)
    assert want.sum() > 1e6
    for grid in got:
        assert np.all(np.abs(grid - want) <= REL * np.abs(want) + ABS)
    # one sub-block more than the scratch holds
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    flat2 = np.concatenate([flat, flat[:3 * 512]])
    d_pos2 = torch.from_numpy(flat2).cuda()
    rc = _call(lib.adeco_deposit_tets_device_noalloc, torch, d_pos2, bbox, 7, 96, 0, MAX_ITEMS + 1, out)
    assert rc == ERR_LIMIT
    assert b"4096" in lib.adeco_last_error()


def test_noalloc_rejects_grids_beyond_its_scratch(env):
    torch, lib = env
    g = load_golden("patches_padded.npz")
    m = int(g["m"])
    d_pos = torch.from_numpy(np.ascontiguousarray(g["positions"], dtype=np.float32)).cuda()
    big = 97  # 97^3 cells > the 96^3 the fixed scratch holds
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    rc = _call(lib.adeco_deposit_tets_device_noalloc, torch, d_pos, g["bbox"], m, big, 0, 1, out)
    assert rc == ERR_LIMIT
    assert b"96" in lib.adeco_last_error()
