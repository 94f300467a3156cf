"""The no-allocation entry point, adeco_deposit_tets_device_noalloc.

It serves callers that cannot allocate device memory when they call the
deposit (code recorded into someone else's CUDA graph, hosts that forbid
cudaMalloc after start-up, applications whose device memory belongs to their
own pool): its scratch is a fixed device array compiled into the library.
This test calls it through the C ABI and checks its output against the
allocating entry point adeco_deposit_tets_device on the same inputs, within
the per-cell tolerance of the parity tests, on two calls in a row (the shared
scratch must not leak one call's sums into the next).  Its name makes pytest
collect it last.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu

REL, ABS = 1e-5, 1e-7


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from adeco_gb300 import _lib, build
    build.build()
    return torch, _lib.load()


def _call(fn, torch, d_pos, g, m, dims, patch_offset, num_patches, out):
    bbox = np.ascontiguousarray(g["bbox"], dtype=np.float32)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    args = [C.c_void_p(d_pos.data_ptr()), d_pos.numel(), patch_offset, num_patches, m,
            C.c_void_p(bbox.ctypes.data), dims, C.c_void_p(out.data_ptr())]
    if fn.__name__.endswith("noalloc"):
        return fn(*args, 0, 1.0, stream)
    return fn(*args, 0, 0, 1.0, stream)  # mixed precision, reference tet order


def test_noalloc_matches_allocating_entry_point_twice(env):
    torch, lib = env
    g = load_golden("patches_padded.npz")
    m, dims = int(g["m"]), int(g["dims"])
    p0, npat = int(g["patch_offset"]), int(g["num_patches"])
    d_pos = torch.from_numpy(np.ascontiguousarray(g["positions"], dtype=np.float32)).cuda()
    ref = torch.zeros(dims ** 3, dtype=torch.float64, device="cuda")
    assert _call(lib.adeco_deposit_tets_device, torch, d_pos, g, m, dims, p0, npat, ref) == 0, \
        lib.adeco_last_error()
    want = ref.cpu().numpy()
    assert want.sum() > 0
    for _ in range(2):
        out = torch.zeros(dims ** 3, dtype=torch.float64, device="cuda")
        rc = _call(lib.adeco_deposit_tets_device_noalloc, torch, d_pos, g, m, dims, p0, npat, out)
        assert rc == 0, lib.adeco_last_error()
        got = out.cpu().numpy()
        assert np.all(np.abs(got - want) <= REL * np.abs(want) + ABS)


def test_noalloc_rejects_sizes_beyond_its_scratch(env):
    torch, lib = env
    g = load_golden("patches_padded.npz")
    m = int(g["m"])
    d_pos = torch.from_numpy(np.ascontiguousarray(g["positions"], dtype=np.float32)).cuda()
    big = 97  # 97^3 cells > the 96^3 the fixed scratch holds
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    rc = _call(lib.adeco_deposit_tets_device_noalloc, torch, d_pos, g, m, big, 0, 1, out)
    assert rc == 9  # ADECO_ERR_LIMIT
    assert b"96" in lib.adeco_last_error()
