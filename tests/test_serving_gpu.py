"""GPU tests of continuous batching (zoom requests over a resident lattice)
and of the failure paths a caller sees: admission refusal, queueing inside
the library, a full route list, a bounded wait that runs out, tuning
parameters.

A request's masses are exact 64-bit fixed-point sums, so they are the same
bit for bit alone, in a batch, and while other batches run.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL, ABS = 1e-5, 1e-7
ERR_MEMORY, ERR_LIMIT, ERR_CUDA = 5, 9, 4


@pytest.fixture(scope="module")
def adeco():
    from adeco_gb300 import build, deposit
    build.build()
    return deposit


@pytest.fixture(scope="module")
def lattice64():
    from adeco_gb300.synthetic import zeldovich_lattice
    return zeldovich_lattice(64, L=100.0, seed=3, rms_disp=3.0)


def test_submit_while_another_batch_runs(adeco, lattice64):
    """A small batch submitted while a large one is on the GPU is admitted at
    once (both run together) and gives the same masses, bit for bit, as the
    same request inside the large batch."""
    small = ((47.0, 52.0, 49.0), 5.0, 64)
    big = [((50.0 + 3 * k, 50.0, 50.0), 40.0, 128) for k in range(7)] + [small]
    with adeco.Session(lattice64) as s:
        warm = s.submit([small])
        s.release(warm)
        a = s.submit(big)
        b = s.submit([small])
        a_done_at_b = s.poll(a)
        s.wait(b)
        s.wait(a)
        st = s.serving_stats()
        assert not a_done_at_b, "the large batch finished before the small one was submitted"
        assert st["max_running"] >= 2, st
        assert np.array_equal(s.result(b, 0, 64), s.result(a, len(big) - 1, 64))
        s.release(a)
        s.release(b)


def test_batches_queue_inside_the_library(adeco, lattice64):
    """With an admission budget that holds one batch at a time, later batches
    wait inside the library (no ERR_MEMORY) and each gives its alone result."""
    torch = pytest.importorskip("torch")
    reqs = [((30.0 + 10 * k, 40.0, 60.0), 12.0, 96) for k in range(4)]
    with adeco.Session(lattice64) as s:
        alone = []
        for r in reqs:
            b = s.submit([r])
            alone.append(s.result(b, 0, 96))
            s.release(b)
    import re
    with adeco.Session(lattice64, hbm_fraction=1e-9) as s:  # the library states what one batch needs
        with pytest.raises(adeco.AdecoError) as e:
            s.submit([reqs[0]])
        one = int(re.search(r"needs (\d+) bytes", str(e.value)).group(1))
    free, _ = torch.cuda.mem_get_info()
    with adeco.Session(lattice64, hbm_fraction=1.5 * one / free) as s:
        ids = [s.submit([r]) for r in reqs]
        for b, want in zip(ids, alone):
            assert np.array_equal(s.result(b, 0, 96), want)
            s.release(b)
        st = s.serving_stats()
        assert st["max_running"] == 1, st
        assert st["admission_waits"] > 0, st
        assert st["completed"] == len(reqs)


def test_admission_refuses_a_batch_beyond_the_budget(adeco, lattice64):
    with adeco.Session(lattice64, hbm_fraction=1e-9) as s:
        with pytest.raises(adeco.AdecoError) as e:
            s.submit([((50.0, 50.0, 50.0), 10.0, 64)])
        assert e.value.code == ERR_MEMORY


def test_full_route_list_is_reported(adeco):
    """A route list too small for the ill-conditioned tets of a clustered
    lattice: the deposit reports ADECO_ERR_LIMIT instead of a silent loss."""
    from adeco_gb300.synthetic import zeldovich_lattice
    pos = zeldovich_lattice(32, L=100.0, seed=4, rms_disp=3.0, infall=20)
    with adeco.Session(pos) as s:
        s.build_octree(20000, 8, leaf_dims=8)
        _, t = s.deposit_leaves()
        assert t["routed_tets"] > 1
        s.set_tuning(route_capacity=1)
        with pytest.raises(adeco.AdecoError) as e:
            s.deposit_leaves()
        assert e.value.code == ERR_LIMIT and "route list" in str(e.value)
        b = s.submit([((50.0, 50.0, 50.0), 60.0, 48)])
        with pytest.raises(adeco.AdecoError) as e:
            s.result(b, 0, 48)
        assert e.value.code == ERR_LIMIT
        s.release(b)
        s.set_tuning(route_capacity=0)
        s.deposit_leaves()


def test_bounded_wait_runs_out_and_reports(adeco):
    """The bounded wait of the deposit kernels, on a count nothing lowers,
    gives up after its limit and reports error bit 3 as ADECO_ERR_CUDA; the
    context stays usable."""
    from adeco_gb300 import _lib
    lib = _lib.load()
    rc = lib.adeco_debug_bounded_wait(4096)
    assert rc == ERR_CUDA
    assert b"timed out" in lib.adeco_last_error()
    from adeco_gb300.synthetic import zeldovich_lattice
    pos = zeldovich_lattice(10, L=10.0, seed=1, rms_disp=0.5)
    p = pos.reshape(-1, 3)
    lo, hi = float(p.min()) - 1.0, float(p.max()) + 1.0  # every tet inside the grid box
    grid = adeco.deposit_tets_ex(pos.reshape(-1), 9, np.array([lo, hi, lo, hi, lo, hi], np.float32), 8)
    assert abs(grid.sum() - 6 * 9 ** 3) <= 1e-6 * 6 * 9 ** 3


def test_tuning_parameters(adeco, oracle, lattice64):
    """Parameters that only change scheduling leave every mass bit-identical;
    a different zoom tile moves the frames the pairs are clipped in, so the
    masses stay within the per-cell bar of the FP64 oracle."""
    pos = lattice64
    n = pos.shape[0]
    reqs = [((40.0, 55.0, 50.0), 9.0, 80), ((60.0, 40.0, 45.0), 30.0, 40)]
    with adeco.Session(pos) as s:
        s.build_octree(262144 // 8, 8, leaf_dims=16)
        leaves0, _ = s.deposit_leaves()
        b = s.submit(reqs)
        zoom0 = [s.result(b, k, r[2]) for k, r in enumerate(reqs)]
        s.release(b)
        t0 = s.get_tuning()
        assert (t0["zoom_tile"], t0["share_chunk"], t0["clip_batch"]) == (64, 512, 128)
        s.set_tuning(clip_batch=64, ctas_per_sm=1, share_chunk=128)
        leaves1, _ = s.deposit_leaves()
        assert np.array_equal(leaves0, leaves1)
        b = s.submit(reqs)
        assert all(np.array_equal(s.result(b, k, r[2]), zoom0[k]) for k, r in enumerate(reqs))
        s.release(b)
        s.set_tuning(zoom_tile=32)
        b = s.submit(reqs)
        flat = np.ascontiguousarray(pos.reshape(-1))
        cd = -(-(n - 1) // 7)
        ids = np.arange(cd ** 3, dtype=np.uint64)
        for k, (c, side, d) in enumerate(reqs):
            got = s.result(b, k, d).reshape(-1)
            h = np.float32(0.5) * np.float32(side)
            box = np.array([np.float32(c[0]) - h, np.float32(c[0]) + h, np.float32(c[1]) - h, np.float32(c[1]) + h,
                            np.float32(c[2]) - h, np.float32(c[2]) + h], np.float32)
            ref = oracle.deposit_meta(flat, (n, n, n), ids, box, d, fp64=True)
            assert np.all(np.abs(got - ref) <= REL * np.abs(ref) + ABS)
        s.release(b)
        with pytest.raises(adeco.AdecoError):
            s.set_tuning(zoom_tile=8)
