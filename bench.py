#!/usr/bin/env python3
"""Benchmark: phase-space tetrahedron mass deposit on one GB300.

Workload (one step): the octree deposit of a 256^3-particle Zel'dovich
lattice -- RMS displacement 3 lattice spacings, seed 0, box L = 100 --
into an adaptive octree (max depth 8, 16^3-cell leaf blocks, refine while a
node's tet estimate exceeds 64 * 16^3 = 262144), every leaf deposited.
  value  : distinct tets / s of the batched persistent mixed-precision
           deposit (one CUDA-graph replay per step, lattice resident in HBM)
  e2e    : the same tets / s through the public C ABI with host buffers:
           session create (H2D of the positions from pinned memory), octree,
           deposit, D2H of every leaf grid, destroy -- per step
  plain  : the one-request-per-launch FP64 deposit (one launch per leaf)
Multi-GPU: the deposit does not exchange data between GPUs ("replicas
only"): each rank deposits its own replica, value = all ranks' tets / max
time.

--impl reference times the reference algorithm's CPU deposit (the oracle
restatement, FP32, all host threads) on a bounded sample of the same leaves
per step, and extrapolates to the whole workload.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import re
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_PART = 256
L_BOX = 100.0
RMS_DISP = 3.0
SEED = 0
INFALL = 0
MAX_TETS = 64 * 16 ** 3
MAX_LEVEL = 8
LEAF = 16
WORKLOAD = ("octree deposit of a 256^3 Zel'dovich lattice (rms disp 3 spacings, seed 0, L=100; the reference's "
            "non-periodic cube set, 255^3 cubes = 99,488,250 tets): depth <= 8, 16^3-cell leaves, refine while tet "
            "estimate > 262144 (64 per cell)")
ZOOM_COUNT, ZOOM_SEED = 512, 1
SERVE_SEED = 2


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    """Barrier / max / sum over ranks (torch.distributed) for N > 1: NCCL on the
    GPUs, or gloo with CPU tensors (the multi-rank logic tested without a GPU).
    Collectives and the rendezvous give up after `timeout_s` (default from
    ADECO_PG_TIMEOUT_S, else 600 s), so a rank that never joins ends the others'
    wait with an error instead of a hang."""

    def __init__(self, ws, local, backend="nccl", timeout_s=None):
        self.ws = ws
        self.pg = None
        if ws > 1:
            import datetime

            import torch
            import torch.distributed as dist
            if backend == "nccl":
                torch.cuda.set_device(local)
            if timeout_s is None:
                timeout_s = float(os.environ.get("ADECO_PG_TIMEOUT_S", "600"))
            dist.init_process_group(backend, timeout=datetime.timedelta(seconds=timeout_s))
            self.torch, self.dist = torch, dist
            self.device = "cuda" if backend == "nccl" else "cpu"

    def agree(self, ok):
        """True when every rank reports ok.  A rank whose host work failed
        reports False before it leaves; a rank that died, or never reaches this
        point within the timeout, makes the collective fail, which counts as
        False here."""
        if self.ws == 1:
            return bool(ok)
        try:
            return self._reduce(1.0 if ok else 0.0, self.dist.ReduceOp.MIN) == 1.0
        except Exception:  # noqa: BLE001 -- a peer that is gone or timed out
            return False

    def barrier(self):
        if self.ws > 1:
            self.dist.barrier()

    def _reduce(self, x, op):
        t = self.torch.tensor([x], dtype=self.torch.float64, device=self.device)
        self.dist.all_reduce(t, op=op)
        return float(t.item())

    def max(self, x):
        return x if self.ws == 1 else self._reduce(x, self.dist.ReduceOp.MAX)

    def sum(self, x):
        return x if self.ws == 1 else self._reduce(x, self.dist.ReduceOp.SUM)

    def close(self):
        if self.ws > 1:
            self.dist.destroy_process_group()


class RankFailure(RuntimeError):
    """Another rank failed before the timed region; no number is reported."""


def gated(dist, fn, what):
    """Runs this rank's untimed work fn(), then has all ranks agree that each
    got through its own before any rank enters the timed region (a rank leaves
    only here, between steps, with no kernel or collective of its own in
    flight).  The failing rank re-raises its own error; the others raise
    RankFailure."""
    try:
        r = fn()
    except BaseException:
        dist.agree(False)
        raise
    if not dist.agree(True):
        raise RankFailure(f"another rank failed during {what}; no number is reported")
    return r


def replica_value(dist, tets, ms):
    """Whole-job throughput of N replicas: all ranks' tets over the slowest
    rank's time.  Returns (tets/s, max ms)."""
    ms_max = dist.max(ms)
    return dist.sum(float(tets)) / (ms_max * 1e-3), ms_max


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-i", str(self.gpu), "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def workload_positions():
    from adeco_gb300.synthetic import zeldovich_lattice
    return zeldovich_lattice(N_PART, L=L_BOX, seed=SEED, rms_disp=RMS_DISP, infall=INFALL)


def set_size(n):
    """Lattice size (256 for the benchmark; smaller only for checking this script)."""
    global N_PART
    N_PART = n


def set_workload(name):
    """c2: the benchmark (256^3 octree deposit).  c4: 512^3 lattice with 2000
    infall regions (seed 4), octree depth <= 12.  c1: 64^3 periodic lattice
    onto a uniform 128^3 grid through the reference boundary.  zoom and serve
    run on the c2 lattice; c5 serves zoom requests of 32^3 to 512^3 cells
    against the resident c4 lattice."""
    global N_PART, SEED, INFALL, MAX_LEVEL, WORKLOAD, RMS_DISP
    if name == "c1":
        N_PART, SEED, RMS_DISP = 64, 0, 0.5
        WORKLOAD = ("periodic 64^3 Zel'dovich lattice (rms disp 0.5 spacings, seed 0, L=100; 64^3 cubes = 1,572,864 "
                    "tets from ghost planes shifted by +L, 64 patches of 16^3 cubes) onto a uniform 128^3 grid over "
                    "the box through the reference boundary; periodic wrap = sum over the box's 27 images")
    if name in ("c4", "c5"):
        N_PART, SEED, INFALL, MAX_LEVEL = 512, 4, 2000, 12
        WORKLOAD = ("octree deposit of a 512^3 Zel'dovich lattice with 2000 infall regions (rms disp 3 spacings, "
                    "seed 4, L=100): depth <= 12, 16^3-cell leaves, refine while tet estimate > 262144")


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def profile_figure(name):
    """A per-launch figure of the deposit kernel (`name: value`) from the
    committed ncu summary: dram_bytes_per_launch_full_workload (DRAM read +
    write), fp32_flops_per_launch_full_workload (executed FADD + FMUL + 2 FFMA)."""
    path = os.path.join(ROOT, "profiles", "deposit_mixed_kernel_c2.md")
    try:
        text = open(path).read()
    except OSError:
        return None
    m = re.search(name + r":\s*([0-9.eE+]+)", text)
    return float(m.group(1)) if m else None


# --------------------------------------------------------------- CPU side
def oracle_sample(pos, n, leaves_budget_s, threads, nodes, off, ids, leaves, seed_leaf=0):
    """Deposit a spread sample of leaves with the oracle (FP32, the reference's
    precision) on `threads` host threads; returns (seconds, meta-tets done)."""
    from concurrent.futures import ThreadPoolExecutor

    from oracle import oracle as O
    flat = np.ascontiguousarray(pos.reshape(-1))
    nl = len(leaves)

    def leaf_box(L):
        nd = nodes[L]
        return np.array([nd["min"][0], nd["min"][0] + nd["ext"], nd["min"][1], nd["min"][1] + nd["ext"],
                         nd["min"][2], nd["min"][2] + nd["ext"]], np.float32)

    def work(q):
        L = leaves[q]
        mids = ids[off[L]:off[L + 1]]
        O.deposit_meta(flat, (n, n, n), mids, leaf_box(L), LEAF, fp64=False)
        return len(mids)

    # calibrate on one leaf, then run a spread sample sized to the budget
    t0 = time.perf_counter()
    m0 = work(seed_leaf % nl)
    t1 = time.perf_counter() - t0
    per_mc = t1 / max(1, m0)
    target_mc = int(leaves_budget_s * threads / max(per_mc, 1e-9))
    order = [(seed_leaf + 1 + k * 7919) % nl for k in range(nl)]
    chosen, acc = [], 0
    for q in order:
        if acc >= target_mc:
            break
        if q in chosen:
            continue
        chosen.append(q)
        acc += int(off[leaves[q] + 1] - off[leaves[q]])
    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=threads) as ex:
        done = sum(ex.map(work, chosen))
    return time.perf_counter() - t0, done, len(chosen)


def cpu_tree(pos, n):
    from oracle import oracle as O
    p = pos.reshape(-1, 3)
    box = np.array([*p.min(0), *p.max(0)], np.float32)
    roi = np.array([1, 1, 1, 0, 0, 0], np.float32)
    max_tets = min(6 * (n - 1) ** 3, MAX_TETS)
    return O.generate_tree(np.ascontiguousarray(pos.reshape(-1)), (n, n, n), box, roi, max_tets, MAX_LEVEL)


def run_reference(args, rank, ws):
    """--impl reference: the reference algorithm on the host cores."""
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    pos = workload_positions()
    n = N_PART
    nodes, off, ids, leaves = cpu_tree(pos, n)
    total_mc = int(sum(off[L + 1] - off[L] for L in leaves))
    tets = 6 * (n - 1) ** 3
    vals, times = [], []
    for step in range(args.warmup + args.steps):
        sec, mc, nleaf = oracle_sample(pos, n, args.ref_step_s, threads, nodes, off, ids, leaves, seed_leaf=step)
        full = sec * total_mc / max(1, mc)           # extrapolated time of the whole workload
        if step >= args.warmup:
            vals.append(tets / full)
            times.append(full * 1e3)
    value = statistics.median(vals)
    line = {
        "impl": "reference", "metric": "tets/s deposited", "value": value, "unit": "tets/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": statistics.median(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "tets": tets, "leaves": len(leaves)},
        "cpu_baseline": {"value": value, "unit": "tets/s", "cores": threads, "kind": "port",
                         "sample": f"each step: a spread sample of octree leaves sized to ~{args.ref_step_s:.0f} s "
                                   f"on {threads} threads (FP32 oracle restatement of the reference deposit), "
                                   f"extrapolated by meta-cell count to all {len(leaves)} leaves"},
        "e2e": {"value": value, "unit": "tets/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# --------------------------------------------------------------- GPU side
def algorithmic_flops(pos, n, nodes, off, ids, leaves, sample_leaves=3):
    """Reference-algorithm FLOPs per meta-cell tet, counted by the instrumented
    oracle on a spread sample of leaves (single thread)."""
    from oracle import oracle as O
    L_ = O.lib()
    flat = np.ascontiguousarray(pos.reshape(-1))
    flops, mcs = 0, 0
    for k in range(sample_leaves):
        L = leaves[(k * len(leaves)) // sample_leaves]
        nd = nodes[L]
        bb = np.array([nd["min"][0], nd["min"][0] + nd["ext"], nd["min"][1], nd["min"][1] + nd["ext"],
                       nd["min"][2], nd["min"][2] + nd["ext"]], np.float32)
        mids = ids[off[L]:off[L + 1]]
        L_.ora_flops_reset()
        O.deposit_meta(flat, (n, n, n), mids, bb, LEAF, fp64=False)
        flops += L_.ora_flops_get()
        mcs += len(mids)
    return flops / max(1, mcs)


def run_ours(args, rank, ws, local):
    from adeco_gb300 import _lib as LB
    from adeco_gb300 import deposit as D
    dist = Dist(ws, local)
    lib = LB.load(build_if_missing=True)
    pos = workload_positions()
    n = N_PART
    tets = 6 * (n - 1) ** 3
    out = {}
    with D.Session(pos, device=local if ws > 1 else args.device) as s:
        def setup():
            info = s.build_octree(MAX_TETS, MAX_LEVEL, leaf_dims=LEAF)
            out["gpu_tree"] = (info, [s.leaf_meta(q) for q in range(len(info.leaves))])
            # launch shape and staging depth: picked by the autotuner for this GPU and workload
            if not args.no_tune:
                from adeco_gb300 import tune
                params, tinfo = tune.tune_leaves(s, WORKLOAD, device=local if ws > 1 else args.device,
                                                 force=args.retune)
                out["tuning"] = {"leaf": params, **{k: v for k, v in tinfo.items() if k != "key"}}
            else:
                out["tuning"] = {"leaf": s.get_tuning(), "source": "defaults"}
            # one untimed pass with the pair counters on
            grids, st = s.deposit_leaves(stats=True)
            for _ in range(args.warmup):
                s.replay_leaves(1)
            kern = [s.deposit_leaves(fetch=False)[1]["kernel_ms"] for _ in range(2)]
            return info, grids, st, kern

        info, grids, st, kern = gated(dist, setup, "the octree build and warm-up")
        nleaf = len(info.leaves)
        mixed_total = float(grids.sum())
        dist.barrier()
        with ClockSampler(local if ws > 1 else args.device) as clk:
            t = s.replay_leaves(args.steps)
        dist.barrier()
        out["value"], ms_step = replica_value(dist, tets, t["kernel_ms"])
        out["ms_per_step"] = ms_step
        out["clocks"] = clk.summary()
        out["kernel_ms"] = min(kern)
        out["stats"] = st
        out["nleaf"] = nleaf
        out["levels"] = info.levels
        # plain FP64, one launch per leaf
        plain = {}
        if not args.skip_plain:
            pg, pt = s.deposit_leaves(precision=1)
            plain = {"ms_per_step": pt["kernel_ms"], "tets_per_s": tets / (pt["kernel_ms"] * 1e-3),
                     "launches": pt["launches"], "steps": 1}
            d = np.abs(pg - grids)
            err = {}
            for th in (1.0, 1e-2, 1e-3):
                sel = pg > th
                err[f"max_rel_cells_gt_{th:g}"] = float((d[sel] / pg[sel]).max()) if sel.any() else 0.0
                err[f"cells_gt_{th:g}"] = int(sel.sum())
            err["max_abs_tet_masses"] = float(d.max())
            err["cells_nonzero"] = int((pg > 0).sum())
            err["bar_1e-5_rel_plus_1e-7_abs_ok"] = bool(np.all(d <= 1e-5 * pg + 1e-7))
            # smallest absolute floor (tet masses) with which every cell meets 1e-5 relative
            excess = (d - 1e-5 * pg).ravel()
            worst = int(np.argmax(excess))
            err["abs_floor_needed_tet_masses"] = float(max(excess[worst], 0.0))
            err["worst_cell"] = {"fp64": float(pg.flat[worst]), "abs_err": float(d.flat[worst])}
            for fl in (1e-7, 1e-6):
                err[f"cells_over_1e-5_rel_plus_{fl:g}"] = int((excess > fl).sum())
            plain["mixed_vs_fp64"] = err
            plain["total_mass_rel_diff"] = abs(mixed_total - float(pg.sum())) / float(pg.sum())
            del pg
        out["plain"] = plain
        out["mass"] = {"mixed_total": mixed_total, "tet_count": tets}
        leaf_values = grids.size
        out["grids"] = grids
        # octree generation: the device builder against the host one (same tree)
        tree_ms = {}
        for builder in ("host", "device"):
            ts = []
            for _ in range(4):
                t0 = time.perf_counter()
                tinfo = s.build_octree(MAX_TETS, MAX_LEVEL, leaf_dims=LEAF, builder=builder)
                ts.append((time.perf_counter() - t0) * 1e3)
            tree_ms[builder] = statistics.median(ts[1:])
            tree_ms[builder + "_nodes"] = tinfo.nodes.copy()
        tree_ms["same_tree"] = bool(np.array_equal(tree_ms.pop("host_nodes"), tree_ms.pop("device_nodes")))
        out["octree_build_ms"] = tree_ms
    # e2e through the public C ABI with host buffers (pinned), per step
    e2e = None
    if not args.skip_e2e:
        import torch
        pin_pos = torch.empty(pos.size, dtype=torch.float32, pin_memory=True)
        pin_pos.numpy()[:] = pos.reshape(-1)
        pin_out = torch.empty(leaf_values, dtype=torch.float64, pin_memory=True)
        cfg = LB.SessionConfig(local if ws > 1 else args.device, 0, 1.0, 0.75, 1)
        tim = LB.Timing()
        e2e_times = []
        for step in range(args.e2e_warmup + args.e2e_steps):
            dist.barrier()
            t0 = time.perf_counter()
            h = C.c_void_p()
            LB.check(lib.adeco_session_create(C.byref(cfg), C.c_void_p(pin_pos.data_ptr()), n, n, n, C.byref(h)))
            LB.check(lib.adeco_session_build_octree(h, None, None, MAX_TETS, MAX_LEVEL, LEAF))
            LB.check(lib.adeco_session_deposit_leaves(h, 0, C.c_void_p(pin_out.data_ptr()), 0, C.byref(tim)))
            LB.check(lib.adeco_session_destroy(h))
            dt = time.perf_counter() - t0
            if step >= args.e2e_warmup:
                e2e_times.append(dist.max(dt))
        e2e_s = statistics.median(e2e_times)
        e2e = {"value": dist.sum(float(tets)) / e2e_s, "unit": "tets/s", "ms_per_step": e2e_s * 1e3,
               "h2d_bytes_per_step": int(pos.size * 4), "d2h_bytes_per_step": int(leaf_values * 8),
               "steps": args.e2e_steps, "warmup": args.e2e_warmup}
    dist.close()
    if rank != 0:
        return 0
    # the oracle's octree (generate_tree restated on the CPU) against the GPU's, node for node
    nodes, off, ids, leaves = cpu_tree(pos, n)
    g_info, g_metas = out.pop("gpu_tree")
    tree_same = same_tree(g_info, g_metas, nodes, off, ids, leaves)
    # per-cell parity of the timed path's grids against the FP64 oracle on a spread sample of leaves
    oracle_check = None if args.skip_oracle_check else oracle_leaf_check(pos, n, out["grids"], nodes, off, ids,
                                                                          leaves, args.oracle_leaves)
    del out["grids"]
    # roofline of the deposit kernel (FP32-pipe bound; HBM figure beside it)
    flops_per_mc = algorithmic_flops(pos, n, nodes, off, ids, leaves)
    total_mc = int(sum(off[L + 1] - off[L] for L in leaves))
    alg_flops = flops_per_mc * total_mc
    peak = C.c_double()
    LB.check(lib.adeco_probe_fp32_tflops(args.device, C.byref(peak)))
    k_s = out["kernel_ms"] * 1e-3
    achieved = alg_flops / k_s / 1e12
    alg_bytes = 12.0 * n ** 3 + 8.0 * out["nleaf"] * LEAF ** 3
    peaks = measured_peaks()
    hbm = peaks.get("hbm_gbs")
    # the committed ncu summary covers the default 256^3 workload only
    c2 = (N_PART, SEED, INFALL, MAX_LEVEL) == (256, 0, 0, 8)
    traffic = profile_figure("dram_bytes_per_launch_full_workload") if c2 else None
    exec_flops = profile_figure("fp32_flops_per_launch_full_workload") if c2 else None
    roof = {"bound": "fp32", "achieved": achieved, "peak": peak.value, "unit": "TFLOP/s", "frac": achieved / peak.value,
            "traffic": traffic, "peak_source": "measured FP32 FMA probe (adeco_probe_fp32_tflops) on this GPU",
            "flops_per_launch": alg_flops, "flops_model": "reference-algorithm FLOPs counted by the instrumented "
            "oracle on a spread sample of leaves, per meta-cell tet, x all leaves' meta-cell tets",
            "kernel_ms": out["kernel_ms"],
            # the FP32 operations the kernel executes (ncu, scaled to this workload) over the same time
            "executed_fp32": None if exec_flops is None else {
                "flops_per_launch": exec_flops, "achieved_tflops": exec_flops / k_s / 1e12,
                "frac": exec_flops / k_s / 1e12 / peak.value,
                "source": "ncu smsp__sass_thread_inst_executed_op_{fadd,fmul,ffma}_pred_on (FFMA x2), profiles/"},
            "hbm": {"achieved_gbs": alg_bytes / k_s / 1e9, "peak_gbs": hbm, "frac_of_measured":
                    (alg_bytes / k_s / 1e9 / hbm) if hbm else None, "algorithmic_bytes": alg_bytes}}
    # CPU baseline: the oracle (reference algorithm, FP32) on a bounded sample
    cpu = None
    if ws == 1 and not args.skip_cpu:
        threads = os.cpu_count() or 1
        sec, mc, nl = oracle_sample(pos, n, args.cpu_budget_s, threads, nodes, off, ids, leaves)
        full = sec * total_mc / max(1, mc)
        cpu = {"value": tets / full, "unit": "tets/s", "cores": threads, "kind": "port",
               "sample": f"{nl} of {len(leaves)} octree leaves ({mc} meta-cells, {sec:.1f} s on {threads} threads, "
                         f"FP32 oracle restatement of the reference deposit), extrapolated by meta-cell count"}
    st = out["stats"]
    line = {
        "metric": "tets/s deposited", "value": out["value"], "unit": "tets/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": out["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "tets": tets, "leaves": out["nleaf"], "octree_levels": out["levels"],
                   "precision": "FP32 clipping in mirrored cell frames (kappa>32 tets: barycentric, double-float shares); "
                                "FP64 near-degenerate classification and volume normalisers; "
                                "64-bit fixed-point accumulation",
                   "l2": f"inputs larger than L2 ({16 * n ** 3 / 1e6:.0f} MB float4 lattice); no flush", "cuda_graph": True,
                   "parallelism": "replicas" if ws > 1 else "single GPU"},
        "roofline": roof,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": 3 * args.steps,  # per step: deposit, ill-conditioned tets, fixed point -> FP64
        "clocks": out["clocks"],
        "plain_fp64": out["plain"],
        "batched_over_plain": (out["value"] / ws / out["plain"]["tets_per_s"]) if out["plain"] else None,
        "tet_cell_pairs_per_s": {"candidate": st["candidate_pairs"] / (out["ms_per_step"] * 1e-3),
                                 "partial": st["partial_pairs"] / (out["ms_per_step"] * 1e-3)},
        "pair_counts": st,
        "mass": out["mass"],
        "octree_build_ms": out["octree_build_ms"],
        "tree_equals_oracle": tree_same,
        "oracle_check": oracle_check,
        "oracle_sample_max_rel": oracle_check["max_rel_cells_gt_1"] if oracle_check else None,
        "tuning": out["tuning"],
    }
    # serving and zoom legs (one GPU, rank 0): the library's continuous batching
    if ws == 1 and not args.skip_serve:
        sv = serve_leg(args, pos)
        line["serve"] = sv
        line["serve_p50_ms"], line["serve_p99_ms"] = sv["p50_ms"], sv["p99_ms"]
        line["serve_rate_req_s"] = sv["offered_rate"]
        if args.serve_rate_high:  # a second, heavier load point
            hi = serve_leg(args, pos, args.serve_rate_high)
            line["serve_high"] = {k: hi[k] for k in ("offered_rate", "achieved_rate", "p50_ms", "p90_ms", "p99_ms",
                                                     "max_ms", "requests", "unfinished_at_deadline")}
    if ws == 1 and not args.skip_zoom:
        zm = zoom_leg(args, pos)
        line["zoom"] = zm
        line["zoom_requests_per_s"] = zm["requests_per_s"]
    print(json.dumps(line), flush=True)
    return 0


def same_tree(info, metas, nodes, off, ids, leaves):
    """True when the GPU octree equals the oracle's: every node's box, level,
    parent, first child and estimate, the leaf order, every leaf's meta-cells."""
    g = info.nodes
    if len(g) != len(nodes) or not np.array_equal(info.leaves, leaves):
        return False
    for f in ("ext", "level", "parent", "first_child", "estimate"):
        if not np.array_equal(g[f], nodes[f]):
            return False
    if not np.array_equal(g["min"], nodes["min"]):
        return False
    return all(np.array_equal(m, ids[off[L]:off[L + 1]]) for m, L in zip(metas, leaves))


def oracle_leaf_check(pos, n, grids, nodes, off, ids, leaves, count):
    """The timed path's leaf grids against the FP64 oracle (the reference's
    deposit_tet_2_grid<double,double> restated) on `count` leaves spread over
    the leaf order, per cell: relative error on cells above 1 and 1e-2 tet
    masses, and the 1e-5 relative + 1e-7 tet-mass bar on every cell."""
    from concurrent.futures import ThreadPoolExecutor

    from oracle import oracle as O
    flat = np.ascontiguousarray(pos.reshape(-1))
    nl = len(leaves)
    pick = sorted(set(int(round(k * (nl - 1) / max(1, count - 1))) for k in range(min(count, nl))))

    def leaf_box(L):
        nd = nodes[L]
        return np.array([nd["min"][0], nd["min"][0] + nd["ext"], nd["min"][1], nd["min"][1] + nd["ext"],
                         nd["min"][2], nd["min"][2] + nd["ext"]], np.float32)

    def ref(q):
        L = leaves[q]
        return O.deposit_meta(flat, (n, n, n), ids[off[L]:off[L + 1]], leaf_box(L), LEAF, fp64=True)

    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 1) as ex:
        refs = list(ex.map(ref, pick))
    got = np.concatenate([grids[q].reshape(-1) for q in pick])
    want = np.concatenate([r.reshape(-1) for r in refs])
    d = np.abs(got - want)
    out = {"leaves": len(pick), "of_leaves": nl, "cells": int(want.size), "seconds": time.perf_counter() - t0}
    for th in (1.0, 1e-2):
        sel = want > th
        out[f"max_rel_cells_gt_{th:g}"] = float((d[sel] / want[sel]).max()) if sel.any() else 0.0
    out["max_abs_tet_masses"] = float(d.max())
    out["bar_1e-5_rel_plus_1e-7_abs_ok"] = bool(np.all(d <= 1e-5 * want + 1e-7))
    out["mass_rel_diff"] = float(abs(got.sum() - want.sum()) / want.sum())
    return out


def serve_leg(args, pos, rate=None):
    """Poisson stream of 128^3-cell zoom requests against the resident lattice."""
    from adeco_gb300 import deposit as D
    from adeco_gb300.synthetic import poisson_requests
    rate = args.serve_rate if rate is None else rate
    stream = poisson_requests(rate, args.serve_seconds, L=L_BOX, seed=SERVE_SEED, dims=tuple(args.serve_dims))
    with D.Session(pos, device=args.device) as s:
        res = serve_stream(s, stream, args.serve_seconds + args.serve_drain_s)
    lat = np.sort(np.asarray(res["lat"]))
    return {"workload": f"Poisson arrivals at {rate:g} req/s for {args.serve_seconds:g} s (seed "
                        f"{SERVE_SEED}): zoom boxes, centre uniform, side log-uniform [0.005L, 0.5L], resolution "
                        f"from {args.serve_dims}; one batch per request, submitted at its arrival",
            "p50_ms": float(np.percentile(lat, 50)), "p90_ms": float(np.percentile(lat, 90)),
            "p99_ms": float(np.percentile(lat, 99)), "max_ms": float(lat[-1]), "requests": int(lat.size),
            "offered_rate": rate, "achieved_rate": lat.size / res["wall"],
            "unfinished_at_deadline": res["unfinished"], "serving_stats": res["stats"]}


def zoom_leg(args, pos):
    """512 zoom requests (C3) in one batch: autotuned tile / item size / chunk /
    staging depth on every other request, then whole batches timed on the
    device."""
    from adeco_gb300 import deposit as D
    from adeco_gb300 import tune
    from adeco_gb300.synthetic import zoom_requests
    reqs = zoom_requests(args.zoom_count, L=L_BOX, seed=ZOOM_SEED, dims=tuple(args.zoom_dims))
    cells = sum(r[2] ** 3 for r in reqs)
    with D.Session(pos, device=args.device) as s:
        if args.no_tune:
            params, tinfo = s.get_tuning(), {"source": "defaults"}
        else:
            params, tinfo = tune.tune_zoom(s, reqs[::2], f"{len(reqs)} zoom requests, seed {ZOOM_SEED}",
                                           device=args.device, force=args.retune)
        ms = []
        for k in range(1 + args.zoom_steps):
            b = s.submit(reqs)
            t = s.device_ms(b)
            if k == 0:
                j = min(range(len(reqs)), key=lambda i: reqs[i][2])
                b1 = s.submit([reqs[j]])
                same = bool(np.array_equal(s.result(b1, 0, reqs[j][2]), s.result(b, j, reqs[j][2])))
                s.release(b1)
            else:
                ms.append(t)
            s.release(b)
    m = statistics.median(ms)
    return {"workload": f"{len(reqs)} zoom requests (seed {ZOOM_SEED}): centres uniform, side log-uniform "
                        f"[0.01L, 0.25L], resolution from {args.zoom_dims}, one batch", "cells": cells,
            "ms_per_batch": m, "requests_per_s": len(reqs) / (m * 1e-3), "cells_per_s": cells / (m * 1e-3),
            "steps": args.zoom_steps, "alone_equals_in_batch": same,
            "tuning": {"zoom": {k: params[k] for k in ("zoom_tile", "item_pairs", "share_chunk", "clip_batch")},
                       **{k: v for k, v in tinfo.items() if k != "key"}}}


# --------------------------------------------------------------- C1: the reference boundary
def run_c1(args, rank, ws, local):
    """C1: periodic 64^3 lattice onto a uniform 128^3 grid, through the
    reference boundary (27 image boxes, each call accumulating).  value: the
    device-pointer entry point with the patches resident; e2e: the reference
    signature (adeco_deposit_tets_ex, host buffers, FP64 output) per step."""
    import torch

    from adeco_gb300 import _lib as LB
    from adeco_gb300.synthetic import image_boxes, lattice_patches, periodic_ghost_lattice, zeldovich_lattice
    if rank != 0:
        return 0
    n, m, dims = N_PART, 16, 128
    pos = zeldovich_lattice(n, L=L_BOX, seed=SEED, rms_disp=RMS_DISP)
    patches = lattice_patches(periodic_ghost_lattice(pos, L_BOX), m)
    boxes = image_boxes(np.array([0, L_BOX, 0, L_BOX, 0, L_BOX], np.float32), L_BOX)
    tets = 6 * n ** 3
    lib = LB.load(build_if_missing=True)
    npatch = patches.size // (3 * (m + 1) ** 3)
    d_pos = torch.from_numpy(patches).cuda(args.device)
    d_out = torch.zeros(dims ** 3, dtype=torch.float64, device=f"cuda:{args.device}")
    st = torch.cuda.current_stream(args.device)
    sp = C.c_void_p(st.cuda_stream)

    def device_step():
        d_out.zero_()
        for b in boxes:
            LB.check(lib.adeco_deposit_tets_device(C.c_void_p(d_pos.data_ptr()), patches.size, 0, npatch, m,
                                                   C.c_void_p(b.ctypes.data), dims, C.c_void_p(d_out.data_ptr()),
                                                   0, 0, 1.0, sp))

    for _ in range(args.warmup):
        device_step()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    with ClockSampler(args.device) as clk:
        e0.record(st)
        for _ in range(args.steps):
            device_step()
        e1.record(st)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    total = float(d_out.sum().item())
    # e2e: host positions, host FP64 grid, through the reference-shaped entry point
    from adeco_gb300 import deposit as D
    host = np.zeros(dims ** 3)
    e2e_t = []
    for k in range(1 + args.e2e_steps):
        host[:] = 0.0
        t0 = time.perf_counter()
        for b in boxes:
            D.deposit_tets_ex(patches, m, b, dims, data=host)
        if k:
            e2e_t.append(time.perf_counter() - t0)
    e2e_s = statistics.median(e2e_t)
    # CPU baseline: the reference algorithm (FP32 oracle) over every image, all host threads
    cpu = None
    if not args.skip_cpu:
        from oracle import oracle as O
        threads = os.cpu_count() or 1
        g32 = np.zeros(dims ** 3, np.float32)
        t0 = time.perf_counter()
        for b in boxes:
            O.deposit_patches(patches, m, b, dims, fp64=False, grid=g32, threads=threads)
        sec = time.perf_counter() - t0
        cpu = {"value": tets / sec, "unit": "tets/s", "cores": threads, "kind": "port",
               "sample": f"the whole workload ({npatch} patches x 27 images, {sec:.1f} s on {threads} threads, FP32 "
                         f"oracle restatement of the reference deposit)"}
    line = {
        "metric": "tets/s deposited", "value": tets / (ms * 1e-3), "unit": "tets/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "tets": tets, "grid": f"{dims}^3", "calls_per_step": len(boxes),
                   "l2": "inputs smaller than L2; the grid (16 MB) stays in L2 between steps"},
        "e2e": {"value": tets / e2e_s, "unit": "tets/s", "ms_per_step": e2e_s * 1e3,
                "h2d_bytes_per_step": int(patches.size * 4 * len(boxes)),
                "d2h_bytes_per_step": int(dims ** 3 * 8 * len(boxes))},
        "cpu_baseline": cpu, "clocks": clk.summary(),
        "mass": {"total": total, "tet_count": tets, "rel_diff": abs(total - tets) / tets},
    }
    print(json.dumps(line), flush=True)
    return 0


# --------------------------------------------------------------- zoom batches and serving
def run_zoom(args, rank, ws, local):
    """512 zoom requests on the resident 256^3 lattice, one batch (one launch) per step."""
    from adeco_gb300 import deposit as D
    from adeco_gb300.synthetic import zoom_requests
    if rank != 0:
        return 0
    pos = workload_positions()
    reqs = zoom_requests(args.zoom_count, L=L_BOX, seed=ZOOM_SEED, dims=tuple(args.zoom_dims))
    cells = sum(r[2] ** 3 for r in reqs)
    dev, host = [], []
    same = None
    with D.Session(pos, device=args.device) as s:
        for step in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            b = s.submit(reqs)
            s.wait(b)
            t1 = time.perf_counter()
            ms = s.device_ms(b)
            if step == 0:
                # a request alone gives the same masses as inside the batch
                k = min(range(len(reqs)), key=lambda i: reqs[i][2])
                b1 = s.submit([reqs[k]])
                same = bool(np.array_equal(s.result(b1, 0, reqs[k][2]), s.result(b, k, reqs[k][2])))
                s.release(b1)
            s.release(b)
            if step >= args.warmup:
                dev.append(ms)
                host.append((t1 - t0) * 1e3)
    ms = statistics.median(dev)
    line = {
        "metric": "zoom requests/s", "value": len(reqs) / (ms * 1e-3), "unit": "requests/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"{len(reqs)} zoom requests (seed {ZOOM_SEED}): centres uniform, side log-uniform "
                               f"[0.01L, 0.25L], resolution from {args.zoom_dims}, on the 256^3 lattice (seed 0)",
                   "cells": cells, "batch": "all requests in one batch, one launch per step"},
        "cells_per_s": cells / (ms * 1e-3),
        "host_ms_per_batch": statistics.median(host),
        "alone_equals_in_batch": same,
    }
    print(json.dumps(line), flush=True)
    return 0


def run_serve(args, rank, ws, local):
    """Poisson stream of zoom requests, one batch per request as it arrives;
    latency = arrival -> results ready on the device (host clock)."""
    from adeco_gb300 import deposit as D
    from adeco_gb300.synthetic import poisson_requests
    if rank != 0:
        return 0
    pos = workload_positions()
    stream = poisson_requests(args.serve_rate, args.serve_seconds, L=L_BOX, seed=SERVE_SEED,
                              dims=tuple(args.serve_dims))
    with D.Session(pos, device=args.device) as s:
        res = serve_stream(s, stream, args.serve_seconds + args.serve_drain_s)
    lat, wall, unfinished, stats = res["lat"], res["wall"], res["unfinished"], res["stats"]
    lat = np.sort(np.asarray(lat))
    line = {
        "metric": "serving latency p50", "value": float(np.percentile(lat, 50)), "unit": "ms", "n_gpus": 1,
        "steps": len(lat), "warmup": 3, "ms_per_step": float(np.mean(lat)), "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"Poisson arrivals at {args.serve_rate:g} req/s for {args.serve_seconds:g} s "
                               f"(seed {SERVE_SEED}): zoom boxes, side log-uniform [0.005L, 0.5L], resolution from "
                               f"{args.serve_dims}, depth 0 (a uniform grid per request), on the resident "
                               f"{N_PART}^3 lattice (seed {SEED}{', 2000 infall regions' if INFALL else ''}); "
                               f"one batch per request"},
        "p50_ms": float(np.percentile(lat, 50)), "p90_ms": float(np.percentile(lat, 90)),
        "p99_ms": float(np.percentile(lat, 99)), "max_ms": float(lat[-1]),
        "requests": len(lat), "offered_rate": args.serve_rate, "achieved_rate": len(lat) / wall,
        "unfinished_at_deadline": unfinished, "serving_stats": stats,
    }
    print(json.dumps(line), flush=True)
    return 0


def serve_stream(s, stream, deadline_s):
    """Replays a Poisson stream [(arrival_s, request)] against session `s`, one
    batch per request submitted at its arrival time; latency = arrival ->
    results in host memory (the completion time the library stamps).  The
    library admits and queues; this loop only submits and polls."""
    for _, r in stream[:3]:  # warm-up: the server's arena, streams and first chunks
        b = s.submit([r])
        s.wait(b)
        s.release(b)
    lat, pending = [], {}
    t_start = time.perf_counter()
    i = 0
    while i < len(stream) or pending:
        now = time.perf_counter() - t_start
        if now > deadline_s:
            break  # overloaded: stop waiting, report what finished and what did not
        while i < len(stream) and stream[i][0] <= now:
            pending[s.submit([stream[i][1]])] = (stream[i][0], time.perf_counter() - t_start)
            i += 1
        for b in list(pending):
            if s.poll(b):
                arrival, submitted = pending.pop(b)
                # the library's own submit -> done time, plus the arrival -> submit lag of this loop
                lat.append(s.latency_ms(b, 0) + (submitted - arrival) * 1e3)
                s.release(b)
        time.sleep(0.0002)
    wall = time.perf_counter() - t_start
    unfinished = len(pending) + (len(stream) - i)
    for b in list(pending):
        s.wait(b)
        s.release(b)
    return {"lat": lat, "wall": wall, "unfinished": unfinished, "stats": s.serving_stats()}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--e2e-warmup", type=int, default=1)
    ap.add_argument("--cpu-budget-s", type=float, default=12.0)
    ap.add_argument("--ref-step-s", type=float, default=6.0)
    ap.add_argument("--skip-plain", action="store_true")
    ap.add_argument("--skip-e2e", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--n", type=int, default=None, help="lattice size; the benchmark workload is 256")
    ap.add_argument("--workload", default="c2", choices=["c2", "c1", "c4", "zoom", "serve", "c5"])
    ap.add_argument("--zoom-dims", type=int, nargs="+", default=[32, 64, 128, 256])
    ap.add_argument("--zoom-count", type=int, default=ZOOM_COUNT)
    ap.add_argument("--serve-rate", type=float, default=None, help="req/s (30; c5: 10)")
    ap.add_argument("--serve-rate-high", type=float, default=100.0, help="default run: a second serving load point (0: none)")
    ap.add_argument("--serve-seconds", type=float, default=8.0)
    ap.add_argument("--serve-dims", type=int, nargs="+", default=None, help="resolutions (128; c5: 32 .. 512)")
    ap.add_argument("--serve-drain-s", type=float, default=30.0)
    ap.add_argument("--skip-serve", action="store_true", help="default run: no serving leg")
    ap.add_argument("--skip-zoom", action="store_true", help="default run: no zoom-batch leg")
    ap.add_argument("--skip-oracle-check", action="store_true")
    ap.add_argument("--oracle-leaves", type=int, default=48)
    ap.add_argument("--zoom-steps", type=int, default=2)
    ap.add_argument("--no-tune", action="store_true", help="library defaults instead of the autotuner")
    ap.add_argument("--retune", action="store_true", help="search again even when the tuning cache has a result")
    args = ap.parse_args()
    c5 = args.workload == "c5"
    if args.serve_rate is None:
        args.serve_rate = 10.0 if c5 else 30.0
    if args.serve_dims is None:
        args.serve_dims = [32, 64, 128, 256, 512] if c5 else [128]
    set_workload(args.workload)
    if args.n:
        set_size(args.n)
    if args.warmup < 3:
        args.warmup = 3
    ws, rank, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, rank, ws)
    if args.workload == "zoom":
        return run_zoom(args, rank, ws, local)
    if args.workload in ("serve", "c5"):
        return run_serve(args, rank, ws, local)
    if args.workload == "c1":
        return run_c1(args, rank, ws, local)
    return run_ours(args, rank, ws, local)


if __name__ == "__main__":
    sys.exit(main())
