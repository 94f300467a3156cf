"""Autotuner for the deposit's launch-shape and batching parameters.

The parameters (``adeco_tuning`` in include/adeco_deposit.h) change how work
is cut and scheduled, never the arithmetic of a (tet, cell) pair, except the
zoom tile, which moves the frame pairs are clipped in (results stay within
the per-cell bar):

* ``zoom_tile``   -- cells per tile edge of a zoom grid: one work item per
  (tile, meta-cell); smaller tiles balance fine grids better but stage and
  cull each meta-cell's vertex block more often;
* ``share_chunk`` -- candidate pairs per chunk when the warps of an item share
  a large tet group (zoom grids);
* ``clip_batch``  -- the staging depth of the clip engine: partial pairs a
  warp lists before it clips them together (deeper lists keep more lanes
  busy, shallower ones clip sooner);
* ``ctas_per_sm`` -- CTAs per SM of the persistent leaf launch;
* ``item_pairs``  -- the expected candidate pairs above which a zoom
  request's tile edge is halved (fine grids: smaller items, shorter tails).

The number of tets a warp sets up at once is the warp width (32, one per
lane); it is not a parameter.  The reference has no tuner: its launch shape
is the compile-time pair AMD_CUDA_GRID_DIM / AMD_CUDA_BLOCK_DIM
(src/AdDeposit2Grid.h:51-52, <<<512, 64>>>).

The search is coordinate descent from the library defaults: each parameter
in turn takes every candidate value with the others held, the fastest is
kept, and passes repeat until one changes nothing (at most `max_passes`).
Results are cached per GPU (name and SM count) and workload class in a JSON
file (``ADECO_TUNE_CACHE``, default ~/.cache/adeco_gb300/tuning.json).
"""
from __future__ import annotations

import json
import os
import statistics
import time

SPACES = {
    # octree leaf blocks (coarse grids: a tet meets a few cells)
    "leaf": {"clip_batch": [64, 96, 128], "ctas_per_sm": [1, 2]},
    # zoom grids (fine grids: cells much smaller than tets)
    "zoom": {"zoom_tile": [32, 64, 128], "item_pairs": [1 << 16, 1 << 17, 1 << 18, 1 << 20],
             "share_chunk": [256, 512, 1024], "clip_batch": [96, 128]},
}
DEFAULTS = {"zoom_tile": 64, "share_chunk": 512, "clip_batch": 128, "ctas_per_sm": 2, "item_pairs": 1 << 18}


def search(space, measure, start=None, max_passes=2, log=None):
    """Coordinate descent over `space` ({name: [values]}), minimising
    measure(params) -> seconds.  Returns (best params, best time, trials)
    where trials lists every (params, time) measured; a setting is measured
    once."""
    best = dict(start or {k: DEFAULTS.get(k, v[0]) for k, v in space.items()})
    seen = {}

    def cost(p):
        key = tuple(sorted(p.items()))
        if key not in seen:
            seen[key] = float(measure(dict(p)))
            if log:
                log(dict(p), seen[key])
        return seen[key]

    best_t = cost(best)
    for _ in range(max_passes):
        changed = False
        for name, values in space.items():
            for v in values:
                if v == best[name]:
                    continue
                trial = dict(best)
                trial[name] = v
                t = cost(trial)
                if t < best_t:
                    best, best_t, changed = trial, t, True
        if not changed:
            break
    trials = [(dict(k), t) for k, t in seen.items()]
    return best, best_t, trials


def cache_path():
    return os.environ.get("ADECO_TUNE_CACHE") or os.path.join(os.path.expanduser("~"), ".cache", "adeco_gb300",
                                                              "tuning.json")


class TuneCache:
    """Tuned parameters per key (GPU | workload class | workload), in a JSON file."""

    def __init__(self, path=None):
        self.path = path or cache_path()
        try:
            with open(self.path) as f:
                self.data = json.load(f)
            if not isinstance(self.data, dict):
                self.data = {}
        except (OSError, ValueError):
            self.data = {}

    @staticmethod
    def key(gpu, cls, workload):
        return f"{gpu}|{cls}|{workload}"

    def get(self, key):
        e = self.data.get(key)
        return dict(e["params"]) if isinstance(e, dict) and "params" in e else None

    def put(self, key, params, seconds, trials):
        self.data[key] = {"params": dict(params), "seconds": float(seconds), "trials": int(trials),
                          "when": time.strftime("%Y-%m-%dT%H:%M:%S")}
        os.makedirs(os.path.dirname(os.path.abspath(self.path)), exist_ok=True)
        tmp = self.path + ".tmp"
        with open(tmp, "w") as f:
            json.dump(self.data, f, indent=1, sort_keys=True)
        os.replace(tmp, self.path)


def gpu_id(device=0):
    """GPU name and SM count, the part of a cache key that says where a result holds."""
    try:
        import torch
        p = torch.cuda.get_device_properties(device)
        return f"{p.name}/{p.multi_processor_count}sm"
    except Exception:  # noqa: BLE001 -- a key without the GPU still works, it is just less specific
        return "unknown-gpu"


def _apply(session, params):
    session.set_tuning(**params)


def tune_leaves(session, workload, reps=3, cache=None, device=0, force=False, log=None):
    """Tunes the leaf deposit of a session whose octree is built: each trial is
    the median device time of `reps` graph replays.  Returns (params, info)."""
    cache = cache or TuneCache()
    key = TuneCache.key(gpu_id(device), "leaf", workload)
    hit = None if force else cache.get(key)
    if hit:
        _apply(session, hit)
        return hit, {"source": "cache", "key": key}

    def measure(p):
        _apply(session, p)
        session.replay_leaves(1)  # capture with these parameters
        return statistics.median(session.replay_leaves(1)["kernel_ms"] for _ in range(reps)) * 1e-3

    best, t, trials = search(SPACES["leaf"], measure, log=log)
    _apply(session, best)
    cache.put(key, best, t, len(trials))
    return best, {"source": "search", "key": key, "trials": len(trials), "best_ms": t * 1e3}


def tune_zoom(session, requests, workload, reps=1, cache=None, device=0, force=False, log=None):
    """Tunes zoom batches on a sample batch `requests`: each trial is the
    device time of the batch (median of `reps`).  The sample must load the GPU
    like the batches to be served: a batch of 64 of the 512 zoom requests
    picked a tile and item size 15% slower on the whole batch than the
    defaults.  Returns (params, info)."""
    cache = cache or TuneCache()
    key = TuneCache.key(gpu_id(device), "zoom", workload)
    hit = None if force else cache.get(key)
    if hit:
        _apply(session, hit)
        return hit, {"source": "cache", "key": key}

    def one():
        b = session.submit(requests)
        ms = session.device_ms(b)
        session.release(b)
        return ms

    def measure(p):
        _apply(session, p)
        return statistics.median(one() for _ in range(reps)) * 1e-3

    one()  # warm-up: the serving arena and streams
    best, t, trials = search(SPACES["zoom"], measure, log=log)
    _apply(session, best)
    cache.put(key, best, t, len(trials))
    return best, {"source": "search", "key": key, "trials": len(trials), "best_ms": t * 1e3}
