"""Seeded synthetic inputs: Zel'dovich-displaced Lagrangian lattices.

ADECO reads N-body snapshots (Dark Sky files, src/AdPointDataReaders.h); no
dataset is available here, so the workloads are generated from the recipe
the benchmark configurations name:

* lattice q = (i+1/2, j+1/2, k+1/2) * L/n, ids x fastest
  (the SORTED_BY_ID layout, src/AdPointDataReaders.h:770-910);
* a Gaussian random field delta(k) with P(k) ∝ k^-2 exp(-(k/k_c)^2),
  k_c = 8 * 2pi / L, from ``numpy.random.default_rng(seed)``;
* the Zel'dovich displacement psi(k) = i k / k^2 delta(k), rescaled to a
  stated RMS |psi| in lattice spacings; x = q + psi.

Positions are returned already unwrapped (q + psi, not wrapped into [0, L)):
that is what the reference's periodic unwrap (``apply_boundary_corrections``,
src/AdPointDataReaders.h:154-204) reconstructs for displacements below L/4.
"""
from __future__ import annotations

import numpy as np


def zeldovich_lattice(n: int, L: float = 100.0, seed: int = 0, rms_disp: float = 0.5,
                      kc_factor: float = 8.0, infall: int = 0, infall_seed: int | None = None,
                      dtype=np.float32) -> np.ndarray:
    """Return positions of shape (n, n, n, 3) indexed [k, j, i] (x fastest)."""
    rng = np.random.default_rng(seed)
    white = rng.standard_normal((n, n, n))
    dk = np.fft.rfftn(white)
    del white
    kf = 2.0 * np.pi / L
    kx = np.fft.rfftfreq(n, d=1.0 / n) * kf          # last axis (x) is the rfft axis
    ky = np.fft.fftfreq(n, d=1.0 / n) * kf
    kz = np.fft.fftfreq(n, d=1.0 / n) * kf
    k2 = kz[:, None, None] ** 2 + ky[None, :, None] ** 2 + kx[None, None, :] ** 2
    kc = kc_factor * kf
    with np.errstate(divide="ignore", invalid="ignore"):
        amp = np.where(k2 > 0, np.sqrt(1.0 / k2 * np.exp(-k2 / kc ** 2)), 0.0)
        dk *= amp
        inv_k2 = np.where(k2 > 0, 1.0 / k2, 0.0)
    del amp
    psi = np.empty((n, n, n, 3), dtype=np.float64)
    for a, kv in enumerate((kx[None, None, :], ky[None, :, None], kz[:, None, None])):
        psi[..., a] = np.fft.irfftn(1j * kv * inv_k2 * dk, s=(n, n, n), axes=(0, 1, 2))
    del dk
    rms = np.sqrt(np.mean(np.sum(psi ** 2, axis=-1)))
    spacing = L / n
    if rms > 0:
        psi *= (rms_disp * spacing) / rms
    q1 = (np.arange(n) + 0.5) * spacing
    pos = psi
    pos[..., 0] += q1[None, None, :]
    pos[..., 1] += q1[None, :, None]
    pos[..., 2] += q1[:, None, None]
    if infall > 0:
        _apply_infall(pos, n, L, infall, seed if infall_seed is None else infall_seed)
    return pos.astype(dtype)


def _apply_infall(pos, n, L, count, seed, concentration=10.0):
    """Spherical infall regions: centres uniform, radii log-uniform in
    [0.5, 5] lattice spacings, NFW-like radial compression of the particles
    within 3 radii of the centre.  A region looks at the lattice sites within
    (3 radii + the largest displacement so far) of its centre, so the cost is
    local; the regions are applied in order."""
    rng = np.random.default_rng(seed + 1000003)
    spacing = L / n
    centres = rng.uniform(0.0, L, size=(count, 3))
    radii = np.exp(rng.uniform(np.log(0.5), np.log(5.0), size=count)) * spacing
    q1 = (np.arange(n) + 0.5) * spacing
    disp = 0.0
    for a, sl in enumerate((np.s_[None, None, :], np.s_[None, :, None], np.s_[:, None, None])):
        d = pos[..., a] - q1[sl]
        d -= L * np.round(d / L)
        disp = max(disp, float(np.abs(d).max()))
    for c, r in zip(centres, radii):
        reach = 3.0 * r
        w = reach + disp
        idx = []
        for a in range(3):
            lo = int(np.floor((c[a] - w) / spacing)) - 1
            hi = int(np.ceil((c[a] + w) / spacing)) + 1
            idx.append(np.arange(n) if hi - lo + 1 >= n else np.arange(lo, hi + 1) % n)
        win = np.ix_(idx[2], idx[1], idx[0])
        sub = pos[win]
        d = sub - c
        d -= L * np.round(d / L)
        dist = np.sqrt(np.sum(d * d, axis=-1))
        sel = dist < reach
        if not np.any(sel):
            continue
        x = dist[sel] / reach
        # enclosed-mass-like profile: shrink radii toward the centre
        g = np.log1p(concentration * x) / np.log1p(concentration)
        new = reach * (x * 0.5 + 0.5 * g * x)
        scale = np.where(dist[sel] > 0, new / np.maximum(dist[sel], 1e-12), 1.0)
        moved = c + d[sel] * scale[:, None]
        site = np.stack(np.broadcast_arrays(q1[idx[0]][None, None, :], q1[idx[1]][None, :, None],
                                            q1[idx[2]][:, None, None]), axis=-1)[sel]
        dq = moved - site
        dq -= L * np.round(dq / L)
        disp = max(disp, float(np.abs(dq).max()))
        sub[sel] = moved
        pos[win] = sub


def zoom_requests(count: int = 512, L: float = 100.0, seed: int = 1, side=(0.01, 0.25),
                  dims=(32, 64, 128, 256)):
    """Zoom requests (centre, side, dims): centres uniform in the box, sides
    log-uniform in side * L, resolution drawn uniformly from `dims`."""
    rng = np.random.default_rng(seed)
    centres = rng.uniform(0.0, L, size=(count, 3))
    sides = L * np.exp(rng.uniform(np.log(side[0]), np.log(side[1]), size=count))
    res = rng.choice(np.asarray(dims), size=count)
    return [(tuple(float(v) for v in c), float(s_), int(d)) for c, s_, d in zip(centres, sides, res)]


def poisson_requests(rate: float, duration_s: float, L: float = 100.0, seed: int = 2, side=(0.005, 0.5),
                     dims=(32, 64, 128, 256, 512)):
    """Serving stream: Poisson arrivals at `rate` per second over `duration_s`;
    each request a zoom box (side log-uniform in side * L, resolution drawn
    uniformly from `dims`).  Returns [(arrival_s, (centre, side, dims))]."""
    rng = np.random.default_rng(seed)
    out, t = [], 0.0
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration_s:
            return out
        c = rng.uniform(0.0, L, size=3)
        s_ = L * np.exp(rng.uniform(np.log(side[0]), np.log(side[1])))
        d = int(rng.choice(np.asarray(dims)))
        out.append((t, (tuple(float(v) for v in c), float(s_), d)))


def periodic_ghost_lattice(pos: np.ndarray, L: float) -> np.ndarray:
    """(n,n,n,3) periodic lattice -> (n+1)^3 lattice whose last plane along
    each axis is the first plane shifted by +L: its (n)^3 cubes are the n^3
    periodic cubes, in the reference's non-periodic cube convention."""
    n = pos.shape[0]
    out = np.empty((n + 1, n + 1, n + 1, 3), dtype=pos.dtype)
    out[:n, :n, :n] = pos
    out[:n, :n, n] = pos[:, :, 0] + np.array([L, 0, 0], dtype=pos.dtype)
    out[:n, n, :] = out[:n, 0, :] + np.array([0, L, 0], dtype=pos.dtype)
    out[n, :, :] = out[0, :, :] + np.array([0, 0, L], dtype=pos.dtype)
    return out


def lattice_patches(vertices: np.ndarray, m: int) -> np.ndarray:
    """Cut an (N+1)^3 vertex lattice (shape (N+1, N+1, N+1, 3), x fastest)
    into (N/m)^3 patches of (m+1)^3 vertices -- the reference boundary's input
    layout, neighbouring patches sharing a vertex plane -- flattened, patches
    x fastest."""
    n = vertices.shape[0] - 1
    if n % m:
        raise ValueError(f"{n} cubes per axis is not a multiple of m = {m}")
    k = n // m
    out = np.empty((k, k, k, m + 1, m + 1, m + 1, 3), dtype=vertices.dtype)
    for pz in range(k):
        for py in range(k):
            for px in range(k):
                out[pz, py, px] = vertices[pz * m:pz * m + m + 1, py * m:py * m + m + 1, px * m:px * m + m + 1]
    return out.reshape(-1)


def image_boxes(bbox, L: float):
    """The 27 periodic images (shifts by -L, 0, +L per axis) of a grid box
    (xmin, xmax, ymin, ymax, zmin, zmax): depositing into every image and
    summing wraps the mass that periodic tets carry across the box faces."""
    b = np.asarray(bbox, dtype=np.float32)
    out = []
    for sz in (-1, 0, 1):
        for sy in (-1, 0, 1):
            for sx in (-1, 0, 1):
                sh = np.array([sx, sx, sy, sy, sz, sz], dtype=np.float32) * np.float32(L)
                out.append((b + sh).astype(np.float32))
    return out


def bbox6(pos: np.ndarray):
    """(xmin, xmax, ymin, ymax, zmin, zmax) of a position array."""
    p = pos.reshape(-1, 3)
    mn, mx = p.min(axis=0), p.max(axis=0)
    return np.array([mn[0], mx[0], mn[1], mx[1], mn[2], mx[2]], dtype=np.float32)
