"""Restatement of the reference's single-rank particle readers -- TEST
INFRASTRUCTURE ONLY (used by tests/ and tests/golden/make_golden.py as the
checker of the library's readers; the product never imports it).

* SORTED_BY_ID (src/AdPointDataReaders.h:770-911): float32 x, y, z per
  particle in id order; n^3 particles (n = round(cbrt(count)), checked);
  stride is ignored by the reference (:783-786).
* DARK_SKY (src/AdPointDataReaders.h:361-767): an SDF text header ending with
  the line "# SDF-EOH", followed by sha1_chunks x (4 + 20) bytes (the header
  size rule of get_header_size, :425-467); then records of float32 x, y, z,
  vx, vy, vz and int64 id (:508-516).  The id's low 48 bits are a Morton key:
  bit 3l -> x, 3l+1 -> y, 3l+2 -> z (morton_2_grid, :366-394, after its swap
  of the first and last axis).  With stride s only particles whose three
  lattice indices are multiples of s are kept, at index / s (:622-634).
  The linear id is x + n (y + n z) (:637).
* Periodic unwrap, apply_boundary_corrections (src/AdPointDataReaders.h:154-204),
  over the global bbox of the particles read (get_global_bbox_mpi, :136),
  in float32: for each axis, a particle whose lattice index is above n/2
  and whose position is below min + ext/4 moves up by ext; one with index
  below n/2 and position above min + (3/4) ext moves down by ext.
"""
from __future__ import annotations

import numpy as np

REC = np.dtype([("pos", "<f4", 3), ("vel", "<f4", 3), ("id", "<i8")])


def sdf_header_size(raw: bytes) -> int:
    sha1_chunks, pos = -1, 0
    for _ in range(100000):
        end = raw.find(b"\n", pos)
        if end < 0:
            break
        line = raw[pos:end].decode("latin-1")
        pos = end + 1
        if line.startswith("int sha1_chunks ="):
            sha1_chunks = int(line[line.find("=") + 1:line.find(";")])
        if line.startswith("# SDF-EOH"):
            if sha1_chunks < 0:
                break
            return pos + sha1_chunks * (4 + 20)
    raise ValueError("failed to parse the SDF header")


def morton_decode(key):
    key = np.asarray(key, np.int64) & ((1 << 48) - 1)
    out = np.zeros((key.size, 3), np.int64)
    for level in range(16):
        for a in range(3):
            out[:, a] |= ((key >> (3 * level + a)) & 1) << level
    return out


def morton_encode(ijk):
    ijk = np.asarray(ijk, np.int64)
    key = np.zeros(len(ijk), np.int64)
    for level in range(16):
        for a in range(3):
            key |= ((ijk[:, a] >> level) & 1) << (3 * level + a)
    return key


def read_particles(path: str, fmt: str, stride: int = 1, periodic: bool = True):
    """(positions (n, n, n, 3) float32 indexed [k, j, i], bbox6) as the reference reads them."""
    raw = open(path, "rb").read()
    if "SORTED_BY_ID" in fmt:
        if len(raw) % 12:
            raise ValueError("inconsistent file size")
        pos = np.frombuffer(raw, "<f4").reshape(-1, 3).copy()
        n = int(round(len(pos) ** (1.0 / 3.0)))
        if n ** 3 != len(pos):
            raise ValueError("lagrangian grid not cubical")
        ids = np.arange(n ** 3)
    elif "DARK_SKY" in fmt:
        hs = sdf_header_size(raw)
        if (len(raw) - hs) % REC.itemsize:
            raise ValueError("inconsistent file size")
        rec = np.frombuffer(raw[hs:], REC)
        n0 = int(np.rint(np.cbrt(len(rec))))
        if n0 ** 3 != len(rec):
            raise ValueError("lagrangian grid not cubical")
        if n0 % stride:
            raise ValueError("invalid stride for data dimensions")
        lid = morton_decode(rec["id"])
        keep = np.all(lid % stride == 0, axis=1) if stride != 1 else np.ones(len(rec), bool)
        lid = lid[keep] // stride
        n = n0 // stride
        pos = rec["pos"][keep].copy()
        ids = lid[:, 0] + n * (lid[:, 1] + n * lid[:, 2])
        if len(ids) != n ** 3:
            raise ValueError("inconsistent global particle number")
    else:
        raise ValueError(f"id_type {fmt} not supported")
    mn, mx = pos.min(axis=0), pos.max(axis=0)
    if periodic:
        ext = (mx - mn).astype(np.float32)
        h1 = (mn + ext / np.float32(4.0)).astype(np.float32)
        h2 = (mn + np.float32(0.75) * ext).astype(np.float32)
        half = np.float32(n) / np.float32(2.0)
        idx = np.stack([ids % n, (ids // n) % n, ids // (n * n)], axis=1).astype(np.float32)
        up = (idx > half) & (pos < h1)
        down = (idx < half) & (pos > h2) & ~up
        pos = np.where(up, pos + ext, np.where(down, pos - ext, pos)).astype(np.float32)
    out = np.empty((n ** 3, 3), np.float32)
    out[ids] = pos
    bbox = np.array([mn[0], mx[0], mn[1], mx[1], mn[2], mx[2]], np.float32)
    return out.reshape(n, n, n, 3), bbox


def write_sorted_by_id(path: str, pos) -> None:
    np.ascontiguousarray(pos, np.float32).reshape(-1).tofile(path)


def write_dark_sky(path: str, pos, *, seed: int = 0, sha1_chunks: int = 3, vel=None) -> None:
    """An SDF file of the lattice `pos` (n, n, n, 3), records in a shuffled order."""
    pos = np.asarray(pos, np.float32)
    n = pos.shape[0]
    k, j, i = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    ijk = np.stack([i.ravel(), j.ravel(), k.ravel()], axis=1)
    rec = np.zeros(n ** 3, REC)
    rec["pos"] = pos.reshape(-1, 3)
    rec["vel"] = 0.0 if vel is None else vel
    rec["id"] = morton_encode(ijk) | (np.int64(5) << 50)   # bits above 48 are not part of the key
    rec = rec[np.random.default_rng(seed).permutation(n ** 3)]
    header = ("# SDF 1.0\nparameter byteorder = 0x78563412;\nint npart = %d;\nint sha1_chunks = %d;\n"
              "struct {\n float x, y, z;\n float vx, vy, vz;\n int64_t ident;\n}[%d];\n# SDF-EOH\n"
              % (n ** 3, sha1_chunks, n ** 3)).encode()
    with open(path, "wb") as f:
        f.write(header)
        f.write(b"\x01" * (sha1_chunks * 24))
        f.write(rec.tobytes())
