"""Golden fixtures for the particle readers, from the reference's own readers.

Run here, where the reference tree exists (oracle/_ref/libadeco_ref_readers.so
is built from it by ``make -C oracle ref``):

    python tests/golden/make_golden_readers.py

The input lattice (a wrapped Zel'dovich lattice, seed 9) is stored in
readers.npz; the tests write the SORTED_BY_ID and DARK_SKY files from it with
oracle/readers.py (DARK_SKY records shuffled with seed 1, 3 sha1 chunks) and
check the reader under test against the lattices the reference's readers
(src/AdPointDataReaders.h, one rank, periodic unwrap on or off) made from the
same files, stored here.
"""
from __future__ import annotations

import ctypes as C
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from adeco_gb300.synthetic import zeldovich_lattice  # noqa: E402
from oracle import readers as R  # noqa: E402

CASES = [("SORTED_BY_ID", 1, 0), ("SORTED_BY_ID", 1, 1), ("DARK_SKY", 1, 0), ("DARK_SKY", 1, 1),
         ("DARK_SKY", 2, 1), ("DARK_SKY", 4, 0)]
N, L = 16, 30.0


def write_inputs(lattice, tmp):
    paths = {"SORTED_BY_ID": os.path.join(tmp, "particles.bin"), "DARK_SKY": os.path.join(tmp, "particles.sdf")}
    R.write_sorted_by_id(paths["SORTED_BY_ID"], lattice)
    R.write_dark_sky(paths["DARK_SKY"], lattice, seed=1, sha1_chunks=3)
    return paths


def main():
    lib = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libadeco_ref_readers.so"))
    f32p = np.ctypeslib.ndpointer(np.float32)
    lib.ref_read_particles.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.c_int, f32p, C.c_longlong,
                                       np.ctypeslib.ndpointer(np.int32), f32p]
    lattice = np.mod(zeldovich_lattice(N, L=L, seed=9, rms_disp=2.0), L).astype(np.float32)
    out = {"lattice": lattice, "cases": np.array([f"{f}:{s}:{p}" for f, s, p in CASES])}
    with tempfile.TemporaryDirectory() as tmp:
        paths = write_inputs(lattice, tmp)
        for k, (fmt, stride, periodic) in enumerate(CASES):
            n = N // stride if fmt == "DARK_SKY" else N
            xyz = np.zeros(n ** 3 * 3, np.float32)
            dims = np.zeros(3, np.int32)
            bbox = np.zeros(6, np.float32)
            rc = lib.ref_read_particles(paths[fmt].encode(), fmt.encode(), stride, periodic, xyz, n ** 3, dims, bbox)
            assert rc == 0 and list(dims) == [n, n, n], (fmt, stride, rc, dims)
            out[f"xyz_{k}"] = xyz.reshape(n, n, n, 3)
            out[f"bbox_{k}"] = bbox
    np.savez_compressed(os.path.join(HERE, "readers.npz"), **out)
    print("wrote readers.npz:", [f"{f}:{s}:{p}" for f, s, p in CASES])


if __name__ == "__main__":
    main()
