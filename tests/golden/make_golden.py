"""Writes tests/golden/potrf_golden.npz — run here, where the reference checkout exists.

Generator pins come from the reference's own PLASMA generator (examples/potrf/core_plgsy.h,
compiled unmodified into oracle/_ref/ref_plgsy by oracle/build.py):
  * plgsy_N100_NB32:  the full ragged tile set (N=100, NB=32, bump=N, seed=3872) as floats64
  * sha256 of the tile sets for (N=160, NB=32) — the reference driver's default size — and
    (N=1000, NB=128), the ragged size the device tests use.
Factor pins come from the oracle's restated flowgraph with plain-loop tile kernels:
  * factor_N100_NB32: L of plgsy_N100_NB32 (lower tiles)
  * uniform_N64_seed42: a few entries of the counter-based generator for seed 42.
"""
import hashlib
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
import oracle  # noqa: E402
from oracle import build as obuild  # noqa: E402


def ref_plgsy(N, NB, bump, seed):
    exe = obuild.build_ref()
    if exe is None:
        raise SystemExit("reference checkout not found; golden fixtures cannot be regenerated")
    with tempfile.TemporaryDirectory() as d:
        out = os.path.join(d, "t.bin")
        subprocess.check_call([exe, str(N), str(NB), repr(float(bump)), str(seed), out])
        return np.fromfile(out, dtype=np.float64)


def main():
    g = {}
    t100 = ref_plgsy(100, 32, 100, 3872)
    g["plgsy_N100_NB32"] = t100
    for (N, NB) in [(160, 32), (1000, 128)]:
        t = ref_plgsy(N, NB, N, 3872)
        g["sha256_plgsy_N%d_NB%d" % (N, NB)] = np.frombuffer(hashlib.sha256(t.tobytes()).digest(), dtype=np.uint8)
    f = t100.copy()
    st, info, _ = oracle.potrf_tiled(f, 100, 32, nthreads=2)
    assert st == 0
    g["factor_N100_NB32"] = f
    idx = np.array([[0, 0], [1, 0], [0, 1], [63, 17], [17, 63], [1000, 999]], dtype=np.int64)
    g["uniform_seed42_idx"] = idx
    g["uniform_seed42_val"] = np.array([oracle.lib().orc_uniform_elem(42, int(i), int(j)) for i, j in idx])
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "potrf_golden.npz")
    np.savez_compressed(path, **g)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
