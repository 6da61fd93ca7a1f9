"""Times the oracle's C restatement (the port) against the reference library
built from the reference's own sources, on this host's cores, at the same
OpenMP thread count T and on the same seeded 512^3 log-normal field
(eb = 1e-4 of range, L = 32): best of `reps` passes after one warm-up of
compress, decompress and the two-way homomorphic add.  Prints one JSON line
per (T, code).  The bench's CPU baseline is the port; the ratio printed here
tells how far a GPU-over-port ratio is from a GPU-over-reference one.

    python oracle/calibrate.py [--side 512] [--T 8 1] [--reps 3]

Needs the reference library (oracle/_ref, built by `make -C oracle ref`)."""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

from oracle import zoracle  # noqa: E402


def field(side: int, seed: int) -> np.ndarray:
    import torch
    from zccl_gb300.workloads import grf_lognormal
    return grf_lognormal(side, seed, torch.device("cpu")).numpy()


def best(fn, reps):
    fn()
    t = []
    for _ in range(reps):
        t0 = time.perf_counter()
        fn()
        t.append(time.perf_counter() - t0)
    return min(t)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--side", type=int, default=512)
    ap.add_argument("--T", type=int, nargs="+", default=[8, 1])
    ap.add_argument("--reps", type=int, default=3)
    a = ap.parse_args()
    if not zoracle.ref_available():
        sys.exit("reference library not built (make -C oracle ref)")
    x, y = field(a.side, 0), field(a.side, 1)
    n, L = x.size, 32
    eb = float(np.float32(1e-4 * max(float(x.max() - x.min()), float(y.max() - y.min()))))
    for T in a.T:
        for name, c in (("port", zoracle.port()), ("reference library", zoracle.ref())):
            sa, sb = c.compress(x, eb, L, T), c.compress(y, eb, L, T)
            tc = best(lambda: c.compress(x, eb, L, T), a.reps)
            td = best(lambda: c.decompress(sa, n, eb, L, T), a.reps)
            th = best(lambda: c.homadd(sa, sb, n, eb, L, T), a.reps)
            gb = 4 * n / 1e9
            print(json.dumps({"T": T, "code": name, "n": n, "compress_GBps": round(gb / tc, 3),
                              "decompress_GBps": round(gb / td, 3), "homadd_GBps": round(gb / th, 3),
                              "step_GBps": round(3 * gb / (tc + td + th), 3)}), flush=True)


if __name__ == "__main__":
    main()
