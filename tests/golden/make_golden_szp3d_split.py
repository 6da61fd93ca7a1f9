"""Generate golden vectors of the SZp 3-D codec's OpenMP form in tests/golden/
from the REFERENCE codec.

Runs the reference's own SZp_compress3D_fast_openmp
(ZCCL/src/ZCCL_float.c:1862-2048) and SZp_decompress3D_fast_openmp
(ZCCL/src/ZCCLd_float.c:2873-3034) from ``oracle/_ref/libzccl_ref.so``, with
the thread count set through omp_set_num_threads, on seeded volumes, and
stores per case the input, the stream and the SHA-256 of the decompressed
floats:

    szp3d_split.npz    x<i> (input volume, flattened), s<i> (stream)
    szp3d_split.json   per case: dims, bs, eb, T, tdims, kind, dec (digest)

Thread counts 1, 3, 8 and 12 give thread grids 1x1x1, 3x1x1, 2x2x2 and
3x2x2; shapes that the grids do not divide evenly give uneven sub-volumes;
block sides 2, 3, 4 and 8 cut the sub-volumes' edge blocks short.

Usage (where the reference checkout exists):  python tests/golden/make_golden_szp3d_split.py
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle import zoracle  # noqa: E402

SHAPES = [((16, 16, 16), 4), ((13, 20, 33), 8), ((24, 17, 9), 2), ((10, 7, 14), 3), ((9, 30, 11), 4)]
THREADS = (1, 3, 8, 12)
KINDS = ("smooth", "noisy")


def volume(dims, kind, seed):
    rng = np.random.default_rng(seed)
    i, j, k = np.meshgrid(*[np.arange(d, dtype=np.float64) for d in dims], indexing="ij")
    base = np.sin(i / 5.0) + np.cos(j / 7.0) * np.sin(k / 3.0)
    x = {"smooth": base, "noisy": base + rng.normal(0, 0.3, dims)}[kind]
    return x.astype(np.float32).ravel()


def main():
    zoracle.build(ref=True)
    if not zoracle.ref_available():
        sys.exit("the reference library is not available here")
    ref = zoracle.ref()
    arrays, cases = {}, []
    for si, (dims, bs) in enumerate(SHAPES):
        for ki, kind in enumerate(KINDS):
            x = volume(dims, kind, 300 + 10 * si + ki)
            for T in THREADS:
                eb = 1e-3 if (si + T) % 2 else 1e-2
                s = ref.szp3d_compress_split(x, dims, bs, eb, T)
                y = ref.szp3d_decompress_split(s, dims, bs, eb, T)
                i = len(cases)
                arrays[f"x{i}"] = x
                arrays[f"s{i}"] = np.frombuffer(s, np.uint8)
                cases.append({"i": i, "dims": list(dims), "bs": bs, "eb": eb, "T": T, "tdims": ref.dims3(T),
                              "kind": kind, "dec": hashlib.sha256(y.tobytes()).hexdigest()})
    np.savez_compressed(os.path.join(HERE, "szp3d_split.npz"), **arrays)
    with open(os.path.join(HERE, "szp3d_split.json"), "w") as f:
        json.dump({"cases": cases}, f, indent=1)
    print(len(cases), "cases")


if __name__ == "__main__":
    main()
