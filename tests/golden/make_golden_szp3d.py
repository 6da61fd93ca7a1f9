"""Generate the SZp 3-D golden vectors in tests/golden/ from the REFERENCE codec.

Runs the reference's own serial 3-D codec (SZp_compress3D_fast and
SZp_compress3D, ZCCL/src/ZCCL_float.c:1706-1860; SZp_decompress3D,
ZCCL/src/ZCCLd_float.c:2801-2871) from ``oracle/_ref/libzccl_ref.so`` on
seeded volumes and stores, per case, the input, the stream (both compress
forms must agree) and the SHA-256 of the decompressed floats:

    szp3d.npz    x<i> (input volume, flattened), s<i> (stream)
    szp3d.json   per case: dims, bs, eb, kind, dec (digest)

Shapes cover whole and cut-short edge blocks on every axis, single-block
volumes and degenerate axes; block sides 2, 3, 4 and 8; smooth, noisy,
constant and wide-range (large rates) inputs; two error bounds.

Usage (where the reference checkout exists):  python tests/golden/make_golden_szp3d.py
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

SHAPES = [((7, 9, 11), 4), ((16, 16, 16), 4), ((13, 20, 33), 8), ((5, 5, 5), 8), ((1, 1, 40), 4),
          ((24, 17, 9), 2), ((10, 6, 14), 3)]
KINDS = ("smooth", "noisy", "const", "wide")


def volume(dims, kind, seed):
    rng = np.random.default_rng(seed)
    i, j, k = np.meshgrid(*[np.arange(d, dtype=np.float64) for d in dims], indexing="ij")
    base = np.sin(i / 5.0) + np.cos(j / 7.0) * np.sin(k / 3.0)
    x = {"smooth": base, "noisy": base + rng.normal(0, 0.3, dims), "const": np.full(dims, 2.5),
         "wide": base * 1e4 + rng.normal(0, 1e3, dims)}[kind]
    return x.astype(np.float32).ravel()


def main():
    zoracle.build(ref=True)
    if not zoracle.ref_available():
        sys.exit("the reference library is not available here")
    ref = zoracle.ref()
    arrays, cases = {}, []
    for si, (dims, bs) in enumerate(SHAPES):
        for ki, kind in enumerate(KINDS):
            x = volume(dims, kind, 100 * si + ki)
            for eb in (1e-2, 1e-4):
                s = ref.szp3d_compress(x, dims, bs, eb, "fast")
                assert s == ref.szp3d_compress(x, dims, bs, eb, "plain")
                y = ref.szp3d_decompress(s, dims, bs, eb)
                i = len(cases)
                arrays[f"x{i}"] = x
                arrays[f"s{i}"] = np.frombuffer(s, np.uint8)
                cases.append({"i": i, "dims": list(dims), "bs": bs, "eb": eb, "kind": kind,
                              "dec": hashlib.sha256(y.tobytes()).hexdigest()})
    np.savez_compressed(os.path.join(HERE, "szp3d.npz"), **arrays)
    with open(os.path.join(HERE, "szp3d.json"), "w") as f:
        json.dump({"cases": cases}, f, indent=1)
    print(len(cases), "cases")


if __name__ == "__main__":
    main()
