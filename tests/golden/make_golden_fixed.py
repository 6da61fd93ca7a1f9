"""Generate the golden vectors of the fixed-rate appendix codec in tests/golden/.

Runs the reference's ZCCL_float_openmp_threadblock_arg_2 and
ZCCL_float_decompress_openmp_threadblock_arg_2 (ZCCL/src/ZCCL_appendix.c:65-590,
from ``oracle/_ref/libzccl_ref.so``) on seeded inputs and stores, per case,
the input, the stream and the SHA-256 of the decompressed floats:

    fixed.npz    x<i> (input), s<i> (stream)
    fixed.json   per case: n, T, L, eb, kind, dec (digest)

The reference's compressor writes the remainder segment's tail block with
the regular segments' tail count (ZCCL_appendix.c:318-330 passes
num_remainder_in_tb where its decompressor reads num_remainder_in_rm), so
for geometries where the two differ its streams do not decode, and where
the regular count is 0 it overruns a heap buffer.  Only geometries without
that mismatch are recorded; there both sides of the reference agree.

Usage (where the reference checkout exists):  python tests/golden/make_golden_fixed.py
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


def self_consistent(n, T, L):
    """The reference writes a readable stream for this geometry."""
    tbs, rem = n // T, n % T
    if rem == 0:
        return True
    tb_rem, rm_rem = (tbs - 1) % L, (rem - 1) % L
    return rm_rem == 0 or rm_rem == tb_rem


def main():
    zoracle.build(ref=True)
    if not zoracle.ref_available():
        sys.exit("the reference library is not available here")
    ref = zoracle.ref()
    rng = np.random.default_rng(11)
    arrays, cases = {}, []
    for n in (97, 1000, 4097):
        for T in (1, 3, 8):
            for L in (8, 32, 36):
                if not self_consistent(n, T, L):
                    continue
                for kind in ("smooth", "wide", "const"):
                    x = {"smooth": np.cumsum(rng.normal(0, 0.1, n)), "wide": rng.normal(0, 1, n) * 1e3,
                         "const": np.full(n, 3.0)}[kind].astype(np.float32)
                    for ebr in (1e-2, 1e-5):
                        eb = float(np.float32(ebr * max(float(x.max() - x.min()), 1.0)))
                        s = ref.compress_fixed(x, eb, L, T)
                        if not zoracle.ref_scratch_ok(s, n, T):
                            continue
                        y = ref.decompress_fixed(s, n, eb, L, T)
                        i = len(cases)
                        arrays[f"x{i}"] = x
                        arrays[f"s{i}"] = np.frombuffer(s, np.uint8)
                        cases.append({"i": i, "n": n, "T": T, "L": L, "eb": eb, "kind": kind,
                                      "dec": hashlib.sha256(y.tobytes()).hexdigest()})
    np.savez_compressed(os.path.join(HERE, "fixed.npz"), **arrays)
    with open(os.path.join(HERE, "fixed.json"), "w") as f:
        json.dump({"cases": cases}, f, indent=1)
    print(len(cases), "cases")


if __name__ == "__main__":
    main()
