"""Generate the golden vectors in tests/golden/ from the REFERENCE codec.

Runs the reference's own compress / decompress / homomorphic-add
(``oracle/_ref/libzccl_ref.so``, compiled in place from the reference
sources by ``oracle/Makefile``) on seeded inputs and stores inputs, streams,
homomorphic sums and SHA-256 digests of the decompressed floats:

    golden.npz   arrays  in_<digest> (inputs, stored once), s<i> (stream of
                         case i's x), t<i> (stream of its y), h<i> (their
                         homomorphic sum)
    golden.json  per case: n, T, L, eb, kind, digests; plus the reference
                 host's width thresholds

Cases cover every remainder branch of the layout (grid of n, T, L), three
error bounds, constant / zero / large-magnitude / sign-alternating inputs,
and a P = 8 homomorphic reduction folded the way the ring folds it.  Cases
whose chunks would overflow the reference's per-thread scratch
(oracle/zoracle.py: ref_scratch_ok) are left out.

Usage (where the reference checkout exists):  python tests/golden/make_golden.py
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


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def smooth_noisy(n, seed, amp=3.0, noise=0.01):
    rng = np.random.default_rng(seed)
    i = np.arange(n, dtype=np.float64)
    x = amp * np.sin(i * 0.05 + seed) + 0.3 * np.sin(i * 0.31) + rng.normal(0, noise, n)
    return x.astype(np.float32)


def value_range(x):
    r = float(np.float32(x.max()) - np.float32(x.min()))
    return r if r > 0 else 1.0


def main():
    zoracle.build(ref=True)
    R = zoracle.ref()
    arrays, cases = {}, []

    P = zoracle.port()

    def add(kind, x, y, eb, L, T):
        n = x.size
        eb = float(np.float32(eb))
        # the port screens out cases that would overflow the reference's scratch
        sp, tp = P.compress(x, eb, L, T), P.compress(y, eb, L, T)
        hp = P.homadd(sp, tp, n, eb, L, T)
        if not all(zoracle.ref_scratch_ok(b, n, T) for b in (sp, tp, hp)):
            return
        s = R.compress(x, eb, L, T)
        t = R.compress(y, eb, L, T)
        h = R.homadd(s, t, n, eb, L, T)
        i = len(cases)
        kx, ky = "in_" + sha(x)[:16], "in_" + sha(y)[:16]  # inputs stored once
        arrays[kx] = x
        arrays[ky] = y
        arrays[f"s{i}"] = np.frombuffer(s, np.uint8)
        arrays[f"t{i}"] = np.frombuffer(t, np.uint8)
        arrays[f"h{i}"] = np.frombuffer(h, np.uint8)
        cases.append(dict(i=i, kind=kind, n=n, T=T, L=L, eb=eb, x=kx, y=ky,
                          dec_s=sha(R.decompress(s, n, eb, L, T)),
                          dec_h=sha(R.decompress(h, n, eb, L, T))))

    # every remainder branch: (tbs-1) % L, (rem-1) % L, tbs == 1, N == T
    for n in list(range(1, 81)) + [100, 127, 128, 129, 200, 255, 257, 1000, 4097]:
        for T in (1, 3, 8):
            if n < T:
                continue
            for L in (8, 32, 36):
                x = smooth_noisy(n, seed=n * 7 + T)
                y = smooth_noisy(n, seed=n * 7 + T + 1000, amp=2.0, noise=0.02)
                add("grid", x, y, 1e-3 * max(value_range(x), value_range(y)), L, T)

    # error bounds across three decades, several writer counts
    n = 32768 + 13
    x = smooth_noisy(n, seed=1, noise=0.05)
    y = smooth_noisy(n, seed=2, noise=0.05)
    rg = max(value_range(x), value_range(y))
    for T in (1, 8, 72):
        for rel in (1e-3, 1e-4, 1e-5):
            add("eb", x, y, rel * rg, 32, T)

    # special inputs
    n = 5000
    rng = np.random.default_rng(7)
    zeros = np.zeros(n, np.float32)
    const = np.full(n, 1.2345, np.float32)
    ramp = np.linspace(-50, 50, n).astype(np.float32)
    alt = (np.where(np.arange(n) % 2 == 0, 1.0, -1.0) * rng.uniform(0.5, 1.0, n)).astype(np.float32)
    big = rng.uniform(-1.0, 1.0, n).astype(np.float32)  # |x/eb| up to ~1e9: slow quantize path
    spiky = smooth_noisy(n, 3)
    spiky[::97] *= 1000.0
    for T in (1, 4):
        add("zeros", zeros, zeros, 1e-3, 32, T)
        add("const", const, const, 1e-4, 32, T)
        add("const_vs_noise", const, smooth_noisy(n, 9), 1e-3, 32, T)
        add("ramp", ramp, -ramp, 1e-3, 32, T)
        add("alternating", alt, alt[::-1].copy(), 1e-4, 32, T)
        add("large_q", big, big[::-1].copy(), 1e-9, 32, T)
        add("spiky", spiky, smooth_noisy(n, 4), 1e-4, 32, T)
        add("alternating_L36", alt, ramp, 1e-4, 36, T)

    # P = 8 reduction folded like the ring's reduce-scatter
    n, T, L, NP = 20000 + 3, 4, 32, 8
    base = smooth_noisy(n, seed=11, noise=0.0)
    chunks = [(base + np.random.default_rng(100 + r).normal(0, 0.05, n)).astype(np.float32)
              for r in range(NP)]
    eb = float(np.float32(1e-4 * max(value_range(c) for c in chunks)))
    streams = [R.compress(c, eb, L, T) for c in chunks]
    fold = R.homadd_fold(streams, n, eb, L, T)
    for r, c in enumerate(chunks):
        arrays[f"p8x{r}"] = c
    arrays["p8sum"] = np.frombuffer(fold, np.uint8)
    reduction = dict(n=n, T=T, L=L, P=NP, eb=eb, dec_sum=sha(R.decompress(fold, n, eb, L, T)))

    np.savez_compressed(os.path.join(HERE, "golden.npz"), **arrays)
    meta = dict(
        generator="tests/golden/make_golden.py",
        source="reference codec (ZCCL/src/ZCCL_float.c, ZCCLd_float.c, ZCCL_TypeManager.c)",
        width_thresholds=zoracle.width_thresholds(),
        cases=cases,
        reduction=reduction,
    )
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(meta, f, indent=0)
    print(f"{len(cases)} cases written")


if __name__ == "__main__":
    main()
