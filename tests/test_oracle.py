"""Pin the oracle: the C restatement (oracle/zccl_port.c) must reproduce every
golden vector written by the reference codec, and agree with the reference
library itself wherever that library can run here."""
from __future__ import annotations

import hashlib

import numpy as np
import pytest

from oracle import zoracle


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def test_port_reproduces_golden_streams(golden, port):
    for c in golden.cases:
        n, T, L, eb = c["n"], c["T"], c["L"], c["eb"]
        s = port.compress(golden.x(c), eb, L, T)
        assert s == golden.stream(c, "s"), c
        t = port.compress(golden.y(c), eb, L, T)
        assert t == golden.stream(c, "t"), c
        assert port.homadd(s, t, n, eb, L, T) == golden.stream(c, "h"), c
        assert sha(port.decompress(s, n, eb, L, T)) == c["dec_s"], c
        assert sha(port.decompress(golden.stream(c, "h"), n, eb, L, T)) == c["dec_h"], c


def test_port_reproduces_golden_reduction(golden, port):
    r = golden.meta["reduction"]
    chunks = [golden.arr[f"p8x{k}"] for k in range(r["P"])]
    streams = [port.compress(x, r["eb"], r["L"], r["T"]) for x in chunks]
    fold = port.homadd_fold(streams, r["n"], r["eb"], r["L"], r["T"])
    assert fold == golden.arr["p8sum"].tobytes()
    assert sha(port.decompress(fold, r["n"], r["eb"], r["L"], r["T"])) == r["dec_sum"]


def test_fold_order_does_not_matter(golden, port):
    """The homomorphic sum is the canonical encoding of the summed deltas, so
    any fold order gives the same bytes (why a one-pass P-way add is exact)."""
    r = golden.meta["reduction"]
    chunks = [golden.arr[f"p8x{k}"] for k in range(r["P"])]
    streams = [port.compress(x, r["eb"], r["L"], r["T"]) for x in chunks]
    fwd = port.homadd_fold(streams, r["n"], r["eb"], r["L"], r["T"])
    bwd = port.homadd_fold(streams[::-1], r["n"], r["eb"], r["L"], r["T"])
    assert fwd == bwd


def test_width_thresholds_match_reference_host(golden, port):
    """glibc's log2f rounds 5,876 integers just below powers of two up to the
    power; the width table captured with the reference equals this host's."""
    thr = zoracle.width_thresholds(port.width)
    assert thr == golden.meta["width_thresholds"]
    assert sum((1 << w) - t for w, t in enumerate(thr) if t and w < 32) == 5876 - 2943
    assert port.width(2**21 - 1) == 22 and port.width(2**21 - 2) == 21


def error_slack(x, P=1):
    """Tolerance of the reference codec's error bound, elementwise: truncation
    keeps |x - q*eb| < P*eb exactly, and the float reciprocal (1.0f/eb) plus
    the float reconstruction (float)q*eb add a few ulps of |x|."""
    return 4.0 * np.spacing(np.abs(x).astype(np.float32)).astype(np.float64) * P


def test_error_bounds_on_golden(golden, port):
    for c in golden.cases[::7]:
        n, T, L, eb = c["n"], c["T"], c["L"], c["eb"]
        x, y = golden.x(c).astype(np.float64), golden.y(c).astype(np.float64)
        d = port.decompress(golden.stream(c, "s"), n, eb, L, T)
        assert np.all(np.abs(d - x) <= eb + error_slack(x)), c
        dh = port.decompress(golden.stream(c, "h"), n, eb, L, T)
        assert np.all(np.abs(dh - (x + y)) <= 2 * eb + error_slack(np.abs(x) + np.abs(y), 2)), c


@pytest.mark.skipif(not zoracle.ref_available(), reason="reference library not built on this host")
def test_port_matches_reference_library(port):
    R = zoracle.ref()
    rng = np.random.default_rng(5)
    for trial in range(60):
        n = int(rng.integers(50, 3000))
        T = int(rng.choice([1, 2, 5, 16]))
        L = int(rng.choice([4, 16, 32, 36, 64]))
        x = np.cumsum(rng.normal(0, 1, n)).astype(np.float32)
        y = np.cumsum(rng.normal(0, 1, n)).astype(np.float32)
        eb = float(np.float32(10 ** rng.uniform(-4, -1) * (x.max() - x.min())))
        s, t = port.compress(x, eb, L, T), port.compress(y, eb, L, T)
        h = port.homadd(s, t, n, eb, L, T)
        if not all(zoracle.ref_scratch_ok(b, n, T) for b in (s, t, h)):
            continue
        assert R.compress(x, eb, L, T) == s
        assert R.homadd(s, t, n, eb, L, T) == h
        assert np.array_equal(R.decompress(s, n, eb, L, T), port.decompress(s, n, eb, L, T))
