"""Bit-exact parity of the measured workloads' shapes with the oracle, on the
GPU through the C ABI, at sizes the oracle finishes in seconds:

* the log-normal Gaussian random field at 256^3 (the benchmark's 512^3
  field at an eighth of the size), eb = 1e-4 and 1e-3 of range, L = 32,
  T = 16: both compressed streams, their homomorphic sum, and the
  decompressed floats of a stream and of the sum;
* the gradient-bucket mix (log-uniform sizes, Laplace(0, 1e-3) values, 5 %
  constant pairs, eb per pair from three decades) compressed by one batch
  launch and summed pairwise by another: every whole stream and sum of 96
  pairs against the oracle's.
"""
from __future__ import annotations

import numpy as np
import pytest

import zccl_gb300 as Z
from zccl_gb300.workloads import error_bound, gradient_buckets, grf_lognormal

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    if not t.cuda.is_available():
        pytest.skip("no CUDA device")
    Z.lib()
    return t


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


@pytest.mark.parametrize("rel", [1e-4, 1e-3])
def test_lognormal_field_matches_oracle(torch, port, rel):
    side, L, T = 256, 32, 16
    x, y = grf_lognormal(side, 0, "cuda"), grf_lognormal(side, 1, "cuda")
    n = x.numel()
    eb = error_bound(rel, x, y)
    codec = Z.Codec(n, L, T)
    a, b = codec.compress(x, eb), codec.compress(y, eb)
    h = codec.homadd([a, b])
    da, dh = codec.decompress(a, eb), codec.decompress(h, eb)
    codec.check()
    xh, yh = x.cpu().numpy(), y.cpu().numpy()
    sa, sb = port.compress(xh, eb, L, T), port.compress(yh, eb, L, T)
    assert a.tobytes() == sa and b.tobytes() == sb
    sh = port.homadd(sa, sb, n, eb, L, T)
    assert h.tobytes() == sh
    assert np.array_equal(bits(da.cpu().numpy()), bits(port.decompress(sa, n, eb, L, T)))
    ref_h = port.decompress(sh, n, eb, L, T)
    assert np.array_equal(bits(dh.cpu().numpy()), bits(ref_h))
    # the error bounds, as properties (ulp slack for the float reconstruction)
    slack = 8 * float(np.spacing(np.float32(max(float(x.abs().max()), float(y.abs().max())) * 2)))
    assert float((da.double() - x.double()).abs().max()) <= eb + slack
    assert float((dh.double() - (x.double() + y.double())).abs().max()) <= 2 * eb + slack


def test_gradient_bucket_batch_matches_oracle(torch, port):
    npairs, L, T = 96, 32, 1
    bk = gradient_buckets(npairs, 3, "cuda", lo_bytes=4 << 10, hi_bytes=4 << 20)
    codecs = {}

    def codec(n):
        if n not in codecs:
            codecs[n] = Z.Codec(n, L, T)
        return codecs[n]

    trios = [[codec(n).new_stream() for _ in range(3)] for n in bk.sizes]
    bc = Z.Batch(Z.BATCH_COMPRESS, [(bk.xs[k][r], bk.ebs[k], T, trios[k][r])
                                    for k in range(npairs) for r in range(2)], L)
    bc.run()
    bc.check()
    bh = Z.Batch(Z.BATCH_HOMADD, [([trios[k][0], trios[k][1]], T, trios[k][2]) for k in range(npairs)], L)
    bh.run()
    bh.check()
    assert sum(bk.const) > 0  # the mix has constant pairs
    for k, n in enumerate(bk.sizes):
        a, b = bk.xs[k][0].cpu().numpy(), bk.xs[k][1].cpu().numpy()
        ra, rb = port.compress(a, bk.ebs[k], L, T), port.compress(b, bk.ebs[k], L, T)
        assert trios[k][0].tobytes() == ra, k
        assert trios[k][1].tobytes() == rb, k
        assert trios[k][2].tobytes() == port.homadd(ra, rb, n, bk.ebs[k], L, T), k
