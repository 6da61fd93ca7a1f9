"""Seeded synthetic inputs of the measured workloads, shared by bench.py and
the parity tests so that both see the same floats.

* ``grf_lognormal(side, seed)``: a side^3 log-normal Gaussian random field,
  white noise shaped to P(k) ~ k^-3 in Fourier space, normalised to unit
  variance, then exp(1.5 g).  It stands in for the NYX 512^3 density fields
  the reference evaluates its codec on (ZCCL/jobs/evaluate_compressor_NYX.sh),
  which are not available here.
* ``rank_chunks(n, P, seed)``: P ranks' chunks of a ring allreduce, a shared
  smooth base (a sum of 8 random-phase sinusoids) plus each rank's own
  N(0, 0.05) perturbation from seed r.
* ``gradient_buckets(npairs, seed)``: gradient-bucket-like buffers, pairs of
  equal size, log-uniform sizes, Laplace(0, 1e-3) values, 5 % of them
  constant, an error bound per pair drawn from {1e-3, 1e-4, 1e-5} x range.

All generators run on the given torch device and return float32 tensors.
"""
from __future__ import annotations

import math

import numpy as np


def grf_lognormal(side: int, seed: int, device):
    """Flat float32 tensor of side^3 elements (z fastest)."""
    import torch
    g = torch.Generator(device=device).manual_seed(seed)
    kx = torch.fft.fftfreq(side, device=device)
    kz = torch.fft.rfftfreq(side, device=device)
    k2 = kx[:, None, None] ** 2 + kx[None, :, None] ** 2 + kz[None, None, :] ** 2
    amp = torch.where(k2 > 0, k2.clamp_min(1e-12) ** (-0.75), torch.zeros_like(k2))  # |k|^-1.5
    del k2
    shape = (side, side, side // 2 + 1)
    spec = torch.complex(torch.randn(shape, generator=g, device=device),
                         torch.randn(shape, generator=g, device=device)) * amp
    del amp
    f = torch.fft.irfftn(spec, s=(side, side, side))
    del spec
    f = (f - f.mean()) / f.std()
    return torch.exp(1.5 * f).reshape(-1).contiguous().float()


def rank_chunks(n: int, P: int, seed: int, device):
    """List of P float32 tensors of n elements."""
    import torch
    g = torch.Generator(device=device).manual_seed(seed)
    i = torch.arange(n, device=device, dtype=torch.float64)
    period = 500.0 + 49500.0 * torch.rand(8, generator=g, device=device, dtype=torch.float64)
    phase = 2 * math.pi * torch.rand(8, generator=g, device=device, dtype=torch.float64)
    base = torch.zeros(n, device=device, dtype=torch.float64)
    for k in range(8):
        base += torch.sin(2 * math.pi * i / period[k] + phase[k])
    del i
    xs = []
    for r in range(P):
        gr = torch.Generator(device=device).manual_seed(r)
        xs.append((base + 0.05 * torch.randn(n, generator=gr, device=device, dtype=torch.float64)).float())
    return xs


def error_bound(rel: float, *xs) -> float:
    """rel x (max - min) over all the tensors, rounded to float32 the way the
    reference's callers pass it (a float argument)."""
    lo = min(float(x.min()) for x in xs)
    hi = max(float(x.max()) for x in xs)
    return float(np.float32(rel * (hi - lo)))


class Buckets:
    """``gradient_buckets`` result: sizes[k] floats per buffer of pair k,
    xs[k] = [a, b] views into one device tensor, ebs[k] the pair's bound,
    const[k] whether the pair is constant."""

    def __init__(self, sizes, xs, ebs, const, data):
        self.sizes, self.xs, self.ebs, self.const, self.data = sizes, xs, ebs, const, data


def gradient_buckets(npairs: int, seed: int, device, lo_bytes: int = 4 << 10, hi_bytes: int = 16 << 20):
    """npairs pairs of equal-size float32 buffers, sizes log-uniform in
    [lo_bytes, hi_bytes] of float32, Laplace(0, 1e-3) values, 5 % of pairs
    constant (0.5 and 0.25), eb per pair from {1e-3, 1e-4, 1e-5} x the
    pair's range (at least 1e-3)."""
    import torch
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(lo_bytes // 4), np.log(hi_bytes // 4), npairs)).astype(np.int64)
    const = rng.random(npairs) < 0.05
    eb_rel = rng.choice([1e-3, 1e-4, 1e-5], npairs)
    total = int(2 * sizes.sum())
    data = torch.empty(total, dtype=torch.float32, device=device)
    g = torch.Generator(device=device).manual_seed(seed)
    u = (torch.rand(total, generator=g, device=device, dtype=torch.float32) - 0.5).clamp_(-0.4999999, 0.4999999)
    data.copy_(-1e-3 * torch.sign(u) * torch.log1p(-2 * u.abs()))  # Laplace(0, 1e-3)
    del u
    off, xs = 0, []
    for k in range(npairs):
        n = int(sizes[k])
        pair = [data[off: off + n], data[off + n: off + 2 * n]]
        off += 2 * n
        if const[k]:
            pair[0].fill_(0.5)
            pair[1].fill_(0.25)
        xs.append(pair)
    ebs = []
    for k in range(npairs):
        lo = min(float(xs[k][0].min()), float(xs[k][1].min()))
        hi = max(float(xs[k][0].max()), float(xs[k][1].max()))
        ebs.append(float(np.float32(eb_rel[k] * max(hi - lo, 1e-3))))
    return Buckets([int(s) for s in sizes], xs, ebs, [bool(c) for c in const], data)
