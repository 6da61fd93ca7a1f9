"""Batches (the zccl_gpu_batch_* calls): streams of many uneven buffers
compressed and summed in one persistent launch each, byte for byte the
same as one call per buffer, also when the launches replay from a CUDA
graph; argument checks without a device."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

import zccl_gb300 as Z


def test_batch_rejects_bad_jobs_without_device():
    lib = Z.lib()
    arr = (Z.BatchJobDesc * 1)()
    assert lib.zccl_gpu_batch_bytes(Z.BATCH_COMPRESS, arr, 1, 32) == 0  # null pointers
    assert lib.zccl_gpu_batch_bytes(7, arr, 1, 32) == 0                 # no such kind
    assert lib.zccl_gpu_batch_bytes(Z.BATCH_COMPRESS, arr, 0, 32) == 0  # empty
    d = Z.BatchDesc()
    assert lib.zccl_gpu_batch_run(ctypes.byref(d), None) == -1          # never planned


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    if not t.cuda.is_available():
        pytest.skip("no CUDA device")
    Z.lib()
    return t


def buckets(torch, seed=0):
    """Pairs of equal-size buffers of uneven sizes (a few floats to a few
    hundred thousand), Laplace values, some constant, per-pair eb and T.
    The last two pairs have T = 1 and several full tiles: one in aligned
    buffers (its full tiles arrive as TMA boxes through the job's own tensor
    map), one in buffers that start 4 bytes past an aligned address (no
    tensor map, every tile copied into padded rows)."""
    rng = np.random.default_rng(seed)
    sizes = [5, 17, 31, 32, 33, 64, 1000, 4097, 8193, 65537] + [int(v) for v in np.exp(rng.uniform(np.log(40), np.log(400000), 20))]
    sizes += [3 * 8192 + 7, 3 * 8192 + 7]
    pairs = []
    for k, n in enumerate(sizes):
        T = int(rng.choice([1, 1, 3, 4])) if n >= 4 else 1
        shift = 1 if k == len(sizes) - 1 else 0
        if k >= len(sizes) - 2:
            T = 1
        xs = []
        for r in range(2):
            if k % 9 == 4 and k < len(sizes) - 2:
                x = np.full(n, 0.25 * (r + 1), np.float32)
            else:
                x = rng.laplace(0, 1e-3, n).astype(np.float32)
            xs.append(torch.from_numpy(np.concatenate([np.zeros(shift, np.float32), x])).cuda()[shift:])
        rng_ = max(float(max(x.max() for x in xs) - min(x.min() for x in xs)), 1e-3)
        eb = float(np.float32(float(rng.choice([1e-3, 1e-4, 1e-5])) * rng_))
        pairs.append((n, T, eb, xs))
    return pairs


@pytest.mark.gpu
def test_batch_matches_single_calls_and_graph_replay(torch):
    pairs = buckets(torch)
    codecs = {}
    singles, comp_jobs, sum_jobs, outs = [], [], [], []
    for n, T, eb, xs in pairs:
        c = codecs.setdefault((n, T), Z.Codec(n, 32, T))
        a = [c.compress(x, eb) for x in xs]
        singles.append((a, c.homadd(a)))
        c.check()
        bo = [c.new_stream() for _ in xs]
        comp_jobs += [(x, eb, T, o) for x, o in zip(xs, bo)]
        so = c.new_stream()
        sum_jobs.append((bo, T, so))
        outs.append((bo, so))
    bc = Z.Batch(Z.BATCH_COMPRESS, comp_jobs)
    bh = Z.Batch(Z.BATCH_HOMADD, sum_jobs)
    assert bc.desc.rows_off != 0  # some jobs have tensor maps

    def check_all():
        for (a, s), (bo, so) in zip(singles, outs):
            for x, y in zip(a, bo):
                assert y.tobytes() == x.tobytes()
                assert torch.equal(y.index, x.index)
            assert so.tobytes() == s.tobytes()
            assert torch.equal(so.index, s.index)

    bc.run()
    bh.run()
    bc.check()
    bh.check()
    check_all()
    # the autotuner picks a grid; the output stays the same
    bc.tune()
    bh.tune()
    bc.run()
    bh.run()
    check_all()
    # both launches recorded into one CUDA graph and replayed
    for bo, so in outs:
        so.buf.zero_()
        for y in bo:
            y.buf.zero_()
    g = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.graph(g, stream=side, capture_error_mode="relaxed"):
        bc.run(side)
        bh.run(side)
    g.replay()
    torch.cuda.synchronize()
    bc.check()
    bh.check()
    check_all()


@pytest.mark.gpu
def test_batch_one_cta_uneven_sums_wrap_the_ring(torch):
    """One CTA takes every tile in ticket order, so packed sums of very
    different sizes follow each other through its output ring: a small sum
    (widths 8) and then one of widths 23, too large for the rest of the ring
    and larger than the part the small one used, which has to start at the
    ring's beginning once everything before it is out."""
    rng = np.random.default_rng(9)
    n, T, eb = 8193, 1, 1.0  # one full tile per buffer; integer values are exact
    codec = Z.Codec(n, 32, T)
    jobs, singles = [], []
    for w in (6, 21, 6, 21, 21, 6):
        xs = [torch.from_numpy(rng.integers(-(1 << (w - 1)), 1 << (w - 1), n).astype(np.float32)).cuda()
              for _ in range(2)]
        ins = [codec.compress(x, eb) for x in xs]
        singles.append(codec.homadd(ins))
        jobs.append((ins, T, codec.new_stream()))
    codec.check()
    bh = Z.Batch(Z.BATCH_HOMADD, jobs)
    bh.desc.grid = 1
    bh.run()
    bh.check()
    for (ins, _, out), s in zip(jobs, singles):
        assert out.tobytes() == s.tobytes()
        assert torch.equal(out.index, s.index)
