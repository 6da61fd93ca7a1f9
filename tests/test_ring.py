"""The compressed ring allreduce run for P ranks on one device
(zccl_gb300/ring.py) against the same ring run by the oracle on the CPU:
reduced compressed chunks bit for bit, the allreduced floats bit for bit,
every rank's copy alike, and the error bounds of the homomorphic sum
(P * eb) next to decompress-add-recompress.  The chunking rule runs on
the CPU."""
from __future__ import annotations

import numpy as np
import pytest

from zccl_gb300.ring import ring_counts


def test_ring_counts_follow_the_reference():
    # ceil(count / P) per chunk, the last one shorter (ZCCL_ring_ho.c:219-233)
    assert ring_counts(80011, 8) == ([10002] * 7 + [9997], [10002 * i for i in range(8)])
    assert ring_counts(64, 8) == ([8] * 8, [8 * i for i in range(8)])
    cnts, displs = ring_counts(10, 4)
    assert cnts == [3, 3, 3, 1] and displs == [0, 3, 6, 9]
    cnts, _ = ring_counts(5, 4)  # 2 + 2 + 1 + nothing
    assert cnts == [2, 2, 1, 0]


def rank_data(count, P, seed=0):
    """P ranks' arrays: a shared smooth base (8 random-phase sinusoids) plus
    a rank's own N(0, 0.05) from seed r."""
    rng = np.random.default_rng(seed)
    i = np.arange(count, dtype=np.float64)
    base = sum(np.sin(2 * np.pi * i / rng.uniform(500, 50000) + rng.uniform(0, 2 * np.pi))
               for _ in range(8))
    return [(base + np.random.default_rng(r).normal(0, 0.05, count)).astype(np.float32) for r in range(P)]


def oracle_ring_ho(port, xs, eb, L, T, P):
    cnts, displs = ring_counts(xs[0].size, P)
    chunk = lambda x, c: np.ascontiguousarray(x[displs[c]: displs[c] + cnts[c]])
    S = [[port.compress(chunk(xs[r], c), eb, L, T) for c in range(P)] for r in range(P)]
    for i in range(P - 1):
        for r in range(P):
            src, c = (r - 1) % P, (r - 2 - i) % P
            S[r][c] = port.homadd(S[src][c], S[r][c], cnts[c], eb, L, T)
    reduced = [S[c][c] for c in range(P)]
    y = np.concatenate([port.decompress(reduced[c], cnts[c], eb, L, T) for c in range(P)])
    return reduced, y


def oracle_ring_doc(port, xs, eb, L, T, P):
    cnts, displs = ring_counts(xs[0].size, P)
    acc = [x.copy() for x in xs]
    sl = lambda c: slice(displs[c], displs[c] + cnts[c])
    for i in range(P - 1):
        msgs = [port.compress(np.ascontiguousarray(acc[r][sl((r - 1 - i) % P)]), eb, L, T) for r in range(P)]
        for r in range(P):
            src, c = (r - 1) % P, (r - 2 - i) % P
            acc[r][sl(c)] += port.decompress(msgs[src], cnts[c], eb, L, T)
    reduced = [port.compress(np.ascontiguousarray(acc[c][sl(c)]), eb, L, T) for c in range(P)]
    y = np.concatenate([port.decompress(reduced[c], cnts[c], eb, L, T) for c in range(P)])
    return reduced, y


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    if not t.cuda.is_available():
        pytest.skip("no CUDA device")
    return t


@pytest.mark.gpu
@pytest.mark.parametrize("count,P,T,batched", [(80011, 8, 3, True), (24000, 4, 1, True), (80011, 8, 3, False)])
def test_homomorphic_ring_matches_oracle(torch, port, count, P, T, batched):
    from zccl_gb300.ring import RingAllreduce
    L = 32
    xs = rank_data(count, P)
    eb = float(np.float32(1e-4 * (max(x.max() for x in xs) - min(x.min() for x in xs))))
    ring = RingAllreduce(count, P, L, T, batched=batched)
    ys = ring.homomorphic([torch.from_numpy(x).cuda() for x in xs], eb, per_rank_outputs=True)
    reduced, y_ref = oracle_ring_ho(port, xs, eb, L, T, P)
    for c in range(P):
        assert ring.reduced[c].tobytes() == reduced[c], c
    for y in ys:  # every rank ends with the same floats
        assert np.array_equal(y.cpu().numpy().view(np.uint32), y_ref.view(np.uint32))
    exact = np.sum([x.astype(np.float64) for x in xs], axis=0)
    err = np.abs(y_ref.astype(np.float64) - exact).max()
    assert err <= P * eb + 8 * np.spacing(np.float32(np.abs(exact).max())), (err, eb)


@pytest.mark.gpu
@pytest.mark.parametrize("batched", [True, False])
def test_doc_ring_matches_oracle(torch, port, batched):
    from zccl_gb300.ring import RingAllreduce
    count, P, T, L = 80011, 8, 3, 32
    xs = rank_data(count, P, seed=1)
    eb = float(np.float32(1e-4 * (max(x.max() for x in xs) - min(x.min() for x in xs))))
    ring = RingAllreduce(count, P, L, T, batched=batched)
    ys = ring.doc([torch.from_numpy(x).cuda() for x in xs], eb, per_rank_outputs=True)
    reduced, y_ref = oracle_ring_doc(port, xs, eb, L, T, P)
    for c in range(P):
        assert ring.reduced[c].tobytes() == reduced[c], c
    for y in ys:
        assert np.array_equal(y.cpu().numpy().view(np.uint32), y_ref.view(np.uint32))


@pytest.mark.gpu
def test_batched_ring_repeats_and_keeps_variants_apart(torch, port):
    """Repeated calls replay the cached batches and give the same floats;
    the two variants' results live in different buffers."""
    from zccl_gb300.ring import RingAllreduce
    count, P, T, L = 50021, 4, 2, 32
    xs = rank_data(count, P, seed=6)
    eb = float(np.float32(1e-4 * (max(x.max() for x in xs) - min(x.min() for x in xs))))
    ring = RingAllreduce(count, P, L, T)
    xd = [torch.from_numpy(x).cuda() for x in xs]
    _, y_ho = oracle_ring_ho(port, xs, eb, L, T, P)
    _, y_doc = oracle_ring_doc(port, xs, eb, L, T, P)
    for _ in range(2):
        a = ring.homomorphic(xd, eb)
        b = ring.doc(xd, eb)
        assert np.array_equal(a.cpu().numpy().view(np.uint32), y_ho.view(np.uint32))
        assert np.array_equal(b.cpu().numpy().view(np.uint32), y_doc.view(np.uint32))


@pytest.mark.gpu
def test_decompress_accumulate_and_decompress_batch(torch, port):
    """acc += decompress(stream) in one pass equals the float sum of the
    oracle's floats; a decompression batch of uneven streams (one of them
    accumulating) equals the oracle's floats."""
    import zccl_gb300 as Z
    rng = np.random.default_rng(14)
    L = 32
    sizes = [(5, 1), (33, 1), (8193, 2), (100003, 4), (300001, 3)]
    streams, refs, ys, jobs = [], [], [], []
    for k, (n, T) in enumerate(sizes):
        x = np.cumsum(rng.normal(0, 0.05, n)).astype(np.float32)
        eb = float(np.float32(1e-4 * (float(x.max() - x.min()) + 1e-3)))
        codec = Z.Codec(n, L, T)
        s = codec.compress(torch.from_numpy(x).cuda(), eb)
        sx = port.compress(x, eb, L, T)
        assert s.tobytes() == sx
        ref = port.decompress(sx, n, eb, L, T)
        base = rng.normal(0, 1.0, n).astype(np.float32)
        acc = torch.from_numpy(base.copy()).cuda()
        codec.decompress_accumulate(s, eb, acc)
        codec.check()
        assert np.array_equal(acc.cpu().numpy().view(np.uint32), (base + ref).view(np.uint32)), n
        accumulate = k == 3
        y = torch.from_numpy(base.copy()).cuda() if accumulate else torch.full((n,), np.nan, device="cuda")
        jobs.append((s, eb, T, y, accumulate))
        refs.append(base + ref if accumulate else ref)
        ys.append(y)
    b = Z.Batch(Z.BATCH_DECOMPRESS, jobs, L)
    b.run()
    b.check()
    for y, ref in zip(ys, refs):
        assert np.array_equal(y.cpu().numpy().view(np.uint32), ref.view(np.uint32))


@pytest.mark.gpu
def test_one_shot_reductions_match_oracle(torch, port):
    import zccl_gb300 as Z
    from zccl_gb300.ring import PairwiseTree, reduce_doc, reduce_homomorphic, reduce_pairwise
    n, P, T, L = 100003, 8, 4, 32
    xs = rank_data(n, P, seed=2)
    eb = float(np.float32(1e-4 * (max(x.max() for x in xs) - min(x.min() for x in xs))))
    codec = Z.Codec(n, L, T)
    streams = [codec.compress(torch.from_numpy(x).cuda(), eb) for x in xs]
    host = [port.compress(x, eb, L, T) for x in xs]
    for s, h in zip(streams, host):
        assert s.tobytes() == h
    fold = port.homadd_fold(host, n, eb, L, T)
    assert reduce_homomorphic(codec, streams).tobytes() == fold
    assert reduce_pairwise(codec, streams).tobytes() == fold
    tree = PairwiseTree(codec, streams)
    assert len(tree.plans) == 3
    assert tree.run().tobytes() == fold
    assert tree.run().tobytes() == fold  # replayed
    tree.check()
    # an odd count: the odd one out goes up a level unchanged
    tree5 = PairwiseTree(codec, streams[:5])
    assert len(tree5.plans) == 3 and len(tree5.sums) == 4
    assert tree5.run().tobytes() == port.homadd_fold(host[:5], n, eb, L, T)
    tree5.check()
    doc, _ = reduce_doc(codec, streams, eb)
    total = np.zeros(n, np.float32)
    for h in host:
        total += port.decompress(h, n, eb, L, T)
    assert doc.tobytes() == port.compress(total, eb, L, T)
    codec.check()


@pytest.mark.gpu
@pytest.mark.parametrize("variant", ["homomorphic", "doc"])
def test_ring_raises_on_an_early_failed_step(torch, variant):
    """An error in the first step (a compressed chunk written into a stream
    too small for it) must surface when the ring returns, although many
    later calls run on the same codec before it checks."""
    import zccl_gb300 as Z
    from zccl_gb300.ring import RingAllreduce
    count, P, T, L = 24000, 4, 1, 32
    xs = rank_data(count, P, seed=4)
    eb = float(np.float32(1e-4 * (max(x.max() for x in xs) - min(x.min() for x in xs))))
    ring = RingAllreduce(count, P, L, T)
    cd = ring.codec(0)
    orig, calls = cd.new_stream, [0]

    def first_too_small(capacity=None):
        calls[0] += 1
        return orig(64) if calls[0] == 1 else orig(capacity)

    cd.new_stream = first_too_small
    with pytest.raises(Z.ZcclError):
        getattr(ring, variant)([torch.from_numpy(x).cuda() for x in xs], eb)
    assert calls[0] > 1
