"""The segmented compressed ring allgatherv run for P ranks on one device
(zccl_gb300/allgather.py) against the same allgatherv run by the oracle on
the CPU: the frames (size prefix and stream bytes) bit for bit, every
rank's receive buffer bit for bit (its own chunk the original floats, the
others decompressed from wire bytes).  The segment rule runs on the CPU."""
from __future__ import annotations

import numpy as np
import pytest

from zccl_gb300.allgather import SEGSIZE, segments


def test_segments_follow_the_reference():
    # SEGSIZE bytes of floats each, the last one the rest (ZCCL_ring.c:1666-1670)
    assert SEGSIZE == 8 * 1024 * 1024
    assert segments(5 * 1024 * 1024) == ([2097152, 2097152, 1048576], [0, 2097152, 4194304])
    assert segments(2097152) == ([2097152], [0])
    assert segments(10, segsize=16) == ([4, 4, 2], [0, 4, 8])
    assert segments(0) == ([], [])


def test_segments_shorter_than_the_writer_count_are_refused():
    # a segment of n < T floats leaves a writer without elements, which the
    # reference's chunking does not allow (tbs = n / T must be >= 1)
    from zccl_gb300.allgather import SegmentedAllgatherv
    with pytest.raises(ValueError):
        SegmentedAllgatherv([2 * 1024 * 1024 + 5], T=16)


def oracle_allgatherv(port, xs, eb, L, T, segsize, fixed=False):
    comp = port.compress_fixed if fixed else port.compress
    decomp = port.decompress_fixed if fixed else port.decompress
    frames = []
    for x in xs:
        cnts, offs = segments(x.size, segsize)
        fr = []
        for n, o in zip(cnts, offs):
            s = comp(np.ascontiguousarray(x[o: o + n]), eb, L, T)
            fr.append(len(s).to_bytes(8, "little") + s)
        frames.append(fr)
    recv = []
    for r in range(len(xs)):
        parts = []
        for c, x in enumerate(xs):
            if c == r:
                parts.append(x)
            else:
                cnts, _ = segments(x.size, segsize)
                parts += [decomp(f[8:], n, eb, L, T) for f, n in zip(frames[c], cnts)]
        recv.append(np.concatenate(parts))
    return frames, recv


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    if not t.cuda.is_available():
        pytest.skip("no CUDA device")
    return t


def frame_bytes(f):
    a = f.cpu().numpy()
    size = int(np.frombuffer(a[:8].tobytes(), "<u8")[0])
    return a[: 8 + size].tobytes()


@pytest.mark.gpu
@pytest.mark.parametrize("counts,T,segsize", [([70000, 65536, 50001, 80003], 3, 64 * 1024),
                                              ([3 * 1024 * 1024, 2 * 1024 * 1024 + 37], 16, SEGSIZE)])
def test_segmented_allgatherv_matches_oracle(torch, port, counts, T, segsize):
    from zccl_gb300.allgather import SegmentedAllgatherv
    L = 32
    rng = np.random.default_rng(len(counts))
    xs = [np.cumsum(rng.normal(0, 0.01, c)).astype(np.float32) for c in counts]
    eb = float(np.float32(1e-4 * (max(x.max() for x in xs) - min(x.min() for x in xs))))
    ag = SegmentedAllgatherv(counts, L, T, segsize=segsize)
    ys = ag.run([torch.from_numpy(x).cuda() for x in xs], eb, per_rank_outputs=True)
    frames, recv = oracle_allgatherv(port, xs, eb, L, T, segsize)
    for c in range(len(xs)):
        assert len(ag.sent[c]) == len(frames[c])
        for f, g in zip(ag.sent[c], frames[c]):
            assert frame_bytes(f) == g
    for r, y in enumerate(ys):
        assert np.array_equal(y.cpu().numpy().view(np.uint32), recv[r].view(np.uint32)), r
    xd = [torch.from_numpy(x).cuda() for x in xs]
    y0 = ag.run(xd, eb)  # rank 0 only
    assert np.array_equal(y0.cpu().numpy().view(np.uint32), recv[0].view(np.uint32))
    g, yg = ag.capture(xd, eb)  # the same exchange replayed from a CUDA graph
    yg.zero_()
    g.replay()
    torch.cuda.synchronize()
    ag.check()
    assert np.array_equal(yg.cpu().numpy().view(np.uint32), recv[0].view(np.uint32))


@pytest.mark.gpu
def test_segmented_allgatherv_fixed_rate_matches_oracle(torch, port):
    """The appendix variant (ZCCL/src/ZCCL_appendix.c:756-941): the same
    frames with the fixed-rate codec."""
    from zccl_gb300.allgather import SegmentedAllgatherv
    counts, T, L, segsize = [48000, 40000, 36000], 4, 32, 64 * 1024
    rng = np.random.default_rng(5)
    xs = [np.cumsum(rng.normal(0, 0.01, c)).astype(np.float32) for c in counts]
    eb = float(np.float32(1e-4 * (max(x.max() for x in xs) - min(x.min() for x in xs))))
    ag = SegmentedAllgatherv(counts, L, T, segsize=segsize, fixed=True)
    ys = ag.run([torch.from_numpy(x).cuda() for x in xs], eb, per_rank_outputs=True)
    frames, recv = oracle_allgatherv(port, xs, eb, L, T, segsize, fixed=True)
    for c in range(len(xs)):
        for f, g in zip(ag.sent[c], frames[c]):
            assert frame_bytes(f) == g
    for r, y in enumerate(ys):
        assert np.array_equal(y.cpu().numpy().view(np.uint32), recv[r].view(np.uint32)), r
