"""The request loop (zccl_gb300/serve.py): requests served concurrently and
batched as they arrive give the same streams and floats as the same
requests served alone, one at a time, with the plain calls; the budget
holds requests back; latency percentiles."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from zccl_gb300.serve import percentile


def test_percentile():
    assert percentile([], 50) is None
    assert percentile([3.0], 99) == 3.0
    v = list(range(1, 101))
    assert percentile(v, 50) in (50, 51) and percentile(v, 99) == 99


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    if not t.cuda.is_available():
        pytest.skip("no CUDA device")
    return t


def build(torch, budget, slots, batching, seed=0):
    from zccl_gb300.serve import COMPRESS, DECOMPRESS, HOMADD, Request, Server
    rng = np.random.default_rng(seed)
    base = torch.from_numpy(np.cumsum(rng.normal(0, 1, 1 << 20)).astype(np.float32)).cuda()
    eb = float(np.float32(1e-4 * float(base.max() - base.min())))
    srv = Server(budget, slots=slots, batching=batching, keep_results=True)
    groups = []
    for gi, n in enumerate([777, 20000, 100003]):
        T = 1 if gi == 0 else 3
        keys = []
        for r in range(5):
            off = int(rng.integers(0, base.numel() - n))
            srv.put((gi, r), base[off: off + n].clone(), eb, T)
            keys.append((gi, r))
        groups.append(keys)
    reqs = []
    for i in range(60):
        u = rng.random()
        t = float(rng.uniform(0, 0.004))
        if u < 0.5:
            n = int(np.exp(rng.uniform(np.log(50), np.log(300000))))
            off = int(rng.integers(0, base.numel() - n))
            reqs.append(Request(t, i, COMPRESS, x=base[off: off + n].clone(), eb=eb, T=int(rng.choice([1, 2]))))
        elif u < 0.8:
            g = groups[int(rng.integers(0, 3))]
            reqs.append(Request(t, i, DECOMPRESS, ins=[g[int(rng.integers(0, 5))]]))
        else:
            g = groups[int(rng.integers(0, 3))]
            P = int(rng.integers(2, 6))
            reqs.append(Request(t, i, HOMADD, ins=[g[int(k)] for k in rng.choice(len(g), P, replace=False)]))
    return srv, reqs


def alone(torch, srv, q):
    """The request served by itself with the plain calls."""
    import zccl_gb300 as Z
    from zccl_gb300.serve import COMPRESS, DECOMPRESS
    if q.kind == COMPRESS:
        c = Z.Codec(q.x.numel(), 32, q.T)
        s = c.compress(q.x, q.eb)
        c.check()
        return s.tobytes()
    rs = [srv.store[k] for k in q.ins]
    c = Z.Codec(rs[0].n, 32, rs[0].T)
    ins = []
    for r in rs:
        d = Z.DeviceStream(c, data=r.buf)
        d.index = r.index
        d.desc = Z.StreamDesc(r.buf.data_ptr(), r.buf.numel(), r.index.data_ptr(), r.desc.indexed,
                              r.desc.qprev_valid)
        ins.append(d)
    if q.kind == DECOMPRESS:
        y = c.decompress(ins[0], rs[0].eb)
        c.check()
        return y.cpu().numpy().view(np.uint32).tobytes()
    s = c.homadd(ins)
    c.check()
    return s.tobytes()


def served(q):
    from zccl_gb300 import lib
    from zccl_gb300.serve import DECOMPRESS
    if q.kind == DECOMPRESS:
        return q.result.cpu().numpy().view(np.uint32).tobytes()
    r = q.result
    size = ctypes.c_size_t(0)
    assert lib().zccl_gpu_stream_size(ctypes.byref(r.desc), r.n, 32, r.T, ctypes.byref(size), None) == 0
    return r.buf[: size.value].cpu().numpy().tobytes()


@pytest.mark.gpu
@pytest.mark.parametrize("batching,slots", [(True, 3), (False, 2)])
def test_results_same_alone_and_in_the_mix(torch, batching, slots):
    srv, reqs = build(torch, budget=1 << 30, slots=slots, batching=batching)
    for q in reqs:
        srv.submit(q)
    log = srv.run()
    assert len(log) == len(reqs) and srv.in_use == 0
    for q in reqs:
        assert q.done is not None and q.done >= q.arrival
        assert served(q) == alone(torch, srv, q), (q.kind, q.rid)
    lat = [q.done - q.arrival for q in reqs]
    assert percentile(lat, 50) <= percentile(lat, 99)


@pytest.mark.gpu
def test_budget_holds_requests_back(torch):
    # a budget for a few requests at a time: still every request completes, in full
    srv, reqs = build(torch, budget=4 << 20, slots=3, batching=True, seed=1)
    for q in reqs:
        srv.submit(q)
    log = srv.run()
    assert len(log) == len(reqs) and srv.in_use == 0
    for q in reqs:
        assert served(q) == alone(torch, srv, q), (q.kind, q.rid)


@pytest.mark.gpu
def test_units_overlap_on_the_device(torch):
    """Units on different slots run at the same time on the device: three
    8-way sums of 32M-element streams arriving together, one per slot, are
    all incomplete on the device at some enqueue, and their device intervals
    (start and end events) overlap.  The budget counts each unit's output and
    scratch, and every byte is returned."""
    from zccl_gb300.serve import HOMADD, Request, Server, device_overlap
    n = 1 << 25
    t = torch.arange(n, dtype=torch.float32, device="cuda")
    base = torch.sin(t * 1e-4) + 0.01 * torch.sin(t * 0.37)
    eb = float(np.float32(1e-4 * 2.0))
    srv = Server(8 << 30, slots=3, batching=False)
    keys = []
    for r in range(8):
        srv.put(r, torch.roll(base, 1000 * r), eb, 1)
        keys.append(r)
    del t
    for warm in range(2):  # the first pass grows the slots' scratch
        srv.units, srv.max_inflight, srv.log = [], 0, []
        for i in range(3):
            srv.submit(Request(0.0, 10 * warm + i, HOMADD, ins=keys))
        log = srv.run()
    assert len(log) == 3 and srv.in_use == 0
    ov = device_overlap(srv.units)
    assert srv.max_inflight >= 2, srv.max_inflight
    assert ov["max_concurrent"] >= 2 and ov["overlap_ms"] > 0, ov


def test_device_overlap_arithmetic():
    """Busy time, time with two units running and the peak concurrency, from
    start and end marks (event stand-ins)."""
    from zccl_gb300.serve import device_overlap

    class Mark:
        def __init__(self, t):
            self.t = t

        def elapsed_time(self, other):
            return other.t - self.t

    units = [(Mark(0.0), Mark(10.0), None), (Mark(5.0), Mark(12.0), None), (Mark(20.0), Mark(21.0), None)]
    ov = device_overlap(units)
    assert ov == {"span_ms": 21.0, "busy_ms": 13.0, "overlap_ms": 5.0, "max_concurrent": 2}
    assert device_overlap([])["max_concurrent"] == 0


def test_buffer_pool_stays_bounded():
    """Released output buffers go to a per-shape pool that keeps at most
    pool_bytes, dropping the oldest shapes first; a pooled buffer is reused
    for its shape.  Host-side logic, on stand-in buffers."""
    from zccl_gb300.serve import Resident, Server
    srv = Server.__new__(Server)
    srv._sizes, srv._pool, srv._pool_bytes, srv._pool_cap = {}, {}, 0, 1000
    srv._size = lambda n, T: (n, 10, 0)  # capacity n, index 10 bytes
    for n in (100, 200, 300, 100, 400):
        srv._release(Resident(n, 1.0, 1, object(), object(), None))
        assert srv._pool_bytes <= 1000
        assert srv._pool_bytes == sum(srv._size(*k)[0] + 10 for k, v in srv._pool.items() for _ in v)
    assert (400, 1) in srv._pool and all(v for v in srv._pool.values())
    srv._release(Resident(2000, 1.0, 1, object(), object(), None))  # larger than the pool: not kept
    assert (2000, 1) not in srv._pool


def test_admission_takes_the_oldest_kind_in_fifo_order():
    """Admission moves arrived requests to per-kind queues and forms each
    unit from the oldest arrived request and the next ones of its kind (up
    to max_batch, while they fit the budget); decompressions go alone.
    Host-side logic with a stand-in launch."""
    from collections import deque
    from zccl_gb300.serve import COMPRESS, DECOMPRESS, HOMADD, Request, Server
    srv = Server.__new__(Server)
    srv.queue, srv.inflight, srv.log = [], [], []
    srv.ready = {COMPRESS: deque(), DECOMPRESS: deque(), HOMADD: deque()}
    srv.free_slots, srv.batching, srv.max_batch = [0, 1, 2], True, 3
    srv.budget, srv.in_use = 100, 0
    srv.now = lambda: 10.0
    srv._bytes = lambda q: q.eb  # the request's size stands in the eb field
    units = []
    srv._launch = lambda slot, group: units.append([q.rid for q in group])
    import heapq
    kinds = [HOMADD, COMPRESS, COMPRESS, DECOMPRESS, COMPRESS, COMPRESS, COMPRESS, HOMADD]
    for i, k in enumerate(kinds):
        heapq.heappush(srv.queue, (float(i), i, Request(float(i), i, k, eb=10.0)))
    heapq.heappush(srv.queue, (99.0, 99, Request(99.0, 99, COMPRESS, eb=10.0)))  # not arrived yet
    srv._admit()
    assert units == [[0, 7], [1, 2, 4], [3]]  # oldest first; batches of up to 3; decompress alone
    assert srv.in_use == 60 and [q.rid for q in srv.ready[COMPRESS]] == [5, 6] and len(srv.queue) == 1
    srv.free_slots, srv.in_use = [0], 95  # the oldest does not fit: nothing is launched
    srv._admit()
    assert len(units) == 3 and [q.rid for q in srv.ready[COMPRESS]] == [5, 6]


@pytest.mark.gpu
@pytest.mark.parametrize("batching", [True, False])
def test_device_status_of_a_unit_is_raised(torch, batching):
    """A compression whose input holds a NaN reports ERANGE on the device
    (no fault); the loop reads the unit's status words when the unit ends
    and raises, whether the request went out in a compression batch or as
    a lone call."""
    import zccl_gb300 as Z
    from zccl_gb300.serve import COMPRESS, Request, Server
    n = 20000
    good = torch.linspace(-1, 1, n, device="cuda")
    bad = good.clone()
    bad[1234] = float("nan")
    srv = Server(1 << 30, slots=2, batching=batching)
    srv.submit(Request(0.0, 1, COMPRESS, x=good, eb=1e-3, T=1))
    srv.submit(Request(0.0, 2, COMPRESS, x=bad, eb=1e-3, T=1))
    with pytest.raises(Z.ZcclError) as e:
        srv.run()
    assert e.value.status == -3
