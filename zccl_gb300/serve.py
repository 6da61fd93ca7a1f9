"""A request loop over device-resident compressed buffers.

Requests -- compress a float buffer, decompress a resident stream, or add
2-8 resident streams homomorphically -- arrive over time.  The server keeps
the compressed buffers resident on the device and works with continuous
batching: every time it looks, it admits queued requests while a slot (a
CUDA stream with its own scratch) and the device-memory budget allow,
launches the queued compressions together as one batch and the queued sums
as another (one persistent launch each, zccl_gpu_batch_*), and a lone
request or a decompression with the ordinary calls.  Work on different
slots overlaps on the device; a request's latency runs from its arrival to
the completion event of the launch that carried it, and its bytes and slot
are released then.

The admission budget counts everything a request holds on the device while
it is in flight: its input floats (compress), its outputs (stream and side
index, or floats) and the scratch of its geometry.  Geometry sizes are
cached per shape, and released output buffers go back to a per-shape pool,
so admission makes no library size queries or allocator calls for shapes it
has seen.  Every unit of work is bracketed by device events, so the device
time of each unit and the overlap between units can be read back.

Results do not depend on the mix: every stream is the reference's byte
layout for its own input, and batching or concurrency changes only which
launch carries the work.
"""
from __future__ import annotations

import ctypes
import heapq
import time
import types
from collections import deque
from dataclasses import dataclass, field

from . import BATCH_COMPRESS, BATCH_HOMADD, Batch, StreamDesc, ZcclError, _check, lib

COMPRESS, DECOMPRESS, HOMADD = "compress", "decompress", "homadd"


@dataclass
class Resident:
    """A compressed stream kept on the device."""
    n: int
    eb: float
    T: int
    buf: object  # uint8 tensor, the wire bytes
    index: object  # uint8 tensor, the side index
    desc: StreamDesc


@dataclass(order=True)
class Request:
    arrival: float                          # seconds on the server's clock
    rid: int
    kind: str = field(compare=False)
    x: object = field(compare=False, default=None)       # compress: CUDA float tensor
    eb: float = field(compare=False, default=0.0)
    T: int = field(compare=False, default=1)
    ins: list = field(compare=False, default=None)       # decompress: [key]; homadd: keys
    # filled in by the server
    result: object = field(compare=False, default=None)  # Resident or float tensor
    done: float = field(compare=False, default=None)
    nbytes: int = field(compare=False, default=0)


class Server:
    """Continuous-batching request loop on one device.  With keep_results
    False a request's result is dropped once it completes (handed back), so
    device memory stays within the budget over a long run."""

    def __init__(self, budget_bytes: int, slots: int = 4, L: int = 32, device: str = "cuda",
                 batching: bool = True, keep_results: bool = False, pool_bytes: int = 1 << 30,
                 max_batch: int = 256):
        import torch
        self.torch = torch
        self.L, self.device, self.batching, self.keep = int(L), device, batching, keep_results
        self.budget, self.in_use = int(budget_bytes), 0
        self.streams = [torch.cuda.Stream(device=device) for _ in range(slots)]
        self.free_slots = list(range(slots))
        self.ws = [None] * slots  # per-slot scratch, grown on demand
        self.store: dict = {}     # key -> Resident
        self.queue: list = []     # (arrival, rid, Request) not yet arrived
        self.ready = {COMPRESS: deque(), DECOMPRESS: deque(), HOMADD: deque()}  # arrived, per kind
        self.max_batch = int(max_batch)
        self.inflight: list = []  # (event, slot, [requests], keep-alive objects)
        self.t0 = time.perf_counter()
        self.log: list = []
        self._sizes: dict = {}    # (n, T) -> (stream capacity, index bytes, workspace bytes)
        self._pool: dict = {}     # (n, T) -> released (buf, idx) pairs, oldest shape first
        self._pool_bytes, self._pool_cap = 0, int(pool_bytes)
        self.units: list = []     # (start event, end event, requests) of every unit launched
        self.max_inflight = 0     # most units incomplete on the device at one enqueue
        self.host_launch_s = 0.0  # host time spent enqueueing units

    # ---- resident buffers -------------------------------------------------
    def _size(self, n: int, T: int):
        """(stream capacity, index bytes, workspace bytes) of a geometry, cached."""
        key = (n, T)
        v = self._sizes.get(key)
        if v is None:
            v = (lib().zccl_gpu_max_stream_bytes(n, self.L, T), lib().zccl_gpu_index_bytes(n, self.L, T),
                 lib().zccl_gpu_workspace_bytes(n, self.L, T))
            if not v[0] or not v[1]:
                raise ZcclError(-1, f"geometry n={n} T={T}")
            self._sizes[key] = v
        return v

    def _stream_for(self, n: int, T: int):
        torch = self.torch
        cap, ib, _ = self._size(n, T)
        pool = self._pool.get((n, T))
        if pool:
            buf, idx = pool.pop()
            self._pool_bytes -= cap + ib
            if not pool:
                del self._pool[(n, T)]
        else:
            buf = torch.empty(cap, dtype=torch.uint8, device=self.device)
            idx = torch.zeros(ib, dtype=torch.uint8, device=self.device)
        return buf, idx, StreamDesc(buf.data_ptr(), cap, idx.data_ptr(), 0, 0)

    def _release(self, res) -> None:
        """Give a handed-back result's stream buffers to the pool, which
        keeps at most pool_bytes (the oldest shapes leave first)."""
        if not isinstance(res, Resident):
            return
        cap, ib, _ = self._size(res.n, res.T)
        if cap + ib > self._pool_cap:
            return
        while self._pool and self._pool_bytes + cap + ib > self._pool_cap:
            key = next(iter(self._pool))
            lst = self._pool[key]
            c, i, _ = self._size(*key)
            if lst:
                lst.pop()
                self._pool_bytes -= c + i
            if not lst:
                del self._pool[key]
        self._pool.setdefault((res.n, res.T), []).append((res.buf, res.index))
        self._pool_bytes += cap + ib

    def _workspace(self, slot: int, n: int, T: int):
        need = self._size(n, T)[2]
        ws = self.ws[slot]
        if ws is None or ws.numel() < need:
            ws = self.torch.zeros(need, dtype=self.torch.uint8, device=self.device)
            self.ws[slot] = ws
        return ws

    def put(self, key, x, eb: float, T: int = 1) -> Resident:
        """Compress x into a resident stream under `key` (setup, not a request)."""
        buf, idx, d = self._stream_for(x.numel(), T)
        st = self.torch.cuda.current_stream()
        ws = self._workspace(0, x.numel(), T)
        _check(lib().zccl_gpu_compress(ctypes.byref(d), x.data_ptr(), x.numel(), eb, self.L, T,
                                       ws.data_ptr(), ctypes.c_void_p(st.cuda_stream)), "compress")
        _check(lib().zccl_gpu_check(ws.data_ptr(), ctypes.c_void_p(st.cuda_stream)), "compress")
        r = Resident(x.numel(), eb, T, buf, idx, d)
        self.store[key] = r
        return r

    # ---- the loop ---------------------------------------------------------
    def now(self) -> float:
        return time.perf_counter() - self.t0

    def submit(self, req: Request) -> None:
        """Queue a request; one that could never fit the budget is refused."""
        if self._bytes(req) > self.budget:
            raise ValueError(f"request {req.rid} needs more than the {self.budget}-byte budget")
        heapq.heappush(self.queue, (req.arrival, req.rid, req))

    def _bytes(self, req: Request) -> int:
        """Device bytes the request holds while in flight: its input floats
        (compress), its outputs and the scratch of its geometry."""
        if req.kind == COMPRESS:
            n, T = req.x.numel(), req.T
            cap, ib, ws = self._size(n, T)
            return 4 * n + cap + ib + ws
        r = self.store[req.ins[0]]
        cap, ib, ws = self._size(r.n, r.T)
        if req.kind == DECOMPRESS:
            return 4 * r.n + ws
        return cap + ib + ws

    def _launch(self, slot: int, reqs: list) -> None:
        """Enqueue one unit of work (a batch or a lone request) on a slot."""
        h0 = time.perf_counter()
        torch = self.torch
        st = self.streams[slot]
        sp = ctypes.c_void_p(st.cuda_stream)
        keep = []
        kind = reqs[0].kind
        busy = sum(1 for u in self.inflight if not u[0].query())
        self.max_inflight = max(self.max_inflight, busy + 1)
        with torch.cuda.stream(st):
            ev0 = torch.cuda.Event(enable_timing=True)
            ev0.record(st)
            if kind == DECOMPRESS or len(reqs) == 1:
                for q in reqs:
                    if q.kind == COMPRESS:
                        buf, idx, d = self._stream_for(q.x.numel(), q.T)
                        ws = self._workspace(slot, q.x.numel(), q.T)
                        _check(lib().zccl_gpu_compress(ctypes.byref(d), q.x.data_ptr(), q.x.numel(), q.eb,
                                                       self.L, q.T, ws.data_ptr(), sp), "compress")
                        q.result = Resident(q.x.numel(), q.eb, q.T, buf, idx, d)
                    elif q.kind == DECOMPRESS:
                        r = self.store[q.ins[0]]
                        y = torch.empty(r.n, dtype=torch.float32, device=self.device)
                        ws = self._workspace(slot, r.n, r.T)
                        _check(lib().zccl_gpu_decompress(y.data_ptr(), ctypes.byref(r.desc), r.n, r.eb,
                                                         self.L, r.T, ws.data_ptr(), sp), "decompress")
                        q.result = y
                    else:
                        rs = [self.store[k] for k in q.ins]
                        buf, idx, d = self._stream_for(rs[0].n, rs[0].T)
                        arr = (StreamDesc * len(rs))(*[r.desc for r in rs])
                        ws = self._workspace(slot, rs[0].n, rs[0].T)
                        _check(lib().zccl_gpu_homadd(ctypes.byref(d), arr, len(rs), rs[0].n, self.L, rs[0].T,
                                                     ws.data_ptr(), sp), "homadd")
                        q.result = Resident(rs[0].n, rs[0].eb, rs[0].T, buf, idx, d)
                    keep.append(ws)
            elif kind == COMPRESS:
                jobs = []
                for q in reqs:
                    buf, idx, d = self._stream_for(q.x.numel(), q.T)
                    q.result = Resident(q.x.numel(), q.eb, q.T, buf, idx, d)
                    jobs.append((q.x, q.eb, q.T, types.SimpleNamespace(desc=d)))
                b = Batch(BATCH_COMPRESS, jobs, self.L, stream=st)
                b.run(st)
                keep.append(b)
            else:
                jobs = []
                for q in reqs:
                    rs = [self.store[k] for k in q.ins]
                    buf, idx, d = self._stream_for(rs[0].n, rs[0].T)
                    q.result = Resident(rs[0].n, rs[0].eb, rs[0].T, buf, idx, d)
                    ins = [types.SimpleNamespace(desc=r.desc) for r in rs]
                    out = types.SimpleNamespace(desc=d, codec=types.SimpleNamespace(n=rs[0].n))
                    jobs.append((ins, rs[0].T, out))
                b = Batch(BATCH_HOMADD, jobs, self.L, stream=st)
                b.run(st)
                keep.append(b)
            ev = torch.cuda.Event(enable_timing=True)
            ev.record(st)
        self.inflight.append((ev, slot, reqs, keep))
        self.units.append((ev0, ev, reqs))
        self.host_launch_s += time.perf_counter() - h0

    def _retire(self) -> None:
        still = []
        for ev, slot, reqs, keep in self.inflight:
            if ev.query():
                t = self.now()
                sp = ctypes.c_void_p(self.streams[slot].cuda_stream)
                for k in keep:  # device status of the unit
                    if isinstance(k, Batch):
                        k.check(self.streams[slot])
                    else:
                        _check(lib().zccl_gpu_check(k.data_ptr(), sp), "device status")
                for q in reqs:
                    q.done = t
                    self.in_use -= q.nbytes
                    if not self.keep:  # the result has been handed back: its memory is free
                        self._release(q.result)
                        q.result, q.x = None, None
                    self.log.append(q)
                self.free_slots.append(slot)
            else:
                still.append((ev, slot, reqs, keep))
        self.inflight = still

    def _admit(self) -> None:
        """Move arrived requests to their kind's FIFO, then fill free slots:
        the oldest arrived request and, with batching, the next ones of its
        kind (up to max_batch, while they fit the budget) form one unit.
        Costs O(arrived) per call, however long the backlog."""
        now = self.now()
        while self.queue and self.queue[0][0] <= now:
            _, _, q = heapq.heappop(self.queue)
            self.ready[q.kind].append(q)
        while self.free_slots:
            heads = [d[0] for d in self.ready.values() if d]
            if not heads:
                return
            head = min(heads, key=lambda q: (q.arrival, q.rid))
            dq = self.ready[head.kind]
            group = []
            while dq and len(group) < self.max_batch:
                q = dq[0]
                need = self._bytes(q)
                if self.in_use + need > self.budget:
                    break
                dq.popleft()
                q.nbytes = need
                self.in_use += need
                group.append(q)
                if not self.batching or q.kind == DECOMPRESS:
                    break
            if not group:
                return  # the oldest does not fit the budget yet
            self._launch(self.free_slots.pop(0), group)

    def _pending(self) -> bool:
        return bool(self.queue or self.inflight or any(self.ready.values()))

    def run(self, deadline: float | None = None) -> list:
        """Serve until every submitted request is done (or the deadline)."""
        while self._pending():
            self._retire()
            self._admit()
            if deadline is not None and self.now() > deadline:
                break
            if not self.free_slots:
                continue  # every slot busy: poll the units, so that a freed slot is refilled at once
            if self.inflight or (self.queue and self.queue[0][0] > self.now()):
                time.sleep(0.00005)
        self.torch.cuda.synchronize()
        self._retire()
        return self.log


def device_overlap(units) -> dict:
    """Device timeline of completed units (start and end events, as
    Server.units holds them): the span from the first start to the last end,
    the busy time (at least one unit running), the time with two or more
    running, and the most running at once."""
    if not units:
        return {"span_ms": 0.0, "busy_ms": 0.0, "overlap_ms": 0.0, "max_concurrent": 0}
    ref = units[0][0]
    marks = []
    for e0, e1, _ in units:
        a, b = ref.elapsed_time(e0), ref.elapsed_time(e1)
        marks.append((a, 1))
        marks.append((b, -1))
    marks.sort(key=lambda m: (m[0], m[1]))
    busy = over = 0.0
    cur = top = 0
    prev = marks[0][0]
    for t, d in marks:
        if cur >= 1:
            busy += t - prev
        if cur >= 2:
            over += t - prev
        cur += d
        top = max(top, cur)
        prev = t
    return {"span_ms": marks[-1][0] - marks[0][0], "busy_ms": busy, "overlap_ms": over, "max_concurrent": top}


def percentile(vals, p):
    """The p-th percentile (nearest rank) of vals, None when empty."""
    if not vals:
        return None
    s = sorted(vals)
    k = min(len(s) - 1, max(0, int(round(p / 100.0 * (len(s) - 1)))))
    return s[k]
