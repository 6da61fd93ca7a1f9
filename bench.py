#!/usr/bin/env python
"""Throughput of the fastmode1 hot path on one GB300 (or N, as replicas).

Workload: a 512^3 float32 field (512 MiB), a log-normal Gaussian random
field with P(k) ~ k^-3 (exp(1.5 g)), error bound eb = 1e-4 * range, block
size 32, writer thread count T = the host's core count.  One step is one
pass of the hot path over it:

    compress(field A) -> decompress(that stream) -> homomorphic add of that
    stream and the (resident) stream of a second field B.

value  = uncompressed bytes handled per second, 3 * 4N per step (GB/s), the
         reference's own convention (one input's bytes per operation),
         device-resident inputs, CUDA events on the launching stream.
e2e    = the same step through the reference-facing C-ABI entry points with
         host buffers in pinned memory (host->device and device->host copies
         inside); e2e.pageable_value the same with ordinary pageable arrays.
roofline: algorithmic bytes of the dominant kernel per launch over its mean
         event-timed duration, against the measured HBM copy bandwidth.
cpu_baseline: the oracle's C restatement of the reference codec with every
         host core, on the same field.
parity: the GPU streams, homomorphic sums and decompressed floats of the
         timed field (at eb = 1e-4 and 1e-3 of range) and of the P = 8 x 16M
         reduction compared byte for byte with the oracle on the same
         inputs; a mismatch fails the run after the line is printed.

Launched as ``python bench.py --gpus N --steps K --warmup W``; for N > 1
under torchrun every rank compresses its own field (weak scaling, no
collective on the data path).  ``--impl reference`` times the CPU codec
instead.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "compress/decompress/homo-add GB/s vs HBM peak; batched speedup; p50/p99 at eb=1e-4"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=300)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--side", type=int, default=512)
    p.add_argument("--eb-rel", type=float, default=1e-4)
    p.add_argument("--L", type=int, default=32)
    p.add_argument("--T", type=int, default=0, help="writer thread count (default: host cores)")
    p.add_argument("--e2e-steps", type=int, default=3)
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-parity", action="store_true", help="skip the byte-for-byte checks against the oracle")
    p.add_argument("--no-extras", action="store_true",
                   help="skip the P-way reduction, batched and serving measurements")
    p.add_argument("--extras", default="reduction,szp3d,batched,serving",
                   help="comma-separated extra measurements to run")
    p.add_argument("--red-n", type=int, default=1 << 24, help="floats per rank chunk (reduction)")
    p.add_argument("--red-p", type=int, default=8, help="ranks (reduction)")
    p.add_argument("--batch-pairs", type=int, default=2048, help="buffer pairs (batched)")
    p.add_argument("--serve-side", type=int, default=400, help="side of the serving field")
    p.add_argument("--serve-slots", type=int, default=4)
    p.add_argument("--serve-secs", type=float, default=2.0, help="arrival window per load point")
    p.add_argument("--serve-max", type=int, default=60000, help="most requests per load point")
    return p.parse_args()


def host_cores() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


# dram__bytes_read.sum + dram__bytes_write.sum of one launch of each kernel on
# the 512^3 field at eb = 1e-4 * range, L = 32 (ncu, one pass, a warm step)
DRAM_TRAFFIC_512 = {"compress": 614956288, "decompress": 564624896, "homadd": 250268160}


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def make_field(side: int, seed: int, device):
    from zccl_gb300.workloads import grf_lognormal
    return grf_lognormal(side, seed, device)


class ClockSampler:
    """SM clock and throttle-reason samples while the timed region runs.

    Reads NVML (libnvidia-ml, shipped with the driver) every 2 ms from a
    background thread, so even a timed region of a few milliseconds gets
    samples; where NVML cannot be loaded, nvidia-smi every 50 ms instead.
    Only reads: no clock or other GPU setting is changed."""

    NAMES = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
    # nvmlClocksEventReason* bits
    BITS = {"sw_power_cap": 0x4, "hw_slowdown": 0x8, "sw_thermal_slowdown": 0x20, "hw_thermal_slowdown": 0x40}
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_id: str):
        self.gpu_id = gpu_id
        self.samples = []  # (sm_mhz, max_mhz, set of reasons)
        self.proc = None
        self.stop = threading.Event()
        self.thread = None
        self.source = None

    def _nvml(self):
        import ctypes
        try:
            nv = ctypes.CDLL("libnvidia-ml.so.1")
        except OSError:
            return None
        if nv.nvmlInit_v2() != 0:
            return None
        h = ctypes.c_void_p()
        gid = self.gpu_id.strip()
        rc = (nv.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(int(gid)), ctypes.byref(h)) if gid.isdigit()
              else nv.nvmlDeviceGetHandleByUUID(gid.encode(), ctypes.byref(h)))
        if rc != 0:
            return None
        reasons_fn = getattr(nv, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            nv.nvmlDeviceGetCurrentClocksThrottleReasons
        return nv, h, reasons_fn

    def _poll_nvml(self, nv, h, reasons_fn):
        import ctypes
        mhz, mx, rs = ctypes.c_uint(), ctypes.c_uint(), ctypes.c_ulonglong()
        while not self.stop.is_set():
            if (nv.nvmlDeviceGetClockInfo(h, 1, ctypes.byref(mhz)) == 0 and
                    nv.nvmlDeviceGetMaxClockInfo(h, 1, ctypes.byref(mx)) == 0 and
                    reasons_fn(h, ctypes.byref(rs)) == 0):
                active = {k for k, b in self.BITS.items() if rs.value & b}
                self.samples.append((float(mhz.value), float(mx.value), active))
            time.sleep(0.002)

    def _read_smi(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.strip().split(",")]
            if len(parts) < 9:
                continue
            try:
                sm, mx = float(parts[1]), float(parts[2])
            except ValueError:
                continue
            active = {n for n, v in zip(self.NAMES, parts[5:9]) if v.lower().startswith("active")}
            self.samples.append((sm, mx, active))

    def __enter__(self):
        nvml = self._nvml()
        if nvml:
            self.source = "nvml, 2 ms"
            self.thread = threading.Thread(target=self._poll_nvml, args=nvml, daemon=True)
            self.thread.start()
        else:
            try:
                self.proc = subprocess.Popen(
                    ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                     "-lms", "50", "-i", self.gpu_id], stdout=subprocess.PIPE,
                    stderr=subprocess.DEVNULL, text=True)
                self.source = "nvidia-smi, 50 ms"
                threading.Thread(target=self._read_smi, daemon=True).start()
            except OSError:
                self.proc = None
        # sampling is live before the timed region starts
        t0 = time.perf_counter()
        while (self.thread or self.proc) and not self.samples and time.perf_counter() - t0 < 3.0:
            time.sleep(0.001)
        self.samples = []  # keep only samples taken from here on
        return self

    def __exit__(self, *exc):
        self.stop.set()
        if self.thread:
            self.thread.join(timeout=2)
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        samples = list(self.samples)
        if not samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0, "source": self.source}
        reasons = set()
        for _, _, r in samples:
            reasons |= r
        return {"sm_mhz": statistics.median(s[0] for s in samples), "sm_max_mhz": max(s[1] for s in samples),
                "reasons": sorted(reasons), "samples": len(samples), "source": self.source}


def seg_worst(length: int, L: int) -> int:
    """Largest encoding of a segment (every block at width 32)."""
    if length == 0:
        return 0
    nfull, ntail = (length - 1) // L, (length - 1) % L
    s = 4 + nfull * (1 + (L + 7) // 8 + 4 * L)
    return s + (1 + (ntail + 7) // 8 + 4 * ntail if ntail else 0)


def host_read_bytes(stream_bytes: bytes, n: int, L: int, T: int) -> int:
    """Bytes the drop-in copies to the device for a host stream: the chunk
    offsets give all but the last chunk, which is read at twice the others'
    average length (plus 64 KiB), and again up to its largest possible size
    (not past 4*n bytes) only when its headers run past that."""
    last = int.from_bytes(stream_bytes[8 * (T - 1): 8 * T], "little")
    known = 8 * T + last
    want = known + seg_worst(n // T, L) + seg_worst(n % T, L)
    first = min(want, max(4 * n, known + 4))
    if T > 1:
        first = min(first, known + 2 * (last // (T - 1)) + 65536)
    if len(stream_bytes) > first:  # the walk runs past the first read: read again in full
        first += want
    return first


def cpu_codec_rate(x, y, eb, L, T, reps=1):
    """GB/s of uncompressed input for compress + decompress + homomorphic add
    with the oracle port on T host threads: the best of `reps` passes after
    one warm-up pass; returns (GB/s, seconds/pass, outputs of the last pass:
    stream of x, its decompressed floats, stream of x + y)."""
    from oracle import zoracle
    port = zoracle.port()
    n = x.size
    sb = port.compress(y, eb, L, T)
    best = None
    for k in range(reps + 1):
        t0 = time.perf_counter()
        sa = port.compress(x, eb, L, T)
        ya = port.decompress(sa, n, eb, L, T)
        ha = port.homadd(sa, sb, n, eb, L, T)
        dt = time.perf_counter() - t0
        if k:
            best = dt if best is None else min(best, dt)
    return 3 * 4 * n / best / 1e9, best, {"stream": sa, "floats": ya, "sum": ha}


def same_bits(a, b) -> bool:
    """Two float32 arrays equal bit for bit (signed zeros and NaNs included)."""
    import numpy as np
    a, b = np.ascontiguousarray(a, np.float32), np.ascontiguousarray(b, np.float32)
    return a.shape == b.shape and bool(np.array_equal(a.view(np.uint32), b.view(np.uint32)))


def oracle_outputs(xh, yh, eb, L, T):
    """The oracle's stream of x, decompressed floats and stream of x + y."""
    from oracle import zoracle
    port = zoracle.port()
    n = xh.size
    sa = port.compress(xh, eb, L, T)
    return {"stream": sa, "floats": port.decompress(sa, n, eb, L, T),
            "sum": port.homadd(sa, port.compress(yh, eb, L, T), n, eb, L, T)}


def max_over_ranks(v: float, world: int, device) -> float:
    """The largest of every rank's v (the whole job is as slow as its
    slowest rank); v itself on one rank."""
    if world <= 1:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def run_reference(args, rank, world):
    """--impl reference: the reference codec's CPU path on the host cores."""
    import numpy as np
    import torch
    if rank != 0:
        return
    T = args.T or host_cores()
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    x = make_field(args.side, 0, dev).cpu().numpy()
    y = make_field(args.side, 1, dev).cpu().numpy()
    eb = float(np.float32(args.eb_rel * max(float(x.max() - x.min()), float(y.max() - y.min()))))
    from oracle import zoracle
    port = zoracle.port()
    n = x.size
    sb = port.compress(y, eb, args.L, T)
    times = []
    for s in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        sa = port.compress(x, eb, args.L, T)
        port.decompress(sa, n, eb, args.L, T)
        port.homadd(sa, sb, n, eb, args.L, T)
        if s >= args.warmup:
            times.append(time.perf_counter() - t0)
    tot = sum(times)
    value = 3 * 4 * n * args.steps / tot / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": "GB/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1e3 * tot / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "config": workload_config(args, n, T),
        "cpu_baseline": {"value": round(value, 3), "unit": "GB/s", "cores": T, "kind": "port",
                         "sample": "whole 512^3 field per step; oracle C restatement, OpenMP"},
        "e2e": {"value": round(value, 3), "unit": "GB/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def make_rank_chunks(n: int, P: int, seed: int, device):
    from zccl_gb300.workloads import rank_chunks
    return rank_chunks(n, P, seed, device)


def timed(fn, reps, stream):
    """Mean device ms of fn over reps runs (after one warm-up), CUDA events
    on the launching stream."""
    import torch
    fn()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def reduction_bench(args, L, T, dev):
    """P ranks' chunks of red_n floats (P = 8 x 16M by default), eb =
    1e-4 * range: the P-way homomorphic add against the pairwise fold and
    decompress-add-recompress, their errors against the exact sum, and the
    ring allreduce run for the P ranks on this device, both variants."""
    import numpy as np
    import torch
    import zccl_gb300 as Z
    from zccl_gb300.ring import PairwiseTree, RingAllreduce, reduce_doc, reduce_homomorphic, reduce_pairwise
    n, P = args.red_n, args.red_p
    xs = make_rank_chunks(n, P, 3, dev)
    lo = min(float(x.min()) for x in xs)
    hi = max(float(x.max()) for x in xs)
    eb = float(np.float32(1e-4 * (hi - lo)))
    codec = Z.Codec(n, L, T, device=str(dev))
    st = codec.torch_stream
    streams = [codec.new_stream() for _ in range(P)]
    out = codec.new_stream()
    ms_compress = timed(lambda: [codec.compress(x, eb, out=s) for x, s in zip(xs, streams)], 3, st)
    ms_pway = timed(lambda: reduce_homomorphic(codec, streams, out=out), 5, st)
    pair_outs = [codec.new_stream(), codec.new_stream()]
    ms_pair = timed(lambda: reduce_pairwise(codec, streams, pair_outs), 5, st)
    tree = PairwiseTree(codec, streams, stream=st)
    ms_tree = timed(tree.run, 5, st)
    docs = codec.new_stream()
    doc_total = torch.empty(n, dtype=torch.float32, device=dev)
    ms_doc = timed(lambda: reduce_doc(codec, streams, eb, out=docs, total=doc_total), 5, st)
    # the same three reductions replayed from CUDA graphs: device time alone,
    # without the host's per-call enqueue between the fold's and DOC's calls
    graph = {}
    gst = torch.cuda.Stream(dev)
    gcodec = Z.Codec(n, L, T, device=str(dev), stream=gst)
    gtree = PairwiseTree(gcodec, streams, stream=gst)
    keep = []
    for name, fn in (("pway_homadd_ms", lambda: reduce_homomorphic(gcodec, streams, out=out)),
                     ("pairwise_fold_ms", lambda: reduce_pairwise(gcodec, streams, pair_outs)),
                     ("pairwise_tree_ms", gtree.run),
                     ("doc_ms", lambda: reduce_doc(gcodec, streams, eb, out=docs, total=doc_total))):
        try:
            with torch.cuda.stream(gst):
                fn()
                gst.synchronize()
                g = torch.cuda.CUDAGraph()
                with torch.cuda.graph(g, stream=gst, capture_error_mode="relaxed"):
                    fn()
                graph[name] = round(timed(g.replay, 10, gst), 4)
            keep.append(g)
        except Exception as e:  # a call that cannot be captured: report it, keep going
            graph[name] = f"not captured: {type(e).__name__}"
    gcodec.check()
    gtree.check()
    del keep, gtree
    codec.check()
    same = reduce_homomorphic(codec, streams, out=out).tobytes() == reduce_pairwise(codec, streams).tobytes()
    same_tree = tree.run().tobytes() == out.tobytes()
    tree.check()
    del tree
    exact = torch.zeros(n, dtype=torch.float64, device=dev)
    for x in xs:
        exact += x.double()
    y_ho = codec.decompress(out, eb)
    doc_stream, _ = reduce_doc(codec, streams, eb, out=docs)
    y_doc = codec.decompress(doc_stream, eb)
    err_ho = float((y_ho.double() - exact).abs().max()) / eb
    err_doc = float((y_doc.double() - exact).abs().max()) / eb
    cin = sum(s.size() for s in streams)
    cout = out.size()
    ring = RingAllreduce(n, P, L, T, device=str(dev))
    ms_ring_ho = timed(lambda: ring.homomorphic(xs, eb), 5, st)
    ms_ring_doc = timed(lambda: ring.doc(xs, eb), 5, st)
    y_rho = ring.homomorphic(xs, eb)
    y_rdoc = ring.doc(xs, eb)
    ring1 = RingAllreduce(n, P, L, T, device=str(dev), batched=False)
    ms_ring1_ho = timed(lambda: ring1.homomorphic(xs, eb), 2, st)
    ms_ring1_doc = timed(lambda: ring1.doc(xs, eb), 2, st)
    del ring1
    # the segmented allgatherv of the P chunks (8 MiB segments, frames
    # decompressed by the receiver as wire bytes), rank 0's receive buffer
    from zccl_gb300.allgather import SegmentedAllgatherv
    ag = SegmentedAllgatherv([n] * P, L, T, device=str(dev))
    ms_ag = timed(lambda: ag.run(xs, eb), 2, st)
    g_ag, y_ag = ag.capture(xs, eb)
    ms_ag_graph = timed(g_ag.replay, 3, st)
    ag.check()
    err_ag = max(float((y_ag[c * n:(c + 1) * n].double() - xs[c].double()).abs().max()) for c in range(1, P)) / eb
    wire = sum(int(np.frombuffer(f[:8].cpu().numpy().tobytes(), "<u8")[0]) + 8 for fr in ag.sent for f in fr)
    nseg = sum(len(fr) for fr in ag.sent)
    res = {
        "workload": f"P={P} ranks x {n} float32 (smooth base of 8 random-phase sinusoids + rank N(0,0.05)), "
                    f"eb=1e-4*range, L={L}, T={T}",
        "pway_homadd_ms": round(ms_pway, 4),
        "pway_homadd_GBps_alg": round((cin + cout) / (ms_pway * 1e-3) / 1e9, 1),
        "pway_homadd_GBps_uncompressed": round(4 * n * P / (ms_pway * 1e-3) / 1e9, 1),
        "pairwise_fold_ms": round(ms_pair, 4),
        "pairwise_tree_ms": round(ms_tree, 4),
        "doc_ms": round(ms_doc, 4),
        "graph_replay_ms": graph,
        "compress_all_ms": round(ms_compress, 4),
        "pway_equals_pairwise_bytes": same,
        "pway_equals_pairwise_tree_bytes": same_tree,
        "max_err_over_eb": {"homomorphic": round(err_ho, 3), "doc": round(err_doc, 3), "bound": P},
        "ring_allreduce_emulated_ms": {"homomorphic": round(ms_ring_ho, 3), "doc": round(ms_ring_doc, 3),
                                       "note": f"all {P} ranks' codec work on one GPU, each step's {P} codec "
                                               f"calls as one batch launch (cached plans)",
                                       "one_call_per_chunk": {"homomorphic": round(ms_ring1_ho, 3),
                                                              "doc": round(ms_ring1_doc, 3)}},
        "segmented_allgatherv": {
            "ms": round(ms_ag, 3), "graph_replay_ms": round(ms_ag_graph, 3), "segments": nseg, "wire_bytes": wire,
            "gathered_GBps": round(4 * n * P / (ms_ag_graph * 1e-3) / 1e9, 1),
            "max_err_over_eb": round(err_ag, 3),
            "note": f"{P} chunks compressed once in 8 MiB segments (size-prefixed frames), rank 0 "
                    f"decompresses the {P - 1} it receives from wire bytes, on a second stream as "
                    f"frames complete; ms eager, graph_replay_ms recorded once as a CUDA graph"},
        "ring_max_err_over_eb": {
            "homomorphic": round(float((y_rho.double() - exact).abs().max()) / eb, 3),
            "doc": round(float((y_rdoc.double() - exact).abs().max()) / eb, 3)},
    }
    if not args.no_parity:
        res["parity"] = reduction_parity(codec, xs, streams, out, y_ho, ring, eb, L, T)
    del xs, exact
    torch.cuda.empty_cache()
    return res


def reduction_parity(codec, xs, streams, out, y_ho, ring, eb, L, T):
    """The P-way sum against the oracle's pairwise fold of the oracle's own
    streams (the reference ring's acc = add(received, acc) order), every
    rank's stream, the decompressed sum, and the emulated homomorphic ring's
    reduced chunks against the same ring run by the oracle."""
    from oracle import zoracle
    port = zoracle.port()
    n, P = codec.n, len(xs)
    xh = [x.cpu().numpy() for x in xs]
    sref = [port.compress(v, eb, L, T) for v in xh]
    fold = port.homadd_fold(sref, n, eb, L, T)
    chunks_ok = True
    ring.homomorphic(xs, eb)
    for c in range(P):
        lo, m = ring.displs[c], ring.cnts[c]
        S = [port.compress(xh[r][lo: lo + m], eb, L, T) for r in range(P)]
        for i in range(P - 1):
            for r in range(P):
                src, cc = (r - 1) % P, (r - 2 - i) % P
                if cc == c:
                    S[r] = port.homadd(S[src], S[r], m, eb, L, T)
        chunks_ok &= ring.reduced[c].tobytes() == S[c]
    return {"rank_streams": all(s.tobytes() == r for s, r in zip(streams, sref)),
            "pway_sum": out.tobytes() == fold,
            "floats": same_bits(y_ho.cpu().numpy(), port.decompress(fold, n, eb, L, T)),
            "ring_reduced_chunks": bool(chunks_ok)}


def szp3d_bench(args, dev):
    """The SZp 3-D codec on the side^3 field (eb = 1e-4 * range, block sides
    4 and 8): device-timed compress and decompress, compression ratio, max
    error over eb; the serial reference restatement (one host core, the
    reference's form is serial) on a 128^3 corner of the field."""
    import time
    import numpy as np
    import torch
    from oracle import zoracle
    from zccl_gb300.szp3d import Szp3D
    side = args.side
    x = make_field(side, 0, dev)
    eb = float(1e-4 * float(x.max() - x.min()))
    dims = (side, side, side)
    res = {"workload": f"{side}^3 log-normal GRF, eb=1e-4*range (float64 {eb:.6g})"}
    for bs in (4, 8):
        codec = Szp3D(dims, bs, device=str(dev))
        st = codec.torch_stream
        buf, size = codec.compress(x, eb)
        n = codec.size(size)
        y = torch.empty_like(x)
        ms_c = timed(lambda: codec.compress(x, eb, out=buf), 5, st)
        ms_d = timed(lambda: codec.decompress(buf, eb, out=y, avail=n), 5, st)
        codec.check()
        err = float((y.double() - x.double()).abs().max()) / eb
        alg = 4 * x.numel() + n
        res[f"bs{bs}"] = {"compress_ms": round(ms_c, 3), "decompress_ms": round(ms_d, 3),
                          "compress_GBps_uncompressed": round(4 * x.numel() / (ms_c * 1e-3) / 1e9, 1),
                          "decompress_GBps_uncompressed": round(4 * x.numel() / (ms_d * 1e-3) / 1e9, 1),
                          "algorithmic_GBps": {"compress": round(alg / (ms_c * 1e-3) / 1e9, 1),
                                               "decompress": round(alg / (ms_d * 1e-3) / 1e9, 1)},
                          "ratio": round(4 * x.numel() / n, 3), "max_err_over_eb": round(err, 4)}
    if not args.no_cpu:
        c = 128
        sub = x.view(side, side, side)[:c, :c, :c].contiguous().cpu().numpy().ravel()
        port = zoracle.port()
        t0 = time.perf_counter()
        s = port.szp3d_compress(sub, (c, c, c), 4, eb)
        t1 = time.perf_counter()
        port.szp3d_decompress(s, (c, c, c), 4, eb)
        t2 = time.perf_counter()
        res["cpu_baseline"] = {"kind": "port", "cores": 1, "sample": f"{c}^3 corner, block side 4",
                               "compress_GBps": round(4 * sub.size / (t1 - t0) / 1e9, 3),
                               "decompress_GBps": round(4 * sub.size / (t2 - t1) / 1e9, 3)}
    del x
    torch.cuda.empty_cache()
    return res


def batched_bench(args, L, dev):
    """4096 gradient-bucket-like buffers (2048 pairs of equal size, log-
    uniform 4 KB - 16 MB, Laplace(0, 1e-3), 5 % constant, eb per pair from
    {1e-3, 1e-4, 1e-5} * range, T = 1): compress all, then add each pair
    homomorphically.  Batched: one persistent launch for all compressions
    and one for all sums (launch shape from the autotuner), replayed from a
    CUDA graph.  Against: one C-ABI call (memset + launch) per buffer, run
    eagerly and also replayed from a CUDA graph."""
    import ctypes
    import types
    import numpy as np
    import torch
    import zccl_gb300 as Z
    from zccl_gb300.workloads import gradient_buckets
    lib = Z.lib()
    npairs = args.batch_pairs
    T = 1
    bk = gradient_buckets(npairs, 7, dev)
    sizes, xs, ebs, data = bk.sizes, bk.xs, bk.ebs, bk.data
    total = data.numel()
    caps = [lib.zccl_gpu_max_stream_bytes(int(n), L, T) for n in sizes]
    idxb = [lib.zccl_gpu_index_bytes(int(n), L, T) for n in sizes]
    a16 = lambda v: (v + 255) // 256 * 256
    sbytes = torch.empty(sum(3 * a16(c) for c in caps), dtype=torch.uint8, device=dev)
    ibytes = torch.zeros(sum(3 * a16(i) for i in idxb), dtype=torch.uint8, device=dev)

    def streams():
        so = io = 0
        out = []
        for k in range(npairs):
            trio = []
            for _ in range(3):
                d = Z.StreamDesc(sbytes.data_ptr() + so, caps[k], ibytes.data_ptr() + io, 0, 0)
                trio.append(types.SimpleNamespace(desc=d, codec=types.SimpleNamespace(n=int(sizes[k]))))
                so += a16(caps[k])
                io += a16(idxb[k])
            out.append(trio)
        return out

    st = torch.cuda.current_stream()
    sp = ctypes.c_void_p(st.cuda_stream)
    S = streams()
    bc = Z.Batch(Z.BATCH_COMPRESS, [(xs[k][r], ebs[k], T, S[k][r]) for k in range(npairs) for r in range(2)], L)
    bh = Z.Batch(Z.BATCH_HOMADD, [([S[k][0], S[k][1]], T, S[k][2]) for k in range(npairs)], L)
    grid_c, grid_h = bc.tune(), bh.tune()

    def batched():
        bc.run()
        bh.run()

    batched()
    bc.check()
    bh.check()
    # whole streams of 64 pairs spread over the size range, against the oracle
    parity = None
    step = max(1, npairs // 64)
    sample = list(range(0, npairs, step))[:64]

    def whole(k, r):
        n = int(sizes[k])
        sz = ctypes.c_size_t(0)
        lib.zccl_gpu_stream_size(ctypes.byref(S[k][r].desc), n, L, T, ctypes.byref(sz), sp)
        o = S[k][r].desc.bytes - sbytes.data_ptr()
        return bytes(sbytes[o: o + sz.value].cpu().numpy())

    if not args.no_parity:
        from oracle import zoracle
        port = zoracle.port()
        ok_c = ok_h = True
        for k in sample:
            n = int(sizes[k])
            a, b = xs[k][0].cpu().numpy(), xs[k][1].cpu().numpy()
            ra, rb = port.compress(a, ebs[k], L, T), port.compress(b, ebs[k], L, T)
            ok_c &= whole(k, 0) == ra and whole(k, 1) == rb
            ok_h &= whole(k, 2) == port.homadd(ra, rb, n, ebs[k], L, T)
        parity = {"pairs_checked": len(sample), "streams": bool(ok_c), "sums": bool(ok_h)}
    sum_b = [(S[k][2].desc.index, S[k][2].desc.bytes) for k in range(0, npairs, 97)]
    digest_b = [bytes(sbytes[d - sbytes.data_ptr(): d - sbytes.data_ptr() + 64].cpu().numpy())
                for _, d in sum_b]

    ws = torch.zeros(max(lib.zccl_gpu_workspace_bytes(int(n), L, T) for n in sizes), dtype=torch.uint8,
                     device=dev)
    pairs_desc = [(Z.StreamDesc * 2)(S[k][0].desc, S[k][1].desc) for k in range(npairs)]

    def per_buffer():
        for k in range(npairs):
            n = int(sizes[k])
            for r in range(2):
                lib.zccl_gpu_compress(ctypes.byref(S[k][r].desc), xs[k][r].data_ptr(), n, ebs[k], L, T,
                                      ws.data_ptr(), sp)
            pairs_desc[k][0], pairs_desc[k][1] = S[k][0].desc, S[k][1].desc
            lib.zccl_gpu_homadd(ctypes.byref(S[k][2].desc), pairs_desc[k], 2, n, L, T, ws.data_ptr(), sp)

    per_buffer()
    lib.zccl_gpu_check(ws.data_ptr(), sp)
    digest_p = [bytes(sbytes[d - sbytes.data_ptr(): d - sbytes.data_ptr() + 64].cpu().numpy())
                for _, d in sum_b]
    same = digest_p == digest_b
    ms_eager = timed(per_buffer, 2, st)
    gp = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    side.wait_stream(st)
    with torch.cuda.graph(gp, stream=side, capture_error_mode="relaxed"):
        sp_saved = sp
        sp = ctypes.c_void_p(side.cuda_stream)
        per_buffer()
        sp = sp_saved
    ms_graph_per = timed(gp.replay, 3, st)
    gb = torch.cuda.CUDAGraph()
    with torch.cuda.graph(gb, stream=side, capture_error_mode="relaxed"):
        bc.run(side)
        bh.run(side)
    ms_batch = timed(gb.replay, 5, st)
    ms_bc = timed(lambda: bc.run(st), 5, st)
    ms_bh = timed(lambda: bh.run(st), 5, st)
    bc.check()
    bh.check()
    unc = 4 * total
    res = {
        "workload": f"{2 * npairs} buffers ({npairs} pairs of equal size), log-uniform 4 KB-16 MB float32, "
                    f"Laplace(0,1e-3), 5% constant, eb in {{1e-3,1e-4,1e-5}}*range, L={L}, T={T}: compress "
                    f"all + pairwise homomorphic add",
        "uncompressed_bytes": unc,
        "batched_graph_ms": round(ms_batch, 3),
        "per_buffer_eager_ms": round(ms_eager, 3),
        "per_buffer_graph_ms": round(ms_graph_per, 3),
        "speedup_vs_per_buffer_eager": round(ms_eager / ms_batch, 2),
        "speedup_vs_per_buffer_graph": round(ms_graph_per / ms_batch, 2),
        "batched_GBps_uncompressed": round(unc / (ms_batch * 1e-3) / 1e9, 1),
        "compress_batch_ms": round(ms_bc, 3),
        "homadd_batch_ms": round(ms_bh, 3),
        "launches": {"batched": 2, "per_buffer": 3 * npairs},
        "autotuned_grid": {"compress": grid_c, "homadd": grid_h},
        "outputs_equal_sampled": same,
    }
    if parity:
        res["parity"] = parity
    del data, xs, sbytes, ibytes, ws, gp, gb
    torch.cuda.empty_cache()
    return res


def serving_bench(args, L, dev):
    """Poisson arrivals: 50 % compress, 30 % decompress, 20 % homomorphic
    add of 2-8 resident streams; sizes log-uniform 64 KB - 256 MB of float32
    cut from a log-normal GRF (as the 512^3 field, at 400^3); eb = 1e-4 *
    range; 120 GB admission budget (inputs, outputs and scratch counted).
    The peak is the saturated open-loop throughput: arrivals offered far
    faster than the device serves them for serve_secs.  The sweep then
    offers 10 % - 200 % of the peak, serve_secs of arrivals per point (at
    most serve_max requests), and reports achieved throughput, p50 / p99
    latency, the device overlap of units and the host's enqueue time per
    point; max_sustained is the highest load served at >= 95 % of the
    offered rate."""
    import numpy as np
    import torch
    from zccl_gb300.serve import COMPRESS, DECOMPRESS, HOMADD, Request, Server, device_overlap, percentile
    field = make_field(args.serve_side, 5, dev)
    nf = field.numel()
    eb = float(np.float32(1e-4 * float(field.max() - field.min())))
    rng = np.random.default_rng(11)
    lo_n, hi_n = (64 << 10) // 4, min((256 << 20) // 4, nf)
    draw_n = lambda: int(np.exp(rng.uniform(np.log(lo_n), np.log(hi_n))))
    srv = Server(120 << 30, slots=args.serve_slots, L=L)
    groups = []
    for gi in range(8):
        n = draw_n()
        keys = []
        for r in range(8):
            off = int(rng.integers(0, nf - n + 1))
            srv.put((gi, r), field[off: off + n], eb, 1)
            keys.append((gi, r))
        groups.append((n, keys))
    rid = [0]

    def make(t):
        u = rng.random()
        rid[0] += 1
        if u < 0.5:
            n = draw_n()
            off = int(rng.integers(0, nf - n + 1))
            return Request(t, rid[0], COMPRESS, x=field[off: off + n], eb=eb, T=1), 4 * n
        n, keys = groups[int(rng.integers(0, len(groups)))]
        if u < 0.8:
            return Request(t, rid[0], DECOMPRESS, ins=[keys[int(rng.integers(0, 8))]]), 4 * n
        P = int(rng.integers(2, 9))
        return Request(t, rid[0], HOMADD, ins=[keys[int(k)] for k in rng.choice(8, P, replace=False)]), 4 * n * P

    def serve(reqs):
        srv.log, srv.units, srv.max_inflight, srv.host_launch_s = [], [], 0, 0.0
        base = srv.now()
        for q, _ in reqs:
            q.arrival += base
            srv.submit(q)
        log = srv.run()
        nbytes = sum(b for _, b in reqs)
        span = max(q.done for q in log) - min(q.arrival for q in log)
        lat = [1e3 * (q.done - q.arrival) for q in log]
        ov = device_overlap(srv.units)
        return {"GBps": nbytes / span / 1e9, "p50": percentile(lat, 50), "p99": percentile(lat, 99),
                "count": len(log), "span_s": span, "overlap": ov, "max_inflight": srv.max_inflight,
                "host_launch_frac": srv.host_launch_s / span}

    def arrivals(rate_gbs, secs, cap):
        lam = rate_gbs * 1e9 / mean_b  # requests per second
        t, reqs = 0.0, []
        while t < secs and len(reqs) < cap:
            t += float(rng.exponential(1.0 / lam))
            reqs.append(make(t))
        return reqs

    serve([make(0.0) for _ in range(60)])  # warm-up: allocator, first launches
    burst = serve([make(0.0) for _ in range(400)])
    mean_b = float(np.mean([make(0.0)[1] for _ in range(4000)]))
    # saturation: offered at four times the closed burst's rate
    sat = serve(arrivals(4.0 * burst["GBps"], args.serve_secs, args.serve_max))
    peak = sat["GBps"]
    points = []
    for load in (0.1, 0.25, 0.5, 0.75, 0.9, 1.0, 1.2, 1.5, 2.0):
        reqs = arrivals(load * peak, args.serve_secs, args.serve_max)
        r = serve(reqs)
        points.append({"offered_frac": load, "offered_GBps": round(load * peak, 1), "achieved_GBps": round(r["GBps"], 1),
                       "p50_ms": round(r["p50"], 3), "p99_ms": round(r["p99"], 3), "requests": r["count"],
                       "arrival_s": round(reqs[-1][0].arrival - reqs[0][0].arrival if len(reqs) > 1 else 0.0, 3),
                       "device_busy_frac": round(r["overlap"]["busy_ms"] / (1e3 * r["span_s"]), 3),
                       "device_overlap_ms": round(r["overlap"]["overlap_ms"], 2),
                       "max_units_in_flight": r["max_inflight"],
                       "host_launch_frac": round(r["host_launch_frac"], 3)})
        if load >= 1.0 and r["GBps"] < 0.95 * load * peak:
            break
    sustained = [p for p in points if p["achieved_GBps"] >= 0.95 * p["offered_GBps"]]
    res = {
        "workload": "Poisson arrivals, 50% compress / 30% decompress / 20% homomorphic add of 2-8 resident "
                    f"streams, log-uniform 64 KB-256 MB float32 from a {args.serve_side}^3 log-normal GRF, "
                    f"eb=1e-4*range, 120 GB budget, {args.serve_slots} slots, continuous batching",
        "peak_GBps_saturated": round(peak, 1),
        "saturated": {"offered_GBps": round(4.0 * burst["GBps"], 1), "requests": sat["count"],
                      "p50_ms": round(sat["p50"], 3), "p99_ms": round(sat["p99"], 3),
                      "max_units_in_flight": sat["max_inflight"],
                      "device_busy_frac": round(sat["overlap"]["busy_ms"] / (1e3 * sat["span_s"]), 3),
                      "host_launch_frac": round(sat["host_launch_frac"], 3)},
        "closed_burst_GBps": round(burst["GBps"], 1),
        "sweep": points,
        "max_sustained": sustained[-1] if sustained else None,
        "bytes_counted": "uncompressed input floats: 4n (compress, decompress), 4n*P (add)",
    }
    del field, srv
    torch.cuda.empty_cache()
    return res


def workload_config(args, n, T):
    return {"workload": f"{args.side}^3 float32 log-normal GRF ({4 * n >> 20} MiB): compress + "
                        f"decompress + 2-way homomorphic add, eb={args.eb_rel:g}*range",
            "elements": n, "eb_rel": args.eb_rel, "block_size": args.L, "writer_threads_T": T,
            "l2": "inputs 512 MiB > 129 MB L2, no flush needed"}


def run_ours(args, rank, world, local_rank):
    import numpy as np
    import torch

    import zccl_gb300 as Z
    dev = torch.device("cuda", local_rank)
    torch.cuda.set_device(dev)
    T = args.T or host_cores()
    L = args.L
    x = make_field(args.side, 2 * rank, dev)
    y = make_field(args.side, 2 * rank + 1, dev)
    n = x.numel()
    eb = float(np.float32(args.eb_rel * max(float(x.max() - x.min()), float(y.max() - y.min()))))
    codec = Z.Codec(n, L, T, device=str(dev))
    st = codec.torch_stream
    sa, sb, ss = codec.new_stream(), codec.new_stream(), codec.new_stream()
    xo = torch.empty(n, dtype=torch.float32, device=dev)
    codec.compress(y, eb, out=sb)

    def step(ev=None):
        if ev:
            ev[0].record(st)
        codec.compress(x, eb, out=sa)
        if ev:
            ev[1].record(st)
        codec.decompress(sa, eb, out=xo)
        if ev:
            ev[2].record(st)
        codec.homadd([sa, sb], out=ss)
        if ev:
            ev[3].record(st)

    for _ in range(args.warmup):
        step()
    codec.check()
    ca, cb, cs = sa.size(), sb.size(), ss.size()
    # correctness guard on the timed workload: decompression error within eb
    err = (xo.double() - x.double()).abs().max().item()
    assert err <= eb * (1 + 1e-3) + 4 * np.spacing(np.float32(x.abs().max().item())), err

    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(args.steps)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    gpu_id = os.environ.get("CUDA_VISIBLE_DEVICES", str(local_rank)).split(",")[0] or "0"
    with ClockSampler(gpu_id) as clk:
        t_start = torch.cuda.Event(enable_timing=True)
        t_end = torch.cuda.Event(enable_timing=True)
        t_start.record(st)
        for k in range(args.steps):
            step(evs[k])
        t_end.record(st)
        torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    codec.check()
    ms = t_start.elapsed_time(t_end) / args.steps
    ms = max_over_ranks(ms, world, dev)
    op_ms = [statistics.mean(e[i].elapsed_time(e[i + 1]) for e in evs) for i in range(3)]
    value = world * 3 * 4 * n / (ms * 1e-3) / 1e9
    peak, peak_kind = peaks()
    alg = {"compress": 4 * n + ca, "decompress": ca + 4 * n, "homadd": ca + cb + cs}
    per_op = {}
    for name, t_ms in zip(("compress", "decompress", "homadd"), op_ms):
        gbs = alg[name] / (t_ms * 1e-3) / 1e9
        per_op[name] = {"ms": round(t_ms, 4), "uncompressed_GBps": round(4 * n / (t_ms * 1e-3) / 1e9, 1),
                        "algorithmic_GBps": round(gbs, 1), "roofline_frac": round(gbs / peak, 4),
                        "algorithmic_bytes": alg[name]}
    dom = max(per_op, key=lambda k: per_op[k]["ms"])
    traffic = DRAM_TRAFFIC_512.get(dom) if (args.side, L, args.eb_rel) == (512, 32, 1e-4) else None
    roofline = {"bound": "hbm", "achieved": per_op[dom]["algorithmic_GBps"], "peak": peak,
                "unit": "GB/s", "frac": per_op[dom]["roofline_frac"], "traffic": traffic,
                "kernel": dom, "peak_source": f"{peak_kind} hbm_gbs"}

    # e2e through the reference-facing entry points with host buffers: the
    # fields, streams and floats in pinned host memory (a caller's MPI
    # buffers), then the same step once more on ordinary pageable arrays
    Z.set_omp_threads(T)
    cap = max(4 * n, codec.max_stream_bytes)

    def host_array(count, dtype, pinned):
        if pinned:
            return torch.zeros(count, dtype=dtype, pin_memory=True).numpy()
        return np.zeros(count, {torch.float32: np.float32, torch.uint8: np.uint8}[dtype])

    def e2e_run(pinned):
        xh, yh = host_array(n, torch.float32, pinned), host_array(n, torch.float32, pinned)
        xh[:], yh[:] = x.cpu().numpy(), y.cpu().numpy()
        bufs = [host_array(cap, torch.uint8, pinned) for _ in range(3)] + [host_array(n, torch.float32, pinned)]
        hs_a, hs_b, hs_s, hy = bufs
        Z.ZCCL_float_openmp_threadblock_arg(hs_b, yh, 0, eb, n, L)

        def e2e_step():
            Z.ZCCL_float_openmp_threadblock_arg(hs_a, xh, 0, eb, n, L)
            Z.ZCCL_float_decompress_openmp_threadblock_arg(hy, n, eb, L, hs_a)
            Z.ZCCL_float_homomophic_add_openmp_threadblock(hs_s, 0, n, eb, L, hs_a, hs_b)

        e2e_step()
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            e2e_step()
        return (time.perf_counter() - t0) / args.e2e_steps, xh, yh, bufs

    e2e_s, xh, yh, (hs_a, hs_b, hs_s, hy) = e2e_run(True)
    e2e_pageable_s = e2e_run(False)[0]
    rd_a = host_read_bytes(hs_a[:ca].tobytes(), n, L, T)
    rd_b = host_read_bytes(hs_b[:cb].tobytes(), n, L, T)
    e2e = {"value": round(world * 3 * 4 * n / e2e_s / 1e9, 3), "unit": "GB/s",
           "h2d_bytes_per_step": 4 * n + 2 * rd_a + rd_b,
           "d2h_bytes_per_step": ca + 4 * n + cs,
           "host_memory": "pinned",
           "pageable_value": round(world * 3 * 4 * n / e2e_pageable_s / 1e9, 3),
           "api": "ZCCL_float_openmp_threadblock_arg / _decompress_ / _homomophic_add_ (host)"}

    cpu, ref_out = None, None
    if rank == 0 and world == 1 and not args.no_cpu:
        rate, secs, ref_out = cpu_codec_rate(xh, yh, eb, L, T, reps=5)
        m = n // 16
        Z.set_omp_threads(1)
        rate1, secs1, _ = cpu_codec_rate(xh[:m], yh[:m], eb, L, 1, reps=1)
        Z.set_omp_threads(T)
        cpu = {"value": round(rate, 3), "unit": "GB/s", "cores": T, "kind": "port",
               "sample": f"whole field, best of 5 passes after one warm-up ({secs:.2f} s a pass) of "
                         f"compress+decompress+homadd, oracle C restatement, OpenMP {T} threads",
               "single_thread": {"value": round(rate1, 3), "unit": "GB/s", "cores": 1,
                                 "sample": f"first {m} elements, T=1, best of 1 after one warm-up "
                                           f"({secs1:.2f} s a pass)"}}

    # byte-for-byte parity of the timed workload with the oracle: the device
    # path's resident stream, sum and floats, and the host-buffer entry
    # points' outputs
    parity = {}
    eb_sweep = {}
    if rank == 0 and not args.no_parity:
        if ref_out is None:
            ref_out = oracle_outputs(xh, yh, eb, L, T)
        parity[f"eb{args.eb_rel:g}"] = {
            "stream": sa.tobytes() == ref_out["stream"],
            "sum": ss.tobytes() == ref_out["sum"],
            "floats": same_bits(xo.cpu().numpy(), ref_out["floats"]),
            "e2e_stream": hs_a[:ca].tobytes() == ref_out["stream"],
            "e2e_sum": hs_s[:cs].tobytes() == ref_out["sum"],
            "e2e_floats": same_bits(hy, ref_out["floats"]),
        }
        del ref_out
        # the same field at the other error bound of the sweep (1e-3 of range)
        for rel in (1e-3, 1e-4):
            if rel == args.eb_rel:
                continue
            eb2 = float(np.float32(rel * max(float(x.max() - x.min()), float(y.max() - y.min()))))
            sa2, sb2, ss2 = codec.new_stream(), codec.new_stream(), codec.new_stream()
            xo2 = torch.empty(n, dtype=torch.float32, device=dev)
            codec.compress(y, eb2, out=sb2)
            t_c = timed(lambda: codec.compress(x, eb2, out=sa2), 20, st)
            t_d = timed(lambda: codec.decompress(sa2, eb2, out=xo2), 20, st)
            t_h = timed(lambda: codec.homadd([sa2, sb2], out=ss2), 20, st)
            codec.check()
            c2a, c2b, c2s = sa2.size(), sb2.size(), ss2.size()
            alg2 = {"compress": 4 * n + c2a, "decompress": c2a + 4 * n, "homadd": c2a + c2b + c2s}
            ops = {}
            for name, t_ms in zip(("compress", "decompress", "homadd"), (t_c, t_d, t_h)):
                gbs = alg2[name] / (t_ms * 1e-3) / 1e9
                ops[name] = {"ms": round(t_ms, 4), "uncompressed_GBps": round(4 * n / (t_ms * 1e-3) / 1e9, 1),
                             "algorithmic_GBps": round(gbs, 1), "roofline_frac": round(gbs / peak, 4)}
            r2 = oracle_outputs(xh, yh, eb2, L, T)
            parity[f"eb{rel:g}"] = {"stream": sa2.tobytes() == r2["stream"], "sum": ss2.tobytes() == r2["sum"],
                                    "floats": same_bits(xo2.cpu().numpy(), r2["floats"])}
            eb_sweep[f"{rel:g}"] = {"eb": eb2, "per_op": ops,
                                    "compression_ratio": {"A": round(4 * n / c2a, 3), "sum": round(4 * n / c2s, 3)}}
            del sa2, sb2, ss2, xo2, r2

    extras = {}
    if rank == 0 and not args.no_extras:
        del hs_a, hs_b, hs_s, hy
        want = set(args.extras.split(","))
        for name, fn in (("reduction", lambda: reduction_bench(args, L, T, dev)), ("szp3d", lambda: szp3d_bench(args, dev)),
                         ("batched", lambda: batched_bench(args, L, dev)), ("serving", lambda: serving_bench(args, L, dev))):
            if name in want:
                extras[name] = fn()

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 2), "unit": "GB/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic: seeded log-normal GRF, P(k)~k^-3, exp(1.5 g) (stands in for NYX 512^3)",
            "config": workload_config(args, n, T),
            "roofline": roofline, "per_op": per_op,
            "compression_ratio": {"A": round(4 * n / ca, 3), "B": round(4 * n / cb, 3),
                                  "sum": round(4 * n / cs, 3)},
            "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": 3 * args.steps,
            "clocks": clk.summary(),
        }
        if eb_sweep:
            line["eb_sweep"] = eb_sweep
        line.update(extras)
        red = extras.get("reduction", {}).get("parity")
        if red:
            parity["reduction_p8"] = red
        bat = extras.get("batched", {}).get("parity")
        if bat:
            parity["batched"] = bat
        if parity:
            line["parity"] = parity
        print(json.dumps(line), flush=True)
        bad = [f"{k}.{kk}" for k, v in parity.items() for kk, vv in v.items() if vv is False]
        if bad:
            sys.stderr.write(f"parity with the oracle FAILED: {', '.join(bad)}\n")
            sys.exit(1)


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        backend = "nccl" if torch.cuda.is_available() and args.impl == "ours" else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local_rank)
        torch.distributed.init_process_group(backend)
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world, local_rank)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
