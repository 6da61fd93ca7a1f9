"""The segmented compressed ring allgatherv, run for P ranks on one device.

MPIR_Allgatherv_intra_ring_RI2_mt_oa_record_seg (ZCCL/src/ZCCL_ring.c:1599-1774)
gathers every rank's chunk of floats onto every rank with compressed
messages cut into segments:

* every rank copies its own floats into its receive buffer (:1633-1637);
* its chunk is cut into segments of SEGSIZE = 8 MiB of floats
  (ZCCL/include/ZCCL_libs.h:31; ZCCL_ring.c:1666-1670), each compressed
  once by the fastmode1 codec into a frame: the stream's size as a
  little-endian size_t, then the stream bytes (:1671-1675);
* P - 1 ring steps (:1684-1774): at step i a rank forwards the frames of
  chunk (rank - i) unchanged to its right-hand neighbour and receives those
  of chunk (rank - 1 - i) from the left, decompressing every frame as soon
  as it has arrived into its place in the receive buffer while it goes on
  sending (:1708-1756).

So chunk c's floats are the owner's originals on rank c and the same
decompressed floats on every other rank; frames are never recompressed.
MPIR_Allgatherv_intra_ring_RI2_mt_oa_record_seg_2 (ZCCL/src/ZCCL_appendix.c:756-941)
is the same exchange with the fixed-rate appendix codec (`fixed=True`).
The reference measures the element extent as sizeof(MPI_Datatype), which is
4 bytes under MPICH (an int handle) and equals sizeof(float); 4 is used here.

On one device the P ranks' buffers are device tensors and a frame on the
wire is the sender's frame buffer itself.  The receiver sees wire bytes
only, so every frame is decompressed as a byte stream (the side index is
rebuilt by the header walk), exactly as a receiving GPU would.  The
overlap of the reference (decompress one segment while sending the next)
becomes two CUDA streams: frames are compressed on one, and each frame's
decompression on the other starts as soon as an event says that frame is
complete.
"""
from __future__ import annotations

import ctypes

from . import Codec, DeviceStream, _check, lib

SEGSIZE = 8 * 1024 * 1024  # bytes of floats per segment (ZCCL/include/ZCCL_libs.h:31)
EXTENT = 4                 # bytes per element


def segments(count: int, segsize: int = SEGSIZE) -> tuple[list[int], list[int]]:
    """Element counts and offsets of a chunk's segments (ZCCL_ring.c:1666-1670):
    segsize bytes each, the last one the rest."""
    nbytes = count * EXTENT
    nseg = (nbytes + segsize - 1) // segsize
    cnts = [(segsize if i < nseg - 1 else nbytes - i * segsize) // EXTENT for i in range(nseg)]
    return cnts, [i * segsize // EXTENT for i in range(nseg)]


class SegmentedAllgatherv:
    """The segmented allgatherv for P ranks with `counts[r]` floats each,
    placed at `displs[r]` of every receive buffer (contiguous by default)."""

    def __init__(self, counts, L: int = 32, T: int = 1, segsize: int = SEGSIZE, displs=None,
                 device: str = "cuda", fixed: bool = False):
        import torch
        self.counts = [int(c) for c in counts]
        self.P, self.L, self.T, self.segsize = len(self.counts), int(L), int(T), int(segsize)
        self.fixed = bool(fixed)
        if segsize % EXTENT or segsize <= 0:
            raise ValueError("segsize must be a positive multiple of 4 bytes")
        if displs is None:
            displs, acc = [], 0
            for c in self.counts:
                displs.append(acc)
                acc += c
        self.displs = [int(d) for d in displs]
        self.total = max(d + c for d, c in zip(self.displs, self.counts))
        self.segs = [segments(c, self.segsize) for c in self.counts]
        for cnts, _ in self.segs:
            if any(n < self.T for n in cnts):
                raise ValueError(f"every segment needs at least T={T} floats: {cnts}")
        self.device = torch.device(device)
        self.sc = torch.cuda.Stream(device=self.device)  # compression
        self.sd = torch.cuda.Stream(device=self.device)  # decompression
        self._codecs: dict = {}

    def codec(self, n: int, which: str) -> Codec:
        key = (n, which)
        if key not in self._codecs:
            self._codecs[key] = Codec(n, self.L, self.T, device=str(self.device),
                                      stream=self.sc if which == "c" else self.sd, fixed=self.fixed)
        return self._codecs[key]

    def frames(self, x, eb: float, events: bool = False):
        """One rank's chunk as frames (uint8 device tensors of 8 + capacity
        bytes: the stream's size, then its bytes), compressed on the
        compression stream; with `events`, also an event per frame."""
        import torch
        cnts, offs = segments(x.numel(), self.segsize)
        out, evs = [], []
        for n, o in zip(cnts, offs):
            c = self.codec(n, "c")
            with torch.cuda.stream(self.sc):  # allocated (and its index zeroed) where it is written
                frame = torch.empty(8 + c.max_stream_bytes, dtype=torch.uint8, device=self.device)
                s = DeviceStream(c, data=frame[8:])
            if not torch.cuda.is_current_stream_capturing():
                frame.record_stream(self.sd)  # read there by the receivers (a graph keeps its own pool)
            c.compress(x[o: o + n], eb, out=s)
            _check(lib().zccl_gpu_frame_size(ctypes.byref(s.desc), frame.data_ptr(),
                                             ctypes.c_void_p(self.sc.cuda_stream)), "zccl_gpu_frame_size")
            out.append(frame)
            if events:
                ev = torch.cuda.Event()
                ev.record(self.sc)
                evs.append(ev)
        return (out, evs) if events else out

    def _unframe(self, frame, y, n: int, eb: float) -> None:
        """Decompress one received frame (wire bytes only) into y[0:n]."""
        import torch
        c = self.codec(n, "d")
        with torch.cuda.stream(self.sd):
            s = DeviceStream(c, data=frame[8:])  # a fresh index: the header walk rebuilds it
        c.decompress(s, eb, out=y)

    def run(self, xs, eb: float, per_rank_outputs: bool = False, _check: bool = True):
        """Allgather the P tensors in xs.  Returns rank 0's receive buffer, or
        every rank's with per_rank_outputs, and keeps the frames in
        self.sent (chunk c's frames are rank c's)."""
        import torch
        P = self.P
        cur = torch.cuda.current_stream(self.device)
        ranks = range(P) if per_rank_outputs else [0]
        recv = {r: torch.empty(self.total, dtype=torch.float32, device=self.device) for r in ranks}
        self.sc.wait_stream(cur)
        self.sd.wait_stream(cur)
        with torch.cuda.stream(self.sd):
            for r in ranks:  # own floats in place (ZCCL_ring.c:1633-1637)
                recv[r][self.displs[r]: self.displs[r] + self.counts[r]].copy_(xs[r])
        # every rank compresses its chunk once (ZCCL_ring.c:1666-1675)
        sent = [self.frames(xs[c], eb, events=True) for c in range(P)]
        # P - 1 steps: rank r receives chunk (r - 1 - i) and decompresses its
        # frames as they arrive (ZCCL_ring.c:1684-1774)
        for i in range(P - 1):
            for r in ranks:
                c = (r - 1 - i) % P
                frames, evs = sent[c]
                cnts, offs = self.segs[c]
                for f, ev, n, o in zip(frames, evs, cnts, offs):
                    self.sd.wait_event(ev)
                    d = self.displs[c] + o
                    self._unframe(f, recv[r][d: d + n], n, eb)
        self.sent = [f for f, _ in sent]
        cur.wait_stream(self.sd)
        cur.wait_stream(self.sc)
        if _check:
            for cd in self._codecs.values():
                cd.check()
        return [recv[r] for r in ranks] if per_rank_outputs else recv[0]

    def capture(self, xs, eb: float, per_rank_outputs: bool = False):
        """Record the whole exchange (P compressions, every decompression on
        the second stream, the events between them) into one CUDA graph
        once; returns (graph, outputs).  graph.replay() repeats it on the
        same input tensors (write new data into them) and outputs, without
        host work per codec call.  check() reads the device status after
        replays."""
        import torch
        self.run(xs, eb, per_rank_outputs)  # the codecs and their scratch exist before capture
        side = torch.cuda.Stream(device=self.device)
        side.wait_stream(torch.cuda.current_stream(self.device))
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=side, capture_error_mode="relaxed"):
            outs = self.run(xs, eb, per_rank_outputs, _check=False)
        torch.cuda.current_stream(self.device).wait_stream(side)
        return g, outs

    def check(self) -> None:
        for cd in self._codecs.values():
            cd.check()
