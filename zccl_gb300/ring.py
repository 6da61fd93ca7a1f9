"""The compressed ring allreduce that calls the codec, run for P ranks on one
device.

ZCCL's allreduce hands the codec its data in ring order: every rank splits
its `count` floats into P chunks (ZCCL/src/ZCCL_ring_ho.c:221-233), and
P - 1 reduce-scatter steps pass chunks to the right-hand neighbour, which
adds them into its own copy, before an allgather spreads the reduced chunks.
The two variants differ in what travels:

* homomorphic (MPI_Allreduce_ZCCL_RI2_mt_oa_ho_record,
  ZCCL/src/ZCCL_ring_ho.c:177-317): every rank compresses its P chunks once;
  each step adds the received compressed chunk into the local compressed
  chunk with the homomorphic add; the allgather (ZCCL_ring_ho.c:12-175)
  passes the reduced compressed chunks around and every rank decompresses
  all P of them.
* decompress-add-recompress, "DOC" (MPI_Allreduce_ZCCL_RI2_mt_oa_record,
  ZCCL/src/ZCCL_ring.c:979-1108): each step compresses the float chunk being
  sent, and the receiver decompresses it and adds it to its float chunk; the
  allgather (ZCCL_ring.c:814-978) compresses each rank's reduced chunk,
  passes it around, and every rank decompresses all P chunks.

Here the P ranks' buffers are P device tensors, a send is the hand-over of
a device stream, and every rank's codec work runs, in ring order, on one
stream of one GPU.  All ranks end with the same floats, so one copy of the
result is returned; `per_rank_outputs=True` keeps every rank's copy.

Also here: the one-shot reduction of P ranks' chunks (the P-way
homomorphic add, the pairwise fold, the pairwise tree, against
decompress-add-recompress) that the P = 8 x 16M benchmark measures.
"""
from __future__ import annotations

from . import BATCH_COMPRESS, BATCH_DECOMPRESS, BATCH_HOMADD, Batch, Codec, DeviceStream, check_all


def ring_counts(count: int, P: int) -> tuple[list[int], list[int]]:
    """Chunk sizes and offsets of the ring (ZCCL/src/ZCCL_ring_ho.c:219-233):
    ceil(count / P) each, the last one shorter, zero-size chunks after it."""
    cnts, total = [0] * P, 0
    for i in range(P):
        c = (count + P - 1) // P
        if total + c > count:
            cnts[i] = count - total
            break
        cnts[i] = c
        total += c
    displs = [0] * P
    for i in range(1, P):
        displs[i] = displs[i - 1] + cnts[i - 1]
    return cnts, displs


class RingAllreduce:
    """Both ring allreduces for P ranks of `count` floats on one device.

    batched (default): every step's P codec calls of the same kind run as
    one batch launch (zccl_gpu_batch_*): the homomorphic ring is one
    compression batch of the P x P chunks, P - 1 sum batches and one
    decompression batch; the DOC ring, per step, a compression batch and a
    decompress-and-accumulate batch, then the allgather's compression and
    decompression batches.  The streams and float buffers the steps pass
    around belong to the ring object and the batches are planned once per
    input and error bound, so repeated calls replay the same launches; the
    returned floats live in a buffer the next call reuses.
    batched=False: one C-ABI call per chunk and step, the reference's call
    sequence (the results are the same bytes)."""

    def __init__(self, count: int, P: int, L: int = 32, T: int = 1, device: str = "cuda", batched: bool = True):
        self.count, self.P, self.L, self.T = int(count), int(P), int(L), int(T)
        self.cnts, self.displs = ring_counts(self.count, self.P)
        if min(self.cnts) < self.T:
            raise ValueError(f"every ring chunk needs at least T={T} floats: {self.cnts}")
        self.device = device
        self.batched = bool(batched)
        self._codecs: dict[int, Codec] = {}
        self._plans: dict = {}
        self._bufs = None

    def codec(self, c: int) -> Codec:
        n = self.cnts[c]
        if n not in self._codecs:
            self._codecs[n] = Codec(n, self.L, self.T, device=self.device)
        return self._codecs[n]

    def _chunk(self, x, c):
        return x[self.displs[c]: self.displs[c] + self.cnts[c]]

    def _check(self, extra=()):
        """Raise if any call on any chunk's codec, or any batch, failed since
        the last check (the device status words keep every call's errors
        until read); one device-to-host read for all of them."""
        check_all(list(self._codecs.values()) + list(self._plans.values()) + list(extra))

    # ---- one call per chunk and step -------------------------------------
    def _allgather_decompress(self, reduced, eb, per_rank_outputs):
        """Every rank decompresses all P reduced chunks into its result."""
        import torch
        outs = []
        for r in range(self.P if per_rank_outputs else 1):
            y = torch.empty(self.count, dtype=torch.float32, device=self.device)
            for c in range(self.P):
                self.codec(c).decompress(reduced[c], eb, out=self._chunk(y, c))
            outs.append(y)
        self._check()
        return outs if per_rank_outputs else outs[0]

    def homomorphic(self, xs, eb: float, per_rank_outputs: bool = False):
        """MPI_Allreduce_ZCCL_RI2_mt_oa_ho_record for the P tensors in xs.
        Returns the allreduced floats (or every rank's copy) and leaves the
        reduced compressed chunks in self.reduced (chunk c is rank c's)."""
        if self.batched:
            return self._homomorphic_batched(xs, eb, per_rank_outputs)
        P = self.P
        # every rank compresses its P chunks (ZCCL_ring_ho.c:250-258)
        S = [[self.codec(c).compress(self._chunk(xs[r], c), eb) for c in range(P)] for r in range(P)]
        # P - 1 reduce-scatter steps (ZCCL_ring_ho.c:260-297): rank r receives
        # chunk (r - 2 - i) from rank r - 1 and adds it into its own copy
        for i in range(P - 1):
            for r in range(P):
                src, c = (r - 1) % P, (r - 2 - i) % P
                S[r][c] = self.codec(c).homadd([S[src][c], S[r][c]])
        self.reduced = [S[c][c] for c in range(P)]
        self._check()
        return self._allgather_decompress(self.reduced, eb, per_rank_outputs)

    def doc(self, xs, eb: float, per_rank_outputs: bool = False):
        """MPI_Allreduce_ZCCL_RI2_mt_oa_record for the P tensors in xs."""
        if self.batched:
            return self._doc_batched(xs, eb, per_rank_outputs)
        P = self.P
        acc = [x.clone() for x in xs]
        for i in range(P - 1):
            # every rank compresses the chunk it sends (ZCCL_ring.c:1050-1058) ...
            msgs = [self.codec((r - 1 - i) % P).compress(self._chunk(acc[r], (r - 1 - i) % P), eb)
                    for r in range(P)]
            # ... and adds the decompressed chunk it receives (ZCCL_ring.c:1074-1077)
            for r in range(P):
                src, c = (r - 1) % P, (r - 2 - i) % P
                self.codec(c).decompress_accumulate(msgs[src], eb, self._chunk(acc[r], c))
        # the allgather compresses each rank's reduced chunk (ZCCL_ring.c:863-869)
        self.reduced = [self.codec(c).compress(self._chunk(acc[c], c), eb) for c in range(P)]
        self._check()
        return self._allgather_decompress(self.reduced, eb, per_rank_outputs)

    # ---- one batch per step ----------------------------------------------
    def _buffers(self, variant: str):
        """The ring's own streams and floats for one variant, made on its
        first run: the P x P chunk streams and a spare stream per rank
        ("ho"), or P float accumulators, P message streams and P reduced
        streams ("doc"); and the variant's result."""
        import torch
        if self._bufs is None:
            self._bufs = {}
        b = self._bufs.get(variant)
        if b is None:
            P = self.P
            if variant == "ho":
                b = {"S": [[self.codec(c).new_stream() for c in range(P)] for _ in range(P)],
                     "spare": [self.codec(c).new_stream() for c in range(P)]}
            else:
                b = {"acc": [torch.empty(self.count, dtype=torch.float32, device=self.device) for _ in range(P)],
                     "msg": [self.codec(c).new_stream() for c in range(P)],
                     "red": [self.codec(c).new_stream() for c in range(P)]}
            b["y"] = torch.empty(self.count, dtype=torch.float32, device=self.device)
            self._bufs[variant] = b
        return b

    def _plan(self, key, kind, jobs):
        b = self._plans.get(key)
        if b is None:
            b = Batch(kind, jobs, self.L, device=self.device)
            self._plans[key] = b
        return b

    def _gather_batched(self, reduced, eb, per_rank_outputs, tag):
        import torch
        P = self.P
        if per_rank_outputs:  # every rank's copy, one batch of P x P decompressions
            ys = [torch.empty(self.count, dtype=torch.float32, device=self.device) for _ in range(P)]
            jobs = [(reduced[c], eb, self.T, self._chunk(y, c), False) for y in ys for c in range(P)]
            b = Batch(BATCH_DECOMPRESS, jobs, self.L, device=self.device)
            b.run()
            self._check([b])
            return ys
        y = self._buffers(tag)["y"]
        self._plan((tag, "gather", eb), BATCH_DECOMPRESS,
                   [(reduced[c], eb, self.T, self._chunk(y, c), False) for c in range(P)]).run()
        self._check()
        return y

    def _homomorphic_batched(self, xs, eb, per_rank_outputs):
        P = self.P
        B = self._buffers("ho")
        S = [row[:] for row in B["S"]]
        spare = B["spare"][:]
        key = ("ho", "compress", eb, tuple(x.data_ptr() for x in xs))
        if key not in self._plans:  # a new input: forget the previous one's plan
            for k in [k for k in self._plans if k[:2] == ("ho", "compress")]:
                del self._plans[k]
        self._plan(key, BATCH_COMPRESS,
                   [(self._chunk(xs[r], c), eb, self.T, S[r][c]) for r in range(P) for c in range(P)]).run()
        for i in range(P - 1):
            jobs = []
            for r in range(P):
                src, c = (r - 1) % P, (r - 2 - i) % P
                jobs.append(([S[src][c], S[r][c]], self.T, spare[c]))
            self._plan(("ho", "step", i), BATCH_HOMADD, jobs).run()
            for r in range(P):  # the sums become the ranks' chunks; the old chunks the spares
                c = (r - 2 - i) % P
                S[r][c], spare[c] = spare[c], S[r][c]
        self.reduced = [S[c][c] for c in range(P)]
        return self._gather_batched(self.reduced, eb, per_rank_outputs, "ho")

    def _doc_batched(self, xs, eb, per_rank_outputs):
        P = self.P
        B = self._buffers("doc")
        acc, msg, red = B["acc"], B["msg"], B["red"]
        for a, x in zip(acc, xs):
            a.copy_(x)
        for i in range(P - 1):
            # every rank compresses the chunk it sends (a message per chunk:
            # the P ranks send P different chunks in a step) ...
            self._plan(("doc", "send", i, eb), BATCH_COMPRESS,
                       [(self._chunk(acc[r], (r - 1 - i) % P), eb, self.T, msg[(r - 1 - i) % P])
                        for r in range(P)]).run()
            # ... and adds the one it receives, decompressed, into its own
            jobs = []
            for r in range(P):
                c = (r - 2 - i) % P
                jobs.append((msg[c], eb, self.T, self._chunk(acc[r], c), True))
            self._plan(("doc", "add", i, eb), BATCH_DECOMPRESS, jobs).run()
        self._plan(("doc", "reduced", eb), BATCH_COMPRESS,
                   [(self._chunk(acc[c], c), eb, self.T, red[c]) for c in range(P)]).run()
        self.reduced = red[:]
        return self._gather_batched(self.reduced, eb, per_rank_outputs, "doc")


def reduce_homomorphic(codec: Codec, streams: list[DeviceStream], out: DeviceStream | None = None):
    """The P ranks' compressed chunks summed by one P-way homomorphic add."""
    return codec.homadd(streams, out=out)


def reduce_pairwise(codec: Codec, streams: list[DeviceStream], outs: list[DeviceStream] | None = None):
    """The same sum folded pairwise, as the ring's P - 1 steps do
    (acc = received + acc, ZCCL/src/ZCCL_ring_ho.c:281-287).  With outs (two
    streams) the partial sums alternate between them instead of new ones."""
    acc = streams[0]
    for i, s in enumerate(streams[1:]):
        acc = codec.homadd([s, acc], out=outs[i & 1] if outs else None)
    return acc


class PairwiseTree:
    """The same sum by two-way adds arranged as a binary tree: level k adds
    pairs of level k - 1's sums (an odd one out goes up unchanged), every
    pair of a level in one batch launch, so ceil(log2 P) launches instead of
    the fold's P - 1 calls.  Addition modulo 2^32 is associative and a
    sum's encoding depends on its values alone, so the result is the fold's
    bytes.  Planned once for the given streams, whose buffers the plans
    bind; each sum gets a stream of its own (P - 1 in all), so no add
    writes over a stream another add of its level reads.  run() replays the
    levels on `stream` (a torch stream, default the current one) and returns
    the sum."""

    def __init__(self, codec: Codec, streams: list[DeviceStream], stream=None):
        if len(streams) < 2:
            raise ValueError("a pairwise tree needs at least two streams")
        self.stream = stream
        self.plans: list[Batch] = []
        self.sums: list[DeviceStream] = []
        cur = list(streams)
        while len(cur) > 1:
            nxt, jobs = [], []
            for i in range(0, len(cur) - 1, 2):
                o = codec.new_stream()
                self.sums.append(o)
                jobs.append(([cur[i], cur[i + 1]], codec.T, o))
                nxt.append(o)
            if len(cur) & 1:
                nxt.append(cur[-1])
            self.plans.append(Batch(BATCH_HOMADD, jobs, codec.L, device=codec.device, stream=stream))
            cur = nxt
        self.result = cur[0]

    def run(self) -> DeviceStream:
        for b in self.plans:
            b.run(self.stream)
        return self.result

    def check(self):
        check_all(self.plans)


def reduce_doc(codec: Codec, streams: list[DeviceStream], eb: float, out: DeviceStream | None = None,
               total=None):
    """Decompress every chunk, add the floats in rank order, recompress: the
    first chunk decompressed, each later one decompressed and added in one
    pass (the float sum of MPI_Reduce_local, ZCCL/src/ZCCL_ring.c:1074-1076).
    total, if given, is the float buffer to use."""
    import torch
    if total is None:
        total = torch.empty(codec.n, dtype=torch.float32, device=codec.device)
    codec.decompress(streams[0], eb, out=total)
    for s in streams[1:]:
        codec.decompress_accumulate(s, eb, total)
    return codec.compress(total, eb, out=out), total
