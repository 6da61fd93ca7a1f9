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
homomorphic add against decompress-add-recompress) that the P = 8 x 16M
benchmark measures.
"""
from __future__ import annotations

from . import Codec, DeviceStream


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
    """Both ring allreduces for P ranks of `count` floats on one device."""

    def __init__(self, count: int, P: int, L: int = 32, T: int = 1, device: str = "cuda"):
        self.count, self.P, self.L, self.T = int(count), int(P), int(L), int(T)
        self.cnts, self.displs = ring_counts(self.count, self.P)
        if min(self.cnts) < self.T:
            raise ValueError(f"every ring chunk needs at least T={T} floats: {self.cnts}")
        self.device = device
        self._codecs: dict[int, Codec] = {}

    def codec(self, c: int) -> Codec:
        n = self.cnts[c]
        if n not in self._codecs:
            self._codecs[n] = Codec(n, self.L, self.T, device=self.device)
        return self._codecs[n]

    def _chunk(self, x, c):
        return x[self.displs[c]: self.displs[c] + self.cnts[c]]

    def _check(self):
        """Raise if any call on any chunk's codec failed since the last check
        (the device status words keep every call's errors until read)."""
        for cd in self._codecs.values():
            cd.check()

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
        P = self.P
        acc = [x.clone() for x in xs]
        for i in range(P - 1):
            # every rank compresses the chunk it sends (ZCCL_ring.c:1050-1058) ...
            msgs = [self.codec((r - 1 - i) % P).compress(self._chunk(acc[r], (r - 1 - i) % P), eb)
                    for r in range(P)]
            # ... and adds the decompressed chunk it receives (ZCCL_ring.c:1074-1077)
            for r in range(P):
                src, c = (r - 1) % P, (r - 2 - i) % P
                self._chunk(acc[r], c).add_(self.codec(c).decompress(msgs[src], eb))
        # the allgather compresses each rank's reduced chunk (ZCCL_ring.c:863-869)
        self.reduced = [self.codec(c).compress(self._chunk(acc[c], c), eb) for c in range(P)]
        self._check()
        return self._allgather_decompress(self.reduced, eb, per_rank_outputs)


def reduce_homomorphic(codec: Codec, streams: list[DeviceStream], out: DeviceStream | None = None):
    """The P ranks' compressed chunks summed by one P-way homomorphic add."""
    return codec.homadd(streams, out=out)


def reduce_pairwise(codec: Codec, streams: list[DeviceStream]):
    """The same sum folded pairwise, as the ring's P - 1 steps do
    (acc = received + acc, ZCCL/src/ZCCL_ring_ho.c:281-287)."""
    acc = streams[0]
    for s in streams[1:]:
        acc = codec.homadd([s, acc])
    return acc


def reduce_doc(codec: Codec, streams: list[DeviceStream], eb: float, out: DeviceStream | None = None):
    """Decompress every chunk, add the floats in rank order, recompress."""
    import torch
    total = torch.zeros(codec.n, dtype=torch.float32, device=codec.device)
    for s in streams:
        total.add_(codec.decompress(s, eb))
    return codec.compress(total, eb, out=out), total
