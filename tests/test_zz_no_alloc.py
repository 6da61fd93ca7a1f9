"""zccl_gpu_compress_noalloc, called through the C ABI: the same stream and
side index as zccl_gpu_compress, on consecutive calls that share the fixed
scratch array, and a clear rejection of inputs that need more scratch than
the array holds.  The file name keeps it last in collection, so it also runs
after every other GPU test has used the device."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

import zccl_gb300 as Z

ESCRATCH = -9
SCRATCH_BYTES = 1 << 20
TILE_FLOATS = 256 * 32  # blocks per tile x block size at L = 32


def _status(rc):
    return f"{rc}: {Z.STATUS.get(rc, '?')}"


def test_oversized_input_rejected_before_any_device_work():
    lib = Z.lib()
    desc = Z.StreamDesc(0, 0, 0, 0, 0)
    scratch = ctypes.c_void_p(1)
    # one segment: 16 + 8 * tiles bytes must fit; one float more than the
    # largest input that fits adds a block, and with it a tile
    n_max = 1 + ((SCRATCH_BYTES - 16) // 8) * TILE_FLOATS
    rc = lib.zccl_gpu_compress_noalloc(ctypes.byref(desc), None, n_max + 1, 1e-3, 32, 1, None,
                                       ctypes.byref(scratch))
    assert rc == ESCRATCH, _status(rc)
    assert scratch.value is None
    assert lib.zccl_gpu_strerror(ESCRATCH).decode() == Z.STATUS[ESCRATCH]
    rc = lib.zccl_gpu_compress_noalloc(ctypes.byref(desc), None, 2 ** 31, 1e-3, 32, 1, None, None)
    assert rc == ESCRATCH, _status(rc)
    # bad geometry is still an argument error
    rc = lib.zccl_gpu_compress_noalloc(ctypes.byref(desc), None, 3, 1e-3, 32, 4, None, None)
    assert rc == -1, _status(rc)


@pytest.mark.gpu
def test_noalloc_matches_compress_on_consecutive_calls():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = Z.lib()
    n, L, T = 3_000_017, 32, 5  # a remainder segment and a ragged last tile
    st = torch.cuda.current_stream().cuda_stream
    cap = lib.zccl_gpu_max_stream_bytes(n, L, T)
    nidx = lib.zccl_gpu_index_bytes(n, L, T)
    ws = torch.zeros(lib.zccl_gpu_workspace_bytes(n, L, T), dtype=torch.uint8, device="cuda")

    def stream():
        buf = torch.full((cap,), 0xA5, dtype=torch.uint8, device="cuda")
        idx = torch.zeros(nidx, dtype=torch.uint8, device="cuda")
        return buf, idx, Z.StreamDesc(buf.data_ptr(), cap, idx.data_ptr(), 0, 0)

    def size_of(desc):
        s = ctypes.c_size_t(0)
        assert lib.zccl_gpu_stream_size(ctypes.byref(desc), n, L, T, ctypes.byref(s), st) == 0
        return s.value

    g = torch.Generator(device="cuda").manual_seed(11)
    fields = [torch.randn(n, generator=g, device="cuda").cumsum_(0),
              torch.rand(n, generator=g, device="cuda") * 50.0 - 25.0]
    addrs, outs = [], []
    for x in fields:  # two calls in a row on the one scratch array
        eb = float(np.float32(1e-4 * float(x.max() - x.min())))
        rbuf, ridx, rdesc = stream()
        rc = lib.zccl_gpu_compress(ctypes.byref(rdesc), x.data_ptr(), n, eb, L, T, ws.data_ptr(), st)
        assert rc == 0, _status(rc)
        assert lib.zccl_gpu_check(ws.data_ptr(), st) == 0

        buf, idx, desc = stream()
        scratch = ctypes.c_void_p(0)
        rc = lib.zccl_gpu_compress_noalloc(ctypes.byref(desc), x.data_ptr(), n, eb, L, T, st,
                                           ctypes.byref(scratch))
        assert rc == 0, _status(rc)
        assert scratch.value
        rc = lib.zccl_gpu_check(scratch, st)
        assert rc == 0, _status(rc)
        addrs.append(scratch.value)
        assert desc.indexed == 1 and desc.qprev_valid == 1
        size = size_of(desc)
        assert size == size_of(rdesc)
        assert torch.equal(buf[:size], rbuf[:size])
        assert torch.equal(idx, ridx)
        outs.append((x, eb, bytes(buf[:size].cpu().numpy())))
    assert addrs[0] == addrs[1]
    # and both streams are the oracle's
    from oracle import zoracle
    port = zoracle.port()
    for x, eb, got in outs:
        assert got == port.compress(x.cpu().numpy(), eb, L, T)


@pytest.mark.gpu
def test_noalloc_at_the_scratch_limit():
    """An input whose status words fill the array to its last word: one
    segment of 131070 tiles at L = 8 (2048 floats a tile, 1.07 GB of
    input), 16 + 8 * 131070 = 1 MiB exactly.  Same bytes and index as
    zccl_gpu_compress; one float more is refused."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = Z.lib()
    L, T = 8, 1
    tiles = (SCRATCH_BYTES - 16) // 8
    n = 1 + tiles * 256 * L
    st = torch.cuda.current_stream().cuda_stream
    cap = lib.zccl_gpu_max_stream_bytes(n, L, T)
    nidx = lib.zccl_gpu_index_bytes(n, L, T)
    g = torch.Generator(device="cuda").manual_seed(5)
    x = (torch.randn(n, generator=g, device="cuda") * 0.01).cumsum_(0)
    eb = float(np.float32(1e-3 * float(x.max() - x.min())))
    ws = torch.zeros(lib.zccl_gpu_workspace_bytes(n, L, T), dtype=torch.uint8, device="cuda")
    sizes = []
    descs = []
    for noalloc in (False, True):
        buf = torch.zeros(cap, dtype=torch.uint8, device="cuda")
        idx = torch.zeros(nidx, dtype=torch.uint8, device="cuda")
        d = Z.StreamDesc(buf.data_ptr(), cap, idx.data_ptr(), 0, 0)
        if noalloc:
            scratch = ctypes.c_void_p(0)
            rc = lib.zccl_gpu_compress_noalloc(ctypes.byref(d), x.data_ptr(), n, eb, L, T, st,
                                               ctypes.byref(scratch))
            assert rc == 0, _status(rc)
            rc = lib.zccl_gpu_check(scratch, st)
        else:
            rc = lib.zccl_gpu_compress(ctypes.byref(d), x.data_ptr(), n, eb, L, T, ws.data_ptr(), st)
            assert rc == 0, _status(rc)
            rc = lib.zccl_gpu_check(ws.data_ptr(), st)
        assert rc == 0, _status(rc)
        s = ctypes.c_size_t(0)
        assert lib.zccl_gpu_stream_size(ctypes.byref(d), n, L, T, ctypes.byref(s), st) == 0
        sizes.append(s.value)
        descs.append((buf, idx))
    assert sizes[0] == sizes[1]
    assert torch.equal(descs[0][0][: sizes[0]], descs[1][0][: sizes[1]])
    assert torch.equal(descs[0][1], descs[1][1])
    del descs
    empty = Z.StreamDesc(0, 0, 0, 0, 0)
    rc = lib.zccl_gpu_compress_noalloc(ctypes.byref(empty), None, n + 1, eb, L, T, st, None)
    assert rc == ESCRATCH, _status(rc)
