"""GPU parity: every result of the CUDA path, called through the C ABI, must be
bit-identical to the reference codec's (golden vectors written by the
reference itself) or to the oracle port on larger inputs.  Floats are
compared bit for bit; the error bounds are checked as properties."""
from __future__ import annotations

import hashlib

import numpy as np
import pytest

import zccl_gb300 as Z

pytestmark = pytest.mark.gpu


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    if not t.cuda.is_available():
        pytest.skip("no CUDA device")
    Z.lib()
    return t


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def test_compress_matches_reference(golden, torch):
    for c in golden.cases:
        codec = Z.Codec(c["n"], c["L"], c["T"])
        s = codec.compress(dev(torch, golden.x(c)), c["eb"])
        codec.check()
        assert s.tobytes() == golden.stream(c, "s"), c


def test_decompress_matches_reference(golden, torch):
    for c in golden.cases:
        codec = Z.Codec(c["n"], c["L"], c["T"])
        own = codec.compress(dev(torch, golden.x(c)), c["eb"])
        y = codec.decompress(own, c["eb"])
        codec.check()
        assert sha(y.cpu().numpy()) == c["dec_s"], c
        foreign = Z.DeviceStream.from_bytes(codec, golden.stream(c, "s"))
        y2 = codec.decompress(foreign, c["eb"])  # walks the headers, then value look-back
        codec.check()
        assert sha(y2.cpu().numpy()) == c["dec_s"], c
        y3 = codec.decompress(foreign, c["eb"])  # second pass uses the recovered index
        codec.check()
        assert sha(y3.cpu().numpy()) == c["dec_s"], c


def test_homadd_matches_reference(golden, torch):
    for c in golden.cases:
        codec = Z.Codec(c["n"], c["L"], c["T"])
        a = codec.compress(dev(torch, golden.x(c)), c["eb"])
        b = codec.compress(dev(torch, golden.y(c)), c["eb"])
        h = codec.homadd([a, b])
        codec.check()
        assert h.tobytes() == golden.stream(c, "h"), c
        assert sha(codec.decompress(h, c["eb"]).cpu().numpy()) == c["dec_h"], c
        fa = Z.DeviceStream.from_bytes(codec, golden.stream(c, "s"))
        fb = Z.DeviceStream.from_bytes(codec, golden.stream(c, "t"))
        hf = codec.homadd([fa, fb])
        codec.check()
        assert hf.tobytes() == golden.stream(c, "h"), c
        assert sha(codec.decompress(hf, c["eb"]).cpu().numpy()) == c["dec_h"], c


def test_pway_reduction_equals_reference_fold(golden, torch):
    r = golden.meta["reduction"]
    codec = Z.Codec(r["n"], r["L"], r["T"])
    streams = [codec.compress(dev(torch, golden.arr[f"p8x{k}"]), r["eb"]) for k in range(r["P"])]
    s = codec.homadd(streams)
    codec.check()
    assert s.tobytes() == golden.arr["p8sum"].tobytes()
    assert sha(codec.decompress(s, r["eb"]).cpu().numpy()) == r["dec_sum"]
    foreign = [Z.DeviceStream.from_bytes(codec, st.tobytes()) for st in streams]
    assert codec.homadd(foreign[::-1]).tobytes() == golden.arr["p8sum"].tobytes()


def n_blocks(n, L, T):
    def seg(m):
        return -(-(m - 1) // L) if m else 0
    return T * seg(n // T) + seg(n % T)


def test_branch_case_counters(golden, torch):
    """The reference's four two-input branch counters (ZCCLd_float.c:2175-2764):
    a constant input against a noisy one only takes 'first zero' (or 'both
    zero' where the noisy block happens to be flat)."""
    c = next(c for c in golden.cases if c["kind"] == "const_vs_noise")
    codec = Z.Codec(c["n"], c["L"], c["T"])
    a = codec.compress(dev(torch, golden.x(c)), c["eb"])
    b = codec.compress(dev(torch, golden.y(c)), c["eb"])
    cases = torch.zeros(4, dtype=torch.int64, device="cuda")
    codec.homadd([a, b], cases=cases)
    codec.check()
    both0, first0, second0, both = cases.cpu().tolist()
    assert second0 == 0 and both == 0
    assert both0 + first0 == n_blocks(c["n"], c["L"], c["T"])
    assert first0 > 0


@pytest.mark.parametrize("T", [1, 3])
def test_dropin_host_pointers(golden, torch, T):
    Z.set_omp_threads(T)
    picked = [c for c in golden.cases if c["T"] == T][::9]
    for c in picked:
        n, L, eb = c["n"], c["L"], c["eb"]
        x, y = golden.x(c), golden.y(c)
        cap = 4 * n + 8 * T + 4096
        s = np.zeros(cap, np.uint8)
        size = Z.ZCCL_float_openmp_threadblock_arg(s, x, 0, eb, n, L)
        assert s[:size].tobytes() == golden.stream(c, "s"), c
        t = np.zeros(cap, np.uint8)
        tsize = Z.ZCCL_float_openmp_threadblock_arg(t, y, 0, eb, n, L)
        out = np.zeros(n, np.float32)
        Z.ZCCL_float_decompress_openmp_threadblock_arg(out, n, eb, L, s)
        assert sha(out) == c["dec_s"], c
        # in place, as the ring does: result written over the second input
        acc = Z.ZCCL_float_homomophic_add_openmp_threadblock(t, 5, n, eb, L, s, t)
        assert acc - 5 == len(golden.stream(c, "h"))  # *final_cmpSize is incremented
        assert t[: acc - 5].tobytes() == golden.stream(c, "h"), c
        assert tsize > 0


def test_dropin_single_thread_variants(golden, torch):
    for c in [c for c in golden.cases if c["T"] == 1][::11]:
        n, L, eb = c["n"], c["L"], c["eb"]
        s = np.zeros(4 * n + 4096, np.uint8)
        size = Z.ZCCL_float_single_thread_arg(s, golden.x(c), 0, eb, n, L)
        assert s[:size].tobytes() == golden.stream(c, "s")
        out = np.zeros(n, np.float32)
        Z.ZCCL_float_decompress_single_thread_arg(out, n, eb, L, s)
        assert sha(out) == c["dec_s"]
        t = np.frombuffer(golden.stream(c, "t"), np.uint8).copy()
        h = np.zeros(4 * n + 4096, np.uint8)
        hs = Z.ZCCL_float_homomophic_add_single_thread(h, 0, n, eb, L, s, t)
        assert h[:hs].tobytes() == golden.stream(c, "h")


def test_dropin_device_pointers(golden, torch):
    Z.set_omp_threads(8)
    for c in [c for c in golden.cases if c["T"] == 8][::13]:
        n, L, eb = c["n"], c["L"], c["eb"]
        x = dev(torch, golden.x(c))
        s = torch.zeros(4 * n + 8192, dtype=torch.uint8, device="cuda")
        size = Z.ZCCL_float_openmp_threadblock_arg(s, x, 0, eb, n, L)
        assert s[:size].cpu().numpy().tobytes() == golden.stream(c, "s")
        out = torch.zeros(n, dtype=torch.float32, device="cuda")
        Z.ZCCL_float_decompress_openmp_threadblock_arg(out, n, eb, L, s)
        assert sha(out.cpu().numpy()) == c["dec_s"]
        t = dev(torch, np.frombuffer(golden.stream(c, "t"), np.uint8).copy())
        t2 = torch.zeros(4 * n + 8192, dtype=torch.uint8, device="cuda")
        t2[: t.numel()] = t
        hs = Z.ZCCL_float_homomophic_add_openmp_threadblock(t2, 0, n, eb, L, s, t2)
        assert t2[:hs].cpu().numpy().tobytes() == golden.stream(c, "h")


def test_generic_block_sizes_against_port(port, torch):
    rng = np.random.default_rng(3)
    for L in (33, 64, 100, 256):
        for T in (1, 5):
            n = 20000 + L
            x = np.cumsum(rng.normal(0, 0.1, n)).astype(np.float32)
            y = np.cumsum(rng.normal(0, 0.1, n)).astype(np.float32)
            eb = float(np.float32(1e-4 * (x.max() - x.min())))
            codec = Z.Codec(n, L, T)
            a, b = codec.compress(dev(torch, x), eb), codec.compress(dev(torch, y), eb)
            sa, sb = port.compress(x, eb, L, T), port.compress(y, eb, L, T)
            assert a.tobytes() == sa
            assert codec.homadd([a, b]).tobytes() == port.homadd(sa, sb, n, eb, L, T)
            assert np.array_equal(codec.decompress(a, eb).cpu().numpy(),
                                  port.decompress(sa, n, eb, L, T))
            codec.check()


def test_dropin_host_stream_with_a_long_last_chunk(port, torch):
    """A host stream carries no length: its last chunk is first read at
    twice the other chunks' average size, and read again in full when the
    walk runs past that.  Here the last of four chunks is noise and the rest
    nearly constant, so the first read falls short; decompress and the add
    must still give the oracle's floats and bytes."""
    T, L = 4, 32
    Z.set_omp_threads(T)
    rng = np.random.default_rng(23)
    n = 4 * 50000 + 3
    x = np.full(n, 1.0, np.float32)
    x[3 * (n // 4):] = rng.normal(0, 1.0, n - 3 * (n // 4)).astype(np.float32)
    y = (x + np.float32(0.5)).astype(np.float32)
    eb = float(np.float32(1e-4 * (x.max() - x.min())))
    sx, sy = port.compress(x, eb, L, T), port.compress(y, eb, L, T)
    last = int.from_bytes(sx[8 * (T - 1): 8 * T], "little")
    assert len(sx) - 8 * T - last > 2 * last // (T - 1) + 65536  # the first read is short
    cap = 4 * n + 8 * T + 4096
    s = np.zeros(cap, np.uint8)
    s[: len(sx)] = np.frombuffer(sx, np.uint8)
    t = np.zeros(cap, np.uint8)
    t[: len(sy)] = np.frombuffer(sy, np.uint8)
    out = np.zeros(n, np.float32)
    Z.ZCCL_float_decompress_openmp_threadblock_arg(out, n, eb, L, s)
    assert np.array_equal(out.view(np.uint32), port.decompress(sx, n, eb, L, T).view(np.uint32))
    acc = Z.ZCCL_float_homomophic_add_openmp_threadblock(t, 0, n, eb, L, s, t)
    assert t[:acc].tobytes() == port.homadd(sx, sy, n, eb, L, T)


def test_walk_long_blocks_against_port(port, torch):
    """Byte-only streams (the header walk rebuilds the index) with blocks of
    up to 64, 128 and 256 elements: blocks of 256 bytes or more take the
    walk's 32-bit window tables and, at 256 elements, its final pass with
    fewer warps.  Noisy data with a wide range gives widths up to the top;
    decompress and the add of two such streams must equal the oracle's."""
    rng = np.random.default_rng(19)
    for L in (48, 64, 128, 256):
        for T in (1, 3):
            n = 40 * L * 64 + 5 * L + 7
            x = (np.cumsum(rng.normal(0, 1.0, n)) * rng.choice([1.0, 3e3], n)).astype(np.float32)
            y = np.cumsum(rng.normal(0, 0.01, n)).astype(np.float32)
            eb = float(np.float32(1e-4 * (x.max() - x.min())))
            sa, sb = port.compress(x, eb, L, T), port.compress(y, eb, L, T)
            codec = Z.Codec(n, L, T)
            fa = Z.DeviceStream.from_bytes(codec, sa)
            assert np.array_equal(codec.decompress(fa, eb).cpu().numpy(), port.decompress(sa, n, eb, L, T)), (L, T)
            fa, fb = Z.DeviceStream.from_bytes(codec, sa), Z.DeviceStream.from_bytes(codec, sb)
            assert codec.homadd([fa, fb]).tobytes() == port.homadd(sa, sb, n, eb, L, T), (L, T)
            codec.check()


def test_box_tiles_and_exact_quantization_against_port(port, torch):
    """Full tiles whose element before them starts a 32-float row of a
    16-byte-aligned buffer move as TMA boxes; the others (segments starting
    off a row, a buffer 4 bytes off alignment) do not.  Both must give the
    oracle's bytes and floats, also when products reach 2^24 and the exact
    quantization takes over: everywhere (a large offset) or block by block
    (spikes, one on the last element of a tile and one right after it)."""
    rng = np.random.default_rng(11)
    L = 32
    for T, n in ((1, 5 * 8192 + 77), (4, 4 * 24576 + 3), (3, 2 * 3 * 8192 + 23)):
        base = np.cumsum(rng.normal(0, 0.01, n)).astype(np.float32)
        eb = float(np.float32(1e-4 * (base.max() - base.min())))
        spiky = base.copy()
        spiky[[8192, 8193, 5000, n - 2]] = np.float32(2.0e7 * eb)
        for x in (base, (base + np.float32(2.0e7 * eb)).astype(np.float32), spiky):
            codec = Z.Codec(n, L, T)
            sx = port.compress(x, eb, L, T)
            a = codec.compress(dev(torch, x), eb)
            assert a.tobytes() == sx, (T, n)
            off = torch.zeros(n + 1, dtype=torch.float32, device="cuda")
            off[1:] = dev(torch, x)
            assert codec.compress(off[1:], eb).tobytes() == sx, (T, n)
            ref = port.decompress(sx, n, eb, L, T)
            assert np.array_equal(codec.decompress(a, eb).cpu().numpy(), ref)
            y = torch.zeros(n + 1, dtype=torch.float32, device="cuda")
            codec.decompress(a, eb, out=y[1:])
            assert np.array_equal(y[1:].cpu().numpy(), ref)
            codec.check()


def test_every_block_width_against_port(port, torch):
    """Blocks of every width 0..31 side by side (block k's values spread
    over 2^(k mod 32) quantization steps), through compress, decompress
    and the homomorphic add, in full tiles and in a ragged tail."""
    rng = np.random.default_rng(5)
    L, eb = 32, 1.0e-3
    for T, n in ((1, 3 * 8192 + 1000), (3, 3 * 8192 + 7)):
        k = np.arange(n) // L
        amp = np.ldexp(1.0, (k % 32).astype(np.int64) - 1)
        x = (eb * np.round(rng.uniform(-1, 1, n) * amp)).astype(np.float32)
        x[(k % 32) == 0] = np.float32(eb * 7)  # constant blocks: width 0
        y = (eb * np.round(rng.uniform(-1, 1, n) * amp[::-1])).astype(np.float32)
        codec = Z.Codec(n, L, T)
        sx, sy = port.compress(x, eb, L, T), port.compress(y, eb, L, T)
        a, b = codec.compress(dev(torch, x), eb), codec.compress(dev(torch, y), eb)
        assert a.tobytes() == sx and b.tobytes() == sy, (T, n)
        assert np.array_equal(codec.decompress(a, eb).cpu().numpy(), port.decompress(sx, n, eb, L, T))
        h = codec.homadd([a, b])
        sh = port.homadd(sx, sy, n, eb, L, T)
        assert h.tobytes() == sh
        assert np.array_equal(codec.decompress(h, eb).cpu().numpy(), port.decompress(sh, n, eb, L, T))
        codec.check()


def sinusoid_config1(n, seed):
    """16M-element test signal: sin(2 pi i/4096) + 0.3 sin(2 pi i/97) + N(0, 0.01)."""
    i = np.arange(n, dtype=np.float64)
    rng = np.random.default_rng(seed)
    return (np.sin(2 * np.pi * i / 4096) + 0.3 * np.sin(2 * np.pi * i / 97)
            + rng.normal(0, 0.01, n)).astype(np.float32)


def test_full_size_sinusoid_against_port(port, torch):
    n, L, T = 16_777_216, 32, 16
    x, y = sinusoid_config1(n, 0), sinusoid_config1(n, 1)
    eb = float(np.float32(1e-4 * max(x.max() - x.min(), y.max() - y.min())))
    codec = Z.Codec(n, L, T)
    a, b = codec.compress(dev(torch, x), eb), codec.compress(dev(torch, y), eb)
    h = codec.homadd([a, b])
    da, dh = codec.decompress(a, eb).cpu().numpy(), codec.decompress(h, eb).cpu().numpy()
    codec.check()
    sa, sb = port.compress(x, eb, L, T), port.compress(y, eb, L, T)
    assert a.tobytes() == sa and b.tobytes() == sb
    assert h.tobytes() == port.homadd(sa, sb, n, eb, L, T)
    assert np.array_equal(da, port.decompress(sa, n, eb, L, T))
    slack = 4.0 * np.spacing(np.float32(2.0))
    assert np.max(np.abs(da.astype(np.float64) - x)) <= eb + slack
    assert np.max(np.abs(dh.astype(np.float64) - (x.astype(np.float64) + y))) <= 2 * eb + 2 * slack


def test_errors_are_reported_not_faulted(torch):
    n, L, T = 10000, 32, 2
    codec = Z.Codec(n, L, T)
    x = np.linspace(-1, 1, n).astype(np.float32)
    x[1234] = np.nan
    codec.compress(dev(torch, x), 1e-3)
    with pytest.raises(Z.ZcclError) as e:
        codec.check()
    assert e.value.status == -3
    good = codec.compress(dev(torch, np.linspace(-1, 1, n).astype(np.float32)), 1e-3)
    codec.check()
    raw = good.tobytes()
    # truncated: the walk runs past the readable bytes
    short = Z.DeviceStream.from_bytes(codec, raw[: len(raw) // 2])
    codec.decompress(short, 1e-3)
    with pytest.raises(Z.ZcclError) as e:
        codec.check()
    assert e.value.status in (-4, -5)
    # a chunk offset that disagrees with the block walk
    bad = bytearray(raw)
    bad[8] ^= 0x01
    codec.decompress(Z.DeviceStream.from_bytes(codec, bytes(bad)), 1e-3)
    with pytest.raises(Z.ZcclError) as e:
        codec.check()
    assert e.value.status in (-4, -5)
    # output capacity too small
    tiny = codec.new_stream(capacity=64)
    codec.compress(dev(torch, np.linspace(-1, 1, n).astype(np.float32)), 1e-3, out=tiny)
    with pytest.raises(Z.ZcclError) as e:
        codec.check()
    assert e.value.status == -8


def test_errors_stay_until_checked(torch):
    """The device status words keep every call's errors until a check reads
    and clears them: an early failed call is still reported after later
    calls on the same workspace succeeded, and the check after that is
    clean again."""
    n, L, T = 20000, 32, 2
    codec = Z.Codec(n, L, T)
    x = dev(torch, np.linspace(-1, 1, n).astype(np.float32))
    codec.compress(x, 1e-3, out=codec.new_stream(capacity=64))  # ECAPACITY
    good = codec.compress(x, 1e-3)
    codec.decompress(good, 1e-3)
    codec.homadd([good, good])
    with pytest.raises(Z.ZcclError) as e:
        codec.check()
    assert e.value.status == -8
    codec.compress(x, 1e-3)
    codec.check()


def test_record_and_split_variants_with_device_pointers(port, torch):
    """The T = 1 _record variants and the split variant on device memory:
    the oracle's stream and floats, the reference's counts (restated by the
    oracle), and the size slot written into a device frame table."""
    rng = np.random.default_rng(31)
    n, L = 200003, 32
    x = np.cumsum(rng.normal(0, 0.02, n)).astype(np.float32)
    x[5000:60000] = np.float32(1.5)
    eb = float(np.float32(1e-4 * float(x.max() - x.min())))
    s1 = port.compress(x, eb, L, 1)
    cc, dc = port.record_counts(s1, n, L)
    xd = dev(torch, x)
    out = torch.zeros(len(s1) + 4096, dtype=torch.uint8, device="cuda")
    size, count = Z.ZCCL_float_single_thread_arg_record(out, xd, eb, n, L)
    assert out[:size].cpu().numpy().tobytes() == s1 and count == cc
    y = torch.zeros(n, dtype=torch.float32, device="cuda")
    assert Z.ZCCL_float_decompress_single_thread_arg_record(y, n, eb, L, out) == dc
    assert np.array_equal(y.cpu().numpy(), port.decompress(s1, n, eb, L, 1))
    frame = torch.zeros(len(s1) + 4096, dtype=torch.uint8, device="cuda")
    size = Z.ZCCL_float_single_thread_arg_split_record(frame[24:], xd, eb, n, L, frame, 2)
    assert size == len(s1)
    assert frame[24: 24 + size].cpu().numpy().tobytes() == s1
    assert int(np.frombuffer(frame[16:24].cpu().numpy().tobytes(), "<u8")[0]) == len(s1)
    Z.set_omp_threads(3)
    assert Z.ZCCL_float_openmp_threadblock(x, eb, n, L) == port.compress(x, eb, L, 3)
    sx = port.compress(x, eb, L, 3)
    host = np.zeros(4 * n + 4096, np.uint8)  # the 4*nbEle bytes a reference caller gives a stream
    host[: len(sx)] = np.frombuffer(sx, np.uint8)
    assert np.array_equal(Z.ZCCL_float_decompress_openmp_threadblock(n, eb, L, host),
                          port.decompress(sx, n, eb, L, 3))


def test_lookback_wait_gives_up_and_reports_timeout(torch, monkeypatch):
    """A bounded device wait that runs out: with the library's test hook the
    compressor hands out tiles from 1 on, so tile 0 never publishes its size
    and tile 1's look-back gives up after 4096 polls.  The call returns at
    once, the check reports ZCCL_GPU_ETIMEOUT (no fault, no hang), and the
    next call on the same workspace is clean and exact again."""
    import time
    n, L, T = 1 << 20, 32, 1
    codec = Z.Codec(n, L, T)
    x = dev(torch, np.sin(np.arange(n, dtype=np.float64) * 1e-3).astype(np.float32))
    ref = codec.compress(x, 1e-4)
    codec.check()
    monkeypatch.setenv("ZCCL_GPU_TEST_STALL_TILE0", "1")
    t0 = time.perf_counter()
    codec.compress(x, 1e-4)
    with pytest.raises(Z.ZcclError) as e:
        codec.check()
    assert time.perf_counter() - t0 < 10.0
    assert e.value.status == -6
    monkeypatch.delenv("ZCCL_GPU_TEST_STALL_TILE0")
    again = codec.compress(x, 1e-4)
    codec.check()
    assert again.tobytes() == ref.tobytes()


@pytest.mark.parametrize("T,extra", [(16, 0), (16, 9), (7, 3), (3, 0)])
def test_host_dropins_pipelined_by_chunk_groups(port, torch, T, extra):
    """Host buffers of 2^22 floats and more go through the pipelined drop-ins
    (groups of chunks copied in on one stream, coded and copied out on four
    more).
    Their streams, floats and sums are the oracle's: remainder segments that
    force the last group to hold several chunks, pageable and pinned
    buffers, and the sum written over its second input as the ring does and
    into a buffer of its own."""
    n = (1 << 22) + extra
    L = 32
    rng = np.random.default_rng(T + extra)
    t = np.arange(n, dtype=np.float64)
    x = (np.sin(t * 1e-3) + rng.normal(0, 0.01, n)).astype(np.float32)
    y = (np.cos(t * 7e-4) + rng.normal(0, 0.01, n)).astype(np.float32)
    eb = float(np.float32(2e-4))
    sx, sy = port.compress(x, eb, L, T), port.compress(y, eb, L, T)
    dx = port.decompress(sx, n, eb, L, T)
    sxy = port.homadd(sx, sy, n, eb, L, T)
    Z.set_omp_threads(T)
    cap = 4 * n + 8 * T + 4096

    def host(count, dtype, pinned):
        if pinned:
            return torch.zeros(count, dtype=dtype, pin_memory=True).numpy()
        return np.zeros(count, {torch.float32: np.float32, torch.uint8: np.uint8}[dtype])

    for pinned in (False, True):
        xh = host(n, torch.float32, pinned)
        xh[:] = x
        hs = host(cap, torch.uint8, pinned)
        size = Z.ZCCL_float_openmp_threadblock_arg(hs, xh, 0, eb, n, L)
        assert hs[:size].tobytes() == sx, (T, extra, pinned)
        out = host(n, torch.float32, pinned)
        Z.ZCCL_float_decompress_openmp_threadblock_arg(out, n, eb, L, hs)
        assert np.array_equal(out.view(np.uint32), dx.view(np.uint32)), (T, extra, pinned)
        acc = host(cap, torch.uint8, pinned)
        acc[: len(sy)] = np.frombuffer(sy, np.uint8)
        ys = acc.copy() if not pinned else host(cap, torch.uint8, True)
        ys[: len(sy)] = np.frombuffer(sy, np.uint8)
        total = Z.ZCCL_float_homomophic_add_openmp_threadblock(acc, 0, n, eb, L, hs, acc)
        assert total == len(sxy) and acc[:total].tobytes() == sxy, (T, extra, pinned)
        # into a separate buffer: the outputs leave group by group while inputs arrive
        sep = host(cap, torch.uint8, pinned)
        total = Z.ZCCL_float_homomophic_add_openmp_threadblock(sep, 0, n, eb, L, hs, ys)
        assert total == len(sxy) and sep[:total].tobytes() == sxy, (T, extra, pinned)


def test_host_dropins_pipelined_report_bad_streams(port, torch):
    """Damaged host streams on the pipelined path end in a status code, not a
    fault or a hang: header bytes above 32 inside a middle chunk group, a
    chunk offset that runs past the stream, and the add of a damaged input.
    A good call right after each is exact again."""
    n, L, T = 1 << 22, 32, 16
    x = np.sin(np.arange(n, dtype=np.float64) * 1e-3).astype(np.float32)
    eb = float(np.float32(2e-4))
    good = port.compress(x, eb, L, T)
    Z.set_omp_threads(T)
    cap = 4 * n + 8 * T + 4096
    hdr = np.frombuffer(good[: 8 * T], "<u8")
    out = np.zeros(n, np.float32)
    ref = port.decompress(good, n, eb, L, T)

    def host(b):
        h = np.zeros(cap, np.uint8)
        h[: len(b)] = np.frombuffer(b, np.uint8)
        return h

    bad = host(good)
    mid = 8 * T + int(hdr[6]) + 64  # inside chunk 6, in the fourth of eight groups
    bad[mid: mid + 32] = 0xEE       # not a width byte
    with pytest.raises(Z.ZcclError):
        Z.ZCCL_float_decompress_openmp_threadblock_arg(out, n, eb, L, bad)
    Z.ZCCL_float_decompress_openmp_threadblock_arg(out, n, eb, L, host(good))
    assert np.array_equal(out.view(np.uint32), ref.view(np.uint32))

    far = host(good)
    far[8 * 5: 8 * 6] = np.frombuffer(np.uint64(3 * cap).tobytes(), np.uint8)  # chunk 5 starts past the end
    with pytest.raises(Z.ZcclError):
        Z.ZCCL_float_decompress_openmp_threadblock_arg(out, n, eb, L, far)

    acc = host(good)
    with pytest.raises(Z.ZcclError):
        Z.ZCCL_float_homomophic_add_openmp_threadblock(acc, 0, n, eb, L, bad, acc)
    acc = host(good)
    total = Z.ZCCL_float_homomophic_add_openmp_threadblock(acc, 0, n, eb, L, host(good), acc)
    assert acc[:total].tobytes() == port.homadd(good, good, n, eb, L, T)
