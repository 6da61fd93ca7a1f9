"""CPU checkers for the fastmode1 codec.  TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg may
import this module.  It wraps two shared libraries:

* ``port`` -- ``oracle/libzccl_port.so``, our C restatement of the reference
  codec (``oracle/zccl_port.c``); builds on any host.
* ``ref``  -- ``oracle/_ref/libzccl_ref.so``, the reference's own codec
  compiled in place from its sources by ``oracle/Makefile``; only where the
  reference checkout exists and the binary matches this host.

Both take the OpenMP thread count T explicitly because T fixes the stream
layout (``ZCCL/src/ZCCL_float.c:532-545``).  For ``ref`` it is set through
``omp_set_num_threads`` right before each call, which is the only way the
reference learns it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "libzccl_port.so")
REF_SO = os.path.join(HERE, "_ref", "libzccl_ref.so")

_u8p = ctypes.POINTER(ctypes.c_ubyte)
_f32p = ctypes.POINTER(ctypes.c_float)
_szp = ctypes.POINTER(ctypes.c_size_t)


def reference_root() -> str | None:
    """The reference checkout the oracle compiles from: $ZCCL_REFERENCE_ROOT,
    else a checkout named ``reference`` beside this repository; None when
    neither holds the codec sources."""
    cands = [os.environ.get("ZCCL_REFERENCE_ROOT"),
             os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")]
    for c in cands:
        if c and os.path.isfile(os.path.join(c, "ZCCL", "src", "ZCCL_float.c")):
            return os.path.abspath(c)
    return None


def build(ref: bool = True) -> None:
    """Compile the port (and the reference library when its sources exist)."""
    root = reference_root() if ref else None
    targets = ["port"] + (["ref", f"REF_ROOT={root}"] if root else [])
    subprocess.run(["make", "-s", "-C", HERE] + targets, check=True)


def _ptr(a, typ):
    return a.ctypes.data_as(typ)


def worst_stream_bytes(n: int, L: int, T: int) -> int:
    """Capacity that always holds a stream (every block at width 32)."""
    tbs, rem = n // T, n % T

    def seg(length):
        if length == 0:
            return 0
        nfull, ntail = (length - 1) // L, (length - 1) % L
        s = 4 + nfull * (1 + (L + 7) // 8 + 4 * L)
        if ntail:
            s += 1 + (ntail + 7) // 8 + 4 * ntail
        return s

    return 8 * T + T * seg(tbs) + seg(rem) + 64


class _Codec:
    def __init__(self, path: str, kind: str):
        self.kind = kind
        self.lib = ctypes.CDLL(path)
        if kind == "port":
            self._c = self.lib.port_compress
            self._c.argtypes = [_u8p, _f32p, _szp, ctypes.c_float, ctypes.c_size_t,
                                ctypes.c_int, ctypes.c_int]
            self._d = self.lib.port_decompress
            self._d.argtypes = [_f32p, ctypes.c_size_t, ctypes.c_float, ctypes.c_int, _u8p,
                                ctypes.c_int]
            self._h = self.lib.port_homadd
            self._h.argtypes = [_u8p, _szp, ctypes.c_size_t, ctypes.c_float, ctypes.c_int,
                                _u8p, _u8p, ctypes.c_int]
            self.width = self.lib.port_width
            self.width.argtypes = [ctypes.c_uint32]
            self.width.restype = ctypes.c_int
        else:
            self._c = self.lib.ZCCL_float_openmp_threadblock_arg
            self._c.argtypes = [_u8p, _f32p, _szp, ctypes.c_float, ctypes.c_size_t, ctypes.c_int]
            self._d = self.lib.ZCCL_float_decompress_openmp_threadblock_arg
            self._d.argtypes = [_f32p, ctypes.c_size_t, ctypes.c_float, ctypes.c_int, _u8p]
            self._h = self.lib.ZCCL_float_homomophic_add_openmp_threadblock
            self._h.argtypes = [_u8p, _szp, ctypes.c_size_t, ctypes.c_float, ctypes.c_int,
                                _u8p, _u8p]
            self._set_threads = self.lib.omp_set_num_threads
            self._set_threads.argtypes = [ctypes.c_int]
        for f in (self._c, self._d, self._h):
            f.restype = None
        # the fixed-rate appendix codec (ZCCL/src/ZCCL_appendix.c:65-590)
        if kind == "port":
            self._cf = self.lib.port_compress_f
            self._cf.argtypes = [_u8p, _f32p, _szp, ctypes.c_float, ctypes.c_size_t, ctypes.c_int,
                                 ctypes.c_int, ctypes.c_int]
            self._df = self.lib.port_decompress_f
            self._df.argtypes = [_f32p, ctypes.c_size_t, ctypes.c_float, ctypes.c_int, _u8p, ctypes.c_int,
                                 ctypes.c_int]
        else:
            self._cf = self.lib.ZCCL_float_openmp_threadblock_arg_2
            self._cf.argtypes = [_u8p, _f32p, _szp, ctypes.c_float, ctypes.c_size_t, ctypes.c_int]
            self._df = self.lib.ZCCL_float_decompress_openmp_threadblock_arg_2
            self._df.argtypes = [_f32p, ctypes.c_size_t, ctypes.c_float, ctypes.c_int, _u8p]
        self._cf.restype = self._df.restype = None
        # the serial SZp 3-D codec (ZCCL/src/ZCCL_float.c:1706-1860, ZCCLd_float.c:2801-2871)
        c3 = [_f32p, _u8p, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_int,
              ctypes.c_double, _szp]
        d3 = [_f32p, _u8p, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_int, ctypes.c_double]
        names = ({"fast": "port_szp3d_compress", "plain": "port_szp3d_compress"}, "port_szp3d_decompress") \
            if kind == "port" else ({"fast": "SZp_compress3D_fast", "plain": "SZp_compress3D"}, "SZp_decompress3D")
        self._c3 = {}
        for k, nm in names[0].items():
            f = getattr(self.lib, nm)
            f.argtypes, f.restype = c3, None
            self._c3[k] = f
        self._d3 = getattr(self.lib, names[1])
        self._d3.argtypes, self._d3.restype = d3, None

    def _args_T(self, T):
        if self.kind == "port":
            return (ctypes.c_int(T),)
        self._set_threads(T)
        return ()

    def compress(self, x: np.ndarray, eb: float, L: int, T: int) -> bytes:
        x = np.ascontiguousarray(x, dtype=np.float32)
        n = x.size
        out = np.zeros(worst_stream_bytes(n, L, T), dtype=np.uint8)
        size = ctypes.c_size_t(0)
        self._c(_ptr(out, _u8p), _ptr(x, _f32p), ctypes.byref(size), ctypes.c_float(eb),
                ctypes.c_size_t(n), ctypes.c_int(L), *self._args_T(T))
        return out[: size.value].tobytes()

    def decompress(self, stream: bytes, n: int, eb: float, L: int, T: int) -> np.ndarray:
        buf = np.frombuffer(stream, dtype=np.uint8).copy()
        # the reference's 3/5/6/7-bit unpackers may read one byte past a field
        buf = np.concatenate([buf, np.zeros(16, np.uint8)])
        y = np.zeros(n, dtype=np.float32)
        self._d(_ptr(y, _f32p), ctypes.c_size_t(n), ctypes.c_float(eb), ctypes.c_int(L),
                _ptr(buf, _u8p), *self._args_T(T))
        return y

    def homadd(self, s1: bytes, s2: bytes, n: int, eb: float, L: int, T: int) -> bytes:
        a = np.concatenate([np.frombuffer(s1, np.uint8), np.zeros(16, np.uint8)])
        b = np.concatenate([np.frombuffer(s2, np.uint8), np.zeros(16, np.uint8)])
        out = np.zeros(worst_stream_bytes(n, L, T), dtype=np.uint8)
        size = ctypes.c_size_t(0)
        self._h(_ptr(out, _u8p), ctypes.byref(size), ctypes.c_size_t(n), ctypes.c_float(eb),
                ctypes.c_int(L), _ptr(a, _u8p), _ptr(b, _u8p), *self._args_T(T))
        return out[: size.value].tobytes()

    def _fmt(self):
        return (ctypes.c_int(1),) if self.kind == "port" else ()

    def compress_fixed(self, x: np.ndarray, eb: float, L: int, T: int) -> bytes:
        """The fixed-rate appendix codec (ZCCL_float_openmp_threadblock_arg_2)."""
        x = np.ascontiguousarray(x, dtype=np.float32)
        n = x.size
        out = np.zeros(worst_stream_bytes(n, L, T), dtype=np.uint8)
        size = ctypes.c_size_t(0)
        self._cf(_ptr(out, _u8p), _ptr(x, _f32p), ctypes.byref(size), ctypes.c_float(eb),
                 ctypes.c_size_t(n), ctypes.c_int(L), *self._args_T(T), *self._fmt())
        return out[: size.value].tobytes()

    def decompress_fixed(self, stream: bytes, n: int, eb: float, L: int, T: int) -> np.ndarray:
        buf = np.concatenate([np.frombuffer(stream, dtype=np.uint8), np.zeros(16, np.uint8)])
        y = np.zeros(n, dtype=np.float32)
        self._df(_ptr(y, _f32p), ctypes.c_size_t(n), ctypes.c_float(eb), ctypes.c_int(L), _ptr(buf, _u8p),
                 *self._args_T(T), *self._fmt())
        return y

    def szp3d_compress(self, x: np.ndarray, dims, bs: int, eb: float, form: str = "fast") -> bytes:
        x = np.ascontiguousarray(x, dtype=np.float32).ravel()
        n = int(np.prod(dims))
        nb = 1
        for d in dims:
            nb *= (d - 1) // bs + 1
        out = np.zeros(nb + nb * (bs ** 3) * 5 + 64, dtype=np.uint8)  # rates + worst payloads
        size = ctypes.c_size_t(0)
        assert x.size == n
        self._c3[form](_ptr(x, _f32p), _ptr(out, _u8p), *[ctypes.c_size_t(d) for d in dims],
                       ctypes.c_int(bs), ctypes.c_double(eb), ctypes.byref(size))
        return out[: size.value].tobytes()

    def szp3d_decompress(self, stream: bytes, dims, bs: int, eb: float) -> np.ndarray:
        buf = np.concatenate([np.frombuffer(stream, dtype=np.uint8), np.zeros(64, np.uint8)])
        y = np.zeros(int(np.prod(dims)), dtype=np.float32)
        self._d3(_ptr(y, _f32p), _ptr(buf, _u8p), *[ctypes.c_size_t(d) for d in dims], ctypes.c_int(bs),
                 ctypes.c_double(eb))
        return y

    # ---- the _record variants' counts ------------------------------------
    def record_counts(self, stream: bytes, n: int, L: int):
        """(compress count, decompress count) the reference's T = 1 _record
        variants return for this stream (port only)."""
        c, d = ctypes.c_size_t(0), ctypes.c_size_t(0)
        f = self.lib.port_record_counts
        f.argtypes = [_u8p, ctypes.c_size_t, ctypes.c_int, _szp, _szp]
        f.restype = None
        buf = np.frombuffer(stream, np.uint8).copy()
        f(_ptr(buf, _u8p), n, L, ctypes.byref(c), ctypes.byref(d))
        return c.value, d.value

    def homadd_cases(self, s1: bytes, s2: bytes, n: int, L: int, T: int):
        """The four branch counters of the two-input add (port only)."""
        out = (ctypes.c_ulonglong * 4)()
        f = self.lib.port_homadd_cases
        f.argtypes = [_u8p, _u8p, ctypes.c_size_t, ctypes.c_int, ctypes.c_int, ctypes.c_ulonglong * 4]
        f.restype = None
        a, b = np.frombuffer(s1, np.uint8).copy(), np.frombuffer(s2, np.uint8).copy()
        f(_ptr(a, _u8p), _ptr(b, _u8p), n, L, T, out)
        return list(out)

    def ref_record(self, x: np.ndarray, eb: float, L: int):
        """The reference library's ZCCL_float_single_thread_arg_record and
        ZCCL_float_decompress_single_thread_arg_record on x: (stream,
        compress count, decompressed floats, decompress count)."""
        x = np.ascontiguousarray(x, dtype=np.float32)
        n = x.size
        out = np.zeros(worst_stream_bytes(n, L, 1), dtype=np.uint8)
        size = ctypes.c_size_t(0)
        fc = self.lib.ZCCL_float_single_thread_arg_record
        fc.argtypes = [_u8p, _f32p, _szp, ctypes.c_float, ctypes.c_size_t, ctypes.c_int]
        fc.restype = ctypes.c_size_t
        cc = fc(_ptr(out, _u8p), _ptr(x, _f32p), ctypes.byref(size), ctypes.c_float(eb), n, L)
        stream = out[: size.value].tobytes()
        buf = np.concatenate([out[: size.value], np.zeros(16, np.uint8)])
        y = np.zeros(n, np.float32)
        fd = self.lib.ZCCL_float_decompress_single_thread_arg_record
        fd.argtypes = [_f32p, ctypes.c_size_t, ctypes.c_float, ctypes.c_int, _u8p]
        fd.restype = ctypes.c_size_t
        dc = fd(_ptr(y, _f32p), n, ctypes.c_float(eb), L, _ptr(buf, _u8p))
        return stream, cc, y, dc

    def ref_homadd_record(self, s1: bytes, s2: bytes, n: int, eb: float, L: int, T: int):
        """The reference's ZCCL_float_homomophic_add_openmp_threadblock_record
        with T threads: (sum stream, [counter_1 .. counter_4])."""
        a = np.concatenate([np.frombuffer(s1, np.uint8), np.zeros(16, np.uint8)])
        b = np.concatenate([np.frombuffer(s2, np.uint8), np.zeros(16, np.uint8)])
        out = np.zeros(worst_stream_bytes(n, L, T), dtype=np.uint8)
        size = ctypes.c_size_t(0)
        cnt = [ctypes.c_int(0) for _ in range(4)]
        f = self.lib.ZCCL_float_homomophic_add_openmp_threadblock_record
        f.argtypes = [_u8p, _szp, ctypes.c_size_t, ctypes.c_float, ctypes.c_int, _u8p, _u8p] + \
            [ctypes.POINTER(ctypes.c_int)] * 4
        f.restype = None
        self._set_threads(T)
        f(_ptr(out, _u8p), ctypes.byref(size), n, ctypes.c_float(eb), L, _ptr(a, _u8p), _ptr(b, _u8p),
          *[ctypes.byref(c) for c in cnt])
        return out[: size.value].tobytes(), [c.value for c in cnt]

    # ---- the OpenMP form of the SZp 3-D codec -------------------------------
    def szp3d_compress_split(self, x: np.ndarray, dims, bs: int, eb: float, T: int) -> bytes:
        """SZp_compress3D_fast_openmp with T threads (the reference through
        omp_set_num_threads; the port with T explicit)."""
        x = np.ascontiguousarray(x, dtype=np.float32).ravel()
        nb = 1
        for d in dims:
            nb *= (d - 1) // bs + 1
        out = np.zeros(8 * T + T * 64 + nb + nb * (bs ** 3) * 5 + 64, dtype=np.uint8)
        size = ctypes.c_size_t(0)
        args = [_ptr(x, _f32p), _ptr(out, _u8p), *[ctypes.c_size_t(d) for d in dims], ctypes.c_int(bs),
                ctypes.c_double(eb)]
        if self.kind == "port":
            f = self.lib.port_szp3d_compress_split
            f.argtypes = [_f32p, _u8p, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_int,
                          ctypes.c_double, ctypes.c_int, _szp]
            f.restype = None
            f(*args, ctypes.c_int(T), ctypes.byref(size))
        else:
            f = self.lib.SZp_compress3D_fast_openmp
            f.argtypes = [_f32p, _u8p, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_int,
                          ctypes.c_double, _szp]
            f.restype = None
            self._set_threads(T)
            f(*args, ctypes.byref(size))
        return out[: size.value].tobytes()

    def szp3d_decompress_split(self, stream: bytes, dims, bs: int, eb: float, T: int) -> np.ndarray:
        buf = np.concatenate([np.frombuffer(stream, dtype=np.uint8), np.zeros(64, np.uint8)])
        y = np.zeros(int(np.prod(dims)), dtype=np.float32)
        args = [_ptr(y, _f32p), _ptr(buf, _u8p), *[ctypes.c_size_t(d) for d in dims], ctypes.c_int(bs),
                ctypes.c_double(eb)]
        if self.kind == "port":
            f = self.lib.port_szp3d_decompress_split
            f.argtypes = [_f32p, _u8p, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_int,
                          ctypes.c_double, ctypes.c_int]
            f.restype = None
            f(*args, ctypes.c_int(T))
        else:
            f = self.lib.SZp_decompress3D_fast_openmp
            f.argtypes = [_f32p, _u8p, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_int,
                          ctypes.c_double]
            f.restype = None
            self._set_threads(T)
            f(*args)
        return y

    def dims3(self, n: int):
        """My_Dims_create(n, 3, {0, 0, 0}): the reference's own, or the port's."""
        d = (ctypes.c_int * 3)(0, 0, 0)
        if self.kind == "port":
            self.lib.port_dims3(ctypes.c_int(n), d)
        else:
            self.lib.My_Dims_create(ctypes.c_int(n), ctypes.c_int(3), d)
        return list(d)

    def homadd_fold(self, streams, n: int, eb: float, L: int, T: int) -> bytes:
        """P-way sum folded pairwise the way the ring's reduce-scatter does it
        (acc = add(received, acc), ZCCL/src/ZCCL_ring_ho.c:281-287)."""
        acc = streams[0]
        for s in streams[1:]:
            acc = self.homadd(s, acc, n, eb, L, T)
        return acc


_cache: dict = {}


def port() -> _Codec:
    if "port" not in _cache:
        if not os.path.exists(PORT_SO):
            build(ref=False)
        _cache["port"] = _Codec(PORT_SO, "port")
    return _cache["port"]


def ref_available() -> bool:
    if not os.path.exists(REF_SO):
        return False
    try:
        ref()
        return True
    except OSError:
        return False


def ref() -> _Codec:
    if "ref" not in _cache:
        _cache["ref"] = _Codec(REF_SO, "ref")
    return _cache["ref"]


def chunk_sizes(stream: bytes, T: int) -> list:
    """Byte length of each of the T chunks of a stream, from its header."""
    hdr = np.frombuffer(stream[: 8 * T], dtype="<u8").astype(np.int64)
    ends = list(hdr[1:]) + [len(stream) - 8 * T]
    return [int(e - b) for b, e in zip(hdr, ends)]


def ref_scratch_ok(stream: bytes, n: int, T: int) -> bool:
    """True when every chunk of ``stream`` fits the reference's per-thread
    scratch of ceil(4n/T) bytes (ZCCL/src/ZCCL_float.c:539,548-549 and
    ZCCL/src/ZCCLd_float.c:1031,1040-1041).  Larger chunks overflow that heap
    buffer inside the reference, so the reference only runs on cases where
    this holds."""
    cap = (4 * n + T - 1) // T
    return max(chunk_sizes(stream, T)) <= cap


def width_thresholds(width_fn=None) -> list:
    """thr[w] = smallest m with bit length w whose width is w+1 (0 if none),
    found by scanning down from 2**w - 1 (the width is monotone in m)."""
    f = width_fn or port().width
    thr = [0] * 33
    for w in range(1, 33):
        lo, m = 1 << (w - 1), (1 << w) - 1
        first = 0
        while m >= lo and f(m) == w + 1:
            first = m
            m -= 1
        thr[w] = first
    return thr
