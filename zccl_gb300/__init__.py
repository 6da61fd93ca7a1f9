"""GB300 implementation of ZCCL's fastmode1 compression hot path.

Python bindings of the C ABI in ``include/zccl_gpu.h`` (the shared library
``zccl_gb300/libzccl_gpu.so``).  Two layers, mirroring the C header:

* the reference's entry points under their own names
  (``ZCCL_float_openmp_threadblock_arg`` ...), taking numpy arrays (host
  memory) or torch CUDA tensors (device memory);
* ``Codec``: the device API with explicit writer thread count T, resident
  compressed streams (``DeviceStream``) that carry their side index, and a
  CUDA stream.

The library is required: nothing here falls back to a CPU implementation.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libzccl_gpu.so")

STATUS = {
    0: "ok", -1: "invalid argument", -2: "CUDA runtime error",
    -3: "input not finite or |x/eb| >= 2^31", -4: "stream inconsistent with its geometry",
    -5: "stream runs past its readable bytes", -6: "device wait timed out",
    -7: "out of memory", -8: "destination buffer too small",
    -9: "input needs more than the fixed scratch array",
}

EXPORTS = [
    "ZCCL_float_openmp_threadblock_arg", "ZCCL_float_single_thread_arg",
    "ZCCL_float_decompress_openmp_threadblock_arg", "ZCCL_float_decompress_single_thread_arg",
    "ZCCL_float_homomophic_add_openmp_threadblock", "ZCCL_float_homomophic_add_single_thread",
    "ZCCL_float_openmp_threadblock", "ZCCL_float_decompress_openmp_threadblock",
    "ZCCL_float_single_thread_arg_record", "ZCCL_float_decompress_single_thread_arg_record",
    "ZCCL_float_single_thread_arg_split_record", "ZCCL_float_homomophic_add_openmp_threadblock_record",
    "zccl_gpu_max_stream_bytes", "zccl_gpu_index_bytes", "zccl_gpu_workspace_bytes",
    "zccl_gpu_compress", "zccl_gpu_decompress", "zccl_gpu_homadd", "zccl_gpu_homadd_cases",
    "zccl_gpu_decompress_accumulate",
    "zccl_gpu_build_index", "zccl_gpu_stream_size", "zccl_gpu_frame_size", "zccl_gpu_check", "zccl_gpu_last_status",
    "zccl_gpu_strerror", "zccl_gpu_width_table", "zccl_gpu_compress_noalloc",
    "zccl_gpu_batch_bytes", "zccl_gpu_batch_plan", "zccl_gpu_batch_run", "zccl_gpu_batch_tune",
    "zccl_gpu_batch_check",
    "SZp_compress3D_fast", "SZp_compress3D", "SZp_decompress3D", "SZp_decompress3D_fast",
    "ZCCL_float_openmp_threadblock_arg_2", "ZCCL_float_decompress_openmp_threadblock_arg_2",
    "zccl_gpu_compress_fixed", "zccl_gpu_decompress_fixed",
    "zccl_gpu_szp3d_max_bytes", "zccl_gpu_szp3d_workspace_bytes", "zccl_gpu_szp3d_compress",
    "zccl_gpu_szp3d_decompress",
    "SZp_compress3D_fast_openmp", "SZp_decompress3D_fast_openmp", "zccl_gpu_szp3d_split_max_bytes",
    "zccl_gpu_szp3d_split_workspace_bytes", "zccl_gpu_szp3d_compress_split", "zccl_gpu_szp3d_decompress_split",
]


class ZcclError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        super().__init__(f"{what}: {STATUS.get(status, status)} ({status})")


class StreamDesc(ctypes.Structure):
    """``zccl_gpu_stream`` of include/zccl_gpu.h."""
    _fields_ = [("bytes", ctypes.c_void_p), ("capacity", ctypes.c_size_t),
                ("index", ctypes.c_void_p), ("indexed", ctypes.c_int),
                ("qprev_valid", ctypes.c_int)]


class BatchJobDesc(ctypes.Structure):
    """``zccl_gpu_batch_job`` of include/zccl_gpu.h."""
    _fields_ = [("d_in", ctypes.c_void_p), ("ins", ctypes.POINTER(StreamDesc)), ("P", ctypes.c_int),
                ("n", ctypes.c_size_t), ("eb", ctypes.c_float), ("T", ctypes.c_int),
                ("out", ctypes.POINTER(StreamDesc)), ("d_out", ctypes.c_void_p), ("accumulate", ctypes.c_int)]


class BatchDesc(ctypes.Structure):
    """``zccl_gpu_batch`` of include/zccl_gpu.h."""
    _fields_ = [("kind", ctypes.c_int), ("L", ctypes.c_int), ("grid", ctypes.c_uint),
                ("njobs", ctypes.c_size_t), ("ntiles", ctypes.c_size_t), ("d_mem", ctypes.c_void_p),
                ("clear_bytes", ctypes.c_size_t), ("jobs_off", ctypes.c_size_t),
                ("map_off", ctypes.c_size_t), ("tile0_off", ctypes.c_size_t), ("tb", ctypes.c_uint),
                ("smem", ctypes.c_uint * 6), ("qprev_valid", ctypes.c_int), ("rows_off", ctypes.c_size_t)]


_lib = None


def lib() -> ctypes.CDLL:
    """Load libzccl_gpu.so (build it first with ``python -m zccl_gb300.build``)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing; build it with `python -m zccl_gb300.build`")
    L = ctypes.CDLL(LIB_PATH)
    vp, sz, i, f = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_float
    sp = ctypes.POINTER(StreamDesc)
    sig = {
        "ZCCL_float_openmp_threadblock_arg": (None, [vp, vp, vp, f, sz, i]),
        "ZCCL_float_single_thread_arg": (None, [vp, vp, vp, f, sz, i]),
        "ZCCL_float_decompress_openmp_threadblock_arg": (None, [vp, sz, f, i, vp]),
        "ZCCL_float_decompress_single_thread_arg": (None, [vp, sz, f, i, vp]),
        "ZCCL_float_homomophic_add_openmp_threadblock": (None, [vp, vp, sz, f, i, vp, vp]),
        "ZCCL_float_homomophic_add_single_thread": (None, [vp, vp, sz, f, i, vp, vp]),
        "ZCCL_float_openmp_threadblock": (vp, [vp, vp, f, sz, i]),
        "ZCCL_float_decompress_openmp_threadblock": (None, [vp, sz, f, i, vp]),
        "ZCCL_float_single_thread_arg_record": (sz, [vp, vp, vp, f, sz, i]),
        "ZCCL_float_decompress_single_thread_arg_record": (sz, [vp, sz, f, i, vp]),
        "ZCCL_float_single_thread_arg_split_record": (None, [vp, vp, vp, f, sz, i, vp, sz]),
        "ZCCL_float_homomophic_add_openmp_threadblock_record": (None, [vp, vp, sz, f, i, vp, vp, vp, vp, vp, vp]),
        "zccl_gpu_max_stream_bytes": (sz, [sz, i, i]),
        "zccl_gpu_index_bytes": (sz, [sz, i, i]),
        "zccl_gpu_workspace_bytes": (sz, [sz, i, i]),
        "zccl_gpu_compress": (i, [sp, vp, sz, f, i, i, vp, vp]),
        "zccl_gpu_decompress": (i, [vp, sp, sz, f, i, i, vp, vp]),
        "zccl_gpu_compress_fixed": (i, [sp, vp, sz, f, i, i, vp, vp]),
        "zccl_gpu_decompress_fixed": (i, [vp, sp, sz, f, i, i, vp, vp]),
        "ZCCL_float_openmp_threadblock_arg_2": (None, [vp, vp, vp, f, sz, i]),
        "ZCCL_float_decompress_openmp_threadblock_arg_2": (None, [vp, sz, f, i, vp]),
        "zccl_gpu_homadd": (i, [sp, sp, i, sz, i, i, vp, vp]),
        "zccl_gpu_decompress_accumulate": (i, [vp, sp, sz, f, i, i, vp, vp]),
        "zccl_gpu_homadd_cases": (i, [sp, sp, i, sz, i, i, vp, vp, vp]),
        "zccl_gpu_build_index": (i, [sp, sz, i, i, vp, vp]),
        "zccl_gpu_stream_size": (i, [sp, sz, i, i, ctypes.POINTER(sz), vp]),
        "zccl_gpu_frame_size": (i, [sp, vp, vp]),
        "SZp_compress3D_fast": (None, [vp, vp, sz, sz, sz, i, ctypes.c_double, ctypes.POINTER(sz)]),
        "SZp_compress3D": (None, [vp, vp, sz, sz, sz, i, ctypes.c_double, ctypes.POINTER(sz)]),
        "SZp_decompress3D": (None, [vp, vp, sz, sz, sz, i, ctypes.c_double]),
        "SZp_decompress3D_fast": (None, [vp, vp, sz, sz, sz, i, ctypes.c_double]),
        "zccl_gpu_szp3d_max_bytes": (sz, [sz, sz, sz, i]),
        "zccl_gpu_szp3d_workspace_bytes": (sz, [sz, sz, sz, i]),
        "zccl_gpu_szp3d_compress": (i, [vp, sz, vp, sz, sz, sz, i, ctypes.c_double, vp, vp, vp]),
        "zccl_gpu_szp3d_decompress": (i, [vp, vp, sz, sz, sz, sz, i, ctypes.c_double, vp, vp]),
        "SZp_compress3D_fast_openmp": (None, [vp, vp, sz, sz, sz, i, ctypes.c_double, ctypes.POINTER(sz)]),
        "SZp_decompress3D_fast_openmp": (None, [vp, vp, sz, sz, sz, i, ctypes.c_double]),
        "zccl_gpu_szp3d_split_max_bytes": (sz, [sz, sz, sz, i, i]),
        "zccl_gpu_szp3d_split_workspace_bytes": (sz, [sz, sz, sz, i, i]),
        "zccl_gpu_szp3d_compress_split": (i, [vp, sz, vp, sz, sz, sz, i, ctypes.c_double, i, vp, vp, vp]),
        "zccl_gpu_szp3d_decompress_split": (i, [vp, vp, sz, sz, sz, sz, i, ctypes.c_double, i, vp, vp]),
        "zccl_gpu_check": (i, [vp, vp]),
        "zccl_gpu_last_status": (i, []),
        "zccl_gpu_strerror": (ctypes.c_char_p, [i]),
        "zccl_gpu_width_table": (None, [ctypes.POINTER(ctypes.c_uint32)]),
        "zccl_gpu_compress_noalloc": (i, [sp, vp, sz, f, i, i, vp, ctypes.POINTER(vp)]),
        "zccl_gpu_batch_bytes": (sz, [i, ctypes.POINTER(BatchJobDesc), sz, i]),
        "zccl_gpu_batch_plan": (i, [ctypes.POINTER(BatchDesc), i, ctypes.POINTER(BatchJobDesc), sz, i, vp,
                                    sz, vp]),
        "zccl_gpu_batch_run": (i, [ctypes.POINTER(BatchDesc), vp]),
        "zccl_gpu_batch_tune": (i, [ctypes.POINTER(BatchDesc), vp]),
        "zccl_gpu_batch_check": (i, [ctypes.POINTER(BatchDesc), vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def set_omp_threads(T: int) -> None:
    """Set the OpenMP thread count the drop-in entry points read as T."""
    fn = lib().omp_set_num_threads
    fn.argtypes = [ctypes.c_int]
    fn(T)


def width_table() -> list:
    arr = (ctypes.c_uint32 * 33)()
    lib().zccl_gpu_width_table(arr)
    return list(arr)


def _check(rc: int, what: str) -> None:
    if rc != 0:
        raise ZcclError(rc, what)


def _ptr(a) -> int:
    """Data pointer of a numpy array or a torch tensor."""
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return a.data_ptr()


# ---------------------------------------------------------------------------
# Reference entry points (host numpy arrays or device torch tensors)
# ---------------------------------------------------------------------------

def _size_slot(outSize):
    return outSize if isinstance(outSize, ctypes.c_size_t) else ctypes.c_size_t(int(outSize or 0))


def ZCCL_float_openmp_threadblock_arg(outputBytes, oriData, outSize, absErrBound, nbEle, blockSize):
    """ZCCL/src/ZCCL_float.c:501; returns the assigned size."""
    s = _size_slot(outSize)
    lib().ZCCL_float_openmp_threadblock_arg(_ptr(outputBytes), _ptr(oriData), ctypes.byref(s),
                                            absErrBound, nbEle, blockSize)
    _check(lib().zccl_gpu_last_status(), "ZCCL_float_openmp_threadblock_arg")
    return s.value


def ZCCL_float_single_thread_arg(outputBytes, oriData, outSize, absErrBound, nbEle, blockSize):
    """ZCCL/src/ZCCL_float.c:809; returns the assigned size."""
    s = _size_slot(outSize)
    lib().ZCCL_float_single_thread_arg(_ptr(outputBytes), _ptr(oriData), ctypes.byref(s),
                                       absErrBound, nbEle, blockSize)
    _check(lib().zccl_gpu_last_status(), "ZCCL_float_single_thread_arg")
    return s.value


def ZCCL_float_decompress_openmp_threadblock_arg(newData, nbEle, absErrBound, blockSize, cmpBytes):
    """ZCCL/src/ZCCLd_float.c:538."""
    lib().ZCCL_float_decompress_openmp_threadblock_arg(_ptr(newData), nbEle, absErrBound,
                                                       blockSize, _ptr(cmpBytes))
    _check(lib().zccl_gpu_last_status(), "ZCCL_float_decompress_openmp_threadblock_arg")


def ZCCL_float_decompress_single_thread_arg(newData, nbEle, absErrBound, blockSize, cmpBytes):
    """ZCCL/src/ZCCLd_float.c:247."""
    lib().ZCCL_float_decompress_single_thread_arg(_ptr(newData), nbEle, absErrBound, blockSize,
                                                  _ptr(cmpBytes))
    _check(lib().zccl_gpu_last_status(), "ZCCL_float_decompress_single_thread_arg")


def ZCCL_float_openmp_threadblock_arg_2(outputBytes, oriData, outSize, absErrBound, nbEle, blockSize):
    """The fixed-rate appendix codec, ZCCL/src/ZCCL_appendix.c:65; returns the assigned size."""
    s = _size_slot(outSize)
    lib().ZCCL_float_openmp_threadblock_arg_2(_ptr(outputBytes), _ptr(oriData), ctypes.byref(s),
                                              absErrBound, nbEle, blockSize)
    _check(lib().zccl_gpu_last_status(), "ZCCL_float_openmp_threadblock_arg_2")
    return s.value


def ZCCL_float_decompress_openmp_threadblock_arg_2(newData, nbEle, absErrBound, blockSize, cmpBytes):
    """ZCCL/src/ZCCL_appendix.c:373."""
    lib().ZCCL_float_decompress_openmp_threadblock_arg_2(_ptr(newData), nbEle, absErrBound, blockSize,
                                                         _ptr(cmpBytes))
    _check(lib().zccl_gpu_last_status(), "ZCCL_float_decompress_openmp_threadblock_arg_2")


def ZCCL_float_homomophic_add_openmp_threadblock(final_cmpBytes, final_cmpSize, nbEle, absErrBound,
                                                 blockSize, cmpBytes, cmpBytes2):
    """ZCCL/src/ZCCLd_float.c:988; returns the accumulated size (the
    reference adds the result size to *final_cmpSize)."""
    s = _size_slot(final_cmpSize)
    lib().ZCCL_float_homomophic_add_openmp_threadblock(_ptr(final_cmpBytes), ctypes.byref(s),
                                                       nbEle, absErrBound, blockSize,
                                                       _ptr(cmpBytes), _ptr(cmpBytes2))
    _check(lib().zccl_gpu_last_status(), "ZCCL_float_homomophic_add_openmp_threadblock")
    return s.value


def ZCCL_float_homomophic_add_single_thread(final_cmpBytes, final_cmpSize, nbEle, absErrBound,
                                            blockSize, cmpBytes, cmpBytes2):
    """ZCCL/src/ZCCLd_float.c:1681; returns the accumulated size."""
    s = _size_slot(final_cmpSize)
    lib().ZCCL_float_homomophic_add_single_thread(_ptr(final_cmpBytes), ctypes.byref(s), nbEle,
                                                  absErrBound, blockSize, _ptr(cmpBytes),
                                                  _ptr(cmpBytes2))
    _check(lib().zccl_gpu_last_status(), "ZCCL_float_homomophic_add_single_thread")
    return s.value


def _libc():
    return ctypes.CDLL(None)


def ZCCL_float_openmp_threadblock(oriData, absErrBound, nbEle, blockSize) -> bytes:
    """ZCCL/src/ZCCL_float.c:192: compresses into a buffer the library
    mallocs; returns the stream's bytes (the buffer is freed here)."""
    s = ctypes.c_size_t(0)
    p = lib().ZCCL_float_openmp_threadblock(_ptr(oriData), ctypes.byref(s), absErrBound, nbEle, blockSize)
    _check(lib().zccl_gpu_last_status(), "ZCCL_float_openmp_threadblock")
    try:
        return ctypes.string_at(p, s.value)
    finally:
        _libc().free(ctypes.c_void_p(p))


def ZCCL_float_decompress_openmp_threadblock(nbEle, absErrBound, blockSize, cmpBytes) -> np.ndarray:
    """ZCCL/src/ZCCLd_float.c:22: decompresses into a buffer the library
    mallocs; returns a copy of the floats (the buffer is freed here)."""
    out = ctypes.c_void_p(0)
    lib().ZCCL_float_decompress_openmp_threadblock(ctypes.byref(out), nbEle, absErrBound, blockSize,
                                                   _ptr(cmpBytes))
    try:
        _check(lib().zccl_gpu_last_status(), "ZCCL_float_decompress_openmp_threadblock")
        return np.ctypeslib.as_array(ctypes.cast(out, ctypes.POINTER(ctypes.c_float)), (nbEle,)).copy()
    finally:
        _libc().free(out)


def ZCCL_float_single_thread_arg_record(outputBytes, oriData, absErrBound, nbEle, blockSize):
    """ZCCL/src/ZCCL_float.c:990; returns (size, the reference's memory-access count)."""
    s = ctypes.c_size_t(0)
    cnt = lib().ZCCL_float_single_thread_arg_record(_ptr(outputBytes), _ptr(oriData), ctypes.byref(s),
                                                    absErrBound, nbEle, blockSize)
    _check(lib().zccl_gpu_last_status(), "ZCCL_float_single_thread_arg_record")
    return s.value, cnt


def ZCCL_float_decompress_single_thread_arg_record(newData, nbEle, absErrBound, blockSize, cmpBytes) -> int:
    """ZCCL/src/ZCCLd_float.c:376; returns the reference's memory-access count."""
    cnt = lib().ZCCL_float_decompress_single_thread_arg_record(_ptr(newData), nbEle, absErrBound, blockSize,
                                                               _ptr(cmpBytes))
    _check(lib().zccl_gpu_last_status(), "ZCCL_float_decompress_single_thread_arg_record")
    return cnt


def ZCCL_float_single_thread_arg_split_record(outputBytes, oriData, absErrBound, nbEle, blockSize, chunk_arr,
                                              chunk_iter):
    """ZCCL/src/ZCCL_float.c:1530; returns the assigned size (also stored
    as size_t number chunk_iter of chunk_arr)."""
    s = ctypes.c_size_t(0)
    lib().ZCCL_float_single_thread_arg_split_record(_ptr(outputBytes), _ptr(oriData), ctypes.byref(s),
                                                    absErrBound, nbEle, blockSize, _ptr(chunk_arr), chunk_iter)
    _check(lib().zccl_gpu_last_status(), "ZCCL_float_single_thread_arg_split_record")
    return s.value


def ZCCL_float_homomophic_add_openmp_threadblock_record(final_cmpBytes, final_cmpSize, nbEle, absErrBound,
                                                        blockSize, cmpBytes, cmpBytes2, counters=None):
    """ZCCL/src/ZCCLd_float.c:2067; returns (accumulated size, the four
    counters after the call's increments, starting from `counters`)."""
    s = _size_slot(final_cmpSize)
    c = [ctypes.c_int(v) for v in (counters or [0, 0, 0, 0])]
    lib().ZCCL_float_homomophic_add_openmp_threadblock_record(
        _ptr(final_cmpBytes), ctypes.byref(s), nbEle, absErrBound, blockSize, _ptr(cmpBytes), _ptr(cmpBytes2),
        *[ctypes.byref(v) for v in c])
    _check(lib().zccl_gpu_last_status(), "ZCCL_float_homomophic_add_openmp_threadblock_record")
    return s.value, [v.value for v in c]


# ---------------------------------------------------------------------------
# Device API
# ---------------------------------------------------------------------------

class DeviceStream:
    """A compressed stream resident in device memory with its side index."""

    def __init__(self, codec: "Codec", capacity: int | None = None, data=None):
        import torch
        self.codec = codec
        cap = capacity if capacity is not None else codec.max_stream_bytes
        if data is not None:
            self.buf = data
            cap = data.numel()
        else:
            self.buf = torch.empty(max(cap, 16), dtype=torch.uint8, device=codec.device)
        self.index = torch.zeros(codec.index_bytes, dtype=torch.uint8, device=codec.device)
        self.desc = StreamDesc(self.buf.data_ptr(), cap, self.index.data_ptr(), 0, 0)

    @classmethod
    def from_bytes(cls, codec: "Codec", data) -> "DeviceStream":
        """Wrap wire bytes (a CUDA uint8 tensor, or bytes copied to the device)."""
        import torch
        if not isinstance(data, torch.Tensor):
            data = torch.frombuffer(bytearray(data), dtype=torch.uint8).to(codec.device)
        return cls(codec, data=data)

    def size(self) -> int:
        s = ctypes.c_size_t(0)
        _check(lib().zccl_gpu_stream_size(ctypes.byref(self.desc), self.codec.n, self.codec.L,
                                          self.codec.T, ctypes.byref(s), self.codec.stream_ptr),
               "zccl_gpu_stream_size")
        return s.value

    def tobytes(self) -> bytes:
        return self.buf[: self.size()].cpu().numpy().tobytes()


class Codec:
    """Device API for one geometry (n floats, block size L, writer count T)."""

    def __init__(self, n: int, L: int = 32, T: int = 1, device: str = "cuda", stream=None,
                 fixed: bool = False):
        """fixed: the fixed-rate appendix codec's block layout
        (ZCCL/src/ZCCL_appendix.c:65-590) instead of fastmode1's; such
        streams compress and decompress only (no homomorphic add)."""
        import torch
        self.n, self.L, self.T = int(n), int(L), int(T)
        self.fixed = bool(fixed)
        self.device = torch.device(device)
        self.max_stream_bytes = lib().zccl_gpu_max_stream_bytes(self.n, self.L, self.T)
        self.index_bytes = lib().zccl_gpu_index_bytes(self.n, self.L, self.T)
        ws = lib().zccl_gpu_workspace_bytes(self.n, self.L, self.T)
        if not (self.max_stream_bytes and self.index_bytes and ws):
            raise ZcclError(-1, f"geometry n={n} L={L} T={T}")
        self.ws = torch.zeros(ws, dtype=torch.uint8, device=self.device)
        self.torch_stream = stream or torch.cuda.current_stream(self.device)
        self.stream_ptr = ctypes.c_void_p(self.torch_stream.cuda_stream)

    def new_stream(self, capacity: int | None = None) -> DeviceStream:
        return DeviceStream(self, capacity)

    def compress(self, x, eb: float, out: DeviceStream | None = None) -> DeviceStream:
        out = out or self.new_stream()
        fn = lib().zccl_gpu_compress_fixed if self.fixed else lib().zccl_gpu_compress
        _check(fn(ctypes.byref(out.desc), x.data_ptr(), self.n, eb, self.L, self.T, self.ws.data_ptr(),
                  self.stream_ptr), "zccl_gpu_compress")
        return out

    def decompress(self, s: DeviceStream, eb: float, out=None):
        import torch
        out = out if out is not None else torch.empty(self.n, dtype=torch.float32,
                                                      device=self.device)
        fn = lib().zccl_gpu_decompress_fixed if self.fixed else lib().zccl_gpu_decompress
        _check(fn(out.data_ptr(), ctypes.byref(s.desc), self.n, eb, self.L, self.T, self.ws.data_ptr(),
                  self.stream_ptr), "zccl_gpu_decompress")
        return out

    def decompress_accumulate(self, s: DeviceStream, eb: float, acc):
        """acc += the stream's floats (one rounding per sum), in one pass; the
        stream must carry its tile starting values (compressed or summed on
        the device)."""
        _check(lib().zccl_gpu_decompress_accumulate(acc.data_ptr(), ctypes.byref(s.desc), self.n, eb, self.L,
                                                    self.T, self.ws.data_ptr(), self.stream_ptr),
               "zccl_gpu_decompress_accumulate")
        return acc

    def homadd(self, ins, out: DeviceStream | None = None, cases=None) -> DeviceStream:
        if self.fixed:
            raise ZcclError(-1, "the fixed-rate layout has no homomorphic add")
        out = out or self.new_stream()
        arr = (StreamDesc * len(ins))(*[s.desc for s in ins])
        rc = lib().zccl_gpu_homadd_cases(ctypes.byref(out.desc), arr, len(ins), self.n, self.L,
                                         self.T, self.ws.data_ptr(),
                                         cases.data_ptr() if cases is not None else None,
                                         self.stream_ptr)
        for s, d in zip(ins, arr):  # the call may have indexed the inputs
            s.desc.indexed, s.desc.qprev_valid = d.indexed, d.qprev_valid
        _check(rc, "zccl_gpu_homadd")
        return out

    def build_index(self, s: DeviceStream) -> None:
        _check(lib().zccl_gpu_build_index(ctypes.byref(s.desc), self.n, self.L, self.T,
                                          self.ws.data_ptr(), self.stream_ptr),
               "zccl_gpu_build_index")

    def check(self) -> None:
        _check(lib().zccl_gpu_check(self.ws.data_ptr(), self.stream_ptr), "device status")

    def _status_words(self):
        return self.ws[:8]


def check_all(objs) -> None:
    """Check many Codecs and Batches with one device-to-host read: their
    status words (the first 8 bytes of each workspace or batch memory) are
    gathered into one tensor and read once; only when one is non-zero is
    that object checked the usual way (which decodes, clears and raises)
    and the others cleared.  Every object's work must be on the current
    stream or ordered before it."""
    import torch
    objs = list(objs)
    if not objs:
        return
    words = torch.stack([o._status_words() for o in objs]).cpu()
    bad = [o for o, w in zip(objs, words) if bool(w.any())]
    if bad:
        for o in objs:
            if o is not bad[0]:
                o._status_words().zero_()
        bad[0].check()


BATCH_COMPRESS, BATCH_HOMADD, BATCH_DECOMPRESS = 0, 1, 2


class Batch:
    """Many streams in one persistent launch (the zccl_gpu_batch_* calls).

    kind BATCH_COMPRESS: jobs are (x, eb, T, out) with x a CUDA float
    tensor and out a DeviceStream; kind BATCH_HOMADD: jobs are (ins, T, out)
    with ins a list of indexed DeviceStreams of one geometry; kind
    BATCH_DECOMPRESS: jobs are (s, eb, T, y, accumulate) with s an indexed
    DeviceStream (with its tile starting values) and y a CUDA float tensor
    that receives (or, with accumulate, is added) the floats.  Planned once;
    run() is one memset and one launch on `stream` (a torch stream, default
    the current one), which can be recorded into a CUDA graph."""

    def __init__(self, kind: int, jobs, L: int = 32, device: str = "cuda", stream=None):
        import torch
        self.kind, self.L = kind, int(L)
        self.torch_stream = stream or torch.cuda.current_stream(torch.device(device))
        n = len(jobs)
        arr = (BatchJobDesc * n)()
        self._keep = []  # ctypes arrays the descriptors point into
        self.outs = []
        for k, job in enumerate(jobs):
            d = arr[k]
            if kind == BATCH_COMPRESS:
                x, eb, T, out = job
                d.d_in, d.n, d.eb, d.T = x.data_ptr(), x.numel(), float(eb), int(T)
            elif kind == BATCH_DECOMPRESS:
                s, eb, T, y, accumulate = job
                d.ins = ctypes.pointer(s.desc)
                d.P, d.n, d.eb, d.T = 1, y.numel(), float(eb), int(T)
                d.d_out, d.accumulate = y.data_ptr(), int(bool(accumulate))
                self._keep.append((s, y))
                continue
            else:
                ins, T, out = job
                ia = (StreamDesc * len(ins))(*[s.desc for s in ins])
                self._keep.append(ia)
                d.ins, d.P, d.n, d.T = ia, len(ins), out.codec.n, int(T)
            d.out = ctypes.pointer(out.desc)
            self.outs.append(out)
        self._jobs = arr
        nbytes = lib().zccl_gpu_batch_bytes(kind, arr, n, self.L)
        if not nbytes:
            raise ZcclError(-1, "zccl_gpu_batch_bytes")
        self.mem = torch.empty(nbytes, dtype=torch.uint8, device=device)
        self.desc = BatchDesc()
        _check(lib().zccl_gpu_batch_plan(ctypes.byref(self.desc), kind, arr, n, self.L, self.mem.data_ptr(),
                                         nbytes, ctypes.c_void_p(self.torch_stream.cuda_stream)),
               "zccl_gpu_batch_plan")

    def _st(self, stream):
        import torch
        s = stream or torch.cuda.current_stream()
        return ctypes.c_void_p(s.cuda_stream)

    def run(self, stream=None) -> None:
        _check(lib().zccl_gpu_batch_run(ctypes.byref(self.desc), self._st(stream)), "zccl_gpu_batch_run")

    def tune(self, stream=None) -> int:
        _check(lib().zccl_gpu_batch_tune(ctypes.byref(self.desc), self._st(stream)), "zccl_gpu_batch_tune")
        return self.desc.grid

    def check(self, stream=None) -> None:
        _check(lib().zccl_gpu_batch_check(ctypes.byref(self.desc), self._st(stream)), "batch status")

    def _status_words(self):
        return self.mem[:8]
