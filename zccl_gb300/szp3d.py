"""The SZp 3-D Lorenzo codec on device tensors (zccl_gpu_szp3d_*).

The serial stream form of ZCCL's 3-D codec (SZp_compress3D_fast /
SZp_compress3D, ZCCL/src/ZCCL_float.c:1706-1860; SZp_decompress3D,
ZCCL/src/ZCCLd_float.c:2801-2871): a (d1, d2, d3) float volume, d3 fastest,
in blocks of bs^3; the stream is one rate byte per block, then each block's
sign bits and fixed-length magnitude bits.  With T given, its OpenMP form
(SZp_compress3D_fast_openmp, ZCCL/src/ZCCL_float.c:1862-2048;
SZp_decompress3D_fast_openmp, ZCCL/src/ZCCLd_float.c:2873-3034): T size_t
offsets, then the serial-form streams of the T sub-volumes of the thread
grid.  The drop-in entry points of the same names take host or device
pointers.
"""
from __future__ import annotations

import ctypes

from . import ZcclError, _check, lib


class Szp3D:
    """Device codec for one volume shape and block side."""

    def __init__(self, dims, bs: int, device: str = "cuda", stream=None, T: int | None = None):
        import torch
        self.dims = tuple(int(d) for d in dims)
        self.bs = int(bs)
        self.T = None if T is None else int(T)
        self.device = torch.device(device)
        if self.T is None:
            self.max_bytes = lib().zccl_gpu_szp3d_max_bytes(*self.dims, self.bs)
            ws = lib().zccl_gpu_szp3d_workspace_bytes(*self.dims, self.bs)
        else:
            self.max_bytes = lib().zccl_gpu_szp3d_split_max_bytes(*self.dims, self.bs, self.T)
            ws = lib().zccl_gpu_szp3d_split_workspace_bytes(*self.dims, self.bs, self.T)
        if not (self.max_bytes and ws):
            raise ZcclError(-1, f"geometry {self.dims} bs={bs}")
        self.ws = torch.zeros(ws + 16, dtype=torch.uint8, device=self.device)
        self._size_at = ws  # a device size_t after the scratch
        self.torch_stream = stream or torch.cuda.current_stream(self.device)
        self.stream_ptr = ctypes.c_void_p(self.torch_stream.cuda_stream)

    def compress(self, x, eb: float, out=None):
        """Compress the float tensor x (numel d1*d2*d3); returns (stream
        buffer, size tensor): the first size bytes of the buffer are the
        stream."""
        import torch
        out = out if out is not None else torch.empty(self.max_bytes, dtype=torch.uint8, device=self.device)
        size = self.ws[self._size_at: self._size_at + 8]
        if self.T is None:
            rc = lib().zccl_gpu_szp3d_compress(out.data_ptr(), out.numel(), x.data_ptr(), *self.dims, self.bs,
                                               float(eb), self.ws.data_ptr(), size.data_ptr(), self.stream_ptr)
        else:
            rc = lib().zccl_gpu_szp3d_compress_split(out.data_ptr(), out.numel(), x.data_ptr(), *self.dims, self.bs,
                                                     float(eb), self.T, self.ws.data_ptr(), size.data_ptr(),
                                                     self.stream_ptr)
        _check(rc, "zccl_gpu_szp3d_compress")
        return out, size

    def size(self, size_tensor) -> int:
        import numpy as np
        return int(np.frombuffer(size_tensor.cpu().numpy().tobytes(), "<u8")[0])

    def decompress(self, stream, eb: float, out=None, avail: int | None = None):
        import torch
        out = out if out is not None else torch.empty(self.dims[0] * self.dims[1] * self.dims[2],
                                                      dtype=torch.float32, device=self.device)
        n = stream.numel() if avail is None else avail
        if self.T is None:
            rc = lib().zccl_gpu_szp3d_decompress(out.data_ptr(), stream.data_ptr(), n, *self.dims, self.bs, float(eb),
                                                 self.ws.data_ptr(), self.stream_ptr)
        else:
            rc = lib().zccl_gpu_szp3d_decompress_split(out.data_ptr(), stream.data_ptr(), n, *self.dims, self.bs,
                                                       float(eb), self.T, self.ws.data_ptr(), self.stream_ptr)
        _check(rc, "zccl_gpu_szp3d_decompress")
        return out

    def check(self) -> None:
        _check(lib().zccl_gpu_check(self.ws.data_ptr(), self.stream_ptr), "device status")


def SZp_compress3D_fast(oriData, cmpData, dim1, dim2, dim3, blockSideLength, errorBound) -> int:
    """ZCCL/src/ZCCL_float.c:1706 (host numpy arrays or device tensors);
    returns the assigned size."""
    from . import _ptr
    s = ctypes.c_size_t(0)
    lib().SZp_compress3D_fast(_ptr(oriData), _ptr(cmpData), dim1, dim2, dim3, blockSideLength, errorBound,
                              ctypes.byref(s))
    _check(lib().zccl_gpu_last_status(), "SZp_compress3D_fast")
    return s.value


def SZp_compress3D(oriData, cmpData, dim1, dim2, dim3, blockSideLength, errorBound) -> int:
    """ZCCL/src/ZCCL_float.c:1791; the same stream as SZp_compress3D_fast."""
    from . import _ptr
    s = ctypes.c_size_t(0)
    lib().SZp_compress3D(_ptr(oriData), _ptr(cmpData), dim1, dim2, dim3, blockSideLength, errorBound,
                         ctypes.byref(s))
    _check(lib().zccl_gpu_last_status(), "SZp_compress3D")
    return s.value


def SZp_decompress3D(decData, cmpData, dim1, dim2, dim3, blockSideLength, errorBound) -> None:
    """ZCCL/src/ZCCLd_float.c:2801."""
    from . import _ptr
    lib().SZp_decompress3D(_ptr(decData), _ptr(cmpData), dim1, dim2, dim3, blockSideLength, errorBound)
    _check(lib().zccl_gpu_last_status(), "SZp_decompress3D")


def SZp_compress3D_fast_openmp(oriData, cmpData, dim1, dim2, dim3, blockSideLength, errorBound) -> int:
    """ZCCL/src/ZCCL_float.c:1862, T = the OpenMP thread count (set it with
    zccl_gb300.set_omp_threads); returns the assigned size."""
    from . import _ptr
    s = ctypes.c_size_t(0)
    lib().SZp_compress3D_fast_openmp(_ptr(oriData), _ptr(cmpData), dim1, dim2, dim3, blockSideLength, errorBound,
                                     ctypes.byref(s))
    _check(lib().zccl_gpu_last_status(), "SZp_compress3D_fast_openmp")
    return s.value


def SZp_decompress3D_fast_openmp(decData, cmpData, dim1, dim2, dim3, blockSideLength, errorBound) -> None:
    """ZCCL/src/ZCCLd_float.c:2873, T = the OpenMP thread count."""
    from . import _ptr
    lib().SZp_decompress3D_fast_openmp(_ptr(decData), _ptr(cmpData), dim1, dim2, dim3, blockSideLength, errorBound)
    _check(lib().zccl_gpu_last_status(), "SZp_decompress3D_fast_openmp")
