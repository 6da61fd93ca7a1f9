"""The C-ABI library: loads without a GPU, exports every function
include/zccl_gpu.h declares, and answers its host-side queries (sizes, width
table) consistently with the oracle.  No device work happens here."""
from __future__ import annotations

import ctypes
import os
import re

import pytest

import zccl_gb300 as Z
from oracle import zoracle

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                      "zccl_gpu.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = "\n".join(l for l in text.splitlines() if not l.lstrip().startswith("#"))
    return sorted(set(re.findall(r"\b((?:ZCCL|zccl)_\w+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(Z.LIB_PATH):
        Z_build = __import__("zccl_gb300.build", fromlist=["build"])
        Z_build.build()
    return Z.lib()


def test_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 19
    for name in names:
        assert hasattr(lib, name), name
    assert set(names) <= set(Z.EXPORTS)


def test_reference_entry_points_present(lib):
    for name in ("ZCCL_float_openmp_threadblock_arg", "ZCCL_float_decompress_openmp_threadblock_arg",
                 "ZCCL_float_homomophic_add_openmp_threadblock", "ZCCL_float_single_thread_arg",
                 "ZCCL_float_decompress_single_thread_arg", "ZCCL_float_homomophic_add_single_thread"):
        assert name in declared_functions()


@pytest.mark.parametrize("n,L,T", [(1, 32, 1), (77, 8, 3), (4097, 36, 8), (16777216, 32, 72),
                                   (134217728, 32, 16), (1000, 256, 4)])
def test_size_queries(lib, n, L, T):
    # the library's worst case equals the oracle's (which adds 64 bytes of slack)
    assert lib.zccl_gpu_max_stream_bytes(n, L, T) == zoracle.worst_stream_bytes(n, L, T) - 64
    ib = lib.zccl_gpu_index_bytes(n, L, T)
    nblocks = T * -(-(n // T - 1) // L) + (-(-((n % T) - 1) // L) if n % T else 0)
    assert nblocks <= ib <= nblocks + 64 + 16 * (n // L + 2)
    assert lib.zccl_gpu_workspace_bytes(n, L, T) >= 32


@pytest.mark.parametrize("n,L,T", [(3, 32, 4), (100, 0, 1), (100, 257, 1), (100, 32, 0)])
def test_invalid_geometry_rejected(lib, n, L, T):
    assert lib.zccl_gpu_max_stream_bytes(n, L, T) == 0
    assert lib.zccl_gpu_index_bytes(n, L, T) == 0
    assert lib.zccl_gpu_workspace_bytes(n, L, T) == 0


def test_width_table_is_host_libm(lib, port):
    assert Z.width_table()[1:] == [t if t else 0xFFFFFFFF
                                   for t in zoracle.width_thresholds(port.width)][1:]


def test_status_strings(lib):
    for code, text in Z.STATUS.items():
        assert lib.zccl_gpu_strerror(code).decode() == text


def test_null_arguments_rejected_without_device(lib):
    d = Z.StreamDesc(0, 0, 0, 0, 0)
    assert lib.zccl_gpu_compress(ctypes.byref(d), None, 100, 1e-3, 32, 1, None, None) == -1
    assert lib.zccl_gpu_build_index(ctypes.byref(d), 100, 32, 1, None, None) == -1
