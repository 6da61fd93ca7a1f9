"""The drop-in boundary as C callers see it.

* CPU: one C translation unit includes the reference's codec headers and
  include/zccl_gpu.h together, so any prototype that drifted from the
  reference's fails to compile.
* CPU: the reference's own codec driver
  (examples/testfloat_homocompress_fastmode1_arg.c) links against
  libzccl_gpu.so ahead of an archive of the reference's objects, the link
  line a maintainer uses, and its codec calls resolve to the library.
* CPU: the oracle restates the reference's _record counts and branch
  counters exactly (checked against the reference library).
* GPU: a C program (tests/native/dropin_driver.c) compiled against the
  header calls every drop-in entry point, the allocating and _record
  variants included; its outputs equal the oracle's.
The reference checkout is only needed by the first three, which skip
without it.
"""
from __future__ import annotations

import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import zoracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")
LIBDIR = os.path.join(ROOT, "zccl_gb300")
SHIM = os.path.join(ROOT, "oracle", "shim")


def ref_root():
    r = zoracle.reference_root()
    if not r:
        pytest.skip("no reference checkout")
    return r


def cc(*args, cwd=None):
    r = subprocess.run(["gcc", *args], capture_output=True, text=True, cwd=cwd)
    assert r.returncode == 0, r.stderr[-3000:]
    return r


def test_prototypes_agree_with_reference_headers(tmp_path):
    ref = ref_root()
    src = tmp_path / "both.c"
    src.write_text('#include "ZCCL_float.h"\n#include "ZCCLd_float.h"\n#include "ZCCL_appendix.h"\n'
                   '#include "zccl_gpu.h"\nint main(void) { return 0; }\n')
    cc("-std=c99", "-D_DEFAULT_SOURCE", "-fsyntax-only", f"-I{SHIM}", f"-I{ref}/ZCCL/include", f"-I{INCLUDE}",
       str(src))


CODEC_SYMBOLS = ["ZCCL_float_openmp_threadblock_arg", "ZCCL_float_decompress_openmp_threadblock_arg",
                 "ZCCL_float_homomophic_add_openmp_threadblock"]


def test_reference_driver_links_against_the_library(tmp_path):
    ref = ref_root()
    lib = os.path.join(LIBDIR, "libzccl_gpu.so")
    if not os.path.exists(lib):
        pytest.skip("library not built")
    # an archive of the reference's objects that the driver needs (the MPI
    # collectives stay out: there is no MPI here)
    srcs = ["ZCCL.c", "ZCCL_rw.c", "ZCCL_BytesToolkit.c", "ZCCL_TypeManager.c", "ZCCL_dataCompression.c",
            "ZCCL_utility.c", "ZCCL_float.c", "ZCCLd_float.c", "ZCCL_helper.c", "ZCCL_libs.c", "ZCCL_utils.c"]
    flags = ["-O1", "-std=c99", "-D_DEFAULT_SOURCE", "-fopenmp", "-w", f"-I{SHIM}", f"-I{ref}/ZCCL/include"]
    objs = []
    for s in srcs:
        o = str(tmp_path / (s[:-2] + ".o"))
        cc(*flags, "-c", f"{ref}/ZCCL/src/{s}", "-o", o)
        objs.append(o)
    cc(*flags, "-c", os.path.join(ROOT, "oracle", "shim", "ref_stubs.c"), "-o", str(tmp_path / "stubs.o"))
    objs.append(str(tmp_path / "stubs.o"))
    r = subprocess.run(["ar", "rcs", str(tmp_path / "libZCCL.a"), *objs], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    drv = str(tmp_path / "testfloat_homocompress_fastmode1_arg")
    # the integration guide's link line: the GPU library ahead of libZCCL.a
    cc(*flags, f"{ref}/examples/testfloat_homocompress_fastmode1_arg.c", f"-L{LIBDIR}", "-lzccl_gpu",
       str(tmp_path / "libZCCL.a"), "-lm", "-o", drv)
    nm = subprocess.run(["nm", drv], capture_output=True, text=True).stdout
    table = {ln.split()[-1]: ln.split()[-2] for ln in nm.splitlines() if len(ln.split()) >= 2}
    for sym in CODEC_SYMBOLS:
        assert table.get(sym) == "U", f"{sym} is {table.get(sym)} in the driver (defined by the archive?)"
    ldd = subprocess.run(["ldd", drv], capture_output=True, text=True,
                         env={**os.environ, "LD_LIBRARY_PATH": LIBDIR}).stdout
    assert "libzccl_gpu.so" in ldd


def test_record_counts_restated_exactly():
    if not zoracle.ref_available():
        pytest.skip("reference library not built")
    port, ref = zoracle.port(), zoracle.ref()
    rng = np.random.default_rng(8)
    for n, L in [(1, 32), (2, 32), (33, 32), (4097, 8), (10000, 36), (77777, 32), (5, 8), (65, 64)]:
        x = np.cumsum(rng.normal(0, 0.05, n)).astype(np.float32)
        x[n // 3: n // 2] = np.float32(0.25)  # constant stretches: zero-width blocks
        eb = float(np.float32(1e-3 * (float(x.max() - x.min()) + 1e-3)))
        stream, c_count, y, d_count = ref.ref_record(x, eb, L)
        assert stream == port.compress(x, eb, L, 1)
        assert np.array_equal(y, port.decompress(stream, n, eb, L, 1))
        assert port.record_counts(stream, n, L) == (c_count, d_count), (n, L)


def test_branch_counters_restated_exactly():
    if not zoracle.ref_available():
        pytest.skip("reference library not built")
    port, ref = zoracle.port(), zoracle.ref()
    rng = np.random.default_rng(9)
    n, L = 60013, 32
    x = np.cumsum(rng.normal(0, 0.05, n)).astype(np.float32)
    y = np.cumsum(rng.normal(0, 0.05, n)).astype(np.float32)
    x[:15000] = 1.0   # first zero
    y[10000:30000] = 2.0  # second zero, and both zero where they overlap
    eb = float(np.float32(1e-3 * float(x.max() - x.min())))
    for T in (1, 3, 8):
        sx, sy = port.compress(x, eb, L, T), port.compress(y, eb, L, T)
        h, cnt = ref.ref_homadd_record(sx, sy, n, eb, L, T)
        assert h == port.homadd(sx, sy, n, eb, L, T)
        assert min(cnt) > 0
        assert port.homadd_cases(sx, sy, n, L, T) == cnt, T


@pytest.mark.gpu
def test_c_caller_matches_oracle(tmp_path, port):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    exe = str(tmp_path / "dropin_driver")
    cc("-O2", "-std=c11", "-fopenmp", f"-I{INCLUDE}", os.path.join(ROOT, "tests", "native", "dropin_driver.c"),
       f"-L{LIBDIR}", "-lzccl_gpu", f"-Wl,-rpath,{LIBDIR}", "-o", exe)
    rng = np.random.default_rng(12)
    n, L, T = 300007, 32, 4
    x = np.cumsum(rng.normal(0, 0.02, n)).astype(np.float32)
    y = np.cumsum(rng.normal(0, 0.02, n)).astype(np.float32)
    x[1000:40000] = np.float32(0.5)
    y[30000:90000] = np.float32(-0.5)
    eb = float(np.float32(1e-4 * max(float(x.max() - x.min()), float(y.max() - y.min()))))
    x.tofile(tmp_path / "x.f32")
    y.tofile(tmp_path / "y.f32")
    r = subprocess.run([exe, str(tmp_path), str(n), str(L), repr(eb), str(T)], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    out = {ln.split()[0]: [int(v) for v in ln.split()[1:]] for ln in r.stdout.splitlines()}
    sx, sy = port.compress(x, eb, L, T), port.compress(y, eb, L, T)
    assert (tmp_path / "a.zc").read_bytes() == sx
    assert np.array_equal(np.fromfile(tmp_path / "a.dec", np.float32), port.decompress(sx, n, eb, L, T))
    assert (tmp_path / "h.zc").read_bytes() == port.homadd(sx, sy, n, eb, L, T)
    assert out["malloc_stream_equal"] == [1] and out["malloc_floats_equal"] == [1]
    assert out["cases"] == port.homadd_cases(sx, sy, n, L, T)
    s1 = port.compress(x, eb, L, 1)
    assert (tmp_path / "a1.zc").read_bytes() == s1
    assert np.array_equal(np.fromfile(tmp_path / "a1.dec", np.float32), port.decompress(s1, n, eb, L, 1))
    assert tuple(out["compress_count"] + out["decompress_count"]) == port.record_counts(s1, n, L)
    assert out["split_slot"] == [len(s1)] and out["split_stream_equal"] == [1]
