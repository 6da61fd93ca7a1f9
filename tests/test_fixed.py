"""The fixed-rate appendix codec (ZCCL_float_openmp_threadblock_arg_2 and its
decompressor, ZCCL/src/ZCCL_appendix.c:65-590): the oracle port against the
reference's golden streams on the CPU; the CUDA path (device API, byte-only
streams through the header walk, drop-in entry points) against both on the
GPU, bytes and floats bit for bit."""
from __future__ import annotations

import hashlib
import json
import os

import numpy as np
import pytest

import zccl_gb300 as Z

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def load_golden():
    with open(os.path.join(GOLD, "fixed.json")) as f:
        cases = json.load(f)["cases"]
    return cases, np.load(os.path.join(GOLD, "fixed.npz"))


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def test_port_matches_reference_golden(port):
    cases, arr = load_golden()
    assert len(cases) == 144
    for c in cases:
        x, s = arr[f"x{c['i']}"], arr[f"s{c['i']}"].tobytes()
        assert port.compress_fixed(x, c["eb"], c["L"], c["T"]) == s, c
        assert sha(port.decompress_fixed(s, c["n"], c["eb"], c["L"], c["T"])) == c["dec"], c


def test_fixed_layout_differs_from_fastmode1(port):
    # whole bytes per magnitude: a wide block takes more bytes than fastmode1's bit packing
    x = (np.random.default_rng(3).normal(0, 1, 4097) * 1e3).astype(np.float32)
    eb = float(np.float32(1e-3))
    assert len(port.compress_fixed(x, eb, 32, 1)) > len(port.compress(x, eb, 32, 1))


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    if not t.cuda.is_available():
        pytest.skip("no CUDA device")
    Z.lib()
    return t


@pytest.mark.gpu
def test_gpu_matches_reference_golden(torch):
    cases, arr = load_golden()
    for c in cases:
        x, s = arr[f"x{c['i']}"], arr[f"s{c['i']}"].tobytes()
        codec = Z.Codec(c["n"], c["L"], c["T"], fixed=True)
        st = codec.compress(torch.from_numpy(x).cuda(), c["eb"])
        codec.check()
        assert st.tobytes() == s, c
        assert sha(codec.decompress(st, c["eb"]).cpu().numpy()) == c["dec"], c
        foreign = Z.DeviceStream.from_bytes(codec, s)  # the header walk in this layout
        assert sha(codec.decompress(foreign, c["eb"]).cpu().numpy()) == c["dec"], c
        codec.check()


@pytest.mark.gpu
def test_dropin_host_pointers(torch):
    cases, arr = load_golden()
    for c in [c for c in cases if c["T"] in (1, 3)][::7]:
        Z.set_omp_threads(c["T"])
        x, s = arr[f"x{c['i']}"], arr[f"s{c['i']}"].tobytes()
        out = np.zeros(4 * c["n"] + 8 * c["T"] + 4096, np.uint8)
        size = Z.ZCCL_float_openmp_threadblock_arg_2(out, x, 0, c["eb"], c["n"], c["L"])
        assert out[:size].tobytes() == s, c
        y = np.zeros(c["n"], np.float32)
        Z.ZCCL_float_decompress_openmp_threadblock_arg_2(y, c["n"], c["eb"], c["L"], out)
        assert sha(y) == c["dec"], c


@pytest.mark.gpu
def test_large_field_against_port(torch, port):
    n, L, T = 3 * 1024 * 1024 + 16, 32, 16
    rng = np.random.default_rng(8)
    x = (np.cumsum(rng.normal(0, 0.01, n)) + rng.normal(0, 0.2, n)).astype(np.float32)
    eb = float(np.float32(1e-4 * (x.max() - x.min())))
    codec = Z.Codec(n, L, T, fixed=True)
    st = codec.compress(torch.from_numpy(x).cuda(), eb)
    s = port.compress_fixed(x, eb, L, T)
    assert st.tobytes() == s
    y = codec.decompress(st, eb).cpu().numpy()
    codec.check()
    assert np.array_equal(y.view(np.uint32), port.decompress_fixed(s, n, eb, L, T).view(np.uint32))
