"""The SZp 3-D codec (serial stream form): the oracle port against the
reference's golden streams on the CPU, and the CUDA path, through the C ABI
and the drop-in entry points, against both on the GPU.  Streams bit for
bit, decompressed floats by digest or bit for bit, |x' - x| <= eb."""
from __future__ import annotations

import hashlib
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def load_golden():
    with open(os.path.join(GOLD, "szp3d.json")) as f:
        meta = json.load(f)
    arr = np.load(os.path.join(GOLD, "szp3d.npz"))
    return meta["cases"], arr


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def test_float_rounding_tiers_match_double(tmp_path):
    """The codec's float quantization and reconstruction tiers (one FMA,
    float pairs, then the double steps near ties), restated in C with IEEE
    float arithmetic, give the double steps' integers and floats on about
    80 million seeded random, near-tie and wide-range inputs."""
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    exe = tmp_path / "sz3_rounding"
    src = os.path.join(os.path.dirname(__file__), "native", "sz3_rounding.c")
    subprocess.run([cc, "-O2", "-ffp-contract=off", "-o", str(exe), src, "-lm"], check=True)
    out = subprocess.run([str(exe), "160000"], capture_output=True, text=True, timeout=120)
    bad, checks = map(int, out.stdout.split())
    assert checks > 50_000_000
    assert bad == 0


def test_port_matches_reference_golden(port):
    cases, arr = load_golden()
    assert len(cases) == 56
    for c in cases:
        x, s = arr[f"x{c['i']}"], arr[f"s{c['i']}"].tobytes()
        dims, bs, eb = tuple(c["dims"]), c["bs"], c["eb"]
        assert port.szp3d_compress(x, dims, bs, eb) == s, c
        y = port.szp3d_decompress(s, dims, bs, eb)
        assert sha(y) == c["dec"], c
        assert np.abs(y.astype(np.float64) - x).max() <= eb * (1 + 1e-6) + 1e-6 * np.abs(x).max()


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    if not t.cuda.is_available():
        pytest.skip("no CUDA device")
    return t


@pytest.mark.gpu
def test_gpu_matches_reference_golden(torch):
    from zccl_gb300.szp3d import Szp3D
    cases, arr = load_golden()
    for c in cases:
        x, s = arr[f"x{c['i']}"], arr[f"s{c['i']}"].tobytes()
        dims, bs, eb = tuple(c["dims"]), c["bs"], c["eb"]
        codec = Szp3D(dims, bs)
        buf, size = codec.compress(torch.from_numpy(x).cuda(), eb)
        n = codec.size(size)
        codec.check()
        assert buf[:n].cpu().numpy().tobytes() == s, c
        y = codec.decompress(buf, eb, avail=n)
        codec.check()
        assert sha(y.cpu().numpy()) == c["dec"], c


@pytest.mark.gpu
@pytest.mark.parametrize("dims,bs", [((64, 80, 96), 4), ((37, 129, 70), 8), ((200, 3, 150), 2), ((40, 40, 40), 16)])
def test_gpu_volumes_against_port(torch, port, dims, bs):
    from zccl_gb300.szp3d import Szp3D
    rng = np.random.default_rng(sum(dims))
    i, j, k = np.meshgrid(*[np.arange(d, dtype=np.float64) for d in dims], indexing="ij")
    x = (np.exp(np.sin(i / 9.0) + np.cos(j / 13.0) * np.sin(k / 7.0)) + rng.normal(0, 0.05, dims)).astype(np.float32).ravel()
    eb = float(1e-4 * (x.max() - x.min()))
    s = port.szp3d_compress(x, dims, bs, eb)
    codec = Szp3D(dims, bs)
    buf, size = codec.compress(torch.from_numpy(x).cuda(), eb)
    n = codec.size(size)
    assert buf[:n].cpu().numpy().tobytes() == s
    y = codec.decompress(buf, eb, avail=n).cpu().numpy()
    codec.check()
    assert np.array_equal(y.view(np.uint32), port.szp3d_decompress(s, dims, bs, eb).view(np.uint32))
    assert np.abs(y.astype(np.float64) - x).max() <= eb * (1 + 1e-6) + 1e-6 * np.abs(x).max()


@pytest.mark.gpu
def test_dropin_host_and_device_pointers(torch):
    import zccl_gb300.szp3d as Z3
    cases, arr = load_golden()
    for c in cases[::5]:
        x, s = arr[f"x{c['i']}"], arr[f"s{c['i']}"].tobytes()
        dims, bs, eb = tuple(c["dims"]), c["bs"], c["eb"]
        out = np.zeros(len(s) + 64 * 1024, np.uint8)
        n = Z3.SZp_compress3D_fast(x, out, *dims, bs, eb)
        assert out[:n].tobytes() == s
        assert Z3.SZp_compress3D(x, out, *dims, bs, eb) == n
        y = np.zeros(x.size, np.float32)
        Z3.SZp_decompress3D(y, np.frombuffer(s, np.uint8).copy(), *dims, bs, eb)
        assert sha(y) == c["dec"]
        dx = torch.from_numpy(x).cuda()
        dout = torch.zeros(len(s) + 64 * 1024, dtype=torch.uint8, device="cuda")
        assert Z3.SZp_compress3D_fast(dx, dout, *dims, bs, eb) == n
        assert dout[:n].cpu().numpy().tobytes() == s
        dy = torch.zeros(x.size, dtype=torch.float32, device="cuda")
        Z3.SZp_decompress3D(dy, dout, *dims, bs, eb)
        assert sha(dy.cpu().numpy()) == c["dec"]


@pytest.mark.gpu
@pytest.mark.parametrize("eb", [1e-4 * 1.37, 2.0 ** -9, 3.3e-7])
def test_gpu_rounding_near_ties(torch, port, eb):
    """Inputs placed on and one to three ulps either side of the points where
    x * (0.5 / eb) + 0.5 is an integer, with quantized values up to 2^27 (both
    sides of 2^24 and 2^26), so that quantization and reconstruction meet the
    cases their double rounding decides; stream and floats must equal the
    oracle's bit for bit."""
    from zccl_gb300.szp3d import Szp3D
    dims, bs = (48, 40, 56), 4
    n = dims[0] * dims[1] * dims[2]
    rng = np.random.default_rng(7)
    inv = 0.5 / eb
    mag = np.where(rng.random(n) < 0.5, 2.0 ** 12, 2.0 ** rng.integers(20, 28, n))
    j = np.floor(rng.uniform(-1, 1, n) * mag)
    x = ((j - 0.5) / inv).astype(np.float32)
    x = (x.view(np.int32) + rng.integers(-3, 4, n).astype(np.int32)).view(np.float32)
    assert np.isfinite(x).all()
    s = port.szp3d_compress(x, dims, bs, eb)
    codec = Szp3D(dims, bs)
    buf, size = codec.compress(torch.from_numpy(x).cuda(), eb)
    m = codec.size(size)
    assert buf[:m].cpu().numpy().tobytes() == s
    y = codec.decompress(buf, eb, avail=m).cpu().numpy()
    codec.check()
    assert np.array_equal(y.view(np.uint32), port.szp3d_decompress(s, dims, bs, eb).view(np.uint32))


# ---- the OpenMP stream form (T sub-volumes) -------------------------------

def load_split_golden():
    with open(os.path.join(GOLD, "szp3d_split.json")) as f:
        meta = json.load(f)
    return meta["cases"], np.load(os.path.join(GOLD, "szp3d_split.npz"))


def test_split_port_matches_reference_golden(port):
    cases, arr = load_split_golden()
    assert len(cases) == 40
    for c in cases:
        x, s = arr[f"x{c['i']}"], arr[f"s{c['i']}"].tobytes()
        dims, bs, eb, T = tuple(c["dims"]), c["bs"], c["eb"], c["T"]
        assert port.dims3(T) == c["tdims"]
        assert port.szp3d_compress_split(x, dims, bs, eb, T) == s, c
        assert sha(port.szp3d_decompress_split(s, dims, bs, eb, T)) == c["dec"], c


def test_split_port_matches_reference_library(port):
    from oracle import zoracle
    if not zoracle.ref_available():
        pytest.skip("reference library not built")
    ref = zoracle.ref()
    for n in list(range(1, 70)) + [72, 96, 144, 1024]:
        assert port.dims3(n) == ref.dims3(n), n
    rng = np.random.default_rng(4)
    for dims in [(17, 19, 23), (40, 9, 12), (6, 6, 50)]:
        x = np.cumsum(rng.normal(0, 0.1, int(np.prod(dims)))).astype(np.float32)
        for bs, T in [(4, 5), (8, 6), (2, 4), (3, 16)]:
            eb = 1e-3 * float(x.max() - x.min())
            s = ref.szp3d_compress_split(x, dims, bs, eb, T)
            assert port.szp3d_compress_split(x, dims, bs, eb, T) == s, (dims, bs, T)
            assert np.array_equal(port.szp3d_decompress_split(s, dims, bs, eb, T).view(np.uint32),
                                  ref.szp3d_decompress_split(s, dims, bs, eb, T).view(np.uint32))


@pytest.mark.gpu
def test_split_gpu_matches_reference_golden(torch):
    import zccl_gb300 as Z
    from zccl_gb300 import szp3d as S
    cases, arr = load_split_golden()
    for c in cases:
        x, s = arr[f"x{c['i']}"], arr[f"s{c['i']}"].tobytes()
        dims, bs, eb, T = tuple(c["dims"]), c["bs"], c["eb"], c["T"]
        codec = S.Szp3D(dims, bs, T=T)
        buf, size = codec.compress(torch.from_numpy(x).cuda(), eb)
        n = codec.size(size)
        assert buf[:n].cpu().numpy().tobytes() == s, c
        y = codec.decompress(buf, eb, avail=n)
        codec.check()
        assert sha(y.cpu().numpy()) == c["dec"], c
        # the drop-ins, host pointers, T from the OpenMP thread count
        Z.set_omp_threads(T)
        out = np.zeros(codec.max_bytes + 64, np.uint8)
        m = S.SZp_compress3D_fast_openmp(x, out, *dims, bs, eb)
        assert out[:m].tobytes() == s, c
        yh = np.zeros(x.size, np.float32)
        S.SZp_decompress3D_fast_openmp(yh, np.frombuffer(s, np.uint8).copy(), *dims, bs, eb)
        assert sha(yh) == c["dec"], c


@pytest.mark.gpu
def test_split_gpu_on_a_field_against_port(torch, port):
    """A 96 x 80 x 100 log-normal field at T = 16 (a 4 x 2 x 2 grid), block
    side 4, device pointers through the drop-ins."""
    import zccl_gb300 as Z
    from zccl_gb300 import szp3d as S
    from zccl_gb300.workloads import grf_lognormal
    f = grf_lognormal(100, 9, "cuda")[: 96 * 80 * 100].contiguous()
    dims, bs, T = (96, 80, 100), 4, 16
    eb = float(1e-4 * float(f.max() - f.min()))
    ref = port.szp3d_compress_split(f.cpu().numpy(), dims, bs, eb, T)
    Z.set_omp_threads(T)
    out = torch.zeros(len(ref) + 4096, dtype=torch.uint8, device="cuda")
    m = S.SZp_compress3D_fast_openmp(f, out, *dims, bs, eb)
    assert out[:m].cpu().numpy().tobytes() == ref
    y = torch.zeros_like(f)
    S.SZp_decompress3D_fast_openmp(y, out, *dims, bs, eb)
    assert np.array_equal(y.cpu().numpy().view(np.uint32),
                          port.szp3d_decompress_split(ref, dims, bs, eb, T).view(np.uint32))


def test_split_rejects_more_parts_than_planes():
    import zccl_gb300 as Z
    lib = Z.lib()
    # T = 8 is a 2 x 2 x 2 grid: every axis needs two planes
    assert lib.zccl_gpu_szp3d_split_max_bytes(2, 64, 64, 4, 8) > 0
    assert lib.zccl_gpu_szp3d_split_max_bytes(1, 64, 64, 4, 8) == 0
    assert lib.zccl_gpu_szp3d_split_max_bytes(64, 64, 1, 4, 8) == 0
    assert lib.zccl_gpu_szp3d_split_workspace_bytes(64, 64, 1, 4, 8) == 0
    assert lib.zccl_gpu_szp3d_split_max_bytes(64, 64, 64, 4, 0) == 0
