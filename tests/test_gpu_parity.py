"""GPU parity: the sm_103a kernels, called through the C-ABI (matx_gb300 ->
libgbfir.so), against the reference's golden vectors and the CPU oracle.

Tolerances: FP32 results must be within rel-L2 1e-5 of the FP64 oracle (the
accuracy bar for the plain FP32 path); FP64 results within 1e-12.  The Harris
known-answer tests keep the reference's own per-component absolute thresholds
(1e-3 for float, 1e-12 for double, test/00_transform/ChannelizePoly.cu:52-60).
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, load_cases, rel_l2, seed_of

pytestmark = pytest.mark.gpu

FP32_TOL = 1e-5
FP64_TOL = 1e-12


@pytest.fixture(scope="module")
def mx():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import matx_gb300
    from matx_gb300 import build
    build.build()
    return matx_gb300


@pytest.fixture(scope="module")
def orc():
    import oracle
    oracle.build()
    return oracle


def dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    return t.cpu().numpy()


def tol_for(a):
    return FP64_TOL if a.dtype in (np.float64, np.complex128) else FP32_TOL


# ---- conv1d / corr -------------------------------------------------------------

@pytest.mark.parametrize("case", sorted(load_cases("conv.npz")))
def test_conv_golden(mx, case):
    c = load_cases("conv.npz")[case]
    a, b = c["a_op"], c["b_op"]
    tol = tol_for(a)
    for key, mode in (("conv_full", 0), ("conv_same", 1), ("conv_valid", 2)):
        y = host(mx.conv1d(dev(a), dev(b), mode))
        assert y.shape == c[key].shape
        assert rel_l2(y, c[key]) < tol, key
    assert rel_l2(host(mx.corr(dev(a), dev(b), 0)), c["corr"]) < tol
    assert rel_l2(host(mx.corr(dev(b), dev(a), 0)), c["corr_swap"]) < tol


def test_conv_known_answer(mx):
    x = np.array([1, 2, 3, 4], dtype=np.float32)
    h = np.array([2, 1, -1], dtype=np.float32)
    assert np.array_equal(host(mx.conv1d(dev(x), dev(h), 0)), [2, 5, 7, 9, 1, -4])
    assert np.array_equal(host(mx.conv1d(dev(x), dev(h), 1)), [5, 7, 9, 1])
    assert np.array_equal(host(mx.conv1d(dev(x), dev(h), 2)), [7, 9])


CONV_SHAPES = [(3, 5000, 63), (2, 4097, 64), (1, 100, 1), (2, 1, 1), (2, 7, 300), (1, 3000, 1500),
               (2, 9000, 2500), (4, 2048, 16), (1, 33, 33)]


@pytest.mark.parametrize("shape", CONV_SHAPES)
@pytest.mark.parametrize("mode", [0, 1, 2])
@pytest.mark.parametrize("kind", ["f32", "c64_rh", "c64_ch", "f32_ch", "f64", "c128"])
@pytest.mark.parametrize("is_corr", [False, True])
def test_conv_random(mx, orc, shape, mode, kind, is_corr):
    B, N, L = shape
    rng = np.random.default_rng(seed_of(shape, mode, kind, is_corr))
    dbl = kind in ("f64", "c128")
    x = rng.uniform(-1, 1, (B, N))
    h = rng.standard_normal(L)
    if kind.startswith("c"):
        x = x + 1j * rng.uniform(-1, 1, (B, N))
    if kind in ("c64_ch", "c128", "f32_ch"):
        h = h + 1j * rng.standard_normal(L)
    if dbl:
        x = x.astype(np.complex128 if np.iscomplexobj(x) else np.float64)
        h = h.astype(np.complex128 if np.iscomplexobj(h) else np.float64)
    else:
        x = x.astype(np.complex64 if np.iscomplexobj(x) else np.float32)
        h = h.astype(np.complex64 if np.iscomplexobj(h) else np.float32)
    y = host((mx.corr if is_corr else mx.conv1d)(dev(x), dev(h), mode))
    r = orc.conv1d(x, h, mode, is_corr)
    assert y.shape == r.shape
    # rel-L2 against the result, or against the magnitude of the products (the forward
    # error bound of a sum) where the result itself cancels to much less than that
    scale = np.linalg.norm(orc.conv1d(np.abs(x), np.abs(h), mode, is_corr))
    err = np.linalg.norm(y - r) / max(np.linalg.norm(r), 0.1 * scale)
    assert err < (FP64_TOL if dbl else FP32_TOL)


def test_conv_batched_filters(mx, orc):
    rng = np.random.default_rng(3)
    x = rng.standard_normal((4, 3000)).astype(np.float32)
    h = rng.standard_normal((4, 51)).astype(np.float32)
    y = host(mx.conv1d(dev(x), dev(h), 1))
    r = np.stack([orc.conv1d(x[i], h[i], 1)[0] for i in range(4)])
    assert rel_l2(y, r) < FP32_TOL


def test_conv_broadcast_signal(mx, orc):
    # the 1-D operand is cloned across the other's batch (conv.h:467-532), whichever it is
    rng = np.random.default_rng(4)
    x = rng.standard_normal(3000).astype(np.float32)
    h = rng.standard_normal((3, 40)).astype(np.float32)
    y = host(mx.conv1d(dev(x), dev(h), 0))
    r = np.stack([orc.conv1d(x, h[i], 0)[0] for i in range(3)])
    assert y.shape == r.shape and rel_l2(y, r) < FP32_TOL


@pytest.mark.parametrize("B,N,L", [(2, 5000, 63), (5, 3001, 17), (3, 9000, 1024), (4, 40, 300), (7, 1, 1),
                                   (9, 70000, 64), (2, 4100, 1000), (3, 2047, 8), (2, 3000, 40), (2, 3000, 52)])
@pytest.mark.parametrize("mode", [0, 1, 2])
@pytest.mark.parametrize("is_corr", [False, True])
@pytest.mark.parametrize("offset", [0, 1])
def test_conv_real_stream_matches_tile_kernel(mx, orc, B, N, L, mode, is_corr, offset):
    """Real rows with one shared filter of at most 1024 taps run on the persistent,
    prefetching kernel; the same filter given once per row runs on the one-tile-per-CTA
    kernel. Both make the same multiply-adds in the same order, so they agree bit for
    bit. offset = 1 takes the rows from a slice one sample in (unaligned windows: the
    4-byte copy path); odd output lengths give unaligned output rows."""
    import torch
    from matx_gb300 import _lib
    rng = np.random.default_rng(seed_of("stream", B, N, L, mode, is_corr, offset))
    x = rng.uniform(-1, 1, (B, N + offset)).astype(np.float32)
    h = rng.standard_normal(L).astype(np.float32)
    olen = (N + L - 1, max(N, L), max(N, L) - min(N, L) + 1)[mode]
    xd, hd, hrows = dev(x), dev(h), dev(np.tile(h, (B, 1)))
    f32 = mx._DT[torch.float32]
    xb = _lib.Buf(xd.data_ptr() + 4 * offset, B, N, N + offset, f32)  # rows of a slice
    lib = _lib.load()
    ys = []
    for hb in (_lib.Buf(hd.data_ptr(), 1, L, 0, f32), _lib.Buf(hrows.data_ptr(), B, L, L, f32)):
        y = torch.empty(B, olen, device="cuda")
        _lib.check(lib.gbfir_conv1d(_lib.Buf(y.data_ptr(), B, olen, olen, f32), xb, hb, mode, int(is_corr), 0,
                                    mx._stream()))
        ys.append(y)
    y = ys[0]
    assert torch.equal(y, ys[1])
    r = orc.conv1d(np.ascontiguousarray(x[:, offset:]), h, mode, is_corr)
    scale = np.linalg.norm(orc.conv1d(np.abs(x[:, offset:]), np.abs(h), mode, is_corr))
    assert np.linalg.norm(host(y) - r) / max(np.linalg.norm(r), 0.1 * scale) < FP32_TOL


def test_conv_config_rows(mx, orc):
    # C1: 8 x 2^20 real, 63-tap Hamming sinc, FULL; every row checked on a sample of rows
    rng = np.random.default_rng(2024)
    x = rng.uniform(-1, 1, (8, 1 << 20)).astype(np.float32)
    n = np.arange(63) - 31
    h = (np.sinc(0.25 * n) * np.hamming(63)).astype(np.float64)
    h = (h / h.sum()).astype(np.float32)
    y = host(mx.conv1d(dev(x), dev(h), 0))
    assert y.shape == (8, (1 << 20) + 62)
    for row in (0, 5):
        assert rel_l2(y[row], orc.conv1d(x[row], h, 0)[0]) < FP32_TOL


# ---- resample_poly -----------------------------------------------------------------

@pytest.mark.parametrize("case", sorted(load_cases("resample.npz")))
def test_resample_golden(mx, case):
    c = load_cases("resample.npz")[case]
    up, down = (int(v) for v in c["updown"])
    y = host(mx.resample_poly(dev(c["a"]), dev(c["h"]), up, down))
    assert y.shape == c["y"].shape
    tol = FP64_TOL if c["a"].dtype == np.float64 else FP32_TOL
    assert rel_l2(y, c["y"]) < tol


def kaiser_filter(up, down):
    from scipy import signal
    m = max(up, down)
    return signal.firwin(2 * 10 * m + 1, 1.0 / m, window=("kaiser", 5.0))


RATIOS = [(3, 2), (4, 5), (160, 147), (1, 2), (2, 3), (3, 4), (5, 4), (2, 1), (7, 1), (1, 7), (1, 16),
          (384, 3125), (6, 4), (5, 5)]


@pytest.mark.parametrize("updown", RATIOS)
@pytest.mark.parametrize("kind", ["c64_rh", "f32", "c64_ch", "f32_ch", "c128_rh", "f64"])
def test_resample_random(mx, orc, updown, kind):
    up, down = updown
    rng = np.random.default_rng(seed_of(updown, kind))
    B, N = 3, 5003
    dbl = kind.startswith("c128") or kind == "f64"
    x = rng.standard_normal((B, N))
    if kind.startswith("c"):
        x = (x + 1j * rng.standard_normal((B, N))) / np.sqrt(2)
    h = kaiser_filter(up, down)
    if kind.endswith("_ch"):
        h = h * np.exp(1j * rng.uniform(0, 2 * np.pi, h.size))
    fdt = (np.complex128 if np.iscomplexobj(h) else np.float64) if dbl else \
        (np.complex64 if np.iscomplexobj(h) else np.float32)
    xdt = (np.complex128 if np.iscomplexobj(x) else np.float64) if dbl else \
        (np.complex64 if np.iscomplexobj(x) else np.float32)
    x, h = x.astype(xdt), h.astype(fdt)
    y = host(mx.resample_poly(dev(x), dev(h), up, down))
    r = orc.resample_poly(x, h, up, down)
    assert y.shape == r.shape
    assert rel_l2(y, r) < (FP64_TOL if dbl else FP32_TOL)


@pytest.mark.parametrize("N,L,up,down", [(1, 3, 3, 1), (1, 2, 3, 1), (1, 1, 3, 2), (10, 1, 1, 3),
                                         (5, 100, 7, 3), (3, 4001, 160, 147), (64, 12, 3, 2),
                                         (1000, 2, 2, 3), (257, 255, 4, 5), (3500, 62501, 384, 3125)])
def test_resample_edges(mx, orc, N, L, up, down):
    rng = np.random.default_rng(N * 7 + L)
    x = (rng.standard_normal((2, N)) + 1j * rng.standard_normal((2, N))).astype(np.complex64)
    h = rng.standard_normal(L).astype(np.float32)
    y = host(mx.resample_poly(dev(x), dev(h), up, down))
    r = orc.resample_poly(x, h, up, down)
    assert y.shape == r.shape
    assert rel_l2(y, r) < FP32_TOL


def test_resample_identity_ignores_filter(mx):
    # up == down after the gcd is a copy (resample_poly.h:333-336)
    rng = np.random.default_rng(1)
    x = (rng.standard_normal((2, 999)) + 1j).astype(np.complex64)
    y = host(mx.resample_poly(dev(x), dev(np.ones(7, np.float32)), 6, 6))
    assert np.array_equal(y, x)


def test_resample_tile_overrides_agree(mx, orc):
    rng = np.random.default_rng(9)
    x = (rng.standard_normal((2, 20000)) + 1j * rng.standard_normal((2, 20000))).astype(np.complex64)
    for up, down in ((3, 2), (4, 5), (160, 147)):
        h = kaiser_filter(up, down).astype(np.float32)
        r = orc.resample_poly(x, h, up, down)
        try:
            for rq, wc, g, nb in ((1, 1, 0, 0), (4, 1, 0, 1), (2, 2, 0, 2), (1, 8, 0, 1), (2, 1, 2, 0),
                                  (1, 4, 4, 2), (4, 2, 16, 1), (1, 10, 0, 1), (1, 12, 8, 2), (1, 16, 32, 1),
                                  (2, 10, 0, 1), (2, 16, 32, 6)):
                mx.set_resample_tile(rq, wc, g, nb)
                y = host(mx.resample_poly(dev(x), dev(h), up, down))
                assert rel_l2(y, r) < FP32_TOL, (up, down, rq, wc, g, nb)
        finally:
            mx.set_resample_tile(0, 0, 0, 0)


@pytest.mark.parametrize("case", [
    # (up, down, batch, N, tile): rows of Nt = 24, 4, 2, 160, 20 outputs, whole and partial last rows
    (3, 2, 2, 20001, (4, 2, 8, 1)), (3, 2, 3, 20000, (2, 1, 8, 2)), (4, 5, 1, 20003, (2, 1, 1, 2)),
    (4, 5, 2, 20000, (4, 1, 1, 1)), (1, 2, 2, 9999, (2, 2, 2, 2)), (160, 147, 2, 20000, (1, 10, 1, 1)),
    (160, 147, 1, 20011, (1, 8, 1, 2)), (5, 4, 2, 20002, (2, 2, 0, 1)), (2, 1, 3, 7777, (4, 1, 0, 2)),
    # odd row stride, double-buffered windows with one staging buffer per warp (two CTAs per
    # SM): long rows, rows of one or two tiles (every window reaches past a signal end and is
    # staged by cp.async), and signals shorter than one window
    (160, 147, 2, 20000, (1, 10, 1, 2)), (160, 147, 8, 3001, (1, 10, 1, 2)),
    (160, 147, 16, 500, (1, 10, 1, 2)), (160, 147, 6, 7003, (1, 10, 1, 1)),
])
def test_resample_tma_store_epilogue(mx, orc, case):
    """Buffers + 4 sends the outputs through shared memory and TMA tensor stores: the result
    equals the direct stores bit for bit (same arithmetic) and the oracle within FP32_TOL;
    rows past the last whole row and odd batch strides take the direct stores."""
    import torch
    up, down, B, N, (rq, wc, g, nb) = case
    rng = np.random.default_rng(seed_of("tma_store", *case[:4]))
    x = (rng.standard_normal((B, N)) + 1j * rng.standard_normal((B, N))).astype(np.complex64)
    h = kaiser_filter(up, down).astype(np.float32)
    try:
        mx.set_resample_tile(rq, wc, g, nb)
        y_direct = mx.resample_poly(dev(x), dev(h), up, down)
        mx.set_resample_tile(rq, wc, g, nb | 4)
        y_tma = mx.resample_poly(dev(x), dev(h), up, down)
        torch.cuda.synchronize()
    finally:
        mx.set_resample_tile(0, 0, 0, 0)
    assert torch.equal(y_tma, y_direct), case
    assert rel_l2(host(y_tma), orc.resample_poly(x, h, up, down)) < FP32_TOL, case


@pytest.mark.parametrize("case", [
    # (up, down, batch, N, (rows per thread, column warps, group)): even row strides (cp.async
    # into the XOR layout), odd ones (bulk copies), windows past the signal ends, partial
    # last rows and tiles, and many tiles per CTA so that the ring wraps many times
    (3, 2, 2, 20001, (2, 2, 8)), (3, 2, 3, 20000, (1, 1, 4)), (4, 5, 1, 20003, (2, 2, 3)),
    (4, 5, 2, 20000, (1, 1, 1)), (160, 147, 2, 20011, (1, 10, 1)), (160, 147, 1, 20000, (2, 16, 1)),
    (1, 2, 2, 9999, (2, 2, 2)), (2, 1, 3, 7777, (1, 4, 0)), (3, 2, 64, 1 << 18, (1, 1, 2)),
    (4, 5, 64, 1 << 18, (2, 1, 1)), (3, 2, 2, 20001, (4, 2, 8)), (160, 147, 2, 20011, (4, 8, 1)),
    (4, 5, 64, 1 << 18, (4, 1, 3)),
    # paired walk: S/2 odd (plain layout, bulk copies) and S/2 = 2^t * odd, t = 1..4 (unit XOR)
    (3, 2, 2, 20001, (2, 2, 3)), (3, 2, 3, 20011, (2, 8, 20)), (4, 5, 2, 20000, (2, 2, 2)),
    (4, 5, 2, 20003, (1, 1, 4)), (160, 147, 2, 20011, (2, 10, 2)), (3, 2, 64, 1 << 18, (2, 4, 12)),
    (1, 2, 2, 9999, (2, 1, 8)), (4, 5, 64, 1 << 18, (2, 1, 6)), (3, 2, 2, 30000, (1, 8, 32)),
])
def test_resample_ring_form(mx, orc, case):
    """Buffers = 3 is the ring form (a staging warp, 3-4 window slots, mbarriers instead of
    CTA barriers) and + 8 the paired walk (two samples per load, bands from even k): the same
    multiply-adds in the same order as the two-buffer form (a leading zero tap adds +-0), so
    bit for bit the same outputs, with direct and with TMA-store epilogues; rows checked
    against the oracle."""
    import torch
    up, down, B, N, (rq, wc, g) = case
    rng = np.random.default_rng(seed_of("ring", *case[:4]))
    x = (rng.standard_normal((B, N)) + 1j * rng.standard_normal((B, N))).astype(np.complex64)
    h = kaiser_filter(up, down).astype(np.float32)
    xd, hd = dev(x), dev(h)
    try:
        mx.set_resample_tile(rq, wc, g, 2)
        y2 = mx.resample_poly(xd, hd, up, down)
        ys = {}
        # ring; + TMA-store epilogue; + paired walk (even strides), also in the one- and
        # two-buffer forms
        for nb in (3, 7, 11, 15, 9, 10, 14):
            mx.set_resample_tile(rq, wc, g, nb)
            ys[nb] = mx.resample_poly(xd, hd, up, down)
        torch.cuda.synchronize()
        assert mx._lib.load().gbfir_tc_status() == 0
    finally:
        mx.set_resample_tile(0, 0, 0, 0)
    for nb, y in ys.items():
        assert torch.equal(y, y2), (case, nb)
    y3 = ys[3]
    rows = [0, B - 1] if B > 1 else [0]
    assert rel_l2(host(y3[rows]), orc.resample_poly(x[rows], h, up, down, nthreads=2)) < FP32_TOL, case


@pytest.mark.parametrize("updown", [(3, 2), (4, 5), (160, 147)])
def test_resample_config_rows(mx, orc, updown):
    # C2 at full size: 64 x 2^20 complex Gaussian; sampled rows against the oracle,
    # plus linearity across the whole batch (a size-independent property).
    import torch
    up, down = updown
    g = torch.Generator(device="cuda").manual_seed(up * 1000 + down)
    x = torch.randn(64, 1 << 20, dtype=torch.complex64, device="cuda", generator=g)
    h = torch.from_numpy(kaiser_filter(up, down).astype(np.float32)).cuda()
    y = mx.resample_poly(x, h, up, down)
    assert y.shape == (64, mx.resample_out_len(1 << 20, up, down))
    xs = host(x[[0, 37, 63]])
    ys = host(y[[0, 37, 63]])
    assert rel_l2(ys, orc.resample_poly(xs, host(h), up, down, nthreads=3)) < FP32_TOL
    y2 = mx.resample_poly(2.0 * x[:8] - 0.5j * x[8:16], h, up, down)
    lin = 2.0 * y[:8] - 0.5j * y[8:16]
    assert float((y2 - lin).abs().norm() / lin.abs().norm()) < FP32_TOL


# ---- channelize_poly ------------------------------------------------------------------

@pytest.mark.parametrize("case", sorted(load_cases("channelize.npz")))
def test_channelize_golden(mx, case):
    c = load_cases("channelize.npz")[case]
    M, D = (int(v) for v in c["md"])
    a = c["a"]
    y = host(mx.channelize_poly(dev(a), dev(c["h"]), M, D))
    assert y.shape == c["y"].shape
    tol = FP64_TOL * 10 if a.dtype == np.complex128 else FP32_TOL
    assert rel_l2(y, c["y"]) < tol
    if "y_hreal" in c:
        yr = host(mx.channelize_poly(dev(a), dev(np.real(c["h"]).copy()), M, D))
        assert rel_l2(yr, c["y_hreal"]) < tol


@pytest.mark.parametrize("double", [False, True])
def test_channelize_harris2003(mx, double):
    z = np.load(os.path.join(GOLDEN, "harris2003.npz"))
    M = int(z["M"][0])
    dt = np.float64 if double else np.float32
    y = host(mx.channelize_poly(dev(z["x"].astype(dt)), dev(z["h"].astype(dt)), M, M))
    thresh = 1e-12 if double else 1e-3
    assert np.max(np.abs(y.real - z["y"].real)) < thresh
    assert np.max(np.abs(y.imag - z["y"].imag)) < thresh


@pytest.mark.parametrize("double", [False, True])
def test_channelize_harris2003_oversampled(mx, double):
    z = np.load(os.path.join(GOLDEN, "harris2003_oversampled.npz"))
    M, D = (int(v) for v in z["MD"])
    cdt, rdt = (np.complex128, np.float64) if double else (np.complex64, np.float32)
    y = host(mx.channelize_poly(dev(z["x"].astype(cdt)), dev(z["h"].astype(rdt)), M, D))
    thresh = 1e-12 if double else 1e-3
    assert np.max(np.abs(y - z["y"])) < thresh


@pytest.mark.parametrize("MD", [(64, 64), (256, 256), (8, 8), (10, 10), (181, 181), (1, 1), (2, 2), (32, 32),
                                (128, 128), (512, 512), (40, 28), (16, 12), (64, 48), (9, 4), (256, 192)])
@pytest.mark.parametrize("taps_per", [1, 5, 16, 32])
@pytest.mark.parametrize("kind", ["c64_rh", "c64_ch", "f32"])
def test_channelize_random(mx, orc, MD, taps_per, kind):
    M, D = MD
    rng = np.random.default_rng(seed_of(MD, taps_per, kind))
    N = 40 * M + 17
    x = rng.standard_normal((2, N))
    if kind.startswith("c"):
        x = x + 1j * rng.standard_normal((2, N))
    L = max(1, taps_per * M - 3)
    h = rng.standard_normal(L) / np.sqrt(L)
    if kind == "c64_ch":
        h = h + 1j * rng.standard_normal(L) / np.sqrt(L)
    x = x.astype(np.complex64 if np.iscomplexobj(x) else np.float32)
    h = h.astype(np.complex64 if np.iscomplexobj(h) else np.float32)
    y = host(mx.channelize_poly(dev(x), dev(h), M, D))
    r = orc.channelize_poly(x, h, M, D)
    assert y.shape == r.shape
    assert rel_l2(y, r) < FP32_TOL


@pytest.mark.parametrize("MP", [(64, 32), (256, 16)])
def test_channelize_config_rows(mx, orc, MP):
    # C3 at full size: 4 x 2^24 complex Gaussian, D == M; one sampled row segment
    # against the oracle and linearity over the batch.
    import torch
    M, P = MP
    g = torch.Generator(device="cuda").manual_seed(M)
    x = torch.randn(4, 1 << 24, dtype=torch.complex64, device="cuda", generator=g)
    n = np.arange(M * P) - (M * P - 1) / 2
    h = np.sinc(n / M) * np.kaiser(M * P, 5.0) / M
    h = torch.from_numpy(h.astype(np.float32)).cuda()
    y = mx.channelize_poly(x, h, M, M)
    assert y.shape == (4, (1 << 24) // M, M)
    seg = 1 << 18  # first 2^18 samples of row 2: its outputs are the first seg/M steps
    r = orc.channelize_poly(host(x[2, :seg]), host(h), M, M, nthreads=4)[0]
    assert rel_l2(host(y[2, : seg // M]), r) < FP32_TOL
    y2 = mx.channelize_poly(x[:2] + 3.0 * x[2:], h, M, M)
    lin = y[:2] + 3.0 * y[2:]
    assert float((y2 - lin).abs().norm() / lin.abs().norm()) < FP32_TOL


def test_launches_are_counted(mx):
    import torch
    before = mx.launch_count()
    mx.resample_poly(torch.zeros(2, 100, dtype=torch.complex64, device="cuda"),
                     torch.ones(5, device="cuda"), 3, 2)
    assert mx.launch_count() == before + 1
