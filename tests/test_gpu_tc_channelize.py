"""Tensor-core forms of channelize_poly (tcgen05 DFT GEMM over the polyphase FIR
outputs) against the FP64 oracle.  Stated error bars (rel-L2 vs FP64): bf16 <= 1e-2,
fp16 <= 2e-3, bf16x3 <= 1e-6.  The forms cover the maximally decimated channelizer
(D == M) with M in {16, 32, 64} (one M-point DFT GEMM) and M in {128, 256} (a radix-2/4
stage in FP32, then a 64-point DFT GEMM); anything else is rejected with
GBFIR_ERR_NOT_SUPPORTED rather than silently run in FP32."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu
TOL = {"bf16": 1e-2, "fp16": 2e-3, "bf16x3": 1e-6}


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


def prototype(M, P):
    """Kaiser-windowed sinc low-pass of M*P taps, cut-off at 1/M of Nyquist."""
    n = np.arange(M * P) - (M * P - 1) / 2
    return np.sinc(n / M) * np.kaiser(M * P, 5.0) / M


@pytest.mark.parametrize("M,P", [(64, 32), (64, 8), (32, 16), (32, 3), (16, 8), (16, 1), (128, 8), (128, 24),
                                 (256, 16), (256, 1), (256, 5)])
@pytest.mark.parametrize("form", ["bf16x3", "bf16", "fp16"])
def test_tc_channelize_vs_fp64(mx, orc, M, P, form):
    import torch
    rng = np.random.default_rng(M * 7 + P)
    B, N = 2, M * 300 + 5  # ragged tail: the last frame is zero-padded
    x = ((rng.standard_normal((B, N)) + 1j * rng.standard_normal((B, N))) / np.sqrt(2)).astype(np.complex64)
    h = prototype(M, P).astype(np.float32)
    y = mx.channelize_poly(torch.from_numpy(x).cuda(), torch.from_numpy(h).cuda(), M, M,
                           precision=form).cpu().numpy()
    assert mx._lib.load().gbfir_tc_status() == 0
    r = orc.channelize_poly(x.astype(np.complex128), h.astype(np.float64), M, M)
    assert y.shape == r.shape
    assert rel_l2(y, r) < TOL[form], (M, P, form, rel_l2(y, r))


@pytest.mark.parametrize("L", [1, 17, 63, 65, 200])
def test_tc_channelize_filter_lengths(mx, orc, L):
    """Filters that are not a multiple of M are zero-padded to whole branches."""
    import torch
    M = 32
    rng = np.random.default_rng(L)
    x = ((rng.standard_normal((3, 4001)) + 1j * rng.standard_normal((3, 4001))) / np.sqrt(2)).astype(np.complex64)
    h = rng.standard_normal(L).astype(np.float32)
    y = mx.channelize_poly(torch.from_numpy(x).cuda(), torch.from_numpy(h).cuda(), M, M,
                           precision="bf16x3").cpu().numpy()
    r = orc.channelize_poly(x.astype(np.complex128), h.astype(np.float64), M, M)
    assert rel_l2(y, r) < 1e-6


@pytest.mark.parametrize("M,D,real", [(512, 512, False), (48, 48, False), (64, 32, False), (64, 64, True),
                                      (256, 192, False)])
def test_tc_channelize_rejects_uncovered_shapes(mx, M, D, real):
    import torch
    x = torch.randn(1, 4096, device="cuda")
    if not real:
        x = x.to(torch.complex64)
    h = torch.randn(4 * M, device="cuda")
    with pytest.raises(mx.GbfirError) as ei:
        mx.channelize_poly(x, h, M, D, precision="bf16x3")
    assert ei.value.code == 5  # GBFIR_ERR_NOT_SUPPORTED


@pytest.mark.parametrize("L", [1, 300, 4096])
def test_tc_channelize_m256_filter_lengths(mx, orc, L):
    """M = 256: filters of any length are zero-padded to whole branches (the radix path)."""
    import torch
    M = 256
    rng = np.random.default_rng(L + 5)
    x = ((rng.standard_normal((2, 9000)) + 1j * rng.standard_normal((2, 9000))) / np.sqrt(2)).astype(np.complex64)
    h = rng.standard_normal(L).astype(np.float32)
    y = mx.channelize_poly(torch.from_numpy(x).cuda(), torch.from_numpy(h).cuda(), M, M,
                           precision="bf16x3").cpu().numpy()
    assert mx._lib.load().gbfir_tc_status() == 0
    r = orc.channelize_poly(x.astype(np.complex128), h.astype(np.float64), M, M)
    assert rel_l2(y, r) < 1e-6


def test_tc_channelize_config_c3_m256(mx, orc):
    """The 4 x 2^24 c64 workload at M = 256 with a 256 x 16 Kaiser sinc prototype in bf16x3:
    sampled stretches of two rows against FP64, and linearity over the whole batch
    (channelize(a*x1 + x2) = a*channelize(x1) + channelize(x2), which a wrong row or tile
    offset anywhere would break)."""
    import torch
    M, P, B, N = 256, 16, 4, 1 << 24
    g = torch.Generator(device="cuda").manual_seed(31)
    x1 = torch.randn(B, N, dtype=torch.complex64, device="cuda", generator=g)
    x2 = torch.randn(B, N, dtype=torch.complex64, device="cuda", generator=g)
    h = torch.from_numpy(prototype(M, P).astype(np.float32)).cuda()
    y1 = mx.channelize_poly(x1, h, M, M, precision="bf16x3")
    assert mx._lib.load().gbfir_tc_status() == 0
    for row, t0 in ((1, 0), (3, 40000)):
        xs = x1[row, t0 * M:(t0 + 2048) * M].cpu().numpy().astype(np.complex128)
        pre = x1[row, max(0, t0 - P) * M:t0 * M].cpu().numpy().astype(np.complex128)
        r = orc.channelize_poly(np.concatenate([pre, xs])[None], h.cpu().numpy().astype(np.float64), M, M)[0]
        r = r[len(pre) // M:]
        assert rel_l2(y1[row, t0:t0 + 2048].cpu().numpy(), r) < 1e-6
    a = 0.75
    y2 = mx.channelize_poly(x2, h, M, M, precision="bf16x3")
    y12 = mx.channelize_poly(a * x1 + x2, h, M, M, precision="bf16x3")
    lin = float(((y12 - (a * y1 + y2)).abs().pow(2).sum() / y12.abs().pow(2).sum()).sqrt())
    assert lin < 2e-6, lin
