"""Tensor-core forms of channelize_poly (tcgen05 DFT GEMM over the polyphase FIR
outputs) against the FP64 oracle.  Stated error bars (rel-L2 vs FP64): bf16 <= 1e-2,
fp16 <= 2e-3, bf16x3 <= 1e-6.  The forms cover the maximally decimated channelizer
(D == M) with M in {16, 32, 64}; anything else is rejected with
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


@pytest.mark.parametrize("M,P", [(64, 32), (64, 8), (32, 16), (32, 3), (16, 8), (16, 1)])
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


@pytest.mark.parametrize("M,D,real", [(128, 128, False), (48, 48, False), (64, 32, False), (64, 64, True)])
def test_tc_channelize_rejects_uncovered_shapes(mx, M, D, real):
    import torch
    x = torch.randn(1, 4096, device="cuda")
    if not real:
        x = x.to(torch.complex64)
    h = torch.randn(4 * M, device="cuda")
    with pytest.raises(mx.GbfirError) as ei:
        mx.channelize_poly(x, h, M, D, precision="bf16x3")
    assert ei.value.code == 5  # GBFIR_ERR_NOT_SUPPORTED
