"""Tensor-core forms of conv1d / corr (tcgen05 Toeplitz MMAs, up = down = 1) against the
FP64 oracle.  Stated error bars (rel-L2 vs FP64): bf16 <= 1e-2, fp16 <= 2e-3, bf16x3 <=
1e-6.  The forms take a real float32 filter row shared by every signal row and a signal
at least as long as the filter; other operands are rejected with GBFIR_ERR_NOT_SUPPORTED."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu
TOL = {"bf16": 1e-2, "fp16": 2e-3, "bf16x3": 1e-6}
MODES = {"full": 0, "same": 1, "valid": 2}


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


@pytest.mark.parametrize("L", [63, 64, 1, 2, 127, 301])
@pytest.mark.parametrize("mode", ["full", "same", "valid"])
@pytest.mark.parametrize("form", ["bf16x3", "bf16", "fp16"])
@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("is_corr", [False, True])
def test_tc_conv_vs_fp64(mx, orc, L, mode, form, cplx, is_corr):
    import torch
    rng = np.random.default_rng(L * 7 + MODES[mode] + 3 * cplx + 11 * is_corr)
    B, N = 3, 20011
    x = rng.uniform(-1, 1, (B, N))
    if cplx:
        x = x + 1j * rng.uniform(-1, 1, (B, N))
    h = rng.standard_normal(L) / np.sqrt(L)
    xd = torch.from_numpy(x.astype(np.complex64 if cplx else np.float32)).cuda()
    hd = torch.from_numpy(h.astype(np.float32)).cuda()
    fn = mx.corr if is_corr else mx.conv1d
    y = fn(xd, hd, mode, precision=form).cpu().numpy()
    assert mx._lib.load().gbfir_tc_status() == 0
    r = orc.conv1d(xd.cpu().numpy().astype(np.complex128 if cplx else np.float64),
                   hd.cpu().numpy().astype(np.float64), MODES[mode], is_corr=is_corr)
    assert y.shape == r.shape
    assert rel_l2(y, r) < TOL[form], (L, mode, form, rel_l2(y, r))


def test_tc_conv_config_c1(mx, orc):
    """The 8 x 2^20 real FULL workload with a 63-tap Hamming sinc: sampled rows vs FP64."""
    import torch
    from scipy import signal
    rng = np.random.default_rng(21)
    x = rng.uniform(-1, 1, (8, 1 << 20)).astype(np.float32)
    h = signal.firwin(63, 0.25, window="hamming").astype(np.float32)
    y = mx.conv1d(torch.from_numpy(x).cuda(), torch.from_numpy(h).cuda(), "full", precision="bf16x3")
    for row in (0, 7):
        r = orc.conv1d(x[row:row + 1].astype(np.float64), h.astype(np.float64), 0)
        assert rel_l2(y[row:row + 1].cpu().numpy(), r) < 1e-6


def test_tc_conv_rejects_uncovered_operands(mx):
    import torch
    x = torch.randn(2, 4096, device="cuda")
    with pytest.raises(mx.GbfirError) as ei:   # filter longer than the signal (operand swap)
        mx.conv1d(torch.randn(2, 50, device="cuda"), torch.randn(80, device="cuda"), precision="bf16x3")
    assert ei.value.code == 5
    with pytest.raises(mx.GbfirError) as ei:   # one filter per row
        mx.conv1d(x, torch.randn(2, 31, device="cuda"), precision="bf16")
    assert ei.value.code == 5
    with pytest.raises(mx.GbfirError) as ei:   # complex taps
        mx.conv1d(x, torch.randn(31, dtype=torch.complex64, device="cuda"), precision="bf16x3")
    assert ei.value.code == 5
