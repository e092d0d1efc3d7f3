"""Tensor-core forms of resample_poly (tcgen05 Toeplitz MMAs) against the FP64
oracle.  Stated error bars (rel-L2 vs FP64): bf16 <= 1e-2, fp16 <= 2e-3,
bf16x3 <= 1e-6.  Rates whose rows alias an 8- or 64-sample operand pitch run the
Hankel kernels; the others (160/147, 40/3, 7/19, and decimators whose Hankel slab does
not fit shared memory, 1/17 with a 341-tap filter) the column-blocked kernel over
materialised rows, in K chunks.  Double-precision signals and complex taps are rejected
with GBFIR_ERR_NOT_SUPPORTED."""
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


def kaiser(up, down):
    from scipy import signal
    m = max(up, down)
    return signal.firwin(2 * 10 * m + 1, 1.0 / m, window=("kaiser", 5.0))


@pytest.mark.parametrize("updown", [(3, 2), (4, 5), (1, 2), (2, 3), (3, 4), (5, 4), (2, 1), (7, 1), (1, 7),
                                    (6, 4), (3, 8), (5, 3), (160, 147), (40, 3), (7, 19), (1, 17)])
@pytest.mark.parametrize("form", ["bf16x3", "bf16", "fp16"])
@pytest.mark.parametrize("cplx", [True, False])
def test_tc_resample_vs_fp64(mx, orc, updown, form, cplx):
    import torch
    up, down = updown
    rng = np.random.default_rng(up * 13 + down)
    B, N = 3, 20011
    x = rng.standard_normal((B, N))
    if cplx:
        x = (x + 1j * rng.standard_normal((B, N))) / np.sqrt(2)
    h = kaiser(up, down)
    xd = torch.from_numpy(x.astype(np.complex64 if cplx else np.float32)).cuda()
    hd = torch.from_numpy(h.astype(np.float32)).cuda()
    y = mx.resample_poly(xd, hd, up, down, precision=form).cpu().numpy()
    assert mx._lib.load().gbfir_tc_status() == 0
    r = orc.resample_poly(xd.cpu().numpy().astype(np.complex128 if cplx else np.float64),
                          hd.cpu().numpy().astype(np.float64), up, down)
    assert y.shape == r.shape
    assert rel_l2(y, r) < TOL[form], (updown, form, rel_l2(y, r))


@pytest.mark.parametrize("L", [30, 31, 2, 1, 301, 401, 801])
def test_tc_resample_filter_lengths(mx, orc, L):
    import torch
    rng = np.random.default_rng(L)
    x = ((rng.standard_normal((2, 5000)) + 1j * rng.standard_normal((2, 5000))) / np.sqrt(2)).astype(np.complex64)
    h = rng.standard_normal(L).astype(np.float32)
    for up, down in ((3, 2), (4, 5)):
        y = mx.resample_poly(torch.from_numpy(x).cuda(), torch.from_numpy(h).cuda(), up, down,
                             precision="bf16x3").cpu().numpy()
        r = orc.resample_poly(x.astype(np.complex128), h.astype(np.float64), up, down)
        assert rel_l2(y, r) < 1e-6


def test_tc_config_rows(mx, orc):
    """The 64 x 2^20 c64 workload at its three rates in bf16x3: sampled rows against FP64,
    and linearity over the whole batch (resample(a*x1 + x2) = a*resample(x1) +
    resample(x2)), which a wrong row, tile or column-block offset anywhere would break."""
    import torch
    g = torch.Generator(device="cuda").manual_seed(7)
    x = torch.randn(64, 1 << 20, dtype=torch.complex64, device="cuda", generator=g)
    x2 = torch.randn(64, 1 << 20, dtype=torch.complex64, device="cuda", generator=g)
    a = 0.625
    for up, down in ((3, 2), (4, 5), (160, 147)):
        h = torch.from_numpy(kaiser(up, down).astype(np.float32)).cuda()
        y = mx.resample_poly(x, h, up, down, precision="bf16x3")
        assert mx._lib.load().gbfir_tc_status() == 0
        rows = [0, 33, 63]
        r = orc.resample_poly(x[rows].cpu().numpy().astype(np.complex128), h.cpu().numpy().astype(np.float64),
                              up, down, nthreads=3)
        assert rel_l2(y[rows].cpu().numpy(), r) < 1e-6
        y2 = mx.resample_poly(x2, h, up, down, precision="bf16x3")
        y12 = mx.resample_poly(a * x + x2, h, up, down, precision="bf16x3")
        lin = float(((y12 - (a * y + y2)).abs().pow(2).sum() / y12.abs().pow(2).sum()).sqrt())
        assert lin < 2e-6, (up, down, lin)
        del y, y2, y12


def test_tc_unsupported_operands_are_rejected(mx):
    import torch
    x = torch.zeros(1, 1000, dtype=torch.complex64, device="cuda")
    with pytest.raises(mx.GbfirError) as e:   # complex taps
        mx.resample_poly(x, torch.ones(31, dtype=torch.complex64, device="cuda"), 3, 2, precision="bf16x3")
    assert e.value.code == 5
    with pytest.raises(mx.GbfirError) as e:   # double-precision signal
        mx.resample_poly(x.to(torch.complex128), torch.ones(31, dtype=torch.float64, device="cuda"), 3, 2,
                         precision="bf16")
    assert e.value.code == 5
