"""Tensor-core dL/dx and dL/dh of resample_poly (gbfir_resample_poly_bwd_prec) against the
FP64 oracle adjoint.  Stated error bars (rel-L2 vs FP64), for dx and dh alike: bf16 <= 1e-2,
fp16 <= 2e-3, bf16x3 <= 1e-6.  dh is reduced on the tensor cores (FP32 in TMEM per CTA, FP64
across CTAs) and is deterministic: two calls give identical bits."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu
TOL = {"bf16": 1e-2, "fp16": 2e-3, "bf16x3": 1e-6}


@pytest.fixture(scope="module")
def ag():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from matx_gb300 import autograd, build
    build.build()
    return autograd


@pytest.fixture(scope="module")
def orc():
    import oracle
    oracle.build()
    return oracle


@pytest.mark.parametrize("updown", [(3, 2), (4, 5), (1, 2), (2, 1), (5, 4), (1, 4)])
@pytest.mark.parametrize("form", ["bf16x3", "bf16", "fp16"])
def test_tc_dx_vs_fp64(ag, orc, updown, form):
    import torch
    up, down = updown
    rng = np.random.default_rng(up * 31 + down)
    B, N, L = 4, 12007, 127
    x = rng.uniform(-1, 1, (B, N)).astype(np.float32)
    h = (rng.standard_normal(L) / np.sqrt(L)).astype(np.float32)
    ny = (N * up + down - 1) // down
    gy = rng.standard_normal((B, ny)).astype(np.float32)
    dev = lambda a: torch.from_numpy(a).cuda()
    dx, dh = ag.resample_poly_bwd(dev(gy), dev(x), dev(h), up, down, precision=form)
    _, dh2 = ag.resample_poly_bwd(dev(gy), dev(x), dev(h), up, down, False, True, precision=form)
    _, dh32 = ag.resample_poly_bwd(dev(gy), dev(x), dev(h), up, down, False, True)
    torch.cuda.synchronize()
    rdx, rdh = orc.resample_poly_bwd(gy.astype(np.float64), x.astype(np.float64), h.astype(np.float64), up, down)
    assert rel_l2(dx.cpu().numpy(), rdx) < TOL[form], (updown, form, rel_l2(dx.cpu().numpy(), rdx))
    e = rel_l2(dh.cpu().numpy(), rdh)
    assert e < TOL[form], (updown, form, e)
    assert torch.equal(dh, dh2)
    assert rel_l2(dh32.cpu().numpy(), rdh) < 1e-5
    if form != "bf16x3":
        # single-term operands round every product: the tensor-core reduction ran, not the FP32 one
        assert e > 1e-5, (updown, form, e)


@pytest.mark.parametrize("updown,L", [((3, 2), 127), ((3, 2), 128), ((4, 5), 101), ((1, 4), 61), ((2, 3), 30),
                                      ((7, 3), 255), ((5, 1), 9), ((160, 147), 3201)])
def test_tc_dh_rates_and_edges(ag, orc, updown, L):
    """dh in bf16x3 across rates, even filters, short signals and a rate whose row tile does not
    fit the tensor-core kernel (160/147 with 3201 taps: the FP32 reduction answers instead)."""
    import torch
    up, down = updown
    rng = np.random.default_rng(up * 7 + down + L)
    for B, N in ((3, 5003), (1, 37), (2, 1)):
        x = rng.uniform(-1, 1, (B, N)).astype(np.float32)
        h = (rng.standard_normal(L) / np.sqrt(L)).astype(np.float32)
        ny = (N * up + down - 1) // down
        gy = rng.standard_normal((B, ny)).astype(np.float32)
        dev = lambda a: torch.from_numpy(a).cuda()
        _, dh = ag.resample_poly_bwd(dev(gy), dev(x), dev(h), up, down, False, True, precision="bf16x3")
        torch.cuda.synchronize()
        _, rdh = orc.resample_poly_bwd(gy.astype(np.float64), x.astype(np.float64), h.astype(np.float64), up, down)
        e = rel_l2(dh.cpu().numpy(), rdh)
        assert e < 1e-6, (updown, L, B, N, e)


def test_tc_fwd_bwd_autograd_bf16x3(ag, orc):
    """The differentiable config (256 x 16384, 127 taps, 3/2) end to end in bf16x3."""
    import torch
    g = torch.Generator(device="cuda").manual_seed(5)
    x = (torch.rand(256, 16384, device="cuda", generator=g) * 2 - 1).requires_grad_(True)
    h = (torch.randn(127, device="cuda", generator=g) / 127 ** 0.5).requires_grad_(True)
    y = ag.resample_poly(x, h, 3, 2, precision="bf16x3")
    gy = torch.randn(y.shape, device="cuda", generator=g)
    y.backward(gy)
    xs, hs, gs = (t.detach().cpu().numpy().astype(np.float64) for t in (x, h, gy))
    rows = slice(0, 8)
    rdx, _ = orc.resample_poly_bwd(gs[rows], xs[rows], hs, 3, 2)
    assert rel_l2(x.grad[rows].cpu().numpy(), rdx) < 1e-6
    _, rdh = orc.resample_poly_bwd(gs, xs, hs, 3, 2, nthreads=8)
    assert rel_l2(h.grad.cpu().numpy(), rdh) < 1e-6
    ry = orc.resample_poly(xs[rows], hs, 3, 2)
    assert rel_l2(y[rows].detach().cpu().numpy(), ry) < 1e-6


@pytest.mark.parametrize("mode", [0, 1, 2])
@pytest.mark.parametrize("form", ["bf16x3", "bf16", "fp16"])
def test_tc_conv_bwd_vs_fp64(ag, orc, mode, form):
    """conv1d's dL/dx and dL/dh on the tensor cores (gbfir_conv1d_bwd_prec), FULL / SAME / VALID."""
    import torch
    rng = np.random.default_rng(17 + mode)
    B, N, L = 3, 9001, 127
    x = rng.uniform(-1, 1, (B, N)).astype(np.float32)
    h = (rng.standard_normal(L) / np.sqrt(L)).astype(np.float32)
    olen = {0: N + L - 1, 1: N, 2: N - L + 1}[mode]
    gy = rng.standard_normal((B, olen)).astype(np.float32)
    dev = lambda a: torch.from_numpy(a).cuda()
    dx, dh = ag.conv1d_bwd(dev(gy), dev(x), dev(h), mode, precision=form)
    _, dh2 = ag.conv1d_bwd(dev(gy), dev(x), dev(h), mode, False, True, precision=form)
    torch.cuda.synchronize()
    rdx, rdh = orc.conv1d_bwd(gy.astype(np.float64), x.astype(np.float64), h.astype(np.float64), mode)
    ex, eh = rel_l2(dx.cpu().numpy(), rdx), rel_l2(dh.cpu().numpy(), rdh)
    assert ex < TOL[form] and eh < TOL[form], (mode, form, ex, eh)
    assert torch.equal(dh, dh2)
    if form != "bf16x3":
        assert ex > 1e-5 and eh > 1e-5, (mode, form, ex, eh)


def test_tc_conv_fwd_bwd_autograd_bf16x3(ag, orc):
    """The differentiable conv1d SAME case (256 x 16384, 127 taps) end to end in bf16x3."""
    import torch
    g = torch.Generator(device="cuda").manual_seed(9)
    x = (torch.rand(256, 16384, device="cuda", generator=g) * 2 - 1).requires_grad_(True)
    h = (torch.randn(127, device="cuda", generator=g) / 127 ** 0.5).requires_grad_(True)
    y = ag.conv1d(x, h, "same", precision="bf16x3")
    gy = torch.randn(y.shape, device="cuda", generator=g)
    y.backward(gy)
    xs, hs, gs = (t.detach().cpu().numpy().astype(np.float64) for t in (x, h, gy))
    rows = slice(0, 8)
    rdx, _ = orc.conv1d_bwd(gs[rows], xs[rows], hs, 1)
    assert rel_l2(x.grad[rows].cpu().numpy(), rdx) < 1e-6
    _, rdh = orc.conv1d_bwd(gs, xs, hs, 1, nthreads=8)
    assert rel_l2(h.grad.cpu().numpy(), rdh) < 1e-6
