"""GPU parity of the hand-written adjoints (matx_gb300.autograd, gbfir_*_bwd).

Checked against: the FP64 oracle adjoint (itself pinned to MatX-built gradients
and finite differences in tests/test_oracle.py), gradients composed from MatX's
own corr / resample_poly (tests/golden/grad_refs.npz), and FP64 central finite
differences (eps = 1e-6) of the oracle loss on 64 random coordinates.
FP32 tolerance: rel-L2 1e-5 on whole gradients, 1e-4 relative per FD coordinate.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-5


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


def dev(a, dt=np.float32):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, dtype=dt)).cuda()


def test_adjoints_match_matx_built_gradients(mx):
    from matx_gb300 import autograd as ag
    z = np.load(os.path.join(GOLDEN, "grad_refs.npz"))
    x, h = dev(z["x"]), dev(z["h"])
    for mode, name in ((0, "full"), (1, "same"), (2, "valid")):
        dx, dh = ag.conv1d_bwd(dev(z[f"conv_{name}__gy"]), x, h, mode)
        assert rel_l2(dx.cpu().numpy(), z[f"conv_{name}__dx"]) < TOL
        assert rel_l2(dh.cpu().numpy(), z[f"conv_{name}__dh"]) < TOL
    for up, down in ((3, 2), (2, 3), (4, 5)):
        dx, _ = ag.resample_poly_bwd(dev(z[f"rs_{up}_{down}__gy"]), x, h, up, down, True, False)
        assert rel_l2(dx.cpu().numpy(), z[f"rs_{up}_{down}__dx"]) < TOL


@pytest.mark.parametrize("updown", [(3, 2), (2, 3), (4, 5), (1, 2), (5, 4), (160, 147), (7, 1), (1, 7), (1, 1),
                                    (6, 4), (384, 3125)])
@pytest.mark.parametrize("L", [127, 126, 15, 1, 801])
def test_resample_bwd_vs_oracle(mx, orc, updown, L):
    from matx_gb300 import autograd as ag
    up, down = updown
    rng = np.random.default_rng(up * 31 + down * 7 + L)
    B, N = 3, 3001
    x = rng.uniform(-1, 1, (B, N)).astype(np.float32)
    h = (rng.standard_normal(L) / np.sqrt(L)).astype(np.float32)
    ny = orc.resample_poly(x[:1], h, up, down).shape[1]
    gy = rng.standard_normal((B, ny)).astype(np.float32)
    dx, dh = ag.resample_poly_bwd(dev(gy), dev(x), dev(h), up, down)
    rdx, rdh = orc.resample_poly_bwd(gy, x, h, up, down)
    assert rel_l2(dx.cpu().numpy(), rdx) < TOL
    if np.linalg.norm(rdh) == 0:
        assert np.all(dh.cpu().numpy() == 0)
    else:
        assert rel_l2(dh.cpu().numpy(), rdh) < TOL


@pytest.mark.parametrize("mode", [0, 1, 2])
@pytest.mark.parametrize("NL", [(5000, 127), (4096, 64), (300, 300), (1000, 1), (17, 40), (20000, 1500)])
def test_conv_bwd_vs_oracle(mx, orc, mode, NL):
    from matx_gb300 import autograd as ag
    N, L = NL
    rng = np.random.default_rng(N + L + mode)
    B = 3
    x = rng.uniform(-1, 1, (B, N)).astype(np.float32)
    h = (rng.standard_normal(L) / np.sqrt(L)).astype(np.float32)
    ny = orc.conv1d(x[:1], h, mode).shape[1]
    gy = rng.standard_normal((B, ny)).astype(np.float32)
    dx, dh = ag.conv1d_bwd(dev(gy), dev(x), dev(h), mode)
    rdx, rdh = orc.conv1d_bwd(gy, x, h, mode)
    assert rel_l2(dx.cpu().numpy(), rdx) < TOL
    assert rel_l2(dh.cpu().numpy(), rdh) < TOL


def test_dh_is_deterministic(mx):
    import torch
    from matx_gb300 import autograd as ag
    g = torch.Generator(device="cuda").manual_seed(3)
    x = torch.rand(64, 50000, device="cuda", generator=g) * 2 - 1
    h = torch.randn(127, device="cuda", generator=g)
    gy = torch.randn(64, 75000, device="cuda", generator=g)
    _, a = ag.resample_poly_bwd(gy, x, h, 3, 2, False, True)
    _, b = ag.resample_poly_bwd(gy, x, h, 3, 2, False, True)
    assert torch.equal(a, b)


def _kaiser(up, down, L=127):
    from scipy import signal
    m = max(up, down)
    return signal.firwin(L, 1.0 / m, window=("kaiser", 5.0))


@pytest.mark.parametrize("form", ["resample_3_2", "conv_same"])
def test_c4_autograd_vs_fd(mx, orc, form):
    """C4: 256 x 16384 uniform[-1,1], learnable 127-tap filter ~ N(0, 1/127), target from
    a fixed seeded Kaiser filter, MSE loss; autograd gradients vs FP64 central finite
    differences (eps = 1e-6) on 64 random coordinates and vs the exact FP64 adjoint."""
    import torch
    from matx_gb300 import autograd as ag
    rng = np.random.default_rng(4096)
    B, N, L = 256, 16384, 127
    x64 = rng.uniform(-1, 1, (B, N))
    h64 = rng.standard_normal(L) / np.sqrt(L)
    hk = _kaiser(3, 2)
    if form == "resample_3_2":
        fwd64 = lambda xx, hh: orc.resample_poly(xx, hh, 3, 2, nthreads=8)
    else:
        fwd64 = lambda xx, hh: orc.conv1d(xx, hh, 1, nthreads=8)
    target = fwd64(x64, hk)
    x = dev(x64).requires_grad_(True)
    h = dev(h64).requires_grad_(True)
    y = ag.resample_poly(x, h, 3, 2) if form == "resample_3_2" else ag.conv1d(x, h, 1)
    loss = torch.mean((y - dev(target)) ** 2)
    loss.backward()
    gx, gh = x.grad.cpu().numpy().astype(np.float64), h.grad.cpu().numpy().astype(np.float64)

    # exact FP64 adjoint of the MSE loss
    y64 = fwd64(x64, h64)
    gy64 = 2.0 * (y64 - target) / y64.size
    if form == "resample_3_2":
        rdx, rdh = orc.resample_poly_bwd(gy64, x64, h64, 3, 2, nthreads=8)
    else:
        rdx, rdh = orc.conv1d_bwd(gy64, x64, h64, 1, nthreads=8)
    assert rel_l2(gh, rdh) < TOL
    assert rel_l2(gx, rdx) < TOL

    # FP64 central differences on 64 coordinates: 16 filter taps (whole batch) and
    # 48 signal samples (their own row; rows are independent)
    eps = 1e-6
    def loss_rows(xx, hh, rows):
        yy = fwd64(xx, hh)
        return float(np.sum((yy - target[rows]) ** 2) / y64.size)
    for k in rng.choice(L, 16, replace=False):
        hp, hm = h64.copy(), h64.copy()
        hp[k] += eps
        hm[k] -= eps
        fd = (loss_rows(x64, hp, slice(None)) - loss_rows(x64, hm, slice(None))) / (2 * eps)
        assert abs(gh[k] - fd) <= 1e-4 * abs(fd) + 1e-9, (k, gh[k], fd)
    for _ in range(48):
        b, i = int(rng.integers(B)), int(rng.integers(N))
        xp, xm = x64[b:b + 1].copy(), x64[b:b + 1].copy()
        xp[0, i] += eps
        xm[0, i] -= eps
        fd = (loss_rows(xp, h64, slice(b, b + 1)) - loss_rows(xm, h64, slice(b, b + 1))) / (2 * eps)
        assert abs(gx[b, i] - fd) <= 1e-4 * abs(fd) + 1e-9, (b, i, gx[b, i], fd)
