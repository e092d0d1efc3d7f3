"""upsample / downsample (bit-exact against numpy indexing) and upfirdn =
downsample(conv1d(upsample(x, up), h, mode), down) against the FP64 oracle applied to the
literal composition (zero-stuffed signal, oracle conv1d, strided slice)."""
import numpy as np
import pytest

from conftest import seed_of

pytestmark = pytest.mark.gpu
FP32_TOL = 1e-5


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


def _rand(rng, shape, cplx, dt=np.float32):
    a = rng.uniform(-1, 1, shape)
    if cplx:
        a = a + 1j * rng.uniform(-1, 1, shape)
        return a.astype(np.complex64 if dt == np.float32 else np.complex128)
    return a.astype(dt)


@pytest.mark.parametrize("n", [1, 2, 3, 7])
@pytest.mark.parametrize("dt", [np.float32, np.complex64, np.float64, np.complex128])
def test_upsample_downsample_exact(mx, n, dt):
    import torch
    rng = np.random.default_rng(seed_of("updown", n, str(dt)))
    x = rng.standard_normal((3, 4, 1001)).astype(dt)
    xd = torch.from_numpy(x).cuda()
    up = mx.upsample(xd, n).cpu().numpy()
    ref = np.zeros((3, 4, 1001 * n), dt)
    ref[..., ::n] = x
    assert np.array_equal(up, ref)
    assert np.array_equal(mx.downsample(xd, n).cpu().numpy(), x[..., ::n])
    # another dimension
    assert np.array_equal(mx.downsample(xd, n, dim=1).cpu().numpy(), x[:, ::n])
    ref1 = np.zeros((3 * n, 4, 1001), dt)
    ref1[::n] = x
    assert np.array_equal(mx.upsample(xd, n, dim=0).cpu().numpy(), ref1)


def _oracle_upfirdn(orc, x, h, up, down, mode):
    u = np.zeros(x.shape[:-1] + (x.shape[-1] * up,), x.dtype)
    u[..., ::up] = x
    r = orc.conv1d(np.ascontiguousarray(u.reshape(-1, u.shape[-1])), h, mode)
    return r[:, ::down].reshape(x.shape[:-1] + (-1,))


@pytest.mark.parametrize("updown", [(1, 1), (2, 1), (1, 3), (3, 2), (4, 5), (2, 4), (3, 3), (7, 1), (1, 8)])
@pytest.mark.parametrize("L", [5, 24, 63])
@pytest.mark.parametrize("mode", [0, 1, 2])
def test_upfirdn_vs_composition(mx, orc, updown, L, mode):
    import torch
    up, down = updown
    rng = np.random.default_rng(seed_of("upfirdn", up, down, L, mode))
    for xc, hc in ((True, False), (False, False), (True, True)):
        x = _rand(rng, (3, 2000), xc)
        h = _rand(rng, (L,), hc)
        y = mx.upfirdn(torch.from_numpy(x).cuda(), torch.from_numpy(h).cuda(), up, down, mode).cpu().numpy()
        r = _oracle_upfirdn(orc, x, h, up, down, mode)
        assert y.shape == r.shape, (y.shape, r.shape)
        scale = np.linalg.norm(_oracle_upfirdn(orc, np.abs(x), np.abs(h), up, down, mode))
        err = np.linalg.norm(y - r) / max(np.linalg.norm(r), 0.1 * scale)
        assert err < FP32_TOL, (xc, hc, err)


def test_upfirdn_short_signal_and_double(mx, orc):
    import torch
    rng = np.random.default_rng(8)
    for mode in (0, 1, 2):
        # upsampled signal shorter than the filter (MatX swaps the conv operands)
        x = _rand(rng, (2, 5), True)
        h = _rand(rng, (40,), False)
        y = mx.upfirdn(torch.from_numpy(x).cuda(), torch.from_numpy(h).cuda(), 3, 2, mode).cpu().numpy()
        r = _oracle_upfirdn(orc, x, h, 3, 2, mode)
        assert y.shape == r.shape and np.linalg.norm(y - r) <= 1e-5 * np.linalg.norm(r) + 1e-6, mode
    x = _rand(rng, (4, 3001), True, np.float64)
    h = _rand(rng, (31,), False, np.float64)
    y = mx.upfirdn(torch.from_numpy(x).cuda(), torch.from_numpy(h).cuda(), 5, 3, "same").cpu().numpy()
    r = _oracle_upfirdn(orc, x, h, 5, 3, 1)
    assert np.linalg.norm(y - r) / np.linalg.norm(r) < 1e-13


def test_updown_validation(mx):
    import torch
    x = torch.zeros(10, device="cuda")
    with pytest.raises(mx.GbfirError):
        mx.upsample(x, 0)
    with pytest.raises(mx.GbfirError):
        mx.upfirdn(x, torch.zeros(3, device="cuda"), 0, 1)
