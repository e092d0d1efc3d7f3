"""conv1d / corr along a strided axis (gbfir_conv1d_axis) against the FP64 oracle run on
the transposed rows, bit-equality with the row kernel on the same transposed data (same
tap order and madd), and the radar three-pulse canceller's permuted view
(examples/simple_radar_pipeline.h:321-327)."""
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


def _oracle_axis(orc, x, h, mode, corr, axis):
    """FP64 oracle on rows: move `axis` last, convolve each row, move it back."""
    xr = np.moveaxis(x, axis, -1)
    shp = xr.shape
    r = orc.conv1d(np.ascontiguousarray(xr.reshape(-1, shp[-1])), h, mode, corr)
    return np.moveaxis(r.reshape(shp[:-1] + (r.shape[-1],)), -1, axis)


def _err(orc, y, x, h, mode, corr, axis):
    r = _oracle_axis(orc, x, h, mode, corr, axis)
    scale = np.linalg.norm(_oracle_axis(orc, np.abs(x), np.abs(h), mode, corr, axis))
    return np.linalg.norm(y - r) / max(np.linalg.norm(r), 0.1 * scale)


@pytest.mark.parametrize("shape,axis", [((3, 200, 77), 1), ((500, 300), 0), ((2, 5, 64, 33), 2),
                                        ((4, 37, 1000), 1)])
@pytest.mark.parametrize("L", [3, 6, 13, 40])
@pytest.mark.parametrize("mode", [0, 1, 2])
def test_axis_vs_oracle_and_row_kernel(mx, orc, shape, axis, L, mode):
    import torch
    rng = np.random.default_rng(seed_of("axis", shape, axis, L, mode))
    for xc, hc, corr in ((True, False, False), (False, False, True), (True, True, False), (True, True, True)):
        x = _rand(rng, shape, xc)
        h = _rand(rng, (L,), hc)
        y = mx.conv1d(torch.from_numpy(x).cuda(), torch.from_numpy(h).cuda(), mode, axis=axis, _corr=corr)
        assert _err(orc, y.cpu().numpy(), x, h, mode, corr, axis) < FP32_TOL, (xc, hc, corr)
        if shape[axis] >= L:
            # the row kernel on the moved-axis copy: same taps in the same order
            xr = torch.from_numpy(np.ascontiguousarray(np.moveaxis(x, axis, -1))).cuda()
            yr = mx.conv1d(xr, torch.from_numpy(h).cuda(), mode, _corr=corr)
            assert torch.equal(torch.movedim(yr, -1, axis), y), (xc, hc, corr)


def test_axis_double_precision(mx, orc):
    import torch
    rng = np.random.default_rng(3)
    x = _rand(rng, (6, 129, 50), True, np.float64)
    h = _rand(rng, (7,), False, np.float64)
    y = mx.conv1d(torch.from_numpy(x).cuda(), torch.from_numpy(h).cuda(), 1, axis=1)
    r = _oracle_axis(orc, x, h, 1, False, 1)
    assert np.linalg.norm(y.cpu().numpy() - r) / np.linalg.norm(r) < 1e-13


def test_axis_signal_shorter_than_filter(mx, orc):
    # MatX swaps the operands when the signal is the shorter one (conv.h:427); the full
    # convolution is the same, SAME/VALID start from the shorter length
    import torch
    rng = np.random.default_rng(4)
    for mode in (0, 1, 2):
        x = _rand(rng, (3, 9, 40), True)
        h = _rand(rng, (14,), False)
        y = mx.conv1d(torch.from_numpy(x).cuda(), torch.from_numpy(h).cuda(), mode, axis=1)
        assert _err(orc, y.cpu().numpy(), x, h, mode, False, 1) < FP32_TOL, mode


def test_three_pulse_canceller_view(mx, orc):
    """conv1d SAME of [1, -2, 1] over the pulses of a [channel][pulse][sample] cube whose
    rows are padded (the compressed samples are a slice), taken as the permuted
    [channel][sample][pulse] view: no copy, and the output is the same kind of view."""
    import torch
    rng = np.random.default_rng(5)
    C, P, S, SR = 4, 128, 2001, 2048
    cube = _rand(rng, (C, P, SR), True)
    mask = np.array([1, -2, 1], np.complex64)
    xv = torch.from_numpy(cube).cuda()[:, :, :S].permute(0, 2, 1)
    full = torch.zeros(C, P, SR, dtype=torch.complex64, device="cuda")
    out = full[:, :, :S].permute(0, 2, 1)
    y = mx.conv1d(xv, torch.from_numpy(mask).cuda(), "same", out=out)
    assert y.data_ptr() == out.data_ptr() and y.shape == (C, S, P)
    ref_in = np.ascontiguousarray(np.transpose(cube[:, :, :S], (0, 2, 1)).reshape(-1, P))
    r = orc.conv1d(ref_in, mask, 1)
    got = y.cpu().numpy().reshape(-1, P)
    assert np.linalg.norm(got - r) / np.linalg.norm(r) < FP32_TOL
    # the padding columns of the output cube are untouched
    assert torch.count_nonzero(full[:, :, S:]) == 0
    # without out= the result is a fresh tensor in the input's dimension order
    y2 = mx.conv1d(xv, torch.from_numpy(mask).cuda(), "same")
    assert y2.stride(-1) != 1 and torch.equal(y2, y)
