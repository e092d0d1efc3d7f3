"""FFT-method conv1d / corr (gbfir_conv1d_fft, MatX MATX_C_METHOD_FFT) against the FP64
oracle's direct convolution (the same outputs up to FP32 rounding) and the direct method
on the GPU, across transform lengths 1024..8192, all modes and operand kinds."""
import numpy as np
import pytest

from conftest import seed_of

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


def _rand(rng, shape, cplx):
    a = rng.uniform(-1, 1, shape)
    if cplx:
        return (a + 1j * rng.uniform(-1, 1, shape)).astype(np.complex64)
    return a.astype(np.float32)


def _err(orc, y, x, h, mode, corr):
    r = orc.conv1d(x, h, mode, corr)
    scale = np.linalg.norm(orc.conv1d(np.abs(x), np.abs(h), mode, corr))
    return np.linalg.norm(y - r) / max(np.linalg.norm(r), 0.1 * scale)


@pytest.mark.parametrize("L,N", [(1, 3000), (2, 3000), (63, 5000), (500, 20000), (1000, 1000), (1025, 9000),
                                 (2049, 40000), (4096, 30000), (7169, 20000)])
@pytest.mark.parametrize("mode", [0, 1, 2])
def test_fft_conv_vs_oracle(mx, orc, L, N, mode):
    import torch
    rng = np.random.default_rng(seed_of("fftconv", L, N, mode))
    for xc, hc, corr in ((True, False, False), (True, True, True), (False, False, False), (False, True, False)):
        x = _rand(rng, (2, N), xc)
        h = _rand(rng, (L,), hc)
        xd, hd = torch.from_numpy(x).cuda(), torch.from_numpy(h).cuda()
        y = mx.conv1d(xd, hd, mode, method="fft", _corr=corr)
        assert y.shape[-1] == orc.conv1d(x[:1], h, mode, corr).shape[-1]
        assert y.is_complex() == (xc or hc)
        assert _err(orc, y.cpu().numpy(), x, h, mode, corr) < TOL, (xc, hc, corr)
        if L <= 1024:
            yd = mx.conv1d(xd, hd, mode, _corr=corr)
            assert np.linalg.norm((y - yd).cpu().numpy()) <= TOL * max(np.linalg.norm(yd.cpu().numpy()), 1e-3)


def test_fft_conv_batch_broadcast_and_limits(mx, orc):
    import torch
    rng = np.random.default_rng(2)
    x = _rand(rng, (7, 12345), True)
    h = _rand(rng, (300,), False)
    y = mx.conv1d(torch.from_numpy(x).cuda(), torch.from_numpy(h).cuda(), "same", method="fft")
    assert _err(orc, y.cpu().numpy(), x, h, 1, False) < TOL
    with pytest.raises(mx.GbfirError):  # longer than the largest transform allows
        mx.conv1d(torch.zeros(2, 20000, dtype=torch.complex64, device="cuda"),
                  torch.zeros(7170, device="cuda"), method="fft")
    with pytest.raises(mx.GbfirError):  # signal shorter than the filter
        mx.conv1d(torch.zeros(2, 100, dtype=torch.complex64, device="cuda"), torch.zeros(200, device="cuda"),
                  method="fft")
    with pytest.raises(mx.GbfirError):  # double precision
        mx.conv1d(torch.zeros(2, 100, dtype=torch.complex128, device="cuda"),
                  torch.zeros(20, dtype=torch.float64, device="cuda"), method="fft")
