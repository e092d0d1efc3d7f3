"""Direct conv2d (gbfir_conv2d, MatX conv2d) against the reference's scipy-generated
vectors (ConvCorr.cu conv2d cases, tests/golden/conv2d.npz), its hand-computed case and the
FP64 oracle restating MatX's host loop."""
import numpy as np
import pytest

from conftest import load_cases, rel_l2, seed_of

pytestmark = pytest.mark.gpu


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


@pytest.mark.parametrize("case", sorted(load_cases("conv2d.npz")))
def test_conv2d_reference_vectors(mx, case):
    c = load_cases("conv2d.npz")[case]
    a, b = c["a_op"], c["b_op"]
    tol = 1e-12 if a.dtype == np.float64 else 1e-5
    for mode, key in ((0, "conv_full"), (1, "conv_same"), (2, "conv_valid")):
        y = mx.conv2d(dev(a), dev(b), mode).cpu().numpy()
        assert y.shape == c[key].shape and rel_l2(y, c[key]) < tol, (case, mode)
        ys = mx.conv2d(dev(b), dev(a), mode).cpu().numpy()  # swapped operands (ConvCorr.cu:783-787)
        assert rel_l2(ys, c[key]) < tol, (case, mode)


def test_conv2d_known_answer(mx):
    x = np.arange(1, 10, dtype=np.float32).reshape(3, 3)
    h = np.array([[1, 2], [3, 4]], np.float32)
    full = np.array([[1, 4, 7, 6], [7, 23, 33, 24], [19, 53, 63, 42], [21, 52, 59, 36]], np.float32)
    assert np.array_equal(mx.conv2d(dev(x), dev(h), "full").cpu().numpy(), full)
    assert np.array_equal(mx.conv2d(dev(x), dev(h), "same").cpu().numpy(), full[:3, :3])
    assert np.array_equal(mx.conv2d(dev(x), dev(h), "valid").cpu().numpy(), full[1:3, 1:3])


@pytest.mark.parametrize("img,filt", [((3, 70, 45), (5, 3)), ((2, 129, 200), (16, 8)), ((1, 64, 32), (64, 32)),
                                      ((4, 33, 97), (1, 1)), ((2, 300, 300), (64, 64)), ((2, 40, 50), (2, 40, 50))])
@pytest.mark.parametrize("mode", [0, 1, 2])
def test_conv2d_vs_oracle(mx, orc, img, filt, mode):
    rng = np.random.default_rng(seed_of("conv2d", img, filt, mode))
    for xc, hc in ((False, False), (True, False), (True, True), (False, True)):
        x = rng.uniform(-1, 1, img) + (1j * rng.uniform(-1, 1, img) if xc else 0)
        h = rng.uniform(-1, 1, filt) + (1j * rng.uniform(-1, 1, filt) if hc else 0)
        x = x.astype(np.complex64 if xc else np.float32)
        h = h.astype(np.complex64 if hc else np.float32)
        y = mx.conv2d(dev(x), dev(h), mode).cpu().numpy()
        r = orc.conv2d(x.astype(np.complex128 if xc else np.float64), h.astype(np.complex128 if hc else np.float64),
                       mode)
        assert y.shape == r.shape, (y.shape, r.shape)
        scale = np.linalg.norm(orc.conv2d(np.abs(x).astype(np.float64), np.abs(h).astype(np.float64), mode))
        err = np.linalg.norm(y - r) / max(np.linalg.norm(r), 0.1 * scale)
        assert err < 1e-5, (xc, hc, err)


def test_conv2d_double_and_limits(mx, orc):
    import torch
    rng = np.random.default_rng(6)
    x = rng.standard_normal((2, 100, 90)) + 1j * rng.standard_normal((2, 100, 90))
    h = rng.standard_normal((7, 9))
    y = mx.conv2d(dev(x), dev(h), "same").cpu().numpy()
    r = orc.conv2d(x, h, 1)
    assert rel_l2(y, r) < 1e-13
    with pytest.raises(mx.GbfirError):
        mx.conv2d(torch.zeros(200, 200, device="cuda"), torch.zeros(65, 65, device="cuda"))
