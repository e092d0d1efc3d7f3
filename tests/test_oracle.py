"""Pins the CPU oracle to the reference: its golden vectors, its known-answer
tests, and (where MatX compiles here) MatX's HostExecutor on the same inputs."""
import numpy as np
import pytest

from conftest import load_cases, rel_l2, seed_of

MODES = {"conv_full": 0, "conv_same": 1, "conv_valid": 2}


def test_conv_known_answer(oracle_mod):
    # test/00_transform/ConvCorr.cu:250-288 — in {1,2,3,4}, h {2,1,-1}
    x = np.array([1, 2, 3, 4], dtype=np.float64)
    h = np.array([2, 1, -1], dtype=np.float64)
    assert np.array_equal(oracle_mod.conv1d(x, h, 0)[0], [2, 5, 7, 9, 1, -4])
    assert np.array_equal(oracle_mod.conv1d(x, h, 1)[0], [5, 7, 9, 1])
    assert np.array_equal(oracle_mod.conv1d(x, h, 2)[0], [7, 9])


@pytest.mark.parametrize("case", sorted(load_cases("conv.npz")))
def test_conv_golden(oracle_mod, case):
    c = load_cases("conv.npz")[case]
    a, b = c["a_op"], c["b_op"]
    for key, mode in MODES.items():
        y = oracle_mod.conv1d(a, b, mode)[0]
        assert y.shape == c[key].shape, key
        assert rel_l2(y, c[key]) < 1e-6, key
    assert rel_l2(oracle_mod.conv1d(a, b, 0, is_corr=True)[0], c["corr"]) < 1e-6
    assert rel_l2(oracle_mod.conv1d(b, a, 0, is_corr=True)[0], c["corr_swap"]) < 1e-6


@pytest.mark.parametrize("case", sorted(load_cases("resample.npz")))
def test_resample_golden(oracle_mod, case):
    c = load_cases("resample.npz")[case]
    up, down = (int(v) for v in c["updown"])
    y = oracle_mod.resample_poly(c["a"], c["h"], up, down)[0]
    assert y.shape == c["y"].shape
    tol = 1e-12 if c["a"].dtype == np.float64 else 1e-6
    assert rel_l2(y, c["y"]) < tol


@pytest.mark.parametrize("case", sorted(load_cases("channelize.npz")))
def test_channelize_golden(oracle_mod, case):
    c = load_cases("channelize.npz")[case]
    M, D = (int(v) for v in c["md"])
    a = c["a"]
    batch_shape = a.shape[:-1]
    y = oracle_mod.channelize_poly(a.reshape(-1, a.shape[-1]), c["h"], M, D)
    y = y.reshape(*batch_shape, y.shape[-2], M) if batch_shape else y[0]
    tol = 1e-10 if a.dtype == np.complex128 else 1e-5
    assert y.shape == c["y"].shape
    assert rel_l2(y, c["y"]) < tol
    if "y_hreal" in c:
        yr = oracle_mod.channelize_poly(a.reshape(-1, a.shape[-1]), np.real(c["h"]), M, D)
        yr = yr.reshape(c["y_hreal"].shape)
        assert rel_l2(yr, c["y_hreal"]) < tol


def test_harris2003_known_answer(oracle_mod):
    # ChannelizePoly.cu:820-1100, double, thresh 1e-12 absolute per component
    import os
    from conftest import GOLDEN
    z = np.load(os.path.join(GOLDEN, "harris2003.npz"))
    M = int(z["M"][0])
    y = oracle_mod.channelize_poly(z["x"], z["h"], M, M)[0]
    assert np.max(np.abs(y.real - z["y"].real)) < 1e-12
    assert np.max(np.abs(y.imag - z["y"].imag)) < 1e-12


def test_harris2003_oversampled(oracle_mod):
    # ChannelizePoly.cu:1104-1132, M=40, D=28, golden from the reference's .bin
    import os
    from conftest import GOLDEN
    z = np.load(os.path.join(GOLDEN, "harris2003_oversampled.npz"))
    M, D = (int(v) for v in z["MD"])
    y = oracle_mod.channelize_poly(z["x"], z["h"], M, D)[0]
    assert y.shape == z["y"].shape
    assert np.max(np.abs(y - z["y"])) < 1e-10


def test_float_oracle_close_to_double(oracle_mod):
    rng = np.random.default_rng(5)
    x = (rng.standard_normal((3, 4000)) + 1j * rng.standard_normal((3, 4000))).astype(np.complex64)
    h = rng.standard_normal(61).astype(np.float32)
    assert rel_l2(oracle_mod.resample_poly(x, h, 3, 2, double=False),
                  oracle_mod.resample_poly(x, h, 3, 2)) < 1e-6
    assert rel_l2(oracle_mod.channelize_poly(x, h, 16, 16, double=False),
                  oracle_mod.channelize_poly(x, h, 16, 16)) < 1e-5


def test_threads_do_not_change_results(oracle_mod):
    rng = np.random.default_rng(6)
    x = rng.standard_normal((8, 3000)).astype(np.float32)
    h = rng.standard_normal(63).astype(np.float32)
    a = oracle_mod.conv1d(x, h, 0, double=False, nthreads=1)
    b = oracle_mod.conv1d(x, h, 0, double=False, nthreads=4)
    assert np.array_equal(a, b)
    a = oracle_mod.resample_poly(x, h, 4, 5, double=False, nthreads=1)
    b = oracle_mod.resample_poly(x, h, 4, 5, double=False, nthreads=4)
    assert np.array_equal(a, b)


# ---- pin against MatX's own HostExecutor (only where MatX was compiled) ------

def _need_ref(oracle_mod):
    if oracle_mod.ref_lib() is None:
        pytest.skip("MatX HostExecutor library (oracle/_ref) not built on this host")


@pytest.mark.parametrize("mode", [0, 1, 2])
@pytest.mark.parametrize("is_corr", [0, 1])
@pytest.mark.parametrize("shape", [(3, 200, 17), (2, 64, 64), (2, 30, 100), (1, 1000, 16)])
@pytest.mark.parametrize("cplx", ["real", "cx_rh", "cx_ch"])
def test_conv_matches_matx_host(oracle_mod, mode, is_corr, shape, cplx):
    _need_ref(oracle_mod)
    B, N, L = shape
    rng = np.random.default_rng(seed_of(mode, is_corr, shape, cplx))
    x = rng.standard_normal((B, N))
    h = rng.standard_normal(L)
    if cplx != "real":
        x = x + 1j * rng.standard_normal((B, N))
    if cplx == "cx_ch":
        h = h + 1j * rng.standard_normal(L)
    for double in (True, False):
        r = oracle_mod.ref_conv1d(x, h, mode, bool(is_corr), double=double)
        o = oracle_mod.conv1d(x, h, mode, bool(is_corr), double=double)
        assert r.shape == o.shape
        assert rel_l2(o, r) < (1e-13 if double else 1e-6)


@pytest.mark.parametrize("updown", [(3, 2), (4, 5), (160, 147), (1, 3), (2, 1), (6, 4), (5, 5)])
@pytest.mark.parametrize("L", [31, 30, 5, 401])
@pytest.mark.parametrize("cplx", ["real", "cx_rh", "cx_ch"])
def test_resample_matches_matx_host(oracle_mod, updown, L, cplx):
    _need_ref(oracle_mod)
    up, down = updown
    rng = np.random.default_rng(seed_of(updown, L, cplx))
    x = rng.standard_normal((2, 777))
    h = rng.standard_normal(L)
    if cplx != "real":
        x = x + 1j * rng.standard_normal((2, 777))
    if cplx == "cx_ch":
        h = h + 1j * rng.standard_normal(L)
    for double in (True, False):
        r = oracle_mod.ref_resample_poly(x, h, up, down, double=double)
        if r is None:
            continue
        o = oracle_mod.resample_poly(x, h, up, down, double=double)
        assert rel_l2(o, r) < (1e-13 if double else 1e-6)


@pytest.mark.parametrize("MD", [(8, 8), (10, 10), (13, 13), (16, 12), (40, 28), (9, 4), (1, 1), (64, 64)])
@pytest.mark.parametrize("L", [100, 64, 7])
@pytest.mark.parametrize("cplx", ["cx_rh", "cx_ch", "real"])
def test_channelize_matches_matx_host(oracle_mod, MD, L, cplx):
    _need_ref(oracle_mod)
    M, D = MD
    rng = np.random.default_rng(seed_of(MD, L, cplx))
    x = rng.standard_normal((2, 1001))
    h = rng.standard_normal(L)
    if cplx != "real":
        x = x + 1j * rng.standard_normal((2, 1001))
    if cplx == "cx_ch":
        h = h + 1j * rng.standard_normal(L)
    for double in (True, False):
        r = oracle_mod.ref_channelize_poly(x, h, M, D, double=double)
        if r is None:
            continue
        o = oracle_mod.channelize_poly(x, h, M, D, double=double)
        assert rel_l2(o, r) < (1e-12 if double else 1e-5)


# ---- adjoint oracle against FP64 central finite differences ------------------

@pytest.mark.parametrize("updown", [(3, 2), (1, 1), (4, 5), (2, 3)])
@pytest.mark.parametrize("L", [13, 12])
def test_resample_adjoint_oracle_fd(oracle_mod, updown, L):
    up, down = updown
    rng = np.random.default_rng(11)
    x = rng.standard_normal((2, 60))
    h = rng.standard_normal(L)
    ny = oracle_mod.resample_poly(x, h, up, down).shape[1]
    gy = rng.standard_normal((2, ny))
    dx, dh = oracle_mod.resample_poly_bwd(gy, x, h, up, down)
    f = lambda xx, hh: float(np.sum(gy * oracle_mod.resample_poly(xx, hh, up, down)))
    eps = 1e-6
    for _ in range(8):
        b, i = rng.integers(2), rng.integers(60)
        xp, xm = x.copy(), x.copy()
        xp[b, i] += eps
        xm[b, i] -= eps
        assert abs((f(xp, h) - f(xm, h)) / (2 * eps) - dx[b, i]) < 1e-6
        k = rng.integers(L)
        hp, hm = h.copy(), h.copy()
        hp[k] += eps
        hm[k] -= eps
        assert abs((f(x, hp) - f(x, hm)) / (2 * eps) - dh[k]) < 1e-6


@pytest.mark.parametrize("mode", [0, 1, 2])
@pytest.mark.parametrize("L", [9, 8])
def test_conv_adjoint_oracle_fd(oracle_mod, mode, L):
    rng = np.random.default_rng(12)
    x = rng.standard_normal((2, 50))
    h = rng.standard_normal(L)
    ny = oracle_mod.conv1d(x, h, mode).shape[1]
    gy = rng.standard_normal((2, ny))
    dx, dh = oracle_mod.conv1d_bwd(gy, x, h, mode)
    f = lambda xx, hh: float(np.sum(gy * oracle_mod.conv1d(xx, hh, mode)))
    eps = 1e-6
    for _ in range(8):
        b, i = rng.integers(2), rng.integers(50)
        xp, xm = x.copy(), x.copy()
        xp[b, i] += eps
        xm[b, i] -= eps
        assert abs((f(xp, h) - f(xm, h)) / (2 * eps) - dx[b, i]) < 1e-6
        k = rng.integers(L)
        hp, hm = h.copy(), h.copy()
        hp[k] += eps
        hm[k] -= eps
        assert abs((f(x, hp) - f(x, hm)) / (2 * eps) - dh[k]) < 1e-6


def test_adjoint_oracle_matches_matx_built_gradients(oracle_mod):
    # grad_refs.npz: gradients composed from MatX's own corr / resample_poly (FP64)
    import os
    from conftest import GOLDEN
    z = np.load(os.path.join(GOLDEN, "grad_refs.npz"))
    x, h = z["x"], z["h"]
    for mode, name in ((0, "full"), (1, "same"), (2, "valid")):
        dx, dh = oracle_mod.conv1d_bwd(z[f"conv_{name}__gy"], x, h, mode)
        assert rel_l2(dx, z[f"conv_{name}__dx"]) < 1e-12
        assert rel_l2(dh, z[f"conv_{name}__dh"]) < 1e-12
    for up, down in ((3, 2), (2, 3), (4, 5)):
        dx, _ = oracle_mod.resample_poly_bwd(z[f"rs_{up}_{down}__gy"], x, h, up, down)
        assert rel_l2(dx, z[f"rs_{up}_{down}__dx"]) < 1e-12


def _filter_test_regression_expected(batches, n, h_rec, h_nonrec):
    """The sequential loop of MatX's own IIR test (test/00_operators/filter_test.cu:19-47)."""
    x = np.array([[((((i + 11 * b) % 23) - 11)) / 7.0 for i in range(n)] for b in range(batches)])
    exp = np.zeros((batches, n))
    for b in range(batches):
        for i in range(n):
            y = 0.0
            for nr, c in enumerate(h_nonrec):
                if i >= nr:
                    y += c * x[b, i - nr]
            for r, c in enumerate(h_rec):
                if i >= r + 1:
                    y += c * exp[b, i - r - 1]
            exp[b, i] = y
    return x, exp


def test_oracle_iir_matches_reference_test(oracle_mod):
    # IIRNonMultipleOfChunkSize: 3 rows of 8192 + 37 samples, h_rec {0.4, -0.1}, h_nonrec {2, 1}
    x, exp = _filter_test_regression_expected(3, 8192 + 37, (0.4, -0.1), (2.0, 1.0))
    y = oracle_mod.iir_filter(x, [0.4, -0.1], [2.0, 1.0])
    assert np.max(np.abs(y - exp)) < 1e-12
    yf = oracle_mod.iir_filter(x.astype(np.float32), np.float32([0.4, -0.1]), np.float32([2.0, 1.0]), double=False)
    assert np.max(np.abs(yf - exp)) < 1e-2  # the reference test's float tolerance


def test_oracle_iir_matches_lfilter(oracle_mod):
    signal = pytest.importorskip("scipy.signal")
    rng = np.random.default_rng(seed_of("iir_lfilter"))
    for na, nb, cplx in ((1, 1, False), (4, 4, True), (3, 2, True), (2, 4, False)):
        a = rng.uniform(-0.3, 0.3, na) + (1j * rng.uniform(-0.2, 0.2, na) if cplx else 0)
        b = rng.standard_normal(nb) + (1j * rng.standard_normal(nb) if cplx else 0)
        x = rng.standard_normal((2, 3000)) + (1j * rng.standard_normal((2, 3000)) if cplx else 0)
        y = oracle_mod.iir_filter(x, a, b)
        r = signal.lfilter(b, np.concatenate([[1.0], -a]), x, axis=-1)
        assert np.max(np.abs(y - r)) < 1e-9 * np.max(np.abs(r)), (na, nb, cplx)
    # FIR only: conv1d SAME (transforms/filter.h:185)
    x = rng.standard_normal((2, 500))
    assert np.array_equal(oracle_mod.iir_filter(x, [], [1.0, -2.0, 1.0]),
                          oracle_mod.conv1d(x, np.array([1.0, -2.0, 1.0]), 1))


def test_oracle_conv2d_known_answer(oracle_mod):
    # ConvCorr.cu:395-440: 3 x 3 ramp against [[1, 2], [3, 4]]
    x = np.arange(1, 10, dtype=np.float64).reshape(3, 3)
    h = np.array([[1.0, 2.0], [3.0, 4.0]])
    full = np.array([[1, 4, 7, 6], [7, 23, 33, 24], [19, 53, 63, 42], [21, 52, 59, 36]], np.float64)
    assert np.array_equal(oracle_mod.conv2d(x, h, 0), full)
    assert np.array_equal(oracle_mod.conv2d(x, h, 1), full[:3, :3])
    assert np.array_equal(oracle_mod.conv2d(x, h, 2), np.array([[23, 33], [53, 63]], np.float64))


@pytest.mark.parametrize("case", sorted(load_cases("conv2d.npz")))
def test_oracle_conv2d_matches_reference_vectors(oracle_mod, case):
    c = load_cases("conv2d.npz")[case]
    a, b = c["a_op"], c["b_op"]
    tol = 1e-12 if a.dtype == np.float64 else 1e-5
    for mode, key in ((0, "conv_full"), (1, "conv_same"), (2, "conv_valid")):
        r = oracle_mod.conv2d(a, b, mode)
        assert r.shape == c[key].shape, (mode, r.shape, c[key].shape)
        assert rel_l2(r, c[key]) < tol, (case, mode)
        # the swapped call conv2d(filter, image) gives the same result (ConvCorr.cu:783-787)
        assert rel_l2(oracle_mod.conv2d(b, a, mode), c[key]) < tol
