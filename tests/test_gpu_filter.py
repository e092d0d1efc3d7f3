"""MatX filter(): the recursive (IIR) filter against the FP64 oracle recurrence (pinned to
MatX's own IIR test loop, test/00_operators/filter_test.cu:19-47, in test_oracle.py) and the
FIR-only form against conv1d SAME (transforms/filter.h:185)."""
import numpy as np
import pytest

from conftest import rel_l2, seed_of

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


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_reference_regression_case(mx, orc, dt):
    # IIRNonMultipleOfChunkSize: 3 rows of 8192 + 37 samples, h_rec {0.4, -0.1}, h_nonrec {2, 1}
    import torch
    n = 8192 + 37
    x = np.array([[((((i + 11 * b) % 23) - 11)) / 7.0 for i in range(n)] for b in range(3)]).astype(dt)
    y = mx.filter(torch.from_numpy(x).cuda(), [0.4, -0.1], [2.0, 1.0]).cpu().numpy()
    r = orc.iir_filter(x.astype(np.float64), [0.4, -0.1], [2.0, 1.0])
    assert np.max(np.abs(y - r)) < (1e-2 if dt == np.float32 else 1e-8)  # the reference test's bounds
    assert rel_l2(y, r) < (1e-6 if dt == np.float32 else 1e-14)


@pytest.mark.parametrize("N", [1, 31, 8192, 8193, 100003])
@pytest.mark.parametrize("na,nb", [(1, 1), (2, 2), (4, 4), (3, 1), (1, 4)])
def test_iir_vs_oracle(mx, orc, N, na, nb):
    import torch
    rng = np.random.default_rng(seed_of("iir", N, na, nb))
    for xc, cc, dt in ((False, False, np.float32), (True, False, np.float32), (True, True, np.float32),
                       (False, True, np.float32), (True, True, np.float64), (False, False, np.float64)):
        a = rng.uniform(-0.2, 0.2, na) + (1j * rng.uniform(-0.2, 0.2, na) if cc else 0)
        b = rng.standard_normal(nb) + (1j * rng.standard_normal(nb) if cc else 0)
        x = rng.uniform(-1, 1, (3, N)) + (1j * rng.uniform(-1, 1, (3, N)) if xc else 0)
        x = x.astype((np.complex64 if xc else np.float32) if dt == np.float32 else (np.complex128 if xc else np.float64))
        y = mx.filter(torch.from_numpy(x).cuda(), a, b).cpu().numpy()
        r = orc.iir_filter(x, a.astype(np.complex128 if cc else np.float64), b.astype(np.complex128 if cc else np.float64))
        assert y.shape == r.shape and (np.iscomplexobj(y) == (xc or cc))
        assert rel_l2(y, r) < (2e-6 if dt == np.float32 else 1e-13), (xc, cc, dt, rel_l2(y, r))


def test_iir_long_memory_carries(mx, orc):
    # a pole at 0.999: the state carries across ~100 CTAs of 8192 samples
    import torch
    rng = np.random.default_rng(7)
    x = rng.uniform(-1, 1, (2, 800_000)).astype(np.float32)
    y = mx.filter(torch.from_numpy(x).cuda(), [0.999], [1.0]).cpu().numpy()
    r = orc.iir_filter(x.astype(np.float64), [0.999], [1.0])
    assert rel_l2(y, r) < 1e-4
    # second order resonator with poles at radius 0.99
    a = [2 * 0.99 * np.cos(0.3), -0.99 ** 2]
    y = mx.filter(torch.from_numpy(x).cuda(), a, [1.0, 0.5]).cpu().numpy()
    r = orc.iir_filter(x.astype(np.float64), a, [1.0, 0.5])
    assert rel_l2(y, r) < 1e-4
    # every chained-carry wait completed (a wait that gives up is recorded, not hung on)
    from matx_gb300 import _lib
    assert _lib.load().gbfir_tc_status() == 0


def test_iir_many_rows_and_blocks(mx, orc):
    # 300 rows x 40 blocks: tickets interleave rows, carries chain within each row only
    import torch
    rng = np.random.default_rng(9)
    x = rng.uniform(-1, 1, (300, 40 * 8192 - 5)).astype(np.float32)
    y = mx.filter(torch.from_numpy(x).cuda(), [0.9, -0.2], [1.0, -1.0]).cpu().numpy()
    for row in (0, 1, 150, 299):
        r = orc.iir_filter(x[row:row + 1].astype(np.float64), [0.9, -0.2], [1.0, -1.0])
        assert rel_l2(y[row:row + 1], r) < 2e-6, row
    from matx_gb300 import _lib
    assert _lib.load().gbfir_tc_status() == 0


@pytest.mark.parametrize("nb", [1, 2, 3, 4])
def test_fir_only_is_conv1d_same(mx, orc, nb):
    import torch
    rng = np.random.default_rng(seed_of("fir_only", nb))
    for cplx in (False, True):
        x = rng.uniform(-1, 1, (4, 5000)).astype(np.float32)
        if cplx:
            x = (x + 1j * rng.uniform(-1, 1, (4, 5000))).astype(np.complex64)
        b = rng.standard_normal(nb).astype(np.float32)
        y = mx.filter(torch.from_numpy(x).cuda(), [], b)
        yc = mx.conv1d(torch.from_numpy(x).cuda(), torch.from_numpy(b).cuda(), "same")
        assert torch.allclose(y, yc, rtol=1e-6, atol=1e-6)
        assert rel_l2(y.cpu().numpy(), orc.iir_filter(x, [], b.astype(np.float64))) < 1e-6


def test_filter_validation(mx):
    import torch
    x = torch.zeros(2, 100, device="cuda")
    with pytest.raises(mx.GbfirError):
        mx.filter(x, [0.1] * 5, [1.0])
    with pytest.raises(mx.GbfirError):
        mx.filter(x, [0.1], [])
    with pytest.raises(mx.GbfirError):
        mx.filter(torch.zeros(2, 3, device="cuda"), [], [1.0, 2.0, 3.0, 4.0])
