"""GPU parity of the ragged persistent launch: every signal against its own
single-signal resample_poly launch and against the oracle; CUDA-graph capture.  The
tensor-core forms (bf16, fp16, bf16x3: column-blocked Toeplitz MMAs per work item) are
checked against the FP64 oracle with the tensor-core error bars (bf16 <= 1e-2, fp16 <=
2e-3, bf16x3 <= 1e-6 rel-L2 per signal)."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

RATIOS = [(1, 2), (2, 3), (3, 4), (5, 4), (160, 147), (1, 1), (3, 2)]


@pytest.fixture(scope="module")
def mx():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import matx_gb300
    from matx_gb300 import build
    build.build()
    return matx_gb300


def make_signals(n, seed, lo=1e3, hi=1e5):
    import torch
    from scipy import signal
    rng = np.random.default_rng(seed)
    sigs = []
    for i in range(n):
        N = int(np.exp(rng.uniform(np.log(lo), np.log(hi))))
        L = int(rng.integers(7, 256)) * 2 + 1
        up, down = RATIOS[int(rng.integers(len(RATIOS)))]
        x = ((rng.standard_normal(N) + 1j * rng.standard_normal(N)) / np.sqrt(2)).astype(np.complex64)
        h = signal.firwin(L, 1.0 / max(up, down, 2), window=("kaiser", 5.0)).astype(np.float32)
        sigs.append((torch.from_numpy(x).cuda(), torch.from_numpy(h).cuda(), up, down))
    return sigs


def test_ragged_matches_single_launches(mx):
    import torch
    from matx_gb300.ragged import RaggedPlan
    sigs = make_signals(300, 1)
    plan = RaggedPlan(sigs)
    outs = plan.run()
    torch.cuda.synchronize()
    for (x, h, up, down), y in zip(sigs, outs):
        ref = mx.resample_poly(x, h, up, down)
        assert y.shape == ref.shape
        assert rel_l2(y.cpu().numpy(), ref.cpu().numpy()) < 1e-6


def test_ragged_vs_oracle_sample(mx):
    import oracle
    import torch
    from matx_gb300.ragged import RaggedPlan
    oracle.build()
    sigs = make_signals(40, 2, 500, 20000)
    outs = RaggedPlan(sigs).run()
    torch.cuda.synchronize()
    for (x, h, up, down), y in zip(sigs, outs):
        r = oracle.resample_poly(x.cpu().numpy(), h.cpu().numpy(), up, down)[0]
        assert rel_l2(y.cpu().numpy(), r) < 1e-5


def test_ragged_graph_capture(mx):
    import torch
    from matx_gb300.ragged import RaggedPlan
    sigs = make_signals(64, 3)
    plan = RaggedPlan(sigs)
    ref = [y.clone() for y in plan.run()]
    torch.cuda.synchronize()
    for y in plan.outputs:
        y.zero_()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        plan.run()  # warm-up on the capture stream
    torch.cuda.current_stream().wait_stream(s)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        plan.run()
    for y in plan.outputs:
        y.zero_()
    g.replay()
    g.replay()
    torch.cuda.synchronize()
    for a, b in zip(plan.outputs, ref):
        assert torch.equal(a, b)


def test_ragged_one_launch(mx):
    import torch
    from matx_gb300.ragged import RaggedPlan
    plan = RaggedPlan(make_signals(100, 4))
    before = mx.launch_count()
    plan.run()
    torch.cuda.synchronize()
    assert mx.launch_count() - before == 1


TC_TOL = {"bf16": 1e-2, "fp16": 2e-3, "bf16x3": 1e-6}


@pytest.mark.parametrize("form", ["bf16x3", "bf16", "fp16"])
def test_ragged_tc_forms_vs_fp64(mx, form):
    import oracle
    import torch
    from matx_gb300.ragged import RaggedPlan
    oracle.build()
    sigs = make_signals(48, 9, 500, 30000)
    plan = RaggedPlan(sigs, precision=form)
    outs = plan.run()
    torch.cuda.synchronize()
    assert mx._lib.load().gbfir_tc_status() == 0
    for (x, h, up, down), y in zip(sigs, outs):
        r = oracle.resample_poly(x.cpu().numpy(), h.cpu().numpy(), up, down)[0]
        assert y.shape[0] == r.shape[0]
        assert rel_l2(y.cpu().numpy(), r) < TC_TOL[form], (up, down, h.shape[0], x.shape[0], form)


def test_ragged_tc_long_decimators_and_graph(mx):
    """1/2 decimators with up to 511 taps (the tap matrices that need K chunks of 32) next to
    160/147 and 1/1 signals, in one graph-captured bf16x3 launch, replayed twice."""
    import oracle
    import torch
    from scipy import signal
    from matx_gb300.ragged import RaggedPlan
    oracle.build()
    rng = np.random.default_rng(77)
    sigs = []
    for i, (up, down, L, N) in enumerate([(1, 2, 511, 40000), (1, 2, 509, 1001), (160, 147, 511, 20000),
                                          (1, 1, 15, 5000), (2, 3, 255, 30000), (5, 4, 101, 12345)]):
        x = ((rng.standard_normal(N) + 1j * rng.standard_normal(N)) / np.sqrt(2)).astype(np.complex64)
        h = signal.firwin(L, 1.0 / max(up, down, 2), window=("kaiser", 5.0)).astype(np.float32)
        sigs.append((torch.from_numpy(x).cuda(), torch.from_numpy(h).cuda(), up, down))
    plan = RaggedPlan(sigs, precision="bf16x3")
    ref = [y.clone() for y in plan.run()]
    torch.cuda.synchronize()
    for (x, h, up, down), y in zip(sigs, ref):
        r = oracle.resample_poly(x.cpu().numpy(), h.cpu().numpy(), up, down)[0]
        assert rel_l2(y.cpu().numpy(), r) < 1e-6, (up, down, h.shape[0])
    for y in plan.outputs:
        y.zero_()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        plan.run()
    torch.cuda.current_stream().wait_stream(s)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        plan.run()
    for y in plan.outputs:
        y.zero_()
    g.replay()
    g.replay()
    torch.cuda.synchronize()
    assert mx._lib.load().gbfir_tc_status() == 0
    for a, b in zip(plan.outputs, ref):
        assert torch.equal(a, b)
