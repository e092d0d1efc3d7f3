"""The host-buffer row pipeline (matx_gb300.streaming.RowPipeline) gives exactly the
device-resident results: every row of every output equals the direct call."""
import numpy as np
import pytest

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


@pytest.mark.parametrize("rows,chunk", [(13, 4), (8, 8), (5, 16), (1, 1)])
def test_row_pipeline_matches_device_path(mx, rows, chunk):
    import torch
    from matx_gb300.streaming import RowPipeline
    dev = torch.device("cuda")
    g = torch.Generator().manual_seed(rows * 31 + chunk)
    x = torch.randn(rows, 30011, dtype=torch.complex64, generator=g).pin_memory()
    h1 = torch.randn(61, generator=g).to(dev)
    h2 = torch.randn(101, generator=g).to(dev)
    n1, n2 = mx.resample_out_len(30011, 3, 2), mx.resample_out_len(30011, 4, 5)
    y1 = torch.empty(rows, n1, dtype=torch.complex64).pin_memory()
    y2 = torch.empty(rows, n2, dtype=torch.complex64).pin_memory()
    pipe = RowPipeline(dev, rows_per_chunk=chunk)
    for _ in range(2):  # the second run reuses the chunk buffers
        y1.zero_()
        y2.zero_()
        pipe.run(x, [y1, y2], lambda xd, oc: [mx.resample_poly(xd, h1, 3, 2, out=oc[0]),
                                               mx.resample_poly(xd, h2, 4, 5, out=oc[1])])
        torch.cuda.synchronize()
        xd = x.to(dev)
        assert torch.equal(y1, mx.resample_poly(xd, h1, 3, 2).cpu())
        assert torch.equal(y2, mx.resample_poly(xd, h2, 4, 5).cpu())


def test_row_pipeline_rejects_device_and_pageable_tensors(mx):
    import torch
    from matx_gb300.streaming import RowPipeline
    pipe = RowPipeline(torch.device("cuda"), rows_per_chunk=2)
    with pytest.raises(ValueError):
        pipe.run(torch.zeros(4, 16, device="cuda"), [torch.zeros(4, 16).pin_memory()], lambda a, b: None)
    with pytest.raises(ValueError):
        pipe.run(torch.zeros(4, 16), [torch.zeros(4, 16).pin_memory()], lambda a, b: None)
