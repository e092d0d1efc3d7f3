"""The allocation-free backward entry point, gbfir_resample_poly_bwd_noalloc.

This entry point is for callers that cannot give the library a device workspace,
either because their calling convention has no place for one or because they must
not call the device allocator while they run.  It keeps its FP64 partial gradients
in a scratch array compiled into the library.  This file checks, through the C-ABI,
that two calls in a row give the same dx and dh as gbfir_resample_poly_bwd with a
caller workspace, within the rel-L2 1e-5 used by the other FP32 tests, and that a
filter whose partials do not fit in the built-in scratch is rejected before any
device work.  It is named so that pytest collects it after every other test file,
and it also passes when run on its own in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-5


@pytest.fixture(scope="module")
def lib():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from matx_gb300 import _lib, build
    build.build()
    return _lib.load()


def _buf(t):
    from matx_gb300 import _buf as mkbuf
    return mkbuf(t, "t")


def _stream():
    import torch
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _with_workspace(lib, gy, x, h, up, down):
    import torch
    dx, dh = torch.empty_like(x), torch.empty_like(h)
    B = x.shape[0]
    nb = lib.gbfir_resample_poly_bwd_workspace_size(B, x.shape[-1], h.shape[-1], up, down)
    ws = torch.empty(nb, dtype=torch.uint8, device=x.device)
    rc = lib.gbfir_resample_poly_bwd(_buf(dx), _buf(dh), _buf(gy), _buf(x), _buf(h), up, down,
                                     ctypes.c_void_p(ws.data_ptr()), ws.numel(), _stream())
    assert rc == 0, lib.gbfir_last_error()
    return dx, dh


def _noalloc(lib, gy, x, h, up, down):
    import torch
    dx, dh = torch.empty_like(x), torch.empty_like(h)
    rc = lib.gbfir_resample_poly_bwd_noalloc(_buf(dx), _buf(dh), _buf(gy), _buf(x), _buf(h), up, down, _stream())
    assert rc == 0, lib.gbfir_last_error()
    return dx, dh


def _case(seed, B, N, L, up, down):
    import torch
    g = torch.Generator(device="cuda").manual_seed(seed)
    x = torch.rand(B, N, device="cuda", generator=g) * 2 - 1
    h = torch.randn(L, device="cuda", generator=g) / L ** 0.5
    ny = (N * up + down - 1) // down
    gy = torch.randn(B, ny, device="cuda", generator=g)
    return gy, x, h


@pytest.mark.parametrize("updown,L", [((3, 2), 127), ((4, 5), 101), ((160, 147), 321), ((1, 1), 31)])
def test_noalloc_matches_workspace_entry_point_twice(lib, updown, L):
    import torch
    up, down = updown
    # two calls in a row on different data: the shared scratch must not leak state
    for seed in (1, 2):
        gy, x, h = _case(seed * 100 + up, 16, 20000 + seed, L, up, down)
        rdx, rdh = _with_workspace(lib, gy, x, h, up, down)
        dx, dh = _noalloc(lib, gy, x, h, up, down)
        torch.cuda.synchronize()
        assert rel_l2(dx.cpu().numpy(), rdx.cpu().numpy()) < TOL
        if float(rdh.abs().max()) == 0.0:
            assert float(dh.abs().max()) == 0.0
        else:
            assert rel_l2(dh.cpu().numpy(), rdh.cpu().numpy()) < TOL


def test_noalloc_rejects_filters_beyond_the_scratch(lib):
    import torch
    # 1,000,001 taps need far more partial gradients than the built-in scratch holds
    gy, x, h = _case(7, 2, 4000, 1_000_001, 3, 2)
    dx, dh = torch.empty_like(x), torch.empty_like(h)
    rc = lib.gbfir_resample_poly_bwd_noalloc(_buf(dx), _buf(dh), _buf(gy), _buf(x), _buf(h), 3, 2, _stream())
    assert rc == 3  # GBFIR_ERR_INVALID_SIZE
    assert b"scratch" in lib.gbfir_last_error()
