"""Differentiable resample_poly / conv1d (no MatX counterpart).

``resample_poly(x, h, up, down)`` and ``conv1d(x, h, mode)`` here are
torch.autograd.Function wrappers over the forward kernels and the hand-written
adjoints of libgbfir (gbfir_resample_poly_bwd_prec / gbfir_conv1d_bwd_prec):

  dL/dx = the transposed resampler applied to dL/dy (correlation with the taps,
          up and down swapped; for conv1d, corr(dL/dy, h) cropped to the signal),
  dL/dh = the batched cross-correlation of dL/dy with x, reduced over the batch
          and over thread blocks in FP64.

Only x and h are saved for the backward pass (no recomputation, no stored
intermediates).  Real float32 operands; h is one row shared by the batch.
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib
from . import conv1d as _conv1d_fwd
from . import resample_poly as _resample_fwd
from . import _buf, _mode, _prec, _stream

_WS = {}


def _workspace(nbytes: int, device) -> torch.Tensor:
    key = (device.index if device.index is not None else torch.cuda.current_device())
    ws = _WS.get(key)
    if ws is None or ws.numel() < nbytes:
        ws = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=device)
        _WS[key] = ws
    return ws


def _null_buf():
    return _lib.Buf(None, 1, 1, 0, _lib.GBFIR_F32)


def resample_poly_bwd(gy: torch.Tensor, x: torch.Tensor, h: torch.Tensor, up: int, down: int,
                      need_dx: bool = True, need_dh: bool = True, precision="fp32"):
    """(dx, dh) of y = resample_poly(x, h, up, down) for upstream gradient gy.

    ``precision`` other than "fp32" computes dx (bf16, fp16 or bf16x3 Toeplitz MMAs) and
    dh (a GEMM over the signal rows, FP64 across CTAs) on the tensor cores; dh falls back
    to the FP32 reduction where its row tile does not fit the tensor-core kernel.
    """
    lib = _lib.load()
    gy = gy.contiguous()
    x = x.contiguous()
    h = h.contiguous()
    dx = torch.empty_like(x) if need_dx else None
    dh = torch.empty_like(h) if need_dh else None
    B = x.numel() // x.shape[-1]
    nb = lib.gbfir_resample_poly_bwd_workspace_size(B, x.shape[-1], h.shape[-1], up, down)
    ws = _workspace(nb, x.device)
    _lib.check(lib.gbfir_resample_poly_bwd_prec(
        _buf(dx, "dx") if need_dx else _null_buf(), _buf(dh, "dh") if need_dh else _null_buf(),
        _buf(gy, "gy"), _buf(x, "x"), _buf(h, "h"), int(up), int(down), _prec(precision),
        ctypes.c_void_p(ws.data_ptr()), ws.numel(), _stream()))
    return dx, dh


def conv1d_bwd(gy: torch.Tensor, x: torch.Tensor, h: torch.Tensor, mode, need_dx: bool = True,
               need_dh: bool = True, precision="fp32"):
    """(dx, dh) of y = conv1d(x, h, mode) for upstream gradient gy.

    ``precision`` other than "fp32" computes dx (the reversed-tap Toeplitz MMA pass over gy)
    and dh (the GEMM over the signal rows) on the tensor cores.
    """
    lib = _lib.load()
    m = _mode(mode)
    gy = gy.contiguous()
    x = x.contiguous()
    h = h.contiguous()
    dx = torch.empty_like(x) if need_dx else None
    dh = torch.empty_like(h) if need_dh else None
    B = x.numel() // x.shape[-1]
    nb = lib.gbfir_conv1d_bwd_workspace_size(B, x.shape[-1], h.shape[-1], m)
    ws = _workspace(nb, x.device)
    _lib.check(lib.gbfir_conv1d_bwd_prec(
        _buf(dx, "dx") if need_dx else _null_buf(), _buf(dh, "dh") if need_dh else _null_buf(),
        _buf(gy, "gy"), _buf(x, "x"), _buf(h, "h"), m, _prec(precision),
        ctypes.c_void_p(ws.data_ptr()), ws.numel(), _stream()))
    return dx, dh


class ResamplePolyFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, h, up, down, precision="fp32"):
        ctx.save_for_backward(x, h)
        ctx.up, ctx.down, ctx.precision = int(up), int(down), precision
        return _resample_fwd(x, h, up, down, precision=precision)

    @staticmethod
    def backward(ctx, gy):
        x, h = ctx.saved_tensors
        dx, dh = resample_poly_bwd(gy, x, h, ctx.up, ctx.down, ctx.needs_input_grad[0], ctx.needs_input_grad[1],
                                   precision=ctx.precision)
        return dx, dh, None, None, None


class Conv1dFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, h, mode, precision="fp32"):
        ctx.save_for_backward(x, h)
        ctx.mode, ctx.precision = _mode(mode), precision
        return _conv1d_fwd(x, h, mode, precision=precision)

    @staticmethod
    def backward(ctx, gy):
        x, h = ctx.saved_tensors
        dx, dh = conv1d_bwd(gy, x, h, ctx.mode, ctx.needs_input_grad[0], ctx.needs_input_grad[1],
                            precision=ctx.precision)
        return dx, dh, None, None


def resample_poly(x: torch.Tensor, h: torch.Tensor, up: int, down: int, precision="fp32") -> torch.Tensor:
    """Differentiable resample_poly; ``precision`` selects the forward, dL/dx and dL/dh arithmetic."""
    if x.dtype != torch.float32 or h.dtype != torch.float32 or h.dim() != 1:
        raise TypeError("matx_gb300.autograd.resample_poly: real float32 x and a 1-D float32 filter")
    return ResamplePolyFn.apply(x, h, up, down, precision)


def conv1d(x: torch.Tensor, h: torch.Tensor, mode=0, precision="fp32") -> torch.Tensor:
    """Differentiable conv1d; ``precision`` selects the forward, dL/dx and dL/dh arithmetic."""
    if x.dtype != torch.float32 or h.dtype != torch.float32 or h.dim() != 1:
        raise TypeError("matx_gb300.autograd.conv1d: real float32 x and a 1-D float32 filter")
    return Conv1dFn.apply(x, h, mode, precision)
