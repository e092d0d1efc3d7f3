"""matx_gb300 — GB300-native (sm_103a) direct-FIR operators behind MatX's operator API.

Python host mirror of MatX's direct-FIR operators.  Each function keeps the MatX
operator's name, argument meaning, output shape and error class, and runs the
CUDA library libgbfir.so (include/gbfir.h) on torch's current CUDA stream:

    conv1d(x, h, mode)                 include/matx/operators/conv.h:243-274
    corr(x, h, mode)                   include/matx/operators/corr.h:224-253
    resample_poly(x, h, up, down)      include/matx/operators/resample_poly.h:182-186
    channelize_poly(x, h, M, D)        include/matx/operators/channelize_poly.h:275-278

Tensors are torch CUDA tensors; the last dimension is the signal axis and every
leading dimension is a batch dimension (MatX's BlockToIdx batch folding,
core/operator_utils.h:244-267).  There is no CPU path: a CPU tensor or a missing
library raises.
"""
from __future__ import annotations

import ctypes
import math

import torch

from . import _lib
from ._lib import GbfirError, PREC

MATX_C_MODE_FULL, MATX_C_MODE_SAME, MATX_C_MODE_VALID = 0, 1, 2
_MODE_NAMES = {"full": 0, "same": 1, "valid": 2}

__all__ = ["conv1d", "corr", "resample_poly", "channelize_poly", "GbfirError",
           "MATX_C_MODE_FULL", "MATX_C_MODE_SAME", "MATX_C_MODE_VALID", "launch_count",
           "resample_out_len", "set_resample_tile", "upsample", "downsample", "upfirdn", "filter",
           "iir_filter", "conv2d"]

_DT = {torch.float32: _lib.GBFIR_F32, torch.complex64: _lib.GBFIR_C64,
       torch.float64: _lib.GBFIR_F64, torch.complex128: _lib.GBFIR_C128}


def _mode(mode) -> int:
    if isinstance(mode, str):
        return _MODE_NAMES[mode.lower()]
    return int(mode)


def _prec(precision) -> int:
    if isinstance(precision, str):
        return PREC[precision.lower()]
    return int(precision)


def _stream() -> ctypes.c_void_p:
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _rows(t: torch.Tensor, name: str) -> torch.Tensor:
    if not t.is_cuda:
        raise ValueError(f"{name}: matx_gb300 runs on CUDA tensors only (got {t.device})")
    if t.dtype not in _DT:
        raise TypeError(f"{name}: unsupported dtype {t.dtype}")
    if t.dim() == 0:
        raise ValueError(f"{name}: needs at least one dimension")
    return t


def _buf(t: torch.Tensor, name: str) -> _lib.Buf:
    """Describe a tensor as rows of its last dimension (materialises other layouts)."""
    t = _rows(t, name)
    if t.stride(-1) != 1:
        raise ValueError(f"{name}: last dimension must be unit-stride")
    n = t.shape[-1]
    batch = t.numel() // n if n else 0
    if t.dim() == 1:
        bstride = 0
    else:
        flat = t.reshape(-1, n)
        if flat.data_ptr() != t.data_ptr() or (batch > 1 and flat.stride(0) < n):
            raise ValueError(f"{name}: leading dimensions must fold into one batch dimension")
        bstride = flat.stride(0) if batch > 1 else 0
    return _lib.Buf(t.data_ptr(), max(batch, 1), n, bstride, _DT[t.dtype])


def _prep_in(t: torch.Tensor, name: str) -> torch.Tensor:
    t = _rows(t, name)
    if t.stride(-1) != 1 or (t.dim() > 1 and not t.is_contiguous()):
        t = t.contiguous()  # MatX's shim materialises strided views the same way
    return t


def _out_dtype(*ts) -> torch.dtype:
    cplx = any(t.is_complex() for t in ts)
    dbl = any(t.dtype in (torch.float64, torch.complex128) for t in ts)
    if cplx:
        return torch.complex128 if dbl else torch.complex64
    return torch.float64 if dbl else torch.float32


def _cast(t: torch.Tensor, double: bool) -> torch.Tensor:
    if t.is_complex():
        want = torch.complex128 if double else torch.complex64
    else:
        want = torch.float64 if double else torch.float32
    return t if t.dtype == want else t.to(want)


def launch_count() -> int:
    """Kernels libgbfir has launched in this process."""
    return int(_lib.load().gbfir_launch_count())


def set_resample_tile(rows_per_thread: int = 0, col_warps: int = 0, group: int = 0, buffers: int = 0):
    """Force a resample_poly tile shape (zeros restore the heuristic)."""
    _lib.check(_lib.load().gbfir_set_resample_tile(rows_per_thread, col_warps, group, buffers))


def _olen(m: int, N: int, L: int) -> int:
    if m == 0:
        return N + L - 1
    if m == 1:
        return max(N, L)
    return max(N, L) - min(N, L) + 1


def _axis_layout(t: torch.Tensor, a: int):
    """Signals of t along dimension a as base + o*ostride + n*step + i: returns
    (inner_dim, inner, step, outer_dims, outer, ostride), or None when the other
    dimensions do not fold into one unit-stride inner index and one outer index."""
    dims = [d for d in range(t.dim()) if d != a and t.shape[d] > 1]
    unit = [d for d in dims if t.stride(d) == 1]
    d_in = unit[-1] if unit else None
    rest = sorted((d for d in dims if d != d_in), key=lambda d: -t.stride(d))
    for u, v in zip(rest, rest[1:]):
        if t.stride(u) != t.stride(v) * t.shape[v]:
            return None
    inner = t.shape[d_in] if d_in is not None else 1
    outer = math.prod(t.shape[d] for d in rest)
    return d_in, inner, t.stride(a), rest, outer, (t.stride(rest[-1]) if rest else 0)


def _empty_like_order(t: torch.Tensor, shape, dtype) -> torch.Tensor:
    """A fresh tensor of `shape` whose dimensions are laid out in t's stride order."""
    order = sorted(range(t.dim()), key=lambda d: (-t.stride(d), d))
    base = torch.empty([shape[d] for d in order], dtype=dtype, device=t.device)
    return base.permute([order.index(d) for d in range(t.dim())])


def _conv1d_axis(x, h, m, a, out, corr):
    """conv1d of a 1-D filter along dimension a of x in place of its layout
    (gbfir_conv1d_axis): no transpose is materialised when the other dimensions fold into
    one unit-stride inner index and one outer index."""
    lib = _lib.load()
    double = _out_dtype(x, h) in (torch.float64, torch.complex128)
    x = _rows(_cast(x, double), "conv1d x")
    h = _prep_in(_cast(h, double), "conv1d h")
    if h.dim() != 1:
        raise GbfirError(2, "conv1d (axis): the filter must be 1-D")
    lx = _axis_layout(x, a)
    if lx is None:
        x = x.contiguous()  # MatX's shim materialises such views the same way
        lx = _axis_layout(x, a)
    N, L = x.shape[a], h.shape[0]
    oshape = list(x.shape)
    oshape[a] = _olen(m, N, L)
    odt = _out_dtype(x, h)
    if out is None:
        out = _empty_like_order(x, oshape, odt)
    elif list(out.shape) != oshape or out.dtype != odt or not out.is_cuda:
        raise ValueError(f"conv1d (axis): out must be a {odt} CUDA tensor of shape {oshape}")
    lo = _axis_layout(out, a)
    if lo is None or lo[0] != lx[0] or lo[3] != lx[3] or (lo[0] is not None and lo[2] < lo[1]):
        raise ValueError("conv1d (axis): out must have the layout of the input along the other dimensions")
    d_in, inner, sx, _, outer, ox = lx
    bx = _lib.Buf(x.data_ptr(), outer, N, ox, _DT[x.dtype])
    bo = _lib.Buf(out.data_ptr(), outer, oshape[a], lo[5], _DT[out.dtype])
    _lib.check(lib.gbfir_conv1d_axis(bo, bx, _buf(h, "conv1d h"), inner, sx, lo[2], m, int(corr), 0, _stream()))
    return out


def conv1d(x: torch.Tensor, h: torch.Tensor, mode=MATX_C_MODE_FULL, *, out: torch.Tensor | None = None,
           precision="fp32", axis: int = -1, method="direct", _corr: bool = False) -> torch.Tensor:
    """1-D convolution (MatX conv1d; ``method`` "direct" = MATX_C_METHOD_DIRECT, "fft" =
    MATX_C_METHOD_FFT, the overlap-save FFT form for long filters, transforms/conv.h:51-172).

    Output length: N+L-1 (FULL), max(N,L) (SAME), max(N,L)-min(N,L)+1 (VALID).
    The operand with more dimensions sets the batch shape; a 1-D operand is
    broadcast across the other's batch (conv.h:467-532).  ``precision`` "bf16",
    "fp16" or "bf16x3" runs the Toeplitz MMA form on the tensor cores (a real
    float32 filter shared by all rows, signal at least as long as the filter).
    ``axis`` convolves another dimension with a 1-D filter (MatX's
    conv1d(a, b, {axis}, mode), operators/conv.h:263-274); so does a last dimension that
    is a transposed view of a contiguous tensor (the radar three-pulse canceller's
    permuted view, examples/simple_radar_pipeline.h:321-327): the data is not moved, and
    the result is the same kind of view.
    """
    m = _mode(mode)
    nd = max(x.dim(), 1)
    if method not in ("direct", "fft"):
        raise GbfirError(1, f"conv1d: unknown method {method!r}")
    if method == "fft" and _prec(precision) != 0:
        raise GbfirError(5, "conv1d: the FFT method is FP32 only")
    if x.dim() > 1 and h.dim() == 1 and x.is_cuda and _prec(precision) == 0 and method == "direct":
        a = axis % nd
        if a != nd - 1 or x.stride(-1) != 1:
            return _conv1d_axis(x, h, m, a, out, _corr)
    elif axis % nd != nd - 1:
        raise GbfirError(2, "conv1d: an axis other than the last needs a 1-D filter and FP32")
    lib = _lib.load()
    double = _out_dtype(x, h) in (torch.float64, torch.complex128)
    x = _prep_in(_cast(x, double), "conv1d x")
    h = _prep_in(_cast(h, double), "conv1d h")
    N, L = x.shape[-1], h.shape[-1]
    if m == 0:
        olen = N + L - 1
    elif m == 1:
        olen = max(N, L)
    else:
        olen = max(N, L) - min(N, L) + 1
    batch_shape = x.shape[:-1] if x.dim() >= h.dim() else h.shape[:-1]
    if x.dim() > 1 and h.dim() > 1 and x.shape[:-1] != h.shape[:-1]:
        raise GbfirError(2, "conv1d: batched operands must have the same batch shape")
    odt = _out_dtype(x, h)
    if out is None:
        out = torch.empty(*batch_shape, olen, dtype=odt, device=x.device)
    if method == "fft":
        _lib.check(lib.gbfir_conv1d_fft(_buf(out, "conv1d out"), _buf(x, "conv1d x"), _buf(h, "conv1d h"),
                                        m, int(_corr), _stream()))
        return out
    _lib.check(lib.gbfir_conv1d(_buf(out, "conv1d out"), _buf(x, "conv1d x"), _buf(h, "conv1d h"),
                                m, int(_corr), _prec(precision), _stream()))
    return out


def corr(x: torch.Tensor, h: torch.Tensor, mode=MATX_C_MODE_FULL, *, out: torch.Tensor | None = None,
         precision="fp32", axis: int = -1, method="direct"):
    """Correlation: corr(x, h) = conv1d(x, reverse(conj(h))) (corr.h:67)."""
    return conv1d(x, h, mode, out=out, precision=precision, axis=axis, method=method, _corr=True)


def _buf2d(t: torch.Tensor, name: str) -> _lib.Buf2d:
    """Images of the last two dimensions; the leading ones must fold into one batch stride."""
    t = _rows(t, name)
    if t.dim() < 2:
        raise ValueError(f"{name}: needs at least two dimensions")
    if t.stride(-1) != 1:
        t = t.contiguous()
    rows, cols = t.shape[-2], t.shape[-1]
    batch = t.numel() // max(rows * cols, 1)
    bstride = 0
    if batch > 1:
        flat = t.reshape(-1, rows, cols)
        if flat.data_ptr() != t.data_ptr():
            raise ValueError(f"{name}: leading dimensions must fold into one batch dimension")
        bstride = flat.stride(0)
    return _lib.Buf2d(t.data_ptr(), max(batch, 1), rows, cols, bstride, t.stride(-2) if rows > 1 else cols,
                      _DT[t.dtype])


def conv2d(x: torch.Tensor, h: torch.Tensor, mode=MATX_C_MODE_FULL, *, out: torch.Tensor | None = None):
    """MatX conv2d (transforms/conv.h:548-600, direct): 2-D convolution of the last two
    dimensions; sizes per axis max+min-1 (FULL), max (SAME), max-min+1 (VALID); the operand
    with more elements is the image; either operand may be one image broadcast over the
    other's batch."""
    m = _mode(mode)
    double = _out_dtype(x, h) in (torch.float64, torch.complex128)
    x = _prep_in(_cast(x, double), "conv2d x")
    h = _prep_in(_cast(h, double), "conv2d h")
    if x.dim() < 2 or h.dim() < 2:
        raise GbfirError(2, "conv2d: operands need at least two dimensions")
    size = lambda a, b: (a + b - 1) if m == 0 else (max(a, b) if m == 1 else max(a, b) - min(a, b) + 1)
    oshape = (*(x.shape[:-2] if x.dim() >= h.dim() else h.shape[:-2]),
              size(x.shape[-2], h.shape[-2]), size(x.shape[-1], h.shape[-1]))
    if x.dim() > 2 and h.dim() > 2 and x.shape[:-2] != h.shape[:-2]:
        raise GbfirError(2, "conv2d: batched operands must have the same batch shape")
    if out is None:
        out = torch.empty(oshape, dtype=_out_dtype(x, h), device=x.device)
    _lib.check(_lib.load().gbfir_conv2d(_buf2d(out, "conv2d out"), _buf2d(x, "conv2d x"), _buf2d(h, "conv2d h"),
                                        m, _stream()))
    return out


def _along_last(x: torch.Tensor, dim: int):
    """x with `dim` moved last and made unit-stride, and the inverse move for the result."""
    d = dim % max(x.dim(), 1)
    if d == x.dim() - 1:
        return _prep_in(x, "x"), (lambda y: y)
    return x.movedim(d, -1).contiguous(), (lambda y: y.movedim(-1, d))


def _updown(x: torch.Tensor, n: int, dim: int, up: bool) -> torch.Tensor:
    what = "upsample" if up else "downsample"
    if n < 1:
        raise GbfirError(1, f"{what}: the rate must be >= 1")
    xl, back = _along_last(_rows(x, what), dim)
    N = xl.shape[-1]
    olen = N * n if up else (N + n - 1) // n
    out = torch.empty(*xl.shape[:-1], olen, dtype=xl.dtype, device=xl.device)
    fn = _lib.load().gbfir_upsample if up else _lib.load().gbfir_downsample
    _lib.check(fn(_buf(out, f"{what} out"), _buf(xl, f"{what} x"), n, _stream()))
    return back(out)


def upsample(x: torch.Tensor, n: int, dim: int = -1) -> torch.Tensor:
    """MatX upsample(x, dim, n): n-fold zero stuffing along `dim`, x[i/n] where n divides i
    (operators/updownsample.h:254-257); the result has n times the samples."""
    return _updown(x, n, dim, True)


def downsample(x: torch.Tensor, n: int, dim: int = -1) -> torch.Tensor:
    """MatX downsample(x, dim, n): every n-th sample along `dim`, ceil(N/n) of them
    (operators/updownsample.h:268-279, a strided slice)."""
    return _updown(x, n, dim, False)


def upfirdn(x: torch.Tensor, h: torch.Tensor, up: int = 1, down: int = 1, mode=MATX_C_MODE_FULL, *,
            out: torch.Tensor | None = None) -> torch.Tensor:
    """downsample(conv1d(upsample(x, up), h, mode), down) along the last dimension in one
    polyphase pass (gbfir_upfirdn): out[m] = sum_k x[k] h[start + m*down - k*up], start the
    conv1d mode offset of the upsampled length; no zero-stuffed signal is formed and no
    discarded output is computed.  h is 1-D."""
    m = _mode(mode)
    if up < 1 or down < 1:
        raise GbfirError(1, "upfirdn: up and down must be >= 1")
    double = _out_dtype(x, h) in (torch.float64, torch.complex128)
    x = _prep_in(_cast(x, double), "upfirdn x")
    h = _prep_in(_cast(h, double), "upfirdn h")
    if h.dim() != 1:
        raise GbfirError(2, "upfirdn: the filter must be 1-D")
    olen = -(-_olen(m, x.shape[-1] * up, h.shape[0]) // down)
    if out is None:
        out = torch.empty(*x.shape[:-1], olen, dtype=_out_dtype(x, h), device=x.device)
    _lib.check(_lib.load().gbfir_upfirdn(_buf(out, "upfirdn out"), _buf(x, "upfirdn x"), _buf(h, "upfirdn h"),
                                         up, down, m, 0, _stream()))
    return out


def iir_filter(x: torch.Tensor, h_rec, h_nonrec, *, out: torch.Tensor | None = None) -> torch.Tensor:
    """MatX filter(x, h_rec, h_nonrec) along the last dimension (transforms/filter.h:159-188):
    with no recursive coefficients conv1d(x, h_nonrec, SAME); else the causal recurrence
    y[n] = sum_j h_nonrec[j] x[n-j] + sum_k h_rec[k] y[n-1-k] from a zero state.  At most 4
    coefficients of each kind (host sequences, as MatX's cuda::std::array arguments)."""
    import numpy as np
    a = np.asarray(h_rec.cpu() if isinstance(h_rec, torch.Tensor) else h_rec).ravel()
    b = np.asarray(h_nonrec.cpu() if isinstance(h_nonrec, torch.Tensor) else h_nonrec).ravel()
    x = _prep_in(x, "filter x")
    dbl = x.dtype in (torch.float64, torch.complex128)
    cc = np.iscomplexobj(a) or np.iscomplexobj(b)
    cdt = (np.complex128 if dbl else np.complex64) if cc else (np.float64 if dbl else np.float32)
    ac, bc = np.ascontiguousarray(a.astype(cdt)), np.ascontiguousarray(b.astype(cdt))
    coef_dt = {np.float32: _lib.GBFIR_F32, np.complex64: _lib.GBFIR_C64, np.float64: _lib.GBFIR_F64,
               np.complex128: _lib.GBFIR_C128}[cdt]
    odt = x.dtype
    if cc and not x.is_complex():
        odt = torch.complex128 if dbl else torch.complex64
    if out is None:
        out = torch.empty(x.shape, dtype=odt, device=x.device)
    lib = _lib.load()
    ob = _buf(out, "filter out")
    ws = None
    nbytes = 0
    if a.size:
        nbytes = int(lib.gbfir_filter_workspace_size(ob.batch, x.shape[-1], _DT[odt]))
        ws = torch.empty(max(nbytes, 16), dtype=torch.uint8, device=x.device)
    _lib.check(lib.gbfir_filter(ob, _buf(x, "filter x"), ac.ctypes.data if a.size else None, int(a.size),
                                bc.ctypes.data, int(b.size), coef_dt, ws.data_ptr() if ws is not None else None,
                                nbytes, _stream()))
    return out


filter = iir_filter  # MatX's name for it


def resample_out_len(n: int, up: int, down: int) -> int:
    """ceil(n*up/down) with the unreduced up/down (resample_poly.h:67-79)."""
    s = n * up
    return s // down + (1 if s % down else 0)


def resample_poly(x: torch.Tensor, h: torch.Tensor, up: int, down: int, *, precision="fp32",
                  out: torch.Tensor | None = None) -> torch.Tensor:
    """Polyphase resampler (MatX resample_poly, scipy centring and gain).

    ``precision`` selects the tap-contraction form: "fp32" (CUDA cores),
    "bf16", "fp16" or "bf16x3" (tcgen05 tensor cores, FP32 accumulate).
    """
    lib = _lib.load()
    double = _out_dtype(x, h) in (torch.float64, torch.complex128)
    x = _prep_in(_cast(x, double), "resample_poly x")
    h = _prep_in(_cast(h, double), "resample_poly h")
    if h.dim() != 1:
        raise GbfirError(2, "resample_poly: currently only support 1D filters")
    if up <= 0 or down <= 0:
        raise GbfirError(1, "resample_poly: up and down must be positive")
    olen = resample_out_len(x.shape[-1], up, down)
    if out is None:
        out = torch.empty(*x.shape[:-1], olen, dtype=_out_dtype(x, h), device=x.device)
    _lib.check(lib.gbfir_resample_poly(_buf(out, "resample_poly out"), _buf(x, "resample_poly x"),
                                       _buf(h, "resample_poly h"), int(up), int(down), _prec(precision),
                                       _stream()))
    return out


def channelize_poly(x: torch.Tensor, h: torch.Tensor, num_channels: int, decimation_factor: int, *,
                    precision="fp32", out: torch.Tensor | None = None) -> torch.Tensor:
    """Polyphase channelizer, output [..., ceil(N/D), M] complex (channelize_poly.h:81-88)."""
    lib = _lib.load()
    double = _out_dtype(x, h) in (torch.float64, torch.complex128)
    x = _prep_in(_cast(x, double), "channelize_poly x")
    h = _prep_in(_cast(h, double), "channelize_poly h")
    M, D = int(num_channels), int(decimation_factor)
    if h.dim() != 1:
        raise GbfirError(2, "channelize_poly: currently only support 1D filters")
    if M <= 0 or D <= 0 or D > M:
        raise GbfirError(1, "channelize_poly: need 0 < decimation_factor <= num_channels")
    T = (x.shape[-1] + D - 1) // D
    odt = torch.complex128 if double else torch.complex64
    if out is None:
        out = torch.empty(*x.shape[:-1], T, M, dtype=odt, device=x.device)
    flat = out.view(*out.shape[:-2], T * M)
    _lib.check(lib.gbfir_channelize_poly(_buf(flat, "channelize_poly out"), _buf(x, "channelize_poly x"),
                                         _buf(h, "channelize_poly h"), M, D, _prec(precision), _stream()))
    return out
