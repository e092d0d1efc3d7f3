"""CPU oracle for the direct-FIR path — TEST INFRASTRUCTURE ONLY.

Two CPU implementations live here, both used only as checkers (tests/,
``__graft_entry__.smoke()``) and as the timed CPU baseline (``bench.py``):

* ``liboracle.so`` — a plain-C restatement of MatX's HostExecutor algorithms
  (gbfir_oracle.c / oracle_impl.h), in float and double.  Builds anywhere with
  gcc (``make -C oracle``).
* ``_ref/libmatxref.so`` — MatX's own HostExecutor operators, compiled from the
  MatX headers by ``make -C oracle ref`` where those headers exist.  Used to pin
  the restatement to the reference on identical inputs.

The product library (``matx_gb300``) never imports this package.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
_REF = None

_i64 = ctypes.c_int64
_int = ctypes.c_int
_p = ctypes.c_void_p


def matx_root():
    """Root of the MatX source tree the reference build reads: ``$MATX_REF`` if set, else
    the default named by this directory's Makefile recipe (``MATX ?= ...``); None where no
    MatX headers are present (the GPU machine, any machine without the tree)."""
    root = os.environ.get("MATX_REF")
    if not root:
        try:
            for line in open(os.path.join(_HERE, "Makefile")):
                if line.replace(" ", "").startswith("MATX?="):
                    root = line.split("=", 1)[1].strip()
                    break
        except OSError:
            root = None
    if root and os.path.isdir(os.path.join(root, "include", "matx")):
        return root
    return None


def build(ref: bool = False) -> None:
    """Compile the C oracle (and MatX's host reference when ``ref`` and the MatX tree is
    present)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    root = matx_root() if ref else None
    if root:
        subprocess.run(["make", "-s", "-C", _HERE, "ref", f"MATX={root}"], check=True)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        for suf in ("_d", "_f"):
            getattr(L, "oracle_conv1d" + suf).argtypes = [
                _p, _p, _i64, _i64, _p, _i64, _i64, _i64, _int, _int, _int, _int, _int]
            getattr(L, "oracle_resample_poly" + suf).argtypes = [
                _p, _i64, _p, _i64, _i64, _p, _i64, _i64, _i64, _i64, _int, _int, _int]
            getattr(L, "oracle_channelize_poly" + suf).argtypes = [
                _p, _p, _i64, _i64, _p, _i64, _i64, _i64, _i64, _int, _int, _int]
            getattr(L, "oracle_resample_poly_bwd" + suf).argtypes = [
                _p, _p, _p, _i64, _p, _i64, _p, _i64, _i64, _i64, _i64, _int]
            getattr(L, "oracle_iir_filter" + suf).argtypes = [_p, _p, _i64, _i64, _p, _int, _p, _int, _int, _int]
            getattr(L, "oracle_conv2d" + suf).argtypes = [_p, _i64, _i64, _p, _i64, _i64, _i64, _p, _i64, _i64, _i64,
                                                        _i64, _int, _int, _int]
            getattr(L, "oracle_conv1d_bwd" + suf).argtypes = [
                _p, _p, _p, _i64, _p, _i64, _p, _i64, _i64, _int, _int]
        L.oracle_max_threads.restype = _int
        _LIB = L
    return _LIB


def ref_lib():
    """MatX HostExecutor library, or None where it was not built."""
    global _REF
    if _REF is None:
        path = os.path.join(_HERE, "_ref", "libmatxref.so")
        if not os.path.exists(path):
            return None
        R = ctypes.CDLL(path)
        R.matxref_conv1d.argtypes = [_int, _p, _p, _i64, _p, _i64, _i64, _int, _int, _int, _int]
        R.matxref_resample_poly.argtypes = [_int, _p, _i64, _p, _i64, _p, _i64, _i64, _i64, _i64, _int]
        R.matxref_channelize_poly.argtypes = [_int, _p, _p, _i64, _p, _i64, _i64, _i64, _i64, _int]
        _REF = R
    return _REF


def max_threads() -> int:
    return int(lib().oracle_max_threads())


def _prep(a, double: bool):
    a = np.asarray(a)
    cplx = np.iscomplexobj(a)
    if double:
        dt = np.complex128 if cplx else np.float64
    else:
        dt = np.complex64 if cplx else np.float32
    a = np.ascontiguousarray(a, dtype=dt)
    if a.ndim == 1:
        a = a[None, :]
    return a, cplx


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _suffix(double):
    return "_d" if double else "_f"


def conv1d(x, h, mode: int = 0, is_corr: bool = False, double: bool = True,
           nthreads: int = 1):
    """Direct conv1d/corr of every row of x with h (h 1-D or one row per x row)."""
    xs, xc = _prep(x, double)
    hs, hc = _prep(h, double)
    B, N = xs.shape
    L = hs.shape[1]
    h_bstride = L if hs.shape[0] > 1 else 0
    if mode == 0:
        out_len = N + L - 1
    elif mode == 1:
        out_len = max(N, L)
    else:
        out_len = max(N, L) - min(N, L) + 1
    oc = xc or hc
    odt = (np.complex128 if double else np.complex64) if oc else (np.float64 if double else np.float32)
    out = np.empty((B, out_len), dtype=odt)
    rc = getattr(lib(), "oracle_conv1d" + _suffix(double))(
        _ptr(out), _ptr(xs), N, N, _ptr(hs), h_bstride, L, B, mode, int(is_corr),
        int(xc), int(hc), nthreads)
    if rc:
        raise ValueError(f"oracle_conv1d failed ({rc})")
    return out


def resample_out_len(n: int, up: int, down: int) -> int:
    s = n * up
    return s // down + (1 if s % down else 0)


def resample_poly(x, h, up: int, down: int, double: bool = True, nthreads: int = 1):
    xs, xc = _prep(x, double)
    hs, hc = _prep(h, double)
    B, N = xs.shape
    L = hs.shape[1]
    out_len = resample_out_len(N, up, down)
    oc = xc or hc
    odt = (np.complex128 if double else np.complex64) if oc else (np.float64 if double else np.float32)
    out = np.empty((B, out_len), dtype=odt)
    rc = getattr(lib(), "oracle_resample_poly" + _suffix(double))(
        _ptr(out), out_len, _ptr(xs), N, N, _ptr(hs), L, B, up, down, int(xc), int(hc), nthreads)
    if rc:
        raise ValueError(f"oracle_resample_poly failed ({rc})")
    return out


def channelize_poly(x, h, M: int, D: int, double: bool = True, nthreads: int = 1):
    xs, xc = _prep(x, double)
    hs, hc = _prep(h, double)
    B, N = xs.shape
    L = hs.shape[1]
    T = (N + D - 1) // D
    out = np.empty((B, T, M), dtype=np.complex128 if double else np.complex64)
    rc = getattr(lib(), "oracle_channelize_poly" + _suffix(double))(
        _ptr(out), _ptr(xs), N, N, _ptr(hs), L, B, M, D, int(xc), int(hc), nthreads)
    if rc:
        raise ValueError(f"oracle_channelize_poly failed ({rc})")
    return out


def resample_poly_bwd(gy, x, h, up: int, down: int, nthreads: int = 1):
    """FP64 exact adjoint (dx, dh) of the real resampler."""
    gs, _ = _prep(gy, True)
    xs, _ = _prep(x, True)
    hs, _ = _prep(h, True)
    B, N = xs.shape
    L = hs.shape[1]
    dx = np.empty((B, N), dtype=np.float64)
    dh = np.empty((L,), dtype=np.float64)
    rc = lib().oracle_resample_poly_bwd_d(_ptr(dx), _ptr(dh), _ptr(gs), gs.shape[1],
                                          _ptr(xs), N, _ptr(hs), L, B, up, down, nthreads)
    if rc:
        raise ValueError(f"oracle_resample_poly_bwd failed ({rc})")
    return dx, dh


def conv1d_bwd(gy, x, h, mode: int, nthreads: int = 1):
    """FP64 exact adjoint (dx, dh) of the real direct conv1d."""
    gs, _ = _prep(gy, True)
    xs, _ = _prep(x, True)
    hs, _ = _prep(h, True)
    B, N = xs.shape
    L = hs.shape[1]
    dx = np.empty((B, N), dtype=np.float64)
    dh = np.empty((L,), dtype=np.float64)
    rc = lib().oracle_conv1d_bwd_d(_ptr(dx), _ptr(dh), _ptr(gs), gs.shape[1],
                                   _ptr(xs), N, _ptr(hs), L, B, mode, nthreads)
    if rc:
        raise ValueError(f"oracle_conv1d_bwd failed ({rc})")
    return dx, dh


def conv2d(x, h, mode: int = 0, double: bool = True):
    """MatX conv2d of images x [..., N1, M1] with h [N2, M2] (or one filter per image):
    the larger image by element count is the signal (transforms/conv.h:569-576)."""
    x = np.asarray(x)
    h = np.asarray(h)
    if h.shape[-2] * h.shape[-1] > x.shape[-2] * x.shape[-1]:
        x, h = h, x
    xc, hc = np.iscomplexobj(x), np.iscomplexobj(h)
    rt = np.float64 if double else np.float32
    ct = np.complex128 if double else np.complex64
    bshape = x.shape[:-2] if x.ndim >= h.ndim else h.shape[:-2]
    B = int(np.prod(bshape)) if len(bshape) else 1
    xs = np.ascontiguousarray(np.broadcast_to(x, tuple(bshape) + x.shape[-2:]).reshape(B, *x.shape[-2:]),
                              dtype=ct if xc else rt)
    hs = np.ascontiguousarray(h.reshape(-1, *h.shape[-2:]), dtype=ct if hc else rt)
    N1, M1 = xs.shape[-2:]
    N2, M2 = hs.shape[-2:]
    size = lambda a, b: (a + b - 1) if mode == 0 else (max(a, b) if mode == 1 else max(a, b) - min(a, b) + 1)
    ON, OM = size(N1, N2), size(M1, M2)
    out = np.empty((B, ON, OM), dtype=ct if (xc or hc) else rt)
    rc = getattr(lib(), "oracle_conv2d" + _suffix(double))(
        _ptr(out), ON, OM, _ptr(xs), N1 * M1, N1, M1, _ptr(hs), N2 * M2 if hs.shape[0] > 1 else 0, N2, M2, B,
        mode, int(xc), int(hc))
    if rc:
        raise ValueError(f"oracle_conv2d failed ({rc})")
    return out.reshape(tuple(bshape) + (ON, OM))


def iir_filter(x, h_rec, h_nonrec, double: bool = True):
    """MatX filter(x, h_rec, h_nonrec) on rows: conv1d SAME with h_nonrec when h_rec is
    empty (transforms/filter.h:185), else the causal recurrence
    y[n] = sum_j h_nonrec[j] x[n-j] + sum_k h_rec[k] y[n-1-k] (kernels/filter.cuh)."""
    a = np.asarray(h_rec)
    b = np.asarray(h_nonrec)
    if a.size == 0:
        return conv1d(x, b, 1, double=double)
    xs, xc = _prep(x, double)
    cc = np.iscomplexobj(a) or np.iscomplexobj(b)
    ct = (np.complex128 if double else np.complex64) if cc else (np.float64 if double else np.float32)
    ac, bc = np.ascontiguousarray(a.astype(ct)), np.ascontiguousarray(b.astype(ct))
    B, N = xs.shape
    oc = xc or cc
    if cc and not xc:
        xs = np.ascontiguousarray(xs.astype(np.complex128 if double else np.complex64))
        xc = True
    odt = (np.complex128 if double else np.complex64) if oc else (np.float64 if double else np.float32)
    out = np.empty((B, N), dtype=odt)
    rc = getattr(lib(), "oracle_iir_filter" + _suffix(double))(
        _ptr(out), _ptr(xs), N, B, _ptr(ac), a.size, _ptr(bc), b.size, int(xc), int(cc))
    if rc:
        raise ValueError(f"oracle_iir_filter failed ({rc})")
    return out


# ---- MatX HostExecutor (reference) wrappers ---------------------------------

def _kind_conv(xc, hc, double):
    if double:
        return 5 if (xc and hc) else (4 if xc else 3)
    return 2 if (xc and hc) else (1 if xc else 0)


def ref_conv1d(x, h, mode=0, is_corr=False, double=False, nthreads=1):
    R = ref_lib()
    if R is None:
        return None
    xs, xc = _prep(x, double)
    hs, hc = _prep(h, double)
    if hc and not xc:
        return None  # combination not instantiated
    B, N = xs.shape
    L = hs.shape[1]
    out_len = N + L - 1 if mode == 0 else (max(N, L) if mode == 1 else max(N, L) - min(N, L) + 1)
    oc = xc or hc
    odt = (np.complex128 if double else np.complex64) if oc else (np.float64 if double else np.float32)
    out = np.empty((B, out_len), dtype=odt)
    rc = R.matxref_conv1d(_kind_conv(xc, hc, double), _ptr(out), _ptr(xs), N, _ptr(hs), L, B,
                          mode, int(is_corr), int(hs.shape[0] > 1), nthreads)
    if rc:
        raise ValueError(f"matxref_conv1d failed ({rc})")
    return out


def ref_resample_poly(x, h, up, down, double=False, nthreads=1):
    R = ref_lib()
    if R is None:
        return None
    xs, xc = _prep(x, double)
    hs, hc = _prep(h, double)
    if hc and not xc:
        return None
    if double:
        kind = 4 if xc else 3
        if hc:
            return None
    else:
        kind = 2 if (xc and hc) else (1 if xc else 0)
    B, N = xs.shape
    L = hs.shape[1]
    out_len = resample_out_len(N, up, down)
    oc = xc or hc
    odt = (np.complex128 if double else np.complex64) if oc else (np.float64 if double else np.float32)
    out = np.empty((B, out_len), dtype=odt)
    rc = R.matxref_resample_poly(kind, _ptr(out), out_len, _ptr(xs), N, _ptr(hs), L, B, up, down, nthreads)
    if rc:
        raise ValueError(f"matxref_resample_poly failed ({rc})")
    return out


def ref_channelize_poly(x, h, M, D, double=False, nthreads=1):
    R = ref_lib()
    if R is None:
        return None
    xs, xc = _prep(x, double)
    hs, hc = _prep(h, double)
    if double:
        if not xc or hc:
            return None
        kind = 2
    elif not xc:
        if hc:
            return None
        kind = 3
    else:
        kind = 1 if hc else 0
    B, N = xs.shape
    L = hs.shape[1]
    T = (N + D - 1) // D
    out = np.empty((B, T, M), dtype=np.complex128 if double else np.complex64)
    rc = R.matxref_channelize_poly(kind, _ptr(out), _ptr(xs), N, _ptr(hs), L, B, M, D, nthreads)
    if rc:
        raise ValueError(f"matxref_channelize_poly failed ({rc})")
    return out
