"""CPU-side checks of the C-ABI library: it loads, exports every symbol the
header declares, and its host-side validation returns the MatX error classes
before any device work (fake, never-dereferenced pointers)."""
import ctypes
import math
import os
import re

import pytest

from conftest import ROOT


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__ as g
    from matx_gb300 import build
    build.build()
    from matx_gb300 import _lib
    return _lib.load()


def header_functions():
    names = []
    for fn in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if not fn.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", fn)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"\b(gbfir_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = header_functions()
    for must in ("gbfir_conv1d", "gbfir_resample_poly", "gbfir_channelize_poly"):
        assert must in names


def test_every_header_symbol_is_exported(lib):
    from matx_gb300 import _lib
    bound = {n for n, _, _ in _lib.SIGNATURES}
    for name in header_functions():
        assert hasattr(lib, name), f"{name} not exported"
        assert name in bound, f"{name} has no ctypes signature"


def test_status_strings(lib):
    assert lib.gbfir_status_string(0) == b"success"
    assert lib.gbfir_status_string(2) == b"invalid dimension"
    assert lib.gbfir_version() >= 100


FAKE = 0x100000  # aligned, never dereferenced: validation fails first


def buf(n, batch=1, dtype=1, stride=None, ptr=FAKE):
    from matx_gb300._lib import Buf
    return Buf(ptr, batch, n, n if stride is None else stride, dtype)


def last(lib):
    return lib.gbfir_last_error().decode()


def test_resample_validation(lib):
    # output length must be ceil(N*up/down) with unreduced up/down (resample_poly.h:318-320)
    assert lib.gbfir_resample_poly(buf(100), buf(67), buf(61, dtype=0), 3, 2, 0, None) == 2
    assert "output size mismatch" in last(lib)
    assert lib.gbfir_resample_poly(buf(101), buf(67), buf(61, dtype=0), 0, 2, 0, None) == 1
    assert lib.gbfir_resample_poly(buf(101), buf(67), buf(61, dtype=0), 3, -1, 0, None) == 1
    # batch mismatch
    assert lib.gbfir_resample_poly(buf(101, batch=2), buf(67, batch=3), buf(61, dtype=0), 3, 2, 0, None) == 2
    # null pointer
    assert lib.gbfir_resample_poly(buf(101, ptr=0), buf(67), buf(61, dtype=0), 3, 2, 0, None) == 7
    # complex input needs complex output
    assert lib.gbfir_resample_poly(buf(101, dtype=0), buf(67), buf(61, dtype=0), 3, 2, 0, None) == 4
    # misaligned complex pointer
    assert lib.gbfir_resample_poly(buf(101, ptr=FAKE + 4), buf(67), buf(61, dtype=0), 3, 2, 0, None) == 8
    # unknown precision
    assert lib.gbfir_resample_poly(buf(101), buf(67), buf(61, dtype=0), 3, 2, 9, None) == 1
    # filter must be one row
    assert lib.gbfir_resample_poly(buf(101), buf(67), buf(61, batch=2, dtype=0), 3, 2, 0, None) == 2


def test_conv_validation(lib):
    assert lib.gbfir_conv1d(buf(100, dtype=0), buf(64, dtype=0), buf(16, dtype=0), 0, 0, 0, None) == 3
    assert lib.gbfir_conv1d(buf(79, dtype=0), buf(64, dtype=0), buf(16, dtype=0), 3, 0, 0, None) == 1
    # SAME is max(N, L), VALID is max-min+1 — wrong sizes rejected
    assert lib.gbfir_conv1d(buf(63, dtype=0), buf(64, dtype=0), buf(16, dtype=0), 1, 0, 0, None) == 3
    assert lib.gbfir_conv1d(buf(48, dtype=0), buf(64, dtype=0), buf(16, dtype=0), 2, 0, 0, None) == 3
    # batch mismatch between operands and output
    assert lib.gbfir_conv1d(buf(79, batch=4, dtype=0), buf(64, batch=3, dtype=0), buf(16, dtype=0),
                            0, 0, 0, None) == 2
    # mixed precision operands
    assert lib.gbfir_conv1d(buf(79, dtype=0), buf(64, dtype=2), buf(16, dtype=0), 0, 0, 0, None) == 4


def test_conv_axis_validation(lib):
    # 4 blocks of [64][10], 16 taps: FULL needs 79 x 10 per block
    def f(o, i, h, mode=0, inner=10, si=10, so=10, prec=0):
        return lib.gbfir_conv1d_axis(o, i, h, inner, si, so, mode, 0, prec, None)
    x = lambda n=64, b=4, st=None: buf(n, batch=b, dtype=0, stride=n * 10 if st is None else st)
    h = buf(16, dtype=0)
    assert f(x(79), x(), h, mode=3) == 1
    assert f(x(80), x(), h) == 3
    assert f(x(79), x(), h, inner=0) == 1
    assert f(x(79), x(), h, si=0) == 1
    assert f(x(79), x(), buf(16, batch=4, dtype=0)) == 2
    assert f(x(79), x(b=3), h) == 2
    # output signals that would overlap: a step below the inner count, blocks too close
    assert f(x(79), x(), h, so=9) == 1
    assert f(x(79, st=779), x(), h) == 1
    # tensor-core forms are not built for the axis form
    assert f(x(79), x(), h, prec=1) == 5


def test_updown_validation(lib):
    assert lib.gbfir_upsample(buf(31, dtype=0), buf(10, dtype=0), 3, None) == 3
    assert lib.gbfir_upsample(buf(30, dtype=1), buf(10, dtype=0), 3, None) == 4
    assert lib.gbfir_downsample(buf(3, dtype=0), buf(10, dtype=0), 3, None) == 3
    assert lib.gbfir_downsample(buf(4, dtype=0), buf(10, dtype=0), 0, None) == 1
    # upfirdn: FULL of the 3x upsampled 64 samples with 16 taps is 207, then ceil(/2) = 104
    f = lambda o, mode=0, up=3, dn=2, prec=0: lib.gbfir_upfirdn(o, buf(64, dtype=0), buf(16, dtype=0), up, dn,
                                                               mode, 0 if prec == 0 else prec, None)
    assert f(buf(105, dtype=0)) == 3
    assert f(buf(97, dtype=0), mode=1) == 3        # SAME: ceil(192 / 2) = 96
    assert f(buf(104, dtype=0), up=0) == 1
    assert f(buf(104, dtype=0), mode=4) == 1
    assert f(buf(104, dtype=0), prec=1) == 5


def test_filter_validation(lib):
    a = (ctypes.c_float * 4)(0.4, -0.1, 0, 0)
    b = (ctypes.c_float * 4)(2.0, 1.0, 0, 0)
    f = lambda o, i, na=2, nb=2, cdt=0, ws=None, wsb=0: lib.gbfir_filter(o, i, a, na, b, nb, cdt, ws, wsb, None)
    x = buf(1000, batch=3, dtype=0)
    # ticket (16 B) + one flag per (row, block) rounded to 16 B + aggregate and inclusive states
    assert lib.gbfir_filter_workspace_size(3, 1000, 0) == 16 + 16 + 2 * 3 * 1 * 4 * 4
    assert lib.gbfir_filter_workspace_size(3, 8193, 1) == 16 + 32 + 2 * 3 * 2 * 4 * 8
    assert f(buf(999, batch=3, dtype=0), x) == 3
    assert f(buf(1000, batch=3, dtype=1), x) == 4           # real in, real taps -> real out
    assert f(buf(1000, batch=3, dtype=0), x, na=5) == 5
    assert f(buf(1000, batch=3, dtype=0), x, nb=0) == 1
    assert f(buf(1000, batch=3, dtype=0), x) == 9            # no workspace for the recursive form
    assert f(buf(1000, batch=3, dtype=0), x, ws=FAKE, wsb=47) == 9
    assert f(buf(3, dtype=0), buf(3, dtype=0), na=0, nb=4) == 3   # FIR-only: conv1d SAME size rule
    assert f(buf(1000, batch=3, dtype=2), x) == 4           # mixed precision


def test_conv_fft_validation(lib):
    f = lambda o, i, h, mode=0: lib.gbfir_conv1d_fft(o, i, h, mode, 0, None)
    assert f(buf(100, dtype=1), buf(64, dtype=1), buf(16, dtype=0)) == 3
    assert f(buf(79, dtype=1), buf(64, dtype=1), buf(16, dtype=0), mode=3) == 1
    assert f(buf(79, dtype=3), buf(64, dtype=3), buf(16, dtype=2)) == 5            # double: not built
    assert f(buf(79, dtype=1), buf(64, dtype=1), buf(16, batch=2, dtype=0)) == 5   # batched filter
    assert f(buf(20063, dtype=1), buf(12894, dtype=1), buf(7170, dtype=0)) == 5    # too many taps
    assert f(buf(79, dtype=1), buf(16, dtype=1), buf(64, dtype=0)) == 5            # signal shorter


def test_conv2d_validation(lib):
    from matx_gb300._lib import Buf2d
    img = lambda r, c, b=1, dt=0, bs=None: Buf2d(FAKE, b, r, c, r * c if bs is None else bs, c, dt)
    f = lambda o, i, h, mode=0: lib.gbfir_conv2d(o, i, h, mode, None)
    assert f(img(101, 100), img(90, 90), img(11, 11)) == 3              # FULL is 100 x 100
    assert f(img(100, 100), img(90, 90), img(11, 11), mode=4) == 1
    assert f(img(90, 90, dt=1), img(90, 90), img(11, 11), mode=1) == 4  # real operands, complex out
    assert f(img(90, 90), img(90, 90, b=2), img(11, 11), mode=1) == 2   # batch mismatch
    assert f(img(90, 90, b=2, bs=10), img(90, 90, b=2), img(11, 11), mode=1) == 1  # batch stride too short
    assert f(img(90, 65), img(90, 40), img(2, 65), mode=1) == 5         # filter wider than the image


def test_channelize_validation(lib):
    # D > M
    assert lib.gbfir_channelize_poly(buf(16 * 8), buf(128), buf(64, dtype=0), 8, 9, 0, None) == 1
    # output row must hold T*M
    assert lib.gbfir_channelize_poly(buf(16 * 8 + 1), buf(128), buf(64, dtype=0), 8, 8, 0, None) == 2
    # output must be complex even for real inputs
    assert lib.gbfir_channelize_poly(buf(128, dtype=0), buf(128, dtype=0), buf(64, dtype=0), 8, 8, 0, None) == 4
    assert lib.gbfir_channelize_poly(buf(128), buf(128), buf(64, dtype=0), 0, 1, 0, None) == 1


def test_resample_tile_hook(lib):
    assert lib.gbfir_set_resample_tile(3, 1, 1, 0) == 1
    assert lib.gbfir_set_resample_tile(2, 4, 1, 16) == 1
    assert lib.gbfir_set_resample_tile(2, 4, 1, 1) == 0
    assert lib.gbfir_set_resample_tile(2, 4, 1, 3) == 0   # the ring form
    assert lib.gbfir_set_resample_tile(0, 0, 0, 0) == 0


def test_package_refuses_cpu_tensors():
    import torch
    import matx_gb300 as mx
    with pytest.raises(ValueError):
        mx.resample_poly(torch.zeros(10, dtype=torch.complex64), torch.zeros(5), 3, 2)


def test_ragged_plan_validation(lib):
    from matx_gb300._lib import RaggedDesc, RaggedPlanInfo
    d = (RaggedDesc * 2)()
    d[0] = RaggedDesc(FAKE, FAKE, FAKE, 1000, 1500, 61, 3, 2, 0)
    d[1] = RaggedDesc(FAKE, FAKE, FAKE, 1000, 800, 101, 4, 5, 0)
    info = RaggedPlanInfo()
    n = lib.gbfir_ragged_plan(d, 2, None, ctypes.byref(info))
    assert n > 0 and info.num_tiles == n and info.shared_bytes > info.table_bytes >= 0
    d[1] = RaggedDesc(FAKE, FAKE, FAKE, 1000, 801, 101, 4, 5, 0)  # wrong out_len
    assert lib.gbfir_ragged_plan(d, 2, None, ctypes.byref(info)) == -2
    d[1] = RaggedDesc(FAKE, 0, FAKE, 1000, 800, 101, 4, 5, 0)  # null output
    assert lib.gbfir_ragged_plan(d, 2, None, ctypes.byref(info)) == -7
    d[1] = RaggedDesc(FAKE + 4, FAKE, FAKE, 1000, 800, 101, 4, 5, 0)  # misaligned complex input
    assert lib.gbfir_ragged_plan(d, 2, None, ctypes.byref(info)) == -8
    # work items cover every row of every signal exactly once, in runs of consecutive rows
    d[1] = RaggedDesc(FAKE, FAKE, FAKE, 100000, 80000, 101, 4, 5, 0)
    n = lib.gbfir_ragged_plan(d, 2, None, ctypes.byref(info))
    import numpy as np
    t = np.empty((n, 4), dtype=np.int64)
    assert lib.gbfir_ragged_plan(d, 2, t.ctypes.data_as(ctypes.c_void_p), ctypes.byref(info)) == n
    assert set(t[:, 0].tolist()) == {0, 1}
    for sig in (0, 1):
        runs = sorted((int(r0), int(nr)) for s_, r0, nr, _ in t if s_ == sig)
        assert runs[0][0] == 0 and all(nr > 0 for _, nr in runs)
        assert all(a[0] + a[1] == b[0] for a, b in zip(runs, runs[1:]))
    assert info.buffers in (1, 2) and info.window_elems > 0
    assert info.window_elems % 2 == 0 and info.table_bytes % 16 == 0   # 16-byte aligned buffers
    assert info.table_bytes + info.buffers * info.window_elems * 8 <= info.shared_bytes
    # a registered tile shape reaches the items of its rate and tap-length bucket
    assert lib.gbfir_ragged_tile_register(8, 10, 100, 2, 4, 2) == 0   # (4,5), taps 65..128
    n2 = lib.gbfir_ragged_plan(d, 2, None, ctypes.byref(info))
    t2 = np.empty((n2, 4), dtype=np.int64)
    lib.gbfir_ragged_plan(d, 2, t2.ctypes.data_as(ctypes.c_void_p), ctypes.byref(info))
    # (bit 16: the paired walk, set by the planner for 16-byte aligned signals)
    assert set((t2[t2[:, 0] == 1, 3] & 0xFFFF).tolist()) == {2 | (4 << 4) | (2 << 8)}
    assert set((t2[t2[:, 0] == 0, 3] & 0xFFFF).tolist()) == {0}
    assert all(int(v) & (1 << 16) for v in t2[:, 3])
    assert lib.gbfir_ragged_tile_register(4, 5, 100, 3, 4, 2) == 1     # rows per thread 1 or 2
    assert lib.gbfir_ragged_tile_clear() == 0
    # launch refuses a plan that does not come from the planner (before touching the device)
    bad = RaggedPlanInfo(n, 300 * 1024, 0, 1, 2, 0)
    assert lib.gbfir_ragged_resample(FAKE, 2, FAKE, ctypes.byref(bad), 0, FAKE, 256, None) == 1
    # tensor-core plans: items carry each signal's packed block geometry; the launch refuses a
    # plan made for another precision
    n3 = lib.gbfir_ragged_plan_prec(d, 2, 3, None, ctypes.byref(info))
    assert n3 > 0 and info.precision == 3 and info.window_elems in (32, 64)
    t3 = np.empty((n3, 4), dtype=np.int64)
    assert lib.gbfir_ragged_plan_prec(d, 2, 3, t3.ctypes.data_as(ctypes.c_void_p), ctypes.byref(info)) == n3
    assert set(t3[:, 0].tolist()) == {0, 1} and (t3[:, 3] > 0).all()
    assert lib.gbfir_ragged_resample(FAKE, 2, FAKE, ctypes.byref(info), 0, FAKE, 256, None) == 1
    assert lib.gbfir_ragged_plan_prec(d, 2, 9, None, ctypes.byref(info)) == -1


@pytest.mark.parametrize("updown", [(3, 2), (4, 5), (160, 147), (2, 1), (1, 7), (6, 4)])
@pytest.mark.parametrize("tma_store", [False, True])
def test_tuner_candidates_are_valid_tiles(lib, updown, tma_store):
    """Every tile the autotuner would time is one the library accepts (registration is
    host-only), the enumeration has no duplicates, and malformed tiles are refused."""
    from matx_gb300 import autotune
    up, down = updown
    cands = list(autotune.candidates(up, down, tma_store))
    assert cands and len(cands) == len(set(cands))
    try:
        for rq, wc, grp, nb in cands:
            assert lib.gbfir_resample_tile_register(up, down, 61, rq, wc, grp, nb) == 0, (rq, wc, grp, nb)
            assert (nb & 4 == 0) or tma_store
            g = math.gcd(up, down)
            assert (nb & 8 == 0) or (tma_store and (down // g * grp) % 2 == 0)
        for bad in ((3, 1, 4, 1), (1, 3, 4, 1), (4, 12, 4, 1), (1, 1, 65, 1), (1, 1, 4, 16), (1, 1, 4, 32),
                    (1, 17, 4, 1), (-1, 1, 4, 1)):
            assert lib.gbfir_resample_tile_register(up, down, 61, *bad) != 0, bad
        assert lib.gbfir_resample_tile_register(0, down, 61, 1, 1, 4, 1) != 0
        assert lib.gbfir_resample_tile_register(up, down, 0, 1, 1, 4, 1) != 0
    finally:
        assert lib.gbfir_resample_tile_clear() == 0


def test_tuner_cache_round_trip(tmp_path, monkeypatch):
    from matx_gb300 import autotune
    path = tmp_path / "sub" / "tiles.json"
    monkeypatch.setattr(autotune, "CACHE", str(path))
    assert autotune.load_cache() == {}
    ent = {"GB300|torch.complex64|torch.float32|3/2|L61|N1048576|B64":
           {"best": [4, 8, 20, 5], "best_ms": 0.37, "default_ms": 0.41}}
    autotune._save_cache(ent)
    assert autotune.load_cache() == ent
    assert not os.path.exists(str(path) + ".tmp")
    path.write_text("{not json")
    assert autotune.load_cache() == {}
