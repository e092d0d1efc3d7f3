#!/usr/bin/env python3
"""Regenerate the golden fixtures in tests/golden/ from the MatX reference.

Run once in a container where the MatX source tree is mounted (the tree the oracle's
Makefile recipe names, or MATX_REF=...):

    python tests/golden/make_golden.py

Sources, all from the reference's own test suite:

* conv.npz, conv2d.npz, resample.npz, channelize.npz — produced by the reference's
  numpy/scipy generator classes (test/test_vectors/generators/00_transforms.py):
  ``conv_operators`` (:14-36), ``conv2d_operators`` (:38-52), ``resample_poly_operators`` (:119-158),
  ``channelize_poly_operators.channelize`` (:194-247) and
  ``.channelize_oversampled`` (:249-334).  Case shapes follow the reference's
  tests (test/00_transform/ConvCorr.cu:491-835, ResamplePoly.cu:304-529,
  ChannelizePoly.cu:300-370,1141-1343); the few reference shapes whose arrays run
  to megabytes are scaled down in length, keeping their filter length and rates.
* harris2003.npz — the maximally decimated known-answer test whose filter,
  input and output are written inline in test/00_transform/ChannelizePoly.cu:820-1100
  (M = 10), parsed from that file as text.
* grad_refs.npz — adjoints of conv1d (all modes) and resample_poly composed from MatX's
  own HostExecutor corr / resample_poly in double (oracle/_ref), on seeded inputs.
* harris2003_oversampled.npz — the M=40, D=28 oversampled case: input and golden
  output from test/test_vectors/channelize_poly/harris2003_oversampled_testvector.bin,
  filter from the generator's remez design (00_transforms.py:336-397).

The fixtures are committed; nothing at test time reads the reference tree.
"""
import importlib
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
import oracle  # noqa: E402

REF = oracle.matx_root()
if REF is None:
    raise SystemExit("make_golden.py: no MatX source tree found (set MATX_REF)")
GEN = os.path.join(REF, "test", "test_vectors", "generators")


def _gen():
    sys.path.insert(0, GEN)
    return importlib.import_module("00_transforms")


def make_conv(T):
    out = {}
    # ConvCorr.cu:491-835 — N=256 against L=16 and L=15, float and complex; swap cases.
    cases = [("f32", np.float32, 256, 16), ("f32", np.float32, 256, 15),
             ("c64", np.complex64, 256, 16), ("c64", np.complex64, 256, 15),
             ("f64", np.float64, 256, 15), ("c128", np.complex128, 256, 16),
             ("f32", np.float32, 16, 256), ("c64", np.complex64, 15, 256),
             ("f32", np.float32, 4096, 209)]  # long case of ConvCorr.cu:61-63, shortened
    for i, (tag, dt, n, l) in enumerate(cases):
        g = T.conv_operators(dt, [n, l])
        r = g.conv()
        r = g.corr()
        r = g.corr_swap()
        key = f"c{i}_{tag}_{n}_{l}"
        for k in ("a_op", "b_op", "conv_full", "conv_same", "conv_valid", "corr", "corr_swap"):
            out[f"{key}__{k}"] = np.asarray(r[k])
    np.savez_compressed(os.path.join(HERE, "conv.npz"), **out)
    return len(cases)


def make_conv2d(T):
    out = {}
    # ConvCorr.cu:520-830 — a 256 x 128 image against 16 x 8 (even) and 15 x 7 (odd) filters,
    # float and complex; the swapped call conv2d(filter, image) (:783-787) uses the same vectors.
    cases = [("f32", np.float32, 16, 8), ("c64", np.complex64, 15, 7), ("f64", np.float64, 16, 8)]
    for i, (tag, dt, b0, b1) in enumerate(cases):
        g = T.conv2d_operators(dt, [256, 128, b0, b1])
        r = g.conv2d()
        key = f"d{i}_{tag}_{b0}x{b1}"
        for k in ("a_op", "b_op", "conv_full", "conv_same", "conv_valid"):
            out[f"{key}__{k}"] = np.asarray(r[k])
    np.savez_compressed(os.path.join(HERE, "conv2d.npz"), **out)
    return len(cases)


def make_resample(T):
    out = {}
    # ResamplePoly.cu:316-328 (odd random filters), :381-393 (even), :440-451 (default
    # scipy Kaiser filter).  Long signals are shortened; taps and rates are the reference's.
    rand_cases = [(3500, 62501, 384, 3125), (3501, 137, 384, 3125), (1173, 173, 7, 1),
                  (7173, 173, 1, 7), (2173, 151, 1, 16), (1, 3, 3, 1),
                  (3501, 62500, 384, 3125), (3104, 138, 384, 3125), (1173, 174, 7, 1),
                  (7173, 174, 1, 7), (2735, 150, 1, 16), (1, 2, 3, 1),
                  (1000, 61, 3, 2), (1000, 101, 4, 5), (1200, 3201, 160, 147)]
    default_cases = [(350, 384, 3125), (1173, 7, 1), (7173, 1, 7), (3500, 1, 16),
                     (3501, 1, 16), (15, 1, 16), (2000, 3, 2), (2000, 4, 5), (1500, 160, 147)]
    n = 0
    for tag, dt in (("f32", np.float32), ("c64", np.complex64), ("f64", np.float64)):
        for (a_len, f_len, up, down) in rand_cases:
            if dt is not np.float32 and (f_len > 10000 or a_len > 3000):
                continue
            if dt is np.float64 and (a_len, f_len) not in ((1000, 61), (1200, 3201), (1173, 174), (1, 3)):
                continue
            g = T.resample_poly_operators(dt, [a_len, f_len, up, down])
            r = g.resample()
            key = f"r{n}_{tag}_{a_len}_{f_len}_{up}_{down}"
            out[f"{key}__a"] = r["a"]
            out[f"{key}__h"] = r["filter_random"]
            out[f"{key}__y"] = np.asarray(r["b_random"])
            out[f"{key}__updown"] = np.array([up, down])
            n += 1
        for (a_len, up, down) in default_cases:
            if dt is not np.float32 and (max(up, down) > 1000 or a_len > 2500):
                continue
            if dt is np.float64 and (up, down) not in ((3, 2), (160, 147)):
                continue
            g = T.resample_poly_operators(dt, [a_len, 1, up, down])
            r = g.resample()
            key = f"d{n}_{tag}_{a_len}_{up}_{down}"
            out[f"{key}__a"] = r["a"]
            out[f"{key}__h"] = r["filter_default"]
            out[f"{key}__y"] = np.asarray(r["b_default"])
            out[f"{key}__updown"] = np.array([up, down])
            n += 1
    np.savez_compressed(os.path.join(HERE, "resample.npz"), **out)
    return n


def make_channelize(T):
    out = {}
    # ChannelizePoly.cu:311-330 (maximally decimated, unaligned filter lengths; long
    # signals shortened) and :1141-1343 (oversampled integer and rational D).
    md = [(2500, 170, 10), (2500, 187, 11), (1800, 120, 2), (1800, 120, 3),
          (1800, 5 * 180 + 33, 180), (1810, 5 * 181 + 17, 181), (2000, 41 * 8 + 4, 8),
          (2000, 41 * 9 + 8, 9), (2000, 301 * 13 + 3, 13), (2002, 301 * 14 + 4, 14),
          (3000, 32 * 16, 32), (3000, 40 * 16, 40), (4096, 64 * 8, 64), (4096, 256 * 4, 256),
          (1000, 7, 1)]
    ov = [(3000, 180, 40, 28), (1000, 97, 16, 12), (2000, 64, 16, 8), (500, 33, 9, 4),
          (2048, 256, 64, 48), (3001, 300, 32, 24), (777, 50, 5, 3)]
    n = 0
    for tag, dt in (("c64", np.complex64), ("c128", np.complex128)):
        for (a_len, f_len, m) in md:
            if dt is np.complex128 and (a_len, m) not in ((2500, 10), (1800, 3), (1000, 1), (2000, 8)):
                continue
            g = T.channelize_poly_operators(dt, [a_len, f_len, m, m])
            r = g.channelize()
            key = f"m{n}_{tag}_{a_len}_{f_len}_{m}_{m}"
            out[f"{key}__a"] = r["a"]
            out[f"{key}__h"] = r["filter_random"]
            out[f"{key}__y"] = r["b_random"].astype(dt)
            if a_len <= 2500:
                out[f"{key}__y_hreal"] = r["b_random_hreal"].astype(dt)
            out[f"{key}__md"] = np.array([m, m])
            n += 1
        for (a_len, f_len, m, d) in ov:
            if dt is np.complex128 and (a_len, m) not in ((1000, 16), (500, 9)):
                continue
            g = T.channelize_poly_operators(dt, [a_len, f_len, m, d])
            r = g.channelize_oversampled()
            key = f"o{n}_{tag}_{a_len}_{f_len}_{m}_{d}"
            out[f"{key}__a"] = r["a"]
            out[f"{key}__h"] = r["filter_random"]
            out[f"{key}__y"] = r["b_random"].astype(dt)
            if a_len <= 1000:
                out[f"{key}__y_hreal"] = r["b_random_hreal"].astype(dt)
            out[f"{key}__md"] = np.array([m, d])
            n += 1
    # batched case, ChannelizePoly.cu:664-726 (batch dims [2, 3])
    g = T.channelize_poly_operators(np.complex64, [400, 64, 8, 8, 2, 3])
    r = g.channelize()
    out["batched__a"] = r["a"]
    out["batched__h"] = r["filter_random"]
    out["batched__y"] = r["b_random"].astype(np.complex64)
    out["batched__md"] = np.array([8, 8])
    np.savez_compressed(os.path.join(HERE, "channelize.npz"), **out)
    return n + 1


def _parse_vec(text, name):
    m = re.search(r"const std::vector<[^>]*>+\s+" + name + r"\s*=\s*\{(.*?)\};", text, re.S)
    body = m.group(1)
    nums = [float(v) for v in re.findall(r"[-+]?\d+\.\d+e[-+]\d+", body)]
    return np.array(nums)


def make_harris():
    src = os.path.join(REF, "test", "00_transform", "ChannelizePoly.cu")
    with open(src) as f:
        text = f.read()
    h = _parse_vec(text, "filter")
    x = _parse_vec(text, "input")
    yv = _parse_vec(text, "output")
    y = yv[0::2] + 1j * yv[1::2]
    M = 10
    T_out = x.size // M
    # output[chan * T + k] is channel-major; store as [T, M] (MatX layout)
    y = y.reshape(M, T_out).T
    np.savez_compressed(os.path.join(HERE, "harris2003.npz"), h=h, x=x, y=y, M=np.array([M]))

    T = _gen()
    g = T.harris2003_oversampled_operators(np.complex128, [5600])
    r = g.channelize()
    np.savez_compressed(os.path.join(HERE, "harris2003_oversampled.npz"),
                        h=r["filter"], x=r["a"], y=r["b_golden"], MD=np.array([40, 28]))
    return h.size, x.size, y.shape


def make_grad_refs():
    """Gradients composed from MatX's own host operators (oracle/_ref, FP64):
    conv1d:   dx = corr(gy, h, FULL)[L-1-start : L-1-start+N]
              dh[f] = sum_b corr(x_b, gy_b, FULL)[Ly-1+start-f]
    resample: dx = (up/down) * resample_poly(gy, reverse(h), down, up)[:N]  (odd L)
    for y = conv1d(x, h, mode) / resample_poly(x, h, up, down) and a seeded gy."""
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    import oracle
    oracle.build(ref=True)
    rng = np.random.default_rng(77)
    B, N, L = 4, 1000, 127
    x = rng.uniform(-1, 1, (B, N))
    h = rng.standard_normal(L) / np.sqrt(L)
    out = {"x": x, "h": h}
    for mode, name in ((0, "full"), (1, "same"), (2, "valid")):
        Ly = N + L - 1 if mode == 0 else (N if mode == 1 else N - L + 1)
        start = 0 if mode == 0 else ((L - 1) // 2 if mode == 1 else L - 1)
        gy = rng.standard_normal((B, Ly))
        cf = oracle.ref_conv1d(gy, h, 0, is_corr=True, double=True)
        dx = cf[:, L - 1 - start: L - 1 - start + N]
        dh = np.zeros(L)
        for b in range(B):
            c2 = oracle.ref_conv1d(x[b], gy[b], 0, is_corr=True, double=True)[0]
            dh += c2[Ly - 1 + start - np.arange(L)]
        out[f"conv_{name}__gy"] = gy
        out[f"conv_{name}__dx"] = dx
        out[f"conv_{name}__dh"] = dh
    for up, down in ((3, 2), (2, 3), (4, 5)):
        Ly = (N * up + down - 1) // down
        gy = rng.standard_normal((B, Ly))
        t = oracle.ref_resample_poly(gy, h[::-1].copy(), down, up, double=True)
        out[f"rs_{up}_{down}__gy"] = gy
        out[f"rs_{up}_{down}__dx"] = (up / down) * t[:, :N]
    np.savez_compressed(os.path.join(HERE, "grad_refs.npz"), **out)
    return len(out)


def main():
    print("grad refs", make_grad_refs())
    T = _gen()
    print("conv cases", make_conv(T))
    print("conv2d cases", make_conv2d(T))
    print("resample cases", make_resample(T))
    print("channelize cases", make_channelize(T))
    print("harris", make_harris())


if __name__ == "__main__":
    main()
