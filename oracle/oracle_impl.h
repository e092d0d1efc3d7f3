/*
 * oracle_impl.h — body of the CPU oracle, instantiated once for double and
 * once for float by gbfir_oracle.c (T = scalar type, SUF = name suffix).
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of MatX's host
 * (HostExecutor) algorithms for the direct-FIR path.  It is the checker for the
 * CUDA library and the timed CPU baseline; the product never calls it.
 *
 * Complex data is interleaved (re, im) pairs.  The flags xc / hc say whether
 * the signal / taps are complex; the output is complex when either is.
 */

#define CAT_(a, b) a##b
#define CAT(a, b) CAT_(a, b)
#define FN(name) CAT(name, SUF)

/* ---------------------------------------------------------------------------
 * Direct conv1d / corr.
 * Follows include/matx/transforms/conv.h:226-289 (host direct conv: one output
 * per iteration, sum over f of signal[full_idx - f] * filter[f] with detail::madd,
 * include/matx/core/utils.h:165-210), the operand swap of conv.h:427-450 (the
 * longer operand is the signal), the SAME/VALID start offsets of conv.h:249-255,
 * and corr = conv1d(a, reverse(conj(b))) from include/matx/transforms/corr.h:67.
 * ------------------------------------------------------------------------- */
int FN(oracle_conv1d)(T *out, const T *x, int64_t x_bstride, int64_t N,
                      const T *h, int64_t h_bstride, int64_t L, int64_t B,
                      int mode, int is_corr, int xc, int hc, int nthreads) {
  if (N <= 0 || L <= 0 || B <= 0) return 1;
  const int oc = xc || hc;
  /* Logical operands after the corr transform: a = x, b[f] = corr ? conj(h[L-1-f]) : h[f]. */
  const int swap = N < L; /* conv.h:427: i1.Size < i2.Size -> signal = i2 */
  const int64_t sig_len = swap ? L : N;
  const int64_t fil_len = swap ? N : L;
  int64_t out_len, start = 0;
  if (mode == 0) {
    out_len = N + L - 1;
  } else if (mode == 1) {
    out_len = sig_len;
    start = (fil_len & 1) ? (fil_len - 1) / 2 : fil_len / 2 - 1;
  } else if (mode == 2) {
    out_len = sig_len - fil_len + 1;
    start = fil_len - 1;
  } else {
    return 2;
  }
  const int64_t total = B * out_len;
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads) if (nthreads > 1) schedule(static)
#endif
  for (int64_t abs_i = 0; abs_i < total; abs_i++) {
    const int64_t b = abs_i / out_len;
    const int64_t o = abs_i % out_len;
    const T *xr = x + b * x_bstride * (xc ? 2 : 1);
    const T *hr = h + b * h_bstride * (hc ? 2 : 1);
    const int64_t full_idx = o + start;
    T sr = 0, si = 0;
    for (int64_t f = 0; f < fil_len; f++) {
      const int64_t s = full_idx - f;
      if (s < 0 || s >= sig_len) continue;
      /* index of the x sample and the b sample feeding this product */
      const int64_t xi_idx = swap ? f : s;
      const int64_t bi_idx = swap ? s : f;
      T ar, ai, br, bi;
      if (xc) { ar = xr[2 * xi_idx]; ai = xr[2 * xi_idx + 1]; } else { ar = xr[xi_idx]; ai = 0; }
      const int64_t hidx = is_corr ? (L - 1 - bi_idx) : bi_idx;
      if (hc) { br = hr[2 * hidx]; bi = hr[2 * hidx + 1]; } else { br = hr[hidx]; bi = 0; }
      if (is_corr) bi = -bi;
      /* madd(ival, fval, sum): ival is the signal operand, fval the filter operand */
      T vr, vi, wr, wi;
      if (swap) { vr = br; vi = bi; wr = ar; wi = ai; } else { vr = ar; vi = ai; wr = br; wi = bi; }
      if (oc) {
        sr = sr + vr * wr;
        sr = sr - vi * wi;
        si = si + vi * wr;
        si = si + vr * wi;
      } else {
        sr = sr + vr * wr;
      }
    }
    if (oc) { out[2 * abs_i] = sr; out[2 * abs_i + 1] = si; } else { out[abs_i] = sr; }
  }
  return 0;
}

/* ---------------------------------------------------------------------------
 * Polyphase resampler.
 * Follows include/matx/transforms/resample_poly.h:212-281 (host impl: even
 * filters act as if a zero were prepended, centre tap (Lodd-1)/2, taps walked
 * with stride -up, result scaled by up) and resample_poly.h:299-354 (gcd
 * reduction; up==down after the reduction copies the input).  `up`/`down` here
 * are the caller's unreduced values; out_len must be ceil(N*up/down).
 * ------------------------------------------------------------------------- */
int FN(oracle_resample_poly)(T *out, int64_t out_len, const T *x,
                             int64_t x_bstride, int64_t N, const T *h,
                             int64_t L, int64_t B, int64_t up, int64_t down,
                             int xc, int hc, int nthreads) {
  if (up <= 0 || down <= 0 || N <= 0 || L <= 0 || B <= 0) return 1;
  const int64_t up_size = N * up;
  const int64_t expect = up_size / down + ((up_size % down) ? 1 : 0);
  if (out_len != expect) return 3;
  int64_t a = up, c = down;
  while (c) { int64_t t = a % c; a = c; c = t; }
  up /= a;
  down /= a;
  const int oc = xc || hc;
  if (up == 1 && down == 1) {
    for (int64_t b = 0; b < B; b++) {
      for (int64_t i = 0; i < N; i++) {
        const T *xr = x + b * x_bstride * (xc ? 2 : 1);
        if (oc) {
          out[2 * (b * out_len + i)] = xc ? xr[2 * i] : xr[i];
          out[2 * (b * out_len + i) + 1] = xc ? xr[2 * i + 1] : 0;
        } else {
          out[b * out_len + i] = xr[i];
        }
      }
    }
    return 0;
  }
  const int is_even = (L % 2) == 0;
  const int64_t flen = is_even ? L + 1 : L;
  const int64_t half = flen / 2;
  const int64_t central = (flen - 1) / 2;
  const int64_t max_in = N - 1;
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads) if (nthreads > 1) schedule(dynamic, 1)
#endif
  for (int64_t b = 0; b < B; b++) {
    const T *xr = x + b * x_bstride * (xc ? 2 : 1);
    T *orow = out + b * out_len * (oc ? 2 : 1);
    for (int64_t n = 0; n < out_len; n++) {
      const int64_t up_ind = n * down;
      const int64_t up_start = (up_ind > half) ? up_ind - half : 0;
      const int64_t up_end = (max_in * up < up_ind + half) ? max_in * up : up_ind + half;
      const int64_t x_start = (up_start + up - 1) / up;
      const int64_t x_end = up_end / up;
      int64_t h_ind = central + (up_ind - up * x_start);
      T ar = 0, ai = 0;
      for (int64_t i = x_start; i <= x_end; i++) {
        if (!is_even || h_ind > 0) {
          const int64_t fi = is_even ? h_ind - 1 : h_ind;
          const T vr = xc ? xr[2 * i] : xr[i];
          const T vi = xc ? xr[2 * i + 1] : 0;
          const T wr = hc ? h[2 * fi] : h[fi];
          const T wi = hc ? h[2 * fi + 1] : 0;
          if (oc) {
            /* accum += in_val * filter(fi): complex product, then add */
            T pr, pi;
            if (xc && hc) { pr = vr * wr - vi * wi; pi = vr * wi + vi * wr; }
            else if (xc) { pr = vr * wr; pi = vi * wr; }
            else { pr = vr * wr; pi = vr * wi; }
            ar = ar + pr;
            ai = ai + pi;
          } else {
            ar = ar + vr * wr;
          }
        }
        h_ind -= up;
      }
      const T scale = (T)up;
      if (oc) { orow[2 * n] = ar * scale; orow[2 * n + 1] = ai * scale; }
      else { orow[n] = ar * scale; }
    }
  }
  return 0;
}

/* ---------------------------------------------------------------------------
 * Polyphase channelizer (maximally decimated D == M and oversampled D < M).
 * Follows include/matx/transforms/channelize_poly.h:858-1029 (host impl):
 * per-branch direct FIR with the h_skip / available_taps rules, the oversampled
 * branch remap r' = (c + M - D) mod M and phase rotation (c + t*D) mod M, the
 * complex multiply-accumulate order of HostChannelizeCmac (:243-270), then an
 * O(M^2) unnormalised positive-sign DFT with double twiddles cast to the
 * accumulator type (HostTwiddle, :320-329).  Output is [B][T][M] complex.
 * ------------------------------------------------------------------------- */
int FN(oracle_channelize_poly)(T *out, const T *x, int64_t x_bstride,
                               int64_t N, const T *h, int64_t L, int64_t B,
                               int64_t M, int64_t D, int xc, int hc,
                               int nthreads) {
  if (M <= 0 || D <= 0 || D > M || N <= 0 || L <= 0 || B <= 0) return 1;
  const int64_t T_out = (N + D - 1) / D;
  const int64_t P = (L + M - 1) / M;
  const int fc = xc || hc; /* filtering accumulator is complex */
  T *tw = (T *)malloc(sizeof(T) * 2 * (size_t)(M * M));
  if (!tw) return 4;
  const double pi = 3.141592653589793238462643383279502884;
  for (int64_t ch = 0; ch < M; ch++) {
    for (int64_t br = 0; br < M; br++) {
      const double arg = 2.0 * pi * (double)ch * (double)br / (double)M;
      tw[2 * (ch * M + br)] = (T)cos(arg);
      tw[2 * (ch * M + br) + 1] = (T)sin(arg);
    }
  }
  const int64_t total = B * T_out;
  int err = 0;
#ifdef _OPENMP
#pragma omp parallel num_threads(nthreads) if (nthreads > 1)
#endif
  {
    T *filt = (T *)malloc(sizeof(T) * 2 * (size_t)M);
    if (!filt) {
#ifdef _OPENMP
#pragma omp atomic write
#endif
      err = 4;
    } else {
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
      for (int64_t it = 0; it < total; it++) {
        const int64_t b = it / T_out;
        const int64_t t = it % T_out;
        const T *xr = x + b * x_bstride * (xc ? 2 : 1);
        for (int64_t branch = 0; branch < M; branch++) {
          T ar = 0, ai = 0;
          int64_t h_ind = branch, sample = 0, niter = 0;
          if (D == M) {
            const int64_t s = M - 1 - branch;
            sample = s + t * M;
            int64_t h_skip = 0;
            if (sample >= N) { h_skip = 1; sample -= M; }
            int64_t avail = P;
            if (P > 0 && ((P - 1) * M + branch) >= L) avail--;
            if (avail > h_skip && (t + 1) > h_skip) {
              niter = (avail - h_skip < t + 1 - h_skip) ? avail - h_skip : t + 1 - h_skip;
              h_ind = branch + h_skip * M;
            }
          } else {
            const int64_t rr = (branch + M - D) % M;
            const int64_t s = M - 1 - rr;
            const int64_t last = t * D + D - 1;
            if (last >= s) {
              const int64_t A = last - s;
              sample = last - (A % M);
              const int64_t causal = A / M + 1;
              const int64_t phase = (branch + t * D) % M;
              int64_t h_skip = 0;
              if (sample >= N) { h_skip = 1; sample -= M; }
              int64_t avail = P;
              if (P > 0 && ((P - 1) * M + phase) >= L) avail--;
              if (avail > h_skip && causal > h_skip) {
                niter = (avail - h_skip < causal - h_skip) ? avail - h_skip : causal - h_skip;
                h_ind = phase + h_skip * M;
              }
            }
          }
          for (int64_t i = 0; i < niter; i++) {
            const T vr = xc ? xr[2 * sample] : xr[sample];
            const T vi = xc ? xr[2 * sample + 1] : 0;
            const T wr = hc ? h[2 * h_ind] : h[h_ind];
            const T wi = hc ? h[2 * h_ind + 1] : 0;
            if (xc && hc) {
              ar = wr * vr + ar;
              ar = -(wi * vi) + ar;
              ai = wr * vi + ai;
              ai = wi * vr + ai;
            } else if (xc) {
              ar = wr * vr + ar;
              ai = wr * vi + ai;
            } else if (hc) {
              ar = wr * vr + ar;
              ai = wi * vr + ai;
            } else {
              ar += wr * vr;
            }
            h_ind += M;
            sample -= M;
          }
          filt[2 * branch] = ar;
          filt[2 * branch + 1] = fc ? ai : 0;
        }
        T *orow = out + 2 * (b * T_out * M + t * M);
        for (int64_t ch = 0; ch < M; ch++) {
          T dr = 0, di = 0;
          for (int64_t br = 0; br < M; br++) {
            const T fr = filt[2 * br], fi = filt[2 * br + 1];
            const T cr = tw[2 * (ch * M + br)], ci = tw[2 * (ch * M + br) + 1];
            /* dft += filtered * twiddle (complex product, then add) */
            const T pr = fr * cr - fi * ci;
            const T pim = fr * ci + fi * cr;
            dr = dr + pr;
            di = di + pim;
          }
          orow[2 * ch] = dr;
          orow[2 * ch + 1] = di;
        }
      }
      free(filt);
    }
  }
  free(tw);
  return err;
}

/* ---------------------------------------------------------------------------
 * Adjoint of the real resampler (no MatX counterpart).
 * For y[n] = up * sum_i x[i] * he[c + n*down - i*up] (he = taps with the even
 * leading zero, c = centre tap, gcd-reduced up/down), the exact adjoints are
 *   dx[b][i] = up * sum_n gy[b][n] * he[c + n*down - i*up]
 *   dh[k]    = up * sum_b sum_n gy[b][n] * x[b][i]  where c + n*down - i*up = k (+1 if L even).
 * up == down after reduction: dx = gy (identity copy), dh = 0.
 * ------------------------------------------------------------------------- */
int FN(oracle_resample_poly_bwd)(T *dx, T *dh, const T *gy, int64_t out_len,
                                 const T *x, int64_t N, const T *h, int64_t L,
                                 int64_t B, int64_t up, int64_t down,
                                 int nthreads) {
  if (up <= 0 || down <= 0 || N <= 0 || L <= 0 || B <= 0) return 1;
  int64_t a = up, c0 = down;
  while (c0) { int64_t t = a % c0; a = c0; c0 = t; }
  up /= a;
  down /= a;
  if (up == 1 && down == 1) {
    if (dx) for (int64_t i = 0; i < B * N; i++) dx[i] = gy[(i / N) * out_len + i % N];
    if (dh) for (int64_t k = 0; k < L; k++) dh[k] = 0;
    return 0;
  }
  const int is_even = (L % 2) == 0;
  const int64_t flen = is_even ? L + 1 : L;
  const int64_t central = (flen - 1) / 2;
  if (dx) {
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads) if (nthreads > 1) schedule(static)
#endif
    for (int64_t bi = 0; bi < B * N; bi++) {
      const int64_t b = bi / N, i = bi % N;
      double acc = 0;
      /* n with 0 <= central + n*down - i*up < flen */
      const int64_t lo_num = i * up - central;            /* n*down >= lo_num */
      const int64_t hi_num = i * up - central + flen - 1; /* n*down <= hi_num */
      int64_t n0 = lo_num <= 0 ? 0 : (lo_num + down - 1) / down;
      int64_t n1 = hi_num < 0 ? -1 : hi_num / down;
      if (n1 > out_len - 1) n1 = out_len - 1;
      for (int64_t n = n0; n <= n1; n++) {
        const int64_t k = central + n * down - i * up;
        if (is_even && k == 0) continue;
        const int64_t fi = is_even ? k - 1 : k;
        acc += (double)gy[b * out_len + n] * (double)h[fi];
      }
      dx[bi] = (T)(acc * (double)up);
    }
  }
  if (dh) {
    double *acc = (double *)calloc((size_t)flen, sizeof(double));
    if (!acc) return 4;
    for (int64_t k = 0; k < flen; k++) {
      if (is_even && k == 0) continue;
      double s = 0;
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads) if (nthreads > 1) reduction(+ : s) schedule(static)
#endif
      for (int64_t bn = 0; bn < B * out_len; bn++) {
        const int64_t b = bn / out_len, n = bn % out_len;
        const int64_t num = central + n * down - k; /* = i*up */
        if (num < 0 || num % up) continue;
        const int64_t i = num / up;
        if (i >= N) continue;
        s += (double)gy[bn] * (double)x[b * N + i];
      }
      acc[k] = s;
    }
    for (int64_t m = 0; m < L; m++) dh[m] = (T)(acc[is_even ? m + 1 : m] * (double)up);
    free(acc);
  }
  return 0;
}

/* ---------------------------------------------------------------------------
 * Adjoint of the real direct conv1d (no MatX counterpart).
 * y[b][o] = sum_i x[b][i] * h[o + start - i]  (start per mode, from min(N, L)):
 *   dx[b][i] = sum_o gy[b][o] * h[o + start - i]
 *   dh[f]    = sum_b sum_o gy[b][o] * x[b][o + start - f]
 * ------------------------------------------------------------------------- */
int FN(oracle_conv1d_bwd)(T *dx, T *dh, const T *gy, int64_t out_len,
                          const T *x, int64_t N, const T *h, int64_t L,
                          int64_t B, int mode, int nthreads) {
  if (N <= 0 || L <= 0 || B <= 0) return 1;
  const int64_t mn = N < L ? N : L;
  int64_t start = 0;
  if (mode == 1) start = (mn & 1) ? (mn - 1) / 2 : mn / 2 - 1;
  else if (mode == 2) start = mn - 1;
  if (dx) {
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads) if (nthreads > 1) schedule(static)
#endif
    for (int64_t bi = 0; bi < B * N; bi++) {
      const int64_t b = bi / N, i = bi % N;
      double acc = 0;
      for (int64_t f = 0; f < L; f++) {
        const int64_t o = i + f - start;
        if (o < 0 || o >= out_len) continue;
        acc += (double)gy[b * out_len + o] * (double)h[f];
      }
      dx[bi] = (T)acc;
    }
  }
  if (dh) {
    for (int64_t f = 0; f < L; f++) {
      double s = 0;
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads) if (nthreads > 1) reduction(+ : s) schedule(static)
#endif
      for (int64_t bo = 0; bo < B * out_len; bo++) {
        const int64_t b = bo / out_len, o = bo % out_len;
        const int64_t i = o + start - f;
        if (i < 0 || i >= N) continue;
        s += (double)gy[bo] * (double)x[b * N + i];
      }
      dh[f] = (T)s;
    }
  }
  return 0;
}

/* ---------------------------------------------------------------------------
 * Direct conv2d of `B` images [N1][M1] with filters [N2][M2] (h_bstride 0: one filter).
 * Follows MatX's host loop include/matx/transforms/conv.h:325-395: per output
 * (oy, ox), sum over fy (outer) and fx (inner) of x[oy+fy-dy][ox+fx-dx] *
 * h[N2-1-fy][M2-1-fx] with detail::madd, x outside the image skipped, dy/dx =
 * N2-1/M2-1 (FULL), N2/2, M2/2 (SAME), 0 (VALID); output sizes per axis
 * max+min-1, max, max-min+1 (operators/conv.h:335-357).  The caller passes the
 * larger image as x (conv.h:569-576 swaps by total size).
 * ------------------------------------------------------------------------- */
int FN(oracle_conv2d)(T *out, int64_t ON, int64_t OM, const T *x, int64_t x_bstride, int64_t N1, int64_t M1,
                      const T *h, int64_t h_bstride, int64_t N2, int64_t M2, int64_t B, int mode, int xc, int hc) {
  if (N1 <= 0 || M1 <= 0 || N2 <= 0 || M2 <= 0 || B <= 0) return 1;
  int64_t dy = 0, dx = 0;
  if (mode == 1) {
    dy = N2 / 2;
    dx = M2 / 2;
  } else if (mode == 0) {
    dy = N2 - 1;
    dx = M2 - 1;
  } else if (mode != 2) {
    return 2;
  }
  const int oc = xc || hc;
  for (int64_t b = 0; b < B; b++) {
    const T *xb = x + b * x_bstride * (xc ? 2 : 1);
    const T *hb = h + b * h_bstride * (hc ? 2 : 1);
    T *ob = out + b * ON * OM * (oc ? 2 : 1);
    for (int64_t oy = 0; oy < ON; oy++)
      for (int64_t ox = 0; ox < OM; ox++) {
        T sr = 0, si = 0;
        for (int64_t fy = 0; fy < N2; fy++) {
          const int64_t iy = oy + fy - dy;
          if (iy < 0 || iy >= N1) continue;
          for (int64_t fx = 0; fx < M2; fx++) {
            const int64_t ix = ox + fx - dx;
            if (ix < 0 || ix >= M1) continue;
            const int64_t xi = iy * M1 + ix, hi = (N2 - 1 - fy) * M2 + (M2 - 1 - fx);
            const T xr = xc ? xb[2 * xi] : xb[xi], xm = xc ? xb[2 * xi + 1] : 0;
            const T hr = hc ? hb[2 * hi] : hb[hi], hm = hc ? hb[2 * hi + 1] : 0;
            /* madd order (core/utils.h:165-210): re += xr hr; re -= xi hi; im += xi hr; im += xr hi */
            sr += xr * hr;
            sr -= xm * hm;
            si += xm * hr;
            si += xr * hm;
          }
        }
        const int64_t o = oy * OM + ox;
        if (oc) {
          ob[2 * o] = sr;
          ob[2 * o + 1] = si;
        } else {
          ob[o] = sr;
        }
      }
  }
  return 0;
}

/* ---------------------------------------------------------------------------
 * Recursive filter() (MatX filter(in, h_rec, h_nonrec) with h_rec non-empty):
 *   y[n] = sum_{j<nb} b[j] x[n-j] + sum_{k<na} a[k] y[n-1-k],  zero initial state,
 * one row at a time, in order.  This is the recurrence MatX's RecursiveFilter
 * solves in parallel (include/matx/kernels/filter.cuh:44-, correction factors of
 * include/matx/transforms/filter.h:206-250) and the sequential loop its own test
 * checks it against (test/00_operators/filter_test.cu:19-47).  x / y complex when
 * xc or cc; coefficients complex when cc.  (MatX's FIR-only filter is conv1d SAME,
 * transforms/filter.h:185: the oracle wrapper routes it to oracle_conv1d.)
 * ------------------------------------------------------------------------- */
int FN(oracle_iir_filter)(T *out, const T *x, int64_t N, int64_t B, const T *a, int na, const T *b, int nb,
                          int xc, int cc) {
  if (N <= 0 || B <= 0 || na < 0 || nb < 0) return 1;
  const int oc = xc || cc;
  for (int64_t r = 0; r < B; r++) {
    const T *xr = x + r * N * (xc ? 2 : 1);
    T *yr = out + r * N * (oc ? 2 : 1);
    for (int64_t n = 0; n < N; n++) {
      T sr = 0, si = 0;
      for (int j = 0; j < nb; j++) {
        if (n - j < 0) continue;
        const T xre = xc ? xr[2 * (n - j)] : xr[n - j], xim = xc ? xr[2 * (n - j) + 1] : 0;
        const T cre = cc ? b[2 * j] : b[j], cim = cc ? b[2 * j + 1] : 0;
        sr += xre * cre - xim * cim;
        si += xre * cim + xim * cre;
      }
      for (int k = 0; k < na; k++) {
        if (n - 1 - k < 0) continue;
        const T yre = oc ? yr[2 * (n - 1 - k)] : yr[n - 1 - k], yim = oc ? yr[2 * (n - 1 - k) + 1] : 0;
        const T cre = cc ? a[2 * k] : a[k], cim = cc ? a[2 * k + 1] : 0;
        sr += yre * cre - yim * cim;
        si += yre * cim + yim * cre;
      }
      if (oc) {
        yr[2 * n] = sr;
        yr[2 * n + 1] = si;
      } else {
        yr[n] = sr;
      }
    }
  }
  return 0;
}

#undef FN
#undef CAT
#undef CAT_
