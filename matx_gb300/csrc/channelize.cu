// channelize.cu — fused polyphase channelizer (FIR branches + M-point DFT) for sm_103a.
//
// Semantics are MatX's channelize_poly (include/matx/transforms/channelize_poly.h:724-849
// CUDA path, :858-1029 host path, include/matx/kernels/channelize_poly.cuh:134-310):
//   D == M:  F[t][c] = sum_p h[p*M + c] * x[(t - p)*M + (M-1-c)]
//   D <  M:  r' = (c + M - D) mod M, s = M-1-r', last = t*D + D - 1, A = last - s,
//            newest = last - (A mod M), causal = A/M + 1, phase = (c + t*D) mod M,
//            F[t][c] = sum_{p < min(P, causal)} h[phase + p*M] * x[newest - p*M]
//   with h zero-padded to P*M (P = ceil(L/M)) and x zero outside [0, N), then
//   Y[t][k] = sum_c F[t][c] * exp(+2*pi*i*c*k/M)  (unnormalised; MatX runs this
//   as a separate in-place cuFFT ifft(FFTNorm::FORWARD) pass, channelize_poly.h:846).
//
// Schedule (no MatX counterpart).  One CTA owns TT consecutive output steps of
// one row and all M channels, so the DFT never leaves shared memory: the input
// window is staged once (cp.async, zero-filled), the branch filters write F into
// shared memory, the DFT runs in shared memory/registers, and each output row
// is stored once.  HBM traffic is 8 B in + 8 B out per output sample, against
// 32 B for FIR-then-FFT.
//   * FIR, D == M: a thread owns one channel and 8 consecutive steps; taps in
//     blocks of 8 with a 16-sample register window (64 FMAs per 8 loads).
//   * FIR, D <  M: one (step, channel) per thread iteration (phases rotate).
//   * DFT, M = M1*M2 <= 256 (powers of two): four-step FFT, radix-M1 and radix-M2
//     passes in registers, twiddle W_M^(c2*k1) between them, padded layouts so both
//     passes are bank-conflict free.  Other M: direct DFT with a twiddle table.
//   * D == M with M = 32 or 64 (float, real taps): the warp-FFT form below keeps F and the
//     DFT in registers (shuffles across the warp) instead.
#include "common.cuh"

namespace gbfir {

constexpr int kChThreads = 256;
constexpr int kChE = 8;

struct ChParams {
  const void *x;
  int64_t x_bstride, N;
  const void *h;
  int64_t L;
  void *out;
  int64_t out_bstride;
  int64_t M, D, P, Ppad, T;
  int32_t TT;
  int64_t tiles_per_row, ntiles;
  int32_t W;           // window samples
  int32_t tap_stride;  // D==M: row stride of the [c][p] tap table
  int32_t Mf, Mp;      // F/Y row stride, A row stride
  int32_t r2_elems;    // elements in region 2 (window / A / generic Y); warp-FFT form: window buffer stride
  int32_t out_aligned; // warp-FFT form: 16-byte stores of bin pairs are aligned
};

// W_16^k = exp(+2*pi*i*k/16), k = 0..7 (cos/sin of multiples of pi/8).
template <typename T>
__device__ __forceinline__ void w16(int k, T &c, T &s) {
  const T a = T(0.92387953251128675613), b = T(0.38268343236508977173), r = T(0.70710678118654752440);
  switch (k & 7) {
    case 0: c = 1; s = 0; break;
    case 1: c = a; s = b; break;
    case 2: c = r; s = r; break;
    case 3: c = b; s = a; break;
    case 4: c = 0; s = 1; break;
    case 5: c = -b; s = a; break;
    case 6: c = -r; s = r; break;
    default: c = -a; s = b; break;
  }
}

template <int R>
__host__ __device__ constexpr int bitrev(int i) {
  int r = 0;
  for (int b = 1; b < R; b <<= 1) {
    r = (r << 1) | (i & 1);
    i >>= 1;
  }
  return r;
}

// In-register radix-2 FFT, positive exponent: v[k] <- sum_n v[n] exp(+2*pi*i*n*k/R).
template <typename T, int R>
__device__ __forceinline__ void fft_reg(T (&re)[R], T (&im)[R]) {
  if constexpr (R > 1) {
#pragma unroll
  for (int i = 0; i < R; i++) {
    const int j = bitrev<R>(i);
    if (j > i) {
      T t = re[i]; re[i] = re[j]; re[j] = t;
      t = im[i]; im[i] = im[j]; im[j] = t;
    }
  }
#pragma unroll
  for (int len = 2; len <= R; len <<= 1) {
#pragma unroll
    for (int i = 0; i < R; i += len) {
#pragma unroll
      for (int k = 0; k < len / 2; k++) {
        T wc, ws;
        w16<T>(k * (16 / len), wc, ws);
        const int a = i + k, b = i + k + len / 2;
        const T br = re[b] * wc - im[b] * ws;
        const T bi = re[b] * ws + im[b] * wc;
        re[b] = re[a] - br;
        im[b] = im[a] - bi;
        re[a] = re[a] + br;
        im[a] = im[a] + bi;
      }
    }
  }
  }
}

template <typename T>
__device__ __forceinline__ void twiddle_of(int64_t m, int64_t M, T &c, T &s);
template <>
__device__ __forceinline__ void twiddle_of<float>(int64_t m, int64_t M, float &c, float &s) {
  // exp(+2*pi*i*m/M); the argument 2m/M is reduced to [0, 2) exactly in integers first.
  sincospif((float)(2 * m) / (float)M, &s, &c);
}
template <>
__device__ __forceinline__ void twiddle_of<double>(int64_t m, int64_t M, double &c, double &s) {
  sincospi((double)(2 * m) / (double)M, &s, &c);
}

// DFT kind: (M1, M2) with M = M1*M2; M1 == 0 selects the direct DFT.
// The 8 taps th[0..7] of one channel row.  Float rows are 16-byte aligned (the table's row
// stride is a multiple of 4 and blocks start at multiples of 8), so they come in as two
// 16-byte loads: lanes of a quarter warp read rows 16*stride bytes apart, distinct 16-byte
// bank groups, where eight 4-byte loads per lane would hit the same bank four times.
template <typename HT, int E>
__device__ __forceinline__ void load_tap_block(const HT *th, HT (&t)[E]) {
  if constexpr (std::is_same<HT, float>::value && E == 8) {
    const float4 a = *reinterpret_cast<const float4 *>(th), b = *reinterpret_cast<const float4 *>(th + 4);
    t[0] = a.x, t[1] = a.y, t[2] = a.z, t[3] = a.w, t[4] = b.x, t[5] = b.y, t[6] = b.z, t[7] = b.w;
  } else {
#pragma unroll
    for (int kk = 0; kk < E; kk++) t[kk] = th[kk];
  }
}

template <typename T, bool XC, bool HC, int M1, int M2>
__global__ void __launch_bounds__(kChThreads) channelize_fused(const ChParams p) {
  using XT = typename val_of<T, XC>::type;
  using HT = typename val_of<T, HC>::type;
  using CT = typename cplx_of<T>::type;
  constexpr bool FC = XC || HC;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int M = (int)p.M;
  const bool md = p.D == p.M;
  // layout: [taps][twiddles][region 1: F / Y][region 2: window / A / generic Y]
  const size_t tap_elems = md ? (size_t)M * p.tap_stride : (size_t)p.Ppad * M;
  size_t off = (tap_elems * sizeof(HT) + 15) & ~(size_t)15;
  HT *taps = reinterpret_cast<HT *>(smem_raw);
  CT *tw = reinterpret_cast<CT *>(smem_raw + off);
  off += ((size_t)M * sizeof(CT) + 15) & ~(size_t)15;
  CT *r1 = reinterpret_cast<CT *>(smem_raw + off);
  off += ((size_t)p.TT * p.Mf * sizeof(CT) + 15) & ~(size_t)15;
  unsigned char *r2raw = smem_raw + off;
  XT *win = reinterpret_cast<XT *>(r2raw);
  CT *r2 = reinterpret_cast<CT *>(r2raw);

  const int tid = threadIdx.x;
  const HT *hp = reinterpret_cast<const HT *>(p.h);
  const XT *xp = reinterpret_cast<const XT *>(p.x);
  CT *op = reinterpret_cast<CT *>(p.out);

  // taps: D==M -> [c][p] rows of tap_stride; D<M -> natural zero-padded P*M
  for (size_t e = tid; e < tap_elems; e += kChThreads) {
    HT v = zero_val<HT>();
    if (md) {
      const int c = (int)(e / p.tap_stride), pp = (int)(e - (size_t)c * p.tap_stride);
      const int64_t idx = (int64_t)pp * M + c;
      if (pp < p.P && idx < p.L) v = hp[idx];
    } else if ((int64_t)e < p.L) {
      v = hp[e];
    }
    taps[e] = v;
  }
  for (int m = tid; m < M; m += kChThreads) {
    T c, s;
    twiddle_of<T>(m, p.M, c, s);
    tw[m].x = c;
    tw[m].y = s;
  }

  for (int64_t tile = blockIdx.x; tile < p.ntiles; tile += gridDim.x) {
    const int64_t b = tile / p.tiles_per_row;
    const int64_t t0 = (tile - b * p.tiles_per_row) * p.TT;
    const XT *row = xp + b * p.x_bstride;
    const int64_t w0 = t0 * p.D + p.D - (p.Ppad + 1) * p.M;
    __syncthreads();  // previous tile fully stored, tables written
    for (int e = tid; e < p.W; e += kChThreads) {
      const int64_t gi = w0 + e;
      const bool ok = gi >= 0 && gi < p.N;
      cp_async_zfill<sizeof(XT)>(&win[e], ok ? (const void *)(row + gi) : (const void *)row, ok);
    }
    cp_async_commit();
    cp_async_wait<0>();
    __syncthreads();

    // ---- FIR branch filters -> F in r1 ([TT][Mf]) ----
    if (md) {
      constexpr int E = kChE;
      const int nitems = M * (p.TT / E);
      const int Pp = (int)p.Ppad;
      for (int w = tid; w < nitems; w += kChThreads) {
        const int c = w % M, r = w / M;
        const int sc = M - 1 - c;
        Acc<T, FC> acc[E];
#pragma unroll
        for (int e = 0; e < E; e++) acc[e].zero();
        const HT *th = taps + (size_t)c * p.tap_stride;
        XT cur[E], prv[E];
        int rowi = r * E + Pp;  // window row of (t = t0 + r*E, p = 0)
#pragma unroll
        for (int e = 0; e < E; e++) cur[e] = win[(rowi + e) * M + sc];
        for (int kb = 0; kb < Pp; kb += E) {
          rowi -= E;
#pragma unroll
          for (int e = 0; e < E; e++) prv[e] = win[(rowi + e) * M + sc];
          HT t[E];
          load_tap_block<HT, E>(th + kb, t);
#pragma unroll
          for (int kk = 0; kk < E; kk++) {
#pragma unroll
            for (int e = 0; e < E; e++) {
              const XT xv = (e >= kk) ? cur[e - kk] : prv[E + e - kk];
              mac<T, XC, HC>(acc[e], xv, t[kk]);
            }
          }
#pragma unroll
          for (int e = 0; e < E; e++) cur[e] = prv[e];
        }
#pragma unroll
        for (int e = 0; e < E; e++) {
          CT v;
          v.x = acc[e].re;
          if constexpr (FC) v.y = acc[e].im;
          else v.y = 0;
          r1[(r * E + e) * p.Mf + c] = v;
        }
      }
    } else {
      const int nitems = M * p.TT;
      for (int w = tid; w < nitems; w += kChThreads) {
        const int c = w % M, tl = w / M;
        const int64_t t = t0 + tl;
        const int64_t rr = (c + p.M - p.D) % p.M;
        const int64_t s = p.M - 1 - rr;
        const int64_t last = t * p.D + p.D - 1;
        Acc<T, FC> acc;
        acc.zero();
        if (last >= s) {
          const int64_t A = last - s;
          const int64_t newest = last - (A % p.M);
          const int64_t causal = A / p.M + 1;
          const int64_t phase = (c + t * p.D) % p.M;
          const int64_t niter = min(p.P, causal);
          int widx = (int)(newest - w0);
          int hidx = (int)phase;
          for (int64_t i = 0; i < niter; i++) {
            mac<T, XC, HC>(acc, win[widx], taps[hidx]);
            widx -= M;
            hidx += M;
          }
        }
        CT v;
        v.x = acc.re;
        if constexpr (FC) v.y = acc.im;
        else v.y = 0;
        r1[tl * p.Mf + c] = v;
      }
    }
    __syncthreads();

    // ---- M-point DFT ----
    CT *ybuf = r1;
    if constexpr (M1 > 0) {
      // step 1: radix-M1 over c1 for each (t, c2); twiddle; A[t][k1*(M2+1) + c2]
      const int n1 = p.TT * M2;
      for (int w = tid; w < n1; w += kChThreads) {
        const int c2 = w % M2, tl = w / M2;
        T re[M1], im[M1];
#pragma unroll
        for (int c1 = 0; c1 < M1; c1++) {
          const CT v = r1[tl * p.Mf + M2 * c1 + c2];
          re[c1] = v.x;
          im[c1] = v.y;
        }
        fft_reg<T, M1>(re, im);
#pragma unroll
        for (int k1 = 0; k1 < M1; k1++) {
          CT v;
          if (M2 > 1 && k1 > 0 && c2 > 0) {
            const CT wv = tw[c2 * k1];
            v.x = re[k1] * wv.x - im[k1] * wv.y;
            v.y = re[k1] * wv.y + im[k1] * wv.x;
          } else {
            v.x = re[k1];
            v.y = im[k1];
          }
          r2[tl * p.Mp + k1 * (M2 + 1) + c2] = v;
        }
      }
      __syncthreads();
      // step 2: radix-M2 over c2 for each (t, k1); Y[t][k1 + M1*k2] into r1
      const int n2 = p.TT * M1;
      for (int w = tid; w < n2; w += kChThreads) {
        const int k1 = w % M1, tl = w / M1;
        T re[M2], im[M2];
#pragma unroll
        for (int c2 = 0; c2 < M2; c2++) {
          const CT v = r2[tl * p.Mp + k1 * (M2 + 1) + c2];
          re[c2] = v.x;
          im[c2] = v.y;
        }
        fft_reg<T, M2>(re, im);
#pragma unroll
        for (int k2 = 0; k2 < M2; k2++) {
          CT v;
          v.x = re[k2];
          v.y = im[k2];
          r1[tl * p.Mf + k1 + M1 * k2] = v;
        }
      }
    } else {
      // direct DFT: Y[t][k] = sum_c F[t][c] * tw[(c*k) mod M], into r2
      const int n2 = p.TT * M;
      for (int w = tid; w < n2; w += kChThreads) {
        const int k = w % M, tl = w / M;
        T ar = 0, ai = 0;
        int idx = 0;
        for (int c = 0; c < M; c++) {
          const CT f = r1[tl * p.Mf + c];
          const CT wv = tw[idx];
          ar = fma(f.x, wv.x, ar);
          ar = fma(-f.y, wv.y, ar);
          ai = fma(f.x, wv.y, ai);
          ai = fma(f.y, wv.x, ai);
          idx += k;
          if (idx >= M) idx -= M;
        }
        CT v;
        v.x = ar;
        v.y = ai;
        r2[tl * p.Mf + k] = v;
      }
      ybuf = r2;
    }
    __syncthreads();

    // ---- store rows t0 .. t0+TT-1 (contiguous [TT][M] block of the output row) ----
    const int64_t nrows = min((int64_t)p.TT, p.T - t0);
    CT *orow = op + b * p.out_bstride + t0 * p.M;
    const int64_t nel = nrows * p.M;
    for (int64_t e = tid; e < nel; e += kChThreads) {
      const int64_t tl = e / M, k = e - tl * M;
      orow[e] = ybuf[tl * p.Mf + k];
    }
  }
}

// ---- warp-FFT form: D == M with M = 32 or 64, float, real taps ----
// A warp owns E = 8 consecutive output steps and all M channels (lane L: channel L and, for
// M = 64, channel L + 32).  It runs the branch filters in registers exactly as the fused
// kernel does (same taps, same multiply-add order), then the M-point DFT of each step across
// the warp: radix-2 decimation in frequency, for M = 64 one stage inside the lane (channels
// n and n + 32) and then five stages across lanes with shuffles (lane distance 16 .. 1, the
// upper lane of a pair taking (partner - own) times its twiddle).  Lane L then holds bin
// bitrev5(L) (M = 32), or bins 2*bitrev5(L) and 2*bitrev5(L) + 1 (M = 64), so each step's M
// outputs leave as one store instruction per warp: 8 or 16 bytes a lane, the whole output
// row.  F and Y never touch shared memory; the input window is double-buffered with
// cp.async, the next tile's window in flight while the current one is filtered.
__device__ __forceinline__ float2 cmulf(float2 a, float2 w) {
  return make_float2(a.x * w.x - a.y * w.y, a.x * w.y + a.y * w.x);
}
__device__ __forceinline__ int bitrev5(int v) { return (int)(__brev((unsigned)v) >> 27); }

template <bool XC, int M>
__global__ void __launch_bounds__(kChThreads) channelize_warpfft(const ChParams p) {
  using XT = typename val_of<float, XC>::type;
  constexpr int C = M / 32;  // channels per lane
  constexpr int E = kChE;    // steps per warp item
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float *taps = reinterpret_cast<float *>(smem_raw);  // [c][pp], rows of tap_stride
  const size_t toff = ((size_t)M * p.tap_stride * sizeof(float) + 15) & ~(size_t)15;
  XT *wbuf0 = reinterpret_cast<XT *>(smem_raw + toff);
  XT *wbuf1 = wbuf0 + p.r2_elems;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const float *hp = reinterpret_cast<const float *>(p.h);
  const XT *xp = reinterpret_cast<const XT *>(p.x);
  float2 *op = reinterpret_cast<float2 *>(p.out);

  for (int e = tid; e < M * p.tap_stride; e += kChThreads) {
    const int c = e / p.tap_stride, pp = e - c * p.tap_stride;
    const int64_t idx = (int64_t)pp * M + c;
    taps[e] = (pp < p.P && idx < p.L) ? hp[idx] : 0.f;
  }
  // twiddles exp(+2*pi*i*m/M) of this lane, arguments reduced exactly in integers
  float2 w0 = make_float2(1.f, 0.f), ws[4];
  if constexpr (M == 64) sincospif((float)(2 * lane) / 64.f, &w0.y, &w0.x);
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const int s = 16 >> i, ex = (lane & (s - 1)) * (16 / s);  // W_{2s}^(L mod s) = W_32^ex
    sincospif((float)(2 * ex) / 32.f, &ws[i].y, &ws[i].x);
  }

  auto issue = [&](int64_t tile, XT *buf) {
    const int64_t b = tile / p.tiles_per_row;
    const int64_t t0 = (tile - b * p.tiles_per_row) * p.TT;
    const XT *row = xp + b * p.x_bstride;
    const int64_t w0i = t0 * p.D + p.D - (p.Ppad + 1) * p.M;
    for (int e = tid; e < p.W; e += kChThreads) {
      const int64_t gi = w0i + e;
      const bool ok = gi >= 0 && gi < p.N;
      cp_async_zfill<sizeof(XT)>(&buf[e], ok ? (const void *)(row + gi) : (const void *)row, ok);
    }
  };
  int64_t tile = blockIdx.x;
  if (tile < p.ntiles) issue(tile, wbuf0);
  cp_async_commit();
  const int Pp = (int)p.Ppad;
  for (int it = 0; tile < p.ntiles; tile += gridDim.x, ++it) {
    const XT *win = (it & 1) ? wbuf1 : wbuf0;
    const int64_t next = tile + gridDim.x;
    if (next < p.ntiles) issue(next, (it & 1) ? wbuf0 : wbuf1);
    cp_async_commit();
    cp_async_wait<1>();
    __syncthreads();  // this tile's window (and, the first time, the taps) is in
    const int64_t b = tile / p.tiles_per_row;
    const int64_t t0 = (tile - b * p.tiles_per_row) * p.TT;
    float2 *orow = op + b * p.out_bstride;
    for (int r = warp; r < p.TT / E; r += kChThreads / 32) {
      Acc<float, XC> acc[C][E];
#pragma unroll
      for (int ci = 0; ci < C; ci++) {
        const int c = lane + 32 * ci, sc = M - 1 - c;
#pragma unroll
        for (int e = 0; e < E; e++) acc[ci][e].zero();
        const float *th = taps + (size_t)c * p.tap_stride;
        XT cur[E], prv[E];
        int rowi = r * E + Pp;  // window row of (t = t0 + r*E, p = 0)
#pragma unroll
        for (int e = 0; e < E; e++) cur[e] = win[(rowi + e) * M + sc];
        for (int kb = 0; kb < Pp; kb += E) {
          rowi -= E;
#pragma unroll
          for (int e = 0; e < E; e++) prv[e] = win[(rowi + e) * M + sc];
          float tv[E];
          load_tap_block<float, E>(th + kb, tv);
#pragma unroll
          for (int kk = 0; kk < E; kk++) {
#pragma unroll
            for (int e = 0; e < E; e++) {
              const XT xv = (e >= kk) ? cur[e - kk] : prv[E + e - kk];
              mac<float, XC, false>(acc[ci][e], xv, tv[kk]);
            }
          }
#pragma unroll
          for (int e = 0; e < E; e++) cur[e] = prv[e];
        }
      }
      const int kb5 = bitrev5(lane);
#pragma unroll
      for (int e = 0; e < E; e++) {
        float2 a, bv = make_float2(0.f, 0.f);
        if constexpr (XC) a = make_float2(acc[0][e].re, acc[0][e].im);
        else a = make_float2(acc[0][e].re, 0.f);
        if constexpr (C == 2) {
          if constexpr (XC) bv = make_float2(acc[1][e].re, acc[1][e].im);
          else bv = make_float2(acc[1][e].re, 0.f);
          // channels n and n + 32: even bins from the sum, odd bins from the twiddled difference
          const float2 sum = make_float2(a.x + bv.x, a.y + bv.y);
          bv = cmulf(make_float2(a.x - bv.x, a.y - bv.y), w0);
          a = sum;
        }
#pragma unroll
        for (int i = 0; i < 5; i++) {
          const int s = 16 >> i;
          const bool up = (lane & s) != 0;
          {
            const float2 pa = make_float2(__shfl_xor_sync(0xffffffffu, a.x, s), __shfl_xor_sync(0xffffffffu, a.y, s));
            const float2 d = make_float2(pa.x - a.x, pa.y - a.y);
            a = up ? (i < 4 ? cmulf(d, ws[i]) : d) : make_float2(a.x + pa.x, a.y + pa.y);
          }
          if constexpr (C == 2) {
            const float2 pb = make_float2(__shfl_xor_sync(0xffffffffu, bv.x, s), __shfl_xor_sync(0xffffffffu, bv.y, s));
            const float2 d = make_float2(pb.x - bv.x, pb.y - bv.y);
            bv = up ? (i < 4 ? cmulf(d, ws[i]) : d) : make_float2(bv.x + pb.x, bv.y + pb.y);
          }
        }
        const int64_t t = t0 + r * E + e;
        if (t < p.T) {
          float2 *dst = orow + t * M;
          if constexpr (C == 2) {
            if (p.out_aligned) *reinterpret_cast<float4 *>(dst + 2 * kb5) = make_float4(a.x, a.y, bv.x, bv.y);
            else {
              dst[2 * kb5] = a;
              dst[2 * kb5 + 1] = bv;
            }
          } else {
            dst[kb5] = a;
          }
        }
      }
    }
    __syncthreads();  // the window is read before the next-next tile's copy reuses the buffer
  }
  cp_async_wait<0>();
}

template <bool XC, int M>
static int launch_warpfft(ChParams &p, int64_t batch, cudaStream_t s) {
  using XT = typename val_of<float, XC>::type;
  p.tap_stride = (int)(p.Ppad + ((p.Ppad % 8) == 0 ? 4 : 0));
  const size_t taps_b = ((size_t)M * p.tap_stride * sizeof(float) + 15) & ~(size_t)15;
  // steps per tile: 64 (one 8-step item per warp), more while two CTAs still share an SM
  auto smem_for = [&](int TT) -> size_t {
    const int64_t W = (int64_t)(TT - 1) * p.D + (p.Ppad + 1) * p.M;
    const int64_t stride = (W + 1) / 2 * 2;  // buffers 16-byte aligned
    return taps_b + 2 * (size_t)stride * sizeof(XT);
  };
  int TT = 64;
  while (smem_for(TT + 64) <= 110 * 1024) TT += 64;
  const size_t smem = smem_for(TT);
  if (smem > 200 * 1024) return -1;
  p.TT = TT;
  p.W = (int32_t)((int64_t)(TT - 1) * p.D + (p.Ppad + 1) * p.M);
  p.r2_elems = (p.W + 1) / 2 * 2;
  p.tiles_per_row = (p.T + TT - 1) / TT;
  p.ntiles = p.tiles_per_row * batch;
  p.out_aligned = (reinterpret_cast<uintptr_t>(p.out) & 15) == 0 && (batch == 1 || p.out_bstride % 2 == 0) ? 1 : 0;
  auto fn = channelize_warpfft<XC, M>;
  int rc = ensure_smem((const void *)fn, smem, "channelize_poly");
  if (rc) return rc;
  int occ = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, kChThreads, smem);
  if (occ < 1) occ = 1;
  int64_t grid = (int64_t)num_sms() * occ;
  if (grid > p.ntiles) grid = p.ntiles;
  fn<<<(unsigned)grid, kChThreads, smem, s>>>(p);
  return check_launch("channelize_poly");
}

// ---- split path for large M*P: FIR into the output, then an in-place row DFT ----
// Used when the fused tile does not fit in shared memory.  The FIR reads x and h
// through L1 (lanes over channels read consecutive samples), writes F[t][c] into
// the output buffer, and a second kernel replaces each row by its M-point DFT.
template <typename T, bool XC, bool HC>
__global__ void __launch_bounds__(kChThreads) channelize_fir_split(const ChParams p) {
  using XT = typename val_of<T, XC>::type;
  using HT = typename val_of<T, HC>::type;
  using CT = typename cplx_of<T>::type;
  constexpr bool FC = XC || HC;
  const XT *xp = reinterpret_cast<const XT *>(p.x);
  const HT *hp = reinterpret_cast<const HT *>(p.h);
  CT *op = reinterpret_cast<CT *>(p.out);
  const int64_t per_row = p.T * p.M;
  const int64_t total = per_row * p.ntiles;  // ntiles == batch on this path
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / per_row, r = e - b * per_row;
    const int64_t t = r / p.M, c = r - t * p.M;
    const XT *row = xp + b * p.x_bstride;
    const int64_t rr = (c + p.M - p.D) % p.M;
    const int64_t s = p.M - 1 - rr;
    const int64_t last = t * p.D + p.D - 1;
    Acc<T, FC> acc;
    acc.zero();
    if (last >= s) {
      const int64_t A = last - s;
      int64_t idx = last - (A % p.M);
      const int64_t causal = A / p.M + 1;
      int64_t hidx = (p.D == p.M) ? c : (c + t * p.D) % p.M;
      const int64_t niter = min(p.P, causal);
      for (int64_t i = 0; i < niter; i++, idx -= p.M, hidx += p.M) {
        if (idx < p.N && hidx < p.L) mac<T, XC, HC>(acc, row[idx], hp[hidx]);
      }
    }
    CT v;
    v.x = acc.re;
    if constexpr (FC) v.y = acc.im;
    else v.y = 0;
    op[b * p.out_bstride + r] = v;
  }
}

template <typename T>
__global__ void __launch_bounds__(kChThreads) dft_rows_inplace(void *out, int64_t out_bstride, int64_t T_rows,
                                                               int64_t M, int64_t batch) {
  using CT = typename cplx_of<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  CT *tw = reinterpret_cast<CT *>(smem_raw);
  CT *rowbuf = tw + M;
  for (int m = threadIdx.x; m < M; m += kChThreads) {
    T c, s;
    twiddle_of<T>(m, M, c, s);
    tw[m].x = c;
    tw[m].y = s;
  }
  CT *op = reinterpret_cast<CT *>(out);
  const int64_t nrows = T_rows * batch;
  for (int64_t rix = blockIdx.x; rix < nrows; rix += gridDim.x) {
    const int64_t b = rix / T_rows, t = rix - b * T_rows;
    CT *row = op + b * out_bstride + t * M;
    __syncthreads();
    for (int m = threadIdx.x; m < M; m += kChThreads) rowbuf[m] = row[m];
    __syncthreads();
    for (int k = threadIdx.x; k < M; k += kChThreads) {
      T ar = 0, ai = 0;
      int idx = 0;
      for (int c = 0; c < M; c++) {
        const CT f = rowbuf[c];
        const CT wv = tw[idx];
        ar = fma(f.x, wv.x, ar);
        ar = fma(-f.y, wv.y, ar);
        ai = fma(f.x, wv.y, ai);
        ai = fma(f.y, wv.x, ai);
        idx += k;
        if (idx >= M) idx -= M;
      }
      CT v;
      v.x = ar;
      v.y = ai;
      row[k] = v;
    }
  }
}

template <typename T, bool XC, bool HC>
static int launch_split(ChParams &p, int64_t batch, cudaStream_t s) {
  using CT = typename cplx_of<T>::type;
  p.ntiles = batch;
  const int64_t total = p.T * p.M * batch;
  int64_t grid = (total + kChThreads - 1) / kChThreads;
  const int64_t cap = (int64_t)num_sms() * 8;
  if (grid > cap) grid = cap;
  channelize_fir_split<T, XC, HC><<<(unsigned)grid, kChThreads, 0, s>>>(p);
  int rc = check_launch("channelize_poly (split FIR)");
  if (rc) return rc;
  const size_t smem = 2 * (size_t)p.M * sizeof(CT);
  if (smem > 200 * 1024)
    GBFIR_FAIL(GBFIR_ERR_NOT_SUPPORTED, "channelize_poly: M=%lld is too large for the row DFT", (long long)p.M);
  auto fn = dft_rows_inplace<T>;
  rc = ensure_smem((const void *)fn, smem, "channelize_poly");
  if (rc) return rc;
  int64_t g2 = p.T * batch;
  const int64_t cap2 = (int64_t)num_sms() * 4;
  if (g2 > cap2) g2 = cap2;
  fn<<<(unsigned)g2, kChThreads, smem, s>>>(p.out, p.out_bstride, p.T, p.M, batch);
  return check_launch("channelize_poly (row DFT)");
}

template <typename T, bool XC, bool HC, int M1, int M2>
static int launch_ch(ChParams &p, int64_t batch, cudaStream_t s) {
  using XT = typename val_of<T, XC>::type;
  using HT = typename val_of<T, HC>::type;
  using CT = typename cplx_of<T>::type;
  const bool md = p.D == p.M;
  const int M = (int)p.M;
  p.Mf = (M1 > 0 && M2 < 16) ? M + M2 : M;
  if (M1 == 0) p.Mf = M;
  p.Mp = M1 > 0 ? M1 * (M2 + 1) : 0;
  p.tap_stride = md ? (int)(p.Ppad + ((p.Ppad % 8) == 0 ? 4 : 0)) : 0;
  const size_t tap_elems = md ? (size_t)M * p.tap_stride : (size_t)p.Ppad * M;
  auto smem_for = [&](int TT, int32_t &W, int32_t &r2e) -> size_t {
    W = (int32_t)((TT - 1) * p.D + (p.Ppad + 1) * p.M);
    size_t r2b = (size_t)W * sizeof(XT);
    const size_t ab = (size_t)TT * (M1 > 0 ? p.Mp : p.Mf) * sizeof(CT);
    if (ab > r2b) r2b = ab;
    r2e = (int32_t)(r2b / sizeof(XT));
    size_t sz = ((tap_elems * sizeof(HT) + 15) & ~(size_t)15) + (((size_t)M * sizeof(CT) + 15) & ~(size_t)15) +
                (((size_t)TT * p.Mf * sizeof(CT) + 15) & ~(size_t)15) + r2b;
    return sz;
  };
  int TT = 64;
  int32_t W = 0, r2e = 0;
  size_t smem = smem_for(TT, W, r2e);
  while (TT > kChE && smem > 100 * 1024) {
    TT -= kChE;
    smem = smem_for(TT, W, r2e);
  }
  if (smem > 200 * 1024) return launch_split<T, XC, HC>(p, batch, s);
  p.TT = TT;
  p.W = W;
  p.r2_elems = r2e;
  p.tiles_per_row = (p.T + TT - 1) / TT;
  p.ntiles = p.tiles_per_row * batch;
  auto fn = channelize_fused<T, XC, HC, M1, M2>;
  int rc = ensure_smem((const void *)fn, smem, "channelize_poly");
  if (rc) return rc;
  int occ = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, kChThreads, smem);
  if (occ < 1) occ = 1;
  int64_t grid = (int64_t)num_sms() * occ;
  if (grid > p.ntiles) grid = p.ntiles;
  fn<<<(unsigned)grid, kChThreads, smem, s>>>(p);
  return check_launch("channelize_poly");
}

template <typename T, bool XC, bool HC>
static int dispatch_ch(ChParams &p, int64_t batch, cudaStream_t s) {
  if constexpr (sizeof(T) == 4 && !HC) {
    // D == M with M = 32 or 64: the warp-FFT form (the fused kernel where its tile does not fit)
    if (p.D == p.M && (p.M == 32 || p.M == 64)) {
      const int rc = p.M == 32 ? launch_warpfft<XC, 32>(p, batch, s) : launch_warpfft<XC, 64>(p, batch, s);
      if (rc >= 0) return rc;
    }
  }
  if constexpr (sizeof(T) == 4) {
    switch (p.M) {
      case 2: return launch_ch<T, XC, HC, 2, 1>(p, batch, s);
      case 4: return launch_ch<T, XC, HC, 4, 1>(p, batch, s);
      case 8: return launch_ch<T, XC, HC, 8, 1>(p, batch, s);
      case 16: return launch_ch<T, XC, HC, 16, 1>(p, batch, s);
      case 32: return launch_ch<T, XC, HC, 8, 4>(p, batch, s);
      case 64: return launch_ch<T, XC, HC, 8, 8>(p, batch, s);
      case 128: return launch_ch<T, XC, HC, 16, 8>(p, batch, s);
      case 256: return launch_ch<T, XC, HC, 16, 16>(p, batch, s);
      default: break;
    }
  }
  return launch_ch<T, XC, HC, 0, 0>(p, batch, s);
}

int channelize_poly_fp(const gbfir_buf &out, const gbfir_buf &in, const gbfir_buf &h, int64_t M, int64_t D,
                       cudaStream_t s) {
  ChParams p{};
  p.x = in.ptr;
  p.x_bstride = in.batch > 1 ? in.batch_stride : 0;
  p.N = in.len;
  p.h = h.ptr;
  p.L = h.len;
  p.out = out.ptr;
  p.out_bstride = out.batch_stride;
  p.M = M;
  p.D = D;
  p.P = (h.len + M - 1) / M;
  p.Ppad = (p.P + kChE - 1) / kChE * kChE;
  p.T = (in.len + D - 1) / D;
  const bool xc = dtype_complex(in.dtype), hc = dtype_complex(h.dtype);
  if (dtype_double(in.dtype)) {
    if (xc && hc) return dispatch_ch<double, true, true>(p, out.batch, s);
    if (xc) return dispatch_ch<double, true, false>(p, out.batch, s);
    if (hc) return dispatch_ch<double, false, true>(p, out.batch, s);
    return dispatch_ch<double, false, false>(p, out.batch, s);
  }
  if (xc && hc) return dispatch_ch<float, true, true>(p, out.batch, s);
  if (xc) return dispatch_ch<float, true, false>(p, out.batch, s);
  if (hc) return dispatch_ch<float, false, true>(p, out.batch, s);
  return dispatch_ch<float, false, false>(p, out.batch, s);
}

}  // namespace gbfir
