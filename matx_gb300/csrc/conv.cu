// conv.cu — plain FP32/FP64 direct conv1d / corr for sm_103a.
//
// Semantics are MatX's direct conv1d (include/matx/transforms/conv.h:402-532 for
// the broadcast and the operand swap, :226-289 for the host loop, and
// include/matx/kernels/conv.cuh:27-185 for the CUDA path): the longer operand is
// the signal s, the shorter the filter f, and
//   full[n] = sum_k f[k] * s[n - k],   out[o] = full[o + start],
// start = 0 (FULL), (Lf-1)/2 or Lf/2-1 (SAME, odd/even Lf), Lf-1 (VALID).
// corr(a, b) = conv1d(a, reverse(conj(b))) (include/matx/transforms/corr.h:67);
// the reverse-conjugate is applied while staging the operand into shared memory.
//
// Schedule (no MatX counterpart): a CTA owns 2048 consecutive outputs of one row.
// Each thread owns E = 8 consecutive outputs and walks the taps in blocks of E
// with a register window of 2E signal samples: per block it loads E new samples
// (128-bit shared loads) and E taps (warp-broadcast 128-bit loads) and issues
// E*E multiply-adds.  Long filters are processed in chunks of up to 1024 taps,
// accumulators staying in registers.  Results are staged through shared memory
// so the global stores are fully coalesced whatever the row alignment.
// Real rows with one shared real filter of at most 1024 taps take conv1d_real_stream
// (persistent CTAs, prefetched windows, unrolled tap blocks), which makes the same
// multiply-adds in the same order.
#include <map>
#include <mutex>
#include <tuple>

#include "common.cuh"

namespace gbfir {

constexpr int kConvThreads = 256;
constexpr int kConvE = 8;
constexpr int kConvNB = kConvThreads * kConvE;  // outputs per CTA
constexpr int kConvChunk = 1024;                // taps per shared-memory chunk

struct ConvParams {
  const void *s;  // signal rows
  int64_t s_bstride, Ns;
  int32_t s_rc;   // reverse-conjugate the signal while staging (corr with swap)
  const void *f;  // filter rows
  int64_t f_bstride, Lf;
  int32_t f_rc;   // reverse-conjugate the filter while staging (corr)
  void *out;
  int64_t out_bstride, out_len, start;
  int64_t chunks_per_row;
};

template <typename V>
__device__ __forceinline__ V conj_val(V v) {
  if constexpr (!std::is_arithmetic<V>::value) {
    v.y = -v.y;
  }
  return v;
}

template <typename T, bool SC, bool FC>
__global__ void __launch_bounds__(kConvThreads) conv1d_direct(const ConvParams p) {
  using ST = typename val_of<T, SC>::type;
  using FT = typename val_of<T, FC>::type;
  constexpr bool OC = SC || FC;
  using OT = typename val_of<T, OC>::type;
  constexpr int E = kConvE;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  FT *taps = reinterpret_cast<FT *>(smem_raw);
  const int lc_max = (int)((p.Lf < kConvChunk ? (p.Lf + E - 1) / E * E : kConvChunk));
  ST *win = reinterpret_cast<ST *>(smem_raw + (((size_t)lc_max * sizeof(FT) + 15) & ~(size_t)15));

  const int64_t b = blockIdx.x / p.chunks_per_row;
  const int64_t o0 = (blockIdx.x - b * p.chunks_per_row) * (int64_t)kConvNB;
  const ST *srow = reinterpret_cast<const ST *>(p.s) + b * p.s_bstride;
  const FT *frow = reinterpret_cast<const FT *>(p.f) + b * p.f_bstride;
  const int64_t n0 = o0 + p.start;  // full-conv index of the CTA's first output
  const int tid = threadIdx.x;

  Acc<T, OC> acc[E];
#pragma unroll
  for (int e = 0; e < E; e++) acc[e].zero();

  for (int64_t fc = 0; fc < p.Lf; fc += kConvChunk) {
    const int lc_real = (int)min((int64_t)kConvChunk, p.Lf - fc);
    const int LC = (lc_real + E - 1) / E * E;
    __syncthreads();
    for (int k = tid; k < LC; k += kConvThreads) {
      FT v = zero_val<FT>();
      if (k < lc_real) {
        const int64_t kk = fc + k;
        v = p.f_rc ? conj_val(frow[p.Lf - 1 - kk]) : frow[kk];
      }
      taps[k] = v;
    }
    // window covers signal indices [wb, wb + NB + LC)
    const int64_t wb = n0 - fc - LC;
    const int wlen = kConvNB + LC;
    for (int e = tid; e < wlen; e += kConvThreads) {
      const int64_t gi = wb + e;
      ST v = zero_val<ST>();
      if (gi >= 0 && gi < p.Ns) v = p.s_rc ? conj_val(srow[p.Ns - 1 - gi]) : srow[gi];
      win[e] = v;
    }
    __syncthreads();

    // register window: cur = s[nb - kb .. nb - kb + E), prv = s[nb - kb - E .. nb - kb)
    ST cur[E], prv[E];
    int pos = tid * E + LC;  // shared index of s[nb - fc]
#pragma unroll
    for (int e = 0; e < E; e++) cur[e] = win[pos + e];
    for (int kb = 0; kb < LC; kb += E) {
      pos -= E;
#pragma unroll
      for (int e = 0; e < E; e++) prv[e] = win[pos + e];
      FT t[E];
#pragma unroll
      for (int kk = 0; kk < E; kk++) t[kk] = taps[kb + kk];
#pragma unroll
      for (int kk = 0; kk < E; kk++) {
#pragma unroll
        for (int e = 0; e < E; e++) {
          const ST sv = (e >= kk) ? cur[e - kk] : prv[E + e - kk];
          mac<T, SC, FC>(acc[e], sv, t[kk]);
        }
      }
#pragma unroll
      for (int e = 0; e < E; e++) cur[e] = prv[e];
    }
  }

  // stage and write out coalesced
  __syncthreads();
  OT *stage = reinterpret_cast<OT *>(win);
#pragma unroll
  for (int e = 0; e < E; e++) stage[tid * E + e] = pack<T, OC>(acc[e], T(1));
  __syncthreads();
  OT *orow = reinterpret_cast<OT *>(p.out) + b * p.out_bstride;
  const int64_t nvalid = min((int64_t)kConvNB, p.out_len - o0);
  for (int e = tid; e < nvalid; e += kConvThreads) orow[o0 + e] = stage[e];
}

// ---- real fp32 rows, one shared filter of at most 1024 taps: persistent and pipelined ----
//
// The one-tile-per-CTA kernel above waits on its window load before its short compute
// (8 tap blocks at 63 taps), so it runs latency-bound. Here a persistent CTA walks its
// tiles (row, 2048 outputs) with the taps loaded once and the next tile's window
// prefetched by cp.async into the second of two buffers while the current one computes.
// The multiply-adds are those of conv1d_direct in the same order: results are identical.
//
// Window layout: float i sits at i ^ (((i >> 5) & 1) << 2). A thread reads its 8 samples
// as two 16-byte loads, lanes 32 bytes apart; the swap of 16-byte halves on bit 5 puts the
// 8 lanes of a quarter warp on 8 distinct bank groups. 16-byte units stay whole, so an
// aligned window is copied in 16-byte pieces.
__device__ __forceinline__ int win_swz(int i) { return i ^ (((i >> 5) & 1) << 2); }

__device__ __forceinline__ void stream_issue(const ConvParams &p, int64_t t, float *buf, int LC, int tid) {
  const int64_t b = t / p.chunks_per_row;
  const int64_t o0 = (t - b * p.chunks_per_row) * (int64_t)kConvNB;
  const int64_t wb = o0 + p.start - LC;  // signal index of window float 0
  const int wlen = kConvNB + LC;         // a multiple of 8
  const float *srow = reinterpret_cast<const float *>(p.s) + b * p.s_bstride;
  if (!p.s_rc && (reinterpret_cast<uintptr_t>(srow + wb) & 15) == 0) {
    for (int u = tid; u < wlen / 4; u += kConvThreads) {
      const int64_t g = wb + 4 * u;
      float *dst = buf + win_swz(4 * u);
      if (g >= 0 && g + 4 <= p.Ns) {
        cp_async_zfill<16>(dst, srow + g, true);
      } else {
#pragma unroll
        for (int r = 0; r < 4; r++) {
          const bool ok = g + r >= 0 && g + r < p.Ns;
          cp_async_zfill<4>(dst + r, ok ? srow + g + r : srow, ok);
        }
      }
    }
  } else {
    for (int e = tid; e < wlen; e += kConvThreads) {
      const int64_t gi = wb + e;
      const bool ok = gi >= 0 && gi < p.Ns;
      const int64_t si = p.s_rc ? p.Ns - 1 - gi : gi;
      cp_async_zfill<4>(buf + win_swz(e), ok ? srow + si : srow, ok);
    }
  }
}

// One block of 8 taps: acc[e] += s[n_e - k] * tap[k] over k = kb..kb+7, where the 16 samples
// below each thread's outputs are `prv` (older) then `cur`: the order of conv1d_direct.
__device__ __forceinline__ void tap_block(float (&acc)[kConvE], const float (&cur)[kConvE],
                                          const float (&prv)[kConvE], const float *tap) {
  const float4 t0 = *reinterpret_cast<const float4 *>(tap);
  const float4 t1 = *reinterpret_cast<const float4 *>(tap + 4);
  const float tk[kConvE] = {t0.x, t0.y, t0.z, t0.w, t1.x, t1.y, t1.z, t1.w};
#pragma unroll
  for (int kk = 0; kk < kConvE; kk++) {
#pragma unroll
    for (int e = 0; e < kConvE; e++)
      acc[e] = fmaf((e >= kk) ? cur[e - kk] : prv[kConvE + e - kk], tk[kk], acc[e]);
  }
}

// The 8 window samples at pos (a multiple of 8): two whole 16-byte units.
__device__ __forceinline__ void load_block(float (&w)[kConvE], const float *win, int pos) {
  const int a = win_swz(pos);
  const float4 v0 = *reinterpret_cast<const float4 *>(win + a);
  const float4 v1 = *reinterpret_cast<const float4 *>(win + (a ^ 4));
  w[0] = v0.x; w[1] = v0.y; w[2] = v0.z; w[3] = v0.w;
  w[4] = v1.x; w[5] = v1.y; w[6] = v1.z; w[7] = v1.w;
}

// NKB > 0: the filter is NKB blocks of 8 taps, fully unrolled; NKB == 0: any length up to
// 1024 taps, two blocks per loop trip. Either way the two register windows swap roles from
// block to block instead of being copied.
template <int NKB>
__global__ void __launch_bounds__(kConvThreads) conv1d_real_stream(const ConvParams p, int64_t ntiles) {
  constexpr int E = kConvE;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int LC = NKB > 0 ? NKB * E : (int)((p.Lf + E - 1) / E * E);
  const int nkb = LC / E;
  const int wlen = kConvNB + LC;
  float *taps = reinterpret_cast<float *>(smem_raw);
  float *bufs = taps + LC;  // LC is a multiple of 8: 32-byte aligned
  const float *frow = reinterpret_cast<const float *>(p.f);
  const int tid = threadIdx.x;

  for (int k = tid; k < LC; k += kConvThreads) taps[k] = k < p.Lf ? (p.f_rc ? frow[p.Lf - 1 - k] : frow[k]) : 0.f;

  int64_t t = blockIdx.x;
  if (t < ntiles) stream_issue(p, t, bufs, LC, tid);
  cp_async_commit();
  for (int it = 0; t < ntiles; it++, t += gridDim.x) {
    const float *win = bufs + (it & 1) * wlen;
    if (t + gridDim.x < ntiles) stream_issue(p, t + gridDim.x, bufs + ((it + 1) & 1) * wlen, LC, tid);
    cp_async_commit();
    cp_async_wait<1>();
    __syncthreads();

    float acc[E];
#pragma unroll
    for (int e = 0; e < E; e++) acc[e] = 0.f;
    float wa[E], wb[E];
    const int top = tid * E + LC;  // window index of the thread's first output sample
    load_block(wa, win, top);
    if constexpr (NKB > 0) {
#pragma unroll
      for (int j = 0; j < NKB; j += 2) {
        load_block(wb, win, top - E * (j + 1));
        tap_block(acc, wa, wb, taps + E * j);
        if (j + 1 < NKB) {
          load_block(wa, win, top - E * (j + 2));
          tap_block(acc, wb, wa, taps + E * (j + 1));
        }
      }
    } else {
      int j = 0;
#pragma unroll 1
      for (; j + 2 <= nkb; j += 2) {
        load_block(wb, win, top - E * (j + 1));
        tap_block(acc, wa, wb, taps + E * j);
        load_block(wa, win, top - E * (j + 2));
        tap_block(acc, wb, wa, taps + E * (j + 1));
      }
      if (j < nkb) {
        load_block(wb, win, top - E * (j + 1));
        tap_block(acc, wa, wb, taps + E * j);
      }
    }

    // each thread writes its 8 consecutive outputs (whole 32-byte sectors when aligned)
    const int64_t b = t / p.chunks_per_row;
    const int64_t o0 = (t - b * p.chunks_per_row) * (int64_t)kConvNB;
    float *dst = reinterpret_cast<float *>(p.out) + b * p.out_bstride + o0 + tid * E;
    const int64_t left = p.out_len - o0 - (int64_t)tid * E;
    if (left >= E && (reinterpret_cast<uintptr_t>(dst) & 15) == 0) {
      reinterpret_cast<float4 *>(dst)[0] = make_float4(acc[0], acc[1], acc[2], acc[3]);
      reinterpret_cast<float4 *>(dst)[1] = make_float4(acc[4], acc[5], acc[6], acc[7]);
    } else {
#pragma unroll
      for (int e = 0; e < E; e++)
        if (e < left) dst[e] = acc[e];
    }
    __syncthreads();  // the buffer just read is the target of the next prefetch
  }
  cp_async_wait<0>();
}

static int launch_conv_real_stream(const ConvParams &p, int64_t batch, cudaStream_t s) {
  const int LC = (int)((p.Lf + kConvE - 1) / kConvE * kConvE);
  const size_t smem = (size_t)(LC + 2 * (kConvNB + LC)) * sizeof(float);
  const void *fn;
  switch (LC / kConvE) {
    case 1: fn = (const void *)conv1d_real_stream<1>; break;
    case 2: fn = (const void *)conv1d_real_stream<2>; break;
    case 3: fn = (const void *)conv1d_real_stream<3>; break;
    case 4: fn = (const void *)conv1d_real_stream<4>; break;
    case 5: fn = (const void *)conv1d_real_stream<5>; break;
    case 6: fn = (const void *)conv1d_real_stream<6>; break;
    case 7: fn = (const void *)conv1d_real_stream<7>; break;
    case 8: fn = (const void *)conv1d_real_stream<8>; break;
    default: fn = (const void *)conv1d_real_stream<0>; break;
  }
  int rc = ensure_smem(fn, smem, "conv1d");
  if (rc) return rc;
  // resident CTAs per SM of this variant at this shared-memory size, per device
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) dev = 0;
  int occ = 0;
  {
    static std::mutex mu;
    static std::map<std::tuple<int, const void *, size_t>, int> occ_cache;
    std::lock_guard<std::mutex> lk(mu);
    const auto key = std::make_tuple(dev, fn, smem);
    auto it = occ_cache.find(key);
    if (it != occ_cache.end()) {
      occ = it->second;
    } else {
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, kConvThreads, smem) != cudaSuccess || occ < 1)
        occ = 1;
      occ_cache[key] = occ;
    }
  }
  const int64_t ntiles = p.chunks_per_row * batch;
  const int64_t grid = std::min<int64_t>(ntiles, (int64_t)num_sms() * occ);
  ConvParams pa = p;
  int64_t nt = ntiles;
  void *args[] = {(void *)&pa, (void *)&nt};
  const cudaError_t e = cudaLaunchKernel(fn, dim3((unsigned)grid), dim3(kConvThreads), args, smem, s);
  if (e != cudaSuccess) GBFIR_FAIL(GBFIR_ERR_CUDA, "conv1d: %s", cudaGetErrorString(e));
  return check_launch("conv1d");
}

template <typename T, bool SC, bool FC>
static int launch_conv(const ConvParams &p, int64_t batch, cudaStream_t s) {
  using ST = typename val_of<T, SC>::type;
  using FT = typename val_of<T, FC>::type;
  using OT = typename val_of<T, SC || FC>::type;
  const int lc_max = (int)((p.Lf < kConvChunk ? (p.Lf + kConvE - 1) / kConvE * kConvE : kConvChunk));
  const size_t taps_bytes = ((size_t)lc_max * sizeof(FT) + 15) & ~(size_t)15;
  size_t win_bytes = (size_t)(kConvNB + lc_max) * sizeof(ST);
  if (win_bytes < (size_t)kConvNB * sizeof(OT)) win_bytes = (size_t)kConvNB * sizeof(OT);
  const size_t smem = taps_bytes + win_bytes;
  auto fn = conv1d_direct<T, SC, FC>;
  int rc = ensure_smem((const void *)fn, smem, "conv1d");
  if (rc) return rc;
  const int64_t grid = p.chunks_per_row * batch;
  if (grid > 0x7fffffffLL) GBFIR_FAIL(GBFIR_ERR_INVALID_SIZE, "conv1d: too many output chunks");
  fn<<<(unsigned)grid, kConvThreads, smem, s>>>(p);
  return check_launch("conv1d");
}

// in / h already validated.  x is `in`, the second operand is `h`.
int conv1d_fp(const gbfir_buf &out, const gbfir_buf &in, const gbfir_buf &h, int mode, int is_corr, cudaStream_t s) {
  const bool swap = in.len < h.len;  // conv.h:427
  const gbfir_buf &sig = swap ? h : in;
  const gbfir_buf &fil = swap ? in : h;
  ConvParams p{};
  p.s = sig.ptr;
  p.s_bstride = sig.batch > 1 ? sig.batch_stride : 0;
  p.Ns = sig.len;
  p.f = fil.ptr;
  p.f_bstride = fil.batch > 1 ? fil.batch_stride : 0;
  p.Lf = fil.len;
  p.s_rc = is_corr && swap;
  p.f_rc = is_corr && !swap;
  p.out = out.ptr;
  p.out_bstride = out.batch_stride;
  p.out_len = out.len;
  const int64_t Lmin = fil.len;
  p.start = mode == GBFIR_MODE_SAME ? ((Lmin & 1) ? (Lmin - 1) / 2 : Lmin / 2 - 1)
          : mode == GBFIR_MODE_VALID ? Lmin - 1 : 0;
  p.chunks_per_row = (out.len + kConvNB - 1) / kConvNB;
  const bool sc = dtype_complex(sig.dtype), fcx = dtype_complex(fil.dtype);
  if (dtype_double(in.dtype)) {
    if (sc && fcx) return launch_conv<double, true, true>(p, out.batch, s);
    if (sc) return launch_conv<double, true, false>(p, out.batch, s);
    if (fcx) return launch_conv<double, false, true>(p, out.batch, s);
    return launch_conv<double, false, false>(p, out.batch, s);
  }
  if (sc && fcx) return launch_conv<float, true, true>(p, out.batch, s);
  if (sc) return launch_conv<float, true, false>(p, out.batch, s);
  if (fcx) return launch_conv<float, false, true>(p, out.batch, s);
  if (p.f_bstride == 0 && p.Lf <= kConvChunk) return launch_conv_real_stream(p, out.batch, s);
  return launch_conv<float, false, false>(p, out.batch, s);
}

}  // namespace gbfir
