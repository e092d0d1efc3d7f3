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
  return launch_conv<float, false, false>(p, out.batch, s);
}

}  // namespace gbfir
