// conv_axis.cu — direct conv1d / corr along a strided axis, for sm_103a.
//
// Semantics are MatX's direct conv1d applied to a view whose convolved dimension is not
// the innermost one: conv1d(a, b, {axis}, mode) permutes the axis last
// (include/matx/operators/conv.h:263-274) and the radar three-pulse canceller convolves a
// permuted [channel][sample][pulse] view along the pulses
// (examples/simple_radar_pipeline.h:321-327).  Signal (o, i), o < outer, i < inner, is
// x[o*ostride + n*step + i] (n < len; a [outer][len][inner] tensor or a slice of one) and
//   full[n] = sum_k f[k] * s[n - k],   out[o][m][i] = full[m + start],
// start = 0 (FULL), (Lmin-1)/2 or Lmin/2-1 (SAME, odd/even Lmin = min(len, L)), Lmin-1
// (VALID), samples outside [0, len) zero (include/matx/transforms/conv.h:226-289);
// corr uses f = reverse(conj(h)) (include/matx/transforms/corr.h:67).  The taps are
// accumulated in ascending k with MatX's madd, as in conv1d_direct, so for len >= L the
// result equals the row kernel's on the transposed data.
//
// Schedule (no MatX counterpart): threads of a warp take consecutive inner positions, so
// every sample load and output store is a coalesced row of the tensor; a thread walks
// SEG outputs of its signal with the last LMAX + U - 1 samples in registers (U = 4 new
// samples are loaded ahead of each group of 4 outputs, keeping 4 loads in flight), so HBM
// sees each sample about once.  Longer filters read the samples through L1.
#include "common.cuh"

namespace gbfir {

struct AxisParams {
  const void *s;
  int64_t s_ostride, s_step, len, inner;
  const void *h;
  int64_t L;
  int32_t rc;  // reverse-conjugate the filter (corr)
  void *out;
  int64_t o_ostride, o_step, out_len, start;
  int64_t outer, nseg;
  int32_t ti;  // inner positions per CTA (the rest of the CTA's threads take more segments)
};

constexpr int kAxisThreads = 256;
constexpr int kAxisSeg = 32;  // outputs per thread
constexpr int kAxisU = 4;     // outputs per register-window step

template <typename V>
__device__ __forceinline__ V axis_conj(V v) {
  if constexpr (!std::is_arithmetic<V>::value) v.y = -v.y;
  return v;
}

template <typename T, bool SC, bool FC, int LMAX>
__global__ void __launch_bounds__(kAxisThreads) conv1d_axis(const AxisParams p) {
  using ST = typename val_of<T, SC>::type;
  using FT = typename val_of<T, FC>::type;
  constexpr bool OC = SC || FC;
  using OT = typename val_of<T, OC>::type;
  constexpr int U = kAxisU;
  const int tsg = kAxisThreads / p.ti;  // segments per CTA
  const int64_t i = (int64_t)blockIdx.x * p.ti + (threadIdx.x % p.ti);
  const int64_t seg = (int64_t)blockIdx.y * tsg + threadIdx.x / p.ti;
  if (i >= p.inner || seg >= p.nseg) return;
  const FT *hp = reinterpret_cast<const FT *>(p.h);
  for (int64_t o = blockIdx.z; o < p.outer; o += gridDim.z) {
    const ST *sp = reinterpret_cast<const ST *>(p.s) + o * p.s_ostride + i;
    OT *op = reinterpret_cast<OT *>(p.out) + o * p.o_ostride + i;
    const int64_t n0 = seg * kAxisSeg, n1 = min(n0 + kAxisSeg, p.out_len);
    auto ld = [&](int64_t m) -> ST {
      return (m >= 0 && m < p.len) ? __ldg(sp + m * p.s_step) : zero_val<ST>();
    };
    if constexpr (LMAX > 0) {
      FT f[LMAX];
#pragma unroll
      for (int k = 0; k < LMAX; k++) {
        f[k] = zero_val<FT>();
        if (k < p.L) f[k] = p.rc ? axis_conj(__ldg(hp + p.L - 1 - k)) : __ldg(hp + k);
      }
      // w[j] = s[m + U - 1 - j] for the group of outputs m .. m + U - 1 (full-conv index)
      constexpr int W = LMAX + U - 1;
      ST w[W];
      int64_t m = n0 + p.start;
#pragma unroll
      for (int j = 0; j < W; j++) w[j] = ld(m + U - 1 - j);
      for (int64_t n = n0; n < n1; n += U, m += U) {
        ST nx[U];
#pragma unroll
        for (int u = 0; u < U; u++) nx[u] = ld(m + 2 * U - 1 - u);  // next group's newest samples
#pragma unroll
        for (int u = 0; u < U; u++) {
          Acc<T, OC> acc;
          acc.zero();
#pragma unroll
          for (int k = 0; k < LMAX; k++)
            if (k < p.L) mac<T, SC, FC>(acc, w[U - 1 - u + k], f[k]);
          if (n + u < n1) op[(n + u) * p.o_step] = pack<T, OC>(acc, T(1));
        }
#pragma unroll
        for (int j = W - 1; j >= U; j--) w[j] = w[j - U];
#pragma unroll
        for (int u = 0; u < U; u++) w[u] = nx[u];
      }
    } else {
      for (int64_t n = n0; n < n1; n++) {
        const int64_t m = n + p.start;
        Acc<T, OC> acc;
        acc.zero();
        for (int64_t k = 0; k < p.L; k++) {
          const FT t = p.rc ? axis_conj(__ldg(hp + p.L - 1 - k)) : __ldg(hp + k);
          mac<T, SC, FC>(acc, ld(m - k), t);
        }
        op[n * p.o_step] = pack<T, OC>(acc, T(1));
      }
    }
  }
}

template <typename T, bool SC, bool FC>
static int launch_axis(const AxisParams &p0, cudaStream_t s) {
  AxisParams p = p0;
  int ti = 32;
  while (ti < kAxisThreads && ti < p.inner) ti *= 2;
  p.ti = ti;
  const int tsg = kAxisThreads / ti;
  const int64_t gx = (p.inner + ti - 1) / ti, gy = (p.nseg + tsg - 1) / tsg;
  if (gx > 0x7fffffffLL || gy > 65535) GBFIR_FAIL(GBFIR_ERR_INVALID_SIZE, "conv1d (axis): grid too large");
  const unsigned gz = (unsigned)(p.outer < 65535 ? p.outer : 65535);
  const dim3 grid((unsigned)gx, (unsigned)gy, gz);
  // register windows up to 16 taps (8 for double), without spills
  if (p.L <= 4) conv1d_axis<T, SC, FC, 4><<<grid, kAxisThreads, 0, s>>>(p);
  else if (p.L <= 8) conv1d_axis<T, SC, FC, 8><<<grid, kAxisThreads, 0, s>>>(p);
  else if (sizeof(T) == 4 && p.L <= 16) conv1d_axis<T, SC, FC, sizeof(T) == 4 ? 16 : 8><<<grid, kAxisThreads, 0, s>>>(p);
  else conv1d_axis<T, SC, FC, 0><<<grid, kAxisThreads, 0, s>>>(p);
  return check_launch("conv1d (axis)");
}

// out / in / h validated by the caller: signal (b, i) of in / out starts at
// b*batch_stride + i and steps by in_step / out_step elements; h one row.
int conv1d_axis_fp(const gbfir_buf &out, const gbfir_buf &in, const gbfir_buf &h, int64_t inner, int64_t in_step,
                   int64_t out_step, int mode, int is_corr, cudaStream_t s) {
  AxisParams p{};
  p.s = in.ptr;
  p.s_ostride = in.batch > 1 ? in.batch_stride : 0;
  p.s_step = in_step;
  p.len = in.len;
  p.inner = inner;
  p.h = h.ptr;
  p.L = h.len;
  p.rc = is_corr ? 1 : 0;
  p.out = out.ptr;
  p.o_ostride = out.batch > 1 ? out.batch_stride : 0;
  p.o_step = out_step;
  p.out_len = out.len;
  const int64_t Lmin = in.len < h.len ? in.len : h.len;
  p.start = mode == GBFIR_MODE_SAME ? ((Lmin & 1) ? (Lmin - 1) / 2 : Lmin / 2 - 1)
          : mode == GBFIR_MODE_VALID ? Lmin - 1 : 0;
  p.outer = out.batch;
  p.nseg = (out.len + kAxisSeg - 1) / kAxisSeg;
  const bool sc = dtype_complex(in.dtype), fc = dtype_complex(h.dtype);
  if (dtype_double(in.dtype)) {
    if (sc && fc) return launch_axis<double, true, true>(p, s);
    if (sc) return launch_axis<double, true, false>(p, s);
    if (fc) return launch_axis<double, false, true>(p, s);
    return launch_axis<double, false, false>(p, s);
  }
  if (sc && fc) return launch_axis<float, true, true>(p, s);
  if (sc) return launch_axis<float, true, false>(p, s);
  if (fc) return launch_axis<float, false, true>(p, s);
  return launch_axis<float, false, false>(p, s);
}

}  // namespace gbfir
