// conv_fft.cu — FFT-method conv1d / corr (MatX MATX_C_METHOD_FFT), for sm_103a.
//
// Semantics are MatX's FFT convolution (include/matx/transforms/conv.h:51-172): the full
// linear convolution of each row with the filter (a circular convolution of length N+L-1
// there), then the FULL / SAME / VALID slice with the SAME start (L-1)/2 for odd L, L/2-1
// for even L; corr is conv1d with reverse(conj(h)) (include/matx/transforms/corr.h:67).
// Real operands give real outputs.  Results equal the direct method up to FP32 rounding.
//
// Schedule (no MatX counterpart; MatX pads every row to N+L-1 and runs cuFFT forward on
// signal and filter, a product and an inverse, through HBM temporaries): overlap-save with
// a transform of NF = 2^n points (1024..8192, at least 2L) in shared memory.  A persistent
// CTA builds the twiddle table and the filter's spectrum once, then walks blocks of
// B = NF - L + 1 outputs: it loads the NF-sample window that ends at the block (zero
// outside the row), transforms it in place (radix-16 decimation-in-frequency stages with a
// last stage of radix 4..32, each lane holding one butterfly's points in registers), multiplies by
// the spectrum (both in the same digit-reversed order, so no reordering pass), runs the
// mirror-image decimation-in-time inverse back to natural order and writes the B valid
// outputs.  HBM sees each input about NF/B times (once plus the L-1 overlap) and each
// output once.
#include "common.cuh"

namespace gbfir {

constexpr int kFftThreads = 512;
constexpr int kFftMaxLog = 13;  // NF <= 8192

struct FftConvParams {
  const void *s;
  int64_t s_bstride, N;
  const void *h;
  int64_t L;
  int32_t rc;  // reverse-conjugate the filter (corr)
  int32_t sc, hc;
  void *out;
  int64_t o_bstride, out_len, start;
  int64_t batch, nblk;  // output blocks per row
  int32_t lognf, B;     // transform length 2^lognf, outputs per block
};

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
// a * (-i) (forward) or a * (+i) (inverse)
template <bool INV>
__device__ __forceinline__ float2 mul_mi(float2 a) {
  return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

// In-register DFTs, natural order in and out; INV uses the conjugate roots.
template <bool INV>
__device__ __forceinline__ void dft2(float2 &a, float2 &b) {
  const float2 t = a;
  a = cadd(t, b);
  b = csub(t, b);
}
template <bool INV>
__device__ __forceinline__ void dft4(float2 (&v)[4]) {
  // split on the index: c_r = v[r] + v[r+2], d_r = (v[r] - v[r+2]) W4^r; X[2k] = DFT2(c), X[2k+1] = DFT2(d)
  float2 c0 = cadd(v[0], v[2]), c1 = cadd(v[1], v[3]);
  float2 d0 = csub(v[0], v[2]), d1 = mul_mi<INV>(csub(v[1], v[3]));
  v[0] = cadd(c0, c1);
  v[2] = csub(c0, c1);
  v[1] = cadd(d0, d1);
  v[3] = csub(d0, d1);
}

// cos(2 pi m / 32), m = 0..31 (exact constants of the 32-point circle); a switch, so that
// unrolled callers with constant m fold it away.
__host__ __device__ constexpr float cos32(int m) {
  switch (m & 31) {
    case 0: return 1.0f;
    case 1: return 0.98078528040323044913f;
    case 2: return 0.92387953251128675613f;
    case 3: return 0.83146961230254523708f;
    case 4: return 0.70710678118654752440f;
    case 5: return 0.55557023301960222474f;
    case 6: return 0.38268343236508977173f;
    case 7: return 0.19509032201612826785f;
    case 8: return 0.0f;
    case 9: return -0.19509032201612826785f;
    case 10: return -0.38268343236508977173f;
    case 11: return -0.55557023301960222474f;
    case 12: return -0.70710678118654752440f;
    case 13: return -0.83146961230254523708f;
    case 14: return -0.92387953251128675613f;
    case 15: return -0.98078528040323044913f;
    case 16: return -1.0f;
    case 17: return -0.98078528040323044913f;
    case 18: return -0.92387953251128675613f;
    case 19: return -0.83146961230254523708f;
    case 20: return -0.70710678118654752440f;
    case 21: return -0.55557023301960222474f;
    case 22: return -0.38268343236508977173f;
    case 23: return -0.19509032201612826785f;
    case 24: return 0.0f;
    case 25: return 0.19509032201612826785f;
    case 26: return 0.38268343236508977173f;
    case 27: return 0.55557023301960222474f;
    case 28: return 0.70710678118654752440f;
    case 29: return 0.83146961230254523708f;
    case 30: return 0.92387953251128675613f;
    case 31: return 0.98078528040323044913f;
  }
  return 0.0f;
}

// The R-point DFT (R a power of two up to 32) in registers, natural order in and out, by
// recursive decimation in frequency: a_r = v_r + v_(r+R/2), b_r = (v_r - v_(r+R/2)) W_R^r,
// X_2k = DFT(a)_k, X_2k+1 = DFT(b)_k.  INV uses the conjugate roots.
template <int R, bool INV>
__device__ __forceinline__ void dftp(float2 (&v)[R]) {
  if constexpr (R == 2) {
    dft2<INV>(v[0], v[1]);
  } else if constexpr (R == 4) {
    dft4<INV>(v);
  } else {
    constexpr int Hh = R / 2;
    float2 a[Hh], b[Hh];
#pragma unroll
    for (int r = 0; r < Hh; r++) {
      a[r] = cadd(v[r], v[r + Hh]);
      const float2 d = csub(v[r], v[r + Hh]);
      const int m = r * (32 / R);
      const float c = cos32(m), sn = cos32(m + 24);  // sin(2 pi m / 32) = cos(2 pi (m - 8) / 32)
      b[r] = r == 0 ? d : cmul(d, make_float2(c, INV ? sn : -sn));
    }
    dftp<Hh, INV>(a);
    dftp<Hh, INV>(b);
#pragma unroll
    for (int k = 0; k < Hh; k++) {
      v[2 * k] = a[k];
      v[2 * k + 1] = b[k];
    }
  }
}

// Element p of a transform lives at p + p/16 in shared memory (one pad per 128 bytes): the
// late stages' butterflies, whose points are 8-128 elements apart, then fall on distinct
// banks for the lanes of a half-warp.
__device__ __forceinline__ int fpad(int p) { return p + (p >> 4); }

// The stages of a 2^lognf-point transform: radix-16, then one of radix 4..32; stage s
// works on sub-transforms of ls[s] points, and its twiddles W_ls^(r*k), r = 1..R-1, k <
// ls/R, sit at tw[off[s] + (r-1)*(ls/R) + k] (consecutive lanes read consecutive entries).
struct FftPlan {
  int ns, rad[6], ls[6], off[6], tw_len;
};
__host__ __device__ inline FftPlan fft_plan(int lognf) {
  FftPlan f{};
  int rem = lognf, len = 1 << lognf, off = 0;
  while (rem > 0) {
    const int lr = rem > 5 ? 4 : rem;  // radix-16 stages, the last of up to radix 32
    f.rad[f.ns] = 1 << lr;
    f.ls[f.ns] = len;
    f.off[f.ns] = off;
    off += ((1 << lr) - 1) * (len >> lr);
    len >>= lr;
    rem -= lr;
    f.ns++;
  }
  f.tw_len = off;
  return f;
}

// One stage in shared memory: butterfly (g, k) on X[g*ls + k + r*ls/R].  Forward
// (decimation in frequency): R-point DFT, then twiddle W_ls^(r*k).  Inverse (the mirror,
// decimation in time): the conjugate twiddle, then the inverse R-point DFT.
template <int R, bool INV>
__device__ __forceinline__ void fft_stage(float2 *X, const float2 *tw, int nf, int ls) {
  const int q = ls / R;
  for (int t = threadIdx.x; t < nf / R; t += blockDim.x) {
    const int g = t / q, k = t - g * q;
    const int base = g * ls + k;
    float2 v[R];
#pragma unroll
    for (int r = 0; r < R; r++) v[r] = X[fpad(base + r * q)];
    if constexpr (INV) {
#pragma unroll
      for (int r = 1; r < R; r++) v[r] = cmul(v[r], cconj(tw[(r - 1) * q + k]));
    }
    dftp<R, INV>(v);
    if constexpr (!INV) {
#pragma unroll
      for (int r = 1; r < R; r++) v[r] = cmul(v[r], tw[(r - 1) * q + k]);
    }
#pragma unroll
    for (int r = 0; r < R; r++) X[fpad(base + r * q)] = v[r];
  }
}

template <bool INV>
__device__ __forceinline__ void stage_any(float2 *X, const float2 *tw, const FftPlan &f, int s, int nf) {
  __syncthreads();
  switch (f.rad[s]) {
    case 32: fft_stage<32, INV>(X, tw + f.off[s], nf, f.ls[s]); break;
    case 16: fft_stage<16, INV>(X, tw + f.off[s], nf, f.ls[s]); break;
    case 8: fft_stage<8, INV>(X, tw + f.off[s], nf, f.ls[s]); break;
    case 4: fft_stage<4, INV>(X, tw + f.off[s], nf, f.ls[s]); break;
    default: fft_stage<2, INV>(X, tw + f.off[s], nf, f.ls[s]); break;
  }
}

// The full forward transform in shared memory (for the filter's spectrum); the result is
// in digit-reversed order.
__device__ void fft_forward(float2 *X, const float2 *tw, const FftPlan &f, int nf) {
  for (int s = 0; s < f.ns; s++) stage_any<false>(X, tw, f, s, nf);
  __syncthreads();
}

// The last forward stage, the product with the spectrum and the first inverse stage on the
// same butterflies: their twiddles cancel (|W| = 1), so only the two DFTs remain.
template <int R>
__device__ __forceinline__ void fft_middle(float2 *X, const float2 *H, int nf, int ls) {
  const int q = ls / R;
  for (int t = threadIdx.x; t < nf / R; t += blockDim.x) {
    const int g = t / q, k = t - g * q;
    const int base = g * ls + k;
    float2 v[R];
#pragma unroll
    for (int r = 0; r < R; r++) v[r] = X[fpad(base + r * q)];
    dftp<R, false>(v);
#pragma unroll
    for (int r = 0; r < R; r++) v[r] = cmul(v[r], H[fpad(base + r * q)]);
    dftp<R, true>(v);
#pragma unroll
    for (int r = 0; r < R; r++) X[fpad(base + r * q)] = v[r];
  }
}

// The first forward stage (radix 16, ls = nf) straight from the global window: lane k loads
// window samples k + r*nf/16, coalesced across the warp.
template <bool SC>
__device__ __forceinline__ void fft_first(float2 *X, const float2 *tw, const FftConvParams &p, int nf, int64_t b,
                                          int64_t ws) {
  constexpr int R = 16;
  const int q = nf / R;
  for (int k = threadIdx.x; k < q; k += blockDim.x) {
    float2 v[R];
#pragma unroll
    for (int r = 0; r < R; r++) {
      const int64_t n = ws + k + r * q;
      v[r] = make_float2(0.f, 0.f);
      if (n >= 0 && n < p.N) {
        if constexpr (SC) v[r] = reinterpret_cast<const float2 *>(p.s)[b * p.s_bstride + n];
        else v[r].x = reinterpret_cast<const float *>(p.s)[b * p.s_bstride + n];
      }
    }
    dftp<R, false>(v);
#pragma unroll
    for (int r = 1; r < R; r++) v[r] = cmul(v[r], tw[(r - 1) * q + k]);
#pragma unroll
    for (int r = 0; r < R; r++) X[fpad(k + r * q)] = v[r];
  }
}

// The last inverse stage (radix 16, ls = nf) straight to the output: positions k + r*nf/16
// in [L-1, L-1+B) are block outputs.
template <bool OC>
__device__ __forceinline__ void fft_last(const float2 *X, const float2 *tw, const FftConvParams &p, int nf,
                                         int64_t b, int64_t o0) {
  constexpr int R = 16;
  const int q = nf / R;
  for (int k = threadIdx.x; k < q; k += blockDim.x) {
    float2 v[R];
#pragma unroll
    for (int r = 0; r < R; r++) v[r] = X[fpad(k + r * q)];
#pragma unroll
    for (int r = 1; r < R; r++) v[r] = cmul(v[r], cconj(tw[(r - 1) * q + k]));
    dftp<R, true>(v);
#pragma unroll
    for (int r = 0; r < R; r++) {
      const int pos = k + r * q;
      const int64_t o = o0 + pos - (p.L - 1);
      if (pos >= p.L - 1 && pos < p.L - 1 + p.B && o < p.out_len) {
        if constexpr (OC) reinterpret_cast<float2 *>(p.out)[b * p.o_bstride + o] = v[r];
        else reinterpret_cast<float *>(p.out)[b * p.o_bstride + o] = v[r].x;
      }
    }
  }
}

template <bool SC, bool HC>
__global__ void __launch_bounds__(kFftThreads) conv1d_fft(const FftConvParams p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int nf = 1 << p.lognf, npad = fpad(nf);
  const FftPlan f = fft_plan(p.lognf);
  float2 *H = reinterpret_cast<float2 *>(smem_raw);
  float2 *X = H + npad;
  float2 *tw = X + npad;
  const int tid = threadIdx.x;
  for (int s = 0; s < f.ns; s++) {
    const int q = f.ls[s] / f.rad[s];
    for (int e = tid; e < (f.rad[s] - 1) * q; e += blockDim.x) {
      const int r = e / q + 1, k = e - (r - 1) * q;
      float sn, cs;
      sincospif(-2.0f * (float)(r * k) / (float)f.ls[s], &sn, &cs);  // exp(-2 pi i r k / ls)
      tw[f.off[s] + e] = make_float2(cs, sn);
    }
  }
  for (int m = tid; m < nf; m += blockDim.x) {
    float2 v = make_float2(0.f, 0.f);
    if (m < p.L) {
      const int64_t k = p.rc ? p.L - 1 - m : m;
      if constexpr (HC) {
        v = reinterpret_cast<const float2 *>(p.h)[k];
        if (p.rc) v.y = -v.y;
      } else {
        v.x = reinterpret_cast<const float *>(p.h)[k];
      }
    }
    H[fpad(m)] = v;
  }
  fft_forward(H, tw, f, nf);
  const float inv = 1.0f / (float)nf;  // the inverse transform's 1/NF, folded into the spectrum
  for (int m = tid; m < nf; m += blockDim.x) {
    const float2 v = H[fpad(m)];
    H[fpad(m)] = make_float2(v.x * inv, v.y * inv);
  }

  const int64_t work = p.batch * p.nblk;
  const int last = f.ns - 1;
  for (int64_t w = blockIdx.x; w < work; w += gridDim.x) {
    const int64_t b = w / p.nblk, j = w - b * p.nblk;
    const int64_t o0 = j * p.B;
    const int64_t ws = o0 + p.start - (p.L - 1);  // first window sample
    __syncthreads();  // the previous block is drained (and the spectrum is ready)
    fft_first<SC>(X, tw + f.off[0], p, nf, b, ws);
    for (int s = 1; s < last; s++) stage_any<false>(X, tw, f, s, nf);
    __syncthreads();
    switch (f.rad[last]) {
      case 32: fft_middle<32>(X, H, nf, f.ls[last]); break;
      case 16: fft_middle<16>(X, H, nf, f.ls[last]); break;
      case 8: fft_middle<8>(X, H, nf, f.ls[last]); break;
      default: fft_middle<4>(X, H, nf, f.ls[last]); break;
    }
    for (int s = last - 1; s >= 1; s--) stage_any<true>(X, tw, f, s, nf);
    __syncthreads();
    fft_last<SC || HC>(X, tw + f.off[0], p, nf, b, o0);
  }
}

// The transform length for an L-tap filter: at least 2L and 1024, at most 8192 with at
// least 1024 outputs per block; 0 when the filter is too long.
int fft_conv_lognf(int64_t L) {
  int lg = 10;
  while ((1LL << lg) < 2 * L && lg < kFftMaxLog) lg++;
  if ((1LL << lg) < 2 * L && (1LL << lg) - L + 1 < 1024) return 0;
  return lg;
}

// Shapes validated by the caller (h one row, float32 / complex64 operands).
int conv1d_fft_fp(const gbfir_buf &out, const gbfir_buf &in, const gbfir_buf &h, int mode, int is_corr,
                  cudaStream_t s) {
  FftConvParams p{};
  p.s = in.ptr;
  p.s_bstride = in.batch > 1 ? in.batch_stride : 0;
  p.N = in.len;
  p.h = h.ptr;
  p.L = h.len;
  p.rc = is_corr ? 1 : 0;
  p.sc = dtype_complex(in.dtype);
  p.hc = dtype_complex(h.dtype);
  p.out = out.ptr;
  p.o_bstride = out.batch_stride;
  p.out_len = out.len;
  // MatX slices the full convolution with the filter's length (transforms/conv.h:139-160)
  p.start = mode == GBFIR_MODE_SAME ? ((h.len & 1) ? (h.len - 1) / 2 : h.len / 2 - 1)
          : mode == GBFIR_MODE_VALID ? h.len - 1 : 0;
  p.lognf = fft_conv_lognf(h.len);
  if (p.lognf == 0) GBFIR_FAIL(GBFIR_ERR_NOT_SUPPORTED, "conv1d (FFT): filters longer than 7169 taps");
  p.B = (1 << p.lognf) - (int)h.len + 1;
  p.batch = out.batch;
  p.nblk = (out.len + p.B - 1) / p.B;
  const int nf = 1 << p.lognf;
  const size_t smem = (size_t)(2 * (nf + (nf >> 4)) + fft_plan(p.lognf).tw_len) * sizeof(float2);
  auto launch = [&](auto fn) -> int {
    int rc = ensure_smem((const void *)fn, smem, "conv1d (FFT)");
    if (rc) return rc;
    int occ = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, kFftThreads, smem);
    if (occ < 1) occ = 1;
    int64_t grid = (int64_t)num_sms() * occ;
    if (grid > p.batch * p.nblk) grid = p.batch * p.nblk;
    fn<<<(unsigned)grid, kFftThreads, smem, s>>>(p);
    return check_launch("conv1d (FFT)");
  };
  if (p.sc && p.hc) return launch(conv1d_fft<true, true>);
  if (p.sc) return launch(conv1d_fft<true, false>);
  if (p.hc) return launch(conv1d_fft<false, true>);
  return launch(conv1d_fft<false, false>);
}

}  // namespace gbfir
