// tc_channelize.cu — channelize_poly with the M-point DFT as a dense complex GEMM on the
// tcgen05 tensor cores (bf16, fp16, bf16x3; FP32 accumulate in TMEM).  No MatX counterpart.
//
// Semantics are those of channelize_fused (channelize.cu) for D == M: the branch filters
// F[t][c] = sum_p h[p*M + c] * x[(t - p)*M + (M-1-c)] run on the CUDA cores in FP32 and
// stay in registers; then
//   Y[t][k] = sum_c F[t][c] * exp(+2*pi*i*c*k/M)
// is computed as real GEMMs with D[t][k] = sum_c A[t][c] * B[k][c]:
//   D_re = F_re * C^T - F_im * S^T,   D_im = F_re * S^T + F_im * C^T,
//   C[k][c] = cos(2*pi*c*k/M), S[k][c] = sin(2*pi*c*k/M)
// (the minus sign through the instruction descriptor's negate-A bit).  One CTA owns 128
// consecutive output steps (MMA M = 128) and all M <= 64 channels: N = M columns per
// accumulator, K = M input channels.  bf16x3 splits F and the twiddles into three bf16
// terms and accumulates the six products of order <= 2 (smallest first).
// The FIR results are written as MMA operands into the input-window buffer once every
// thread has finished reading the window, so the kernel needs window + twiddles of
// shared memory.  All waits are bounded (tc.cuh).
#include "common.cuh"
#include "tc.cuh"

namespace gbfir {

constexpr int kTcChThreads = 256;
constexpr int kTcChTT = 128;  // output steps per tile (MMA M)
constexpr int kTcChE = 8;

struct TcChParams {
  const float2 *x;
  int64_t x_bstride, N;
  const float *h;
  int64_t L;
  float2 *out;
  int64_t out_bstride;
  int32_t M, P, Ppad;
  int64_t T, tiles_per_row, ntiles;
  int32_t terms, fp16;
  int32_t tap_stride;
  int32_t W;  // window samples
};

// Bounded-wait status of the channelizer kernels of this file (1 = a wait gave up); read and
// cleared by gbfir_tc_status() through tc_channelize_status_take().
__device__ int32_t g_tcch_status;

int tc_channelize_status_take() {
  int32_t v = 0, zero = 0;
  if (cudaMemcpyFromSymbol(&v, g_tcch_status, sizeof(v)) != cudaSuccess) return -1;
  cudaMemcpyToSymbol(g_tcch_status, &zero, sizeof(zero));
  return v;
}

__global__ void __launch_bounds__(kTcChThreads) tc_channelize_kernel(const TcChParams p) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ uint64_t bar;
  __shared__ uint32_t tmem_slot;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int M = p.M;
  // layout: [twiddle terms: {C, S} x terms x (M x M) bf16][taps: M x tap_stride f32][window / A operands]
  const uint32_t tbytes = (uint32_t)M * M * 2u;  // one twiddle matrix, one term
  unsigned char *tw = smem;
  auto twm = [&](int which, int t) { return tw + ((size_t)which * p.terms + t) * tbytes; };
  size_t off = ((size_t)2 * p.terms * tbytes + 127) / 128 * 128;
  float *taps = reinterpret_cast<float *>(smem + off);
  off += ((size_t)M * p.tap_stride * 4 + 127) / 128 * 128;
  unsigned char *region = smem + off;
  float2 *win = reinterpret_cast<float2 *>(region);
  const uint32_t abytes = (uint32_t)kTcChTT * M * 2u;  // one A operand (128 x M), one term
  auto aop = [&](int part, int t) { return region + ((size_t)part * p.terms + t) * abytes; };

  if (warp == 0) tc::tmem_alloc(&tmem_slot, (uint32_t)(2 * M < 32 ? 32 : 2 * M));
  if (tid == 0) {
    tc::mbar_init(&bar, 1);
    tc::mbar_fence_init();
  }
  // twiddles C[k][c], S[k][c] in the K-major core layout (rows k, K = c), split into terms
  for (int e = tid; e < M * M; e += kTcChThreads) {
    const int k = e / M, c = e - k * M;
    float sv, cv;
    sincospif((float)(2 * ((k * c) % M)) / (float)M, &sv, &cv);
    const uint32_t o = tc::kmajor_offset(k, c, M);
    if (p.fp16) {
      *reinterpret_cast<__half *>(twm(0, 0) + o) = __float2half_rn(cv);
      *reinterpret_cast<__half *>(twm(1, 0) + o) = __float2half_rn(sv);
    } else {
      __nv_bfloat16 a0, a1, a2, b0, b1, b2;
      tc::split3_bf16(cv, a0, a1, a2);
      tc::split3_bf16(sv, b0, b1, b2);
      *reinterpret_cast<__nv_bfloat16 *>(twm(0, 0) + o) = a0;
      *reinterpret_cast<__nv_bfloat16 *>(twm(1, 0) + o) = b0;
      if (p.terms == 3) {
        *reinterpret_cast<__nv_bfloat16 *>(twm(0, 1) + o) = a1;
        *reinterpret_cast<__nv_bfloat16 *>(twm(0, 2) + o) = a2;
        *reinterpret_cast<__nv_bfloat16 *>(twm(1, 1) + o) = b1;
        *reinterpret_cast<__nv_bfloat16 *>(twm(1, 2) + o) = b2;
      }
    }
  }
  for (int e = tid; e < M * p.tap_stride; e += kTcChThreads) {
    const int c = e / p.tap_stride, pp = e - c * p.tap_stride;
    const int64_t idx = (int64_t)pp * M + c;
    taps[e] = (pp < p.P && idx < p.L) ? p.h[idx] : 0.f;
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = tmem_slot;
  const uint32_t idesc = tc::idesc_f16(128, (uint32_t)M, p.fp16 ? 0u : 1u);
  const uint32_t idesc_neg = idesc | (1u << 13);  // negate A
  const int pa3[6] = {2, 1, 0, 1, 0, 0}, pb3[6] = {0, 1, 2, 0, 1, 0};
  const int npairs = p.terms == 3 ? 6 : 1;
  constexpr int E = kTcChE;
  const int items_per_thread = (M * (kTcChTT / E) + kTcChThreads - 1) / kTcChThreads;  // <= 4 for M <= 64
  uint32_t phase = 0;
  bool ok = true;

  for (int64_t tile = blockIdx.x; tile < p.ntiles; tile += gridDim.x) {
    const int64_t b = tile / p.tiles_per_row;
    const int64_t t0 = (tile - b * p.tiles_per_row) * kTcChTT;
    const float2 *row = p.x + b * p.x_bstride;
    const int64_t w0 = (t0 - p.Ppad) * (int64_t)M;
    for (int e = tid; e < p.W; e += kTcChThreads) {
      const int64_t gi = w0 + e;
      const bool okk = gi >= 0 && gi < p.N;
      cp_async_zfill<8>(&win[e], okk ? (const void *)(row + gi) : (const void *)row, okk);
    }
    cp_async_commit();
    cp_async_wait<0>();
    __syncthreads();

    // ---- FIR: items (channel c, run r of 8 steps); results kept in registers ----
    float fr[4][E], fi[4][E];
#pragma unroll
    for (int it = 0; it < 4; it++) {
      const int w = tid + it * kTcChThreads;
#pragma unroll
      for (int e = 0; e < E; e++) {
        fr[it][e] = 0.f;
        fi[it][e] = 0.f;
      }
      if (it >= items_per_thread || w >= M * (kTcChTT / E)) continue;
      const int c = w % M, r = w / M;
      const int sc = M - 1 - c;
      const float *th = taps + (size_t)c * p.tap_stride;
      float2 cur[E], prv[E];
      int rowi = r * E + p.Ppad;
#pragma unroll
      for (int e = 0; e < E; e++) cur[e] = win[(rowi + e) * M + sc];
      for (int kb = 0; kb < p.Ppad; kb += E) {
        rowi -= E;
#pragma unroll
        for (int e = 0; e < E; e++) prv[e] = win[(rowi + e) * M + sc];
#pragma unroll
        for (int kk = 0; kk < E; kk++) {
          const float t = th[kb + kk];
#pragma unroll
          for (int e = 0; e < E; e++) {
            const float2 xv = (e >= kk) ? cur[e - kk] : prv[E + e - kk];
            fr[it][e] = fmaf(xv.x, t, fr[it][e]);
            fi[it][e] = fmaf(xv.y, t, fi[it][e]);
          }
        }
#pragma unroll
        for (int e = 0; e < E; e++) cur[e] = prv[e];
      }
    }
    __syncthreads();  // window no longer read: reuse it for the A operands
#pragma unroll
    for (int it = 0; it < 4; it++) {
      const int w = tid + it * kTcChThreads;
      if (it >= items_per_thread || w >= M * (kTcChTT / E)) continue;
      const int c = w % M, r = w / M;
#pragma unroll
      for (int e = 0; e < E; e++) {
        const int t = r * E + e;
        const uint32_t o = tc::kmajor_offset(t, c, M);
        if (p.fp16) {
          *reinterpret_cast<__half *>(aop(0, 0) + o) = __float2half_rn(fr[it][e]);
          *reinterpret_cast<__half *>(aop(1, 0) + o) = __float2half_rn(fi[it][e]);
        } else {
          __nv_bfloat16 a0, a1, a2, b0, b1, b2;
          tc::split3_bf16(fr[it][e], a0, a1, a2);
          tc::split3_bf16(fi[it][e], b0, b1, b2);
          *reinterpret_cast<__nv_bfloat16 *>(aop(0, 0) + o) = a0;
          *reinterpret_cast<__nv_bfloat16 *>(aop(1, 0) + o) = b0;
          if (p.terms == 3) {
            *reinterpret_cast<__nv_bfloat16 *>(aop(0, 1) + o) = a1;
            *reinterpret_cast<__nv_bfloat16 *>(aop(0, 2) + o) = a2;
            *reinterpret_cast<__nv_bfloat16 *>(aop(1, 1) + o) = b1;
            *reinterpret_cast<__nv_bfloat16 *>(aop(1, 2) + o) = b2;
          }
        }
      }
    }
    tc::fence_async_smem();
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();

    // ---- DFT GEMM: D_re at columns [0, M), D_im at [M, 2M) ----
    if (tid == 0) {
      const uint32_t sbo = (uint32_t)(M / 8) * 128u;
      const int nks = M / 16;
      for (int dpart = 0; dpart < 2; dpart++) {
        const uint32_t d = tmem + (uint32_t)(dpart * M);
        uint32_t acc = 0;
        for (int pi = 0; pi < npairs; pi++) {
          const int ta = p.terms == 3 ? pa3[pi] : 0, tb = p.terms == 3 ? pb3[pi] : 0;
          // D_re += F_re C - F_im S ; D_im += F_re S + F_im C
          for (int src = 0; src < 2; src++) {
            const int which = (dpart == 0) ? (src == 0 ? 0 : 1) : (src == 0 ? 1 : 0);
            const uint32_t id = (dpart == 0 && src == 1) ? idesc_neg : idesc;
            uint64_t ad = tc::smem_desc(tc::smem_u32(aop(src, ta)), 128u, sbo);
            uint64_t bd = tc::smem_desc(tc::smem_u32(twm(which, tb)), 128u, sbo);
            for (int ks = 0; ks < nks; ks++) {
              tc::mma_f16(d, ad, bd, id, acc);
              acc = 1;
              ad += 16;  // +256 B = two core matrices along K
              bd += 16;
            }
          }
        }
      }
      tc::mma_commit(&bar);
    }
    const bool got = tc::mbar_wait(&bar, phase);
    phase ^= 1u;
    if (!got) {
      ok = false;
      if (tid == 0) atomicExch(&g_tcch_status, 1);
    }
    tc::tc_fence_after();
    if (got && warp < 4) {
      const int64_t t = t0 + 32 * warp + lane;
      float2 *orow = p.out + b * p.out_bstride + t * M;
      const uint32_t lane_base = (uint32_t)(32 * warp) << 16;
      for (int col = 0; col < M; col += 16) {
        uint32_t rr[16], ri[16];
        tc::tmem_ld16(tmem + lane_base + (uint32_t)col, rr);
        tc::tmem_ld16(tmem + lane_base + (uint32_t)(M + col), ri);
        tc::tmem_ld_wait();
        if (t < p.T) {
#pragma unroll
          for (int i = 0; i < 16; i++) orow[col + i] = make_float2(__uint_as_float(rr[i]), __uint_as_float(ri[i]));
        }
      }
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    if (!ok) break;
  }
  if (!ok && tid == 0) (void)tc::mbar_wait(&bar, phase);
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc::tc_fence_after();
    tc::tmem_dealloc(tmem, (uint32_t)(2 * M < 32 ? 32 : 2 * M));
  }
}

// ---- M = 64 * R (R = 2, 4): a radix-R stage in FP32 registers, then one 64-point DFT GEMM ----
// With c = 64a + c' and k = k1 + R*k2 (a, k1 < R; c', k2 < 64):
//   exp(2*pi*i*c*k/M) = exp(2*pi*i*a*k1/R) * exp(2*pi*i*c'*k1/M) * exp(2*pi*i*c'*k2/64),
// so Y[t][k1 + R*k2] = sum_c' G[t][k1][c'] * exp(2*pi*i*c'*k2/64) with
//   G[t][k1][c'] = exp(2*pi*i*c'*k1/M) * sum_a F[t][64a + c'] * exp(2*pi*i*a*k1/R)
// (R-point DFTs and twiddles, FP32, straight after the branch filters).  The GEMM's 128 MMA
// rows are the (step, k1) pairs of 128/R consecutive steps (row = R*t + k1), K = c' (64),
// and N = 128: the twiddle matrices [C | S] and [-S | C] put D_re in columns 0-63 and D_im in
// 64-127 (D = G_re [C|S] + G_im [-S|C]).  Only the 64-point twiddles are stored (bf16x3:
// 96 KB), so M = 256 fits where its 256-point matrices would not.  Lane L of an epilogue warp
// holds row R*t + k1: the R lanes of one step write R consecutive channels per column.
template <int R>
__global__ void __launch_bounds__(kTcChThreads) tc_channelize_rad_kernel(const TcChParams p) {
  constexpr int TS = kTcChTT / R;  // output steps per tile
  constexpr int E = kTcChE;
  constexpr int NIT = (64 * (TS / E) + kTcChThreads - 1) / kTcChThreads;  // FIR items per thread
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ uint64_t bar;
  __shared__ uint32_t tmem_slot;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int M = p.M;  // 64 * R
  // layout: [B1 = [C|S], B2 = [-S|C] : terms x (128 x 64) bf16][taps: M x tap_stride f32][window / A]
  const uint32_t bbytes = 128u * 64u * 2u;
  auto bmat = [&](int which, int t) { return smem + ((size_t)which * p.terms + t) * bbytes; };
  size_t off = (size_t)2 * p.terms * bbytes;
  float *taps = reinterpret_cast<float *>(smem + off);
  off += ((size_t)M * p.tap_stride * 4 + 127) / 128 * 128;
  unsigned char *region = smem + off;
  float2 *win = reinterpret_cast<float2 *>(region);
  const uint32_t abytes = 128u * 64u * 2u;  // one A operand (128 rows x 64), one term
  auto aop = [&](int part, int t) { return region + ((size_t)part * p.terms + t) * abytes; };

  if (warp == 0) tc::tmem_alloc(&tmem_slot, 128u);
  if (tid == 0) {
    tc::mbar_init(&bar, 1);
    tc::mbar_fence_init();
  }
  for (int e = tid; e < 128 * 64; e += kTcChThreads) {
    const int n = e / 64, c = e - n * 64;
    const int k = n & 63;
    float sv, cv;
    sincospif((float)(2 * ((k * c) & 63)) / 64.f, &sv, &cv);
    const float v1 = n < 64 ? cv : sv, v2 = n < 64 ? -sv : cv;
    const uint32_t o = tc::kmajor_offset(n, c, 64);
    if (p.fp16) {
      *reinterpret_cast<__half *>(bmat(0, 0) + o) = __float2half_rn(v1);
      *reinterpret_cast<__half *>(bmat(1, 0) + o) = __float2half_rn(v2);
    } else {
      __nv_bfloat16 a0, a1, a2, b0, b1, b2;
      tc::split3_bf16(v1, a0, a1, a2);
      tc::split3_bf16(v2, b0, b1, b2);
      *reinterpret_cast<__nv_bfloat16 *>(bmat(0, 0) + o) = a0;
      *reinterpret_cast<__nv_bfloat16 *>(bmat(1, 0) + o) = b0;
      if (p.terms == 3) {
        *reinterpret_cast<__nv_bfloat16 *>(bmat(0, 1) + o) = a1;
        *reinterpret_cast<__nv_bfloat16 *>(bmat(0, 2) + o) = a2;
        *reinterpret_cast<__nv_bfloat16 *>(bmat(1, 1) + o) = b1;
        *reinterpret_cast<__nv_bfloat16 *>(bmat(1, 2) + o) = b2;
      }
    }
  }
  for (int e = tid; e < M * p.tap_stride; e += kTcChThreads) {
    const int c = e / p.tap_stride, pp = e - c * p.tap_stride;
    const int64_t idx = (int64_t)pp * M + c;
    taps[e] = (pp < p.P && idx < p.L) ? p.h[idx] : 0.f;
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = tmem_slot;
  const uint32_t idesc = tc::idesc_f16(128, 128, p.fp16 ? 0u : 1u);
  const int pa3[6] = {2, 1, 0, 1, 0, 0}, pb3[6] = {0, 1, 2, 0, 1, 0};
  const int npairs = p.terms == 3 ? 6 : 1;
  uint32_t phase = 0;
  bool ok = true;

  for (int64_t tile = blockIdx.x; tile < p.ntiles; tile += gridDim.x) {
    const int64_t b = tile / p.tiles_per_row;
    const int64_t t0 = (tile - b * p.tiles_per_row) * TS;
    const float2 *row = p.x + b * p.x_bstride;
    const int64_t w0 = (t0 - p.Ppad) * (int64_t)M;
    for (int e = tid; e < p.W; e += kTcChThreads) {
      const int64_t gi = w0 + e;
      const bool okk = gi >= 0 && gi < p.N;
      cp_async_zfill<8>(&win[e], okk ? (const void *)(row + gi) : (const void *)row, okk);
    }
    cp_async_commit();
    cp_async_wait<0>();
    __syncthreads();
    // ---- branch filters: item (c', run r of 8 steps) computes channels c' + 64a, a < R ----
    float fr[NIT][R][E], fi[NIT][R][E];
#pragma unroll
    for (int it = 0; it < NIT; it++) {
      const int w = tid + it * kTcChThreads;
#pragma unroll
      for (int a = 0; a < R; a++)
#pragma unroll
        for (int e = 0; e < E; e++) {
          fr[it][a][e] = 0.f;
          fi[it][a][e] = 0.f;
        }
      if (w >= 64 * (TS / E)) continue;
      const int cp = w & 63, r = w >> 6;
#pragma unroll
      for (int a = 0; a < R; a++) {
        const int c = cp + 64 * a;
        const int sc = M - 1 - c;
        const float *th = taps + (size_t)c * p.tap_stride;
        float2 cur[E], prv[E];
        int rowi = r * E + p.Ppad;
#pragma unroll
        for (int e = 0; e < E; e++) cur[e] = win[(rowi + e) * M + sc];
        for (int kb = 0; kb < p.Ppad; kb += E) {
          rowi -= E;
#pragma unroll
          for (int e = 0; e < E; e++) prv[e] = win[(rowi + e) * M + sc];
#pragma unroll
          for (int kk = 0; kk < E; kk++) {
            const float t = th[kb + kk];
#pragma unroll
            for (int e = 0; e < E; e++) {
              const float2 xv = (e >= kk) ? cur[e - kk] : prv[E + e - kk];
              fr[it][a][e] = fmaf(xv.x, t, fr[it][a][e]);
              fi[it][a][e] = fmaf(xv.y, t, fi[it][a][e]);
            }
          }
#pragma unroll
          for (int e = 0; e < E; e++) cur[e] = prv[e];
        }
      }
    }
    __syncthreads();  // window no longer read: reuse it for the A operands
    // ---- R-point DFTs (positive sign) and twiddles exp(2*pi*i*c'*k1/M); A[R*t + k1][c'] ----
#pragma unroll
    for (int it = 0; it < NIT; it++) {
      const int w = tid + it * kTcChThreads;
      if (w >= 64 * (TS / E)) continue;
      const int cp = w & 63, r = w >> 6;
      float twc[R], tws[R];
#pragma unroll
      for (int k1 = 0; k1 < R; k1++) sincospif((float)(2 * ((cp * k1) % M)) / (float)M, &tws[k1], &twc[k1]);
#pragma unroll
      for (int e = 0; e < E; e++) {
        float xr[R], xi[R];
        if constexpr (R == 2) {
          xr[0] = fr[it][0][e] + fr[it][1][e];
          xi[0] = fi[it][0][e] + fi[it][1][e];
          xr[1] = fr[it][0][e] - fr[it][1][e];
          xi[1] = fi[it][0][e] - fi[it][1][e];
        } else {
          const float s02r = fr[it][0][e] + fr[it][2][e], s02i = fi[it][0][e] + fi[it][2][e];
          const float d02r = fr[it][0][e] - fr[it][2][e], d02i = fi[it][0][e] - fi[it][2][e];
          const float s13r = fr[it][1][e] + fr[it][3][e], s13i = fi[it][1][e] + fi[it][3][e];
          const float d13r = fr[it][1][e] - fr[it][3][e], d13i = fi[it][1][e] - fi[it][3][e];
          xr[0] = s02r + s13r;  // F0 + F1 + F2 + F3
          xi[0] = s02i + s13i;
          xr[1] = d02r - d13i;  // F0 + i F1 - F2 - i F3
          xi[1] = d02i + d13r;
          xr[2] = s02r - s13r;  // F0 - F1 + F2 - F3
          xi[2] = s02i - s13i;
          xr[3] = d02r + d13i;  // F0 - i F1 - F2 + i F3
          xi[3] = d02i - d13r;
        }
        const int t = r * E + e;
#pragma unroll
        for (int k1 = 0; k1 < R; k1++) {
          const float gr = xr[k1] * twc[k1] - xi[k1] * tws[k1];
          const float gi = xr[k1] * tws[k1] + xi[k1] * twc[k1];
          const uint32_t o = tc::kmajor_offset(R * t + k1, cp, 64);
          if (p.fp16) {
            *reinterpret_cast<__half *>(aop(0, 0) + o) = __float2half_rn(gr);
            *reinterpret_cast<__half *>(aop(1, 0) + o) = __float2half_rn(gi);
          } else {
            __nv_bfloat16 a0, a1, a2, b0, b1, b2;
            tc::split3_bf16(gr, a0, a1, a2);
            tc::split3_bf16(gi, b0, b1, b2);
            *reinterpret_cast<__nv_bfloat16 *>(aop(0, 0) + o) = a0;
            *reinterpret_cast<__nv_bfloat16 *>(aop(1, 0) + o) = b0;
            if (p.terms == 3) {
              *reinterpret_cast<__nv_bfloat16 *>(aop(0, 1) + o) = a1;
              *reinterpret_cast<__nv_bfloat16 *>(aop(0, 2) + o) = a2;
              *reinterpret_cast<__nv_bfloat16 *>(aop(1, 1) + o) = b1;
              *reinterpret_cast<__nv_bfloat16 *>(aop(1, 2) + o) = b2;
            }
          }
        }
      }
    }
    tc::fence_async_smem();
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    // ---- 64-point DFT GEMM: D[row][0:64) = Y_re, D[row][64:128) = Y_im ----
    if (tid == 0) {
      uint32_t acc = 0;
      for (int pi = 0; pi < npairs; pi++) {
        const int ta = p.terms == 3 ? pa3[pi] : 0, tb = p.terms == 3 ? pb3[pi] : 0;
        for (int src = 0; src < 2; src++) {  // G_re [C|S], G_im [-S|C]
          uint64_t ad = tc::smem_desc(tc::smem_u32(aop(src, ta)), 128u, 1024u);
          uint64_t bd = tc::smem_desc(tc::smem_u32(bmat(src, tb)), 128u, 1024u);
          for (int ks = 0; ks < 4; ks++) {
            tc::mma_f16(tmem, ad, bd, idesc, acc);
            acc = 1;
            ad += 16;  // +256 B = two core matrices along K
            bd += 16;
          }
        }
      }
      tc::mma_commit(&bar);
    }
    const bool got = tc::mbar_wait(&bar, phase);
    phase ^= 1u;
    if (!got) {
      ok = false;
      if (tid == 0) atomicExch(&g_tcch_status, 1);
    }
    tc::tc_fence_after();
    if (got && warp < 4) {
      const int rowl = 32 * warp + lane;
      const int64_t t = t0 + rowl / R;
      const int k1 = rowl % R;
      float2 *orow = p.out + b * p.out_bstride + t * M + k1;
      const uint32_t lane_base = (uint32_t)(32 * warp) << 16;
      for (int col = 0; col < 64; col += 16) {
        uint32_t rr[16], ri[16];
        tc::tmem_ld16(tmem + lane_base + (uint32_t)col, rr);
        tc::tmem_ld16(tmem + lane_base + (uint32_t)(64 + col), ri);
        tc::tmem_ld_wait();
        if (t < p.T) {
#pragma unroll
          for (int i = 0; i < 16; i++)
            orow[(int64_t)R * (col + i)] = make_float2(__uint_as_float(rr[i]), __uint_as_float(ri[i]));
        }
      }
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    if (!ok) break;
  }
  if (!ok && tid == 0) (void)tc::mbar_wait(&bar, phase);
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc::tc_fence_after();
    tc::tmem_dealloc(tmem, 128u);
  }
}

static int channelize_poly_tc_rad(const gbfir_buf &out, const gbfir_buf &in, const gbfir_buf &h, int64_t M,
                                  int precision, cudaStream_t s) {
  const int R = (int)(M / 64);
  TcChParams p{};
  p.x = reinterpret_cast<const float2 *>(in.ptr);
  p.x_bstride = out.batch > 1 ? in.batch_stride : 0;
  p.N = in.len;
  p.h = reinterpret_cast<const float *>(h.ptr);
  p.L = h.len;
  p.out = reinterpret_cast<float2 *>(out.ptr);
  p.out_bstride = out.batch_stride;
  p.M = (int32_t)M;
  p.P = (int32_t)((h.len + M - 1) / M);
  p.Ppad = (p.P + kTcChE - 1) / kTcChE * kTcChE;
  p.T = (in.len + M - 1) / M;
  const int TS = kTcChTT / R;
  p.tiles_per_row = (p.T + TS - 1) / TS;
  p.ntiles = p.tiles_per_row * out.batch;
  p.terms = precision == GBFIR_PREC_BF16X3 ? 3 : 1;
  p.fp16 = precision == GBFIR_PREC_FP16;
  p.tap_stride = p.Ppad + ((p.Ppad % 8) == 0 ? 4 : 0);
  p.W = (int32_t)((TS + p.Ppad) * M);
  const size_t bb = (size_t)2 * p.terms * 128 * 64 * 2;
  const size_t tapb = ((size_t)M * p.tap_stride * 4 + 127) / 128 * 128;
  const size_t winb = (size_t)p.W * 8;
  const size_t ab = (size_t)2 * p.terms * 128 * 64 * 2;
  const size_t smem = bb + tapb + std::max(winb, ab);
  if (smem > 220 * 1024)
    GBFIR_FAIL(GBFIR_ERR_NOT_SUPPORTED, "channelize_poly: tensor-core tile needs %zu B of shared memory (P=%d)", smem,
               p.P);
  const void *fn = R == 2 ? (const void *)tc_channelize_rad_kernel<2> : (const void *)tc_channelize_rad_kernel<4>;
  int rc = ensure_smem(fn, smem, "channelize_poly (tensor cores)");
  if (rc) return rc;
  int occ = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, kTcChThreads, smem);
  if (occ < 1) occ = 1;
  occ = std::min(occ, 4);  // 128 TMEM columns per CTA
  int64_t grid = (int64_t)num_sms() * occ;
  if (grid > p.ntiles) grid = p.ntiles;
  void *args[] = {&p};
  const cudaError_t e = cudaLaunchKernel(fn, dim3((unsigned)grid), dim3(kTcChThreads), args, smem, s);
  if (e != cudaSuccess) GBFIR_FAIL(GBFIR_ERR_CUDA, "channelize_poly (tensor cores): %s", cudaGetErrorString(e));
  count_launch();
  return GBFIR_SUCCESS;
}

int channelize_poly_tc(const gbfir_buf &out, const gbfir_buf &in, const gbfir_buf &h, int64_t M, int64_t D,
                       int precision, cudaStream_t s) {
  if (in.dtype != GBFIR_C64 || h.dtype != GBFIR_F32)
    GBFIR_FAIL(GBFIR_ERR_NOT_SUPPORTED, "channelize_poly: tensor-core forms take complex64 signals and float32 taps");
  if (D == M && (M == 128 || M == 256)) return channelize_poly_tc_rad(out, in, h, M, precision, s);
  if (D != M || (M != 16 && M != 32 && M != 64))
    GBFIR_FAIL(GBFIR_ERR_NOT_SUPPORTED, "channelize_poly: tensor-core forms cover D == M with M in {16, 32, 64, "
                                        "128, 256} (got M=%lld, D=%lld)", (long long)M, (long long)D);
  TcChParams p{};
  p.x = reinterpret_cast<const float2 *>(in.ptr);
  p.x_bstride = out.batch > 1 ? in.batch_stride : 0;
  p.N = in.len;
  p.h = reinterpret_cast<const float *>(h.ptr);
  p.L = h.len;
  p.out = reinterpret_cast<float2 *>(out.ptr);
  p.out_bstride = out.batch_stride;
  p.M = (int32_t)M;
  p.P = (int32_t)((h.len + M - 1) / M);
  p.Ppad = (p.P + kTcChE - 1) / kTcChE * kTcChE;
  p.T = (in.len + D - 1) / D;
  p.tiles_per_row = (p.T + kTcChTT - 1) / kTcChTT;
  p.ntiles = p.tiles_per_row * out.batch;
  p.terms = precision == GBFIR_PREC_BF16X3 ? 3 : 1;
  p.fp16 = precision == GBFIR_PREC_FP16;
  p.tap_stride = p.Ppad + ((p.Ppad % 8) == 0 ? 4 : 0);
  p.W = (int32_t)((kTcChTT + p.Ppad) * M);
  const size_t twb = ((size_t)2 * p.terms * M * M * 2 + 127) / 128 * 128;
  const size_t tapb = ((size_t)M * p.tap_stride * 4 + 127) / 128 * 128;
  const size_t winb = (size_t)p.W * 8;
  const size_t ab = (size_t)2 * p.terms * kTcChTT * M * 2;
  const size_t smem = twb + tapb + std::max(winb, ab);
  if (smem > 220 * 1024)
    GBFIR_FAIL(GBFIR_ERR_NOT_SUPPORTED, "channelize_poly: tensor-core tile needs %zu B of shared memory (P=%d)", smem,
               p.P);
  int rc = ensure_smem((const void *)tc_channelize_kernel, smem, "channelize_poly (tensor cores)");
  if (rc) return rc;
  int occ = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, tc_channelize_kernel, kTcChThreads, smem);
  if (occ < 1) occ = 1;
  occ = std::min(occ, 512 / std::max(32, 2 * (int)M));
  int64_t grid = (int64_t)num_sms() * occ;
  if (grid > p.ntiles) grid = p.ntiles;
  tc_channelize_kernel<<<(unsigned)grid, kTcChThreads, smem, s>>>(p);
  return check_launch("channelize_poly (tensor cores)");
}

}  // namespace gbfir
