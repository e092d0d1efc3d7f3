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

extern __device__ int32_t g_tc_status;

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
      if (tid == 0) atomicExch(&g_tc_status, 1);
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

int channelize_poly_tc(const gbfir_buf &out, const gbfir_buf &in, const gbfir_buf &h, int64_t M, int64_t D,
                       int precision, cudaStream_t s) {
  if (in.dtype != GBFIR_C64 || h.dtype != GBFIR_F32)
    GBFIR_FAIL(GBFIR_ERR_NOT_SUPPORTED, "channelize_poly: tensor-core forms take complex64 signals and float32 taps");
  if (D != M || (M != 16 && M != 32 && M != 64))
    GBFIR_FAIL(GBFIR_ERR_NOT_SUPPORTED, "channelize_poly: tensor-core forms cover D == M with M in {16, 32, 64} "
                                        "(got M=%lld, D=%lld)", (long long)M, (long long)D);
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
