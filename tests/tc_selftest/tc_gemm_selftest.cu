// tc_gemm_selftest.cu — test-only self-test GEMM of the library's tcgen05 building blocks
// (matx_gb300/csrc/tc.cuh).  Built by tests/tc_selftest/build.py into a library of its own;
// nothing in the product links or loads it.
//
//   C[M][N] = A[M][K] * B[N][K]^T   (FP32 in and out)
// with the operands rounded to bf16 (terms = 1) or split into three bf16 terms
// (terms = 3; the six products of order <= 2, smallest first, accumulated in FP32 TMEM).
// One CTA of 128 threads per 128-row block: pack operands into the K-major core-matrix
// layout, one thread issues the MMAs and a commit to an mbarrier, all four warps wait
// (bounded) and read their 32 TMEM lanes back.  A timed-out wait sets *status = 1.
#include <cuda_runtime.h>
#include <stdint.h>

#include "tc.cuh"

namespace gbfir {

__global__ void __launch_bounds__(128) tc_gemm_selftest_kernel(const float *A, const float *B, float *C, int M,
                                                               int N, int K, int terms, int *status) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ uint64_t bar;
  __shared__ uint32_t tmem_slot;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * 128;
  const uint32_t abytes = 128u * K * 2u, bbytes = (uint32_t)N * K * 2u;
  unsigned char *abuf[3], *bbuf[3];
  for (int t = 0; t < 3; t++) {
    abuf[t] = smem + t * abytes;
    bbuf[t] = smem + 3 * abytes + t * bbytes;
  }
  uint32_t ncols = 32;
  while (ncols < (uint32_t)N) ncols <<= 1;

  if (warp == 0) tc::tmem_alloc(&tmem_slot, ncols);
  if (tid == 0) {
    tc::mbar_init(&bar, 1);
    tc::mbar_fence_init();
  }
  for (int e = tid; e < 128 * K; e += 128) {
    const int r = e / K, k = e - r * K;
    const float a = A[(size_t)(m0 + r) * K + k];
    __nv_bfloat16 t0, t1, t2;
    tc::split3_bf16(a, t0, t1, t2);
    const uint32_t off = tc::kmajor_offset(r, k, K);
    *reinterpret_cast<__nv_bfloat16 *>(abuf[0] + off) = t0;
    if (terms == 3) {
      *reinterpret_cast<__nv_bfloat16 *>(abuf[1] + off) = t1;
      *reinterpret_cast<__nv_bfloat16 *>(abuf[2] + off) = t2;
    }
  }
  for (int e = tid; e < N * K; e += 128) {
    const int r = e / K, k = e - r * K;
    const float b = B[(size_t)r * K + k];
    __nv_bfloat16 t0, t1, t2;
    tc::split3_bf16(b, t0, t1, t2);
    const uint32_t off = tc::kmajor_offset(r, k, K);
    *reinterpret_cast<__nv_bfloat16 *>(bbuf[0] + off) = t0;
    if (terms == 3) {
      *reinterpret_cast<__nv_bfloat16 *>(bbuf[1] + off) = t1;
      *reinterpret_cast<__nv_bfloat16 *>(bbuf[2] + off) = t2;
    }
  }
  tc::fence_async_smem();
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = tmem_slot;

  if (tid == 0) {
    const uint32_t kstride = 128, rstride = (uint32_t)(K / 8) * 128;  // layout of kmajor_offset
    const uint32_t lbo = kstride, sbo = rstride;
    const uint32_t idesc = tc::idesc_f16(128, (uint32_t)N, 1);
    const int pa3[6] = {2, 1, 0, 1, 0, 0}, pb3[6] = {0, 1, 2, 0, 1, 0};
    const int npairs = terms == 3 ? 6 : 1;
    uint32_t acc = 0;
    for (int pidx = 0; pidx < npairs; pidx++) {
      const int pa = terms == 3 ? pa3[pidx] : 0, pb = terms == 3 ? pb3[pidx] : 0;
      for (int ks = 0; ks < K / 16; ks++) {
        const uint64_t ad = tc::smem_desc(tc::smem_u32(abuf[pa]) + ks * 256, lbo, sbo);
        const uint64_t bd = tc::smem_desc(tc::smem_u32(bbuf[pb]) + ks * 256, lbo, sbo);
        tc::mma_f16(tmem, ad, bd, idesc, acc);
        acc = 1;
      }
    }
    tc::mma_commit(&bar);
  }
  const bool ok = tc::mbar_wait(&bar, 0);
  tc::tc_fence_after();
  if (ok) {
    for (int col = 0; col < N; col += 16) {
      uint32_t r[16];
      tc::tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)col, r);
      tc::tmem_ld_wait();
      float *crow = C + (size_t)(m0 + 32 * warp + lane) * N + col;
#pragma unroll
      for (int i = 0; i < 16; i++) crow[i] = __uint_as_float(r[i]);
    }
  } else if (lane == 0) {
    atomicExch(status, 1);
    (void)tc::mbar_wait(&bar, 0);  // give in-flight MMAs a second bounded chance before freeing TMEM
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc::tc_fence_after();
    tc::tmem_dealloc(tmem, ncols);
  }
}

}  // namespace gbfir

using namespace gbfir;

// 0 on success; 1 = null pointer, 2 = unsupported size, 3 = CUDA error.
extern "C" __attribute__((visibility("default"))) int tc_gemm_selftest(const float *A, const float *B, float *C,
                                                                        int32_t M, int32_t N, int32_t K,
                                                                        int32_t terms, int32_t *status,
                                                                        void *stream) {
  if (!A || !B || !C || !status) return 1;
  if (M <= 0 || M % 128 || N < 16 || N > 256 || N % 16 || K < 16 || K > 64 || K % 16 || (terms != 1 && terms != 3))
    return 2;
  const size_t smem = 3 * (128u * K * 2u) + 3 * ((size_t)N * K * 2u);
  if (cudaFuncSetAttribute(tc_gemm_selftest_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess)
    return 3;
  tc_gemm_selftest_kernel<<<M / 128, 128, smem, reinterpret_cast<cudaStream_t>(stream)>>>(A, B, C, M, N, K, terms,
                                                                                           status);
  return cudaGetLastError() == cudaSuccess ? 0 : 3;
}
