// tc.cuh — tcgen05 (5th-generation tensor core) building blocks for sm_103a, in inline PTX.
//
// Conventions used by every tensor-core kernel of this library:
//  * One CTA, cta_group::1, MMA shape M = 128 (TMEM lane m = row m), N = 16..256, K = 16
//    (kind::f16, bf16 or fp16 operands, FP32 accumulate).
//  * Operands live in shared memory in the no-swizzle K-major canonical layout: 8-row x
//    16-byte core matrices (8 rows x 8 bf16 along K, 128 contiguous bytes); the core
//    matrix (row group i, K group j) sits at  base + i * SBO + j * LBO.
//  * One elected thread issues the MMAs and a tcgen05.commit that arrives on an mbarrier;
//    every wait on an mbarrier is bounded: after kSpinLimit failed polls the waiter sets
//    an error flag and the kernel skips the work that depended on it, so a fault in the
//    pipeline becomes a status code, never a hung GPU.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>

namespace gbfir {
namespace tc {

constexpr uint32_t kSpinLimit = 1u << 22;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// ---- mbarrier ---------------------------------------------------------------------
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return done != 0;
}
// Bounded wait; returns false (and leaves the barrier untouched) if it gave up.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
  for (uint32_t i = 0; i < kSpinLimit; i++) {
    if (mbar_try_wait(bar, parity)) return true;
  }
  return false;
}

// Bounded wait whose polls let the thread sleep until the phase completes or about
// kSleepHintNs have passed, so waiting warps leave the issue slots to the warps that work;
// gives up (returns false) after kSleepLimit polls, well under a second.
constexpr uint32_t kSleepHintNs = 200;
constexpr uint32_t kSleepLimit = 1u << 21;
__device__ __forceinline__ bool mbar_wait_sleep(uint64_t *bar, uint32_t parity) {
  for (uint32_t i = 0; i < kSleepLimit; i++) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity), "r"(kSleepHintNs)
        : "memory");
    if (done) return true;
  }
  return false;
}

// Arrive on `bar` and add `bytes` to the transaction count it waits for.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(
                   smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive_plain(uint64_t *bar) {
  asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(smem_u32(bar))
               : "memory");
}
// TMA bulk copy global -> shared, completing `bytes` of transactions on `bar`.  Both
// addresses must be 16-byte aligned and bytes a multiple of 16.
__device__ __forceinline__ void bulk_copy_g2s(void *dst_smem, const void *src_gmem, uint32_t bytes, uint64_t *bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst_smem)),
               "l"(src_gmem), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

// Bulk prefetch of `bytes` of global memory into L2 (16-byte aligned address, bytes a
// multiple of 16); nothing waits for it.
__device__ __forceinline__ void bulk_prefetch_l2(const void *src_gmem, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src_gmem), "r"(bytes) : "memory");
}

// TMA tensor store shared -> global of one 3-D box (coordinates in elements, innermost
// first; the innermost times the element size a multiple of 16 bytes, none negative),
// tracked by the issuing thread's bulk groups.
__device__ __forceinline__ void tma_store_3d(const void *tmap, const void *src_smem, int x, int y, int z) {
  asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.bulk_group [%0, {%2, %3, %4}], [%1];" ::"l"(
                   reinterpret_cast<uint64_t>(tmap)),
               "r"(smem_u32(src_smem)), "r"(x), "r"(y), "r"(z)
               : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// at most N of this thread's bulk groups still reading shared memory
template <int N>
__device__ __forceinline__ void bulk_wait_read() {
  asm volatile("cp.async.bulk.wait_group.read %0;" ::"n"(N) : "memory");
}
// all of this thread's bulk groups complete
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// ---- proxy / tcgen05 ordering fences ---------------------------------------------------
// generic-proxy shared-memory writes -> visible to the tensor core (async proxy)
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// ---- tensor memory ---------------------------------------------------------------------
// Executed by one full warp.  ncols is a power of two in [32, 512].
__device__ __forceinline__ void tmem_alloc(uint32_t *dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst_smem)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// ---- descriptors ---------------------------------------------------------------------
// Shared-memory matrix descriptor, no swizzle: start, leading (K-direction core matrix)
// and stride (row-group direction) byte offsets, all multiples of 16 bytes.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version for this architecture
  return d;                // base offset 0, relative LBO, layout type 0 (no swizzle)
}

// Instruction descriptor for kind::f16 with FP32 accumulate, both operands K-major.
// ab_bf16: 1 = bf16 operands, 0 = fp16.
__host__ __device__ constexpr uint32_t idesc_f16(uint32_t M, uint32_t N, uint32_t ab_bf16) {
  return (1u << 4)                  // D format: F32
         | (ab_bf16 << 7)           // A format
         | (ab_bf16 << 10)          // B format
         | ((N >> 3) << 17)         // N / 8
         | ((M >> 4) << 24);        // M / 16
}

// D[tmem] (+)= A[smem] * B[smem]^T ; issued by one thread.
__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                        uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// Arrive on `bar` once every MMA this thread issued so far has completed.
__device__ __forceinline__ void mma_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// Warp w (0..3) reads its 32 TMEM lanes, 16 consecutive FP32 columns starting at `col`.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
}
// Warp w reads 16 of its TMEM lanes (from the lane in taddr) x 8 FP32 columns: lane L gets
// (lane L/4, columns 2*(L%4) and 2*(L%4)+1) in r[0], r[1] and the same columns of lane
// L/4 + 8 in r[2], r[3].
__device__ __forceinline__ void tmem_ld_16x256b(uint32_t taddr, uint32_t (&r)[4]) {
  asm volatile("tcgen05.ld.sync.aligned.16x256b.x1.b32 {%0, %1, %2, %3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(taddr)
               : "memory");
}
// The same for 32 columns: r[4g .. 4g+3] hold the 8-column group g (columns 8g .. 8g+7)
// laid out as above.
__device__ __forceinline__ void tmem_ld_16x256b_x4(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.16x256b.x4.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
}
__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// ---- operand packing ----------------------------------------------------------------------
// Byte offset of element (row, k) in the K-major no-swizzle layout with K-adjacent core
// matrices contiguous: core (row/8, k/8) at ((row/8) * (K/8) + k/8) * 128.
__device__ __forceinline__ uint32_t kmajor_offset(uint32_t row, uint32_t k, uint32_t K) {
  return (((row >> 3) * (K >> 3) + (k >> 3)) << 7) + ((row & 7) << 4) + ((k & 7) << 1);
}

// Split an FP32 value into three bf16 terms a0 + a1 + a2 (24 significant bits).
__device__ __forceinline__ void split3_bf16(float a, __nv_bfloat16 &a0, __nv_bfloat16 &a1, __nv_bfloat16 &a2) {
  a0 = __float2bfloat16_rn(a);
  const float r1 = a - __bfloat162float(a0);
  a1 = __float2bfloat16_rn(r1);
  const float r2 = r1 - __bfloat162float(a1);
  a2 = __float2bfloat16_rn(r2);
}

// The same split for two values at once: each bf16x2 conversion rounds both lanes to
// nearest, and the residuals are exact, so t_i.x / t_i.y equal split3_bf16 of a.x / a.y.
__device__ __forceinline__ void split3_bf16x2(float2 a, __nv_bfloat162 &t0, __nv_bfloat162 &t1,
                                              __nv_bfloat162 &t2) {
  t0 = __float22bfloat162_rn(a);
  const float2 b0 = __bfloat1622float2(t0);
  const float2 r1 = __fadd2_rn(a, make_float2(-b0.x, -b0.y));
  t1 = __float22bfloat162_rn(r1);
  const float2 b1 = __bfloat1622float2(t1);
  const float2 r2 = __fadd2_rn(r1, make_float2(-b1.x, -b1.y));
  t2 = __float22bfloat162_rn(r2);
}

}  // namespace tc
}  // namespace gbfir
