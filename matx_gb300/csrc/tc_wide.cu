// tc_wide.cu — resample_poly and conv1d/corr on the tcgen05 tensor cores with 64-sample
// Toeplitz rows: the taps are the MMA's A operand in tensor memory and the signal is an
// aliased Hankel B operand in 128-byte-swizzled shared memory.  No MatX counterpart.
//
// Math (gcd-reduced rates, down divides 64).  Row q of a signal holds Nt = 64*up/down
// consecutive outputs and needs the inputs x[64q + k0 + k], k < Kp, so with the linear
// bf16/fp16 array xs[u] = x[64 q0 + k0 + u] of a tile of NR rows starting at row q0
//   D[j][n] = sum_k W[j][k] * xs[64n + k],   W[j][k] = scale * he[c + j*down - (k0 + k)*up],
//   out[(q0 + n)*Nt + j] = D[j][n]            (j < Nt, lanes j >= Nt idle).
// A 128-byte swizzled K-major operand row is 64 bf16, so B[n][k] = xs[64n + k] is exactly
// the swizzled layout of xs with rows 128 bytes apart (SBO = 1024 per 8-row group) and
// K-step s starting 32*s bytes in; no Hankel matrix is materialised.  W (M = 128 lanes =
// output phases, K = Kp) is built once per CTA into TMEM with tcgen05.st, bf16 pairs
// packed low-k-first.  bf16x3 splits both operands into three bf16 terms and accumulates
// the six products of order <= 2 into one FP32 accumulator.
//
// Pipeline (persistent, warp-specialised CTA, 384 threads).  A stage is one part (real or
// imaginary) of one tile.  Warps 1-7 bring each tile's input window into a raw slot (one
// TMA bulk copy; element loads with zeros outside the signal at the row ends), staged up
// to two tiles ahead, and convert one part into the swizzled term arrays of a 2-slot
// operand ring; warp 0 lane 0 issues the MMAs into one of two TMEM accumulator sets (a set
// holds every part of one tile); warps 8-11 (one per TMEM lane quarter, lane = output
// phase) store the tile's outputs as whole (complex) values.  Every wait on an mbarrier is bounded; a wait that gives up sets the kernel's
// status word.
#include <cstdio>
#include <cstdlib>

#include "common.cuh"
#include "tc.cuh"
#include "tc_wide.h"

namespace gbfir {

// Bounded-wait status of this kernel (1 = a wait gave up); read and cleared by
// gbfir_tc_status() through tc_wide_status_take().
__device__ int32_t g_tcw_status;

int tc_wide_status_take() {
  int32_t v = 0, zero = 0;
  if (cudaMemcpyFromSymbol(&v, g_tcw_status, sizeof(v)) != cudaSuccess) return -1;
  cudaMemcpyToSymbol(g_tcw_status, &zero, sizeof(zero));
  return v;
}

constexpr int kTwThreads = 384;
constexpr int kTwProd0 = 1, kTwProdWarps = 7, kTwEpi0 = 8;
constexpr int kTwNProd = kTwProdWarps * 32;

__device__ __forceinline__ void tw_named_sync(int id, int nthreads) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}
__device__ __forceinline__ void tw_tmem_st16(uint32_t taddr, const uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15, %16};" ::"r"(taddr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]), "r"(r[8]), "r"(r[9]),
      "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15])
      : "memory");
}
__device__ __forceinline__ void tw_tmem_st_wait() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }
// D[tmem] (+)= A[tmem] * B[smem]^T, issued by one thread.
__device__ __forceinline__ void tw_mma_ts(uint32_t d, uint32_t a_tmem, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}" ::"r"(d),
      "r"(a_tmem), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
// 128-byte-swizzled K-major descriptor: 8-row groups 1024 bytes apart, base offset 0 (the
// swizzle follows the absolute shared-memory address, so a start inside a row works).
__device__ __forceinline__ uint64_t tw_desc_sw128(uint32_t saddr) {
  return tc::smem_desc(saddr, 16u, 1024u) | ((uint64_t)2 << 61);
}

__device__ __forceinline__ uint32_t tw_pack_fp16(float a, float b) {
  return (uint32_t)__half_as_ushort(__float2half_rn(a)) | ((uint32_t)__half_as_ushort(__float2half_rn(b)) << 16);
}

template <bool XC>
__global__ void __launch_bounds__(kTwThreads, 1) tc_wide_kernel(const TwParams p) {
  using XT = typename val_of<float, XC>::type;
  constexpr int NPARTS = XC ? 2 : 1;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ uint64_t op_full[2], op_empty[2], tm_full[2], tm_empty[2], raw_full[2];
  __shared__ uint32_t tmem_slot;
  __shared__ int s_fail, s_pok, s_eok;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  // shared layout (1024-aligned): operand ring [2 slots][terms] x xarr, then the raw ring
  unsigned char *base = smem_raw + ((1024u - (tc::smem_u32(smem_raw) & 1023u)) & 1023u);
  auto xarrp = [&](int slot, int t) { return base + ((size_t)slot * p.terms + t) * (size_t)p.xarr; };
  XT *raw0 = reinterpret_cast<XT *>(base + (size_t)2 * p.terms * p.xarr);
  auto rawp = [&](int slot) { return raw0 + (size_t)slot * p.raw_elems; };
  const XT *xp = reinterpret_cast<const XT *>(p.x);

  if (warp == 0) tc::tmem_alloc(&tmem_slot, (uint32_t)p.tmem_cols);
  if (tid == 0) {
    for (int i = 0; i < 2; i++) {
      tc::mbar_init(&op_full[i], 1);
      tc::mbar_init(&op_empty[i], 1);
      tc::mbar_init(&tm_full[i], 1);
      tc::mbar_init(&tm_empty[i], 1);
      tc::mbar_init(&raw_full[i], 1);
    }
    s_fail = 0;
    tc::mbar_fence_init();
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = tmem_slot;

  // ---- the taps, scaled and split into the operand terms once (hterm[t][e] = term t of
  // scale * h[e], 16-bit), staged in the raw ring (not in use yet) ----
  const int64_t Lh = p.Lo - p.even;
  const bool h_staged = (size_t)Lh * 2 * p.terms <= (size_t)p.nraw * p.raw_elems * sizeof(XT);
  uint16_t *hterm = reinterpret_cast<uint16_t *>(raw0);
  auto split_terms = [&](float v, uint16_t (&o)[3]) {
    if (p.fp16) {
      o[0] = __half_as_ushort(__float2half_rn(v));
      o[1] = o[2] = 0;
    } else {
      __nv_bfloat16 t0, t1, t2;
      tc::split3_bf16(v, t0, t1, t2);
      o[0] = __bfloat16_as_ushort(t0);
      o[1] = __bfloat16_as_ushort(t1);
      o[2] = __bfloat16_as_ushort(t2);
    }
  };
  if (h_staged) {
    for (int64_t e = tid; e < Lh; e += kTwThreads) {
      uint16_t o[3];
      split_terms(p.h[e] * (float)p.scale, o);
      for (int t = 0; t < p.terms; t++) hterm[t * Lh + e] = o[t];
    }
  }
  __syncthreads();
  // term t of W at tap position tp (he read reversed when rev, 0 outside the filter)
  auto w_term = [&](int t, int64_t tp) -> uint32_t {
    if (tp < 0 || tp >= p.Lo) return 0u;
    const int64_t te = p.rev ? p.Lo - 1 - tp : tp;
    if (p.even && te == 0) return 0u;
    const int64_t e = te - p.even;
    if (h_staged) return hterm[t * Lh + e];
    uint16_t o[3];
    split_terms(p.h[e] * (float)p.scale, o);
    return o[t];
  };
  // ---- W into TMEM: lane j = output phase, columns = K packed two per column ----
  if (warp >= kTwEpi0) {
    const int quarter = warp - kTwEpi0;
    const int j = 32 * quarter + lane;
    const uint32_t lane_base = (uint32_t)(32 * quarter) << 16;
    const int half = p.Kp / 2;
    for (int t = 0; t < p.terms; t++) {
      for (int kc = 0; kc < half; kc += 16) {
        uint32_t r[16];
#pragma unroll
        for (int i = 0; i < 16; i++) {
          const int k = 2 * (kc + i);
          r[i] = 0u;
          if (j < p.Nt) {
            const int64_t tb = p.c + (int64_t)j * p.down - (p.k0 + k) * p.up;
            r[i] = w_term(t, tb) | (w_term(t, tb - p.up) << 16);
          }
        }
        tw_tmem_st16(tmem + lane_base + (uint32_t)(p.wcol0 + t * half + kc), r);
      }
    }
    tw_tmem_st_wait();
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();

  // this CTA's tiles: blockIdx.x, blockIdx.x + gridDim.x, ...; a stage = (tile, part)
  const int64_t my_tiles = p.ntiles > blockIdx.x ? (p.ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
  const int64_t nstages = my_tiles * NPARTS;
  auto tile_of = [&](int64_t i, int64_t &b, int64_t &q0) {
    const int64_t t = blockIdx.x + i * (int64_t)gridDim.x;
    b = t / p.tiles_per_row;
    q0 = (t - b * p.tiles_per_row) * (int64_t)p.NR;
  };
  if (warp >= kTwProd0 && warp < kTwProd0 + kTwProdWarps) {
    // ================= producers =================
    // The tile's input window comes into one of nraw raw slots by one TMA bulk copy
    // (element loads with zeros outside the signal for the edge tiles), staged nraw tiles
    // ahead.  Each stage converts one part: lane v takes the element pair (2v, 2v+1) with
    // one 16-byte shared load and writes 4 bytes per term, so a warp reads 512 contiguous
    // bytes and writes one 128-byte swizzled row of each term array (conflict-free).
    const int ptid = tid - kTwProd0 * 32;
    constexpr int ES = (int)sizeof(XT), G = 16 / ES;
    auto raw_origin = [&](int64_t i, int64_t &w0, const XT *&row) -> int {
      int64_t b, q0;
      tile_of(i, b, q0);
      row = xp + b * p.x_bstride;
      const int64_t ws = 64 * q0 + p.k0;
      const int a = (int)((reinterpret_cast<uintptr_t>(row + ws) & 15) / ES);
      w0 = ws - a;
      return a;
    };
    auto fetch = [&](int64_t i, int rslot) {
      int64_t w0;
      const XT *row;
      const int a = raw_origin(i, w0, row);
      const int64_t wl = (p.win + a + G - 1) / G * G;
      XT *dst = rawp(rslot);
      const bool aligned = ((reinterpret_cast<uintptr_t>(row + w0) | (uintptr_t)tc::smem_u32(dst)) & 15) == 0;
      if (aligned && w0 >= 0 && w0 + wl <= p.N) {
        if (ptid == 0) {
          const uint32_t bytes = (uint32_t)(wl * ES);
          tc::fence_async_smem();
          tc::mbar_arrive_expect_tx(&raw_full[rslot], bytes);
          tc::bulk_copy_g2s(dst, row + w0, bytes, &raw_full[rslot]);
        }
      } else {
        for (int64_t e = ptid; e < wl; e += kTwNProd) {
          const int64_t gi = w0 + e;
          dst[e] = (gi >= 0 && gi < p.N) ? row[gi] : zero_val<XT>();
        }
        tw_named_sync(1, kTwNProd);
        if (ptid == 0) tc::mbar_arrive_plain(&raw_full[rslot]);
      }
    };
    if (my_tiles > 0) fetch(0, 0);
    if (p.nraw == 2 && my_tiles > 1) fetch(1, 1);
    const int npairs = p.win / 2;
    for (int64_t s = 0; s < nstages; ++s) {
      const int64_t i = s / NPARTS;
      const int part = (int)(s - i * NPARTS);
      const int rslot = p.nraw == 2 ? (int)(i & 1) : 0;
      const int slot = (int)(s & 1);
      if (ptid == 0) {
        bool ok = true;
        if (part == 0) ok = tc::mbar_wait(&raw_full[rslot], (uint32_t)((i / p.nraw) & 1));
        if (ok && s >= 2) ok = tc::mbar_wait(&op_empty[slot], (uint32_t)(((s - 2) >> 1) & 1));
        s_pok = ok ? 1 : 0;
      }
      tw_named_sync(1, kTwNProd);
      if (!s_pok) {
        s_fail = 1;
        break;
      }
      int64_t w0;
      const XT *rowp;
      const int a = raw_origin(i, w0, rowp);
      const XT *src = rawp(rslot) + a;
      unsigned char *d0 = xarrp(slot, 0), *d1 = xarrp(slot, p.terms == 3 ? 1 : 0),
                    *d2 = xarrp(slot, p.terms == 3 ? 2 : 0);
#pragma unroll 4
      for (int v = ptid; v < npairs; v += kTwNProd) {
        XT x0, x1;
        if constexpr (XC) {
          if (a == 0) {
            const float4 w4 = *reinterpret_cast<const float4 *>(src + 2 * v);
            x0 = make_float2(w4.x, w4.y);
            x1 = make_float2(w4.z, w4.w);
          } else {
            x0 = src[2 * v];
            x1 = src[2 * v + 1];
          }
        } else {
          x0 = src[2 * v];
          x1 = src[2 * v + 1];
        }
        const float2 f = part == 0 ? make_float2(re_of(x0), re_of(x1)) : make_float2(im_of(x0), im_of(x1));
        const uint32_t o = 4u * (uint32_t)v;               // byte offset of element 2v
        const uint32_t phys = o ^ (((o >> 7) & 7u) << 4);  // 128-byte swizzle
        if (p.fp16) {
          *reinterpret_cast<uint32_t *>(d0 + phys) = tw_pack_fp16(f.x, f.y);
        } else {
          __nv_bfloat162 t0, t1, t2;
          tc::split3_bf16x2(f, t0, t1, t2);
          *reinterpret_cast<__nv_bfloat162 *>(d0 + phys) = t0;
          if (p.terms == 3) {
            *reinterpret_cast<__nv_bfloat162 *>(d1 + phys) = t1;
            *reinterpret_cast<__nv_bfloat162 *>(d2 + phys) = t2;
          }
        }
      }
      tc::fence_async_smem();
      tw_named_sync(1, kTwNProd);
      if (ptid == 0) tc::mbar_arrive_plain(&op_full[slot]);
      // the last part of the tile releases its raw slot: stage the tile nraw ahead into it
      if (part == NPARTS - 1 && i + p.nraw < my_tiles) fetch(i + p.nraw, rslot);
    }
  } else if (warp == 0) {
    // ================= MMA issuer =================
    // every TMEM column the MMAs touch lies inside the allocation (checked once)
    const bool geom_ok = p.NR % 16 == 0 && p.Kp % 32 == 0 && (p.nsets == 1 || p.nsets == 2) &&
                         p.wcol0 >= p.nsets * NPARTS * p.NR &&
                         p.wcol0 + p.terms * (p.Kp / 2) <= p.tmem_cols && (p.terms == 1 || p.terms == 3);
    if (lane == 0 && !geom_ok) s_fail = 1;
    if (lane == 0 && geom_ok) {
      const uint32_t idesc = tc::idesc_f16(128, (uint32_t)p.NR, p.fp16 ? 0u : 1u);
      const int nks = p.Kp / 16, half = p.Kp / 2;
      // products of order <= 2 (W term, x term), smallest first: (1,1) (2,0) (0,2) (1,0)
      // (0,1) (0,0), packed one nibble per product
      constexpr uint32_t kPw = 0x001021u, kPx = 0x010201u;
      const int npairs = p.terms == 3 ? 6 : 1;
      for (int64_t s = 0; s < nstages; ++s) {
        const int64_t i = s / NPARTS;
        const int part = (int)(s - i * NPARTS);
        const int slot = (int)(s & 1), tset = (int)(i % p.nsets);
        if (!tc::mbar_wait(&op_full[slot], (uint32_t)((s >> 1) & 1))) { s_fail = 1; break; }
        // accumulator set tset holds every part of tile i; it is free once the epilogue has
        // drained tile i - nsets
        if (part == 0 && i >= p.nsets &&
            !tc::mbar_wait(&tm_empty[tset], (uint32_t)(((i - p.nsets) / p.nsets) & 1))) {
          s_fail = 1;
          break;
        }
        tc::tc_fence_after();
        const uint32_t d = tmem + (uint32_t)((tset * NPARTS + part) * p.NR);
        for (int ks = 0; ks < nks; ks++) {
          for (int pr = 0; pr < npairs; pr++) {
            const int tw = p.terms == 3 ? (int)((kPw >> (4 * pr)) & 15u) : 0;
            const int tx = p.terms == 3 ? (int)((kPx >> (4 * pr)) & 15u) : 0;
            const uint32_t a = tmem + (uint32_t)(p.wcol0 + tw * half + 8 * ks);
            const uint64_t bd = tw_desc_sw128(tc::smem_u32(xarrp(slot, tx)) + 32u * ks);
            tw_mma_ts(d, a, bd, idesc, (ks > 0 || pr > 0) ? 1u : 0u);
          }
        }
        tc::mma_commit(&op_empty[slot]);
        if (part == NPARTS - 1) tc::mma_commit(&tm_full[tset]);
      }
    }
  } else {
    // ================= epilogue: lane j of quarter q = output phase 32q + j =================
    // one tile at a time, both parts together, so each output is one whole store and a
    // warp's 32 phases of one row are 32 consecutive outputs
    const int quarter = warp - kTwEpi0;
    const int j = 32 * quarter + lane;
    const uint32_t lane_base = (uint32_t)(32 * quarter) << 16;
    for (int64_t i = 0; i < my_tiles; ++i) {
      const int tset = (int)(i % p.nsets);
      if (quarter == 0 && lane == 0) s_eok = tc::mbar_wait(&tm_full[tset], (uint32_t)((i / p.nsets) & 1)) ? 1 : 0;
      tw_named_sync(2, 128);
      if (!s_eok) {
        s_fail = 1;
        break;
      }
      tc::tc_fence_after();
      int64_t b, q0;
      tile_of(i, b, q0);
      XT *orow = reinterpret_cast<XT *>(p.out) + (size_t)b * p.out_bstride;
      // rows n < nv hold a valid output for this phase
      const int64_t left = p.out_len - q0 * p.Nt - j;
      const int nv = (j >= p.Nt || left <= 0) ? 0 : (int)std::min<int64_t>(p.NR, (left + p.Nt - 1) / p.Nt);
      XT *dst = orow + q0 * p.Nt + j;
      const uint32_t dre = tmem + lane_base + (uint32_t)(tset * NPARTS * p.NR);
      for (int c = 0; c < p.NR; c += 16) {
        uint32_t r0[16], r1[16];
        tc::tmem_ld16(dre + (uint32_t)c, r0);
        if constexpr (XC) tc::tmem_ld16(dre + (uint32_t)(p.NR + c), r1);
        tc::tmem_ld_wait();
#pragma unroll
        for (int e = 0; e < 16; e++) {
          if (c + e < nv) {
            if constexpr (XC) dst[(int64_t)(c + e) * p.Nt] = make_float2(__uint_as_float(r0[e]), __uint_as_float(r1[e]));
            else dst[(int64_t)(c + e) * p.Nt] = __uint_as_float(r0[e]);
          }
        }
      }
      tc::tc_fence_before();
      tw_named_sync(2, 128);
      if (quarter == 0 && lane == 0) tc::mbar_arrive_plain(&tm_empty[tset]);
    }
  }
  __syncthreads();
  if (s_fail && tid == 0) {
    atomicExch(&g_tcw_status, 1);
    // give work still in flight a bounded chance to finish before the TMEM is freed
    (void)tc::mbar_wait(&tm_full[0], 0);
    (void)tc::mbar_wait(&tm_full[1], 0);
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc::tc_fence_after();
    tc::tmem_dealloc(tmem, (uint32_t)p.tmem_cols);
  }
}

// Plan of the 64-sample-row form.  Covers down | 64 with Nt = 64*up/down <= 128 and a
// tap band whose W fits TMEM next to two accumulator sets; returns ok = false otherwise.
TwPlan plan_tc_wide(int64_t up, int64_t down, int64_t Lo, int64_t c, int even, int rev, double scale, int64_t N_in,
                    int64_t out_len, int64_t batch, int xc, int precision) {
  TwPlan pl{};
  TwParams &p = pl.p;
  if (64 % down != 0 || 64 * up / down > 128) {
    snprintf(pl.why, sizeof(pl.why), "64-sample rows need down | 64 and 64*up/down <= 128");
    return pl;
  }
  p.Lo = Lo;
  p.c = c;
  p.even = even;
  p.rev = rev;
  p.scale = scale;
  p.up = up;
  p.down = down;
  p.N = N_in;
  p.out_len = out_len;
  p.Nt = (int32_t)(64 * up / down);
  p.fp16 = precision == GBFIR_PREC_FP16;
  p.terms = precision == GBFIR_PREC_BF16X3 ? 3 : 1;
  const int64_t kmin = ceil_div(c - Lo + 1, up);
  const int64_t kmax = floor_div(c + (int64_t)(p.Nt - 1) * down, up);
  p.k0 = kmin;
  p.Kp = (int32_t)((kmax - kmin + 1 + 31) / 32 * 32);  // W is written to TMEM 16 columns (32 k) at a time
  const int ES = xc ? 8 : 4, G = 16 / ES;
  const size_t kMaxSmem = 225 * 1024;
  const int nparts = xc ? 2 : 1;
  // Candidates: two TMEM accumulator sets (the epilogue of one tile overlaps the MMAs of the
  // next) or one set with more rows per MMA; a single set counts 0.8 of its rows, the
  // measured cost of the serialised epilogue.  Two raw slots before one.
  // GBFIR_TC_WIDE_SHAPE="sets,raw,rows" restricts the candidates to one shape (for tuning)
  int want[3] = {0, 0, 0};
  if (const char* env = getenv("GBFIR_TC_WIDE_SHAPE"))
    if (sscanf(env, "%d,%d,%d", &want[0], &want[1], &want[2]) != 3) want[0] = want[1] = want[2] = 0;
  int best_score = 0;
  TwParams best{};
  size_t best_smem = 0;
  for (int nsets : {2, 1}) {
    for (int nraw : {2, 1}) {
      for (int NR : {128, 112, 96, 80, 64}) {
        const int64_t win = 64LL * (NR - 1) + p.Kp;
        const size_t xarr = ((size_t)win * 2 + 1023) / 1024 * 1024;
        const int64_t raw_elems = (win + 3 * G - 1) / G * G;
        const size_t smem = 1024 + (size_t)2 * p.terms * xarr + (size_t)nraw * raw_elems * ES;
        const int wcols = p.terms * p.Kp / 2;
        if (smem > kMaxSmem || nsets * nparts * NR + wcols > 512) continue;
        if (want[0] && (nsets != want[0] || nraw != want[1] || NR != want[2])) continue;
        const int score = (nsets == 2 ? 10 * NR : 8 * NR) + (nraw == 2 ? 1 : 0);
        if (score <= best_score) continue;
        TwParams q = p;
        q.NR = NR;
        q.nraw = nraw;
        q.nsets = nsets;
        q.win = (int32_t)win;
        q.xarr = (int32_t)xarr;
        q.raw_elems = (int32_t)raw_elems;
        q.wcol0 = nsets * nparts * NR;
        uint32_t cols = 32;
        while (cols < (uint32_t)(q.wcol0 + wcols)) cols <<= 1;
        q.tmem_cols = (int32_t)cols;
        q.rows = (out_len + q.Nt - 1) / q.Nt;
        q.tiles_per_row = (q.rows + NR - 1) / NR;
        q.ntiles = q.tiles_per_row * batch;
        best = q;
        best_smem = smem;
        best_score = score;
      }
    }
  }
  if (best_score > 0) {
    p = best;
    pl.smem = best_smem;
    pl.ok = true;
    return pl;
  }
  snprintf(pl.why, sizeof(pl.why), "a band of %d taps does not fit next to the accumulators", p.Kp);
  return pl;
}

int launch_tc_wide(TwPlan &pl, const gbfir_buf &out, const gbfir_buf &in, const gbfir_buf &h, bool xc,
                   const char *what, cudaStream_t s) {
  TwParams &p = pl.p;
  p.x = in.ptr;
  p.x_bstride = (out.batch > 1 && in.batch > 1) ? in.batch_stride : 0;
  p.h = reinterpret_cast<const float *>(h.ptr);
  p.out = out.ptr;
  p.out_bstride = out.batch_stride;
  const void *fn = xc ? (const void *)tc_wide_kernel<true> : (const void *)tc_wide_kernel<false>;
  int rc = ensure_smem(fn, pl.smem, what);
  if (rc) return rc;
  int64_t grid = num_sms();  // one CTA per SM (TMEM and shared memory)
  if (grid > p.ntiles) grid = p.ntiles;
  if (grid < 1) return GBFIR_SUCCESS;
  void *args[] = {&p};
  cudaError_t e = cudaLaunchKernel(fn, dim3((unsigned)grid), dim3(kTwThreads), args, pl.smem, s);
  if (e != cudaSuccess) GBFIR_FAIL(GBFIR_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  count_launch();
  return GBFIR_SUCCESS;
}

}  // namespace gbfir
