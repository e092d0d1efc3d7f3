// tc_blocks.cu — resample_poly as Toeplitz MMAs over materialised Hankel rows, in column
// blocks and K chunks (tcgen05; bf16, fp16, bf16x3 split precision; FP32 accumulate in TMEM).
// No MatX counterpart: the same outputs as MatX's resample_poly (include/matx/transforms/
// resample_poly.h:212-281 semantics) for rates whose rows advance by a number of input
// samples the aliased layouts of tc_resample.cu cannot express (160/147: rows of 160
// outputs advance 147 samples), and the tensor-core form of the ragged launch (many signals
// of their own rate, length and taps in one persistent launch; MatX runs one resample_poly
// per signal, include/matx/transforms/resample_poly.h:299-354).
//
// Math.  Rows of Nt = up*G outputs advance S = down*G input samples.  The row's phases are
// cut into column blocks of NB; block b (phases j in [b*NB, b*NB + NB)) only reads the band
// k in [k0_b, k0_b + Kb) (k0_b = the smallest k any of its phases reads), so
//   out[q*Nt + b*NB + n] = sum_k A_b[q][k] * W_b[n][k],
//   A_b[q][k] = x[q*S + k0_b + k],   W_b[n][k] = up * he[c + (b*NB + n)*down - (k0_b + k)*up].
// The band is taken in chunks of Kc = 64 (32 where the tap matrix needs the room; a block's
// accumulator sums its chunks), so the shared-memory slab does not grow with the filter.  The producers materialise each A chunk
// (a Hankel slab: neighbouring rows overlap) straight from global memory, split into the
// operand terms, in the no-swizzle K-major layout.  A complex signal puts the real parts of
// 64 rows in MMA rows 0-63 and their imaginary parts in rows 64-127 of the same MMA (the taps
// are real), so one MMA covers both parts.  W_b of every block is built once per signal.
//
// Pipeline (persistent, warp-specialised, 384 threads): a stage is (tile of rows, column
// block, K chunk).  Warps 1-7 materialise A into a 2-slot ring; warp 0 lane 0 issues the MMAs
// into one of two TMEM accumulator sets (one per (tile, block); bf16x3: a leading and a
// correction accumulator per set, summed in FP32 on the way out); warps 8-11 drain a set
// through a padded shared staging tile and store whole (complex) outputs, a warp per row at a
// time, coalesced.  The ragged launch takes work items (runs of tiles of one signal) from an
// atomic counter; between items every role is idle, the CTA rebuilds W for the item's signal
// and the stage counters (and so the mbarrier phases) carry on.  Every mbarrier wait is
// bounded: one that gives up sets the status word read by gbfir_tc_status().
#include <algorithm>
#include <cstdio>
#include <vector>

#include "common.cuh"
#include "tc.cuh"

namespace gbfir {

__device__ int32_t g_tcb_status;

int tc_blocks_status_take() {
  int32_t v = 0, zero = 0;
  if (cudaMemcpyFromSymbol(&v, g_tcb_status, sizeof(v)) != cudaSuccess) return -1;
  cudaMemcpyToSymbol(g_tcb_status, &zero, sizeof(zero));
  return v;
}

constexpr int kTbThreads = 384;
constexpr int kTbProd0 = 1, kTbProdWarps = 7, kTbEpi0 = 8;
constexpr int kTbNProd = kTbProdWarps * 32;
constexpr int kTbBatch = 3;     // producer items whose loads are in flight together

// Column-blocked geometry of one signal.
struct TbGeom {
  const void *x;
  int64_t x_bstride, N;
  const float *h;
  int64_t Lo, c;
  int32_t even, rev;
  double scale;
  void *out;
  int64_t out_bstride, out_len;
  int64_t up, down, Nt, S;
  int32_t NB, nblk, Kb, nkc, identity;
  int64_t rows, tiles_per_row, ntiles;
};

struct TbParams {
  TbGeom g;            // the single-signal launch's geometry
  int32_t terms, fp16;
  int32_t RT;          // rows per tile: 64 (complex: both parts in the 128 MMA rows) or 128
  int32_t NBmax;       // widest column block of the launch (TMEM, staging pitch NBmax + 4)
  int32_t wbytes;      // bytes of the W region
  int32_t Kc;          // K chunk: 64, or 32 where a launch needs the room for its W
  // ragged launch (ragged = 1)
  int32_t ragged;
  const gbfir_ragged_desc *descs;
  const int64_t *items;  // [nitems][4]: signal, first row, rows, packed geometry
  int64_t nitems;
  unsigned long long *counter;
};

// packed per-signal geometry of a ragged work item: G | NB << 8 | nblk << 16 | Kb << 32, or
// kTbIdentity for a signal whose rates reduce to 1/1 (a copy)
constexpr int64_t kTbIdentity = -1;
__host__ __device__ inline int64_t tb_pack(int64_t G, int64_t NB, int64_t nblk, int64_t Kb) {
  return G | (NB << 8) | (nblk << 16) | (Kb << 32);
}

// Timing hooks of the pipeline roles (role, stage, event); they compile to nothing unless a
// tracing build defines them.
#ifndef GBFIR_TC_TRACE
#define GBFIR_TC_TRACE(role, stage, event) \
  do {                                     \
  } while (0)
#endif

__device__ __forceinline__ void tb_sync(int id, int nthreads) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

// smallest k any phase of block b reads
__device__ __forceinline__ int64_t tb_k0(const TbGeom &g, int b) {
  return ceil_div(g.c + (int64_t)b * g.NB * g.down - g.Lo + 1, g.up);
}

__device__ __forceinline__ int64_t tb_gcd(int64_t a, int64_t b) {
  while (b) {
    const int64_t t = a % b;
    a = b;
    b = t;
  }
  return a;
}

template <bool XC>
__global__ void __launch_bounds__(kTbThreads, 1) tc_blocks_kernel(const TbParams p) {
  using XT = typename val_of<float, XC>::type;
  extern __shared__ __align__(1024) unsigned char smem_dyn[];
  __shared__ uint64_t op_full[2], op_empty[2], tm_full[2], tm_empty[2];
  __shared__ uint32_t tmem_slot;
  __shared__ int s_fail, s_pok, s_eok;
  __shared__ TbGeom sg;
  __shared__ long long s_item;
  __shared__ int64_t s_row0, s_ntiles;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) GBFIR_TC_TRACE(3, 0, 1);

  // layout: W [nblk][terms][NB x Kb] ; A ring [2][terms][128 x Kc] ; staging [128][NBmax + 4] f32
  unsigned char *smem = smem_dyn + ((1024u - (tc::smem_u32(smem_dyn) & 1023u)) & 1023u);
  const int Kc = p.Kc;
  const uint32_t abytes = 128u * (uint32_t)Kc * 2u;
  unsigned char *abase = smem + ((size_t)p.wbytes + 1023) / 1024 * 1024;
  auto amat = [&](int slot, int t) { return abase + ((size_t)slot * p.terms + t) * abytes; };
  const int sstride = p.NBmax + 4;
  float *stage = reinterpret_cast<float *>(abase + (size_t)2 * p.terms * abytes);

  // two accumulator sets of acc_cols columns, rounded up to a power of two >= 32.  bf16x3
  // keeps the leading product a0*b0 alone in the first NBmax columns of a set and the five
  // smaller ones in the next NBmax.  Every MMA instruction loses about one FP32 rounding of
  // its accumulator (six products a K-step into one accumulator measured 1.7e-6 rel-L2 at 475
  // taps), so the big sum takes one loss per K-step instead of six and the correction sum's
  // losses are 2^-8 smaller.
  const int acc_cols = p.terms == 3 ? 2 * p.NBmax : p.NBmax;
  const uint32_t tcols = 2 * acc_cols <= 32 ? 32u : 2 * acc_cols <= 64 ? 64u : 2 * acc_cols <= 128 ? 128u
                         : 2 * acc_cols <= 256 ? 256u : 512u;
  if (warp == 0) tc::tmem_alloc(&tmem_slot, tcols);
  if (tid == 0) {
    for (int i = 0; i < 2; i++) {
      tc::mbar_init(&op_full[i], 1);
      tc::mbar_init(&op_empty[i], 1);
      tc::mbar_init(&tm_full[i], 1);
      tc::mbar_init(&tm_empty[i], 1);
    }
    s_fail = 0;
    tc::mbar_fence_init();
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = tmem_slot;
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
  // stage counters of each role; they carry on across work items, so the mbarrier phases do
  int64_t ps = 0, ms = 0, me = 0, es = 0;
  for (int pass = 0;; pass++) {
    // ---- next work item: the whole launch's tiles (single signal) or one ragged item ----
    if (tid == 0) {
      if (!p.ragged) {
        s_item = pass == 0 ? 0 : -1;
        if (pass == 0) {
          sg = p.g;
          s_row0 = 0;
          s_ntiles = p.g.ntiles > blockIdx.x ? (p.g.ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
        }
      } else {
        const long long it = (long long)atomicAdd(p.counter, 1ULL);
        s_item = it < p.nitems ? it : -1;
        if (it < p.nitems) {
          const int64_t sig = p.items[4 * it], packed = p.items[4 * it + 3];
          const gbfir_ragged_desc d = p.descs[sig];
          TbGeom g{};
          g.x = d.in;
          g.N = d.in_len;
          g.h = d.h;
          g.out = d.out;
          g.out_len = d.out_len;
          const int64_t gg = tb_gcd(d.up, d.down);
          g.up = d.up / gg;
          g.down = d.down / gg;
          g.identity = packed == kTbIdentity;
          if (!g.identity) {
            g.even = (d.h_len % 2) == 0;
            g.Lo = d.h_len + g.even;
            g.c = (g.Lo - 1) / 2;
            g.scale = (double)g.up;
            const int64_t G = packed & 255;
            g.NB = (int32_t)((packed >> 8) & 255);
            g.nblk = (int32_t)((packed >> 16) & 65535);
            g.Kb = (int32_t)((packed >> 32) & 65535);
            g.nkc = (g.Kb + Kc - 1) / Kc;
            g.Nt = g.up * G;
            g.S = g.down * G;
            g.rows = (g.out_len + g.Nt - 1) / g.Nt;
          }
          sg = g;
          s_row0 = p.items[4 * it + 1];
          s_ntiles = (p.items[4 * it + 2] + p.RT - 1) / p.RT;
        }
      }
    }
    __syncthreads();
    if (s_item < 0 || s_fail) break;
    // a private copy: read through the shared struct, every field would be reloaded after each
    // store the compiler cannot prove does not alias it (a dependent shared load per element)
    const TbGeom g = sg;
    const int64_t row0 = s_row0, ntl = s_ntiles;
    if (g.identity) {
      // rates that reduce to 1/1: MatX's resample_poly copies the input (the taps are ignored);
      // a ragged item's rows are runs of RT elements here
      const XT *xi = reinterpret_cast<const XT *>(g.x);
      XT *yo = reinterpret_cast<XT *>(g.out);
      const int64_t e0 = row0, e1 = min(g.out_len, row0 + ntl * p.RT);
      for (int64_t e = e0 + tid; e < e1; e += kTbThreads) yo[e] = xi[e];
      __syncthreads();
      continue;
    }
    auto tile_of = [&](int64_t i, int64_t &bb, int64_t &q0) {
      if (p.ragged) {
        bb = 0;
        q0 = row0 + i * (int64_t)p.RT;
      } else {
        const int64_t t = blockIdx.x + i * (int64_t)gridDim.x;
        bb = t / g.tiles_per_row;
        q0 = (t - bb * g.tiles_per_row) * (int64_t)p.RT;
      }
    };
    // ---- W of this signal: the taps split into terms once (staged in the A ring, idle
    // here), then one item per (block, term, row n, 8-wide K chunk), one 16-byte store ----
    const uint32_t wbytes_b = (uint32_t)g.NB * g.Kb * 2u;
    auto wmat = [&](int b, int t) { return smem + ((size_t)b * p.terms + t) * wbytes_b; };
    const int64_t Lh = g.Lo - g.even;
    const bool h_staged = (size_t)Lh * 2 * p.terms <= (size_t)2 * p.terms * abytes;
    uint16_t *hterm = reinterpret_cast<uint16_t *>(abase);
    if (h_staged) {
      for (int64_t e = tid; e < Lh; e += kTbThreads) {
        uint16_t o[3];
        split_terms(g.h[e] * (float)g.scale, o);
        for (int t = 0; t < p.terms; t++) hterm[t * Lh + e] = o[t];
      }
    }
    __syncthreads();
    auto w_term = [&](int t, int64_t tp) -> uint32_t {
      if (tp < 0 || tp >= g.Lo) return 0u;
      const int64_t te = g.rev ? g.Lo - 1 - tp : tp;
      if (g.even && te == 0) return 0u;
      const int64_t e = te - g.even;
      if (h_staged) return hterm[t * Lh + e];
      uint16_t o[3];
      split_terms(g.h[e] * (float)g.scale, o);
      return o[t];
    };
    const int kch = g.Kb / 8;
    for (int it = tid; it < g.nblk * p.terms * g.NB * kch; it += kTbThreads) {
      const int rr = it / kch, kc = it - rr * kch;
      const int bt = rr / g.NB, n = rr - bt * g.NB;
      const int b = bt / p.terms, t = bt - b * p.terms;
      const int64_t j = (int64_t)b * g.NB + n;
      uint32_t w[4] = {0u, 0u, 0u, 0u};
      if (j < g.Nt) {
        const int64_t tp0 = g.c + j * g.down - (tb_k0(g, b) + 8 * kc) * g.up;
#pragma unroll
        for (int e = 0; e < 8; e++) w[e >> 1] |= w_term(t, tp0 - e * g.up) << (16 * (e & 1));
      }
      *reinterpret_cast<uint4 *>(wmat(b, t) + tc::kmajor_offset(n, 8 * kc, g.Kb)) = make_uint4(w[0], w[1], w[2], w[3]);
    }
    tc::fence_async_smem();
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    if (tid == 0) GBFIR_TC_TRACE(3, 0, 0);
    const XT *xp = reinterpret_cast<const XT *>(g.x);
    const int64_t nblocks = ntl * g.nblk;          // epilogue stages of the item
    const int64_t nstages = nblocks * g.nkc;       // producer / MMA stages of the item

    if (warp >= kTbProd0 && warp < kTbProd0 + kTbProdWarps) {
      // ================= producers: A chunks, from global memory =================
      // item (q, 8-wide K chunk): lanes take consecutive rows q, so a warp's 16-byte stores
      // fill whole 128-byte core matrices (conflict-free)
      const int ptid = tid - kTbProd0 * 32;
      for (int64_t k = 0; k < nstages; ++k, ++ps) {
        const int slot = (int)(ps & 1);
        const int64_t blk = k / g.nkc;
        const int kcn = (int)(k - blk * g.nkc);
        const int64_t i = blk / g.nblk;
        const int b = (int)(blk - i * g.nblk);
        if (ptid == 0) GBFIR_TC_TRACE(0, (int)k, 0);
        if (ptid == 0) s_pok = (ps < 2) ? 1 : (tc::mbar_wait(&op_empty[slot], (uint32_t)(((ps - 2) >> 1) & 1)) ? 1 : 0);
        tb_sync(1, kTbNProd);
        if (ptid == 0) GBFIR_TC_TRACE(0, (int)k, 1);
        if (!s_pok) {
          s_fail = 1;
          break;
        }
        int64_t bb, q0;
        tile_of(i, bb, q0);
        const XT *row = xp + bb * g.x_bstride;
        const int64_t k0 = tb_k0(g, b) + (int64_t)Kc * kcn;
        const int klen = min(Kc, g.Kb - Kc * kcn);
        const int nitems = p.RT * (klen / 8);
        // at a tile's first stage, the next tile's input (one contiguous run of its rows) is
        // prefetched into L2, so its slabs gather from L2 rather than DRAM
        if (b == 0 && kcn == 0 && ptid == 0 && i + 1 < ntl) {
          int64_t bn, qn;
          tile_of(i + 1, bn, qn);
          const XT *rown = xp + bn * g.x_bstride;
          int64_t lo = qn * g.S + tb_k0(g, 0), hi = (qn + p.RT) * g.S + tb_k0(g, g.nblk - 1) + g.Kb;
          lo = lo < 0 ? 0 : lo;
          hi = hi > g.N ? g.N : hi;
          // 16-byte boundaries inside [lo, hi): nothing outside the signal is touched
          uintptr_t a0 = (reinterpret_cast<uintptr_t>(rown + lo) + 15) & ~(uintptr_t)15;
          const uintptr_t a1 = reinterpret_cast<uintptr_t>(rown + hi) & ~(uintptr_t)15;
          for (; a0 < a1; a0 += 65536) {
            const uintptr_t n = a1 - a0 < 65536 ? a1 - a0 : 65536;
            tc::bulk_prefetch_l2(reinterpret_cast<const void *>(a0), (uint32_t)n);
          }
        }
        // kTbBatch items per thread at a time, every load of the batch issued before any
        // conversion, so a stage pays the global-load latency once per batch
        for (int i0 = ptid; i0 < nitems; i0 += kTbBatch * kTbNProd) {
          XT v[kTbBatch][8];
#pragma unroll
          for (int bi = 0; bi < kTbBatch; bi++) {
            const int itm = i0 + bi * kTbNProd;
            const int kc = itm / p.RT, q = itm - kc * p.RT;
            const int64_t g0 = (q0 + q) * g.S + k0 + 8 * kc;
#pragma unroll
            for (int e = 0; e < 8; e++) {
              const int64_t gi = g0 + e;
              v[bi][e] = (itm < nitems && gi >= 0 && gi < g.N) ? __ldg(row + gi) : zero_val<XT>();
            }
          }
#pragma unroll
          for (int bi = 0; bi < kTbBatch; bi++) {
            const int itm = i0 + bi * kTbNProd;
            if (itm >= nitems) break;
            const int kc = itm / p.RT, q = itm - kc * p.RT;
#pragma unroll
            for (int part = 0; part < (XC ? 2 : 1); part++) {
              uint32_t w[3][4];
#pragma unroll
              for (int e2 = 0; e2 < 4; e2++) {
                const float2 f = part == 0 ? make_float2(re_of(v[bi][2 * e2]), re_of(v[bi][2 * e2 + 1]))
                                           : make_float2(im_of(v[bi][2 * e2]), im_of(v[bi][2 * e2 + 1]));
                if (p.fp16) {
                  const __half2 hh = __floats2half2_rn(f.x, f.y);
                  w[0][e2] = *reinterpret_cast<const uint32_t *>(&hh);
                  w[1][e2] = w[2][e2] = 0u;
                } else {
                  __nv_bfloat162 t0, t1, t2;
                  tc::split3_bf16x2(f, t0, t1, t2);
                  w[0][e2] = *reinterpret_cast<uint32_t *>(&t0);
                  w[1][e2] = *reinterpret_cast<uint32_t *>(&t1);
                  w[2][e2] = *reinterpret_cast<uint32_t *>(&t2);
                }
              }
              const uint32_t off = tc::kmajor_offset(part * 64 + q, 8 * kc, Kc);
              *reinterpret_cast<uint4 *>(amat(slot, 0) + off) = make_uint4(w[0][0], w[0][1], w[0][2], w[0][3]);
              if (p.terms == 3) {
                *reinterpret_cast<uint4 *>(amat(slot, 1) + off) = make_uint4(w[1][0], w[1][1], w[1][2], w[1][3]);
                *reinterpret_cast<uint4 *>(amat(slot, 2) + off) = make_uint4(w[2][0], w[2][1], w[2][2], w[2][3]);
              }
            }
          }
        }
        tc::fence_async_smem();
        tb_sync(1, kTbNProd);
        if (ptid == 0) tc::mbar_arrive_plain(&op_full[slot]);
        if (ptid == 0) GBFIR_TC_TRACE(0, (int)k, 2);
      }
    } else if (warp == 0) {
      // ================= MMA issuer =================
      if (lane == 0) {
        const bool geom_ok = g.NB % 16 == 0 && g.NB <= p.NBmax && g.Kb % 16 == 0;
        if (!geom_ok) s_fail = 1;
        const uint32_t idesc = tc::idesc_f16(128, (uint32_t)g.NB, p.fp16 ? 0u : 1u);
        const uint32_t asbo = (uint32_t)(Kc / 8) * 128u, wsbo = (uint32_t)(g.Kb / 8) * 128u;
        // products of order <= 2 (signal term tx, tap term tw), smallest first
        constexpr uint32_t kTx = 0x001021u, kTw = 0x010201u;
        const int npairs = p.terms == 3 ? 6 : 1;
        for (int64_t k = 0; geom_ok && k < nstages; ++k, ++ms) {
          const int slot = (int)(ms & 1);
          const int64_t blk = k / g.nkc;
          const int kcn = (int)(k - blk * g.nkc);
          const int b = (int)(blk % g.nblk);
          const int set = (int)(me & 1);
          GBFIR_TC_TRACE(1, (int)k, 0);
          if (!tc::mbar_wait(&op_full[slot], (uint32_t)((ms >> 1) & 1))) { s_fail = 1; break; }
          // a block's first chunk needs its accumulator set drained by the epilogue
          if (kcn == 0 && me >= 2 && !tc::mbar_wait(&tm_empty[set], (uint32_t)(((me - 2) >> 1) & 1))) {
            s_fail = 1;
            break;
          }
          GBFIR_TC_TRACE(1, (int)k, 1);
          tc::tc_fence_after();
          const uint32_t d = tmem + (uint32_t)(set * acc_cols);
          const int nks = min(Kc, g.Kb - Kc * kcn) / 16;
          for (int pr = 0; pr < npairs; pr++) {
            const int tx = p.terms == 3 ? (int)((kTx >> (4 * pr)) & 15u) : 0;
            const int tw = p.terms == 3 ? (int)((kTw >> (4 * pr)) & 15u) : 0;
            // bf16x3: (0,0), the last pair, into the leading accumulator; the rest, first of them
            // pair 0, into the correction accumulator NBmax columns on
            const bool lead = pr == npairs - 1;
            const uint32_t dd = d + (p.terms == 3 && !lead ? (uint32_t)p.NBmax : 0u);
            const bool first_pair = lead || pr == 0;
            uint64_t ad = tc::smem_desc(tc::smem_u32(amat(slot, tx)), 128u, asbo);
            uint64_t bd = tc::smem_desc(tc::smem_u32(wmat(b, tw)) + (uint32_t)(kcn * (Kc / 8) * 128), 128u, wsbo);
            for (int ks = 0; ks < nks; ks++) {
              tc::mma_f16(dd, ad, bd, idesc, (kcn > 0 || !first_pair || ks > 0) ? 1u : 0u);
              ad += 16;  // +256 B: two core matrices along K
              bd += 16;
            }
          }
          tc::mma_commit(&op_empty[slot]);
          if (kcn == g.nkc - 1) {
            tc::mma_commit(&tm_full[set]);
            ++me;
          }
          GBFIR_TC_TRACE(1, (int)k, 2);
        }
      }
    } else if (warp >= kTbEpi0) {
      // ================= epilogue =================
      // quarter w holds TMEM lanes 32w..32w+31 = staging rows; for a complex signal rows
      // 0-63 are real parts and 64-127 imaginary parts of the tile's 64 rows
      const int quarter = warp - kTbEpi0;
      const int srow = 32 * quarter + lane;
      const uint32_t lane_base = (uint32_t)(32 * quarter) << 16;
      for (int64_t e = 0; e < nblocks; ++e, ++es) {
        const int set = (int)(es & 1);
        const int64_t i = e / g.nblk;
        const int b = (int)(e - i * g.nblk);
        if (quarter == 0 && lane == 0) GBFIR_TC_TRACE(2, (int)e, 0);
        if (quarter == 0 && lane == 0) s_eok = tc::mbar_wait(&tm_full[set], (uint32_t)((es >> 1) & 1)) ? 1 : 0;
        tb_sync(2, 128);
        if (quarter == 0 && lane == 0) GBFIR_TC_TRACE(2, (int)e, 1);
        if (!s_eok) {
          s_fail = 1;
          break;
        }
        tc::tc_fence_after();
        float *srow_p = stage + (size_t)srow * sstride;
        for (int col = 0; col < g.NB; col += 16) {
          uint32_t r[16], rc[16];
          tc::tmem_ld16(tmem + lane_base + (uint32_t)(set * acc_cols + col), r);
          if (p.terms == 3) tc::tmem_ld16(tmem + lane_base + (uint32_t)(set * acc_cols + p.NBmax + col), rc);
          tc::tmem_ld_wait();
          if (p.terms == 3) {
#pragma unroll
            for (int q = 0; q < 16; q++) r[q] = __float_as_uint(__uint_as_float(r[q]) + __uint_as_float(rc[q]));
          }
#pragma unroll
          for (int q = 0; q < 16; q += 4)
            *reinterpret_cast<float4 *>(srow_p + col + q) =
                make_float4(__uint_as_float(r[q]), __uint_as_float(r[q + 1]), __uint_as_float(r[q + 2]),
                            __uint_as_float(r[q + 3]));
        }
        tc::tc_fence_before();
        tb_sync(2, 128);
        if (quarter == 0 && lane == 0) tc::mbar_arrive_plain(&tm_empty[set]);
        if (quarter == 0 && lane == 0) GBFIR_TC_TRACE(2, (int)e, 3);
        // whole outputs, a warp per row at a time: lanes take consecutive phases (coalesced)
        int64_t bb, q0;
        tile_of(i, bb, q0);
        XT *orow = reinterpret_cast<XT *>(g.out) + bb * g.out_bstride;
        const int64_t j0 = (int64_t)b * g.NB;
        // the row's valid phases of this block, worked out once per row; the loop body is two
        // shared loads and one store, two phases a lane in flight
        const int64_t cols = std::min<int64_t>(g.NB, g.Nt - j0);
        for (int q = quarter; q < p.RT; q += 4) {
          const int64_t n0 = (q0 + q) * g.Nt + j0;
          const int lim = (int)std::max<int64_t>(0, std::min<int64_t>(cols, g.out_len - n0));
          const float *sr = stage + (size_t)q * sstride;
          XT *dst = orow + n0;
          if constexpr (XC) {
            const float *si = stage + (size_t)(64 + q) * sstride;
#pragma unroll 2
            for (int n = lane; n < lim; n += 32) dst[n] = make_float2(sr[n], si[n]);
          } else {
#pragma unroll 2
            for (int n = lane; n < lim; n += 32) dst[n] = sr[n];
          }
        }
        tb_sync(2, 128);  // the staging tile is read before the next stage overwrites it
        if (quarter == 0 && lane == 0) GBFIR_TC_TRACE(2, (int)e, 2);
      }
    }
    __syncthreads();  // the item is drained: W and the rings may be rewritten
  }
  __syncthreads();
  if (s_fail && tid == 0) {
    atomicExch(&g_tcb_status, 1);
    // give MMAs still in flight a bounded chance to finish before the TMEM is freed
    (void)tc::mbar_wait(&tm_full[0], 0);
    (void)tc::mbar_wait(&tm_full[1], 0);
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc::tc_fence_after();
    tc::tmem_dealloc(tmem, tcols);
  }
}

// Shared memory of a launch: W region + A ring + staging (+ alignment slack).
static size_t tb_smem(size_t wbytes, int terms, int NBmax, int Kc) {
  return 1024 + (wbytes + 1023) / 1024 * 1024 + (size_t)2 * terms * 128 * Kc * 2 + (size_t)128 * (NBmax + 4) * 4;
}

// Column-blocked geometry of one signal: rows of Nt = up*G outputs (G the smallest with
// Nt >= 32), blocks of NB phases (64, 48, 32 or 16: the widest whose W fits wmax bytes).
// Returns false where no block width fits.
static bool tb_geometry(int64_t up, int64_t down, int64_t Lo, int64_t c, int terms, size_t wmax, int Kc, TbGeom &g) {
  int64_t G = 1;
  while (up * G < 32 && G < 64) G++;
  g.up = up;
  g.down = down;
  g.Lo = Lo;
  g.c = c;
  g.Nt = up * G;
  g.S = down * G;
  for (int NB : {64, 48, 32, 16}) {
    if (NB > ((g.Nt + 15) / 16) * 16 && NB > 16) continue;
    const int nblk = (int)((g.Nt + NB - 1) / NB);
    int64_t span = 1;
    for (int b = 0; b < nblk; b++) {
      const int64_t j0 = (int64_t)b * NB, j1 = std::min<int64_t>(g.Nt - 1, j0 + NB - 1);
      const int64_t k0 = ceil_div(c + j0 * down - Lo + 1, up);
      const int64_t k1 = floor_div(c + j1 * down, up);
      span = std::max<int64_t>(span, k1 - k0 + 1);
    }
    const int64_t Kb = (span + 15) / 16 * 16;
    const size_t w = (size_t)nblk * terms * NB * Kb * 2;
    if (w > wmax || Kb > 65535 || nblk > 65535) continue;
    g.NB = NB;
    g.nblk = nblk;
    g.Kb = (int32_t)Kb;
    g.nkc = (int32_t)((Kb + Kc - 1) / Kc);
    return true;
  }
  return false;
}

// The W budget of a launch whose widest block is 64 phases, with K chunks of Kc.
static size_t tb_wmax(int terms, int Kc) { return 225 * 1024 - tb_smem(0, terms, 64, Kc); }

// Plans and launches the column-blocked pass for out = scale * sum x * he(c + n*down - k*up);
// returns GBFIR_ERR_NOT_SUPPORTED (with the reason) where no tile fits.
int launch_tc_blocks(const gbfir_buf &out, const gbfir_buf &in, const gbfir_buf &h, int64_t up, int64_t down,
                     int64_t Lo, int64_t c, int even, int rev, double scale, int precision, const char *what,
                     cudaStream_t s) {
  const bool xc = dtype_complex(in.dtype);
  TbParams p{};
  p.terms = precision == GBFIR_PREC_BF16X3 ? 3 : 1;
  p.fp16 = precision == GBFIR_PREC_FP16;
  p.RT = xc ? 64 : 128;
  TbGeom &g = p.g;
  // K chunks of 64, or of 32 where the tap matrix needs the room
  p.Kc = 64;
  if (!tb_geometry(up, down, Lo, c, p.terms, tb_wmax(p.terms, 64), 64, g)) p.Kc = 32;
  if (p.Kc == 32 && !tb_geometry(up, down, Lo, c, p.terms, tb_wmax(p.terms, 32), 32, g))
    GBFIR_FAIL(GBFIR_ERR_NOT_SUPPORTED, "%s: column-blocked tensor-core form unavailable: the tap matrix of a %lld-tap "
               "filter at %lld/%lld does not fit shared memory", what, (long long)Lo, (long long)up, (long long)down);
  g.even = even;
  g.rev = rev;
  g.scale = scale;
  g.N = in.len;
  g.out_len = out.len;
  g.x = in.ptr;
  g.x_bstride = (out.batch > 1 && in.batch > 1) ? in.batch_stride : 0;
  g.h = reinterpret_cast<const float *>(h.ptr);
  g.out = out.ptr;
  g.out_bstride = out.batch_stride;
  g.rows = (out.len + g.Nt - 1) / g.Nt;
  g.tiles_per_row = (g.rows + p.RT - 1) / p.RT;
  g.ntiles = g.tiles_per_row * out.batch;
  p.NBmax = g.NB;
  p.wbytes = (int32_t)((size_t)g.nblk * p.terms * g.NB * g.Kb * 2);
  const size_t smem = tb_smem((size_t)p.wbytes, p.terms, p.NBmax, p.Kc);
  const void *fn = xc ? (const void *)tc_blocks_kernel<true> : (const void *)tc_blocks_kernel<false>;
  int rc = ensure_smem(fn, smem, what);
  if (rc) return rc;
  int64_t grid = num_sms();  // one CTA per SM
  if (grid > g.ntiles) grid = g.ntiles;
  if (grid < 1) return GBFIR_SUCCESS;
  void *args[] = {&p};
  const cudaError_t e = cudaLaunchKernel(fn, dim3((unsigned)grid), dim3(kTbThreads), args, smem, s);
  if (e != cudaSuccess) GBFIR_FAIL(GBFIR_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  count_launch();
  return GBFIR_SUCCESS;
}

// ---- ragged tensor-core form ------------------------------------------------------------
// Host plan: per signal the column-blocked geometry (W within the launch's budget) packed into
// its work items; items are runs of 64-row tiles of one signal of about 1/8 of a CTA's fair
// share, most expensive first.  Returns the item count or a negative status.
int64_t ragged_plan_tc(const gbfir_ragged_desc *descs, int64_t count, int precision, int64_t *table,
                       int64_t *shared_bytes, int64_t *kchunk) {
  const int terms = precision == GBFIR_PREC_BF16X3 ? 3 : 1;
  constexpr int RT = 64;
  // K chunks of 64 unless some signal's tap matrix needs the room of chunks of 32
  int Kc = 64;
  for (int64_t s = 0; s < count && Kc == 64; s++) {
    const gbfir_ragged_desc &d = descs[s];
    const int64_t gg = gcd64(d.up, d.down);
    if (d.up / gg == 1 && d.down / gg == 1) continue;
    const int64_t Lo = d.h_len + ((d.h_len % 2) == 0);
    TbGeom g{};
    if (!tb_geometry(d.up / gg, d.down / gg, Lo, (Lo - 1) / 2, terms, tb_wmax(terms, 64), 64, g)) Kc = 32;
  }
  const size_t wmax = tb_wmax(terms, Kc);
  struct Item {
    double cost;
    int64_t sig, row0, nrows, packed;
  };
  std::vector<Item> items;
  std::vector<int64_t> ntiles_of, packs, rows_of;
  std::vector<double> cost_of;
  size_t wneed = 0;
  double total = 0;
  for (int64_t s = 0; s < count; s++) {
    const gbfir_ragged_desc &d = descs[s];
    const int64_t gg = gcd64(d.up, d.down);
    const int64_t up = d.up / gg, down = d.down / gg;
    // a 1/1 signal is copied in runs of RT elements: its "rows" are elements
    int64_t packed = kTbIdentity, rows = d.out_len;
    double tile_cost = RT;
    if (!(up == 1 && down == 1)) {
      const int even = (d.h_len % 2) == 0;
      const int64_t Lo = d.h_len + even;
      TbGeom g{};
      if (!tb_geometry(up, down, Lo, (Lo - 1) / 2, terms, wmax, Kc, g)) {
        char buf[200];
        snprintf(buf, sizeof(buf), "ragged_plan: signal %lld (%lld taps at %lld/%lld) has no tensor-core tile that fits",
                 (long long)s, (long long)d.h_len, (long long)d.up, (long long)d.down);
        set_error(buf);
        return -GBFIR_ERR_NOT_SUPPORTED;
      }
      wneed = std::max(wneed, (size_t)g.nblk * terms * g.NB * g.Kb * 2);
      packed = tb_pack(g.Nt / up, g.NB, g.nblk, g.Kb);
      rows = (d.out_len + g.Nt - 1) / g.Nt;
      // MMA issues of a tile (per block and K chunk) and its output stores
      tile_cost = (double)RT * g.nblk * g.nkc * 4.0 + (double)RT * g.Nt;
    }
    const int64_t ntiles = (rows + RT - 1) / RT;
    ntiles_of.push_back(ntiles);
    cost_of.push_back(tile_cost);
    packs.push_back(packed);
    rows_of.push_back(rows);
    total += tile_cost * (double)ntiles;
  }
  const double target = total / ((double)num_sms() * 8.0);
  for (int64_t s = 0; s < count; s++) {
    const int64_t ntiles = ntiles_of[(size_t)s];
    const double tc = cost_of[(size_t)s];
    int64_t per = (int64_t)(target / std::max(tc, 1.0));
    per = std::max<int64_t>(1, std::min<int64_t>(per, ntiles));
    for (int64_t k = 0; k < ntiles; k += per) {
      const int64_t n = std::min<int64_t>(per, ntiles - k);
      const int64_t row0 = k * RT;
      items.push_back({tc * (double)n, s, row0, std::min<int64_t>(n * RT, rows_of[(size_t)s] - row0),
                       packs[(size_t)s]});
    }
  }
  if (table) {
    std::stable_sort(items.begin(), items.end(), [](const Item &a, const Item &b) { return a.cost > b.cost; });
    for (size_t i = 0; i < items.size(); i++) {
      table[4 * i] = items[i].sig;
      table[4 * i + 1] = items[i].row0;
      table[4 * i + 2] = items[i].nrows;
      table[4 * i + 3] = items[i].packed;
    }
  }
  *shared_bytes = (int64_t)tb_smem(wneed, terms, 64, Kc);
  *kchunk = Kc;
  return (int64_t)items.size();
}

int ragged_resample_tc(const gbfir_ragged_desc *device_descs, const int64_t *device_items, int64_t nitems,
                       int64_t shared_bytes, int64_t kchunk, int precision, void *workspace, cudaStream_t s) {
  TbParams p{};
  p.terms = precision == GBFIR_PREC_BF16X3 ? 3 : 1;
  p.fp16 = precision == GBFIR_PREC_FP16;
  p.RT = 64;
  p.NBmax = 64;
  if (kchunk != 32 && kchunk != 64)
    GBFIR_FAIL(GBFIR_ERR_INVALID_PARAMETER, "ragged_resample: plan info does not come from gbfir_ragged_plan_prec");
  p.Kc = (int32_t)kchunk;
  const int64_t base = (int64_t)tb_smem(0, p.terms, 64, p.Kc);
  if (shared_bytes < base || shared_bytes > 225 * 1024)
    GBFIR_FAIL(GBFIR_ERR_INVALID_PARAMETER, "ragged_resample: plan info does not come from gbfir_ragged_plan_prec");
  p.wbytes = (int32_t)(shared_bytes - base);
  p.ragged = 1;
  p.descs = device_descs;
  p.items = device_items;
  p.nitems = nitems;
  p.counter = reinterpret_cast<unsigned long long *>(workspace);
  cudaError_t e = cudaMemsetAsync(workspace, 0, 8, s);
  if (e != cudaSuccess) GBFIR_FAIL(GBFIR_ERR_CUDA, "ragged_resample: %s", cudaGetErrorString(e));
  const void *fn = (const void *)tc_blocks_kernel<true>;
  int rc = ensure_smem(fn, (size_t)shared_bytes, "ragged_resample (tensor cores)");
  if (rc) return rc;
  int64_t grid = num_sms();
  if (grid > nitems) grid = nitems;
  void *args[] = {&p};
  e = cudaLaunchKernel(fn, dim3((unsigned)grid), dim3(kTbThreads), args, (size_t)shared_bytes, s);
  if (e != cudaSuccess) GBFIR_FAIL(GBFIR_ERR_CUDA, "ragged_resample (tensor cores): %s", cudaGetErrorString(e));
  count_launch();
  return GBFIR_SUCCESS;
}

}  // namespace gbfir
