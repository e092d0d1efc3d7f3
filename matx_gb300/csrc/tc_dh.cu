// tc_dh.cu — the tap gradient dL/dh of resample_poly on the tensor cores (tcgen05; bf16,
// fp16, bf16x3 split precision; FP32 accumulate in TMEM, FP64 across CTAs).  No MatX
// counterpart: MatX has no adjoints; the gradient it must agree with is the one composed
// from MatX's corr (include/matx/transforms/corr.h:60-69) over the forward of
// include/matx/transforms/resample_poly.h:212-281.
//
// Math.  The forward is y[b][n] = scale * sum_i x[b][i] * he[c + n*down - i*up].  Cut the
// outputs into rows of Nt = up*G (row q holds n = q*Nt + j) and read each row's inputs from
// i = q*S + kmin + k (S = down*G).  The tap an (n, i) pair uses,
//   t = c + j*down - (kmin + k)*up,
// does not depend on q, so the tap gradient is a GEMM reduced over the rows:
//   dB[k][j] = sum_{b,q} X[q][k] * GY[q][j],   X[q][k] = x[b][q*S + kmin + k],
//                                              GY[q][j] = gy[b][q*Nt + j],
//   dh[t] = scale * sum_{(k, j) -> t} dB[k][j].
// dB is a (band of W input positions) x (Nt phases) matrix: M = k in MT tiles of 128 TMEM
// lanes, N = j (Nt padded to NP, a multiple of 16), K = rows, 16 per MMA.  Each CTA reduces
// its share of the rows in TMEM (a persistent CTA per SM, rows in stages of KR), then folds
// its dB onto the taps in FP64, in a fixed order, into its row of partials; a second kernel
// adds the CTAs' partials in a fixed order.  The result is deterministic.
//
// Pipeline (384 threads): warps 1-11 materialise each stage's operands straight from global
// memory — the X Hankel slab and the GY slab, split into the operand terms — into a ring of
// 2 to 4 slots, each warp arriving on the slot's barrier when its own items are stored (no
// CTA-wide barrier); warp 0 lane 0 issues the MMAs.  Stages of 64 rows use the 128-byte
// swizzled K-major layout (the tensor core reads it at about twice the rate of the
// no-swizzle layout at N = 128), with the no-swizzle layout and 32- or 16-row stages where
// those do not fit.  bf16x3 keeps the leading product x0*g0 in its own accumulator (every MMA
// costs about one FP32 rounding of its accumulator): where two gradient terms fit one MMA
// (N = 2*NP <= 256) it issues four MMAs a K-step into [x0*g0 | x0*g1 + x1*g0 | x1*g1 + x2*g0
// + x0*g2] (B = [g0 | g1] for two of them), else six into x0*g0 and the rest.  At the end
// every warp drains part of TMEM through shared memory and every thread folds taps.  Every mbarrier
// wait is bounded: one that gives up sets the status word read by gbfir_tc_status().
#include <algorithm>

#include "common.cuh"
#include "tc.cuh"

namespace gbfir {

__device__ int32_t g_tcd_status;

int tc_dh_status_take() {
  int32_t v = 0, zero = 0;
  if (cudaMemcpyFromSymbol(&v, g_tcd_status, sizeof(v)) != cudaSuccess) return -1;
  cudaMemcpyToSymbol(g_tcd_status, &zero, sizeof(zero));
  return v;
}

constexpr int kTdThreads = 384;
constexpr int kTdProd0 = 1, kTdProdWarps = 11;
constexpr int kTdNProd = kTdProdWarps * 32;
constexpr int kTdBatch = 8;     // producer items whose loads are in flight together
constexpr int kTdMaxItems = 8;  // producer items per thread and stage (planner bound)
constexpr int kTdMaxSlots = 4;  // operand ring slots

struct TdParams {
  const float *x;
  int64_t x_bstride, N;
  const float *gy;
  int64_t gy_bstride, out_len;
  int64_t up, down, Lo, c, kmin, inv_down;
  int64_t Nt, S;
  int32_t NP, MT, KR, terms, fp16;
  int32_t nslot;  // operand ring slots (2..4)
  int32_t sw;     // 1: 128-byte-swizzled K-major operands (KR = 64: a row of a tile is 128 bytes)
  int32_t nsub, fold_off;  // threads per tap in the fold; byte offset of its FP64 sums
  int32_t cat;    // bf16x3 with the gradient terms concatenated along N: 4 MMAs a K-step into
                  // three accumulators [x0*g0 | x0*g1 + x1*g0 | x1*g1 + x2*g0 + x0*g2]
  int64_t tiles_per_row, ntiles;
  double *partial;  // [gridDim.x][Lo]
};


// Timing hooks of the pipeline roles (role, stage, event); they compile to nothing unless a
// tracing build defines them.
#ifndef GBFIR_TC_TRACE
#define GBFIR_TC_TRACE(role, stage, event) \
  do {                                     \
  } while (0)
#endif

// Byte offset of the 16-byte chunk (row, 8-wide K chunk kc) in a tile of KR-wide K-major rows:
// the no-swizzle core-matrix layout, or with sw the 128-byte swizzle (rows of 128 bytes, the
// chunk index XORed with the row's position in its 8-row, 1024-byte group; tiles 1024-aligned).
__device__ __forceinline__ uint32_t td_chunk_offset(uint32_t row, uint32_t kc, uint32_t KR, bool sw) {
  return sw ? (row << 7) + ((kc ^ (row & 7u)) << 4) : tc::kmajor_offset(row, 8u * kc, KR);
}

__global__ void __launch_bounds__(kTdThreads, 1) tc_dh_kernel(const TdParams p) {
  extern __shared__ __align__(1024) unsigned char smem_dyn[];
  __shared__ uint64_t op_full[kTdMaxSlots], op_empty[kTdMaxSlots], acc_full;
  __shared__ uint32_t tmem_slot;
  __shared__ int s_fail, s_aok;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) GBFIR_TC_TRACE(3, 0, 1);

  // ring slot: X tiles [terms][MT][128 x KR] then GY tiles [terms][NP x KR], bf16/fp16
  unsigned char *smem = smem_dyn + ((1024u - (tc::smem_u32(smem_dyn) & 1023u)) & 1023u);
  const int KR = p.KR;
  const uint32_t abytes = 128u * (uint32_t)KR * 2u, bbytes = (uint32_t)p.NP * KR * 2u;
  const size_t slot_bytes = ((size_t)p.MT * abytes + bbytes) * p.terms;
  auto amat = [&](int slot, int mt, int t) { return smem + slot * slot_bytes + ((size_t)t * p.MT + mt) * abytes; };
  auto bmat = [&](int slot, int t) {
    return smem + slot * slot_bytes + (size_t)p.terms * p.MT * abytes + (size_t)t * bbytes;
  };
  const bool split = p.terms == 3 && !p.cat;
  const int acc_cols = p.MT * p.NP;  // M-tile mt in columns [mt*NP, mt*NP + NP) (cat: [mt*3*NP, +3*NP))
  const int need = p.cat ? 3 * acc_cols : split ? 2 * acc_cols : acc_cols;
  const uint32_t tcols = need <= 32 ? 32u : need <= 64 ? 64u : need <= 128 ? 128u : need <= 256 ? 256u : 512u;
  if (warp == 0) tc::tmem_alloc(&tmem_slot, tcols);
  if (tid == 0) {
    for (int i = 0; i < p.nslot; i++) {
      tc::mbar_init(&op_full[i], kTdProdWarps);
      tc::mbar_init(&op_empty[i], 1);
    }
    tc::mbar_init(&acc_full, 1);
    s_fail = 0;
    tc::mbar_fence_init();
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = tmem_slot;
  const int64_t my_tiles = p.ntiles > blockIdx.x ? (p.ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;

  if (warp >= kTdProd0) {
    // ================= producers =================
    // items: (X row m, 8-row K chunk) then (GY phase n, 8-row K chunk); lanes take
    // consecutive m (n): the 8 loads of an item are rows apart, a warp's loads coalesced,
    // and its 16-byte stores fill whole 128-byte core matrices.  A thread's items are the
    // same in every stage (only the rows move), so their offsets are worked out once.
    const int ptid = tid - kTdProd0 * 32;
    const int mrows = p.MT * 128, kch = KR / 8;
    const int nA = mrows * kch, nitems = nA + p.NP * kch;
    const int Si = (int)p.S, Nti = (int)p.Nt;
    int it_g[kTdMaxItems];       // element offset from the stage's first sample (X) or gradient (GY)
    uint32_t it_s[kTdMaxItems];  // byte offset of term 0 in the ring slot; bit 31: GY item, bit 30: zero
#pragma unroll
    for (int j = 0; j < kTdMaxItems; j++) {
      const int itm = ptid + j * kTdNProd;
      it_g[j] = 0;
      it_s[j] = 1u << 30;
      if (itm < nA) {
        const int kc = itm / mrows, m = itm - kc * mrows;
        it_g[j] = 8 * kc * Si + m;
        it_s[j] = (uint32_t)(m >> 7) * abytes + td_chunk_offset((uint32_t)(m & 127), (uint32_t)kc, (uint32_t)KR, p.sw);
      } else if (itm < nitems) {
        const int i2 = itm - nA;
        const int kc = i2 / p.NP, n = i2 - kc * p.NP;
        it_g[j] = 8 * kc * Nti + n;
        it_s[j] = (1u << 31) | (n < Nti ? 0u : 1u << 30) |
                  ((uint32_t)p.terms * p.MT * abytes + td_chunk_offset((uint32_t)n, (uint32_t)kc, (uint32_t)KR, p.sw));
      }
    }
    const uint32_t tstride_a = (uint32_t)p.MT * abytes;
    for (int64_t i = 0; i < my_tiles; ++i) {
      const int slot = (int)(i % p.nslot);
      const int64_t round = i / p.nslot;
      if (ptid == 0) GBFIR_TC_TRACE(0, (int)i, 0);
      int ok = 1;
      if (lane == 0 && round > 0) ok = tc::mbar_wait(&op_empty[slot], (uint32_t)((round - 1) & 1)) ? 1 : 0;
      if (!__shfl_sync(0xffffffffu, ok, 0)) {
        s_fail = 1;
        break;
      }
      if (ptid == 0) GBFIR_TC_TRACE(0, (int)i, 1);
      const int64_t t = blockIdx.x + i * (int64_t)gridDim.x;
      const int64_t b = t / p.tiles_per_row;
      const int64_t q0 = (t - b * p.tiles_per_row) * KR;
      const int64_t xbase = q0 * p.S + p.kmin, gbase = q0 * p.Nt;
      const float *xr = p.x + b * p.x_bstride;
      const float *gr = p.gy + b * p.gy_bstride;
      unsigned char *sbase = smem + slot * slot_bytes;
#pragma unroll
      for (int j0 = 0; j0 < kTdMaxItems; j0 += kTdBatch) {
        if (ptid + j0 * kTdNProd >= nitems) break;
        float v[kTdBatch][8];
        // every load of the batch is issued before any conversion
#pragma unroll
        for (int bi = 0; bi < kTdBatch; bi++) {
          const int j = j0 + bi;
          const uint32_t sd = it_s[j];
          if (sd & (1u << 30)) {
#pragma unroll
            for (int e = 0; e < 8; e++) v[bi][e] = 0.f;
          } else if (!(sd >> 31)) {
            const int64_t g0 = xbase + it_g[j];
            const float *src = xr + g0;
            if (g0 >= 0 && g0 + 7 * (int64_t)Si < p.N) {
#pragma unroll
              for (int e = 0; e < 8; e++) v[bi][e] = __ldg(src + e * Si);
            } else {
#pragma unroll
              for (int e = 0; e < 8; e++) {
                const int64_t gi = g0 + e * (int64_t)Si;
                v[bi][e] = (gi >= 0 && gi < p.N) ? __ldg(xr + gi) : 0.f;
              }
            }
          } else {
            const int64_t g0 = gbase + it_g[j];
            const float *src = gr + g0;
            if (g0 + 7 * (int64_t)Nti < p.out_len) {
#pragma unroll
              for (int e = 0; e < 8; e++) v[bi][e] = __ldg(src + e * Nti);
            } else {
#pragma unroll
              for (int e = 0; e < 8; e++) v[bi][e] = g0 + e * (int64_t)Nti < p.out_len ? __ldg(src + e * Nti) : 0.f;
            }
          }
        }
#pragma unroll
        for (int bi = 0; bi < kTdBatch; bi++) {
          const int j = j0 + bi;
          if (ptid + j * kTdNProd >= nitems) break;
          uint32_t w[3][4];
#pragma unroll
          for (int e2 = 0; e2 < 4; e2++) {
            const float2 f = make_float2(v[bi][2 * e2], v[bi][2 * e2 + 1]);
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
          const uint32_t sd = it_s[j];
          unsigned char *dst = sbase + (sd & 0x3FFFFFFFu);
          const uint32_t ts = (sd >> 31) ? bbytes : tstride_a;
          *reinterpret_cast<uint4 *>(dst) = make_uint4(w[0][0], w[0][1], w[0][2], w[0][3]);
          if (p.terms == 3) {
            *reinterpret_cast<uint4 *>(dst + ts) = make_uint4(w[1][0], w[1][1], w[1][2], w[1][3]);
            *reinterpret_cast<uint4 *>(dst + 2 * ts) = make_uint4(w[2][0], w[2][1], w[2][2], w[2][3]);
          }
        }
      }
      tc::fence_async_smem();
      __syncwarp();
      if (lane == 0) tc::mbar_arrive_plain(&op_full[slot]);
      if (ptid == 0) GBFIR_TC_TRACE(0, (int)i, 2);
    }
  } else if (lane == 0) {
    // ================= MMA issuer (warp 0, one thread) =================
    const uint32_t idesc = tc::idesc_f16(128, (uint32_t)p.NP, p.fp16 ? 0u : 1u);
    const uint32_t idesc2 = tc::idesc_f16(128, 2u * (uint32_t)p.NP, 1u);
    const uint32_t sbo = (uint32_t)(KR / 8) * 128u;
    // no swizzle: K-adjacent core matrices 128 bytes apart, row groups sbo apart; 128-byte
    // swizzle (layout type 2): row groups 1024 bytes apart, K-step s starting 32*s bytes in
    auto desc = [&](const unsigned char *tile) -> uint64_t {
      return p.sw ? (tc::smem_desc(tc::smem_u32(tile), 16u, 1024u) | ((uint64_t)2 << 61))
                  : tc::smem_desc(tc::smem_u32(tile), 128u, sbo);
    };
    const uint64_t kstep = p.sw ? 2 : 16;  // in 16-byte units
    // products of order <= 2 (signal term tx, gradient term tg), smallest first; the last,
    // x0*g0, goes to the leading accumulator
    constexpr uint32_t kTx = 0x001021u, kTg = 0x010201u;
    const int npairs = split ? 6 : 1;
    for (int64_t i = 0; i < my_tiles; ++i) {
      const int slot = (int)(i % p.nslot);
      GBFIR_TC_TRACE(1, (int)i, 0);
      if (!tc::mbar_wait(&op_full[slot], (uint32_t)((i / p.nslot) & 1))) {
        s_fail = 1;
        break;
      }
      GBFIR_TC_TRACE(1, (int)i, 1);
      tc::tc_fence_after();
      for (int mt = 0; p.cat && mt < p.MT; mt++) {
        // C2 is initialised first (x0*g2), so the x1*[g0|g1] MMA, which spans C1 and C2, only
        // ever accumulates; B = [g0 | g1] is the two term tiles back to back (N = 2*NP)
        const uint32_t L = tmem + (uint32_t)(mt * 3 * p.NP), C1 = L + (uint32_t)p.NP, C2 = L + 2u * p.NP;
        uint64_t a0 = desc(amat(slot, mt, 0)), a1 = desc(amat(slot, mt, 1)), a2 = desc(amat(slot, mt, 2));
        uint64_t g01 = desc(bmat(slot, 0)), g2 = desc(bmat(slot, 2));
        for (int ks = 0; ks < KR / 16; ks++) {
          const uint32_t acc = (i > 0 || ks > 0) ? 1u : 0u;
          tc::mma_f16(C2, a0, g2, idesc, acc);
          tc::mma_f16(C2, a2, g01, idesc, 1u);
          tc::mma_f16(L, a0, g01, idesc2, acc);
          tc::mma_f16(C1, a1, g01, idesc2, 1u);
          a0 += kstep;
          a1 += kstep;
          a2 += kstep;
          g01 += kstep;
          g2 += kstep;
        }
      }
      for (int mt = 0; !p.cat && mt < p.MT; mt++) {
        for (int pr = 0; pr < npairs; pr++) {
          const int tx = split ? (int)((kTx >> (4 * pr)) & 15u) : 0;
          const int tg = split ? (int)((kTg >> (4 * pr)) & 15u) : 0;
          const bool lead = pr == npairs - 1;
          const uint32_t d = tmem + (uint32_t)(mt * p.NP) + (split && !lead ? (uint32_t)acc_cols : 0u);
          const bool first_pair = lead || pr == 0;
          uint64_t ad = desc(amat(slot, mt, tx));
          uint64_t bd = desc(bmat(slot, tg));
          for (int ks = 0; ks < KR / 16; ks++) {
            tc::mma_f16(d, ad, bd, idesc, (i > 0 || !first_pair || ks > 0) ? 1u : 0u);
            ad += kstep;
            bd += kstep;
          }
        }
      }
      tc::mma_commit(&op_empty[slot]);
      GBFIR_TC_TRACE(1, (int)i, 2);
    }
    // arrives once every MMA issued above has completed (at once if there were none)
    tc::mma_commit(&acc_full);
  }

  // ================= drain and fold =================
  if (tid == 0) GBFIR_TC_TRACE(2, 0, 0);
  if (tid == 0) s_aok = tc::mbar_wait(&acc_full, 0u) ? 1 : 0;
  __syncthreads();
  if (tid == 0) GBFIR_TC_TRACE(2, 0, 1);
  const bool have = my_tiles > 0 && s_aok && !s_fail;
  const int sstride = p.NP + 4;
  float *stage = reinterpret_cast<float *>(smem);  // [MT*128][NP + 4] FP32, over the idle ring
  tc::tc_fence_after();
  if (have) {
    // every warp drains: warp w reads TMEM lane quarter w % 4, column chunks w / 4, + 3, ...
    const int quarter = warp & 3, cset = warp >> 2;
    const uint32_t lane_base = (uint32_t)(32 * quarter) << 16;
    for (int mt = 0; mt < p.MT; mt++) {
      float *srow = stage + (size_t)(mt * 128 + 32 * quarter + lane) * sstride;
      for (int col = 16 * cset; col < p.NP; col += 16 * (kTdThreads / 128)) {
        uint32_t r[16], rc[16], rd[16];
        if (p.cat) {
          const uint32_t base = lane_base + (uint32_t)(mt * 3 * p.NP + col);
          tc::tmem_ld16(tmem + base, r);
          tc::tmem_ld16(tmem + base + (uint32_t)p.NP, rc);
          tc::tmem_ld16(tmem + base + 2u * p.NP, rd);
        } else {
          tc::tmem_ld16(tmem + lane_base + (uint32_t)(mt * p.NP + col), r);
          if (split) tc::tmem_ld16(tmem + lane_base + (uint32_t)(acc_cols + mt * p.NP + col), rc);
        }
        tc::tmem_ld_wait();
        if (p.cat) {
#pragma unroll
          for (int q = 0; q < 16; q++)
            r[q] = __float_as_uint(__uint_as_float(r[q]) + (__uint_as_float(rc[q]) + __uint_as_float(rd[q])));
        } else if (split) {
#pragma unroll
          for (int q = 0; q < 16; q++) r[q] = __float_as_uint(__uint_as_float(r[q]) + __uint_as_float(rc[q]));
        }
#pragma unroll
        for (int q = 0; q < 16; q += 4)
          *reinterpret_cast<float4 *>(srow + col + q) = make_float4(
              __uint_as_float(r[q]), __uint_as_float(r[q + 1]), __uint_as_float(r[q + 2]), __uint_as_float(r[q + 3]));
      }
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (tid == 0) GBFIR_TC_TRACE(2, 1, 0);
  // tap t collects dB[k][j] over the phases j = j0, j0 + up, ... (j*down = t - c mod up),
  // k = (c + j*down - t)/up - kmin.  With nsub > 1 threads per tap (few taps), thread sub
  // sums the phases j0 + up*(sub + nsub*m) in increasing m, and the nsub sums are added in
  // sub order: a fixed order either way.  A thread's sum is compensated FP32 (Kahan: the
  // rounding error of each addition carried into the next), as exact as an FP64 sum of these
  // few FP32 terms while staying off the FP64 pipe; the sums are combined in FP64.
  double *part = p.partial + (size_t)blockIdx.x * p.Lo;
  const int mrows = p.MT * 128;
  const int nsub = p.nsub;
  double *fsum = reinterpret_cast<double *>(smem + p.fold_off);  // [Lo][nsub] when nsub > 1
  for (int64_t e = tid; e < p.Lo * nsub; e += kTdThreads) {
    const int64_t tp = e / nsub;
    const int sub = (int)(e - tp * nsub);
    double s = 0.0;
    if (have) {
      int64_t res = (tp - p.c) % p.up;
      if (res < 0) res += p.up;
      const int j0 = (int)((res * p.inv_down) % p.up);
      // along the phases j0, j0 + up, ... the input position k steps by down
      int k = (int)((p.c + j0 * p.down - tp) / p.up - p.kmin) + sub * (int)p.down;
      const int Nti = (int)p.Nt, ustep = (int)p.up * nsub, dstep = (int)p.down * nsub;
      float sf = 0.f, cf = 0.f;
      for (int j = j0 + sub * (int)p.up; j < Nti; j += ustep, k += dstep) {
        if (k >= 0 && k < mrows) {
          const float y = __fsub_rn(stage[(size_t)k * sstride + j], cf);
          const float t = __fadd_rn(sf, y);
          cf = __fsub_rn(__fsub_rn(t, sf), y);
          sf = t;
        }
      }
      s = (double)sf - (double)cf;
    }
    if (nsub == 1) part[tp] = s;
    else fsum[e] = s;
  }
  if (nsub > 1) {
    __syncthreads();
    for (int64_t tp = tid; tp < p.Lo; tp += kTdThreads) {
      double s = fsum[tp * nsub];
      for (int sub = 1; sub < nsub; sub++) s += fsum[tp * nsub + sub];
      part[tp] = s;
    }
  }
  if (tid == 0) GBFIR_TC_TRACE(2, 0, 2);
  if ((s_fail || !s_aok) && tid == 0 && my_tiles > 0) atomicExch(&g_tcd_status, 1);
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc::tc_fence_after();
    tc::tmem_dealloc(tmem, tcols);
  }
}

// Plan of one tap-gradient launch.
struct TdPlan {
  TdParams p;
  size_t smem;
  int64_t grid;
  bool ok;
};

static int64_t td_inverse(int64_t a, int64_t m) {
  if (m == 1) return 0;
  a %= m;
  for (int64_t v = 1; v < m; v++)
    if ((a * v) % m == 1) return v;
  return 0;
}

// Rows of Nt = up*G phases: the G with the least MMA and operand work per output
// ((MT*NP + MT*128 + NP) / Nt), NP = Nt padded to 16 <= 256 and MT*NP <= 256 (two FP32
// accumulators within the 512 TMEM columns; the FP32 staging of dB within the ring).
static TdPlan plan_tc_dh(int64_t up, int64_t down, int64_t Lo, int64_t c, int64_t out_len, int64_t batch,
                         int precision) {
  TdPlan pl{};
  TdParams &p = pl.p;
  p.terms = precision == GBFIR_PREC_BF16X3 ? 3 : 1;
  p.fp16 = precision == GBFIR_PREC_FP16;
  const int64_t kmin = ceil_div(c - Lo + 1, up);
  const size_t budget = 200 * 1024;
  auto slot_bytes = [&](int64_t MT, int64_t NP, int kr) { return ((size_t)MT * 128 + NP) * kr * 2 * p.terms; };
  double best = 0.0;
  int64_t bestG = 0;
  for (int64_t G = 1; up * G <= 256; G++) {
    const int64_t Nt = up * G, NP = (Nt + 15) / 16 * 16;
    const int64_t W = floor_div(c + (Nt - 1) * down, up) - kmin + 1;
    const int64_t MT = (W + 127) / 128;
    if (MT * NP > 256 || 2 * slot_bytes(MT, NP, 16) > budget || (MT * 128 + NP) * 2 > (int64_t)kTdMaxItems * kTdNProd)
      continue;
    const double cost = (double)(MT * NP + MT * 128 + NP) / (double)Nt;
    if (bestG == 0 || cost < best - 1e-9) {
      best = cost;
      bestG = G;
    }
  }
  if (bestG == 0) return pl;
  p.up = up;
  p.down = down;
  p.Lo = Lo;
  p.c = c;
  p.kmin = kmin;
  p.inv_down = td_inverse(down, up);
  p.Nt = up * bestG;
  p.S = down * bestG;
  p.NP = (int32_t)((p.Nt + 15) / 16 * 16);
  p.MT = (int32_t)((floor_div(c + (p.Nt - 1) * down, up) - kmin + 1 + 127) / 128);
  // rows per stage and ring slots: stages of 32 rows in up to four slots (the producers run
  // up to three stages ahead of the MMAs), else 64 or 16 rows in at least two; each producer
  // thread has at most kTdMaxItems items (8-row chunks of an X row or a GY phase) per stage
  auto items = [&](int kr) { return ((int64_t)p.MT * 128 + p.NP) * (kr / 8); };
  // 64-row stages in the 128-byte-swizzled layout where two slots fit (the tensor core reads
  // those operands faster than the no-swizzle ones), else the no-swizzle layout
  p.KR = 0;
  p.sw = 0;
  {
    const int ns = (int)std::min<size_t>(kTdMaxSlots, budget / slot_bytes(p.MT, p.NP, 64));
    if (ns >= 2 && items(64) <= (int64_t)kTdMaxItems * kTdNProd) {
      p.KR = 64;
      p.nslot = ns;
      p.sw = 1;
    }
  }
  for (int kr : {32, 64, 16}) {
    if (p.KR) break;
    const int ns = (int)std::min<size_t>(kTdMaxSlots, budget / slot_bytes(p.MT, p.NP, kr));
    if (ns >= 2 && items(kr) <= (int64_t)kTdMaxItems * kTdNProd) {
      p.KR = kr;
      p.nslot = ns;
      break;
    }
  }
  if (p.KR == 0) return pl;
  p.cat = (p.terms == 3 && 2 * p.NP <= 256 && 3 * p.MT * p.NP <= 512) ? 1 : 0;
  const size_t ring = (size_t)p.nslot * slot_bytes(p.MT, p.NP, p.KR);
  const size_t staging = (size_t)p.MT * 128 * (p.NP + 4) * 4;
  // the fold: up to four threads per tap where taps are few, their FP64 sums after the staging
  p.nsub = Lo >= kTdThreads ? 1 : (int32_t)std::min<int64_t>(4, kTdThreads / Lo);
  p.fold_off = (int32_t)((staging + 15) / 16 * 16);
  const size_t fold = p.nsub > 1 ? (size_t)p.fold_off + (size_t)Lo * p.nsub * 8 : staging;
  pl.smem = 1024 + std::max(ring, fold);
  const int64_t rows = (out_len + p.Nt - 1) / p.Nt;
  p.tiles_per_row = (rows + p.KR - 1) / p.KR;
  p.ntiles = p.tiles_per_row * batch;
  pl.grid = std::max<int64_t>(1, std::min<int64_t>(p.ntiles, num_sms()));
  pl.ok = true;
  return pl;
}

// The per-CTA FP64 partials of dh_e[t] = sum over (n, i) with c + n*down - i*up = t of
// gy[n]*x[i] (extended taps t in [0, Lo)), written to partial[0 .. nparts)[Lo]; returns
// GBFIR_ERR_NOT_SUPPORTED (nothing launched) where no row tile fits.
int tc_dh_partials(const float *x, int64_t x_bstride, int64_t N, const float *gy, int64_t gy_bstride, int64_t out_len,
                   int64_t batch, int64_t up, int64_t down, int64_t Lo, int64_t c, int precision, double *partial,
                   size_t partial_bytes, int64_t *nparts, cudaStream_t s) {
  TdPlan pl = plan_tc_dh(up, down, Lo, c, out_len, batch, precision);
  if (!pl.ok) return GBFIR_ERR_NOT_SUPPORTED;
  TdParams &p = pl.p;
  p.x = x;
  p.x_bstride = batch > 1 ? x_bstride : 0;
  p.N = N;
  p.gy = gy;
  p.gy_bstride = batch > 1 ? gy_bstride : 0;
  p.out_len = out_len;
  p.partial = partial;
  if ((size_t)pl.grid * Lo * sizeof(double) > partial_bytes)
    GBFIR_FAIL(GBFIR_ERR_WORKSPACE, "backward dh (tensor cores): needs %zu B of workspace, got %zu",
               (size_t)pl.grid * Lo * sizeof(double), partial_bytes);
  int rc = ensure_smem((const void *)tc_dh_kernel, pl.smem, "backward dh (tensor cores)");
  if (rc) return rc;
  tc_dh_kernel<<<(unsigned)pl.grid, kTdThreads, pl.smem, s>>>(p);
  rc = check_launch("backward dh (tensor cores)");
  if (rc) return rc;
  *nparts = pl.grid;
  return GBFIR_SUCCESS;
}

}  // namespace gbfir
