// tc_resample.cu — resample_poly as Toeplitz MMAs on the tcgen05 tensor cores
// (bf16, fp16 and bf16x3 split precision, FP32 accumulate in TMEM).  No MatX counterpart.
//
// Math.  With gcd-reduced rates, y[n] = up * sum_i x[i] * he[c + n*down - i*up].
// The kernel groups outputs into rows whose inputs advance by exactly R samples (the row
// pitch, 8 or 64) of a linear array xs, so that the Hankel operand A[q][k] = xs[R*q + k]
// is a K-major shared-memory matrix with overlapping rows and no Hankel matrix is ever
// materialised:
//   R = 8:  no-swizzle layout; the 8-row x 16-byte core matrices are 16 bytes apart along
//           K (LBO = 16) and 128 bytes apart along rows (SBO = 128).
//   R = 64: 128-byte-swizzled layout; an operand row is 64 bf16 = 128 bytes, so xs stored
//           linearly with the swizzle applied at its (1024-aligned) addresses is exactly
//           A with rows 128 bytes apart (SBO = 1024 per 8-row group), K-step s starting
//           32*s bytes in.  Rows of 64 inputs give N = 64*up/down MMA columns instead of
//           8*up/down, so each MMA does eight times the work for the same issue cost.
//   path A (down divides R): xs[u] = x[u + k0]; a row holds Nt = R*up/down outputs and
//     D[q][j] = sum_k xs[R*q + k] * W[j][k],  W[j][k] = up*he[c + j*down - (k + k0)*up].
//   path B (other down): x is split into its `down` polyphase components
//     xs_b[a] = x[down*a + b]; each is an interpolator (rate up) and a row holds
//     Nt = R*up outputs:  D[q][j] = sum_b sum_k xs_b[R*q + k + k0] * W_b[j][k],
//     W_b[j][k] = up*he[c + down*j - up*(b + down*(k + k0))].
// The tap matrices W (N = Nt rounded up to 16 columns, Kp = band rounded to 16) are
// built once per CTA.  Complex x runs as two M = 128 MMAs (real, imaginary rows) on the
// same W.  bf16x3 splits both operands into three bf16 terms and accumulates the six
// products of order <= 2 (smallest first) — 24 significant bits, FP32-class accuracy.
//
// bf16x3 with 3*N <= 256 concatenates the three tap terms along N (W_cat = [b0 | b1 | b2])
// so one K-step is three MMAs — a0*[b0|b1|b2] into D[0:3N), a1*[b0|b1] into D[N:3N), a2*b0
// into D[2N:3N) — and the epilogue sums the three column blocks: exactly the six products
// of order <= 2, with the small terms accumulated apart from a0*b0.  Wider rows issue the
// six products as six MMAs of N columns: into one accumulator for bands of up to 8 K-steps,
// else a0*b0 into one and the five smaller products into a second (every MMA instruction
// costs the accumulator about one FP32 rounding, so long bands keep the big sum's count low).
//
// Pipeline (persistent, warp-specialised CTA; roles below).  A stage covers MT M-tiles
// of 128 rows; raw input is staged two stages ahead with cp.async, converted into a
// two-slot operand ring, multiplied into one of two TMEM accumulator sets and drained
// by the epilogue warps while the next stage's MMAs run.
#include <cstdlib>
#include <cstring>

#include "rowtile.cuh"
#include "tc.cuh"

namespace gbfir {


struct TcParams {
  const void *x;
  int64_t x_bstride, N;
  const float *h;
  int64_t Lo, c;
  int32_t even, rev;
  void *out;
  int64_t out_bstride, out_len;
  int64_t up, down;
  int32_t path;     // 0: A, 1: B
  int32_t P;        // arrays per term (1 or down)
  int32_t Nt, Nmma; // useful outputs per row, MMA N
  int32_t Kp;       // K band (multiple of 16)
  int64_t k0;       // aligned band start (multiple of 8)
  int32_t MT;       // M-tiles (128 rows) per iteration
  int32_t LA;       // elements per xs array per buffer = rp*128*MT + Kp
  int32_t terms;    // 1 or 3
  int32_t fp16;     // 1: fp16 operands (single term), 0: bf16
  int64_t rows;     // rows per signal row = ceil(out_len / Nt)
  int64_t iters_per_row, niters;
  double scale;     // up
  int32_t tmem_cols;
  int32_t nbuf;     // operand ring slots (1 or 2)
  int32_t nsets;    // TMEM accumulator sets (1 or 2)
  int32_t nraw;     // raw staging slots: 2 = stage two iterations ahead, 1 = one ahead
  int32_t rp;       // Hankel row pitch in samples: 8 (no swizzle) or 64 (128-byte swizzle)
  int32_t concat;   // bf16x3: 1 = tap terms concatenated along N, 0 = six MMAs of N columns
  int32_t split;    // bf16x3 without concat: 1 = a0*b0 and the five smaller products in two
                    // accumulators (long K bands), 0 = all six in one
  int32_t acols;    // TMEM accumulator columns per (M-tile, part): 3*Nmma (concat), 2*Nmma
                    // (split) or Nmma
};

// Bounded-wait status of the tensor-core kernels (1 = a wait gave up); read and
// cleared by gbfir_tc_status().
__device__ int32_t g_tc_status;

// Two floats as an fp16 pair (round to nearest), low half first.
__device__ __forceinline__ uint32_t tw_pack_h2(float a, float b) {
  const __half2 h = __floats2half2_rn(a, b);
  return *reinterpret_cast<const uint32_t *>(&h);
}

// Timing hooks of the pipeline roles (role, stage, event); they compile to nothing unless a
// tracing build defines them.
#ifndef GBFIR_TC_TRACE
#define GBFIR_TC_TRACE(role, stage, event) \
  do {                                     \
  } while (0)
#endif

// Warp roles (12 warps): warp 0 lane 0 issues the MMAs; warps 1-7 stage raw input with
// cp.async and convert it into the operand ring; warps 8-11 (one per TMEM lane quarter)
// drain finished accumulators.  Handoffs use mbarriers: op_full / op_empty per operand
// slot, tm_full / tm_empty per TMEM accumulator set.  Every wait is bounded.
constexpr int kWsThreads = 384;
constexpr int kProdWarp0 = 1, kProdWarps = 7, kEpiWarp0 = 8;
constexpr int kNProd = kProdWarps * 32;

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(tc::smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void named_sync(int id, int nthreads) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

// Epilogue of one 16-lane half of a warp's TMEM lane quarter (tb: its TMEM address, columns of
// one M-tile).  16x256b loads: for TMEM lanes l0 + L/4 and l0 + L/4 + 8, lane L holds columns
// c and c + 1 of each 8-column group, c = 2 * (L % 4); so four lanes hold 8 consecutive outputs
// of one row and each store instruction writes 32 (real) or 64 (complex) contiguous bytes of
// 8 rows: whole sectors.  GCH 32-column chunks (16x256b.x4 loads of every part and of the BLK
// concatenated term blocks) go per TMEM wait, up to 64 registers; 8-column groups for a
// remainder.  qa: the signal row of lane L's first TMEM lane.
template <bool XC, int BLK>
__device__ __forceinline__ void tcr_drain_half(const TcParams &p, uint32_t tb,
                                               typename val_of<float, XC>::type *orow, int64_t qa, int lane) {
  using XT = typename val_of<float, XC>::type;
  constexpr int NPARTS = XC ? 2 : 1;
  constexpr int GCH = (64 / (16 * NPARTS * BLK)) > 0 ? 64 / (16 * NPARTS * BLK) : 1;
  auto valid = [&](int64_t n0) -> int {
    const int64_t left = p.out_len - n0;
    return left < p.Nt ? (left > 0 ? (int)left : 0) : p.Nt;
  };
  const int64_t na = qa * p.Nt, nb = (qa + 8) * p.Nt;
  const int nva = valid(na), nvb = valid(nb);
  XT *da = orow + na, *db = orow + nb;
  // c is even, so a pair of outputs is one vector store wherever the row start is aligned to
  // the pair (8 bytes real, 16 bytes complex)
  constexpr uintptr_t kPairAlign = XC ? 15 : 7;
  const bool ala = (reinterpret_cast<uintptr_t>(da) & kPairAlign) == 0;
  const bool alb = (reinterpret_cast<uintptr_t>(db) & kPairAlign) == 0;
  auto put = [&](XT *d, int nv, bool al, int c, const float (&w)[NPARTS][2]) {
    if (al && c + 1 < nv) {
      if constexpr (XC) *reinterpret_cast<float4 *>(d + c) = make_float4(w[0][0], w[1][0], w[0][1], w[1][1]);
      else *reinterpret_cast<float2 *>(d + c) = make_float2(w[0][0], w[0][1]);
    } else {
      if constexpr (XC) {
        if (c < nv) d[c] = make_float2(w[0][0], w[1][0]);
        if (c + 1 < nv) d[c + 1] = make_float2(w[0][1], w[1][1]);
      } else {
        if (c < nv) d[c] = w[0][0];
        if (c + 1 < nv) d[c + 1] = w[0][1];
      }
    }
  };
  const int nfull = p.Nmma / 32;
  for (int c0 = 0; c0 < nfull; c0 += GCH) {
    uint32_t rb[GCH][NPARTS][BLK][16];
#pragma unroll
    for (int g = 0; g < GCH; g++) {
      if (c0 + g >= nfull) break;
#pragma unroll
      for (int part = 0; part < NPARTS; part++)
#pragma unroll
        for (int bk = 0; bk < BLK; bk++)
          tc::tmem_ld_16x256b_x4(tb + (uint32_t)(part * p.acols + bk * p.Nmma + 32 * (c0 + g)), rb[g][part][bk]);
    }
    tc::tmem_ld_wait();
#pragma unroll
    for (int g = 0; g < GCH; g++) {
      if (c0 + g >= nfull) break;
#pragma unroll
      for (int grp = 0; grp < 4; grp++) {
        float va[NPARTS][2], vb[NPARTS][2];
#pragma unroll
        for (int part = 0; part < NPARTS; part++) {
          float v[4];
#pragma unroll
          for (int i = 0; i < 4; i++) {
            const int r = 4 * grp + i;
            if constexpr (BLK == 3)
              v[i] = __uint_as_float(rb[g][part][0][r]) +
                     (__uint_as_float(rb[g][part][1][r]) + __uint_as_float(rb[g][part][2][r]));
            else if constexpr (BLK == 2)
              v[i] = __uint_as_float(rb[g][part][0][r]) + __uint_as_float(rb[g][part][1][r]);
            else
              v[i] = __uint_as_float(rb[g][part][0][r]);
          }
          va[part][0] = v[0];
          va[part][1] = v[1];
          vb[part][0] = v[2];
          vb[part][1] = v[3];
        }
        const int c = 32 * (c0 + g) + 8 * grp + 2 * (lane & 3);
        put(da, nva, ala, c, va);
        put(db, nvb, alb, c, vb);
      }
    }
  }
  for (int cg = 32 * nfull; cg < p.Nmma; cg += 8) {
    float va[NPARTS][2], vb[NPARTS][2];
    uint32_t r[NPARTS][BLK][4];
#pragma unroll
    for (int part = 0; part < NPARTS; part++)
#pragma unroll
      for (int bk = 0; bk < BLK; bk++)
        tc::tmem_ld_16x256b(tb + (uint32_t)(part * p.acols + bk * p.Nmma + cg), r[part][bk]);
    tc::tmem_ld_wait();
#pragma unroll
    for (int part = 0; part < NPARTS; part++) {
      float v[4];
#pragma unroll
      for (int i = 0; i < 4; i++) {
        if constexpr (BLK == 3)
          v[i] = __uint_as_float(r[part][0][i]) + (__uint_as_float(r[part][1][i]) + __uint_as_float(r[part][2][i]));
        else if constexpr (BLK == 2)
          v[i] = __uint_as_float(r[part][0][i]) + __uint_as_float(r[part][1][i]);
        else
          v[i] = __uint_as_float(r[part][0][i]);
      }
      va[part][0] = v[0];
      va[part][1] = v[1];
      vb[part][0] = v[2];
      vb[part][1] = v[3];
    }
    const int c = cg + 2 * (lane & 3);
    put(da, nva, ala, c, va);
    put(db, nvb, alb, c, vb);
  }
}

template <bool XC>
__global__ void __launch_bounds__(kWsThreads, 1) tc_resample_kernel(const TcParams p) {
  using XT = typename val_of<float, XC>::type;
  constexpr int NPARTS = XC ? 2 : 1;  // real / imaginary operand rows
  extern __shared__ __align__(1024) unsigned char smem_dyn[];
  __shared__ uint64_t op_full[2], op_empty[2], tm_full[2], tm_empty[2], raw_full[2];
  __shared__ uint32_t tmem_slot;
  __shared__ int s_fail, s_pok, s_eok;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) GBFIR_TC_TRACE(3, 0, 1);

  // shared layout (1024-aligned; the 128-byte swizzle pattern follows address bits 4-9):
  // W_cat [P][terms*Nmma rows][Kp] ; operand ring [nbuf][NPARTS][terms][P][LA] ; raw ring
  // [nraw][P*LA]
  unsigned char *smem = smem_dyn + ((1024u - (tc::smem_u32(smem_dyn) & 1023u)) & 1023u);
  const int wrows = p.terms * p.Nmma;
  const uint32_t wbytes = (uint32_t)wrows * p.Kp * 2u;
  unsigned char *wbase = smem;
  unsigned char *xbase = smem + ((size_t)p.P * wbytes + 1023) / 1024 * 1024;
  const size_t xalign = p.rp == 64 ? 1024 : 128;
  const size_t xarr = ((size_t)p.LA * 2 + xalign - 1) / xalign * xalign;
  auto warr = [&](int pp) { return wbase + (size_t)pp * wbytes; };
  auto xarrp = [&](int slot, int part, int t, int pp) {
    return xbase + ((((size_t)slot * NPARTS + part) * p.terms + t) * p.P + pp) * xarr;
  };
  const size_t raw_elems = (size_t)p.P * p.LA;
  XT *raw0 = reinterpret_cast<XT *>(xbase + (size_t)p.nbuf * NPARTS * p.terms * p.P * xarr);
  auto rawp = [&](int slot) { return raw0 + (size_t)slot * raw_elems; };

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
  __syncthreads();  // the barriers are initialised
  const XT *xp = reinterpret_cast<const XT *>(p.x);
  const int ptid = tid - kProdWarp0 * 32;
  const bool producer = warp >= kProdWarp0 && warp < kProdWarp0 + kProdWarps;
  // An iteration's raw window (one contiguous run of P*LA samples of the signal from base)
  // comes in with TMA bulk copies completing on raw_full[slot] when it lies inside the
  // signal with a 16-byte aligned start; other windows (at the row ends) are staged with
  // plain loads, zeros outside the signal.  Windows are staged nraw iterations ahead; the
  // first ones are in flight while the tap matrices are built.
  auto fetch = [&](int64_t itx, int slot) {
    const int64_t b = itx / p.iters_per_row;
    const int64_t q0 = (itx - b * p.iters_per_row) * (int64_t)(128 * p.MT);
    const XT *row = xp + b * p.x_bstride;
    const int64_t base = p.path == 0 ? p.rp * q0 + p.k0 : p.down * (p.rp * q0 + p.k0);
    XT *dst = rawp(slot);
    const size_t bytes = raw_elems * sizeof(XT);
    const bool bulk = ((reinterpret_cast<uintptr_t>(row + base) | (uintptr_t)tc::smem_u32(dst)) & 15) == 0 &&
                      base >= 0 && base + (int64_t)raw_elems <= p.N && bytes % 16 == 0 && bytes < (1u << 20);
    if (bulk) {
      // four bulk copies (16-byte multiples) from four lanes, so the pieces are in flight
      // together; the transaction count is set before any of them is issued
      if (ptid < 32) {
        if (ptid == 0) {
          tc::fence_async_smem();
          tc::mbar_arrive_expect_tx(&raw_full[slot], (uint32_t)bytes);
        }
        __syncwarp();
        const uint32_t piece = (uint32_t)(((bytes / 4) + 15) & ~(size_t)15);
        const uint32_t off = (uint32_t)ptid * piece;
        if (ptid < 4 && off < bytes) {
          const uint32_t nb = (uint32_t)std::min<size_t>(piece, bytes - off);
          tc::bulk_copy_g2s(reinterpret_cast<unsigned char *>(dst) + off,
                            reinterpret_cast<const unsigned char *>(row + base) + off, nb, &raw_full[slot]);
        }
      }
    } else {
#pragma unroll 4
      for (int v = ptid; v < (int)raw_elems; v += kNProd) {
        const int64_t gi = base + v;
        dst[v] = (gi >= 0 && gi < p.N) ? __ldg(row + gi) : zero_val<XT>();
      }
      named_sync(1, kNProd);
      if (ptid == 0) tc::mbar_arrive_plain(&raw_full[slot]);
    }
  };
  const int nraw = p.nraw;
  const int64_t my_iters = p.niters > blockIdx.x ? (p.niters - 1 - blockIdx.x) / gridDim.x + 1 : 0;
  if (producer) {
    if (my_iters > 0) fetch(blockIdx.x, 0);
    if (nraw == 2 && my_iters > 1) fetch(blockIdx.x + gridDim.x, 1);
  }
  // The filter's taps, scaled and split into the operand terms once (hterm[t][e] = term t
  // of scale * h[e], 16-bit), staged in the operand ring (not in use yet), so that the W
  // build gathers 8 taps per 16-byte store instead of splitting every element.
  const int64_t Lh = p.Lo - p.even;
  const size_t scratch_bytes = (size_t)p.nbuf * NPARTS * p.terms * p.P * xarr;
  const bool h_staged = (size_t)Lh * 2 * p.terms <= scratch_bytes;
  uint16_t *hterm = reinterpret_cast<uint16_t *>(xbase);
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
    for (int64_t e = tid; e < Lh; e += kWsThreads) {
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
  // ---- W_cat[pp][t*Nmma + j][k] = term t of up*he[tap(j, k)] (K-major core layout) ----
  // Every tap position a W element reads lies in [tp_lo, tp_hi]; zline[t][tp - tp_lo] holds
  // its term t (0 outside the filter), so each element is one branch-free shared load.  An
  // item is one 8-wide K chunk of one row (one 16-byte store); along a chunk the tap position
  // steps by -up (path A) or -up*down (path B).
  if (tid == 0) GBFIR_TC_TRACE(3, 1, 0);
  const int kch = p.Kp / 8;
  const int64_t dtp = p.path == 0 ? -p.up : -p.up * p.down;
  const int64_t kk_hi = p.k0 + p.Kp - 1;
  const int64_t tp_lo = p.path == 0 ? p.c - kk_hi * p.up : p.c - p.up * ((p.P - 1) + p.down * kk_hi);
  const int64_t tp_hi = p.path == 0 ? p.c + (int64_t)(p.Nt - 1) * p.down - p.k0 * p.up
                                    : p.c + p.down * (int64_t)(p.Nt - 1) - p.up * p.down * p.k0;
  const int64_t zlen = tp_hi - tp_lo + 1;
  uint16_t *zline = hterm + (h_staged ? (size_t)p.terms * Lh : 0);
  const bool z_staged = h_staged && zlen > 0 && ((size_t)p.terms * Lh + (size_t)p.terms * zlen) * 2 <= scratch_bytes;
  if (z_staged) {
    for (int64_t i = tid; i < p.terms * zlen; i += kWsThreads) {
      const int t = (int)(i / zlen);
      zline[i] = (uint16_t)w_term(t, tp_lo + (i - (int64_t)t * zlen));
    }
  }
  __syncthreads();
  if (tid == 0) GBFIR_TC_TRACE(3, 2, 0);
  // A thread owns one row of W and every tpr-th of its 8-wide K chunks (consecutive lanes take
  // consecutive rows of one chunk, so their 16-byte stores fill whole 128-byte core matrices:
  // conflict-free); the row's constants are derived once, and along the row the tap position
  // steps by 8*dtp per chunk (32-bit: every position lies within a few Kp*up of the filter).
  // A chunk whose tap range misses the filter is stored as zeros without gathers.
  const int nrows_w = p.P * wrows;
  const int tpr = kWsThreads >= nrows_w ? kWsThreads / nrows_w : 1;  // threads per row
  const int dt = (int)dtp;
  for (int sl = tid; sl < nrows_w * tpr; sl += kWsThreads) {
    const int rr = sl % nrows_w, kc0 = sl / nrows_w;
    const int pp = rr / wrows, row = rr - pp * wrows;
    const int t = row / p.Nmma, j = row - t * p.Nmma;
    unsigned char *wrow = warr(pp);
    const bool live = j < p.Nt;
    // tap position of chunk 0's first element
    const int tpj = (int)(p.path == 0 ? p.c + (int64_t)j * p.down - p.k0 * p.up
                                      : p.c + p.down * (int64_t)j - p.up * (pp + p.down * p.k0));
    const uint16_t *zt0 = zline + (size_t)t * zlen;
    const int ztl = (int)tp_lo;
    const int Lo = (int)p.Lo;
    for (int kc = kc0; kc < kch; kc += tpr) {
      uint32_t w[4] = {0u, 0u, 0u, 0u};
      const int tp0 = tpj + 8 * kc * dt;
      const int tp7 = tp0 + 7 * dt;  // dt < 0: the chunk reads taps tp7..tp0
      if (live && tp0 >= 0 && tp7 < Lo) {
        if (z_staged) {
          const uint16_t *zt = zt0 + (tp0 - ztl);
#pragma unroll
          for (int e = 0; e < 8; e++) w[e >> 1] |= (uint32_t)zt[e * dt] << (16 * (e & 1));
        } else {
#pragma unroll
          for (int e = 0; e < 8; e++) w[e >> 1] |= w_term(t, tp0 + e * dt) << (16 * (e & 1));
        }
      }
      *reinterpret_cast<uint4 *>(wrow + tc::kmajor_offset(row, 8 * kc, p.Kp)) = make_uint4(w[0], w[1], w[2], w[3]);
    }
  }
  if (tid == 0) GBFIR_TC_TRACE(3, 3, 0);
  tc::fence_async_smem();
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = tmem_slot;
  if (tid == 0) GBFIR_TC_TRACE(3, 0, 0);
  const uint32_t set_cols = (uint32_t)(p.MT * NPARTS * p.acols);

  if (producer) {
    // ================= producers =================
    const int nslots = p.nbuf;
    const uint32_t swz = p.rp == 64 ? 7u : 0u;
    const int half = p.LA / 2;
    for (int64_t k = 0; k < my_iters; ++k) {
      const int slot = (int)(k % nslots);
      if (ptid == 0) GBFIR_TC_TRACE(0, (int)k, 0);
      const int rslot = nraw == 2 ? (int)(k & 1) : 0;
      // one thread waits for the raw window and the operand slot; the named barrier publishes
      // its verdict to all producers, so the role leaves the loop together
      if (ptid == 0) {
        bool ok = tc::mbar_wait(&raw_full[rslot], (uint32_t)((k / nraw) & 1));
        if (ok && k >= nslots) ok = tc::mbar_wait(&op_empty[slot], (uint32_t)(((k - nslots) / nslots) & 1));
        s_pok = ok ? 1 : 0;
      }
      named_sync(1, kNProd);
      if (ptid == 0) GBFIR_TC_TRACE(0, (int)k, 1);
      if (!s_pok) {
        s_fail = 1;
        // windows still in flight land before the CTA's shared memory goes away
        if (ptid == 0)
          for (int64_t j = k; j < my_iters && j < k + nraw; j++)
            (void)tc::mbar_wait(&raw_full[nraw == 2 ? (int)(j & 1) : 0], (uint32_t)((j / nraw) & 1));
        break;
      }
      // convert raw slot -> operand slot.  One component (P == 1): eight consecutive samples
      // per item, 16-byte shared loads and one 16-byte store per term and part (with 64-sample
      // rows the 16-byte chunk at byte o goes to o ^ ((o >> 7) & 7) << 4 of the 128-byte
      // swizzle; a quarter warp writes one 128-byte row, conflict-free).  Polyphase
      // components (P > 1): pairs of samples of one component per item.
      const XT *src = rawp(rslot);
      if (p.P == 1) {
        unsigned char *dst[NPARTS][3];
#pragma unroll
        for (int part = 0; part < NPARTS; part++)
#pragma unroll
          for (int t = 0; t < 3; t++) dst[part][t] = xarrp(slot, part, t < p.terms ? t : 0, 0);
        const int n8 = p.LA / 8;
        for (int u = ptid; u < n8; u += kNProd) {
          float vr[8], vi[8];
          if constexpr (XC) {
            const float4 *s4 = reinterpret_cast<const float4 *>(src + 8 * u);
#pragma unroll
            for (int q = 0; q < 4; q++) {
              const float4 w = s4[q];
              vr[2 * q] = w.x;
              vi[2 * q] = w.y;
              vr[2 * q + 1] = w.z;
              vi[2 * q + 1] = w.w;
            }
          } else {
            const float4 *s4 = reinterpret_cast<const float4 *>(src + 8 * u);
            const float4 w0 = s4[0], w1 = s4[1];
            vr[0] = w0.x; vr[1] = w0.y; vr[2] = w0.z; vr[3] = w0.w;
            vr[4] = w1.x; vr[5] = w1.y; vr[6] = w1.z; vr[7] = w1.w;
          }
          const uint32_t o = 16u * (uint32_t)u;
          const uint32_t po = o ^ (((o >> 7) & swz) << 4);
#pragma unroll
          for (int part = 0; part < NPARTS; part++) {
            const float *v = part == 0 ? vr : vi;
            if (p.fp16) {
              uint4 h4;
              h4.x = tw_pack_h2(v[0], v[1]);
              h4.y = tw_pack_h2(v[2], v[3]);
              h4.z = tw_pack_h2(v[4], v[5]);
              h4.w = tw_pack_h2(v[6], v[7]);
              *reinterpret_cast<uint4 *>(dst[part][0] + po) = h4;
            } else {
              uint32_t w0[4], w1[4], w2[4];
#pragma unroll
              for (int q = 0; q < 4; q++) {
                __nv_bfloat162 t0, t1, t2;
                tc::split3_bf16x2(make_float2(v[2 * q], v[2 * q + 1]), t0, t1, t2);
                w0[q] = *reinterpret_cast<uint32_t *>(&t0);
                w1[q] = *reinterpret_cast<uint32_t *>(&t1);
                w2[q] = *reinterpret_cast<uint32_t *>(&t2);
              }
              *reinterpret_cast<uint4 *>(dst[part][0] + po) = make_uint4(w0[0], w0[1], w0[2], w0[3]);
              if (p.terms == 3) {
                *reinterpret_cast<uint4 *>(dst[part][1] + po) = make_uint4(w1[0], w1[1], w1[2], w1[3]);
                *reinterpret_cast<uint4 *>(dst[part][2] + po) = make_uint4(w2[0], w2[1], w2[2], w2[3]);
              }
            }
          }
        }
      } else {
        for (int pp = 0; pp < p.P; pp++) {
          unsigned char *dst[NPARTS][3];
#pragma unroll
          for (int part = 0; part < NPARTS; part++)
#pragma unroll
            for (int t = 0; t < 3; t++) dst[part][t] = xarrp(slot, part, t < p.terms ? t : 0, pp);
          for (int v = ptid; v < half; v += kNProd) {
            const int u = 2 * v;
            const XT a0 = src[(size_t)u * p.P + pp], a1 = src[(size_t)(u + 1) * p.P + pp];
            const uint32_t o = 4u * (uint32_t)v;
            const uint32_t po = o ^ (((o >> 7) & swz) << 4);
#pragma unroll
            for (int part = 0; part < NPARTS; part++) {
              const float2 f = part == 0 ? make_float2(re_of(a0), re_of(a1)) : make_float2(im_of(a0), im_of(a1));
              if (p.fp16) {
                *reinterpret_cast<uint32_t *>(dst[part][0] + po) = tw_pack_h2(f.x, f.y);
              } else {
                __nv_bfloat162 t0, t1, t2;
                tc::split3_bf16x2(f, t0, t1, t2);
                *reinterpret_cast<__nv_bfloat162 *>(dst[part][0] + po) = t0;
                if (p.terms == 3) {
                  *reinterpret_cast<__nv_bfloat162 *>(dst[part][1] + po) = t1;
                  *reinterpret_cast<__nv_bfloat162 *>(dst[part][2] + po) = t2;
                }
              }
            }
          }
        }
      }
      tc::fence_async_smem();
      named_sync(1, kNProd);
      if (ptid == 0) mbar_arrive(&op_full[slot]);
      if (ptid == 0) GBFIR_TC_TRACE(0, (int)k, 2);
      // the raw slot is consumed (every producer passed the barrier): stage iteration
      // k + nraw into it
      if (k + nraw < my_iters) fetch(blockIdx.x + (k + nraw) * (int64_t)gridDim.x, rslot);
    }
  } else if (warp == 0) {
    // ================= MMA issuer =================
    // every TMEM column the MMAs touch lies inside the allocation (checked once)
    const bool geom_ok = (p.rp == 8 || p.rp == 64) && p.Nmma % 16 == 0 && p.Nmma <= 256 &&
                         (!p.concat || 3 * p.Nmma <= 256) && p.Kp % 16 == 0 &&
                         (uint32_t)p.nsets * set_cols <= (uint32_t)p.tmem_cols;
    if (lane == 0 && !geom_ok) s_fail = 1;
    if (lane == 0 && geom_ok) {
      const uint32_t idesc3 = tc::idesc_f16(128, (uint32_t)(3 * p.Nmma), 1u);
      const uint32_t idesc2 = tc::idesc_f16(128, (uint32_t)(2 * p.Nmma), 1u);
      const uint32_t idesc1 = tc::idesc_f16(128, (uint32_t)p.Nmma, p.fp16 ? 0u : 1u);
      const uint32_t wsbo = (uint32_t)(p.Kp / 8) * 128u;
      const int nks = p.Kp / 16;
      // descriptor fields that never change; only the 14-bit start address (bytes >> 4) moves.
      // 64-sample rows: 128-byte swizzle (layout type 2), 8-row groups 1024 bytes apart, base
      // offset 0 (the swizzle follows the absolute address, so starts inside a row are exact)
      const uint64_t afix = p.rp == 64 ? (tc::smem_desc(0u, 16u, 1024u) | ((uint64_t)2 << 61))
                                       : tc::smem_desc(0u, 16u, 128u);
      const uint64_t bfix = tc::smem_desc(0u, 128u, wsbo);
      const uint32_t xs0 = tc::smem_u32(xbase), w0 = tc::smem_u32(wbase);
      const uint32_t mtile_bytes = (uint32_t)p.rp * 128u * 2u;    // one M-tile of 128 rows
      const uint64_t term_step = (uint64_t)p.Nmma * p.Kp / 8;      // W term block, in 16-byte units
      int64_t it = blockIdx.x;
      for (int k = 0; it < p.niters; it += gridDim.x, ++k) {
        const int slot = k % p.nbuf, tset = k % p.nsets;
        GBFIR_TC_TRACE(1, k, 0);
        if (!tc::mbar_wait(&op_full[slot], (k / p.nbuf) & 1)) { s_fail = 1; break; }
        if (k >= p.nsets && !tc::mbar_wait(&tm_empty[tset], ((k - p.nsets) / p.nsets) & 1)) { s_fail = 1; break; }
        GBFIR_TC_TRACE(1, k, 1);
        tc::tc_fence_after();
        const uint32_t dset = tmem + (uint32_t)tset * set_cols;
        // Issue order (measured): with three terms, accumulator-major — per (M-tile, part)
        // the K-steps, each step's a0*[b0|b1|b2], a1*[b0|b1], a2*b0 back to back; with one
        // term, step-major — consecutive MMAs write different accumulators.
        const int nacc = p.MT * NPARTS;
        auto a_desc = [&](int a, int t, int pp, int ks) -> uint64_t {
          const int m = a / NPARTS, part = a - m * NPARTS;
          const uint32_t aaddr = xs0 + (uint32_t)((((slot * NPARTS + part) * p.terms + t) * p.P + pp) * xarr) +
                                 mtile_bytes * (uint32_t)m;
          return (afix | (uint64_t)(aaddr >> 4)) + (uint64_t)(2 * ks);
        };
        if (p.terms == 3 && p.concat) {
          for (int a = 0; a < nacc; a++) {
            const uint32_t d = dset + (uint32_t)(a * p.acols);
            for (int pp = 0; pp < p.P; pp++) {
              const uint64_t bd0 = bfix | (uint64_t)((w0 + (uint32_t)pp * wbytes) >> 4);
              for (int ks = 0; ks < nks; ks++) {
                const uint64_t bd = bd0 + (uint64_t)(16 * ks);
                // D[0:3N) (+)= a0 * [b0|b1|b2];  D[N:3N) += a1 * [b0|b1];  D[2N:3N) += a2 * b0
                tc::mma_f16(d, a_desc(a, 0, pp, ks), bd, idesc3, (pp > 0 || ks > 0) ? 1u : 0u);
                tc::mma_f16(d + (uint32_t)p.Nmma, a_desc(a, 1, pp, ks), bd, idesc2, 1u);
                tc::mma_f16(d + (uint32_t)(2 * p.Nmma), a_desc(a, 2, pp, ks), bd, idesc1, 1u);
              }
            }
          }
        } else if (p.terms == 3) {
          // six MMAs of N columns per K-step, products of order <= 2 (signal term tx, tap
          // term tw), smallest first: (1,1) (2,0) (0,2) (1,0) (0,1) (0,0); split: the last,
          // a0*b0, into the first N columns and the other five into the next N
          constexpr uint32_t kTx = 0x001021u, kTw = 0x010201u;
          for (int a = 0; a < nacc; a++) {
            const uint32_t d = dset + (uint32_t)(a * p.acols);
            for (int pp = 0; pp < p.P; pp++) {
              const uint64_t bd0 = bfix | (uint64_t)((w0 + (uint32_t)pp * wbytes) >> 4);
              for (int ks = 0; ks < nks; ks++) {
                for (int pr = 0; pr < 6; pr++) {
                  const int tx = (int)((kTx >> (4 * pr)) & 15u), tw = (int)((kTw >> (4 * pr)) & 15u);
                  const uint64_t bd = bd0 + (uint64_t)tw * term_step + (uint64_t)(16 * ks);
                  const bool small = p.split && pr < 5;
                  const bool first = p.split ? (pr == 0 || pr == 5) : pr == 0;
                  tc::mma_f16(d + (small ? (uint32_t)p.Nmma : 0u), a_desc(a, tx, pp, ks), bd, idesc1,
                              (pp > 0 || ks > 0 || !first) ? 1u : 0u);
                }
              }
            }
          }
        } else {
          for (int pp = 0; pp < p.P; pp++) {
            const uint64_t bd0 = bfix | (uint64_t)((w0 + (uint32_t)pp * wbytes) >> 4);
            for (int ks = 0; ks < nks; ks++) {
              const uint64_t bd = bd0 + (uint64_t)(16 * ks);
              for (int a = 0; a < nacc; a++)
                tc::mma_f16(dset + (uint32_t)(a * p.acols), a_desc(a, 0, pp, ks), bd, idesc1,
                            (pp > 0 || ks > 0) ? 1u : 0u);
            }
          }
        }
        tc::mma_commit(&op_empty[slot]);
        GBFIR_TC_TRACE(1, k, 2);
        tc::mma_commit(&tm_full[tset]);
      }
    }
  } else {
    // ================= epilogue (warps 8-11: TMEM lane quarters 0-3) =================
    const int quarter = warp - kEpiWarp0;
    int64_t it = blockIdx.x;
    for (int k = 0; it < p.niters; it += gridDim.x, ++k) {
      const int slot = k % p.nsets;
      if (quarter == 0 && lane == 0) GBFIR_TC_TRACE(2, k, 0);
      if (quarter == 0 && lane == 0) s_eok = tc::mbar_wait(&tm_full[slot], (k / p.nsets) & 1) ? 1 : 0;
      named_sync(2, 128);
      if (quarter == 0 && lane == 0) GBFIR_TC_TRACE(2, k, 1);
      if (!s_eok) {
        s_fail = 1;
        break;
      }
      tc::tc_fence_after();
      const uint32_t dset = tmem + (uint32_t)slot * set_cols;
      const int64_t b = it / p.iters_per_row;
      const int64_t q0 = (it - b * p.iters_per_row) * (int64_t)(128 * p.MT);
      XT *orow = reinterpret_cast<XT *>(p.out) + b * p.out_bstride;
      const bool blocks3 = p.terms == 3 && p.concat, blocks2 = p.terms == 3 && p.split;
      for (int m = 0; m < p.MT; m++) {
        for (int half = 0; half < 2; half++) {
          const int64_t qa = q0 + 128 * m + 32 * quarter + 16 * half + (lane >> 2);
          const uint32_t tb = dset + ((uint32_t)(32 * quarter + 16 * half) << 16) + (uint32_t)(m * NPARTS * p.acols);
          if (blocks3) tcr_drain_half<XC, 3>(p, tb, orow, qa, lane);
          else if (blocks2) tcr_drain_half<XC, 2>(p, tb, orow, qa, lane);
          else tcr_drain_half<XC, 1>(p, tb, orow, qa, lane);
        }
      }
      tc::tc_fence_before();
      named_sync(2, 128);
      if (quarter == 0 && lane == 0) mbar_arrive(&tm_empty[slot]);
      if (quarter == 0 && lane == 0) GBFIR_TC_TRACE(2, k, 2);
    }
  }
  __syncthreads();
  if (s_fail && tid == 0) {
    atomicExch(&g_tc_status, 1);
    // give MMAs still in flight a bounded chance to finish before the TMEM is freed
    for (int i = 0; i < p.nsets; i++) (void)tc::mbar_wait(&tm_full[i], 0);
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc::tc_fence_after();
    tc::tmem_dealloc(tmem, (uint32_t)p.tmem_cols);
  }
}

// ---------------------------------------------------------------------------------
struct TcPlan {
  TcParams p;
  size_t smem;
  bool ok;
  char why[160];
};

// Tap geometry of one pass: y[n] = scale * sum_i x[i] * he(c + n*down - i*up), with he the
// filter of logical length Lo (a virtual leading zero when `even`), read reversed when rev.
struct TcTaps {
  int64_t Lo, c;
  int32_t even, rev;
  double scale;
};

// resample_poly: scipy centring, even filters extended by a leading zero, gain up.
static TcTaps resample_taps(int64_t L, int64_t up) {
  TcTaps t{};
  t.even = (L % 2) == 0;
  t.Lo = L + t.even;
  t.c = (t.Lo - 1) / 2;
  t.rev = 0;
  t.scale = (double)up;
  return t;
}

// rp: Hankel row pitch, 8 or 64 samples.
static TcPlan plan_tc(int64_t up, int64_t down, const TcTaps &taps, int64_t N_in, int64_t out_len, int64_t batch,
                      int xc, int precision, int rp) {
  TcPlan pl{};
  TcParams &p = pl.p;
  p.even = taps.even;
  p.Lo = taps.Lo;
  p.c = taps.c;
  p.rev = taps.rev;
  p.up = up;
  p.down = down;
  p.N = N_in;
  p.out_len = out_len;
  p.scale = taps.scale;
  p.fp16 = precision == GBFIR_PREC_FP16;
  p.terms = precision == GBFIR_PREC_BF16X3 ? 3 : 1;
  p.rp = rp;
  p.path = (rp % down == 0) ? 0 : 1;
  p.P = p.path == 0 ? 1 : (int32_t)down;
  if (up > 256 || (p.path == 0 ? up * (rp / down) : rp * up) > 256) {
    snprintf(pl.why, sizeof(pl.why), "a row of %lld outputs exceeds the MMA N limit of 256",
             (long long)(p.path == 0 ? up * (rp / down) : rp * up));
    return pl;
  }
  int64_t kmin, kmax;
  if (p.path == 0) {
    p.Nt = (int32_t)(up * (rp / down));
    kmin = ceil_div(p.c - p.Lo + 1, up);
    kmax = floor_div(p.c + (int64_t)(p.Nt - 1) * down, up);
  } else {
    p.Nt = (int32_t)(rp * up);
    kmin = INT64_MAX;
    kmax = INT64_MIN;
    for (int64_t b = 0; b < down; b++) {
      kmin = std::min(kmin, ceil_div(p.c - up * b - p.Lo + 1, up * down));
      kmax = std::max(kmax, floor_div(p.c + down * (int64_t)(p.Nt - 1) - up * b, up * down));
    }
  }
  p.Nmma = (p.Nt + 15) / 16 * 16;
  p.k0 = floor_div(kmin, 8) * 8;
  p.Kp = (int32_t)((kmax - p.k0 + 1 + 15) / 16 * 16);
  if (p.Nmma > 256) {
    snprintf(pl.why, sizeof(pl.why), "a row of %d outputs exceeds the MMA N limit of 256", p.Nt);
    return pl;
  }
  if (p.P > 16) {
    snprintf(pl.why, sizeof(pl.why), "down = %lld polyphase components are too many", (long long)down);
    return pl;
  }
  const int nparts = xc ? 2 : 1;
  // bf16x3: the tap terms concatenated along N wherever 3*N fits one MMA (measured: three
  // MMAs of N = 192/128/64 per K-step take half the time of six of N = 64, and the small
  // terms accumulate apart from a0*b0: 1e-7 rel-L2 for a 301-tap conv where one accumulator
  // over all six products gave 2e-6); wider rows issue six MMAs of N per K-step, into two
  // accumulators (a0*b0 apart from the rest) where the band is longer than 8 K-steps
  p.concat = (p.terms == 3 && 3 * p.Nmma <= 256) ? 1 : 0;
  p.split = (p.terms == 3 && !p.concat && p.P * (p.Kp / 16) > 8) ? 1 : 0;
  p.acols = p.concat ? 3 * p.Nmma : p.split ? 2 * p.Nmma : p.Nmma;
  const int wrows = p.terms * p.Nmma;
  const size_t xalign = rp == 64 ? 1024 : 128;
  auto smem_for = [&](int MT, int nraw, int nslots) -> size_t {
    const size_t w = (size_t)p.P * wrows * p.Kp * 2;
    const size_t la = (size_t)rp * 128 * MT + p.Kp;
    const size_t xa = (la * 2 + xalign - 1) / xalign * xalign;
    const size_t raw = (size_t)nraw * p.P * la * (xc ? 8 : 4);
    // 1024 bytes of slack to align the dynamic shared memory base
    return 1024 + (w + 1023) / 1024 * 1024 + (size_t)nslots * nparts * p.terms * p.P * xa + raw;
  };
  // A stage holds MT M-tiles of 128 rows.  Shrink, in this order, until it fits: MT, the raw
  // staging depth, the number of TMEM accumulator sets (512 columns), the operand ring depth.
  const size_t kMaxSmem = 225 * 1024;
  int MT = rp == 64 ? 1 : 4, nraw = 2, nsets = 2, nslots = 2;
  auto smem_ok = [&]() { return smem_for(MT, nraw, nslots) <= kMaxSmem; };
  auto tmem_ok = [&]() { return nsets * MT * nparts * p.acols <= 512; };
  while (MT > 1 && !(smem_ok() && tmem_ok())) MT /= 2;
  if (!smem_ok()) nraw = 1;
  if (!tmem_ok()) nsets = 1;
  if (!smem_ok()) nslots = 1;
  if (!smem_ok() || !tmem_ok()) {
    snprintf(pl.why, sizeof(pl.why), "tile needs %zu B of shared memory", smem_for(MT, nraw, nslots));
    return pl;
  }
  p.MT = MT;
  p.nbuf = nslots;
  p.nraw = nraw;
  p.nsets = nsets;
  p.LA = rp * 128 * MT + p.Kp;
  uint32_t cols = 32;
  while (cols < (uint32_t)(nsets * MT * nparts * p.acols)) cols <<= 1;
  p.tmem_cols = (int32_t)cols;
  p.rows = (out_len + p.Nt - 1) / p.Nt;
  p.iters_per_row = (p.rows + 128 * MT - 1) / (128 * MT);
  p.niters = p.iters_per_row * batch;
  pl.smem = smem_for(MT, nraw, nslots);
  pl.ok = true;
  return pl;
}

}  // namespace gbfir
#include "tc_wide.h"
namespace gbfir {

int launch_tc_blocks(const gbfir_buf &out, const gbfir_buf &in, const gbfir_buf &h, int64_t up, int64_t down,
                     int64_t Lo, int64_t c, int even, int rev, double scale, int precision, const char *what,
                     cudaStream_t s);

static int launch_tc(TcPlan &pl, const gbfir_buf &out, const gbfir_buf &in, const gbfir_buf &h, bool xc,
                     const char *what, cudaStream_t s) {
  TcParams &p = pl.p;
  p.x = in.ptr;
  p.x_bstride = (out.batch > 1 && in.batch > 1) ? in.batch_stride : 0;
  p.h = reinterpret_cast<const float *>(h.ptr);
  p.out = out.ptr;
  p.out_bstride = out.batch_stride;
  const void *fn = xc ? (const void *)tc_resample_kernel<true> : (const void *)tc_resample_kernel<false>;
  int rc = ensure_smem(fn, pl.smem, what);
  if (rc) return rc;
  int occ = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, kWsThreads, pl.smem);
  if (occ < 1) occ = 1;
  occ = std::min(occ, 512 / p.tmem_cols);  // each CTA holds tmem_cols of the SM's 512 TMEM columns
  int64_t grid = (int64_t)num_sms() * occ;
  if (grid > p.niters) grid = p.niters;
  void *args[] = {&p};
  cudaError_t e = cudaLaunchKernel(fn, dim3((unsigned)grid), dim3(kWsThreads), args, pl.smem, s);
  if (e != cudaSuccess) GBFIR_FAIL(GBFIR_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  count_launch();
  return GBFIR_SUCCESS;
}

// Which tensor-core kernel a pass prefers: 0 = the built-in order, 8 / 64 = the Toeplitz kernel
// with that row pitch only, 1 = the 64-sample-row kernel with the taps in TMEM (tc_wide.cu)
// first.  GBFIR_TC_ROWS ("8", "64", "wide") pins one for measurements.
static int tc_rows_pref() {
  const char *e = getenv("GBFIR_TC_ROWS");
  if (e == nullptr) return 0;
  if (strcmp(e, "8") == 0) return 8;
  if (strcmp(e, "64") == 0) return 64;
  if (strcmp(e, "wide") == 0) return 1;
  return 0;
}

// The Toeplitz plan to run, or the one the preference pins: 64-sample rows where the tile
// fits (measured faster even with one operand slot), else 8-sample rows.
static TcPlan plan_tc_rows(int64_t up, int64_t down, const TcTaps &taps, int64_t N_in, int64_t out_len,
                           int64_t batch, int xc, int precision, int pref) {
  if (pref == 8 || pref == 64) return plan_tc(up, down, taps, N_in, out_len, batch, xc, precision, pref);
  TcPlan wide = plan_tc(up, down, taps, N_in, out_len, batch, xc, precision, 64);
  if (wide.ok) return wide;
  return plan_tc(up, down, taps, N_in, out_len, batch, xc, precision, 8);
}

int resample_poly_tc(const gbfir_buf &out, const gbfir_buf &in, const gbfir_buf &h, int64_t up, int64_t down,
                     int precision, cudaStream_t s) {
  if (dtype_double(in.dtype) || dtype_complex(h.dtype))
    GBFIR_FAIL(GBFIR_ERR_NOT_SUPPORTED, "resample_poly: tensor-core forms take float32/complex64 signals and real "
                                        "float32 taps");
  const bool xc = dtype_complex(in.dtype);
  const TcTaps taps = resample_taps(h.len, up);
  const int pref = tc_rows_pref();
  // The Toeplitz kernel with 64-sample rows where its tile fits (measured fastest); else
  // 64-sample rows with the taps in TMEM where they fill at least half of the 128 MMA lanes
  // with output phases; else the Toeplitz kernel with 8-sample rows.
  if (pref == 0) {
    TcPlan wide = plan_tc(up, down, taps, in.len, out.len, out.batch, xc, precision, 64);
    if (wide.ok) return launch_tc(wide, out, in, h, xc, "resample_poly (tensor cores)", s);
  }
  if ((pref == 0 || pref == 1) && 64 % down == 0 && 64 * up / down >= 64) {
    TwPlan wp = plan_tc_wide(up, down, taps.Lo, taps.c, taps.even, taps.rev, taps.scale, in.len, out.len, out.batch,
                             xc, precision);
    if (wp.ok) return launch_tc_wide(wp, out, in, h, xc, "resample_poly (tensor cores)", s);
  }
  TcPlan pl = plan_tc_rows(up, down, taps, in.len, out.len, out.batch, xc, precision, pref);
  if (pl.ok) return launch_tc(pl, out, in, h, xc, "resample_poly (tensor cores)", s);
  // rows that advance a number of samples no aliased layout expresses (e.g. 160/147):
  // materialised Hankel rows in column blocks
  return launch_tc_blocks(out, in, h, up, down, taps.Lo, taps.c, taps.even, taps.rev, taps.scale, precision,
                          "resample_poly (tensor cores)", s);
}

// conv1d / corr on the tensor cores: the Toeplitz pass with up = down = 1, no even-length
// extension, gain 1 and the mode's start offset as the centre (conv.h:155-168 semantics:
// out[o] = full[o + start], start = 0 FULL, (L-1)/2 or L/2-1 SAME, L-1 VALID); corr reads
// the (real) taps reversed.  Covers a real float32 filter row shared by every signal row,
// with the signal at least as long as the filter (no operand swap).  Rows of 64 outputs
// (64-sample Hankel rows) where the tile fits, 8 otherwise.
int conv1d_tc(const gbfir_buf &out, const gbfir_buf &in, const gbfir_buf &h, int mode, int is_corr, int precision,
              cudaStream_t s) {
  if (dtype_double(in.dtype) || dtype_complex(h.dtype))
    GBFIR_FAIL(GBFIR_ERR_NOT_SUPPORTED, "conv1d: tensor-core forms take float32/complex64 signals and real "
                                        "float32 taps");
  if (h.batch > 1)
    GBFIR_FAIL(GBFIR_ERR_NOT_SUPPORTED, "conv1d: tensor-core forms take one filter row for all signal rows");
  if (in.len < h.len)
    GBFIR_FAIL(GBFIR_ERR_NOT_SUPPORTED, "conv1d: tensor-core forms need the signal at least as long as the filter "
                                        "(%lld < %lld)", (long long)in.len, (long long)h.len);
  const int64_t L = h.len;
  TcTaps t{};
  t.Lo = L;
  t.even = 0;
  t.rev = is_corr ? 1 : 0;
  t.scale = 1.0;
  t.c = mode == GBFIR_MODE_SAME ? ((L & 1) ? (L - 1) / 2 : L / 2 - 1) : mode == GBFIR_MODE_VALID ? L - 1 : 0;
  const bool xc = dtype_complex(in.dtype);
  TcPlan pl = plan_tc_rows(1, 1, t, in.len, out.len, out.batch, xc, precision, tc_rows_pref());
  if (!pl.ok) GBFIR_FAIL(GBFIR_ERR_NOT_SUPPORTED, "conv1d: tensor-core form unavailable: %s", pl.why);
  return launch_tc(pl, out, in, h, xc, "conv1d (tensor cores)", s);
}

// dL/dx of conv1d on the tensor cores: dx[i] = sum_n gy[n] * h[start + n - i] is the forward
// pass over gy with the taps read reversed about the centre L - 1 - start (the FP32 adjoint
// runs the same pass on the CUDA cores).  Real float32 operands.
int conv1d_bwd_dx_tc(const gbfir_buf &dx, const gbfir_buf &gy, const gbfir_buf &h, int64_t start, int precision,
                     cudaStream_t s) {
  TcTaps t{};
  t.Lo = h.len;
  t.even = 0;
  t.rev = 1;
  t.scale = 1.0;
  t.c = h.len - 1 - start;
  TcPlan pl = plan_tc_rows(1, 1, t, gy.len, dx.len, dx.batch, 0, precision, tc_rows_pref());
  if (!pl.ok) GBFIR_FAIL(GBFIR_ERR_NOT_SUPPORTED, "conv1d_bwd: tensor-core dx unavailable: %s", pl.why);
  return launch_tc(pl, dx, gy, h, false, "conv1d_bwd dx (tensor cores)", s);
}

// dL/dx of resample_poly on the tensor cores: the transposed resampler
//   dx[m] = up * sum_k gy[k] * he(Lo - 1 - (c + m*up - k*down))
// is the forward pass with the rates swapped and the taps read reversed (the FP32 adjoint
// runs the same pass on the CUDA cores).  Real float32 operands, gcd-reduced rates.
int resample_poly_bwd_dx_tc(const gbfir_buf &dx, const gbfir_buf &gy, const gbfir_buf &h, int64_t up, int64_t down,
                            int precision, cudaStream_t s) {
  TcTaps taps = resample_taps(h.len, up);
  taps.rev = 1;
  const int pref = tc_rows_pref();
  if (pref == 0) {
    TcPlan wide = plan_tc(down, up, taps, gy.len, dx.len, dx.batch, 0, precision, 64);
    if (wide.ok) return launch_tc(wide, dx, gy, h, false, "resample_poly_bwd dx (tensor cores)", s);
  }
  if (pref == 0 || pref == 1) {
    TwPlan wp = plan_tc_wide(down, up, taps.Lo, taps.c, taps.even, taps.rev, taps.scale, gy.len, dx.len, dx.batch, 0,
                             precision);
    if (wp.ok) return launch_tc_wide(wp, dx, gy, h, false, "resample_poly_bwd dx (tensor cores)", s);
  }
  TcPlan pl = plan_tc_rows(down, up, taps, gy.len, dx.len, dx.batch, 0, precision, pref);
  if (pl.ok) return launch_tc(pl, dx, gy, h, false, "resample_poly_bwd dx (tensor cores)", s);
  return launch_tc_blocks(dx, gy, h, down, up, taps.Lo, taps.c, taps.even, taps.rev, taps.scale, precision,
                          "resample_poly_bwd dx (tensor cores)", s);
}

int tc_status_read_and_clear() {
  int32_t v = 0, zero = 0;
  if (cudaMemcpyFromSymbol(&v, g_tc_status, sizeof(v)) != cudaSuccess) return -1;
  cudaMemcpyToSymbol(g_tc_status, &zero, sizeof(zero));
  return v;
}

}  // namespace gbfir

namespace gbfir {
int resample_rowtile_status();
int adjoint_rowtile_status();
int tc_wide_status_take();
int tc_channelize_status_take();
int tc_blocks_status_take();
int tc_dh_status_take();
int iir_status_take();
}  // namespace gbfir

// 0 if every bounded wait of the pipelined kernels (tensor-core kernels, the TMA-fed row
// tile, the filter's chained carries) completed since the last call; 1 if one gave up; -1 if
// the status could not be read.
extern "C" int gbfir_tc_status(void) {
  const int a = gbfir::tc_status_read_and_clear();
  const int b = gbfir::resample_rowtile_status();
  const int c = gbfir::adjoint_rowtile_status();
  const int d = gbfir::tc_wide_status_take();
  const int e = gbfir::iir_status_take();
  const int f = gbfir::tc_channelize_status_take();
  const int g = gbfir::tc_blocks_status_take();
  const int k = gbfir::tc_dh_status_take();
  if (a < 0 || b < 0 || c < 0 || d < 0 || e < 0 || f < 0 || g < 0 || k < 0) return -1;
  return (a | b | c | d | e | f | g | k) ? 1 : 0;
}
