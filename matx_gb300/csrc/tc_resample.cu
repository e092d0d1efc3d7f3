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
// six products as six MMAs of N columns into one accumulator.
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
  int32_t concat;   // bf16x3: 1 = tap terms concatenated along N, 0 = six MMAs into one
  int32_t acols;    // TMEM accumulator columns per (M-tile, part): 3*Nmma (concat) or Nmma
};

// Bounded-wait status of the tensor-core kernels (1 = a wait gave up); read and
// cleared by gbfir_tc_status().
__device__ int32_t g_tc_status;

// Tap he(tp) of the logical filter (reversed when rev, 0 outside), read from hs: the filter's
// taps staged in shared memory, or the global row.
__device__ __forceinline__ float tap_value(const TcParams &p, const float *hs, int64_t tp) {
  if (tp < 0 || tp >= p.Lo) return 0.f;
  const int64_t te = p.rev ? p.Lo - 1 - tp : tp;
  if (p.even && te == 0) return 0.f;
  return hs[te - p.even];
}

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

template <bool XC>
__global__ void __launch_bounds__(kWsThreads, 1) tc_resample_kernel(const TcParams p) {
  using XT = typename val_of<float, XC>::type;
  constexpr int NPARTS = XC ? 2 : 1;  // real / imaginary operand rows
  extern __shared__ __align__(1024) unsigned char smem_dyn[];
  __shared__ uint64_t op_full[2], op_empty[2], tm_full[2], tm_empty[2];
  __shared__ uint32_t tmem_slot;
  __shared__ int s_fail, s_pok, s_eok;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

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
    }
    s_fail = 0;
    tc::mbar_fence_init();
  }
  // The filter's taps, staged once into the raw ring (not in use yet) so that the W build
  // reads shared memory instead of making one dependent global load per element.
  const int64_t Lh = p.Lo - p.even;
  const bool h_staged = (size_t)Lh * sizeof(float) <= (size_t)p.nraw * raw_elems * sizeof(XT);
  float *hs_stage = reinterpret_cast<float *>(raw0);
  if (h_staged)
    for (int64_t e = tid; e < Lh; e += kWsThreads) hs_stage[e] = p.h[e];
  __syncthreads();
  const float *hsrc = h_staged ? hs_stage : p.h;
  // ---- W_cat[pp][t*Nmma + j][k] = term t of up*he[tap(j, k)] (K-major core layout) ----
  const int wel = wrows * p.Kp;
  for (int e = tid; e < p.P * wel; e += kWsThreads) {
    const int pp = e / wel, r = e - pp * wel;
    const int row = r / p.Kp, k = r - row * p.Kp;
    const int t = row / p.Nmma, j = row - t * p.Nmma;
    float v = 0.f;
    if (j < p.Nt) {
      const int64_t kk = k + p.k0;
      const int64_t tp = p.path == 0 ? p.c + (int64_t)j * p.down - kk * p.up
                                     : p.c + p.down * (int64_t)j - p.up * (pp + p.down * kk);
      v = tap_value(p, hsrc, tp) * (float)p.scale;
    }
    const uint32_t off = tc::kmajor_offset(row, k, p.Kp);
    if (p.fp16) {
      *reinterpret_cast<__half *>(warr(pp) + off) = __float2half_rn(v);
    } else {
      __nv_bfloat16 t0, t1, t2;
      tc::split3_bf16(v, t0, t1, t2);
      *reinterpret_cast<__nv_bfloat16 *>(warr(pp) + off) = t == 0 ? t0 : (t == 1 ? t1 : t2);
    }
  }
  tc::fence_async_smem();
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = tmem_slot;
  const uint32_t set_cols = (uint32_t)(p.MT * NPARTS * p.acols);
  const XT *xp = reinterpret_cast<const XT *>(p.x);
  (void)xp;

  if (warp >= kProdWarp0 && warp < kProdWarp0 + kProdWarps) {
    // ================= producers =================
    const int ptid = tid - kProdWarp0 * 32;
    auto fetch = [&](int64_t itx, int slot) {
      const int64_t b = itx / p.iters_per_row;
      const int64_t q0 = (itx - b * p.iters_per_row) * (int64_t)(128 * p.MT);
      const XT *row = xp + b * p.x_bstride;
      const int64_t base = p.path == 0 ? p.rp * q0 + p.k0 : p.down * (p.rp * q0 + p.k0);
      XT *dst = rawp(slot);
      constexpr int G = 16 / (int)sizeof(XT);
      // windows inside the signal with a 16-byte aligned start come in 16-byte pieces; the
      // others element by element, zero-filled outside the signal
      const bool vec = ((reinterpret_cast<uintptr_t>(row + base) | (uintptr_t)tc::smem_u32(dst)) & 15) == 0 &&
                       base >= 0 && base + (int64_t)raw_elems <= p.N && raw_elems % G == 0;
      if (vec) {
        for (int v = ptid; v < (int)(raw_elems / G); v += kNProd)
          cp_async_zfill<16>(dst + (size_t)v * G, row + base + (int64_t)v * G, true);
      } else {
        for (int v = ptid; v < (int)raw_elems; v += kNProd) {
          const int64_t gi = base + v;
          const bool okk = gi >= 0 && gi < p.N;
          cp_async_zfill<sizeof(XT)>(dst + v, okk ? (const void *)(row + gi) : (const void *)row, okk);
        }
      }
    };
    const int nraw = p.nraw;
    int64_t it = blockIdx.x;
    if (it < p.niters) fetch(it, 0);
    cp_async_commit();
    if (nraw == 2 && it + gridDim.x < p.niters) fetch(it + gridDim.x, 1);
    cp_async_commit();
    const int nslots = p.nbuf;
    for (int k = 0; it < p.niters; it += gridDim.x, ++k) {
      const int slot = k % nslots;
      const int rslot = nraw == 2 ? (k & 1) : 0;
      // with two raw slots this iteration's group is the older of two outstanding ones;
      // with one slot it is the most recent group
      if (nraw == 2) cp_async_wait<1>();
      else cp_async_wait<0>();
      // one thread waits for the slot; the named barrier publishes its verdict (and every
      // producer's landed copies) to all producers, so the role leaves the loop together
      if (ptid == 0)
        s_pok = (k < nslots) ? 1 : (tc::mbar_wait(&op_empty[slot], ((k - nslots) / nslots) & 1) ? 1 : 0);
      named_sync(1, kNProd);
      if (!s_pok) {
        s_fail = 1;
        break;
      }
      // convert raw slot -> operand slot: two consecutive samples of one component per item
      // (with 64-sample rows the 4-byte pair at byte o goes to the 128-byte-swizzled slot
      // o ^ ((o >> 7) & 7) << 4; a warp writes one 128-byte row, conflict-free)
      const XT *src = rawp(rslot);
      const int half = p.LA / 2;
      const uint32_t swz = p.rp == 64 ? 7u : 0u;
      for (int pp = 0; pp < p.P; pp++) {
        unsigned char *dst[NPARTS][3];
#pragma unroll
        for (int part = 0; part < NPARTS; part++)
#pragma unroll
          for (int t = 0; t < 3; t++) dst[part][t] = xarrp(slot, part, t < p.terms ? t : 0, pp);
        for (int v = ptid; v < half; v += kNProd) {
          const int u = 2 * v;
          const uint32_t o = 4u * (uint32_t)v;
          const uint32_t po = o ^ (((o >> 7) & swz) << 4);
          XT v0, v1;
          if (p.P == 1) {
            if constexpr (XC) {
              const float4 w = *reinterpret_cast<const float4 *>(src + u);
              v0 = make_float2(w.x, w.y);
              v1 = make_float2(w.z, w.w);
            } else {
              const float2 w = *reinterpret_cast<const float2 *>(src + u);
              v0 = w.x;
              v1 = w.y;
            }
          } else {
            v0 = src[(size_t)u * p.P + pp];
            v1 = src[(size_t)(u + 1) * p.P + pp];
          }
#pragma unroll
          for (int part = 0; part < NPARTS; part++) {
            const float2 f = part == 0 ? make_float2(re_of(v0), re_of(v1)) : make_float2(im_of(v0), im_of(v1));
            if (p.fp16) {
              *reinterpret_cast<__half2 *>(dst[part][0] + po) = __float22half2_rn(f);
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
      tc::fence_async_smem();
      named_sync(1, kNProd);
      if (ptid == 0) mbar_arrive(&op_full[slot]);
      // the raw slot is consumed: stage iteration k + nraw into it
      const int64_t it2 = it + (int64_t)nraw * gridDim.x;
      if (it2 < p.niters) fetch(it2, rslot);
      cp_async_commit();
    }
    cp_async_wait<0>();
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
        if (!tc::mbar_wait(&op_full[slot], (k / p.nbuf) & 1)) { s_fail = 1; break; }
        if (k >= p.nsets && !tc::mbar_wait(&tm_empty[tset], ((k - p.nsets) / p.nsets) & 1)) { s_fail = 1; break; }
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
          // six MMAs of N columns into one accumulator per K-step, products of order <= 2
          // (signal term tx, tap term tw), smallest first: (1,1) (2,0) (0,2) (1,0) (0,1) (0,0)
          constexpr uint32_t kTx = 0x001021u, kTw = 0x010201u;
          for (int a = 0; a < nacc; a++) {
            const uint32_t d = dset + (uint32_t)(a * p.acols);
            for (int pp = 0; pp < p.P; pp++) {
              const uint64_t bd0 = bfix | (uint64_t)((w0 + (uint32_t)pp * wbytes) >> 4);
              for (int ks = 0; ks < nks; ks++) {
                for (int pr = 0; pr < 6; pr++) {
                  const int tx = (int)((kTx >> (4 * pr)) & 15u), tw = (int)((kTw >> (4 * pr)) & 15u);
                  const uint64_t bd = bd0 + (uint64_t)tw * term_step + (uint64_t)(16 * ks);
                  tc::mma_f16(d, a_desc(a, tx, pp, ks), bd, idesc1, (pp > 0 || ks > 0 || pr > 0) ? 1u : 0u);
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
        tc::mma_commit(&tm_full[tset]);
      }
    }
  } else {
    // ================= epilogue (warps 8-11: TMEM lane quarters 0-3) =================
    const int quarter = warp - kEpiWarp0;
    const uint32_t lane_base = (uint32_t)(32 * quarter) << 16;
    int64_t it = blockIdx.x;
    for (int k = 0; it < p.niters; it += gridDim.x, ++k) {
      const int slot = k % p.nsets;
      if (quarter == 0 && lane == 0) s_eok = tc::mbar_wait(&tm_full[slot], (k / p.nsets) & 1) ? 1 : 0;
      named_sync(2, 128);
      if (!s_eok) {
        s_fail = 1;
        break;
      }
      tc::tc_fence_after();
      const uint32_t dset = tmem + (uint32_t)slot * set_cols;
      const int64_t b = it / p.iters_per_row;
      const int64_t q0 = (it - b * p.iters_per_row) * (int64_t)(128 * p.MT);
      XT *orow = reinterpret_cast<XT *>(p.out) + b * p.out_bstride;
      for (int m = 0; m < p.MT; m++) {
        const int64_t q = q0 + 128 * m + 32 * quarter + lane;
        const int64_t n0 = q * p.Nt;
        const int64_t left64 = p.out_len - n0;
        const int nv = left64 < p.Nt ? (left64 > 0 ? (int)left64 : 0) : p.Nt;  // valid outputs of this row
        XT *dst = orow + n0;
        const bool vec = (reinterpret_cast<uintptr_t>(dst) & 15) == 0;
        const bool blocks3 = p.terms == 3 && p.concat;
        for (int col = 0; col < p.Nmma; col += 16) {
          float acc[NPARTS][16];
#pragma unroll
          for (int part = 0; part < NPARTS; part++) {
            const uint32_t base = dset + lane_base + (uint32_t)((m * NPARTS + part) * p.acols + col);
            uint32_t r0[16], r1[16], r2[16];
            tc::tmem_ld16(base, r0);
            if (blocks3) {
              tc::tmem_ld16(base + (uint32_t)p.Nmma, r1);
              tc::tmem_ld16(base + (uint32_t)(2 * p.Nmma), r2);
            }
            tc::tmem_ld_wait();
            if (blocks3) {
#pragma unroll
              for (int i = 0; i < 16; i++)
                acc[part][i] = (__uint_as_float(r0[i]) + __uint_as_float(r1[i])) + __uint_as_float(r2[i]);
            } else {
#pragma unroll
              for (int i = 0; i < 16; i++) acc[part][i] = __uint_as_float(r0[i]);
            }
          }
          if constexpr (XC) {
            // pairs of outputs as one 16-byte store where the row start is 16-byte aligned
#pragma unroll
            for (int i = 0; i < 16; i += 2) {
              if (vec && col + i + 1 < nv) {
                *reinterpret_cast<float4 *>(dst + col + i) =
                    make_float4(acc[0][i], acc[1][i], acc[0][i + 1], acc[1][i + 1]);
              } else {
                if (col + i < nv) dst[col + i] = make_float2(acc[0][i], acc[1][i]);
                if (col + i + 1 < nv) dst[col + i + 1] = make_float2(acc[0][i + 1], acc[1][i + 1]);
              }
            }
          } else {
            // groups of four outputs as one 16-byte store where the row start is aligned
#pragma unroll
            for (int i = 0; i < 16; i += 4) {
              if (vec && col + i + 3 < nv) {
                *reinterpret_cast<float4 *>(dst + col + i) =
                    make_float4(acc[0][i], acc[0][i + 1], acc[0][i + 2], acc[0][i + 3]);
              } else {
#pragma unroll
                for (int e = 0; e < 4; e++)
                  if (col + i + e < nv) dst[col + i + e] = acc[0][i + e];
              }
            }
          }
        }
      }
      tc::tc_fence_before();
      named_sync(2, 128);
      if (quarter == 0 && lane == 0) mbar_arrive(&tm_empty[slot]);
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
  // bf16x3: concatenate the tap terms along N where 3*N fits one MMA, else six MMAs of N
  p.concat = (p.terms == 3 && 3 * p.Nmma <= 256) ? 1 : 0;
  p.acols = p.concat ? 3 * p.Nmma : p.Nmma;
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

// The Toeplitz plan to run, or the one the preference pins: 64-sample rows where they keep
// the whole pipeline (two operand slots, two accumulator sets), else 8-sample rows, else
// 64-sample rows with whatever pipeline fits.
static TcPlan plan_tc_rows(int64_t up, int64_t down, const TcTaps &taps, int64_t N_in, int64_t out_len,
                           int64_t batch, int xc, int precision, int pref) {
  if (pref == 8 || pref == 64) return plan_tc(up, down, taps, N_in, out_len, batch, xc, precision, pref);
  TcPlan wide = plan_tc(up, down, taps, N_in, out_len, batch, xc, precision, 64);
  if (wide.ok && wide.p.nbuf == 2 && wide.p.nsets == 2) return wide;
  TcPlan narrow = plan_tc(up, down, taps, N_in, out_len, batch, xc, precision, 8);
  if (narrow.ok || !wide.ok) return narrow;
  return wide;
}

int resample_poly_tc(const gbfir_buf &out, const gbfir_buf &in, const gbfir_buf &h, int64_t up, int64_t down,
                     int precision, cudaStream_t s) {
  if (dtype_double(in.dtype) || dtype_complex(h.dtype))
    GBFIR_FAIL(GBFIR_ERR_NOT_SUPPORTED, "resample_poly: tensor-core forms take float32/complex64 signals and real "
                                        "float32 taps");
  const bool xc = dtype_complex(in.dtype);
  const TcTaps taps = resample_taps(h.len, up);
  const int pref = tc_rows_pref();
  // 64-sample rows with the taps in TMEM where they fill at least half of the 128 MMA lanes
  // with output phases (measured faster there); the Toeplitz kernel otherwise
  if ((pref == 0 || pref == 1) && 64 % down == 0 && 64 * up / down >= 64) {
    TwPlan wp = plan_tc_wide(up, down, taps.Lo, taps.c, taps.even, taps.rev, taps.scale, in.len, out.len, out.batch,
                             xc, precision);
    if (wp.ok) return launch_tc_wide(wp, out, in, h, xc, "resample_poly (tensor cores)", s);
  }
  TcPlan pl = plan_tc_rows(up, down, taps, in.len, out.len, out.batch, xc, precision, pref);
  if (!pl.ok)
    GBFIR_FAIL(GBFIR_ERR_NOT_SUPPORTED, "resample_poly: tensor-core form unavailable for up=%lld down=%lld: %s",
               (long long)up, (long long)down, pl.why);
  return launch_tc(pl, out, in, h, xc, "resample_poly (tensor cores)", s);
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

// dL/dx of resample_poly on the tensor cores: the transposed resampler
//   dx[m] = up * sum_k gy[k] * he(Lo - 1 - (c + m*up - k*down))
// is the forward pass with the rates swapped and the taps read reversed (the FP32 adjoint
// runs the same pass on the CUDA cores).  Real float32 operands, gcd-reduced rates.
int resample_poly_bwd_dx_tc(const gbfir_buf &dx, const gbfir_buf &gy, const gbfir_buf &h, int64_t up, int64_t down,
                            int precision, cudaStream_t s) {
  TcTaps taps = resample_taps(h.len, up);
  taps.rev = 1;
  const int pref = tc_rows_pref();
  if (pref == 0 || pref == 1) {
    TwPlan wp = plan_tc_wide(down, up, taps.Lo, taps.c, taps.even, taps.rev, taps.scale, gy.len, dx.len, dx.batch, 0,
                             precision);
    if (wp.ok) return launch_tc_wide(wp, dx, gy, h, false, "resample_poly_bwd dx (tensor cores)", s);
  }
  TcPlan pl = plan_tc_rows(down, up, taps, gy.len, dx.len, dx.batch, 0, precision, pref);
  if (!pl.ok)
    GBFIR_FAIL(GBFIR_ERR_NOT_SUPPORTED, "resample_poly_bwd: tensor-core dx unavailable for up=%lld down=%lld: %s",
               (long long)up, (long long)down, pl.why);
  return launch_tc(pl, dx, gy, h, false, "resample_poly_bwd dx (tensor cores)", s);
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
  if (a < 0 || b < 0 || c < 0 || d < 0 || e < 0) return -1;
  return (a | b | c | d | e) ? 1 : 0;
}
