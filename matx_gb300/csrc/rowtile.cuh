// rowtile.cuh — the polyphase "row tile" kernel shared by the forward resampler,
// its adjoints and the ragged launch.
//
// Outputs are grouped into rows of Nt = up*G consecutive outputs; row q needs
// inputs from q*S + k with S = down*G, so every row sees the same tap matrix
// B[k][j] = he[c + j*down - k*up].  The columns j are cut into groups of 4
// adjacent phases; group g only needs the band k in [kl0(g), kl0(g)+span) (its
// union band), stored in shared memory as one 4-vector of taps per k.  A thread
// owns 8 adjacent phases (two bands, the second starting d samples later) of RQ
// rows and walks the union of the two bands in three ranges (A only, both, B
// only), so each input sample read from shared memory feeds up to 8 phases x RQ
// rows of FMAs with no multiply by a padding zero between the bands.  A warp's
// 32 lanes take 32 different rows of the same phases, so tap reads are warp-wide
// broadcasts.  A persistent CTA walks tiles of QC rows; with nbuf = 2 the next
// tile's input window is prefetched with cp.async (zero-filled outside the
// signal) while the current one is computed.
//
// With rev = 1 the taps are read reversed (he[Lo-1-tp]); with up and down
// swapped this computes the transposed resampler used by the adjoint.
#pragma once
#include <cuda.h>

#include <algorithm>
#include <cstring>

#include "common.cuh"
#include "tc.cuh"

namespace gbfir {

// Timing hooks of the ring form's roles (role, stage, event); they compile to nothing unless
// a tracing build defines them.
#ifndef GBFIR_TC_TRACE
#define GBFIR_TC_TRACE(role, stage, event) \
  do {                                     \
  } while (0)
#endif

// Bounded-wait status of the row-tile kernels of this translation unit (1 = a window copy
// did not complete within the spin limit); read and cleared through rowtile_status_take().
static __device__ int32_t g_rowtile_status;

static inline int rowtile_status_take() {
  int32_t v = 0, zero = 0;
  if (cudaMemcpyFromSymbol(&v, g_rowtile_status, sizeof(v)) != cudaSuccess) return -1;
  cudaMemcpyToSymbol(g_rowtile_status, &zero, sizeof(zero));
  return v;
}

struct RsParams {
  const void *x;
  int64_t x_bstride, N;
  const void *h;
  int64_t Lo;      // logical (odd) filter length
  int32_t even;    // 1: h has a virtual leading zero
  int64_t c;       // centre tap
  void *out;
  int64_t out_bstride, out_len;
  int64_t up, down;  // reduced
  int64_t Nt, S;     // outputs per row, input stride per row
  int32_t ncg, span; // column groups, padded band length
  int64_t kmin;      // smallest k any group reads
  int64_t rows, tiles_per_row, ntiles;
  int32_t QC, WC;    // rows per tile, column warps
  int32_t win;       // input samples per tile window
  int32_t win_alloc; // shared elements per window buffer (with padding)
  double scale;      // output scale (up for resample_poly)
  int32_t rev;       // read taps reversed
  int32_t nbuf;      // 2: prefetch the next tile's window while computing; 1: single buffer
  int32_t ostore;    // 1: outputs leave through shared memory and TMA tensor stores
  int32_t ost_rb;    // bytes of one row of a stored box (16, 32 or 64)
  int32_t stg_off;   // byte offset of the store staging area in dynamic shared memory
  int64_t rows_full; // rows holding Nt outputs (the tensor map's row count)
  int32_t pair;      // 1: bands start at even k and rows read two samples per 16-byte load
  int32_t ost_single; // 1: one staging buffer per warp instead of two (one row per thread)
};

// Batch row of tile t: a 32-bit division wherever the tile count allows it (the 64-bit one
// is a long instruction sequence, on the path between two tiles).
__device__ __forceinline__ int64_t tile_row(const RsParams &p, int64_t t) {
  if (p.ntiles <= 0x7fffffffLL) return (int64_t)((uint32_t)t / (uint32_t)p.tiles_per_row);
  return t / p.tiles_per_row;
}

// Output staging of one warp for the TMA-store epilogue: two buffers of 32 rows x ost_rb
// bytes, alternating (or one, reused once its previous box has been read); `n` counts the
// boxes this warp has stored.
struct OutStage {
  const void *map;  // CUtensorMap over (2*Nt floats, rows_full, batch)
  unsigned char *buf;
  int n;
  int64_t b;
};

template <typename T, bool HC>
struct TapVec;  // 4 taps of one k
template <typename T>
struct TapVec<T, false> {
  T v[4];
};
template <typename T>
struct TapVec<T, true> {
  typename cplx_of<T>::type v[4];
};
template <typename T, bool XC, bool HC>
struct TapEntry {
  using type = TapVec<T, HC>;
};

// Shared bytes of the tap table: ncg*span entries, then one int32 band offset per group.
template <typename T, bool XC, bool HC>
__host__ __device__ inline size_t tap_table_bytes(int64_t ncg, int64_t span) {
  const size_t taps = ((size_t)ncg * span * sizeof(typename TapEntry<T, XC, HC>::type) + 15) & ~(size_t)15;
  return taps + (((size_t)ncg * 4 + 15) & ~(size_t)15);
}

// Window layouts against bank conflicts of the row-strided reads (lanes read rows q*S + k;
// a 64-bit shared load is served per half-warp, so 16 lanes at stride S must hit distinct
// 8-byte slots of 128 bytes).  PAD = 10 + t, t = ctz(S) (1..7): XOR the low min(t, 4) bits
// of the index with the bits from max(t, 4) up, a permutation inside each block of 16
// elements that is conflict-free for every even S below 256; PAD = 1 is the t = 3 form;
// PAD = 30 + t: the same for 4-byte real samples (32 lanes at stride S hit 32 distinct
// banks), a permutation inside each block of 32 elements; PAD = 4 puts one pad element
// after every 16 elements (the other element types); PAD = 0 is the plain layout (odd S).
template <int PAD>
__device__ __forceinline__ int smem_idx(int p) {
  if constexpr (PAD > 30) {
    // 4-byte elements (real float), row stride S with t = PAD - 30 trailing zero bits: the
    // row bits above the bank bits are XORed into them, a permutation inside blocks of 32
    constexpr int t = PAD - 30, sh = t > 5 ? t : 5, m = (1 << (t < 5 ? t : 5)) - 1;
    return p ^ ((p >> sh) & m);
  } else if constexpr (PAD > 10) {
    constexpr int t = PAD - 10, sh = t > 4 ? t : 4, m = (1 << (t < 4 ? t : 4)) - 1;
    return p ^ ((p >> sh) & m);
  } else if constexpr (PAD == 1) {
    return p ^ ((p >> 4) & 7);
  } else if constexpr (PAD > 0) {
    return p + (p >> PAD);
  } else {
    return p;
  }
}

// First k that column group g (phases 4g..4g+3) reads.  In the paired form it is rounded
// down to even (at most one leading zero tap), so every row's reads start on a 16-byte pair
// of complex samples when the row stride is even.
__host__ __device__ inline int64_t band_start(int64_t c, int64_t g, int64_t down, int64_t Lo, int64_t up, bool pair) {
  const int64_t k = ceil_div(c + 4 * g * down - Lo + 1, up);
  return pair ? floor_div(k, 2) * 2 : k;
}

// table[g*span + kk] holds the 4 taps he[c + (4g+jj)*down - (kl0(g)+kk)*up] (reversed when
// rev, 0 outside); goff[g] = kl0(g) - kmin is where band g starts in the tile window.
template <typename T, bool XC, bool HC>
__device__ __forceinline__ void build_tap_table(const RsParams &p, const typename val_of<T, HC>::type *hp,
                                                unsigned char *table_raw, int tid, int nthreads) {
  using HT = typename val_of<T, HC>::type;
  using TE = typename TapEntry<T, XC, HC>::type;
  TE *table = reinterpret_cast<TE *>(table_raw);
  int *goff = reinterpret_cast<int *>(table_raw + (((size_t)p.ncg * p.span * sizeof(TE) + 15) & ~(size_t)15));
  const int nent = p.ncg * p.span * 4;
  // four entries a thread per pass, their tap loads all in flight before the stores
  constexpr int U = 4;
  for (int e0 = tid; e0 < nent; e0 += U * nthreads) {
    HT v[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int e = e0 + u * nthreads;
      v[u] = zero_val<HT>();
      if (e < nent) {
        const int g = e / (p.span * 4);
        const int rem = e - g * (p.span * 4);
        const int kk = rem >> 2, jj = rem & 3;
        const int64_t j = 4 * (int64_t)g + jj;
        const int64_t kl0 = band_start(p.c, g, p.down, p.Lo, p.up, p.pair != 0);
        const int64_t tp = p.c + j * p.down - (kl0 + kk) * p.up;
        if (j < p.Nt && tp >= 0 && tp < p.Lo) {
          const int64_t te = p.rev ? p.Lo - 1 - tp : tp;  // index into he
          if (!(p.even && te == 0)) v[u] = hp[te - p.even];
        }
      }
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int e = e0 + u * nthreads;
      if (e < nent) {
        const int g = e / (p.span * 4);
        const int rem = e - g * (p.span * 4);
        table[g * p.span + (rem >> 2)].v[rem & 3] = v[u];
      }
    }
  }
  for (int g = tid; g < p.ncg; g += nthreads)
    goff[g] = (int)(band_start(p.c, g, p.down, p.Lo, p.up, p.pair != 0) - p.kmin);
}

__device__ __forceinline__ const int *tap_goff(const RsParams &p, const unsigned char *table_raw, size_t entry) {
  return reinterpret_cast<const int *>(table_raw + (((size_t)p.ncg * p.span * entry + 15) & ~(size_t)15));
}

// Packed FP32 pair arithmetic: one f32x2 instruction, each lane an IEEE round-to-nearest
// fma / mul, so the values equal two scalar fmaf / __fmul_rn calls.
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }

// The 8 phases of super-group sg for a thread's RQ rows, scaled, to the output: through the
// warp's staging buffer and a TMA tensor store when os.buf is set, else direct stores (four
// 16-byte stores per whole, aligned row).
template <int RQ>
__device__ __forceinline__ void c2_store_rows(const RsParams &p, const float2 (&acc)[RQ][8], int sg, int64_t q0,
                                              int rbase, int lane, float2 sc, float2 *orow, OutStage &os) {
  const int Nt = (int)p.Nt;
  const int j0 = 8 * sg;
  const int ncol = min(8, Nt - j0);
#pragma unroll
  for (int i = 0; i < RQ; i++) {
    const int64_t n0 = (q0 + rbase + 32 * i) * p.Nt + j0;
    const int64_t left = p.out_len - n0;
    const int nv = left < ncol ? (left > 0 ? (int)left : 0) : ncol;
    float2 *dst = orow + n0;
    if (os.buf) {
      // stage the warp's 32 rows x 8 phases (swizzled like the tensor map: 16-byte chunk
      // u of row r at chunk u ^ f(r), conflict-free), then one lane stores the box; rows
      // past rows_full are clipped by the map and the one partial row is stored here
      unsigned char *buf = os.buf + (p.ost_single ? 0 : (os.n & 1) * 2048);
      if (lane == 0 && os.n >= 1) {
        if (p.ost_single) tc::bulk_wait_read<0>();
        else if (os.n >= 2) tc::bulk_wait_read<1>();
      }
      __syncwarp();
      const int rb = p.ost_rb;
      const int sw = rb == 64 ? ((lane >> 1) & 3) : rb == 32 ? ((lane >> 2) & 1) : 0;
#pragma unroll
      for (int u = 0; u < 4; u++) {
        if (u * 16 < rb) {
          const float2 lo = mul2(acc[i][2 * u], sc), hi = mul2(acc[i][2 * u + 1], sc);
          *reinterpret_cast<float4 *>(buf + lane * rb + ((u ^ sw) << 4)) = make_float4(lo.x, lo.y, hi.x, hi.y);
        }
      }
      tc::fence_async_smem();
      __syncwarp();
      if (lane == 0) {
        tc::tma_store_3d(os.map, buf, 2 * j0, (int)(q0 + rbase - lane + 32 * i), (int)os.b);
        tc::bulk_commit();
      }
      os.n++;
      if (q0 + rbase + 32 * i == p.rows_full) {
#pragma unroll
        for (int jj = 0; jj < 8; jj++)
          if (jj < nv) dst[jj] = mul2(acc[i][jj], sc);
      }
    } else if (nv == 8 && ((reinterpret_cast<uintptr_t>(dst) & 15) == 0)) {
      float4 *d4 = reinterpret_cast<float4 *>(dst);
#pragma unroll
      for (int u = 0; u < 4; u++) {
        const float2 lo = mul2(acc[i][2 * u], sc), hi = mul2(acc[i][2 * u + 1], sc);
        d4[u] = make_float4(lo.x, lo.y, hi.x, hi.y);
      }
    } else {
#pragma unroll
      for (int jj = 0; jj < 8; jj++)
        if (jj < nv) dst[jj] = mul2(acc[i][jj], sc);
    }
  }
}

// Complex float signal x real float taps, the hot case: the same three-range walk as the
// generic form below with (re, im) accumulated by one f32x2 FMA per sample and phase
// (each lane is the fma of MatX's madd for a real tap, so results are unchanged; the
// (t, t) operand pairs are formed in registers from one 16-byte load of 4 taps), and
// each row's 8 outputs written as four 16-byte stores when they are whole and aligned.
template <int RQ, int PAD>
__device__ __forceinline__ void rowtile_compute_c2(const RsParams &p, const float2 *cur,
                                                   const unsigned char *table_raw, float2 *orow, int64_t q0, int wr,
                                                   int wc, int lane, float scale, int woff, OutStage &os) {
  using TV = TapVec<float, false>;
  const TV *table = reinterpret_cast<const TV *>(table_raw);
  const int *goff = tap_goff(p, table_raw, sizeof(TV));
  const int nsg = (p.ncg + 1) / 2;
  const int rbase = wr * 32 * RQ + lane;
  const float2 sc = make_float2(scale, scale);
  for (int sg = wc; sg < nsg; sg += p.WC) {
    const int gA = 2 * sg, gB = 2 * sg + 1;
    const bool hasB = gB < p.ncg;
    const int oA = goff[gA];
    const int d = hasB ? goff[gB] - oA : 0;
    int base[RQ];
#pragma unroll
    for (int i = 0; i < RQ; i++) base[i] = (rbase + 32 * i) * (int)p.S + oA + woff;
    float2 acc[RQ][8];
#pragma unroll
    for (int i = 0; i < RQ; i++)
#pragma unroll
      for (int jj = 0; jj < 8; jj++) acc[i][jj] = make_float2(0.f, 0.f);
    const TV *tA = table + gA * p.span;
    const TV *tB = table + (hasB ? gB : gA) * p.span;
    const int e1 = hasB ? min(d, p.span) : p.span;
#pragma unroll 2
    for (int kk = 0; kk < e1; kk++) {
      const float4 a = *reinterpret_cast<const float4 *>(tA[kk].v);
      const float4 a0 = make_float4(a.x, a.x, a.y, a.y), a1 = make_float4(a.z, a.z, a.w, a.w);
#pragma unroll
      for (int i = 0; i < RQ; i++) {
        const float2 xv = cur[smem_idx<PAD>(base[i] + kk)];
        acc[i][0] = fma2(xv, make_float2(a0.x, a0.y), acc[i][0]);
        acc[i][1] = fma2(xv, make_float2(a0.z, a0.w), acc[i][1]);
        acc[i][2] = fma2(xv, make_float2(a1.x, a1.y), acc[i][2]);
        acc[i][3] = fma2(xv, make_float2(a1.z, a1.w), acc[i][3]);
      }
    }
    if (hasB) {
#pragma unroll 2
      for (int kk = d; kk < p.span; kk++) {
        const float4 a = *reinterpret_cast<const float4 *>(tA[kk].v);
        const float4 b = *reinterpret_cast<const float4 *>(tB[kk - d].v);
        const float4 a0 = make_float4(a.x, a.x, a.y, a.y), a1 = make_float4(a.z, a.z, a.w, a.w);
        const float4 b0 = make_float4(b.x, b.x, b.y, b.y), b1 = make_float4(b.z, b.z, b.w, b.w);
#pragma unroll
        for (int i = 0; i < RQ; i++) {
          const float2 xv = cur[smem_idx<PAD>(base[i] + kk)];
          acc[i][0] = fma2(xv, make_float2(a0.x, a0.y), acc[i][0]);
          acc[i][1] = fma2(xv, make_float2(a0.z, a0.w), acc[i][1]);
          acc[i][2] = fma2(xv, make_float2(a1.x, a1.y), acc[i][2]);
          acc[i][3] = fma2(xv, make_float2(a1.z, a1.w), acc[i][3]);
          acc[i][4] = fma2(xv, make_float2(b0.x, b0.y), acc[i][4]);
          acc[i][5] = fma2(xv, make_float2(b0.z, b0.w), acc[i][5]);
          acc[i][6] = fma2(xv, make_float2(b1.x, b1.y), acc[i][6]);
          acc[i][7] = fma2(xv, make_float2(b1.z, b1.w), acc[i][7]);
        }
      }
#pragma unroll 2
      for (int kk = max(p.span, d); kk < d + p.span; kk++) {
        const float4 b = *reinterpret_cast<const float4 *>(tB[kk - d].v);
        const float4 b0 = make_float4(b.x, b.x, b.y, b.y), b1 = make_float4(b.z, b.z, b.w, b.w);
#pragma unroll
        for (int i = 0; i < RQ; i++) {
          const float2 xv = cur[smem_idx<PAD>(base[i] + kk)];
          acc[i][4] = fma2(xv, make_float2(b0.x, b0.y), acc[i][4]);
          acc[i][5] = fma2(xv, make_float2(b0.z, b0.w), acc[i][5]);
          acc[i][6] = fma2(xv, make_float2(b1.x, b1.y), acc[i][6]);
          acc[i][7] = fma2(xv, make_float2(b1.z, b1.w), acc[i][7]);
        }
      }
    }
    c2_store_rows<RQ>(p, acc, sg, q0, rbase, lane, sc, orow, os);
  }
}

// Paired form of the window (even row strides): 16-byte units of two complex samples.  PAD =
// 20 is the plain layout (S/2 odd: the 8 lanes of a quarter-warp, which share one 128-byte
// wavefront of 16-byte loads, hit 8 different units mod 8); PAD = 20 + t, t = ctz(S/2) (1..7),
// XORs the low min(t, 3) bits of the unit index with the bits from max(t, 3) up, a
// permutation inside each block of 8 units that is conflict-free for those strides.
template <int PAD>
__device__ __forceinline__ int unit_idx(int u) {
  if constexpr (PAD > 20) {
    constexpr int t = PAD - 20, sh = t > 3 ? t : 3, m = (1 << (t < 3 ? t : 3)) - 1;
    return u ^ ((u >> sh) & m);
  } else {
    return u;
  }
}

// cp.async of one 16-byte unit reading `src_bytes` (0, 8 or 16) of it, zeros for the rest.
__device__ __forceinline__ void cp_async16_part(void *smem_dst, const void *gmem_src, int src_bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(tc::smem_u32(smem_dst)), "l"(gmem_src),
               "r"(src_bytes)
               : "memory");
}

// cp.async completion on an mbarrier: the barrier's pending count is raised by one now and
// lowered again once every cp.async this thread issued before it has landed.
__device__ __forceinline__ void cp_async_mbar_arrive_inc(uint64_t *bar) {
  asm volatile("cp.async.mbarrier.arrive.shared::cta.b64 [%0];" ::"r"(tc::smem_u32(bar)) : "memory");
}

// The paired walk of rowtile_compute_c2: every band starts at an even k and the row stride is
// even, so each row reads samples k and k+1 with one 16-byte load and the loop runs two k a
// step — half the window loads and index arithmetic for the same f32x2 FMAs, in the same
// order (a leading zero tap adds +-0).  The window is addressed in units of two samples.
template <int RQ, int PAD>
__device__ __forceinline__ void rowtile_compute_c2pair(const RsParams &p, const float2 *cur,
                                                       const unsigned char *table_raw, float2 *orow, int64_t q0,
                                                       int wr, int wc, int lane, float scale, OutStage &os) {
  using TV = TapVec<float, false>;
  const TV *table = reinterpret_cast<const TV *>(table_raw);
  const int *goff = tap_goff(p, table_raw, sizeof(TV));
  const float4 *cu = reinterpret_cast<const float4 *>(cur);
  const int nsg = (p.ncg + 1) / 2;
  const int rbase = wr * 32 * RQ + lane;
  const float2 sc = make_float2(scale, scale);
  const int S2 = (int)(p.S >> 1);
  for (int sg = wc; sg < nsg; sg += p.WC) {
    const int gA = 2 * sg, gB = 2 * sg + 1;
    const bool hasB = gB < p.ncg;
    const int oA = goff[gA];               // even
    const int d = hasB ? goff[gB] - oA : 0;  // even
    int ub[RQ];                            // unit of each row's band start
#pragma unroll
    for (int i = 0; i < RQ; i++) ub[i] = (rbase + 32 * i) * S2 + (oA >> 1);
    float2 acc[RQ][8];
#pragma unroll
    for (int i = 0; i < RQ; i++)
#pragma unroll
      for (int jj = 0; jj < 8; jj++) acc[i][jj] = make_float2(0.f, 0.f);
    const TV *tA = table + gA * p.span;
    const TV *tB = table + (hasB ? gB : gA) * p.span;
    const int e1 = hasB ? min(d, p.span) : p.span;  // even: span and d are
    for (int kk = 0; kk < e1; kk += 2) {
      const float4 a = *reinterpret_cast<const float4 *>(tA[kk].v);
      const float4 a2 = *reinterpret_cast<const float4 *>(tA[kk + 1].v);
#pragma unroll
      for (int i = 0; i < RQ; i++) {
        const float4 xv = cu[unit_idx<PAD>(ub[i] + (kk >> 1))];
        const float2 x0 = make_float2(xv.x, xv.y), x1 = make_float2(xv.z, xv.w);
        acc[i][0] = fma2(x0, make_float2(a.x, a.x), acc[i][0]);
        acc[i][1] = fma2(x0, make_float2(a.y, a.y), acc[i][1]);
        acc[i][2] = fma2(x0, make_float2(a.z, a.z), acc[i][2]);
        acc[i][3] = fma2(x0, make_float2(a.w, a.w), acc[i][3]);
        acc[i][0] = fma2(x1, make_float2(a2.x, a2.x), acc[i][0]);
        acc[i][1] = fma2(x1, make_float2(a2.y, a2.y), acc[i][1]);
        acc[i][2] = fma2(x1, make_float2(a2.z, a2.z), acc[i][2]);
        acc[i][3] = fma2(x1, make_float2(a2.w, a2.w), acc[i][3]);
      }
    }
    if (hasB) {
      for (int kk = d; kk < p.span; kk += 2) {
        const float4 a = *reinterpret_cast<const float4 *>(tA[kk].v);
        const float4 a2 = *reinterpret_cast<const float4 *>(tA[kk + 1].v);
        const float4 b = *reinterpret_cast<const float4 *>(tB[kk - d].v);
        const float4 b2 = *reinterpret_cast<const float4 *>(tB[kk - d + 1].v);
#pragma unroll
        for (int i = 0; i < RQ; i++) {
          const float4 xv = cu[unit_idx<PAD>(ub[i] + (kk >> 1))];
          const float2 x0 = make_float2(xv.x, xv.y), x1 = make_float2(xv.z, xv.w);
          acc[i][0] = fma2(x0, make_float2(a.x, a.x), acc[i][0]);
          acc[i][1] = fma2(x0, make_float2(a.y, a.y), acc[i][1]);
          acc[i][2] = fma2(x0, make_float2(a.z, a.z), acc[i][2]);
          acc[i][3] = fma2(x0, make_float2(a.w, a.w), acc[i][3]);
          acc[i][4] = fma2(x0, make_float2(b.x, b.x), acc[i][4]);
          acc[i][5] = fma2(x0, make_float2(b.y, b.y), acc[i][5]);
          acc[i][6] = fma2(x0, make_float2(b.z, b.z), acc[i][6]);
          acc[i][7] = fma2(x0, make_float2(b.w, b.w), acc[i][7]);
          acc[i][0] = fma2(x1, make_float2(a2.x, a2.x), acc[i][0]);
          acc[i][1] = fma2(x1, make_float2(a2.y, a2.y), acc[i][1]);
          acc[i][2] = fma2(x1, make_float2(a2.z, a2.z), acc[i][2]);
          acc[i][3] = fma2(x1, make_float2(a2.w, a2.w), acc[i][3]);
          acc[i][4] = fma2(x1, make_float2(b2.x, b2.x), acc[i][4]);
          acc[i][5] = fma2(x1, make_float2(b2.y, b2.y), acc[i][5]);
          acc[i][6] = fma2(x1, make_float2(b2.z, b2.z), acc[i][6]);
          acc[i][7] = fma2(x1, make_float2(b2.w, b2.w), acc[i][7]);
        }
      }
      for (int kk = max(p.span, d); kk < d + p.span; kk += 2) {
        const float4 b = *reinterpret_cast<const float4 *>(tB[kk - d].v);
        const float4 b2 = *reinterpret_cast<const float4 *>(tB[kk - d + 1].v);
#pragma unroll
        for (int i = 0; i < RQ; i++) {
          const float4 xv = cu[unit_idx<PAD>(ub[i] + (kk >> 1))];
          const float2 x0 = make_float2(xv.x, xv.y), x1 = make_float2(xv.z, xv.w);
          acc[i][4] = fma2(x0, make_float2(b.x, b.x), acc[i][4]);
          acc[i][5] = fma2(x0, make_float2(b.y, b.y), acc[i][5]);
          acc[i][6] = fma2(x0, make_float2(b.z, b.z), acc[i][6]);
          acc[i][7] = fma2(x0, make_float2(b.w, b.w), acc[i][7]);
          acc[i][4] = fma2(x1, make_float2(b2.x, b2.x), acc[i][4]);
          acc[i][5] = fma2(x1, make_float2(b2.y, b2.y), acc[i][5]);
          acc[i][6] = fma2(x1, make_float2(b2.z, b2.z), acc[i][6]);
          acc[i][7] = fma2(x1, make_float2(b2.w, b2.w), acc[i][7]);
        }
      }
    }
    c2_store_rows<RQ>(p, acc, sg, q0, rbase, lane, sc, orow, os);
  }
}

// Real float signal x real float taps: the generic walk with each accumulator a pair of
// adjacent phases, updated by one f32x2 FMA against (x, x) and two taps of one 16-byte tap
// load (each lane is exactly the scalar fma of the generic form, so results are unchanged):
// half the FMA instructions of the scalar form.  Outputs leave as two 16-byte stores per row
// where they are whole and aligned.
template <int RQ, int PAD>
__device__ __forceinline__ void rowtile_compute_r2(const RsParams &p, const float *cur, const unsigned char *table_raw,
                                                   float *orow, int64_t q0, int wr, int wc, int lane, float scale,
                                                   int woff) {
  using TV = TapVec<float, false>;
  const TV *table = reinterpret_cast<const TV *>(table_raw);
  const int *goff = tap_goff(p, table_raw, sizeof(TV));
  const int nsg = (p.ncg + 1) / 2;
  const int rbase = wr * 32 * RQ + lane;
  const float2 sc = make_float2(scale, scale);
  const int Nt = (int)p.Nt;
  for (int sg = wc; sg < nsg; sg += p.WC) {
    const int gA = 2 * sg, gB = 2 * sg + 1;
    const bool hasB = gB < p.ncg;
    const int oA = goff[gA];
    const int d = hasB ? goff[gB] - oA : 0;
    int base[RQ];
#pragma unroll
    for (int i = 0; i < RQ; i++) base[i] = (rbase + 32 * i) * (int)p.S + oA + woff;
    float2 acc[RQ][4];  // phase pairs (0,1) (2,3) of band A, (4,5) (6,7) of band B
#pragma unroll
    for (int i = 0; i < RQ; i++)
#pragma unroll
      for (int jj = 0; jj < 4; jj++) acc[i][jj] = make_float2(0.f, 0.f);
    const TV *tA = table + gA * p.span;
    const TV *tB = table + (hasB ? gB : gA) * p.span;
    const int e1 = hasB ? min(d, p.span) : p.span;
#pragma unroll 2
    for (int kk = 0; kk < e1; kk++) {
      const float4 a = *reinterpret_cast<const float4 *>(tA[kk].v);
#pragma unroll
      for (int i = 0; i < RQ; i++) {
        const float xv = cur[smem_idx<PAD>(base[i] + kk)];
        const float2 x2 = make_float2(xv, xv);
        acc[i][0] = fma2(x2, make_float2(a.x, a.y), acc[i][0]);
        acc[i][1] = fma2(x2, make_float2(a.z, a.w), acc[i][1]);
      }
    }
    if (hasB) {
#pragma unroll 2
      for (int kk = d; kk < p.span; kk++) {
        const float4 a = *reinterpret_cast<const float4 *>(tA[kk].v);
        const float4 b = *reinterpret_cast<const float4 *>(tB[kk - d].v);
#pragma unroll
        for (int i = 0; i < RQ; i++) {
          const float xv = cur[smem_idx<PAD>(base[i] + kk)];
          const float2 x2 = make_float2(xv, xv);
          acc[i][0] = fma2(x2, make_float2(a.x, a.y), acc[i][0]);
          acc[i][1] = fma2(x2, make_float2(a.z, a.w), acc[i][1]);
          acc[i][2] = fma2(x2, make_float2(b.x, b.y), acc[i][2]);
          acc[i][3] = fma2(x2, make_float2(b.z, b.w), acc[i][3]);
        }
      }
#pragma unroll 2
      for (int kk = max(p.span, d); kk < d + p.span; kk++) {
        const float4 b = *reinterpret_cast<const float4 *>(tB[kk - d].v);
#pragma unroll
        for (int i = 0; i < RQ; i++) {
          const float xv = cur[smem_idx<PAD>(base[i] + kk)];
          const float2 x2 = make_float2(xv, xv);
          acc[i][2] = fma2(x2, make_float2(b.x, b.y), acc[i][2]);
          acc[i][3] = fma2(x2, make_float2(b.z, b.w), acc[i][3]);
        }
      }
    }
    const int j0 = 8 * sg;
    const int ncol = min(8, Nt - j0);
#pragma unroll
    for (int i = 0; i < RQ; i++) {
      const int64_t n0 = (q0 + rbase + 32 * i) * p.Nt + j0;
      const int64_t left = p.out_len - n0;
      const int nv = left < ncol ? (left > 0 ? (int)left : 0) : ncol;
      float *dst = orow + n0;
      float v[8];
#pragma unroll
      for (int u = 0; u < 4; u++) {
        const float2 t = mul2(acc[i][u], sc);
        v[2 * u] = t.x;
        v[2 * u + 1] = t.y;
      }
      if (nv == 8 && ((reinterpret_cast<uintptr_t>(dst) & 15) == 0)) {
        reinterpret_cast<float4 *>(dst)[0] = make_float4(v[0], v[1], v[2], v[3]);
        reinterpret_cast<float4 *>(dst)[1] = make_float4(v[4], v[5], v[6], v[7]);
      } else {
#pragma unroll
        for (int jj = 0; jj < 8; jj++)
          if (jj < nv) dst[jj] = v[jj];
      }
    }
  }
}

// One tile of QC rows starting at row q0: every warp (wr, wc) accumulates its 8-phase
// super-groups for RQ rows per lane and stores them (masked by Nt and out_len).
// woff: where element 0 of the tile's logical window sits in `cur` (the window copy may
// start up to 15 bytes early so that it is 16-byte aligned).
template <typename T, bool XC, bool HC, int RQ, int PAD>
__device__ __forceinline__ void rowtile_compute(const RsParams &p, const typename val_of<T, XC>::type *cur,
                                                const unsigned char *table_raw,
                                                typename val_of<T, XC || HC>::type *orow, int64_t q0, int wr, int wc,
                                                int lane, T scale, int woff, OutStage &os) {
  if constexpr (std::is_same<T, float>::value && XC && !HC) {
    if constexpr (PAD >= 20)
      rowtile_compute_c2pair<RQ, PAD>(p, cur, table_raw, orow, q0, wr, wc, lane, scale, os);
    else
      rowtile_compute_c2<RQ, PAD>(p, cur, table_raw, orow, q0, wr, wc, lane, scale, woff, os);
  } else if constexpr (std::is_same<T, float>::value && !XC && !HC) {
    rowtile_compute_r2<RQ, PAD>(p, cur, table_raw, orow, q0, wr, wc, lane, scale, woff);
  } else {
    using XT = typename val_of<T, XC>::type;
    constexpr bool OC = XC || HC;
    const TapVec<T, HC> *table = reinterpret_cast<const TapVec<T, HC> *>(table_raw);
    const int *goff = tap_goff(p, table_raw, sizeof(TapVec<T, HC>));
    const int nsg = (p.ncg + 1) / 2;
    const int rbase = wr * 32 * RQ + lane;  // local row of slice i is rbase + 32*i
    for (int sg = wc; sg < nsg; sg += p.WC) {
      const int gA = 2 * sg, gB = 2 * sg + 1;
      const bool hasB = gB < p.ncg;
      const int oA = goff[gA];
      const int d = hasB ? goff[gB] - oA : 0;  // band B starts d samples after band A
      int base[RQ];
#pragma unroll
      for (int i = 0; i < RQ; i++) base[i] = (rbase + 32 * i) * (int)p.S + oA + woff;
      Acc<T, OC> acc[RQ][8];
#pragma unroll
      for (int i = 0; i < RQ; i++)
#pragma unroll
        for (int jj = 0; jj < 8; jj++) acc[i][jj].zero();
      const TapVec<T, HC> *tA = table + gA * p.span;
      const TapVec<T, HC> *tB = table + (hasB ? gB : gA) * p.span;
      // range 1: band A only
      const int e1 = hasB ? min(d, p.span) : p.span;
#pragma unroll 2
      for (int kk = 0; kk < e1; kk++) {
        const TapVec<T, HC> t = tA[kk];
#pragma unroll
        for (int i = 0; i < RQ; i++) {
          const XT xv = cur[smem_idx<PAD>(base[i] + kk)];
#pragma unroll
          for (int jj = 0; jj < 4; jj++) mac<T, XC, HC>(acc[i][jj], xv, t.v[jj]);
        }
      }
      if (hasB) {
        // range 2: both bands
#pragma unroll 2
        for (int kk = d; kk < p.span; kk++) {
          const TapVec<T, HC> ta = tA[kk];
          const TapVec<T, HC> tb = tB[kk - d];
#pragma unroll
          for (int i = 0; i < RQ; i++) {
            const XT xv = cur[smem_idx<PAD>(base[i] + kk)];
#pragma unroll
            for (int jj = 0; jj < 4; jj++) mac<T, XC, HC>(acc[i][jj], xv, ta.v[jj]);
#pragma unroll
            for (int jj = 0; jj < 4; jj++) mac<T, XC, HC>(acc[i][4 + jj], xv, tb.v[jj]);
          }
        }
        // range 3: band B only
#pragma unroll 2
        for (int kk = max(p.span, d); kk < d + p.span; kk++) {
          const TapVec<T, HC> tb = tB[kk - d];
#pragma unroll
          for (int i = 0; i < RQ; i++) {
            const XT xv = cur[smem_idx<PAD>(base[i] + kk)];
#pragma unroll
            for (int jj = 0; jj < 4; jj++) mac<T, XC, HC>(acc[i][4 + jj], xv, tb.v[jj]);
          }
        }
      }
      const int j0 = 8 * sg;
      const int ncol = min(8, (int)p.Nt - j0);
#pragma unroll
      for (int i = 0; i < RQ; i++) {
        const int64_t n0 = (q0 + rbase + 32 * i) * p.Nt + j0;
        const int64_t left = p.out_len - n0;
        const int nv = left < ncol ? (left > 0 ? (int)left : 0) : ncol;
#pragma unroll
        for (int jj = 0; jj < 8; jj++)
          if (jj < nv) orow[n0 + jj] = pack<T, OC>(acc[i][jj], scale);
      }
    }
  }
}

// Same, with every output stored directly (no staging).
template <typename T, bool XC, bool HC, int RQ, int PAD>
__device__ __forceinline__ void rowtile_compute(const RsParams &p, const typename val_of<T, XC>::type *cur,
                                                const unsigned char *table_raw,
                                                typename val_of<T, XC || HC>::type *orow, int64_t q0, int wr, int wc,
                                                int lane, T scale, int woff) {
  OutStage none{nullptr, nullptr, 0, 0};
  rowtile_compute<T, XC, HC, RQ, PAD>(p, cur, table_raw, orow, q0, wr, wc, lane, scale, woff, none);
}

// 256 threads (8 warps) per CTA, or up to 512 (one row slice of 9..16 column warps) with one
// or two rows per thread.
template <typename T, bool XC, bool HC, int RQ, int PAD>
__global__ void __launch_bounds__(RQ <= 2 ? 512 : 256)
    resample_rowtile(const RsParams p, const __grid_constant__ CUtensorMap omap) {
  using XT = typename val_of<T, XC>::type;
  using HT = typename val_of<T, HC>::type;
  using OT = typename val_of<T, XC || HC>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned char *table = smem_raw;
  const size_t table_bytes = tap_table_bytes<T, XC, HC>(p.ncg, p.span);
  XT *xbuf0 = reinterpret_cast<XT *>(smem_raw + table_bytes);
  XT *xbuf1 = xbuf0 + p.win_alloc;

  const int tid = threadIdx.x;
  const HT *hp = reinterpret_cast<const HT *>(p.h);
  const XT *xp = reinterpret_cast<const XT *>(p.x);
  OT *op = reinterpret_cast<OT *>(p.out);

  if (tid == 0) GBFIR_TC_TRACE(3, 0, 1);
  // (odd row strides build the table after issuing the first window copy)
  if constexpr (PAD > 0 && PAD != 20) build_tap_table<T, XC, HC>(p, hp, table, tid, blockDim.x);

  const int wid = tid >> 5, lane = tid & 31;
  const int wr = wid / p.WC, wc = wid - wr * p.WC;
  const T scale = T(p.scale);
  const bool dbuf = p.nbuf == 2;
  // TMA-store epilogue: each warp's two staging buffers, 1024-byte aligned (the swizzle
  // pattern repeats every 512 bytes)
  OutStage ostage{&omap, nullptr, 0, 0};
  if constexpr (std::is_same<T, float>::value && XC && !HC) {
    if (p.ostore) {
      unsigned char *base = smem_raw + p.stg_off;
      base += (1024 - (tc::smem_u32(base) & 1023)) & 1023;
      ostage.buf = base + wid * (p.ost_single ? 2048 : 4096);
    }
  }

  if constexpr (PAD > 0 && PAD != 20) {
    // Even row stride: the window is stored in a bank-conflict-free layout (an element
    // permutation inside blocks of 16 or 32, a unit permutation of the paired walk, or one pad per
    // 16), which a bulk copy cannot produce; stage it with cp.async (zero-filled outside the
    // signal).
    auto issue_loads = [&](int64_t tile, XT *buf) {
      const int64_t b = tile_row(p, tile);
      const int64_t q0 = (tile - b * p.tiles_per_row) * p.QC;
      const int64_t xs0 = q0 * p.S + p.kmin;
      const XT *row = xp + b * p.x_bstride;
      if constexpr (PAD > 20 && PAD < 30) {
        // units of two samples (xs0 is even); the last may hold one sample of the signal
        float4 *bu = reinterpret_cast<float4 *>(buf);
        const int nu = (p.win + 1) >> 1;
        for (int u = tid; u < nu; u += blockDim.x) {
          const int64_t gi = xs0 + 2 * u;
          const int nb = (gi >= 0 && gi < p.N) ? (gi + 1 < p.N ? 16 : 8) : 0;
          cp_async16_part(&bu[unit_idx<PAD>(u)], nb ? (const void *)(row + gi) : (const void *)row, nb);
        }
      } else if (xs0 >= 0 && xs0 + p.win <= p.N) {
        const XT *src = row + xs0;
        for (int e = tid; e < p.win; e += blockDim.x) cp_async_zfill<sizeof(XT)>(&buf[smem_idx<PAD>(e)], src + e, true);
      } else {
        for (int e = tid; e < p.win; e += blockDim.x) {
          const int64_t gi = xs0 + e;
          const bool ok = gi >= 0 && gi < p.N;
          cp_async_zfill<sizeof(XT)>(&buf[smem_idx<PAD>(e)], ok ? (const void *)(row + gi) : (const void *)row, ok);
        }
      }
    };

    int64_t tile = blockIdx.x;
    if (tile < p.ntiles) issue_loads(tile, xbuf0);
    cp_async_commit();
    for (int it = 0; tile < p.ntiles; tile += gridDim.x, ++it) {
      XT *cur = (dbuf && (it & 1)) ? xbuf1 : xbuf0;
      const int64_t next = tile + gridDim.x;
      if (dbuf) {
        if (next < p.ntiles) issue_loads(next, (it & 1) ? xbuf0 : xbuf1);
        cp_async_commit();
        cp_async_wait<1>();
      } else {
        cp_async_wait<0>();
      }
      __syncthreads();

      const int64_t b = tile_row(p, tile);
      const int64_t q0 = (tile - b * p.tiles_per_row) * p.QC;
      OT *orow = op + b * p.out_bstride;
      ostage.b = b;
      rowtile_compute<T, XC, HC, RQ, PAD>(p, cur, table, orow, q0, wr, wc, lane, scale, 0, ostage);
      __syncthreads();
      if (!dbuf && next < p.ntiles) {
        issue_loads(next, xbuf0);
        cp_async_commit();
      }
    }
    cp_async_wait<0>();
  } else {
    // Odd row stride: the window is one contiguous run of the signal, brought in by one
    // TMA bulk copy (thread 0) that completes on an mbarrier.  The copy starts at the
    // 16-byte boundary at or below the window start (`a` elements early) and covers a
    // multiple of 16 bytes; windows that reach past either end of the signal are staged
    // element by element (cp.async, zeros outside) on the same barrier instead.
    constexpr int ES = (int)sizeof(XT), G = 16 / ES;
    __shared__ uint64_t s_bar[2];
    __shared__ int s_ok;
    if (tid == 0) {
      tc::mbar_init(&s_bar[0], 1);
      tc::mbar_init(&s_bar[1], 1);
      tc::mbar_fence_init();
    }
    __syncthreads();
    // tile t: its batch row, first row, and the elements its window copy starts early; every
    // thread computes the same values once per tile (for the copy one tile ahead, then the
    // compute)
    struct Origin {
      int64_t b, q0, w0;
      int a;
    };
    auto origin = [&](int64_t t) -> Origin {
      Origin o;
      o.b = tile_row(p, t);
      o.q0 = (t - o.b * p.tiles_per_row) * p.QC;
      const int64_t xs0 = o.q0 * p.S + p.kmin;
      o.a = (int)((reinterpret_cast<uintptr_t>(xp + o.b * p.x_bstride + xs0) & 15) / ES);
      o.w0 = xs0 - o.a;
      return o;
    };
    auto issue_window = [&](const Origin &o, XT *buf, uint64_t *bar, int ts) {
      const int64_t w0 = o.w0;
      const int64_t wl = (p.win + o.a + G - 1) / G * G;
      const XT *row = xp + o.b * p.x_bstride;
      // the bulk copy's alignment rules hold by construction; check them anyway and take
      // the element path if they do not
      const bool aligned = ((reinterpret_cast<uintptr_t>(row + w0) | (uintptr_t)tc::smem_u32(buf)) & 15) == 0;
      if (aligned && w0 >= 0 && w0 + wl <= p.N) {
        if (tid == 0) {
          const uint32_t bytes = (uint32_t)(wl * ES);
          GBFIR_TC_TRACE(2, ts, 1);
          tc::fence_async_smem();
          GBFIR_TC_TRACE(2, ts, 2);
          tc::mbar_arrive_expect_tx(bar, bytes);
          tc::bulk_copy_g2s(buf, row + w0, bytes, bar);
          GBFIR_TC_TRACE(2, ts, 3);
        }
      } else {
        // one cp.async per sample (zeros outside the signal), each thread's copies completing
        // on the barrier; the barrier's one expected arrival comes from thread 0 once every
        // thread has registered its copies, so the window lands while the CTA computes
        for (int64_t e = tid; e < wl; e += blockDim.x) {
          const int64_t gi = w0 + e;
          const bool ok = gi >= 0 && gi < p.N;
          cp_async_zfill<ES>(&buf[e], ok ? (const void *)(row + gi) : (const void *)row, ok);
        }
        cp_async_mbar_arrive_inc(bar);
        __syncthreads();
        if (tid == 0) tc::mbar_arrive_plain(bar);
      }
    };

    int64_t tile = blockIdx.x;
    if (tid == 0) GBFIR_TC_TRACE(3, 0, 0);
    Origin oc{};
    if (tile < p.ntiles) {
      oc = origin(tile);
      issue_window(oc, xbuf0, &s_bar[0], 16);
    }
    // the table is complete before any thread reads it: the loop's first barrier follows
    build_tap_table<T, XC, HC>(p, hp, table, tid, blockDim.x);
    for (int it = 0; tile < p.ntiles; tile += gridDim.x, ++it) {
      if (tid == 0) GBFIR_TC_TRACE(2, it, 0);
      const int k = dbuf ? (it & 1) : 0;
      XT *cur = k ? xbuf1 : xbuf0;
      const uint32_t parity = dbuf ? ((it >> 1) & 1) : (it & 1);
      const int64_t next = tile + gridDim.x;
      Origin on{};
      if (next < p.ntiles) on = origin(next);
      // the other buffer was released by the barrier that ended the previous tile
      if (dbuf && next < p.ntiles) issue_window(on, k ? xbuf0 : xbuf1, &s_bar[k ^ 1], it);
      if (tid == 0) GBFIR_TC_TRACE(0, it, 0);
      if (tid == 0) s_ok = tc::mbar_wait(&s_bar[k], parity) ? 1 : 0;
      __syncthreads();
      if (tid == 0) GBFIR_TC_TRACE(0, it, 1);
      if (!s_ok) {
        // a copy that never completed: record it and stop; give the copies in flight a
        // bounded chance to land before the CTA (and its shared memory) goes away
        if (tid == 0) {
          atomicExch(&g_rowtile_status, 1);
          (void)tc::mbar_wait(&s_bar[k], parity);
          if (dbuf) (void)tc::mbar_wait(&s_bar[k ^ 1], parity);
        }
        __syncthreads();
        break;
      }
      OT *orow = op + oc.b * p.out_bstride;
      ostage.b = oc.b;
      rowtile_compute<T, XC, HC, RQ, PAD>(p, cur, table, orow, oc.q0, wr, wc, lane, scale, oc.a, ostage);
      if (tid == 0) GBFIR_TC_TRACE(0, it, 2);
      if (lane == 0 && wid == (int)(blockDim.x >> 5) - 1) GBFIR_TC_TRACE(1, it, 2);
      __syncthreads();
      if (tid == 0) GBFIR_TC_TRACE(0, it, 3);
      if (!dbuf && next < p.ntiles) issue_window(on, xbuf0, &s_bar[0], it);
      oc = on;
    }
  }
  // the staged boxes are read and written before the CTA's shared memory goes away
  if (ostage.buf && lane == 0) tc::bulk_wait_all();
}

// cp.async completion on an mbarrier: the arrival fires once every cp.async this thread issued
// before it has landed (.noinc: the barrier's expected count includes the arrival).
__device__ __forceinline__ void cp_async_mbar_arrive(uint64_t *bar) {
  asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(tc::smem_u32(bar)) : "memory");
}


constexpr int kRingMax = 4;       // window slots of the ring form
constexpr int kRingStageMax = 2;  // staging warps of the ring form (ring_stages)
constexpr int kRingThreads = 32 * (kRingStageMax + 16);  // + up to 16 compute warps

// Staging warps of the ring form for a window layout: two where the window is one bulk copy
// (PAD 0, 20), one where cp.async stages it per sample or unit.  Measured on the fixed-tile
// step (two runs each, same box): 3/2 (PAD 22) 0.302 ms with one, 0.322 with two; 4/5 (PAD
// 20) 0.248 with one, 0.239 with two.  A count chosen at run time instead cost 4-13 %.
__host__ __device__ constexpr int ring_stages(int pad) { return (pad == 0 || pad == 20) ? 2 : 1; }

// Ring form of the row tile (complex float signal, real taps; one CTA per SM).  The first
// ring_stages(PAD) warps stage the windows of the CTA's tiles into a ring of p.nbuf (3 or 4)
// slots, up to p.nbuf - 1 tiles ahead of the compute warps — one TMA bulk copy per window for an odd row stride or the plain paired layout (PAD
// 0, 20), cp.async into the conflict-free layouts otherwise (per sample for PAD 11..17, per
// 16-byte unit for PAD 21..27; two staging warps take alternate 32-element groups) — and
// the other warps compute as in the two-buffer form (PAD >= 20: the paired walk).  A full and an empty
// mbarrier per slot take the place of the CTA-wide barriers, so a compute warp waits only
// when the copies fall behind and the next windows are already in flight while a tile is
// computed.  Every wait is bounded; one that gives up records the status read by
// rowtile_status_take() and ends the CTA's loop.
template <int RQ, int PAD>
__global__ void __launch_bounds__(kRingThreads, 1)
    resample_rowtile_ring(const RsParams p, const __grid_constant__ CUtensorMap omap) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ uint64_t full[kRingMax], empty[kRingMax];
  __shared__ int s_fail;
  unsigned char *table = smem_raw;
  float2 *xbuf0 = reinterpret_cast<float2 *>(smem_raw + tap_table_bytes<float, true, false>(p.ncg, p.span));
  const int tid = threadIdx.x, wid = tid >> 5, lane = tid & 31;
  constexpr int nstage = ring_stages(PAD);
  const int ncw = (int)(blockDim.x >> 5) - nstage;
  const int R = p.nbuf;
  const float2 *xp = reinterpret_cast<const float2 *>(p.x);
  if (tid == 0) GBFIR_TC_TRACE(3, 0, 1);
  build_tap_table<float, true, false>(p, reinterpret_cast<const float *>(p.h), table, tid, blockDim.x);
  if (tid == 0) {
    for (int i = 0; i < R; i++) {
      tc::mbar_init(&full[i], 32 * nstage);  // every lane of the staging warps
      tc::mbar_init(&empty[i], ncw); // lane 0 of every compute warp
    }
    s_fail = 0;
    tc::mbar_fence_init();
  }
  __syncthreads();
  // tile t: its batch row, first row, and (odd strides) the elements its window copy starts
  // early so that the bulk copy is 16-byte aligned
  auto origin = [&](int64_t t, int64_t &b, int64_t &q0, int64_t &w0) -> int {
    b = tile_row(p, t);
    q0 = (t - b * p.tiles_per_row) * p.QC;
    const int64_t xs0 = q0 * p.S + p.kmin;
    int a = 0;
    if constexpr (PAD == 0) a = (int)((reinterpret_cast<uintptr_t>(xp + b * p.x_bstride + xs0) & 15) / 8);
    w0 = xs0 - a;
    return a;
  };

  if (tid == 0) GBFIR_TC_TRACE(3, 0, 0);
  if (wid < nstage) {
    // ================= staging warps =================
    const int sl = wid * 32 + lane, nsl = 32 * nstage;  // this lane's share of a window
    int64_t n = 0;
    for (int64_t tile = blockIdx.x; tile < p.ntiles; tile += gridDim.x, ++n) {
      const int slot = (int)(n % R);
      if (sl == 0) GBFIR_TC_TRACE(0, (int)n, 0);
      if (n >= R) {
        int ok = 1;
        if (lane == 0) ok = tc::mbar_wait_sleep(&empty[slot], (uint32_t)((n / R - 1) & 1)) ? 1 : 0;
        if (!__shfl_sync(0xffffffffu, ok, 0)) {
          if (lane == 0) s_fail = 1;
          break;
        }
      }
      float2 *buf = xbuf0 + (size_t)slot * p.win_alloc;
      int64_t b, q0, w0;
      const int a = origin(tile, b, q0, w0);
      const float2 *row = xp + b * p.x_bstride;
      if constexpr (PAD > 20) {
        // units of two samples (w0 is even); the last may hold one sample of the signal
        float4 *bu = reinterpret_cast<float4 *>(buf);
        const int nu = (p.win + 1) >> 1;
        if (w0 >= 0 && w0 + 2 * (int64_t)nu <= p.N) {
          for (int u = sl; u < nu; u += nsl) cp_async16_part(&bu[unit_idx<PAD>(u)], row + w0 + 2 * u, 16);
        } else {
          for (int u = sl; u < nu; u += nsl) {
            const int64_t gi = w0 + 2 * u;
            const int nb = (gi >= 0 && gi < p.N) ? (gi + 1 < p.N ? 16 : 8) : 0;
            cp_async16_part(&bu[unit_idx<PAD>(u)], nb ? (const void *)(row + gi) : (const void *)row, nb);
          }
        }
        cp_async_mbar_arrive(&full[slot]);
      } else if constexpr (PAD > 0 && PAD != 20) {
        if (w0 >= 0 && w0 + p.win <= p.N) {
          for (int e = sl; e < p.win; e += nsl) cp_async_zfill<8>(&buf[smem_idx<PAD>(e)], row + w0 + e, true);
        } else {
          for (int e = sl; e < p.win; e += nsl) {
            const int64_t gi = w0 + e;
            const bool ok = gi >= 0 && gi < p.N;
            cp_async_zfill<8>(&buf[smem_idx<PAD>(e)], ok ? (const void *)(row + gi) : (const void *)row, ok);
          }
        }
        cp_async_mbar_arrive(&full[slot]);
      } else {
        const int64_t wl = (p.win + a + 1) / 2 * 2;  // whole 16-byte units
        const bool aligned = ((reinterpret_cast<uintptr_t>(row + w0) | (uintptr_t)tc::smem_u32(buf)) & 15) == 0;
        if (aligned && w0 >= 0 && w0 + wl <= p.N) {
          if (sl == 0) {
            const uint32_t bytes = (uint32_t)(wl * 8);
            tc::fence_async_smem();
            tc::mbar_arrive_expect_tx(&full[slot], bytes);
            tc::bulk_copy_g2s(buf, row + w0, bytes, &full[slot]);
          } else {
            tc::mbar_arrive_plain(&full[slot]);
          }
        } else {
          // one cp.async per sample (zeros outside the signal), each lane's arrival made when
          // its copies have landed, so the staging warps go on to the next slot at once
          for (int64_t e = sl; e < wl; e += nsl) {
            const int64_t gi = w0 + e;
            const bool ok = gi >= 0 && gi < p.N;
            cp_async_zfill<8>(&buf[e], ok ? (const void *)(row + gi) : (const void *)row, ok);
          }
          cp_async_mbar_arrive(&full[slot]);
        }
      }
      if (sl == 0) GBFIR_TC_TRACE(0, (int)n, 1);
    }
    cp_async_commit();  // the copies were never grouped: group them, then wait for all
    cp_async_wait<0>();
  } else {
    // ================= compute warps =================
    const int cw = wid - nstage;
    const int wr = p.WC <= 8 ? cw / p.WC : 0, wc = p.WC <= 8 ? cw - wr * p.WC : cw;
    const float scale = (float)p.scale;
    OutStage ostage{&omap, nullptr, 0, 0};
    if (p.ostore) {
      unsigned char *base = smem_raw + p.stg_off;
      base += (1024 - (tc::smem_u32(base) & 1023)) & 1023;
      ostage.buf = base + cw * 4096;
    }
    int64_t n = 0;
    for (int64_t tile = blockIdx.x; tile < p.ntiles; tile += gridDim.x, ++n) {
      const int slot = (int)(n % R);
      const int trole = cw == 0 ? 1 : cw == ncw - 1 ? 2 : -1;
      if (lane == 0 && trole > 0) GBFIR_TC_TRACE(trole, (int)n, 0);
      // every lane waits: its own acquire makes the window's bytes visible to it
      const bool ok = tc::mbar_wait_sleep(&full[slot], (uint32_t)((n / R) & 1));
      if (!__all_sync(0xffffffffu, ok)) {
        if (lane == 0) s_fail = 1;
        break;
      }
      if (lane == 0 && trole > 0) GBFIR_TC_TRACE(trole, (int)n, 1);
      int64_t b, q0, w0;
      const int a = origin(tile, b, q0, w0);
      ostage.b = b;
      if constexpr (PAD >= 20)
        rowtile_compute_c2pair<RQ, PAD>(p, xbuf0 + (size_t)slot * p.win_alloc, table,
                                        reinterpret_cast<float2 *>(p.out) + b * p.out_bstride, q0, wr, wc, lane, scale,
                                        ostage);
      else
        rowtile_compute_c2<RQ, PAD>(p, xbuf0 + (size_t)slot * p.win_alloc, table,
                                    reinterpret_cast<float2 *>(p.out) + b * p.out_bstride, q0, wr, wc, lane, scale, a,
                                    ostage);
      __syncwarp();
      if (lane == 0) tc::mbar_arrive_plain(&empty[slot]);
      if (lane == 0 && trole > 0) GBFIR_TC_TRACE(trole, (int)n, 2);
    }
    // the staged boxes are read before the CTA's shared memory goes away
    if (ostage.buf && lane == 0) tc::bulk_wait_all();
  }
  __syncthreads();
  if (s_fail && tid == 0) {
    atomicExch(&g_rowtile_status, 1);
    // copies a stopped loop left in flight: a bounded chance to land before the CTA ends
    for (int i = 0; i < R; i++) {
      (void)tc::mbar_wait(&full[i], 0);
      (void)tc::mbar_wait(&full[i], 1);
    }
  }
  __syncthreads();
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (the library does not
// link the driver, so it loads where no GPU driver is installed); null if unavailable.
using TensorMapEncodeFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                       const cuuint64_t *, const cuuint32_t *, const cuuint32_t *,
                                       CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion,
                                       CUtensorMapFloatOOBfill);
inline TensorMapEncodeFn tensor_map_encoder() {
  static TensorMapEncodeFn fn = [] {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      f = nullptr;
    return reinterpret_cast<TensorMapEncodeFn>(f);
  }();
  return fn;
}

// Host planning shared by the forward launch and the ragged planner.
struct RsGeom {
  int64_t up, down, Lo, c, Nt, S, kmin, kmax, rows;
  int32_t even, ncg, span;
};

inline RsGeom plan_geometry(int64_t up, int64_t down, int64_t L, int64_t out_len, int64_t G, int64_t c_override = -1,
                            bool odd_extend = true, bool pair = false) {
  RsGeom g{};
  g.up = up;
  g.down = down;
  g.even = odd_extend ? (L % 2) == 0 : 0;
  g.Lo = L + g.even;
  g.c = c_override >= 0 ? c_override : (g.Lo - 1) / 2;
  g.Nt = up * G;
  g.S = down * G;
  g.ncg = (int32_t)((g.Nt + 3) / 4);
  int64_t span = 1;
  for (int64_t grp = 0; grp < g.ncg; grp++) {
    const int64_t j0 = 4 * grp;
    const int64_t jl = std::min<int64_t>(j0 + 3, g.Nt - 1);
    const int64_t kl0 = band_start(g.c, grp, down, g.Lo, up, pair);
    const int64_t kh = floor_div(g.c + jl * down, up);
    span = std::max<int64_t>(span, kh - kl0 + 1);
  }
  span = (span + 1) & ~1LL;  // even, for the 2x unrolled band loop
  g.span = (int32_t)span;
  g.kmin = band_start(g.c, 0, down, g.Lo, up, pair);
  g.kmax = band_start(g.c, g.ncg - 1, down, g.Lo, up, pair) + span - 1;
  g.rows = (out_len + g.Nt - 1) / g.Nt;
  return g;
}

// Direct form for tap/rate combinations whose row tile does not fit in shared
// memory (very large up or down): one output per thread iteration,
//   out[m] = scale * sum_k in[k] * hh(c + m*dn - k*upk),  hh(t) = he(rev ? Lo-1-t : t),
// the input read through L1, the filter from shared memory when it fits.  With
// dn = down, upk = up, rev = 0 this is the MatX host loop (resample_poly.h:239-262).
template <typename T, bool XC, bool HC>
__global__ void __launch_bounds__(256) resample_direct(const RsParams p, int h_in_smem, int64_t batch) {
  using XT = typename val_of<T, XC>::type;
  using HT = typename val_of<T, HC>::type;
  using OT = typename val_of<T, XC || HC>::type;
  constexpr bool OC = XC || HC;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  HT *hs = reinterpret_cast<HT *>(smem_raw);
  const HT *hg = reinterpret_cast<const HT *>(p.h);
  const int64_t L = p.Lo - p.even;
  if (h_in_smem) {
    for (int64_t k = threadIdx.x; k < L; k += blockDim.x) hs[k] = hg[k];
    __syncthreads();
  }
  const HT *hh = h_in_smem ? hs : hg;
  const XT *xp = reinterpret_cast<const XT *>(p.x);
  OT *op = reinterpret_cast<OT *>(p.out);
  const int64_t total = p.out_len * batch;
  const T scale = T(p.scale);
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / p.out_len, m = e - b * p.out_len;
    const XT *row = xp + b * p.x_bstride;
    const int64_t a = p.c + m * p.down;
    int64_t k0 = ceil_div(a - p.Lo + 1, p.up), k1 = floor_div(a, p.up);
    if (k0 < 0) k0 = 0;
    if (k1 > p.N - 1) k1 = p.N - 1;
    Acc<T, OC> acc;
    acc.zero();
    for (int64_t k = k0; k <= k1; k++) {
      const int64_t t = a - k * p.up;
      const int64_t te = p.rev ? p.Lo - 1 - t : t;
      if (p.even && te == 0) continue;
      mac<T, XC, HC>(acc, row[k], hh[te - p.even]);
    }
    op[b * p.out_bstride + m] = pack<T, OC>(acc, scale);
  }
}

template <typename T, bool XC, bool HC, int RQ, int PAD>
inline int launch_rowtile(RsParams &p, const CUtensorMap &omap, size_t smem, cudaStream_t s, int threads) {
  auto fn = resample_rowtile<T, XC, HC, RQ, PAD>;
  int rc = ensure_smem((const void *)fn, smem, "resample_poly");
  if (rc) return rc;
  int occ = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, threads, smem);
  if (occ < 1) GBFIR_FAIL(GBFIR_ERR_NOT_SUPPORTED, "resample_poly: tile needs %zu B of shared memory", smem);
  int64_t grid = (int64_t)num_sms() * occ;
  if (grid > p.ntiles) grid = p.ntiles;
  fn<<<(unsigned)grid, (unsigned)threads, smem, s>>>(p, omap);
  return check_launch("resample_poly");
}

template <typename T, bool XC, bool HC, int PAD>
inline int dispatch_rq_pad(RsParams &p, const CUtensorMap &m, int rq, size_t smem, cudaStream_t s, int threads) {
  if (rq == 1) return launch_rowtile<T, XC, HC, 1, PAD>(p, m, smem, s, threads);
  if constexpr (sizeof(T) == 4) {
    if (rq == 2) return launch_rowtile<T, XC, HC, 2, PAD>(p, m, smem, s, threads);
    return launch_rowtile<T, XC, HC, 4, PAD>(p, m, smem, s, threads);
  }
  return launch_rowtile<T, XC, HC, 1, PAD>(p, m, smem, s, threads);
}

// pad: 0 (odd row stride), 4 (one pad per 16), or the XOR layouts 11..17 (complex float
// samples) and 31..37 (real float samples)
template <typename T, bool XC, bool HC>
inline int dispatch_rq(RsParams &p, const CUtensorMap &m, int rq, int pad, size_t smem, cudaStream_t s,
                       int threads) {
  if (pad == 0) return dispatch_rq_pad<T, XC, HC, 0>(p, m, rq, smem, s, threads);
  if constexpr (std::is_same<T, float>::value && !XC && !HC) {
    switch (pad) {
      case 31: return dispatch_rq_pad<T, XC, HC, 31>(p, m, rq, smem, s, threads);
      case 32: return dispatch_rq_pad<T, XC, HC, 32>(p, m, rq, smem, s, threads);
      case 33: return dispatch_rq_pad<T, XC, HC, 33>(p, m, rq, smem, s, threads);
      case 34: return dispatch_rq_pad<T, XC, HC, 34>(p, m, rq, smem, s, threads);
      case 35: return dispatch_rq_pad<T, XC, HC, 35>(p, m, rq, smem, s, threads);
      case 36: return dispatch_rq_pad<T, XC, HC, 36>(p, m, rq, smem, s, threads);
      default: return dispatch_rq_pad<T, XC, HC, 37>(p, m, rq, smem, s, threads);
    }
  }
  if constexpr (std::is_same<T, float>::value && XC && !HC) {
    switch (pad) {
      case 11: return dispatch_rq_pad<T, XC, HC, 11>(p, m, rq, smem, s, threads);
      case 12: return dispatch_rq_pad<T, XC, HC, 12>(p, m, rq, smem, s, threads);
      case 13: return dispatch_rq_pad<T, XC, HC, 13>(p, m, rq, smem, s, threads);
      case 14: return dispatch_rq_pad<T, XC, HC, 14>(p, m, rq, smem, s, threads);
      case 15: return dispatch_rq_pad<T, XC, HC, 15>(p, m, rq, smem, s, threads);
      case 16: return dispatch_rq_pad<T, XC, HC, 16>(p, m, rq, smem, s, threads);
      default: return dispatch_rq_pad<T, XC, HC, 17>(p, m, rq, smem, s, threads);
    }
  }
  return dispatch_rq_pad<T, XC, HC, 4>(p, m, rq, smem, s, threads);
}

template <int RQ, int PAD>
inline int launch_ring(RsParams &p, const CUtensorMap &omap, size_t smem, cudaStream_t s, int threads) {
  auto fn = resample_rowtile_ring<RQ, PAD>;
  int rc = ensure_smem((const void *)fn, smem, "resample_poly");
  if (rc) return rc;
  int occ = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, threads, smem);
  if (occ < 1) GBFIR_FAIL(GBFIR_ERR_NOT_SUPPORTED, "resample_poly: ring tile needs %zu B of shared memory", smem);
  int64_t grid = (int64_t)num_sms() * occ;
  if (grid > p.ntiles) grid = p.ntiles;
  fn<<<(unsigned)grid, (unsigned)threads, smem, s>>>(p, omap);
  return check_launch("resample_poly");
}

template <int PAD>
inline int dispatch_ring_rq(RsParams &p, const CUtensorMap &m, int rq, size_t smem, cudaStream_t s, int threads) {
  if (rq == 1) return launch_ring<1, PAD>(p, m, smem, s, threads);
  return launch_ring<2, PAD>(p, m, smem, s, threads);
}

inline int dispatch_ring(RsParams &p, const CUtensorMap &m, int rq, int pad, size_t smem, cudaStream_t s,
                         int threads) {
  switch (pad) {
    case 0: return dispatch_ring_rq<0>(p, m, rq, smem, s, threads);
    case 11: return dispatch_ring_rq<11>(p, m, rq, smem, s, threads);
    case 12: return dispatch_ring_rq<12>(p, m, rq, smem, s, threads);
    case 13: return dispatch_ring_rq<13>(p, m, rq, smem, s, threads);
    case 14: return dispatch_ring_rq<14>(p, m, rq, smem, s, threads);
    case 15: return dispatch_ring_rq<15>(p, m, rq, smem, s, threads);
    case 16: return dispatch_ring_rq<16>(p, m, rq, smem, s, threads);
    case 17: return dispatch_ring_rq<17>(p, m, rq, smem, s, threads);
    case 20: return dispatch_ring_rq<20>(p, m, rq, smem, s, threads);
    case 21: return dispatch_ring_rq<21>(p, m, rq, smem, s, threads);
    case 22: return dispatch_ring_rq<22>(p, m, rq, smem, s, threads);
    case 23: return dispatch_ring_rq<23>(p, m, rq, smem, s, threads);
    case 24: return dispatch_ring_rq<24>(p, m, rq, smem, s, threads);
    case 25: return dispatch_ring_rq<25>(p, m, rq, smem, s, threads);
    case 26: return dispatch_ring_rq<26>(p, m, rq, smem, s, threads);
    default: return dispatch_ring_rq<27>(p, m, rq, smem, s, threads);
  }
}

// The two-buffer form's paired walk (complex float signal, real taps): pad 20..27.
template <int PAD>
inline int dispatch_pair_rq(RsParams &p, const CUtensorMap &m, int rq, size_t smem, cudaStream_t s, int threads) {
  if (rq == 1) return launch_rowtile<float, true, false, 1, PAD>(p, m, smem, s, threads);
  if (rq == 2) return launch_rowtile<float, true, false, 2, PAD>(p, m, smem, s, threads);
  return launch_rowtile<float, true, false, 4, PAD>(p, m, smem, s, threads);
}

inline int dispatch_pair(RsParams &p, const CUtensorMap &m, int rq, int pad, size_t smem, cudaStream_t s,
                         int threads) {
  switch (pad) {
    case 20: return dispatch_pair_rq<20>(p, m, rq, smem, s, threads);
    case 21: return dispatch_pair_rq<21>(p, m, rq, smem, s, threads);
    case 22: return dispatch_pair_rq<22>(p, m, rq, smem, s, threads);
    case 23: return dispatch_pair_rq<23>(p, m, rq, smem, s, threads);
    case 24: return dispatch_pair_rq<24>(p, m, rq, smem, s, threads);
    case 25: return dispatch_pair_rq<25>(p, m, rq, smem, s, threads);
    case 26: return dispatch_pair_rq<26>(p, m, rq, smem, s, threads);
    default: return dispatch_pair_rq<27>(p, m, rq, smem, s, threads);
  }
}

// Tile shape knobs: rq rows per thread (1, 2, 4), wc column warps (1..8), G row
// grouping.  Zero picks the built-in heuristic.
struct TileChoice {
  int rq = 0, wc = 0, nbuf = 0;  // nbuf 3: the ring form (staging warp, 3-4 window slots)
  int ostore = -1;  // 1: TMA-store epilogue where the output layout allows it, 0: direct
                    // stores, -1: the epilogue for rows of 8 or more outputs
  bool pair = false;  // the paired walk where the row stride is even
  int64_t group = 0;
};

// One resampling pass
//   out[b][m] = scale * sum_k in[b][k] * hh(c + m*dn - k*upk)
// (forward: dn = down, upk = up; adjoint: dn = up, upk = down, rev = 1).
// Uses the row tile when it fits in shared memory, else the direct form.  RING: the caller
// may ask for the ring form (complex float signals, real taps); other callers do not
// instantiate it.
template <typename T, bool XC, bool HC, bool RING = false>
inline int resample_pass(const void *in, int64_t in_bstride, int64_t N_in, const void *h, int64_t L, void *out,
                         int64_t out_bstride, int64_t out_len, int64_t batch, int64_t upk, int64_t dn,
                         int64_t c_override, bool odd_extend, int rev, double scale, TileChoice tc, cudaStream_t s) {
  using XT = typename val_of<T, XC>::type;
  using HT = typename val_of<T, HC>::type;
  // real float rows: at least 8 phases, so a thread's 8-phase super-group is not half empty
  constexpr bool kReal32 = std::is_same<T, float>::value && !XC && !HC;
  int64_t G = tc.group > 0 ? tc.group : 4 / gcd64(upk, 4);
  if (tc.group <= 0 && kReal32 && upk * G < 8) G = 8 / gcd64(upk, 8);
  RsGeom geo = plan_geometry(upk, dn, L, out_len, G, c_override, odd_extend);
  const int nsg = (geo.ncg + 1) / 2;
  int wc = 1;
  if (tc.wc > 0) {
    wc = tc.wc;
  } else {
    // the largest power of two <= 8 that divides the super-group count (balanced warps)
    while (wc < 8 && nsg % (wc * 2) == 0) wc *= 2;
  }
  if (wc > nsg || wc < 1 || wc > 16 || (wc <= 8 && 8 % wc != 0)) wc = 1;
  constexpr bool kRingType = RING && std::is_same<T, float>::value && XC && !HC;
  bool ring = kRingType && tc.nbuf == 3;
  // row slices per CTA: 8/wc for 1, 2, 4, 8 column warps, one slice (one row per thread)
  // for 9..16, so the CTA has 8 warps or wc of them; the ring form has 16 compute warps
  // (16/wc slices) or wc, plus its staging warps
  int wr = wc <= 8 ? (ring ? 16 : 8) / wc : 1;
  // the paired walk: an even row stride and 16-byte aligned signal rows; its bands start at
  // even k
  int t2 = 0;
  while (t2 < 8 && (((geo.S >> 1) >> t2) & 1) == 0) t2++;
  const bool pair = kRingType && tc.pair && geo.S % 2 == 0 && t2 <= 7 && (reinterpret_cast<uintptr_t>(in) & 15) == 0 &&
                    (batch == 1 || in_bstride % 2 == 0);
  if (pair) geo = plan_geometry(upk, dn, L, out_len, G, c_override, odd_extend, true);
  // even row strides need a conflict-free window layout: the XOR permutation for ctz(S)
  // (complex float signals with real taps), one pad per 16 elements otherwise; the paired
  // walk takes the unit layout for ctz(S/2)
  auto pad_for = [&](bool paired) -> int {
    if (paired) return 20 + t2;
    int pd = (geo.S % 2) ? 0 : 4;
    if (pd && ((std::is_same<T, float>::value && XC && !HC) || kReal32)) {
      int t = 0;
      while (t < 7 && ((geo.S >> t) & 1) == 0) t++;
      pd = (kReal32 ? 30 : 10) + t;
    }
    return pd;
  };
  int pad = pad_for(pair);
  const int nstage = ring_stages(pad);
  int threads = 32 * wc * wr + (ring ? 32 * nstage : 0);
  // window buffer: padded layout for even S; for odd S room for the 16-byte-aligned bulk copy
  constexpr int64_t G16 = 16 / (int64_t)sizeof(XT);
  auto window_alloc = [&](int64_t win) -> int64_t {
    if (pad > 30) return (win + 31) / 32 * 32;             // permutations inside blocks of 32
    if (pad == 1 || pad > 10) return (win + 15) / 16 * 16;  // the permutations stay inside blocks of 16
    return pad ? win + (win >> pad) + 1 : (win + 3 * G16 - 1) / G16 * G16;
  };
  // TMA-store epilogue (complex float outputs): rows of an even Nt >= 8 (64-byte boxes), 4
  // or 2 (32, 16), a 16-byte aligned output with an even batch stride, at least one whole row
  const int64_t rows_full = out_len / geo.Nt;
  int ost_rb = geo.Nt >= 8 ? 64 : geo.Nt == 4 ? 32 : geo.Nt == 2 ? 16 : 0;
  const bool ostore = (tc.ostore == 1 || (tc.ostore < 0 && geo.Nt >= 8)) && std::is_same<T, float>::value && XC && !HC && geo.Nt % 2 == 0 &&
                      ost_rb > 0 && (reinterpret_cast<uintptr_t>(out) & 15) == 0 &&
                      (batch == 1 || out_bstride % 2 == 0) && rows_full >= 1;
  size_t stg_bytes = ostore ? 1024 + (size_t)(threads / 32 - (ring ? nstage : 0)) * 4096 : 0;
  bool ost_single = false;
  auto smem_for = [&](int rq, int nbuf) -> size_t {
    const int64_t QC = 32LL * rq * wr;
    const int64_t win = (QC - 1) * geo.S + (geo.kmax - geo.kmin) + 1;
    const int64_t alloc = window_alloc(win);
    return tap_table_bytes<T, XC, HC>(geo.ncg, geo.span) + (size_t)nbuf * (size_t)alloc * sizeof(XT) + stg_bytes;
  };
  // four rows per thread for real float rows: the f32x2 FMAs of a sample need one 16-byte
  // tap load per band and k, shared by the thread's rows
  int rq = tc.rq > 0 ? tc.rq : kReal32 ? 4 : 2;
  int nbuf = tc.nbuf > 0 ? tc.nbuf : 2;
  if (ring) {
    // one CTA per SM of up to 18 warps (112 registers a thread: one or two rows per thread); four
    // window slots, else three, else fewer rows per thread; the two-buffer form where even
    // one row per thread does not fit
    if (rq > 2) rq = 2;
    nbuf = 4;
    while (smem_for(rq, nbuf) > 225 * 1024 && (nbuf > 3 || rq > 1)) {
      if (nbuf == 4) nbuf = 3;
      else {
        rq /= 2;
        nbuf = 4;
      }
    }
    if (smem_for(rq, nbuf) > 225 * 1024) {
      ring = false;
      wr = wc <= 8 ? 8 / wc : 1;
      threads = 32 * wc * wr;
      stg_bytes = ostore ? 1024 + (size_t)(threads / 32) * 4096 : 0;
      rq = tc.rq > 0 ? tc.rq : 2;
      nbuf = 2;
    }
  }
  if (!ring) {
    if (nbuf > 2) nbuf = 2;
    if (sizeof(T) == 8) rq = 1;
    else if (threads > 256 && rq > 2) rq = 2;  // CTAs of 9-16 column warps: 1 or 2 rows per thread
    // two CTAs per SM (228 KB per SM, 1 KB of it reserved per CTA): prefer double buffering,
    // then fewer rows, then (one row per thread, whose warps compute a whole super-group
    // between two boxes) one staging buffer per warp, then a single window buffer
    const size_t stg_two = stg_bytes;
    while (smem_for(rq, nbuf) > 112 * 1024 && (rq > 1 || nbuf > 1)) {
      if (nbuf == 2 && rq == 1 && ostore && !ost_single) {
        ost_single = true;
        stg_bytes = 1024 + (size_t)(threads / 32) * 2048;
      } else if (nbuf == 2 && rq == 1) {
        nbuf = 1;
      } else if (rq > 1) {
        rq /= 2;
      } else {
        nbuf = 1;
      }
    }
    if (nbuf == 1 && ost_single) {
      ost_single = false;
      stg_bytes = stg_two;
    }
  }
  const size_t smem = smem_for(rq, nbuf);

  RsParams p{};
  p.x = in;
  p.x_bstride = batch > 1 ? in_bstride : 0;
  p.N = N_in;
  p.h = h;
  p.Lo = geo.Lo;
  p.even = geo.even;
  p.c = geo.c;
  p.out = out;
  p.out_bstride = out_bstride;
  p.out_len = out_len;
  p.up = upk;
  p.down = dn;
  p.scale = scale;
  p.rev = rev;
  p.nbuf = nbuf;
  p.pair = pair ? 1 : 0;
  if (smem <= (ring ? 225 : 200) * 1024) {
    p.Nt = geo.Nt;
    p.S = geo.S;
    p.ncg = geo.ncg;
    p.span = geo.span;
    p.kmin = geo.kmin;
    p.rows = geo.rows;
    p.QC = 32 * rq * wr;
    p.WC = wc;
    p.tiles_per_row = (geo.rows + p.QC - 1) / p.QC;
    p.ntiles = p.tiles_per_row * batch;
    const int64_t win = (int64_t)(p.QC - 1) * geo.S + (geo.kmax - geo.kmin) + 1;
    p.win = (int32_t)win;
    p.win_alloc = (int32_t)window_alloc(win);
    CUtensorMap omap;
    memset(&omap, 0, sizeof(omap));
    if (ostore) {
      // the output as (2*Nt floats, rows_full rows, batch); boxes of 32 rows x ost_rb bytes
      const cuuint64_t dims[3] = {(cuuint64_t)(2 * geo.Nt), (cuuint64_t)rows_full, (cuuint64_t)batch};
      const cuuint64_t strides[2] = {(cuuint64_t)(geo.Nt * 8),
                                     (cuuint64_t)((batch > 1 ? out_bstride : rows_full * geo.Nt) * 8)};
      const cuuint32_t box[3] = {(cuuint32_t)(ost_rb / 4), 32, 1}, es[3] = {1, 1, 1};
      const CUtensorMapSwizzle sw = ost_rb == 64   ? CU_TENSOR_MAP_SWIZZLE_64B
                                    : ost_rb == 32 ? CU_TENSOR_MAP_SWIZZLE_32B
                                                   : CU_TENSOR_MAP_SWIZZLE_NONE;
      const TensorMapEncodeFn enc = tensor_map_encoder();
      const CUresult r = enc == nullptr ? CUDA_ERROR_NOT_SUPPORTED : enc(&omap, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, out, dims, strides, box,
                                                es, CU_TENSOR_MAP_INTERLEAVE_NONE, sw,
                                                CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
      if (r == CUDA_SUCCESS) {
        p.ostore = 1;
        p.ost_rb = ost_rb;
        p.rows_full = rows_full;
        p.stg_off = (int32_t)(smem - stg_bytes);
        p.ost_single = ost_single ? 1 : 0;
      }
    }
    if constexpr (kRingType) {
      if (ring) return dispatch_ring(p, omap, rq, pad, smem, s, threads);
      if (pair) return dispatch_pair(p, omap, rq, pad, smem, s, threads);
    }
    return dispatch_rq<T, XC, HC>(p, omap, rq, pad, smem, s, threads);
  }
  // row tile too large for shared memory: direct form
  const size_t hbytes = (size_t)L * sizeof(HT);
  const int h_in_smem = hbytes <= 96 * 1024;
  const size_t dsmem = h_in_smem ? hbytes : 0;
  auto fn = resample_direct<T, XC, HC>;
  int rc = ensure_smem((const void *)fn, dsmem, "resample_poly");
  if (rc) return rc;
  const int64_t total = out_len * batch;
  int64_t grid = (total + 255) / 256;
  const int64_t cap = (int64_t)num_sms() * 4;
  if (grid > cap) grid = cap;
  if (grid < 1) grid = 1;
  fn<<<(unsigned)grid, 256, dsmem, s>>>(p, h_in_smem, batch);
  return check_launch("resample_poly (direct)");
}

}  // namespace gbfir
