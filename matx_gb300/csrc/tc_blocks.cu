// tc_blocks.cu — resample_poly as Toeplitz MMAs over materialised Hankel rows, in column
// blocks (tcgen05; bf16, fp16, bf16x3 split precision; FP32 accumulate in TMEM).  No MatX
// counterpart: the same outputs as MatX's resample_poly (include/matx/transforms/
// resample_poly.h:212-281 semantics) for rates whose rows advance by a number of input
// samples the aliased layouts of tc_resample.cu cannot express (160/147: rows of 160
// outputs advance 147 samples).
//
// Math.  Rows of Nt = up*G outputs advance S = down*G input samples.  The row's phases are
// cut into column blocks of NB; block b (phases j in [b*NB, b*NB + NB)) only reads the band
// k in [k0_b, k0_b + Kb) (k0_b = the smallest k any of its phases reads), so
//   out[q*Nt + b*NB + n] = sum_k A_b[q][k] * W_b[n][k],
//   A_b[q][k] = x[q*S + k0_b + k],   W_b[n][k] = up * he[c + (b*NB + n)*down - (k0_b + k)*up].
// The producers materialise A_b (a Hankel slab: neighbouring rows overlap) straight from
// global memory, already split into the operand terms, in the no-swizzle K-major layout.  A
// complex signal puts the real parts of 64 rows in MMA rows 0-63 and their imaginary parts
// in rows 64-127 of the same MMA (the taps are real), so one MMA covers both parts.  The W_b
// of every block are built once per CTA.
//
// Pipeline (persistent, warp-specialised, 384 threads): a stage is (tile of rows, column
// block).  Warps 1-7 materialise A into a 2-slot ring; warp 0 lane 0 issues the MMAs into one
// of two TMEM accumulator sets; warps 8-11 drain a set through a padded shared staging tile
// and store whole (complex) outputs, a warp per row slice, coalesced.  Every mbarrier wait is
// bounded: one that gives up sets the status word read by gbfir_tc_status().
#include <algorithm>
#include <cstdio>

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

struct TbParams {
  const void *x;
  int64_t x_bstride, N;
  const float *h;
  int64_t Lo, c;
  int32_t even, rev;
  double scale;
  void *out;
  int64_t out_bstride, out_len;
  int64_t up, down;  // gcd-reduced
  int64_t Nt, S;     // outputs per row, input samples a row advances
  int32_t NB;        // phases per column block (MMA N, multiple of 16)
  int32_t nblk;      // column blocks per row
  int32_t Kb;        // K band per block (multiple of 16)
  int32_t terms, fp16;
  int32_t RT;        // rows per tile: 64 (complex: both parts in the 128 MMA rows) or 128
  int64_t rows, tiles_per_row, ntiles;
  int32_t stage_stride;  // staging row pitch in floats (NB + 4)
};

constexpr int kTbThreads = 384;
constexpr int kTbProd0 = 1, kTbProdWarps = 7, kTbEpi0 = 8;
constexpr int kTbNProd = kTbProdWarps * 32;
constexpr int kTbBatch = 3;  // producer items whose loads are in flight together

__device__ __forceinline__ void tb_sync(int id, int nthreads) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

// smallest k any phase of block b reads
__device__ __forceinline__ int64_t tb_k0(const TbParams &p, int b) {
  return ceil_div(p.c + (int64_t)b * p.NB * p.down - p.Lo + 1, p.up);
}

template <bool XC>
__global__ void __launch_bounds__(kTbThreads, 1) tc_blocks_kernel(const TbParams p) {
  using XT = typename val_of<float, XC>::type;
  extern __shared__ __align__(1024) unsigned char smem_dyn[];
  __shared__ uint64_t op_full[2], op_empty[2], tm_full[2], tm_empty[2];
  __shared__ uint32_t tmem_slot;
  __shared__ int s_fail, s_pok, s_eok;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  // layout: W [nblk][terms][NB x Kb] ; A ring [2][terms][128 x Kb] ; staging [128][stage_stride] f32
  unsigned char *smem = smem_dyn + ((1024u - (tc::smem_u32(smem_dyn) & 1023u)) & 1023u);
  const uint32_t wbytes = (uint32_t)p.NB * p.Kb * 2u, abytes = 128u * p.Kb * 2u;
  auto wmat = [&](int b, int t) { return smem + ((size_t)b * p.terms + t) * wbytes; };
  unsigned char *abase = smem + ((size_t)p.nblk * p.terms * wbytes + 1023) / 1024 * 1024;
  auto amat = [&](int slot, int t) { return abase + ((size_t)slot * p.terms + t) * abytes; };
  float *stage = reinterpret_cast<float *>(abase + (size_t)2 * p.terms * abytes);

  // two accumulator sets of NB columns, rounded up to a power of two >= 32
  const uint32_t tcols = 2 * p.NB <= 32 ? 32u : 2 * p.NB <= 64 ? 64u : 2 * p.NB <= 128 ? 128u : 256u;
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
  // ---- the taps, scaled and split into the operand terms once, staged in the A ring (not in
  // use yet); then every W_b element is a lookup ----
  const int64_t Lh = p.Lo - p.even;
  const bool h_staged = (size_t)Lh * 2 * p.terms <= (size_t)2 * p.terms * abytes;
  uint16_t *hterm = reinterpret_cast<uint16_t *>(abase);
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
    for (int64_t e = tid; e < Lh; e += kTbThreads) {
      uint16_t o[3];
      split_terms(p.h[e] * (float)p.scale, o);
      for (int t = 0; t < p.terms; t++) hterm[t * Lh + e] = o[t];
    }
  }
  __syncthreads();
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
  // W_b[t][n][k]: one item per (block, term, row n, 8-wide K chunk), one 16-byte store
  const int kch = p.Kb / 8;
  for (int it = tid; it < p.nblk * p.terms * p.NB * kch; it += kTbThreads) {
    const int rr = it / kch, kc = it - rr * kch;
    const int bt = rr / p.NB, n = rr - bt * p.NB;
    const int b = bt / p.terms, t = bt - b * p.terms;
    const int64_t j = (int64_t)b * p.NB + n;
    uint32_t w[4] = {0u, 0u, 0u, 0u};
    if (j < p.Nt) {
      const int64_t tp0 = p.c + j * p.down - (tb_k0(p, b) + 8 * kc) * p.up;
#pragma unroll
      for (int e = 0; e < 8; e++) w[e >> 1] |= w_term(t, tp0 - e * p.up) << (16 * (e & 1));
    }
    *reinterpret_cast<uint4 *>(wmat(b, t) + tc::kmajor_offset(n, 8 * kc, p.Kb)) = make_uint4(w[0], w[1], w[2], w[3]);
  }
  tc::fence_async_smem();
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = tmem_slot;
  const XT *xp = reinterpret_cast<const XT *>(p.x);
  const int64_t my_tiles = p.ntiles > blockIdx.x ? (p.ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
  const int64_t nstages = my_tiles * p.nblk;
  auto tile_of = [&](int64_t i, int64_t &bb, int64_t &q0) {
    const int64_t t = blockIdx.x + i * (int64_t)gridDim.x;
    bb = t / p.tiles_per_row;
    q0 = (t - bb * p.tiles_per_row) * (int64_t)p.RT;
  };

  if (warp >= kTbProd0 && warp < kTbProd0 + kTbProdWarps) {
    // ================= producers: A_b of each stage, from global memory =================
    // item (q, 8-wide K chunk): lanes take consecutive rows q, so a warp's 16-byte stores fill
    // whole 128-byte core matrices (conflict-free)
    const int ptid = tid - kTbProd0 * 32;
    for (int64_t s = 0; s < nstages; ++s) {
      const int slot = (int)(s & 1);
      const int64_t i = s / p.nblk;
      const int b = (int)(s - i * p.nblk);
      if (ptid == 0) s_pok = (s < 2) ? 1 : (tc::mbar_wait(&op_empty[slot], (uint32_t)(((s - 2) >> 1) & 1)) ? 1 : 0);
      tb_sync(1, kTbNProd);
      if (!s_pok) {
        s_fail = 1;
        break;
      }
      int64_t bb, q0;
      tile_of(i, bb, q0);
      const XT *row = xp + bb * p.x_bstride;
      const int64_t k0 = tb_k0(p, b);
      const int nitems = p.RT * kch;
      // kTbBatch items per thread at a time, every load of the batch issued before any
      // conversion, so a stage pays the global-load latency once per batch
      for (int i0 = ptid; i0 < nitems; i0 += kTbBatch * kTbNProd) {
        XT v[kTbBatch][8];
#pragma unroll
        for (int bi = 0; bi < kTbBatch; bi++) {
          const int itm = i0 + bi * kTbNProd;
          const int kc = itm / p.RT, q = itm - kc * p.RT;
          const int64_t g0 = (q0 + q) * p.S + k0 + 8 * kc;
#pragma unroll
          for (int e = 0; e < 8; e++) {
            const int64_t gi = g0 + e;
            v[bi][e] = (itm < nitems && gi >= 0 && gi < p.N) ? __ldg(row + gi) : zero_val<XT>();
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
            const uint32_t off = tc::kmajor_offset(part * 64 + q, 8 * kc, p.Kb);
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
    }
  } else if (warp == 0) {
    // ================= MMA issuer =================
    const bool geom_ok = p.NB % 16 == 0 && p.NB <= 256 && p.Kb % 16 == 0;
    if (lane == 0 && !geom_ok) s_fail = 1;
    if (lane == 0 && geom_ok) {
      const uint32_t idesc = tc::idesc_f16(128, (uint32_t)p.NB, p.fp16 ? 0u : 1u);
      const uint32_t sbo = (uint32_t)(p.Kb / 8) * 128u;
      const int nks = p.Kb / 16;
      // products of order <= 2 (signal term tx, tap term tw), smallest first
      constexpr uint32_t kTx = 0x001021u, kTw = 0x010201u;
      const int npairs = p.terms == 3 ? 6 : 1;
      for (int64_t s = 0; s < nstages; ++s) {
        const int slot = (int)(s & 1);
        const int b = (int)(s % p.nblk);
        if (!tc::mbar_wait(&op_full[slot], (uint32_t)((s >> 1) & 1))) { s_fail = 1; break; }
        if (s >= 2 && !tc::mbar_wait(&tm_empty[slot], (uint32_t)(((s - 2) >> 1) & 1))) { s_fail = 1; break; }
        tc::tc_fence_after();
        const uint32_t d = tmem + (uint32_t)(slot * p.NB);
        for (int pr = 0; pr < npairs; pr++) {
          const int tx = p.terms == 3 ? (int)((kTx >> (4 * pr)) & 15u) : 0;
          const int tw = p.terms == 3 ? (int)((kTw >> (4 * pr)) & 15u) : 0;
          uint64_t ad = tc::smem_desc(tc::smem_u32(amat(slot, tx)), 128u, sbo);
          uint64_t bd = tc::smem_desc(tc::smem_u32(wmat(b, tw)), 128u, sbo);
          for (int ks = 0; ks < nks; ks++) {
            tc::mma_f16(d, ad, bd, idesc, (pr > 0 || ks > 0) ? 1u : 0u);
            ad += 16;  // +256 B: two core matrices along K
            bd += 16;
          }
        }
        tc::mma_commit(&op_empty[slot]);
        tc::mma_commit(&tm_full[slot]);
      }
    }
  } else if (warp >= kTbEpi0) {
    // ================= epilogue =================
    // quarter w holds TMEM lanes 32w..32w+31 = staging rows; for a complex signal rows 0-63
    // are real parts and 64-127 imaginary parts of the tile's 64 rows
    const int quarter = warp - kTbEpi0;
    const int srow = 32 * quarter + lane;
    const uint32_t lane_base = (uint32_t)(32 * quarter) << 16;
    for (int64_t s = 0; s < nstages; ++s) {
      const int slot = (int)(s & 1);
      const int64_t i = s / p.nblk;
      const int b = (int)(s - i * p.nblk);
      if (quarter == 0 && lane == 0) s_eok = tc::mbar_wait(&tm_full[slot], (uint32_t)((s >> 1) & 1)) ? 1 : 0;
      tb_sync(2, 128);
      if (!s_eok) {
        s_fail = 1;
        break;
      }
      tc::tc_fence_after();
      float *srow_p = stage + (size_t)srow * p.stage_stride;
      for (int col = 0; col < p.NB; col += 16) {
        uint32_t r[16];
        tc::tmem_ld16(tmem + lane_base + (uint32_t)(slot * p.NB + col), r);
        tc::tmem_ld_wait();
#pragma unroll
        for (int e = 0; e < 16; e += 4)
          *reinterpret_cast<float4 *>(srow_p + col + e) = make_float4(__uint_as_float(r[e]), __uint_as_float(r[e + 1]),
                                                                       __uint_as_float(r[e + 2]), __uint_as_float(r[e + 3]));
      }
      tc::tc_fence_before();
      tb_sync(2, 128);
      if (quarter == 0 && lane == 0) tc::mbar_arrive_plain(&tm_empty[slot]);
      // whole outputs, a warp per row at a time: lanes take consecutive phases (coalesced)
      int64_t bb, q0;
      tile_of(i, bb, q0);
      XT *orow = reinterpret_cast<XT *>(p.out) + bb * p.out_bstride;
      const int64_t j0 = (int64_t)b * p.NB;
      for (int q = quarter; q < p.RT; q += 4) {
        const int64_t n0 = (q0 + q) * p.Nt + j0;
        for (int n = lane; n < p.NB; n += 32) {
          if (j0 + n >= p.Nt || n0 + n >= p.out_len) continue;
          if constexpr (XC) {
            orow[n0 + n] = make_float2(stage[(size_t)q * p.stage_stride + n], stage[(size_t)(64 + q) * p.stage_stride + n]);
          } else {
            orow[n0 + n] = stage[(size_t)q * p.stage_stride + n];
          }
        }
      }
      tb_sync(2, 128);  // the staging tile is read before the next stage overwrites it
    }
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

struct TbPlan {
  TbParams p;
  size_t smem;
  bool ok;
  char why[160];
};

// Column-blocked plan: rows of Nt = up*G outputs (G the smallest with Nt >= 32), blocks of
// NB phases (64, 48, 32 or 16: the widest whose tile fits 225 KB of shared memory).
static TbPlan plan_tc_blocks(int64_t up, int64_t down, int64_t Lo, int64_t c, int even, int rev, double scale,
                             int64_t N_in, int64_t out_len, int64_t batch, int xc, int precision) {
  TbPlan pl{};
  TbParams &p = pl.p;
  p.Lo = Lo;
  p.c = c;
  p.even = even;
  p.rev = rev;
  p.scale = scale;
  p.up = up;
  p.down = down;
  p.N = N_in;
  p.out_len = out_len;
  p.fp16 = precision == GBFIR_PREC_FP16;
  p.terms = precision == GBFIR_PREC_BF16X3 ? 3 : 1;
  p.RT = xc ? 64 : 128;
  int64_t G = 1;
  while (up * G < 32 && G < 64) G++;
  p.Nt = up * G;
  p.S = down * G;
  for (int NB : {64, 48, 32, 16}) {
    if (NB > ((p.Nt + 15) / 16) * 16 && NB > 16) continue;
    const int nblk = (int)((p.Nt + NB - 1) / NB);
    int64_t span = 1;
    for (int b = 0; b < nblk; b++) {
      const int64_t j0 = (int64_t)b * NB, j1 = std::min<int64_t>(p.Nt - 1, j0 + NB - 1);
      const int64_t k0 = ceil_div(c + j0 * down - Lo + 1, up);
      const int64_t k1 = floor_div(c + j1 * down, up);
      span = std::max<int64_t>(span, k1 - k0 + 1);
    }
    const int Kb = (int)((span + 15) / 16 * 16);
    const size_t w = (size_t)nblk * p.terms * NB * Kb * 2;
    const size_t a = (size_t)2 * p.terms * 128 * Kb * 2;
    const size_t st = (size_t)128 * (NB + 4) * 4;
    const size_t smem = 1024 + (w + 1023) / 1024 * 1024 + a + st;
    if (smem > 225 * 1024 || Kb > 512) continue;
    p.NB = NB;
    p.nblk = nblk;
    p.Kb = Kb;
    p.stage_stride = NB + 4;
    p.rows = (out_len + p.Nt - 1) / p.Nt;
    p.tiles_per_row = (p.rows + p.RT - 1) / p.RT;
    p.ntiles = p.tiles_per_row * batch;
    pl.smem = smem;
    pl.ok = true;
    return pl;
  }
  snprintf(pl.why, sizeof(pl.why), "no column block of 16..64 phases fits shared memory (filter of %lld taps)",
           (long long)Lo);
  return pl;
}

// Plans and launches the column-blocked pass for out = scale * sum x * he(c + n*down - k*up);
// returns GBFIR_ERR_NOT_SUPPORTED (with the reason) where no tile fits.
int launch_tc_blocks(const gbfir_buf &out, const gbfir_buf &in, const gbfir_buf &h, int64_t up, int64_t down,
                     int64_t Lo, int64_t c, int even, int rev, double scale, int precision, const char *what,
                     cudaStream_t s) {
  const bool xc = dtype_complex(in.dtype);
  TbPlan pl = plan_tc_blocks(up, down, Lo, c, even, rev, scale, in.len, out.len, out.batch, xc, precision);
  if (!pl.ok) GBFIR_FAIL(GBFIR_ERR_NOT_SUPPORTED, "%s: column-blocked tensor-core form unavailable: %s", what, pl.why);
  TbParams &p = pl.p;
  p.x = in.ptr;
  p.x_bstride = (out.batch > 1 && in.batch > 1) ? in.batch_stride : 0;
  p.h = reinterpret_cast<const float *>(h.ptr);
  p.out = out.ptr;
  p.out_bstride = out.batch_stride;
  const void *fn = xc ? (const void *)tc_blocks_kernel<true> : (const void *)tc_blocks_kernel<false>;
  int rc = ensure_smem(fn, pl.smem, what);
  if (rc) return rc;
  int64_t grid = num_sms();  // one CTA per SM
  if (grid > p.ntiles) grid = p.ntiles;
  if (grid < 1) return GBFIR_SUCCESS;
  void *args[] = {&p};
  const cudaError_t e = cudaLaunchKernel(fn, dim3((unsigned)grid), dim3(kTbThreads), args, pl.smem, s);
  if (e != cudaSuccess) GBFIR_FAIL(GBFIR_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  count_launch();
  return GBFIR_SUCCESS;
}

}  // namespace gbfir
