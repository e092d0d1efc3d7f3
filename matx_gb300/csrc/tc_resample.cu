// tc_resample.cu — resample_poly as Toeplitz MMAs on the tcgen05 tensor cores
// (bf16, fp16 and bf16x3 split precision, FP32 accumulate in TMEM).  No MatX counterpart.
//
// Math.  With gcd-reduced rates, y[n] = up * sum_i x[i] * he[c + n*down - i*up].
// The kernel groups outputs into rows whose inputs advance by exactly 8 samples of a
// linear array xs, so that the Hankel operand A[q][k] = xs[8q + k] is a plain
// K-major shared-memory matrix with overlapping rows: its 8-row x 16-byte core
// matrices are 16 bytes apart along K (LBO = 16) and 128 bytes apart along rows
// (SBO = 128), and no Hankel matrix is ever materialised.
//   path A (down divides 8): xs[u] = x[u + k0]; a row holds Nt = 8*up/down outputs and
//     D[q][j] = sum_k xs[8q + k] * W[j][k],  W[j][k] = up*he[c + j*down - (k + k0)*up].
//   path B (other down): x is split into its `down` polyphase components
//     xs_b[a] = x[down*a + b]; each is an interpolator (rate up) and a row holds
//     Nt = 8*up outputs:  D[q][j] = sum_b sum_k xs_b[8q + k + k0] * W_b[j][k],
//     W_b[j][k] = up*he[c + down*j - up*(b + down*(k + k0))].
// The tap matrices W (N = Nt rounded up to 16 columns, Kp = band rounded to 16) are
// built once per CTA.  Complex x runs as two M = 128 MMAs (real, imaginary rows) on the
// same W.  bf16x3 splits both operands into three bf16 terms and accumulates the six
// products of order <= 2 (smallest first) — 24 significant bits, FP32-class accuracy.
//
// Pipeline (persistent CTA, 256 threads).  An iteration covers MT M-tiles of 128 rows.
// Threads convert the next iteration's input samples into the bf16 term arrays of the
// other shared buffer while one thread's MMAs for the current iteration run into one
// of two TMEM accumulator sets; after a bounded mbarrier wait every warp reads its TMEM
// lanes back and stores the outputs.
#include "rowtile.cuh"
#include "tc.cuh"

namespace gbfir {

constexpr int kTcThreads = 256;

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
  int32_t LA;       // elements per xs array per buffer = 8*128*MT + Kp
  int32_t terms;    // 1 or 3
  int32_t fp16;     // 1: fp16 operands (single term), 0: bf16
  int64_t rows;     // rows per signal row = ceil(out_len / Nt)
  int64_t iters_per_row, niters;
  double scale;     // up
  int32_t tmem_cols;
  int32_t nbuf;     // 2: convert the next iteration during the MMAs; 1: after them
};

// Bounded-wait status of the tensor-core kernels (1 = a wait gave up); read and
// cleared by gbfir_tc_status().
__device__ int32_t g_tc_status;

__device__ __forceinline__ float tap_value(const TcParams &p, int64_t tp) {
  if (tp < 0 || tp >= p.Lo) return 0.f;
  const int64_t te = p.rev ? p.Lo - 1 - tp : tp;
  if (p.even && te == 0) return 0.f;
  return p.h[te - p.even];
}

template <bool XC>
__global__ void __launch_bounds__(kTcThreads) tc_resample_kernel(const TcParams p) {
  using XT = typename val_of<float, XC>::type;
  constexpr int NPARTS = XC ? 2 : 1;  // real / imaginary operand rows
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ uint64_t bars[2];
  __shared__ uint32_t tmem_slot;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  // shared layout: W [P][terms][Nmma x Kp] ; xs [2 bufs][NPARTS][terms][P][LA]
  const uint32_t wbytes = (uint32_t)p.Nmma * p.Kp * 2u;
  unsigned char *wbase = smem;
  unsigned char *xbase = smem + ((size_t)p.P * p.terms * wbytes + 127) / 128 * 128;
  const size_t xarr = ((size_t)p.LA * 2 + 127) / 128 * 128;  // bytes per xs array
  auto warr = [&](int pp, int t) { return wbase + ((size_t)pp * p.terms + t) * wbytes; };
  auto xarrp = [&](int buf, int part, int t, int pp) {
    return xbase + ((((size_t)buf * NPARTS + part) * p.terms + t) * p.P + pp) * xarr;
  };
  // raw input ring: two slots of P*LA samples (x as stored in HBM), filled by cp.async
  const size_t raw_elems = (size_t)p.P * p.LA;
  XT *raw0 = reinterpret_cast<XT *>(xbase + (size_t)p.nbuf * NPARTS * p.terms * p.P * xarr);
  auto rawp = [&](int slot) { return raw0 + (size_t)slot * raw_elems; };

  if (warp == 0) tc::tmem_alloc(&tmem_slot, (uint32_t)p.tmem_cols);
  if (tid == 0) {
    tc::mbar_init(&bars[0], 1);
    tc::mbar_init(&bars[1], 1);
    tc::mbar_fence_init();
  }
  // ---- tap matrices W_p[j][k] (K-major core layout), split into terms ----
  const int wel = p.Nmma * p.Kp;
  for (int e = tid; e < p.P * wel; e += kTcThreads) {
    const int pp = e / wel, r = e - pp * wel;
    const int j = r / p.Kp, k = r - j * p.Kp;
    float v = 0.f;
    if (j < p.Nt) {
      const int64_t kk = k + p.k0;
      const int64_t tp = p.path == 0 ? p.c + (int64_t)j * p.down - kk * p.up
                                     : p.c + p.down * (int64_t)j - p.up * (pp + p.down * kk);
      v = tap_value(p, tp) * (float)p.scale;
    }
    const uint32_t off = tc::kmajor_offset(j, k, p.Kp);
    if (p.fp16) {
      *reinterpret_cast<__half *>(warr(pp, 0) + off) = __float2half_rn(v);
    } else {
      __nv_bfloat16 t0, t1, t2;
      tc::split3_bf16(v, t0, t1, t2);
      *reinterpret_cast<__nv_bfloat16 *>(warr(pp, 0) + off) = t0;
      if (p.terms == 3) {
        *reinterpret_cast<__nv_bfloat16 *>(warr(pp, 1) + off) = t1;
        *reinterpret_cast<__nv_bfloat16 *>(warr(pp, 2) + off) = t2;
      }
    }
  }

  // ---- input staging: raw samples of one iteration into a ring slot (cp.async, zero-filled) ----
  const XT *xp = reinterpret_cast<const XT *>(p.x);
  auto fetch = [&](int64_t itx, int slot) {
    const int64_t b = itx / p.iters_per_row;
    const int64_t q0 = (itx - b * p.iters_per_row) * (int64_t)(128 * p.MT);
    const XT *row = xp + b * p.x_bstride;
    // path A: raw[v] = x[8*q0 + k0 + v]; path B: raw[v] = x[down*(8*q0 + k0) + v], v = P*u + b
    const int64_t base = p.path == 0 ? 8 * q0 + p.k0 : p.down * (8 * q0 + p.k0);
    XT *dst = rawp(slot);
    for (int v = tid; v < (int)raw_elems; v += kTcThreads) {
      const int64_t gi = base + v;
      const bool okk = gi >= 0 && gi < p.N;
      cp_async_zfill<sizeof(XT)>(dst + v, okk ? (const void *)(row + gi) : (const void *)row, okk);
    }
  };
  // ---- conversion of a staged slot into the bf16/fp16 term arrays of buffer `buf` ----
  // Each thread converts two consecutive samples of one component (4-byte stores).
  auto convert = [&](int slot, int buf) {
    const XT *src = rawp(slot);
    const int half = (p.LA + 1) / 2;
    for (int e = tid; e < p.P * half; e += kTcThreads) {
      const int pp = e / half, u = 2 * (e - pp * half);
      const XT v0 = src[(size_t)u * p.P + pp];
      const XT v1 = (u + 1 < p.LA) ? src[(size_t)(u + 1) * p.P + pp] : zero_val<XT>();
#pragma unroll
      for (int part = 0; part < NPARTS; part++) {
        const float f0 = part == 0 ? re_of(v0) : im_of(v0);
        const float f1 = part == 0 ? re_of(v1) : im_of(v1);
        if (p.fp16) {
          *reinterpret_cast<__half2 *>(reinterpret_cast<__half *>(xarrp(buf, part, 0, pp)) + u) =
              __floats2half2_rn(f0, f1);
        } else {
          __nv_bfloat16 a0, a1, a2, b0, b1, b2;
          tc::split3_bf16(f0, a0, a1, a2);
          tc::split3_bf16(f1, b0, b1, b2);
          *reinterpret_cast<__nv_bfloat162 *>(reinterpret_cast<__nv_bfloat16 *>(xarrp(buf, part, 0, pp)) + u) =
              __halves2bfloat162(a0, b0);
          if (p.terms == 3) {
            *reinterpret_cast<__nv_bfloat162 *>(reinterpret_cast<__nv_bfloat16 *>(xarrp(buf, part, 1, pp)) + u) =
                __halves2bfloat162(a1, b1);
            *reinterpret_cast<__nv_bfloat162 *>(reinterpret_cast<__nv_bfloat16 *>(xarrp(buf, part, 2, pp)) + u) =
                __halves2bfloat162(a2, b2);
          }
        }
      }
    }
  };

  int64_t it = blockIdx.x;
  if (it < p.niters) fetch(it, 0);
  cp_async_commit();
  if (p.nbuf == 2 && it + gridDim.x < p.niters) fetch(it + gridDim.x, 1);
  cp_async_commit();
  cp_async_wait<1>();
  __syncthreads();
  if (it < p.niters) convert(0, 0);
  tc::fence_async_smem();
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = tmem_slot;
  const uint32_t set_cols = (uint32_t)(p.MT * NPARTS * p.Nmma);
  const uint32_t idesc = tc::idesc_f16(128, (uint32_t)p.Nmma, p.fp16 ? 0u : 1u);
  const int pa3[6] = {2, 1, 0, 1, 0, 0}, pb3[6] = {0, 1, 2, 0, 1, 0};
  const int npairs = p.terms == 3 ? 6 : 1;
  bool ok = true;
  uint32_t phase[2] = {0, 0};

  const bool dbuf = p.nbuf == 2;
  for (int k = 0; it < p.niters; it += gridDim.x, ++k) {
    const int buf = dbuf ? (k & 1) : 0;  // shared operand buffer
    const int ts = k & 1;                // TMEM accumulator set and mbarrier
    const uint32_t dset = tmem + (uint32_t)ts * set_cols;
    if (tid == 0) {
      // A: xs_p + (8*128*m + 16*ks) elements, LBO 16 B, SBO 128 B;  W: K-major, LBO 128 B, SBO Kp/8*128 B.
      // Advancing one K-step adds 32 B to A's start address and 256 B to W's (start field is in 16 B units).
      const uint32_t wsbo = (uint32_t)(p.Kp / 8) * 128u;
      const int nks = p.Kp / 16;
      for (int m = 0; m < p.MT; m++) {
        for (int part = 0; part < NPARTS; part++) {
          const uint32_t d = dset + (uint32_t)((m * NPARTS + part) * p.Nmma);
          uint32_t acc = 0;
          for (int pi = 0; pi < npairs; pi++) {
            const int ta = p.terms == 3 ? pa3[pi] : 0, tb = p.terms == 3 ? pb3[pi] : 0;
            for (int pp = 0; pp < p.P; pp++) {
              uint64_t ad = tc::smem_desc(tc::smem_u32(xarrp(buf, part, ta, pp)) + (uint32_t)(8 * 128 * m) * 2u, 16u,
                                          128u);
              uint64_t bd = tc::smem_desc(tc::smem_u32(warr(pp, tb)), 128u, wsbo);
              for (int ks = 0; ks < nks; ks++) {
                tc::mma_f16(d, ad, bd, idesc, acc);
                acc = 1;
                ad += 2;   // +32 B
                bd += 16;  // +256 B
              }
            }
          }
        }
      }
      tc::mma_commit(&bars[ts]);
    }
    // stage iteration k+2 into the raw slot iteration k used, then convert iteration k+1
    // (staged one iteration ago) into the other operand buffer while the MMAs run
    const int64_t nxt = it + gridDim.x;
    const int64_t nxt2 = nxt + gridDim.x;
    if (dbuf) {
      if (nxt2 < p.niters) fetch(nxt2, k & 1);
      cp_async_commit();
      cp_async_wait<1>();
      __syncthreads();
      if (nxt < p.niters) convert((k + 1) & 1, buf ^ 1);
    }
    tc::fence_async_smem();
    const bool got = tc::mbar_wait(&bars[ts], phase[ts]);
    phase[ts] ^= 1u;
    if (!got) {
      ok = false;
      if (tid == 0) atomicExch(&g_tc_status, 1);
    }
    tc::tc_fence_after();
    // ---- epilogue: warp quarter w%4 owns TMEM lanes 32*(w%4) .. +32 (rows); warps 0-3 take
    // even M-tiles, 4-7 odd ones ----
    if (got) {
      const int64_t b = it / p.iters_per_row;
      const int64_t q0 = (it - b * p.iters_per_row) * (int64_t)(128 * p.MT);
      XT *orow = reinterpret_cast<XT *>(p.out) + b * p.out_bstride;
      for (int m = warp >> 2; m < p.MT; m += 2) {
        const int64_t q = q0 + 128 * m + 32 * (warp & 3) + lane;
        for (int col = 0; col < p.Nmma; col += 16) {
          uint32_t rr[16], ri[16];
          const uint32_t lane_base = (uint32_t)(32 * (warp & 3)) << 16;
          tc::tmem_ld16(dset + lane_base + (uint32_t)((m * NPARTS) * p.Nmma + col), rr);
          if constexpr (XC) tc::tmem_ld16(dset + lane_base + (uint32_t)((m * NPARTS + 1) * p.Nmma + col), ri);
          tc::tmem_ld_wait();
#pragma unroll
          for (int i = 0; i < 16; i++) {
            const int j = col + i;
            const int64_t n = q * p.Nt + j;
            if (j < p.Nt && n < p.out_len) {
              if constexpr (XC) {
                float2 v;
                v.x = __uint_as_float(rr[i]);
                v.y = __uint_as_float(ri[i]);
                orow[n] = v;
              } else {
                orow[n] = __uint_as_float(rr[i]);
              }
            }
          }
        }
      }
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    if (!ok) break;
    if (!dbuf && nxt < p.niters) {
      fetch(nxt, 0);
      cp_async_commit();
      cp_async_wait<0>();
      __syncthreads();
      convert(0, 0);
      tc::fence_async_smem();
      tc::tc_fence_before();
      __syncthreads();
      tc::tc_fence_after();
    }
  }
  cp_async_wait<0>();
  // drain: a timed-out wait above leaves MMAs possibly in flight; wait once more (bounded)
  if (!ok && tid == 0) {
    (void)tc::mbar_wait(&bars[0], phase[0]);
    (void)tc::mbar_wait(&bars[1], phase[1]);
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

static TcPlan plan_tc(int64_t up, int64_t down, int64_t L, int64_t N_in, int64_t out_len, int64_t batch, int xc,
                      int precision, int rev) {
  TcPlan pl{};
  TcParams &p = pl.p;
  p.even = (L % 2) == 0;
  p.Lo = L + p.even;
  p.c = (p.Lo - 1) / 2;
  p.rev = rev;
  p.up = up;
  p.down = down;
  p.N = N_in;
  p.out_len = out_len;
  p.scale = (double)up;
  p.fp16 = precision == GBFIR_PREC_FP16;
  p.terms = precision == GBFIR_PREC_BF16X3 ? 3 : 1;
  p.path = (8 % down == 0) ? 0 : 1;
  p.P = p.path == 0 ? 1 : (int32_t)down;
  int64_t kmin, kmax;
  if (p.path == 0) {
    p.Nt = (int32_t)(up * (8 / down));
    kmin = ceil_div(p.c - p.Lo + 1, up);
    kmax = floor_div(p.c + (int64_t)(p.Nt - 1) * down, up);
  } else {
    p.Nt = (int32_t)(8 * up);
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
  auto smem_for = [&](int MT, int nbuf) -> size_t {
    const size_t w = (size_t)p.P * p.terms * p.Nmma * p.Kp * 2;
    const size_t la = (size_t)8 * 128 * MT + p.Kp;
    const size_t xa = (la * 2 + 127) / 128 * 128;
    const size_t raw = (size_t)nbuf * p.P * la * (xc ? 8 : 4);
    return (w + 127) / 128 * 128 + (size_t)nbuf * nparts * p.terms * p.P * xa + raw;
  };
  // prefer two CTAs per SM (<= 110 KB each), then one CTA with double buffering, then single
  int MT = 4, nbuf = 2;
  while (MT > 1 && (smem_for(MT, nbuf) > 110 * 1024 || 2 * MT * nparts * p.Nmma > 256)) MT /= 2;
  if (smem_for(MT, nbuf) > 200 * 1024) nbuf = 1;
  if (2 * MT * nparts * p.Nmma > 512 || smem_for(MT, nbuf) > 200 * 1024) {
    snprintf(pl.why, sizeof(pl.why), "tile needs %zu B of shared memory", smem_for(MT, nbuf));
    return pl;
  }
  p.MT = MT;
  p.nbuf = nbuf;
  p.LA = 8 * 128 * MT + p.Kp;
  uint32_t cols = 32;
  while (cols < (uint32_t)(2 * MT * nparts * p.Nmma)) cols <<= 1;
  p.tmem_cols = (int32_t)cols;
  p.rows = (out_len + p.Nt - 1) / p.Nt;
  p.iters_per_row = (p.rows + 128 * MT - 1) / (128 * MT);
  p.niters = p.iters_per_row * batch;
  pl.smem = smem_for(MT, nbuf);
  pl.ok = true;
  return pl;
}

int resample_poly_tc(const gbfir_buf &out, const gbfir_buf &in, const gbfir_buf &h, int64_t up, int64_t down,
                     int precision, cudaStream_t s) {
  if (dtype_double(in.dtype) || dtype_complex(h.dtype))
    GBFIR_FAIL(GBFIR_ERR_NOT_SUPPORTED, "resample_poly: tensor-core forms take float32/complex64 signals and real "
                                        "float32 taps");
  const bool xc = dtype_complex(in.dtype);
  TcPlan pl = plan_tc(up, down, h.len, in.len, out.len, out.batch, xc, precision, 0);
  if (!pl.ok)
    GBFIR_FAIL(GBFIR_ERR_NOT_SUPPORTED, "resample_poly: tensor-core form unavailable for up=%lld down=%lld: %s",
               (long long)up, (long long)down, pl.why);
  TcParams &p = pl.p;
  p.x = in.ptr;
  p.x_bstride = out.batch > 1 ? in.batch_stride : 0;
  p.h = reinterpret_cast<const float *>(h.ptr);
  p.out = out.ptr;
  p.out_bstride = out.batch_stride;
  const void *fn = xc ? (const void *)tc_resample_kernel<true> : (const void *)tc_resample_kernel<false>;
  int rc = ensure_smem(fn, pl.smem, "resample_poly (tensor cores)");
  if (rc) return rc;
  int occ = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, kTcThreads, pl.smem);
  if (pl.smem <= 110 * 1024) occ = std::max(occ, 2);
  if (occ < 1) occ = 1;
  // each CTA holds tmem_cols of the SM's 512 TMEM columns
  occ = std::min(occ, 512 / p.tmem_cols);
  int64_t grid = (int64_t)num_sms() * occ;
  if (grid > p.niters) grid = p.niters;
  void *args[] = {&p};
  cudaError_t e = cudaLaunchKernel(fn, dim3((unsigned)grid), dim3(kTcThreads), args, pl.smem, s);
  if (e != cudaSuccess) GBFIR_FAIL(GBFIR_ERR_CUDA, "resample_poly (tensor cores): %s", cudaGetErrorString(e));
  count_launch();
  return GBFIR_SUCCESS;
}

int tc_status_read_and_clear() {
  int32_t v = 0, zero = 0;
  if (cudaMemcpyFromSymbol(&v, g_tc_status, sizeof(v)) != cudaSuccess) return -1;
  cudaMemcpyToSymbol(g_tc_status, &zero, sizeof(zero));
  return v;
}

}  // namespace gbfir

extern "C" int gbfir_tc_status(void) { return gbfir::tc_status_read_and_clear(); }
