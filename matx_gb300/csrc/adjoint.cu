// adjoint.cu — hand-written adjoints of resample_poly and direct conv1d (no MatX
// counterpart).  Real FP32 operands.
//
// Forward (row-tile form, rowtile.cuh):  y[b][n] = scale * sum_i x[b][i] * he[c + n*dn - i*upk]
//   resample_poly: dn = down, upk = up, scale = up, c = (Lodd-1)/2, he = h with the
//                  even-length leading zero;   conv1d: dn = upk = 1, c = start, he = h.
// Adjoints:
//   dx[b][i] = scale * sum_n gy[b][n] * he[c + n*dn - i*upk]
//            = the same row-tile pass on gy with dn and upk swapped and the taps
//              reversed (the transposed resampler; for conv it is corr(gy, h)).
//   dh[t]    = scale * sum_b sum_{(n, i): c + n*dn - i*upk = t} gy[b][n] * x[b][i]
//            = the tap-matrix gradient dB[k][j] = sum_q X[q][k] * GY[q][j] of every
//              row tile, folded back onto the taps.
// The dh kernel keeps dB entries of 4 k x 4 j in registers per thread while a
// persistent CTA walks its row tiles (x window and gy tile double-buffered with
// cp.async); the per-thread FP32 sums are reduced across row slices and CTAs in
// FP64, in a fixed order, so the result is deterministic.
#include <mutex>

#include "rowtile.cuh"

namespace gbfir {

struct DhParams {
  const float *x;
  int64_t x_bstride, N;
  const float *gy;
  int64_t gy_bstride, out_len;
  int64_t up, down, Lo, c;
  int64_t Nt, S;
  int32_t ncg, span;  // span is a multiple of 4 here
  int64_t kmin;
  int64_t rows, tiles_per_row, ntiles;
  int32_t QC, win, win_alloc;
  int32_t U, RS;      // work units (g, 4 k) and row slices
  int64_t G, inv_down;
  int32_t gal;        // 1: gradient rows 16-byte aligned (16-byte tile copies)
  double *partial;    // [gridDim.x][Lo]
};

constexpr int kDhThreads = 256;

// Timing hooks (role, stage, event); they compile to nothing unless a tracing build defines them.
#ifndef GBFIR_TC_TRACE
#define GBFIR_TC_TRACE(role, stage, event) \
  do {                                     \
  } while (0)
#endif

template <bool PAD, int UPT>
__global__ void __launch_bounds__(kDhThreads) rowtile_dh(const DhParams p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float *xb0 = reinterpret_cast<float *>(smem_raw);
  float *xb1 = xb0 + p.win_alloc;
  const int gyn = p.QC * (int)p.Nt;
  float *gb0 = xb1 + p.win_alloc;
  float *gb1 = gb0 + gyn;
  float *red = gb1 + gyn;  // [RS][U][16]
  const int tid = threadIdx.x;
  const int units_per_g = p.span / 4;

  auto issue = [&](int64_t tile, float *xb, float *gb) {
    const int64_t b = tile / p.tiles_per_row;
    const int64_t q0 = (tile - b * p.tiles_per_row) * p.QC;
    const float *xr = p.x + b * p.x_bstride;
    const int64_t xs0 = q0 * p.S + p.kmin;
    if (xs0 >= 0 && xs0 + p.win <= p.N) {
      // interior window: no range checks
      const float *src = xr + xs0;
      for (int e = tid; e < p.win; e += kDhThreads) cp_async_zfill<4>(&xb[smem_idx<PAD ? 4 : 0>(e)], src + e, true);
    } else {
      for (int e = tid; e < p.win; e += kDhThreads) {
        const int64_t gi = xs0 + e;
        const bool ok = gi >= 0 && gi < p.N;
        cp_async_zfill<4>(&xb[smem_idx<PAD ? 4 : 0>(e)], ok ? (const void *)(xr + gi) : (const void *)xr, ok);
      }
    }
    const float *gr = p.gy + b * p.gy_bstride;
    const int64_t g0 = q0 * p.Nt;
    if (p.gal && g0 + gyn <= p.out_len) {
      // a whole tile of 16-byte aligned gradient rows: 16-byte copies
      const float *src = gr + g0;
      for (int e4 = tid; e4 < gyn / 4; e4 += kDhThreads) cp_async_zfill<16>(&gb[4 * e4], src + 4 * e4, true);
    } else {
      for (int e = tid; e < gyn; e += kDhThreads) {
        const int64_t gi = g0 + e;
        const bool ok = gi < p.out_len;
        cp_async_zfill<4>(&gb[e], ok ? (const void *)(gr + gi) : (const void *)gr, ok);
      }
    }
  };

  // unit assignment: thread -> (unit u, row slice r) for UPT units spaced by U/UPT... kept simple:
  // units u = tid % Ueff + m * Ueff (m < UPT), slice r = tid / Ueff
  const int Ueff = (p.U + UPT - 1) / UPT;
  const int r = tid / Ueff;
  const bool active = r < p.RS;
  int kb[UPT], gcol[UPT];
  bool uok[UPT];
#pragma unroll
  for (int m = 0; m < UPT; m++) {
    const int u = (tid % Ueff) + m * Ueff;
    uok[m] = active && u < p.U;
    const int g = uok[m] ? u / units_per_g : 0;
    const int kq = uok[m] ? (u - g * units_per_g) * 4 : 0;
    const int64_t kl0 = ceil_div(p.c + 4 * (int64_t)g * p.down - p.Lo + 1, p.up);
    kb[m] = (int)(kl0 - p.kmin) + kq;
    gcol[m] = 4 * g;
  }
  float acc[UPT][16];
#pragma unroll
  for (int m = 0; m < UPT; m++)
#pragma unroll
    for (int e = 0; e < 16; e++) acc[m][e] = 0.f;

  if (tid == 0) GBFIR_TC_TRACE(3, 0, 1);
  int64_t tile = blockIdx.x;
  if (tile < p.ntiles) issue(tile, xb0, gb0);
  cp_async_commit();
  for (int it = 0; tile < p.ntiles; tile += gridDim.x, ++it) {
    float *xc = (it & 1) ? xb1 : xb0;
    float *gc = (it & 1) ? gb1 : gb0;
    const int64_t next = tile + gridDim.x;
    if (tid == 0) GBFIR_TC_TRACE(0, it, 0);
    if (next < p.ntiles) issue(next, (it & 1) ? xb0 : xb1, (it & 1) ? gb0 : gb1);
    cp_async_commit();
    if (tid == 0) GBFIR_TC_TRACE(0, it, 1);
    cp_async_wait<1>();
    __syncthreads();
    if (tid == 0) GBFIR_TC_TRACE(0, it, 2);
    if (active) {
      for (int q = r; q < p.QC; q += p.RS) {
        const int xq = q * (int)p.S;
        const float *gq = gc + q * (int)p.Nt;
#pragma unroll
        for (int m = 0; m < UPT; m++) {
          if (!uok[m]) continue;
          const float4 gv = *reinterpret_cast<const float4 *>(gq + gcol[m]);
          float xv[4];
#pragma unroll
          for (int kk = 0; kk < 4; kk++) xv[kk] = xc[smem_idx<PAD ? 4 : 0>(xq + kb[m] + kk)];
#pragma unroll
          for (int kk = 0; kk < 4; kk++) {
            acc[m][kk * 4 + 0] = fmaf(xv[kk], gv.x, acc[m][kk * 4 + 0]);
            acc[m][kk * 4 + 1] = fmaf(xv[kk], gv.y, acc[m][kk * 4 + 1]);
            acc[m][kk * 4 + 2] = fmaf(xv[kk], gv.z, acc[m][kk * 4 + 2]);
            acc[m][kk * 4 + 3] = fmaf(xv[kk], gv.w, acc[m][kk * 4 + 3]);
          }
        }
      }
    }
    __syncthreads();
  }
  cp_async_wait<0>();
  if (tid == 0) GBFIR_TC_TRACE(2, 0, 0);

  // ---- deterministic reduction: row slices, then taps -------------------------------
#pragma unroll
  for (int m = 0; m < UPT; m++) {
    if (!uok[m]) continue;
    const int u = (tid % Ueff) + m * Ueff;
#pragma unroll
    for (int e = 0; e < 16; e++) red[((size_t)r * p.U + u) * 16 + e] = acc[m][e];
  }
  __syncthreads();
  if (tid == 0) GBFIR_TC_TRACE(2, 0, 1);
  double *dred = reinterpret_cast<double *>(xb0);  // window buffers are free now: [U][16] doubles
  // the row slices' sums: compensated FP32 (the rounding error of each addition carried into
  // the next, in slice order), kept as a double — as exact as FP64 additions of these few
  // FP32 terms, without the slow FP64 pipe
  for (int e = tid; e < p.U * 16; e += kDhThreads) {
    float sf = 0.f, cf = 0.f;
    for (int rr = 0; rr < p.RS; rr++) {
      const float y = __fsub_rn(red[(size_t)rr * p.U * 16 + e], cf);
      const float t = __fadd_rn(sf, y);
      cf = __fsub_rn(__fsub_rn(t, sf), y);
      sf = t;
    }
    dred[e] = (double)sf - (double)cf;
  }
  __syncthreads();
  if (tid == 0) GBFIR_TC_TRACE(2, 0, 3);
  double *part = p.partial + (size_t)blockIdx.x * p.Lo;
  // 32-bit index arithmetic (tile-local quantities); along the phases j0, j0 + up, ... the
  // input position k steps by down
  const int upi = (int)p.up, dni = (int)p.down, ci = (int)p.c, Loi = (int)p.Lo, Nti = (int)p.Nt;
  for (int tp = tid; tp < Loi; tp += kDhThreads) {
    int res = (tp - ci) % upi;
    if (res < 0) res += upi;
    const int j0 = (int)(((int64_t)res * p.inv_down) % upi);
    int k = (ci + j0 * dni - tp) / upi;
    double s = 0.0;
    for (int mm = 0, j = j0; mm < (int)p.G && j < Nti; mm++, j += upi, k += dni) {
      const int g = j >> 2, jj = j & 3;
      const int num = ci + 4 * g * dni - Loi + 1;  // kl0 = ceil(num / up)
      const int kl0 = num >= 0 ? (num + upi - 1) / upi : -((-num) / upi);
      const int kk = k - kl0;
      if (kk < 0 || kk >= p.span) continue;
      s += dred[((g * units_per_g + kk / 4) * 16) + (kk % 4) * 4 + jj];
    }
    part[tp] = s;
  }
  if (tid == 0) GBFIR_TC_TRACE(2, 0, 2);
}

// dh[m] = scale * sum_p partial[p][m + off]  (fixed order over the partial rows)
// One warp per tap: lane l sums the partials l, l + 32, ... in FP64, then the 32 lane sums
// are added in a fixed shuffle tree — a fixed order, so the result is deterministic — and the
// partials' loads of a warp are in flight together instead of one dependent chain per tap.
__global__ void dh_reduce(const double *partial, int64_t nparts, int64_t Lo, int64_t off, int64_t L, double scale,
                          float *dh) {
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t m = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); m < L; m += nwarps) {
    double s = 0.0;
    for (int64_t q = lane; q < nparts; q += 32) s += partial[q * Lo + m + off];
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) s += __shfl_xor_sync(0xffffffffu, s, d);
    if (lane == 0) dh[m] = (float)(s * scale);
  }
}

// Direct dh for rates whose row tile is too large: thread per (tap, chunk of lattice
// points) over all rows:  dh[t] = sum_b sum_s gy[n0 + upk*s] * x[i0 + dn*s].
__global__ void dh_direct(DhParams p, int64_t batch, int64_t nchunks) {
  const int64_t total = p.Lo * nchunks;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t ch = e / p.Lo, tp = e - ch * p.Lo;
    // n*dn - i*upk = tp - c; smallest n >= 0 with a valid i >= 0
    int64_t res = (tp - p.c) % p.up;
    if (res < 0) res += p.up;
    int64_t n = (res * p.inv_down) % p.up;  // n*dn == tp - c (mod upk)
    int64_t i = (p.c + n * p.down - tp) / p.up;
    if (i < 0) {  // step along the lattice until i >= 0
      const int64_t steps = (-i + p.down - 1) / p.down;
      n += steps * p.up;
      i += steps * p.down;
    }
    const int64_t nmax_s = min((p.out_len - 1 - n) / p.up, (p.N - 1 - i) / p.down);
    double s = 0.0;
    if (n < p.out_len && i < p.N && nmax_s >= 0) {
      const int64_t per = (nmax_s + nchunks) / nchunks;
      const int64_t s0 = ch * per, s1 = min(nmax_s, s0 + per - 1);
      for (int64_t b = 0; b < batch; b++) {
        const float *gr = p.gy + b * p.gy_bstride;
        const float *xr = p.x + b * p.x_bstride;
        float acc = 0.f;
        for (int64_t q = s0; q <= s1; q++) acc = fmaf(gr[n + p.up * q], xr[i + p.down * q], acc);
        s += (double)acc;
      }
    }
    p.partial[ch * p.Lo + tp] = s;
  }
}

static int64_t mod_inverse(int64_t a, int64_t m) {
  if (m == 1) return 0;
  int64_t g = m, x = 0, x1 = 1, aa = a % m;
  while (aa) {
    const int64_t q = g / aa;
    int64_t t = g - q * aa;
    g = aa;
    aa = t;
    t = x - q * x1;
    x = x1;
    x1 = t;
  }
  return ((x % m) + m) % m;
}

static int max_parts() { return 2 * num_sms(); }

struct DhPlan {
  DhParams p;
  bool tiled;
  int upt;
  bool pad;
  size_t smem;
  int64_t grid, nchunks;
};

static DhPlan plan_dh(const float *x, int64_t x_bstride, int64_t N, const float *gy, int64_t gy_bstride,
                      int64_t out_len, int64_t batch, int64_t L, int64_t upk, int64_t dn, int64_t c_override,
                      bool odd_extend) {
  DhPlan pl{};
  const int64_t G = 4 / gcd64(upk, 4);
  RsGeom geo = plan_geometry(upk, dn, L, out_len, G, c_override, odd_extend);
  const int span4 = (geo.span + 3) & ~3;
  DhParams &p = pl.p;
  p.x = x;
  p.x_bstride = batch > 1 ? x_bstride : 0;
  p.N = N;
  p.gy = gy;
  p.gy_bstride = batch > 1 ? gy_bstride : 0;
  p.out_len = out_len;
  p.gal = (reinterpret_cast<uintptr_t>(gy) % 16 == 0 && p.gy_bstride % 4 == 0) ? 1 : 0;
  p.up = upk;
  p.down = dn;
  p.Lo = geo.Lo;
  p.c = geo.c;
  p.Nt = geo.Nt;
  p.S = geo.S;
  p.ncg = geo.ncg;
  p.span = span4;
  p.kmin = geo.kmin;
  p.rows = geo.rows;
  p.G = G;
  p.inv_down = mod_inverse(dn % upk, upk);
  p.U = geo.ncg * (span4 / 4);
  pl.pad = (geo.S % 2) == 0;
  pl.upt = (p.U + kDhThreads - 1) / kDhThreads;
  const int64_t kmax = ceil_div(geo.c + 4 * (int64_t)(geo.ncg - 1) * dn - geo.Lo + 1, upk) + span4 - 1;
  if (pl.upt == 3) pl.upt = 4;
  pl.tiled = pl.upt <= 4;
  if (pl.tiled) {
    const int Ueff = (p.U + pl.upt - 1) / pl.upt;
    p.RS = kDhThreads / Ueff;
    int QC = 256;
    size_t smem = 0;
    int64_t win = 0, alloc = 0;
    for (;; QC /= 2) {
      win = (int64_t)(QC - 1) * geo.S + (kmax - geo.kmin) + 1;
      alloc = pl.pad ? win + (win >> 4) + 1 : win;
      // the two window buffers also hold the [U][16] FP64 reduction at the end
      alloc = std::max<int64_t>(alloc, (int64_t)p.U * 16);
      alloc = (alloc + 3) & ~3LL;  // keep the gy tiles 16-byte aligned
      smem = 2 * (size_t)alloc * sizeof(float) + 2 * (size_t)QC * geo.Nt * sizeof(float) +
             (size_t)p.RS * p.U * 16 * sizeof(float);
      if (smem <= 96 * 1024 || QC <= 8) break;
    }
    p.win = (int32_t)win;
    p.win_alloc = (int32_t)alloc;
    p.QC = QC;
    p.tiles_per_row = (geo.rows + QC - 1) / QC;
    p.ntiles = p.tiles_per_row * batch;
    pl.smem = smem;
    pl.tiled = smem <= 200 * 1024;
    pl.grid = std::min<int64_t>(p.ntiles, max_parts());
  }
  if (!pl.tiled) {
    pl.nchunks = std::max<int64_t>(1, std::min<int64_t>(max_parts(), (int64_t)(4 * num_sms() * 256 / geo.Lo) + 1));
    pl.grid = pl.nchunks;
  }
  return pl;
}

static int reduce_dh(const double *partial, int64_t nparts, int64_t Lo, int64_t even_off, int64_t L, double scale,
                     float *dh, cudaStream_t s) {
  dh_reduce<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>((L + 7) / 8, 4 * num_sms())), 256, 0, s>>>(
      partial, nparts, Lo, even_off, L, scale, dh);
  return check_launch("backward dh reduce");
}

static int run_dh(DhPlan &pl, int64_t batch, int64_t L, int64_t even_off, double scale, float *dh, void *ws,
                  size_t ws_bytes, cudaStream_t s) {
  DhParams &p = pl.p;
  const size_t need = (size_t)pl.grid * p.Lo * sizeof(double);
  if (ws == nullptr || ws_bytes < need)
    GBFIR_FAIL(GBFIR_ERR_WORKSPACE, "backward: dh needs %zu B of workspace, got %zu", need, ws_bytes);
  if (reinterpret_cast<uintptr_t>(ws) % 8) GBFIR_FAIL(GBFIR_ERR_ALIGNMENT, "backward: workspace not 8-byte aligned");
  p.partial = reinterpret_cast<double *>(ws);
  int rc;
  if (pl.tiled) {
    const void *fn = nullptr;
    if (pl.pad) {
      fn = pl.upt == 1 ? (const void *)rowtile_dh<true, 1> : pl.upt == 2 ? (const void *)rowtile_dh<true, 2>
                                                                        : (const void *)rowtile_dh<true, 4>;
    } else {
      fn = pl.upt == 1 ? (const void *)rowtile_dh<false, 1> : pl.upt == 2 ? (const void *)rowtile_dh<false, 2>
                                                                         : (const void *)rowtile_dh<false, 4>;
    }
    rc = ensure_smem(fn, pl.smem, "backward dh");
    if (rc) return rc;
    void *args[] = {&p};
    cudaError_t e = cudaLaunchKernel(fn, dim3((unsigned)pl.grid), dim3(kDhThreads), args, pl.smem, s);
    if (e != cudaSuccess) GBFIR_FAIL(GBFIR_ERR_CUDA, "backward dh: launch failed: %s", cudaGetErrorString(e));
    count_launch();
  } else {
    dh_direct<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>((p.Lo * pl.nchunks + 255) / 256, 4 * num_sms())),
                256, 0, s>>>(p, batch, pl.nchunks);
    rc = check_launch("backward dh (direct)");
    if (rc) return rc;
  }
  return reduce_dh(p.partial, pl.grid, p.Lo, even_off, L, scale, dh, s);
}

int tc_dh_partials(const float *x, int64_t x_bstride, int64_t N, const float *gy, int64_t gy_bstride, int64_t out_len,
                   int64_t batch, int64_t up, int64_t down, int64_t Lo, int64_t c, int precision, double *partial,
                   size_t partial_bytes, int64_t *nparts, cudaStream_t s);

// dh on the tensor cores (tc_dh.cu) where a row tile fits, else the FP32 reduction above.
static int run_dh_prec(DhPlan &pl, int precision, int64_t batch, int64_t L, int64_t even_off, double scale, float *dh,
                       void *ws, size_t ws_bytes, cudaStream_t s) {
  if (precision != GBFIR_PREC_FP32) {
    const DhParams &p = pl.p;
    if (ws == nullptr || reinterpret_cast<uintptr_t>(ws) % 8)
      GBFIR_FAIL(GBFIR_ERR_WORKSPACE, "backward dh: needs an 8-byte aligned workspace");
    int64_t nparts = 0;
    const int rc = tc_dh_partials(p.x, p.x_bstride, p.N, p.gy, p.gy_bstride, p.out_len, batch, p.up, p.down, p.Lo,
                                  p.c, precision, reinterpret_cast<double *>(ws), ws_bytes, &nparts, s);
    if (rc == GBFIR_SUCCESS) return reduce_dh(reinterpret_cast<double *>(ws), nparts, p.Lo, even_off, L, scale, dh, s);
    if (rc != GBFIR_ERR_NOT_SUPPORTED) return rc;
  }
  return run_dh(pl, batch, L, even_off, scale, dh, ws, ws_bytes, s);
}


// ---- allocation-free backward -----------------------------------------------------
// Scratch for gbfir_resample_poly_bwd_noalloc: the FP64 partial tap gradients of the
// dh reduction, GBFIR_NOALLOC_SCRATCH_BYTES per device.  Host code must not use the
// array's name as an address (it is a host-side stand-in); the device address is
// looked up per device with cudaGetSymbolAddress and passed to the kernels.  Each call
// writes every partial it later reads, so nothing has to be cleared between calls.
static __device__ __align__(256) double g_noalloc_scratch[GBFIR_NOALLOC_SCRATCH_BYTES / sizeof(double)];

static void *noalloc_scratch_address(int *rc_out) {
  static std::mutex mu;
  static void *addr[128] = {nullptr};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= 128) {
    *rc_out = GBFIR_ERR_CUDA;
    return nullptr;
  }
  std::lock_guard<std::mutex> lk(mu);
  if (!addr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      *rc_out = GBFIR_ERR_CUDA;
      return nullptr;
    }
    addr[dev] = p;
  }
  *rc_out = GBFIR_SUCCESS;
  return addr[dev];
}

static int check_real(const gbfir_buf &b, const char *name, bool allow_broadcast) {
  int rc = check_buf(b, name, allow_broadcast);
  if (rc) return rc;
  if (b.dtype != GBFIR_F32) GBFIR_FAIL(GBFIR_ERR_NOT_SUPPORTED, "%s: the adjoints take real float32 operands", name);
  return GBFIR_SUCCESS;
}

// Bounded-wait status of the row-tile launches made from this file (1 = a window copy
// did not complete); read and cleared by gbfir_tc_status().
int adjoint_rowtile_status() { return rowtile_status_take(); }

}  // namespace gbfir

using namespace gbfir;

namespace gbfir {
int conv1d_bwd_dx_tc(const gbfir_buf &dx, const gbfir_buf &gy, const gbfir_buf &h, int64_t start, int precision,
                     cudaStream_t s);
int resample_poly_bwd_dx_tc(const gbfir_buf &dx, const gbfir_buf &gy, const gbfir_buf &h, int64_t up, int64_t down,
                            int precision, cudaStream_t s);
}  // namespace gbfir

extern "C" {

size_t gbfir_resample_poly_bwd_workspace_size(int64_t batch, int64_t in_len, int64_t h_len, int64_t up,
                                              int64_t down) {
  (void)batch;
  (void)in_len;
  (void)up;
  (void)down;
  if (h_len < 1) return 0;
  return (size_t)max_parts() * (size_t)(h_len + 1) * sizeof(double);
}

static int resample_bwd_impl(gbfir_buf dx, gbfir_buf dh, gbfir_buf gy, gbfir_buf x, gbfir_buf h, int64_t up,
                             int64_t down, int32_t precision, void *workspace, size_t workspace_bytes,
                             gbfir_stream_t stream) {
  try {
    int rc;
    if ((rc = check_real(gy, "resample_poly_bwd gy", false))) return rc;
    if ((rc = check_real(x, "resample_poly_bwd x", false))) return rc;
    if ((rc = check_real(h, "resample_poly_bwd h", false))) return rc;
    if (up <= 0 || down <= 0) GBFIR_FAIL(GBFIR_ERR_INVALID_PARAMETER, "resample_poly_bwd: up/down must be positive");
    if (h.batch != 1) GBFIR_FAIL(GBFIR_ERR_INVALID_DIM, "resample_poly_bwd: the filter must be one row");
    if (gy.batch != x.batch) GBFIR_FAIL(GBFIR_ERR_INVALID_DIM, "resample_poly_bwd: gy/x batch mismatch");
    const int64_t up_size = x.len * up;
    const int64_t olen = up_size / down + ((up_size % down) ? 1 : 0);
    if (gy.len != olen) GBFIR_FAIL(GBFIR_ERR_INVALID_DIM, "resample_poly_bwd: gy length %lld, expected %lld",
                                   (long long)gy.len, (long long)olen);
    if (dx.ptr) {
      if ((rc = check_real(dx, "resample_poly_bwd dx", false))) return rc;
      if (dx.batch != x.batch || dx.len != x.len) GBFIR_FAIL(GBFIR_ERR_INVALID_DIM, "resample_poly_bwd: dx shape");
    }
    if (dh.ptr) {
      if ((rc = check_real(dh, "resample_poly_bwd dh", false))) return rc;
      if (dh.batch != 1 || dh.len != h.len) GBFIR_FAIL(GBFIR_ERR_INVALID_DIM, "resample_poly_bwd: dh shape");
    }
    const int64_t g = gcd64(up, down);
    up /= g;
    down /= g;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (up == 1 && down == 1) {  // forward was an identity copy
      if (dx.ptr) {
        cudaError_t e = cudaMemcpy2DAsync(dx.ptr, (size_t)std::max<int64_t>(dx.batch_stride, dx.len) * 4, gy.ptr,
                                          (size_t)std::max<int64_t>(gy.batch_stride, gy.len) * 4, (size_t)x.len * 4,
                                          (size_t)x.batch, cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess) GBFIR_FAIL(GBFIR_ERR_CUDA, "resample_poly_bwd: copy failed: %s", cudaGetErrorString(e));
      }
      if (dh.ptr) {
        cudaError_t e = cudaMemsetAsync(dh.ptr, 0, (size_t)h.len * 4, s);
        if (e != cudaSuccess) GBFIR_FAIL(GBFIR_ERR_CUDA, "resample_poly_bwd: memset failed: %s", cudaGetErrorString(e));
      }
      return GBFIR_SUCCESS;
    }
    if (dx.ptr && precision != GBFIR_PREC_FP32) {
      // dL/dx on the tensor cores: the transposed resampler as a Toeplitz MMA pass
      rc = resample_poly_bwd_dx_tc(dx, gy, h, up, down, precision, s);
      if (rc) return rc;
    } else if (dx.ptr) {
      TileChoice tc;
      rc = resample_pass<float, false, false>(gy.ptr, gy.batch_stride, gy.len, h.ptr, h.len, dx.ptr, dx.batch_stride,
                                              x.len, x.batch, down, up, -1, true, 1, (double)up, tc, s);
      if (rc) return rc;
    }
    if (dh.ptr) {
      DhPlan pl = plan_dh((const float *)x.ptr, x.batch_stride, x.len, (const float *)gy.ptr, gy.batch_stride, gy.len,
                          x.batch, h.len, up, down, -1, true);
      const int64_t even = (h.len % 2) == 0;
      return run_dh_prec(pl, precision, x.batch, h.len, even, (double)up, (float *)dh.ptr, workspace, workspace_bytes,
                         s);
    }
    return GBFIR_SUCCESS;
  } catch (...) {
    GBFIR_FAIL(GBFIR_ERR_CUDA, "resample_poly_bwd: internal exception");
  }
}


int gbfir_resample_poly_bwd(gbfir_buf dx, gbfir_buf dh, gbfir_buf gy, gbfir_buf x, gbfir_buf h, int64_t up,
                            int64_t down, void *workspace, size_t workspace_bytes, gbfir_stream_t stream) {
  return resample_bwd_impl(dx, dh, gy, x, h, up, down, GBFIR_PREC_FP32, workspace, workspace_bytes, stream);
}

int gbfir_resample_poly_bwd_prec(gbfir_buf dx, gbfir_buf dh, gbfir_buf gy, gbfir_buf x, gbfir_buf h, int64_t up,
                                 int64_t down, int32_t precision, void *workspace, size_t workspace_bytes,
                                 gbfir_stream_t stream) {
  if (precision < GBFIR_PREC_FP32 || precision > GBFIR_PREC_BF16X3)
    GBFIR_FAIL(GBFIR_ERR_INVALID_PARAMETER, "resample_poly_bwd: unknown precision %d", (int)precision);
  return resample_bwd_impl(dx, dh, gy, x, h, up, down, precision, workspace, workspace_bytes, stream);
}

int gbfir_resample_poly_bwd_noalloc(gbfir_buf dx, gbfir_buf dh, gbfir_buf gy, gbfir_buf x, gbfir_buf h, int64_t up,
                                    int64_t down, gbfir_stream_t stream) {
  try {
    int rc;
    if ((rc = check_real(gy, "resample_poly_bwd_noalloc gy", false))) return rc;
    if ((rc = check_real(x, "resample_poly_bwd_noalloc x", false))) return rc;
    if ((rc = check_real(h, "resample_poly_bwd_noalloc h", false))) return rc;
    if (up <= 0 || down <= 0)
      GBFIR_FAIL(GBFIR_ERR_INVALID_PARAMETER, "resample_poly_bwd_noalloc: up/down must be positive");
    if (h.batch != 1) GBFIR_FAIL(GBFIR_ERR_INVALID_DIM, "resample_poly_bwd_noalloc: the filter must be one row");
    if (gy.batch != x.batch) GBFIR_FAIL(GBFIR_ERR_INVALID_DIM, "resample_poly_bwd_noalloc: gy/x batch mismatch");
    const int64_t up_size = x.len * up;
    const int64_t olen = up_size / down + ((up_size % down) ? 1 : 0);
    if (gy.len != olen)
      GBFIR_FAIL(GBFIR_ERR_INVALID_DIM, "resample_poly_bwd_noalloc: gy length %lld, expected %lld",
                 (long long)gy.len, (long long)olen);
    if (dx.ptr) {
      if ((rc = check_real(dx, "resample_poly_bwd_noalloc dx", false))) return rc;
      if (dx.batch != x.batch || dx.len != x.len)
        GBFIR_FAIL(GBFIR_ERR_INVALID_DIM, "resample_poly_bwd_noalloc: dx shape");
    }
    if (dh.ptr) {
      if ((rc = check_real(dh, "resample_poly_bwd_noalloc dh", false))) return rc;
      if (dh.batch != 1 || dh.len != h.len) GBFIR_FAIL(GBFIR_ERR_INVALID_DIM, "resample_poly_bwd_noalloc: dh shape");
    }
    const int64_t g = gcd64(up, down);
    up /= g;
    down /= g;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    DhPlan pl{};
    const bool need_dh = dh.ptr && !(up == 1 && down == 1);
    if (need_dh) {
      pl = plan_dh((const float *)x.ptr, x.batch_stride, x.len, (const float *)gy.ptr, gy.batch_stride, gy.len,
                   x.batch, h.len, up, down, -1, true);
      const size_t need = (size_t)pl.grid * pl.p.Lo * sizeof(double);
      if (need > GBFIR_NOALLOC_SCRATCH_BYTES)
        GBFIR_FAIL(GBFIR_ERR_INVALID_SIZE,
                   "resample_poly_bwd_noalloc: %lld taps need %zu B of scratch, the built-in maximum is %u B; use "
                   "gbfir_resample_poly_bwd with a workspace",
                   (long long)h.len, need, (unsigned)GBFIR_NOALLOC_SCRATCH_BYTES);
    }
    int src = GBFIR_SUCCESS;
    void *scratch = need_dh ? noalloc_scratch_address(&src) : nullptr;
    if (need_dh && !scratch)
      GBFIR_FAIL(src, "resample_poly_bwd_noalloc: cannot look up the scratch address on the current device");
    if (up == 1 && down == 1) {  // forward was an identity copy
      if (dx.ptr) {
        cudaError_t e = cudaMemcpy2DAsync(dx.ptr, (size_t)std::max<int64_t>(dx.batch_stride, dx.len) * 4, gy.ptr,
                                          (size_t)std::max<int64_t>(gy.batch_stride, gy.len) * 4, (size_t)x.len * 4,
                                          (size_t)x.batch, cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess)
          GBFIR_FAIL(GBFIR_ERR_CUDA, "resample_poly_bwd_noalloc: copy failed: %s", cudaGetErrorString(e));
      }
      if (dh.ptr) {
        cudaError_t e = cudaMemsetAsync(dh.ptr, 0, (size_t)h.len * 4, s);
        if (e != cudaSuccess)
          GBFIR_FAIL(GBFIR_ERR_CUDA, "resample_poly_bwd_noalloc: memset failed: %s", cudaGetErrorString(e));
      }
      return GBFIR_SUCCESS;
    }
    if (dx.ptr) {
      TileChoice tc;
      rc = resample_pass<float, false, false>(gy.ptr, gy.batch_stride, gy.len, h.ptr, h.len, dx.ptr, dx.batch_stride,
                                              x.len, x.batch, down, up, -1, true, 1, (double)up, tc, s);
      if (rc) return rc;
    }
    if (need_dh) {
      const int64_t even = (h.len % 2) == 0;
      return run_dh(pl, x.batch, h.len, even, (double)up, (float *)dh.ptr, scratch, GBFIR_NOALLOC_SCRATCH_BYTES, s);
    }
    return GBFIR_SUCCESS;
  } catch (...) {
    GBFIR_FAIL(GBFIR_ERR_CUDA, "resample_poly_bwd_noalloc: internal exception");
  }
}

size_t gbfir_conv1d_bwd_workspace_size(int64_t batch, int64_t in_len, int64_t h_len, int32_t mode) {
  (void)batch;
  (void)in_len;
  (void)mode;
  if (h_len < 1) return 0;
  return (size_t)max_parts() * (size_t)h_len * sizeof(double);
}

static int conv_bwd_impl(gbfir_buf dx, gbfir_buf dh, gbfir_buf gy, gbfir_buf x, gbfir_buf h, int32_t mode,
                         int32_t precision, void *workspace, size_t workspace_bytes, gbfir_stream_t stream) {
  try {
    int rc;
    if ((rc = check_real(gy, "conv1d_bwd gy", false))) return rc;
    if ((rc = check_real(x, "conv1d_bwd x", false))) return rc;
    if ((rc = check_real(h, "conv1d_bwd h", false))) return rc;
    if (h.batch != 1) GBFIR_FAIL(GBFIR_ERR_NOT_SUPPORTED, "conv1d_bwd: the filter must be one broadcast row");
    if (gy.batch != x.batch) GBFIR_FAIL(GBFIR_ERR_INVALID_DIM, "conv1d_bwd: gy/x batch mismatch");
    if (mode < GBFIR_MODE_FULL || mode > GBFIR_MODE_VALID)
      GBFIR_FAIL(GBFIR_ERR_INVALID_PARAMETER, "conv1d_bwd: unknown mode %d", (int)mode);
    const int64_t N = x.len, L = h.len, mx = std::max(N, L), mn = std::min(N, L);
    const int64_t olen = mode == GBFIR_MODE_FULL ? N + L - 1 : mode == GBFIR_MODE_SAME ? mx : mx - mn + 1;
    if (gy.len != olen) GBFIR_FAIL(GBFIR_ERR_INVALID_SIZE, "conv1d_bwd: gy length %lld, expected %lld",
                                   (long long)gy.len, (long long)olen);
    if (dx.ptr) {
      if ((rc = check_real(dx, "conv1d_bwd dx", false))) return rc;
      if (dx.batch != x.batch || dx.len != N) GBFIR_FAIL(GBFIR_ERR_INVALID_DIM, "conv1d_bwd: dx shape");
    }
    if (dh.ptr) {
      if ((rc = check_real(dh, "conv1d_bwd dh", false))) return rc;
      if (dh.batch != 1 || dh.len != L) GBFIR_FAIL(GBFIR_ERR_INVALID_DIM, "conv1d_bwd: dh shape");
    }
    const int64_t start = mode == GBFIR_MODE_SAME ? ((mn & 1) ? (mn - 1) / 2 : mn / 2 - 1)
                        : mode == GBFIR_MODE_VALID ? mn - 1 : 0;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (dx.ptr && precision != GBFIR_PREC_FP32) {
      rc = conv1d_bwd_dx_tc(dx, gy, h, start, precision, s);
      if (rc) return rc;
    } else if (dx.ptr) {
      TileChoice tc;
      rc = resample_pass<float, false, false>(gy.ptr, gy.batch_stride, gy.len, h.ptr, L, dx.ptr, dx.batch_stride, N,
                                              x.batch, 1, 1, L - 1 - start, false, 1, 1.0, tc, s);
      if (rc) return rc;
    }
    if (dh.ptr) {
      DhPlan pl = plan_dh((const float *)x.ptr, x.batch_stride, N, (const float *)gy.ptr, gy.batch_stride, gy.len,
                          x.batch, L, 1, 1, start, false);
      return run_dh_prec(pl, precision, x.batch, L, 0, 1.0, (float *)dh.ptr, workspace, workspace_bytes, s);
    }
    return GBFIR_SUCCESS;
  } catch (...) {
    GBFIR_FAIL(GBFIR_ERR_CUDA, "conv1d_bwd: internal exception");
  }
}

int gbfir_conv1d_bwd(gbfir_buf dx, gbfir_buf dh, gbfir_buf gy, gbfir_buf x, gbfir_buf h, int32_t mode,
                     void *workspace, size_t workspace_bytes, gbfir_stream_t stream) {
  return conv_bwd_impl(dx, dh, gy, x, h, mode, GBFIR_PREC_FP32, workspace, workspace_bytes, stream);
}

int gbfir_conv1d_bwd_prec(gbfir_buf dx, gbfir_buf dh, gbfir_buf gy, gbfir_buf x, gbfir_buf h, int32_t mode,
                          int32_t precision, void *workspace, size_t workspace_bytes, gbfir_stream_t stream) {
  if (precision < GBFIR_PREC_FP32 || precision > GBFIR_PREC_BF16X3)
    GBFIR_FAIL(GBFIR_ERR_INVALID_PARAMETER, "conv1d_bwd: unknown precision %d", (int)precision);
  return conv_bwd_impl(dx, dh, gy, x, h, mode, precision, workspace, workspace_bytes, stream);
}

}  // extern "C"
