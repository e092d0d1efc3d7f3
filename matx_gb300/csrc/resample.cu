// resample.cu — plain FP32/FP64 polyphase resampler for sm_103a.
//
// Semantics are MatX's resample_poly (include/matx/transforms/resample_poly.h:212-281
// host loop, :299-354 gcd/identity, include/matx/kernels/resample_poly.cuh:269-376):
//   y[n] = up * sum_i x[i] * he[c + n*down - i*up],  he = h with a leading zero
//   when L is even, c = (Lodd-1)/2, taps outside [0, Lodd) and x outside [0, N) are 0.
//
// Schedule ("row tiles", no MatX counterpart).  Outputs are grouped into rows of
// Nt = up*G consecutive outputs; row q needs inputs from q*S + k with S = down*G,
// so every row sees the same tap matrix B[k][j] = he[c + j*down - k*up].  The
// columns j are cut into groups of 4 adjacent phases; group g only needs the
// band k in [kl0(g), kl0(g)+span) (its union band), stored in shared memory as
// one float4 (real taps) per k.  A warp's 32 lanes take 32 different rows of the
// same column group, so the tap read is a warp-wide broadcast and each input
// sample read from shared memory feeds 4 phases x RQ rows of FMAs.
// A persistent CTA walks tiles of QC rows; the next tile's input window is
// prefetched with cp.async (zero-filled outside the signal) while the current
// one is computed.
#include "common.cuh"

namespace gbfir {

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
  double scale;      // up
};

// Resample tile override set by the autotuner hook.
static int g_rq_override = 0, g_wc_override = 0, g_group_override = 0;

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

template <bool PAD>
__device__ __forceinline__ int smem_idx(int p) {
  if constexpr (PAD) return p + (p >> 4);
  else return p;
}

template <typename T, bool XC, bool HC, int RQ, bool PAD>
__global__ void __launch_bounds__(256) resample_rowtile(const RsParams p) {
  using XT = typename val_of<T, XC>::type;
  using HT = typename val_of<T, HC>::type;
  using OT = typename val_of<T, XC || HC>::type;
  constexpr bool OC = XC || HC;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  TapVec<T, HC> *table = reinterpret_cast<TapVec<T, HC> *>(smem_raw);
  const size_t table_bytes = ((size_t)p.ncg * p.span * sizeof(TapVec<T, HC>) + 15) & ~(size_t)15;
  XT *xbuf0 = reinterpret_cast<XT *>(smem_raw + table_bytes);
  XT *xbuf1 = xbuf0 + p.win_alloc;

  const int tid = threadIdx.x;
  const HT *hp = reinterpret_cast<const HT *>(p.h);
  const XT *xp = reinterpret_cast<const XT *>(p.x);
  OT *op = reinterpret_cast<OT *>(p.out);

  // ---- tap table: table[g*span + kk].v[jj] = he[c + (4g+jj)*down - (kl0(g)+kk)*up]
  const int nent = p.ncg * p.span * 4;
  for (int e = tid; e < nent; e += blockDim.x) {
    const int g = e / (p.span * 4);
    const int rem = e - g * (p.span * 4);
    const int kk = rem >> 2, jj = rem & 3;
    const int64_t j = 4 * (int64_t)g + jj;
    const int64_t kl0 = ceil_div(p.c + 4 * (int64_t)g * p.down - p.Lo + 1, p.up);
    const int64_t tp = p.c + j * p.down - (kl0 + kk) * p.up;
    HT v = zero_val<HT>();
    if (j < p.Nt && tp >= 0 && tp < p.Lo && !(p.even && tp == 0)) v = hp[tp - p.even];
    table[g * p.span + kk].v[jj] = v;
  }

  auto issue_loads = [&](int64_t tile, XT *buf) {
    const int64_t b = tile / p.tiles_per_row;
    const int64_t q0 = (tile - b * p.tiles_per_row) * p.QC;
    const int64_t xs0 = q0 * p.S + p.kmin;
    const XT *row = xp + b * p.x_bstride;
    for (int e = tid; e < p.win; e += blockDim.x) {
      const int64_t gi = xs0 + e;
      const bool ok = gi >= 0 && gi < p.N;
      cp_async_zfill<sizeof(XT)>(&buf[smem_idx<PAD>(e)], ok ? (const void *)(row + gi) : (const void *)row, ok);
    }
  };

  int64_t tile = blockIdx.x;
  if (tile < p.ntiles) issue_loads(tile, xbuf0);
  cp_async_commit();

  const int wid = tid >> 5, lane = tid & 31;
  const int wr = wid / p.WC, wc = wid - wr * p.WC;
  const T scale = T(p.scale);

  for (int it = 0; tile < p.ntiles; tile += gridDim.x, ++it) {
    XT *cur = (it & 1) ? xbuf1 : xbuf0;
    XT *nxt = (it & 1) ? xbuf0 : xbuf1;
    const int64_t next = tile + gridDim.x;
    if (next < p.ntiles) issue_loads(next, nxt);
    cp_async_commit();
    cp_async_wait<1>();
    __syncthreads();

    const int64_t b = tile / p.tiles_per_row;
    const int64_t q0 = (tile - b * p.tiles_per_row) * p.QC;
    OT *orow = op + b * p.out_bstride;
    const int rbase = wr * 32 * RQ + lane;  // local row of slice i is rbase + 32*i

    for (int g = wc; g < p.ncg; g += p.WC) {
      const int64_t kl0 = ceil_div(p.c + 4 * (int64_t)g * p.down - p.Lo + 1, p.up);
      const int kb = (int)(kl0 - p.kmin);
      int base[RQ];
#pragma unroll
      for (int i = 0; i < RQ; i++) base[i] = (rbase + 32 * i) * (int)p.S + kb;
      Acc<T, OC> acc[RQ][4];
#pragma unroll
      for (int i = 0; i < RQ; i++)
#pragma unroll
        for (int jj = 0; jj < 4; jj++) acc[i][jj].zero();
      const TapVec<T, HC> *tg = table + g * p.span;
#pragma unroll 2
      for (int kk = 0; kk < p.span; kk++) {
        const TapVec<T, HC> t = tg[kk];
#pragma unroll
        for (int i = 0; i < RQ; i++) {
          const XT xv = cur[smem_idx<PAD>(base[i] + kk)];
#pragma unroll
          for (int jj = 0; jj < 4; jj++) mac<T, XC, HC>(acc[i][jj], xv, t.v[jj]);
        }
      }
#pragma unroll
      for (int i = 0; i < RQ; i++) {
        const int64_t q = q0 + rbase + 32 * i;
#pragma unroll
        for (int jj = 0; jj < 4; jj++) {
          const int64_t j = 4 * (int64_t)g + jj;
          const int64_t n = q * p.Nt + j;
          if (j < p.Nt && n < p.out_len) orow[n] = pack<T, OC>(acc[i][jj], scale);
        }
      }
    }
    __syncthreads();
  }
  cp_async_wait<0>();
}

// Direct form for tap/rate combinations whose row tile does not fit in shared
// memory (very large up or down): one output per thread iteration, the input
// window read through L1, the filter from shared memory when it fits.  Same
// index arithmetic as the MatX host loop (resample_poly.h:239-262).
template <typename T, bool XC, bool HC>
__global__ void __launch_bounds__(256) resample_direct(const RsParams p, int h_in_smem) {
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
  const int64_t half = p.Lo / 2;
  const int64_t total = p.out_len * p.rows;  // rows == batch here
  const T scale = T(p.scale);
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / p.out_len, n = e - b * p.out_len;
    const XT *row = xp + b * p.x_bstride;
    const int64_t up_ind = n * p.down;
    const int64_t up_start = up_ind > half ? up_ind - half : 0;
    const int64_t up_end = min((p.N - 1) * p.up, up_ind + half);
    const int64_t x_start = (up_start + p.up - 1) / p.up;
    const int64_t x_end = up_end / p.up;
    int64_t h_ind = p.c + (up_ind - p.up * x_start);
    Acc<T, OC> acc;
    acc.zero();
    for (int64_t i = x_start; i <= x_end; i++, h_ind -= p.up) {
      if (p.even && h_ind == 0) continue;
      mac<T, XC, HC>(acc, row[i], hh[h_ind - p.even]);
    }
    op[b * p.out_bstride + n] = pack<T, OC>(acc, scale);
  }
}

// Identity (up == down after the gcd): out = in, with real->complex widening.
template <typename T, bool XC, bool OC>
__global__ void resample_identity(const void *x, int64_t x_bstride, void *out, int64_t out_bstride,
                                  int64_t n, int64_t batch) {
  using XT = typename val_of<T, XC>::type;
  using OT = typename val_of<T, OC>::type;
  const XT *xp = reinterpret_cast<const XT *>(x);
  OT *op = reinterpret_cast<OT *>(out);
  const int64_t total = n * batch;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / n, i = e - b * n;
    const XT v = xp[b * x_bstride + i];
    if constexpr (OC && !XC) {
      OT o;
      o.x = v;
      o.y = 0;
      op[b * out_bstride + i] = o;
    } else {
      op[b * out_bstride + i] = v;
    }
  }
}

// ---------------------------------------------------------------------------------

struct RsChoice {
  int rq, wc;
  int64_t group;
};

template <typename T, bool XC, bool HC, int RQ, bool PAD>
static int launch_rowtile(RsParams &p, size_t smem, cudaStream_t s) {
  auto fn = resample_rowtile<T, XC, HC, RQ, PAD>;
  int rc = ensure_smem((const void *)fn, smem, "resample_poly");
  if (rc) return rc;
  int occ = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, 256, smem);
  if (occ < 1) GBFIR_FAIL(GBFIR_ERR_NOT_SUPPORTED, "resample_poly: tile needs %zu B of shared memory", smem);
  int64_t grid = (int64_t)num_sms() * occ;
  if (grid > p.ntiles) grid = p.ntiles;
  fn<<<(unsigned)grid, 256, smem, s>>>(p);
  return check_launch("resample_poly");
}

template <typename T, bool XC, bool HC>
static int dispatch_rq(RsParams &p, int rq, bool pad, size_t smem, cudaStream_t s) {
  if (pad) {
    if (rq == 1) return launch_rowtile<T, XC, HC, 1, true>(p, smem, s);
    if constexpr (sizeof(T) == 4) {
      if (rq == 2) return launch_rowtile<T, XC, HC, 2, true>(p, smem, s);
      return launch_rowtile<T, XC, HC, 4, true>(p, smem, s);
    }
  } else {
    if (rq == 1) return launch_rowtile<T, XC, HC, 1, false>(p, smem, s);
    if constexpr (sizeof(T) == 4) {
      if (rq == 2) return launch_rowtile<T, XC, HC, 2, false>(p, smem, s);
      return launch_rowtile<T, XC, HC, 4, false>(p, smem, s);
    }
  }
  return launch_rowtile<T, XC, HC, 1, false>(p, smem, s);
}

// Host planning shared by the forward launch and the ragged planner.
struct RsGeom {
  int64_t up, down, Lo, c, Nt, S, kmin, kmax, rows;
  int32_t even, ncg, span;
};

static RsGeom plan_geometry(int64_t up, int64_t down, int64_t L, int64_t out_len, int64_t G) {
  RsGeom g{};
  g.up = up;
  g.down = down;
  g.even = (L % 2) == 0;
  g.Lo = L + g.even;
  g.c = (g.Lo - 1) / 2;
  g.Nt = up * G;
  g.S = down * G;
  g.ncg = (int32_t)((g.Nt + 3) / 4);
  int64_t span = 1;
  for (int64_t grp = 0; grp < g.ncg; grp++) {
    const int64_t j0 = 4 * grp;
    const int64_t jl = std::min<int64_t>(j0 + 3, g.Nt - 1);
    const int64_t kl0 = ceil_div(g.c + j0 * down - g.Lo + 1, up);
    const int64_t kh = floor_div(g.c + jl * down, up);
    span = std::max<int64_t>(span, kh - kl0 + 1);
  }
  span = (span + 1) & ~1LL;  // even, for the 2x unrolled band loop
  g.span = (int32_t)span;
  g.kmin = ceil_div(g.c - g.Lo + 1, up);
  g.kmax = ceil_div(g.c + 4 * (int64_t)(g.ncg - 1) * down - g.Lo + 1, up) + span - 1;
  g.rows = (out_len + g.Nt - 1) / g.Nt;
  return g;
}

template <typename T, bool XC, bool HC>
static int run_resample(const gbfir_buf &out, const gbfir_buf &in, const gbfir_buf &h, int64_t up, int64_t down,
                        cudaStream_t s) {
  using XT = typename val_of<T, XC>::type;
  using HT = typename val_of<T, HC>::type;
  // Row grouping: the smallest G with Nt = up*G a multiple of 4.
  int64_t G = g_group_override > 0 ? g_group_override : 4 / gcd64(up, 4);
  RsGeom geo = plan_geometry(up, down, h.len, out.len, G);
  int wc = 1;
  if (g_wc_override > 0) {
    wc = g_wc_override;
  } else {
    while (wc < 8 && wc * 2 <= geo.ncg) wc *= 2;
  }
  if (wc > geo.ncg) wc = 1;
  const bool pad = (geo.S % 2) == 0;
  auto smem_for = [&](int rq) -> size_t {
    const int64_t QC = 32LL * rq * (8 / wc);
    const int64_t win = (QC - 1) * geo.S + (geo.kmax - geo.kmin) + 1;
    const int64_t alloc = pad ? win + (win >> 4) + 1 : win;
    const size_t table = ((size_t)geo.ncg * geo.span * 4 * sizeof(HT) + 15) & ~(size_t)15;
    return table + 2 * (size_t)alloc * sizeof(XT);
  };
  int rq = g_rq_override > 0 ? g_rq_override : 2;
  if (sizeof(T) == 8) rq = 1;
  while (rq > 1 && smem_for(rq) > 110 * 1024) rq /= 2;
  const size_t smem = smem_for(rq);

  RsParams p{};
  p.x = in.ptr;
  p.x_bstride = in.batch_stride;
  p.N = in.len;
  p.h = h.ptr;
  p.Lo = geo.Lo;
  p.even = geo.even;
  p.c = geo.c;
  p.out = out.ptr;
  p.out_bstride = out.batch_stride;
  p.out_len = out.len;
  p.up = up;
  p.down = down;
  p.Nt = geo.Nt;
  p.S = geo.S;
  p.ncg = geo.ncg;
  p.span = geo.span;
  p.kmin = geo.kmin;
  p.rows = geo.rows;
  p.QC = 32 * rq * (8 / wc);
  p.WC = wc;
  p.tiles_per_row = (geo.rows + p.QC - 1) / p.QC;
  p.ntiles = p.tiles_per_row * out.batch;
  const int64_t win = (int64_t)(p.QC - 1) * geo.S + (geo.kmax - geo.kmin) + 1;
  p.win = (int32_t)win;
  p.win_alloc = (int32_t)(pad ? win + (win >> 4) + 1 : win);
  p.scale = (double)up;
  if (out.batch > 1 && in.batch_stride == 0) p.x_bstride = 0;
  if (smem <= 200 * 1024) return dispatch_rq<T, XC, HC>(p, rq, pad, smem, s);

  // row tile too large for shared memory: direct form
  p.rows = out.batch;
  const size_t hbytes = (size_t)h.len * sizeof(HT);
  const int h_in_smem = hbytes <= 96 * 1024;
  const size_t dsmem = h_in_smem ? hbytes : 0;
  auto fn = resample_direct<T, XC, HC>;
  int rc = ensure_smem((const void *)fn, dsmem, "resample_poly");
  if (rc) return rc;
  const int64_t total = out.len * out.batch;
  int64_t grid = (total + 255) / 256;
  const int64_t cap = (int64_t)num_sms() * 4;
  if (grid > cap) grid = cap;
  fn<<<(unsigned)grid, 256, dsmem, s>>>(p, h_in_smem);
  return check_launch("resample_poly (direct)");
}

template <typename T, bool XC, bool OC>
static int run_identity(const gbfir_buf &out, const gbfir_buf &in, cudaStream_t s) {
  const int64_t total = out.batch * in.len;
  int64_t grid = (total + 255) / 256;
  const int64_t cap = (int64_t)num_sms() * 8;
  if (grid > cap) grid = cap;
  if (grid < 1) grid = 1;
  resample_identity<T, XC, OC><<<(unsigned)grid, 256, 0, s>>>(in.ptr, in.batch_stride, out.ptr, out.batch_stride,
                                                               in.len, out.batch);
  return check_launch("resample_poly (identity)");
}

int resample_poly_fp(const gbfir_buf &out, const gbfir_buf &in, const gbfir_buf &h, int64_t up, int64_t down,
                     cudaStream_t s) {
  const bool xc = dtype_complex(in.dtype), hc = dtype_complex(h.dtype);
  const bool dbl = dtype_double(in.dtype);
  if (up == 1 && down == 1) {
    const bool oc = dtype_complex(out.dtype);
    if (dbl) {
      if (xc) return run_identity<double, true, true>(out, in, s);
      return oc ? run_identity<double, false, true>(out, in, s) : run_identity<double, false, false>(out, in, s);
    }
    if (xc) return run_identity<float, true, true>(out, in, s);
    return oc ? run_identity<float, false, true>(out, in, s) : run_identity<float, false, false>(out, in, s);
  }
  if (dbl) {
    if (xc && hc) return run_resample<double, true, true>(out, in, h, up, down, s);
    if (xc) return run_resample<double, true, false>(out, in, h, up, down, s);
    if (hc) return run_resample<double, false, true>(out, in, h, up, down, s);
    return run_resample<double, false, false>(out, in, h, up, down, s);
  }
  if (xc && hc) return run_resample<float, true, true>(out, in, h, up, down, s);
  if (xc) return run_resample<float, true, false>(out, in, h, up, down, s);
  if (hc) return run_resample<float, false, true>(out, in, h, up, down, s);
  return run_resample<float, false, false>(out, in, h, up, down, s);
}

int set_resample_tile(int rq, int wc, int group) {
  if (rq != 0 && rq != 1 && rq != 2 && rq != 4) return GBFIR_ERR_INVALID_PARAMETER;
  if (wc != 0 && wc != 1 && wc != 2 && wc != 4 && wc != 8) return GBFIR_ERR_INVALID_PARAMETER;
  if (group < 0 || group > 64) return GBFIR_ERR_INVALID_PARAMETER;
  g_rq_override = rq;
  g_wc_override = wc;
  g_group_override = group;
  return GBFIR_SUCCESS;
}

}  // namespace gbfir
