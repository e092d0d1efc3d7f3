// resample.cu — plain FP32/FP64 polyphase resampler for sm_103a.
//
// Semantics are MatX's resample_poly (include/matx/transforms/resample_poly.h:212-281
// host loop, :299-354 gcd/identity, include/matx/kernels/resample_poly.cuh:269-376):
//   y[n] = up * sum_i x[i] * he[c + n*down - i*up],  he = h with a leading zero
//   when L is even, c = (Lodd-1)/2, taps outside [0, Lodd) and x outside [0, N) are 0.
//
// Schedule (no MatX counterpart): the row-tile kernel of rowtile.cuh, with a
// direct per-output kernel for rates whose tiles do not fit in shared memory.
#include <mutex>
#include <unordered_map>

#include "rowtile.cuh"

namespace gbfir {

// Resample tile override set by the autotuner hook.
static int g_rq_override = 0, g_wc_override = 0, g_group_override = 0, g_nbuf_override = 0;

// Autotuned tiles per (reduced up, reduced down, filter length).
struct TileKey {
  int64_t up, down, L;
  bool operator==(const TileKey &o) const { return up == o.up && down == o.down && L == o.L; }
};
struct TileKeyHash {
  size_t operator()(const TileKey &k) const {
    return std::hash<int64_t>()(k.up * 1000003 + k.down * 7919 + k.L);
  }
};
static std::mutex g_tile_mu;
static std::unordered_map<TileKey, TileChoice, TileKeyHash> g_tiles;

static bool valid_tile(int rq, int wc, int group, int nbuf) {
  // column warps: 1, 2, 4, 8 (8/wc row slices per CTA) or 9..16 (one row slice, rows per thread 1 or 2)
  // buffers: 1 or 2 window buffers (0 = heuristic) or 3 = the ring form (a staging warp and
  // 3-4 window slots; complex float signals with real taps, else 2), plus 4 for the
  // TMA-store epilogue, plus 8 for the ring form's paired walk (even row strides)
  return (rq == 0 || rq == 1 || rq == 2 || rq == 4) && (wc >= 0 && wc <= 16 && (wc <= 8 ? 8 % (wc ? wc : 1) == 0 : rq <= 2)) &&
         group >= 0 && group <= 64 && (nbuf & ~15) == 0;
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

template <typename T, bool XC, bool HC>
static int run_resample(const gbfir_buf &out, const gbfir_buf &in, const gbfir_buf &h, int64_t up, int64_t down,
                        cudaStream_t s) {
  TileChoice tc;
  {
    std::lock_guard<std::mutex> lk(g_tile_mu);
    auto it = g_tiles.find(TileKey{up, down, h.len});
    if (it != g_tiles.end()) tc = it->second;
  }
  if (g_rq_override) tc.rq = g_rq_override;
  if (g_wc_override) tc.wc = g_wc_override;
  if (g_group_override) tc.group = g_group_override;
  if (g_nbuf_override) tc.nbuf = g_nbuf_override;
  // buffers + 4 asks for the TMA-store epilogue (an explicit 1, 2 or 3 without it: direct
  // stores), + 8 the ring form's paired walk
  tc.ostore = (tc.nbuf & 4) ? 1 : tc.nbuf ? 0 : -1;
  tc.pair = (tc.nbuf & 8) != 0;
  tc.nbuf &= 3;
  return resample_pass<T, XC, HC, true>(in.ptr, in.batch_stride, in.len, h.ptr, h.len, out.ptr, out.batch_stride, out.len,
                                  out.batch, up, down, -1, true, 0, (double)up, tc, s);
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

int register_resample_tile(int64_t up, int64_t down, int64_t L, int rq, int wc, int group, int nbuf) {
  if (!valid_tile(rq, wc, group, nbuf) || up <= 0 || down <= 0 || L <= 0) return GBFIR_ERR_INVALID_PARAMETER;
  const int64_t g = gcd64(up, down);
  TileChoice tc;
  tc.rq = rq;
  tc.wc = wc;
  tc.group = group;
  tc.nbuf = nbuf;
  std::lock_guard<std::mutex> lk(g_tile_mu);
  g_tiles[TileKey{up / g, down / g, L}] = tc;
  return GBFIR_SUCCESS;
}

int clear_resample_tiles() {
  std::lock_guard<std::mutex> lk(g_tile_mu);
  g_tiles.clear();
  return GBFIR_SUCCESS;
}

int set_resample_tile(int rq, int wc, int group, int nbuf) {
  if (!valid_tile(rq, wc, group, nbuf)) return GBFIR_ERR_INVALID_PARAMETER;
  g_rq_override = rq;
  g_wc_override = wc;
  g_group_override = group;
  g_nbuf_override = nbuf;
  return GBFIR_SUCCESS;
}

// Bounded-wait status of the row-tile launches made from this file (1 = a window copy
// did not complete); read and cleared by gbfir_tc_status().
int resample_rowtile_status() { return rowtile_status_take(); }

}  // namespace gbfir
