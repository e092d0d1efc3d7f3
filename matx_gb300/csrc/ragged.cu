// ragged.cu — one persistent launch over thousands of uneven resampling jobs
// (no MatX counterpart; MatX runs one resample_poly launch per signal,
// include/matx/transforms/resample_poly.h:299-354).
//
// Every signal (complex64 in/out, real taps, its own length, tap count and up/down) is
// cut by the host planner into row tiles of its own row-tile geometry (rowtile.cuh):
// rows of Nt = up*G outputs, QC = 32*RQ*(8/WC) rows per tile, 8-phase super-groups split
// over WC warps.  The tile shape (RQ, WC, G) of a signal comes from the tile registry
// (gbfir_ragged_tile_register, filled by the autotuner per reduced rate and tap-length
// bucket) or from the built-in heuristic.  Consecutive tiles of one signal are grouped
// into work items of roughly equal cost, ordered most expensive first.  CTAs take work
// items from an atomic counter (dynamic scheduling: a 1e6-sample signal next to a
// 1e3-sample one costs no idle SMs); per item a CTA derives the geometry once, builds the
// signal's tap table once and walks the item's tiles with the next tile's input window
// prefetched by cp.async into the second of two buffers while the current one is
// computed (even strides in the conflict-free XOR layout of rowtile.cuh for that
// signal's stride).  The per-tile compute is the single-signal kernel's.  Taking an item
// is one atomicAdd: no CTA ever waits on another, so nothing can spin.  The launch
// contains no host synchronisation and can be captured in a CUDA graph.
#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "rowtile.cuh"

namespace gbfir {

constexpr int kRgThreads = 256;
constexpr int kIdentityChunk = 8192;
constexpr int64_t kRgWindowCap = 6144;  // samples per window the heuristic aims to stay under

// Tile shape of one signal, packed into one int64 of its work items:
// rows per thread | column warps << 4 | row group << 8 (0 fields: heuristic).
__host__ __device__ inline int64_t rg_pack(int rq, int wc, int group) {
  return (int64_t)rq | ((int64_t)wc << 4) | ((int64_t)group << 8);
}
// shape bit of a signal whose tiles take the paired walk (even row stride, 16-byte aligned
// signal): set by the planner, not by the tile registry
constexpr int64_t kRgPair = (int64_t)1 << 16;

// Row-tile geometry of one ragged signal; identical on host and device.
struct RgGeom {
  int64_t up, down, Lo, c, Nt, S, kmin, kmax, rows;
  int32_t even, ncg, span, WC, QC, RQ, identity, pair;
};

__host__ __device__ inline int64_t gcd_hd(int64_t a, int64_t b) {
  while (b) {
    const int64_t t = a % b;
    a = b;
    b = t;
  }
  return a;
}

__host__ __device__ inline int64_t rg_window(const RgGeom &g) {
  return (int64_t)(g.QC - 1) * g.S + (g.kmax - g.kmin) + 1;
}
__host__ __device__ inline int64_t rg_window_alloc(const RgGeom &g) {
  const int64_t w = rg_window(g);
  return (g.S % 2 == 0) ? (w + 15) / 16 * 16 : w;  // the XOR layouts permute inside blocks of 16
}

// Geometry for a packed shape.  The heuristic: G = 4 / gcd(up, 4) (rows of a multiple of 4
// outputs), RQ = 1, and the column warps the largest power of two <= 8 dividing the
// super-groups, or more (unbalanced) while the window exceeds kRgWindowCap samples.
__host__ __device__ inline RgGeom rg_geometry(int64_t up, int64_t down, int64_t L, int64_t out_len, int64_t shape) {
  RgGeom g{};
  const int64_t gg = gcd_hd(up, down);
  up /= gg;
  down /= gg;
  g.up = up;
  g.down = down;
  g.identity = (up == 1 && down == 1);
  if (g.identity) {
    g.rows = (out_len + kIdentityChunk - 1) / kIdentityChunk;
    g.QC = 1;
    g.RQ = 1;
    return g;
  }
  const int srq = (int)(shape & 15), swc = (int)((shape >> 4) & 15), sgroup = (int)((shape >> 8) & 255);
  const int64_t G = sgroup > 0 ? sgroup : 4 / gcd_hd(up, 4);
  g.even = (L % 2) == 0;
  g.Lo = L + g.even;
  g.c = (g.Lo - 1) / 2;
  g.Nt = up * G;
  g.S = down * G;
  g.ncg = (int32_t)((g.Nt + 3) / 4);
  // the paired walk needs an even row stride with ctz(S/2) <= 7 (rowtile.cuh's unit layouts)
  g.pair = ((shape & kRgPair) && g.S % 2 == 0 && ((g.S >> 1) & 255) != 0) ? 1 : 0;
  int64_t span = 1;
  for (int64_t grp = 0; grp < g.ncg; grp++) {
    const int64_t j0 = 4 * grp;
    const int64_t jl = (j0 + 3 < g.Nt - 1) ? j0 + 3 : g.Nt - 1;
    const int64_t kl0 = band_start(g.c, grp, down, g.Lo, up, g.pair != 0);
    const int64_t kh = floor_div(g.c + jl * down, up);
    if (kh - kl0 + 1 > span) span = kh - kl0 + 1;
  }
  g.span = (int32_t)((span + 1) & ~1LL);
  g.kmin = band_start(g.c, 0, down, g.Lo, up, g.pair != 0);
  g.kmax = band_start(g.c, g.ncg - 1, down, g.Lo, up, g.pair != 0) + g.span - 1;
  g.rows = (out_len + g.Nt - 1) / g.Nt;
  const int nsg = (g.ncg + 1) / 2;
  g.RQ = (srq == 1 || srq == 2) ? srq : 1;
  if (swc == 1 || swc == 2 || swc == 4 || swc == 8) {
    g.WC = swc;
  } else {
    int wc = 1;
    while (wc < 8 && nsg % (wc * 2) == 0) wc *= 2;
    g.WC = wc;
    g.QC = 32 * g.RQ * (8 / wc);
    while (g.WC < 8 && g.WC < nsg && rg_window(g) > kRgWindowCap) {
      g.WC *= 2;
      g.QC = 32 * g.RQ * (8 / g.WC);
    }
  }
  g.QC = 32 * g.RQ * (8 / g.WC);
  return g;
}

struct RgParams {
  const gbfir_ragged_desc *descs;
  const int64_t *items;  // [nitems][4]: signal, first row, rows, packed shape
  int64_t nitems;
  unsigned long long *counter;
  int32_t table_bytes;   // shared bytes reserved for the tap table
  int32_t win_elems;     // elements per window buffer
  int32_t nbuf;          // window buffers (2: prefetch the next tile of the item)
};

// The tiles of one work item: rows [row0, row0 + nrows) of signal p, QC rows per tile.
template <int RQ, int PAD>
__device__ __forceinline__ void rg_run_item(const RsParams &p, int64_t row0, int64_t nrows, float2 *buf0, float2 *buf1,
                                            int nbuf, const unsigned char *table, int tid) {
  const int wid = tid >> 5, lane = tid & 31;
  const int wr = wid / p.WC, wc = wid - wr * p.WC;
  const float2 *row = reinterpret_cast<const float2 *>(p.x);
  float2 *orow = reinterpret_cast<float2 *>(p.out);
  const int ntl = (int)((nrows + p.QC - 1) / p.QC);
  auto issue = [&](int t, float2 *buf) {
    const int64_t xs0 = (row0 + (int64_t)t * p.QC) * p.S + p.kmin;
    if constexpr (PAD >= 20) {
      // paired walk: units of two samples (xs0 is even); the last may hold one of the signal
      float4 *bu = reinterpret_cast<float4 *>(buf);
      const int nu = (p.win + 1) >> 1;
      for (int u = tid; u < nu; u += kRgThreads) {
        const int64_t gi = xs0 + 2 * u;
        const int nb = (gi >= 0 && gi < p.N) ? (gi + 1 < p.N ? 16 : 8) : 0;
        cp_async16_part(&bu[unit_idx<PAD>(u)], nb ? (const void *)(row + gi) : (const void *)row, nb);
      }
    } else if (xs0 >= 0 && xs0 + p.win <= p.N) {
      const float2 *src = row + xs0;
      for (int e = tid; e < p.win; e += kRgThreads) cp_async_zfill<8>(&buf[smem_idx<PAD>(e)], src + e, true);
    } else {
      for (int e = tid; e < p.win; e += kRgThreads) {
        const int64_t gi = xs0 + e;
        const bool ok = gi >= 0 && gi < p.N;
        cp_async_zfill<8>(&buf[smem_idx<PAD>(e)], ok ? (const void *)(row + gi) : (const void *)row, ok);
      }
    }
  };
  issue(0, buf0);
  cp_async_commit();
  for (int t = 0; t < ntl; t++) {
    float2 *cur = (nbuf == 2 && (t & 1)) ? buf1 : buf0;
    if (nbuf == 2) {
      if (t + 1 < ntl) issue(t + 1, (t & 1) ? buf0 : buf1);
      cp_async_commit();
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
    rowtile_compute<float, true, false, RQ, PAD>(p, cur, table, orow, row0 + (int64_t)t * p.QC, wr, wc, lane,
                                                 (float)p.scale, 0);
    __syncthreads();
    if (nbuf == 1 && t + 1 < ntl) {
      issue(t + 1, buf0);
      cp_async_commit();
    }
  }
  cp_async_wait<0>();
}

template <int RQ>
__device__ __forceinline__ void rg_dispatch_pad(int pad, const RsParams &p, int64_t row0, int64_t nrows, float2 *b0,
                                                float2 *b1, int nbuf, const unsigned char *table, int tid) {
  switch (pad) {
    case 0: rg_run_item<RQ, 0>(p, row0, nrows, b0, b1, nbuf, table, tid); break;
    case 11: rg_run_item<RQ, 11>(p, row0, nrows, b0, b1, nbuf, table, tid); break;
    case 12: rg_run_item<RQ, 12>(p, row0, nrows, b0, b1, nbuf, table, tid); break;
    case 13: rg_run_item<RQ, 13>(p, row0, nrows, b0, b1, nbuf, table, tid); break;
    case 14: rg_run_item<RQ, 14>(p, row0, nrows, b0, b1, nbuf, table, tid); break;
    case 15: rg_run_item<RQ, 15>(p, row0, nrows, b0, b1, nbuf, table, tid); break;
    case 16: rg_run_item<RQ, 16>(p, row0, nrows, b0, b1, nbuf, table, tid); break;
    case 17: rg_run_item<RQ, 17>(p, row0, nrows, b0, b1, nbuf, table, tid); break;
    case 20: rg_run_item<RQ, 20>(p, row0, nrows, b0, b1, nbuf, table, tid); break;
    case 21: rg_run_item<RQ, 21>(p, row0, nrows, b0, b1, nbuf, table, tid); break;
    case 22: rg_run_item<RQ, 22>(p, row0, nrows, b0, b1, nbuf, table, tid); break;
    case 23: rg_run_item<RQ, 23>(p, row0, nrows, b0, b1, nbuf, table, tid); break;
    case 24: rg_run_item<RQ, 24>(p, row0, nrows, b0, b1, nbuf, table, tid); break;
    case 25: rg_run_item<RQ, 25>(p, row0, nrows, b0, b1, nbuf, table, tid); break;
    case 26: rg_run_item<RQ, 26>(p, row0, nrows, b0, b1, nbuf, table, tid); break;
    default: rg_run_item<RQ, 27>(p, row0, nrows, b0, b1, nbuf, table, tid); break;
  }
}

__global__ void __launch_bounds__(kRgThreads) ragged_rowtile(const RgParams rp) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned char *table = smem_raw;
  float2 *xbuf0 = reinterpret_cast<float2 *>(smem_raw + rp.table_bytes);
  float2 *xbuf1 = xbuf0 + rp.win_elems;
  __shared__ long long s_item;
  __shared__ RsParams s_p;
  __shared__ int s_identity, s_pad, s_rq;
  const int tid = threadIdx.x;

  for (;;) {
    if (tid == 0) s_item = (long long)atomicAdd(rp.counter, 1ULL);
    __syncthreads();
    const int64_t it = s_item;
    if (it >= rp.nitems) break;
    const int64_t sig = rp.items[4 * it], row0 = rp.items[4 * it + 1], nrows = rp.items[4 * it + 2];
    const int64_t shape = rp.items[4 * it + 3];
    const gbfir_ragged_desc d = rp.descs[sig];
    if (tid == 0) {
      const RgGeom g = rg_geometry(d.up, d.down, d.h_len, d.out_len, shape);
      RsParams p{};
      p.x = d.in;
      p.N = d.in_len;
      p.h = d.h;
      p.Lo = g.Lo;
      p.even = g.even;
      p.c = g.c;
      p.out = d.out;
      p.out_len = d.out_len;
      p.up = g.up;
      p.down = g.down;
      p.Nt = g.Nt;
      p.S = g.S;
      p.ncg = g.ncg;
      p.span = g.span;
      p.kmin = g.kmin;
      p.rows = g.rows;
      p.QC = g.QC;
      p.WC = g.WC;
      p.win = (int32_t)rg_window(g);
      p.scale = (double)g.up;
      p.pair = g.pair;
      s_p = p;
      s_identity = g.identity;
      s_rq = g.RQ;
      // even row strides: the conflict-free XOR window layout for t = ctz(S), or the paired
      // walk's unit layout for ctz(S/2) (rowtile.cuh)
      int t = 0;
      while (t < 7 && ((g.S >> t) & 1) == 0) t++;
      if (g.pair) {
        int t2 = 0;
        while (t2 < 7 && (((g.S >> 1) >> t2) & 1) == 0) t2++;
        s_pad = 20 + t2;
      } else {
        s_pad = t ? 10 + t : 0;
      }
    }
    __syncthreads();
    // a private copy: read through the shared struct, the fields would be reloaded after every
    // store the compiler cannot prove does not alias it
    const RsParams p = s_p;
    if (s_identity) {
      const float2 *xi = reinterpret_cast<const float2 *>(d.in);
      float2 *yo = reinterpret_cast<float2 *>(d.out);
      const int64_t e0 = row0 * kIdentityChunk;
      const int64_t e1 = min(d.out_len, (row0 + nrows) * kIdentityChunk);
      for (int64_t e = e0 + tid; e < e1; e += kRgThreads) yo[e] = xi[e];
      __syncthreads();
      continue;
    }
    // the tap table is read only after the first window wait's barrier inside the item
    build_tap_table<float, true, false>(p, reinterpret_cast<const float *>(p.h), table, tid, kRgThreads);
    if (s_rq == 2) rg_dispatch_pad<2>(s_pad, p, row0, nrows, xbuf0, xbuf1, rp.nbuf, table, tid);
    else rg_dispatch_pad<1>(s_pad, p, row0, nrows, xbuf0, xbuf1, rp.nbuf, table, tid);
    __syncthreads();
  }
}

static int64_t table_bytes_of(const RgGeom &g) {
  return g.identity ? 0 : (int64_t)tap_table_bytes<float, true, false>(g.ncg, g.span);
}

// Tile registry of the ragged planner: packed shape per (reduced up, reduced down, tap-length
// bucket = the smallest power of two >= the tap count).
static std::mutex g_rg_mu;
static std::map<std::tuple<int64_t, int64_t, int64_t>, int64_t> g_rg_tiles;

static int64_t rg_bucket(int64_t L) {
  int64_t b = 1;
  while (b < L) b <<= 1;
  return b;
}

static int64_t rg_shape_for(int64_t up, int64_t down, int64_t L) {
  const int64_t g = gcd_hd(up, down);
  std::lock_guard<std::mutex> lk(g_rg_mu);
  auto it = g_rg_tiles.find(std::make_tuple(up / g, down / g, rg_bucket(L)));
  return it == g_rg_tiles.end() ? 0 : it->second;
}

// Descriptor checks shared by the planners (host copies): 0 or a negative status.
static int64_t rg_validate(const gbfir_ragged_desc *descs, int64_t count) {
  for (int64_t s = 0; s < count; s++) {
    const gbfir_ragged_desc &d = descs[s];
    char buf[256];
    if (!d.in || !d.out || !d.h) {
      snprintf(buf, sizeof(buf), "ragged_plan: signal %lld has a null pointer", (long long)s);
      set_error(buf);
      return -GBFIR_ERR_NULL_POINTER;
    }
    if (d.in_len < 1 || d.h_len < 1 || d.up < 1 || d.down < 1) {
      snprintf(buf, sizeof(buf), "ragged_plan: signal %lld has a non-positive length or rate", (long long)s);
      set_error(buf);
      return -GBFIR_ERR_INVALID_PARAMETER;
    }
    const int64_t up_size = d.in_len * d.up;
    const int64_t olen = up_size / d.down + ((up_size % d.down) ? 1 : 0);
    if (d.out_len != olen) {
      snprintf(buf, sizeof(buf), "ragged_plan: signal %lld out_len %lld, expected %lld", (long long)s,
               (long long)d.out_len, (long long)olen);
      set_error(buf);
      return -GBFIR_ERR_INVALID_DIM;
    }
    if ((reinterpret_cast<uintptr_t>(d.in) | reinterpret_cast<uintptr_t>(d.out)) % 8 ||
        reinterpret_cast<uintptr_t>(d.h) % 4) {
      snprintf(buf, sizeof(buf), "ragged_plan: signal %lld has a misaligned pointer", (long long)s);
      set_error(buf);
      return -GBFIR_ERR_ALIGNMENT;
    }
  }
  return 0;
}

// tensor-core form (tc_blocks.cu)
int64_t ragged_plan_tc(const gbfir_ragged_desc *descs, int64_t count, int precision, int64_t *table,
                       int64_t *shared_bytes, int64_t *kchunk);
int ragged_resample_tc(const gbfir_ragged_desc *device_descs, const int64_t *device_items, int64_t nitems,
                       int64_t shared_bytes, int64_t kchunk, int precision, void *workspace, cudaStream_t s);

}  // namespace gbfir

using namespace gbfir;

extern "C" {

size_t gbfir_ragged_workspace_size(int64_t count, int64_t num_tiles) {
  (void)count;
  (void)num_tiles;
  return 256;
}

int gbfir_ragged_tile_register(int64_t up, int64_t down, int64_t h_len, int32_t rows_per_thread, int32_t col_warps,
                               int32_t group) {
  if (up > 0 && down > 0 && h_len > 0 && rows_per_thread == 0 && col_warps == 0 && group == 0) {
    const int64_t g = gcd64(up, down);
    std::lock_guard<std::mutex> lk(g_rg_mu);
    g_rg_tiles.erase(std::make_tuple(up / g, down / g, rg_bucket(h_len)));
    return GBFIR_SUCCESS;
  }
  if (up <= 0 || down <= 0 || h_len <= 0 || (rows_per_thread != 1 && rows_per_thread != 2) ||
      (col_warps != 1 && col_warps != 2 && col_warps != 4 && col_warps != 8) || group < 1 || group > 64)
    GBFIR_FAIL(GBFIR_ERR_INVALID_PARAMETER,
               "ragged_tile_register: rows_per_thread 1 or 2, col_warps 1/2/4/8, group 1..64, positive rates");
  const int64_t g = gcd64(up, down);
  std::lock_guard<std::mutex> lk(g_rg_mu);
  g_rg_tiles[std::make_tuple(up / g, down / g, rg_bucket(h_len))] = rg_pack(rows_per_thread, col_warps, group);
  return GBFIR_SUCCESS;
}

int gbfir_ragged_tile_clear(void) {
  std::lock_guard<std::mutex> lk(g_rg_mu);
  g_rg_tiles.clear();
  return GBFIR_SUCCESS;
}

int64_t gbfir_ragged_plan(const gbfir_ragged_desc *descs, int64_t count, int64_t *tile_table,
                          gbfir_ragged_plan_info *info) {
  if (descs == nullptr || count <= 0) {
    set_error("ragged_plan: no descriptors");
    return -GBFIR_ERR_INVALID_PARAMETER;
  }
  {
    const int64_t rc = rg_validate(descs, count);
    if (rc) return rc;
  }
  struct Sig {
    RgGeom g;
    int64_t shape, ntiles;
    double tile_cost;
  };
  std::vector<Sig> sigs((size_t)count);
  int64_t max_table = 0, max_win = 0;
  double total = 0;
  for (int64_t s = 0; s < count; s++) {
    const gbfir_ragged_desc &d = descs[s];
    Sig &sg = sigs[(size_t)s];
    sg.shape = rg_shape_for(d.up, d.down, d.h_len);
    // the paired walk where the signal is 16-byte aligned (its row stride decides the rest)
    if ((reinterpret_cast<uintptr_t>(d.in) & 15) == 0) sg.shape |= kRgPair;
    sg.g = rg_geometry(d.up, d.down, d.h_len, d.out_len, sg.shape);
    const RgGeom &g = sg.g;
    if (!g.identity) {
      max_table = std::max(max_table, table_bytes_of(g));
      max_win = std::max(max_win, rg_window_alloc(g));
    }
    sg.ntiles = (g.rows + g.QC - 1) / g.QC;
    // cost of one tile: its multiply-adds plus its window traffic (in MAC-equivalents)
    sg.tile_cost = g.identity ? (double)kIdentityChunk
                              : (double)g.QC * g.Nt * ((double)d.h_len / g.up + 1) + 4.0 * (double)rg_window(g);
    total += sg.tile_cost * (double)sg.ntiles;
  }
  const int64_t tb = (max_table + 15) & ~15LL;
  // whole 16-byte units per buffer, so the second buffer keeps the 16-byte alignment the paired
  // walk's unit copies and loads need
  max_win = (max_win + 1) / 2 * 2;
  int nbuf = 2;
  int64_t smem = tb + 2 * max_win * 8;
  if (smem > 200 * 1024) {
    nbuf = 1;
    smem = tb + max_win * 8;
  }
  if (smem > 200 * 1024) {
    set_error("ragged_plan: a signal's tile needs more than 200 KB of shared memory");
    return -GBFIR_ERR_NOT_SUPPORTED;
  }
  // Work items: runs of consecutive tiles of one signal, each about 1/8 of a CTA's fair share
  // (SMs x 2 resident CTAs), so the tap table and geometry are set up once per run while
  // the most-expensive-first order still balances the tail.
  const double target = total / ((double)num_sms() * 2.0 * 8.0);
  struct Item {
    double cost;
    int64_t sig, row0, nrows, shape;
  };
  std::vector<Item> items;
  for (int64_t s = 0; s < count; s++) {
    const Sig &sg = sigs[(size_t)s];
    int64_t per = (int64_t)(target / std::max(sg.tile_cost, 1.0));
    per = std::max<int64_t>(1, std::min<int64_t>(per, sg.ntiles));
    for (int64_t k = 0; k < sg.ntiles; k += per) {
      const int64_t n = std::min<int64_t>(per, sg.ntiles - k);
      const int64_t row0 = k * sg.g.QC;
      const int64_t nrows = std::min<int64_t>(n * sg.g.QC, sg.g.rows - row0);
      items.push_back({sg.tile_cost * (double)n, s, row0, nrows, sg.shape});
    }
  }
  const int64_t nitems = (int64_t)items.size();
  if (tile_table) {
    std::stable_sort(items.begin(), items.end(), [](const Item &a, const Item &b) { return a.cost > b.cost; });
    for (size_t i = 0; i < items.size(); i++) {
      tile_table[4 * i] = items[i].sig;
      tile_table[4 * i + 1] = items[i].row0;
      tile_table[4 * i + 2] = items[i].nrows;
      tile_table[4 * i + 3] = items[i].shape;
    }
  }
  if (info) {
    info->num_tiles = nitems;
    info->shared_bytes = smem < 16 ? 16 : smem;
    info->table_bytes = tb;
    info->window_elems = max_win;
    info->buffers = nbuf;
    info->precision = GBFIR_PREC_FP32;
  }
  return nitems;
}

int64_t gbfir_ragged_plan_prec(const gbfir_ragged_desc *descs, int64_t count, int32_t precision,
                               int64_t *tile_table, gbfir_ragged_plan_info *info) {
  if (precision == GBFIR_PREC_FP32) return gbfir_ragged_plan(descs, count, tile_table, info);
  if (precision < GBFIR_PREC_FP32 || precision > GBFIR_PREC_BF16X3) {
    set_error("ragged_plan: unknown precision");
    return -GBFIR_ERR_INVALID_PARAMETER;
  }
  if (descs == nullptr || count <= 0) {
    set_error("ragged_plan: no descriptors");
    return -GBFIR_ERR_INVALID_PARAMETER;
  }
  const int64_t rc = rg_validate(descs, count);
  if (rc) return rc;
  int64_t smem = 0, kchunk = 0;
  const int64_t nitems = ragged_plan_tc(descs, count, precision, tile_table, &smem, &kchunk);
  if (nitems < 0) return nitems;
  if (info) {
    info->num_tiles = nitems;
    info->shared_bytes = smem;
    info->table_bytes = 0;
    info->window_elems = kchunk;  // the tensor-core plan's K chunk
    info->buffers = 0;
    info->precision = precision;
  }
  return nitems;
}

int gbfir_ragged_resample(const gbfir_ragged_desc *device_descs, int64_t count, const int64_t *device_tile_table,
                          const gbfir_ragged_plan_info *info, int32_t precision, void *workspace,
                          size_t workspace_bytes, gbfir_stream_t stream) {
  if (!device_descs || !device_tile_table || !info || count <= 0 || info->num_tiles <= 0)
    GBFIR_FAIL(GBFIR_ERR_INVALID_PARAMETER, "ragged_resample: empty plan");
  const int64_t nitems = info->num_tiles;
  if (precision != info->precision)
    GBFIR_FAIL(GBFIR_ERR_INVALID_PARAMETER, "ragged_resample: the plan was made for precision %lld, not %d",
               (long long)info->precision, (int)precision);
  if (!workspace || workspace_bytes < gbfir_ragged_workspace_size(count, nitems))
    GBFIR_FAIL(GBFIR_ERR_WORKSPACE, "ragged_resample: workspace missing or too small");
  if (reinterpret_cast<uintptr_t>(workspace) % 8) GBFIR_FAIL(GBFIR_ERR_ALIGNMENT, "ragged_resample: workspace");
  if (precision != GBFIR_PREC_FP32)
    return ragged_resample_tc(device_descs, device_tile_table, nitems, info->shared_bytes, info->window_elems,
                              precision, workspace, reinterpret_cast<cudaStream_t>(stream));
  const int64_t table_bytes = info->table_bytes;
  const int64_t smem = info->shared_bytes;
  const int64_t nbuf = info->buffers, win = info->window_elems;
  if (smem <= 0 || smem > 200 * 1024 || table_bytes < 0 || table_bytes > smem || (table_bytes & 15) ||
      (nbuf != 1 && nbuf != 2) || win < 0 || table_bytes + nbuf * win * 8 > smem)
    GBFIR_FAIL(GBFIR_ERR_INVALID_PARAMETER, "ragged_resample: plan info does not come from gbfir_ragged_plan");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemsetAsync(workspace, 0, 8, s);
  if (e != cudaSuccess) GBFIR_FAIL(GBFIR_ERR_CUDA, "ragged_resample: %s", cudaGetErrorString(e));
  int rc = ensure_smem((const void *)ragged_rowtile, (size_t)smem, "ragged_resample");
  if (rc) return rc;
  int occ = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, ragged_rowtile, kRgThreads, (size_t)smem);
  if (occ < 1) occ = 1;
  int64_t grid = (int64_t)num_sms() * occ;
  if (grid > nitems) grid = nitems;
  RgParams rp{};
  rp.descs = device_descs;
  rp.items = device_tile_table;
  rp.nitems = nitems;
  rp.counter = reinterpret_cast<unsigned long long *>(workspace);
  rp.table_bytes = (int32_t)table_bytes;
  rp.win_elems = (int32_t)win;
  rp.nbuf = (int32_t)nbuf;
  ragged_rowtile<<<(unsigned)grid, kRgThreads, (size_t)smem, s>>>(rp);
  return check_launch("ragged_resample");
}

}  // extern "C"
