// ragged.cu — one persistent launch over thousands of uneven resampling jobs
// (no MatX counterpart; MatX runs one resample_poly launch per signal).
//
// Every signal (complex64 in/out, real taps, its own length, tap count and up/down)
// is cut by the host planner into row tiles of its own row-tile geometry
// (rowtile.cuh): rows of Nt = up*G outputs, QC rows per tile, 8-phase super-groups
// split over WC warps.  The tile table is ordered most expensive first.  CTAs take
// tiles from an atomic counter (dynamic scheduling, so a 1e6-sample signal next to a
// 1e3-sample one costs no idle SMs), rebuild the tap table only when the signal
// changes, stage the tile's input window with cp.async (zero-filled; even strides in the
// conflict-free XOR layout of rowtile.cuh for that signal's stride) and run the same
// per-tile compute as the single-signal kernel.  Taking a tile is one atomicAdd: no
// CTA ever waits on another, so nothing can spin.  The launch contains no host
// synchronisation and can be captured in a CUDA graph.
#include <vector>

#include "rowtile.cuh"

namespace gbfir {

constexpr int kRgThreads = 256;
constexpr int kIdentityChunk = 8192;

// Row-tile geometry of one ragged signal; identical on host and device.
struct RgGeom {
  int64_t up, down, Lo, c, Nt, S, kmin, kmax, rows;
  int32_t even, ncg, span, WC, QC, identity;
};

__host__ __device__ inline int64_t gcd_hd(int64_t a, int64_t b) {
  while (b) {
    const int64_t t = a % b;
    a = b;
    b = t;
  }
  return a;
}

__host__ __device__ inline RgGeom rg_geometry(int64_t up, int64_t down, int64_t L, int64_t out_len) {
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
    return g;
  }
  const int64_t G = 4 / gcd_hd(up, 4);
  g.even = (L % 2) == 0;
  g.Lo = L + g.even;
  g.c = (g.Lo - 1) / 2;
  g.Nt = up * G;
  g.S = down * G;
  g.ncg = (int32_t)((g.Nt + 3) / 4);
  int64_t span = 1;
  for (int64_t grp = 0; grp < g.ncg; grp++) {
    const int64_t j0 = 4 * grp;
    const int64_t jl = (j0 + 3 < g.Nt - 1) ? j0 + 3 : g.Nt - 1;
    const int64_t kl0 = ceil_div(g.c + j0 * down - g.Lo + 1, up);
    const int64_t kh = floor_div(g.c + jl * down, up);
    if (kh - kl0 + 1 > span) span = kh - kl0 + 1;
  }
  g.span = (int32_t)((span + 1) & ~1LL);
  g.kmin = ceil_div(g.c - g.Lo + 1, up);
  g.kmax = ceil_div(g.c + 4 * (int64_t)(g.ncg - 1) * down - g.Lo + 1, up) + g.span - 1;
  g.rows = (out_len + g.Nt - 1) / g.Nt;
  const int nsg = (g.ncg + 1) / 2;
  int wc = 1;
  while (wc < 8 && nsg % (wc * 2) == 0) wc *= 2;
  g.WC = wc;
  g.QC = 32 * (8 / wc);
  return g;
}

__host__ __device__ inline int64_t rg_window(const RgGeom &g) { return (int64_t)(g.QC - 1) * g.S + (g.kmax - g.kmin) + 1; }
__host__ __device__ inline int64_t rg_window_alloc(const RgGeom &g) {
  const int64_t w = rg_window(g);
  return (g.S % 2 == 0) ? (w + 15) / 16 * 16 : w;  // the XOR layouts permute inside blocks of 16
}

struct RgParams {
  const gbfir_ragged_desc *descs;
  const int64_t *tiles;  // [ntiles][2]: signal, first row
  int64_t ntiles;
  unsigned long long *counter;
  int32_t table_bytes;   // shared bytes reserved for the tap table
};

__global__ void __launch_bounds__(kRgThreads) ragged_rowtile(const RgParams rp) {
  using XT = float2;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned char *table = smem_raw;
  XT *xbuf = reinterpret_cast<XT *>(smem_raw + rp.table_bytes);
  __shared__ long long s_tile;
  __shared__ RsParams s_p;
  __shared__ int s_identity, s_pad;
  const int tid = threadIdx.x;
  const int wid = tid >> 5, lane = tid & 31;
  int64_t last_sig = -1;

  for (;;) {
    if (tid == 0) s_tile = (long long)atomicAdd(rp.counter, 1ULL);
    __syncthreads();
    const int64_t t = s_tile;
    if (t >= rp.ntiles) break;
    const int64_t sig = rp.tiles[2 * t], q0 = rp.tiles[2 * t + 1];
    const gbfir_ragged_desc d = rp.descs[sig];
    if (tid == 0) {
      const RgGeom g = rg_geometry(d.up, d.down, d.h_len, d.out_len);
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
      s_p = p;
      s_identity = g.identity;
      // even row strides: the conflict-free XOR window layout for t = ctz(S) (rowtile.cuh)
      int t = 0;
      while (t < 7 && ((g.S >> t) & 1) == 0) t++;
      s_pad = t ? 10 + t : 0;
    }
    __syncthreads();
    const RsParams &p = s_p;
    if (s_identity) {
      const float2 *xi = reinterpret_cast<const float2 *>(d.in);
      float2 *yo = reinterpret_cast<float2 *>(d.out);
      const int64_t e0 = q0 * kIdentityChunk;
      const int64_t e1 = min(d.out_len, e0 + kIdentityChunk);
      for (int64_t e = e0 + tid; e < e1; e += kRgThreads) yo[e] = xi[e];
      __syncthreads();
      continue;
    }
    if (sig != last_sig) {
      build_tap_table<float, true, false>(p, reinterpret_cast<const float *>(p.h), table, tid, kRgThreads);
      last_sig = sig;
    }
    const int64_t xs0 = q0 * p.S + p.kmin;
    const XT *row = reinterpret_cast<const XT *>(p.x);
    const int wr = wid / p.WC, wc = wid - wr * p.WC;
    float2 *orow = reinterpret_cast<float2 *>(p.out);
    auto stage_and_compute = [&](auto padc) {
      constexpr int PAD = decltype(padc)::value;
      for (int e = tid; e < p.win; e += kRgThreads) {
        const int64_t gi = xs0 + e;
        const bool ok = gi >= 0 && gi < p.N;
        cp_async_zfill<8>(&xbuf[smem_idx<PAD>(e)], ok ? (const void *)(row + gi) : (const void *)row, ok);
      }
      cp_async_commit();
      cp_async_wait<0>();
      __syncthreads();
      rowtile_compute<float, true, false, 1, PAD>(p, xbuf, table, orow, q0, wr, wc, lane, (float)p.scale, 0);
    };
    switch (s_pad) {
      case 0: stage_and_compute(std::integral_constant<int, 0>{}); break;
      case 11: stage_and_compute(std::integral_constant<int, 11>{}); break;
      case 12: stage_and_compute(std::integral_constant<int, 12>{}); break;
      case 13: stage_and_compute(std::integral_constant<int, 13>{}); break;
      case 14: stage_and_compute(std::integral_constant<int, 14>{}); break;
      case 15: stage_and_compute(std::integral_constant<int, 15>{}); break;
      case 16: stage_and_compute(std::integral_constant<int, 16>{}); break;
      default: stage_and_compute(std::integral_constant<int, 17>{}); break;
    }
    __syncthreads();
  }
}

static int64_t table_bytes_of(const RgGeom &g) {
  return g.identity ? 0 : (int64_t)tap_table_bytes<float, true, false>(g.ncg, g.span);
}

}  // namespace gbfir

using namespace gbfir;

extern "C" {

size_t gbfir_ragged_workspace_size(int64_t count, int64_t num_tiles) {
  (void)count;
  (void)num_tiles;
  return 256;
}

int64_t gbfir_ragged_plan(const gbfir_ragged_desc *descs, int64_t count, int64_t *tile_table,
                          gbfir_ragged_plan_info *info) {
  if (descs == nullptr || count <= 0) {
    set_error("ragged_plan: no descriptors");
    return -GBFIR_ERR_INVALID_PARAMETER;
  }
  int64_t ntiles = 0, max_table = 0, max_win = 0;
  std::vector<std::pair<double, std::pair<int64_t, int64_t>>> tiles;
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
    const RgGeom g = rg_geometry(d.up, d.down, d.h_len, d.out_len);
    if (!g.identity) {
      max_table = std::max(max_table, table_bytes_of(g));
      max_win = std::max(max_win, rg_window_alloc(g));
    }
    const int64_t nt = (g.rows + g.QC - 1) / g.QC;
    const double per = g.identity ? (double)kIdentityChunk : (double)g.QC * g.Nt * ((double)d.h_len / g.up + 1);
    for (int64_t k = 0; k < nt; k++) {
      if (tile_table) tiles.push_back({per, {s, k * g.QC}});
    }
    ntiles += nt;
  }
  const int64_t tb = (max_table + 15) & ~15LL;
  const int64_t smem = tb + max_win * 8;
  if (smem > 200 * 1024) {
    set_error("ragged_plan: a signal's tile needs more than 200 KB of shared memory");
    return -GBFIR_ERR_NOT_SUPPORTED;
  }
  if (tile_table) {
    std::stable_sort(tiles.begin(), tiles.end(),
                     [](const auto &a, const auto &b) { return a.first > b.first; });
    for (size_t i = 0; i < tiles.size(); i++) {
      tile_table[2 * i] = tiles[i].second.first;
      tile_table[2 * i + 1] = tiles[i].second.second;
    }
  }
  if (info) {
    info->num_tiles = ntiles;
    info->shared_bytes = smem < 16 ? 16 : smem;
    info->table_bytes = tb;
  }
  return ntiles;
}

int gbfir_ragged_resample(const gbfir_ragged_desc *device_descs, int64_t count, const int64_t *device_tile_table,
                          const gbfir_ragged_plan_info *info, int32_t precision, void *workspace,
                          size_t workspace_bytes, gbfir_stream_t stream) {
  if (!device_descs || !device_tile_table || !info || count <= 0 || info->num_tiles <= 0)
    GBFIR_FAIL(GBFIR_ERR_INVALID_PARAMETER, "ragged_resample: empty plan");
  const int64_t num_tiles = info->num_tiles;
  if (precision != GBFIR_PREC_FP32)
    GBFIR_FAIL(GBFIR_ERR_NOT_SUPPORTED, "ragged_resample: only the FP32 form is available");
  if (!workspace || workspace_bytes < gbfir_ragged_workspace_size(count, num_tiles))
    GBFIR_FAIL(GBFIR_ERR_WORKSPACE, "ragged_resample: workspace missing or too small");
  if (reinterpret_cast<uintptr_t>(workspace) % 8) GBFIR_FAIL(GBFIR_ERR_ALIGNMENT, "ragged_resample: workspace");
  const int64_t table_bytes = info->table_bytes;
  const int64_t smem = info->shared_bytes;
  if (smem <= 0 || smem > 200 * 1024 || table_bytes < 0 || table_bytes > smem || (table_bytes & 15))
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
  if (grid > num_tiles) grid = num_tiles;
  RgParams rp{};
  rp.descs = device_descs;
  rp.tiles = device_tile_table;
  rp.ntiles = num_tiles;
  rp.counter = reinterpret_cast<unsigned long long *>(workspace);
  rp.table_bytes = (int32_t)table_bytes;
  ragged_rowtile<<<(unsigned)grid, kRgThreads, (size_t)smem, s>>>(rp);
  return check_launch("ragged_resample");
}

}  // extern "C"
