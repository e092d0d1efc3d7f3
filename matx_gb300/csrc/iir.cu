// iir.cu — MatX filter(): the recursive (IIR) filter and its FIR-only form, for sm_103a.
//
// Semantics are MatX's filter(in, h_rec, h_nonrec) (include/matx/operators/filter.h:177-181,
// include/matx/transforms/filter.h:159-188):
//   * h_rec empty: conv1d(in, h_nonrec, SAME) (transforms/filter.h:185);
//   * else, per row, y[n] = sum_{j<nb} b[j] x[n-j] + sum_{k<na} a[k] y[n-1-k] with zero
//     initial state (the recurrence of include/matx/kernels/filter.cuh:44-, checked by
//     MatX's own test against this loop, test/00_operators/filter_test.cu:19-47), at most
//     4 coefficients of each kind (kernels/filter.cuh:29-30).
//
// Schedule (no MatX counterpart; MatX solves the recurrence with per-position correction
// factors and a chained block carry): a CTA owns 8192 samples of one row, 32 per thread.
// With the state s = (y[n], ..., y[n-c+1]) the recurrence is s[n] = A s[n-1] + w[n] e0, A
// the companion matrix, so a thread's chunk maps its entry state e to M e + g (M = A^32,
// g its zero-entry final state); the CTA's 256 chunks combine by a Kogge-Stone scan with the
// powers M^(2^k), which the host forms in FP64, and the CTAs of a row by chained carries in
// one pass (iir_onepass below): x is read once and y written once.  The window comes in and
// goes out as coalesced 16-byte accesses through a padded shared buffer, each thread holds
// its 32 samples in registers, and the kernels run 2 or 4 coefficients of each kind
// (zero-padded), fixed at compile time, so no per-sample test is issued.
#include <cstring>

#include "common.cuh"

namespace gbfir {

constexpr int kIirThreads = 256;
constexpr int kIirChunk = 32;                        // samples per thread
constexpr int kIirBlock = kIirThreads * kIirChunk;   // samples per CTA
constexpr int kIirMaxCoef = 4;
constexpr int kIirPowers = 14;  // M^(2^k), k < 14: chunk scans (k < 8), CTAs (8), look-back windows (8..13)

struct IirParams {
  const void *x;
  int64_t x_bstride, N;
  void *y;
  int64_t y_bstride;
  int64_t batch, nblk;
  int32_t na, nb, xc;      // xc: the input is complex
  double a[kIirMaxCoef][2], b[kIirMaxCoef][2];
  double mpow[kIirPowers][kIirMaxCoef][kIirMaxCoef][2];  // (A^32)^(2^k): k = 8 one CTA, 13 32 CTAs
  float fa[kIirMaxCoef][2], fb[kIirMaxCoef][2];  // the same in float (no per-use conversion)
  float fmpow[kIirPowers][kIirMaxCoef][kIirMaxCoef][2];
  void *ws;                                      // [batch][nblk][4] states (output type)
};

// Coefficients in the arithmetic type (read straight from the parameter space).
template <typename T>
struct IirC;
template <>
struct IirC<float> {
  static __device__ __forceinline__ const float *a(const IirParams &p, int k) { return p.fa[k]; }
  static __device__ __forceinline__ const float *b(const IirParams &p, int k) { return p.fb[k]; }
  static __device__ __forceinline__ const float *m(const IirParams &p, int lv, int i, int j) {
    return p.fmpow[lv][i][j];
  }
};
template <>
struct IirC<double> {
  static __device__ __forceinline__ const double *a(const IirParams &p, int k) { return p.a[k]; }
  static __device__ __forceinline__ const double *b(const IirParams &p, int k) { return p.b[k]; }
  static __device__ __forceinline__ const double *m(const IirParams &p, int lv, int i, int j) {
    return p.mpow[lv][i][j];
  }
};

// Arithmetic on the output value type: real T or (re, im) pairs.
template <typename T, bool OC>
struct IV {
  T re, im;
  __device__ __forceinline__ static IV zero() { return IV{T(0), T(0)}; }
};
template <typename T>
struct IV<T, false> {
  T re;
  __device__ __forceinline__ static IV zero() { return IV{T(0)}; }
};

template <typename T, bool OC, bool CC>
__device__ __forceinline__ IV<T, OC> cmad(IV<T, OC> acc, const T *c, IV<T, OC> v) {
  // acc + c * v, c a coefficient (real unless CC)
  const T cr = c[0];
  if constexpr (OC) {
    if constexpr (CC) {
      const T ci = c[1];
      acc.re = fma(cr, v.re, acc.re);
      acc.re = fma(-ci, v.im, acc.re);
      acc.im = fma(cr, v.im, acc.im);
      acc.im = fma(ci, v.re, acc.im);
    } else {
      acc.re = fma(cr, v.re, acc.re);
      acc.im = fma(cr, v.im, acc.im);
    }
  } else {
    acc.re = fma(cr, v.re, acc.re);
  }
  return acc;
}

template <typename T, bool OC>
__device__ __forceinline__ IV<T, OC> vadd(IV<T, OC> a, IV<T, OC> b) {
  a.re += b.re;
  if constexpr (OC) a.im += b.im;
  return a;
}

template <typename T, bool OC>
__device__ __forceinline__ IV<T, OC> iir_load(const IirParams &p, const void *row, int64_t n) {
  IV<T, OC> v = IV<T, OC>::zero();
  if (n < 0 || n >= p.N) return v;
  if constexpr (OC) {
    if (p.xc) {
      const T *q = reinterpret_cast<const T *>(row) + 2 * n;
      v.re = q[0];
      v.im = q[1];
    } else {
      v.re = reinterpret_cast<const T *>(row)[n];
    }
  } else {
    v.re = reinterpret_cast<const T *>(row)[n];
  }
  return v;
}

// v <- M v for the (CAP x CAP) matrix M (complex entries when CC)
template <typename T, bool OC, bool CC, int CAP>
__device__ __forceinline__ void matvec(const IirParams &p, int lv, IV<T, OC> (&v)[kIirMaxCoef]) {
  IV<T, OC> r[CAP];
#pragma unroll
  for (int i = 0; i < CAP; i++) {
    r[i] = IV<T, OC>::zero();
#pragma unroll
    for (int j = 0; j < CAP; j++) r[i] = cmad<T, OC, CC>(r[i], IirC<T>::m(p, lv, i, j), v[j]);
  }
#pragma unroll
  for (int i = 0; i < CAP; i++) v[i] = r[i];
}

// Shared staging of one CTA's 8192 samples: chunk t (32 elements of ES bytes) sits at
// t*(32*ES + 16), so a lane's 16-byte reads of its own chunk are conflict-free across the
// warp and the fill / drain are coalesced 16-byte global accesses (interior CTAs of rows
// whose starts are 16-byte aligned; the rest element by element, zero past the row).
template <int ES>
__device__ __forceinline__ int stg_off(int e) {
  return (e >> 5) * (32 * ES + 16) + (e & 31) * ES;
}

template <typename T, bool XC>
__device__ __forceinline__ void stage_in(const IirParams &p, const unsigned char *row, int64_t n0, bool vec,
                                         unsigned char *sm) {
  using E = typename val_of<T, XC>::type;
  constexpr int ES = (int)sizeof(E), PPC = 32 * ES / 16;
  if (vec && n0 + kIirBlock <= p.N) {
    const float4 *src = reinterpret_cast<const float4 *>(row + n0 * ES);
#pragma unroll 4
    for (int q = threadIdx.x; q < kIirBlock * ES / 16; q += kIirThreads)
      *reinterpret_cast<float4 *>(sm + (q / PPC) * (32 * ES + 16) + (q % PPC) * 16) = __ldg(src + q);
  } else {
    const E *src = reinterpret_cast<const E *>(row);
    for (int e = threadIdx.x; e < kIirBlock; e += kIirThreads) {
      const int64_t n = n0 + e;
      *reinterpret_cast<E *>(sm + stg_off<ES>(e)) = n < p.N ? src[n] : zero_val<E>();
    }
  }
}

// This thread's 32 staged samples as arithmetic values (real input promoted when OC).
template <typename T, bool XC, bool OC>
__device__ __forceinline__ void read_chunk(const unsigned char *sm, IV<T, OC> (&xr)[kIirChunk]) {
  using E = typename val_of<T, XC>::type;
  constexpr int ES = (int)sizeof(E), PER = 16 / ES;
  const unsigned char *base = sm + threadIdx.x * (32 * ES + 16);
#pragma unroll
  for (int v = 0; v < kIirChunk / PER; v++) {
    const float4 w = *reinterpret_cast<const float4 *>(base + 16 * v);
    const T *e = reinterpret_cast<const T *>(&w);
#pragma unroll
    for (int u = 0; u < PER; u++) {
      xr[v * PER + u] = IV<T, OC>::zero();
      if constexpr (XC) {
        xr[v * PER + u].re = e[2 * u];
        xr[v * PER + u].im = e[2 * u + 1];
      } else {
        xr[v * PER + u].re = e[u];
      }
    }
  }
}

// The chunk's recurrence from entry state s (s[k] = y[c-1-k]); halo[i] = x[c-1-i].  CAP
// coefficients of each kind, zero-padded (no per-sample tests).  WRITE replaces xr[j] by y[c+j].
template <typename T, bool OC, bool CC, int CAP, bool WRITE>
__device__ __forceinline__ void run_chunk(const IirParams &p, IV<T, OC> (&xr)[kIirChunk],
                                          const IV<T, OC> (&halo)[kIirMaxCoef - 1], IV<T, OC> (&s)[kIirMaxCoef]) {
  using V = IV<T, OC>;
  V xw[CAP];  // xw[i] = x[n - i]
#pragma unroll
  for (int i = 1; i < CAP; i++) xw[i] = halo[i - 1];
#pragma unroll
  for (int j = 0; j < kIirChunk; j++) {
    xw[0] = xr[j];
    // the feed-forward part first: only the feedback terms sit on the recurrence chain
    V y = V::zero();
#pragma unroll
    for (int i = 0; i < CAP; i++) y = cmad<T, OC, CC>(y, IirC<T>::b(p, i), xw[i]);
#pragma unroll
    for (int k = CAP - 1; k >= 0; k--) y = cmad<T, OC, CC>(y, IirC<T>::a(p, k), s[k]);
#pragma unroll
    for (int k = CAP - 1; k > 0; k--) s[k] = s[k - 1];
    s[0] = y;
#pragma unroll
    for (int i = CAP - 1; i > 0; i--) xw[i] = xw[i - 1];
    if constexpr (WRITE) xr[j] = y;
  }
}

// One bounded device status word for the filter's chained carries: 1 if a wait for a
// predecessor's state gave up since the last read.
static __device__ int32_t g_iir_status;

int iir_status_take() {
  int32_t v = 0, zero = 0;
  if (cudaMemcpyFromSymbol(&v, g_iir_status, sizeof(v)) != cudaSuccess) return -1;
  cudaMemcpyToSymbol(g_iir_status, &zero, sizeof(zero));
  return v;
}

// Single pass over a row with chained carries (decoupled look-back).  CTAs take (row, block)
// tickets in block-major order from a counter, so every block a CTA waits for took its ticket
// earlier and never waits on a later one.  Each CTA stages its window, runs its chunks from a
// zero entry and scans them (the zero-entry inclusive state of every chunk), publishes its
// block aggregate, then warp 0 looks back over the predecessors 32 at a time: the nearest
// inclusive state ends the walk and every aggregate in front of it, d blocks back, adds
// M^(256 d) times itself.  The CTA publishes its own inclusive state, every chunk gets its
// entry M^(32 t) carry + (its zero-entry exclusive state), and the chunks are rerun from
// there and written.  A wait that runs past
// kIirSpinLimit polls records the failure in g_iir_status and proceeds (results then wrong,
// the launch still ends).
constexpr uint32_t kIirSpinLimit = 1u << 22;

template <typename T, bool XC, bool OC, bool CC, int CAP>
__global__ void __launch_bounds__(kIirThreads)
    iir_onepass(const IirParams p, int vec, unsigned long long *ticket, int *flags, IV<T, OC> *agg,
                IV<T, OC> *incl) {
  using V = IV<T, OC>;
  using XE = typename val_of<T, XC>::type;
  using OE = typename val_of<T, OC>::type;
  constexpr int XES = (int)sizeof(XE), OES = (int)sizeof(OE);
  __shared__ V sh[kIirThreads * CAP];
  __shared__ V s_agg[CAP], s_carry[CAP];
  __shared__ unsigned long long s_ticket;
  extern __shared__ __align__(16) unsigned char stg[];
  const int tid = threadIdx.x;
  if (tid == 0) s_ticket = atomicAdd(ticket, 1ULL);
  __syncthreads();
  // tickets run block-major (block j of every row, then block j + 1): a block's predecessor
  // took its ticket a whole column of rows earlier and has usually published its inclusive
  // state by the time the block looks back
  const int64_t blk = (int64_t)(s_ticket / (unsigned long long)p.batch);
  const int64_t row = (int64_t)(s_ticket - (unsigned long long)blk * (unsigned long long)p.batch);
  const int64_t idx = row * p.nblk + blk;
  const int64_t c = blk * kIirBlock + (int64_t)tid * kIirChunk;
  const unsigned char *xrow = reinterpret_cast<const unsigned char *>(p.x) + row * p.x_bstride * XES;
  stage_in<T, XC>(p, xrow, blk * kIirBlock, vec != 0, stg);
  __syncthreads();
  V xr[kIirChunk], halo[kIirMaxCoef - 1];
  read_chunk<T, XC, OC>(stg, xr);
#pragma unroll
  for (int i = 0; i < CAP - 1; i++) {
    if (tid > 0) {
      const XE e = *reinterpret_cast<const XE *>(stg + stg_off<XES>(tid * kIirChunk - 1 - i));
      halo[i] = V::zero();
      if constexpr (XC) {
        halo[i].re = e.x;
        halo[i].im = e.y;
      } else {
        halo[i].re = e;
      }
    } else {
      halo[i] = iir_load<T, OC>(p, xrow, c - 1 - i);
    }
  }
  V s[kIirMaxCoef];
#pragma unroll
  for (int k = 0; k < kIirMaxCoef; k++) s[k] = V::zero();
  run_chunk<T, OC, CC, CAP, false>(p, xr, halo, s);
  // zero-entry inclusive states of the chunks: G_t = M G_{t-1} + g_t
#pragma unroll 1
  for (int lv = 0; lv < 8; lv++) {
    const int d = 1 << lv;
    __syncthreads();
#pragma unroll
    for (int k = 0; k < CAP; k++) sh[k * kIirThreads + tid] = s[k];
    __syncthreads();
    if (tid >= d) {
      V o[kIirMaxCoef];
#pragma unroll
      for (int k = 0; k < CAP; k++) o[k] = sh[k * kIirThreads + tid - d];
      matvec<T, OC, CC, CAP>(p, lv, o);
#pragma unroll
      for (int k = 0; k < CAP; k++) s[k] = vadd<T, OC>(s[k], o[k]);
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < CAP; k++) sh[k * kIirThreads + tid] = s[k];
  if (tid == kIirThreads - 1) {
    // publish the block aggregate (for the first block of a row it is the inclusive state)
#pragma unroll
    for (int k = 0; k < CAP; k++) {
      s_agg[k] = s[k];
      (blk == 0 ? incl : agg)[idx * kIirMaxCoef + k] = s[k];
    }
    __threadfence();
    atomicExch(&flags[idx], blk == 0 ? 2 : 1);
  }
  __syncthreads();
  V excl[kIirMaxCoef];
#pragma unroll
  for (int k = 0; k < CAP; k++) excl[k] = tid ? sh[k * kIirThreads + tid - 1] : V::zero();
  if (tid < 32) {
    // warp 0 looks back over windows of 32 predecessors: lane l takes block blk-1-l of the
    // current window; the nearest inclusive state ends the walk, the aggregates in front of
    // it add M^(256 l) a_l, and each full window of aggregates multiplies the rest by
    // M^(256*32)
    const int lane = tid;
    V carry[kIirMaxCoef];
#pragma unroll
    for (int k = 0; k < CAP; k++) carry[k] = V::zero();
    bool ok = true;
    if (blk > 0) {
      int win = 0;  // windows walked so far (the walk's power is M^(256*32*win))
      for (int64_t j0 = blk - 1; j0 >= 0; j0 -= 32, win++) {
        const int64_t j = j0 - lane;
        int f = 2;  // lanes past block 0 count as "inclusive zero"
        V v[kIirMaxCoef];
#pragma unroll
        for (int k = 0; k < CAP; k++) v[k] = V::zero();
        if (j >= 0) {
          volatile int *fl = flags + row * p.nblk + j;
          f = 0;
          for (uint32_t it = 0; it < kIirSpinLimit && (f = *fl) == 0; it++) __nanosleep(32);
          if (f == 0) {
            ok = false;
            f = 2;  // give up on this block: treat it as a zero inclusive state
          } else {
            __threadfence();
            const V *src = (f == 2 ? incl : agg) + (row * p.nblk + j) * kIirMaxCoef;
#pragma unroll
            for (int k = 0; k < CAP; k++) {
              if constexpr (OC) {
                const OE e = __ldcg(reinterpret_cast<const OE *>(src + k));
                v[k].re = e.x;
                v[k].im = e.y;
              } else {
                v[k].re = __ldcg(reinterpret_cast<const T *>(src + k));
              }
            }
          }
        }
        const unsigned inc_mask = __ballot_sync(0xffffffffu, f == 2);
        const int stop = inc_mask ? __ffs(inc_mask) - 1 : 32;  // lanes <= stop contribute
        if (lane > stop) {
#pragma unroll
          for (int k = 0; k < CAP; k++) v[k] = V::zero();
        }
        // M^(256 (32 win + lane)) v
#pragma unroll
        for (int b = 0; b < 5; b++)
          if ((lane >> b) & 1) matvec<T, OC, CC, CAP>(p, 8 + b, v);
        for (int w = 0; w < win; w++) matvec<T, OC, CC, CAP>(p, 13, v);
        // sum over the warp
#pragma unroll
        for (int k = 0; k < CAP; k++) {
#pragma unroll
          for (int off = 16; off > 0; off >>= 1) {
            v[k].re += __shfl_xor_sync(0xffffffffu, v[k].re, off);
            if constexpr (OC) v[k].im += __shfl_xor_sync(0xffffffffu, v[k].im, off);
          }
          carry[k] = vadd<T, OC>(carry[k], v[k]);
        }
        if (stop < 32) break;
      }
      const bool all_ok = __all_sync(0xffffffffu, ok);
      if (lane == 0) {
        if (!all_ok) atomicExch(&g_iir_status, 1);
        // this block's inclusive state: M^256 carry + aggregate
        V inc[kIirMaxCoef];
#pragma unroll
        for (int k = 0; k < CAP; k++) inc[k] = carry[k];
        matvec<T, OC, CC, CAP>(p, 8, inc);
#pragma unroll
        for (int k = 0; k < CAP; k++) {
          inc[k] = vadd<T, OC>(inc[k], s_agg[k]);
          incl[idx * kIirMaxCoef + k] = inc[k];
        }
        __threadfence();
        atomicExch(&flags[idx], 2);
      }
    }
    if (lane == 0) {
#pragma unroll
      for (int k = 0; k < CAP; k++) s_carry[k] = carry[k];
    }
  }
  __syncthreads();
  // entry of chunk t: M^(32 t) carry + its zero-entry exclusive state
#pragma unroll
  for (int k = 0; k < CAP; k++) s[k] = s_carry[k];
#pragma unroll
  for (int lv = 0; lv < 8; lv++)
    if ((tid >> lv) & 1) matvec<T, OC, CC, CAP>(p, lv, s);
#pragma unroll
  for (int k = 0; k < CAP; k++) s[k] = vadd<T, OC>(s[k], excl[k]);
  run_chunk<T, OC, CC, CAP, true>(p, xr, halo, s);
  // drain through the staging buffer: the chunks in place, then coalesced rows
  __syncthreads();
  unsigned char *mine = stg + tid * (32 * OES + 16);
#pragma unroll
  for (int j = 0; j < kIirChunk; j++) {
    OE o;
    if constexpr (OC) {
      o.x = xr[j].re;
      o.y = xr[j].im;
    } else {
      o = xr[j].re;
    }
    *reinterpret_cast<OE *>(mine + j * OES) = o;
  }
  __syncthreads();
  unsigned char *yrow = reinterpret_cast<unsigned char *>(p.y) + row * p.y_bstride * OES;
  const int64_t n0 = blk * kIirBlock;
  if (vec && n0 + kIirBlock <= p.N) {
    constexpr int PPC = 32 * OES / 16;
    float4 *dst = reinterpret_cast<float4 *>(yrow + n0 * OES);
#pragma unroll 4
    for (int q = tid; q < kIirBlock * OES / 16; q += kIirThreads)
      dst[q] = *reinterpret_cast<const float4 *>(stg + (q / PPC) * (32 * OES + 16) + (q % PPC) * 16);
  } else {
    OE *dst = reinterpret_cast<OE *>(yrow);
    for (int e = tid; e < kIirBlock; e += kIirThreads)
      if (n0 + e < p.N) dst[n0 + e] = *reinterpret_cast<const OE *>(stg + stg_off<OES>(e));
  }
}

// FIR-only filter(): conv1d SAME with the (at most 4) host coefficients, one output per thread.
template <typename T, bool OC, bool CC, int CAP>
__global__ void fir_same(const IirParams p, int start) {
  using V = IV<T, OC>;
  const int64_t total = p.N * p.batch;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = e / p.N, n = e - row * p.N;
    const void *xrow = reinterpret_cast<const unsigned char *>(p.x) +
                       row * p.x_bstride * (int64_t)sizeof(T) * ((OC && p.xc) ? 2 : 1);
    V y = V::zero();
#pragma unroll
    for (int i = 0; i < CAP; i++) y = cmad<T, OC, CC>(y, IirC<T>::b(p, i), iir_load<T, OC>(p, xrow, n + start - i));
    T *yrow = reinterpret_cast<T *>(p.y) + row * p.y_bstride * (OC ? 2 : 1);
    if constexpr (OC) {
      yrow[2 * n] = y.re;
      yrow[2 * n + 1] = y.im;
    } else {
      yrow[n] = y.re;
    }
  }
}

// ---- host ---------------------------------------------------------------------------

namespace {
struct CMat {
  double v[kIirMaxCoef][kIirMaxCoef][2];
};
CMat cmat_mul(const CMat &a, const CMat &b) {
  CMat r{};
  for (int i = 0; i < kIirMaxCoef; i++)
    for (int j = 0; j < kIirMaxCoef; j++)
      for (int k = 0; k < kIirMaxCoef; k++) {
        r.v[i][j][0] += a.v[i][k][0] * b.v[k][j][0] - a.v[i][k][1] * b.v[k][j][1];
        r.v[i][j][1] += a.v[i][k][0] * b.v[k][j][1] + a.v[i][k][1] * b.v[k][j][0];
      }
  return r;
}
}  // namespace

// Workspace of the recursive form: the ticket counter (16 bytes), one flag per (row, block),
// then the blocks' aggregate and inclusive states (4 values each).
static size_t iir_flag_bytes(int64_t batch, int64_t nblk) { return ((size_t)batch * nblk * 4 + 15) & ~(size_t)15; }

size_t filter_workspace_bytes(int64_t batch, int64_t len, int32_t out_dtype) {
  const int64_t nblk = (len + kIirBlock - 1) / kIirBlock;
  return 16 + iir_flag_bytes(batch, nblk) + 2 * (size_t)batch * (size_t)nblk * kIirMaxCoef * dtype_size(out_dtype);
}

template <typename T, bool XC, bool OC, bool CC, int CAP>
static int launch_filter(IirParams &p, cudaStream_t s) {
  if (p.na == 0) {
    // conv1d SAME start for Lmin = nb (the signal is at least as long as the filter)
    const int start = (p.nb & 1) ? (p.nb - 1) / 2 : p.nb / 2 - 1;
    const int64_t total = p.N * p.batch;
    int64_t grid = (total + 255) / 256;
    const int64_t cap = (int64_t)num_sms() * 16;
    if (grid > cap) grid = cap;
    fir_same<T, OC, CC, CAP><<<(unsigned)(grid < 1 ? 1 : grid), 256, 0, s>>>(p, start);
    return check_launch("filter (FIR)");
  }
  using V = IV<T, OC>;
  const size_t xes = sizeof(T) * (XC ? 2 : 1), oes = sizeof(T) * (OC ? 2 : 1);
  const size_t bsmem = (size_t)kIirThreads * (32 * oes + 16);
  int rc = ensure_smem((const void *)iir_onepass<T, XC, OC, CC, CAP>, bsmem, "filter");
  if (rc) return rc;
  // coalesced 16-byte fills and drains when every row start is 16-byte aligned
  const int vec = (reinterpret_cast<uintptr_t>(p.x) % 16 == 0 && reinterpret_cast<uintptr_t>(p.y) % 16 == 0 &&
                   (p.x_bstride * xes) % 16 == 0 && (p.y_bstride * oes) % 16 == 0)
                      ? 1
                      : 0;
  unsigned char *ws = reinterpret_cast<unsigned char *>(p.ws);
  const size_t fbytes = iir_flag_bytes(p.batch, p.nblk);
  auto *ticket = reinterpret_cast<unsigned long long *>(ws);
  int *flags = reinterpret_cast<int *>(ws + 16);
  V *agg = reinterpret_cast<V *>(ws + 16 + fbytes);
  V *incl = agg + (size_t)p.batch * p.nblk * kIirMaxCoef;
  if (cudaMemsetAsync(ws, 0, 16 + fbytes, s) != cudaSuccess) GBFIR_FAIL(GBFIR_ERR_CUDA, "filter: workspace reset failed");
  const int64_t grid = p.batch * p.nblk;
  if (grid > 0x7fffffffLL) GBFIR_FAIL(GBFIR_ERR_INVALID_SIZE, "filter: too many blocks");
  iir_onepass<T, XC, OC, CC, CAP><<<(unsigned)grid, kIirThreads, bsmem, s>>>(p, vec, ticket, flags, agg, incl);
  return check_launch("filter (IIR)");
}

// Shapes validated by the caller.  a / b are host arrays of `na` / `nb` coefficients of
// coef_dtype; workspace holds filter_workspace_bytes(out) when na > 0.
int filter_fp(const gbfir_buf &out, const gbfir_buf &in, const void *a, int na, const void *b, int nb,
              int32_t coef_dtype, void *workspace, cudaStream_t s) {
  IirParams p{};
  p.x = in.ptr;
  p.x_bstride = in.batch > 1 ? in.batch_stride : 0;
  p.N = in.len;
  p.y = out.ptr;
  p.y_bstride = out.batch_stride;
  p.batch = out.batch;
  p.nblk = (in.len + kIirBlock - 1) / kIirBlock;
  p.na = na;
  p.nb = nb;
  p.xc = dtype_complex(in.dtype);
  p.ws = workspace;
  const bool cc = dtype_complex(coef_dtype), dbl = dtype_double(coef_dtype);
  auto coef = [&](const void *src, int i, double (&dst)[2]) {
    if (dbl) {
      const double *q = reinterpret_cast<const double *>(src);
      dst[0] = cc ? q[2 * i] : q[i];
      dst[1] = cc ? q[2 * i + 1] : 0.0;
    } else {
      const float *q = reinterpret_cast<const float *>(src);
      dst[0] = cc ? q[2 * i] : q[i];
      dst[1] = cc ? q[2 * i + 1] : 0.0;
    }
  };
  for (int i = 0; i < na; i++) coef(a, i, p.a[i]);
  for (int i = 0; i < nb; i++) coef(b, i, p.b[i]);
  // kernels run CAP = 2 or 4 coefficients of each kind, zero-padded
  const int cap = (na <= 2 && nb <= 2) ? 2 : 4;
  if (na > 0) {
    // companion matrix of y[n] = w[n] + sum_k a[k] y[n-1-k] on s = (y[n], ..., y[n-cap+1])
    CMat A{};
    for (int k = 0; k < na; k++) {
      A.v[0][k][0] = p.a[k][0];
      A.v[0][k][1] = p.a[k][1];
    }
    for (int i = 1; i < cap; i++) A.v[i][i - 1][0] = 1.0;
    CMat M = A;
    for (int i = 0; i < 5; i++) M = cmat_mul(M, M);  // A^32
    for (int lv = 0; lv < kIirPowers; lv++) {
      memcpy(p.mpow[lv], M.v, sizeof(M.v));
      M = cmat_mul(M, M);
    }
  }
  for (int i = 0; i < kIirMaxCoef; i++)
    for (int c = 0; c < 2; c++) {
      p.fa[i][c] = (float)p.a[i][c];
      p.fb[i][c] = (float)p.b[i][c];
      for (int lv = 0; lv < kIirPowers; lv++)
        for (int j = 0; j < kIirMaxCoef; j++) p.fmpow[lv][i][j][c] = (float)p.mpow[lv][i][j][c];
    }
  const bool xc = dtype_complex(in.dtype);
  auto go = [&](auto capv) -> int {
    constexpr int C = decltype(capv)::value;
    if (dtype_double(in.dtype)) {
      if (xc && cc) return launch_filter<double, true, true, true, C>(p, s);
      if (xc) return launch_filter<double, true, true, false, C>(p, s);
      if (cc) return launch_filter<double, false, true, true, C>(p, s);
      return launch_filter<double, false, false, false, C>(p, s);
    }
    if (xc && cc) return launch_filter<float, true, true, true, C>(p, s);
    if (xc) return launch_filter<float, true, true, false, C>(p, s);
    if (cc) return launch_filter<float, false, true, true, C>(p, s);
    return launch_filter<float, false, false, false, C>(p, s);
  };
  return cap == 2 ? go(std::integral_constant<int, 2>{}) : go(std::integral_constant<int, 4>{});
}

}  // namespace gbfir
