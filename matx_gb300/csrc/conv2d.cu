// conv2d.cu — direct 2-D convolution (MatX conv2d), for sm_103a.
//
// Semantics are MatX's conv2d (include/matx/transforms/conv.h:548-600 dispatch,
// :325-395 host loop, include/matx/kernels/conv.cuh:210-402 CUDA kernel):
//   out[oy][ox] = sum_{fy, fx} x[oy + fy - dy][ox + fx - dx] * h[N2-1-fy][M2-1-fx],
// x outside the image zero, dy/dx = N2-1 / M2-1 (FULL), N2/2, M2/2 (SAME), 0 (VALID), output
// sizes per axis max+min-1 / max / max-min+1 (operators/conv.h:335-357); the operand with
// more elements is the image (conv.h:569-576, applied by the caller); complex products with
// MatX's madd.  Images are batched; the filter is one per image or shared.
//
// Schedule (no MatX counterpart in this form): a CTA owns a 64 x 32 output tile of one image
// (32 x 8 threads, 8 outputs per thread down a column) and stages the tile's input window
// (64 + N2 - 1 rows x 32 + M2 - 1 columns, zero-filled) and the filter in shared memory
// once.  For each filter column a thread keeps its 8 + N2 - 1 input samples in a sliding
// register window, so one shared load feeds up to 8 multiply-adds; warp lanes take
// consecutive columns, so the loads and the output stores are coalesced rows.
#include "common.cuh"

namespace gbfir {

constexpr int kC2X = 32, kC2Y = 8, kC2U = 8;  // tile: kC2X columns x kC2Y*kC2U rows
constexpr int kC2MaxF = 64;

struct Conv2dParams {
  const void *x;
  int64_t x_bstride, x_rstride, N1, M1;
  const void *h;
  int64_t h_bstride, h_rstride, N2, M2;
  void *out;
  int64_t o_bstride, o_rstride, ON, OM;
  int64_t dy, dx, batch;
};

template <typename T, bool XC, bool HC>
__global__ void __launch_bounds__(kC2X *kC2Y) conv2d_direct(const Conv2dParams p) {
  using XT = typename val_of<T, XC>::type;
  using HT = typename val_of<T, HC>::type;
  constexpr bool OC = XC || HC;
  using OT = typename val_of<T, OC>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int wy = kC2Y * kC2U + (int)p.N2 - 1, wx = kC2X + (int)p.M2 - 1;
  XT *win = reinterpret_cast<XT *>(smem_raw);
  HT *filt = reinterpret_cast<HT *>(smem_raw + (((size_t)wy * wx * sizeof(XT) + 15) & ~(size_t)15));
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * kC2X + tx;
  const int64_t ox0 = (int64_t)blockIdx.x * kC2X, oy0 = (int64_t)blockIdx.y * (kC2Y * kC2U);
  for (int64_t b = blockIdx.z; b < p.batch; b += gridDim.z) {
    const XT *xb = reinterpret_cast<const XT *>(p.x) + b * p.x_bstride;
    const HT *hb = reinterpret_cast<const HT *>(p.h) + b * p.h_bstride;
    __syncthreads();
    // the filter, flipped: filt[fy][fx] = h[N2-1-fy][M2-1-fx]
    for (int e = tid; e < p.N2 * p.M2; e += kC2X * kC2Y) {
      const int fy = e / (int)p.M2, fx = e - fy * (int)p.M2;
      filt[e] = hb[(p.N2 - 1 - fy) * p.h_rstride + (p.M2 - 1 - fx)];
    }
    // input rows oy0 - dy .. and columns ox0 - dx .., zero outside the image
    for (int e = tid; e < wy * wx; e += kC2X * kC2Y) {
      const int r = e / wx, c = e - r * wx;
      const int64_t iy = oy0 - p.dy + r, ix = ox0 - p.dx + c;
      win[e] = (iy >= 0 && iy < p.N1 && ix >= 0 && ix < p.M1) ? xb[iy * p.x_rstride + ix] : zero_val<XT>();
    }
    __syncthreads();
    Acc<T, OC> acc[kC2U];
#pragma unroll
    for (int u = 0; u < kC2U; u++) acc[u].zero();
    const int r0 = ty * kC2U;
    for (int fx = 0; fx < p.M2; fx++) {
      const XT *col = win + r0 * wx + tx + fx;
      XT w[kC2U];
#pragma unroll
      for (int u = 0; u < kC2U - 1; u++) w[u + 1] = col[u * wx];
      for (int fy = 0; fy < p.N2; fy++) {
        // w[u] = x of output row r0 + u at filter row fy
#pragma unroll
        for (int u = 0; u < kC2U - 1; u++) w[u] = w[u + 1];
        w[kC2U - 1] = col[(fy + kC2U - 1) * wx];
        const HT t = filt[fy * (int)p.M2 + fx];
#pragma unroll
        for (int u = 0; u < kC2U; u++) mac<T, XC, HC>(acc[u], w[u], t);
      }
    }
    OT *ob = reinterpret_cast<OT *>(p.out) + b * p.o_bstride;
    const int64_t ox = ox0 + tx;
#pragma unroll
    for (int u = 0; u < kC2U; u++) {
      const int64_t oy = oy0 + r0 + u;
      if (oy < p.ON && ox < p.OM) ob[oy * p.o_rstride + ox] = pack<T, OC>(acc[u], T(1));
    }
  }
}

template <typename T, bool XC, bool HC>
static int launch_conv2d(const Conv2dParams &p, cudaStream_t s) {
  using XT = typename val_of<T, XC>::type;
  using HT = typename val_of<T, HC>::type;
  const int wy = kC2Y * kC2U + (int)p.N2 - 1, wx = kC2X + (int)p.M2 - 1;
  const size_t smem = (((size_t)wy * wx * sizeof(XT) + 15) & ~(size_t)15) + (size_t)p.N2 * p.M2 * sizeof(HT);
  if (smem > 227 * 1024) GBFIR_FAIL(GBFIR_ERR_NOT_SUPPORTED, "conv2d: filter and tile exceed shared memory");
  auto fn = conv2d_direct<T, XC, HC>;
  int rc = ensure_smem((const void *)fn, smem, "conv2d");
  if (rc) return rc;
  const int64_t gx = (p.OM + kC2X - 1) / kC2X, gy = (p.ON + kC2Y * kC2U - 1) / (kC2Y * kC2U);
  if (gx > 0x7fffffffLL || gy > 65535) GBFIR_FAIL(GBFIR_ERR_INVALID_SIZE, "conv2d: image too large");
  const dim3 grid((unsigned)gx, (unsigned)gy, (unsigned)(p.batch < 65535 ? p.batch : 65535));
  fn<<<grid, dim3(kC2X, kC2Y), smem, s>>>(p);
  return check_launch("conv2d");
}

// Operands validated by the caller; x is the larger image (the swap is applied).
int conv2d_fp(const gbfir_buf2d &out, const gbfir_buf2d &x, const gbfir_buf2d &h, int mode, cudaStream_t s) {
  if (h.rows > kC2MaxF || h.cols > kC2MaxF)
    GBFIR_FAIL(GBFIR_ERR_NOT_SUPPORTED, "conv2d: filters of at most %d x %d", kC2MaxF, kC2MaxF);
  Conv2dParams p{};
  p.x = x.ptr;
  p.x_bstride = x.batch > 1 ? x.batch_stride : 0;
  p.x_rstride = x.row_stride;
  p.N1 = x.rows;
  p.M1 = x.cols;
  p.h = h.ptr;
  p.h_bstride = h.batch > 1 ? h.batch_stride : 0;
  p.h_rstride = h.row_stride;
  p.N2 = h.rows;
  p.M2 = h.cols;
  p.out = out.ptr;
  p.o_bstride = out.batch_stride;
  p.o_rstride = out.row_stride;
  p.ON = out.rows;
  p.OM = out.cols;
  p.dy = mode == GBFIR_MODE_SAME ? h.rows / 2 : mode == GBFIR_MODE_FULL ? h.rows - 1 : 0;
  p.dx = mode == GBFIR_MODE_SAME ? h.cols / 2 : mode == GBFIR_MODE_FULL ? h.cols - 1 : 0;
  p.batch = out.batch;
  const bool xc = dtype_complex(x.dtype), hc = dtype_complex(h.dtype);
  if (dtype_double(x.dtype)) {
    if (xc && hc) return launch_conv2d<double, true, true>(p, s);
    if (xc) return launch_conv2d<double, true, false>(p, s);
    if (hc) return launch_conv2d<double, false, true>(p, s);
    return launch_conv2d<double, false, false>(p, s);
  }
  if (xc && hc) return launch_conv2d<float, true, true>(p, s);
  if (xc) return launch_conv2d<float, true, false>(p, s);
  if (hc) return launch_conv2d<float, false, true>(p, s);
  return launch_conv2d<float, false, false>(p, s);
}

}  // namespace gbfir
