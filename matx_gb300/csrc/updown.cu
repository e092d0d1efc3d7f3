// updown.cu — upsample / downsample and their composition with conv1d, for sm_103a.
//
// Semantics are MatX's upsample and downsample operators
// (include/matx/operators/updownsample.h:254-279): upsample(x, n)[i] = x[i/n] when n divides
// i, else 0, of length N*n; downsample(x, n)[i] = x[i*n], of length ceil(N/n) (a slice with
// stride n).  Their composition around conv1d (include/matx/transforms/conv.h:402-532),
//   downsample(conv1d(upsample(x, up), h, mode), down)[m] = sum_k x[k] h[start + m*down - k*up],
// with start the conv1d mode offset for the upsampled length N*up, is the polyphase form the
// row tile of rowtile.cuh computes (taps without the even-length lead zero, no x-up scale),
// so the zero-stuffed signal and the discarded outputs are never formed.
#include "rowtile.cuh"

namespace gbfir {

int conv1d_fp(const gbfir_buf &out, const gbfir_buf &in, const gbfir_buf &h, int mode, int is_corr, cudaStream_t s);

template <typename V>
__global__ void upsample_rows(const V *x, int64_t x_bstride, int64_t N, V *out, int64_t o_bstride, int64_t n,
                              int64_t batch) {
  const int64_t olen = N * n, total = olen * batch;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / olen, i = e - b * olen;
    const int64_t q = i / n;
    out[b * o_bstride + i] = (i - q * n == 0) ? x[b * x_bstride + q] : zero_val<V>();
  }
}

template <typename V>
__global__ void downsample_rows(const V *x, int64_t x_bstride, V *out, int64_t o_bstride, int64_t olen, int64_t n,
                                int64_t batch) {
  const int64_t total = olen * batch;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / olen, i = e - b * olen;
    out[b * o_bstride + i] = x[b * x_bstride + i * n];
  }
}

static dim3 elementwise_grid(int64_t total) {
  int64_t grid = (total + 255) / 256;
  const int64_t cap = (int64_t)num_sms() * 16;
  if (grid > cap) grid = cap;
  if (grid < 1) grid = 1;
  return dim3((unsigned)grid);
}

template <typename V>
static int launch_updown(const gbfir_buf &out, const gbfir_buf &in, int64_t n, bool up, cudaStream_t s) {
  const V *x = reinterpret_cast<const V *>(in.ptr);
  V *o = reinterpret_cast<V *>(out.ptr);
  const int64_t xb = in.batch > 1 ? in.batch_stride : 0;
  if (up) {
    upsample_rows<V><<<elementwise_grid(out.len * out.batch), 256, 0, s>>>(x, xb, in.len, o, out.batch_stride, n,
                                                                           out.batch);
    return check_launch("upsample");
  }
  downsample_rows<V><<<elementwise_grid(out.len * out.batch), 256, 0, s>>>(x, xb, o, out.batch_stride, out.len, n,
                                                                           out.batch);
  return check_launch("downsample");
}

int updown_fp(const gbfir_buf &out, const gbfir_buf &in, int64_t n, bool up, cudaStream_t s) {
  switch (in.dtype) {
    case GBFIR_F32: return launch_updown<float>(out, in, n, up, s);
    case GBFIR_F64: return launch_updown<double>(out, in, n, up, s);
    case GBFIR_C64: return launch_updown<float2>(out, in, n, up, s);
    default: return launch_updown<double2>(out, in, n, up, s);
  }
}

// downsample(conv1d(upsample(in, up), h, mode), down); shapes validated by the caller.
int upfirdn_fp(const gbfir_buf &out, const gbfir_buf &in, const gbfir_buf &h, int64_t up, int64_t down, int mode,
               cudaStream_t s) {
  if (up == 1 && down == 1) return conv1d_fp(out, in, h, mode, 0, s);
  const int64_t Nu = in.len * up, Lmin = Nu < h.len ? Nu : h.len;
  const int64_t start = mode == GBFIR_MODE_SAME ? ((Lmin & 1) ? (Lmin - 1) / 2 : Lmin / 2 - 1)
                      : mode == GBFIR_MODE_VALID ? Lmin - 1 : 0;
  const bool xc = dtype_complex(in.dtype), hc = dtype_complex(h.dtype);
  TileChoice tc;
  auto run = [&](auto tag, auto xcv, auto hcv) {
    using T = decltype(tag);
    return resample_pass<T, decltype(xcv)::value, decltype(hcv)::value>(
        in.ptr, in.batch_stride, in.len, h.ptr, h.len, out.ptr, out.batch_stride, out.len, out.batch, up, down, start,
        false, 0, 1.0, tc, s);
  };
  using Y = std::true_type;
  using F = std::false_type;
  if (dtype_double(in.dtype)) {
    if (xc && hc) return run(0.0, Y{}, Y{});
    if (xc) return run(0.0, Y{}, F{});
    if (hc) return run(0.0, F{}, Y{});
    return run(0.0, F{}, F{});
  }
  if (xc && hc) return run(0.0f, Y{}, Y{});
  if (xc) return run(0.0f, Y{}, F{});
  if (hc) return run(0.0f, F{}, Y{});
  return run(0.0f, F{}, F{});
}

}  // namespace gbfir
