// matx_ref.cu — runs MatX's own HostExecutor operators for the direct-FIR path.
//
// TEST INFRASTRUCTURE ONLY.  Compiled by `make -C oracle ref` against the MatX
// headers (header-only library) into oracle/_ref/libmatxref.so.  The tests use
// it to pin the C oracle (gbfir_oracle.c) to the reference's real behaviour on
// the same inputs.  It runs only on hosts where the MatX headers are present.
//
// Every entry point wraps caller memory in non-owning MatX tensors and runs the
// public operator expression on SelectThreadsHostExecutor, exactly as a MatX
// user would:
//   (y = conv1d(x, h, mode)).run(exec)        operators/conv.h:243-274
//   (y = corr(x, h, mode, DIRECT)).run(exec)  operators/corr.h:224-253
//   (y = resample_poly(x, h, up, down)).run(exec)  operators/resample_poly.h:182-186
//   (y = channelize_poly(x, h, M, D)).run(exec)    operators/channelize_poly.h:275-278
#include "matx.h"

#include <complex>

using namespace matx;

namespace {

template <typename T>
struct host_t { using type = T; };
template <>
struct host_t<std::complex<float>> { using type = cuda::std::complex<float>; };
template <>
struct host_t<std::complex<double>> { using type = cuda::std::complex<double>; };

template <typename XT, typename HT, typename OT>
int run_conv(void *out, const void *x, index_t N, const void *h, index_t L,
             index_t B, int mode, int is_corr, int h_batched, int nthreads) {
  try {
    SelectThreadsHostExecutor exec{HostExecParams{nthreads}};
    auto xt = make_tensor<XT>(reinterpret_cast<XT *>(const_cast<void *>(x)), {B, N});
    const index_t out_len = mode == 0 ? N + L - 1
                          : mode == 1 ? std::max(N, L)
                                      : std::max(N, L) - std::min(N, L) + 1;
    auto yt = make_tensor<OT>(reinterpret_cast<OT *>(out), {B, out_len});
    const auto m = mode == 0 ? MATX_C_MODE_FULL : mode == 1 ? MATX_C_MODE_SAME : MATX_C_MODE_VALID;
    if (h_batched) {
      auto ht = make_tensor<HT>(reinterpret_cast<HT *>(const_cast<void *>(h)), {B, L});
      if (is_corr) (yt = corr(xt, ht, m, MATX_C_METHOD_DIRECT)).run(exec);
      else (yt = conv1d(xt, ht, m)).run(exec);
    } else {
      auto ht = make_tensor<HT>(reinterpret_cast<HT *>(const_cast<void *>(h)), {L});
      if (is_corr) (yt = corr(xt, ht, m, MATX_C_METHOD_DIRECT)).run(exec);
      else (yt = conv1d(xt, ht, m)).run(exec);
    }
    return 0;
  } catch (const std::exception &e) {
    fprintf(stderr, "matxref conv: %s\n", e.what());
    return 1;
  }
}

template <typename XT, typename HT, typename OT>
int run_resample(void *out, index_t out_len, const void *x, index_t N,
                 const void *h, index_t L, index_t B, index_t up, index_t down,
                 int nthreads) {
  try {
    SelectThreadsHostExecutor exec{HostExecParams{nthreads}};
    auto xt = make_tensor<XT>(reinterpret_cast<XT *>(const_cast<void *>(x)), {B, N});
    auto ht = make_tensor<HT>(reinterpret_cast<HT *>(const_cast<void *>(h)), {L});
    auto yt = make_tensor<OT>(reinterpret_cast<OT *>(out), {B, out_len});
    (yt = resample_poly(xt, ht, up, down)).run(exec);
    return 0;
  } catch (const std::exception &e) {
    fprintf(stderr, "matxref resample: %s\n", e.what());
    return 1;
  }
}

template <typename XT, typename HT, typename OT>
int run_channelize(void *out, const void *x, index_t N, const void *h, index_t L,
                   index_t B, index_t M, index_t D, int nthreads) {
  try {
    SelectThreadsHostExecutor exec{HostExecParams{nthreads}};
    const index_t T = (N + D - 1) / D;
    auto xt = make_tensor<XT>(reinterpret_cast<XT *>(const_cast<void *>(x)), {B, N});
    auto ht = make_tensor<HT>(reinterpret_cast<HT *>(const_cast<void *>(h)), {L});
    auto yt = make_tensor<OT>(reinterpret_cast<OT *>(out), {B, T, M});
    (yt = channelize_poly(xt, ht, M, D)).run(exec);
    return 0;
  } catch (const std::exception &e) {
    fprintf(stderr, "matxref channelize: %s\n", e.what());
    return 1;
  }
}

using c64 = cuda::std::complex<float>;
using c128 = cuda::std::complex<double>;

}  // namespace

extern "C" {

// conv1d / corr.  kind: 0 = f32*f32, 1 = c64*f32, 2 = c64*c64, 3 = f64*f64,
// 4 = c128*f64, 5 = c128*c128.
int matxref_conv1d(int kind, void *out, const void *x, int64_t N, const void *h,
                   int64_t L, int64_t B, int mode, int is_corr, int h_batched,
                   int nthreads) {
  switch (kind) {
    case 0: return run_conv<float, float, float>(out, x, N, h, L, B, mode, is_corr, h_batched, nthreads);
    case 1: return run_conv<c64, float, c64>(out, x, N, h, L, B, mode, is_corr, h_batched, nthreads);
    case 2: return run_conv<c64, c64, c64>(out, x, N, h, L, B, mode, is_corr, h_batched, nthreads);
    case 3: return run_conv<double, double, double>(out, x, N, h, L, B, mode, is_corr, h_batched, nthreads);
    case 4: return run_conv<c128, double, c128>(out, x, N, h, L, B, mode, is_corr, h_batched, nthreads);
    case 5: return run_conv<c128, c128, c128>(out, x, N, h, L, B, mode, is_corr, h_batched, nthreads);
    default: return 2;
  }
}

// resample_poly.  kind: 0 = f32 x, f32 h; 1 = c64 x, f32 h; 2 = c64 x, c64 h;
// 3 = f64/f64; 4 = c128 x, f64 h.
int matxref_resample_poly(int kind, void *out, int64_t out_len, const void *x,
                          int64_t N, const void *h, int64_t L, int64_t B,
                          int64_t up, int64_t down, int nthreads) {
  switch (kind) {
    case 0: return run_resample<float, float, float>(out, out_len, x, N, h, L, B, up, down, nthreads);
    case 1: return run_resample<c64, float, c64>(out, out_len, x, N, h, L, B, up, down, nthreads);
    case 2: return run_resample<c64, c64, c64>(out, out_len, x, N, h, L, B, up, down, nthreads);
    case 3: return run_resample<double, double, double>(out, out_len, x, N, h, L, B, up, down, nthreads);
    case 4: return run_resample<c128, double, c128>(out, out_len, x, N, h, L, B, up, down, nthreads);
    default: return 2;
  }
}

// channelize_poly.  kind: 0 = c64 x, f32 h; 1 = c64 x, c64 h; 2 = c128 x, f64 h;
// 3 = f32 x, f32 h (real path: R2C + unpack on the CUDA side, same values).
int matxref_channelize_poly(int kind, void *out, const void *x, int64_t N,
                            const void *h, int64_t L, int64_t B, int64_t M,
                            int64_t D, int nthreads) {
  switch (kind) {
    case 0: return run_channelize<c64, float, c64>(out, x, N, h, L, B, M, D, nthreads);
    case 1: return run_channelize<c64, c64, c64>(out, x, N, h, L, B, M, D, nthreads);
    case 2: return run_channelize<c128, double, c128>(out, x, N, h, L, B, M, D, nthreads);
    case 3: return run_channelize<float, float, c64>(out, x, N, h, L, B, M, D, nthreads);
    default: return 2;
  }
}

}  // extern "C"
