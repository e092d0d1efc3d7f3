// matx_shim_check.cu — MatX user code, unchanged, routed to libgbfir by gbfir_matx.h.
//
// Built by tests/test_shim.py where the MatX headers exist.  The object must
// reference gbfir_resample_poly / gbfir_conv1d / gbfir_channelize_poly /
// gbfir_conv1d_axis / gbfir_filter / gbfir_conv1d_fft / gbfir_conv2d: that
// proves MatX's own operator classes resolved their *_impl calls to the
// gbfir overloads.  Run on a GPU host with MatX, it also compares every result
// with MatX's HostExecutor and returns non-zero on a mismatch.
#include <matx.h>
#include "gbfir_matx.h"

#include <cstdio>

using namespace matx;

template <typename A, typename B>
static double max_abs_diff(const A &a, const B &b, index_t n) {
  double m = 0;
  for (index_t i = 0; i < n; i++) {
    const double d = cuda::std::abs(a.Data()[i] - b.Data()[i]);
    m = d > m ? d : m;
  }
  return m;
}

int main() {
  cudaStream_t stream = 0;
  cudaExecutor exec{stream};
  SingleThreadedHostExecutor host{};
  const index_t B = 4, N = 4096, L = 61;
  auto x = make_tensor<cuda::std::complex<float>>({B, N}, MATX_MANAGED_MEMORY);
  auto h = make_tensor<float>({L}, MATX_MANAGED_MEMORY);
  for (index_t b = 0; b < B; b++)
    for (index_t i = 0; i < N; i++) x(b, i) = {float((i * 7 + b) % 13) - 6.f, float((i * 3) % 5) - 2.f};
  for (index_t k = 0; k < L; k++) h(k) = float((k * 5) % 11 - 5) / 11.f;

  // resample_poly
  const index_t olen = (N * 3 + 1) / 2;
  auto y = make_tensor<cuda::std::complex<float>>({B, olen}, MATX_MANAGED_MEMORY);
  auto yr = make_tensor<cuda::std::complex<float>>({B, olen}, MATX_MANAGED_MEMORY);
  (y = resample_poly(x, h, 3, 2)).run(exec);
  (yr = resample_poly(x, h, 3, 2)).run(host);

  // conv1d and corr, direct
  auto c = make_tensor<cuda::std::complex<float>>({B, N + L - 1}, MATX_MANAGED_MEMORY);
  auto cr = make_tensor<cuda::std::complex<float>>({B, N + L - 1}, MATX_MANAGED_MEMORY);
  (c = conv1d(x, h, MATX_C_MODE_FULL)).run(exec);
  (cr = conv1d(x, h, MATX_C_MODE_FULL)).run(host);
  auto cf = make_tensor<cuda::std::complex<float>>({B, N + L - 1}, MATX_MANAGED_MEMORY);
  (cf = conv1d(x, h, MATX_C_MODE_FULL, MATX_C_METHOD_FFT)).run(exec);
  auto r = make_tensor<cuda::std::complex<float>>({B, N}, MATX_MANAGED_MEMORY);
  auto rr = make_tensor<cuda::std::complex<float>>({B, N}, MATX_MANAGED_MEMORY);
  (r = corr(x, h, MATX_C_MODE_SAME, MATX_C_METHOD_DIRECT)).run(exec);
  (rr = corr(x, h, MATX_C_MODE_SAME, MATX_C_METHOD_DIRECT)).run(host);

  // channelize_poly, M = 64, D = 64
  const index_t M = 64, T = N / M;
  auto hc = make_tensor<float>({M * 8}, MATX_MANAGED_MEMORY);
  for (index_t k = 0; k < M * 8; k++) hc(k) = float((k * 3) % 7 - 3) / 7.f;
  auto z = make_tensor<cuda::std::complex<float>>({B, T, M}, MATX_MANAGED_MEMORY);
  auto zr = make_tensor<cuda::std::complex<float>>({B, T, M}, MATX_MANAGED_MEMORY);
  (z = channelize_poly(x, hc, M, M)).run(exec);
  (zr = channelize_poly(x, hc, M, M)).run(host);
  // radar three-pulse canceller: conv1d SAME over the pulses of a permuted cube
  // (examples/simple_radar_pipeline.h:321-327); runs on the strided view, no transpose
  const index_t C = 2, P = 16, S = 300;
  auto cube = make_tensor<cuda::std::complex<float>>({C, P, S}, MATX_MANAGED_MEMORY);
  auto tpc = make_tensor<cuda::std::complex<float>>({C, P, S}, MATX_MANAGED_MEMORY);
  auto tpcr = make_tensor<cuda::std::complex<float>>({C, S, P}, MATX_MANAGED_MEMORY);
  auto mask = make_tensor<cuda::std::complex<float>>({3}, MATX_MANAGED_MEMORY);
  mask(0) = {1.f, 0.f};
  mask(1) = {-2.f, 0.f};
  mask(2) = {1.f, 0.f};
  for (index_t a = 0; a < C; a++)
    for (index_t p = 0; p < P; p++)
      for (index_t q = 0; q < S; q++) cube(a, p, q) = {float((a + 3 * p + 5 * q) % 9) - 4.f, float((p * q) % 7) - 3.f};
  auto xv = cube.Permute({0, 2, 1});
  auto ov = tpc.Permute({0, 2, 1});
  (ov = conv1d(xv, mask, MATX_C_MODE_SAME)).run(exec);
  (tpcr = conv1d(xv, mask, MATX_C_MODE_SAME)).run(host);

  // conv2d SAME of the 4 images (4 x 4096 viewed as 4 x 64 x 64) with a 5 x 3 filter
  auto img = make_tensor<float>({B, 64, 64}, MATX_MANAGED_MEMORY);
  auto k2 = make_tensor<float>({5, 3}, MATX_MANAGED_MEMORY);
  auto c2 = make_tensor<float>({B, 64, 64}, MATX_MANAGED_MEMORY);
  auto c2r = make_tensor<float>({B, 64, 64}, MATX_MANAGED_MEMORY);
  for (index_t b = 0; b < B; b++)
    for (index_t i = 0; i < 64; i++)
      for (index_t j = 0; j < 64; j++) img(b, i, j) = float((i * 5 + j * 3 + b) % 17) - 8.f;
  for (index_t i = 0; i < 5; i++)
    for (index_t j = 0; j < 3; j++) k2(i, j) = float(i * 3 + j) / 7.f - 1.f;
  (c2 = conv2d(img, k2, MATX_C_MODE_SAME)).run(exec);
  (c2r = conv2d(img, k2, MATX_C_MODE_SAME)).run(host);

  // filter(): the reference test's second-order section
  auto fx = make_tensor<float>({B, N}, MATX_MANAGED_MEMORY);
  auto fy = make_tensor<float>({B, N}, MATX_MANAGED_MEMORY);
  for (index_t b = 0; b < B; b++)
    for (index_t i = 0; i < N; i++) fx(b, i) = float(((i + 11 * b) % 23) - 11) / 7.f;
  const cuda::std::array<float, 2> h_rec{0.4f, -0.1f}, h_nonrec{2.0f, 1.0f};
  (fy = filter(fx, h_rec, h_nonrec)).run(exec);
  exec.sync();

  double e5 = 0;
  for (index_t a = 0; a < C; a++)
    for (index_t q = 0; q < S; q++)
      for (index_t p = 0; p < P; p++) {
        const double d = cuda::std::abs(tpc(a, p, q) - tpcr(a, q, p));
        e5 = d > e5 ? d : e5;
      }
  double e6 = 0;  // the recurrence in double, sequentially
  for (index_t b = 0; b < B; b++) {
    double y1 = 0, y2 = 0;
    for (index_t i = 0; i < N; i++) {
      const double y = 2.0 * fx(b, i) + (i ? 1.0 * fx(b, i - 1) : 0.0) + 0.4 * y1 - 0.1 * y2;
      y2 = y1;
      y1 = y;
      const double d = cuda::std::abs(fy(b, i) - y);
      e6 = d > e6 ? d : e6;
    }
  }

  const double e1 = max_abs_diff(y, yr, B * olen), e2 = max_abs_diff(c, cr, B * (N + L - 1));
  const double e3 = max_abs_diff(r, rr, B * N), e4 = max_abs_diff(z, zr, B * T * M);
  const double e7 = max_abs_diff(cf, cr, B * (N + L - 1));
  const double e8 = max_abs_diff(c2, c2r, B * 64 * 64);
  printf("resample %g conv %g corr %g channelize %g canceller %g filter %g fft-conv %g conv2d %g launches %llu\n",
         e1, e2, e3, e4, e5, e6, e7, e8, (unsigned long long)gbfir_launch_count());
  return (e1 < 1e-3 && e2 < 1e-3 && e3 < 1e-3 && e4 < 1e-2 && e5 < 1e-4 && e6 < 1e-2 && e7 < 1e-3 && e8 < 1e-3) ? 0
                                                                                                          : 1;
}
