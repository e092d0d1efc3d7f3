// matx_shim_check.cu — MatX user code, unchanged, routed to libgbfir by gbfir_matx.h.
//
// Built by tests/test_shim.py where the MatX headers exist.  The object must
// reference gbfir_resample_poly / gbfir_conv1d / gbfir_channelize_poly: that
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
  exec.sync();

  const double e1 = max_abs_diff(y, yr, B * olen), e2 = max_abs_diff(c, cr, B * (N + L - 1));
  const double e3 = max_abs_diff(r, rr, B * N), e4 = max_abs_diff(z, zr, B * T * M);
  printf("resample %g conv %g corr %g channelize %g launches %llu\n", e1, e2, e3, e4,
         (unsigned long long)gbfir_launch_count());
  return (e1 < 1e-3 && e2 < 1e-3 && e3 < 1e-3 && e4 < 1e-2) ? 0 : 1;
}
