// matx_shim_expr.cu — MatX operator expressions as the inputs of the routed operators.
//
// Built by tests/test_shim.py where the MatX headers exist.  Every call here takes an
// expression input (conj(x), h * 2.f, a permuted signal), never a plain tensor, so the
// object references gbfir_resample_poly / gbfir_conv1d / gbfir_channelize_poly /
// gbfir_conv2d only if the expression overloads were selected.  Run on a GPU host with
// MatX, it compares each result with MatX's HostExecutor and returns non-zero on a mismatch.
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
  cudaExecutor exec{cudaStream_t{0}};
  SingleThreadedHostExecutor host{};
  const index_t B = 3, N = 2048, L = 31;
  auto x = make_tensor<cuda::std::complex<float>>({B, N}, MATX_MANAGED_MEMORY);
  auto h = make_tensor<float>({L}, MATX_MANAGED_MEMORY);
  for (index_t b = 0; b < B; b++)
    for (index_t i = 0; i < N; i++) x(b, i) = {float((i * 5 + b) % 11) - 5.f, float((i * 7) % 3) - 1.f};
  for (index_t k = 0; k < L; k++) h(k) = float((k * 3) % 13 - 6) / 13.f;

  const index_t olen = (N * 3 + 1) / 2;
  auto y = make_tensor<cuda::std::complex<float>>({B, olen}, MATX_MANAGED_MEMORY);
  auto yr = make_tensor<cuda::std::complex<float>>({B, olen}, MATX_MANAGED_MEMORY);
  (y = resample_poly(conj(x), h * 2.f, 3, 2)).run(exec);
  (yr = resample_poly(conj(x), h * 2.f, 3, 2)).run(host);

  auto c = make_tensor<cuda::std::complex<float>>({B, N + L - 1}, MATX_MANAGED_MEMORY);
  auto cr = make_tensor<cuda::std::complex<float>>({B, N + L - 1}, MATX_MANAGED_MEMORY);
  (c = conv1d(conj(x), h * 2.f, MATX_C_MODE_FULL)).run(exec);
  (cr = conv1d(conj(x), h * 2.f, MATX_C_MODE_FULL)).run(host);

  const index_t M = 32, T = N / M;
  auto hc = make_tensor<float>({M * 4}, MATX_MANAGED_MEMORY);
  for (index_t k = 0; k < M * 4; k++) hc(k) = float((k * 5) % 9 - 4) / 9.f;
  auto z = make_tensor<cuda::std::complex<float>>({B, T, M}, MATX_MANAGED_MEMORY);
  auto zr = make_tensor<cuda::std::complex<float>>({B, T, M}, MATX_MANAGED_MEMORY);
  (z = channelize_poly(conj(x), hc, M, M)).run(exec);
  (zr = channelize_poly(conj(x), hc, M, M)).run(host);

  auto img = make_tensor<float>({B, 32, 32}, MATX_MANAGED_MEMORY);
  auto k2 = make_tensor<float>({3, 5}, MATX_MANAGED_MEMORY);
  auto c2 = make_tensor<float>({B, 32, 32}, MATX_MANAGED_MEMORY);
  auto c2r = make_tensor<float>({B, 32, 32}, MATX_MANAGED_MEMORY);
  for (index_t b = 0; b < B; b++)
    for (index_t i = 0; i < 32; i++)
      for (index_t j = 0; j < 32; j++) img(b, i, j) = float((i * 3 + j * 7 + b) % 19) - 9.f;
  for (index_t i = 0; i < 3; i++)
    for (index_t j = 0; j < 5; j++) k2(i, j) = float(i * 5 + j) / 9.f - 0.8f;
  (c2 = conv2d(img * 0.5f, k2, MATX_C_MODE_SAME)).run(exec);
  (c2r = conv2d(img * 0.5f, k2, MATX_C_MODE_SAME)).run(host);
  exec.sync();

  const double e1 = max_abs_diff(y, yr, B * olen), e2 = max_abs_diff(c, cr, B * (N + L - 1));
  const double e3 = max_abs_diff(z, zr, B * T * M), e4 = max_abs_diff(c2, c2r, B * 32 * 32);
  printf("resample %g conv %g channelize %g conv2d %g\n", e1, e2, e3, e4);
  return (e1 < 1e-3 && e2 < 1e-3 && e3 < 1e-2 && e4 < 1e-3) ? 0 : 1;
}
