// common.cuh — shared host/device helpers of the gbfir CUDA library (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <cstdio>
#include <string>
#include <type_traits>

#include "../../include/gbfir.h"

namespace gbfir {

// ---- status plumbing ---------------------------------------------------------

void set_error(const std::string &msg);  // thread-local message for gbfir_last_error()
void count_launch(uint64_t n = 1);       // feeds gbfir_launch_count()

#define GBFIR_FAIL(code, ...)                                    \
  do {                                                           \
    char _buf[512];                                              \
    snprintf(_buf, sizeof(_buf), __VA_ARGS__);                   \
    ::gbfir::set_error(_buf);                                    \
    return (code);                                               \
  } while (0)

// Check the launch that was just enqueued.
inline int check_launch(const char *what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    char buf[512];
    snprintf(buf, sizeof(buf), "%s: CUDA launch failed: %s", what, cudaGetErrorString(e));
    set_error(buf);
    return GBFIR_ERR_CUDA;
  }
  count_launch();
  return GBFIR_SUCCESS;
}

int num_sms();  // SM count of the current device (cached per device)

// Opt a kernel in to more than 48 KB of dynamic shared memory (cached per function).
int ensure_smem(const void *func, size_t bytes, const char *what);

// ---- integer helpers -----------------------------------------------------------

__host__ __device__ __forceinline__ int64_t floor_div(int64_t a, int64_t b) {
  // b > 0
  return a >= 0 ? a / b : -((-a + b - 1) / b);
}
__host__ __device__ __forceinline__ int64_t ceil_div(int64_t a, int64_t b) {
  return -floor_div(-a, b);
}
inline int64_t gcd64(int64_t a, int64_t b) {
  while (b) {
    int64_t t = a % b;
    a = b;
    b = t;
  }
  return a;
}

// ---- value types ---------------------------------------------------------------

template <typename T> struct cplx_of;
template <> struct cplx_of<float> { using type = float2; };
template <> struct cplx_of<double> { using type = double2; };

template <typename T, bool C> struct val_of;  // storage type of one element
template <typename T> struct val_of<T, false> { using type = T; };
template <typename T> struct val_of<T, true> { using type = typename cplx_of<T>::type; };

// A value that may be real or complex, with explicit re/im for FMA chains.
template <typename T, bool C> struct Acc;
template <typename T> struct Acc<T, false> {
  T re;
  __device__ __forceinline__ void zero() { re = T(0); }
};
template <typename T> struct Acc<T, true> {
  T re, im;
  __device__ __forceinline__ void zero() { re = T(0); im = T(0); }
};

template <typename T> __device__ __forceinline__ T re_of(T v) { return v; }
template <typename T> __device__ __forceinline__ T im_of(T) { return T(0); }
__device__ __forceinline__ float re_of(float2 v) { return v.x; }
__device__ __forceinline__ float im_of(float2 v) { return v.y; }
__device__ __forceinline__ double re_of(double2 v) { return v.x; }
__device__ __forceinline__ double im_of(double2 v) { return v.y; }

// acc += x * h  with the FMA order of MatX's madd (core/utils.h:204-208):
//   re += xr*hr; re -= xi*hi; im += xi*hr; im += xr*hi.
template <typename T, bool XC, bool HC>
__device__ __forceinline__ void mac(Acc<T, XC || HC> &a,
                                    typename val_of<T, XC>::type x,
                                    typename val_of<T, HC>::type h) {
  if constexpr (XC && HC) {
    a.re = fma(re_of(x), re_of(h), a.re);
    a.re = fma(-im_of(x), im_of(h), a.re);
    a.im = fma(im_of(x), re_of(h), a.im);
    a.im = fma(re_of(x), im_of(h), a.im);
  } else if constexpr (XC) {
    if constexpr (std::is_same<T, float>::value) {
      // one packed f32x2 FMA: each lane is exactly the scalar fma of the line below
      const float2 r = __ffma2_rn(x, make_float2(h, h), make_float2(a.re, a.im));
      a.re = r.x;
      a.im = r.y;
    } else {
      a.re = fma(re_of(x), h, a.re);
      a.im = fma(im_of(x), h, a.im);
    }
  } else if constexpr (HC) {
    a.re = fma(x, re_of(h), a.re);
    a.im = fma(x, im_of(h), a.im);
  } else {
    a.re = fma(x, h, a.re);
  }
}

template <typename T, bool C>
__device__ __forceinline__ typename val_of<T, C>::type pack(const Acc<T, C> &a, T scale) {
  if constexpr (C) {
    typename val_of<T, C>::type v;
    v.x = a.re * scale;
    v.y = a.im * scale;
    return v;
  } else {
    return a.re * scale;
  }
}

template <typename V> __device__ __forceinline__ V zero_val() {
  V v;
  if constexpr (std::is_arithmetic<V>::value) {
    v = V(0);
  } else {
    v.x = 0;
    v.y = 0;
  }
  return v;
}

// ---- cp.async (LDGSTS) with zero fill --------------------------------------------
// `bytes` is 4, 8 or 16; `valid` == false fills the destination with zeros and
// reads nothing (src-size operand 0), so out-of-range halo samples cost no load.

template <int BYTES>
__device__ __forceinline__ void cp_async_zfill(void *smem_dst, const void *gmem_src, bool valid) {
  const uint32_t dst = static_cast<uint32_t>(__cvta_generic_to_shared(smem_dst));
  const int src_size = valid ? BYTES : 0;
  if constexpr (BYTES == 16) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(gmem_src), "r"(src_size)
                 : "memory");
  } else {
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;\n" ::"r"(dst), "l"(gmem_src), "n"(BYTES),
                 "r"(src_size)
                 : "memory");
  }
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// ---- buffer validation -----------------------------------------------------------

inline bool dtype_complex(int32_t dt) { return dt == GBFIR_C64 || dt == GBFIR_C128; }
inline bool dtype_double(int32_t dt) { return dt == GBFIR_F64 || dt == GBFIR_C128; }
inline size_t dtype_size(int32_t dt) {
  switch (dt) {
    case GBFIR_F32: return 4;
    case GBFIR_C64: return 8;
    case GBFIR_F64: return 8;
    case GBFIR_C128: return 16;
    default: return 0;
  }
}

int check_buf(const gbfir_buf &b, const char *name, bool allow_broadcast);

}  // namespace gbfir
