// gbfir_matx.h — drop-in routing of MatX's direct-FIR operators to libgbfir (sm_103a).
//
// Include this header after <matx.h> and link libgbfir.so.  User code is unchanged:
//
//     (out = matx::resample_poly(in, h, up, down)).run(matx::cudaExecutor{stream});
//     (y   = matx::conv1d(x, h, MATX_C_MODE_FULL)).run(exec);
//     (y   = matx::corr(x, h, MATX_C_MODE_FULL, MATX_C_METHOD_DIRECT)).run(exec);
//     (Y   = matx::channelize_poly(x, h, M, D)).run(exec);
//     (y   = matx::filter(x, h_rec, h_nonrec)).run(exec);
//     (z   = matx::conv2d(images, kernel, MATX_C_MODE_SAME)).run(exec);
//
// How: MatX's operator classes call resample_poly_impl / conv1d_impl / corr_impl /
// channelize_poly_impl / filter_impl unqualified from their Exec() (operators/resample_poly.h:
// 113-120, operators/conv.h:178-188, operators/corr.h:170-180, operators/channelize_poly.h:
// 117-134, operators/filter.h:97-101).  conv1d / corr of a 1-D filter over a view whose last
// dimension is strided (conv1d with an axis, or a permuted view as in the radar
// three-pulse canceller) run in place of the view's layout (gbfir_conv1d_axis).
// This header adds, in namespace matx, overloads with the same parameter lists and
// stronger constraints — a CUDA executor, a MatX tensor output and tensor or operator
// expression inputs of float, double, complex<float> or complex<double> — so C++20 overload
// resolution selects them (the executor argument brings namespace matx into argument-
// dependent lookup).  An expression input is evaluated once into a contiguous temporary.
// Host executors, FFT convolutions outside the overlap-save kernel's range and other value
// types keep MatX's own implementation.
//
// Each overload keeps the MatX transform's asserts and error classes: a gbfir_status
// is rethrown as matxException with the matching matxError_t.  Tensors whose batch
// dimensions do not fold into one stride are first copied into contiguous temporaries
// with MatX's own elementwise executor, as MatX does for nested transforms.
#pragma once

#include <matx.h>

#include <numeric>
#include <type_traits>

#include "gbfir.h"

namespace matx {
namespace gbfir_shim {

template <typename T>
constexpr int32_t dtype_of() {
  using V = remove_cvref_t<T>;
  if constexpr (std::is_same_v<V, float>) return GBFIR_F32;
  else if constexpr (std::is_same_v<V, double>) return GBFIR_F64;
  else if constexpr (std::is_same_v<V, cuda::std::complex<float>>) return GBFIR_C64;
  else if constexpr (std::is_same_v<V, cuda::std::complex<double>>) return GBFIR_C128;
  else return -1;
}

template <typename Op>
concept routable_tensor = is_tensor_view_v<remove_cvref_t<Op>> && (remove_cvref_t<Op>::Rank() >= 1) &&
                          (dtype_of<typename remove_cvref_t<Op>::value_type>() >= 0);

// An input operand: a tensor view, or an operator expression (x * 2.f, conj(x), a generator
// ...) of a routable value type.  MatX's kernels read an expression element by element
// (transforms/resample_poly.h:142-146 chooses between the tensor and operator paths); here
// Staged evaluates it once into a contiguous temporary with MatX's elementwise executor,
// after which the C-ABI sees plain rows.
template <typename Op>
concept routable_operand = (is_tensor_view_v<remove_cvref_t<Op>> || is_matx_op_c<Op>) &&
                           (remove_cvref_t<Op>::Rank() >= 1) &&
                           (dtype_of<typename remove_cvref_t<Op>::value_type>() >= 0);

inline matxError_t to_matx_error(int rc) {
  switch (rc) {
    case GBFIR_ERR_INVALID_PARAMETER: return matxInvalidParameter;
    case GBFIR_ERR_INVALID_DIM: return matxInvalidDim;
    case GBFIR_ERR_INVALID_SIZE: return matxInvalidSize;
    case GBFIR_ERR_INVALID_TYPE: return matxInvalidType;
    case GBFIR_ERR_NOT_SUPPORTED: return matxNotSupported;
    default: return matxCudaError;
  }
}

inline void check(int rc) {
  if (rc != GBFIR_SUCCESS) {
    MATX_THROW(to_matx_error(rc), gbfir_last_error());
  }
}

// Rows of the last dimension with one batch stride, or false if the layout does not fold.
template <typename Op>
bool describe(const Op &t, gbfir_buf &b) {
  constexpr int R = remove_cvref_t<Op>::Rank();
  if (t.Size(R - 1) > 1 && t.Stride(R - 1) != 1) return false;
  index_t batch = 1;
  for (int i = 0; i < R - 1; i++) batch *= t.Size(i);
  index_t bstride = 0;
  if constexpr (R >= 2) {
    // innermost non-unit batch dimension sets the stride; every outer one must be dense over it
    int inner = -1;
    for (int i = R - 2; i >= 0; i--) {
      if (t.Size(i) > 1) { inner = i; break; }
    }
    if (inner >= 0) {
      bstride = t.Stride(inner);
      index_t expect = bstride * t.Size(inner);
      for (int i = inner - 1; i >= 0; i--) {
        if (t.Size(i) == 1) continue;
        if (t.Stride(i) != expect) return false;
        expect *= t.Size(i);
      }
    }
  }
  b.ptr = const_cast<void *>(static_cast<const void *>(t.Data()));
  b.batch = batch;
  b.len = t.Size(R - 1);
  b.batch_stride = batch > 1 ? bstride : 0;
  b.dtype = dtype_of<typename remove_cvref_t<Op>::value_type>();
  return true;
}

// An operand as a gbfir_buf, materialised into a contiguous temporary if needed.
template <typename Op, typename Executor>
struct Staged {
  using value_type = typename remove_cvref_t<Op>::value_type;
  static constexpr int R = remove_cvref_t<Op>::Rank();
  gbfir_buf buf{};
  decltype(make_tensor<value_type>(cuda::std::array<index_t, R>{}, MATX_ASYNC_DEVICE_MEMORY,
                                   cudaStream_t{})) tmp;
  Staged(const Op &t, const Executor &exec) {
    bool direct = false;
    if constexpr (is_tensor_view_v<remove_cvref_t<Op>>) direct = describe(t, buf);
    if (!direct) {
      cuda::std::array<index_t, R> shape;
      for (int i = 0; i < R; i++) shape[i] = t.Size(i);
      (void)(tmp = make_tensor<value_type>(shape, MATX_ASYNC_DEVICE_MEMORY, exec.getStream()));
      (tmp = t).run(exec);
      (void)describe(tmp, buf);
    }
  }
};

inline gbfir_stream_t stream_of(cudaStream_t s) { return reinterpret_cast<gbfir_stream_t>(s); }

// A rank >= 2 operand whose last dimension is strided, as signals
// x[o*ostride + n*step + i]: one unit-stride inner dimension, the others folding into one outer
// stride (MatX's permuted views, e.g. the radar three-pulse canceller's).
struct AxisLayout {
  gbfir_buf buf{};
  index_t inner = 1, step = 1;
  int inner_dim = -1, nouter = 0, outer_dims[8] = {};
};
template <typename Op>
bool describe_axis(const Op &t, AxisLayout &l) {
  constexpr int R = remove_cvref_t<Op>::Rank();
  if constexpr (R < 2 || R > 9) {
    return false;
  } else {
    if (t.Size(R - 1) <= 1 || t.Stride(R - 1) == 1) return false;
    l.step = t.Stride(R - 1);
    l.inner_dim = -1;
    for (int i = R - 2; i >= 0; i--)
      if (t.Size(i) > 1 && t.Stride(i) == 1) {
        l.inner_dim = i;
        break;
      }
    if (l.inner_dim < 0) return false;
    l.nouter = 0;
    for (int i = 0; i < R - 1; i++)
      if (i != l.inner_dim && t.Size(i) > 1) l.outer_dims[l.nouter++] = i;
    for (int a = 1; a < l.nouter; a++)  // by stride, largest first
      for (int c = a; c > 0 && t.Stride(l.outer_dims[c]) > t.Stride(l.outer_dims[c - 1]); c--) {
        const int tmp = l.outer_dims[c];
        l.outer_dims[c] = l.outer_dims[c - 1];
        l.outer_dims[c - 1] = tmp;
      }
    index_t outer = 1;
    for (int a = 0; a < l.nouter; a++) {
      outer *= t.Size(l.outer_dims[a]);
      if (a + 1 < l.nouter &&
          t.Stride(l.outer_dims[a]) != t.Stride(l.outer_dims[a + 1]) * t.Size(l.outer_dims[a + 1]))
        return false;
    }
    l.inner = t.Size(l.inner_dim);
    l.buf.ptr = const_cast<void *>(static_cast<const void *>(t.Data()));
    l.buf.batch = outer;
    l.buf.len = t.Size(R - 1);
    l.buf.batch_stride = outer > 1 ? t.Stride(l.outer_dims[l.nouter - 1]) : 0;
    l.buf.dtype = dtype_of<typename remove_cvref_t<Op>::value_type>();
    return true;
  }
}

// conv1d / corr of a 1-D filter along a strided last dimension, in place of the views' layout;
// false when the operands do not have that form (the caller then stages them).
template <typename OutputType, typename In1Type, typename In2Type, typename Executor>
bool conv_axis(OutputType &o, const In1Type &i1, const In2Type &i2, matxConvCorrMode_t mode, int is_corr,
               const Executor &exec) {
  if constexpr (remove_cvref_t<In2Type>::Rank() != 1 || !is_tensor_view_v<remove_cvref_t<In1Type>> ||
                remove_cvref_t<In1Type>::Rank() != remove_cvref_t<OutputType>::Rank()) {
    return false;
  } else {
    AxisLayout lo, li;
    if (!describe_axis(o, lo) || !describe_axis(i1, li)) return false;
    if (lo.inner_dim != li.inner_dim || lo.nouter != li.nouter) return false;
    for (int a = 0; a < lo.nouter; a++)
      if (lo.outer_dims[a] != li.outer_dims[a]) return false;
    Staged<In2Type, Executor> h(i2, exec);
    check(gbfir_conv1d_axis(lo.buf, li.buf, h.buf, li.inner, li.step, lo.step, static_cast<int32_t>(mode),
                            is_corr, GBFIR_PREC_FP32, stream_of(exec.getStream())));
    return true;
  }
}

}  // namespace gbfir_shim

// ---- resample_poly ------------------------------------------------------------------
// Replaces transforms/resample_poly.h:299-354 for CUDA executors.
template <typename OutType, typename InType, typename FilterType, typename Executor>
  requires is_executor<Executor> && is_cuda_executor_v<Executor> && gbfir_shim::routable_tensor<OutType> &&
           gbfir_shim::routable_operand<InType> && gbfir_shim::routable_operand<FilterType>
inline void resample_poly_impl(OutType &out, const InType &in, const FilterType &f, index_t up, index_t down,
                               Executor &&exec) {
  MATX_NVTX_START("gbfir resample_poly", matx::MATX_NVTX_LOG_API)
  static_assert(remove_cvref_t<OutType>::Rank() == remove_cvref_t<InType>::Rank(), "resample_poly: rank mismatch");
  static_assert(remove_cvref_t<FilterType>::Rank() == 1, "resample_poly: currently only support 1D filters");
  gbfir_shim::Staged<OutType, remove_cvref_t<Executor>> o(out, exec);
  gbfir_shim::Staged<InType, remove_cvref_t<Executor>> x(in, exec);
  gbfir_shim::Staged<FilterType, remove_cvref_t<Executor>> h(f, exec);
  gbfir_shim::check(gbfir_resample_poly(o.buf, x.buf, h.buf, up, down, GBFIR_PREC_FP32,
                                        gbfir_shim::stream_of(exec.getStream())));
  if (o.buf.ptr != static_cast<const void *>(out.Data())) (out = o.tmp).run(exec);
}

// ---- conv1d (direct) --------------------------------------------------------------------
// Replaces transforms/conv.h:467-532 for CUDA executors and the direct method.
template <typename OutputType, typename In1Type, typename In2Type, typename Executor>
  requires is_cuda_executor_v<Executor> && gbfir_shim::routable_tensor<OutputType> &&
           gbfir_shim::routable_operand<In1Type> && gbfir_shim::routable_operand<In2Type>
inline void conv1d_impl(OutputType o, const In1Type &i1, const In2Type &i2, matxConvCorrMode_t mode,
                        matxConvCorrMethod_t method, const Executor &exec) {
  MATX_NVTX_START("gbfir conv1d", matx::MATX_NVTX_LOG_API)
  if (method != MATX_C_METHOD_DIRECT) {
    // FFT method: the overlap-save kernel for float / complex<float> rows and one filter row
    // of at most GBFIR_FFT_CONV_MAX_TAPS taps no longer than the signal (gbfir_conv1d_fft)
    using V1 = typename remove_cvref_t<In1Type>::value_type;
    using V2 = typename remove_cvref_t<In2Type>::value_type;
    constexpr bool single = (std::is_same_v<V1, float> || std::is_same_v<V1, cuda::std::complex<float>>) &&
                            (std::is_same_v<V2, float> || std::is_same_v<V2, cuda::std::complex<float>>);
    if constexpr (single && remove_cvref_t<In2Type>::Rank() == 1) {
      const index_t n = i1.Size(remove_cvref_t<In1Type>::Rank() - 1), l = i2.Size(0);
      if (n >= l && l <= GBFIR_FFT_CONV_MAX_TAPS) {
        gbfir_shim::Staged<OutputType, Executor> out(o, exec);
        gbfir_shim::Staged<In1Type, Executor> a(i1, exec);
        gbfir_shim::Staged<In2Type, Executor> b(i2, exec);
        gbfir_shim::check(gbfir_conv1d_fft(out.buf, a.buf, b.buf, static_cast<int32_t>(mode), 0,
                                           gbfir_shim::stream_of(exec.getStream())));
        if (out.buf.ptr != static_cast<const void *>(o.Data())) (o = out.tmp).run(exec);
        return;
      }
    }
    // otherwise MatX's own path (conv1d_impl_internal, transforms/conv.h:402-451), with
    // the lower-rank operand cloned across the batch as conv.h:467-532 does.
    constexpr int R1 = remove_cvref_t<In1Type>::Rank(), R2 = remove_cvref_t<In2Type>::Rank();
    if constexpr (R1 == R2) {
      conv1d_impl_internal(o, i1, i2, mode, method, exec);
    } else if constexpr (R1 > R2) {
      index_t shape[R1];
      for (int i = 0; i < R1; i++) shape[i] = i < R1 - R2 ? i1.Size(i) : matxKeepDim;
      conv1d_impl_internal(o, i1, clone<R1>(i2, shape), mode, method, exec);
    } else {
      index_t shape[R2];
      for (int i = 0; i < R2; i++) shape[i] = i < R2 - R1 ? i2.Size(i) : matxKeepDim;
      conv1d_impl_internal(o, clone<R2>(i1, shape), i2, mode, method, exec);
    }
    return;
  }
  if (gbfir_shim::conv_axis(o, i1, i2, mode, 0, exec)) return;  // strided-axis views, no transpose
  gbfir_shim::Staged<OutputType, Executor> out(o, exec);
  gbfir_shim::Staged<In1Type, Executor> a(i1, exec);
  gbfir_shim::Staged<In2Type, Executor> b(i2, exec);
  gbfir_shim::check(gbfir_conv1d(out.buf, a.buf, b.buf, static_cast<int32_t>(mode), 0, GBFIR_PREC_FP32,
                                 gbfir_shim::stream_of(exec.getStream())));
  if (out.buf.ptr != static_cast<const void *>(o.Data())) (o = out.tmp).run(exec);
}

// ---- corr (direct) ------------------------------------------------------------------------
// Replaces transforms/corr.h:60-69: corr(a, b) = conv1d(a, reverse(conj(b))), applied in-kernel.
template <typename OutputTensor, typename In1Type, typename In2Type, typename Executor>
  requires is_cuda_executor_v<Executor> && gbfir_shim::routable_tensor<OutputTensor> &&
           gbfir_shim::routable_operand<In1Type> && gbfir_shim::routable_operand<In2Type>
__MATX_INLINE__ void corr_impl(OutputTensor o, const In1Type i1, const In2Type i2, matxConvCorrMode_t mode,
                               [[maybe_unused]] matxConvCorrMethod_t method, const Executor &exec) {
  MATX_NVTX_START("gbfir corr", matx::MATX_NVTX_LOG_API)
  if (gbfir_shim::conv_axis(o, i1, i2, mode, 1, exec)) return;
  gbfir_shim::Staged<OutputTensor, Executor> out(o, exec);
  gbfir_shim::Staged<In1Type, Executor> a(i1, exec);
  gbfir_shim::Staged<In2Type, Executor> b(i2, exec);
  gbfir_shim::check(gbfir_conv1d(out.buf, a.buf, b.buf, static_cast<int32_t>(mode), 1, GBFIR_PREC_FP32,
                                 gbfir_shim::stream_of(exec.getStream())));
  if (out.buf.ptr != static_cast<const void *>(o.Data())) (o = out.tmp).run(exec);
}

// ---- conv2d (direct) ------------------------------------------------------------------------
// Replaces transforms/conv.h:548-600 for CUDA executors: images of the last two dimensions,
// the leading ones folding into one batch stride (else MatX's elementwise copy into a
// contiguous temporary first); filters up to 64 x 64 (larger: MatX's kernel).
namespace gbfir_shim {
template <typename Op>
bool describe2d(const Op &t, gbfir_buf2d &b) {
  constexpr int R = remove_cvref_t<Op>::Rank();
  if constexpr (R < 2) {
    return false;
  } else {
    if (t.Size(R - 1) > 1 && t.Stride(R - 1) != 1) return false;
    index_t batch = 1;
    for (int i = 0; i < R - 2; i++) batch *= t.Size(i);
    index_t bstride = 0;
    int inner = -1;
    for (int i = R - 3; i >= 0; i--)
      if (t.Size(i) > 1) {
        inner = i;
        break;
      }
    if (inner >= 0) {
      bstride = t.Stride(inner);
      index_t expect = bstride * t.Size(inner);
      for (int i = inner - 1; i >= 0; i--) {
        if (t.Size(i) == 1) continue;
        if (t.Stride(i) != expect) return false;
        expect *= t.Size(i);
      }
    }
    b.ptr = const_cast<void *>(static_cast<const void *>(t.Data()));
    b.batch = batch;
    b.rows = t.Size(R - 2);
    b.cols = t.Size(R - 1);
    b.batch_stride = batch > 1 ? bstride : 0;
    b.row_stride = t.Size(R - 2) > 1 ? t.Stride(R - 2) : t.Size(R - 1);
    b.dtype = dtype_of<typename remove_cvref_t<Op>::value_type>();
    return true;
  }
}
template <typename Op, typename Executor>
struct Staged2d {
  using value_type = typename remove_cvref_t<Op>::value_type;
  static constexpr int R = remove_cvref_t<Op>::Rank();
  gbfir_buf2d buf{};
  decltype(make_tensor<value_type>(cuda::std::array<index_t, R>{}, MATX_ASYNC_DEVICE_MEMORY,
                                   cudaStream_t{})) tmp;
  Staged2d(const Op &t, const Executor &exec) {
    bool direct = false;
    if constexpr (is_tensor_view_v<remove_cvref_t<Op>>) direct = describe2d(t, buf);
    if (!direct) {
      cuda::std::array<index_t, R> shape;
      for (int i = 0; i < R; i++) shape[i] = t.Size(i);
      (void)(tmp = make_tensor<value_type>(shape, MATX_ASYNC_DEVICE_MEMORY, exec.getStream()));
      (tmp = t).run(exec);
      (void)describe2d(tmp, buf);
    }
  }
};
}  // namespace gbfir_shim

template <typename OutputType, typename In1Type, typename In2Type, typename Executor>
  requires is_cuda_executor_v<Executor> && gbfir_shim::routable_tensor<OutputType> &&
           gbfir_shim::routable_operand<In1Type> && gbfir_shim::routable_operand<In2Type> &&
           (remove_cvref_t<In1Type>::Rank() >= 2) && (remove_cvref_t<In2Type>::Rank() >= 2)
inline void conv2d_impl(OutputType o, const In1Type in1, const In2Type in2, matxConvCorrMode_t mode,
                        const Executor &exec) {
  MATX_NVTX_START("gbfir conv2d", matx::MATX_NVTX_LOG_API)
  constexpr int R1 = remove_cvref_t<In1Type>::Rank(), R2 = remove_cvref_t<In2Type>::Rank();
  const index_t n1 = in1.Size(R1 - 2) * in1.Size(R1 - 1), n2 = in2.Size(R2 - 2) * in2.Size(R2 - 1);
  const index_t fil_rows = n1 >= n2 ? in2.Size(R2 - 2) : in1.Size(R1 - 2);
  const index_t fil_cols = n1 >= n2 ? in2.Size(R2 - 1) : in1.Size(R1 - 1);
  if constexpr (R1 == R2) {
    // filters beyond the kernel's 64 x 64: MatX's own direct kernel (same operand order rule)
    if (fil_rows > 64 || fil_cols > 64) {
      if (n1 >= n2) detail::matxDirectConv2DInternal(o, in1, in2, mode, exec.getStream());
      else detail::matxDirectConv2DInternal(o, in2, in1, mode, exec.getStream());
      return;
    }
  }
  gbfir_shim::Staged2d<OutputType, Executor> out(o, exec);
  gbfir_shim::Staged2d<In1Type, Executor> a(in1, exec);
  gbfir_shim::Staged2d<In2Type, Executor> b(in2, exec);
  gbfir_shim::check(gbfir_conv2d(out.buf, a.buf, b.buf, static_cast<int32_t>(mode),
                                 gbfir_shim::stream_of(exec.getStream())));
  if (out.buf.ptr != static_cast<const void *>(o.Data())) (o = out.tmp).run(exec);
}

// ---- filter() --------------------------------------------------------------------------------
// Replaces transforms/filter.h:456-495: without recursive coefficients conv1d SAME
// (filter.h:185), else the recursive filter, with a workspace from MatX's allocator.
template <size_t NR, size_t NNR, typename OutType, typename InType, typename FilterType>
  requires gbfir_shim::routable_tensor<OutType> && gbfir_shim::routable_operand<InType> &&
           (gbfir_shim::dtype_of<FilterType>() >= 0) && (NR <= 4) && (NNR >= 1) && (NNR <= 4)
void filter_impl(OutType &o, const InType &i, const cuda::std::array<FilterType, NR> h_rec,
                 const cuda::std::array<FilterType, NNR> h_nonrec, const cudaExecutor &exec) {
  MATX_NVTX_START("gbfir filter", matx::MATX_NVTX_LOG_API)
  gbfir_shim::Staged<OutType, cudaExecutor> out(o, exec);
  gbfir_shim::Staged<InType, cudaExecutor> x(i, exec);
  const cudaStream_t stream = exec.getStream();
  void *ws = nullptr;
  size_t need = 0;
  if constexpr (NR > 0) {
    need = gbfir_filter_workspace_size(out.buf.batch, x.buf.len, out.buf.dtype);
    matxAlloc(&ws, need, MATX_ASYNC_DEVICE_MEMORY, stream);
  }
  const int rc = gbfir_filter(out.buf, x.buf, NR > 0 ? static_cast<const void *>(h_rec.data()) : nullptr,
                              static_cast<int32_t>(NR), h_nonrec.data(), static_cast<int32_t>(NNR),
                              gbfir_shim::dtype_of<FilterType>(), ws, need, gbfir_shim::stream_of(stream));
  if (ws != nullptr) matxFree(ws, stream);
  gbfir_shim::check(rc);
  if (out.buf.ptr != static_cast<const void *>(o.Data())) (o = out.tmp).run(exec);
}

// ---- channelize_poly ----------------------------------------------------------------------
// Replaces transforms/channelize_poly.h:724-849 (FIR + in-place cuFFT) with the fused kernel,
// for the default accumulator (the output's inner type).
template <typename OutType, typename InType, typename FilterType, typename AccumType>
  requires gbfir_shim::routable_tensor<OutType> && gbfir_shim::routable_operand<InType> &&
           gbfir_shim::routable_operand<FilterType> &&
           std::is_same_v<AccumType, typename inner_op_type_t<typename remove_cvref_t<OutType>::value_type>::type>
inline void channelize_poly_impl(OutType out, const InType &in, const FilterType &f, index_t num_channels,
                                 index_t decimation_factor, cudaStream_t stream) {
  MATX_NVTX_START("gbfir channelize_poly", matx::MATX_NVTX_LOG_API)
  constexpr int OR = remove_cvref_t<OutType>::Rank();
  static_assert(OR == remove_cvref_t<InType>::Rank() + 1, "channelize_poly: output rank should be 1 higher than input");
  cudaExecutor exec{stream};
  gbfir_shim::Staged<InType, cudaExecutor> x(in, exec);
  gbfir_shim::Staged<FilterType, cudaExecutor> h(f, exec);
  // the output [..., T, M] as rows of T*M elements; a contiguous temporary if it does not fold
  using OV = typename remove_cvref_t<OutType>::value_type;
  auto fold = [&](const auto &t, gbfir_buf &b) {
    if (t.Stride(OR - 1) != 1 || (t.Size(OR - 2) > 1 && t.Stride(OR - 2) != t.Size(OR - 1))) return false;
    index_t batch = 1;
    for (int i = 0; i < OR - 2; i++) batch *= t.Size(i);
    index_t bstride = t.Size(OR - 2) * t.Size(OR - 1), expect = bstride;
    bool first = true;
    for (int i = OR - 3; i >= 0; i--) {
      if (t.Size(i) == 1) continue;
      if (first) {
        bstride = t.Stride(i);
        if (bstride < t.Size(OR - 2) * t.Size(OR - 1)) return false;
        expect = bstride;
        first = false;
      } else if (t.Stride(i) != expect) {
        return false;
      }
      expect *= t.Size(i);
    }
    b.ptr = static_cast<void *>(t.Data());
    b.batch = batch;
    b.len = t.Size(OR - 2) * t.Size(OR - 1);
    b.batch_stride = batch > 1 ? bstride : 0;
    b.dtype = gbfir_shim::dtype_of<OV>();
    return true;
  };
  gbfir_buf ob{};
  if (fold(out, ob)) {
    gbfir_shim::check(gbfir_channelize_poly(ob, x.buf, h.buf, num_channels, decimation_factor, GBFIR_PREC_FP32,
                                            gbfir_shim::stream_of(stream)));
  } else {
    auto tmp = make_tensor<OV>(out.Shape(), MATX_ASYNC_DEVICE_MEMORY, stream);
    (void)fold(tmp, ob);
    gbfir_shim::check(gbfir_channelize_poly(ob, x.buf, h.buf, num_channels, decimation_factor, GBFIR_PREC_FP32,
                                            gbfir_shim::stream_of(stream)));
    (out = tmp).run(exec);
  }
}

}  // namespace matx
