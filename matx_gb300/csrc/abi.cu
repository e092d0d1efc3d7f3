// abi.cu — the extern "C" boundary of libgbfir (include/gbfir.h).
//
// Every entry point validates its arguments with the same rules (and the same
// error classes) as the MatX transform it replaces, then enqueues kernels on the
// caller's stream.  No exception crosses the boundary.
#include <cuda_runtime.h>

#include <mutex>
#include <numeric>
#include <string>
#include <unordered_map>

#include "common.cuh"

namespace gbfir {

int conv1d_fp(const gbfir_buf &out, const gbfir_buf &in, const gbfir_buf &h, int mode, int is_corr, cudaStream_t s);
int conv1d_axis_fp(const gbfir_buf &out, const gbfir_buf &in, const gbfir_buf &h, int64_t inner, int64_t in_step,
                   int64_t out_step, int mode, int is_corr, cudaStream_t s);
int updown_fp(const gbfir_buf &out, const gbfir_buf &in, int64_t n, bool up, cudaStream_t s);
int conv2d_fp(const gbfir_buf2d &out, const gbfir_buf2d &x, const gbfir_buf2d &h, int mode, cudaStream_t s);
int conv1d_fft_fp(const gbfir_buf &out, const gbfir_buf &in, const gbfir_buf &h, int mode, int is_corr,
                  cudaStream_t s);
size_t filter_workspace_bytes(int64_t batch, int64_t len, int32_t out_dtype);
int filter_fp(const gbfir_buf &out, const gbfir_buf &in, const void *a, int na, const void *b, int nb,
              int32_t coef_dtype, void *workspace, cudaStream_t s);
int upfirdn_fp(const gbfir_buf &out, const gbfir_buf &in, const gbfir_buf &h, int64_t up, int64_t down, int mode,
               cudaStream_t s);
int resample_poly_fp(const gbfir_buf &out, const gbfir_buf &in, const gbfir_buf &h, int64_t up, int64_t down,
                     cudaStream_t s);
int channelize_poly_fp(const gbfir_buf &out, const gbfir_buf &in, const gbfir_buf &h, int64_t M, int64_t D,
                       cudaStream_t s);
int resample_poly_tc(const gbfir_buf &out, const gbfir_buf &in, const gbfir_buf &h, int64_t up, int64_t down,
                     int precision, cudaStream_t s);
int channelize_poly_tc(const gbfir_buf &out, const gbfir_buf &in, const gbfir_buf &h, int64_t M, int64_t D,
                       int precision, cudaStream_t s);
int conv1d_tc(const gbfir_buf &out, const gbfir_buf &in, const gbfir_buf &h, int mode, int is_corr, int precision,
              cudaStream_t s);
int set_resample_tile(int rq, int wc, int group, int nbuf);
int register_resample_tile(int64_t up, int64_t down, int64_t L, int rq, int wc, int group, int nbuf);
int clear_resample_tiles();

static thread_local std::string t_last_error;
static std::atomic<uint64_t> g_launches{0};

void set_error(const std::string &msg) { t_last_error = msg; }
void count_launch(uint64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

int num_sms() {
  static std::mutex mu;
  static std::unordered_map<int, int> cache;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(mu);
  auto it = cache.find(dev);
  if (it != cache.end()) return it->second;
  int n = 0;
  cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
  if (n <= 0) n = 1;
  cache[dev] = n;
  return n;
}

int ensure_smem(const void *func, size_t bytes, const char *what) {
  static std::mutex mu;
  static std::unordered_map<uint64_t, size_t> done;  // (device, func) -> bytes granted
  int dev = 0;
  cudaGetDevice(&dev);
  const uint64_t key = (reinterpret_cast<uint64_t>(func) << 4) ^ (uint64_t)dev;
  {
    std::lock_guard<std::mutex> lk(mu);
    auto it = done.find(key);
    if (it != done.end() && it->second >= bytes) return GBFIR_SUCCESS;
  }
  if (bytes > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e != cudaSuccess) {
      char buf[256];
      snprintf(buf, sizeof(buf), "%s: cannot reserve %zu B of shared memory: %s", what, bytes, cudaGetErrorString(e));
      set_error(buf);
      return GBFIR_ERR_CUDA;
    }
  }
  std::lock_guard<std::mutex> lk(mu);
  done[key] = bytes;
  return GBFIR_SUCCESS;
}

int check_buf(const gbfir_buf &b, const char *name, bool allow_broadcast) {
  if (b.ptr == nullptr) GBFIR_FAIL(GBFIR_ERR_NULL_POINTER, "%s: null pointer", name);
  const size_t es = dtype_size(b.dtype);
  if (es == 0) GBFIR_FAIL(GBFIR_ERR_INVALID_TYPE, "%s: unknown dtype %d", name, (int)b.dtype);
  if (b.batch < 1) GBFIR_FAIL(GBFIR_ERR_INVALID_DIM, "%s: batch must be >= 1 (got %lld)", name, (long long)b.batch);
  if (b.len < 1) GBFIR_FAIL(GBFIR_ERR_INVALID_SIZE, "%s: length must be >= 1 (got %lld)", name, (long long)b.len);
  const size_t align = (b.dtype == GBFIR_C128) ? 16 : es;
  if (reinterpret_cast<uintptr_t>(b.ptr) % align)
    GBFIR_FAIL(GBFIR_ERR_ALIGNMENT, "%s: pointer not aligned to %zu bytes", name, align);
  if (b.batch > 1) {
    if (b.batch_stride < 0) GBFIR_FAIL(GBFIR_ERR_INVALID_PARAMETER, "%s: negative batch stride", name);
    if (b.batch_stride == 0 && !allow_broadcast)
      GBFIR_FAIL(GBFIR_ERR_INVALID_PARAMETER, "%s: zero batch stride is only allowed for inputs", name);
    if (b.batch_stride != 0 && b.batch_stride < b.len)
      GBFIR_FAIL(GBFIR_ERR_INVALID_PARAMETER, "%s: batch stride %lld shorter than a row (%lld)", name,
                 (long long)b.batch_stride, (long long)b.len);
  }
  return GBFIR_SUCCESS;
}

// Output dtype rule: complex if either operand is complex, same precision as the inputs.
static int check_types(const gbfir_buf &out, const gbfir_buf &in, const gbfir_buf &h, const char *what,
                       bool out_always_complex) {
  if (dtype_double(in.dtype) != dtype_double(h.dtype) || dtype_double(in.dtype) != dtype_double(out.dtype))
    GBFIR_FAIL(GBFIR_ERR_INVALID_TYPE, "%s: operands must all be single or all be double precision", what);
  const bool oc = out_always_complex || dtype_complex(in.dtype) || dtype_complex(h.dtype);
  if (dtype_complex(out.dtype) != oc)
    GBFIR_FAIL(GBFIR_ERR_INVALID_TYPE, "%s: output must be %s", what, oc ? "complex" : "real");
  return GBFIR_SUCCESS;
}

static int check_precision(int32_t precision, const char *what) {
  if (precision < GBFIR_PREC_FP32 || precision > GBFIR_PREC_BF16X3)
    GBFIR_FAIL(GBFIR_ERR_INVALID_PARAMETER, "%s: unknown precision %d", what, (int)precision);
  return GBFIR_SUCCESS;
}

}  // namespace gbfir

using namespace gbfir;

#define GBFIR_TRY(expr)        \
  do {                         \
    int _rc = (expr);          \
    if (_rc) return _rc;       \
  } while (0)

extern "C" {

int gbfir_conv1d(gbfir_buf out, gbfir_buf in, gbfir_buf h, int32_t mode, int32_t is_corr, int32_t precision,
                 gbfir_stream_t stream) {
  try {
    GBFIR_TRY(check_buf(out, "conv1d out", false));
    GBFIR_TRY(check_buf(in, "conv1d in", true));
    GBFIR_TRY(check_buf(h, "conv1d h", true));
    GBFIR_TRY(check_types(out, in, h, "conv1d", false));
    GBFIR_TRY(check_precision(precision, "conv1d"));
    if (mode < GBFIR_MODE_FULL || mode > GBFIR_MODE_VALID)
      GBFIR_FAIL(GBFIR_ERR_INVALID_PARAMETER, "conv1d: unknown mode %d", (int)mode);
    // batch rule of conv1d_impl (conv.h:467-532): each operand is one row or out.batch rows
    if ((in.batch != 1 && in.batch != out.batch) || (h.batch != 1 && h.batch != out.batch))
      GBFIR_FAIL(GBFIR_ERR_INVALID_DIM, "conv1d: batch sizes do not match (out %lld, in %lld, h %lld)",
                 (long long)out.batch, (long long)in.batch, (long long)h.batch);
    const int64_t mx = std::max(in.len, h.len), mn = std::min(in.len, h.len);
    const int64_t want = mode == GBFIR_MODE_FULL ? in.len + h.len - 1 : mode == GBFIR_MODE_SAME ? mx : mx - mn + 1;
    if (out.len != want)
      GBFIR_FAIL(GBFIR_ERR_INVALID_SIZE, "conv1d: output length %lld, expected %lld", (long long)out.len,
                 (long long)want);
    if (precision != GBFIR_PREC_FP32)
      return conv1d_tc(out, in, h, mode, is_corr != 0, precision, reinterpret_cast<cudaStream_t>(stream));
    return conv1d_fp(out, in, h, mode, is_corr != 0, reinterpret_cast<cudaStream_t>(stream));
  } catch (...) {
    GBFIR_FAIL(GBFIR_ERR_CUDA, "conv1d: internal exception");
  }
}

int gbfir_conv1d_axis(gbfir_buf out, gbfir_buf in, gbfir_buf h, int64_t inner, int64_t in_step, int64_t out_step,
                      int32_t mode, int32_t is_corr, int32_t precision, gbfir_stream_t stream) {
  try {
    GBFIR_TRY(check_buf(h, "conv1d (axis) h", false));
    if (out.ptr == nullptr || in.ptr == nullptr) GBFIR_FAIL(GBFIR_ERR_NULL_POINTER, "conv1d (axis): null pointer");
    if (out.batch < 1 || in.batch < 1) GBFIR_FAIL(GBFIR_ERR_INVALID_DIM, "conv1d (axis): batch must be >= 1");
    if (out.len < 1 || in.len < 1) GBFIR_FAIL(GBFIR_ERR_INVALID_SIZE, "conv1d (axis): lengths must be >= 1");
    if (dtype_size(out.dtype) == 0 || dtype_size(in.dtype) == 0)
      GBFIR_FAIL(GBFIR_ERR_INVALID_TYPE, "conv1d (axis): unknown dtype");
    GBFIR_TRY(check_types(out, in, h, "conv1d (axis)", false));
    GBFIR_TRY(check_precision(precision, "conv1d (axis)"));
    if (precision != GBFIR_PREC_FP32)
      GBFIR_FAIL(GBFIR_ERR_NOT_SUPPORTED, "conv1d (axis): only the FP32/FP64 form is built");
    if (mode < GBFIR_MODE_FULL || mode > GBFIR_MODE_VALID)
      GBFIR_FAIL(GBFIR_ERR_INVALID_PARAMETER, "conv1d (axis): unknown mode %d", (int)mode);
    if (inner < 1) GBFIR_FAIL(GBFIR_ERR_INVALID_PARAMETER, "conv1d (axis): inner count must be >= 1");
    if (in_step < 1 || out_step < 1)
      GBFIR_FAIL(GBFIR_ERR_INVALID_PARAMETER, "conv1d (axis): sample steps must be >= 1");
    if (h.batch != 1) GBFIR_FAIL(GBFIR_ERR_INVALID_DIM, "conv1d (axis): the filter must be one row");
    if (in.batch != 1 && in.batch != out.batch)
      GBFIR_FAIL(GBFIR_ERR_INVALID_DIM, "conv1d (axis): batch sizes do not match (out %lld, in %lld)",
                 (long long)out.batch, (long long)in.batch);
    // output signals must not overlap: inner positions within one step, blocks apart
    if (inner > 1 && out.len > 1 && out_step < inner)
      GBFIR_FAIL(GBFIR_ERR_INVALID_PARAMETER, "conv1d (axis): output step %lld below the inner count %lld",
                 (long long)out_step, (long long)inner);
    if (out.batch > 1 && out.batch_stride < (out.len - 1) * out_step + inner)
      GBFIR_FAIL(GBFIR_ERR_INVALID_PARAMETER, "conv1d (axis): output batch stride shorter than a block");
    if (in.batch > 1 && in.batch_stride < 0)
      GBFIR_FAIL(GBFIR_ERR_INVALID_PARAMETER, "conv1d (axis): negative input batch stride");
    const size_t ia = in.dtype == GBFIR_C128 ? 16 : dtype_size(in.dtype);
    const size_t oa = out.dtype == GBFIR_C128 ? 16 : dtype_size(out.dtype);
    if (reinterpret_cast<uintptr_t>(in.ptr) % ia || reinterpret_cast<uintptr_t>(out.ptr) % oa)
      GBFIR_FAIL(GBFIR_ERR_ALIGNMENT, "conv1d (axis): pointer not aligned to its element type");
    const int64_t mx = std::max(in.len, h.len), mn = std::min(in.len, h.len);
    const int64_t want = mode == GBFIR_MODE_FULL ? in.len + h.len - 1 : mode == GBFIR_MODE_SAME ? mx : mx - mn + 1;
    if (out.len != want)
      GBFIR_FAIL(GBFIR_ERR_INVALID_SIZE, "conv1d (axis): output length %lld, expected %lld", (long long)out.len,
                 (long long)want);
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    return conv1d_axis_fp(out, in, h, inner, in_step, out_step, mode, is_corr != 0, s);
  } catch (...) {
    GBFIR_FAIL(GBFIR_ERR_CUDA, "conv1d (axis): internal exception");
  }
}

size_t gbfir_filter_workspace_size(int64_t batch, int64_t len, int32_t out_dtype) {
  if (batch < 1 || len < 1 || dtype_size(out_dtype) == 0) return 0;
  return filter_workspace_bytes(batch, len, out_dtype);
}

int gbfir_filter(gbfir_buf out, gbfir_buf in, const void *h_rec, int32_t num_rec, const void *h_nonrec,
                 int32_t num_nonrec, int32_t coef_dtype, void *workspace, size_t workspace_bytes,
                 gbfir_stream_t stream) {
  try {
    GBFIR_TRY(check_buf(out, "filter out", false));
    GBFIR_TRY(check_buf(in, "filter in", true));
    if (dtype_size(coef_dtype) == 0) GBFIR_FAIL(GBFIR_ERR_INVALID_TYPE, "filter: unknown coefficient dtype");
    if (dtype_double(in.dtype) != dtype_double(out.dtype) || dtype_double(in.dtype) != dtype_double(coef_dtype))
      GBFIR_FAIL(GBFIR_ERR_INVALID_TYPE, "filter: operands must all be single or all be double precision");
    const bool oc = dtype_complex(in.dtype) || dtype_complex(coef_dtype);
    if (dtype_complex(out.dtype) != oc)
      GBFIR_FAIL(GBFIR_ERR_INVALID_TYPE, "filter: output must be %s", oc ? "complex" : "real");
    if (num_rec < 0 || num_nonrec < 1)
      GBFIR_FAIL(GBFIR_ERR_INVALID_PARAMETER, "filter: need >= 0 recursive and >= 1 non-recursive coefficients");
    if (num_rec > 4 || num_nonrec > 4)
      GBFIR_FAIL(GBFIR_ERR_NOT_SUPPORTED, "filter: at most 4 recursive and 4 non-recursive coefficients");
    if ((num_rec > 0 && h_rec == nullptr) || h_nonrec == nullptr)
      GBFIR_FAIL(GBFIR_ERR_NULL_POINTER, "filter: null coefficient array");
    if (in.batch != 1 && in.batch != out.batch)
      GBFIR_FAIL(GBFIR_ERR_INVALID_DIM, "filter: batch sizes do not match (out %lld, in %lld)",
                 (long long)out.batch, (long long)in.batch);
    if (out.len != in.len)
      GBFIR_FAIL(GBFIR_ERR_INVALID_SIZE, "filter: output length %lld, expected %lld", (long long)out.len,
                 (long long)in.len);
    if (num_rec == 0 && in.len < num_nonrec)
      GBFIR_FAIL(GBFIR_ERR_INVALID_SIZE, "filter: FIR-only filter (conv1d SAME) needs len >= %d", (int)num_nonrec);
    if (num_rec > 0) {
      if (out.batch > 65535) GBFIR_FAIL(GBFIR_ERR_NOT_SUPPORTED, "filter: at most 65535 rows per call");
      const size_t need = filter_workspace_bytes(out.batch, in.len, out.dtype);
      if (workspace == nullptr || workspace_bytes < need)
        GBFIR_FAIL(GBFIR_ERR_WORKSPACE, "filter: workspace of %zu bytes needed", need);
      if (reinterpret_cast<uintptr_t>(workspace) % 16)
        GBFIR_FAIL(GBFIR_ERR_ALIGNMENT, "filter: workspace not 16-byte aligned");
    }
    return filter_fp(out, in, h_rec, num_rec, h_nonrec, num_nonrec, coef_dtype, workspace,
                     reinterpret_cast<cudaStream_t>(stream));
  } catch (...) {
    GBFIR_FAIL(GBFIR_ERR_CUDA, "filter: internal exception");
  }
}

static int check_buf2d(const gbfir_buf2d &b, const char *name, bool allow_broadcast) {
  if (b.ptr == nullptr) GBFIR_FAIL(GBFIR_ERR_NULL_POINTER, "%s: null pointer", name);
  const size_t es = dtype_size(b.dtype);
  if (es == 0) GBFIR_FAIL(GBFIR_ERR_INVALID_TYPE, "%s: unknown dtype %d", name, (int)b.dtype);
  if (b.batch < 1) GBFIR_FAIL(GBFIR_ERR_INVALID_DIM, "%s: batch must be >= 1", name);
  if (b.rows < 1 || b.cols < 1) GBFIR_FAIL(GBFIR_ERR_INVALID_SIZE, "%s: empty image", name);
  const size_t align = (b.dtype == GBFIR_C128) ? 16 : es;
  if (reinterpret_cast<uintptr_t>(b.ptr) % align)
    GBFIR_FAIL(GBFIR_ERR_ALIGNMENT, "%s: pointer not aligned to %zu bytes", name, align);
  if (b.rows > 1 && b.row_stride < b.cols)
    GBFIR_FAIL(GBFIR_ERR_INVALID_PARAMETER, "%s: row stride shorter than a row", name);
  if (b.batch > 1 && b.batch_stride == 0 && !allow_broadcast)
    GBFIR_FAIL(GBFIR_ERR_INVALID_PARAMETER, "%s: zero batch stride is only allowed for inputs", name);
  if (b.batch > 1 && b.batch_stride != 0 && b.batch_stride < (b.rows - 1) * b.row_stride + b.cols)
    GBFIR_FAIL(GBFIR_ERR_INVALID_PARAMETER, "%s: batch stride shorter than an image", name);
  return GBFIR_SUCCESS;
}

int gbfir_conv2d(gbfir_buf2d out, gbfir_buf2d in, gbfir_buf2d h, int32_t mode, gbfir_stream_t stream) {
  try {
    GBFIR_TRY(check_buf2d(out, "conv2d out", false));
    GBFIR_TRY(check_buf2d(in, "conv2d in", true));
    GBFIR_TRY(check_buf2d(h, "conv2d h", true));
    if (dtype_double(in.dtype) != dtype_double(h.dtype) || dtype_double(in.dtype) != dtype_double(out.dtype))
      GBFIR_FAIL(GBFIR_ERR_INVALID_TYPE, "conv2d: operands must all be single or all be double precision");
    const bool oc = dtype_complex(in.dtype) || dtype_complex(h.dtype);
    if (dtype_complex(out.dtype) != oc)
      GBFIR_FAIL(GBFIR_ERR_INVALID_TYPE, "conv2d: output must be %s", oc ? "complex" : "real");
    if (mode < GBFIR_MODE_FULL || mode > GBFIR_MODE_VALID)
      GBFIR_FAIL(GBFIR_ERR_INVALID_PARAMETER, "conv2d: unknown mode %d", (int)mode);
    if ((in.batch != 1 && in.batch != out.batch) || (h.batch != 1 && h.batch != out.batch))
      GBFIR_FAIL(GBFIR_ERR_INVALID_DIM, "conv2d: batch sizes do not match");
    auto size = [&](int64_t a, int64_t b) {
      const int64_t mx = std::max(a, b), mn = std::min(a, b);
      return mode == GBFIR_MODE_FULL ? a + b - 1 : mode == GBFIR_MODE_SAME ? mx : mx - mn + 1;
    };
    if (out.rows != size(in.rows, h.rows) || out.cols != size(in.cols, h.cols))
      GBFIR_FAIL(GBFIR_ERR_INVALID_SIZE, "conv2d: output %lld x %lld, expected %lld x %lld", (long long)out.rows,
                 (long long)out.cols, (long long)size(in.rows, h.rows), (long long)size(in.cols, h.cols));
    // the operand with more elements is the image (transforms/conv.h:569-576)
    const bool swap = in.rows * in.cols < h.rows * h.cols;
    const gbfir_buf2d &img = swap ? h : in, &fil = swap ? in : h;
    if (fil.rows > img.rows || fil.cols > img.cols)
      GBFIR_FAIL(GBFIR_ERR_NOT_SUPPORTED, "conv2d: the filter must fit inside the image along both axes");
    return conv2d_fp(out, img, fil, mode, reinterpret_cast<cudaStream_t>(stream));
  } catch (...) {
    GBFIR_FAIL(GBFIR_ERR_CUDA, "conv2d: internal exception");
  }
}

int gbfir_conv1d_fft(gbfir_buf out, gbfir_buf in, gbfir_buf h, int32_t mode, int32_t is_corr,
                     gbfir_stream_t stream) {
  try {
    GBFIR_TRY(check_buf(out, "conv1d (FFT) out", false));
    GBFIR_TRY(check_buf(in, "conv1d (FFT) in", true));
    GBFIR_TRY(check_buf(h, "conv1d (FFT) h", false));
    GBFIR_TRY(check_types(out, in, h, "conv1d (FFT)", false));
    if (dtype_double(in.dtype))
      GBFIR_FAIL(GBFIR_ERR_NOT_SUPPORTED, "conv1d (FFT): float32 / complex64 operands only");
    if (mode < GBFIR_MODE_FULL || mode > GBFIR_MODE_VALID)
      GBFIR_FAIL(GBFIR_ERR_INVALID_PARAMETER, "conv1d (FFT): unknown mode %d", (int)mode);
    if (h.batch != 1) GBFIR_FAIL(GBFIR_ERR_NOT_SUPPORTED, "conv1d (FFT): the filter must be one row");
    if (in.batch != 1 && in.batch != out.batch)
      GBFIR_FAIL(GBFIR_ERR_INVALID_DIM, "conv1d (FFT): batch sizes do not match (out %lld, in %lld)",
                 (long long)out.batch, (long long)in.batch);
    if (in.len < h.len) GBFIR_FAIL(GBFIR_ERR_NOT_SUPPORTED, "conv1d (FFT): the signal must be at least as long as the filter");
    if (h.len > GBFIR_FFT_CONV_MAX_TAPS)
      GBFIR_FAIL(GBFIR_ERR_NOT_SUPPORTED, "conv1d (FFT): at most %d taps", (int)GBFIR_FFT_CONV_MAX_TAPS);
    const int64_t want = mode == GBFIR_MODE_FULL ? in.len + h.len - 1 : mode == GBFIR_MODE_SAME ? in.len
                                                                      : in.len - h.len + 1;
    if (out.len != want)
      GBFIR_FAIL(GBFIR_ERR_INVALID_SIZE, "conv1d (FFT): output length %lld, expected %lld", (long long)out.len,
                 (long long)want);
    return conv1d_fft_fp(out, in, h, mode, is_corr != 0, reinterpret_cast<cudaStream_t>(stream));
  } catch (...) {
    GBFIR_FAIL(GBFIR_ERR_CUDA, "conv1d (FFT): internal exception");
  }
}

static int updown_entry(gbfir_buf out, gbfir_buf in, int64_t n, bool up, gbfir_stream_t stream) {
  const char *what = up ? "upsample" : "downsample";
  GBFIR_TRY(check_buf(out, what, false));
  GBFIR_TRY(check_buf(in, what, true));
  if (out.dtype != in.dtype) GBFIR_FAIL(GBFIR_ERR_INVALID_TYPE, "%s: input and output types differ", what);
  if (n < 1) GBFIR_FAIL(GBFIR_ERR_INVALID_PARAMETER, "%s: the rate must be >= 1", what);
  if (in.batch != 1 && in.batch != out.batch)
    GBFIR_FAIL(GBFIR_ERR_INVALID_DIM, "%s: batch sizes do not match (out %lld, in %lld)", what,
               (long long)out.batch, (long long)in.batch);
  const int64_t want = up ? in.len * n : (in.len + n - 1) / n;
  if (out.len != want)
    GBFIR_FAIL(GBFIR_ERR_INVALID_SIZE, "%s: output length %lld, expected %lld", what, (long long)out.len,
               (long long)want);
  return updown_fp(out, in, n, up, reinterpret_cast<cudaStream_t>(stream));
}

int gbfir_upsample(gbfir_buf out, gbfir_buf in, int64_t n, gbfir_stream_t stream) {
  try {
    return updown_entry(out, in, n, true, stream);
  } catch (...) {
    GBFIR_FAIL(GBFIR_ERR_CUDA, "upsample: internal exception");
  }
}

int gbfir_downsample(gbfir_buf out, gbfir_buf in, int64_t n, gbfir_stream_t stream) {
  try {
    return updown_entry(out, in, n, false, stream);
  } catch (...) {
    GBFIR_FAIL(GBFIR_ERR_CUDA, "downsample: internal exception");
  }
}

int gbfir_upfirdn(gbfir_buf out, gbfir_buf in, gbfir_buf h, int64_t up, int64_t down, int32_t mode, int32_t precision,
                  gbfir_stream_t stream) {
  try {
    GBFIR_TRY(check_buf(out, "upfirdn out", false));
    GBFIR_TRY(check_buf(in, "upfirdn in", true));
    GBFIR_TRY(check_buf(h, "upfirdn h", false));
    GBFIR_TRY(check_types(out, in, h, "upfirdn", false));
    GBFIR_TRY(check_precision(precision, "upfirdn"));
    if (precision != GBFIR_PREC_FP32)
      GBFIR_FAIL(GBFIR_ERR_NOT_SUPPORTED, "upfirdn: only the FP32/FP64 form is built");
    if (up < 1 || down < 1) GBFIR_FAIL(GBFIR_ERR_INVALID_PARAMETER, "upfirdn: up and down must be >= 1");
    if (mode < GBFIR_MODE_FULL || mode > GBFIR_MODE_VALID)
      GBFIR_FAIL(GBFIR_ERR_INVALID_PARAMETER, "upfirdn: unknown mode %d", (int)mode);
    if (h.batch != 1) GBFIR_FAIL(GBFIR_ERR_INVALID_DIM, "upfirdn: the filter must be one row");
    if (in.batch != 1 && in.batch != out.batch)
      GBFIR_FAIL(GBFIR_ERR_INVALID_DIM, "upfirdn: batch sizes do not match (out %lld, in %lld)",
                 (long long)out.batch, (long long)in.batch);
    const int64_t Nu = in.len * up;
    const int64_t mx = std::max(Nu, h.len), mn = std::min(Nu, h.len);
    const int64_t clen = mode == GBFIR_MODE_FULL ? Nu + h.len - 1 : mode == GBFIR_MODE_SAME ? mx : mx - mn + 1;
    const int64_t want = (clen + down - 1) / down;
    if (out.len != want)
      GBFIR_FAIL(GBFIR_ERR_INVALID_SIZE, "upfirdn: output length %lld, expected %lld", (long long)out.len,
                 (long long)want);
    return upfirdn_fp(out, in, h, up, down, mode, reinterpret_cast<cudaStream_t>(stream));
  } catch (...) {
    GBFIR_FAIL(GBFIR_ERR_CUDA, "upfirdn: internal exception");
  }
}

int gbfir_resample_poly(gbfir_buf out, gbfir_buf in, gbfir_buf h, int64_t up, int64_t down, int32_t precision,
                        gbfir_stream_t stream) {
  try {
    GBFIR_TRY(check_buf(out, "resample_poly out", false));
    GBFIR_TRY(check_buf(in, "resample_poly in", false));
    GBFIR_TRY(check_buf(h, "resample_poly h", false));
    GBFIR_TRY(check_types(out, in, h, "resample_poly", false));
    GBFIR_TRY(check_precision(precision, "resample_poly"));
    if (up <= 0) GBFIR_FAIL(GBFIR_ERR_INVALID_PARAMETER, "resample_poly: up must be positive");
    if (down <= 0) GBFIR_FAIL(GBFIR_ERR_INVALID_PARAMETER, "resample_poly: down must be positive");
    if (h.batch != 1) GBFIR_FAIL(GBFIR_ERR_INVALID_DIM, "resample_poly: the filter must be one row");
    if (out.batch != in.batch)
      GBFIR_FAIL(GBFIR_ERR_INVALID_DIM, "resample_poly: input/output must have matched batch sizes");
    const int64_t up_size = in.len * up;
    const int64_t outlen = up_size / down + ((up_size % down) ? 1 : 0);
    if (out.len != outlen)
      GBFIR_FAIL(GBFIR_ERR_INVALID_DIM, "resample_poly: output size mismatch (%lld, expected %lld)",
                 (long long)out.len, (long long)outlen);
    const int64_t g = std::gcd(up, down);
    up /= g;
    down /= g;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (precision == GBFIR_PREC_FP32 || (up == 1 && down == 1)) return resample_poly_fp(out, in, h, up, down, s);
    return resample_poly_tc(out, in, h, up, down, precision, s);
  } catch (...) {
    GBFIR_FAIL(GBFIR_ERR_CUDA, "resample_poly: internal exception");
  }
}

int gbfir_channelize_poly(gbfir_buf out, gbfir_buf in, gbfir_buf h, int64_t M, int64_t D, int32_t precision,
                          gbfir_stream_t stream) {
  try {
    GBFIR_TRY(check_buf(out, "channelize_poly out", false));
    GBFIR_TRY(check_buf(in, "channelize_poly in", false));
    GBFIR_TRY(check_buf(h, "channelize_poly h", false));
    GBFIR_TRY(check_types(out, in, h, "channelize_poly", true));
    GBFIR_TRY(check_precision(precision, "channelize_poly"));
    if (M <= 0) GBFIR_FAIL(GBFIR_ERR_INVALID_PARAMETER, "channelize_poly: num_channels must be positive");
    if (D <= 0) GBFIR_FAIL(GBFIR_ERR_INVALID_PARAMETER, "channelize_poly: decimation_factor must be positive");
    if (D > M) GBFIR_FAIL(GBFIR_ERR_INVALID_PARAMETER, "channelize_poly: decimation_factor must be <= num_channels");
    if (h.batch != 1) GBFIR_FAIL(GBFIR_ERR_INVALID_DIM, "channelize_poly: currently only support 1D filters");
    if (out.batch != in.batch)
      GBFIR_FAIL(GBFIR_ERR_INVALID_DIM, "channelize_poly: input/output must have matched batch sizes");
    const int64_t T = (in.len + D - 1) / D;
    if (out.len != T * M)
      GBFIR_FAIL(GBFIR_ERR_INVALID_DIM, "channelize_poly: output row must hold T*M = %lld elements (got %lld)",
                 (long long)(T * M), (long long)out.len);
    if (precision != GBFIR_PREC_FP32)
      return channelize_poly_tc(out, in, h, M, D, precision, reinterpret_cast<cudaStream_t>(stream));
    return channelize_poly_fp(out, in, h, M, D, reinterpret_cast<cudaStream_t>(stream));
  } catch (...) {
    GBFIR_FAIL(GBFIR_ERR_CUDA, "channelize_poly: internal exception");
  }
}

int gbfir_set_resample_tile(int32_t rows_per_thread, int32_t col_warps, int32_t group, int32_t buffers) {
  int rc = set_resample_tile(rows_per_thread, col_warps, group, buffers);
  if (rc)
    GBFIR_FAIL(rc, "set_resample_tile: invalid tile (%d, %d, %d, %d)", rows_per_thread, col_warps, group, buffers);
  return rc;
}

int gbfir_resample_tile_register(int64_t up, int64_t down, int64_t h_len, int32_t rows_per_thread, int32_t col_warps,
                                 int32_t group, int32_t buffers) {
  int rc = register_resample_tile(up, down, h_len, rows_per_thread, col_warps, group, buffers);
  if (rc) GBFIR_FAIL(rc, "resample_tile_register: invalid tile");
  return rc;
}

int gbfir_resample_tile_clear(void) { return clear_resample_tiles(); }

uint64_t gbfir_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

const char *gbfir_status_string(int status) {
  switch (status) {
    case GBFIR_SUCCESS: return "success";
    case GBFIR_ERR_INVALID_PARAMETER: return "invalid parameter";
    case GBFIR_ERR_INVALID_DIM: return "invalid dimension";
    case GBFIR_ERR_INVALID_SIZE: return "invalid size";
    case GBFIR_ERR_INVALID_TYPE: return "invalid type";
    case GBFIR_ERR_NOT_SUPPORTED: return "not supported";
    case GBFIR_ERR_CUDA: return "CUDA error";
    case GBFIR_ERR_NULL_POINTER: return "null pointer";
    case GBFIR_ERR_ALIGNMENT: return "misaligned pointer";
    case GBFIR_ERR_WORKSPACE: return "workspace missing or too small";
    case GBFIR_ERR_TIMEOUT: return "device wait timed out";
    default: return "unknown status";
  }
}

const char *gbfir_last_error(void) { return t_last_error.c_str(); }

int gbfir_version(void) { return 100; }

}  // extern "C"
