/*
 * gbfir.h — C ABI of the GB300 (sm_103a) direct-FIR library.
 *
 * This is the drop-in boundary for MatX's direct-FIR operators.  Each entry
 * point replaces the CUDA branch of one MatX transform (the L4 dispatcher
 * plus its L5 kernel) and keeps that transform's argument meaning, shape
 * rules and error classes:
 *
 *   gbfir_conv1d           include/matx/transforms/conv.h:467-532 (conv1d_impl)
 *                          include/matx/transforms/conv.h:402-451 (operand swap)
 *                          include/matx/transforms/conv.h:175-224 (direct CUDA path)
 *                          include/matx/transforms/corr.h:60-69   (corr = conv with reverse(conj(h)))
 *   gbfir_conv1d_fft       include/matx/transforms/conv.h:51-172 (the FFT method)
 *   gbfir_conv2d           include/matx/transforms/conv.h:548-600 (conv2d_impl, direct)
 *   gbfir_conv1d_axis      include/matx/operators/conv.h:263-274 (conv1d with an axis)
 *   gbfir_upsample / gbfir_downsample   include/matx/operators/updownsample.h:254-279
 *   gbfir_upfirdn          downsample(conv1d(upsample(.)), .) of the same operators
 *   gbfir_filter           include/matx/transforms/filter.h:159-188 (filter(): FIR-only
 *                          conv1d SAME, or the recursive filter of kernels/filter.cuh:44)
 *   gbfir_resample_poly    include/matx/transforms/resample_poly.h:299-354 (resample_poly_impl)
 *                          include/matx/transforms/resample_poly.h:64-210  (CUDA dispatcher)
 *   gbfir_channelize_poly  include/matx/transforms/channelize_poly.h:724-849 (CUDA impl incl. the
 *                          cuFFT ifft(FFTNorm::FORWARD) pass at :846, fused here)
 *
 * Entry points with no MatX counterpart (adjoints, ragged batches, plans) say
 * so in their comment.
 *
 * Conventions
 *  - Plain C.  No exception crosses the boundary; every function returns a
 *    gbfir_status.  gbfir_last_error() gives a human-readable message for the
 *    most recent failure on the calling thread.
 *  - All device pointers are caller-owned and must stay valid until the work
 *    enqueued on `stream` has completed.  Nothing here allocates device memory
 *    unless an entry point says so.
 *  - Every launch is enqueued on the given stream and returns asynchronously,
 *    exactly like MatX's cudaExecutor path.
 *  - A gbfir_buf describes a batch of 1-D rows: `batch` rows of `len`
 *    elements, row r starting at ptr + r*batch_stride elements.  A row count of
 *    1 or a batch_stride of 0 broadcasts one row over the batch (MatX's
 *    clone<>() of a lower-rank operand, conv.h:467-532).  The innermost
 *    dimension is always unit-stride; MatX's shim materialises other layouts
 *    before calling in.
 */
#ifndef GBFIR_H_
#define GBFIR_H_

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define GBFIR_API __attribute__((visibility("default")))
#else
#define GBFIR_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* CUDA stream handle; identical to cudaStream_t (struct CUstream_st*). */
typedef struct CUstream_st *gbfir_stream_t;

/* Status codes.  The first block mirrors matxError_t (include/matx/core/error.h:55-75)
 * so the MatX shim can rethrow with the same class. */
typedef enum gbfir_status {
  GBFIR_SUCCESS = 0,
  GBFIR_ERR_INVALID_PARAMETER = 1, /* matxInvalidParameter */
  GBFIR_ERR_INVALID_DIM = 2,       /* matxInvalidDim */
  GBFIR_ERR_INVALID_SIZE = 3,      /* matxInvalidSize */
  GBFIR_ERR_INVALID_TYPE = 4,      /* matxInvalidType */
  GBFIR_ERR_NOT_SUPPORTED = 5,     /* matxNotSupported */
  GBFIR_ERR_CUDA = 6,              /* matxCudaError */
  GBFIR_ERR_NULL_POINTER = 7,      /* a required pointer was NULL */
  GBFIR_ERR_ALIGNMENT = 8,         /* pointer/stride not aligned to its element type */
  GBFIR_ERR_WORKSPACE = 9,         /* workspace missing or too small */
  GBFIR_ERR_TIMEOUT = 10           /* a bounded device-side wait gave up */
} gbfir_status;

typedef enum gbfir_dtype {
  GBFIR_F32 = 0,  /* float                         */
  GBFIR_C64 = 1,  /* cuda::std::complex<float>     */
  GBFIR_F64 = 2,  /* double                        */
  GBFIR_C128 = 3  /* cuda::std::complex<double>    */
} gbfir_dtype;

/* Same order as matxConvCorrMode_t (include/matx/core/operator_options.h:51-55). */
typedef enum gbfir_conv_mode {
  GBFIR_MODE_FULL = 0,
  GBFIR_MODE_SAME = 1,
  GBFIR_MODE_VALID = 2
} gbfir_conv_mode;

/* Arithmetic form of the tap contraction. */
typedef enum gbfir_precision {
  GBFIR_PREC_FP32 = 0,   /* CUDA-core FP32 (FP64 for F64/C128 operands)                 */
  GBFIR_PREC_BF16 = 1,   /* tcgen05 tensor cores, bf16 operands, FP32 accumulate        */
  GBFIR_PREC_FP16 = 2,   /* tcgen05 tensor cores, fp16 operands, FP32 accumulate        */
  GBFIR_PREC_BF16X3 = 3  /* tcgen05, each operand split into three bf16 terms; the six
                            cross products of order <= 2 are accumulated in FP32        */
} gbfir_precision;

typedef struct gbfir_buf {
  void *ptr;            /* device pointer to row 0 element 0                 */
  int64_t batch;        /* number of rows (>= 1)                             */
  int64_t len;          /* elements per row                                  */
  int64_t batch_stride; /* elements between rows; 0 broadcasts row 0         */
  int32_t dtype;        /* gbfir_dtype                                       */
} gbfir_buf;

/* `batch` images of rows x cols elements: element (b, r, c) at
 * ptr + b*batch_stride + r*row_stride + c (batch_stride 0 broadcasts image 0). */
typedef struct gbfir_buf2d {
  void *ptr;
  int64_t batch, rows, cols;
  int64_t batch_stride, row_stride;
  int32_t dtype;
} gbfir_buf2d;

/* ---- forward operators ------------------------------------------------- */

/* Direct 1-D convolution or correlation of every row of `in` with `h`.
 *  out.len must be N+L-1 (FULL), max(N,L) (SAME) or max(N,L)-min(N,L)+1 (VALID),
 *  matching Conv1DOp's output shape (include/matx/operators/conv.h:109-133).
 *  The longer operand is treated as the signal (conv.h:427-450); SAME starts
 *  at (Lmin-1)/2 for odd Lmin and Lmin/2-1 for even Lmin (kernels/conv.cuh:155-168).
 *  is_corr != 0 computes corr(in, h) = conv1d(in, reverse(conj(h))) (corr.h:67).
 *  `in` and `h` may each be batched (same row count as out) or broadcast.
 *  out is complex if either operand is complex.
 *  precision != FP32 runs the Toeplitz MMA form on the tensor cores; it takes float32 /
 *  complex64 signals with one real float32 filter row no longer than the signal, and
 *  returns GBFIR_ERR_NOT_SUPPORTED for other operands. */
GBFIR_API int gbfir_conv1d(gbfir_buf out, gbfir_buf in, gbfir_buf h, int32_t mode,
                 int32_t is_corr, int32_t precision, gbfir_stream_t stream);

/* Direct conv2d of images with filters (MatX conv2d, include/matx/transforms/conv.h:548-600,
 *  kernels/conv.cuh:210-402): out[oy][ox] = sum x[oy+fy-dy][ox+fx-dx] * h[N2-1-fy][M2-1-fx],
 *  dy/dx = N2-1/M2-1 (FULL), N2/2, M2/2 (SAME), 0 (VALID); out rows/cols per axis
 *  max+min-1 / max / max-min+1; the operand with more elements is the image (conv.h:569-576);
 *  each operand one image or out.batch of them; out complex if either operand is.  Filters
 *  up to 64 x 64 (GBFIR_ERR_NOT_SUPPORTED beyond). */
GBFIR_API int gbfir_conv2d(gbfir_buf2d out, gbfir_buf2d in, gbfir_buf2d h, int32_t mode,
                           gbfir_stream_t stream);

/* FFT-method conv1d / corr (MatX MATX_C_METHOD_FFT, include/matx/transforms/conv.h:51-172):
 *  the same outputs as gbfir_conv1d up to FP32 rounding, computed by overlap-save with
 *  transforms of 1024..8192 points in shared memory.  float32 / complex64 operands, h one
 *  row of at most GBFIR_FFT_CONV_MAX_TAPS taps, the signal at least as long as the
 *  filter; other operands return GBFIR_ERR_NOT_SUPPORTED. */
#define GBFIR_FFT_CONV_MAX_TAPS 7169
GBFIR_API int gbfir_conv1d_fft(gbfir_buf out, gbfir_buf in, gbfir_buf h, int32_t mode,
                               int32_t is_corr, gbfir_stream_t stream);

/* conv1d / corr along a strided axis.  Signal (b, i), b < out.batch, i < inner, is
 *  in[b*in.batch_stride + n*in_step + i], n < in.len (in.batch_stride 0 broadcasts one
 *  block); its output is out[b*out.batch_stride + m*out_step + i], m < out.len.  A
 *  contiguous [batch][len][inner] tensor has in_step = inner; a slice of a wider one a
 *  larger step.  This is MatX's conv1d(a, h, {axis}, mode)
 *  (include/matx/operators/conv.h:263-274) and the permuted-view conv1d of the radar
 *  three-pulse canceller (examples/simple_radar_pipeline.h:321-327) without
 *  materialising the permutation.  Output lengths, the SAME start and corr as
 *  gbfir_conv1d; h is one row; out_step >= inner.  FP32 / FP64 only (other precisions:
 *  GBFIR_ERR_NOT_SUPPORTED). */
GBFIR_API int gbfir_conv1d_axis(gbfir_buf out, gbfir_buf in, gbfir_buf h, int64_t inner,
                                int64_t in_step, int64_t out_step, int32_t mode,
                                int32_t is_corr, int32_t precision, gbfir_stream_t stream);

/* Polyphase resampler: out[b] = up * (upsample-by-up, filter with h,
 * downsample-by-down)(in[b]), with the scipy centring of
 * include/matx/transforms/resample_poly.h:212-281 (even h gets a leading zero).
 *  out.len must equal ceil(in.len*up/down) with the UNREDUCED up/down
 *  (resample_poly.h:318-320); up/down are then divided by their gcd; up==down
 *  copies the input and ignores h (resample_poly.h:333-336).
 *  h is one row (broadcast); real or complex.
 *  precision != FP32 runs the Toeplitz MMA form on the tensor cores for float32 /
 *  complex64 signals and real float32 taps; rates whose 8-sample rows need more than
 *  256 MMA columns (for example 160/147) return GBFIR_ERR_NOT_SUPPORTED. */
/* MatX filter(in, h_rec, h_nonrec) along rows (include/matx/operators/filter.h:177-181,
 *  include/matx/transforms/filter.h:159-188).  h_rec / h_nonrec are HOST arrays of
 *  num_rec (0..4) / num_nonrec (1..4) coefficients of coef_dtype (MatX passes
 *  cuda::std::array by value; at most 4 of each, kernels/filter.cuh:29-30):
 *    num_rec == 0: conv1d(in, h_nonrec, SAME) (transforms/filter.h:185), len >= num_nonrec;
 *    else y[n] = sum_{j<num_nonrec} h_nonrec[j] x[n-j] + sum_{k<num_rec} h_rec[k] y[n-1-k],
 *    zero initial state (kernels/filter.cuh:44; test/00_operators/filter_test.cu:19-47).
 *  out.len == in.len; out complex iff in or the coefficients are complex; all single or all
 *  double.  The recursive form needs `workspace` (device, 16-byte aligned) of
 *  gbfir_filter_workspace_size(out.batch, len, out.dtype) bytes (GBFIR_ERR_WORKSPACE if
 *  missing or short); no device memory is allocated. */
GBFIR_API size_t gbfir_filter_workspace_size(int64_t batch, int64_t len, int32_t out_dtype);
GBFIR_API int gbfir_filter(gbfir_buf out, gbfir_buf in, const void *h_rec, int32_t num_rec,
                           const void *h_nonrec, int32_t num_nonrec, int32_t coef_dtype,
                           void *workspace, size_t workspace_bytes, gbfir_stream_t stream);

/* MatX's upsample(in, dim, n) / downsample(in, dim, n) along rows
 *  (include/matx/operators/updownsample.h:254-279): upsample writes in[i/n] where n
 *  divides i and 0 elsewhere, out.len = in.len*n; downsample writes in[i*n],
 *  out.len = ceil(in.len/n).  Same dtype in and out; `in` one row or out.batch rows. */
GBFIR_API int gbfir_upsample(gbfir_buf out, gbfir_buf in, int64_t n, gbfir_stream_t stream);
GBFIR_API int gbfir_downsample(gbfir_buf out, gbfir_buf in, int64_t n, gbfir_stream_t stream);

/* downsample(conv1d(upsample(in, up), h, mode), down) in one polyphase pass that forms
 *  neither the zero-stuffed signal nor the discarded outputs:
 *    out[m] = sum_k in[k] * h[start + m*down - k*up],
 *  start = the conv1d mode offset for the upsampled length N*up (0 FULL, (Lmin-1)/2 or
 *  Lmin/2-1 SAME, Lmin-1 VALID, Lmin = min(N*up, L)), out.len = ceil(conv length / down)
 *  (operators/updownsample.h:254-279 around transforms/conv.h:402-532).  No x-up scale
 *  and no even-length lead zero (those are resample_poly's).  h is one row; FP32 / FP64
 *  only (other precisions: GBFIR_ERR_NOT_SUPPORTED). */
GBFIR_API int gbfir_upfirdn(gbfir_buf out, gbfir_buf in, gbfir_buf h, int64_t up, int64_t down,
                            int32_t mode, int32_t precision, gbfir_stream_t stream);

GBFIR_API int gbfir_resample_poly(gbfir_buf out, gbfir_buf in, gbfir_buf h, int64_t up,
                        int64_t down, int32_t precision, gbfir_stream_t stream);

/* Polyphase channelizer, maximally decimated (D == M) or oversampled (D < M),
 * fused FIR branch filtering + unnormalised positive-sign M-point DFT
 * (include/matx/transforms/channelize_poly.h:724-849, host semantics :858-1029).
 *  out is [batch][T][M] complex with T = ceil(in.len/D): out.len == T*M.
 *  h is one row of any length L; it is zero-padded to P*M with P = ceil(L/M).
 *  precision != FP32 runs the cross-channel DFT as a dense complex GEMM on the tensor
 *  cores (complex64 signal, real float32 taps, D == M with M in {16, 32, 64}); other
 *  shapes return GBFIR_ERR_NOT_SUPPORTED. */
GBFIR_API int gbfir_channelize_poly(gbfir_buf out, gbfir_buf in, gbfir_buf h, int64_t M,
                          int64_t D, int32_t precision, gbfir_stream_t stream);

/* ---- adjoints (no MatX counterpart) --------------------------------------
 * For y = resample_poly(x, h, up, down) and the upstream gradient gy:
 *   dx = transposed resampler of gy (correlation with the taps, up/down swapped),
 *   dh = sum over the batch of the cross-correlation of gy with x,
 *        reduced across blocks in FP64 in `workspace`.
 * Either dx.ptr or dh.ptr may be NULL to skip that gradient.  up==down after
 * the gcd gives dx = gy and dh = 0, matching the forward identity copy.
 * Real FP32 operands only. */
GBFIR_API size_t gbfir_resample_poly_bwd_workspace_size(int64_t batch, int64_t in_len,
                                              int64_t h_len, int64_t up,
                                              int64_t down);
GBFIR_API int gbfir_resample_poly_bwd(gbfir_buf dx, gbfir_buf dh, gbfir_buf gy,
                            gbfir_buf x, gbfir_buf h, int64_t up, int64_t down,
                            void *workspace, size_t workspace_bytes,
                            gbfir_stream_t stream);

/* Adjoint of gbfir_conv1d (is_corr == 0, real FP32, h broadcast):
 *   dx = corr(gy, h) cropped to the signal, dh = sum_b corr(gy_b, x_b) cropped to L. */
GBFIR_API size_t gbfir_conv1d_bwd_workspace_size(int64_t batch, int64_t in_len,
                                       int64_t h_len, int32_t mode);
GBFIR_API int gbfir_conv1d_bwd(gbfir_buf dx, gbfir_buf dh, gbfir_buf gy, gbfir_buf x,
                     gbfir_buf h, int32_t mode, void *workspace,
                     size_t workspace_bytes, gbfir_stream_t stream);

/* gbfir_conv1d_bwd with a choice of arithmetic: precision != FP32 computes dx on the tensor
 * cores (the forward Toeplitz-MMA pass over gy with the taps reversed; NOT_SUPPORTED where no
 * tile fits) and dh as the tensor-core GEMM over the signal rows described for
 * gbfir_resample_poly_bwd_prec (the FP32 reduction where its tile does not fit).  Other
 * arguments and results are those of gbfir_conv1d_bwd. */
GBFIR_API int gbfir_conv1d_bwd_prec(gbfir_buf dx, gbfir_buf dh, gbfir_buf gy, gbfir_buf x,
                                    gbfir_buf h, int32_t mode, int32_t precision, void *workspace,
                                    size_t workspace_bytes, gbfir_stream_t stream);

/* gbfir_resample_poly_bwd with a choice of arithmetic: precision != FP32 computes dx on the
 * tensor cores as a Toeplitz MMA pass over gy (the transposed resampler, taps reversed,
 * rates swapped; same coverage rules as the forward forms, NOT_SUPPORTED otherwise), and dh
 * as a GEMM over the signal rows (input Hankel slab x gradient rows, FP32 in tensor memory
 * per CTA, FP64 across CTAs, deterministic).  Where the tap gradient's row tile does not fit
 * the tensor-core kernel (rows of up * G phases within 256 MMA columns whose input band
 * fits two accumulators, e.g. 160/147 with thousands of taps), dh comes from the FP32
 * row-tile reduction instead.  Other arguments and results are those of
 * gbfir_resample_poly_bwd. */
GBFIR_API int gbfir_resample_poly_bwd_prec(gbfir_buf dx, gbfir_buf dh, gbfir_buf gy, gbfir_buf x,
                                           gbfir_buf h, int64_t up, int64_t down, int32_t precision,
                                           void *workspace, size_t workspace_bytes, gbfir_stream_t stream);

/* Allocation-free variant of gbfir_resample_poly_bwd.  It has no counterpart in
 * the reference library.  It is for callers that cannot hand this library a device
 * workspace: callers whose calling convention has no slot for one (an operator
 * signature fixed by another framework), and callers that must not touch the device
 * allocator while they run (processing loops with a fixed memory budget, plugins
 * inside a host application that owns every device allocation).
 * Arguments and results are those of gbfir_resample_poly_bwd; the FP64 partial tap
 * gradients live in a scratch array compiled into the library instead of in a
 * caller workspace.  That array holds GBFIR_NOALLOC_SCRATCH_BYTES per device and stays
 * resident on every GPU that loads the library until the process exits.  A call whose
 * partials do not fit (about 2 * SMs * (h_len + 1) * 8 bytes) is rejected with
 * GBFIR_ERR_INVALID_SIZE before any device work.  Nothing here calls cudaMalloc or
 * cudaFree.  The first call on each device looks the array's device address up
 * (cudaGetSymbolAddress) with that device current; make that first call before any
 * stream capture.  The address is kept for the life of the process, so a
 * cudaDeviceReset() of a device (which unloads the library's device code there) ends
 * this entry point's use on that device.  All calls share the one array: calls whose
 * work overlaps on the GPU (different streams without ordering, or different host
 * threads) race on it and must be serialised by the caller. */
#define GBFIR_NOALLOC_SCRATCH_BYTES (4u << 20)
GBFIR_API int gbfir_resample_poly_bwd_noalloc(gbfir_buf dx, gbfir_buf dh, gbfir_buf gy,
                                              gbfir_buf x, gbfir_buf h, int64_t up,
                                              int64_t down, gbfir_stream_t stream);

/* ---- ragged batches (no MatX counterpart) --------------------------------
 * One persistent launch resamples `count` independent complex64 signals of
 * uneven length, tap count and up/down ratio.  Descriptors live in device
 * memory (an array of gbfir_ragged_desc).  The launch is stream-ordered and
 * contains no host synchronisation, so it can be captured in a CUDA graph. */
typedef struct gbfir_ragged_desc {
  const void *in;   /* complex64 input row                      */
  void *out;        /* complex64 output row                     */
  const float *h;   /* real taps                                */
  int64_t in_len;
  int64_t out_len;  /* must be ceil(in_len*up/down)             */
  int32_t h_len;
  int32_t up;       /* reduced by gcd in the planner; up==down copies the input */
  int32_t down;
  int32_t pad_;
} gbfir_ragged_desc;

/* Bytes of device workspace gbfir_ragged_resample needs (a work-queue counter). */
GBFIR_API size_t gbfir_ragged_workspace_size(int64_t count, int64_t num_tiles);

/* Launch geometry produced by the planner (host memory). */
typedef struct gbfir_ragged_plan_info {
  int64_t num_tiles;     /* entries (work items) in the tile table             */
  int64_t shared_bytes;  /* dynamic shared memory per CTA                      */
  int64_t table_bytes;   /* of which the tap table (the window buffers follow) */
  int64_t window_elems;  /* complex samples per window buffer (FP32 plans); the K
                            chunk of the tensor-core plans                     */
  int64_t buffers;       /* window buffers per CTA (2: the next tile prefetched) */
  int64_t precision;     /* the gbfir_precision the plan was made for          */
} gbfir_ragged_plan_info;

/* Tile shape the ragged planner uses for signals of one reduced (up, down) whose tap
 * count falls in h_len's bucket (the smallest power of two >= h_len): rows_per_thread
 * 1 or 2, col_warps 1, 2, 4 or 8, group 1..64 (outputs per row = up * group).  Filled
 * by the autotuner (no MatX counterpart); signals without an entry take the built-in
 * heuristic, and rows_per_thread = col_warps = group = 0 removes the entry.  Applies to
 * plans made after the call. */
GBFIR_API int gbfir_ragged_tile_register(int64_t up, int64_t down, int64_t h_len,
                                         int32_t rows_per_thread, int32_t col_warps,
                                         int32_t group);
GBFIR_API int gbfir_ragged_tile_clear(void);

/* Host-side planner.  Validates the descriptors (host copies), cuts every signal
 * into row tiles of its own geometry and groups consecutive tiles of one signal into
 * work items of similar cost; writes `tile_table` (host memory, four int64 per item:
 * signal index, first row, number of rows, packed tile shape), most expensive items
 * first.  Returns the number of items (with tile_table == NULL it only counts) or a
 * negative gbfir_status, and fills *info.  Each signal's up/down are reduced by
 * their gcd. */
GBFIR_API int64_t gbfir_ragged_plan(const gbfir_ragged_desc *host_descs, int64_t count,
                          int64_t *tile_table, gbfir_ragged_plan_info *info);

/* The planner for one arithmetic form (no MatX counterpart): FP32 is gbfir_ragged_plan; the
 * tensor-core forms (BF16, FP16, BF16X3) plan the column-blocked Toeplitz-MMA pass, each
 * signal with its own block geometry packed into its items (four int64 per item: signal,
 * first row, rows, packed geometry), rows in tiles of 64.  A signal whose tap matrix does not
 * fit shared memory fails the plan with GBFIR_ERR_NOT_SUPPORTED.  Pass the same precision to
 * gbfir_ragged_resample. */
GBFIR_API int64_t gbfir_ragged_plan_prec(const gbfir_ragged_desc *host_descs, int64_t count,
                                         int32_t precision, int64_t *tile_table,
                                         gbfir_ragged_plan_info *info);

/* One persistent launch over all work items.  device_descs / device_tile_table are
 * device copies of the descriptors and of the planner's table; info is the
 * planner's host struct, made for `precision` (GBFIR_ERR_INVALID_PARAMETER otherwise).
 * CTAs take items from an atomic counter in `workspace` (zeroed on the stream first), so
 * the launch balances arbitrary length skew and contains no host synchronisation: it can
 * be captured in a CUDA graph. */
GBFIR_API int gbfir_ragged_resample(const gbfir_ragged_desc *device_descs, int64_t count,
                          const int64_t *device_tile_table,
                          const gbfir_ragged_plan_info *info, int32_t precision,
                          void *workspace, size_t workspace_bytes,
                          gbfir_stream_t stream);

/* ---- tuning and diagnostics ---------------------------------------------- */

/* Override the tile shape the dispatcher picks for resample_poly (autotuner
 * hook; no MatX counterpart).  rows_per_thread in {1,2,4}, col_warps in
 * {1,2,4,8} (or 9..16 with one row per thread), group (outputs per row =
 * group*up) >= 1, buffers in {1,2,3} (2 = prefetch the next input window while
 * computing; 3 = the ring form for complex float signals with real taps: one CTA
 * per SM, a staging warp keeping up to three windows in flight ahead of 16 compute
 * warps, col_warps 1/2/4/8 giving 16/col_warps row slices; other signals take 2),
 * plus 4 to write the outputs through shared memory and TMA tensor stores (complex
 * float signals with real taps, rows of 2, 4 or >= 8 even outputs; other cases
 * store directly), plus 8 for the paired walk (even row strides: two samples per
 * 16-byte load, bands from even k).  Zero for a field keeps the built-in heuristic
 * for it.
 * Process-wide setting, not thread-safe. */
GBFIR_API int gbfir_set_resample_tile(int32_t rows_per_thread, int32_t col_warps,
                            int32_t group, int32_t buffers);

/* Register the tile shape resample_poly uses for one (up, down, filter length)
 * (autotuner output; no MatX counterpart).  up/down are reduced by their gcd.
 * Same field meaning as gbfir_set_resample_tile; the global override wins over
 * a registered entry, a registered entry over the built-in heuristic. */
GBFIR_API int gbfir_resample_tile_register(int64_t up, int64_t down, int64_t h_len,
                                 int32_t rows_per_thread, int32_t col_warps,
                                 int32_t group, int32_t buffers);
GBFIR_API int gbfir_resample_tile_clear(void);

/* Status of the bounded waits inside the pipelined kernels of the current device (the
 * tensor-core kernels and the TMA-fed row tile) since the last call: 0 = none gave up,
 * 1 = at least one gave up (its results are incomplete), -1 = could not be read.
 * Synchronous; clears the flags. */
GBFIR_API int gbfir_tc_status(void);

/* Number of device kernels this library has launched in this process. */
GBFIR_API uint64_t gbfir_launch_count(void);

GBFIR_API const char *gbfir_status_string(int status);
GBFIR_API const char *gbfir_last_error(void);
GBFIR_API int gbfir_version(void);

#ifdef __cplusplus
}
#endif

#endif /* GBFIR_H_ */
