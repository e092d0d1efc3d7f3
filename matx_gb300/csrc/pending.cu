// pending.cu — entry points whose kernels are not built yet.  Each returns
// GBFIR_ERR_NOT_SUPPORTED with a message; nothing falls back to another path.
#include "common.cuh"

namespace gbfir {
int resample_poly_tc(const gbfir_buf &, const gbfir_buf &, const gbfir_buf &, int64_t, int64_t, int,
                     cudaStream_t) {
  GBFIR_FAIL(GBFIR_ERR_NOT_SUPPORTED, "resample_poly: tensor-core forms are not available in this build");
}
}  // namespace gbfir

extern "C" {
size_t gbfir_ragged_workspace_size(int64_t, int64_t) { return 0; }
int64_t gbfir_ragged_plan(const gbfir_ragged_desc *, int64_t, int32_t, int64_t *) { return -GBFIR_ERR_NOT_SUPPORTED; }
int gbfir_ragged_resample(const gbfir_ragged_desc *, int64_t, const int64_t *, int64_t, int32_t, int32_t, void *,
                          size_t, gbfir_stream_t) {
  GBFIR_FAIL(GBFIR_ERR_NOT_SUPPORTED, "ragged_resample: not available in this build");
}
}
