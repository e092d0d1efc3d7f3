// pending.cu — entry points whose kernels are not built yet.  Each returns
// GBFIR_ERR_NOT_SUPPORTED with a message; nothing falls back to another path.
#include "common.cuh"

namespace gbfir {
int resample_poly_tc(const gbfir_buf &, const gbfir_buf &, const gbfir_buf &, int64_t, int64_t, int,
                     cudaStream_t) {
  GBFIR_FAIL(GBFIR_ERR_NOT_SUPPORTED, "resample_poly: tensor-core forms are not available in this build");
}
}  // namespace gbfir

