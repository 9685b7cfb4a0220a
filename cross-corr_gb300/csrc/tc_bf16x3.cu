// tc_bf16x3.cu -- split-BF16 tensor-core correlation (tcgen05), FP32 in/out.
#include "xc_common.cuh"
#include "xc_internal.h"

namespace xc {

size_t tc_workspace_size(const Geometry& g, const PairMap& pm) {
  (void)g;
  (void)pm;
  return 0;
}

xc_status tc_correlate(const float* left, const float* right, float* out, const Geometry& g, const PairMap& pm,
                       void* workspace, size_t ws_bytes, cudaStream_t stream) {
  (void)left; (void)right; (void)out; (void)g; (void)pm; (void)workspace; (void)ws_bytes; (void)stream;
  return fail(XC_ERR_UNSUPPORTED, "split-BF16 tensor-core path not built yet");
}

}  // namespace xc
