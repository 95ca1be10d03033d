// BF16 tensor-core NeRF MLP path (placeholder until the tcgen05 kernels land).
#include "nerf_mlp.h"

namespace srf {
size_t mlp_tc_workspace(const MlpLayout&, int64_t, bool) { return 0; }
int mlp_tc_forward(const MlpLayout&, const float* const*, const float*, const float*, int, int64_t, const float*,
                   float*, float*, bool, void*, size_t, cudaStream_t) {
    return SRF_ERR_UNSUPPORTED;
}
int mlp_tc_backward(const MlpLayout&, const float* const*, const float*, const float*, int64_t, int, float* const*,
                    void*, size_t, cudaStream_t) {
    return SRF_ERR_UNSUPPORTED;
}
}  // namespace srf
