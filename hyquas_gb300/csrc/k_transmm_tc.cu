// Tensor-core TransMM contraction (tcgen05): split-BF16 x3 and TF32.
#include <cuda_runtime.h>

#include "common.h"
#include "transmm.h"

namespace hq {

size_t transmm_tc_operand_bytes(int m, int precision) {
    (void)precision;
    return size_t(16) << (2 * m);
}

void launch_u_to_tc_operand(int, int, const double*, void*, cudaStream_t) {
    fail(HQ_ERR_UNSUPPORTED, "tensor-core TransMM not available in this build");
}

void launch_transmm_tc(const TransmmLaunch&, cudaStream_t) {
    fail(HQ_ERR_UNSUPPORTED, "tensor-core TransMM not available in this build");
}

}  // namespace hq
