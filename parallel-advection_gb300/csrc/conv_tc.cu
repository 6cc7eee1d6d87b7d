// BF16 tensor-core conv1d (tcgen05 implicit GEMM). Placeholder until the
// kernel lands: plans asking for it get BKMA_ERR_UNSUPPORTED.
#include "conv.cuh"

namespace bkma {
bkma_status conv_tc_plan_init(ConvPlanImpl &) {
    return fail(BKMA_ERR_UNSUPPORTED, "tensor-core conv1d not built yet");
}
bkma_status conv_tc_run(ConvPlanImpl &, void *, void *, const void *, const void *, cudaStream_t) {
    return fail(BKMA_ERR_UNSUPPORTED, "tensor-core conv1d not built yet");
}
}  // namespace bkma
