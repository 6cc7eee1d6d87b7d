// Batched uneven advection. Placeholder until the persistent kernel lands.
#include "adv_plan.cuh"

extern "C" {
bkma_status bkma_adv_batch_create(const bkma_adv_field *, int32_t, int32_t, bkma_adv_batch **b) {
    if (b) *b = nullptr;
    return bkma::fail(BKMA_ERR_UNSUPPORTED, "batched advection not built yet");
}
bkma_status bkma_adv_batch_step(bkma_adv_batch *, int32_t, void *) {
    return bkma::fail(BKMA_ERR_UNSUPPORTED, "batched advection not built yet");
}
bkma_status bkma_adv_batch_info(const bkma_adv_batch *, int64_t *, int32_t *) {
    return bkma::fail(BKMA_ERR_UNSUPPORTED, "batched advection not built yet");
}
bkma_status bkma_adv_batch_destroy(bkma_adv_batch *) { return BKMA_OK; }
}
