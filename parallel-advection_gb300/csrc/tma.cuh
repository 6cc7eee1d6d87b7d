// Pieces shared by the TMA-staged advection kernels (adv_tma.cu, adv_ds.cu):
// the shared-memory address of a pointer, a bounded wait on a staging
// barrier's first phase, and the plan's cached tensor maps of a field.
#pragma once
#include <cuda.h>

#include <cstdint>

#include "adv_plan.cuh"

namespace bkma {

__device__ __forceinline__ uint32_t smem_u32addr(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// Polls phase 0 of the staging barrier at most `polls` times.
__device__ __forceinline__ bool staging_wait(uint64_t *bar, uint32_t polls) {
    for (uint32_t i = 0; i < polls; ++i) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n"
            " selp.u32 %0, 1, 0, p;\n}"
            : "=r"(done)
            : "r"(smem_u32addr(bar))
            : "memory");
        if (done) return true;
        if (i > 32) __nanosleep(128);
    }
    return false;
}

// One thread: arm the barrier for `bytes` and issue `nbox` 3-D boxes
// (columns c0.., rows b * box_rows.., slab `line`) back to back into `dst`,
// each box box_bytes long.
__device__ __forceinline__ void staging_issue(const CUtensorMap *tmap, uint64_t *bar, void *dst,
                                              uint32_t bytes, int nbox, int box_rows,
                                              uint32_t box_bytes, int c0, int line) {
    asm volatile(
        "{\n .reg .b64 st;\n mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n}" ::"r"(
            smem_u32addr(bar)),
        "r"(bytes)
        : "memory");
    for (int b = 0; b < nbox; ++b) {
        const uint32_t d = smem_u32addr(dst) + (uint32_t)b * box_bytes;
        asm volatile(
            "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes "
            "[%0], [%1, {%2, %3, %4}], [%5];" ::"r"(d),
            "l"(reinterpret_cast<uint64_t>(tmap)), "r"(c0), "r"(b * box_rows), "r"(line),
            "r"(smem_u32addr(bar))
            : "memory");
    }
}

// The plan's tensor map of field `src` (dims n2 x n1 x lines of the plan's
// element type, boxes W x min(256, n1) x 1), encoded once per (pointer, W)
// and cached; null if the driver cannot encode it.
const CUtensorMap *adv_field_tmap(AdvPlanImpl &p, const void *src, int W);

}  // namespace bkma
