// Host-side advection plan (shared by adv.cu and adv_util.cu).
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "adv.cuh"
#include "common.cuh"

namespace bkma {

struct AdvPlanImpl {
    bkma_adv_desc desc{};
    AdvPhys phys{};
    int64_t lines = 0;
    int npts = 6;
    int esize = 4;
    // host tables
    std::vector<int32_t> base;       // per line, tap-0 offset mod n1
    std::vector<double> shift;       // per line, d - 2 at i1 = 0
    std::vector<double> vx;          // per line velocity
    std::vector<double> w64;         // per line weights
    std::vector<int32_t> exc_index;  // per line, -1 or exception slot
    int64_t n_exc = 0;
    // device tables
    int32_t *d_base = nullptr;
    void *d_w = nullptr;  // T weights
    int32_t *d_exc_index = nullptr;
    void *d_exc = nullptr;
    double *d_vx = nullptr;
    // launch shape: path 0 = cp.async staging (any shape), 1 = TMA staging
    int W = 16, R = 1, threads = 256, path = 0;
    bool autotuned = false;
    struct TmapCache {
        const void *ptr;
        int W;
        CUtensorMap map;
    };
    std::vector<TmapCache> tmaps;  // TMA descriptors of recently used fields
    int *d_status = nullptr;       // device status word of the bounded waits
    // host-run buffer
    void *d_host_buf = nullptr;
    size_t host_buf_bytes = 0;
    double *d_partials = nullptr;
    int device = 0;

    ~AdvPlanImpl() {
        cudaFree(d_base);
        cudaFree(d_w);
        cudaFree(d_exc_index);
        cudaFree(d_exc);
        cudaFree(d_vx);
        cudaFree(d_host_buf);
        cudaFree(d_partials);
        cudaFree(d_status);
    }

    int halo() const { return desc.impl == BKMA_ADV_PLAIN ? 0 : npts - 1; }
    int64_t ncb(int w) const { return (desc.n2 + w - 1) / w; }
    // Shared memory of an R-slab tile of w columns: the widest row stride of
    // the full tiles and of the ragged last column tile.
    size_t smem_bytes(int w, int r) const {
        const int wc = (int)std::min<int64_t>(w, desc.n2);
        int ws = staged_row_stride(desc.n2, wc, esize);
        const int last = (int)(desc.n2 % wc);
        if (last) ws = std::max(ws, staged_row_stride(desc.n2, last, esize));
        return (size_t)r * (size_t)slab_stride(desc.n1, halo(), ws, esize) * (size_t)esize;
    }
    int64_t tiles(int w, int r) const { return ((lines + r - 1) / r) * ncb(w); }
};

bool adv_tma_eligible(const AdvPlanImpl &p, const void *src, int W);
size_t adv_tma_smem(const AdvPlanImpl &p, int W);
cudaError_t adv_tma_launch(AdvPlanImpl &p, const void *src, void *dst, int W, int threads,
                           cudaStream_t st);

}  // namespace bkma

struct bkma_adv_plan {
    bkma::AdvPlanImpl impl;
};

namespace bkma {
inline AdvPlanImpl &plan_impl(bkma_adv_plan *p) { return p->impl; }
inline const AdvPlanImpl &plan_impl(const bkma_adv_plan *p) { return p->impl; }
}  // namespace bkma
