// Conv1d plan and kernel argument blocks (conv.cu, conv_tc.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "common.cuh"

namespace bkma {

struct ConvRefArgs {
    const double *src;
    double *dst;
    const double *weight;  // (K, Cin, Cout)
    const double *bias;    // (Cout)
    int64_t n1, n2, K;
    int cin;
    int64_t length;
    int W;
};

template <typename T>
struct ConvTorchArgs {
    const T *x;
    T *out;
    const T *w;     // (Cout, Cin, K)
    const T *bias;  // (Cout) or null
    const T *halo;  // [B][ntiles][Cin][K-1] or null (out of place)
    int64_t B;
    int cin, cout;
    int64_t L;
    int K, TL;
    int64_t ntiles;
    int64_t out_stride;  // row stride of out: L in place, L-K+1 out of place
};

struct ConvPlanImpl {
    bkma_conv_desc desc{};
    int device = 0;
    bool tensor = false;
    int TL = 64;          // output columns per tile
    int64_t ntiles = 0;   // tiles per row
    void *d_halo = nullptr;
    size_t halo_bytes = 0;
    int halo_width = 0;       // halo values kept per channel of a snapshot slot >= K-1
    void *d_wpack = nullptr;  // weights packed for the tensor path
    size_t wpack_bytes = 0;
    void *d_status = nullptr; // device status word of the tensor kernel
    uint32_t wait_polls = kWaitPolls;  // polls of a bounded device wait before it gives up
    int grid = 0;
    ~ConvPlanImpl() {
        cudaFree(d_halo);
        cudaFree(d_wpack);
        cudaFree(d_status);
    }
};

// Argument checks shared by every conv1d entry point (bounds that keep the
// kernels' int fields in range, semantics, dtype).
bkma_status conv_check_desc(const bkma_conv_desc &d);
bkma_status conv_halo_prepass(ConvPlanImpl &p, const void *x, cudaStream_t st);
bkma_status conv_tc_scratch_need(const bkma_conv_desc &d, size_t *halo_bytes, size_t *wpack_bytes);
bkma_status conv_tc_run_into(const bkma_conv_desc &d, void *data, const void *w, const void *bias,
                             void *halo, void *wpack, int *status, cudaStream_t st);
bkma_status conv_tc_plan_init(ConvPlanImpl &p);
bkma_status conv_tc_run(ConvPlanImpl &p, void *data, void *out, const void *w, const void *bias,
                        cudaStream_t st);

}  // namespace bkma

struct bkma_conv_plan {
    bkma::ConvPlanImpl impl;
};
