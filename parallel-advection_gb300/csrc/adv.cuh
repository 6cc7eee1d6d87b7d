// Kernel argument blocks of the advection kernels (adv.cu, batch.cu).
#pragma once
#include <cstdint>

#include "common.cuh"

namespace bkma {

constexpr int kMaxTaps = 10;

// Per-cell stencil of a line whose departure offset varies along n1.
template <typename T>
struct AdvExcCell {
    int32_t base;  // tap-0 row minus i1, modulo n1
    T w[kMaxTaps];
};

template <typename T>
struct AdvStagedArgs {
    const T *src;
    T *dst;
    int64_t n1, n2, lines;
    int W, R;          // tile: W columns (i2) x R slabs (i0) x all n1 rows
    int64_t ncb;       // column blocks per slab
    int vec_ok;        // 16-byte cp.async allowed
    const int32_t *base;       // [lines]
    const T *w;                // [lines][NT]
    const int32_t *exc_index;  // [lines]
    const AdvExcCell<T> *exc;  // [exception lines][n1]
};

struct AdvTmaArgs {
    float *dst;
    int64_t n1, n2;
    int64_t ncb;               // column blocks per slab
    int box_rows, nbox;        // TMA boxes of box_rows rows cover n1
    const int32_t *base;       // [lines]
    const float *w;            // [lines][NT]
    const int32_t *exc_index;  // [lines]
    const AdvExcCell<float> *exc;
    int *status;               // device status word (BKMA_ERR_TIMEOUT on a stuck copy)
};

struct AdvPlainArgs {
    const double *src;
    double *dst;
    int64_t n1, n2, lines;
    int W, R;
    int64_t ncb;
    int vec_ok;
    const double *vx;  // [lines]
    AdvPhys phys;
};

// Shared-memory elements per staged slab, padded to 16 bytes.
__host__ __device__ __forceinline__ int slab_stride(int64_t n1, int halo, int wc, int esize) {
    const int e = (int)(n1 + halo) * wc;
    const int q = 16 / esize;
    return (e + q - 1) / q * q;
}

}  // namespace bkma
