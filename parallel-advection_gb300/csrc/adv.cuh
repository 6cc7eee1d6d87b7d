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
    const int32_t *base;       // [lines]
    const T *w;                // [lines][NT]
    const int32_t *exc_index;  // [lines]
    const AdvExcCell<T> *exc;  // [exception lines][n1]
    const int32_t *line_list;  // optional: tile row lt covers line line_list[lt] (R = 1)
};

// Streamed form (adv_stream.cu): each lane walks one (line, i2) column down
// all n1 rows. A line streams when its offset is constant along n1 and its
// signed tap-0 offset d (base, or base - n1 above n1/2) lies in
// [-kStreamBack, kStreamSeam - npts + 1]; n1 >= kStreamMinN1.
constexpr int kStreamBack = 24;  // d >= -24: every row is read before it is overwritten
constexpr int kStreamSeam = 24;  // rows 0 .. d+npts-2 saved before row 0 is overwritten
constexpr int kStreamMinN1 = 64;

struct StreamField {
    const float *src;
    float *dst;
    int64_t n1, n2, lines;
    const int32_t *base;       // [lines]
    const float *w;            // [lines][npts]
    const int32_t *exc_index;  // [lines]; exception lines are left to the staged pass
    int npts;
    int segs;                  // row segments per 32-column group (warps per group)
    int64_t cta0;              // first CTA of this field in the launch
};

__host__ __device__ __forceinline__ int stream_offset(int32_t base, int64_t n1) {
    return 2 * (int64_t)base > n1 ? (int)(base - n1) : (int)base;
}
__host__ __device__ __forceinline__ bool stream_line_ok(int32_t base, int64_t n1, int npts) {
    const int d = stream_offset(base, n1);
    return n1 >= kStreamMinN1 && d >= -kStreamBack && d + npts - 1 <= kStreamSeam;
}

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
    uint32_t spin_limit;       // polls of the staging barrier before the CTA gives up
};

// FP64-storage kernel with FP32-pair arithmetic (adv_ds.cu): 8-column TMA
// tiles of one slab.
struct AdvDsArgs {
    double *dst;
    int64_t n1, n2;
    int64_t ncb;               // 8-column blocks per slab
    int box_rows, nbox;        // TMA boxes of box_rows rows cover n1
    const int32_t *base;       // [lines]
    const double *w;           // [lines][NT] FP64 weights (FP64 tiles)
    const float2 *w2;          // [lines][NT] (a, b): w = a + b, a = RN32(w), b = RN32(w - a)
    const int32_t *exc_index;  // [lines], or null when the plan has no exception lines
    const AdvExcCell<double> *exc;
    int *status;
    uint32_t spin_limit;
};

struct AdvPlainArgs {
    const double *src;
    double *dst;
    int64_t n1, n2, lines;
    int W, R;
    int64_t ncb;
    const double *vx;  // [lines]
    AdvPhys phys;
};

// Shared-memory row stride of a staged tile of wc columns. It is congruent
// to n2 modulo 16 bytes, so every staged element keeps its global address's
// position inside a 16-byte chunk and the aligned interior of each row is
// copied in 16-byte pieces whatever n2 is.
__host__ __device__ __forceinline__ int staged_row_stride(int64_t n2, int wc, int esize) {
    const int q = 16 / esize;
    const int64_t gap = n2 - wc;
    return wc + (int)(((gap % q) + q) % q);
}

// Shared-memory elements per staged slab: up to q-1 leading elements (the
// slab start's offset inside its 16-byte chunk) plus rows of ws elements,
// rounded up to 16 bytes.
__host__ __device__ __forceinline__ int slab_stride(int64_t n1, int halo, int ws, int esize) {
    const int q = 16 / esize;
    const int e = q - 1 + (int)(n1 + halo) * ws;
    return (e + q - 1) / q * q;
}

}  // namespace bkma
