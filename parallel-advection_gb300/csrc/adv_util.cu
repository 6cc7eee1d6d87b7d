// Device-side init and validation for advected fields:
//  - bkma_adv_fill: fill_buffer_adv (src/tools/init.hpp:31-46) and the seeded
//    sine+noise init of the synthetic workloads;
//  - bkma_adv_error_norms: one-pass max/L2 error against a reference field;
//  - bkma_adv_validate: validate_result_adv (src/tools/validation.hpp:9-80)
//    as one fused reduction over all i2 instead of n2 separate launches.
#include <cmath>
#include <vector>

#include "adv_plan.cuh"
#include "common.cuh"

namespace bkma {

__host__ __device__ __forceinline__ uint64_t splitmix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Same generator as the oracle's bko_uniform.
__host__ __device__ __forceinline__ double uniform01(uint64_t seed, uint64_t idx) {
    const uint64_t h = splitmix64(seed ^ (idx * 0xD1B54A32D192ED03ull));
    return (double)(h >> 11) * (1.0 / 9007199254740992.0);
}

template <typename T>
__global__ void adv_fill_kernel(T *data, int64_t lines, int64_t n1, int64_t n2, int64_t gline0,
                                double minX, double dx, int mode, double amp, uint64_t seed) {
    const double pi = 3.14159265358979323846;
    const int64_t total = lines * n1 * n2;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i1 = (i / n2) % n1;
        const double x = minX + (double)i1 * dx;
        double v;
        if (mode == 0) {
            v = sin(4 * x * pi);
        } else {
            const uint64_t gidx = (uint64_t)(gline0 * n1 * n2 + i);
            v = sin(2 * pi * x) + amp * (2.0 * uniform01(seed, gidx) - 1.0);
        }
        data[i] = (T)v;
    }
}

template <typename TA, typename TB>
__global__ void err_norm_kernel(const TA *a, const TB *b, int64_t n, double *partials) {
    double mx = 0, mref = 0, se = 0, sr = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double x = (double)a[i], r = (double)b[i];
        const double d = x - r;
        mx = fmax(mx, fabs(d));
        mref = fmax(mref, fabs(r));
        se += d * d;
        sr += r * r;
    }
    __shared__ double sh[4][32];
    for (int o = 16; o > 0; o >>= 1) {
        mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        mref = fmax(mref, __shfl_xor_sync(0xffffffffu, mref, o));
        se += __shfl_xor_sync(0xffffffffu, se, o);
        sr += __shfl_xor_sync(0xffffffffu, sr, o);
    }
    const int w = threadIdx.x / 32, l = threadIdx.x % 32;
    if (l == 0) {
        sh[0][w] = mx;
        sh[1][w] = mref;
        sh[2][w] = se;
        sh[3][w] = sr;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const int nw = blockDim.x / 32;
        for (int k = 1; k < nw; ++k) {
            sh[0][0] = fmax(sh[0][0], sh[0][k]);
            sh[1][0] = fmax(sh[1][0], sh[1][k]);
            sh[2][0] += sh[2][k];
            sh[3][0] += sh[3][k];
        }
        for (int q = 0; q < 4; ++q) partials[blockIdx.x * 4 + q] = sh[q][0];
    }
}

// Sum over (i0, i1) of |f - sin(4 pi (x - v t))| for every i2 into
// sums[n2]; the line velocity is the plan's own (reference law or array).
// When n2 fits a block, each thread keeps one i2 column and adds its partial
// sum once; otherwise columns are spread over threads.
template <typename T>
__global__ void validate_kernel(const T *f, int64_t lines, int64_t n1, int64_t n2,
                                const double *vx, double minX, double dx, double t,
                                double *sums) {
    const double pi = 3.14159265358979323846;
    const int64_t nrows = lines * n1;
    if (n2 <= blockDim.x) {
        const int rpb = blockDim.x / (int)n2;
        const int i2 = threadIdx.x % (int)n2;
        const int roff = threadIdx.x / (int)n2;
        if (roff >= rpb) return;
        double acc = 0.0;
        for (int64_t row = (int64_t)blockIdx.x * rpb + roff; row < nrows;
             row += (int64_t)gridDim.x * rpb) {
            const int64_t i1 = row % n1, i0 = row / n1;
            const double x = minX + (double)i1 * dx;
            acc += fabs((double)f[row * n2 + i2] - sin(4 * pi * (x - vx[i0] * t)));
        }
        atomicAdd(&sums[i2], acc);
    } else {
        for (int64_t row = blockIdx.x; row < nrows; row += gridDim.x) {
            const int64_t i1 = row % n1, i0 = row / n1;
            const double x = minX + (double)i1 * dx;
            const double value = sin(4 * pi * (x - vx[i0] * t));
            for (int64_t i2 = threadIdx.x; i2 < n2; i2 += blockDim.x)
                atomicAdd(&sums[i2], fabs((double)f[row * n2 + i2] - value));
        }
    }
}

}  // namespace bkma

using namespace bkma;

namespace {
constexpr int kNormBlocks = 1024;
}

extern "C" {

bkma_status bkma_adv_fill(const bkma_adv_plan *plan, void *data, int32_t mode, double amp,
                          uint64_t seed, void *stream) try {
    BKMA_CHECK_ARG(plan && data, "null argument");
    BKMA_CHECK_ARG(mode == 0 || mode == 1, "mode must be 0 or 1");
    const AdvPlanImpl &p = plan_impl(plan);
    cudaStream_t st = (cudaStream_t)stream;
    const int blocks = 152 * 8, threads = 256;
    if (p.desc.dtype == BKMA_F32)
        adv_fill_kernel<float><<<blocks, threads, 0, st>>>((float *)data, p.lines, p.desc.n1,
                                                          p.desc.n2, p.desc.i0_offset,
                                                          p.phys.minX, p.phys.dx, mode, amp, seed);
    else
        adv_fill_kernel<double><<<blocks, threads, 0, st>>>((double *)data, p.lines, p.desc.n1,
                                                           p.desc.n2, p.desc.i0_offset,
                                                           p.phys.minX, p.phys.dx, mode, amp,
                                                           seed);
    BKMA_CUDA_TRY(cudaGetLastError());
    return BKMA_OK;
} BKMA_ABI_CATCH("bkma_adv_fill")

bkma_status bkma_adv_error_norms(const bkma_adv_plan *plan, const void *data, int32_t data_dtype,
                                 const void *ref, int32_t ref_dtype, double *out, void *stream) try {
    BKMA_CHECK_ARG(plan && data && ref && out, "null argument");
    BKMA_CHECK_ARG((data_dtype == BKMA_F32 || data_dtype == BKMA_F64) &&
                       (ref_dtype == BKMA_F32 || ref_dtype == BKMA_F64),
                   "dtypes must be BKMA_F32 or BKMA_F64");
    AdvPlanImpl &p = plan_impl(const_cast<bkma_adv_plan *>(plan));
    cudaStream_t st = (cudaStream_t)stream;
    if (!p.d_partials) BKMA_CUDA_TRY(cudaMalloc(&p.d_partials, sizeof(double) * 4 * kNormBlocks));
    const int64_t n = p.lines * p.desc.n1 * p.desc.n2;
    if (data_dtype == BKMA_F32 && ref_dtype == BKMA_F64)
        err_norm_kernel<<<kNormBlocks, 256, 0, st>>>((const float *)data, (const double *)ref, n,
                                                     p.d_partials);
    else if (data_dtype == BKMA_F32 && ref_dtype == BKMA_F32)
        err_norm_kernel<<<kNormBlocks, 256, 0, st>>>((const float *)data, (const float *)ref, n,
                                                     p.d_partials);
    else if (data_dtype == BKMA_F64 && ref_dtype == BKMA_F64)
        err_norm_kernel<<<kNormBlocks, 256, 0, st>>>((const double *)data, (const double *)ref, n,
                                                     p.d_partials);
    else
        err_norm_kernel<<<kNormBlocks, 256, 0, st>>>((const double *)data, (const float *)ref, n,
                                                     p.d_partials);
    BKMA_CUDA_TRY(cudaGetLastError());
    std::vector<double> h(4 * kNormBlocks);
    BKMA_CUDA_TRY(cudaMemcpyAsync(h.data(), p.d_partials, sizeof(double) * h.size(),
                                  cudaMemcpyDeviceToHost, st));
    BKMA_CUDA_TRY(cudaStreamSynchronize(st));
    double r[4] = {0, 0, 0, 0};
    for (int b = 0; b < kNormBlocks; ++b) {
        r[0] = std::fmax(r[0], h[b * 4 + 0]);
        r[1] = std::fmax(r[1], h[b * 4 + 1]);
        r[2] += h[b * 4 + 2];
        r[3] += h[b * 4 + 3];
    }
    for (int q = 0; q < 4; ++q) out[q] = r[q];
    return BKMA_OK;
} BKMA_ABI_CATCH("bkma_adv_error_norms")

bkma_status bkma_adv_validate(const bkma_adv_plan *plan, const void *data, int64_t max_iter,
                              double *highest_l1, double *lowest_l1, void *stream) try {
    BKMA_CHECK_ARG(plan && data, "null argument");
    const AdvPlanImpl &p = plan_impl(plan);
    cudaStream_t st = (cudaStream_t)stream;
    const int64_t n2 = p.desc.n2;
    std::vector<double> h((size_t)n2);  // before the device buffers: a throw leaks nothing
    double *sums = nullptr;
    double *vx = nullptr;
    BKMA_CUDA_TRY(cudaMalloc(&sums, sizeof(double) * (size_t)n2));
    cudaError_t e = cudaMalloc(&vx, sizeof(double) * (size_t)p.lines);
    if (e == cudaSuccess) e = cudaMemsetAsync(sums, 0, sizeof(double) * n2, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(vx, p.vx.data(), sizeof(double) * p.lines, cudaMemcpyHostToDevice, st);
    const double t = (double)max_iter * p.phys.dt;
    if (e == cudaSuccess) {
        if (p.desc.dtype == BKMA_F32)
            validate_kernel<<<152 * 8, 256, 0, st>>>((const float *)data, p.lines, p.desc.n1, n2,
                                                     vx, p.phys.minX, p.phys.dx, t, sums);
        else
            validate_kernel<<<152 * 8, 256, 0, st>>>((const double *)data, p.lines, p.desc.n1, n2,
                                                     vx, p.phys.minX, p.phys.dx, t, sums);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(h.data(), sums, sizeof(double) * n2, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(sums);
    cudaFree(vx);
    if (e != cudaSuccess) return cuda_fail(e, "bkma_adv_validate");
    double hi = 0, lo = 0;
    for (int64_t i2 = 0; i2 < n2; ++i2) {
        const double l1 = h[(size_t)i2] / (double)(p.desc.n1 * p.lines);
        if (i2 == 0 || l1 > hi) hi = l1;
        if (i2 == 0 || l1 < lo) lo = l1;
    }
    if (highest_l1) *highest_l1 = hi;
    if (lowest_l1) *lowest_l1 = lo;
    return BKMA_OK;
} BKMA_ABI_CATCH("bkma_adv_validate")

}  // extern "C"
