// Device helpers of the conv1d driver: constant fills (fill_buffer_conv1d,
// src/tools/init.hpp:50-72) and the conv1d result checks in one pass over
// the device field (sum_and_normalize_conv1d and validate_conv1d,
// src/tools/validation.hpp:84-156): the mean of the first nw values of every
// (i0, i2) line, and whether every value at a given i1 < nw is the same
// across all (i0, i2).
#include <cuda_bf16.h>

#include <algorithm>
#include <vector>

#include "common.cuh"

namespace bkma {
namespace {

constexpr int kCheckBlocks = 1024;
constexpr int kCheckThreads = 256;

template <typename T>
__device__ __forceinline__ double as_f64(T v) {
    return (double)v;
}
template <>
__device__ __forceinline__ double as_f64<__nv_bfloat16>(__nv_bfloat16 v) {
    return (double)__bfloat162float(v);
}

template <typename T>
__global__ void fill_kernel(T *data, int64_t count, T value) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count;
         i += (int64_t)gridDim.x * blockDim.x)
        data[i] = value;
}

// Block b sums its share of the (i0, i1 < nw, i2) cells in FP64 and flags a
// value other than data(0, i1, 0) that differs from it (a NaN compares
// unequal, as in the reference's != test, which compares neighbours along i2
// and along i0: the same as all equal to the first); the host adds the block
// partials in order.
template <typename T>
__global__ void conv_check_kernel(const T *__restrict__ data, int64_t n0, int64_t n1, int64_t n2,
                                  int64_t nw, double *partial, int *differ) {
    __shared__ double red[kCheckThreads];
    const int64_t total = n0 * nw * n2;
    double sum = 0.0;
    int diff = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i2 = i % n2;
        const int64_t r = i / n2;
        const int64_t i1 = r % nw;
        const int64_t i0 = r / nw;
        const T v = data[(i0 * n1 + i1) * n2 + i2];
        sum += as_f64(v);
        if ((i0 | i2) != 0 && !(as_f64(v) == as_f64(data[i1 * n2]))) diff = 1;
    }
    red[threadIdx.x] = sum;
    if (__syncthreads_or(diff) && threadIdx.x == 0) atomicOr(differ, 1);
    for (int s = kCheckThreads / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

template <typename T>
bkma_status check_t(const void *data, int64_t n0, int64_t n1, int64_t n2, int64_t nw,
                    double *mean, int32_t *equal, cudaStream_t st) {
    std::vector<double> h(kCheckBlocks);  // before the device buffer: a throw leaks nothing
    double *d_partial = nullptr;
    int *d_differ = nullptr;
    BKMA_CUDA_TRY(cudaMalloc(&d_partial, sizeof(double) * kCheckBlocks + sizeof(int) * 4));
    d_differ = reinterpret_cast<int *>(d_partial + kCheckBlocks);
    cudaError_t e = cudaMemsetAsync(d_differ, 0, sizeof(int), st);
    if (e == cudaSuccess) {
        conv_check_kernel<T><<<kCheckBlocks, kCheckThreads, 0, st>>>(
            (const T *)data, n0, n1, n2, nw, d_partial, d_differ);
        e = cudaGetLastError();
    }
    int differ = 0;
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(h.data(), d_partial, sizeof(double) * kCheckBlocks,
                            cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(&differ, d_differ, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(d_partial);
    if (e != cudaSuccess) return cuda_fail(e, "conv check");
    double sum = 0.0;
    for (double v : h) sum += v;
    if (mean) *mean = sum / (double)(n0 * nw * n2);
    if (equal) *equal = differ ? 0 : 1;
    return BKMA_OK;
}

}  // namespace
}  // namespace bkma

using namespace bkma;

extern "C" {

bkma_status bkma_fill(void *data, int64_t count, int32_t dtype, double value, void *stream) try {
    BKMA_CHECK_ARG(data && count >= 0, "bkma_fill: bad arguments");
    if (count == 0) return BKMA_OK;
    cudaStream_t st = (cudaStream_t)stream;
    const int grid = (int)std::min<int64_t>(4096, (count + 255) / 256);
    switch (dtype) {
    case BKMA_F32: fill_kernel<float><<<grid, 256, 0, st>>>((float *)data, count, (float)value); break;
    case BKMA_F64: fill_kernel<double><<<grid, 256, 0, st>>>((double *)data, count, value); break;
    case BKMA_BF16:
        fill_kernel<__nv_bfloat16><<<grid, 256, 0, st>>>((__nv_bfloat16 *)data, count,
                                                         __float2bfloat16_rn((float)value));
        break;
    default: return fail(BKMA_ERR_INVALID_ARG, "bkma_fill: dtype must be F32, F64 or BF16");
    }
    BKMA_CUDA_TRY(cudaGetLastError());
    return BKMA_OK;
} BKMA_ABI_CATCH("bkma_fill")

bkma_status bkma_conv_check(const void *data, int32_t dtype, int64_t n0, int64_t n1, int64_t n2,
                            int64_t nw, double *mean, int32_t *equal, void *stream) try {
    BKMA_CHECK_ARG(data && n0 > 0 && n1 > 0 && n2 > 0 && nw > 0 && nw <= n1,
                   "bkma_conv_check: need n0, n1, n2 > 0 and 0 < nw <= n1");
    cudaStream_t st = (cudaStream_t)stream;
    switch (dtype) {
    case BKMA_F32: return check_t<float>(data, n0, n1, n2, nw, mean, equal, st);
    case BKMA_F64: return check_t<double>(data, n0, n1, n2, nw, mean, equal, st);
    case BKMA_BF16: return check_t<__nv_bfloat16>(data, n0, n1, n2, nw, mean, equal, st);
    default: return fail(BKMA_ERR_INVALID_ARG, "bkma_conv_check: dtype must be F32, F64 or BF16");
    }
} BKMA_ABI_CATCH("bkma_conv_check")

}  // extern "C"
