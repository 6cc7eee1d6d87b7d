// In-place 1D convolution (the reference's ConvSolver driven by AdaptiveWg
// with window() = K: src/solvers/ConvSolver.hpp:7-45,
// src/core/AdaptiveWg.hpp:82-83,123-134), rebuilt for sm_103a.
//
// Two semantics:
//  - REFERENCE: bit-identical FP64 restatement of ConvSolver + AdaptiveWg on
//    data (n0, C*L, n2): output iw = ii1-(K-1) of a line is
//    bias[oc] + sum_ic sum_k [i_l-k >= 0] line[i_l-k] * W(k,ic,oc) with
//    oc = ii1/L, i_l = ii1%L; it only ever reads the first L samples of a
//    line, so a CTA stages those, then overwrites the line in place.
//  - TORCH: out[b,co,l] = bias[co] + sum_ci sum_k w[co,ci,k] x[b,ci,l+k],
//    l < L-K+1, layout (B, C, L). In place, tile t of a row overwrites
//    columns [l0, l0+TL) that tile t-1 still reads as its right halo. A
//    pre-pass copies every tile's right halo (Cin x (K-1) columns) into plan
//    scratch; the compute kernel then reads its halo from there, so tiles of
//    one row run concurrently with no ordering between CTAs.
//
// The BF16 tensor-core path (conv_tc.cu) runs each CTA's tiles in order and
// snapshots only the rows past each CTA's last tile.
#include <algorithm>
#include <cstring>
#include <memory>
#include <string>

#include "common.cuh"
#include "conv.cuh"

namespace bkma {

// ------------------------------------------------------------ reference

// One CTA = one i0 slab x W columns (i2) x the first L rows of each line.
__global__ void __launch_bounds__(256) conv_ref_kernel(ConvRefArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double *sm = reinterpret_cast<double *>(smem_raw);
    const int64_t ncb = (a.n2 + a.W - 1) / a.W;
    const int64_t i0 = blockIdx.x / ncb;
    const int64_t c0 = (blockIdx.x - i0 * ncb) * a.W;
    const int wc = (int)min((int64_t)a.W, a.n2 - c0);
    const int L = (int)a.length;
    const double *src = a.src + i0 * a.n1 * a.n2 + c0;
    double *dst = a.dst + i0 * a.n1 * a.n2 + c0;
    for (int i = threadIdx.x; i < L * wc; i += blockDim.x) {
        const int r = i / wc, c = i - r * wc;
        sm[i] = src[(int64_t)r * a.n2 + c];
    }
    __syncthreads();
    const int64_t nw = a.n1 - (a.K - 1);
    const int64_t total = nw * wc;
    const int64_t cout = a.cin;
    for (int64_t i = threadIdx.x; i < total; i += blockDim.x) {
        const int64_t iw = i / wc;
        const int c = (int)(i - iw * wc);
        const uint64_t ii1 = (uint64_t)(iw + a.K - 1);
        const uint64_t oc = ii1 / (uint64_t)a.length;
        const uint64_t i_l = ii1 - oc * (uint64_t)a.length;
        double sum = a.bias[oc];
        for (int ic = 0; ic < a.cin; ++ic) {
            for (int k = 0; k < a.K; ++k) {
                const int input_idx = (int)(int64_t)(i_l - (uint64_t)(int64_t)k);
                if ((uint64_t)(int64_t)input_idx < (uint64_t)a.n1) {
                    sum = dadd(sum, dmul(sm[input_idx * wc + c],
                                         a.weight[((int64_t)k * a.cin + ic) * cout + (int64_t)oc]));
                }
            }
        }
        dst[iw * a.n2 + c] = sum;
    }
}

// ---------------------------------------------------------------- torch

// Copy the right halo of every tile: halo[b][t][ci][j] = x[b][ci][(t+1)*TL + j]
// for j < K-1, zero for K-1 <= j < hw (hw >= K-1 pads rows to a vector width;
// columns past L are zero and never used).
template <typename T>
__global__ void conv_halo_kernel(const T *x, T *halo, int64_t B, int64_t cin, int64_t L,
                                 int K, int TL, int64_t ntiles, int hw) {
    const int hk = hw;
    const int64_t total = B * ntiles * cin * hk;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
         i += (int64_t)gridDim.x * blockDim.x) {
        int64_t r = i;
        const int j = (int)(r % hk);
        r /= hk;
        const int64_t ci = r % cin;
        r /= cin;
        const int64_t t = r % ntiles;
        const int64_t b = r / ntiles;
        const int64_t col = (t + 1) * TL + j;
        halo[i] = (col < L && j < K - 1) ? x[(b * cin + ci) * L + col] : T(0);
    }
}

template <typename T>
__device__ __forceinline__ T mac(T acc, T a, T b);
template <>
__device__ __forceinline__ double mac<double>(double acc, double a, double b) {
    return dadd(acc, dmul(a, b));  // oracle order, no contraction
}
template <>
__device__ __forceinline__ float mac<float>(float acc, float a, float b) {
    return fmaf(a, b, acc);
}

// CTA = (row b, tile of TL output columns), all Cout. Shared memory holds
// x[b][:, l0 : l0+TL+K-1]; the last K-1 columns come from the halo snapshot
// when running in place.
template <typename T>
__global__ void __launch_bounds__(256) conv_torch_plain(ConvTorchArgs<T> a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *sm = reinterpret_cast<T *>(smem_raw);
    const int TL = a.TL;
    const int K = a.K;
    const int width = TL + K - 1;
    const int64_t t = blockIdx.x % a.ntiles;
    const int64_t b = blockIdx.x / a.ntiles;
    const int64_t l0 = t * TL;
    const int64_t lout = a.L - K + 1;
    for (int i = threadIdx.x; i < a.cin * width; i += blockDim.x) {
        const int ci = i / width, j = i - ci * width;
        const int64_t col = l0 + j;
        T v = T(0);
        if (j >= TL && a.halo) {
            v = a.halo[((b * a.ntiles + t) * a.cin + ci) * (K - 1) + (j - TL)];
        } else if (col < a.L) {
            v = a.x[(b * a.cin + ci) * a.L + col];
        }
        sm[i] = v;
    }
    __syncthreads();
    const int64_t ostride = a.out_stride;
    for (int i = threadIdx.x; i < a.cout * TL; i += blockDim.x) {
        const int co = i / TL, j = i - co * TL;
        const int64_t l = l0 + j;
        if (l >= lout) continue;
        T s = a.bias ? a.bias[co] : T(0);
        const T *wr = a.w + (int64_t)co * a.cin * K;
        for (int ci = 0; ci < a.cin; ++ci)
            for (int k = 0; k < K; ++k) s = mac<T>(s, wr[ci * K + k], sm[ci * width + j + k]);
        a.out[(b * a.cout + co) * ostride + l] = s;
    }
}

}  // namespace bkma

using namespace bkma;

namespace bkma {

bkma_status conv_halo_prepass(ConvPlanImpl &p, const void *x, cudaStream_t st) {
    const bkma_conv_desc &d = p.desc;
    const int blocks = 152 * 4;
    if (d.dtype == BKMA_F64)
        conv_halo_kernel<double><<<blocks, 256, 0, st>>>((const double *)x, (double *)p.d_halo,
                                                        d.batch, d.cin, d.length, (int)d.ksize,
                                                        p.TL, p.ntiles, p.halo_width);
    else if (d.dtype == BKMA_F32)
        conv_halo_kernel<float><<<blocks, 256, 0, st>>>((const float *)x, (float *)p.d_halo,
                                                       d.batch, d.cin, d.length, (int)d.ksize,
                                                       p.TL, p.ntiles, p.halo_width);
    else
        return fail(BKMA_ERR_UNSUPPORTED, "halo pre-pass: F32 or F64 only (BF16 runs on the tensor path)");
    BKMA_CUDA_TRY(cudaGetLastError());
    return BKMA_OK;
}

namespace {

template <typename T>
bkma_status run_torch_plain(ConvPlanImpl &p, void *data, void *out, const void *w,
                            const void *bias, cudaStream_t st) {
    const bkma_conv_desc &d = p.desc;
    const bool inplace = (out == nullptr || out == data);
    if (inplace) {
        bkma_status s = conv_halo_prepass(p, data, st);
        if (s != BKMA_OK) return s;
    }
    ConvTorchArgs<T> a;
    a.x = (const T *)data;
    a.out = (T *)(inplace ? data : out);
    a.w = (const T *)w;
    a.bias = (const T *)bias;
    a.halo = inplace ? (const T *)p.d_halo : nullptr;
    a.B = d.batch;
    a.cin = (int)d.cin;
    a.cout = (int)d.cout;
    a.L = d.length;
    a.K = (int)d.ksize;
    a.TL = p.TL;
    a.ntiles = p.ntiles;
    a.out_stride = inplace ? d.length : d.length - d.ksize + 1;
    const size_t smem = sizeof(T) * (size_t)(d.cin * (p.TL + d.ksize - 1));
    BKMA_CUDA_TRY(cudaFuncSetAttribute(conv_torch_plain<T>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    conv_torch_plain<T><<<grid_x(d.batch * p.ntiles), 256, smem, st>>>(a);
    BKMA_CUDA_TRY(cudaGetLastError());
    return BKMA_OK;
}

bkma_status run_reference(ConvPlanImpl &p, void *data, void *out, const void *w,
                          const void *bias, cudaStream_t st) {
    const bkma_conv_desc &d = p.desc;
    const bool inplace = (out == nullptr || out == data);
    ConvRefArgs a;
    a.src = (const double *)data;
    a.dst = (double *)(inplace ? data : out);
    a.weight = (const double *)w;
    a.bias = (const double *)bias;
    a.n1 = d.cin * d.length;
    a.n2 = d.n2;
    a.K = d.ksize;
    a.cin = (int)d.cin;
    a.length = d.length;
    a.W = (int)std::min<int64_t>(16, d.n2);
    const size_t smem = sizeof(double) * (size_t)(d.length * a.W);
    if (smem > 227 * 1024) return fail(BKMA_ERR_UNSUPPORTED, "length too long for the reference conv tile");
    if (!inplace) {
        // Out of place: copy the untouched tail (the last K-1 samples of
        // each line keep their values, as in place would).
        BKMA_CUDA_TRY(cudaMemcpyAsync(out, data, sizeof(double) * (size_t)(d.batch * a.n1 * d.n2),
                                      cudaMemcpyDeviceToDevice, st));
    }
    BKMA_CUDA_TRY(cudaFuncSetAttribute(conv_ref_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem));
    const int64_t ncb = (d.n2 + a.W - 1) / a.W;
    conv_ref_kernel<<<grid_x(d.batch * ncb), 256, smem, st>>>(a);
    BKMA_CUDA_TRY(cudaGetLastError());
    return BKMA_OK;
}

}  // namespace

bkma_status conv_check_desc(const bkma_conv_desc &d) {
    BKMA_CHECK_ARG(d.batch > 0 && d.cin > 0 && d.cout > 0 && d.length > 0 && d.ksize > 0,
                   "batch, cin, cout, length, ksize must be positive");
    BKMA_CHECK_ARG(d.ksize <= d.length, "ksize must not exceed length");
    BKMA_CHECK_ARG(d.semantics == BKMA_CONV_TORCH || d.semantics == BKMA_CONV_REFERENCE,
                   "unknown semantics");
    BKMA_CHECK_ARG(d.impl >= BKMA_CONV_AUTO && d.impl <= BKMA_CONV_PLAIN, "unknown impl");
    BKMA_CHECK_ARG(d.cin < 65536 && d.cout < 65536 && d.ksize < 4096, "channel count or ksize too large");
    // the kernels index rows and tiles with 32-bit fields
    BKMA_CHECK_ARG(d.batch < (1ll << 31) && d.length < (1ll << 40), "batch or length too large");
    if (d.semantics == BKMA_CONV_REFERENCE) {
        BKMA_CHECK_ARG(d.cout == d.cin, "reference semantics force channel_out = channel_in");
        BKMA_CHECK_ARG(d.dtype == BKMA_F64, "reference semantics run in FP64");
        BKMA_CHECK_ARG(d.impl != BKMA_CONV_TENSOR, "reference semantics have no tensor-core form");
        BKMA_CHECK_ARG(d.n2 > 0, "n2 must be positive");
    } else {
        BKMA_CHECK_ARG(d.n2 == 0 || d.n2 == 1, "torch semantics take n2 = 1");
        BKMA_CHECK_ARG(d.dtype == BKMA_F64 || d.dtype == BKMA_F32 || d.dtype == BKMA_BF16,
                       "dtype must be F64, F32 or BF16");
        if (d.inplace) BKMA_CHECK_ARG(d.cin == d.cout, "in place needs cin == cout");
    }
    return BKMA_OK;
}

}  // namespace bkma

extern "C" {

bkma_status bkma_conv_plan_create(const bkma_conv_desc *desc, bkma_conv_plan **plan) try {
    bkma::NvtxRange nvtx_range("bkma_conv_plan_create");
    BKMA_CHECK_ARG(desc && plan, "bkma_conv_plan_create: null argument");
    *plan = nullptr;
    const bkma_conv_desc &d = *desc;
    bkma_status cs = conv_check_desc(d);
    if (cs != BKMA_OK) return cs;
    // owned here until complete: an early return or an exception frees it
    std::unique_ptr<bkma_conv_plan> pl(new bkma_conv_plan);
    ConvPlanImpl &p = pl->impl;
    p.desc = d;
    if (p.desc.n2 == 0) p.desc.n2 = 1;
    cudaGetDevice(&p.device);
    bkma_status s = BKMA_OK;
    if (d.semantics == BKMA_CONV_TORCH) {
        const bool tensor = d.dtype == BKMA_BF16 && d.impl != BKMA_CONV_PLAIN;
        if (d.dtype == BKMA_BF16 && !tensor) s = fail(BKMA_ERR_UNSUPPORTED, "BF16 runs on the tensor path");
        if (s == BKMA_OK && tensor) {
            s = conv_tc_plan_init(p);
        } else if (s == BKMA_OK) {
            p.TL = 64;
            p.ntiles = (d.length - d.ksize + 1 + p.TL - 1) / p.TL;
            const size_t es = d.dtype == BKMA_F64 ? 8 : 4;
            const size_t smem = es * (size_t)(d.cin * (p.TL + d.ksize - 1));
            if (smem > 227 * 1024) s = fail(BKMA_ERR_UNSUPPORTED, "cin too large for the plain tile");
            p.halo_width = (int)(d.ksize - 1);
            p.halo_bytes = es * (size_t)(d.batch * p.ntiles * d.cin * p.halo_width);
        }
        if (s == BKMA_OK && d.inplace && p.halo_bytes > 0) {
            cudaError_t e = cudaMalloc(&p.d_halo, p.halo_bytes);
            if (e != cudaSuccess) s = cuda_fail(e, "conv halo scratch");
        }
    }
    if (s != BKMA_OK) return s;
    *plan = pl.release();
    return BKMA_OK;
} BKMA_ABI_CATCH("bkma_conv_plan_create")

bkma_status bkma_conv_plan_scratch_bytes(const bkma_conv_plan *plan, int64_t *bytes) try {
    BKMA_CHECK_ARG(plan && bytes, "null argument");
    *bytes = (int64_t)(plan->impl.halo_bytes + plan->impl.wpack_bytes);
    return BKMA_OK;
} BKMA_ABI_CATCH("bkma_conv_plan_scratch_bytes")

bkma_status bkma_conv_run(bkma_conv_plan *plan, void *data, void *out, const void *weight,
                          const void *bias, void *stream) try {
    bkma::NvtxRange nvtx_range("bkma_conv_run");
    BKMA_CHECK_ARG(plan && data && weight, "bkma_conv_run: null argument");
    ConvPlanImpl &p = plan->impl;
    const bkma_conv_desc &d = p.desc;
    cudaStream_t st = (cudaStream_t)stream;
    const bool inplace = (out == nullptr || out == data);
    if (inplace && d.semantics == BKMA_CONV_TORCH)
        BKMA_CHECK_ARG(d.inplace, "plan was created for out-of-place runs");
    if (d.semantics == BKMA_CONV_REFERENCE) {
        BKMA_CHECK_ARG(bias, "reference semantics need a bias");
        return run_reference(p, data, out, weight, bias, st);
    }
    if (p.tensor) return conv_tc_run(p, data, out, weight, bias, st);
    if (d.dtype == BKMA_F64) return run_torch_plain<double>(p, data, out, weight, bias, st);
    return run_torch_plain<float>(p, data, out, weight, bias, st);
} BKMA_ABI_CATCH("bkma_conv_run")

bkma_status bkma_conv_plan_status(bkma_conv_plan *plan, void *stream) try {
    BKMA_CHECK_ARG(plan, "null argument");
    ConvPlanImpl &p = plan->impl;
    BKMA_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
    if (!p.d_status) return BKMA_OK;
    int st = 0;
    BKMA_CUDA_TRY(cudaMemcpy(&st, p.d_status, sizeof(int), cudaMemcpyDeviceToHost));
    BKMA_CUDA_TRY(cudaMemset(p.d_status, 0, sizeof(int)));
    if (st != 0) return fail((bkma_status)st, "tensor-core conv1d: a bounded device wait timed out");
    return BKMA_OK;
} BKMA_ABI_CATCH("bkma_conv_plan_status")

bkma_status bkma_conv_plan_set_wait_limit(bkma_conv_plan *plan, uint32_t polls) try {
    BKMA_CHECK_ARG(plan, "null argument");
    plan->impl.wait_polls = polls;
    return BKMA_OK;
} BKMA_ABI_CATCH("bkma_conv_plan_set_wait_limit")

bkma_status bkma_conv_plan_destroy(bkma_conv_plan *plan) try {
    delete plan;
    return BKMA_OK;
} BKMA_ABI_CATCH("bkma_conv_plan_destroy")

}  // extern "C"
