// Contiguous-line FP32 advection (n2 = 1): every line is n1 consecutive
// floats, so a run of whole lines is one contiguous block of the field.
//
// A CTA stages R consecutive lines (R * n1 floats) into shared memory with
// one bulk copy (cp.async.bulk, completed on an mbarrier; the block starts on
// a 16-byte boundary and is a multiple of 16 bytes long: n1 % 4 == 0 and a
// 16-byte-aligned field; against 16-byte cp.async from every thread:
// 2^21 lines of 1024 784 -> 836 GCells/s, 2^17 lines of 16384 784 -> 803,
// 2^27 lines of 16 665 -> 669), then each thread computes 4 consecutive cells of
// one line from a register window of npts + 3 staged values (the taps of 4
// neighbouring cells overlap), read as aligned float4s (contiguous across the
// lanes of a line: no bank conflicts; the periodic wrap falls on float4
// boundaries) and shifted in registers by base % 4,
// with the staged kernels' arithmetic f_c + sum_k w_k (f_k - f_c) in the
// same order (same bits), and writes them with one 16-byte store. The CTA
// has read all of its lines before any store and no other CTA touches them,
// so in place is legal. Exception lines (offset not constant along n1) use
// their per-cell stencils.
//
// This replaces the whole-slab staging of the generic kernel for the
// reference's n2 = 1 shapes (benchmark/bench_config.hpp: 2^27 lines of 16
// cells, 2^21 lines of 1024, 2^17 lines of 16384), where one CTA per slab
// or per-cell index arithmetic leaves HBM idle.
#include "adv.cuh"
#include "adv_device.cuh"
#include "adv_plan.cuh"
#include "common.cuh"
#include "tma.cuh"

namespace bkma {

namespace {

constexpr int kRowsThreads = 256;

// `polls` bounds the wait for the staged block; on a timeout the CTA raises
// `status`, lets its copy land (a second bounded wait) and leaves without
// writing.
template <int NT>
__global__ void __launch_bounds__(kRowsThreads) adv_rows_f32(AdvStagedArgs<float> a, int *status,
                                                             uint32_t polls) {
    extern __shared__ __align__(16) float S[];
    __shared__ __align__(8) uint64_t bar;
    constexpr int C = NT / 2 - 1;
    const int n1 = (int)a.n1;
    const int64_t line0 = (int64_t)blockIdx.x * a.R;
    const int nl = (int)min((int64_t)a.R, a.lines - line0);
    const int total = nl * n1;  // a multiple of 4
    const float *g = a.src + line0 * a.n1;
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32addr(&bar)));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const uint32_t bytes = (uint32_t)total * 4u;
        asm volatile(
            "{\n .reg .b64 st;\n mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n}" ::"r"(
                smem_u32addr(&bar)),
            "r"(bytes)
            : "memory");
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
                "r"(smem_u32addr(S)),
            "l"(g), "r"(bytes), "r"(smem_u32addr(&bar))
            : "memory");
    }
    if (!__syncthreads_and(staging_wait(&bar, polls))) {
        if (threadIdx.x == 0) {
            atomicExch(status, (int)BKMA_ERR_TIMEOUT);
            staging_wait(&bar, kWaitPolls);
        }
        return;
    }
    float *G = a.dst + line0 * a.n1;
    for (int i = (int)threadIdx.x * 4; i < total; i += kRowsThreads * 4) {
        const int l = i / n1;
        const int c0 = i - l * n1;
        const int64_t line = line0 + l;
        const float *Sl = S + l * n1;
        const int exc = a.exc_index ? a.exc_index[line] : -1;
        float o[4];
        if (exc < 0) {
            float w[NT];
#pragma unroll
            for (int k = 0; k < NT; ++k) w[k] = a.w[line * NT + k];
            int q = c0 + a.base[line];
            if (q >= n1) q -= n1;
            // the window starts q & 3 floats into an aligned float4 (q & 3 =
            // base & 3: the same for every thread of a line); aligned float4
            // loads are contiguous across the lanes of a line, and n1 % 4 == 0
            // keeps the wrap on float4 boundaries
            constexpr int NV = (NT + 3 + 3 + 3) / 4;  // window + shift <= 3, in float4s
            static_assert(4 * NV >= NT + 3 + 3, "window");
            float v[4 * NV];
            int q4 = q & ~3;
#pragma unroll
            for (int j = 0; j < NV; ++j) {
                const float4 t = *reinterpret_cast<const float4 *>(Sl + q4);
                v[4 * j] = t.x;
                v[4 * j + 1] = t.y;
                v[4 * j + 2] = t.z;
                v[4 * j + 3] = t.w;
                q4 = q4 + 4 == n1 ? 0 : q4 + 4;
            }
            float f[NT + 3];
            switch (q & 3) {
#define BKMA_ROWS_SHIFT(sh)                                   \
    case sh:                                                  \
        _Pragma("unroll") for (int j = 0; j < NT + 3; ++j) f[j] = v[j + sh]; \
        break;
                BKMA_ROWS_SHIFT(0)
                BKMA_ROWS_SHIFT(1)
                BKMA_ROWS_SHIFT(2)
                BKMA_ROWS_SHIFT(3)
#undef BKMA_ROWS_SHIFT
            }
#pragma unroll
            for (int m = 0; m < 4; ++m) {
                const float fc = f[m + C];
                float acc = 0.f;
#pragma unroll
                for (int k = 0; k < NT; ++k)
                    if (k != C) acc = fmaf(w[k], f[m + k] - fc, acc);
                o[m] = fc + acc;
            }
        } else {
            const AdvExcCell<float> *cells = a.exc + (int64_t)exc * n1;
#pragma unroll
            for (int m = 0; m < 4; ++m) {
                const AdvExcCell<float> &e = cells[c0 + m];
                int q = c0 + m + e.base;
                if (q >= n1) q -= n1;
                float f[NT];
#pragma unroll
                for (int k = 0; k < NT; ++k) {
                    f[k] = Sl[q];
                    q = q + 1 == n1 ? 0 : q + 1;
                }
                const float fc = f[C];
                float acc = 0.f;
#pragma unroll
                for (int k = 0; k < NT; ++k)
                    if (k != C) acc = fmaf(e.w[k], f[k] - fc, acc);
                o[m] = fc + acc;
            }
        }
        *reinterpret_cast<float4 *>(G + i) = make_float4(o[0], o[1], o[2], o[3]);
    }
}

template <int NT>
cudaError_t launch_rows(const AdvPlanImpl &p, const void *src, void *dst, int R, cudaStream_t st) {
    AdvStagedArgs<float> a{};
    a.src = (const float *)src;
    a.dst = (float *)dst;
    a.n1 = p.desc.n1;
    a.n2 = 1;
    a.lines = p.lines;
    a.W = 1;
    a.R = R;
    a.ncb = 1;
    a.base = p.d_base;
    a.w = (const float *)p.d_w;
    // no exception lines: the kernel skips the index (4 of the 32 table
    // bytes a 16-cell line reads)
    a.exc_index = p.n_exc > 0 ? p.d_exc_index : nullptr;
    a.exc = (const AdvExcCell<float> *)p.d_exc;
    a.line_list = nullptr;
    const size_t smem = adv_rows_smem(p, R);
    auto kern = adv_rows_f32<NT>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    const int64_t grid = (p.lines + R - 1) / R;
    kern<<<grid_x(grid), kRowsThreads, smem, st>>>(a, p.d_status, p.wait_polls);
    return cudaGetLastError();
}

}  // namespace

size_t adv_rows_smem(const AdvPlanImpl &p, int R) {
    return (size_t)R * (size_t)p.desc.n1 * sizeof(float);
}

bool adv_rows_shape_ok(const AdvPlanImpl &p) {
    return p.desc.dtype == BKMA_F32 && p.desc.impl != BKMA_ADV_PLAIN && p.desc.n2 == 1 &&
           p.desc.n1 % 4 == 0 && p.desc.n1 >= 16 && p.lines * p.desc.n1 < (1ll << 40) &&
           (p.npts == 4 || p.npts == 6 || p.npts == 10);
}

bool adv_rows_eligible(const AdvPlanImpl &p, const void *src, const void *dst, int R) {
    return adv_rows_shape_ok(p) && R >= 1 && ((uintptr_t)src % 16) == 0 &&
           ((uintptr_t)dst % 16) == 0 && (int64_t)R * p.desc.n1 <= (1 << 20) &&
           adv_rows_smem(p, R) <= (size_t)227 * 1024 - 16;  // + the static barrier
}

int adv_rows_default_r(const AdvPlanImpl &p) {
    // about 8192 cells (32 KB of shared memory) per CTA, whole lines; 4096
    // for lines shorter than 256 (2^27 lines of 16: 528 -> 579 GCells/s)
    const int64_t target = p.desc.n1 < 256 ? 4096 : 8192;
    const int64_t r = std::max<int64_t>(1, target / p.desc.n1);
    return (int)std::min<int64_t>(r, p.lines);
}

cudaError_t adv_rows_launch(const AdvPlanImpl &p, const void *src, void *dst, int R,
                            cudaStream_t st) {
    switch (p.npts) {
    case 4: return launch_rows<4>(p, src, dst, R, st);
    case 6: return launch_rows<6>(p, src, dst, R, st);
    case 10: return launch_rows<10>(p, src, dst, R, st);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace bkma
