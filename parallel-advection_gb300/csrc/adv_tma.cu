// TMA-staged FP32 advection kernel (the fast path of adv.cu's staged form).
//
// One CTA = one slab i0 x WC columns (i2) x all n1 rows. One thread issues
// cp.async.bulk.tensor 3-D boxes (WC x box_rows x 1) of the field into shared
// memory and every thread waits on one mbarrier (bounded). The wrap halo
// (rows 0..NT-2 repeated after row n1-1) is copied in shared memory. Each
// thread then owns a 4-column group of a row per pass: NT float4 tap loads
// with immediate offsets (WC is a template constant), the incremental form
// f_c + sum_k w_k (f_k - f_c) in packed FP32x2 FMAs, and one 16-byte store
// straight back to HBM. The tile was read completely before any store, so
// in place is legal.
//
// Used when n2 % 4 == 0, n2 >= WC and the field base is 16-byte aligned
// (TMA's stride/alignment rules); adv.cu keeps the cp.async form for the rest.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <mutex>

#include "adv.cuh"
#include "adv_plan.cuh"
#include "common.cuh"
#include "tma.cuh"

namespace bkma {

namespace {

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return smem_u32addr(p); }

constexpr uint32_t kTmaSpinLimit = kWaitPolls;

template <int NT, int WC>
__global__ void __launch_bounds__(512) adv_tma_f32(const __grid_constant__ CUtensorMap tmap,
                                                   AdvTmaArgs a) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bar;
    constexpr int C = NT / 2 - 1;
    constexpr int TPR = WC / 4;  // threads per row (one float4 each)
    // 128-byte aligned staging base
    const uint32_t raw = smem_addr(smem_raw);
    const uint32_t pad = ((raw + 127u) & ~127u) - raw;
    float *S = reinterpret_cast<float *>(smem_raw + pad);

    const int64_t line = blockIdx.x / a.ncb;
    const int c0 = (int)(blockIdx.x - line * a.ncb) * WC;
    const int n1 = (int)a.n1;

    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&bar)));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const uint32_t bytes = (uint32_t)(a.nbox * a.box_rows * WC * 4);
        asm volatile(
            "{\n .reg .b64 st;\n mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n}" ::"r"(
                smem_addr(&bar)),
            "r"(bytes)
            : "memory");
        for (int b = 0; b < a.nbox; ++b) {
            const uint32_t dst = smem_addr(S + (size_t)b * a.box_rows * WC);
            asm volatile(
                "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes "
                "[%0], [%1, {%2, %3, %4}], [%5];" ::"r"(dst),
                "l"(reinterpret_cast<uint64_t>(&tmap)), "r"(c0), "r"(b * a.box_rows),
                "r"((int)line), "r"(smem_addr(&bar))
                : "memory");
        }
    }
    // Line parameters while the copy is in flight.
    const int exc = a.exc_index[line];
    const int base = a.base[line];
    float2 w2[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) {
        const float wk = a.w[line * NT + k];
        w2[k] = make_float2(wk, wk);
    }
    // Every thread polls the barrier at most a.spin_limit times; the CTA then
    // agrees on one outcome. On a timeout the status word is raised and the
    // issuing thread stays until its copies have landed (a second bounded
    // wait), so that no copy writes into shared memory the CTA has left.
    const bool ok = __syncthreads_and(staging_wait(&bar, a.spin_limit));
    if (!ok) {
        if (threadIdx.x == 0) {
            atomicExch(a.status, (int)BKMA_ERR_TIMEOUT);
            staging_wait(&bar, kTmaSpinLimit);
        }
        return;
    }
    // wrap halo: rows n1 .. n1+NT-2 repeat rows 0 .. NT-2
    for (int i = threadIdx.x; i < (NT - 1) * WC; i += blockDim.x) S[n1 * WC + i] = S[i];
    __syncthreads();

    const int g = threadIdx.x % TPR;
    const int r0 = threadIdx.x / TPR;
    const int rpp = blockDim.x / TPR;
    const bool col_ok = (c0 + 4 * g) < a.n2;
    const float *Sb = S + 4 * g;
    float *Gp = a.dst + (line * a.n1 + r0) * a.n2 + c0 + 4 * g;
    const int64_t gstep = (int64_t)rpp * a.n2;
    const float2 m1 = make_float2(-1.0f, -1.0f);
    for (int r = r0; r < n1; r += rpp, Gp += gstep) {
        int rr;
        const AdvExcCell<float> *cell = nullptr;
        if (exc < 0) {
            rr = r + base;
        } else {
            cell = a.exc + (int64_t)exc * n1 + r;
            rr = r + cell->base;
        }
        if (rr >= n1) rr -= n1;
        const float *p = Sb + rr * WC;
        float4 f[NT];
#pragma unroll
        for (int k = 0; k < NT; ++k) f[k] = *reinterpret_cast<const float4 *>(p + k * WC);
        const float2 cl = make_float2(f[C].x, f[C].y);
        const float2 ch = make_float2(f[C].z, f[C].w);
        float2 al = make_float2(0.f, 0.f), ah = make_float2(0.f, 0.f);
#pragma unroll
        for (int k = 0; k < NT; ++k) {
            if (k == C) continue;
            float2 wk = w2[k];
            if (exc >= 0) wk = make_float2(cell->w[k], cell->w[k]);
            const float2 dl = __ffma2_rn(cl, m1, make_float2(f[k].x, f[k].y));
            const float2 dh = __ffma2_rn(ch, m1, make_float2(f[k].z, f[k].w));
            al = __ffma2_rn(wk, dl, al);
            ah = __ffma2_rn(wk, dh, ah);
        }
        const float2 ol = __fadd2_rn(cl, al);
        const float2 oh = __fadd2_rn(ch, ah);
        if (col_ok) *reinterpret_cast<float4 *>(Gp) = make_float4(ol.x, ol.y, oh.x, oh.y);
    }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static std::once_flag once;
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    std::call_once(once, [] {
        cudaDriverEntryPointQueryResult q;
        void *p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

}  // namespace

void *tensor_map_encoder() { return reinterpret_cast<void *>(encode_fn()); }

namespace {

template <int NT, int WC>
cudaError_t launch_tma_t(const CUtensorMap &tm, const AdvTmaArgs &a, int threads, size_t smem,
                         int64_t grid, cudaStream_t st) {
    auto kern = adv_tma_f32<NT, WC>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<grid_x(grid), threads, smem, st>>>(tm, a);
    return cudaGetLastError();
}

}  // namespace

bool adv_tma_eligible(const AdvPlanImpl &p, const void *src, int W) {
    return p.desc.dtype == BKMA_F32 && p.desc.impl != BKMA_ADV_PLAIN &&
           (W == 8 || W == 16 || W == 32) && (p.npts == 4 || p.npts == 6) &&
           p.desc.n2 % 4 == 0 && p.desc.n2 >= W && ((uintptr_t)src % 16) == 0 &&
           p.lines < (1ll << 31) && encode_fn() != nullptr;
}

size_t adv_tma_smem(const AdvPlanImpl &p, int W) {
    const int64_t n1 = p.desc.n1;
    const int box_rows = (int)std::min<int64_t>(256, n1);
    const int64_t nbox = (n1 + box_rows - 1) / box_rows;
    const int64_t rows = std::max<int64_t>(nbox * box_rows, n1 + p.npts - 1);
    return (size_t)rows * W * 4 + 128;
}

const CUtensorMap *adv_field_tmap(AdvPlanImpl &p, const void *src, int W) {
    for (auto &c : p.tmaps)
        if (c.ptr == src && c.W == W) return &c.map;
    if (!encode_fn()) return nullptr;
    AdvPlanImpl::TmapCache c;
    c.ptr = src;
    c.W = W;
    const int box_rows = (int)std::min<int64_t>(256, p.desc.n1);
    const cuuint64_t es = (cuuint64_t)p.esize;
    const cuuint64_t dims[3] = {(cuuint64_t)p.desc.n2, (cuuint64_t)p.desc.n1, (cuuint64_t)p.lines};
    const cuuint64_t strides[2] = {(cuuint64_t)p.desc.n2 * es, (cuuint64_t)(p.desc.n1 * p.desc.n2) * es};
    const cuuint32_t box[3] = {(cuuint32_t)W, (cuuint32_t)box_rows, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    const CUtensorMapDataType dt =
        p.esize == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
    CUresult r = encode_fn()(&c.map, dt, 3, const_cast<void *>(src), dims, strides, box, estr,
                             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return nullptr;
    if (p.tmaps.size() >= 4) p.tmaps.erase(p.tmaps.begin());
    p.tmaps.push_back(c);
    return &p.tmaps.back().map;
}

cudaError_t adv_tma_launch(AdvPlanImpl &p, const void *src, void *dst, int W, int threads,
                           cudaStream_t st) {
    // tensor map of the source field (cached per pointer)
    const CUtensorMap *tm = adv_field_tmap(p, src, W);
    if (!tm) return cudaErrorInvalidValue;
    AdvTmaArgs a;
    a.dst = (float *)dst;
    a.n1 = p.desc.n1;
    a.n2 = p.desc.n2;
    a.ncb = p.ncb(W);
    a.box_rows = (int)std::min<int64_t>(256, p.desc.n1);
    a.nbox = (int)((p.desc.n1 + a.box_rows - 1) / a.box_rows);
    a.base = p.d_base;
    a.w = (const float *)p.d_w;
    a.exc_index = p.d_exc_index;
    a.exc = (const AdvExcCell<float> *)p.d_exc;
    a.status = p.d_status;
    a.spin_limit = p.wait_polls;
    const size_t smem = adv_tma_smem(p, W);
    const int64_t grid = p.lines * a.ncb;
    if (p.npts == 6) {
        if (W == 16) return launch_tma_t<6, 16>(*tm, a, threads, smem, grid, st);
        if (W == 8) return launch_tma_t<6, 8>(*tm, a, threads, smem, grid, st);
        return launch_tma_t<6, 32>(*tm, a, threads, smem, grid, st);
    }
    if (W == 16) return launch_tma_t<4, 16>(*tm, a, threads, smem, grid, st);
    if (W == 8) return launch_tma_t<4, 8>(*tm, a, threads, smem, grid, st);
    return launch_tma_t<4, 32>(*tm, a, threads, smem, grid, st);
}

}  // namespace bkma
