// Streamed FP64 advection in FP32-pair arithmetic (path 6).
//
// The column-pair kernel (adv_ds.cu) stages whole column strips in shared
// memory: a strip of 16384 rows does not fit, rows 16 MB apart make every TMA
// box row its own DRAM page, and each of its 16-row runs re-splits npts - 1
// taps. This form streams instead, like the FP32 streamed kernel
// (adv_stream.cu):
//
//  * work unit: a group of 32 column pairs (64 consecutive columns of the
//    field's (line, i2) space, one 16-byte pair per lane; n2 is even, so a
//    pair never straddles two lines) and a segment of its n1 rows, one warp;
//  * every lane keeps two register rings: 2 npts raw rows (double2) and npts
//    split taps (the FP32 pairs of the column-pair kernel). Row r's newest tap
//    is split once when it is needed, the stencil is the column-pair kernel's
//    (ds_stencil: the same operations per cell, so the same bits), the output
//    is stored, and the raw slot of the row's oldest tap is reloaded with the
//    row 2 npts further on: npts + 1 rows of loads in flight per lane, with an
//    L2 prefetch further ahead;
//  * a window holding a tap the split cannot carry runs the staged kernel's
//    FP64 arithmetic from the raw ring (the same bits as the staged kernel);
//  * in place: a lane loads every row before it overwrites it (its loads run
//    2 npts + d rows ahead of its stores, and the plan allows this form only
//    for d > -2 npts); rows outside the warp's segment belong to the warps of
//    the neighbouring segments and are read from seams saved in shared
//    memory before one CTA barrier (a segment's first d + npts - 1 rows, and
//    its last -d rows when d < 0), as in the FP32 streamed kernel;
//  * exception lines (offset not constant along n1) are skipped here and run
//    by the staged kernel.
#include <algorithm>

#include "adv.cuh"
#include "adv_plan.cuh"
#include "common.cuh"
#include "ds_arith.cuh"

namespace bkma {

namespace {

constexpr int kDsWarps = 8;         // warps per CTA
constexpr int kDsPrefetchRows = 16;  // L2 prefetch distance beyond the raw ring's loads

struct DsStreamArgs {
    const double *src;
    double *dst;
    int64_t n1, n2, lines;
    const int32_t *base;       // [lines]
    const double *w;           // [lines][NT] FP64 weights (windows the pair cannot carry)
    const float2 *w2;          // [lines][NT] FP32-pair weights
    const int32_t *exc_index;  // [lines]
    int segs;                  // row segments per group, one warp each (1, 2, 4 or 8)
    int sa, sb;                // seam rows per warp: a segment's first sa and last sb rows
};

template <int NT>
__global__ void __launch_bounds__(kDsWarps * 32, 2) adv_stream_ds(DsStreamArgs a) {
    extern __shared__ __align__(16) double2 seams[];  // [kDsWarps][sa + sb][32]
    constexpr int NR = 2 * NT;                        // raw ring rows
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const int S = a.segs;
    const int64_t group = (int64_t)blockIdx.x * (kDsWarps / S) + warp / S;
    const int seg = warp % S;
    const int n1 = (int)a.n1;
    const int64_t n2 = a.n2;
    const int64_t q = group * 64 + 2 * lane;
    bool ok = q < a.lines * n2;
    int64_t line = 0, col = 0;
    int d = 0;
    if (ok) {
        line = q / n2;
        col = q - line * n2;
        ok = a.exc_index[line] < 0;  // exception lines: the staged pass
        d = stream_offset(a.base[line], a.n1);
    }
    const int M = d + NT - 1;  // rows above the segment that it reads
    const int Lseg = (n1 + S - 1) / S;
    const int a0 = seg * Lseg, b0 = min(a0 + Lseg, n1);
    const int sa = a.sa, SR = a.sa + a.sb;
    const int64_t off = line * a.n1 * n2 + col;
    const double *src = a.src + off;
    double *dst = a.dst + off;
    double2 *mine = seams + (size_t)warp * SR * 32;
    if (ok) {
        for (int t = 0; t < M; ++t) {
            int j = a0 + t;
            if (j >= n1) j -= n1;
            mine[t * 32 + lane] = *reinterpret_cast<const double2 *>(src + (int64_t)j * n2);
        }
        for (int t = 0; t < -d; ++t) {
            int j = b0 + d + t;
            if (j < 0) j += n1;
            mine[(sa + t) * 32 + lane] = *reinterpret_cast<const double2 *>(src + (int64_t)j * n2);
        }
    }
    __syncthreads();  // every seam is saved before any warp overwrites rows
    if (!ok || a0 >= b0) return;
    const int g0 = warp - seg;  // first warp of this column group
    const double2 *above = seams + (size_t)(g0 + (seg + 1 == S ? 0 : seg + 1)) * SR * 32;
    const double2 *below = seams + (size_t)(g0 + (seg == 0 ? S - 1 : seg - 1)) * SR * 32;
    // original value of (unwrapped) row j; rows past the last one a window
    // reads give zeros (loaded into ring slots that no output uses)
    auto ld = [&](int j) -> double2 {
        if (j >= b0) {
            const int t = j - b0;
            return t < M ? above[t * 32 + lane] : make_double2(0.0, 0.0);
        }
        if (j < a0) return below[(sa + (j - a0) - d) * 32 + lane];
        return *reinterpret_cast<const double2 *>(src + (int64_t)j * n2);
    };
    float2 A[NT], B[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) {
        const float2 ab = a.w2[line * NT + k];
        A[k] = make_float2(ab.x, ab.x);
        B[k] = make_float2(ab.y, ab.y);
    }
    // raw ring: slot j % NR holds row a0 + d + j; split ring: slot j % NT
    // holds tap j; bad: bit k set when tap (newest - k) cannot be split
    double2 RR[NR];
    float4 T[NT];
    uint32_t bad = 0;
#pragma unroll
    for (int j = 0; j < NR; ++j) RR[j] = ld(a0 + d + j);
#pragma unroll
    for (int j = 0; j < NT - 1; ++j) bad = (bad << 1) | (ds_split2(RR[j], T[j]) ? 0u : 1u);
    double *po = dst + (int64_t)a0 * n2;
    const double *pn = src + (int64_t)(a0 + d + NR) * n2;  // next raw row to load
    for (int r0 = a0; r0 < b0; r0 += NR) {
        // the loads of this block stay inside the segment: plain loads
        const bool inner = a0 + d + (r0 - a0) + NR >= a0 && a0 + d + (r0 - a0) + 2 * NR <= b0;
#pragma unroll
        for (int i = 0; i < NR; ++i) {
            const int r = r0 + i;
            // newest tap of row r: j = (r - a0) + NT - 1, raw slot (i + NT - 1) % NR
            bad = ((bad << 1) | (ds_split2(RR[(i + NT - 1) % NR], T[(i + NT - 1) % NT]) ? 0u : 1u)) &
                  ((1u << NT) - 1u);
            if (r < b0) {
                double2 o;
                if (bad == 0u) {
                    o = ds_stencil<NT>(T, i % NT, A, B);
                } else {
                    // FP64 direct form, the staged kernel's arithmetic
                    double w64[NT];
#pragma unroll
                    for (int k = 0; k < NT; ++k) w64[k] = a.w[line * NT + k];
                    o.x = w64[0] * RR[i % NR].x;
                    o.y = w64[0] * RR[i % NR].y;
#pragma unroll
                    for (int k = 1; k < NT; ++k) {
                        o.x = fma(w64[k], RR[(i + k) % NR].x, o.x);
                        o.y = fma(w64[k], RR[(i + k) % NR].y, o.y);
                    }
                }
                *reinterpret_cast<double2 *>(po) = o;
            }
            po += n2;
            // the oldest tap of row r is not read again: reload its slot with
            // the row NR further on
            const int jn = a0 + d + (r - a0) + NR;
            if (inner) {
                if (jn + kDsPrefetchRows < b0)
                    asm volatile("prefetch.global.L2 [%0];" ::"l"(pn + (int64_t)kDsPrefetchRows * n2));
                RR[i % NR] = *reinterpret_cast<const double2 *>(pn);
            } else {
                RR[i % NR] = ld(jn);
            }
            pn += n2;
        }
    }
}

template <int NT>
cudaError_t launch_t(const DsStreamArgs &a, int64_t ctas, size_t smem, cudaStream_t st) {
    auto kern = adv_stream_ds<NT>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<grid_x(ctas), kDsWarps * 32, smem, st>>>(a);
    return cudaGetLastError();
}

int64_t groups_of(const AdvPlanImpl &p) { return (p.lines * p.desc.n2 + 63) / 64; }

}  // namespace

bool adv_stream_ds_shape_ok(const AdvPlanImpl &p) {
    return p.desc.dtype == BKMA_F64 && p.desc.impl != BKMA_ADV_PLAIN && p.d_w2 != nullptr &&
           p.ds_stream_ok && (p.npts == 4 || p.npts == 6) && p.desc.n2 % 2 == 0 &&
           p.desc.n1 >= kStreamMinN1 && p.desc.n1 < (1 << 30);
}

size_t adv_stream_ds_smem(const AdvPlanImpl &p) {
    return (size_t)kDsWarps * (size_t)(p.ds_sa + p.ds_sb) * 32 * sizeof(double2);
}

bool adv_stream_ds_eligible(const AdvPlanImpl &p, const void *src, const void *dst) {
    return adv_stream_ds_shape_ok(p) && ((uintptr_t)src % 16) == 0 && ((uintptr_t)dst % 16) == 0 &&
           adv_stream_ds_smem(p) <= (size_t)227 * 1024;
}

int adv_stream_ds_segs(const AdvPlanImpl &p, int mode) {
    // mode 0: split rows until there are enough warps to fill the GPU a few
    // times over; mode k >= 1: up to k segments. Segments keep >= 64 rows.
    const int64_t n1 = p.desc.n1, groups = groups_of(p);
    int s = 1;
    if (mode == 0) {
        while (s < kDsWarps && n1 / (2 * s) >= 64 && groups * s < 16384) s *= 2;
    } else {
        while (2 * s <= mode && s < kDsWarps && n1 / (2 * s) >= 64) s *= 2;
    }
    return s;
}

cudaError_t adv_stream_ds_launch(AdvPlanImpl &p, const void *src, void *dst, int segs_mode,
                                 cudaStream_t st) {
    DsStreamArgs a;
    a.src = (const double *)src;
    a.dst = (double *)dst;
    a.n1 = p.desc.n1;
    a.n2 = p.desc.n2;
    a.lines = p.lines;
    a.base = p.d_base;
    a.w = (const double *)p.d_w;
    a.w2 = p.d_w2;
    a.exc_index = p.d_exc_index;
    a.segs = adv_stream_ds_segs(p, segs_mode);
    a.sa = p.ds_sa;
    a.sb = p.ds_sb;
    const int64_t per_cta = kDsWarps / a.segs;
    const int64_t ctas = (groups_of(p) + per_cta - 1) / per_cta;
    const size_t smem = adv_stream_ds_smem(p);
    if (p.npts == 6) return launch_t<6>(a, ctas, smem, st);
    return launch_t<4>(a, ctas, smem, st);
}

}  // namespace bkma
