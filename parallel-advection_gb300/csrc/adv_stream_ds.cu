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
//  * every lane keeps two register rings: npts + 2 raw rows (double2) and
//    npts split taps (the FP32 pairs of the column-pair kernel). Row r's
//    newest tap is split once when it is needed, the stencil is the
//    column-pair kernel's (ds_stencil: the same operations per cell, so the
//    same bits), the output is stored, and the raw slot of the row's oldest
//    tap is reloaded with the row npts + 2 further on: 3 rows of loads in
//    flight per lane, the rows found in L2 by a prefetch 16 rows ahead. A raw
//    row stays in its register until its last window's FP64 fallback could
//    read it, so the ring's length sets the registers it holds (2 npts rows:
//    e2 251, e8 256 GCells/s; npts + 4: 258 / 265; npts + 2: 266 / 277;
//    npts + 1: 257 / 268; npts, one row of loads ahead: 226 / 236);
//  * a window holding a tap the split cannot carry runs the staged kernel's
//    FP64 arithmetic from the raw ring (the same bits as the staged kernel);
//  * in place: a lane loads every row before it overwrites it. Walking up
//    the rows, its loads run npts + 2 + d rows ahead of its stores, which
//    holds for d > -(npts + 2); a warp whose lanes shift further down walks
//    down the rows instead (the mirror image: loads run 3 - d rows ahead,
//    which holds for d <= 2), with its rings filled from the last
//    tap down and the taps taken in the same order as walking up, so every
//    cell gets the same operations. The plan allows this form only when
//    every 64-column group has one direction that suits all its lines. Rows
//    outside the warp's segment belong to the warps of the neighbouring
//    segments and are read from seams saved in shared memory before one CTA
//    barrier (a segment's first d + npts - 1 rows, and its last -d rows when
//    d < 0), as in the FP32 streamed kernel;
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
    int sr;                    // seam rows per warp: a lane's max(d + NT - 1, 0) + max(-d, 0)
};

// One warp's segment [a0, b0) of its column group, walking up (REV false) or
// down the rows. Ring position j holds row y0 + j (up) or y0 - j (down): the
// taps of the segment's first output, then the rows further on.
template <int NT, bool REV>
__device__ __forceinline__ void stream_segment(const DsStreamArgs &a, int64_t line, const double *src,
                                               double *dst, int a0, int b0, int d,
                                               const double2 *above, const double2 *below, int M,
                                               int lane) {
    constexpr int NR = NT + 2;  // raw ring rows
    const int64_t n2 = a.n2;
    const int len = b0 - a0;
    const int K = max(-d, 0);
    const int sg = REV ? -1 : 1;
    const int64_t step = REV ? -n2 : n2;
    // original value of (unwrapped) row j; rows past the last one a window
    // reads give zeros (loaded into ring slots that no output uses)
    auto ld = [&](int j) -> double2 {
        if (j >= b0) {
            const int t = j - b0;
            return t < M ? above[t * 32 + lane] : make_double2(0.0, 0.0);
        }
        if (j < a0) {
            const int t = j - a0 + K;
            return t >= 0 ? below[(M + t) * 32 + lane] : make_double2(0.0, 0.0);
        }
        return *reinterpret_cast<const double2 *>(src + (int64_t)j * n2);
    };
    float2 A[NT], B[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) {
        const float2 ab = a.w2[line * NT + k];
        A[k] = make_float2(ab.x, ab.x);
        B[k] = make_float2(ab.y, ab.y);
    }
    const int y0 = REV ? b0 - 1 + d + NT - 1 : a0 + d;
    // raw ring: slot j % NR holds ring row j; split ring: slot j % NR holds
    // ring tap j (NR slots, so that a block of NR rows maps every ring to the
    // same slots); bad: bit k set when ring tap (newest - k) cannot be split
    double2 RR[NR];
    float4 T[NR];
    uint32_t bad = 0;
#pragma unroll
    for (int j = 0; j < NR; ++j) RR[j] = ld(y0 + sg * j);
#pragma unroll
    for (int j = 0; j < NT - 1; ++j) bad = (bad << 1) | (ds_split2(RR[j], T[j]) ? 0u : 1u);
    double *po = dst + (int64_t)(REV ? b0 - 1 : a0) * n2;
    const double *pn = src + (int64_t)(y0 + sg * NR) * n2;  // next raw row to load
    for (int u0 = 0; u0 < len; u0 += NR) {
        // the loads of this block, ring rows u0 + NR .. u0 + 2 NR - 1, stay
        // inside the segment: plain loads
        const int lo = REV ? y0 - u0 - 2 * NR + 1 : y0 + u0 + NR;
        const bool inner = lo >= a0 && lo + NR <= b0;
#pragma unroll
        for (int i = 0; i < NR; ++i) {
            const int u = u0 + i;
            // newest tap of output u: ring tap u + NT - 1, raw slot (i + NT - 1) % NR
            bad = ((bad << 1) | (ds_split2(RR[(i + NT - 1) % NR], T[(i + NT - 1) % NR]) ? 0u : 1u)) &
                  ((1u << NT) - 1u);
            if (u < len) {
                double2 o;
                if (bad == 0u) {
                    o = ds_stencil<NT, REV>(T, i, A, B);
                } else {
                    // FP64 direct form, the staged kernel's arithmetic; tap k
                    // is ring tap k (up) or NT - 1 - k (down)
                    double w64[NT];
#pragma unroll
                    for (int k = 0; k < NT; ++k) w64[k] = a.w[line * NT + k];
                    constexpr int k0 = REV ? NT - 1 : 0;
                    o.x = w64[0] * RR[(i + k0) % NR].x;
                    o.y = w64[0] * RR[(i + k0) % NR].y;
#pragma unroll
                    for (int k = 1; k < NT; ++k) {
                        const int kk = REV ? NT - 1 - k : k;
                        o.x = fma(w64[k], RR[(i + kk) % NR].x, o.x);
                        o.y = fma(w64[k], RR[(i + kk) % NR].y, o.y);
                    }
                }
                *reinterpret_cast<double2 *>(po) = o;
            }
            po += step;
            // ring row u is not read again: reload its slot with ring row u + NR
            if (inner) {
                const int jn = y0 + sg * (u + NR);
                if (REV ? jn - kDsPrefetchRows >= a0 : jn + kDsPrefetchRows < b0)
                    asm volatile("prefetch.global.L2 [%0];" ::"l"(pn + kDsPrefetchRows * step));
                RR[i % NR] = *reinterpret_cast<const double2 *>(pn);
            } else {
                RR[i % NR] = ld(y0 + sg * (u + NR));
            }
            pn += step;
        }
    }
}

template <int NT>
__global__ void __launch_bounds__(kDsWarps * 32, 2) adv_stream_ds(DsStreamArgs a) {
    extern __shared__ __align__(16) double2 seams[];  // [kDsWarps][sr][32]
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
    // walk up unless a lane shifts too far down for it (the plan checked that
    // walking down then suits every lane of the group)
    const bool up = __all_sync(0xFFFFFFFFu, !ok || d > -(NT + 2));
    // seams of a lane: rows 0 .. M-1 are the segment's first M rows (read by
    // the segment below it), rows M .. M+K-1 its last K rows (read by the one
    // above); a neighbour's same lane has the same line, so the same M and K
    const int M = max(d + NT - 1, 0);
    const int K = max(-d, 0);
    const int Lseg = (n1 + S - 1) / S;
    const int a0 = seg * Lseg, b0 = min(a0 + Lseg, n1);
    const int64_t off = line * a.n1 * n2 + col;
    const double *src = a.src + off;
    double *dst = a.dst + off;
    double2 *mine = seams + (size_t)warp * a.sr * 32;
    if (ok) {
        for (int t = 0; t < M; ++t) {
            int j = a0 + t;
            if (j >= n1) j -= n1;
            mine[t * 32 + lane] = *reinterpret_cast<const double2 *>(src + (int64_t)j * n2);
        }
        for (int t = 0; t < K; ++t) {
            int j = b0 - K + t;
            if (j < 0) j += n1;
            mine[(M + t) * 32 + lane] = *reinterpret_cast<const double2 *>(src + (int64_t)j * n2);
        }
    }
    __syncthreads();  // every seam is saved before any warp overwrites rows
    if (!ok || a0 >= b0) return;
    const int g0 = warp - seg;  // first warp of this column group
    const double2 *above = seams + (size_t)(g0 + (seg + 1 == S ? 0 : seg + 1)) * a.sr * 32;
    const double2 *below = seams + (size_t)(g0 + (seg == 0 ? S - 1 : seg - 1)) * a.sr * 32;
    if (up)
        stream_segment<NT, false>(a, line, src, dst, a0, b0, d, above, below, M, lane);
    else
        stream_segment<NT, true>(a, line, src, dst, a0, b0, d, above, below, M, lane);
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
    return (size_t)kDsWarps * (size_t)p.ds_sr * 32 * sizeof(double2);
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
    a.sr = p.ds_sr;
    const int64_t per_cta = kDsWarps / a.segs;
    const int64_t ctas = (groups_of(p) + per_cta - 1) / per_cta;
    const size_t smem = adv_stream_ds_smem(p);
    if (p.npts == 6) return launch_t<6>(a, ctas, smem, st);
    return launch_t<4>(a, ctas, smem, st);
}

}  // namespace bkma
