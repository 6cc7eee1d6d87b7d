// Streamed FP32 advection: no shared-memory staging of whole column strips.
//
// Work unit: a group of 32 consecutive columns of the field's (line i0,
// column i2) space, one column per lane, so a row of a line is one coalesced
// 128-byte access whatever n2 is (lanes may belong to different lines, each
// with its own offset d and weights). The n1 rows of a group are split into
// `segs` row segments, one warp each; a CTA of 8 warps holds 8/segs groups.
//
// A warp walks its segment [a, b) in blocks of U = 8 rows, keeping the
// stencil window in registers: a ring of kRing blocks holds rows of the
// ORIGINAL field from r0+d on (d = the line's signed tap-0 offset); the loads
// of the block kRing-1 ahead are issued before the current block's stores,
// so kRing-2 blocks of loads are always in flight; an L2 prefetch runs
// kPrefetch blocks further ahead, so that those loads find their rows in L2
// (the registers bound the bytes in flight, and with them the HBM rate at
// DRAM latency). Output row r0+i is the incremental form
// f_c + sum_k w_k (f_k - f_c) over the npts rows from r0+d+i, the same
// operations in the same order as the staged kernels (identical bits).
//
// In place: inside its segment a lane reads every row before it overwrites
// it (loads at block r0 reach rows >= r0 + d + 8 (kRing-1) >= r0 when d >= -24, and a
// lane's loads are ordered before its later stores). Rows outside the
// segment belong to other warps, which overwrite them: before any store,
// each warp saves in shared memory the first d+npts-1 rows of its segment
// (needed by the segment above it, or at the periodic wrap by the last one)
// and, when d < 0, its last -d rows (needed by the segment below it, or by
// the first one at the wrap); one barrier, then every warp streams.
//
// Exception lines (offset not constant along n1) are skipped here and run
// by the staged kernel. This replaces the whole-strip staging of the
// reference's scratch-memory kernels (src/core/AdaptiveWg.hpp:57-140) for
// the usual small per-step displacement.
#include <type_traits>

#include "adv.cuh"
#include "adv_plan.cuh"
#include "common.cuh"

namespace bkma {

namespace {

constexpr int kU = 8;         // output rows per block
// register ring of kRing blocks: kRing - 1 blocks of loads ahead (batched
// workload: 4 blocks 727, 5 blocks 735, 6 blocks 730, 8 blocks 666 GCells/s;
// up to 8 blocks the kernel keeps two CTAs per SM)
constexpr int kRing = 5;
constexpr int kWarps = 8;     // warps per CTA
constexpr int kSeamRows = kStreamSeam + kStreamBack;
constexpr int kPitch = 32;    // shared-memory row pitch (floats) of a warp's seams
// L2 prefetch distance in blocks beyond the register ring's loads (batched
// workload, 4-block ring: 681 GCells/s without, 702 at 4, 716 at 8, 665 at
// 12, 643 at 16, 727 at 8 with the start-of-segment burst; 5-block ring: 744
// at 6, 738 at 8, 729 at 10)
constexpr int kPrefetch = 6;

template <int NT>
__device__ __forceinline__ void stream_group(const StreamField &F, int64_t group, int seg,
                                             float (*seams)[kSeamRows * kPitch]) {
    constexpr int C = NT / 2 - 1;
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const int n1 = (int)F.n1;
    const int64_t n2 = F.n2;
    const int S = F.segs;
    const int64_t q = group * 32 + lane;
    bool ok = q < F.lines * n2;
    int64_t line = 0, col = 0;
    if (ok) {
        line = q / n2;
        col = q - line * n2;
    }
    int d = 0;
    float w[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) w[k] = 0.f;
    if (ok) {
        const int32_t b = F.base[line];
        ok = F.exc_index[line] < 0 && stream_line_ok(b, F.n1, NT);
        d = stream_offset(b, F.n1);
#pragma unroll
        for (int k = 0; k < NT; ++k) w[k] = F.w[line * NT + k];
    }
    const int M = d + NT - 1;  // rows above the segment that it reads
    const int L = (n1 + S - 1) / S;
    const int a = seg * L, b = min(a + L, n1);
    const int64_t off = line * F.n1 * n2 + col;
    const float *src = F.src + off;
    float *dst = F.dst + off;
    // Save this segment's first M rows (seam rows 0..M-1) and, when d < 0,
    // its last -d rows (seam rows kStreamSeam + t = row b + d + t).
    float *mine = seams[warp];
    if (ok) {
        for (int t = 0; t < M; ++t) {
            int j = a + t;
            if (j >= n1) j -= n1;
            mine[t * kPitch + lane] = src[(int64_t)j * n2];
        }
        for (int t = 0; t < -d; ++t) {
            int j = b + d + t;
            if (j < 0) j += n1;
            mine[(kStreamSeam + t) * kPitch + lane] = src[(int64_t)j * n2];
        }
    }
    __syncthreads();  // every seam is saved before any warp overwrites rows
    if (!ok || a >= b) return;
    const int g0 = warp - seg;  // first warp of this column group
    const float *above = seams[g0 + (seg + 1 == S ? 0 : seg + 1)];
    const float *below = seams[g0 + (seg == 0 ? S - 1 : seg - 1)];
    // original value of row j, a + d <= j < b + d + 32 (unwrapped)
    auto ld = [&](int j) -> float {
        if (j >= b) return above[min(j - b, kStreamSeam - 1) * kPitch + lane];
        if (j < a) return below[(kStreamSeam + (j - a) - d) * kPitch + lane];
        return src[(int64_t)j * n2];
    };
    // Ring of kRing blocks of kU rows: slot (t % kRing) holds rows r0(t)+d ..
    // +kU-1 of block t. At block t the loads of block t+kRing-1 are issued
    // (into the slot block t-1 used), and block t's outputs read slots t and
    // t+1, so kRing-2 blocks of loads stay in flight behind the one being
    // computed. Before the first block: the rows the steady-state prefetch
    // would have covered.
    for (int j = max(a, a + d + (kRing - 1) * kU); j < min(b, a + d + (kRing - 1 + kPrefetch) * kU); ++j)
        asm volatile("prefetch.global.L2 [%0];" ::"l"(src + (int64_t)j * n2));
    // outputs are not read again this step: stores are marked first for L2
    // eviction, so the prefetched rows ahead stay resident (batched workload
    // 746 -> 754 GCells/s; the same hint on the loads: 514)
    uint64_t evict_first;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(evict_first));
    float B[kRing * kU];
#pragma unroll
    for (int i = 0; i < (kRing - 1) * kU; ++i) B[i] = ld(a + d + i);
    const float *pn = src + (int64_t)(a + d + (kRing - 1) * kU) * n2;  // first row of block t+kRing-1
    float *po = dst + (int64_t)a * n2;
    auto block = [&](auto ph_c, int r0) {
        constexpr int ph = decltype(ph_c)::value;  // t % kRing
        constexpr int ld_slot = (ph + kRing - 1) % kRing;
        const int j0 = r0 + d + (kRing - 1) * kU;
        {  // L2 prefetch of the rows kPrefetch blocks beyond this load
            const int jp = j0 + kPrefetch * kU;
            if (jp >= a && jp + kU <= b) {
                const float *pp = pn + (int64_t)kPrefetch * kU * n2;
#pragma unroll
                for (int i = 0; i < kU; ++i)
                    asm volatile("prefetch.global.L2 [%0];" ::"l"(pp + (int64_t)i * n2));
            }
        }
        if (j0 >= a && j0 + kU <= b) {
#pragma unroll
            for (int i = 0; i < kU; ++i) {
                B[ld_slot * kU + i] = *pn;
                pn += n2;
            }
        } else {
#pragma unroll
            for (int i = 0; i < kU; ++i) B[ld_slot * kU + i] = ld(j0 + i);
            pn += kU * n2;
        }
        const int nr = min(kU, b - r0);
#pragma unroll
        for (int i = 0; i < kU; ++i) {
            if (i < nr) {
                const float fc = B[(ph * kU + i + C) % (kRing * kU)];
                float acc = 0.f;
#pragma unroll
                for (int k = 0; k < NT; ++k)
                    if (k != C) acc = fmaf(w[k], B[(ph * kU + i + k) % (kRing * kU)] - fc, acc);
                asm volatile("st.global.L1::no_allocate.L2::cache_hint.f32 [%0], %1, %2;" ::"l"(po),
                             "f"(fc + acc), "l"(evict_first)
                             : "memory");
            }
            po += n2;
        }
    };
    for (int r0 = a; r0 < b; r0 += kRing * kU) {
        block(std::integral_constant<int, 0>{}, r0);
        if (r0 + kU >= b) break;
        block(std::integral_constant<int, 1>{}, r0 + kU);
        if (r0 + 2 * kU >= b) break;
        block(std::integral_constant<int, 2>{}, r0 + 2 * kU);
        if (r0 + 3 * kU >= b) break;
        block(std::integral_constant<int, 3>{}, r0 + 3 * kU);
        if constexpr (kRing > 4) {
            if (r0 + 4 * kU >= b) break;
            block(std::integral_constant<int, 4 % kRing>{}, r0 + 4 * kU);
        }
        if constexpr (kRing > 5) {
            if (r0 + 5 * kU >= b) break;
            block(std::integral_constant<int, 5 % kRing>{}, r0 + 5 * kU);
        }
        if constexpr (kRing > 6) {
            if (r0 + 6 * kU >= b) break;
            block(std::integral_constant<int, 6 % kRing>{}, r0 + 6 * kU);
        }
        if constexpr (kRing > 7) {
            if (r0 + 7 * kU >= b) break;
            block(std::integral_constant<int, 7 % kRing>{}, r0 + 7 * kU);
        }
    }
}

// `many` (device array of nfields fields, ascending cta0; all with npts ==
// NT) or, when null, the single field `one`.
template <int NT>
__global__ void __launch_bounds__(kWarps * 32) adv_stream_f32(StreamField one,
                                                               const StreamField *__restrict__ many,
                                                               int nfields) {
    __shared__ float seams[kWarps][kSeamRows * kPitch];
    StreamField F = one;
    if (many) {
        int lo = 0, hi = nfields - 1;  // last field with cta0 <= blockIdx.x
        while (lo < hi) {
            const int mid = (lo + hi + 1) / 2;
            if (many[mid].cta0 <= (int64_t)blockIdx.x) lo = mid;
            else hi = mid - 1;
        }
        F = many[lo];
    }
    const int warp = threadIdx.x >> 5;
    const int per_cta = kWarps / F.segs;  // column groups per CTA
    const int64_t group = ((int64_t)blockIdx.x - F.cta0) * per_cta + warp / F.segs;
    stream_group<NT>(F, group, warp % F.segs, seams);
}

// Fields of 4 and of 6 taps in one launch (batches): the CTAs of a field all
// take its tap count, so the switch is uniform per CTA, and the batch has one
// last wave instead of one per tap count.
__global__ void __launch_bounds__(kWarps * 32) adv_stream_f32_46(const StreamField *__restrict__ many,
                                                                  int nfields) {
    __shared__ float seams[kWarps][kSeamRows * kPitch];
    int lo = 0, hi = nfields - 1;  // last field with cta0 <= blockIdx.x
    while (lo < hi) {
        const int mid = (lo + hi + 1) / 2;
        if (many[mid].cta0 <= (int64_t)blockIdx.x) lo = mid;
        else hi = mid - 1;
    }
    const StreamField F = many[lo];
    const int warp = threadIdx.x >> 5;
    const int per_cta = kWarps / F.segs;
    const int64_t group = ((int64_t)blockIdx.x - F.cta0) * per_cta + warp / F.segs;
    if (F.npts == 4)
        stream_group<4>(F, group, warp % F.segs, seams);
    else
        stream_group<6>(F, group, warp % F.segs, seams);
}

template <int NT>
cudaError_t launch_stream(StreamField one, const StreamField *many, int nfields, int64_t ctas,
                          cudaStream_t st) {
    if (ctas == 0) return cudaSuccess;
    adv_stream_f32<NT><<<grid_x(ctas), kWarps * 32, 0, st>>>(one, many, nfields);
    return cudaGetLastError();
}

cudaError_t launch_stream_npts(int npts, StreamField one, const StreamField *many, int nfields,
                               int64_t ctas, cudaStream_t st) {
    switch (npts) {
    case 4: return launch_stream<4>(one, many, nfields, ctas, st);
    case 6: return launch_stream<6>(one, many, nfields, ctas, st);
    case 10: return launch_stream<10>(one, many, nfields, ctas, st);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace

size_t adv_stream_smem() { return sizeof(float) * kWarps * kSeamRows * kPitch; }

int adv_stream_segs(int64_t n1, int64_t groups, int mode) {
    // mode 0: split rows until there are enough warps to fill the GPU a few
    // times over; mode k >= 1: up to k segments. Segments keep >= 64 rows.
    int s = 1;
    if (mode == 0) {
        while (s < kWarps && n1 / (2 * s) >= 64 && groups * s < 16384) s *= 2;
    } else {
        while (2 * s <= mode && s < kWarps && n1 / (2 * s) >= 64) s *= 2;
    }
    return s;
}

int64_t adv_stream_groups(const AdvPlanImpl &p) { return (p.lines * p.desc.n2 + 31) / 32; }

int64_t adv_stream_ctas(const AdvPlanImpl &p, int segs) {
    const int per_cta = kWarps / segs;
    return (adv_stream_groups(p) + per_cta - 1) / per_cta;
}

StreamField adv_stream_field(const AdvPlanImpl &p, const void *src, void *dst, int segs) {
    StreamField f;
    f.src = (const float *)src;
    f.dst = (float *)dst;
    f.n1 = p.desc.n1;
    f.n2 = p.desc.n2;
    f.lines = p.lines;
    f.base = p.d_base;
    f.w = (const float *)p.d_w;
    f.exc_index = p.d_exc_index;
    f.npts = p.npts;
    f.segs = segs;
    f.cta0 = 0;
    return f;
}

cudaError_t adv_stream_launch(AdvPlanImpl &p, const void *src, void *dst, int segs,
                              cudaStream_t st) {
    const int s = adv_stream_segs(p.desc.n1, adv_stream_groups(p), segs);
    return launch_stream_npts(p.npts, adv_stream_field(p, src, dst, s), nullptr, 1,
                              adv_stream_ctas(p, s), st);
}

cudaError_t adv_stream_launch_fields_46(const StreamField *d_fields, int nfields, int64_t nctas,
                                        cudaStream_t st) {
    if (nctas == 0) return cudaSuccess;
    adv_stream_f32_46<<<grid_x(nctas), kWarps * 32, 0, st>>>(d_fields, nfields);
    return cudaGetLastError();
}

cudaError_t adv_stream_launch_fields(int npts, const StreamField *d_fields, int nfields,
                                     int64_t nctas, cudaStream_t st) {
    StreamField none{};
    return launch_stream_npts(npts, none, d_fields, nfields, nctas, st);
}

}  // namespace bkma
