// Device code of the cp.async-staged advection kernels, shared by adv.cu
// (one field per launch) and batch.cu (many fields per persistent launch).
#pragma once
#include "adv.cuh"
#include "common.cuh"

namespace bkma {

// ----------------------------------------------------------------- device

__device__ __forceinline__ void cp_async(void *smem, const void *gmem, int bytes) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    if (bytes == 16) {
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem));
    } else if (bytes == 8) {
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem));
    } else {
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem));
    }
}
__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.wait_all;\n" ::: "memory");
}

// Element offset of `p` inside its 16-byte chunk.
template <typename T>
__device__ __forceinline__ int chunk_lead(const T *p) {
    return (int)(((uintptr_t)p / sizeof(T)) & (16 / sizeof(T) - 1));
}

// Block j of a run of `len` elements at `grow` -> `srow`: the elements of
// the j-th 16-byte chunk of global memory that the run touches. A chunk that
// lies wholly inside the run, with source and destination at the same place
// inside their 16-byte chunks, moves as one 16-byte copy; the ragged ends
// move element by element. Nothing outside the run is read.
template <typename T>
__device__ __forceinline__ void copy_block(T *srow, const T *grow, int len, int j) {
    constexpr int Q = 16 / (int)sizeof(T);
    const int a = j * Q - chunk_lead(grow);
    const int lo = max(a, 0), hi = min(a + Q, len);
    const bool cong = ((__cvta_generic_to_shared(srow) ^ (uintptr_t)grow) & 15) == 0;
    if (cong && lo == a && hi == a + Q) {
        cp_async(srow + a, grow + a, 16);
    } else {
        for (int e = lo; e < hi; ++e) cp_async(srow + e, grow + e, (int)sizeof(T));
    }
}

// Stage rows [0, n1) plus halo rows [n1, n1+H) (copies of rows 0..H-1) of
// `nslab` slabs x `wc` columns into shared memory. Slab s starts at element
// s*sstride; element (r, c) of the slab sits at chunk_lead(gs) + r*ws + c,
// gs = the slab's first global element (see staged_row_stride). When a tile
// holds whole rows (wc == n2) each slab is one contiguous run in HBM.
template <typename T>
__device__ __forceinline__ void stage_tile(T *sm, const T *__restrict__ g, int64_t n1,
                                           int64_t n2, int64_t line0, int nslab, int64_t c0,
                                           int wc, int ws, int halo, int sstride) {
    constexpr int Q = 16 / (int)sizeof(T);
    if (wc == n2) {
        const int body = (int)n1 * wc;
        const int hal = halo * wc;
        const int nb = (body + 2 * Q - 2) / Q;  // chunks a run of `body` can touch
        const int per_slab = nb + (hal + 2 * Q - 2) / Q;
        if (per_slab < (int)blockDim.x) {
            // small slabs: threads over (slab, chunk) pairs of all slabs
            for (int i = threadIdx.x; i < nslab * per_slab; i += blockDim.x) {
                const int s = i / per_slab;
                const int j = i - s * per_slab;
                const T *gs = g + (line0 + s) * n1 * n2;
                T *ss = sm + (int64_t)s * sstride + chunk_lead(gs);
                if (j < nb)
                    copy_block(ss, gs, body, j);
                else
                    copy_block(ss + body, gs, hal, j - nb);
            }
        } else {
            for (int s = 0; s < nslab; ++s) {
                const T *gs = g + (line0 + s) * n1 * n2;
                T *ss = sm + (int64_t)s * sstride + chunk_lead(gs);
                for (int i = threadIdx.x; i < per_slab; i += blockDim.x) {
                    if (i < nb)
                        copy_block(ss, gs, body, i);
                    else
                        copy_block(ss + body, gs, hal, i - nb);
                }
            }
        }
    } else {
        // (row, chunk) walk with incremental indices. When n2 is a multiple
        // of 16 bytes every row has the same lead and the chunk count is
        // exact; otherwise it is the most a row of wc elements can touch.
        const int rows = (int)n1 + halo;
        const int lead0 = chunk_lead(g + line0 * n1 * n2 + c0);
        const int cpr = (n2 % Q == 0) ? (lead0 + wc + Q - 1) / Q : (wc + 2 * Q - 2) / Q;
        const int per_slab = rows * cpr;
        const int dr = blockDim.x / cpr, dch = blockDim.x - dr * cpr;
        const int r_init = threadIdx.x / cpr, ch_init = threadIdx.x - r_init * cpr;
        for (int s = 0; s < nslab; ++s) {
            const T *gs = g + (line0 + s) * n1 * n2 + c0;
            T *ss = sm + (int64_t)s * sstride + chunk_lead(gs);
            int r = r_init, ch = ch_init;
            for (int i = threadIdx.x; i < per_slab; i += blockDim.x) {
                const int gr = r < n1 ? r : r - (int)n1;
                copy_block(ss + r * ws, gs + (int64_t)gr * n2, wc, ch);
                ch += dch;
                r += dr;
                if (ch >= cpr) {
                    ch -= cpr;
                    r += 1;
                }
            }
        }
    }
    cp_async_wait_all();
    __syncthreads();
}

// Stage like stage_tile, but into rows of ws elements that all start on 16
// bytes (lead 0), element by element. Used for FP32 tiles whose global rows
// do not start on 16 bytes, so the four-column compute can run on them.
template <typename T>
__device__ __forceinline__ void stage_tile_elems(T *sm, const T *__restrict__ g, int64_t n1,
                                                 int64_t n2, int64_t line0, int nslab,
                                                 int64_t c0, int wc, int ws, int halo,
                                                 int sstride) {
    const int rows = (int)n1 + halo;
    const int total = rows * wc;
    if (total < (int)blockDim.x) {
        // small slabs: threads over the elements of all slabs
        for (int i = threadIdx.x; i < nslab * total; i += blockDim.x) {
            const int s = i / total;
            const int e = i - s * total;
            const int r = e / wc, c = e - (e / wc) * wc;
            const int gr = r < n1 ? r : r - (int)n1;
            cp_async(sm + (int64_t)s * sstride + r * ws + c,
                     g + (line0 + s) * n1 * n2 + c0 + (int64_t)gr * n2 + c, (int)sizeof(T));
        }
        cp_async_wait_all();
        __syncthreads();
        return;
    }
    const int dr = blockDim.x / wc, dc = blockDim.x - dr * wc;
    const int r_init = threadIdx.x / wc, c_init = threadIdx.x - r_init * wc;
    for (int s = 0; s < nslab; ++s) {
        const T *gs = g + (line0 + s) * n1 * n2 + c0;
        T *ss = sm + (int64_t)s * sstride;
        int r = r_init, c = c_init;
        for (int i = threadIdx.x; i < total; i += blockDim.x) {
            const int gr = r < n1 ? r : r - (int)n1;
            cp_async(ss + r * ws + c, gs + (int64_t)gr * n2 + c, (int)sizeof(T));
            c += dc;
            r += dr;
            if (c >= wc) {
                c -= wc;
                r += 1;
            }
        }
    }
    cp_async_wait_all();
    __syncthreads();
}

// Tile coordinates of block `t`.
struct TileCoord {
    int64_t line0;
    int nslab;
    int64_t c0;
    int wc;
};

__device__ __forceinline__ TileCoord tile_of(int64_t t, int64_t lines, int64_t n2, int R,
                                             int W, int64_t ncb) {
    TileCoord tc;
    const int64_t lt = t / ncb;
    const int64_t cb = t - lt * ncb;
    tc.line0 = lt * R;
    tc.nslab = (int)min((int64_t)R, lines - tc.line0);
    tc.c0 = cb * W;
    tc.wc = (int)min((int64_t)W, n2 - tc.c0);
    return tc;
}

// FP32 rows of one slab, four columns per thread: NT float4 tap loads and
// packed FMAs in the same order as the scalar loop below (d = f_k - f_c as
// fma(f_c, -1, f_k), acc = fma(w_k, d, acc), out = f_c + acc), so the bits
// match it. Needs ws a multiple of 4 and S on 16 bytes; a last group past
// wc computes on unused shared memory and stores only its columns < wc.
// Stores are 16, 8 or 4 bytes wide as each row's address allows.
template <int NT>
__device__ __forceinline__ void rows_f32x4(const float *S, float *G, int n1, int64_t n2, int ws,
                                           int wc, int base, const float (&wl)[NT]) {
    constexpr int C = NT / 2 - 1;
    const int ng = (wc + 3) >> 2;  // column groups per row
    const int rpp = blockDim.x / ng;
    const int r0 = threadIdx.x / ng;
    if (r0 >= rpp) return;
    const int g4 = (threadIdx.x - r0 * ng) * 4;
    const int nval = min(4, wc - g4);  // columns of this group inside the tile
    float2 w2[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) w2[k] = make_float2(wl[k], wl[k]);
    const float2 m1 = make_float2(-1.0f, -1.0f);
    int rr = r0 + base;
    if (rr >= n1) rr -= n1;
    int rstep = rpp % n1;
    for (int r = r0; r < n1; r += rpp) {
        const float *p = S + rr * ws + g4;
        float4 f[NT];
#pragma unroll
        for (int k = 0; k < NT; ++k) f[k] = *reinterpret_cast<const float4 *>(p + k * ws);
        const float2 cl = make_float2(f[C].x, f[C].y);
        const float2 ch = make_float2(f[C].z, f[C].w);
        float2 al = make_float2(0.f, 0.f), ah = make_float2(0.f, 0.f);
#pragma unroll
        for (int k = 0; k < NT; ++k) {
            if (k == C) continue;
            const float2 dl = __ffma2_rn(cl, m1, make_float2(f[k].x, f[k].y));
            const float2 dh = __ffma2_rn(ch, m1, make_float2(f[k].z, f[k].w));
            al = __ffma2_rn(w2[k], dl, al);
            ah = __ffma2_rn(w2[k], dh, ah);
        }
        const float2 ol = __fadd2_rn(cl, al);
        const float2 oh = __fadd2_rn(ch, ah);
        float *q = G + (int64_t)r * n2 + g4;
        const unsigned qa = (unsigned)(uintptr_t)q & 15u;
        if (nval == 4 && qa == 0) {
            *reinterpret_cast<float4 *>(q) = make_float4(ol.x, ol.y, oh.x, oh.y);
        } else if (nval == 4 && (qa & 7u) == 0) {
            *reinterpret_cast<float2 *>(q) = ol;
            *reinterpret_cast<float2 *>(q + 2) = oh;
        } else {
            q[0] = ol.x;
            if (nval > 1) q[1] = ol.y;
            if (nval > 2) q[2] = oh.x;
            if (nval > 3) q[3] = oh.y;
        }
        rr += rstep;
        if (rr >= n1) rr -= n1;
    }
}

// One staged tile: `tc.nslab` slabs x `tc.wc` columns x all n1 rows of the
// field `a.src` -> `a.dst` (may alias). Shared by the single-field kernel and
// the batched persistent kernel, so both produce the same bits.
// One cell from its npts taps p[0], p[ws], ..., p[(NT-1) ws] and weights w.
// FP32: the incremental form f_c + sum_{k != c} w_k (f_k - f_c), whose
// rounding scales with the small differences rather than with |f| (and the
// same operations as the packed FP32 kernels: same bits). FP64: the direct
// form sum_k w_k f_k, one multiply and NT - 1 FMAs instead of 2 NT - 1
// operations; FP64 issue bounds these kernels on GB300, and FP64 rounding
// (~1e-16 |f| per step) stays far below the stencil's own error.
template <typename T, int NT>
__device__ __forceinline__ T stencil_cell(const T *p, int ws, const T (&w)[NT]) {
    constexpr int C = NT / 2 - 1;
    if constexpr (sizeof(T) == 8) {
        T acc = w[0] * p[0];
#pragma unroll
        for (int k = 1; k < NT; ++k) acc = fma(w[k], p[k * ws], acc);
        return acc;
    } else {
        const T fc = p[C * ws];
        T acc = T(0);
#pragma unroll
        for (int k = 0; k < NT; ++k)
            if (k != C) acc = fma(w[k], p[k * ws] - fc, acc);
        return fc + acc;
    }
}

template <typename T, int NT>
__device__ __forceinline__ void staged_tile(const AdvStagedArgs<T> &a, const TileCoord &tc, T *sm) {
    // Parameters of the first line, loaded before the staging wait so their
    // latency hides behind the copies.
    // a null exception index: the plan has no exception lines
    const int exc0 = a.exc_index ? a.exc_index[tc.line0] : -1;
    const int base0 = a.base[tc.line0];
    T w0[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) w0[k] = a.w[tc.line0 * NT + k];
    // Column tiles narrower than a 16-byte chunk are staged element by
    // element into unpadded rows; FP32 rows of 4+ columns that do not start on
    // 16 bytes element by element into 16-byte-aligned rows, so they run the
    // four-column compute (both `packed`). Otherwise (whole rows, aligned
    // columns) the shared layout keeps each element's place inside its
    // 16-byte chunk and moves 16-byte pieces.
    constexpr int Q = 16 / (int)sizeof(T);
    bool packed = tc.wc < Q && tc.wc < a.n2;
    if constexpr (sizeof(T) == 4)
        packed = packed ||
                 (tc.wc >= 4 && ((a.n2 & 3) != 0 ||
                                 chunk_lead(a.src + tc.line0 * a.n1 * a.n2 + tc.c0) != 0));
    const int ws = !packed ? staged_row_stride(a.n2, tc.wc, (int)sizeof(T))
                   : tc.wc < Q ? tc.wc : (tc.wc + 3) & ~3;
    const int sstride = slab_stride(a.n1, NT - 1, ws, (int)sizeof(T));
    if (packed)
        stage_tile_elems<T>(sm, a.src, a.n1, a.n2, tc.line0, tc.nslab, tc.c0, tc.wc, ws, NT - 1,
                            sstride);
    else
        stage_tile<T>(sm, a.src, a.n1, a.n2, tc.line0, tc.nslab, tc.c0, tc.wc, ws, NT - 1,
                      sstride);

    const int n1 = (int)a.n1;
    const int wc = tc.wc;
    const int total = n1 * wc;
    const int dr = blockDim.x / wc;
    const int dc = blockDim.x - dr * wc;
    const int r_init = threadIdx.x / wc;
    const int c_init = threadIdx.x - r_init * wc;
    // Slabs of at most half a CTA's threads (short lines, few columns):
    // several slabs at once, one thread per cell, same per-cell arithmetic.
    if (tc.nslab > 1 && 2 * total <= (int)blockDim.x) {
        const int conc = (int)blockDim.x / total;
        const int sub = (int)threadIdx.x / total;
        const int e = (int)threadIdx.x - sub * total;
        const int r = e / wc, c = e - (e / wc) * wc;
        for (int s = sub; s < tc.nslab && sub < conc; s += conc) {
            const int64_t line = tc.line0 + s;
            const int64_t g0 = line * a.n1 * a.n2 + tc.c0;
            const int lead = packed ? 0 : chunk_lead(a.src + g0);
            const T *S = sm + (int64_t)s * sstride + lead;
            const int exc = a.exc_index ? a.exc_index[line] : -1;
            int rr;
            T w[NT];
            if (exc < 0) {
                rr = r + a.base[line];
#pragma unroll
                for (int k = 0; k < NT; ++k) w[k] = a.w[line * NT + k];
            } else {
                const AdvExcCell<T> &ec = a.exc[(int64_t)exc * n1 + r];
                rr = r + ec.base;
#pragma unroll
                for (int k = 0; k < NT; ++k) w[k] = ec.w[k];
            }
            if (rr >= n1) rr -= n1;
            a.dst[g0 + (int64_t)r * a.n2 + c] = stencil_cell<T, NT>(S + rr * ws + c, ws, w);
        }
        return;
    }
    for (int s = 0; s < tc.nslab; ++s) {
        const int64_t line = tc.line0 + s;
        const int64_t g0 = line * a.n1 * a.n2 + tc.c0;
        const int lead = packed ? 0 : chunk_lead(a.src + g0);
        const T *S = sm + (int64_t)s * sstride + lead;
        T *G = a.dst + g0;
        const int exc = s == 0 ? exc0 : a.exc_index ? a.exc_index[line] : -1;
        if (exc < 0) {
            const int base = s == 0 ? base0 : a.base[line];
            T w[NT];
#pragma unroll
            for (int k = 0; k < NT; ++k) w[k] = s == 0 ? w0[k] : a.w[line * NT + k];
            if constexpr (sizeof(T) == 4) {
                if (((ws | lead) & 3) == 0) {
                    rows_f32x4<NT>(S, G, n1, a.n2, ws, wc, base, w);
                    continue;
                }
            }
            int r = r_init, c = c_init;
            for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
                int rr = r + base;
                if (rr >= n1) rr -= n1;
                G[(int64_t)r * a.n2 + c] = stencil_cell<T, NT>(S + rr * ws + c, ws, w);
                c += dc;
                r += dr;
                if (c >= wc) {
                    c -= wc;
                    r += 1;
                }
            }
        } else {
            // Line whose departure offset varies along n1: per-cell table.
            const AdvExcCell<T> *cells = a.exc + (int64_t)exc * n1;
            int r = r_init, c = c_init;
            for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
                const AdvExcCell<T> &e = cells[r];
                int rr = r + e.base;
                if (rr >= n1) rr -= n1;
                T we[NT];
#pragma unroll
                for (int k = 0; k < NT; ++k) we[k] = e.w[k];
                G[(int64_t)r * a.n2 + c] = stencil_cell<T, NT>(S + rr * ws + c, ws, we);
                c += dc;
                r += dr;
                if (c >= wc) {
                    c -= wc;
                    r += 1;
                }
            }
        }
    }
}

template <typename T, int NT>
__global__ void __launch_bounds__(512) adv_staged(AdvStagedArgs<T> a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    TileCoord tc = tile_of(blockIdx.x, a.lines, a.n2, a.R, a.W, a.ncb);
    if (a.line_list) tc.line0 = a.line_list[tc.line0];
    staged_tile<T, NT>(a, tc, reinterpret_cast<T *>(smem_raw));
}

}  // namespace bkma
