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

// Stage rows [0, n1) plus halo rows [n1, n1+H) (copies of rows 0..H-1) of
// `nslab` slabs x `wc` columns into shared memory laid out
// [slab (stride sstride elements)][row][col]. When a tile holds whole rows
// (wc == n2) each slab is one contiguous block in HBM and is copied flat.
// vec_ok: the global field allows 16-byte chunks for this tile.
template <typename T>
__device__ __forceinline__ void stage_tile(T *sm, const T *__restrict__ g, int64_t n1,
                                           int64_t n2, int64_t line0, int nslab, int64_t c0,
                                           int wc, int halo, int vec_ok, int sstride) {
    constexpr int VEC = 16 / (int)sizeof(T);
    if (wc == n2) {
        const int body = (int)n1 * wc;
        const int hal = halo * wc;
        const bool v = vec_ok && (body % VEC) == 0;
        const int chunks = v ? body / VEC : body;
        const int per_slab = chunks + hal;
        const int total = nslab * per_slab;
        for (int i = threadIdx.x; i < total; i += blockDim.x) {
            const int s = i / per_slab;
            const int j = i - s * per_slab;
            const T *gs = g + (line0 + s) * n1 * n2;
            T *ss = sm + (int64_t)s * sstride;
            if (j < chunks) {
                if (v)
                    cp_async(ss + j * VEC, gs + (int64_t)j * VEC, 16);
                else
                    cp_async(ss + j, gs + j, (int)sizeof(T));
            } else {
                const int h = j - chunks;
                cp_async(ss + body + h, gs + h, (int)sizeof(T));
            }
        }
    } else {
        const int rows = (int)n1 + halo;
        const int vec = (vec_ok && (wc % VEC) == 0) ? VEC : 1;
        const int cpr = wc / vec;
        const int per_slab = rows * cpr;
        const int total = nslab * per_slab;
        for (int i = threadIdx.x; i < total; i += blockDim.x) {
            const int s = i / per_slab;
            const int rem = i - s * per_slab;
            const int r = rem / cpr;
            const int ch = rem - r * cpr;
            const int gr = r < n1 ? r : r - (int)n1;
            const T *src = g + ((line0 + s) * n1 + gr) * n2 + c0 + (int64_t)ch * vec;
            T *dst = sm + (int64_t)s * sstride + r * wc + ch * vec;
            cp_async(dst, src, vec * (int)sizeof(T));
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

// One staged tile: `tc.nslab` slabs x `tc.wc` columns x all n1 rows of the
// field `a.src` -> `a.dst` (may alias). Shared by the single-field kernel and
// the batched persistent kernel, so both produce the same bits.
template <typename T, int NT>
__device__ __forceinline__ void staged_tile(const AdvStagedArgs<T> &a, const TileCoord &tc, T *sm) {
    constexpr int C = NT / 2 - 1;  // centre tap: the left node of the foot cell
    const int sstride = slab_stride(a.n1, NT - 1, tc.wc, (int)sizeof(T));
    stage_tile<T>(sm, a.src, a.n1, a.n2, tc.line0, tc.nslab, tc.c0, tc.wc, NT - 1, a.vec_ok,
                  sstride);

    const int n1 = (int)a.n1;
    const int wc = tc.wc;
    const int total = n1 * wc;
    const int dr = blockDim.x / wc;
    const int dc = blockDim.x - dr * wc;
    const int r_init = threadIdx.x / wc;
    const int c_init = threadIdx.x - r_init * wc;
    for (int s = 0; s < tc.nslab; ++s) {
        const int64_t line = tc.line0 + s;
        const T *S = sm + (int64_t)s * sstride;
        T *G = a.dst + line * a.n1 * a.n2 + tc.c0;
        const int exc = a.exc_index[line];
        if (exc < 0) {
            const int base = a.base[line];
            T w[NT];
#pragma unroll
            for (int k = 0; k < NT; ++k) w[k] = a.w[line * NT + k];
            int r = r_init, c = c_init;
            for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
                int rr = r + base;
                if (rr >= n1) rr -= n1;
                const T *p = S + rr * wc + c;
                const T fc = p[C * wc];
                T acc = T(0);
#pragma unroll
                for (int k = 0; k < NT; ++k)
                    if (k != C) acc = fma(w[k], p[k * wc] - fc, acc);
                G[(int64_t)r * a.n2 + c] = fc + acc;
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
                const T *p = S + rr * wc + c;
                const T fc = p[C * wc];
                T acc = T(0);
#pragma unroll
                for (int k = 0; k < NT; ++k)
                    if (k != C) acc = fma(e.w[k], p[k * wc] - fc, acc);
                G[(int64_t)r * a.n2 + c] = fc + acc;
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
    const TileCoord tc = tile_of(blockIdx.x, a.lines, a.n2, a.R, a.W, a.ncb);
    staged_tile<T, NT>(a, tc, reinterpret_cast<T *>(smem_raw));
}

}  // namespace bkma
