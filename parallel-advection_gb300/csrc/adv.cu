// Semi-Lagrangian advection along n1 (the reference's AdvectionSolver driven
// by AdaptiveWg/NDRange/BasicRange: src/solvers/AdvectionSolver.hpp:71-99,
// src/core/AdaptiveWg.hpp:57-140, src/core/NDRange.hpp:4-40,
// src/core/BasicRange.hpp:27-69), rebuilt for sm_103a.
//
// Data layout in HBM: field[i0][i1][i2], n2 fastest (layout_right, as
// src/types.hpp:12-30). A "line" is (i0, i2): n1 values at stride n2.
//
// Because the departure point depends on (i0, i1) only, every line of slab
// i0 shares one integer tap offset and one set of weights. The plan computes
// them once on the host in FP64 with the reference's exact formulas (leftNode
// bit-identical), and lists any line whose offset is not constant along n1
// (those get per-cell offsets and weights).
//
// Kernel `adv_staged`: one CTA per tile = a block of W columns (i2) of one
// slab, or R whole slabs when n2 is small, spanning all n1 rows. The tile is
// staged into shared memory with cp.async (16-byte chunks when aligned), with
// the first npts-1 rows repeated after row n1-1 so the periodic wrap needs no
// modulo per tap. After one barrier every output is computed from shared
// memory with register-resident weights in the incremental form
// f_c + sum_k w_k (f_k - f_c), and written straight to global memory: the
// tile was read completely before the first write, so in place is legal
// (the AdaptiveWg scratch/barrier/write-back pattern, with the scratch being
// the input copy).
//
// Kernel `adv_plain`: the same staging, but each output recomputes the
// reference's per-cell FP64 math (displ, floor, lag_basis) with
// non-contracted operations: bit-identical to AdvectionSolver::operator().
// It is the "plain FP64 form" speed baseline.

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <system_error>
#include <thread>
#include <tuple>
#include <vector>

#include "adv.cuh"
#include "adv_device.cuh"
#include "adv_plan.cuh"
#include "common.cuh"

namespace bkma {

// Plain FP64 form: the reference's per-cell math, bit-identical.
__global__ void __launch_bounds__(512) adv_plain(AdvPlainArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double *sm = reinterpret_cast<double *>(smem_raw);
    const TileCoord tc = tile_of(blockIdx.x, a.lines, a.n2, a.R, a.W, a.ncb);
    const int ws = staged_row_stride(a.n2, tc.wc, 8);
    const int sstride = slab_stride(a.n1, 0, ws, 8);
    stage_tile<double>(sm, a.src, a.n1, a.n2, tc.line0, tc.nslab, tc.c0, tc.wc, ws, 0, sstride);
    const int n1 = (int)a.n1;
    const int wc = tc.wc;
    const int total = n1 * wc;
    const uint64_t un1 = (uint64_t)a.n1;
    for (int s = 0; s < tc.nslab; ++s) {
        const int64_t line = tc.line0 + s;
        const int64_t g0 = line * a.n1 * a.n2 + tc.c0;
        const double *S = sm + (int64_t)s * sstride + chunk_lead(a.src + g0);
        double *G = a.dst + g0;
        const double vx = a.vx[line];
        for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
            const int r = idx / wc;
            const int c = idx - r * wc;
            double d;
            const int left = adv_departure(a.phys, r, vx, &d);
            double coef[6];
            lag_basis_ref5(d, coef);
            const int ipos1 = left - 2;
            double value = 0.;
#pragma unroll
            for (int k = 0; k < 6; ++k) {
                const uint64_t id = (un1 + (uint64_t)(int64_t)ipos1 + (uint64_t)k) % un1;
                value = dadd(value, dmul(coef[k], S[(int64_t)id * ws + c]));
            }
            G[(int64_t)r * a.n2 + c] = value;
        }
    }
}

// ----------------------------------------------------------------- host

namespace {

// Textbook Lagrange basis on nodes 0..npts-1 at px.
void lag_textbook(int npts, double px, double *c) {
    for (int j = 0; j < npts; ++j) {
        double num = 1.0, den = 1.0;
        for (int m = 0; m < npts; ++m) {
            if (m == j) continue;
            num *= (px - (double)m);
            den *= (double)(j - m);
        }
        c[j] = num / den;
    }
}

// Weights of the stencil whose tap 0 sits at leftNode-(npts/2-1), for a foot
// point with d = 2 + frac (frac in [0,1)).
void stencil_weights(int weights_kind, int npts, double d, double *w) {
    if (weights_kind == BKMA_W_REFERENCE) {
        lag_basis_ref5(d, w);
    } else {
        lag_textbook(npts, (double)(npts / 2 - 1) + (d - 2.0), w);
    }
}

// Row of tap 0 for point i1, as an offset from i1 modulo n1. The tap index
// is formed like the reference's (n1 + ipos1 + k) % n1 in size_t arithmetic
// (AdvectionSolver.hpp:94), so even a negative foot (a displacement beyond a
// full period) selects the same rows.
int64_t tap0_offset(int left, int NT, int64_t i1, int64_t n1) {
    const uint64_t un1 = (uint64_t)n1;
    const int64_t first = (int64_t)left - (NT / 2 - 1);
    const uint64_t id0 = (un1 + (uint64_t)first) % un1;
    return (int64_t)((id0 + un1 - (uint64_t)i1 % un1) % un1);
}

struct TuneKey {
    int dtype, npts, impl;
    int64_t lines, n1, n2;
    bool operator<(const TuneKey &o) const {
        return std::tie(dtype, npts, impl, lines, n1, n2) <
               std::tie(o.dtype, o.npts, o.impl, o.lines, o.n1, o.n2);
    }
};
struct TuneVal {
    int W, R, threads, path;
};
std::mutex g_tune_mu;
std::map<TuneKey, TuneVal> g_tune_cache;

}  // namespace

}  // namespace bkma

namespace bkma {
namespace {

constexpr size_t kMaxSmem = 227 * 1024;
constexpr int kRunHostChunks = 32;  // slab chunks of bkma_adv_run_host's copy/compute pipeline (8: 759, 16: 784, 32: 788, 64: 781 GCells/s e2e)

// Default tile: columns of one slab when n2 is wide enough for 64-byte row
// segments, otherwise whole slabs; about 32-64 KB of shared memory per CTA.
void default_tile(AdvPlanImpl &p) {
    const int64_t n2 = p.desc.n2;
    const int min_cols = 64 / p.esize;  // 16 FP32 / 8 FP64 columns = 64 B rows
    // Short lines: a column tile would hold few cells, so take whole rows of
    // several slabs when a slab's rows fit in 48 KB.
    const bool short_lines =
        p.desc.n1 * min_cols < 8192 && p.smem_bytes((int)n2, 1) <= 48 * 1024;
    if (n2 >= min_cols && !short_lines) {
        p.W = min_cols;
        p.R = 1;
    } else {
        p.W = (int)n2;
        const size_t per = p.smem_bytes(p.W, 1);
        // very short lines: smaller CTAs (1048576 x 16 x 128: 2 slabs of
        // 10.8 KB and 128 threads run at 744 GCells/s, 4 slabs and 256
        // threads at 600)
        const size_t target = p.desc.n1 <= 64 ? 24 * 1024 : 48 * 1024;
        int r = (int)std::max<size_t>(1, target / std::max<size_t>(per, 1));
        r = (int)std::min<int64_t>(r, p.lines);
        p.R = std::max(1, r);
    }
    while (p.R > 1 && p.smem_bytes(p.W, p.R) > kMaxSmem) p.R /= 2;
    while (p.W > 1 && p.smem_bytes(p.W, p.R) > kMaxSmem) p.W /= 2;
    p.threads = (short_lines && p.desc.n1 <= 64) ? 128 : 256;
    // TMA staging for FP32 column tiles (512 threads: 4-5 % faster than 256
    // on the reference's n1 = 1024 shapes); launch_once falls back per call
    // when a field pointer is not 16-byte aligned.
    const void *aligned_probe = reinterpret_cast<const void *>(uintptr_t(256));
    p.path = (p.R == 1 && adv_tma_eligible(p, aligned_probe, p.W) &&
              adv_tma_smem(p, p.W) <= kMaxSmem) ? 1 : 0;
    if (p.path == 1) {
        // 32-column tiles while a tile stays within ~64 KB (n1 <= 512), and
        // about eight row passes per thread. Measured (GCells/s, 16 columns x
        // 512 threads before): 1024 x 128 x 2048 382 -> 876 (32 x 128),
        // 4096 x 64 x 1024 244 -> 848, 512 x 256 x 2048 578 -> 874 (32 x 256),
        // 2048 x 512 x 512 772 -> 881 (32 x 512); n1 = 1024 keeps 16 x 512.
        if (p.desc.n1 * 32 * p.esize <= 65536 && adv_tma_eligible(p, aligned_probe, 32) &&
            adv_tma_smem(p, 32) <= kMaxSmem)
            p.W = 32;
        const int64_t want = std::max<int64_t>(128, p.desc.n1 * p.W / 32);
        p.threads = want >= 512 ? 512 : want >= 256 ? 256 : 128;
    }
    // Streaming beats TMA tiles when a tile leaves one CTA per SM (n1 >= 2048:
    // 534 vs 760 GCells/s at 1024 x 2048 x 1024) or when rows are 1 MB or
    // more apart (1 x 1024 x 2^21: 400 vs 699, every box row a new page).
    const bool tma_poor = adv_tma_smem(p, p.W) > 100 * 1024 || n2 * p.esize >= (1 << 20);
    if (p.stream_ok && n2 >= 8 && (p.path == 0 || tma_poor)) {
        // rows that are not 16-byte aligned, or tiles too tall for the TMA
        // form: stream the columns (row segments chosen from the size)
        p.path = 2;
        p.R = 0;
        p.W = (int)std::min<int64_t>(16, n2);
    }
    if (adv_rows_shape_ok(p) && adv_rows_smem(p, adv_rows_default_r(p)) <= kMaxSmem) {
        // n2 = 1: runs of whole contiguous lines
        p.path = 3;
        p.W = 1;
        p.R = adv_rows_default_r(p);
        p.threads = 256;  // the contiguous-line kernel's fixed CTA
    }
    if (adv_ds_shape_ok(p, 4) && p.desc.n1 >= 128 && adv_ds_smem(p, 4) <= kMaxSmem) {
        // FP64 storage in FP32-pair arithmetic (GB300's FP64 rate bounds the
        // FP64 staged kernel near 100 GCells/s): 4-column TMA tiles, six CTAs
        // of 128 threads per SM (2048 x 1024 x 512: 333 GCells/s; 8-column
        // tiles, three CTAs of 256 threads: 289). Lines shorter than 128 rows
        // leave runs of one or two rows that re-split most taps: they take
        // whole slabs below (x 128 columns, 2^27 cells, GCells/s column pairs
        // / slabs / staged: n1 = 16 33 / 311 / 100, 64 97 / 311 / 91; 128
        // 151 / - / 98, 256 216 / - / 99, slabs of 128 KB and more leaving
        // one CTA per SM)
        p.path = 4;
        p.W = 4;
        p.R = 1;
        p.threads = adv_ds_threads(4);  // the FP32-pair kernel's CTA for the width
    }
    if (adv_stream_ds_shape_ok(p) && adv_stream_ds_smem(p) <= kMaxSmem && p.desc.n1 >= 128 &&
        (p.path != 4 || n2 * 8 >= (1 << 20))) {
        // FP64 column pairs that the staged form cannot take (strips too tall
        // for shared memory) or takes badly (rows 1 MB or more apart: every
        // TMA box row its own DRAM page): the streamed FP32-pair form
        p.path = 6;
        p.W = (int)std::min<int64_t>(8, n2);  // the staged passes' tile width
        p.R = 0;                              // row-segment mode: from the size
        p.threads = 256;
    }
    if (adv_ds_rows_shape_ok(p) && (n2 == 1 || (p.path == 0 && p.desc.n1 < 128))) {
        // FP64 contiguous lines (n2 = 1), or whole slabs of lines too short
        // for the column-pair kernel, in the same FP32-pair arithmetic
        int W = 1, R = 1;
        adv_ds_rows_default(p, &W, &R);
        if (adv_ds_rows_smem(p, R) <= kMaxSmem) {
            p.path = 5;
            p.W = W;  // lines: 1 = 4 cells per thread, 2 = runs along two
                      // sections, 3 = half lines in 2-CTA clusters, 4 = runs
                      // of 4-cell groups, 5 = lines shared by a warp's lanes,
                      // 6 = half lines in runs of 4-cell groups;
                      // slabs: runs of rows per column pair
            p.R = R;
            p.threads = 256;  // the kernels' fixed CTA
        }
    }
}

template <typename T>
bkma_status upload_tables(AdvPlanImpl &p) {
    const int64_t L = p.lines;
    const int NT = p.npts;
    std::vector<T> w((size_t)(L * NT));
    for (int64_t i = 0; i < L * NT; ++i) w[(size_t)i] = (T)p.w64[(size_t)i];
    BKMA_CUDA_TRY(cudaMalloc(&p.d_base, sizeof(int32_t) * (size_t)L));
    BKMA_CUDA_TRY(cudaMalloc(&p.d_w, sizeof(T) * (size_t)(L * NT)));
    BKMA_CUDA_TRY(cudaMalloc(&p.d_exc_index, sizeof(int32_t) * (size_t)L));
    BKMA_CUDA_TRY(cudaMalloc(&p.d_vx, sizeof(double) * (size_t)L));
    BKMA_CUDA_TRY(cudaMemcpy(p.d_base, p.base.data(), sizeof(int32_t) * L, cudaMemcpyHostToDevice));
    BKMA_CUDA_TRY(cudaMemcpy(p.d_w, w.data(), sizeof(T) * L * NT, cudaMemcpyHostToDevice));
    BKMA_CUDA_TRY(cudaMemcpy(p.d_exc_index, p.exc_index.data(), sizeof(int32_t) * L,
                             cudaMemcpyHostToDevice));
    BKMA_CUDA_TRY(cudaMemcpy(p.d_vx, p.vx.data(), sizeof(double) * L, cudaMemcpyHostToDevice));
    if (sizeof(T) == 8 && p.desc.impl != BKMA_ADV_PLAIN) {
        // FP32-pair weights of the FP64 kernel in FP32-pair arithmetic (adv_ds.cu):
        // w = a + b + r, a = RN32(w), b = RN32(w - a), |r| <= 2^-48 |w|
        std::vector<float2> w2((size_t)(L * NT));
        for (int64_t i = 0; i < L * NT; ++i) {
            const double wd = p.w64[(size_t)i];
            const float a = (float)wd;
            w2[(size_t)i] = make_float2(a, (float)(wd - (double)a));
        }
        BKMA_CUDA_TRY(cudaMalloc(&p.d_w2, sizeof(float2) * (size_t)(L * NT)));
        BKMA_CUDA_TRY(cudaMemcpy(p.d_w2, w2.data(), sizeof(float2) * (size_t)(L * NT),
                                 cudaMemcpyHostToDevice));
    }
    if (p.n_exc > 0) {
        std::vector<int32_t> lst;
        for (int64_t l = 0; l < L; ++l)
            if (p.exc_index[(size_t)l] >= 0) lst.push_back((int32_t)l);
        BKMA_CUDA_TRY(cudaMalloc(&p.d_exc_lines, sizeof(int32_t) * lst.size()));
        BKMA_CUDA_TRY(cudaMemcpy(p.d_exc_lines, lst.data(), sizeof(int32_t) * lst.size(),
                                 cudaMemcpyHostToDevice));
    }
    if (p.n_exc > 0) {
        // Per-cell tables for exception lines.
        const int64_t n1 = p.desc.n1;
        std::vector<AdvExcCell<T>> cells((size_t)(p.n_exc * n1));
        for (int64_t l = 0; l < L; ++l) {
            const int slot = p.exc_index[(size_t)l];
            if (slot < 0) continue;
            for (int64_t i1 = 0; i1 < n1; ++i1) {
                double d;
                const int left = adv_departure(p.phys, (int)i1, p.vx[(size_t)l], &d);
                const int64_t b = tap0_offset(left, NT, i1, n1);
                double wd[16];
                stencil_weights(p.desc.weights, NT, d, wd);
                AdvExcCell<T> &e = cells[(size_t)(slot * n1 + i1)];
                e.base = (int32_t)b;
                int64_t dev = (b - p.base[(size_t)l]) % n1;
                if (dev < 0) dev += n1;
                dev = std::min(dev, n1 - dev);
                p.exc_dev = (int)std::max<int64_t>(p.exc_dev, dev);
                for (int k = 0; k < kMaxTaps; ++k) e.w[k] = k < NT ? (T)wd[k] : T(0);
            }
        }
        BKMA_CUDA_TRY(cudaMalloc(&p.d_exc, sizeof(AdvExcCell<T>) * cells.size()));
        BKMA_CUDA_TRY(cudaMemcpy(p.d_exc, cells.data(), sizeof(AdvExcCell<T>) * cells.size(),
                                 cudaMemcpyHostToDevice));
    }
    return BKMA_OK;
}

// `list`, when given, restricts the launch to its `nlist` lines (R = 1).
template <typename T, int NT>
cudaError_t launch_staged_t(const AdvPlanImpl &p, const T *src, T *dst, int W, int R,
                            int threads, cudaStream_t st, const int32_t *list, int64_t nlist) {
    AdvStagedArgs<T> a;
    a.src = src;
    a.dst = dst;
    a.n1 = p.desc.n1;
    a.n2 = p.desc.n2;
    a.lines = list ? nlist : p.lines;
    a.W = W;
    a.R = list ? 1 : R;
    a.ncb = p.ncb(W);
    a.base = p.d_base;
    a.w = (const T *)p.d_w;
    a.exc_index = p.n_exc > 0 ? p.d_exc_index : nullptr;  // null: no per-line index reads
    a.exc = (const AdvExcCell<T> *)p.d_exc;
    a.line_list = list;
    const size_t smem = p.smem_bytes(W, a.R);
    auto kern = adv_staged<T, NT>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    const int64_t grid = list ? nlist * a.ncb : p.tiles(W, R);
    if (grid == 0) return cudaSuccess;
    kern<<<grid_x(grid), threads, smem, st>>>(a);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_staged_npts(const AdvPlanImpl &p, const void *src, void *dst, int W, int R,
                               int threads, cudaStream_t st, const int32_t *list = nullptr,
                               int64_t nlist = 0) {
    const T *s = (const T *)src;
    T *d = (T *)dst;
    switch (p.npts) {
    case 4: return launch_staged_t<T, 4>(p, s, d, W, R, threads, st, list, nlist);
    case 6: return launch_staged_t<T, 6>(p, s, d, W, R, threads, st, list, nlist);
    case 10: return launch_staged_t<T, 10>(p, s, d, W, R, threads, st, list, nlist);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_plain(const AdvPlanImpl &p, const double *src, double *dst, int W, int R,
                         int threads, cudaStream_t st) {
    AdvPlainArgs a;
    a.src = src;
    a.dst = dst;
    a.n1 = p.desc.n1;
    a.n2 = p.desc.n2;
    a.lines = p.lines;
    a.W = W;
    a.R = R;
    a.ncb = p.ncb(W);
    a.vx = p.d_vx;
    a.phys = p.phys;
    const size_t smem = p.smem_bytes(W, R);
    cudaError_t e =
        cudaFuncSetAttribute(adv_plain, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    adv_plain<<<grid_x(p.tiles(W, R)), threads, smem, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_once(AdvPlanImpl &p, const void *src, void *dst, int W, int R, int threads,
                        int path, cudaStream_t st) {
    // FP32-pair FP64 kernel; a field off the 16-byte grid takes the FP64
    // staged kernel on the same 8-column tiles
    if (path == 4 && adv_ds_eligible(p, src, W)) return adv_ds_launch(p, src, dst, W, st);
    if (path == 1 && R == 1 && adv_tma_eligible(p, src, W))
        return adv_tma_launch(p, src, dst, W, threads, st);
    if (path == 2 && p.stream_ok) {
        // streamed lines, then the exception lines through the staged kernel
        (void)threads;  // the streamed kernel has a fixed CTA; R = row-segment mode
        cudaError_t e = adv_stream_launch(p, src, dst, R, st);
        if (e != cudaSuccess || p.n_exc == 0) return e;
        return launch_staged_npts<float>(p, src, dst, p.exc_tile_w(kMaxSmem), 1, 256, st,
                                         p.d_exc_lines, p.n_exc);
    }
    if (path == 6 && adv_stream_ds_eligible(p, src, dst)) {
        // streamed FP32-pair lines, then the exception lines through the staged kernel
        cudaError_t e = adv_stream_ds_launch(p, src, dst, R, st);
        if (e != cudaSuccess || p.n_exc == 0) return e;
        return launch_staged_npts<double>(p, src, dst, p.exc_tile_w(kMaxSmem), 1, 256, st,
                                          p.d_exc_lines, p.n_exc);
    }
    if (path == 6) {
        // a field off the 16-byte grid: the FP64 staged kernel on strips that fit
        W = std::max(1, p.exc_tile_w(kMaxSmem));
        R = 1;
        threads = 256;
    }
    if (path == 3 || path == 5) {
        if (path == 3 && adv_rows_eligible(p, src, dst, R)) return adv_rows_launch(p, src, dst, R, st);
        if (path == 5 && adv_ds_rows_eligible(p, src, dst, R))
            return adv_ds_rows_launch(p, src, dst, W, R, st);
        // unaligned field: the generic staged kernel on whole rows (n2 = 1)
        // or on 8-column strips of single lines
        W = (int)std::min<int64_t>(8, p.desc.n2);
        if (W > 1) R = 1;
        while (R > 1 && p.smem_bytes(W, R) > kMaxSmem) R /= 2;
    }
    if (p.desc.impl == BKMA_ADV_PLAIN)
        return launch_plain(p, (const double *)src, (double *)dst, W, R, threads, st);
    if (p.desc.dtype == BKMA_F32) return launch_staged_npts<float>(p, src, dst, W, R, threads, st);
    return launch_staged_npts<double>(p, src, dst, W, R, threads, st);
}

}  // namespace

bkma_status adv_launch(AdvPlanImpl &p, void *data, void *out, int nsteps, cudaStream_t st) {
    const bool inplace = (out == nullptr || out == data);
    if (p.fuse > 1 && nsteps > 0) {
        // k steps per launch; out of place the first launch reads `data` and
        // writes `out`, later ones run in place on `out`. FP64 contiguous
        // lines on the FP32-pair kernel fuse in the same arithmetic, the
        // other plans on the staged kernel's.
        const void *src = data;
        void *dst = inplace ? data : out;
        const int Rf = adv_ds_rows_fused_r(p);
        const bool pair = p.path == 5 && adv_ds_rows_fused_ok(p, data, dst, Rf);
        const int W = pair ? 0 : adv_fused_tile_w(p, kMaxSmem);
        for (int done = 0; done < nsteps;) {
            const int k = std::min(p.fuse, nsteps - done);
            cudaError_t e = pair ? adv_ds_rows_fused_launch(p, src, dst, Rf, k, st)
                                 : adv_fused_launch(p, src, dst, W, k, st);
            if (e != cudaSuccess) return cuda_fail(e, "adv fused kernel launch");
            src = dst;
            done += k;
        }
        return BKMA_OK;
    }
    // Out of place: an odd number of steps alternates data->out->data...->out;
    // an even number first steps `data` in place, then alternates.
    int t0 = 0;
    if (!inplace && nsteps > 0 && nsteps % 2 == 0) {
        cudaError_t e = launch_once(p, data, data, p.W, p.R, p.threads, p.path, st);
        if (e != cudaSuccess) return cuda_fail(e, "adv kernel launch");
        t0 = 1;
    }
    for (int t = t0; t < nsteps; ++t) {
        void *src = data, *dst = data;
        if (!inplace) {
            const bool to_out = ((t - t0) % 2) == 0;
            src = to_out ? data : out;
            dst = to_out ? out : data;
        }
        cudaError_t e = launch_once(p, src, dst, p.W, p.R, p.threads, p.path, st);
        if (e != cudaSuccess) return cuda_fail(e, "adv kernel launch");
    }
    return BKMA_OK;
}

// Per-line precompute of a plan (bit-exact leftNode, FP64 weights).
bkma_status adv_precompute(AdvPlanImpl &p) {
    const bkma_adv_desc &d = p.desc;
    const int NT = p.npts;
    p.base.assign((size_t)p.lines, 0);
    p.shift.assign((size_t)p.lines, 0.0);
    p.vx.assign((size_t)p.lines, 0.0);
    p.w64.assign((size_t)(p.lines * NT), 0.0);
    p.exc_index.assign((size_t)p.lines, -1);
    p.n_exc = 0;
    const int64_t n1 = d.n1;
    // A line's tap offset can change along n1 only where its fractional shift
    // lies within rounding error of a cell boundary: the FP64 coordinate
    // arithmetic of the departure point is off by far less than 1e-8 cells
    // for n1 <= 2^24, so a line whose shift (at i1 = 0) is in
    // (kEdge, 1 - kEdge) has one offset for every i1; the others are scanned
    // cell by cell. Lines are independent: host threads split them.
    constexpr double kEdge = 1e-6;
    std::vector<uint8_t> varying((size_t)p.lines, 0);
    auto work = [&](int64_t lo, int64_t hi) {
        for (int64_t l = lo; l < hi; ++l) {
            const int64_t g = d.i0_offset + l;
            const double v =
                d.velocity ? d.velocity[l] : adv_coord((int)g, p.phys.minVx, p.phys.dvx);
            p.vx[(size_t)l] = v;
            double d0;
            const int left0 = adv_departure(p.phys, 0, v, &d0);
            const int64_t b0 = tap0_offset(left0, NT, 0, n1);
            p.base[(size_t)l] = (int32_t)b0;
            p.shift[(size_t)l] = d0 - 2.0;
            stencil_weights(d.weights, NT, d0, &p.w64[(size_t)(l * NT)]);
            if (d.impl == BKMA_ADV_PLAIN) continue;
            const double f = d0 - 2.0;
            if (f > kEdge && f < 1.0 - kEdge) continue;
            for (int64_t i1 = 1; i1 < n1; ++i1) {
                double di;
                const int left = adv_departure(p.phys, (int)i1, v, &di);
                if (tap0_offset(left, NT, i1, n1) != b0) {
                    varying[(size_t)l] = 1;
                    break;
                }
            }
        }
    };
    const int64_t per_thread = 1 << 14;  // lines
    const int nthr = (int)std::min<int64_t>(
        std::max(1u, std::thread::hardware_concurrency()), (p.lines + per_thread - 1) / per_thread);
    if (nthr <= 1) {
        work(0, p.lines);
    } else {
        std::vector<std::thread> pool;
        pool.reserve((size_t)nthr);
        int started = 0;
        try {
            for (; started < nthr; ++started)
                pool.emplace_back(work, p.lines * started / nthr, p.lines * (started + 1) / nthr);
        } catch (const std::system_error &) {
            // a thread that could not start: its share and the rest run here
        }
        for (int t = started; t < nthr; ++t) work(p.lines * t / nthr, p.lines * (t + 1) / nthr);
        for (auto &th : pool) th.join();
    }
    for (int64_t l = 0; l < p.lines; ++l)
        if (varying[(size_t)l]) p.exc_index[(size_t)l] = (int32_t)p.n_exc++;
    if (d.impl == BKMA_ADV_PLAIN) return BKMA_OK;
    p.stream_ok = d.dtype == BKMA_F32;
    for (int64_t l = 0; l < p.lines && p.stream_ok; ++l)
        if (p.exc_index[(size_t)l] < 0 && !stream_line_ok(p.base[(size_t)l], n1, NT))
            p.stream_ok = false;
    if (d.dtype == BKMA_F64 && d.n2 % 2 == 0) {
        // the streamed FP32-pair form: each 64-column group (32 column pairs
        // of the (line, i2) space) walks up its rows, loading NT + 2 rows
        // ahead of its stores (d > -(NT + 2) on all its lines), or down
        // (d <= 2); seams of at most 32 rows each way
        constexpr int kWin = 32;
        p.ds_stream_ok = n1 >= kStreamMinN1;
        p.ds_sr = 0;
        const int64_t cols = p.lines * d.n2, ngroups = (cols + 63) / 64;
        for (int64_t g = 0; g < ngroups && p.ds_stream_ok; ++g) {
            const int64_t l0 = g * 64 / d.n2, l1 = std::min(g * 64 + 63, cols - 1) / d.n2;
            bool up = true, down = true;
            for (int64_t l = l0; l <= l1; ++l) {
                if (p.exc_index[(size_t)l] >= 0) continue;
                const int dd = stream_offset(p.base[(size_t)l], n1);
                if (dd < -kWin || dd + NT - 1 > kWin) p.ds_stream_ok = false;
                up = up && dd > -(NT + 2);
                down = down && dd <= 2;
                p.ds_sr = std::max(p.ds_sr, std::max(dd + NT - 1, 0) + std::max(-dd, 0));
            }
            if (!up && !down) p.ds_stream_ok = false;
        }
    }
    if (d.dtype == BKMA_F32) return upload_tables<float>(p);
    return upload_tables<double>(p);
}

bkma_status adv_autotune(AdvPlanImpl &p, void *field, cudaStream_t st) {
    const TuneKey key{p.desc.dtype, p.npts, p.desc.impl, p.lines, p.desc.n1, p.desc.n2};
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
            p.W = it->second.W;
            p.R = it->second.R;
            p.threads = it->second.threads;
            p.path = it->second.path;
            p.autotuned = true;
            return BKMA_OK;
        }
    }
    // The plan's own tile is the first candidate, so tuning never ends on a
    // tile slower than the default. An FP64 plan on an FP32-pair kernel
    // (paths 4 and 5) keeps it: the other FP64 kernels round differently, and
    // tuning must not change results.
    std::vector<TuneVal> cands{{p.W, p.R, p.threads, p.path}};
    const int64_t n2 = p.desc.n2;
    const int ths[3] = {128, 256, 512};
    if (p.path == 4 || p.path == 6 || (p.path == 5 && n2 > 1)) {
        // the other forms of the same arithmetic per cell (same bits): tile
        // widths of the staged column-pair kernel, row segments of the
        // streamed one, slabs per CTA of the whole-slab one
        for (int W : {4, 8})
            if ((p.path != 4 || W != p.W) && adv_ds_shape_ok(p, W) && p.desc.n1 >= 16)
                cands.push_back({W, 1, adv_ds_threads(W), 4});
        if (adv_stream_ds_eligible(p, field, field))
            for (int segs : {0, 1, 2, 4, 8})
                if (p.path != 6 || segs != p.R)
                    cands.push_back({(int)std::min<int64_t>(8, n2), segs, 256, 6});
        if (p.desc.n1 < 128)
            for (int R = 1; R <= 1024 && R <= p.lines; R *= 2)
                for (int runs : {1, 2, 4, 8})
                    if ((p.path != 5 || R != p.R || runs != p.W) && runs <= p.desc.n1 &&
                        adv_ds_rows_eligible(p, field, field, R) &&
                        (int64_t)R * (n2 / 2) * runs <= 1024)
                        cands.push_back({runs, R, 256, 5});
    } else if (p.path == 5) {
        // other line counts per CTA of the same kernel
        for (int R = 1; R <= 1024 && R <= p.lines; R *= 2)
            for (int W : {1, 2, 4, 5})
                if ((R != p.R || W != p.W) && adv_ds_rows_eligible(p, field, field, R) &&
                    (W != 2 || adv_ds_runs_ok(p, R)) && (W != 5 || adv_ds_lineq_ok(p)))
                    cands.push_back({W, R, 256, 5});
        if (adv_ds_halves_ok(p) && ((uintptr_t)field % 16) == 0)
            for (int W : {3, 6})
                if (W != p.W) cands.push_back({W, 1, 256, 5});
    } else if (n2 >= 8) {
        for (int W : {8, 16, 32, 64})
            if (W <= n2 || W == 8)
                for (int t : ths) {
                    cands.push_back({W, 1, t, 0});
                    if (adv_tma_eligible(p, field, W)) cands.push_back({W, 1, t, 1});
                }
    }
    const bool other = p.path != 4 && p.path != 5 && p.path != 6;
    if (p.stream_ok && other)
        for (int segs : {0, 1, 2, 4, 8}) cands.push_back({(int)std::min<int64_t>(16, n2), segs, 256, 2});
    for (int R : {1, 2, 4, 8, 16, 32, 64, 128, 256, 512, 1024})
        if (other && n2 < 32 && R <= p.lines && p.smem_bytes((int)n2, R) <= kMaxSmem)
            for (int t : ths) cands.push_back({(int)n2, R, t, 0});
    // whole-row tiles of a few slabs for wider rows of short lines
    for (int R : {1, 2, 4, 8, 16})
        if (other && n2 >= 32 && n2 <= 256 && R <= p.lines && p.smem_bytes((int)n2, R) <= 96 * 1024)
            for (int t : ths) cands.push_back({(int)n2, R, t, 0});
    if (other && adv_rows_shape_ok(p))
        for (int R = 1; R <= 4096 && R <= p.lines; R *= 2)
            if (adv_rows_eligible(p, field, field, R)) cands.push_back({1, R, 256, 3});
    cudaEvent_t e0, e1;
    BKMA_CUDA_TRY(cudaEventCreate(&e0));
    BKMA_CUDA_TRY(cudaEventCreate(&e1));
    float best = 1e30f;
    TuneVal bestv{p.W, p.R, p.threads, p.path};
    for (const TuneVal &c : cands) {
        const size_t need = c.path == 1 ? adv_tma_smem(p, c.W)
                            : c.path == 4 ? adv_ds_smem(p, c.W)
                            : c.path == 2 || c.path == 6 ? (c.path == 6 ? adv_stream_ds_smem(p) : 0)
                            : c.path == 3 ? adv_rows_smem(p, c.R)
                            : c.path == 5 ? ((c.W == 3 || c.W == 6) && p.desc.n2 == 1 ? adv_ds_halves_smem(p)
                                                                         : adv_ds_rows_smem(p, c.R))
                                          : p.smem_bytes(c.W, c.R);
        if (need > kMaxSmem) continue;
        cudaError_t err = launch_once(p, field, field, c.W, c.R, c.threads, c.path, st);  // warm-up
        if (err != cudaSuccess) {
            cudaGetLastError();
            continue;
        }
        const int reps = 3;
        cudaEventRecord(e0, st);
        for (int i = 0; i < reps; ++i)
            launch_once(p, field, field, c.W, c.R, c.threads, c.path, st);
        cudaEventRecord(e1, st);
        BKMA_CUDA_TRY(cudaEventSynchronize(e1));
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) {
            best = ms;
            bestv = c;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    p.W = bestv.W;
    p.R = bestv.R;
    p.threads = bestv.threads;
    p.path = bestv.path;
    p.autotuned = true;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_cache[key] = bestv;
    return BKMA_OK;
}

}  // namespace bkma

// ================================================================= C ABI
using namespace bkma;

extern "C" {

bkma_status bkma_adv_plan_create(const bkma_adv_desc *desc, bkma_adv_plan **plan) try {
    bkma::NvtxRange nvtx_range("bkma_adv_plan_create");
    BKMA_CHECK_ARG(desc && plan, "bkma_adv_plan_create: null argument");
    *plan = nullptr;
    const bkma_adv_desc &d = *desc;
    BKMA_CHECK_ARG(d.n0 > 0 && d.n1 > 0 && d.n2 > 0, "n0, n1, n2 must be positive");
    BKMA_CHECK_ARG(d.n1 < (1 << 24) && d.n2 < (1 << 24), "n1 and n2 must be < 2^24");
    // the velocity index i0 is an int in AdvectionSolver::coord
    // (src/solvers/AdvectionSolver.hpp:24); 2^50 cells keep every size product
    // far from int64 overflow
    BKMA_CHECK_ARG(d.n0 < (int64_t(1) << 31), "n0 must be < 2^31");
    BKMA_CHECK_ARG((double)d.n0 * (double)d.n1 * (double)d.n2 < 1125899906842624.0,
                   "n0 * n1 * n2 must be < 2^50");
    BKMA_CHECK_ARG(d.i0_offset >= 0 && d.i0_offset < d.n0, "i0_offset out of range");
    const int64_t count = d.i0_count == 0 ? d.n0 - d.i0_offset : d.i0_count;
    BKMA_CHECK_ARG(count > 0 && d.i0_offset + count <= d.n0, "i0_count out of range");
    BKMA_CHECK_ARG(d.dtype == BKMA_F32 || d.dtype == BKMA_F64, "dtype must be BKMA_F32 or BKMA_F64");
    BKMA_CHECK_ARG(d.impl >= BKMA_ADV_AUTO && d.impl <= BKMA_ADV_PLAIN, "unknown impl");
    BKMA_CHECK_ARG(d.weights >= BKMA_W_REFERENCE && d.weights <= BKMA_W_TABLE, "unknown weights");
    if (d.weights == BKMA_W_REFERENCE)
        BKMA_CHECK_ARG(d.degree == 5, "reference weights (lag_basis) exist for degree 5 only");
    else
        BKMA_CHECK_ARG(d.degree == 3 || d.degree == 5 || d.degree == 9, "degree must be 3, 5 or 9");
    if (d.impl == BKMA_ADV_PLAIN) {
        BKMA_CHECK_ARG(d.dtype == BKMA_F64 && d.weights == BKMA_W_REFERENCE,
                       "the plain form is the reference's FP64 degree-5 operator");
    } else {
        BKMA_CHECK_ARG(d.n1 >= d.degree + 1, "the staged kernel needs n1 >= degree + 1");
    }
    BKMA_CHECK_ARG(d.maxX > d.minX, "maxX must exceed minX");
    BKMA_CHECK_ARG(std::isfinite(d.dt), "dt must be finite");
    BKMA_CHECK_ARG(std::isfinite(d.minX) && std::isfinite(d.maxX) && std::isfinite(d.minVx) &&
                       std::isfinite(d.maxVx),
                   "minX, maxX, minVx and maxVx must be finite");
    // a NaN foot point would reach floor() and an int conversion
    if (d.velocity)
        for (int64_t l = 0; l < count; ++l)
            BKMA_CHECK_ARG(std::isfinite(d.velocity[l]), "velocity values must be finite");

    // owned here until complete: an early return or an exception frees it
    std::unique_ptr<bkma_adv_plan> pl(new bkma_adv_plan);
    AdvPlanImpl &p = pl->impl;
    p.desc = d;
    p.desc.i0_count = count;
    p.desc.velocity = nullptr;
    p.lines = count;
    p.npts = d.degree + 1;
    p.esize = d.dtype == BKMA_F32 ? 4 : 8;
    p.phys.n0 = d.n0;
    p.phys.n1 = d.n1;
    p.phys.dt = d.dt;
    p.phys.minX = d.minX;
    p.phys.maxX = d.maxX;
    p.phys.minVx = d.minVx;
    p.phys.maxVx = d.maxVx;
    adv_update_deltas(p.phys);
    cudaGetDevice(&p.device);
    // velocity pointer is only read during create
    bkma_adv_desc dv = p.desc;
    dv.velocity = d.velocity;
    std::swap(p.desc, dv);
    bkma_status s = adv_precompute(p);
    std::swap(p.desc, dv);
    p.desc.velocity = nullptr;
    if (s == BKMA_OK && d.impl == BKMA_ADV_PLAIN) {
        cudaError_t e = cudaMalloc(&p.d_vx, sizeof(double) * (size_t)p.lines);
        if (e == cudaSuccess)
            e = cudaMemcpy(p.d_vx, p.vx.data(), sizeof(double) * p.lines, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) s = cuda_fail(e, "plan tables");
    }
    if (s != BKMA_OK) return s;
    {
        cudaError_t e = cudaMalloc(&p.d_status, sizeof(int));
        if (e == cudaSuccess) e = cudaMemset(p.d_status, 0, sizeof(int));
        if (e != cudaSuccess) return cuda_fail(e, "plan status word");
    }
    default_tile(p);
    // the staged kernel runs every line, or (streamed form) the exception lines
    const bool too_long = (p.path == 2 || p.path == 6) ? (p.n_exc > 0 && p.exc_tile_w(kMaxSmem) == 0)
                                      : p.smem_bytes(p.W, p.R) > kMaxSmem;
    if (too_long) return fail(BKMA_ERR_UNSUPPORTED, "n1 too long for a shared-memory line tile");
    *plan = pl.release();
    return BKMA_OK;
} BKMA_ABI_CATCH("bkma_adv_plan_create")

bkma_status bkma_adv_plan_info_get(const bkma_adv_plan *plan, bkma_adv_plan_info *info) try {
    BKMA_CHECK_ARG(plan && info, "null argument");
    const AdvPlanImpl &p = plan->impl;
    info->lines = p.lines;
    info->exception_lines = p.n_exc;
    // path 5: the contiguous-line kernel form (1: 4 cells per thread, 2: runs)
    info->tile_cols = (int32_t)(p.path == 5 ? p.W : std::min<int64_t>(p.W, p.desc.n2));
    info->tile_slabs = p.R;
    info->threads = p.threads;
    info->smem_bytes = (int32_t)(p.path == 1   ? adv_tma_smem(p, p.W)
                                 : p.path == 4 ? adv_ds_smem(p, p.W)
                                 : p.path == 2 ? adv_stream_smem()
                                 : p.path == 3 ? adv_rows_smem(p, p.R)
                                 : p.path == 5 ? ((p.W == 3 || p.W == 6) && p.desc.n2 == 1 ? adv_ds_halves_smem(p)
                                                                             : adv_ds_rows_smem(p, p.R))
                                 : p.path == 6 ? adv_stream_ds_smem(p)
                                               : p.smem_bytes(p.W, p.R));
    info->npts = p.npts;
    info->autotuned = p.autotuned ? 1 : 0;
    info->tiles = (p.path == 5 && (p.W == 3 || p.W == 6) && p.desc.n2 == 1) ? 2 * p.lines
                  : (p.path == 3 || p.path == 5)             ? (p.lines + p.R - 1) / p.R
                                                              : p.tiles(p.W, p.R);
    info->path = p.path;
    return BKMA_OK;
} BKMA_ABI_CATCH("bkma_adv_plan_info_get")

bkma_status bkma_adv_plan_status(bkma_adv_plan *plan, void *stream) try {
    BKMA_CHECK_ARG(plan, "null argument");
    AdvPlanImpl &p = plan->impl;
    BKMA_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
    int st = 0;
    BKMA_CUDA_TRY(cudaMemcpy(&st, p.d_status, sizeof(int), cudaMemcpyDeviceToHost));
    BKMA_CUDA_TRY(cudaMemset(p.d_status, 0, sizeof(int)));
    if (st != 0) return fail((bkma_status)st, "advection: a bounded device wait timed out");
    return BKMA_OK;
} BKMA_ABI_CATCH("bkma_adv_plan_status")

bkma_status bkma_adv_plan_set_wait_limit(bkma_adv_plan *plan, uint32_t polls) try {
    BKMA_CHECK_ARG(plan, "null argument");
    plan->impl.wait_polls = polls;
    return BKMA_OK;
} BKMA_ABI_CATCH("bkma_adv_plan_set_wait_limit")

bkma_status bkma_adv_plan_autotune(bkma_adv_plan *plan, void *field, void *stream) try {
    bkma::NvtxRange nvtx_range("bkma_adv_plan_autotune");
    BKMA_CHECK_ARG(plan && field, "null argument");
    return adv_autotune(plan->impl, field, (cudaStream_t)stream);
} BKMA_ABI_CATCH("bkma_adv_plan_autotune")

bkma_status bkma_adv_plan_set_tile(bkma_adv_plan *plan, int32_t W, int32_t R, int32_t threads,
                                   int32_t path) try {
    BKMA_CHECK_ARG(plan, "null argument");
    AdvPlanImpl &p = plan->impl;
    BKMA_CHECK_ARG(W >= 1 && W <= 1024 && R >= (path == 2 || path == 6 ? 0 : 1) && R <= 1024,
                   "W must be in [1,1024], R in [1,1024] (path 2: row-segment mode 0..8)");
    BKMA_CHECK_ARG(threads == 128 || threads == 256 || threads == 512, "threads must be 128, 256 or 512");
    BKMA_CHECK_ARG(path >= 0 && path <= 6, "path must be 0 to 6");
    BKMA_CHECK_ARG(path != 2 || p.stream_ok, "streamed form not available for this plan");
    BKMA_CHECK_ARG(path >= 2 || R == 1 || W >= p.desc.n2, "R > 1 needs whole-row tiles (W >= n2)");
    BKMA_CHECK_ARG((path != 2 && path != 6) || R <= 8,
                   "paths 2 and 6: R is the row-segment mode, 0 (auto) to 8");
    if (path == 1) {
        const void *probe = reinterpret_cast<const void *>(uintptr_t(256));
        BKMA_CHECK_ARG(R == 1 && adv_tma_eligible(p, probe, W), "TMA staging not available for this tile");
        BKMA_CHECK_ARG(adv_tma_smem(p, W) <= kMaxSmem, "tile does not fit shared memory");
    } else if (path == 0) {
        BKMA_CHECK_ARG(p.smem_bytes(W, R) <= kMaxSmem, "tile does not fit shared memory");
    } else if (path == 3) {
        BKMA_CHECK_ARG(adv_rows_shape_ok(p) && W == 1 && adv_rows_smem(p, R) <= kMaxSmem,
                       "path 3 needs an FP32 plan with n2 = 1, n1 % 4 == 0, n1 >= 16, "
                       "W = 1 and R lines that fit shared memory");
    } else if (path == 4) {
        BKMA_CHECK_ARG(adv_ds_shape_ok(p, W) && adv_ds_smem(p, W) <= kMaxSmem && R == 1 &&
                           threads == adv_ds_threads(W),
                       "path 4 needs an FP64 plan of degree 3 or 5 with an even n2 >= W, n1 >= 16, "
                       "lines that fit shared memory, W = 4 (128 threads) or 8 (256 threads) "
                       "and R = 1");
    } else if (path == 6) {
        BKMA_CHECK_ARG(adv_stream_ds_shape_ok(p) && adv_stream_ds_smem(p) <= kMaxSmem,
                       "path 6 needs an FP64 plan of degree 3 or 5 with an even n2, n1 >= 64 and "
                       "every line's per-step shift within the streamed window");
    } else if (path == 5) {
        const bool slabs = p.desc.n2 > 1;
        BKMA_CHECK_ARG(adv_ds_rows_shape_ok(p) &&
                           (slabs ? W <= 64 && adv_ds_rows_smem(p, R) <= kMaxSmem
                                  : ((W == 1 || W == 4 || (W == 5 && adv_ds_lineq_ok(p))) &&
                                     adv_ds_rows_smem(p, R) <= kMaxSmem) ||
                                        (W == 2 && adv_ds_runs_ok(p, R) &&
                                         adv_ds_rows_smem(p, R) <= kMaxSmem) ||
                                        ((W == 3 || W == 6) && R == 1 && adv_ds_halves_ok(p))),
                       "path 5 needs an FP64 plan of degree 3 or 5 with n2 = 1, n1 % 4 == 0, "
                       "n1 >= 16, R lines that fit shared memory and W = 1 (4 cells per thread) "
                       "or W = 2 (runs along two sections: n1 >= 512, R = 1 or an even R <= 16) "
                       "or W = 3 (half lines in 2-CTA clusters: n1 >= 8192, R = 1) "
                       "or W = 4 (runs of 4-cell groups) or W = 5 (lines of 16-128 cells shared "
                       "by a warp's lanes); "
                       "or with an even n2, R whole slabs that fit shared memory and W <= 64 "
                       "runs of rows per column pair");
    }
    p.W = W;
    p.R = R;
    p.threads = threads;
    p.path = path;
    return BKMA_OK;
} BKMA_ABI_CATCH("bkma_adv_plan_set_tile")

bkma_status bkma_adv_plan_set_fusion(bkma_adv_plan *plan, int32_t steps_per_launch) try {
    BKMA_CHECK_ARG(plan && steps_per_launch >= 1, "steps_per_launch must be >= 1");
    AdvPlanImpl &p = plan->impl;
    if (steps_per_launch > 1) {
        if (p.desc.impl == BKMA_ADV_PLAIN)
            return fail(BKMA_ERR_UNSUPPORTED, "the plain FP64 form runs one step per launch");
        if (adv_fused_tile_w(p, kMaxSmem) == 0)
            return fail(BKMA_ERR_UNSUPPORTED, "lines too long for a fused shared-memory strip");
        // FP32 lines too long for the fast strips would run one column per
        // CTA: 2x slower than one step per launch (64 x 8192 x 512: 315-382
        // vs 655 GCells/s), so fusion is refused there
        if (p.desc.dtype == BKMA_F32 && !p.fuse_x2 && !adv_fused_f32_fast(p, kMaxSmem))
            return fail(BKMA_ERR_UNSUPPORTED,
                        "FP32 lines longer than the fused strips hold (4608 rows): one step "
                        "per launch is faster");
    }
    p.fuse = steps_per_launch;
    return BKMA_OK;
} BKMA_ABI_CATCH("bkma_adv_plan_set_fusion")

bkma_status bkma_adv_plan_set_fused_state(bkma_adv_plan *plan, int32_t state) try {
    BKMA_CHECK_ARG(plan && (state == BKMA_FUSED_F32 || state == BKMA_FUSED_F32X2),
                   "state must be BKMA_FUSED_F32 or BKMA_FUSED_F32X2");
    AdvPlanImpl &p = plan->impl;
    if (state == BKMA_FUSED_F32X2) {
        if (p.desc.dtype != BKMA_F32 || p.desc.impl == BKMA_ADV_PLAIN)
            return fail(BKMA_ERR_UNSUPPORTED, "the hi + lo fused state is for FP32 staged plans");
        if (!(p.npts == 4 || p.npts == 6 || p.npts == 10))
            return fail(BKMA_ERR_UNSUPPORTED, "the hi + lo fused state needs degree 3, 5 or 9");
        if (adv_fused_x2_smem(p) > kMaxSmem || p.desc.n1 > 3632)
            return fail(BKMA_ERR_UNSUPPORTED, "lines too long for the hi + lo fused state");
    }
    p.fuse_x2 = state == BKMA_FUSED_F32X2 ? 1 : 0;
    return BKMA_OK;
} BKMA_ABI_CATCH("bkma_adv_plan_set_fused_state")

bkma_status bkma_adv_plan_set_weights(bkma_adv_plan *plan, const float *weights, int32_t on_device) try {
    BKMA_CHECK_ARG(plan && weights, "null argument");
    AdvPlanImpl &p = plan->impl;
    BKMA_CHECK_ARG(p.desc.weights == BKMA_W_TABLE, "plan was not created with BKMA_W_TABLE");
    BKMA_CHECK_ARG(p.desc.dtype == BKMA_F32, "table weights are FP32");
    const size_t bytes = sizeof(float) * (size_t)(p.lines * p.npts);
    BKMA_CUDA_TRY(cudaMemcpy(p.d_w, weights, bytes,
                             on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice));
    return BKMA_OK;
} BKMA_ABI_CATCH("bkma_adv_plan_set_weights")

bkma_status bkma_adv_plan_line_table(const bkma_adv_plan *plan, int32_t *offsets, double *shifts) try {
    BKMA_CHECK_ARG(plan, "null argument");
    const AdvPlanImpl &p = plan->impl;
    if (offsets) std::memcpy(offsets, p.base.data(), sizeof(int32_t) * (size_t)p.lines);
    if (shifts) std::memcpy(shifts, p.shift.data(), sizeof(double) * (size_t)p.lines);
    return BKMA_OK;
} BKMA_ABI_CATCH("bkma_adv_plan_line_table")

bkma_status bkma_adv_plan_destroy(bkma_adv_plan *plan) try {
    delete plan;
    return BKMA_OK;
} BKMA_ABI_CATCH("bkma_adv_plan_destroy")

bkma_status bkma_adv_step(bkma_adv_plan *plan, void *data, void *out, int32_t nsteps, void *stream) try {
    bkma::NvtxRange nvtx_range("bkma_adv_step");
    BKMA_CHECK_ARG(plan && data, "bkma_adv_step: null argument");
    BKMA_CHECK_ARG(nsteps >= 0, "nsteps must be >= 0");
    AdvPlanImpl &p = plan->impl;
    return adv_launch(p, data, out, nsteps, (cudaStream_t)stream);
} BKMA_ABI_CATCH("bkma_adv_step")

bkma_status bkma_adv_run_host(bkma_adv_plan *plan, void *host_data, int32_t nsteps, void *stream) try {
    bkma::NvtxRange nvtx_range("bkma_adv_run_host");
    BKMA_CHECK_ARG(plan && host_data, "bkma_adv_run_host: null argument");
    AdvPlanImpl &p = plan->impl;
    const size_t slab = (size_t)(p.desc.n1 * p.desc.n2) * (size_t)p.esize;
    const size_t bytes = (size_t)p.lines * slab;
    if (p.host_buf_bytes < bytes) {
        cudaFree(p.d_host_buf);
        p.d_host_buf = nullptr;
        p.host_buf_bytes = 0;
        BKMA_CUDA_TRY(cudaMalloc(&p.d_host_buf, bytes));
        p.host_buf_bytes = bytes;
    }
    cudaStream_t st = (cudaStream_t)stream;
    // Small fields, or no steps: copy in, step, copy out on the caller's stream.
    const int nch = (bytes >= ((size_t)256 << 20) && nsteps > 0)
                        ? (int)std::min<int64_t>(kRunHostChunks, p.lines) : 1;
    if (nch <= 1) {
        BKMA_CUDA_TRY(cudaMemcpyAsync(p.d_host_buf, host_data, bytes, cudaMemcpyHostToDevice, st));
        bkma_status s = adv_launch(p, p.d_host_buf, nullptr, nsteps, st);
        if (s != BKMA_OK) return s;
        BKMA_CUDA_TRY(cudaMemcpyAsync(host_data, p.d_host_buf, bytes, cudaMemcpyDeviceToHost, st));
        BKMA_CUDA_TRY(cudaStreamSynchronize(st));
        return BKMA_OK;
    }
    // Pipeline over slab chunks: chunk c = copy in, nsteps steps, copy out;
    // each chunk is a sub-plan of the same lines (same tables, bit-identical
    // results), so copies of one chunk overlap steps of others.
    if ((int)p.chunks.size() != nch) {
        for (auto *c : p.chunks) bkma_adv_plan_destroy(c);
        p.chunks.clear();
        p.chunk_l0.clear();
        for (int c = 0; c < nch; ++c) {
            const int64_t l0 = p.lines * c / nch, l1 = p.lines * (c + 1) / nch;
            bkma_adv_desc d = p.desc;
            d.i0_offset = p.desc.i0_offset + l0;
            d.i0_count = l1 - l0;
            d.velocity = p.vx.data() + l0;
            bkma_adv_plan *sub = nullptr;
            bkma_status s = bkma_adv_plan_create(&d, &sub);
            if (s != BKMA_OK) return s;
            p.chunks.push_back(sub);
            p.chunk_l0.push_back(l0);
        }
    }
    for (auto &q : p.pipe)
        if (!q) BKMA_CUDA_TRY(cudaStreamCreateWithFlags(&q, cudaStreamNonBlocking));
    for (auto &e : p.pipe_ev)
        if (!e) BKMA_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    while ((int)p.chunk_ev.size() < 2 * nch) {
        cudaEvent_t e = nullptr;
        BKMA_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        p.chunk_ev.push_back(e);
    }
    BKMA_CUDA_TRY(cudaEventRecord(p.pipe_ev[4], st));
    for (auto &q : p.pipe) BKMA_CUDA_TRY(cudaStreamWaitEvent(q, p.pipe_ev[4], 0));
    // Copies in run back to back on one stream, so the first chunk arrives
    // at the link's full rate and the steps start early; each chunk's steps
    // wait for its copy, each copy out for its steps.
    for (int c = 0; c < nch; ++c) {
        AdvPlanImpl &sp = plan_impl(p.chunks[(size_t)c]);
        sp.W = p.W;  // the parent's tile choice (set or autotuned)
        sp.R = p.R;
        sp.threads = p.threads;
        sp.path = p.path;
        sp.autotuned = p.autotuned;
        const int64_t l0 = p.chunk_l0[(size_t)c];
        const size_t nb = (size_t)sp.lines * slab;
        char *dev = (char *)p.d_host_buf + (size_t)l0 * slab;
        char *host = (char *)host_data + (size_t)l0 * slab;
        cudaEvent_t in_done = p.chunk_ev[2 * (size_t)c], stepped = p.chunk_ev[2 * (size_t)c + 1];
        BKMA_CUDA_TRY(cudaMemcpyAsync(dev, host, nb, cudaMemcpyHostToDevice, p.pipe[0]));
        BKMA_CUDA_TRY(cudaEventRecord(in_done, p.pipe[0]));
        cudaStream_t q = p.pipe[1 + (c & 1)];
        BKMA_CUDA_TRY(cudaStreamWaitEvent(q, in_done, 0));
        bkma_status s = adv_launch(sp, dev, nullptr, nsteps, q);
        if (s != BKMA_OK) return s;
        BKMA_CUDA_TRY(cudaEventRecord(stepped, q));
        BKMA_CUDA_TRY(cudaStreamWaitEvent(p.pipe[3], stepped, 0));
        BKMA_CUDA_TRY(cudaMemcpyAsync(host, dev, nb, cudaMemcpyDeviceToHost, p.pipe[3]));
    }
    for (int k = 0; k < 4; ++k) {
        BKMA_CUDA_TRY(cudaEventRecord(p.pipe_ev[k], p.pipe[k]));
        BKMA_CUDA_TRY(cudaStreamWaitEvent(st, p.pipe_ev[k], 0));
    }
    BKMA_CUDA_TRY(cudaStreamSynchronize(st));
    for (auto *c : p.chunks) {
        bkma_status s = bkma_adv_plan_status(c, stream);
        if (s != BKMA_OK) return s;
    }
    return BKMA_OK;
} BKMA_ABI_CATCH("bkma_adv_run_host")

}  // extern "C"
