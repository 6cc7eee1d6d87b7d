// FP64-storage advection computed in FP32-pair ("double-single") arithmetic.
//
// GB300 runs FP64 FMAs at a small fraction of its FP32 rate: the staged FP64
// kernel (one DMUL + NT-1 DFMA per cell) tops out near 100 GCells/s, a quarter
// of what HBM allows at 16 B per cell-step. This kernel keeps the field in
// FP64 in HBM and forms each cell's sum_k w_k f_k from FP32 pieces:
//
//  * staging: one CTA = one slab i0 x 4 or 8 columns (32- or 64-byte rows; 4
//    by default, six CTAs of 128 threads per SM) x all n1 rows, copied by TMA
//    (cp.async.bulk.tensor, FP64 tensor map) into shared memory;
//  * split: a thread walks a run of consecutive rows of one column pair and
//    splits every tap it loads once, into a register ring of npts pairs:
//    x = h + l, h = x's leading 24 bits (truncated; integer operations on the
//    bit pattern), l = the remaining 29 bits rounded to 24 (one
//    integer-to-float conversion and a power-of-two scale), so
//    |x - (h + l)| <= 2^-48 |x|; zeros split exactly. A cell pair with a tap
//    outside [2^-74, 2^126) in magnitude (or a subnormal, inf, NaN) is
//    computed in FP64 from the staged doubles (the staged kernel's
//    arithmetic, same bits), as are lines whose departure offset varies along
//    n1 (per-cell stencils);
//  * per tap, with the line's weight w = a + b split the same way on the
//    host: p = a h (rounded) and e = a h - p (exact, one FMA); the p are
//    summed by a pairwise tree of TwoSums into (S, err) so that S + sum(err)
//    is their exact sum (dependence depth 3 for 6 taps instead of 5 in a
//    running sum: 320 -> 330 GCells/s on 2048 x 1024 x 512); the small terms
//    e, err, a l and b h are added in FP32 (b l is below 2^-48 of the term and
//    dropped);
//  * output: S and L widened to FP64 with integer operations and added with
//    one DADD (correct rounding of the pair sum), one 16-byte store per
//    column pair.
//
// The sum is within a few 2^-48 of sum_k |w_k f_k| of the FP64 direct form:
// against the staged FP64 kernel the result differs by at most ~2e-13 max|f|
// per step. One step reads and writes each cell once (16 B per cell-step); the
// tile is read completely before the first store, so in place is legal.
//
// The same arithmetic per cell (ds_arith.cuh), so the same bits, in the other
// staged forms of this file (path 5): contiguous lines (n2 = 1) as 4-cell
// groups (adv_ds_rows, one per thread; adv_ds_qruns, runs of them with
// sliding register rings; adv_ds_lineq, lines of 16-128 cells shared by a
// warp's lanes through shuffles), as runs along two sections (adv_ds_runs),
// as half lines in 2-CTA clusters (adv_ds_halves, adv_ds_halves_q), k fused
// steps (adv_ds_rows_fused); and whole slabs of short lines with an even n2
// (adv_ds_slabs). Each stages its lines by bulk copies completed on an
// mbarrier with a bounded wait (stage_block2).
#include <cuda.h>

#include <algorithm>
#include <type_traits>

#include "adv.cuh"
#include "adv_device.cuh"
#include "adv_plan.cuh"
#include "common.cuh"
#include "ds_arith.cuh"
#include "tma.cuh"

namespace bkma {

namespace {

// A tile is WC FP64 columns (8: 64-byte rows, 4: 32-byte rows) x all n1 rows;
// a CTA has kDsRuns runs of rows per column pair: 32 * WC threads.
constexpr int kDsRuns = 64;
template <int WC> constexpr int ds_threads() { return kDsRuns * WC / 2; }


// Rows per thread run of a CTA with `runs` runs over n1 rows.
__host__ __device__ __forceinline__ int ds_run_rows(int64_t n1, int runs) {
    return (int)((n1 + runs - 1) / runs);
}

// One row of a thread's run: load and split the ring's newest tap (slot
// (u + NT - 1) % NT, row P[NT - 1] of this output's window), then the
// output pair from the window's taps. A tap outside the split's range sets
// `bad` (the pair is then redone in FP64 after the run).
template <int NT, int TPR>
__device__ __forceinline__ void ds_row(const double2 *P, int u, float4 (&T)[NT], bool &bad,
                                       const float2 (&A)[NT], const float2 (&B)[NT], double *G) {
    const int sn = (u + NT - 1) % NT;
    bad |= !ds_split2(P[(NT - 1) * TPR], T[sn]);
    *reinterpret_cast<double2 *>(G) = ds_stencil<NT>(T, u, A, B);
}

// Thread map: column pair g of the 8-column tile, run j of consecutive rows
// [j*RL, (j+1)*RL). A thread splits each staged tap once into a register
// ring of NT pairs (one 16-byte shared load per output row) and computes
// its rows in order. The wrap halo repeats rows 0 .. RL+NT-2 after row n1-1,
// so a run's taps never wrap: the ring walks a plain pointer.
template <int NT, int WC>
__global__ void __launch_bounds__(ds_threads<WC>(), 24 / WC) adv_ds_f64(
    const __grid_constant__ CUtensorMap tmap, AdvDsArgs a) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bar;
    constexpr int W = WC;
    constexpr int TPR = W / 2;  // column pairs per row
    const uint32_t raw = smem_u32addr(smem_raw);
    const uint32_t pad = ((raw + 127u) & ~127u) - raw;
    double *S = reinterpret_cast<double *>(smem_raw + pad);

    const int64_t line = blockIdx.x / a.ncb;
    const int c0 = (int)(blockIdx.x - line * a.ncb) * W;
    const int n1 = (int)a.n1;
    const int runs = blockDim.x / TPR;
    const int RL = ds_run_rows(n1, runs);

    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32addr(&bar)));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0)
        staging_issue(&tmap, &bar, S, (uint32_t)(a.nbox * a.box_rows * W * 8), a.nbox, a.box_rows,
                      (uint32_t)(a.box_rows * W * 8), c0, (int)line);
    const int exc = a.exc_index ? a.exc_index[line] : -1;
    const int base = a.base[line];
    float2 A[NT], B[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) {
        const float2 ab = a.w2[line * NT + k];
        A[k] = make_float2(ab.x, ab.x);
        B[k] = make_float2(ab.y, ab.y);
    }
    const bool ok_wait = __syncthreads_and(staging_wait(&bar, a.spin_limit));
    if (!ok_wait) {
        if (threadIdx.x == 0) {
            atomicExch(a.status, (int)BKMA_ERR_TIMEOUT);
            staging_wait(&bar, kWaitPolls);  // let the copies land before the CTA leaves
        }
        return;
    }
    // wrap halo: rows n1 .. n1+RL+NT-2 repeat rows 0 .. RL+NT-2
    for (int i = threadIdx.x; i < (RL + NT - 1) * W; i += blockDim.x) S[n1 * W + i] = S[i];
    __syncthreads();

    if (exc >= 0) {
        // per-cell stencils: FP64 direct form (the staged kernel's arithmetic)
        const int total = n1 * W;
        for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
            const int r = idx / W, c = idx - (idx / W) * W;
            if (c0 + c >= a.n2) continue;
            const AdvExcCell<double> &ec = a.exc[(int64_t)exc * n1 + r];
            int rr = r + ec.base;
            if (rr >= n1) rr -= n1;
            double we[NT];
#pragma unroll
            for (int k = 0; k < NT; ++k) we[k] = ec.w[k];
            a.dst[(line * a.n1 + r) * a.n2 + c0 + c] = stencil_cell<double, NT>(S + rr * W + c, W, we);
        }
        return;
    }

    const int g = threadIdx.x % TPR;
    const int rs = (int)(threadIdx.x / TPR) * RL;
    const int cnt = min(n1 - rs, RL);
    if (cnt <= 0 || c0 + 2 * g >= a.n2) return;  // n2 is even: a pair is whole or absent
    int q0 = rs + base;  // row of the first output's tap 0
    if (q0 >= n1) q0 -= n1;
    const double2 *P0 = reinterpret_cast<const double2 *>(S) + (size_t)q0 * TPR + g;
    double *G0 = a.dst + (line * a.n1 + rs) * a.n2 + c0 + 2 * g;
    float4 T[NT];
    bool bad = false;
#pragma unroll
    for (int k = 0; k < NT - 1; ++k) bad |= !ds_split2(P0[k * TPR], T[k]);
    int i = 0;
    const double2 *P = P0;
    double *G = G0;
    for (; i + NT <= cnt; i += NT) {
#pragma unroll
        for (int u = 0; u < NT; ++u) ds_row<NT, TPR>(P + u * TPR, u, T, bad, A, B, G + (int64_t)u * a.n2);
        P += NT * TPR;
        G += (int64_t)NT * a.n2;
    }
#pragma unroll
    for (int u = 0; u < NT - 1; ++u)
        if (i + u < cnt) ds_row<NT, TPR>(P + u * TPR, u, T, bad, A, B, G + (int64_t)u * a.n2);
    if (bad) {
        // a tap the split cannot carry: redo the pairs whose window holds one
        // in FP64 (the staged kernel's arithmetic); the same thread wrote them
        double w64[NT];
#pragma unroll
        for (int k = 0; k < NT; ++k) w64[k] = a.w[line * NT + k];
        for (int r = 0; r < cnt; ++r) {
            const double2 *Pr = P0 + r * TPR;
            bool ok = true;
#pragma unroll
            for (int k = 0; k < NT; ++k) {
                const double2 x = Pr[k * TPR];
                ok = ok && ds_splittable(x.x) && ds_splittable(x.y);
            }
            if (ok) continue;
            const double *p = S + (q0 + r) * W + 2 * g;
            *reinterpret_cast<double2 *>(G0 + (int64_t)r * a.n2) =
                make_double2(stencil_cell<double, NT>(p, W, w64),
                             stencil_cell<double, NT>(p + 1, W, w64));
        }
    }
}

template <int NT, int WC>
cudaError_t launch_ds_t(const CUtensorMap &tm, const AdvDsArgs &a, size_t smem, int64_t grid,
                        cudaStream_t st) {
    auto kern = adv_ds_f64<NT, WC>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<grid_x(grid), ds_threads<WC>(), smem, st>>>(tm, a);
    return cudaGetLastError();
}

// ---- contiguous lines (n2 = 1) in FP32-pair arithmetic
//
// A line is n1 consecutive doubles and a run of lines is one contiguous
// block: a CTA stages R whole lines with one bulk copy (completed on an
// mbarrier, bounded wait), then each thread computes 4 consecutive cells of
// one line. Their NT + 3 taps (the windows of 4 neighbouring cells overlap)
// are read as aligned double2s (the periodic wrap falls on double2
// boundaries: n1 % 4 == 0), shifted in registers by the line's offset mod 2
// and split once each; cells (c, c+1) and (c+2, c+3) are two lanes of the
// packed FP32x2 stencil of the column-pair kernel (the same operations per
// cell). A window holding a tap the split cannot carry, and exception lines,
// run the staged kernel's FP64 arithmetic. The CTA has read its lines before
// any store and no other CTA touches them, so in place is legal.
constexpr int kDsRowsThreads = 256;

struct AdvDsRowsArgs {
    const double *src;
    double *dst;
    int64_t n1, n2, lines;     // n2: 1 (lines), or even (slabs: adv_ds_slabs)
    int R;                     // lines per CTA
    int runs;                  // slabs: runs of rows per column pair (threads per pair)
    const int32_t *base;       // [lines]
    const double *w;           // [lines][NT]
    const float2 *w2;          // [lines][NT] FP32-pair weights
    const int32_t *exc_index;  // [lines], or null when the plan has no exception lines
    const AdvExcCell<double> *exc;
    int *status;
    uint32_t spin_limit;
};

// Stage bytes0 bytes from src0, then bytes1 bytes from src1 (0: none), into
// S by bulk copies completed on the barrier *bar (initialised here). Every
// thread of the CTA calls it; false when the bounded wait gave up (the status
// is set, and the copies have been waited for again so that nothing lands
// after the CTA leaves).
__device__ __forceinline__ bool stage_block2(double *S, const double *src0, uint32_t bytes0,
                                             const double *src1, uint32_t bytes1, uint64_t *bar,
                                             int *status, uint32_t polls) {
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32addr(bar)));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        asm volatile(
            "{\n .reg .b64 st;\n mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n}" ::"r"(
                smem_u32addr(bar)),
            "r"(bytes0 + bytes1)
            : "memory");
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
                "r"(smem_u32addr(S)),
            "l"(src0), "r"(bytes0), "r"(smem_u32addr(bar))
            : "memory");
        if (bytes1)
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
                    "r"(smem_u32addr(S) + bytes0),
                "l"(src1), "r"(bytes1), "r"(smem_u32addr(bar))
                : "memory");
    }
    if (__syncthreads_and(staging_wait(bar, polls))) return true;
    if (threadIdx.x == 0) {
        atomicExch(status, (int)BKMA_ERR_TIMEOUT);
        staging_wait(bar, kWaitPolls);  // let the copies land before the CTA leaves
    }
    return false;
}

// One contiguous block by one bulk copy.
__device__ __forceinline__ bool stage_block(double *S, const double *src, uint32_t bytes,
                                            uint64_t *bar, int *status, uint32_t polls) {
    return stage_block2(S, src, bytes, src, 0u, bar, status, polls);
}

// Cells c0 .. c0 + 3 (c0 % 4 == 0) of line `line` after one step, from its
// n1 staged values Sl: two packed pairs of the column-pair kernel's stencil
// from NT + 3 taps split once; a cell whose own window holds a tap the pair
// cannot carry, and exception lines, in FP64 arithmetic.
template <int NT>
__device__ __forceinline__ void ds_quad(const AdvDsRowsArgs &a, const double *Sl, int n1,
                                        int64_t line, int c0, double (&o)[4]) {
    constexpr int NW = NT + 3;            // taps of 4 consecutive cells
    constexpr int NV = (NW + 2) / 2;      // double2s covering them from an even start
    const int exc = a.exc_index ? a.exc_index[line] : -1;
    if (exc < 0) {
        int q = c0 + a.base[line];
        if (q >= n1) q -= n1;
        double v[2 * NV];
        int q2 = q & ~1;
#pragma unroll
        for (int j = 0; j < NV; ++j) {
            const double2 t = *reinterpret_cast<const double2 *>(Sl + q2);
            v[2 * j] = t.x;
            v[2 * j + 1] = t.y;
            q2 = q2 + 2 == n1 ? 0 : q2 + 2;
        }
        double f[NW];
        const bool odd = (q & 1) != 0;  // the same for every thread of a line
#pragma unroll
        for (int j = 0; j < NW; ++j) f[j] = odd ? v[j + 1] : v[j];
        float h[NW], lo[NW];
        bool ok = true;
#pragma unroll
        for (int j = 0; j < NW; ++j) {
            ds_split(f[j], h[j], lo[j]);
            ok = ok && ds_splittable(f[j]);
        }
        float2 A[NT], B[NT];
#pragma unroll
        for (int k = 0; k < NT; ++k) {
            const float2 ab = a.w2[line * NT + k];
            A[k] = make_float2(ab.x, ab.x);
            B[k] = make_float2(ab.y, ab.y);
        }
#pragma unroll
        for (int pr = 0; pr < 2; ++pr) {
            float4 T[NT];
#pragma unroll
            for (int k = 0; k < NT; ++k)
                T[k] = make_float4(h[2 * pr + k], h[2 * pr + k + 1], lo[2 * pr + k],
                                   lo[2 * pr + k + 1]);
            const double2 r = ds_stencil<NT>(T, 0, A, B);
            o[2 * pr] = r.x;
            o[2 * pr + 1] = r.y;
        }
        if (!ok) {
            // a cell whose own window holds a tap the pair cannot carry:
            // FP64 direct form, the staged kernel's arithmetic
            double w64[NT];
#pragma unroll
            for (int k = 0; k < NT; ++k) w64[k] = a.w[line * NT + k];
#pragma unroll
            for (int m = 0; m < 4; ++m) {
                bool own = true;
#pragma unroll
                for (int k = 0; k < NT; ++k) own = own && ds_splittable(f[m + k]);
                if (!own) o[m] = stencil_cell<double, NT>(f + m, 1, w64);
            }
        }
    } else {
        // per-cell stencils of an exception line, FP64 arithmetic
        const AdvExcCell<double> *cells = a.exc + (int64_t)exc * n1;
#pragma unroll
        for (int m = 0; m < 4; ++m) {
            const AdvExcCell<double> &e = cells[c0 + m];
            int q = c0 + m + e.base;
            if (q >= n1) q -= n1;
            double f[NT], we[NT];
#pragma unroll
            for (int k = 0; k < NT; ++k) {
                f[k] = Sl[q];
                we[k] = e.w[k];
                q = q + 1 == n1 ? 0 : q + 1;
            }
            o[m] = stencil_cell<double, NT>(f, 1, we);
        }
    }
}

template <int NT>
__global__ void __launch_bounds__(kDsRowsThreads) adv_ds_rows(AdvDsRowsArgs a) {
    extern __shared__ __align__(16) double Sd[];
    __shared__ __align__(8) uint64_t bar;
    const int n1 = (int)a.n1;
    const int64_t line0 = (int64_t)blockIdx.x * a.R;
    const int nl = (int)min((int64_t)a.R, a.lines - line0);
    const int total = nl * n1;  // a multiple of 4
    if (!stage_block(Sd, a.src + line0 * a.n1, (uint32_t)total * 8u, &bar, a.status, a.spin_limit))
        return;
    double *G = a.dst + line0 * a.n1;
    for (int i = (int)threadIdx.x * 4; i < total; i += kDsRowsThreads * 4) {
        const int l = i / n1;
        double o[4];
        ds_quad<NT>(a, Sd + (size_t)l * n1, n1, line0 + l, i - l * n1, o);
        *reinterpret_cast<double2 *>(G + i) = make_double2(o[0], o[1]);
        *reinterpret_cast<double2 *>(G + i + 2) = make_double2(o[2], o[3]);
    }
}

// k steps in one launch on contiguous lines (n2 = 1): the CTA stages its R
// lines once, then each step computes every cell with ds_quad (the one-step
// kernels' arithmetic, so the same bits as k steps of them) from one
// shared-memory copy into the other, a CTA barrier between steps; the last
// step stores to global memory. HBM traffic is 16 / k bytes per cell-step.
template <int NT>
__global__ void __launch_bounds__(kDsRowsThreads) adv_ds_rows_fused(AdvDsRowsArgs a, int ksteps) {
    extern __shared__ __align__(16) double Sd[];  // [2][R * n1]
    __shared__ __align__(8) uint64_t bar;
    const int n1 = (int)a.n1;
    const int64_t line0 = (int64_t)blockIdx.x * a.R;
    const int nl = (int)min((int64_t)a.R, a.lines - line0);
    const int total = nl * n1;  // a multiple of 4
    if (!stage_block(Sd, a.src + line0 * a.n1, (uint32_t)total * 8u, &bar, a.status, a.spin_limit))
        return;
    double *cur = Sd, *nxt = Sd + (size_t)a.R * n1;
    double *G = a.dst + line0 * a.n1;
    for (int step = 0; step < ksteps; ++step) {
        double *out = step + 1 == ksteps ? G : nxt;
        for (int i = (int)threadIdx.x * 4; i < total; i += kDsRowsThreads * 4) {
            const int l = i / n1;
            double o[4];
            ds_quad<NT>(a, cur + (size_t)l * n1, n1, line0 + l, i - l * n1, o);
            *reinterpret_cast<double2 *>(out + i) = make_double2(o[0], o[1]);
            *reinterpret_cast<double2 *>(out + i + 2) = make_double2(o[2], o[3]);
        }
        __syncthreads();  // the step's cells are written before the next reads them
        double *t = cur;
        cur = nxt;
        nxt = t;
    }
}

// Short contiguous lines shared by the lanes of a warp (path 5, W = 5; n1 =
// 4 G with G = 4, 8, 16 or 32): the G lanes of a line each take one group of
// 4 cells. Lane u of a line loads and splits the line's taps 4u .. 4u + 3
// (cells (q + 4u + e) mod n1, q the line's offset: runtime shared-memory
// addresses, no parity selects) once, and takes the taps 4u + 4 .. 4u + NT + 2
// of its group's windows from the next two lanes of the line by width-G warp
// shuffles: 4 splits per 4 cells, where the 4-cell kernel splits NT + 3. The
// two packed pairs are ds_quad's with the same split taps, so the bits are
// the 4-cell kernel's; windows holding a tap the pair cannot carry, and
// exception lines, are redone by ds_quad after the loop (the same thread
// wrote them). Every lane of a warp runs every
// shuffle (the loop covers whole warps; lanes past the CTA's lines compute
// on line 0 and store nothing). A line's lanes take its groups rotated by
// the line's index, so that the lines of a warp, which often share an
// offset, read different banks.
template <int NT, int G>
__global__ void __launch_bounds__(kDsRowsThreads) adv_ds_lineq(AdvDsRowsArgs a) {
    extern __shared__ __align__(16) double Sd[];
    __shared__ __align__(8) uint64_t bar;
    constexpr int n1 = 4 * G;
    constexpr int NW = NT + 3;  // taps of a group
    const int64_t line0 = (int64_t)blockIdx.x * a.R;
    const int nl = (int)min((int64_t)a.R, a.lines - line0);
    if (!stage_block(Sd, a.src + line0 * n1, (uint32_t)nl * (uint32_t)n1 * 8u, &bar, a.status,
                     a.spin_limit))
        return;
    const int total = (nl * G + 31) & ~31;  // whole warps
    bool any_slow = false;
    for (int t = (int)threadIdx.x; t < total; t += kDsRowsThreads) {
        const int l0 = t / G, j = t % G;
        const bool valid = l0 < nl;
        const int l = valid ? l0 : 0;
        const int u = (j + l) & (G - 1);  // this lane's group of the line
        const int64_t line = line0 + l;
        const double *Sl = Sd + (size_t)l * n1;
        const int q = a.base[line];
        float h[4], lo[4];
        uint32_t badm = 0;
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const double f = Sl[(q + 4 * u + e) & (n1 - 1)];
            ds_split(f, h[e], lo[e]);
            badm |= ds_splittable(f) ? 0u : (1u << e);
        }
        // the next two groups' taps sit with lanes j + 1 and j + 2 of the line
        const int s1 = (j + 1) & (G - 1), s2 = (j + 2) & (G - 1);
        float H[NW], L[NW];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            H[e] = h[e];
            L[e] = lo[e];
        }
#pragma unroll
        for (int e = 0; e < 4 && 4 + e < NW; ++e) {
            H[4 + e] = __shfl_sync(0xFFFFFFFFu, h[e], s1, G);
            L[4 + e] = __shfl_sync(0xFFFFFFFFu, lo[e], s1, G);
        }
#pragma unroll
        for (int e = 0; 8 + e < NW; ++e) {
            H[8 + e] = __shfl_sync(0xFFFFFFFFu, h[e], s2, G);
            L[8 + e] = __shfl_sync(0xFFFFFFFFu, lo[e], s2, G);
        }
        const uint32_t b1 = __shfl_sync(0xFFFFFFFFu, badm, s1, G);
        const uint32_t b2 = __shfl_sync(0xFFFFFFFFu, badm, s2, G);
        if (!valid) continue;  // after every shuffle
        const uint32_t bad = (badm | (b1 << 4) | (b2 << 8)) & ((1u << NW) - 1u);
        const int exc = a.exc_index ? a.exc_index[line] : -1;
        // exception lines and windows holding a tap the pair cannot carry
        // give garbage here and are redone after the loop
        any_slow = any_slow || exc >= 0 || bad != 0u;
        float2 A[NT], B[NT];
#pragma unroll
        for (int k = 0; k < NT; ++k) {
            const float2 ab = a.w2[line * NT + k];
            A[k] = make_float2(ab.x, ab.x);
            B[k] = make_float2(ab.y, ab.y);
        }
        double *Gq = a.dst + line * n1 + 4 * u;
#pragma unroll
        for (int pr = 0; pr < 2; ++pr) {
            float4 T[NT];
#pragma unroll
            for (int k = 0; k < NT; ++k)
                T[k] = make_float4(H[2 * pr + k], H[2 * pr + k + 1], L[2 * pr + k], L[2 * pr + k + 1]);
            *reinterpret_cast<double2 *>(Gq + 2 * pr) = ds_stencil<NT>(T, 0, A, B);
        }
    }
    if (!any_slow) return;
    // this thread's groups that need ds_quad, over its own stores
    for (int t = (int)threadIdx.x; t < nl * G; t += kDsRowsThreads) {
        const int l = t / G;
        const int u = (t % G + l) & (G - 1);
        const int64_t line = line0 + l;
        const double *Sl = Sd + (size_t)l * n1;
        bool slow = a.exc_index && a.exc_index[line] >= 0;
        const int q = a.base[line];
        for (int m = 0; m < NW && !slow; ++m) slow = !ds_splittable(Sl[(q + 4 * u + m) & (n1 - 1)]);
        if (!slow) continue;
        double o[4];
        ds_quad<NT>(a, Sl, n1, line, 4 * u, o);
        double *Gq = a.dst + line * n1 + 4 * u;
        *reinterpret_cast<double2 *>(Gq) = make_double2(o[0], o[1]);
        *reinterpret_cast<double2 *>(Gq + 2) = make_double2(o[2], o[3]);
    }
}

// Contiguous lines in runs of 4-cell groups (path 5, W = 4): each thread
// walks rq consecutive groups of 4 cells of one line. The NT + 3 taps of a
// group's windows slide by 4 cells from one group to the next, so a group
// loads two aligned 16-byte pairs and splits 4 new taps (one per cell, as
// the ring kernels do), and it stores its cells as two 16-byte pairs, 32
// contiguous bytes per lane (adv_ds_runs stores 8 bytes per lane, one L2
// sector per cell: 4x the output in L2 write transactions). The two packed
// pairs are ds_quad's (cells c, c + 1 and c + 2, c + 3 with the same split
// taps), so the bits are the 4-cell kernel's; exception lines go through
// ds_quad itself, and a group whose window holds a tap the pair cannot carry
// is redone by ds_quad after the run (over the same thread's stores: inlined
// in each of the three unrolled groups it made the hot loop 10 % slower).
//
// The split taps sit in a ring of 12 register slots, tap m (cell q + m) in
// slot m % 12. Group u reads taps 4u .. 4u + NT + 2, so with the groups
// unrolled by three every slot index is a compile-time constant. The raw
// values come in aligned pairs (raw value i is cell q2 + i, q2 = q rounded
// down to even); the line's parity (q odd) picks a group's four new taps out
// of its two pairs and one raw value carried from the group before.
constexpr int kDsQrunsThreads = 256;

template <int NT>
__global__ void __launch_bounds__(kDsQrunsThreads, 2) adv_ds_qruns(AdvDsRowsArgs a, int rq) {
    extern __shared__ __align__(16) double Sd[];
    __shared__ __align__(8) uint64_t bar;
    constexpr int NW = NT + 3;  // taps of a group
    constexpr int E = NW - 4;   // a group's first new tap
    constexpr int RA = NW - 3;  // a group's first new raw value (even)
    constexpr int NS = 12;      // ring slots
    const int n1 = (int)a.n1;
    const int64_t line0 = (int64_t)blockIdx.x * a.R;
    const int nl = (int)min((int64_t)a.R, a.lines - line0);
    if (!stage_block(Sd, a.src + line0 * a.n1, (uint32_t)nl * (uint32_t)n1 * 8u, &bar, a.status,
                     a.spin_limit))
        return;
    const int groups = n1 / 4;
    const int runs_pl = (groups + rq - 1) / rq;
    for (int t = (int)threadIdx.x; t < nl * runs_pl; t += kDsQrunsThreads) {
        const int l = t / runs_pl, j = t - l * runs_pl;
        const int g0 = j * rq, gn = min(rq, groups - g0);
        const int64_t line = line0 + l;
        const double *Sl = Sd + (size_t)l * n1;
        double *G = a.dst + line * a.n1 + 4 * g0;
        const int exc = a.exc_index ? a.exc_index[line] : -1;
        if (exc >= 0) {
            for (int u = 0; u < gn; ++u) {
                double o[4];
                ds_quad<NT>(a, Sl, n1, line, 4 * (g0 + u), o);
                *reinterpret_cast<double2 *>(G + 4 * u) = make_double2(o[0], o[1]);
                *reinterpret_cast<double2 *>(G + 4 * u + 2) = make_double2(o[2], o[3]);
            }
            continue;
        }
        float2 A[NT], B[NT];
#pragma unroll
        for (int k = 0; k < NT; ++k) {
            const float2 ab = a.w2[line * NT + k];
            A[k] = make_float2(ab.x, ab.x);
            B[k] = make_float2(ab.y, ab.y);
        }
        int q = 4 * g0 + a.base[line];
        if (q >= n1) q -= n1;
        const bool odd = (q & 1) != 0;
        int pn = q & ~1;  // cell of the next aligned pair to load
        float H[NS], L[NS];
        uint32_t bad = 0;  // bit m: tap (newest - m) cannot be split
        auto load2 = [&]() {
            const double2 v = *reinterpret_cast<const double2 *>(Sl + pn);
            pn = pn + 2 == n1 ? 0 : pn + 2;
            return v;
        };
        auto split = [&](int m, double f) {  // tap m (slot m % NS)
            ds_split(f, H[m % NS], L[m % NS]);
            bad = (bad << 1) | (ds_splittable(f) ? 0u : 1u);
        };
        // raw value i of the run is cell q2 + i and tap m is raw value m + odd:
        // the first group's raw values 0 .. RA - 1 give taps 0 .. E - 1, and
        // each group's two pairs (raw 4u + RA .. 4u + RA + 3) its taps
        // 4u + E .. 4u + NW - 1 with one raw value carried from the group before
        double carry;
        {
            double r[RA];
#pragma unroll
            for (int i = 0; i < RA; i += 2) {
                const double2 v = load2();
                r[i] = v.x;
                r[i + 1] = v.y;
            }
#pragma unroll
            for (int m = 0; m < E; ++m) split(m, odd ? r[m + 1] : r[m]);
            carry = r[RA - 1];
        }
        bool any_bad = false;
        auto group = [&](auto ph_c, int u) {
            constexpr int b = 4 * decltype(ph_c)::value;  // 4 (u % 3)
            const double2 v0 = load2(), v1 = load2();
            const double f[5] = {carry, v0.x, v0.y, v1.x, v1.y};
#pragma unroll
            for (int m = 0; m < NW - E; ++m) split(b + E + m, odd ? f[m + 1] : f[m]);
            carry = v1.y;
            // a window holding a tap the pair cannot carry gives garbage here
            // and is redone after the run
            any_bad = any_bad || (bad & ((1u << NW) - 1u)) != 0u;
#pragma unroll
            for (int pr = 0; pr < 2; ++pr) {
                float4 T[NT];
#pragma unroll
                for (int k = 0; k < NT; ++k) {
                    const int s0 = (b + 2 * pr + k) % NS, s1 = (b + 2 * pr + k + 1) % NS;
                    T[k] = make_float4(H[s0], H[s1], L[s0], L[s1]);
                }
                *reinterpret_cast<double2 *>(G + 4 * u + 2 * pr) = ds_stencil<NT>(T, 0, A, B);
            }
        };
        int u = 0;
        for (; u + 3 <= gn; u += 3) {
            group(std::integral_constant<int, 0>{}, u);
            group(std::integral_constant<int, 1>{}, u + 1);
            group(std::integral_constant<int, 2>{}, u + 2);
        }
        if (u < gn) group(std::integral_constant<int, 0>{}, u);
        if (u + 1 < gn) group(std::integral_constant<int, 1>{}, u + 1);
        if (!any_bad) continue;
        // the groups whose window holds a tap the pair cannot carry: ds_quad,
        // over this thread's own stores
        for (int v = 0; v < gn; ++v) {
            int c = 4 * (g0 + v) + a.base[line];
            if (c >= n1) c -= n1;
            bool ok = true;
            for (int m = 0; m < NW; ++m) {
                ok = ok && ds_splittable(Sl[c]);
                c = c + 1 == n1 ? 0 : c + 1;
            }
            if (ok) continue;
            double o[4];
            ds_quad<NT>(a, Sl, n1, line, 4 * (g0 + v), o);
            *reinterpret_cast<double2 *>(G + 4 * v) = make_double2(o[0], o[1]);
            *reinterpret_cast<double2 *>(G + 4 * v + 2) = make_double2(o[2], o[3]);
        }
    }
}

// Short lines with an even n2 > 1: whole slabs. A line of the field is a
// slab of n1 rows x n2 columns, n1 * n2 consecutive doubles, and R
// consecutive slabs are one contiguous block: a CTA stages them with one bulk
// copy (bounded wait), then each thread takes a run of rows of one column
// pair (`runs` runs per pair: 1 for lines of 16 rows, more for longer lines,
// so that a CTA has about 256 threads) with the column-pair kernel's register
// ring (every tap split once, the same stencil per cell and the same FP64
// redo of windows the pair cannot carry: the same bits as adv_ds_f64), the
// periodic wrap taken by the tap pointer. That kernel spreads 64 runs over
// the rows of each column pair, which leaves lines shorter than 128 rows runs
// of one or two rows.
constexpr int kDsSlabThreads = 256;

template <int NT>
__global__ void __launch_bounds__(kDsSlabThreads, 3) adv_ds_slabs(AdvDsRowsArgs a) {
    extern __shared__ __align__(16) double Sd[];
    __shared__ __align__(8) uint64_t bar;
    const int n1 = (int)a.n1;
    const int P2 = (int)(a.n2 / 2);  // column pairs per row
    const int64_t slab = a.n1 * a.n2;
    const int64_t line0 = (int64_t)blockIdx.x * a.R;
    const int nl = (int)min((int64_t)a.R, a.lines - line0);
    if (!stage_block(Sd, a.src + line0 * slab, (uint32_t)(nl * slab) * 8u, &bar, a.status,
                     a.spin_limit))
        return;
    const int RP = a.runs;
    const int RL = (n1 + RP - 1) / RP;
    const int units = nl * RP * P2;
    // consecutive threads: consecutive column pairs of one run
    auto unit = [&](int t, int &l, int &g, int &r0, int &cnt) {
        const int lj = t / P2;
        g = t - lj * P2;
        l = lj / RP;
        r0 = (lj - l * RP) * RL;
        cnt = min(n1 - r0, RL);
    };
    bool any_bad = false;
    for (int t = threadIdx.x; t < units; t += kDsSlabThreads) {
        int l, g, r0, cnt;
        unit(t, l, g, r0, cnt);
        if (cnt <= 0) continue;
        const int64_t line = line0 + l;
        // row 0 of the thread's column pair
        const double2 *S0 = reinterpret_cast<const double2 *>(Sd + (size_t)l * slab) + g;
        double *G = a.dst + line * slab + 2 * g;
        const int exc = a.exc_index ? a.exc_index[line] : -1;
        if (exc >= 0) {
            // per-cell stencils of an exception line, FP64 arithmetic
            const AdvExcCell<double> *cells = a.exc + (int64_t)exc * n1;
            for (int r = r0; r < r0 + cnt; ++r) {
                const AdvExcCell<double> &e = cells[r];
                int q = r + e.base;
                if (q >= n1) q -= n1;
                double fx[NT], fy[NT], we[NT];
#pragma unroll
                for (int k = 0; k < NT; ++k) {
                    const double2 x = S0[(size_t)q * P2];
                    fx[k] = x.x;
                    fy[k] = x.y;
                    we[k] = e.w[k];
                    q = q + 1 == n1 ? 0 : q + 1;
                }
                *reinterpret_cast<double2 *>(G + (int64_t)r * a.n2) =
                    make_double2(stencil_cell<double, NT>(fx, 1, we), stencil_cell<double, NT>(fy, 1, we));
            }
            continue;
        }
        float2 A[NT], B[NT];
#pragma unroll
        for (int k = 0; k < NT; ++k) {
            const float2 ab = a.w2[line * NT + k];
            A[k] = make_float2(ab.x, ab.x);
            B[k] = make_float2(ab.y, ab.y);
        }
        int q0 = a.base[line] + r0;  // row of output row r0's tap 0
        if (q0 >= n1) q0 -= n1;
        const double2 *P = S0 + (size_t)q0 * P2;
        int left = n1 - q0;  // rows before the tap pointer wraps to row 0
        float4 T[NT];
        bool bad = false;
        auto advance = [&]() {
            P += P2;
            if (--left == 0) {
                P = S0;
                left = n1;
            }
        };
#pragma unroll
        for (int k = 0; k < NT - 1; ++k) {
            bad |= !ds_split2(*P, T[k]);
            advance();
        }
        double *Gr = G + (int64_t)r0 * a.n2;
        auto row = [&](int u) {
            bad |= !ds_split2(*P, T[(u + NT - 1) % NT]);
            advance();
            *reinterpret_cast<double2 *>(Gr) = ds_stencil<NT>(T, u, A, B);
            Gr += a.n2;
        };
        int i = 0;
        for (; i + NT <= cnt; i += NT) {
#pragma unroll
            for (int u = 0; u < NT; ++u) row(u);
        }
#pragma unroll
        for (int u = 0; u < NT - 1; ++u)
            if (i + u < cnt) row(u);
        any_bad |= bad;
    }
    if (!any_bad) return;
    // a tap the split cannot carry: redo the pairs whose window holds one in
    // FP64 (the staged kernel's arithmetic); this thread wrote them
    for (int t = threadIdx.x; t < units; t += kDsSlabThreads) {
        int l, g, r0, cnt;
        unit(t, l, g, r0, cnt);
        const int64_t line = line0 + l;
        if (cnt <= 0 || (a.exc_index && a.exc_index[line] >= 0)) continue;
        const double2 *S0 = reinterpret_cast<const double2 *>(Sd + (size_t)l * slab) + g;
        double *G = a.dst + line * slab + 2 * g;
        double w64[NT];
#pragma unroll
        for (int k = 0; k < NT; ++k) w64[k] = a.w[line * NT + k];
        int q = a.base[line] + r0;
        if (q >= n1) q -= n1;
        for (int r = r0; r < r0 + cnt; ++r) {
            int qk = q;
            double fx[NT], fy[NT];
            bool ok = true;
#pragma unroll
            for (int k = 0; k < NT; ++k) {
                const double2 x = S0[(size_t)qk * P2];
                fx[k] = x.x;
                fy[k] = x.y;
                ok = ok && ds_splittable(x.x) && ds_splittable(x.y);
                qk = qk + 1 == n1 ? 0 : qk + 1;
            }
            q = q + 1 == n1 ? 0 : q + 1;
            if (ok) continue;
            *reinterpret_cast<double2 *>(G + (int64_t)r * a.n2) =
                make_double2(stencil_cell<double, NT>(fx, 1, w64), stencil_cell<double, NT>(fy, 1, w64));
        }
    }
}

// Long contiguous lines (n1 >= 512): each thread walks a run of RL
// consecutive cells (RL odd, so that the 8-byte shared-memory loads of the 32
// runs of a warp fall in distinct banks) of two line sections at once - two
// lines, or the two halves of one line when a CTA holds a single line - as
// the two lanes of the packed pair stencil, each lane with its own line
// weights, splitting every tap once into a register ring (the column-pair
// kernel's scheme). Windows the pair cannot carry and exception lines run the
// staged kernel's FP64 arithmetic from the staged lines.
constexpr int kDsRunsThreads = 256;
// cells either side of a line's offset that its exception cells' offsets may
// take (the staged window of a half line; the plan checks it)
constexpr int kDsHalfMargin = 2;

template <int NT>
__global__ void __launch_bounds__(kDsRunsThreads, 3) adv_ds_runs(AdvDsRowsArgs a, int rl) {
    extern __shared__ __align__(16) double Sd[];
    __shared__ __align__(8) uint64_t bar;
    const int n1 = (int)a.n1;
    const int64_t line0 = (int64_t)blockIdx.x * a.R;
    const int nl = (int)min((int64_t)a.R, a.lines - line0);
    if (!stage_block(Sd, a.src + line0 * a.n1, (uint32_t)nl * (uint32_t)n1 * 8u, &bar, a.status,
                     a.spin_limit))
        return;
    // sections: pairs of lines (an odd last line pairs with itself and stores
    // once), or the two halves of the CTA's single line
    const bool halves = a.R == 1;
    const int runs_pp = halves ? kDsRunsThreads : kDsRunsThreads / (a.R / 2);
    const int p = (int)threadIdx.x / runs_pp, j = (int)threadIdx.x % runs_pp;
    const int npairs = halves ? 1 : (nl + 1) / 2;
    const int seclen = halves ? n1 / 2 : n1;
    const int c0 = j * rl;
    const int cnt = min(rl, seclen - c0);
    if (p >= npairs || cnt <= 0) return;
    int lx = halves ? 0 : 2 * p;
    int ly = halves ? 0 : min(2 * p + 1, nl - 1);
    bool store_y = halves || ly != lx;
    int ox = 0, oy = halves ? n1 / 2 : 0;
    int64_t gx = line0 + lx, gy = line0 + ly;
    const double *Sx = Sd + (size_t)lx * n1, *Sy = Sd + (size_t)ly * n1;
    double *Gx = a.dst + gx * a.n1 + ox + c0, *Gy = a.dst + gy * a.n1 + oy + c0;
    const int ex = a.exc_index ? a.exc_index[gx] : -1;
    const int ey = a.exc_index ? a.exc_index[gy] : -1;
    // an exception line's section: per-cell stencils in FP64 arithmetic (the
    // staged kernel's); its partner, if it is not one, keeps the pair
    // arithmetic (with both lanes on it), so that no cell's bits depend on
    // which lines share a CTA
    for (int s2 = 0; s2 < (store_y ? 2 : 1); ++s2) {
        const int e = s2 ? ey : ex;
        if (e < 0) continue;
        const double *Sl = s2 ? Sy : Sx;
        double *G = s2 ? Gy : Gx;
        const int o = (s2 ? oy : ox) + c0;
        for (int i = 0; i < cnt; ++i) {
            const AdvExcCell<double> &ec = a.exc[(int64_t)e * n1 + o + i];
            int q = o + i + ec.base;
            if (q >= n1) q -= n1;
            double f[NT], we[NT];
#pragma unroll
            for (int k = 0; k < NT; ++k) {
                f[k] = Sl[q];
                we[k] = ec.w[k];
                q = q + 1 == n1 ? 0 : q + 1;
            }
            G[i] = stencil_cell<double, NT>(f, 1, we);
        }
    }
    if (ex >= 0 && (ey >= 0 || !store_y)) return;
    if (ex >= 0 || ey >= 0) {
        // the one normal section on both lanes
        const bool xn = ex < 0;
        lx = xn ? lx : ly;
        ox = xn ? ox : oy;
        gx = xn ? gx : gy;
        Sx = xn ? Sx : Sy;
        Gx = xn ? Gx : Gy;
        ly = lx;
        oy = ox;
        gy = gx;
        Sy = Sx;
        Gy = Gx;
        store_y = false;
    }
    float2 A[NT], B[NT];
    double wx[NT], wy[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) {
        const float2 abx = a.w2[gx * NT + k], aby = a.w2[gy * NT + k];
        A[k] = make_float2(abx.x, aby.x);
        B[k] = make_float2(abx.y, aby.y);
    }
    // tap 0 of the first cell of each section, and the ring of split taps
    int qx = ox + c0 + a.base[gx], qy = oy + c0 + a.base[gy];
    if (qx >= n1) qx -= n1;
    if (qy >= n1) qy -= n1;
    const int qx0 = qx, qy0 = qy;
    float4 T[NT];
    uint32_t bad = 0;
#pragma unroll
    for (int k = 0; k < NT - 1; ++k) {
        bad = (bad << 1) | (ds_split2(make_double2(Sx[qx], Sy[qy]), T[k]) ? 0u : 1u);
        qx = qx + 1 == n1 ? 0 : qx + 1;
        qy = qy + 1 == n1 ? 0 : qy + 1;
    }
    bool any_bad = false;
    int i = 0;
    auto row = [&](auto u_c) {
        constexpr int u = decltype(u_c)::value;
        bad = ((bad << 1) | (ds_split2(make_double2(Sx[qx], Sy[qy]), T[(u + NT - 1) % NT]) ? 0u : 1u)) &
              ((1u << NT) - 1u);
        qx = qx + 1 == n1 ? 0 : qx + 1;
        qy = qy + 1 == n1 ? 0 : qy + 1;
        const double2 r = ds_stencil<NT>(T, u, A, B);
        any_bad = any_bad || bad != 0u;
        Gx[i] = r.x;
        if (store_y) Gy[i] = r.y;
        ++i;
    };
    for (; i + NT <= cnt;) {
        row(std::integral_constant<int, 0>{});
        row(std::integral_constant<int, 1>{});
        row(std::integral_constant<int, 2>{});
        row(std::integral_constant<int, 3>{});
        if constexpr (NT > 4) {
            row(std::integral_constant<int, 4 % NT>{});
            row(std::integral_constant<int, 5 % NT>{});
        }
    }
    if (i < cnt) row(std::integral_constant<int, 0>{});
    if (i < cnt) row(std::integral_constant<int, 1>{});
    if (i < cnt) row(std::integral_constant<int, 2>{});
    if constexpr (NT > 4) {
        if (i < cnt) row(std::integral_constant<int, 3>{});
        if (i < cnt) row(std::integral_constant<int, 4 % NT>{});
    }
    if (any_bad) {
        // windows holding a tap the pair cannot carry: FP64 arithmetic (the
        // staged kernel's) for both sections' cells of those windows
#pragma unroll
        for (int k = 0; k < NT; ++k) {
            wx[k] = a.w[gx * NT + k];
            wy[k] = a.w[gy * NT + k];
        }
        int px = qx0, py = qy0;
        for (int c = 0; c < cnt; ++c) {
            double fx[NT], fy[NT];
            bool okx = true, oky = true;
            int tx = px, ty = py;
#pragma unroll
            for (int k = 0; k < NT; ++k) {
                fx[k] = Sx[tx];
                fy[k] = Sy[ty];
                okx = okx && ds_splittable(fx[k]);
                oky = oky && ds_splittable(fy[k]);
                tx = tx + 1 == n1 ? 0 : tx + 1;
                ty = ty + 1 == n1 ? 0 : ty + 1;
            }
            // each lane's cell by its own window
            if (!okx) Gx[c] = stencil_cell<double, NT>(fx, 1, wx);
            if (!oky && store_y) Gy[c] = stencil_cell<double, NT>(fy, 1, wy);
            px = px + 1 == n1 ? 0 : px + 1;
            py = py + 1 == n1 ? 0 : py + 1;
        }
    }
}

// Lines of 8192 cells and more (64 KB and more: one or two CTAs per SM with
// the whole line staged) split between the two CTAs of a cluster. CTA h of a
// line stages only the cells its half's stencils read - [h n1/2 + base - M,
// (h + 1) n1/2 + base + NT - 1 + M) modulo n1, M = kDsHalfMargin cells for
// the offsets of exception lines, in at most two bulk copies - and computes
// its half's cells as the run kernel does, the two lanes of the packed
// stencil on the half's two quarters. A cluster barrier after the staging
// orders every read of the line's original values before either CTA writes,
// so in place is legal; every thread of both CTAs reaches it once, also after
// a staging timeout. The same per-cell arithmetic as adv_ds_runs: the same bits.
template <int NT>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(kDsRunsThreads, 3)
    adv_ds_halves(AdvDsRowsArgs a, int rl, int win) {
    extern __shared__ __align__(16) double Sd[];  // [win] cells of the line from cell w0
    __shared__ __align__(8) uint64_t bar;
    const int n1 = (int)a.n1;
    const int h = n1 / 2, q = n1 / 4;
    const int64_t line = blockIdx.x >> 1;
    const int s0 = (int)(blockIdx.x & 1) * h;  // first cell of this CTA's half
    const int base = a.base[line];
    // first staged cell, even (16-byte aligned copies)
    int w0 = (s0 + base - kDsHalfMargin) % n1;
    if (w0 < 0) w0 += n1;
    w0 &= ~1;
    const int first = min(win, n1 - w0);
    const double *L = a.src + line * a.n1;
    const bool staged = stage_block2(Sd, L + w0, (uint32_t)first * 8u, L, (uint32_t)(win - first) * 8u,
                                     &bar, a.status, a.spin_limit);
    // both halves of the line are staged before either CTA writes to it
    asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
    asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
    if (!staged) return;
    auto local = [&](int g) {  // staged index of cell g of the line
        int t = g - w0;
        if (t < 0) t += n1;
        return t;
    };
    const int j = (int)threadIdx.x;
    const int c0 = j * rl;
    const int cnt = min(rl, q - c0);
    if (cnt <= 0) return;
    double *Gx = a.dst + line * a.n1 + s0 + c0, *Gy = Gx + q;
    const int e = a.exc_index ? a.exc_index[line] : -1;
    if (e >= 0) {
        // an exception line: per-cell stencils in FP64 arithmetic
        for (int s2 = 0; s2 < 2; ++s2) {
            const int o = s0 + s2 * q + c0;
            double *G = s2 ? Gy : Gx;
            for (int i = 0; i < cnt; ++i) {
                const AdvExcCell<double> &ec = a.exc[(int64_t)e * n1 + o + i];
                int g = o + i + ec.base;
                if (g >= n1) g -= n1;
                int t = local(g);
                double f[NT], we[NT];
#pragma unroll
                for (int k = 0; k < NT; ++k) {
                    f[k] = Sd[t + k];
                    we[k] = ec.w[k];
                }
                G[i] = stencil_cell<double, NT>(f, 1, we);
            }
        }
        return;
    }
    float2 A[NT], B[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) {
        const float2 ab = a.w2[line * NT + k];
        A[k] = make_float2(ab.x, ab.x);
        B[k] = make_float2(ab.y, ab.y);
    }
    // tap 0 of the run's first cell in each quarter; the window never wraps
    int gx = s0 + c0 + base;
    if (gx >= n1) gx -= n1;
    const int qx0 = local(gx), qy0 = qx0 + q;
    int qx = qx0, qy = qy0;
    float4 T[NT];
    uint32_t bad = 0;
#pragma unroll
    for (int k = 0; k < NT - 1; ++k) {
        bad = (bad << 1) | (ds_split2(make_double2(Sd[qx], Sd[qy]), T[k]) ? 0u : 1u);
        ++qx;
        ++qy;
    }
    bool any_bad = false;
    int i = 0;
    auto row = [&](auto u_c) {
        constexpr int u = decltype(u_c)::value;
        bad = ((bad << 1) | (ds_split2(make_double2(Sd[qx], Sd[qy]), T[(u + NT - 1) % NT]) ? 0u : 1u)) &
              ((1u << NT) - 1u);
        ++qx;
        ++qy;
        const double2 r = ds_stencil<NT>(T, u, A, B);
        any_bad = any_bad || bad != 0u;
        Gx[i] = r.x;
        Gy[i] = r.y;
        ++i;
    };
    for (; i + NT <= cnt;) {
        row(std::integral_constant<int, 0>{});
        row(std::integral_constant<int, 1>{});
        row(std::integral_constant<int, 2>{});
        row(std::integral_constant<int, 3>{});
        if constexpr (NT > 4) {
            row(std::integral_constant<int, 4 % NT>{});
            row(std::integral_constant<int, 5 % NT>{});
        }
    }
    if (i < cnt) row(std::integral_constant<int, 0>{});
    if (i < cnt) row(std::integral_constant<int, 1>{});
    if (i < cnt) row(std::integral_constant<int, 2>{});
    if constexpr (NT > 4) {
        if (i < cnt) row(std::integral_constant<int, 3>{});
        if (i < cnt) row(std::integral_constant<int, 4 % NT>{});
    }
    if (any_bad) {
        // windows holding a tap the pair cannot carry: each lane's cell by
        // its own window in FP64 arithmetic (the staged kernel's)
        double w64[NT];
#pragma unroll
        for (int k = 0; k < NT; ++k) w64[k] = a.w[line * NT + k];
        for (int c = 0; c < cnt; ++c) {
            double fx[NT], fy[NT];
            bool okx = true, oky = true;
#pragma unroll
            for (int k = 0; k < NT; ++k) {
                fx[k] = Sd[qx0 + c + k];
                fy[k] = Sd[qy0 + c + k];
                okx = okx && ds_splittable(fx[k]);
                oky = oky && ds_splittable(fy[k]);
            }
            if (!okx) Gx[c] = stencil_cell<double, NT>(fx, 1, w64);
            if (!oky) Gy[c] = stencil_cell<double, NT>(fy, 1, w64);
        }
    }
}

// Half lines in 2-CTA clusters (staged and ordered as in adv_ds_halves)
// computed in runs of 4-cell groups (the rings of adv_ds_qruns, 32
// contiguous bytes stored per lane and group): the half's window needs no
// wrap, so the rings load plain staged indices. A cell whose own window holds
// a tap the pair cannot carry is redone in FP64 after the run, as ds_quad
// does; exception lines take per-cell FP64 stencils. The same bits.
template <int NT>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(kDsQrunsThreads, 2)
    adv_ds_halves_q(AdvDsRowsArgs a, int rq, int win) {
    extern __shared__ __align__(16) double Sd[];  // [win] cells of the line from cell w0
    __shared__ __align__(8) uint64_t bar;
    constexpr int NW = NT + 3;  // taps of a group
    constexpr int E = NW - 4;   // a group's first new tap
    constexpr int RA = NW - 3;  // a group's first new raw value (even)
    constexpr int NS = 12;      // ring slots
    const int n1 = (int)a.n1;
    const int h = n1 / 2;
    const int64_t line = blockIdx.x >> 1;
    const int s0 = (int)(blockIdx.x & 1) * h;  // first cell of this CTA's half
    const int base = a.base[line];
    int w0 = (s0 + base - kDsHalfMargin) % n1;  // first staged cell, even
    if (w0 < 0) w0 += n1;
    w0 &= ~1;
    const int first = min(win, n1 - w0);
    const double *Lp = a.src + line * a.n1;
    const bool staged = stage_block2(Sd, Lp + w0, (uint32_t)first * 8u, Lp,
                                     (uint32_t)(win - first) * 8u, &bar, a.status, a.spin_limit);
    // both halves of the line are staged before either CTA writes to it
    asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
    asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
    if (!staged) return;
    auto local = [&](int g) {  // staged index of cell g of the line
        int t = g - w0;
        if (t < 0) t += n1;
        return t;
    };
    const int off = local(s0 + base >= n1 ? s0 + base - n1 : s0 + base);  // tap 0 of cell s0
    const int groups = h / 4;
    const int e = a.exc_index ? a.exc_index[line] : -1;
    double *G = a.dst + line * a.n1 + s0;
    float2 A[NT], B[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) {
        const float2 ab = a.w2[line * NT + k];
        A[k] = make_float2(ab.x, ab.x);
        B[k] = make_float2(ab.y, ab.y);
    }
    for (int t = (int)threadIdx.x; t * rq < groups; t += kDsQrunsThreads) {
        const int g0 = t * rq, gn = min(rq, groups - g0);
        bool any_bad = e >= 0;
        if (e < 0) {
            const int q = off + 4 * g0;  // staged index of the run's tap 0
            const bool odd = (q & 1) != 0;
            int pn = q & ~1;
            float H[NS], L[NS];
            uint32_t bad = 0;
            auto load2 = [&]() {
                const double2 v = *reinterpret_cast<const double2 *>(Sd + pn);
                pn += 2;
                return v;
            };
            auto split = [&](int m, double f) {
                ds_split(f, H[m % NS], L[m % NS]);
                bad = (bad << 1) | (ds_splittable(f) ? 0u : 1u);
            };
            double carry;
            {
                double r[RA];
#pragma unroll
                for (int i = 0; i < RA; i += 2) {
                    const double2 v = load2();
                    r[i] = v.x;
                    r[i + 1] = v.y;
                }
#pragma unroll
                for (int m = 0; m < E; ++m) split(m, odd ? r[m + 1] : r[m]);
                carry = r[RA - 1];
            }
            auto group = [&](auto ph_c, int u) {
                constexpr int b = 4 * decltype(ph_c)::value;  // 4 (u % 3)
                const double2 v0 = load2(), v1 = load2();
                const double f[5] = {carry, v0.x, v0.y, v1.x, v1.y};
#pragma unroll
                for (int m = 0; m < NW - E; ++m) split(b + E + m, odd ? f[m + 1] : f[m]);
                carry = v1.y;
                any_bad = any_bad || (bad & ((1u << NW) - 1u)) != 0u;
                double *Gq = G + 4 * (g0 + u);
#pragma unroll
                for (int pr = 0; pr < 2; ++pr) {
                    float4 T[NT];
#pragma unroll
                    for (int k = 0; k < NT; ++k) {
                        const int t0 = (b + 2 * pr + k) % NS, t1 = (b + 2 * pr + k + 1) % NS;
                        T[k] = make_float4(H[t0], H[t1], L[t0], L[t1]);
                    }
                    *reinterpret_cast<double2 *>(Gq + 2 * pr) = ds_stencil<NT>(T, 0, A, B);
                }
            };
            int u = 0;
            for (; u + 3 <= gn; u += 3) {
                group(std::integral_constant<int, 0>{}, u);
                group(std::integral_constant<int, 1>{}, u + 1);
                group(std::integral_constant<int, 2>{}, u + 2);
            }
            if (u < gn) group(std::integral_constant<int, 0>{}, u);
            if (u + 1 < gn) group(std::integral_constant<int, 1>{}, u + 1);
        }
        if (!any_bad) continue;
        // per cell in FP64: an exception line's cells with their own weights,
        // otherwise the cells whose own window the pair cannot carry (this
        // thread's own stores)
        double w64[NT];
#pragma unroll
        for (int k = 0; k < NT; ++k) w64[k] = a.w[line * NT + k];
        for (int c = 4 * g0; c < 4 * (g0 + gn); ++c) {
            double fv[NT], we[NT];
            int t0 = off + c;
            if (e >= 0) {
                const AdvExcCell<double> &ec = a.exc[(int64_t)e * n1 + s0 + c];
                int g = s0 + c + ec.base;
                if (g >= n1) g -= n1;
                t0 = local(g);
#pragma unroll
                for (int k = 0; k < NT; ++k) we[k] = ec.w[k];
            } else {
#pragma unroll
                for (int k = 0; k < NT; ++k) we[k] = w64[k];
            }
            bool ok = e < 0;
#pragma unroll
            for (int k = 0; k < NT; ++k) {
                fv[k] = Sd[t0 + k];
                ok = ok && ds_splittable(fv[k]);
            }
            if (!ok) G[c] = stencil_cell<double, NT>(fv, 1, we);
        }
    }
}

}  // namespace

size_t adv_ds_smem(const AdvPlanImpl &p, int W) {
    const int64_t n1 = p.desc.n1;
    const int box_rows = (int)std::min<int64_t>(256, n1);
    const int64_t nbox = (n1 + box_rows - 1) / box_rows;
    const int RL = ds_run_rows(n1, kDsRuns);
    const int64_t rows = std::max<int64_t>(nbox * box_rows, n1 + RL + p.npts - 1);
    return (size_t)rows * W * 8 + 128;
}

bool adv_ds_shape_ok(const AdvPlanImpl &p, int W) {
    return p.desc.dtype == BKMA_F64 && p.desc.impl != BKMA_ADV_PLAIN && p.d_w2 != nullptr &&
           (W == 4 || W == 8) && (p.npts == 4 || p.npts == 6) && p.desc.n2 % 2 == 0 &&
           p.desc.n2 >= W && p.desc.n1 >= 16 && p.lines < (1ll << 31) &&
           tensor_map_encoder() != nullptr;
}

bool adv_ds_eligible(const AdvPlanImpl &p, const void *src, int W) {
    return adv_ds_shape_ok(p, W) && ((uintptr_t)src % 16) == 0;
}

int adv_ds_threads(int W) { return W == 4 ? ds_threads<4>() : ds_threads<8>(); }

cudaError_t adv_ds_launch(AdvPlanImpl &p, const void *src, void *dst, int W, cudaStream_t st) {
    const CUtensorMap *tm = adv_field_tmap(p, src, W);
    if (!tm) return cudaErrorInvalidValue;
    AdvDsArgs a;
    a.dst = (double *)dst;
    a.n1 = p.desc.n1;
    a.n2 = p.desc.n2;
    a.ncb = p.ncb(W);
    a.box_rows = (int)std::min<int64_t>(256, p.desc.n1);
    a.nbox = (int)((p.desc.n1 + a.box_rows - 1) / a.box_rows);
    a.base = p.d_base;
    a.w = (const double *)p.d_w;
    a.w2 = p.d_w2;
    a.exc_index = p.n_exc > 0 ? p.d_exc_index : nullptr;
    a.exc = (const AdvExcCell<double> *)p.d_exc;
    a.status = p.d_status;
    a.spin_limit = p.wait_polls;
    const size_t smem = adv_ds_smem(p, W);
    const int64_t grid = p.lines * a.ncb;
    if (W == 4) {
        if (p.npts == 6) return launch_ds_t<6, 4>(*tm, a, smem, grid, st);
        return launch_ds_t<4, 4>(*tm, a, smem, grid, st);
    }
    if (p.npts == 6) return launch_ds_t<6, 8>(*tm, a, smem, grid, st);
    return launch_ds_t<4, 8>(*tm, a, smem, grid, st);
}

size_t adv_ds_rows_smem(const AdvPlanImpl &p, int R) {
    return (size_t)R * (size_t)p.desc.n1 * (size_t)p.desc.n2 * sizeof(double);
}

bool adv_ds_rows_shape_ok(const AdvPlanImpl &p) {
    const int64_t n1 = p.desc.n1, n2 = p.desc.n2;
    const bool lines = n2 == 1 && n1 % 4 == 0 && n1 >= 16;
    const bool slabs = n2 >= 2 && n2 % 2 == 0;
    return p.desc.dtype == BKMA_F64 && p.desc.impl != BKMA_ADV_PLAIN && p.d_w2 != nullptr &&
           (lines || slabs) && (p.npts == 4 || p.npts == 6) && p.lines * n1 * n2 < (1ll << 40);
}

bool adv_ds_rows_eligible(const AdvPlanImpl &p, const void *src, const void *dst, int R) {
    // one bulk copy per CTA, within the barrier's transaction count
    return adv_ds_rows_shape_ok(p) && R >= 1 && ((uintptr_t)src % 16) == 0 &&
           ((uintptr_t)dst % 16) == 0 && adv_ds_rows_smem(p, R) < (1 << 20) &&
           adv_ds_rows_smem(p, R) <= (size_t)227 * 1024 - 16;  // + the static barrier
}

bool adv_ds_runs_ok(const AdvPlanImpl &p, int R) {
    return adv_ds_rows_shape_ok(p) && p.desc.n2 == 1 && p.desc.n1 >= 512 &&
           (R == 1 || (R % 2 == 0 && R <= 16));
}

void adv_ds_rows_default(const AdvPlanImpl &p, int *W, int *R) {
    if (p.desc.n2 > 1) {
        // slabs: up to 256 column pairs and 64 KB (three CTAs per SM) per
        // CTA, then runs of >= 16 rows per pair up to about 256 threads
        const int64_t pairs = p.desc.n2 / 2, bytes = p.desc.n1 * p.desc.n2 * 8;
        const int64_t r = std::min<int64_t>(
            std::max<int64_t>(1, std::min(kDsSlabThreads / pairs, 65536 / bytes)), p.lines);
        int runs = 1;
        while (runs < 8 && r * pairs * runs * 2 <= kDsSlabThreads && p.desc.n1 / (runs * 2) >= 16)
            runs *= 2;
        *W = runs;
        *R = (int)r;
        return;
    }
    // long lines: the run-based kernel with about 8192 cells (64 KB) per CTA
    // (an even number of lines, or one line from 8192 cells on), when that
    // leaves at least two CTAs per SM; otherwise the 4-cell kernel with
    // about 4096 cells (32 KB) per CTA (512 x 1024 x 1: 55.5 GCells/s against
    // 44.5 for 64 CTAs of 8 lines)
    const int64_t n1 = p.desc.n1;
    if (n1 > 8192 && 2 * p.lines >= 2 * 152 && adv_ds_halves_ok(p)) {
        // a whole line would leave one CTA per SM, its staging not overlapped
        // with any arithmetic: half lines in 2-CTA clusters, in runs of 4-cell
        // groups (2^17 x 16384 x 1, GCells/s: whole lines 190, half lines
        // with runs along the quarters 207, with runs of 4-cell groups 215;
        // at 8192 cells the half lines' 32 KB leave too little in flight:
        // 169 against 233 for whole lines in runs of 4-cell groups)
        *W = 6;
        *R = 1;
        return;
    }
    if (adv_ds_lineq_ok(p)) {
        // lines of 16-128 cells shared by a warp's lanes, 8192 cells (64 KB)
        // per CTA (x 1 lines, 2^27 cells and more, GCells/s, 4-cell kernel ->
        // shared lines: n1 = 16 201 -> 213, 32 200 -> 213, 64 203 -> 219,
        // 128 205 -> 217; 4096 cells per CTA 199-206, 12288 165-173; runs of
        // 4-cell groups 199-225)
        const int64_t r = std::min<int64_t>(8192 / n1, p.lines);
        if ((p.lines + r - 1) / r >= 2 * 152) {
            *W = 5;
            *R = (int)r;
            return;
        }
    }
    if (n1 >= 256 && n1 <= 8192) {
        // runs of 4-cell groups with about 12288 cells (96 KB: two CTAs per
        // SM) per CTA (x 1 lines, 2^27 cells and more, GCells/s, run kernel
        // or 4-cell kernel -> group runs: n1 = 256 210 -> 261, 1024 208 ->
        // 270, 4096 209 -> 272, 8192 205 -> 230; 8192 cells per CTA: 222-248)
        const int64_t r = std::min<int64_t>(std::max<int64_t>(1, 12288 / n1), p.lines);
        if ((p.lines + r - 1) / r >= 2 * 152) {
            *W = 4;
            *R = (int)r;
            return;
        }
    }
    if (n1 >= 512) {
        int64_t r = n1 >= 8192 ? 1 : std::max<int64_t>(2, (8192 / n1) & ~int64_t(1));
        r = std::min<int64_t>(r, p.lines);
        if (r > 1 && r % 2) --r;
        if ((p.lines + r - 1) / r >= 2 * 152 && adv_ds_runs_ok(p, (int)r)) {
            *W = 2;
            *R = (int)r;
            return;
        }
    }
    *W = 1;
    *R = (int)std::min<int64_t>(std::max<int64_t>(1, 4096 / n1), p.lines);
}

namespace {

AdvDsRowsArgs rows_args(const AdvPlanImpl &p, const void *src, void *dst, int R) {
    AdvDsRowsArgs a;
    a.src = (const double *)src;
    a.dst = (double *)dst;
    a.n1 = p.desc.n1;
    a.n2 = p.desc.n2;
    a.lines = p.lines;
    a.R = R;
    a.runs = 1;
    a.base = p.d_base;
    a.w = (const double *)p.d_w;
    a.w2 = p.d_w2;
    a.exc_index = p.n_exc > 0 ? p.d_exc_index : nullptr;
    a.exc = (const AdvExcCell<double> *)p.d_exc;
    a.status = p.d_status;
    a.spin_limit = p.wait_polls;
    return a;
}

}  // namespace

namespace {

int halves_win(const AdvPlanImpl &p) {
    // a half line's cells, its stencils' NT - 1 further taps, the margin
    // either side and one cell of alignment, rounded up to an even count
    return (int)((p.desc.n1 / 2 + p.npts + 2 * kDsHalfMargin + 1) & ~int64_t(1));
}

int halves_rl(const AdvPlanImpl &p) {
    // odd runs over a quarter line
    return (int)((p.desc.n1 / 4 + kDsRunsThreads - 1) / kDsRunsThreads) | 1;
}

}  // namespace

size_t adv_ds_halves_smem(const AdvPlanImpl &p) { return (size_t)halves_win(p) * sizeof(double); }

bool adv_ds_lineq_ok(const AdvPlanImpl &p) {
    const int64_t n1 = p.desc.n1;
    return adv_ds_rows_shape_ok(p) && p.desc.n2 == 1 &&
           (n1 == 16 || n1 == 32 || n1 == 64 || n1 == 128);
}

bool adv_ds_halves_ok(const AdvPlanImpl &p) {
    return adv_ds_rows_shape_ok(p) && p.desc.n2 == 1 && p.desc.n1 >= 8192 &&
           p.desc.n1 < (1 << 28) && p.lines < (1 << 30) && p.exc_dev <= kDsHalfMargin &&
           adv_ds_halves_smem(p) <= (size_t)227 * 1024 - 16;
}

int adv_ds_rows_fused_r(const AdvPlanImpl &p) {
    // about 2048 cells per CTA: two 4-cell groups per thread and step (10
    // steps per launch, x 1024 x 1, GCells/s for 512 / 2048 / 16384 lines:
    // 1024 cells 108 / 159 / 181, 2048 cells 107 / 169 / 197, 4096 cells
    // 98 / 154 / 208)
    return (int)std::min<int64_t>(std::max<int64_t>(1, 2048 / p.desc.n1), p.lines);
}

bool adv_ds_rows_fused_ok(const AdvPlanImpl &p, const void *src, const void *dst, int R) {
    // two copies of the CTA's lines in shared memory
    return adv_ds_rows_shape_ok(p) && p.desc.n2 == 1 && R >= 1 && ((uintptr_t)src % 16) == 0 &&
           ((uintptr_t)dst % 16) == 0 && 2 * adv_ds_rows_smem(p, R) <= (size_t)227 * 1024 - 16;
}

cudaError_t adv_ds_rows_fused_launch(AdvPlanImpl &p, const void *src, void *dst, int R, int k,
                                     cudaStream_t st) {
    const AdvDsRowsArgs a = rows_args(p, src, dst, R);
    const size_t smem = 2 * adv_ds_rows_smem(p, R);
    auto kern = p.npts == 6 ? adv_ds_rows_fused<6> : adv_ds_rows_fused<4>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<grid_x((p.lines + R - 1) / R), kDsRowsThreads, smem, st>>>(a, k);
    return cudaGetLastError();
}

cudaError_t adv_ds_rows_launch(AdvPlanImpl &p, const void *src, void *dst, int W, int R,
                               cudaStream_t st) {
    AdvDsRowsArgs a = rows_args(p, src, dst, R);
    const size_t smem = adv_ds_rows_smem(p, R);
    a.runs = std::max(1, W);
    if (p.desc.n2 > 1) {
        auto kern = p.npts == 6 ? adv_ds_slabs<6> : adv_ds_slabs<4>;
        cudaError_t e =
            cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        kern<<<grid_x((p.lines + R - 1) / R), kDsSlabThreads, smem, st>>>(a);
        return cudaGetLastError();
    }
    if (W == 5 && adv_ds_lineq_ok(p)) {
        // the lanes of a warp share each short line
        auto pick = [&](auto g_c) {
            constexpr int G = decltype(g_c)::value;
            return p.npts == 6 ? adv_ds_lineq<6, G> : adv_ds_lineq<4, G>;
        };
        const int64_t n1 = p.desc.n1;
        auto kern = n1 == 16   ? pick(std::integral_constant<int, 4>{})
                    : n1 == 32 ? pick(std::integral_constant<int, 8>{})
                    : n1 == 64 ? pick(std::integral_constant<int, 16>{})
                               : pick(std::integral_constant<int, 32>{});
        cudaError_t e =
            cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        kern<<<grid_x((p.lines + R - 1) / R), kDsRowsThreads, smem, st>>>(a);
        return cudaGetLastError();
    }
    if (W == 4 && p.desc.n2 == 1) {
        // runs of 4-cell groups: about one run per thread, an odd number of
        // groups per run (the lanes' 16-byte loads then use 4 of the 8 bank groups)
        const int64_t groups = (int64_t)R * (p.desc.n1 / 4);
        const int rq = (int)std::max<int64_t>(1, (groups + kDsQrunsThreads - 1) / kDsQrunsThreads) | 1;
        auto kern = p.npts == 6 ? adv_ds_qruns<6> : adv_ds_qruns<4>;
        cudaError_t e =
            cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        kern<<<grid_x((p.lines + R - 1) / R), kDsQrunsThreads, smem, st>>>(a, rq);
        return cudaGetLastError();
    }
    if (W == 6 && adv_ds_halves_ok(p)) {
        // half lines in 2-CTA clusters, runs of 4-cell groups
        const size_t hs = adv_ds_halves_smem(p);
        const int groups = (int)(p.desc.n1 / 8);
        const int rq = std::max(1, (groups + kDsQrunsThreads - 1) / kDsQrunsThreads) | 1;
        auto kern = p.npts == 6 ? adv_ds_halves_q<6> : adv_ds_halves_q<4>;
        cudaError_t e =
            cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)hs);
        if (e != cudaSuccess) return e;
        kern<<<grid_x(2 * p.lines), kDsQrunsThreads, hs, st>>>(a, rq, halves_win(p));
        return cudaGetLastError();
    }
    if (W == 3 && adv_ds_halves_ok(p)) {
        // half lines, one per CTA of a 2-CTA cluster
        const size_t hs = adv_ds_halves_smem(p);
        auto kern = p.npts == 6 ? adv_ds_halves<6> : adv_ds_halves<4>;
        cudaError_t e =
            cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)hs);
        if (e != cudaSuccess) return e;
        kern<<<grid_x(2 * p.lines), kDsRunsThreads, hs, st>>>(a, halves_rl(p), halves_win(p));
        return cudaGetLastError();
    }
    if (W == 2 && adv_ds_runs_ok(p, R)) {
        // long lines: runs of an odd length along two sections per thread
        const int runs_pp = R == 1 ? kDsRunsThreads : kDsRunsThreads / (R / 2);
        const int64_t seclen = R == 1 ? p.desc.n1 / 2 : p.desc.n1;
        const int rl = (int)((seclen + runs_pp - 1) / runs_pp) | 1;
        auto kern = p.npts == 6 ? adv_ds_runs<6> : adv_ds_runs<4>;
        cudaError_t e =
            cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        kern<<<grid_x((p.lines + R - 1) / R), kDsRunsThreads, smem, st>>>(a, rl);
        return cudaGetLastError();
    }
    auto kern = p.npts == 6 ? adv_ds_rows<6> : adv_ds_rows<4>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<grid_x((p.lines + R - 1) / R), kDsRowsThreads, smem, st>>>(a);
    return cudaGetLastError();
}

}  // namespace bkma
