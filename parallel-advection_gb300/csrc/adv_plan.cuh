// Host-side advection plan (shared by adv.cu and adv_util.cu).
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "adv.cuh"
#include "common.cuh"

namespace bkma {

struct AdvPlanImpl {
    bkma_adv_desc desc{};
    AdvPhys phys{};
    int64_t lines = 0;
    int npts = 6;
    int esize = 4;
    // host tables
    std::vector<int32_t> base;       // per line, tap-0 offset mod n1
    std::vector<double> shift;       // per line, d - 2 at i1 = 0
    std::vector<double> vx;          // per line velocity
    std::vector<double> w64;         // per line weights
    std::vector<int32_t> exc_index;  // per line, -1 or exception slot
    int64_t n_exc = 0;
    // largest distance (cells) of an exception cell's tap offset from its
    // line's offset at i1 = 0
    int exc_dev = 0;
    // device tables
    int32_t *d_base = nullptr;
    void *d_w = nullptr;  // T weights
    float2 *d_w2 = nullptr;  // FP64 plans: each weight split into two FP32 parts (a, b)
    int32_t *d_exc_index = nullptr;
    void *d_exc = nullptr;
    double *d_vx = nullptr;
    int32_t *d_exc_lines = nullptr;  // [n_exc] the exception lines, ascending
    // every non-exception line can stream (FP32 tables, see stream_line_ok)
    bool stream_ok = false;
    // FP64 plans: every non-exception line can stream in FP32-pair arithmetic
    // (adv_stream_ds.cu: |d| <= 32, and every 64-column group walks up, d >
    // -(npts + 2) on all its lines, or down, d <= 2), with ds_sr seam rows per
    // column pair (max(d + npts - 1, 0) + max(-d, 0), the largest over lines)
    bool ds_stream_ok = false;
    int ds_sr = 0;
    // launch shape: path 0 = cp.async staging (any shape), 1 = TMA staging,
    // 2 = streamed columns (+ staged exception lines), 3 = contiguous lines
    // (n2 = 1, R lines per CTA), 4 = FP64 in FP32-pair arithmetic (TMA tiles),
    // 5 = the same on contiguous lines, 6 = the same streamed (+ staged
    // exception lines)
    int W = 16, R = 1, threads = 256, path = 0;
    bool autotuned = false;
    int fuse = 1;  // time steps per launch (adv_fused.cu when > 1)
    int fuse_x2 = 0;  // fused on-chip state: 0 FP32, 1 FP32 hi + lo pair
    struct TmapCache {
        const void *ptr;
        int W;
        CUtensorMap map;
    };
    std::vector<TmapCache> tmaps;  // TMA descriptors of recently used fields
    int *d_status = nullptr;       // device status word of the bounded waits
    uint32_t wait_polls = kWaitPolls;  // polls of a bounded device wait before it gives up
    // host-run buffer, and bkma_adv_run_host's pipeline: sub-plans over slab
    // chunks (lines are independent) on four streams, so the copies of one
    // chunk overlap the time steps of another
    void *d_host_buf = nullptr;
    size_t host_buf_bytes = 0;
    std::vector<bkma_adv_plan *> chunks;
    std::vector<int64_t> chunk_l0;
    // pipe[0]: copies in (one after another), pipe[1..2]: steps of alternate
    // chunks, pipe[3]: copies out; chunk_ev[2c] = chunk c copied in,
    // chunk_ev[2c+1] = chunk c stepped
    cudaStream_t pipe[4] = {nullptr, nullptr, nullptr, nullptr};
    cudaEvent_t pipe_ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    std::vector<cudaEvent_t> chunk_ev;
    double *d_partials = nullptr;
    int device = 0;

    ~AdvPlanImpl() {
        for (auto *c : chunks) bkma_adv_plan_destroy(c);
        for (auto &q : pipe)
            if (q) cudaStreamDestroy(q);
        for (auto &e : pipe_ev)
            if (e) cudaEventDestroy(e);
        for (auto &e : chunk_ev)
            if (e) cudaEventDestroy(e);
        cudaFree(d_base);
        cudaFree(d_w);
        cudaFree(d_w2);
        cudaFree(d_exc_index);
        cudaFree(d_exc);
        cudaFree(d_vx);
        cudaFree(d_exc_lines);
        cudaFree(d_host_buf);
        cudaFree(d_partials);
        cudaFree(d_status);
    }

    int halo() const { return desc.impl == BKMA_ADV_PLAIN ? 0 : npts - 1; }
    int64_t ncb(int w) const { return (desc.n2 + w - 1) / w; }
    // Shared memory of an R-slab tile of w columns: the widest row stride of
    // the full tiles and of the ragged last column tile, in either staged
    // layout (chunk-congruent rows, or rows padded to 16 bytes).
    size_t smem_bytes(int w, int r) const {
        const int q = 16 / esize;
        auto widest = [&](int wc) {
            if (wc < q) return wc;  // narrower than a chunk (or whole rows of n2 < q): unpadded
            const int ws = staged_row_stride(desc.n2, wc, esize);
            // FP32 rows off the 16-byte grid: padded to 16 bytes
            return esize == 4 ? std::max(ws, (wc + q - 1) / q * q) : ws;
        };
        const int wc = (int)std::min<int64_t>(w, desc.n2);
        int ws = widest(wc);
        const int last = (int)(desc.n2 % wc);
        if (last) ws = std::max(ws, widest(last));
        return (size_t)r * (size_t)slab_stride(desc.n1, halo(), ws, esize) * (size_t)esize;
    }
    int64_t tiles(int w, int r) const { return ((lines + r - 1) / r) * ncb(w); }
    // Tile width of the staged pass over the exception lines of a streamed
    // plan: the widest of 16, 8, 4, 2, 1 columns that fits shared memory
    // (0 if none does).
    int exc_tile_w(size_t max_smem) const {
        for (int w : {16, 8, 4, 2, 1})
            if (w <= desc.n2 && smem_bytes(w, 1) <= max_smem) return w;
        return 0;
    }
};

// Streamed form (adv_stream.cu): the kernel over all streamable lines of a
// plan (exception lines are skipped; the caller runs them staged). `segs`:
// row segments per 32-column group, 0 = chosen from the field's size (see
// adv_stream_segs).
cudaError_t adv_stream_launch(AdvPlanImpl &p, const void *src, void *dst, int segs,
                              cudaStream_t st);
// Row segments for a field of n1 rows and `groups` 32-column groups: mode 0
// splits until the GPU is filled a few times over, mode k >= 1 = up to k
// (a power of two <= 8); segments keep at least 64 rows.
int adv_stream_segs(int64_t n1, int64_t groups, int mode);
int64_t adv_stream_groups(const AdvPlanImpl &p);
int64_t adv_stream_ctas(const AdvPlanImpl &p, int segs);
// Device descriptor of a plan's field for the streamed kernel.
StreamField adv_stream_field(const AdvPlanImpl &p, const void *src, void *dst, int segs);
// Contiguous-line form (adv_rows.cu, FP32, n2 = 1, n1 % 4 == 0, n1 >= 16):
// R whole lines per CTA.
bool adv_rows_shape_ok(const AdvPlanImpl &p);
bool adv_rows_eligible(const AdvPlanImpl &p, const void *src, const void *dst, int R);
size_t adv_rows_smem(const AdvPlanImpl &p, int R);
int adv_rows_default_r(const AdvPlanImpl &p);
cudaError_t adv_rows_launch(const AdvPlanImpl &p, const void *src, void *dst, int R,
                            cudaStream_t st);
size_t adv_stream_smem();  // static shared memory per CTA of the streamed kernel
// All fields of `d_fields` (device array, ascending cta0) have npts taps;
// nctas = the sum of their CTA counts.
// Fields of 4 and of 6 taps mixed, in one launch.
cudaError_t adv_stream_launch_fields_46(const StreamField *d_fields, int nfields, int64_t nctas,
                                        cudaStream_t st);
cudaError_t adv_stream_launch_fields(int npts, const StreamField *d_fields, int nfields,
                                     int64_t nctas, cudaStream_t st);

// Multi-step fused form (adv_fused.cu): strip width for a plan (0 if the
// plan's lines are too long), and one launch of k fused steps src -> dst.
int adv_fused_tile_w(const AdvPlanImpl &p, size_t max_smem);
// FP32 plans: whether the fast fused strips (two shared buffers, 4 or 8
// columns) hold the plan's lines.
bool adv_fused_f32_fast(const AdvPlanImpl &p, size_t max_smem);
// Shared memory of the hi + lo fused kernel (four n1 x 4 FP32 buffers).
size_t adv_fused_x2_smem(const AdvPlanImpl &p);
cudaError_t adv_fused_launch(const AdvPlanImpl &p, const void *src, void *dst, int W, int k,
                             cudaStream_t st);

// FP64 storage, FP32-pair arithmetic (adv_ds.cu): TMA tiles of W = 4 or 8
// columns, adv_ds_threads(W) threads per CTA.
bool adv_ds_shape_ok(const AdvPlanImpl &p, int W);
bool adv_ds_eligible(const AdvPlanImpl &p, const void *src, int W);
size_t adv_ds_smem(const AdvPlanImpl &p, int W);
int adv_ds_threads(int W);
cudaError_t adv_ds_launch(AdvPlanImpl &p, const void *src, void *dst, int W, cudaStream_t st);
// The same arithmetic on contiguous lines (FP64, n2 = 1, n1 % 4 == 0, n1 >=
// 16, degree 3 or 5; path 5): R whole lines per CTA; W = 1: 4 cells per
// thread, W = 2: runs along two line sections per thread (n1 >= 512, R = 1 or
// an even R <= 16: adv_ds_runs_ok), W = 3: half lines (adv_ds_halves_ok),
// W = 4: runs of 4-cell groups, W = 5: lines of 16-128 cells shared by a
// warp's lanes (adv_ds_lineq_ok), W = 6: half lines in runs of 4-cell groups
// (adv_ds_halves_ok). All give the same bits; with an even n2 > 1,
// whole slabs with W runs of rows per column pair.
bool adv_ds_rows_shape_ok(const AdvPlanImpl &p);
bool adv_ds_rows_eligible(const AdvPlanImpl &p, const void *src, const void *dst, int R);
bool adv_ds_runs_ok(const AdvPlanImpl &p, int R);
size_t adv_ds_rows_smem(const AdvPlanImpl &p, int R);
void adv_ds_rows_default(const AdvPlanImpl &p, int *W, int *R);
cudaError_t adv_ds_rows_launch(AdvPlanImpl &p, const void *src, void *dst, int W, int R,
                               cudaStream_t st);
// k fused steps per launch on contiguous lines (n2 = 1) in the same
// arithmetic (the bits of k steps of adv_ds_rows_launch): R lines per CTA,
// two copies of them in shared memory.
// W = 3 on path 5: lines of 8192 cells and more split between the two CTAs
// of a cluster (adv_ds_halves), the same bits.
bool adv_ds_halves_ok(const AdvPlanImpl &p);
// W = 5 on path 5: lines of 16, 32, 64 or 128 cells shared by the lanes of a
// warp (adv_ds_lineq), the same bits.
bool adv_ds_lineq_ok(const AdvPlanImpl &p);
size_t adv_ds_halves_smem(const AdvPlanImpl &p);
int adv_ds_rows_fused_r(const AdvPlanImpl &p);
bool adv_ds_rows_fused_ok(const AdvPlanImpl &p, const void *src, const void *dst, int R);
cudaError_t adv_ds_rows_fused_launch(AdvPlanImpl &p, const void *src, void *dst, int R, int k,
                                     cudaStream_t st);
// The same arithmetic streamed down column pairs (adv_stream_ds.cu, path 6;
// FP64, degree 3 or 5, even n2, ds_stream_ok); segs_mode as the FP32
// streamed form's row-segment mode; exception lines are left to the staged pass.
bool adv_stream_ds_shape_ok(const AdvPlanImpl &p);
bool adv_stream_ds_eligible(const AdvPlanImpl &p, const void *src, const void *dst);
size_t adv_stream_ds_smem(const AdvPlanImpl &p);
int adv_stream_ds_segs(const AdvPlanImpl &p, int mode);
cudaError_t adv_stream_ds_launch(AdvPlanImpl &p, const void *src, void *dst, int segs_mode,
                                 cudaStream_t st);

bool adv_tma_eligible(const AdvPlanImpl &p, const void *src, int W);
size_t adv_tma_smem(const AdvPlanImpl &p, int W);
cudaError_t adv_tma_launch(AdvPlanImpl &p, const void *src, void *dst, int W, int threads,
                           cudaStream_t st);

}  // namespace bkma

struct bkma_adv_plan {
    bkma::AdvPlanImpl impl;
};

namespace bkma {
inline AdvPlanImpl &plan_impl(bkma_adv_plan *p) { return p->impl; }
inline const AdvPlanImpl &plan_impl(const bkma_adv_plan *p) { return p->impl; }
}  // namespace bkma
