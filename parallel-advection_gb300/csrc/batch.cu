// Batched uneven advection: many fields of different (n0, n1, n2), degree and
// line velocities advanced by ONE persistent kernel launch per time step.
//
// Each field gets its own per-line tables (the same host precompute as a
// single-field plan, so departure cells are bit-identical to the reference)
// and a tile shape from a cost model: column tiles of W = 32/16/8/4 columns
// when n2 allows, otherwise R whole slabs, each kept under a shared-memory cap
// so several CTAs stay resident per SM. All tiles of all fields form one
// work list; persistent CTAs pull tiles from a global counter (atomicAdd, no
// waiting on other CTAs) and run the same staged-tile device code as the
// single-field kernel. The counter reset and the launch are captured once in
// a CUDA graph; a step is one graph launch. bkma_adv_batch_autotune times the
// candidate caps and CTA sizes on the live fields (this stands in for the
// reference's WorkItemDispatch / adjust_sizes_mem_limit sizing,
// src/core/bkma_tools.hpp:74-107).
#include <algorithm>
#include <cstring>
#include <memory>
#include <vector>

#include "adv_device.cuh"
#include "adv_plan.cuh"
#include "common.cuh"

namespace bkma {

template <typename T>
struct BatchFieldDev {
    AdvStagedArgs<T> args;
    int npts;
    int64_t tile0;  // first tile of this field in the work list
};

template <typename T>
__global__ void __launch_bounds__(256) adv_batch_kernel(const BatchFieldDev<T> *__restrict__ fields,
                                                        int nfields, int64_t ntiles,
                                                        unsigned long long *counter) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ long long t_sh;
    T *sm = reinterpret_cast<T *>(smem_raw);
    for (;;) {
        if (threadIdx.x == 0) t_sh = (long long)atomicAdd(counter, 1ull);
        __syncthreads();
        const long long t = t_sh;
        if (t >= ntiles) break;
        int lo = 0, hi = nfields - 1;  // last field with tile0 <= t
        while (lo < hi) {
            const int mid = (lo + hi + 1) / 2;
            if (fields[mid].tile0 <= t) lo = mid;
            else hi = mid - 1;
        }
        // Copy the field's argument block into registers: read through a
        // pointer to global memory, every store to the field would force
        // the compiler to reload it.
        const AdvStagedArgs<T> args = fields[lo].args;
        const int npts = fields[lo].npts;
        TileCoord tc = tile_of(t - fields[lo].tile0, args.lines, args.n2, args.R, args.W,
                               args.ncb);
        if (args.line_list) tc.line0 = args.line_list[tc.line0];
        if (npts == 6)
            staged_tile<T, 6>(args, tc, sm);
        else
            staged_tile<T, 4>(args, tc, sm);
        __syncthreads();  // shared memory is restaged by the next tile
    }
}

namespace {

struct BatchImpl {
    int dtype = BKMA_F32;
    int esize = 4;
    std::vector<bkma_adv_plan *> plans;
    std::vector<void *> data;
    std::vector<int> W, R;
    void *d_fields = nullptr;  // staged work list entries
    int nstaged = 0;
    unsigned long long *d_counter = nullptr;
    // streamed fields: group 0 the 4- and 6-tap fields (one launch), group 2
    // the 10-tap ones (group 1 unused)
    StreamField *d_stream[3] = {nullptr, nullptr, nullptr};
    int nstream[3] = {0, 0, 0};
    int64_t items[3] = {0, 0, 0};  // CTAs of each streamed launch
    bool stream = true;  // stream the fields that allow it (FP32, small shifts)
    int segs_mode = 0;   // row segments of streamed fields (adv_stream_segs mode)
    int nfields = 0;
    int64_t ntiles = 0, cells = 0;
    size_t smem = 0;
    int threads = 256, grid = 0, launches = 0;
    size_t cap = 48 * 1024;
    cudaGraphExec_t exec = nullptr;
    cudaStream_t cs = nullptr;
    cudaStream_t par[2] = {nullptr, nullptr};  // capture branches of the streamed launches
    cudaEvent_t fork = nullptr, join[2] = {nullptr, nullptr};

    void free_lists() {
        cudaFree(d_fields);
        d_fields = nullptr;
        for (auto &d : d_stream) {
            cudaFree(d);
            d = nullptr;
        }
    }
    ~BatchImpl() {
        if (exec) cudaGraphExecDestroy(exec);
        if (cs) cudaStreamDestroy(cs);
        for (auto &q : par)
            if (q) cudaStreamDestroy(q);
        if (fork) cudaEventDestroy(fork);
        for (auto &e : join)
            if (e) cudaEventDestroy(e);
        free_lists();
        cudaFree(d_counter);
        for (auto *p : plans) bkma_adv_plan_destroy(p);
    }
};

// Streamed launch of a field: 4 and 6 taps share one (adv_stream_f32_46),
// 10 taps have their own.
int stream_group(int npts) { return npts == 10 ? 2 : 0; }

// Streamed when every line allows it and rows have at least 8 columns: with
// fewer, a warp's 32 lanes spread over many lines and rows stop coalescing,
// and whole-row staged tiles do better.
bool streams(const AdvPlanImpl &p) { return p.stream_ok && p.desc.n2 >= 8; }

// Tile of one field under a shared-memory cap.
void choose_tile(const AdvPlanImpl &p, size_t cap, int &W, int &R) {
    const int64_t n2 = p.desc.n2;
    W = (int)n2;
    R = 1;
    // Up to 32 columns: whole rows (no ragged column tile), when they fit.
    if (n2 >= 8 && (n2 > 32 || p.smem_bytes((int)n2, 1) > cap)) {
        for (int w : {32, 16, 8, 4}) {
            if (w <= n2 && p.smem_bytes(w, 1) <= cap) {
                W = w;
                return;
            }
        }
        W = 4;
        return;
    }
    const size_t per = p.smem_bytes((int)n2, 1);
    R = (int)std::max<size_t>(1, cap / std::max<size_t>(per, 1));
    R = (int)std::min<int64_t>(R, p.lines);
}

template <typename T>
void staged_entry(std::vector<BatchFieldDev<T>> &f, BatchImpl &b, const AdvPlanImpl &p,
                  void *data, int W, int R, const int32_t *list, int64_t nlist) {
    BatchFieldDev<T> e{};
    AdvStagedArgs<T> &a = e.args;
    a.src = (const T *)data;
    a.dst = (T *)data;
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
    e.npts = p.npts;
    e.tile0 = b.ntiles;
    b.ntiles += ((a.lines + a.R - 1) / a.R) * a.ncb;
    b.smem = std::max(b.smem, p.smem_bytes(W, a.R));
    f.push_back(e);
}

template <typename T>
bkma_status build_batch(BatchImpl &b, cudaStream_t st) {
    std::vector<BatchFieldDev<T>> f;
    std::vector<StreamField> sf[3];
    b.free_lists();
    b.ntiles = 0;
    b.smem = 0;
    for (int g = 0; g < 3; ++g) b.items[g] = 0;
    int64_t stream_groups = 0;  // 32-column groups of all streamed fields
    for (int i = 0; i < b.nfields; ++i) {
        const AdvPlanImpl &p = plan_impl(b.plans[(size_t)i]);
        if (sizeof(T) == 4 && b.stream && streams(p)) stream_groups += adv_stream_groups(p);
    }
    for (int i = 0; i < b.nfields; ++i) {
        AdvPlanImpl &p = plan_impl(b.plans[(size_t)i]);
        void *data = b.data[(size_t)i];
        int W, R;
        choose_tile(p, b.cap, W, R);
        if (sizeof(T) == 4 && b.stream && streams(p)) {
            // streamed; its exception lines (if any) stay on the staged list
            const int g = stream_group(p.npts);
            const int segs = adv_stream_segs(p.desc.n1, stream_groups, b.segs_mode);
            StreamField s = adv_stream_field(p, data, data, segs);
            s.cta0 = adv_stream_ctas(p, segs);  // the field's CTA count until the ordering below
            sf[g].push_back(s);
            b.W[(size_t)i] = 0;
            b.R[(size_t)i] = segs;
            if (p.n_exc > 0) staged_entry<T>(f, b, p, data, W, 1, p.d_exc_lines, p.n_exc);
            continue;
        }
        b.W[(size_t)i] = W;
        b.R[(size_t)i] = R;
        staged_entry<T>(f, b, p, data, W, R, nullptr, 0);
    }
    // Longest CTAs first: a streamed CTA's time grows with the rows each warp
    // walks (n1 / segs), and CTAs start roughly in index order, so the last
    // wave then holds the short ones (64-field batch 752.7 -> 755.8 GCells/s).
    for (int g = 0; g < 3; ++g) {
        std::stable_sort(sf[g].begin(), sf[g].end(), [](const StreamField &x, const StreamField &y) {
            return (x.n1 + x.segs - 1) / x.segs > (y.n1 + y.segs - 1) / y.segs;
        });
        for (auto &q : sf[g]) {
            const int64_t n = q.cta0;
            q.cta0 = b.items[g];
            b.items[g] += n;
        }
    }
    b.nstaged = (int)f.size();
    if (!f.empty()) {
        BKMA_CUDA_TRY(cudaMalloc(&b.d_fields, sizeof(BatchFieldDev<T>) * f.size()));
        BKMA_CUDA_TRY(cudaMemcpy(b.d_fields, f.data(), sizeof(BatchFieldDev<T>) * f.size(),
                                 cudaMemcpyHostToDevice));
    }
    for (int g = 0; g < 3; ++g) {
        b.nstream[g] = (int)sf[g].size();
        if (sf[g].empty()) continue;
        BKMA_CUDA_TRY(cudaMalloc(&b.d_stream[g], sizeof(StreamField) * sf[g].size()));
        BKMA_CUDA_TRY(cudaMemcpy(b.d_stream[g], sf[g].data(), sizeof(StreamField) * sf[g].size(),
                                 cudaMemcpyHostToDevice));
    }
    auto kern = adv_batch_kernel<T>;
    b.grid = 0;
    if (b.ntiles > 0) {
        BKMA_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)b.smem));
        int per_sm = 0, dev = 0, sms = 0;
        BKMA_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, b.threads, b.smem));
        cudaGetDevice(&dev);
        BKMA_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        if (per_sm < 1) return fail(BKMA_ERR_UNSUPPORTED, "batched tile does not fit an SM");
        b.grid = (int)std::min<int64_t>((int64_t)per_sm * sms, b.ntiles);
    }
    // capture: counter reset + persistent staged launch, then the streamed
    // launches (disjoint lines, so the order does not matter)
    if (b.exec) {
        cudaGraphExecDestroy(b.exec);
        b.exec = nullptr;
    }
    if (!b.cs) BKMA_CUDA_TRY(cudaStreamCreateWithFlags(&b.cs, cudaStreamNonBlocking));
    for (auto &q : b.par)
        if (!q) BKMA_CUDA_TRY(cudaStreamCreateWithFlags(&q, cudaStreamNonBlocking));
    if (!b.fork) BKMA_CUDA_TRY(cudaEventCreateWithFlags(&b.fork, cudaEventDisableTiming));
    for (auto &e : b.join)
        if (!e) BKMA_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    (void)st;
    cudaGraph_t g = nullptr;
    b.launches = 0;
    // the launches touch disjoint lines: capture them as parallel branches,
    // so the last wave of one overlaps the others
    BKMA_CUDA_TRY(cudaStreamBeginCapture(b.cs, cudaStreamCaptureModeThreadLocal));
    cudaEventRecord(b.fork, b.cs);
    for (auto &q : b.par) cudaStreamWaitEvent(q, b.fork, 0);
    cudaStream_t branch[3] = {b.cs, b.par[0], b.par[1]};
    int nb = 0;
    if (b.ntiles > 0) {
        cudaMemsetAsync(b.d_counter, 0, sizeof(unsigned long long), branch[nb]);
        kern<<<b.grid, b.threads, b.smem, branch[nb]>>>((const BatchFieldDev<T> *)b.d_fields,
                                                       b.nstaged, b.ntiles, b.d_counter);
        ++b.launches;
        ++nb;
    }
    for (int k = 0; k < 3; ++k) {
        if (b.items[k] == 0) continue;
        if (k == 0)
            adv_stream_launch_fields_46(b.d_stream[0], b.nstream[0], b.items[0], branch[nb % 3]);
        else
            adv_stream_launch_fields(10, b.d_stream[k], b.nstream[k], b.items[k], branch[nb % 3]);
        ++b.launches;
        ++nb;
    }
    for (int k = 0; k < 2; ++k) {
        cudaEventRecord(b.join[k], b.par[k]);
        cudaStreamWaitEvent(b.cs, b.join[k], 0);
    }
    cudaError_t e = cudaStreamEndCapture(b.cs, &g);
    if (e != cudaSuccess) return cuda_fail(e, "batch graph capture");
    e = cudaGraphInstantiate(&b.exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(e, "batch graph instantiate");
    return BKMA_OK;
}

bkma_status rebuild(BatchImpl &b, cudaStream_t st) {
    return b.dtype == BKMA_F32 ? build_batch<float>(b, st) : build_batch<double>(b, st);
}

}  // namespace
}  // namespace bkma

struct bkma_adv_batch {
    bkma::BatchImpl impl;
};

using namespace bkma;

extern "C" {

bkma_status bkma_adv_batch_create(const bkma_adv_field *fields, int32_t nfields, int32_t dtype,
                                  bkma_adv_batch **batch) try {
    bkma::NvtxRange nvtx_range("bkma_adv_batch_create");
    BKMA_CHECK_ARG(fields && batch && nfields > 0, "bkma_adv_batch_create: bad arguments");
    BKMA_CHECK_ARG(dtype == BKMA_F32 || dtype == BKMA_F64, "dtype must be BKMA_F32 or BKMA_F64");
    *batch = nullptr;
    // owned here until complete: an early return or an exception frees it
    std::unique_ptr<bkma_adv_batch> bb(new bkma_adv_batch);
    BatchImpl &b = bb->impl;
    b.dtype = dtype;
    b.esize = dtype == BKMA_F32 ? 4 : 8;
    b.nfields = nfields;
    b.W.assign((size_t)nfields, 0);
    b.R.assign((size_t)nfields, 1);
    b.plans.reserve((size_t)nfields);  // push_back below cannot throw: no plan leaks
    b.data.reserve((size_t)nfields);
    for (int i = 0; i < nfields; ++i) {
        const bkma_adv_field &f = fields[i];
        if (!f.data) {
            return fail(BKMA_ERR_INVALID_ARG, "field " + std::to_string(i) + ": null data");
        }
        if (f.degree != 3 && f.degree != 5) {
            return fail(BKMA_ERR_INVALID_ARG, "field " + std::to_string(i) + ": degree must be 3 or 5");
        }
        bkma_adv_desc d{};
        d.n0 = f.n0;
        d.n1 = f.n1;
        d.n2 = f.n2;
        d.dtype = dtype;
        d.degree = f.degree;
        d.weights = f.weights;
        d.impl = BKMA_ADV_STAGED;
        d.inplace = 1;
        d.dt = f.dt;
        d.minX = f.minX;
        d.maxX = f.maxX;
        d.minVx = f.minVx;
        d.maxVx = f.maxVx;
        d.velocity = f.velocity;
        bkma_adv_plan *p = nullptr;
        bkma_status s = bkma_adv_plan_create(&d, &p);
        if (s != BKMA_OK) {
            const std::string m = bkma_last_error();
            return fail(s, "field " + std::to_string(i) + ": " + m);
        }
        b.plans.push_back(p);
        b.data.push_back(f.data);
        b.cells += f.n0 * f.n1 * f.n2;
    }
    cudaError_t e = cudaMalloc(&b.d_counter, sizeof(unsigned long long));
    if (e != cudaSuccess) return cuda_fail(e, "batch counter");
    bkma_status s = rebuild(b, nullptr);
    if (s != BKMA_OK) return s;
    *batch = bb.release();
    return BKMA_OK;
} BKMA_ABI_CATCH("bkma_adv_batch_create")

bkma_status bkma_adv_batch_step(bkma_adv_batch *batch, int32_t nsteps, void *stream) try {
    bkma::NvtxRange nvtx_range("bkma_adv_batch_step");
    BKMA_CHECK_ARG(batch && nsteps >= 0, "bkma_adv_batch_step: bad arguments");
    BatchImpl &b = batch->impl;
    for (int i = 0; i < nsteps; ++i) BKMA_CUDA_TRY(cudaGraphLaunch(b.exec, (cudaStream_t)stream));
    return BKMA_OK;
} BKMA_ABI_CATCH("bkma_adv_batch_step")

bkma_status bkma_adv_batch_autotune(bkma_adv_batch *batch, void *stream) try {
    bkma::NvtxRange nvtx_range("bkma_adv_batch_autotune");
    BKMA_CHECK_ARG(batch, "null argument");
    BatchImpl &b = batch->impl;
    cudaStream_t st = (cudaStream_t)stream;
    cudaEvent_t e0, e1;
    BKMA_CUDA_TRY(cudaEventCreate(&e0));
    BKMA_CUDA_TRY(cudaEventCreate(&e1));
    float best = 1e30f;
    size_t best_cap = b.cap;
    int best_thr = b.threads;
    bool best_stream = b.stream;
    int best_segs = b.segs_mode;
    // candidates: streamed fields (row segments: fill the GPU, or up to 8)
    // or none x shared-memory cap x CTA size of the staged kernel
    for (int sm : {0, 8, -1})
    for (size_t cap : {24 * 1024, 32 * 1024, 48 * 1024, 64 * 1024, 96 * 1024}) {
        for (int thr : {128, 256}) {
            b.stream = sm >= 0;
            b.segs_mode = sm >= 0 ? sm : 0;
            b.cap = cap;
            b.threads = thr;
            if (rebuild(b, st) != BKMA_OK) continue;
            // nothing left for the staged kernel: cap and CTA size are moot
            if (b.ntiles == 0 && (cap != 24 * 1024 || thr != 128)) continue;
            cudaGraphLaunch(b.exec, st);  // warm-up
            cudaEventRecord(e0, st);
            for (int r = 0; r < 2; ++r) cudaGraphLaunch(b.exec, st);
            cudaEventRecord(e1, st);
            BKMA_CUDA_TRY(cudaEventSynchronize(e1));
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            if (ms < best) {
                best = ms;
                best_cap = cap;
                best_thr = thr;
                best_stream = b.stream;
                best_segs = b.segs_mode;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b.cap = best_cap;
    b.threads = best_thr;
    b.stream = best_stream;
    b.segs_mode = best_segs;
    return rebuild(b, st);
} BKMA_ABI_CATCH("bkma_adv_batch_autotune")

bkma_status bkma_adv_batch_info(const bkma_adv_batch *batch, int64_t *cells, int32_t *launches_per_step) try {
    BKMA_CHECK_ARG(batch, "null argument");
    if (cells) *cells = batch->impl.cells;
    if (launches_per_step) *launches_per_step = batch->impl.launches;
    return BKMA_OK;
} BKMA_ABI_CATCH("bkma_adv_batch_info")

bkma_status bkma_adv_batch_tiles(const bkma_adv_batch *batch, int32_t *W, int32_t *R, int64_t *tiles,
                                 int32_t *threads, int64_t *smem_bytes) try {
    BKMA_CHECK_ARG(batch, "null argument");
    const BatchImpl &b = batch->impl;
    for (int i = 0; i < b.nfields; ++i) {
        if (W) W[i] = b.W[(size_t)i];
        if (R) R[i] = b.R[(size_t)i];
    }
    if (tiles) *tiles = b.ntiles;
    if (threads) *threads = b.threads;
    if (smem_bytes) *smem_bytes = (int64_t)b.smem;
    return BKMA_OK;
} BKMA_ABI_CATCH("bkma_adv_batch_tiles")

bkma_status bkma_adv_batch_destroy(bkma_adv_batch *batch) try {
    delete batch;
    return BKMA_OK;
} BKMA_ABI_CATCH("bkma_adv_batch_destroy")

}  // extern "C"
