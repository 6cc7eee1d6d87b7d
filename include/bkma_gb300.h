/*
 * bkma_gb300 — C ABI of the GB300-native BKMA hot paths.
 *
 * One shared library (libbkma_gb300.so) with C linkage, plain pointers and
 * sizes. Device pointers are CUDA device addresses on the current device;
 * `stream` is a cudaStream_t passed as void* (NULL = legacy default stream).
 * No call throws; every call returns a bkma_status and leaves a message for
 * bkma_last_error() (thread-local) on failure.
 *
 * Reference interfaces replaced (Maison-de-la-Simulation/parallel-advection):
 *   bkma_run<Solver, Impl>(queue, span3d data, solver, optim, global_scratch)
 *       src/core/bkma_run.hpp:10-62                -> bkma_adv_step / bkma_conv_run
 *   impl_selector<Solver>(name)   src/tools/impl_selector.hpp:31-49
 *                                                  -> bkma_impl_from_name
 *   AdvectionSolver(ADVParams)    src/solvers/AdvectionSolver.hpp:13-100
 *                                                  -> bkma_adv_plan_create
 *   ConvSolver{weight, bias, k, c_in, length}      src/solvers/ConvSolver.hpp:7-45
 *                                                  -> bkma_conv_plan_create
 *   create_optim_params / WorkItemDispatch / WorkGroupDispatch
 *       src/tools/init.hpp:76-102, src/core/bkma_tools.hpp:25-107
 *                                                  -> plan-time tile choice + bkma_adv_plan_autotune
 *   fill_buffer_adv / validate_result_adv
 *       src/tools/init.hpp:31-46, src/tools/validation.hpp:9-80
 *                                                  -> bkma_adv_fill / bkma_adv_error_norms
 */
#ifndef BKMA_GB300_H
#define BKMA_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BKMA_ABI_VERSION 1

typedef enum bkma_status {
    BKMA_OK = 0,
    BKMA_ERR_INVALID_ARG = 1, /* reference: std::invalid_argument (bkma_tools.hpp:38-51, bkma_run.hpp:53) */
    BKMA_ERR_UNSUPPORTED = 2, /* reference: std::runtime_error (impl_selector.hpp:44-47) */
    BKMA_ERR_CUDA = 3,        /* a CUDA runtime error (message holds cudaGetErrorString) */
    BKMA_ERR_TIMEOUT = 4,     /* a bounded device-side wait gave up */
    BKMA_ERR_NO_DEVICE = 5,   /* no CUDA device visible */
    BKMA_ERR_HOST = 6         /* a host-side failure (out of host memory): no C++ exception
                                 ever leaves an entry point */
} bkma_status;

typedef enum bkma_dtype { BKMA_F32 = 0, BKMA_F64 = 1, BKMA_BF16 = 2 } bkma_dtype;

/* Strategy names accepted by bkma_impl_from_name (case-insensitive):
 * "ndrange", "adaptivewg" (the reference's two live strategies), "basicrange"
 * (out of place), "plain" (per-cell FP64 reference math), "staged" and
 * "gb300"/"cuda" (the per-line staged kernel). */
/* AUTO and STAGED run the fastest kernel for the shape. For FP64 fields that
 * is, wherever the shape allows it (degree 3 or 5; column pairs of an even
 * n2 with n1 >= 128, staged in shared memory or, for strips too tall or rows
 * 1 MB or more apart, streamed; whole slabs of lines shorter than 128 rows
 * with an even n2; or n2 = 1 with n1 % 4 == 0; a 16-byte aligned field), a
 * kernel that
 * keeps FP64 in HBM but sums the stencil in FP32-pair arithmetic (GB300's
 * FP64 rate would otherwise bound the step near 100 GCells/s): it agrees with
 * FP64 arithmetic to about 2e-13 max|f| per step. bkma_adv_plan_set_tile
 * with path 0 selects the FP64-arithmetic staged kernel. */
typedef enum bkma_adv_impl {
    BKMA_ADV_AUTO = 0,   /* staged kernels, autotuned tile */
    BKMA_ADV_STAGED = 1, /* per-line FP64 departure + weights, lines staged in shared memory */
    BKMA_ADV_PLAIN = 2   /* per-cell FP64 reference math (AdvectionSolver.hpp:71-99); FP64 only */
} bkma_adv_impl;

typedef enum bkma_adv_weights {
    BKMA_W_REFERENCE = 0, /* AdvectionSolver::lag_basis, degree 5 only (AdvectionSolver.hpp:31-51) */
    BKMA_W_LAGRANGE = 1,  /* textbook Lagrange, degree 3 or 5 (no reference form) */
    BKMA_W_TABLE = 2      /* caller-supplied per-line weights (bkma_adv_plan_set_weights) */
} bkma_adv_weights;

typedef struct bkma_adv_plan bkma_adv_plan;

/* Mirrors ADVParams (src/config/AdvectionParams.hpp:10-57). dx, dvx, inv_dx
 * and the width are derived exactly as ADVParams::update_deltas
 * (AdvectionParams.cpp:96-103). The line velocity is coord(i0, minVx, dvx)
 * (AdvectionSolver.hpp:60) unless `velocity` is given. */
typedef struct bkma_adv_desc {
    int64_t n0, n1, n2;      /* full field extents, layout_right (n2 fastest) */
    int64_t i0_offset;       /* first global line of this shard */
    int64_t i0_count;        /* lines in this shard; 0 = n0 - i0_offset */
    int32_t dtype;           /* BKMA_F32 or BKMA_F64 */
    int32_t degree;          /* 3 or 5 */
    int32_t weights;         /* bkma_adv_weights */
    int32_t impl;            /* bkma_adv_impl */
    int32_t inplace;         /* 1: overwrite data (AdaptiveWg/NDRange); 0: write `out` (BasicRange) */
    int32_t reserved;
    double dt, minX, maxX, minVx, maxVx;
    const double *velocity;  /* optional HOST array of i0_count line velocities */
} bkma_adv_desc;

typedef struct bkma_adv_plan_info {
    int64_t lines;             /* i0_count */
    int64_t exception_lines;   /* lines whose departure offset is not constant along n1 */
    int32_t tile_cols;         /* n2 columns per tile (W) */
    int32_t tile_slabs;        /* n0 lines per tile (R) */
    int32_t threads;           /* threads per CTA */
    int32_t smem_bytes;        /* dynamic shared memory per CTA */
    int32_t npts;              /* stencil points (degree + 1) */
    int32_t autotuned;         /* 1 once bkma_adv_plan_autotune picked the tile */
    int64_t tiles;             /* CTAs per step */
    int32_t path;              /* 0: cp.async staging, 1: TMA (cp.async.bulk.tensor) staging,
                                  2: streamed columns, 3: contiguous lines (n2 = 1),
                                  4: FP64 in FP32-pair arithmetic (TMA staging),
                                  5: FP64 contiguous lines (n2 = 1) or whole slabs (even n2)
                                     in FP32-pair arithmetic,
                                  6: FP64 column pairs streamed in FP32-pair arithmetic */
    int32_t reserved;
} bkma_adv_plan_info;

int32_t bkma_abi_version(void);
const char *bkma_last_error(void);

/* impl_selector (src/tools/impl_selector.hpp:31-49): a strategy name to a
 * bkma_adv_impl; unknown names give BKMA_ERR_UNSUPPORTED with the reference's
 * message "<name> is not a valid implementation name.\nShould be: ...". */
bkma_status bkma_impl_from_name(const char *name, int32_t *impl, int32_t *inplace);

/* AdvectionSolver construction + create_optim_params: validates the
 * descriptor, computes every line's departure offset and weights in FP64 on
 * the host (bit-exact with AdvectionSolver::operator's leftNode), uploads the
 * per-line tables and picks a tile. */
bkma_status bkma_adv_plan_create(const bkma_adv_desc *desc, bkma_adv_plan **plan);
bkma_status bkma_adv_plan_info_get(const bkma_adv_plan *plan, bkma_adv_plan_info *info);
/* Times the candidate tiles on `scratch_field` (a device field of the plan's
 * shape, contents are overwritten) and keeps the fastest; cached per shape. */
bkma_status bkma_adv_plan_autotune(bkma_adv_plan *plan, void *scratch_field, void *stream);
/* Explicit tile choice (the reference's pref_wg_size / seq_size knobs):
 * W columns x R slabs per CTA, `threads` per CTA (128, 256 or 512), staging
 * path 0 (cp.async) or 1 (TMA; FP32, n2 % 4 == 0, W in {8,16,32}, R == 1),
 * or path 2: streamed columns (FP32, every line's per-step shift within the
 * streamed window, n1 >= 64), where R is the row-segment mode (0 = from the
 * field's size, k = up to k segments per 32-column group, k <= 8) and W the
 * tile width of the staged pass over exception lines, or path 3: contiguous
 * lines (FP32, n2 = 1, n1 % 4 == 0, n1 >= 16; W = 1, R whole lines per CTA,
 * `threads` ignored: 256), or path 4: FP64 in FP32-pair arithmetic (FP64,
 * degree 3 or 5, even n2 >= W, n1 >= 16; W = 4 with 128 threads or W = 8 with
 * 256, R = 1; a field off the 16-byte grid runs the FP64 staged kernel on the
 * same tiles), or path 5: FP64 contiguous lines in FP32-pair arithmetic (FP64,
 * degree 3 or 5, n2 = 1, n1 % 4 == 0, n1 >= 16; R whole lines per CTA; W = 1:
 * 4 cells per thread, W = 2: runs along two line sections per thread, for
 * n1 >= 512 and R = 1 or an even R <= 16, W = 3: half lines in the two CTAs
 * of a cluster, for n1 >= 8192 and R = 1, W = 4: runs of 4-cell groups per
 * thread, W = 5: lines of 16, 32, 64 or 128 cells shared by the lanes of a
 * warp, W = 6: half lines in clusters as W = 3, in runs of 4-cell groups as
 * W = 4, all the same bits; or with an even n2,
 * R whole slabs per CTA and W <= 64 runs of rows per column pair, the same
 * bits as path 4; `threads` ignored: 256; a field off the 16-byte grid runs
 * the FP64 staged kernel on whole rows or 8-column strips), or path 6: FP64 column pairs streamed in FP32-pair
 * arithmetic (FP64, degree 3 or 5, even n2, n1 >= 64, every line's tap-0
 * offset d within -32 <= d <= 33 - npts, and in each group of 64 consecutive
 * columns of the (line, i2) space either d > -(npts + 2) on every line,
 * walked up the rows, or d <= 2, walked down; R the row-segment mode as on
 * path 2, `threads` ignored: 256; the same bits as path 4; exception lines
 * and a field off the 16-byte grid run the FP64 staged kernel). R <= 1024 on
 * paths 0, 1, 3 and 5. */
bkma_status bkma_adv_plan_set_tile(bkma_adv_plan *plan, int32_t W, int32_t R, int32_t threads,
                                   int32_t path);
/* Multi-step fusion: bkma_adv_step runs `steps_per_launch` time steps per
 * kernel launch on column strips held in shared memory (the last launch of
 * a call runs the remainder), 1 = one step per launch (default). Results
 * are bit-identical to one step per launch of the staged kernels (FP32; for
 * FP64 the FP64-arithmetic staged kernel, path 0), except for FP64 plans on
 * contiguous lines in FP32-pair arithmetic (path 5 with n2 = 1, a 16-byte
 * aligned field, two copies of about 2048 cells' lines in shared memory):
 * those fuse in that arithmetic, bit-identical to one step per launch of
 * path 5; HBM traffic per cell-step
 * falls by the factor. Out of place, `data` is left unchanged. Not for the plain
 * FP64 form; BKMA_ERR_UNSUPPORTED when a strip of the plan's n1 rows does
 * not fit shared memory, and for FP32 lines longer than 4608 rows (the strips
 * would hold one column: slower than one step per launch). No counterpart in the reference, which runs one
 * step per kernel (src/advection.cpp:55-59). */
bkma_status bkma_adv_plan_set_fusion(bkma_adv_plan *plan, int32_t steps_per_launch);
/* On-chip state of the fused steps (FP32 plans, degree 3, 5 or 9).
 * BKMA_FUSED_F32 (default): FP32, bit-identical to one step per launch.
 * BKMA_FUSED_F32X2: each cell is held as an unevaluated sum hi + lo of two
 * FP32 numbers between the steps of a launch (Fast2Sum renormalisation, exact
 * wherever the cell's value exceeds its one-step change), so the field is
 * rounded to FP32 once per launch instead of once per step;
 * one step per launch still gives the FP32 bits. HBM traffic is unchanged.
 * BKMA_ERR_UNSUPPORTED for FP64 plans, the plain form, or n1 > 3632 (four
 * n1 x 4-column FP32 buffers must fit shared memory). No counterpart in the
 * reference. */
typedef enum bkma_fused_state { BKMA_FUSED_F32 = 0, BKMA_FUSED_F32X2 = 1 } bkma_fused_state;
bkma_status bkma_adv_plan_set_fused_state(bkma_adv_plan *plan, int32_t state);
/* BKMA_W_TABLE: per-line weights, i0_count x (degree+1) floats (host or
 * device pointer), applied on the plan's own departure offsets. */
bkma_status bkma_adv_plan_set_weights(bkma_adv_plan *plan, const float *weights, int32_t on_device);
/* Per-line departure offsets (tap-0 node minus i1, modulo n1) and FP64
 * fractional shifts d - 2 in [0,1) (host arrays of i0_count). */
bkma_status bkma_adv_plan_line_table(const bkma_adv_plan *plan, int32_t *offsets, double *shifts);
/* Synchronizes `stream`, returns the device status of the kernels' bounded
 * waits since the last query (BKMA_OK or BKMA_ERR_TIMEOUT) and clears it. */
bkma_status bkma_adv_plan_status(bkma_adv_plan *plan, void *stream);
/* Polls of each bounded device-side wait before it gives up (default
 * 4194304: with the kernels' back-off, about half a second to a second).
 * 0 makes every such wait give up at once: the launch then stops its tiles
 * without writing them, waits (with the default bound) for its own copies in
 * flight, and bkma_adv_plan_status reports BKMA_ERR_TIMEOUT - a way to test a
 * caller's timeout handling without a stuck GPU. Applies to the TMA-staged
 * kernel (the only advection kernel with a device-side wait). The reference
 * has no device-side waits; its errors are C++ exceptions
 * (src/core/bkma_tools.hpp:38-51). */
bkma_status bkma_adv_plan_set_wait_limit(bkma_adv_plan *plan, uint32_t polls);
bkma_status bkma_adv_plan_destroy(bkma_adv_plan *plan);

/* bkma_run for the advection solver: nsteps time steps of the device field
 * `data` (i0_count x n1 x n2 elements of dtype). In place when out is NULL or
 * equal to data. Out of place: the result lands in `out`; with nsteps > 1,
 * `data` serves as the ping-pong buffer and is overwritten. Asynchronous on
 * `stream`. */
bkma_status bkma_adv_step(bkma_adv_plan *plan, void *data, void *out, int32_t nsteps, void *stream);
/* The same on a HOST field: copies it to a plan-owned device buffer, runs
 * nsteps, copies the result back and synchronizes `stream`. */
bkma_status bkma_adv_run_host(bkma_adv_plan *plan, void *host_data, int32_t nsteps, void *stream);

/* Device init (fill_buffer_adv, init.hpp:31-46, generalised): mode 0 gives
 * sin(4*pi*x) like the reference; mode 1 gives sin(2*pi*x) + amp*(2u-1) with
 * u = bkma_uniform(seed, global cell index). */
bkma_status bkma_adv_fill(const bkma_adv_plan *plan, void *data, int32_t mode, double amp,
                          uint64_t seed, void *stream);
/* Fused error norms of `data` against `ref` (same shape; ref may be FP64 while
 * data is FP32): out[0] = max|data-ref|, out[1] = max|ref|, out[2] =
 * sum (data-ref)^2, out[3] = sum ref^2. Host array out[4]; synchronizes. */
bkma_status bkma_adv_error_norms(const bkma_adv_plan *plan, const void *data, int32_t data_dtype,
                                 const void *ref, int32_t ref_dtype, double *out, void *stream);
/* validate_result_adv (validation.hpp:9-80) on the device: max over i2 of
 * the mean L1 error against sin(4*pi*(x - v*t)), t = max_iter*dt. */
bkma_status bkma_adv_validate(const bkma_adv_plan *plan, const void *data, int64_t max_iter,
                              double *highest_l1, double *lowest_l1, void *stream);

/* ---------------------------------------------------------------- batches */
/* Several independent fields advanced by ONE persistent launch per step over
 * a device descriptor table (captured in a CUDA graph). */
typedef struct bkma_adv_field {
    void *data;              /* device field n0 x n1 x n2 of the batch dtype */
    int64_t n0, n1, n2;
    int32_t degree;          /* 3 or 5 */
    int32_t weights;         /* BKMA_W_REFERENCE or BKMA_W_LAGRANGE */
    double dt, minX, maxX, minVx, maxVx;
    const double *velocity;  /* optional HOST array of n0 line velocities */
} bkma_adv_field;

typedef struct bkma_adv_batch bkma_adv_batch;
bkma_status bkma_adv_batch_create(const bkma_adv_field *fields, int32_t nfields, int32_t dtype,
                                  bkma_adv_batch **batch);
bkma_status bkma_adv_batch_step(bkma_adv_batch *batch, int32_t nsteps, void *stream);
/* Times the tile-model candidates (shared-memory cap per tile, threads per
 * CTA) on the live fields - their contents advance by the timed steps - and
 * keeps the fastest. */
bkma_status bkma_adv_batch_autotune(bkma_adv_batch *batch, void *stream);
/* Chosen tiles: per field W (columns) and R (slabs) (arrays of nfields; for
 * a field that runs in the streamed form W = 0 and R = its row segments per
 * 32-column group, and its exception lines, if any, stay staged), the total
 * staged tile count, and threads and shared memory per CTA of the staged
 * kernel. */
bkma_status bkma_adv_batch_tiles(const bkma_adv_batch *batch, int32_t *W, int32_t *R, int64_t *tiles,
                                 int32_t *threads, int64_t *smem_bytes);
/* Total cells over all fields, and kernel launches per step. */
bkma_status bkma_adv_batch_info(const bkma_adv_batch *batch, int64_t *cells, int32_t *launches_per_step);
bkma_status bkma_adv_batch_destroy(bkma_adv_batch *batch);

/* ------------------------------------------------------------------ conv1d */
typedef enum bkma_conv_semantics {
    BKMA_CONV_TORCH = 0,     /* cross-correlation (B, C, L) like torch.nn.functional.conv1d */
    BKMA_CONV_REFERENCE = 1  /* ConvSolver + AdaptiveWg packing (ConvSolver.hpp:20-44) */
} bkma_conv_semantics;

typedef enum bkma_conv_impl {
    BKMA_CONV_AUTO = 0,
    BKMA_CONV_TENSOR = 1,    /* BF16 tcgen05 implicit GEMM, FP32 accumulate in TMEM */
    BKMA_CONV_PLAIN = 2      /* scalar FP64 / FP32 */
} bkma_conv_impl;

/* TORCH: data (batch, cin, length), weight (cout, cin, ksize), bias (cout).
 * REFERENCE: data (n0, cin*length, n2), weight (ksize, cin, cin), bias (cin),
 * matching Conv1dParams (src/config/Conv1dParams.cpp:44-76) with n0 =
 * batch and n2 as given. In place the output (length - ksize + 1 per
 * channel row, or the packed cin*length - ksize + 1 per line) overwrites the
 * start of each row of `data`. */
typedef struct bkma_conv_desc {
    int64_t batch, cin, cout, length, ksize;
    int64_t n2;              /* REFERENCE semantics only; 1 otherwise */
    int32_t dtype;           /* BKMA_BF16 (TENSOR), BKMA_F32 or BKMA_F64 (PLAIN) */
    int32_t semantics;       /* bkma_conv_semantics */
    int32_t impl;            /* bkma_conv_impl */
    int32_t inplace;
} bkma_conv_desc;

typedef struct bkma_conv_plan bkma_conv_plan;
bkma_status bkma_conv_plan_create(const bkma_conv_desc *desc, bkma_conv_plan **plan);
/* Device bytes of scratch the plan owns (halo snapshots, packed weights). */
bkma_status bkma_conv_plan_scratch_bytes(const bkma_conv_plan *plan, int64_t *bytes);
bkma_status bkma_conv_run(bkma_conv_plan *plan, void *data, void *out, const void *weight,
                          const void *bias, void *stream);
/* Synchronizes `stream` and returns the device status of the tensor-core
 * kernel's bounded waits since the last query (BKMA_OK or BKMA_ERR_TIMEOUT),
 * then clears it. */
bkma_status bkma_conv_plan_status(bkma_conv_plan *plan, void *stream);
/* Polls of each bounded wait of the tensor-core kernel's pipeline before it
 * gives up (default 4194304, about a second); 0 makes the first wait of every
 * role give up at once, so the call stops, drains the MMAs it issued, frees
 * its tensor memory and bkma_conv_plan_status reports BKMA_ERR_TIMEOUT. For
 * testing a caller's timeout handling; no counterpart in the reference. */
bkma_status bkma_conv_plan_set_wait_limit(bkma_conv_plan *plan, uint32_t polls);
bkma_status bkma_conv_plan_destroy(bkma_conv_plan *plan);

/* fill_buffer_conv1d (src/tools/init.hpp:50-72): `count` elements of a
 * device buffer of `dtype` (F32, F64 or BF16) set to `value`. */
bkma_status bkma_fill(void *data, int64_t count, int32_t dtype, double value, void *stream);
/* sum_and_normalize_conv1d + validate_conv1d (src/tools/validation.hpp:
 * 84-156) in one pass over the device field (n0, n1, n2): *mean = the mean of
 * the values (i0, i1 < nw, i2), summed in FP64 in a fixed order; *equal = 1
 * when every value at a given i1 < nw is the same for all (i0, i2) (a NaN
 * counts as different), else 0. Synchronizes `stream`. */
bkma_status bkma_conv_check(const void *data, int32_t dtype, int64_t n0, int64_t n1, int64_t n2,
                            int64_t nw, double *mean, int32_t *equal, void *stream);

/* In-place BF16 tensor-core conv1d (torch semantics, cin = cout = channels,
 * data (batch, channels, length), weight (channels, channels, ksize), bias
 * (channels) or NULL) that allocates nothing. No counterpart in the
 * reference: it exists for callers that must not call cudaMalloc while they
 * run - runtimes that give all device memory to their own pool at start-up
 * and forbid further driver allocations, and loops that cannot afford an
 * allocation's implicit synchronization. Its scratch is one 16 MiB device
 * array inside the library (held by every GPU that loads it until exit):
 * 512 KiB for packed weights and 15.5 MiB for the halo snapshot, which keeps
 * one slot per chunk of consecutive tiles (at most 3840 slots of
 * channels * 2 * max(8, round_up(ksize-1, 8)) bytes: at most 15 MiB for every
 * shape the tensor path takes), so no batch or length is limited by it; a
 * shape that would need more is refused with BKMA_ERR_INVALID_ARG. The
 * arguments obey the same bounds as bkma_conv_plan_create. The first call on
 * a device looks the array's address up, so make it before any stream
 * capture. Calls share the array, which keeps the last call's contents:
 * calls that overlap on the GPU race. */
bkma_status bkma_conv1d_bf16_inplace_noalloc(void *data, const void *weight, const void *bias,
                                             int64_t batch, int64_t channels, int64_t length,
                                             int64_t ksize, void *stream);
/* Status of the last bkma_conv1d_bf16_inplace_noalloc call on the current
 * device: synchronizes `stream`, returns BKMA_OK or BKMA_ERR_TIMEOUT (a
 * bounded device-side wait gave up, so the output is incomplete) and clears
 * it. Allocates nothing. No counterpart in the reference. */
bkma_status bkma_conv1d_noalloc_status(void *stream);

/* ------------------------------------------------------- learned stencil */
/* A small MLP (1 -> 32 -> 32 -> npts, GELU, FP32) maps a line's fractional
 * shift a in [0,1) to a corrected stencil w(a) = L(a) + c(a) - mean(c(a)) of
 * npts = 4 points (L: degree-3 Lagrange on nodes 0..3 at 1 + a) or 6 points
 * (degree-5 Lagrange on nodes 0..5 at 2 + a); the weights keep summing to one.
 * No counterpart in the reference (which only has the fixed degree-5
 * stencil); the trained weights feed an advection plan created with
 * BKMA_W_TABLE and degree npts - 1 through bkma_adv_plan_set_weights.
 * Parameter layout (32 + 32 + 1024 + 32 + 33 npts floats: 1252 for 4 points,
 * 1318 for 6): W1[32] b1[32] W2[32][32] b2[32] W3[npts][32] b3[npts]; the output
 * layer starts at zero, so an untrained model is the Lagrange stencil. */
typedef struct bkma_mlp bkma_mlp;
/* A 4-point model. */
bkma_status bkma_mlp_create(uint64_t seed, bkma_mlp **mlp);
/* A model of npts = 4 or 6 points. */
bkma_status bkma_mlp_create_stencil(uint64_t seed, int32_t npts, bkma_mlp **mlp);
/* The model's stencil points and parameter count. */
bkma_status bkma_mlp_info(const bkma_mlp *mlp, int32_t *npts, int32_t *nparams);
/* Copy the parameters to (set = 0) or from (set = 1) a host array. */
bkma_status bkma_mlp_params(bkma_mlp *mlp, float *host_params, int32_t set);
/* Training samples first .. first+n-1 into device arrays alpha[n],
 * taps4[n][4], target[n]: a random periodic line (32 Fourier modes with
 * amplitudes U[-1,1]/m), its 4 nodes j-1..j+2 and the degree-9 Lagrange value
 * at j + alpha. */
bkma_status bkma_mlp_samples(int64_t n, uint64_t seed, int64_t first, float *alpha, float *taps4,
                             float *target, void *stream);
/* The same on lines sampled on n1 cells, with the npts nodes around node j
 * (taps[n][npts]) and, when exact = 1, the target f(x_j + a/n1) of the line's
 * own Fourier series instead of the degree-9 Lagrange value (for coarse
 * grids, where degree 9 is not accurate either). bkma_mlp_samples is
 * n1 = 1024, npts = 4, exact = 0. */
bkma_status bkma_mlp_samples_grid(int64_t n, uint64_t seed, int64_t first, int64_t n1,
                                  int32_t npts, int32_t exact, float *alpha, float *taps,
                                  float *target, void *stream);
/* Mean squared error over all n samples and its gradient (host float[nparams]);
 * taps is [n][npts] of the model's npts. */
bkma_status bkma_mlp_grad(bkma_mlp *mlp, const float *alpha, const float *taps,
                          const float *target, int64_t n, float *host_grad, double *host_loss,
                          void *stream);
/* `steps` Adam steps on random batches of `batch` samples drawn from the n
 * samples, cosine learning rate from lr_max; host_loss gets the last batch's
 * mean squared error. */
bkma_status bkma_mlp_train(bkma_mlp *mlp, const float *alpha, const float *taps,
                           const float *target, int64_t n, int32_t steps, int32_t batch,
                           float lr_max, uint64_t seed, double *host_loss, void *stream);
/* Stencils of n shifts: device alpha[n] -> device weights[n][npts]. */
bkma_status bkma_mlp_infer(const bkma_mlp *mlp, const float *alpha, int64_t n, float *weights,
                           void *stream);
bkma_status bkma_mlp_destroy(bkma_mlp *mlp);

#ifdef __cplusplus
}
#endif
#endif
