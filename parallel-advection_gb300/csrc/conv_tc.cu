// BF16 tensor-core conv1d (torch semantics) on sm_103a: a persistent implicit
// GEMM with tcgen05.mma, FP32 accumulation in TMEM.
//
// Per row b the convolution is D[co, l] = sum_k W_k[co, :] . X[:, l + k]
// (W_k = weight[:, :, k]). GEMM view per tap: M = Cout (<= 128, zero-padded
// rows), N = output positions, K = Cin.
//
//  * A (weights) stays on chip for the whole kernel. Every MMA has N = 128
//    (a tcgen05.mma costs at least ~51 cycles, so N = 32 or 64 cannot reach
//    the tensor peak; N >= 128 does). Two 128-column FP32 accumulators leave
//    256 TMEM columns for weights: taps 0..3 (Cin = 128) sit in TMEM (lane m
//    = output channel, column (k*Cin + ci)/2 holds the BF16 pair (ci, ci+1)),
//    the remaining taps sit in shared memory as K-major no-swizzle A tiles.
//  * B (activations) is staged K-major without swizzle: 16-byte rows of 8
//    input channels, one row per position l, rows contiguous (SBO = 128 B),
//    ci-chunks at a padded stride (LBO). Tap k is then the same staging
//    buffer with the descriptor start moved by k rows (16*k bytes): the
//    implicit im2col costs nothing.
//  * Producer warps load the tile from HBM with 16-byte loads along l,
//    transpose 8x8 BF16 blocks in registers, and store conflict-free (the
//    odd row count of a chunk spreads the 8 stores of a phase over all
//    banks). A warp covers 8 consecutive channel chunks x 4 consecutive row
//    blocks, so one load instruction touches 8 lines of 64 bytes.
//  * Items ((row, tile) pairs) are grouped in chunks of `chunk` consecutive
//    tiles; CTAs take chunks round-robin (the CTAs of one round read
//    neighbouring stretches of every channel row) and run a chunk's tiles in
//    order. The items left after the full rounds are split evenly, one
//    shorter chunk per CTA, so every CTA runs the same number of items (+-1). In place, the rows past a tile (the next tile's first K-1
//    positions) are then still unwritten when its producer reads them: the
//    next tile's epilogue waits for its MMAs, which wait for this tile's
//    stage. Only the rows past a chunk's last tile belong to another CTA; the
//    prologue kernel snapshots them (one slot per chunk) before the main
//    kernel starts.
//  * One thread issues the MMAs of a 128-position item (K taps x Cin/16
//    K-steps) into a TMEM accumulator; four epilogue warps drain it
//    (tcgen05.ld), add the bias and round to BF16. When the output rows are
//    16-byte strided, each warp writes its 32 channels x 64 positions into a
//    128-byte-swizzled shared tile (conflict-free) and one lane stores it
//    with a TMA tensor store (two tiles per warp stored together after the
//    accumulator is released, or one tile stored per half, by shape);
//    otherwise lanes store their own rows.
//    The shared-memory data path is the limit of this kernel (every N = 128
//    MMA reads a 4 KB B tile: half its bandwidth at the tensor rate), so
//    every other access is shaped for few wavefronts.
//  * Every mbarrier wait is bounded; on timeout the CTA raises a status word,
//    stops, drains its MMAs with a bounded wait and frees TMEM.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cstring>

#include "conv.cuh"

namespace bkma {
namespace tc {

constexpr int TILE = 128;   // output positions per item = N of every MMA
constexpr int STAGES_MAX = 6;
constexpr int TMEM_COLS = 512;
// TMEM: weights of taps 0 .. taps_tmem-1 in columns [0, 512 - 128 nacc), then
// nacc FP32 accumulators of 128 columns. One accumulator leaves 384 columns
// for weights (6 taps of Cin = 128 instead of 4): the MMAs of the next item
// wait only until the epilogue has read the accumulator into registers.
constexpr int SMEM_LIMIT = 232448 - 1024;
constexpr int NUM_EPI_WARPS = 4;
constexpr int NUM_PROD_WARPS = 8;  // two groups of 4 warps, alternate items
constexpr int PROD_GROUP = 128;    // threads per producer group
constexpr int THREADS = 32 * (NUM_EPI_WARPS + NUM_PROD_WARPS + 1);
constexpr uint32_t kSpinLimit = kWaitPolls;  // x ~ 0.25 us backoff: ~1 s
constexpr int MAX_CTAS = 1024;             // grid cap
constexpr int CHUNK_TILES = 64;            // preferred tiles per chunk
constexpr int MAX_SLOTS = 3840;            // halo snapshot slots (chunks) per call: <= 15 MiB

constexpr int EPI_TILE_BYTES = 4096;  // 32 channels x 64 positions BF16
// epilogue tiles per warp: 2 (one per half item, both stored after the
// accumulator is released) or 1 (each half stored as soon as it is staged)
constexpr int epi_bytes(int tiles) { return NUM_EPI_WARPS * tiles * EPI_TILE_BYTES + 1024; }

struct Args {
    CUtensorMap out_map;      // (lout, cout, B) view of out, 64 x 32 x 1 boxes, 128-B swizzle
    const __nv_bfloat16 *x;   // (B, Cin, L)
    __nv_bfloat16 *out;       // (B, Cout, out_stride)
    const __nv_bfloat16 *w;   // (Cout, Cin, K)
    const __nv_bfloat16 *bias;  // (Cout) or null
    const __nv_bfloat16 *halo;  // [chunk slots][Cin][halo_rows]: rows past each chunk, or null
    const uint32_t *wpack_tmem;  // [128][tm_cols] BF16 pairs: TMEM image of taps 0..taps_tmem-1
    const uint4 *wpack_smem;     // shared-memory image of taps taps_tmem..K-1
    int B, cin, cout, K;
    int64_t L, lout, out_stride;
    int ntiles;
    int chunk;       // items per chunk (the last chunk may be shorter)
    int halo_rows;   // rows after the tile: round_up(K-1, 8)
    int chunk_rows;  // TILE + halo_rows + 1 (odd, spreads banks)
    int stage_bytes;
    int stages;      // activation stages (2..STAGES_MAX)
    int taps_tmem;   // taps whose weights live in TMEM; the rest live in shared memory
    int nacc;        // FP32 accumulators in TMEM (1 or 2)
    int tm_cols;     // TMEM columns of the weight image: 512 - 128 * nacc
    int wsmem_bytes; // shared-memory weights, placed before the stages
    int epi_tma;     // 1 or 2: the epilogue stores through out_map from 1 or 2 tiles per warp
    int epi_off;     // offset of the epilogue tiles (after the stages)
    int *status;     // device status word (0 ok, 4 timeout)
    uint32_t spin_limit;  // polls of a pipeline wait before the CTA gives up (the final
                          // drain of the MMAs always uses kSpinLimit)
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile(
        "{\n .reg .b64 st;\n mbarrier.arrive.shared::cta.b64 st, [%0];\n}" ::"r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ bool mbar_try(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait (at most `polls` polls of the barrier). Returns false (and
// raises the CTA abort flag) on timeout, or when another thread already
// aborted.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, volatile int *abort_flag,
                                          int *status, uint32_t polls) {
    for (uint32_t i = 0; i < polls; ++i) {
        if (mbar_try(bar, parity)) return true;
        if (*abort_flag) return false;
        if (i > 64) __nanosleep(256);
    }
    *abort_flag = 1;
    atomicExch(status, (int)BKMA_ERR_TIMEOUT);
    return false;
}

__device__ __forceinline__ void fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// Instruction descriptor: kind::f16, BF16 A and B, FP32 D, both K-major.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
           ((uint32_t)(M >> 4) << 24);
}

// Same MMA with the B descriptor given as its two 32-bit words.
__device__ __forceinline__ void mma_ts2(uint32_t d_tmem, uint32_t a_tmem, uint32_t b_lo,
                                        uint32_t b_hi, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n .reg .b64 bd;\n setp.ne.u32 p, %5, 0;\n mov.b64 bd, {%2, %3};\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], bd, %4, p;\n}" ::"r"(d_tmem),
        "r"(a_tmem), "r"(b_lo), "r"(b_hi), "r"(idesc), "r"(accumulate)
        : "memory");
}

// MMA with both operands in shared memory (descriptor words lo/hi).
__device__ __forceinline__ void mma_ss2(uint32_t d_tmem, uint32_t a_lo, uint32_t a_hi, uint32_t b_lo,
                                        uint32_t b_hi, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n .reg .b64 ad, bd;\n setp.ne.u32 p, %6, 0;\n mov.b64 ad, {%1, %2};\n"
        " mov.b64 bd, {%3, %4};\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], ad, bd, %5, p;\n}" ::"r"(d_tmem),
        "r"(a_lo), "r"(a_hi), "r"(b_lo), "r"(b_hi), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t *bar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void tmem_st32(uint32_t taddr, const uint32_t (&v)[32]) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, "
        "%10, %11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, "
        "%27, %28, %29, %30, %31, %32};" ::"r"(taddr),
        "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]),
        "r"(v[8]), "r"(v[9]), "r"(v[10]), "r"(v[11]), "r"(v[12]), "r"(v[13]), "r"(v[14]),
        "r"(v[15]), "r"(v[16]), "r"(v[17]), "r"(v[18]), "r"(v[19]), "r"(v[20]), "r"(v[21]),
        "r"(v[22]), "r"(v[23]), "r"(v[24]), "r"(v[25]), "r"(v[26]), "r"(v[27]), "r"(v[28]),
        "r"(v[29]), "r"(v[30]), "r"(v[31])
        : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&v)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
        "%11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, "
        "%28, %29, %30, %31}, [%32];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
          "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]),
          "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]),
          "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]),
          "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]),
          "=r"(v[31])
        : "r"(taddr)
        : "memory");
}

__device__ __forceinline__ uint32_t bf16_bits(__nv_bfloat16 h) {
    return (uint32_t)__bfloat16_as_ushort(h);
}

// Load the 8x8 block (ci = 8c..8c+7) x (rows 8q..8q+7 of the tile) into v[j]
// (row j = ci 8c+j, 8 positions). slot >= 0 (in place, the last item of
// chunk `slot`): the rows past the tile come from that halo slot (16-byte
// rows, halo_rows values per channel).
__device__ __forceinline__ void load_block(const Args &a, int b, int tile, int c, int q, int64_t slot,
                                           uint4 (&v)[8]) {
    const int64_t l0 = (int64_t)tile * TILE;
    const int r0 = 8 * q;
    const int64_t col = l0 + r0;
    if (r0 >= TILE + a.K - 1) {  // rows no output reads (K = 1): never touch the next tile
#pragma unroll
        for (int j = 0; j < 8; ++j) v[j] = make_uint4(0, 0, 0, 0);
        return;
    }
    if (slot >= 0 && r0 >= TILE) {
        const __nv_bfloat16 *h = a.halo + (slot * a.cin + 8 * c) * a.halo_rows + (r0 - TILE);
#pragma unroll
        for (int j = 0; j < 8; ++j) v[j] = *reinterpret_cast<const uint4 *>(h + (int64_t)j * a.halo_rows);
        return;
    }
    if (col + 8 <= a.L) {
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int64_t ci = 8 * c + j;
            v[j] = *reinterpret_cast<const uint4 *>(a.x + ((int64_t)b * a.cin + ci) * a.L + col);
        }
        return;
    }
    // past the end of the row: zeros (L is a multiple of 8, so a block is
    // either fully inside or fully outside)
#pragma unroll
    for (int j = 0; j < 8; ++j) v[j] = make_uint4(0, 0, 0, 0);
}

// Chunk k of a launch with `grid` CTAs over `items` items: rounds of grid
// chunks of `chunk` items, then one last chunk per CTA that splits the rest
// evenly (possibly empty). Sets [*begin, *end); slot k = r * grid + c.
__host__ __device__ __forceinline__ void chunk_range(int64_t k, int64_t items, int grid, int chunk,
                                                     int64_t *begin, int64_t *end) {
    const int64_t per_round = (int64_t)grid * chunk;
    const int64_t rounds = items / per_round;
    if (k < rounds * grid) {
        *begin = k * chunk;
        *end = *begin + chunk;
    } else {
        const int64_t base = rounds * per_round, rem = items - base, c = k - rounds * grid;
        *begin = base + (c * rem) / grid;
        *end = base + ((c + 1) * rem) / grid;
    }
}
__host__ __device__ __forceinline__ int64_t chunk_slots(int64_t items, int grid, int chunk) {
    return (items / ((int64_t)grid * chunk) + 1) * grid;
}

// Block p of an item's (channel chunk, row block) pairs. With a multiple of 8
// chunks, 32 consecutive p cover chunks 8g..8g+7 x row blocks 4m..4m+3 of the
// tile body (one 64-byte segment of 8 channel rows per load instruction; the
// chunk residues 0..7 keep the transposed stores conflict-free), then the
// halo blocks; otherwise chunks vary fastest.
__device__ __forceinline__ void block_of(int p, int nchunks, int &c, int &q) {
    const int body = nchunks * (TILE / 8);
    if ((nchunks & 7) == 0 && p < body) {
        c = (p & 7) + 8 * ((p >> 3) / (TILE / 8));
        q = (p >> 3) % (TILE / 8);
    } else if ((nchunks & 7) == 0) {
        c = (p - body) % nchunks;
        q = TILE / 8 + (p - body) / nchunks;
    } else {
        c = p % nchunks;
        q = p / nchunks;
    }
}

// Transpose an 8x8 BF16 block (v[j] = channel j, 8 positions) into 8 rows of
// 8 channels and store them at dst + 16*i.
__device__ __forceinline__ void store_block(unsigned char *dst, const uint4 (&v)[8]) {
    const uint32_t *w = reinterpret_cast<const uint32_t *>(v);
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int wsel = i / 2;
        const uint32_t sel = (i & 1) ? 0x7632u : 0x5410u;
        uint4 o;
        o.x = __byte_perm(w[0 * 4 + wsel], w[1 * 4 + wsel], sel);
        o.y = __byte_perm(w[2 * 4 + wsel], w[3 * 4 + wsel], sel);
        o.z = __byte_perm(w[4 * 4 + wsel], w[5 * 4 + wsel], sel);
        o.w = __byte_perm(w[6 * 4 + wsel], w[7 * 4 + wsel], sel);
        *reinterpret_cast<uint4 *>(dst + (size_t)i * 16) = o;
    }
}

// Prologue of one call (one launch, before the main kernel). Words
// [0, nA + nB): the weight images - the TMEM image of taps 0..taps_tmem-1 (BF16
// pairs (ci, ci+1) per output channel) and the shared-memory image of the
// other taps ([tap][ci-chunk][co][8 ci], K-major no-swizzle A tiles of 128
// rows). Then, in place (halo != null), 16-byte pieces of the halo snapshot:
// slot c = x[b][ci][(t+1)*TILE + j], j < halo_rows, for the last item (b, t)
// of chunk c (chunk_range), zero past L; empty chunks have no slot content.
__global__ void conv_tc_prologue(const __nv_bfloat16 *w, int cin, int cout, int K, int taps_tmem,
                                 int tm_cols, uint32_t *tm_img, uint32_t *sm_img,
                                 const __nv_bfloat16 *x, __nv_bfloat16 *halo, int64_t items,
                                 int grid, int chunk, int ntiles, int64_t L, int halo_rows) {
    const int wcols = taps_tmem * cin / 2;
    const int nA = 128 * tm_cols;
    const int nB = (K - taps_tmem) * (cin / 8) * 128 * 4;  // 32-bit words
    const int pieces = halo_rows / 8;
    const int64_t nS = halo ? chunk_slots(items, grid, chunk) * cin * pieces : 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nA + nB + nS;
         i += (int64_t)gridDim.x * blockDim.x) {
        if (i >= nA + nB) {
            int64_t r = i - nA - nB;
            const int piece = (int)(r % pieces);
            r /= pieces;
            const int ci = (int)(r % cin);
            const int64_t c = r / cin;
            int64_t first, end;
            chunk_range(c, items, grid, chunk, &first, &end);
            if (end == first) continue;
            const int64_t last = end - 1;
            const int64_t b = last / ntiles;
            const int64_t col = (last % ntiles + 1) * TILE + 8 * piece;
            uint4 v = make_uint4(0, 0, 0, 0);
            if (col + 8 <= L) v = *reinterpret_cast<const uint4 *>(x + (b * cin + ci) * L + col);
            *reinterpret_cast<uint4 *>(halo + (c * cin + ci) * halo_rows + 8 * piece) = v;
            continue;
        }
        int co, k, ci;
        if (i < nA) {
            co = (int)(i / tm_cols);
            const int col = (int)(i % tm_cols);
            if (col >= wcols || co >= cout) {
                tm_img[i] = 0;
                continue;
            }
            k = (2 * col) / cin;
            ci = (2 * col) % cin;
        } else {
            int r = (int)(i - nA);
            const int e = r % 4;
            r /= 4;
            co = r % 128;
            r /= 128;
            const int c = r % (cin / 8);
            k = taps_tmem + r / (cin / 8);
            ci = 8 * c + 2 * e;
            if (co >= cout) {
                sm_img[i - nA] = 0;
                continue;
            }
        }
        const __nv_bfloat16 *wr = w + (int64_t)co * cin * K;
        const uint32_t pair = (uint32_t)__bfloat16_as_ushort(wr[(int64_t)ci * K + k]) |
                              ((uint32_t)__bfloat16_as_ushort(wr[(int64_t)(ci + 1) * K + k]) << 16);
        if (i < nA)
            tm_img[i] = pair;
        else
            sm_img[i - nA] = pair;
    }
}

// KC: K16 steps per tap (Cin / 16). kPlanPolls: the pipeline waits poll
// a.spin_limit times (a plan whose wait limit was changed) instead of the
// compile-time kSpinLimit; a runtime bound in the MMA issue loop measured 11 %
// slower on the bench workload, so the default instantiation keeps the constant.
template <int KC, bool kPlanPolls>
__global__ void __launch_bounds__(THREADS, 1) conv_tc_kernel(const __grid_constant__ Args a) {
    const uint32_t polls = kPlanPolls ? a.spin_limit : kSpinLimit;
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ __align__(8) uint64_t full_bar[STAGES_MAX], empty_bar[STAGES_MAX];
    __shared__ __align__(8) uint64_t accf_bar[2], acce_bar[2];
    __shared__ __align__(8) uint64_t drain_bar;
    __shared__ uint32_t tmem_base_sh;
    __shared__ volatile int abort_flag;

    const int warp = threadIdx.x / 32;
    const int lane = threadIdx.x % 32;
    const bool is_epi = warp < NUM_EPI_WARPS;
    const bool is_prod = warp >= NUM_EPI_WARPS && warp < NUM_EPI_WARPS + NUM_PROD_WARPS;
    const bool is_mma = warp == NUM_EPI_WARPS + NUM_PROD_WARPS;
    const int stages = a.stages;

    if (threadIdx.x == 0) {
        abort_flag = 0;
        for (int s = 0; s < stages; ++s) {
            mbar_init(&full_bar[s], PROD_GROUP);
            mbar_init(&empty_bar[s], 1);
        }
        for (int i = 0; i < 2; ++i) {
            mbar_init(&accf_bar[i], 1);
            mbar_init(&acce_bar[i], 32 * NUM_EPI_WARPS);
        }
        mbar_init(&drain_bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(&tmem_base_sh)),
                     "r"(TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = tmem_base_sh;
    const int cin = KC * 16;
    unsigned char *wsm = smem;                      // shared-memory weights
    unsigned char *stages_sm = smem + a.wsmem_bytes;  // activation stages

    // ---- weights on chip from the pre-packed images
    if (is_epi) {  // TMEM part: thread = output channel = TMEM lane
        const int co = threadIdx.x;
        const int wcols = a.taps_tmem * cin / 2;
        const uint32_t lane_addr = tmem + ((uint32_t)(32 * warp) << 16);
        const uint4 *src = reinterpret_cast<const uint4 *>(a.wpack_tmem + (size_t)co * a.tm_cols);
        for (int c0 = 0; c0 < wcols; c0 += 32) {
            uint32_t v[32];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const uint4 q4 = src[c0 / 4 + j];
                v[4 * j] = q4.x;
                v[4 * j + 1] = q4.y;
                v[4 * j + 2] = q4.z;
                v[4 * j + 3] = q4.w;
            }
            tmem_st32(lane_addr + (uint32_t)c0, v);
        }
        asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
    }
    {  // shared-memory part: every thread copies 16-byte chunks
        const int n16 = (a.K - a.taps_tmem) * cin * 256 / 16;
        for (int i = threadIdx.x; i < n16; i += blockDim.x)
            reinterpret_cast<uint4 *>(wsm)[i] = a.wpack_smem[i];
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();

    const int64_t items = (int64_t)a.B * a.ntiles;
    const int64_t chunk_ids = chunk_slots(items, gridDim.x, a.chunk);
    const uint32_t smem_base = smem_u32(smem);
    // Every role walks the same item sequence: chunks blockIdx.x, +gridDim.x,
    // ..., the items of a chunk in order.
#define BKMA_TC_FOR_ITEMS                                                              \
    for (int64_t ch = blockIdx.x, item = 0, iend = 0; ch < chunk_ids; ch += gridDim.x) \
        for (chunk_range(ch, items, gridDim.x, a.chunk, &item, &iend); item < iend; ++item, ++it)

    if (is_prod) {
        const int pidx = threadIdx.x - 32 * NUM_EPI_WARPS;  // 0..255
        const int grp = pidx / PROD_GROUP;                 // items it with it % 2 == grp
        const int pt = pidx % PROD_GROUP;
        const int cchunks = cin / 8;  // 8-channel chunks
        const int qblocks = (TILE + a.halo_rows) / 8;
        const int pairs = cchunks * qblocks;
        int it = 0;
        BKMA_TC_FOR_ITEMS {
            if ((it & 1) != grp) continue;
            const int s = it % stages;
            const uint32_t ph = (uint32_t)(it / stages) & 1u;
            if (!mbar_wait(&empty_bar[s], ph ^ 1u, &abort_flag, a.status, polls)) break;
            const int b = (int)(item / a.ntiles);
            const int tile = (int)(item % a.ntiles);
            unsigned char *stage = stages_sm + (size_t)s * a.stage_bytes;
            const int64_t slot = (a.halo != nullptr && item == iend - 1) ? ch : -1;
            // up to three 8x8 blocks per thread in flight at once (one round trip
            // for Cin = 128: 16 chunks x 17 row blocks = 272 blocks / 128 threads)
            for (int p = pt; p < pairs; p += 3 * PROD_GROUP) {
                uint4 v[3][8];
                int bc[3], bq[3];
#pragma unroll
                for (int h = 0; h < 3; ++h) {
                    const int ph2 = p + h * PROD_GROUP;
                    block_of(ph2, cchunks, bc[h], bq[h]);
                    if (ph2 < pairs) load_block(a, b, tile, bc[h], bq[h], slot, v[h]);
                }
#pragma unroll
                for (int h = 0; h < 3; ++h) {
                    const int ph2 = p + h * PROD_GROUP;
                    if (ph2 < pairs)
                        store_block(stage + ((size_t)bc[h] * a.chunk_rows + 8 * bq[h]) * 16, v[h]);
                }
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            mbar_arrive(&full_bar[s]);
        }
    } else if (is_mma) {
        if (lane == 0) {
            const uint32_t idesc = idesc_bf16(128, TILE);
            const uint32_t lbo16 = (uint32_t)a.chunk_rows;  // B: LBO >> 4 (ci-chunk stride)
            // high word of both descriptors: SBO = 128 B (>> 4 = 8), version 1 (bit 46)
            const uint32_t desc_hi = (128u >> 4) | (1u << 14);
            const uint32_t a_step = (uint32_t)(cin / 2);  // TMEM columns per tap
            // A in shared memory: LBO = 2048 B (chunk of 128 rows x 16 B)
            const uint32_t wlo0 = (smem_base >> 4) | ((2048u >> 4) << 16);
            const uint32_t tap16 = (uint32_t)(cin * 256) >> 4;
            const uint32_t stage0 = smem_base + (uint32_t)a.wsmem_bytes;
            int it = 0;
            BKMA_TC_FOR_ITEMS {
                const int s = it % stages;
                const uint32_t ph = (uint32_t)(it / stages) & 1u;
                if (!mbar_wait(&full_bar[s], ph, &abort_flag, a.status, polls)) break;
                const int acc = a.nacc == 2 ? (it & 1) : 0;
                const uint32_t aph = (uint32_t)(a.nacc == 2 ? (it >> 1) : it) & 1u;
                if (!mbar_wait(&acce_bar[acc], aph ^ 1u, &abort_flag, a.status, polls)) break;
                fence_after();
                const uint32_t d_tmem = tmem + (uint32_t)(a.tm_cols + acc * TILE);
                // descriptor low word: start address >> 4 (bits 0-13, < 256 KB so
                // row / chunk offsets never carry into the LBO field at bit 16)
                const uint32_t lo0 = ((stage0 + (uint32_t)(s * a.stage_bytes)) >> 4) | (lbo16 << 16);
                uint32_t a_k = tmem;
                int k = 0;
                for (; k < a.taps_tmem; ++k, a_k += a_step) {
#pragma unroll
                    for (int j = 0; j < KC; ++j)
                        mma_ts2(d_tmem, a_k + 8u * j, lo0 + (uint32_t)k + 2u * j * lbo16, desc_hi,
                                idesc, (k | j) != 0 ? 1u : 0u);
                }
                for (; k < a.K; ++k) {
                    const uint32_t wk = wlo0 + (uint32_t)(k - a.taps_tmem) * tap16;
#pragma unroll
                    for (int j = 0; j < KC; ++j)
                        mma_ss2(d_tmem, wk + 2u * j * 128u, desc_hi, lo0 + (uint32_t)k + 2u * j * lbo16,
                                desc_hi, idesc, (k | j) != 0 ? 1u : 0u);
                }
                mma_commit(&accf_bar[acc]);
                mma_commit(&empty_bar[s]);
            }
            // all MMAs issued by this thread are complete once this arrives
            mma_commit(&drain_bar);
        }
    } else if (is_epi) {
        const int co = threadIdx.x;
        const float bias = (a.bias && co < a.cout) ? __bfloat162float(a.bias[co]) : 0.0f;
        const uint32_t lane_addr = tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)a.tm_cols;
        // this warp's 4 KB swizzled output tiles: with two, one per half item,
        // stored by one bulk group per item; with one, one bulk group per half
        const uint32_t epi_tile = ((smem_base + (uint32_t)a.epi_off + 1023u) & ~1023u) +
                                  (uint32_t)(warp * a.epi_tma * EPI_TILE_BYTES);
        const bool one_tile = a.epi_tma == 1;
        const bool warp_rows = 32 * warp < a.cout;
        int it = 0;
        BKMA_TC_FOR_ITEMS {
            const int b = (int)(item / a.ntiles);
            const int tile = (int)(item % a.ntiles);
            const int acc = a.nacc == 2 ? (it & 1) : 0;
            const uint32_t aph = (uint32_t)(a.nacc == 2 ? (it >> 1) : it) & 1u;
            if (!mbar_wait(&accf_bar[acc], aph, &abort_flag, a.status, polls)) break;
            fence_after();
            const int64_t l0 = (int64_t)tile * TILE;
            // The tensor map ends at lt = lout rounded down to 8 positions (a
            // tensor store clips in 16-byte units); lanes store the last
            // lout - lt values of their rows themselves.
            const int64_t lt = a.lout & ~(int64_t)7;
            const bool tma_rows = a.epi_tma && warp_rows;
            // both tiles of this warp are free once the previous item's stores read them
            if (tma_rows && !one_tile) {
                if (lane == 0) asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
                __syncwarp();
            }
#pragma unroll 1
            for (int half = 0; half < 2; ++half) {
                uint32_t v[2][32];
                const uint32_t col = lane_addr + (uint32_t)(acc * TILE + 64 * half);
                tmem_ld32(col, v[0]);
                tmem_ld32(col + 32u, v[1]);
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                if (half == 1) {
                    fence_before();
                    mbar_arrive(&acce_bar[acc]);
                }
                const int64_t lh = l0 + 64 * half;
                if (lh >= a.lout || (a.epi_tma && !warp_rows)) continue;
                uint32_t pk[32];
#pragma unroll
                for (int e = 0; e < 32; ++e) {
                    const float f0 = __uint_as_float(v[e / 16][(2 * e) % 32]) + bias;
                    const float f1 = __uint_as_float(v[e / 16][(2 * e + 1) % 32]) + bias;
                    const __nv_bfloat162 h = __floats2bfloat162_rn(f0, f1);
                    pk[e] = *reinterpret_cast<const uint32_t *>(&h);
                }
                __nv_bfloat16 *dst = a.out + ((int64_t)b * a.cout + co) * a.out_stride + lh;
                if (a.epi_tma) {
                    if (lt < a.lout && lt < lh + 64 && co < a.cout) {
#pragma unroll
                        for (int e = 0; e < 64; ++e)
                            if (lh + e >= lt && lh + e < a.lout)
                                dst[e] = __ushort_as_bfloat16(
                                    (uint16_t)((pk[e / 2] >> (16 * (e & 1))) & 0xFFFFu));
                    }
                    if (lh >= lt) continue;
                    if (one_tile) {  // the tile is free once its last store read it
                        if (lane == 0) asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
                        __syncwarp();
                    }
                    const uint32_t tile_addr = epi_tile + (one_tile ? 0u : (uint32_t)half * EPI_TILE_BYTES);
                    const uint32_t row_addr = tile_addr + (uint32_t)lane * 128u;
#pragma unroll
                    for (int e = 0; e < 8; ++e)
                        asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(
                                         row_addr + ((uint32_t)(e ^ (lane & 7)) << 4)),
                                     "r"(pk[4 * e]), "r"(pk[4 * e + 1]), "r"(pk[4 * e + 2]),
                                     "r"(pk[4 * e + 3])
                                     : "memory");
                    if (one_tile) {
                        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                        __syncwarp();
                        if (lane == 0) {
                            asm volatile(
                                "cp.async.bulk.tensor.3d.global.shared::cta.bulk_group [%0, {%2, "
                                "%3, %4}], [%1];" ::"l"(reinterpret_cast<uint64_t>(&a.out_map)),
                                "r"(tile_addr), "r"((int)lh), "r"(32 * warp), "r"(b)
                                : "memory");
                            asm volatile("cp.async.bulk.commit_group;" ::: "memory");
                        }
                    }
                } else if (co < a.cout) {
                    if (lh + 64 <= a.lout && (a.out_stride % 8) == 0) {
                        uint4 *d4 = reinterpret_cast<uint4 *>(dst);
#pragma unroll
                        for (int e = 0; e < 8; ++e)
                            d4[e] = make_uint4(pk[4 * e], pk[4 * e + 1], pk[4 * e + 2], pk[4 * e + 3]);
                    } else {
#pragma unroll
                        for (int e = 0; e < 64; ++e)
                            if (lh + e < a.lout)
                                dst[e] = __ushort_as_bfloat16(
                                    (uint16_t)((pk[e / 2] >> (16 * (e & 1))) & 0xFFFFu));
                    }
                }
            }
            if (tma_rows && !one_tile) {
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                __syncwarp();
                if (lane == 0) {
                    for (int half = 0; half < 2; ++half) {
                        const int64_t lh = l0 + 64 * half;
                        if (lh >= lt) break;
                        asm volatile(
                            "cp.async.bulk.tensor.3d.global.shared::cta.bulk_group [%0, {%2, %3, %4}], "
                            "[%1];" ::"l"(reinterpret_cast<uint64_t>(&a.out_map)),
                            "r"(epi_tile + (uint32_t)half * EPI_TILE_BYTES), "r"((int)lh),
                            "r"(32 * warp), "r"(b)
                            : "memory");
                    }
                    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
                }
            }
        }
        // every tensor store of this warp has completed before teardown
        if (lane == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
    }

#undef BKMA_TC_FOR_ITEMS

    // Drain: the MMA thread's last commit covers every MMA it issued.
    if (threadIdx.x == 32 * (NUM_EPI_WARPS + NUM_PROD_WARPS)) {
        for (uint32_t i = 0; i < kSpinLimit; ++i) {
            if (mbar_try(&drain_bar, 0)) break;
            if (i > 64) __nanosleep(256);
            if (i + 1 == kSpinLimit) atomicExch(a.status, (int)BKMA_ERR_TIMEOUT);
        }
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(TMEM_COLS));
    }
}

}  // namespace tc

namespace {
struct TcLayout {
    int taps_tmem, nacc, tm_cols, wsmem_bytes, halo_rows, chunk_rows, stage_bytes, stages;
    int epi_tma, epi_off;
    size_t smem;
};

// On-chip layout of one launch. epi_tma asks for the tensor-store epilogue:
// two tiles per warp when an item has more than 40 MMAs (stores after the
// accumulator is released: K = 7 at Cin = 128 1453 vs 1404 TFLOP/s, K = 11 at
// Cin = 96 1093 vs 965), one tile per warp below that (each half stored at
// once: K = 1/3/5 +11/13/14 %) or when two tiles leave fewer than 3
// activation stages (K = 9 at Cin = 128: 1605 vs 1222 with per-lane stores);
// none when even one tile leaves fewer than 3.
TcLayout tc_layout(const bkma_conv_desc &d, bool epi_tma = false) {
    TcLayout t;
    const int cin = (int)d.cin, K = (int)d.ksize;
    // one accumulator when that moves more weight taps into TMEM
    const int taps2 = std::min(K, 256 / (cin / 2)), taps1 = std::min(K, 384 / (cin / 2));
    t.nacc = taps1 > taps2 ? 1 : 2;
    t.tm_cols = tc::TMEM_COLS - 128 * t.nacc;
    t.taps_tmem = t.nacc == 1 ? taps1 : taps2;
    t.wsmem_bytes = (K - t.taps_tmem) * cin * 256;
    t.wsmem_bytes = (t.wsmem_bytes + 1023) / 1024 * 1024;
    t.halo_rows = std::max(8, (K - 1 + 7) / 8 * 8);
    t.chunk_rows = tc::TILE + t.halo_rows + 1;
    t.stage_bytes = ((cin / 8) * t.chunk_rows * 16 + 1023) / 1024 * 1024;
    const int avail = tc::SMEM_LIMIT - t.wsmem_bytes;
    t.stages = std::min(tc::STAGES_MAX, avail / t.stage_bytes);
    t.epi_tma = 0;
    if (epi_tma) {
        const int mmas = K * cin / 16;
        for (int tiles : {2, 1}) {
            if (tiles == 2 && mmas <= 40) continue;
            const int bytes = tc::epi_bytes(tiles);
            const int st_epi = std::min(tc::STAGES_MAX, (avail - bytes) / t.stage_bytes);
            if (avail > bytes && st_epi >= 3) {
                t.stages = st_epi;
                t.epi_tma = tiles;
                break;
            }
        }
    }
    t.epi_off = t.wsmem_bytes + t.stages * t.stage_bytes;
    t.smem = (size_t)t.epi_off + (t.epi_tma ? tc::epi_bytes(t.epi_tma) : 0);
    return t;
}

// Encode the output view (lt, cout, B), lt = L-K+1 rounded down to 8
// positions (tensor stores clip the inner dimension in 16-byte units), with
// 64 x 32 x 1 boxes and the 128-byte swizzle the epilogue writes. Needs a row
// stride that is a multiple of 16 bytes.
bool encode_out_map(CUtensorMap *map, const bkma_conv_desc &d, void *out, int64_t out_stride) {
    auto fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(tensor_map_encoder());
    const int64_t lt = (d.length - d.ksize + 1) & ~(int64_t)7;
    if (!fn || (out_stride % 8) != 0 || ((uintptr_t)out % 16) != 0 || lt < 64 || d.cout < 32)
        return false;
    const cuuint64_t dims[3] = {(cuuint64_t)lt, (cuuint64_t)d.cout, (cuuint64_t)d.batch};
    const cuuint64_t strides[2] = {(cuuint64_t)out_stride * 2, (cuuint64_t)(d.cout * out_stride * 2)};
    const cuuint32_t box[3] = {64, 32, 1};
    const cuuint32_t es[3] = {1, 1, 1};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, out, dims, strides, box, es,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
              CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

int64_t tc_items(const bkma_conv_desc &d) {
    return d.batch * ((d.length - d.ksize + 1 + tc::TILE - 1) / tc::TILE);
}

// CTAs of a launch: min(SMs, items, MAX_CTAS).
int tc_grid(int64_t items, int sms) {
    return (int)std::min<int64_t>(std::min<int64_t>(sms, items), tc::MAX_CTAS);
}

// Items per chunk: CHUNK_TILES, or more so that the chunks (slots) stay
// within MAX_SLOTS for any grid up to MAX_CTAS.
int tc_chunk(int64_t items) {
    return (int)std::max<int64_t>(tc::CHUNK_TILES,
                                  (items + tc::MAX_SLOTS - tc::MAX_CTAS - 1) /
                                      (tc::MAX_SLOTS - tc::MAX_CTAS));
}

// Halo snapshot bytes: one slot per chunk; for any grid the chunks number at
// most items / chunk + min(items, MAX_CTAS) <= MAX_SLOTS.
size_t tc_halo_bytes(const bkma_conv_desc &d, int halo_rows) {
    const int64_t items = tc_items(d);
    const int64_t slots = items / tc_chunk(items) + std::min<int64_t>(items, tc::MAX_CTAS);
    return (size_t)slots * (size_t)d.cin * (size_t)halo_rows * 2;
}

// Launch the prologue (weight images; in place, the halo snapshot) and the
// tensor kernel: data is read (in place when out == data, then halo holds
// one slot per chunk), grid = min(sms, items, MAX_CTAS).
bkma_status tc_launch(const bkma_conv_desc &d, const void *data, void *out, int64_t out_stride,
                      const void *w, const void *bias, void *halo, void *wpack, int *status,
                      int64_t ntiles, int sms, uint32_t wait_polls, cudaStream_t st) {
    TcLayout t = tc_layout(d, true);
    tc::Args a;
    memset(&a, 0, sizeof(a));
    if (t.epi_tma && !encode_out_map(&a.out_map, d, out, out_stride)) t = tc_layout(d, false);
    const int64_t items = d.batch * ntiles;
    const int chunk = tc_chunk(items);
    const int grid = tc_grid(items, sms);
    uint32_t *tm_img = (uint32_t *)wpack;
    uint32_t *sm_img = tm_img + 128 * t.tm_cols;
    {
        const int64_t words = (int64_t)128 * t.tm_cols +
                              (int64_t)(d.ksize - t.taps_tmem) * (d.cin / 8) * 128 * 4;
        const int64_t total =
            words + (halo ? tc::chunk_slots(items, grid, chunk) * d.cin * (t.halo_rows / 8) : 0);
        const int blocks = (int)std::min<int64_t>(4 * 152, (total + 255) / 256);
        tc::conv_tc_prologue<<<blocks, 256, 0, st>>>(
            (const __nv_bfloat16 *)w, (int)d.cin, (int)d.cout, (int)d.ksize, t.taps_tmem, t.tm_cols,
            tm_img, sm_img, (const __nv_bfloat16 *)data, (__nv_bfloat16 *)halo, items, grid,
            chunk, (int)ntiles, d.length, t.halo_rows);
        BKMA_CUDA_TRY(cudaGetLastError());
    }
    a.x = (const __nv_bfloat16 *)data;
    a.out = (__nv_bfloat16 *)out;
    a.w = (const __nv_bfloat16 *)w;
    a.bias = (const __nv_bfloat16 *)bias;
    a.halo = (const __nv_bfloat16 *)halo;
    a.B = (int)d.batch;
    a.cin = (int)d.cin;
    a.cout = (int)d.cout;
    a.K = (int)d.ksize;
    a.L = d.length;
    a.lout = d.length - d.ksize + 1;
    a.out_stride = out_stride;
    a.ntiles = (int)ntiles;
    a.chunk = chunk;
    a.halo_rows = t.halo_rows;
    a.chunk_rows = t.chunk_rows;
    a.stage_bytes = t.stage_bytes;
    a.stages = t.stages;
    a.taps_tmem = t.taps_tmem;
    a.nacc = t.nacc;
    a.tm_cols = t.tm_cols;
    a.wsmem_bytes = t.wsmem_bytes;
    a.epi_tma = t.epi_tma;
    a.epi_off = t.epi_off;
    a.wpack_tmem = tm_img;
    a.wpack_smem = reinterpret_cast<const uint4 *>(sm_img);
    a.status = status;
    a.spin_limit = wait_polls;
    void (*kern)(const tc::Args) = nullptr;
    const bool plan_polls = wait_polls != kWaitPolls;
#define BKMA_TC_KERN(kc) (plan_polls ? tc::conv_tc_kernel<kc, true> : tc::conv_tc_kernel<kc, false>)
    switch (a.cin / 16) {
    case 1: kern = BKMA_TC_KERN(1); break;
    case 2: kern = BKMA_TC_KERN(2); break;
    case 3: kern = BKMA_TC_KERN(3); break;
    case 4: kern = BKMA_TC_KERN(4); break;
    case 5: kern = BKMA_TC_KERN(5); break;
    case 6: kern = BKMA_TC_KERN(6); break;
    case 7: kern = BKMA_TC_KERN(7); break;
    case 8: kern = BKMA_TC_KERN(8); break;
    default: return fail(BKMA_ERR_UNSUPPORTED, "tensor path: cin must be 16..128");
    }
#undef BKMA_TC_KERN
    BKMA_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)t.smem));
    kern<<<grid, tc::THREADS, t.smem, st>>>(a);
    BKMA_CUDA_TRY(cudaGetLastError());
    return BKMA_OK;
}
}  // namespace

bkma_status conv_tc_plan_init(ConvPlanImpl &p) {
    const bkma_conv_desc &d = p.desc;
    if (d.cout > 128 || d.cin > 128)
        return fail(BKMA_ERR_UNSUPPORTED, "tensor path: cin and cout must be <= 128");
    if (d.cin % 16 != 0)
        return fail(BKMA_ERR_UNSUPPORTED, "tensor path: cin must be a multiple of 16");
    if (d.length % 8 != 0)
        return fail(BKMA_ERR_UNSUPPORTED, "tensor path: length must be a multiple of 8");
    const TcLayout t = tc_layout(d);
    if (t.stages < 2)
        return fail(BKMA_ERR_UNSUPPORTED,
                    "tensor path: ksize*cin too large for on-chip weights (TMEM + shared memory)");
    p.tensor = true;
    p.TL = tc::TILE;
    p.ntiles = (d.length - d.ksize + 1 + tc::TILE - 1) / tc::TILE;
    p.halo_width = t.halo_rows;
    p.halo_bytes = tc_halo_bytes(d, t.halo_rows);
    p.wpack_bytes = (size_t)128 * t.tm_cols * 4 + (size_t)t.wsmem_bytes;
    BKMA_CUDA_TRY(cudaMalloc(&p.d_wpack, p.wpack_bytes));
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
        sms = 148;
    p.grid = std::min(sms, tc::MAX_CTAS);
    BKMA_CUDA_TRY(cudaMalloc(&p.d_status, sizeof(int)));
    BKMA_CUDA_TRY(cudaMemset(p.d_status, 0, sizeof(int)));
    return BKMA_OK;
}

bkma_status conv_tc_run(ConvPlanImpl &p, void *data, void *out, const void *w, const void *bias,
                        cudaStream_t st) {
    const bkma_conv_desc &d = p.desc;
    const bool inplace = (out == nullptr || out == data);
    const auto misaligned = [](const void *q) { return q && ((uintptr_t)q % 16) != 0; };
    if (misaligned(data) || misaligned(out) || misaligned(w))
        return fail(BKMA_ERR_INVALID_ARG, "tensor path: data, out and weight must be 16-byte aligned");
    return tc_launch(d, data, inplace ? data : out, inplace ? d.length : d.length - d.ksize + 1, w,
                     bias, (inplace && d.ksize > 1) ? p.d_halo : nullptr, p.d_wpack,
                     (int *)p.d_status, p.ntiles, p.grid, p.wait_polls, st);
}

}  // namespace bkma

namespace bkma {

// Scratch needs of the tensor path for one in-place call: the halo snapshot
// (one slot per chunk of tiles, at most MAX_SLOTS) and the packed weights
// (bytes, each rounded to 256).
bkma_status conv_tc_scratch_need(const bkma_conv_desc &d, size_t *halo_bytes, size_t *wpack_bytes) {
    if (d.cout > 128 || d.cin > 128 || d.cin % 16 != 0 || d.length % 8 != 0)
        return fail(BKMA_ERR_UNSUPPORTED,
                    "tensor path: cin = cout <= 128, cin a multiple of 16, length a multiple of 8");
    const TcLayout t = tc_layout(d);
    if (t.stages < 2)
        return fail(BKMA_ERR_UNSUPPORTED,
                    "tensor path: ksize*cin too large for on-chip weights (TMEM + shared memory)");
    *halo_bytes = (tc_halo_bytes(d, t.halo_rows) + 255) / 256 * 256;
    *wpack_bytes = ((size_t)128 * t.tm_cols * 4 + (size_t)t.wsmem_bytes + 255) / 256 * 256;
    return BKMA_OK;
}

// In-place BF16 tensor-core conv1d with caller-provided scratch (halo
// snapshot, packed weights, status word): the same two kernels as
// conv_tc_run, launched without a plan and without allocating.
bkma_status conv_tc_run_into(const bkma_conv_desc &d, void *data, const void *w, const void *bias,
                             void *halo, void *wpack, int *status, cudaStream_t st) {
    const auto misaligned = [](const void *q) { return q && ((uintptr_t)q % 16) != 0; };
    if (misaligned(data) || misaligned(w) || misaligned(halo) || misaligned(wpack))
        return fail(BKMA_ERR_INVALID_ARG, "tensor path: data, weight and scratch must be 16-byte aligned");
    const int64_t ntiles = (d.length - d.ksize + 1 + tc::TILE - 1) / tc::TILE;
    int dev = 0, sms = 0;
    BKMA_CUDA_TRY(cudaGetDevice(&dev));
    BKMA_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    return tc_launch(d, data, data, d.length, w, bias, d.ksize > 1 ? halo : nullptr, wpack, status,
                     ntiles, sms, kWaitPolls, st);
}

}  // namespace bkma
