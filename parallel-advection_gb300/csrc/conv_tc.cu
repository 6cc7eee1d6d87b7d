// BF16 tensor-core conv1d (torch semantics) on sm_103a: a persistent implicit
// GEMM with tcgen05.mma, FP32 accumulation in TMEM.
//
// Per row b the convolution is D[co, l] = sum_k W_k[co, :] . X[:, l + k]
// (W_k = weight[:, :, k]). GEMM view per tap: M = Cout (<= 128, zero-padded
// rows), N = output positions, K = Cin.
//
//  * A (weights) lives in TMEM for the whole kernel: lane m = output channel,
//    column (k*Cin + ci)/2 holds the BF16 pair (ci, ci+1) of tap k. One MMA
//    reads only B from shared memory.
//  * B (activations) is staged K-major without swizzle: 16-byte rows of 8
//    input channels, one row per position l, rows contiguous (SBO = 128 B),
//    ci-chunks at a padded stride (LBO). Tap k is then the same staging
//    buffer with the descriptor start moved by k rows (16*k bytes): the
//    implicit im2col costs nothing.
//  * Producer warps load the tile from HBM with 16-byte loads along l,
//    transpose 8x8 BF16 blocks in registers, and store conflict-free (the
//    odd row count of a chunk spreads the 8 stores of a phase over all
//    banks). Rows past the tile come from the halo snapshot (conv.cu), so
//    tiles of one row can be overwritten in place concurrently.
//  * One thread issues the MMAs (N = 32 per instruction, 4 sub-tiles per
//    128-position stage) into two alternating TMEM accumulators; four
//    epilogue warps drain one accumulator (tcgen05.ld) while the other fills,
//    add the bias, round to BF16 and store.
//  * Every mbarrier wait is bounded; on timeout the CTA raises a status word,
//    stops, drains its MMAs with a bounded wait and frees TMEM.
#include <cuda_bf16.h>

#include <algorithm>

#include "conv.cuh"

namespace bkma {
namespace tc {

constexpr int TILE = 128;          // output positions per stage
constexpr int NSUB = 32;           // positions per MMA (N)
constexpr int SUBS = TILE / NSUB;  // sub-tiles per stage
constexpr int STAGES = 4;
constexpr int ACC_COLS = 2 * NSUB;  // two accumulators
constexpr int TMEM_COLS = 512;
constexpr int W_COLS_MAX = TMEM_COLS - ACC_COLS;  // 448: K*Cin <= 896
constexpr int NUM_EPI_WARPS = 4;
constexpr int NUM_PROD_WARPS = 4;
constexpr int THREADS = 32 * (NUM_EPI_WARPS + NUM_PROD_WARPS + 1);
constexpr uint32_t kSpinLimit = 1u << 22;  // x ~ 0.25 us backoff: ~1 s

struct Args {
    const __nv_bfloat16 *x;   // (B, Cin, L)
    __nv_bfloat16 *out;       // (B, Cout, out_stride)
    const __nv_bfloat16 *w;   // (Cout, Cin, K)
    const __nv_bfloat16 *bias;  // (Cout) or null
    const __nv_bfloat16 *halo;  // [B][ntiles][Cin][K-1] or null
    int B, cin, cout, K;
    int64_t L, lout, out_stride;
    int ntiles;
    int halo_rows;   // rows after the tile: round_up(K-1, 8)
    int chunk_rows;  // TILE + halo_rows + 1 (odd, spreads banks)
    int stage_bytes;
    int *status;     // device status word (0 ok, 4 timeout)
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
// Bounded wait. Returns false (and raises the CTA abort flag) on timeout, or
// when another thread already aborted.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, volatile int *abort_flag,
                                          int *status) {
    for (uint32_t i = 0; i < kSpinLimit; ++i) {
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

// Shared-memory matrix descriptor: K-major, no swizzle.
__device__ __forceinline__ uint64_t desc_kmajor_noswizzle(uint32_t addr, uint32_t lbo,
                                                          uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((addr & 0x3FFFF) >> 4);
    d |= (uint64_t)((lbo & 0x3FFFF) >> 4) << 16;
    d |= (uint64_t)((sbo & 0x3FFFF) >> 4) << 32;
    d |= (uint64_t)1 << 46;  // descriptor version for tcgen05
    return d;                // base offset 0, swizzle mode 0 (none)
}

// Instruction descriptor: kind::f16, BF16 A and B, FP32 D, both K-major.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
           ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_ts(uint32_t d_tmem, uint32_t a_tmem, uint64_t b_desc,
                                       uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n}" ::"r"(d_tmem),
        "r"(a_tmem), "l"(b_desc), "r"(idesc), "r"(accumulate)
        : "memory");
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
// (row j = ci 8c+j, 8 positions).
__device__ __forceinline__ void load_block(const Args &a, int b, int tile, int c, int q,
                                           uint4 (&v)[8]) {
    const int64_t l0 = (int64_t)tile * TILE;
    const int r0 = 8 * q;
    const int64_t col = l0 + r0;
    const bool from_halo = a.halo != nullptr && r0 >= TILE;
    if (!from_halo && col + 8 <= a.L && (a.L % 8) == 0) {
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int64_t ci = 8 * c + j;
            v[j] = *reinterpret_cast<const uint4 *>(a.x + ((int64_t)b * a.cin + ci) * a.L + col);
        }
        return;
    }
    // ragged end or halo rows: element-wise
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const int64_t ci = 8 * c + j;
        uint32_t wv[4];
#pragma unroll
        for (int e2 = 0; e2 < 4; ++e2) {
            uint32_t pair = 0;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int r = r0 + 2 * e2 + h;
                const int64_t l = l0 + r;
                uint32_t bits = 0;
                if (from_halo) {
                    const int hk = r - TILE;
                    if (hk < a.K - 1)
                        bits = bf16_bits(a.halo[(((int64_t)b * a.ntiles + tile) * a.cin + ci) *
                                                    (a.K - 1) + hk]);
                } else if (l < a.L) {
                    bits = bf16_bits(a.x[((int64_t)b * a.cin + ci) * a.L + l]);
                }
                pair |= bits << (16 * h);
            }
            wv[e2] = pair;
        }
        v[j] = make_uint4(wv[0], wv[1], wv[2], wv[3]);
    }
}

template <int KC>  // K16 steps per tap: Cin / 16
__global__ void __launch_bounds__(THREADS, 1) conv_tc_kernel(Args a) {
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ __align__(8) uint64_t full_bar[STAGES], empty_bar[STAGES];
    __shared__ __align__(8) uint64_t accf_bar[2], acce_bar[2];
    __shared__ __align__(8) uint64_t drain_bar;
    __shared__ uint32_t tmem_base_sh;
    __shared__ volatile int abort_flag;

    const int warp = threadIdx.x / 32;
    const int lane = threadIdx.x % 32;
    const bool is_epi = warp < NUM_EPI_WARPS;
    const bool is_prod = warp >= NUM_EPI_WARPS && warp < NUM_EPI_WARPS + NUM_PROD_WARPS;
    const bool is_mma = warp == NUM_EPI_WARPS + NUM_PROD_WARPS;

    if (threadIdx.x == 0) {
        abort_flag = 0;
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(&full_bar[s], 32 * NUM_PROD_WARPS);
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
    const int wcols = a.K * a.cin / 2;   // TMEM columns of A
    const uint32_t acc_col0 = (uint32_t)W_COLS_MAX;

    // ---- weights -> TMEM (epilogue warps: thread = output channel lane)
    if (is_epi) {
        const int co = threadIdx.x;  // 0..127
        const uint32_t lane_addr = tmem + ((uint32_t)(32 * warp) << 16);
        for (int c0 = 0; c0 < wcols; c0 += 32) {
            uint32_t v[32];
#pragma unroll
            for (int j = 0; j < 32; ++j) {
                const int col = c0 + j;
                uint32_t pair = 0;
                if (col < wcols && co < a.cout) {
                    const int k = (2 * col) / a.cin;
                    const int ci = (2 * col) % a.cin;
                    const __nv_bfloat16 *wr = a.w + (int64_t)co * a.cin * a.K;
                    pair = bf16_bits(wr[(int64_t)ci * a.K + k]) |
                           (bf16_bits(wr[(int64_t)(ci + 1) * a.K + k]) << 16);
                }
                v[j] = pair;
            }
            tmem_st32(lane_addr + (uint32_t)c0, v);
        }
        asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();

    const int64_t items = (int64_t)a.B * a.ntiles;
    const uint32_t smem_base = smem_u32(smem);

    if (is_prod) {
        const int pt = threadIdx.x - 32 * NUM_EPI_WARPS;  // 0..127
        const int nchunks = a.cin / 8;
        const int qblocks = (TILE + a.halo_rows) / 8;
        const int pairs = nchunks * qblocks;
        int it = 0;
        for (int64_t item = blockIdx.x; item < items; item += gridDim.x, ++it) {
            const int s = it % STAGES;
            const uint32_t ph = (uint32_t)(it / STAGES) & 1u;
            if (!mbar_wait(&empty_bar[s], ph ^ 1u, &abort_flag, a.status)) break;
            const int b = (int)(item / a.ntiles);
            const int tile = (int)(item % a.ntiles);
            unsigned char *stage = smem + (size_t)s * a.stage_bytes;
            constexpr int PT = 32 * NUM_PROD_WARPS;
            for (int p = pt; p < pairs; p += 2 * PT) {
                // two 8x8 blocks in flight before either is transposed
                uint4 v[2][8];
                const bool second = p + PT < pairs;
                load_block(a, b, tile, p % nchunks, p / nchunks, v[0]);
                if (second) load_block(a, b, tile, (p + PT) % nchunks, (p + PT) / nchunks, v[1]);
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    if (h == 1 && !second) break;
                    const int ph2 = p + h * PT;
                    const int c = ph2 % nchunks;
                    const int q = ph2 / nchunks;
                    const uint32_t *w = reinterpret_cast<const uint32_t *>(v[h]);
                    unsigned char *dst = stage + ((size_t)c * a.chunk_rows + 8 * q) * 16;
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
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            mbar_arrive(&full_bar[s]);
        }
    } else if (is_mma) {
        if (lane == 0) {
            const uint32_t idesc = idesc_bf16(128, NSUB);
            const uint32_t lbo16 = (uint32_t)a.chunk_rows;  // LBO >> 4
            // high word: SBO = 128 B (>> 4 = 8) in bits 32-45, version 1 at bit 46
            const uint32_t desc_hi = (128u >> 4) | (1u << 14);
            const uint32_t a_step = (uint32_t)(a.cin / 2);  // TMEM columns per tap
            int it = 0;
            int n = 0;  // sub-tile counter
            for (int64_t item = blockIdx.x; item < items; item += gridDim.x, ++it) {
                const int s = it % STAGES;
                const uint32_t ph = (uint32_t)(it / STAGES) & 1u;
                if (!mbar_wait(&full_bar[s], ph, &abort_flag, a.status)) break;
                fence_after();
                const uint32_t stage_addr = smem_base + (uint32_t)(s * a.stage_bytes);
                bool ok = true;
                for (int sub = 0; sub < SUBS; ++sub, ++n) {
                    const int acc = n & 1;
                    const uint32_t aph = (uint32_t)(n >> 1) & 1u;
                    if (!mbar_wait(&acce_bar[acc], aph ^ 1u, &abort_flag, a.status)) {
                        ok = false;
                        break;
                    }
                    fence_after();
                    const uint32_t d_tmem = tmem + acc_col0 + (uint32_t)(acc * NSUB);
                    // Descriptor low word: start address >> 4 in bits 0-13
                    // (below 256 KB, so adding row / chunk offsets never
                    // carries into the LBO field in bits 16-29).
                    const uint32_t lo0 = ((stage_addr + (uint32_t)(NSUB * sub) * 16u) >> 4) |
                                         (lbo16 << 16);
                    uint32_t a_k = tmem;
                    for (int k = 0; k < a.K; ++k, a_k += a_step) {
#pragma unroll
                        for (int j = 0; j < KC; ++j) {
                            mma_ts2(d_tmem, a_k + 8u * j, lo0 + (uint32_t)k + 2u * j * lbo16, desc_hi,
                                    idesc, (k | j) != 0 ? 1u : 0u);
                        }
                    }
                    mma_commit(&accf_bar[acc]);
                }
                mma_commit(&empty_bar[s]);
                if (!ok) break;
            }
            // all MMAs issued by this thread are complete once this arrives
            mma_commit(&drain_bar);
        }
    } else if (is_epi) {
        const int co = threadIdx.x;
        const float bias = (a.bias && co < a.cout) ? __bfloat162float(a.bias[co]) : 0.0f;
        const uint32_t lane_addr = tmem + ((uint32_t)(32 * warp) << 16) + acc_col0;
        int n = 0;
        for (int64_t item = blockIdx.x; item < items; item += gridDim.x) {
            const int b = (int)(item / a.ntiles);
            const int tile = (int)(item % a.ntiles);
            bool ok = true;
            for (int sub = 0; sub < SUBS; ++sub, ++n) {
                const int acc = n & 1;
                const uint32_t aph = (uint32_t)(n >> 1) & 1u;
                if (!mbar_wait(&accf_bar[acc], aph, &abort_flag, a.status)) {
                    ok = false;
                    break;
                }
                fence_after();
                uint32_t v[32];
                tmem_ld32(lane_addr + (uint32_t)(acc * NSUB), v);
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                fence_before();
                mbar_arrive(&acce_bar[acc]);
                if (co < a.cout) {
                    const int64_t l0 = (int64_t)tile * TILE + NSUB * sub;
                    __nv_bfloat16 *dst = a.out + ((int64_t)b * a.cout + co) * a.out_stride + l0;
                    uint32_t pk[16];
#pragma unroll
                    for (int e = 0; e < 16; ++e) {
                        const float f0 = __uint_as_float(v[2 * e]) + bias;
                        const float f1 = __uint_as_float(v[2 * e + 1]) + bias;
                        const __nv_bfloat162 h = __floats2bfloat162_rn(f0, f1);
                        pk[e] = *reinterpret_cast<const uint32_t *>(&h);
                    }
                    const bool full = (l0 + NSUB <= a.lout) && ((a.out_stride % 8) == 0);
                    if (full) {
                        uint4 *d4 = reinterpret_cast<uint4 *>(dst);
#pragma unroll
                        for (int e = 0; e < 4; ++e)
                            d4[e] = make_uint4(pk[4 * e], pk[4 * e + 1], pk[4 * e + 2], pk[4 * e + 3]);
                    } else {
                        for (int e = 0; e < NSUB; ++e) {
                            if (l0 + e < a.lout) {
                                const uint16_t bits =
                                    (uint16_t)((pk[e / 2] >> (16 * (e & 1))) & 0xFFFFu);
                                dst[e] = __ushort_as_bfloat16(bits);
                            }
                        }
                    }
                }
            }
            if (!ok) break;
        }
    }

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

bkma_status conv_tc_plan_init(ConvPlanImpl &p) {
    const bkma_conv_desc &d = p.desc;
    if (d.cout > 128 || d.cin > 128)
        return fail(BKMA_ERR_UNSUPPORTED, "tensor path: cin and cout must be <= 128");
    if (d.cin % 16 != 0)
        return fail(BKMA_ERR_UNSUPPORTED, "tensor path: cin must be a multiple of 16");
    if (d.ksize * d.cin > 2 * tc::W_COLS_MAX)
        return fail(BKMA_ERR_UNSUPPORTED, "tensor path: ksize*cin must be <= 896 (TMEM-resident weights)");
    if (d.length % 8 != 0)
        return fail(BKMA_ERR_UNSUPPORTED, "tensor path: length must be a multiple of 8");
    p.tensor = true;
    p.TL = tc::TILE;
    p.ntiles = (d.length - d.ksize + 1 + tc::TILE - 1) / tc::TILE;
    p.halo_bytes = 2 * (size_t)(d.batch * p.ntiles * d.cin * (d.ksize - 1));
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
        sms = 148;
    p.grid = sms;
    BKMA_CUDA_TRY(cudaMalloc(&p.d_status, sizeof(int)));
    BKMA_CUDA_TRY(cudaMemset(p.d_status, 0, sizeof(int)));
    return BKMA_OK;
}

bkma_status conv_tc_run(ConvPlanImpl &p, void *data, void *out, const void *w, const void *bias,
                        cudaStream_t st) {
    const bkma_conv_desc &d = p.desc;
    const bool inplace = (out == nullptr || out == data);
    if (inplace && d.ksize > 1) {
        bkma_status s = conv_halo_prepass(p, data, st);
        if (s != BKMA_OK) return s;
    }
    const auto misaligned = [](const void *q) { return q && ((uintptr_t)q % 16) != 0; };
    if (misaligned(data) || misaligned(out) || misaligned(w))
        return fail(BKMA_ERR_INVALID_ARG, "tensor path: data, out and weight must be 16-byte aligned");
    tc::Args a;
    a.x = (const __nv_bfloat16 *)data;
    a.out = (__nv_bfloat16 *)(inplace ? data : out);
    a.w = (const __nv_bfloat16 *)w;
    a.bias = (const __nv_bfloat16 *)bias;
    a.halo = (inplace && d.ksize > 1) ? (const __nv_bfloat16 *)p.d_halo : nullptr;
    a.B = (int)d.batch;
    a.cin = (int)d.cin;
    a.cout = (int)d.cout;
    a.K = (int)d.ksize;
    a.L = d.length;
    a.lout = d.length - d.ksize + 1;
    a.out_stride = inplace ? d.length : a.lout;
    a.ntiles = (int)p.ntiles;
    a.halo_rows = (int)((d.ksize - 1 + 7) / 8 * 8);
    if (a.halo_rows == 0) a.halo_rows = 8;
    a.chunk_rows = tc::TILE + a.halo_rows + 1;
    a.stage_bytes = (a.cin / 8) * a.chunk_rows * 16;
    a.stage_bytes = (a.stage_bytes + 1023) / 1024 * 1024;
    a.status = (int *)p.d_status;
    const size_t smem = (size_t)tc::STAGES * a.stage_bytes;
    if (smem > 220 * 1024) return fail(BKMA_ERR_UNSUPPORTED, "tensor path: stage too large for shared memory");
    void (*kern)(tc::Args) = nullptr;
    switch (a.cin / 16) {
    case 1: kern = tc::conv_tc_kernel<1>; break;
    case 2: kern = tc::conv_tc_kernel<2>; break;
    case 3: kern = tc::conv_tc_kernel<3>; break;
    case 4: kern = tc::conv_tc_kernel<4>; break;
    case 5: kern = tc::conv_tc_kernel<5>; break;
    case 6: kern = tc::conv_tc_kernel<6>; break;
    case 7: kern = tc::conv_tc_kernel<7>; break;
    case 8: kern = tc::conv_tc_kernel<8>; break;
    default: return fail(BKMA_ERR_UNSUPPORTED, "tensor path: cin must be 16..128");
    }
    BKMA_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int64_t items = (int64_t)a.B * a.ntiles;
    const int grid = (int)std::min<int64_t>(p.grid, items);
    kern<<<grid, tc::THREADS, smem, st>>>(a);
    BKMA_CUDA_TRY(cudaGetLastError());
    return BKMA_OK;
}

}  // namespace bkma
