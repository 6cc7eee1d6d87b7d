// Multi-step fused advection: k time steps per launch for column strips that
// fit in shared memory.
//
// A CTA stages W columns x n1 rows (+ npts-1 wrap rows) of one slab, then
// runs k steps on the shared copy: each thread computes its cells of the
// next step into registers from the shared strip (the same per-cell
// arithmetic as the staged kernel, f_c + sum_k w_k (f_k - f_c), so k fused
// steps give the bits of k separate steps), the CTA waits, writes them back,
// refreshes the wrap rows and waits again; after the last step the strip goes
// back to HBM once. Lines are independent and the departure tables do not
// change with time, so nothing outside the strip is needed between steps.
// HBM traffic is 8/k (FP32) or 16/k (FP64) bytes per cell-step, so results
// are reported apart from the one-step-per-launch roofline. The reference
// runs one step per kernel (src/advection.cpp:55-59).
//
// Thread map: column c = tid % wc, rows r0, r0 + rstep, ... with
// r0 = tid / wc and rstep = blockDim / wc; at most 32 (FP32) or 16 (FP64)
// rows per thread, held in registers across the barrier.
#include "adv.cuh"
#include "adv_device.cuh"
#include "adv_plan.cuh"
#include "common.cuh"

namespace bkma {

namespace {

// cells per thread, held in registers across the barrier
template <typename T>
__host__ __device__ constexpr int fuse_rows() { return sizeof(T) == 4 ? 32 : 16; }
constexpr int kFuseThreads = 512;

template <typename T, int NT>
__global__ void __launch_bounds__(kFuseThreads) adv_fused(AdvStagedArgs<T> a, int ksteps) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *S = reinterpret_cast<T *>(smem_raw);
    TileCoord tc = tile_of(blockIdx.x, a.lines, a.n2, 1, a.W, a.ncb);
    if (a.line_list) tc.line0 = a.line_list[tc.line0];
    const int n1 = (int)a.n1;
    const int wc = tc.wc;
    const int ws = wc;  // unpadded rows, element-wise staging (any alignment)
    const int64_t line = tc.line0;
    stage_tile_elems<T>(S, a.src, a.n1, a.n2, line, 1, tc.c0, wc, ws, NT - 1,
                        slab_stride(a.n1, NT - 1, ws, (int)sizeof(T)));
    const int exc = a.exc_index[line];
    const int base = exc < 0 ? a.base[line] : 0;
    T w[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) w[k] = exc < 0 ? a.w[line * NT + k] : T(0);
    const AdvExcCell<T> *cells = exc < 0 ? nullptr : a.exc + (int64_t)exc * n1;
    const int rstep = (int)blockDim.x / wc;
    const int r0 = (int)threadIdx.x / wc;
    const int c = (int)threadIdx.x - r0 * wc;
    const bool active = r0 < rstep;
    constexpr int kFuseRows = fuse_rows<T>();
    T v[kFuseRows];
    for (int step = 0; step < ksteps; ++step) {
#pragma unroll
        for (int j = 0; j < kFuseRows; ++j) {
            const int r = r0 + j * rstep;
            if (active && r < n1) {
                int rr;
                T wk[NT];
                if (exc < 0) {
                    rr = r + base;
#pragma unroll
                    for (int k = 0; k < NT; ++k) wk[k] = w[k];
                } else {
                    const AdvExcCell<T> &e = cells[r];
                    rr = r + e.base;
#pragma unroll
                    for (int k = 0; k < NT; ++k) wk[k] = e.w[k];
                }
                if (rr >= n1) rr -= n1;
                v[j] = stencil_cell<T, NT>(S + rr * ws + c, ws, wk);
            }
        }
        __syncthreads();  // every thread has read the old strip
#pragma unroll
        for (int j = 0; j < kFuseRows; ++j) {
            const int r = r0 + j * rstep;
            if (active && r < n1) S[r * ws + c] = v[j];
        }
        __syncthreads();
        // wrap rows n1 .. n1+NT-2 repeat rows 0 .. NT-2
        for (int i = threadIdx.x; i < (NT - 1) * wc; i += blockDim.x) {
            const int hr = i / wc, hc = i - hr * wc;
            S[(n1 + hr) * ws + hc] = S[hr * ws + hc];
        }
        __syncthreads();
    }
    T *G = a.dst + line * a.n1 * a.n2 + tc.c0;
    for (int i = threadIdx.x; i < n1 * wc; i += blockDim.x) {
        const int r = i / wc, cc = i - r * wc;
        G[(int64_t)r * a.n2 + cc] = S[r * ws + cc];
    }
}

// FP32 form: two shared buffers (the step reads one and writes the other,
// one barrier per step, the periodic wrap by index arithmetic), four
// columns x kRowsF32 consecutive rows per thread with the taps in a float4
// register ring (one new row load per output row) and packed FP32x2 FMAs in
// the staged kernel's order (same bits). The odd row count puts the rows
// that the eight threads of a 16-byte shared-memory phase read on different
// banks. Lines with per-cell stencils (exception lines) load their taps per
// row.
constexpr int kRowsF32 = 9;

template <int NT>
__global__ void __launch_bounds__(kFuseThreads) adv_fused_f32(AdvStagedArgs<float> a, int ksteps) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int C = NT / 2 - 1;
    TileCoord tc = tile_of(blockIdx.x, a.lines, a.n2, 1, a.W, a.ncb);
    const int n1 = (int)a.n1;
    const int wc = tc.wc;
    const int ws = (wc + 3) & ~3;
    float *buf0 = reinterpret_cast<float *>(smem_raw);
    float *buf1 = buf0 + (size_t)n1 * ws;
    const int64_t line = tc.line0;
    stage_tile_elems<float>(buf0, a.src, a.n1, a.n2, line, 1, tc.c0, wc, ws, 0, n1 * ws);
    const int exc = a.exc_index[line];
    const int base = exc < 0 ? a.base[line] : 0;
    float2 w2[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) {
        const float wk = exc < 0 ? a.w[line * NT + k] : 0.f;
        w2[k] = make_float2(wk, wk);
    }
    const AdvExcCell<float> *cells = exc < 0 ? nullptr : a.exc + (int64_t)exc * n1;
    const float2 m1 = make_float2(-1.0f, -1.0f);
    const int G = ws >> 2;  // column groups
    const int g4 = ((int)threadIdx.x % G) * 4;
    const int r0 = ((int)threadIdx.x / G) * kRowsF32;
    const int nr = max(0, min(kRowsF32, n1 - r0));
    auto cell = [&](const float4 (&f)[NT], const float2 (&wv)[NT]) -> float4 {
        const float2 cl = make_float2(f[C].x, f[C].y);
        const float2 ch = make_float2(f[C].z, f[C].w);
        float2 al = make_float2(0.f, 0.f), ah = make_float2(0.f, 0.f);
#pragma unroll
        for (int k = 0; k < NT; ++k) {
            if (k == C) continue;
            al = __ffma2_rn(wv[k], __ffma2_rn(cl, m1, make_float2(f[k].x, f[k].y)), al);
            ah = __ffma2_rn(wv[k], __ffma2_rn(ch, m1, make_float2(f[k].z, f[k].w)), ah);
        }
        const float2 ol = __fadd2_rn(cl, al), oh = __fadd2_rn(ch, ah);
        return make_float4(ol.x, ol.y, oh.x, oh.y);
    };
    float *in = buf0, *out = buf1;
    for (int step = 0; step < ksteps; ++step) {
        if (nr > 0 && exc < 0) {
            int q0 = r0 + base;
            if (q0 >= n1) q0 -= n1;
            auto row = [&](int i) -> float4 {
                int q = q0 + i;
                if (q >= n1) q -= n1;
                return *reinterpret_cast<const float4 *>(in + q * ws + g4);
            };
            float4 ring[NT];
#pragma unroll
            for (int i = 0; i < NT - 1; ++i) ring[i] = row(i);
#pragma unroll
            for (int i = 0; i < kRowsF32; ++i) {
                ring[(i + NT - 1) % NT] = row(i + NT - 1);
                if (i < nr) {
                    float4 f[NT];
#pragma unroll
                    for (int k = 0; k < NT; ++k) f[k] = ring[(i + k) % NT];
                    *reinterpret_cast<float4 *>(out + (r0 + i) * ws + g4) = cell(f, w2);
                }
            }
        } else if (nr > 0) {
            for (int i = 0; i < nr; ++i) {
                const AdvExcCell<float> &e = cells[r0 + i];
                int q = r0 + i + e.base;
                if (q >= n1) q -= n1;
                float4 f[NT];
                float2 wv[NT];
#pragma unroll
                for (int k = 0; k < NT; ++k) {
                    int qk = q + k;
                    if (qk >= n1) qk -= n1;
                    f[k] = *reinterpret_cast<const float4 *>(in + qk * ws + g4);
                    wv[k] = make_float2(e.w[k], e.w[k]);
                }
                *reinterpret_cast<float4 *>(out + (r0 + i) * ws + g4) = cell(f, wv);
            }
        }
        __syncthreads();
        float *t = in;
        in = out;
        out = t;
    }
    float *Gp = a.dst + line * a.n1 * a.n2 + tc.c0;
    for (int i = threadIdx.x; i < n1 * wc; i += blockDim.x) {
        const int r = i / wc, cc = i - r * wc;
        Gp[(int64_t)r * a.n2 + cc] = in[r * ws + cc];
    }
}

// Extended-precision fused steps: the on-chip state of a cell is the
// unevaluated sum hi + lo of two FP32 numbers (|lo| <= half an ulp of hi);
// HBM still holds FP32 (hi is staged with lo = 0, and hi = RN(hi + lo) is
// written back). Per cell and step, in packed FP32x2:
//   s_h = sum_{k != c} w_k (hi_k - hi_c)   (the staged kernel's fma order),
//   s_l = sum_{k != c} w_k lo_k + (w_c - 1) lo_c  (= sum w_k (lo_k - lo_c),
//         since the weights sum to one; its rounding is far below lo),
//   t = lo_c + (s_h + s_l),  (hi', lo') = Fast2Sum(hi_c, t):
//   hi' = RN(hi_c + t), lo' = t - (hi' - hi_c). It is exact when
//   |hi_c| >= |t| (every cell but those where the field passes near zero
//   and the step's increment t exceeds it; there lo' misses by O(2^-24 |t|),
//   |t| being one step's change of the cell). Measured against TwoSum on the
//   2048x1024x512 field over 50 steps: outputs differ by at most one FP32
//   ulp, and the Fast2Sum form runs 8 % faster.
// With lo = 0 this is the FP32 kernel's arithmetic bit for bit (s_l = +0,
// t = s_h, hi' = RN(hi_c + s_h)), so one step per launch gives the same
// bits; over k steps the field is rounded to FP32 once instead of k times. Thread map: W = 4 columns (one float4 group), R
// consecutive rows per thread, hi and lo register rings.
template <int NT, int R>
__global__ void __launch_bounds__(kFuseThreads) adv_fused_f32x2(AdvStagedArgs<float> a, int ksteps) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int C = NT / 2 - 1;
    TileCoord tc = tile_of(blockIdx.x, a.lines, a.n2, 1, a.W, a.ncb);
    const int n1 = (int)a.n1;
    const int wc = tc.wc;
    constexpr int ws = 4;
    float *hi_in = reinterpret_cast<float *>(smem_raw);
    float *lo_in = hi_in + (size_t)n1 * ws;
    float *hi_out = lo_in + (size_t)n1 * ws;
    float *lo_out = hi_out + (size_t)n1 * ws;
    const int64_t line = tc.line0;
    stage_tile_elems<float>(hi_in, a.src, a.n1, a.n2, line, 1, tc.c0, wc, ws, 0, n1 * ws);
    for (int i = threadIdx.x; i < n1 * ws; i += blockDim.x) lo_in[i] = 0.f;
    __syncthreads();
    const int exc = a.exc_index[line];
    const int base = exc < 0 ? a.base[line] : 0;
    float2 w2[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) {
        const float wk = exc < 0 ? a.w[line * NT + k] : 0.f;
        w2[k] = make_float2(wk, wk);
    }
    const AdvExcCell<float> *cells = exc < 0 ? nullptr : a.exc + (int64_t)exc * n1;
    const float2 m1 = make_float2(-1.0f, -1.0f);
    const int r0 = (int)threadIdx.x * R;
    const int nr = max(0, min(R, n1 - r0));
    // one cell pair (columns 2j, 2j+1 of the group): returns (hi', lo')
    auto pair = [&](const float4 (&h)[NT], const float4 (&l)[NT], const float2 (&wv)[NT], bool upper,
                    float2 &oh, float2 &ol) {
        const float2 hc = upper ? make_float2(h[C].z, h[C].w) : make_float2(h[C].x, h[C].y);
        const float2 lc = upper ? make_float2(l[C].z, l[C].w) : make_float2(l[C].x, l[C].y);
        float2 acc = make_float2(0.f, 0.f), accl = make_float2(0.f, 0.f);
#pragma unroll
        for (int k = 0; k < NT; ++k) {
            const float2 lk = upper ? make_float2(l[k].z, l[k].w) : make_float2(l[k].x, l[k].y);
            if (k == C) {
                accl = __ffma2_rn(make_float2(wv[k].x - 1.0f, wv[k].y - 1.0f), lk, accl);
                continue;
            }
            const float2 hk = upper ? make_float2(h[k].z, h[k].w) : make_float2(h[k].x, h[k].y);
            acc = __ffma2_rn(wv[k], __ffma2_rn(hc, m1, hk), acc);
            accl = __ffma2_rn(wv[k], lk, accl);
        }
        acc = __fadd2_rn(acc, accl);
        const float2 t = __fadd2_rn(lc, acc);
        const float2 sum = __fadd2_rn(hc, t);
        const float2 bb = __ffma2_rn(hc, m1, sum);  // sum - hc
        oh = sum;
        ol = __ffma2_rn(bb, m1, t);                 // t - (sum - hc)
    };
    auto cell4 = [&](const float4 (&h)[NT], const float4 (&l)[NT], const float2 (&wv)[NT], float *dh,
                     float *dl) {
        float2 h0, l0, h1, l1;
        pair(h, l, wv, false, h0, l0);
        pair(h, l, wv, true, h1, l1);
        *reinterpret_cast<float4 *>(dh) = make_float4(h0.x, h0.y, h1.x, h1.y);
        *reinterpret_cast<float4 *>(dl) = make_float4(l0.x, l0.y, l1.x, l1.y);
    };
    for (int step = 0; step < ksteps; ++step) {
        if (nr > 0 && exc < 0) {
            int q0 = r0 + base;
            if (q0 >= n1) q0 -= n1;
            auto row = [&](const float *b, int i) -> float4 {
                int q = q0 + i;
                if (q >= n1) q -= n1;
                return *reinterpret_cast<const float4 *>(b + q * ws);
            };
            float4 rh[NT], rl[NT];
#pragma unroll
            for (int i = 0; i < NT - 1; ++i) {
                rh[i] = row(hi_in, i);
                rl[i] = row(lo_in, i);
            }
#pragma unroll
            for (int i = 0; i < R; ++i) {
                rh[(i + NT - 1) % NT] = row(hi_in, i + NT - 1);
                rl[(i + NT - 1) % NT] = row(lo_in, i + NT - 1);
                if (i < nr) {
                    float4 h[NT], l[NT];
#pragma unroll
                    for (int k = 0; k < NT; ++k) {
                        h[k] = rh[(i + k) % NT];
                        l[k] = rl[(i + k) % NT];
                    }
                    cell4(h, l, w2, hi_out + (r0 + i) * ws, lo_out + (r0 + i) * ws);
                }
            }
        } else if (nr > 0) {
            for (int i = 0; i < nr; ++i) {
                const AdvExcCell<float> &e = cells[r0 + i];
                int q = r0 + i + e.base;
                if (q >= n1) q -= n1;
                float4 h[NT], l[NT];
                float2 wv[NT];
#pragma unroll
                for (int k = 0; k < NT; ++k) {
                    int qk = q + k;
                    if (qk >= n1) qk -= n1;
                    h[k] = *reinterpret_cast<const float4 *>(hi_in + qk * ws);
                    l[k] = *reinterpret_cast<const float4 *>(lo_in + qk * ws);
                    wv[k] = make_float2(e.w[k], e.w[k]);
                }
                cell4(h, l, wv, hi_out + (r0 + i) * ws, lo_out + (r0 + i) * ws);
            }
        }
        __syncthreads();
        float *t = hi_in;
        hi_in = hi_out;
        hi_out = t;
        t = lo_in;
        lo_in = lo_out;
        lo_out = t;
    }
    float *Gp = a.dst + line * a.n1 * a.n2 + tc.c0;
    for (int i = threadIdx.x; i < n1 * wc; i += blockDim.x) {
        const int r = i / wc, cc = i - r * wc;
        Gp[(int64_t)r * a.n2 + cc] = hi_in[r * ws + cc];
    }
}

// Rows per thread of the extended kernel: the fewest of 3, 5, 9 that cover n1
// with 512 threads (0: n1 too long).
int fused_x2_rows(int64_t n1) {
    for (int r : {3, 5, 9})
        if ((int64_t)kFuseThreads * r >= n1) return r;
    return 0;
}

int fused_f32_w(const AdvPlanImpl &p, size_t max_smem) {
    // 8-column strips (three CTAs per SM for n1 = 1024); narrower for longer
    // lines, so that rowblocks x kRowsF32 covers n1
    for (int w : {8, 4}) {
        const int ws = w;
        const int rowblocks = kFuseThreads / (ws / 4);
        const size_t smem = 2 * (size_t)p.desc.n1 * ws * sizeof(float);
        if ((int64_t)rowblocks * kRowsF32 >= p.desc.n1 && smem <= max_smem) return w;
    }
    return 0;
}

template <int NT>
cudaError_t launch_fused_f32(const AdvPlanImpl &p, const void *src, void *dst, int W, int ksteps,
                             cudaStream_t st) {
    AdvStagedArgs<float> a{};
    a.src = (const float *)src;
    a.dst = (float *)dst;
    a.n1 = p.desc.n1;
    a.n2 = p.desc.n2;
    a.lines = p.lines;
    a.W = W;
    a.R = 1;
    a.ncb = p.ncb(W);
    a.base = p.d_base;
    a.w = (const float *)p.d_w;
    a.exc_index = p.d_exc_index;
    a.exc = (const AdvExcCell<float> *)p.d_exc;
    a.line_list = nullptr;
    const size_t smem = 2 * (size_t)p.desc.n1 * ((W + 3) & ~3) * sizeof(float);
    auto kern = adv_fused_f32<NT>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    // threads = column groups x row blocks rounded to warps (256 instead of
    // 512 for n1 = 1024: 1329 -> 1450 G cell-steps/s at k = 10)
    const int G = ((W + 3) & ~3) / 4;
    const int thr = (int)std::min<int64_t>(
        kFuseThreads, (G * ((p.desc.n1 + kRowsF32 - 1) / kRowsF32) + 31) / 32 * 32);
    kern<<<grid_x(p.tiles(W, 1)), thr, smem, st>>>(a, ksteps);
    return cudaGetLastError();
}

template <int NT, int R>
cudaError_t launch_fused_x2(const AdvPlanImpl &p, const void *src, void *dst, int ksteps,
                            cudaStream_t st) {
    AdvStagedArgs<float> a{};
    a.src = (const float *)src;
    a.dst = (float *)dst;
    a.n1 = p.desc.n1;
    a.n2 = p.desc.n2;
    a.lines = p.lines;
    a.W = 4;
    a.R = 1;
    a.ncb = p.ncb(4);
    a.base = p.d_base;
    a.w = (const float *)p.d_w;
    a.exc_index = p.d_exc_index;
    a.exc = (const AdvExcCell<float> *)p.d_exc;
    a.line_list = nullptr;
    const size_t smem = adv_fused_x2_smem(p);
    auto kern = adv_fused_f32x2<NT, R>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    // threads = rows / R rounded to warps (352 for n1 = 1024): two CTAs per
    // SM at 74 registers instead of one 512-thread CTA with 170 idle
    // threads (766 -> 982 G cell-steps/s on 2048 x 1024 x 512, 50 steps)
    const int thr = (int)std::min<int64_t>(kFuseThreads, ((p.desc.n1 + R - 1) / R + 31) / 32 * 32);
    kern<<<grid_x(p.tiles(4, 1)), thr, smem, st>>>(a, ksteps);
    return cudaGetLastError();
}

template <typename T, int NT>
cudaError_t launch_fused_t(const AdvPlanImpl &p, const void *src, void *dst, int W, int ksteps,
                           cudaStream_t st) {
    AdvStagedArgs<T> a{};
    a.src = (const T *)src;
    a.dst = (T *)dst;
    a.n1 = p.desc.n1;
    a.n2 = p.desc.n2;
    a.lines = p.lines;
    a.W = W;
    a.R = 1;
    a.ncb = p.ncb(W);
    a.base = p.d_base;
    a.w = (const T *)p.d_w;
    a.exc_index = p.d_exc_index;
    a.exc = (const AdvExcCell<T> *)p.d_exc;
    a.line_list = nullptr;
    const size_t smem =
        (size_t)slab_stride(p.desc.n1, p.npts - 1, W, p.esize) * (size_t)p.esize;
    auto kern = adv_fused<T, NT>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<grid_x(p.tiles(W, 1)), kFuseThreads, smem, st>>>(a, ksteps);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_fused_npts(const AdvPlanImpl &p, const void *src, void *dst, int W, int k,
                              cudaStream_t st) {
    switch (p.npts) {
    case 4: return launch_fused_t<T, 4>(p, src, dst, W, k, st);
    case 6: return launch_fused_t<T, 6>(p, src, dst, W, k, st);
    case 10: return launch_fused_t<T, 10>(p, src, dst, W, k, st);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace

bool adv_fused_f32_fast(const AdvPlanImpl &p, size_t max_smem) {
    return fused_f32_w(p, max_smem) != 0;
}

size_t adv_fused_x2_smem(const AdvPlanImpl &p) {
    return 4 * (size_t)p.desc.n1 * 4 * sizeof(float);
}

int adv_fused_tile_w(const AdvPlanImpl &p, size_t max_smem) {
    if (p.fuse_x2) return adv_fused_x2_smem(p) <= max_smem && fused_x2_rows(p.desc.n1) ? 4 : 0;
    if (p.desc.dtype == BKMA_F32) {
        const int w = fused_f32_w(p, max_smem);
        if (w) return w;
    }
    // widest strip with at most fuse_rows rows per thread that fits
    for (int w : {16, 8, 4, 2, 1}) {
        if (w > p.desc.n2 && w != 1) continue;
        const int rstep = kFuseThreads / w;
        const size_t smem =
            (size_t)slab_stride(p.desc.n1, p.npts - 1, w, p.esize) * (size_t)p.esize;
        const int rows = p.esize == 4 ? fuse_rows<float>() : fuse_rows<double>();
        if ((p.desc.n1 + rstep - 1) / rstep <= rows && smem <= max_smem) return w;
    }
    return 0;
}

cudaError_t adv_fused_launch(const AdvPlanImpl &p, const void *src, void *dst, int W, int k,
                             cudaStream_t st) {
    if (p.fuse_x2) {
        if (W != 4) return cudaErrorInvalidValue;
        switch (p.npts * 16 + fused_x2_rows(p.desc.n1)) {
        case 4 * 16 + 3: return launch_fused_x2<4, 3>(p, src, dst, k, st);
        case 4 * 16 + 5: return launch_fused_x2<4, 5>(p, src, dst, k, st);
        case 4 * 16 + 9: return launch_fused_x2<4, 9>(p, src, dst, k, st);
        case 6 * 16 + 3: return launch_fused_x2<6, 3>(p, src, dst, k, st);
        case 6 * 16 + 5: return launch_fused_x2<6, 5>(p, src, dst, k, st);
        case 6 * 16 + 9: return launch_fused_x2<6, 9>(p, src, dst, k, st);
        case 10 * 16 + 3: return launch_fused_x2<10, 3>(p, src, dst, k, st);
        case 10 * 16 + 5: return launch_fused_x2<10, 5>(p, src, dst, k, st);
        case 10 * 16 + 9: return launch_fused_x2<10, 9>(p, src, dst, k, st);
        default: return cudaErrorInvalidValue;
        }
    }
    if (p.desc.dtype == BKMA_F32) {
        if (W == fused_f32_w(p, (size_t)227 * 1024)) {
            switch (p.npts) {
            case 4: return launch_fused_f32<4>(p, src, dst, W, k, st);
            case 6: return launch_fused_f32<6>(p, src, dst, W, k, st);
            case 10: return launch_fused_f32<10>(p, src, dst, W, k, st);
            default: return cudaErrorInvalidValue;
            }
        }
        return launch_fused_npts<float>(p, src, dst, W, k, st);
    }
    return launch_fused_npts<double>(p, src, dst, W, k, st);
}

}  // namespace bkma
