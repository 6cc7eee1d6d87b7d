// Learned stencils: a small MLP maps the fractional shift a in [0,1) of a
// line's foot point to a correction of the Lagrange stencil of the same
// points,
//   w(a) = L(a) + c(a) - mean(c(a)),  c = W3 gelu(W2 gelu(W1 a + b1) + b2) + b3,
// so the weights still sum to one (constants are preserved). NO = 4 points
// (degree-3 Lagrange base, nodes 0..3 at 1 + a) or 6 points (degree-5 base,
// nodes 0..5 at 2 + a). Layers 1 -> 32 -> 32 -> NO, FP32, GELU (erf form).
// The output layer starts at zero, so an untrained model is exactly the
// Lagrange method of its degree.
//
// Kernels (all on the GPU): the training-set generator (random periodic
// lines of 32 Fourier modes sampled on n1 cells; the target is the degree-9
// Lagrange interpolation of 10 nodes, or the line's exact value at the
// point), a fused forward/backward over blocks of 128 samples with the
// parameter gradient reduced in shared memory, Adam with a cosine
// learning-rate schedule, and per-line inference whose output is the weight
// table of an advection plan (bkma_adv_plan_set_weights).
//
// Parameter layout (32 + 32 + 1024 + 32 + 32 NO + NO floats: 1252 for NO = 4,
// 1318 for NO = 6): W1[32] b1[32] W2[32][32] b2[32] W3[NO][32] b3[NO].
#include <cmath>
#include <memory>
#include <vector>

#include "common.cuh"

namespace bkma {
namespace mlp {

constexpr int OW1 = 0, OB1 = 32, OW2 = 64, OB2 = 1088, OW3 = 1120;
template <int NO> __host__ __device__ constexpr int ob3() { return OW3 + 32 * NO; }
template <int NO> __host__ __device__ constexpr int nparams() { return ob3<NO>() + NO; }
constexpr int MODES = 32;
constexpr int PER_SAMPLE = 2 + 2 * MODES;
constexpr int TB = 128;   // samples per block in the gradient kernel
// per-sample shared-memory stride (odd: conflict-free)
template <int NO> __host__ __device__ constexpr int sstride() { return (129 + NO) | 1; }
// per-sample slots: [0] a, [1..32] z1 -> dz1, [33..64] h1, [65..96] z2 -> dz2,
// [97..128] h2, [129..129+NO) dc

__host__ __device__ __forceinline__ uint64_t splitmix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
__host__ __device__ __forceinline__ double uniform01(uint64_t seed, uint64_t idx) {
    const uint64_t h = splitmix64(seed ^ (idx * 0xD1B54A32D192ED03ull));
    return (double)(h >> 11) * (1.0 / 9007199254740992.0);
}

__device__ __forceinline__ float gelu(float x) {
    return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f));
}
__device__ __forceinline__ float gelu_grad(float x) {
    return 0.5f * (1.0f + erff(x * 0.70710678118654752f)) +
           x * expf(-0.5f * x * x) * 0.39894228040143268f;
}

// Lagrange weights on nodes 0..NO-1 at (NO/2 - 1) + a.
template <int NO>
__device__ __forceinline__ void lagrange_base(float a, float w[NO]) {
    const float x = (float)(NO / 2 - 1) + a;
#pragma unroll
    for (int j = 0; j < NO; ++j) {
        float num = 1.0f, den = 1.0f;
#pragma unroll
        for (int m = 0; m < NO; ++m) {
            if (m == j) continue;
            num *= (x - (float)m);
            den *= (float)(j - m);
        }
        w[j] = num / den;
    }
}

// ---------------------------------------------------------------- data
// Sample i: a random periodic line f(x) = sum_m a_m cos(2 pi m x) + b_m sin(2 pi m x)
// (a_m, b_m ~ U[-1,1]/m, m = 1..32) at nodes x0 + (k-4)/n1, k = 0..9, and a
// shift a; taps = the npts nodes around node 4 (from node 5 - npts/2); target
// = the degree-9 Lagrange value at 4 + a, or (exact) f(x0 + a/n1).
__global__ void samples_kernel(int64_t n, uint64_t seed, int64_t first, int64_t n1, int npts,
                               int exact, float *alpha, float *taps, float *target) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t base = (uint64_t)(first + i) * PER_SAMPLE;
        const double x0 = uniform01(seed, base);
        const double a = uniform01(seed, base + 1);
        float f[10];
#pragma unroll
        for (int k = 0; k < 10; ++k) f[k] = 0.f;
        double fx = 0.0;  // f(x0 + a/n1), exact
        const double xa = x0 + a / (double)n1;
        for (int m = 1; m <= MODES; ++m) {
            const double amd = (2.0 * uniform01(seed, base + 2 * m) - 1.0) / m;
            const double bmd = (2.0 * uniform01(seed, base + 2 * m + 1) - 1.0) / m;
            const float am = (float)amd, bm = (float)bmd;
#pragma unroll
            for (int k = 0; k < 10; ++k) {
                // phase / pi = 2 m x, reduced modulo 2 in FP64 before sinpi/cospi
                const double x = x0 + (double)(k - 4) / (double)n1;
                double ph = fmod(2.0 * m * x, 2.0);
                float s, c;
                sincospif((float)ph, &s, &c);
                f[k] += am * c + bm * s;
            }
            if (exact) {
                double s, c;
                sincospi(fmod(2.0 * m * xa, 2.0), &s, &c);
                fx += amd * c + bmd * s;
            }
        }
        double t = fx;
        if (!exact) {
            // degree-9 Lagrange target at 4 + a (FP64 weights)
            t = 0.0;
            const double px = 4.0 + a;
#pragma unroll
            for (int j = 0; j < 10; ++j) {
                double num = 1.0, den = 1.0;
                for (int m = 0; m < 10; ++m) {
                    if (m == j) continue;
                    num *= (px - m);
                    den *= (double)(j - m);
                }
                t += num / den * (double)f[j];
            }
        }
        alpha[i] = (float)a;
        const int k0 = 5 - npts / 2;
        for (int k = 0; k < npts; ++k) taps[i * npts + k] = f[k0 + k];
        target[i] = (float)t;
    }
}

// -------------------------------------------------------- forward/backward
// One sample per thread; `idx` (optional) selects samples; the batch mean of
// (pred - target)^2 is the loss. grad and loss are accumulated (zero them).
template <int NO>
__global__ void __launch_bounds__(TB) fwd_bwd_kernel(const float *__restrict__ params,
                                                     const float *__restrict__ alpha,
                                                     const float *__restrict__ taps,
                                                     const float *__restrict__ target,
                                                     int64_t n, int64_t batch, uint64_t pick_seed,
                                                     int pick, float *grad, double *loss_sum) {
    constexpr int NP = nparams<NO>();
    constexpr int OB3 = ob3<NO>();
    constexpr int SS = sstride<NO>();
    extern __shared__ float smem[];
    float *P = smem;            // NP parameters
    float *S = smem + NP + 4;   // TB x SS per-sample slots
    for (int i = threadIdx.x; i < NP; i += blockDim.x) P[i] = params[i];
    __syncthreads();
    const int64_t s_glob = (int64_t)blockIdx.x * TB + threadIdx.x;
    const bool live = s_glob < batch;
    float *Q = S + threadIdx.x * SS;
    float r = 0.f;
    if (live) {
        int64_t si = s_glob;
        if (pick) si = (int64_t)(uniform01(pick_seed, (uint64_t)s_glob) * (double)n);
        if (si >= n) si = n - 1;
        const float a = alpha[si];
        float fk[NO];
#pragma unroll
        for (int k = 0; k < NO; ++k) fk[k] = taps[si * NO + k];
        Q[0] = a;
        float h1[32];
#pragma unroll
        for (int o = 0; o < 32; ++o) {
            const float z = fmaf(P[OW1 + o], a, P[OB1 + o]);
            Q[1 + o] = z;
            h1[o] = gelu(z);
            Q[33 + o] = h1[o];
        }
        float h2[32];
        for (int o = 0; o < 32; ++o) {
            float z = P[OB2 + o];
#pragma unroll
            for (int i = 0; i < 32; ++i) z = fmaf(P[OW2 + o * 32 + i], h1[i], z);
            Q[65 + o] = z;
            h2[o] = gelu(z);
            Q[97 + o] = h2[o];
        }
        float c[NO], w[NO];
        float csum = 0.f;
#pragma unroll
        for (int o = 0; o < NO; ++o) {
            float z = P[OB3 + o];
#pragma unroll
            for (int i = 0; i < 32; ++i) z = fmaf(P[OW3 + o * 32 + i], h2[i], z);
            c[o] = z;
            csum += z;
        }
        const float cm = csum * (1.0f / NO);
        lagrange_base<NO>(a, w);
        float pred = 0.f;
#pragma unroll
        for (int k = 0; k < NO; ++k) pred = fmaf(w[k] + (c[k] - cm), fk[k], pred);
        r = pred - target[si];
        const float dpred = 2.0f * r / (float)batch;
        float dw[NO];
        float dsum = 0.f;
#pragma unroll
        for (int k = 0; k < NO; ++k) {
            dw[k] = dpred * fk[k];
            dsum += dw[k];
        }
        const float dm = dsum * (1.0f / NO);
        float dc[NO];
#pragma unroll
        for (int k = 0; k < NO; ++k) {
            dc[k] = dw[k] - dm;
            Q[129 + k] = dc[k];
        }
        // dz2 = (W3^T dc) * gelu'(z2)  (overwrites z2)
        for (int i = 0; i < 32; ++i) {
            float d = 0.f;
#pragma unroll
            for (int o = 0; o < NO; ++o) d = fmaf(P[OW3 + o * 32 + i], dc[o], d);
            Q[65 + i] = d * gelu_grad(Q[65 + i]);
        }
        // dz1 = (W2^T dz2) * gelu'(z1)  (overwrites z1)
        for (int i = 0; i < 32; ++i) {
            float d = 0.f;
            for (int o = 0; o < 32; ++o) d = fmaf(P[OW2 + o * 32 + i], Q[65 + o], d);
            Q[1 + i] = d * gelu_grad(Q[1 + i]);
        }
    } else {
        for (int j = 0; j < SS; ++j) Q[j] = 0.f;
    }
    __syncthreads();
    // parameter gradient of this block: entry e summed over the block's samples
    for (int e = threadIdx.x; e < NP; e += blockDim.x) {
        float g = 0.f;
        if (e < OB1) {
            for (int s = 0; s < TB; ++s) g = fmaf(S[s * SS + 1 + e], S[s * SS], g);
        } else if (e < OW2) {
            for (int s = 0; s < TB; ++s) g += S[s * SS + 1 + (e - OB1)];
        } else if (e < OB2) {
            const int o = (e - OW2) / 32, i = (e - OW2) % 32;
            for (int s = 0; s < TB; ++s) g = fmaf(S[s * SS + 65 + o], S[s * SS + 33 + i], g);
        } else if (e < OW3) {
            for (int s = 0; s < TB; ++s) g += S[s * SS + 65 + (e - OB2)];
        } else if (e < OB3) {
            const int o = (e - OW3) / 32, i = (e - OW3) % 32;
            for (int s = 0; s < TB; ++s) g = fmaf(S[s * SS + 129 + o], S[s * SS + 97 + i], g);
        } else {
            for (int s = 0; s < TB; ++s) g += S[s * SS + 129 + (e - OB3)];
        }
        atomicAdd(&grad[e], g);
    }
    // loss
    double rr = live ? (double)r * (double)r : 0.0;
    for (int o = 16; o > 0; o >>= 1) rr += __shfl_xor_sync(0xffffffffu, rr, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss_sum, rr);
}

__global__ void adam_kernel(float *params, float *grad, float *m, float *v, int np, float lr,
                            float b1, float b2, float eps, int t) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np) return;
    const float g = grad[i];
    const float mi = b1 * m[i] + (1.f - b1) * g;
    const float vi = b2 * v[i] + (1.f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    const float mh = mi / (1.f - powf(b1, (float)t));
    const float vh = vi / (1.f - powf(b2, (float)t));
    params[i] -= lr * mh / (sqrtf(vh) + eps);
    grad[i] = 0.f;
}

template <int NO>
__global__ void infer_kernel(const float *__restrict__ params, const float *__restrict__ alpha,
                             int64_t n, float *__restrict__ wout) {
    constexpr int NP = nparams<NO>();
    constexpr int OB3 = ob3<NO>();
    __shared__ float P[NP];
    for (int i = threadIdx.x; i < NP; i += blockDim.x) P[i] = params[i];
    __syncthreads();
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n;
         s += (int64_t)gridDim.x * blockDim.x) {
        const float a = alpha[s];
        float h1[32];
#pragma unroll
        for (int o = 0; o < 32; ++o) h1[o] = gelu(fmaf(P[OW1 + o], a, P[OB1 + o]));
        float h2[32];
        for (int o = 0; o < 32; ++o) {
            float z = P[OB2 + o];
#pragma unroll
            for (int i = 0; i < 32; ++i) z = fmaf(P[OW2 + o * 32 + i], h1[i], z);
            h2[o] = gelu(z);
        }
        float c[NO], w[NO];
        float csum = 0.f;
#pragma unroll
        for (int o = 0; o < NO; ++o) {
            float z = P[OB3 + o];
#pragma unroll
            for (int i = 0; i < 32; ++i) z = fmaf(P[OW3 + o * 32 + i], h2[i], z);
            c[o] = z;
            csum += z;
        }
        const float cm = csum * (1.0f / NO);
        lagrange_base<NO>(a, w);
#pragma unroll
        for (int k = 0; k < NO; ++k) wout[s * NO + k] = w[k] + (c[k] - cm);
    }
}

}  // namespace mlp

struct MlpImpl {
    int npts = 4;   // stencil points (4 or 6)
    int np = 0;     // parameters
    float *d_params = nullptr, *d_grad = nullptr, *d_m = nullptr, *d_v = nullptr;
    double *d_loss = nullptr;
    int step = 0;
    ~MlpImpl() {
        cudaFree(d_params);
        cudaFree(d_grad);
        cudaFree(d_m);
        cudaFree(d_v);
        cudaFree(d_loss);
    }
};

}  // namespace bkma

struct bkma_mlp {
    bkma::MlpImpl impl;
};

using namespace bkma;

namespace {
template <int NO>
constexpr size_t fwd_smem() {
    return sizeof(float) * (mlp::nparams<NO>() + 4 + (size_t)mlp::TB * mlp::sstride<NO>());
}

template <int NO>
bkma_status launch_grad_t(MlpImpl &M, const float *alpha, const float *taps, const float *target,
                          int64_t n, int64_t batch, uint64_t pick_seed, int pick, cudaStream_t st) {
    BKMA_CUDA_TRY(cudaFuncSetAttribute(mlp::fwd_bwd_kernel<NO>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)fwd_smem<NO>()));
    const int64_t blocks = (batch + mlp::TB - 1) / mlp::TB;
    mlp::fwd_bwd_kernel<NO><<<grid_x(blocks), mlp::TB, fwd_smem<NO>(), st>>>(
        M.d_params, alpha, taps, target, n, batch, pick_seed, pick, M.d_grad, M.d_loss);
    BKMA_CUDA_TRY(cudaGetLastError());
    return BKMA_OK;
}

bkma_status launch_grad(MlpImpl &M, const float *alpha, const float *taps, const float *target,
                        int64_t n, int64_t batch, uint64_t pick_seed, int pick, cudaStream_t st) {
    if (M.npts == 6) return launch_grad_t<6>(M, alpha, taps, target, n, batch, pick_seed, pick, st);
    return launch_grad_t<4>(M, alpha, taps, target, n, batch, pick_seed, pick, st);
}

bkma_status create(uint64_t seed, int npts, bkma_mlp **out) {
    BKMA_CHECK_ARG(out, "null argument");
    *out = nullptr;
    BKMA_CHECK_ARG(npts == 4 || npts == 6, "a learned stencil has 4 or 6 points");
    // owned here until complete: an early return or an exception frees it
    std::unique_ptr<bkma_mlp> m(new bkma_mlp);
    MlpImpl &M = m->impl;
    M.npts = npts;
    M.np = npts == 6 ? mlp::nparams<6>() : mlp::nparams<4>();
    // hidden layers U[-1,1]*sqrt(6/(fan_in+fan_out)) from the shared generator,
    // output layer zero
    std::vector<float> p((size_t)M.np, 0.f);
    for (int i = mlp::OW1; i < mlp::OB1; ++i)
        p[i] = (float)((2 * mlp::uniform01(seed, (uint64_t)i) - 1) * std::sqrt(6.0 / 33.0));
    for (int i = mlp::OW2; i < mlp::OB2; ++i)
        p[i] = (float)((2 * mlp::uniform01(seed, (uint64_t)i) - 1) * std::sqrt(6.0 / 64.0));
    const size_t b = sizeof(float) * (size_t)M.np;
    cudaError_t e = cudaMalloc(&M.d_params, b);
    if (e == cudaSuccess) e = cudaMalloc(&M.d_grad, b);
    if (e == cudaSuccess) e = cudaMalloc(&M.d_m, b);
    if (e == cudaSuccess) e = cudaMalloc(&M.d_v, b);
    if (e == cudaSuccess) e = cudaMalloc(&M.d_loss, sizeof(double));
    if (e == cudaSuccess) e = cudaMemcpy(M.d_params, p.data(), b, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(M.d_grad, 0, b);
    if (e == cudaSuccess) e = cudaMemset(M.d_m, 0, b);
    if (e == cudaSuccess) e = cudaMemset(M.d_v, 0, b);
    if (e != cudaSuccess) return cuda_fail(e, "bkma_mlp_create");
    *out = m.release();
    return BKMA_OK;
}

bkma_status samples(int64_t n, uint64_t seed, int64_t first, int64_t n1, int npts, int exact,
                    float *alpha, float *taps, float *target, cudaStream_t st) {
    BKMA_CHECK_ARG(n > 0 && alpha && taps && target && first >= 0, "bad arguments");
    BKMA_CHECK_ARG(n1 >= 10 && n1 < (1ll << 30), "n1 must be in [10, 2^30)");
    BKMA_CHECK_ARG(npts == 4 || npts == 6, "a learned stencil has 4 or 6 points");
    const int64_t blocks = std::min<int64_t>((n + 255) / 256, 152 * 16);
    mlp::samples_kernel<<<grid_x(blocks), 256, 0, st>>>(n, seed, first, n1, npts, exact ? 1 : 0,
                                                       alpha, taps, target);
    BKMA_CUDA_TRY(cudaGetLastError());
    return BKMA_OK;
}
}  // namespace

extern "C" {

bkma_status bkma_mlp_create(uint64_t seed, bkma_mlp **out) try {
    return create(seed, 4, out);
} BKMA_ABI_CATCH("bkma_mlp_create")

bkma_status bkma_mlp_create_stencil(uint64_t seed, int32_t npts, bkma_mlp **out) try {
    return create(seed, npts, out);
} BKMA_ABI_CATCH("bkma_mlp_create_stencil")

bkma_status bkma_mlp_info(const bkma_mlp *mlp, int32_t *npts, int32_t *nparams) try {
    BKMA_CHECK_ARG(mlp && npts && nparams, "null argument");
    *npts = mlp->impl.npts;
    *nparams = mlp->impl.np;
    return BKMA_OK;
} BKMA_ABI_CATCH("bkma_mlp_info")

bkma_status bkma_mlp_params(bkma_mlp *mlp, float *host_params, int32_t set) try {
    BKMA_CHECK_ARG(mlp && host_params, "null argument");
    const size_t b = sizeof(float) * (size_t)mlp->impl.np;
    if (set)
        BKMA_CUDA_TRY(cudaMemcpy(mlp->impl.d_params, host_params, b, cudaMemcpyHostToDevice));
    else
        BKMA_CUDA_TRY(cudaMemcpy(host_params, mlp->impl.d_params, b, cudaMemcpyDeviceToHost));
    return BKMA_OK;
} BKMA_ABI_CATCH("bkma_mlp_params")

bkma_status bkma_mlp_samples(int64_t n, uint64_t seed, int64_t first, float *alpha, float *taps4,
                             float *target, void *stream) try {
    return samples(n, seed, first, 1024, 4, 0, alpha, taps4, target, (cudaStream_t)stream);
} BKMA_ABI_CATCH("bkma_mlp_samples")

bkma_status bkma_mlp_samples_grid(int64_t n, uint64_t seed, int64_t first, int64_t n1,
                                  int32_t npts, int32_t exact, float *alpha, float *taps,
                                  float *target, void *stream) try {
    return samples(n, seed, first, n1, npts, exact, alpha, taps, target, (cudaStream_t)stream);
} BKMA_ABI_CATCH("bkma_mlp_samples_grid")

bkma_status bkma_mlp_grad(bkma_mlp *mlp, const float *alpha, const float *taps,
                          const float *target, int64_t n, float *host_grad, double *host_loss,
                          void *stream) try {
    BKMA_CHECK_ARG(mlp && alpha && taps && target && n > 0 && host_grad, "bad arguments");
    MlpImpl &M = mlp->impl;
    cudaStream_t st = (cudaStream_t)stream;
    const size_t b = sizeof(float) * (size_t)M.np;
    BKMA_CUDA_TRY(cudaMemsetAsync(M.d_grad, 0, b, st));
    BKMA_CUDA_TRY(cudaMemsetAsync(M.d_loss, 0, sizeof(double), st));
    bkma_status s = launch_grad(M, alpha, taps, target, n, n, 0, 0, st);
    if (s != BKMA_OK) return s;
    BKMA_CUDA_TRY(cudaMemcpyAsync(host_grad, M.d_grad, b, cudaMemcpyDeviceToHost, st));
    double loss = 0;
    BKMA_CUDA_TRY(cudaMemcpyAsync(&loss, M.d_loss, sizeof(double), cudaMemcpyDeviceToHost, st));
    BKMA_CUDA_TRY(cudaStreamSynchronize(st));
    BKMA_CUDA_TRY(cudaMemsetAsync(M.d_grad, 0, b, st));
    if (host_loss) *host_loss = loss / (double)n;
    return BKMA_OK;
} BKMA_ABI_CATCH("bkma_mlp_grad")

bkma_status bkma_mlp_train(bkma_mlp *mlp, const float *alpha, const float *taps,
                           const float *target, int64_t n, int32_t steps, int32_t batch,
                           float lr_max, uint64_t seed, double *host_loss, void *stream) try {
    BKMA_CHECK_ARG(mlp && alpha && taps && target && n > 0 && steps >= 0 && batch > 0 &&
                       lr_max > 0,
                   "bad arguments");
    MlpImpl &M = mlp->impl;
    cudaStream_t st = (cudaStream_t)stream;
    BKMA_CUDA_TRY(cudaMemsetAsync(M.d_grad, 0, sizeof(float) * (size_t)M.np, st));
    for (int it = 0; it < steps; ++it) {
        BKMA_CUDA_TRY(cudaMemsetAsync(M.d_loss, 0, sizeof(double), st));
        bkma_status s = launch_grad(M, alpha, taps, target, n, batch,
                                    seed ^ (0x5bd1e995ull * (uint64_t)(M.step + 1)), 1, st);
        if (s != BKMA_OK) return s;
        ++M.step;
        // cosine schedule from lr_max to 1e-5 over this call's steps
        const double kPi = 3.14159265358979323846;
        const float lr = (float)(lr_max * 0.5 * (1.0 + std::cos(kPi * (it + 1) / (double)steps)) + 1e-5);
        mlp::adam_kernel<<<(M.np + 255) / 256, 256, 0, st>>>(M.d_params, M.d_grad, M.d_m, M.d_v,
                                                             M.np, lr, 0.9f, 0.999f, 1e-8f, M.step);
        BKMA_CUDA_TRY(cudaGetLastError());
    }
    if (host_loss) {
        double l = 0;
        BKMA_CUDA_TRY(cudaMemcpyAsync(&l, M.d_loss, sizeof(double), cudaMemcpyDeviceToHost, st));
        BKMA_CUDA_TRY(cudaStreamSynchronize(st));
        *host_loss = l / (double)batch;
    }
    return BKMA_OK;
} BKMA_ABI_CATCH("bkma_mlp_train")

bkma_status bkma_mlp_infer(const bkma_mlp *mlp, const float *alpha, int64_t n, float *weights,
                           void *stream) try {
    BKMA_CHECK_ARG(mlp && alpha && weights && n > 0, "bad arguments");
    const int64_t blocks = std::min<int64_t>((n + 127) / 128, 152 * 8);
    cudaStream_t st = (cudaStream_t)stream;
    if (mlp->impl.npts == 6)
        mlp::infer_kernel<6><<<grid_x(blocks), 128, 0, st>>>(mlp->impl.d_params, alpha, n, weights);
    else
        mlp::infer_kernel<4><<<grid_x(blocks), 128, 0, st>>>(mlp->impl.d_params, alpha, n, weights);
    BKMA_CUDA_TRY(cudaGetLastError());
    return BKMA_OK;
} BKMA_ABI_CATCH("bkma_mlp_infer")

bkma_status bkma_mlp_destroy(bkma_mlp *mlp) try {
    delete mlp;
    return BKMA_OK;
} BKMA_ABI_CATCH("bkma_mlp_destroy")

}  // extern "C"
