// Shared helpers of libbkma_gb300: status/error plumbing and FP64 arithmetic
// that is never contracted into FMA (bit parity with the reference's
// operation order on host and device).
#pragma once
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <cstdint>
#include <string>

#include "bkma_gb300.h"

namespace bkma {

void set_error(const std::string &msg) noexcept;
bkma_status fail(bkma_status s, const std::string &msg) noexcept;
bkma_status cuda_fail(cudaError_t e, const char *what) noexcept;
// BKMA_ERR_HOST with the message of the C++ exception being handled (a host
// allocation that failed, a thread that could not start), prefixed by the
// entry point's name. Call only from a catch handler.
bkma_status host_fail(const char *fn) noexcept;
// The driver's cuTensorMapEncodeTiled (a PFN_cuTensorMapEncodeTiled_v12000),
// or null when the CUDA driver does not provide it.
void *tensor_map_encoder();

#define BKMA_CUDA_TRY(expr)                                   \
    do {                                                      \
        cudaError_t e__ = (expr);                             \
        if (e__ != cudaSuccess) return ::bkma::cuda_fail(e__, #expr); \
    } while (0)

#define BKMA_CHECK_ARG(cond, msg)                                            \
    do {                                                                     \
        if (!(cond)) return ::bkma::fail(BKMA_ERR_INVALID_ARG, msg);         \
    } while (0)

// A named NVTX range for the duration of an entry point: the library's calls
// show up by name on a profiler's timeline (Nsight Systems / Compute); without
// a profiler attached a push/pop costs a few nanoseconds.
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

// Polls of a bounded device-side wait before it gives up (with the kernels'
// back-off, roughly half a second to a second): plans start with this limit,
// bkma_adv_plan_set_wait_limit / bkma_conv_plan_set_wait_limit change it.
constexpr uint32_t kWaitPolls = 1u << 22;

// x dimension of a 1-D launch: 0 (a launch error, "invalid configuration")
// when the CTA count is above the 2^31 - 1 limit, never a silently truncated
// grid that would leave tiles unprocessed.
inline unsigned grid_x(int64_t ctas) {
    return ctas > 0 && ctas <= 0x7fffffff ? (unsigned)ctas : 0u;
}

// Every entry point of the C ABI is a function-try-block closed by this
// handler: no C++ exception crosses the ABI, the caller gets BKMA_ERR_HOST.
#define BKMA_ABI_CATCH(fn) \
    catch (...) {          \
        return ::bkma::host_fail(fn); \
    }

// Non-contracted FP64 operations. On the device the _rn intrinsics are never
// fused; on the host the library is compiled with -ffp-contract=off.
#ifdef __CUDA_ARCH__
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
#define BKMA_HD __host__ __device__ __forceinline__
#else
inline double dmul(double a, double b) { return a * b; }
inline double dadd(double a, double b) { return a + b; }
inline double dsub(double a, double b) { return a - b; }
#define BKMA_HD __host__ __device__ inline
#endif

// Physical parameters of one advected field, derived like
// ADVParams::update_deltas (src/config/AdvectionParams.cpp:96-103).
struct AdvPhys {
    int64_t n0, n1;
    double dt, minX, maxX, minVx, maxVx;
    double width, dx, dvx, inv_dx;
};

BKMA_HD void adv_update_deltas(AdvPhys &p) {
    p.width = dsub(p.maxX, p.minX);
    p.dx = p.width / (double)p.n1;
    p.dvx = dsub(p.maxVx, p.minVx) / (double)p.n0;
    p.inv_dx = 1 / p.dx;
}

// AdvectionSolver::coord (src/solvers/AdvectionSolver.hpp:23-26).
BKMA_HD double adv_coord(int i, double min_value, double delta) {
    return dadd(min_value, dmul((double)i, delta));
}

// AdvectionSolver::lag_basis (src/solvers/AdvectionSolver.hpp:31-51), same
// association order, no contraction.
BKMA_HD void lag_basis_ref5(double px, double c[6]) {
    const double l0 = -1. / 24, l1 = 1. / 24., l2 = -1. / 12., l3 = 1. / 12.,
                 l4 = -1. / 24., l5 = 1. / 24.;
    const double pxm2 = dsub(px, 2.);
    const double sqr = dmul(pxm2, pxm2);
    const double p01 = dmul(pxm2, dsub(pxm2, 1.));
    const double five_sqr = dmul(5., sqr);
    c[0] = dmul(dmul(dmul(dmul(l0, p01), dadd(pxm2, 1.)), dsub(pxm2, 2.)), dsub(pxm2, 1.));
    c[1] = dmul(dmul(dmul(l1, p01), dsub(pxm2, 2.)), dsub(dadd(five_sqr, pxm2), 8.));
    c[2] = dmul(dmul(dmul(dmul(l2, dsub(pxm2, 1.)), dsub(pxm2, 2.)), dadd(pxm2, 1.)),
                dsub(dsub(five_sqr, dmul(3., pxm2)), 6.));
    c[3] = dmul(dmul(dmul(dmul(l3, pxm2), dadd(pxm2, 1.)), dsub(pxm2, 2.)),
                dsub(dsub(five_sqr, dmul(7., pxm2)), 4.));
    c[4] = dmul(dmul(dmul(l4, p01), dadd(pxm2, 1.)), dsub(dsub(five_sqr, dmul(11., pxm2)), 2.));
    c[5] = dmul(dmul(dmul(dmul(l5, p01), pxm2), dadd(pxm2, 1.)), dsub(pxm2, 2.));
}

// AdvectionSolver::displ + the leftNode / d computation of operator()
// (src/solvers/AdvectionSolver.hpp:56-85) for a line of velocity vx.
// Returns leftNode; *d = LAG_OFFSET + inv_dx*(foot - coord(leftNode)).
BKMA_HD int adv_departure(const AdvPhys &p, int i1, double vx, double *d) {
    const double x = adv_coord(i1, p.minX, p.dx);
    const double displx = dmul(p.dt, vx);
    const double foot =
        dadd(p.minX, fmod(dsub(dsub(dadd(p.width, x), displx), p.minX), p.width));
    const int left = (int)floor(dmul(dsub(foot, p.minX), p.inv_dx));
    *d = dadd(2., dmul(p.inv_dx, dsub(foot, adv_coord(left, p.minX, p.dx))));
    return left;
}

}  // namespace bkma
