/*
 * Driver that exposes the reference's OWN solver and config code through a C
 * ABI, so tests can pin the oracle restatement (bkma_oracle.c) and generate
 * golden vectors. It is compiled by oracle/build_ref.sh against the reference
 * sources where they lie (AdvectionSolver.hpp, ConvSolver.hpp, ConfigMap.cpp,
 * AdvectionParams.cpp, Conv1dParams.cpp, inih) with the host-only shim in
 * oracle/ref_shim; the result goes to oracle/_ref/ and is never committed.
 *
 * TEST INFRASTRUCTURE ONLY. The schedule around the solvers (compute a whole
 * line into scratch, then write it back) restates src/core/AdaptiveWg.hpp:
 * 111-134 on the CPU; the per-point math is the reference's, unmodified.
 */
#include <AdvectionParams.hpp>
#include <AdvectionSolver.hpp>
#include <ConfigMap.h>
#include <Conv1dParams.hpp>
#include <ConvSolver.hpp>

#include <cstdint>
#include <cstring>
#include <vector>

namespace {
struct LineView {
    double *p;
    std::size_t stride;
    std::size_t n;
    double &operator()(std::size_t i) const { return p[i * stride]; }
    std::size_t extent(int) const { return n; }
};
}  // namespace

extern "C" {

struct ref_adv_params {
    int64_t n0, n1, n2, max_iter;
    double dt, minX, maxX, minVx, maxVx;
    double width, dx, dvx, inv_dx;
    int32_t inplace, gpu;
    int64_t pref_wg_size, seq_size0, seq_size2;
    char kernel_impl[64];
};

static void export_params(const ADVParams &p, ref_adv_params *o) {
    o->n0 = (int64_t)p.n0;
    o->n1 = (int64_t)p.n1;
    o->n2 = (int64_t)p.n2;
    o->max_iter = (int64_t)p.maxIter;
    o->dt = p.dt;
    o->minX = p.minRealX;
    o->maxX = p.maxRealX;
    o->minVx = p.minRealVx;
    o->maxVx = p.maxRealVx;
    o->width = p.realWidthX;
    o->dx = p.dx;
    o->dvx = p.dvx;
    o->inv_dx = p.inv_dx;
    o->gpu = p.gpu;
    o->pref_wg_size = (int64_t)p.pref_wg_size;
}

/* ADVParamsNonCopyable::setup on a .ini (AdvectionParams.cpp:64-92). */
int ref_adv_params_from_ini(const char *path, ref_adv_params *o) {
    ConfigMap cm{std::string(path)};
    if (cm.ParseError() < 0) return -1;
    ADVParamsNonCopyable s;
    s.setup(cm);
    ADVParams p(s);
    export_params(p, o);
    o->inplace = s.inplace;
    o->seq_size0 = (int64_t)s.seq_size0;
    o->seq_size2 = (int64_t)s.seq_size2;
    std::strncpy(o->kernel_impl, s.kernelImpl.c_str(), sizeof(o->kernel_impl) - 1);
    o->kernel_impl[sizeof(o->kernel_impl) - 1] = 0;
    return 0;
}

/* Default-constructed ADVParams (AdvectionParams.hpp:12-53). */
void ref_adv_params_default(ref_adv_params *o) {
    ADVParams p;
    std::memset(o, 0, sizeof(*o));
    export_params(p, o);
}

static ADVParams make_params(const ref_adv_params *in) {
    ADVParams p;
    p.n0 = (std::size_t)in->n0;
    p.n1 = (std::size_t)in->n1;
    p.n2 = (std::size_t)in->n2;
    p.dt = in->dt;
    p.minRealX = in->minX;
    p.maxRealX = in->maxX;
    p.minRealVx = in->minVx;
    p.maxRealVx = in->maxVx;
    p.update_deltas();
    return p;
}

/* nsteps advection steps of the whole field with AdvectionSolver. */
void ref_adv_step(const ref_adv_params *in, double *data, int nsteps) {
    const ADVParams p = make_params(in);
    const AdvectionSolver solver(p);
    const std::size_t n0 = p.n0, n1 = p.n1, n2 = p.n2;
    for (int t = 0; t < nsteps; ++t) {
#pragma omp parallel
        {
            std::vector<double> scratch(n1);
#pragma omp for collapse(2) schedule(static)
            for (std::size_t i0 = 0; i0 < n0; ++i0)
                for (std::size_t i2 = 0; i2 < n2; ++i2) {
                    LineView line{data + i0 * n1 * n2 + i2, n2, n1};
                    for (std::size_t i1 = 0; i1 < n1; ++i1)
                        scratch[i1] = solver(line, i0, i1, i2);
                    for (std::size_t i1 = 0; i1 < n1; ++i1) line(i1) = scratch[i1];
                }
        }
    }
}

/* The reference's stencil of point (i0, i1): out[j] = solver(e_j, i0, i1),
 * i.e. the weight it gives node j of the line (0 if j is not a tap). */
void ref_adv_stencil(const ref_adv_params *in, int64_t i0, int64_t i1,
                     double *out) {
    const ADVParams p = make_params(in);
    const AdvectionSolver solver(p);
    std::vector<double> e(p.n1, 0.0);
    LineView line{e.data(), 1, p.n1};
    for (std::size_t j = 0; j < p.n1; ++j) {
        e[j] = 1.0;
        out[j] = solver(line, (std::size_t)i0, (std::size_t)i1, 0);
        e[j] = 0.0;
    }
}

/* AdvectionSolver::lag_basis, exported for the pinning tests. */
void ref_lag_basis(double px, double *coef) {
    const auto c = AdvectionSolver::lag_basis(px);
    for (int k = 0; k < LAG_PTS; ++k) coef[k] = c[k];
}

struct ref_conv_params {
    int64_t length, channel_in, channel_out, k, total_batch_size,
        batch_size_n2, n0, n1, n2, n_write;
    int32_t inplace, gpu;
    int64_t pref_wg_size, seq_size0, seq_size2;
    char kernel_impl[64];
};

/* Conv1dParamsNonCopyable::setup (Conv1dParams.cpp:44-68). */
int ref_conv_params_from_ini(const char *path, ref_conv_params *o) {
    ConfigMap cm{std::string(path)};
    if (cm.ParseError() < 0) return -1;
    Conv1dParamsNonCopyable s;
    s.setup(cm);
    o->length = (int64_t)s.length;
    o->channel_in = s.channel_in;
    o->channel_out = s.channel_out;
    o->k = s.k;
    o->total_batch_size = (int64_t)s.total_batch_size;
    o->batch_size_n2 = (int64_t)s.batch_size_n2;
    o->n0 = (int64_t)s.n0;
    o->n1 = (int64_t)s.n1;
    o->n2 = (int64_t)s.n2;
    o->n_write = (int64_t)s.n_write;
    o->inplace = s.inplace;
    o->gpu = s.gpu;
    o->pref_wg_size = s.pref_wg_size;
    o->seq_size0 = (int64_t)s.seq_size0;
    o->seq_size2 = (int64_t)s.seq_size2;
    std::strncpy(o->kernel_impl, s.kernelImpl.c_str(), sizeof(o->kernel_impl) - 1);
    o->kernel_impl[sizeof(o->kernel_impl) - 1] = 0;
    return 0;
}

/* One in-place conv step with ConvSolver over data[n0][n1][n2]. */
void ref_conv_step(double *data, int64_t n0, int64_t n1, int64_t n2,
                   double *weight, double *bias, int64_t K, int64_t cin,
                   int64_t length) {
    span3d_t w(weight, (std::size_t)K, (std::size_t)cin, (std::size_t)cin);
    span1d_t b(bias, (std::size_t)cin);
    ConvSolver solver{w, b, (std::size_t)K, (std::size_t)cin, (std::size_t)length};
    const std::size_t window = solver.window();
    const std::size_t nw = (std::size_t)n1 - (window - 1);
#pragma omp parallel
    {
        std::vector<double> scratch(nw);
#pragma omp for collapse(2) schedule(static)
        for (int64_t i0 = 0; i0 < n0; ++i0)
            for (int64_t i2 = 0; i2 < n2; ++i2) {
                LineView line{data + i0 * n1 * n2 + i2, (std::size_t)n2,
                              (std::size_t)n1};
                for (int64_t ii1 = 0; ii1 < n1; ++ii1) {
                    const int64_t iw = ii1 - (int64_t)(window - 1);
                    if (iw >= 0)
                        scratch[iw] = solver(line, (std::size_t)i0,
                                             (std::size_t)ii1, (std::size_t)i2);
                }
                for (std::size_t iw = 0; iw < nw; ++iw) line(iw) = scratch[iw];
            }
    }
}

}  // extern "C"
