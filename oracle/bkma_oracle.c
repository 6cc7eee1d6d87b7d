/*
 * CPU oracle for the BKMA hot paths. TEST INFRASTRUCTURE ONLY (the checker;
 * never linked into the product library). See bkma_oracle.h for the contract
 * and the parity status.
 *
 * Build with -ffp-contract=off: the reference's arithmetic is restated
 * operation by operation, and FMA contraction would change the last bit.
 */
#include "bkma_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* LAG_ORDER / LAG_PTS / LAG_OFFSET and loc[] of
 * src/solvers/AdvectionSolver.hpp:7-11. */
#define REF_LAG_PTS 6
#define REF_LAG_OFFSET 2
static const double ref_loc[6] = {-1. / 24, 1. / 24., -1. / 12.,
                                  1. / 12., -1. / 24., 1. / 24.};

static void set_threads(int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
}

/* src/config/AdvectionParams.cpp:96-103 */
void bko_adv_update_deltas(bko_adv_params *p) {
    p->width = p->maxX - p->minX;
    p->dx = p->width / (double)p->n1;
    p->dvx = (p->maxVx - p->minVx) / (double)p->n0;
    p->inv_dx = 1 / p->dx;
}

/* src/solvers/AdvectionSolver.hpp:23-26 */
double bko_coord(int i, double min_value, double delta) {
    return min_value + i * delta;
}

/* src/solvers/AdvectionSolver.hpp:31-51, same association order. */
void bko_lag_basis_ref5(double px, double coef[6]) {
    const double pxm2 = px - 2.;
    const double sqrpxm2 = pxm2 * pxm2;
    const double pxm2_01 = pxm2 * (pxm2 - 1.);

    coef[0] = ref_loc[0] * pxm2_01 * (pxm2 + 1.) * (pxm2 - 2.) * (pxm2 - 1.);
    coef[1] = ref_loc[1] * pxm2_01 * (pxm2 - 2.) * (5 * sqrpxm2 + pxm2 - 8.);
    coef[2] = ref_loc[2] * (pxm2 - 1.) * (pxm2 - 2.) * (pxm2 + 1.) *
              (5 * sqrpxm2 - 3 * pxm2 - 6.);
    coef[3] = ref_loc[3] * pxm2 * (pxm2 + 1.) * (pxm2 - 2.) *
              (5 * sqrpxm2 - 7 * pxm2 - 4.);
    coef[4] = ref_loc[4] * pxm2_01 * (pxm2 + 1.) *
              (5 * sqrpxm2 - 11 * pxm2 - 2.);
    coef[5] = ref_loc[5] * pxm2_01 * pxm2 * (pxm2 + 1.) * (pxm2 - 2.);
}

void bko_lag_basis_textbook(int npts, double px, double *coef) {
    for (int j = 0; j < npts; ++j) {
        double num = 1.0, den = 1.0;
        for (int m = 0; m < npts; ++m) {
            if (m == j) continue;
            num *= (px - (double)m);
            den *= (double)(j - m);
        }
        coef[j] = num / den;
    }
}

/* src/solvers/AdvectionSolver.hpp:56-66 */
double bko_displ_v(const bko_adv_params *p, int i1, double vx) {
    const double x = bko_coord(i1, p->minX, p->dx);
    const double displx = p->dt * vx;
    return p->minX + fmod(p->width + x - displx - p->minX, p->width);
}

/* coord(i0, minRealVx, dvx), src/solvers/AdvectionSolver.hpp:60 */
double bko_line_velocity(const bko_adv_params *p, int64_t i0) {
    return bko_coord((int)i0, p->minVx, p->dvx);
}

/* src/solvers/AdvectionSolver.hpp:76-85 */
int bko_departure(const bko_adv_params *p, int i1, double vx, double *d_out) {
    const double foot = bko_displ_v(p, i1, vx);
    const int left = (int)floor((foot - p->minX) * p->inv_dx);
    *d_out = REF_LAG_OFFSET +
             p->inv_dx * (foot - bko_coord(left, p->minX, p->dx));
    return left;
}

/* One point of AdvectionSolver::operator() (AdvectionSolver.hpp:71-99) on a
 * strided line, generalised to the textbook bases for other degrees. */
static double adv_point(const bko_adv_params *p, const double *line,
                        int64_t stride, int i1, double vx, int degree,
                        int ref_weights) {
    double d;
    const int left = bko_departure(p, i1, vx, &d);
    const int npts = degree + 1;
    double coef[16];
    int first;
    if (ref_weights) {
        bko_lag_basis_ref5(d, coef);
        first = left - REF_LAG_OFFSET;
    } else {
        const int half = npts / 2 - 1;
        bko_lag_basis_textbook(npts, (double)half + (d - REF_LAG_OFFSET), coef);
        first = left - half;
    }
    const uint64_t n1 = (uint64_t)p->n1;
    double value = 0.;
    for (int k = 0; k < npts; k++) {
        /* (n1 + ipos1 + k) % n1 in size_t arithmetic, AdvectionSolver.hpp:94 */
        const uint64_t id = (n1 + (uint64_t)(int64_t)first + (uint64_t)k) % n1;
        value += coef[k] * line[(int64_t)id * stride];
    }
    return value;
}

/* AdaptiveWg schedule (src/core/AdaptiveWg.hpp:111-134): scratch then
 * write back, one (i0, i2) line at a time. */
void bko_adv_step(const bko_adv_params *p, double *data, int64_t n0_local,
                  int64_t i0_offset, const double *velocity, int degree,
                  int ref_weights, int nthreads) {
    const int64_t n1 = p->n1, n2 = p->n2;
    set_threads(nthreads);
#pragma omp parallel
    {
        double *scratch = (double *)malloc(sizeof(double) * (size_t)n1);
#pragma omp for collapse(2) schedule(static)
        for (int64_t li0 = 0; li0 < n0_local; ++li0) {
            for (int64_t i2 = 0; i2 < n2; ++i2) {
                const int64_t gi0 = li0 + i0_offset;
                const double vx = velocity ? velocity[li0]
                                           : bko_line_velocity(p, gi0);
                double *line = data + li0 * n1 * n2 + i2;
                for (int64_t i1 = 0; i1 < n1; ++i1)
                    scratch[i1] = adv_point(p, line, n2, (int)i1, vx, degree,
                                            ref_weights);
                for (int64_t i1 = 0; i1 < n1; ++i1) line[i1 * n2] = scratch[i1];
            }
        }
        free(scratch);
    }
}

/* src/tools/init.hpp:31-46 */
void bko_fill_adv(const bko_adv_params *p, double *data) {
    const double pi = 3.14159265358979323846;
    for (int64_t i0 = 0; i0 < p->n0; ++i0)
        for (int64_t i1 = 0; i1 < p->n1; ++i1) {
            const double x = p->minX + (double)i1 * p->dx;
            const double v = sin(4 * x * pi);
            for (int64_t i2 = 0; i2 < p->n2; ++i2)
                data[(i0 * p->n1 + i1) * p->n2 + i2] = v;
        }
}

/* src/tools/validation.hpp:9-80 */
double bko_validate_adv(const bko_adv_params *p, const double *data,
                        int64_t max_iter) {
    const double pi = 3.14159265358979323846;
    double highest = 0.0;
    for (int64_t i2 = 0; i2 < p->n2; ++i2) {
        double err = 0.0;
        for (int64_t i0 = 0; i0 < p->n0; ++i0)
            for (int64_t i1 = 0; i1 < p->n1; ++i1) {
                const double f = data[(i0 * p->n1 + i1) * p->n2 + i2];
                const double x = p->minX + (double)i1 * p->dx;
                const double v = p->minVx + (double)i0 * p->dvx;
                const double t = (double)max_iter * p->dt;
                err += fabs(f - sin(4 * pi * (x - v * t)));
            }
        const double l1 = err / (double)(p->n1 * p->n0);
        if (i2 == 0 || l1 > highest) highest = l1;
    }
    return highest;
}

/* ConvSolver::operator() (src/solvers/ConvSolver.hpp:20-44). The line view
 * `line` has stride n2; weight is span3d (K, Cin, Cout) row-major. */
static double conv_ref_point(const double *line, int64_t stride, int64_t n1,
                             const double *weight, const double *bias,
                             int64_t K, int64_t cin, int64_t length,
                             int64_t i1) {
    const int64_t cout = cin; /* out_channels = in_channels_ (:27) */
    const uint64_t oc = (uint64_t)i1 / (uint64_t)length;
    const uint64_t i_l = (uint64_t)i1 - oc * (uint64_t)length;
    double sum = bias[oc];
    for (int ic = 0; ic < cin; ++ic) {
        for (int k = 0; k < K; ++k) {
            /* int input_idx = i_l - k; if (input_idx < extent) ... (:36-37) */
            const int input_idx = (int)(int64_t)(i_l - (uint64_t)(int64_t)k);
            if ((uint64_t)(int64_t)input_idx < (uint64_t)n1) {
                sum += line[(int64_t)input_idx * stride] *
                       weight[((int64_t)k * cin + ic) * cout + (int64_t)oc];
            }
        }
    }
    return sum;
}

void bko_conv_ref_step(double *data, int64_t n0, int64_t n1, int64_t n2,
                       const double *weight, const double *bias, int64_t K,
                       int64_t cin, int64_t length, int nthreads) {
    const int64_t nw = n1 - (K - 1); /* AdaptiveWg.hpp:82-83 */
    set_threads(nthreads);
#pragma omp parallel
    {
        double *scratch = (double *)malloc(sizeof(double) * (size_t)(nw > 0 ? nw : 1));
#pragma omp for collapse(2) schedule(static)
        for (int64_t i0 = 0; i0 < n0; ++i0) {
            for (int64_t i2 = 0; i2 < n2; ++i2) {
                double *line = data + i0 * n1 * n2 + i2;
                for (int64_t ii1 = 0; ii1 < n1; ++ii1) {
                    const int64_t iw = ii1 - (K - 1);
                    if (iw >= 0)
                        scratch[iw] = conv_ref_point(line, n2, n1, weight, bias,
                                                     K, cin, length, ii1);
                }
                for (int64_t iw = 0; iw < nw; ++iw) line[iw * n2] = scratch[iw];
            }
        }
        free(scratch);
    }
}

void bko_conv_torch(const double *x, double *out, int64_t B, int64_t cin,
                    int64_t cout, int64_t L, int64_t K, const double *w,
                    const double *bias, int nthreads) {
    const int64_t lout = L - K + 1;
    set_threads(nthreads);
#pragma omp parallel
    {
        double *row = (double *)malloc(sizeof(double) * (size_t)(cout * lout));
#pragma omp for schedule(static)
        for (int64_t b = 0; b < B; ++b) {
            const double *xb = x + b * cin * L;
            for (int64_t co = 0; co < cout; ++co)
                for (int64_t l = 0; l < lout; ++l) {
                    double s = bias ? bias[co] : 0.0;
                    for (int64_t ci = 0; ci < cin; ++ci)
                        for (int64_t k = 0; k < K; ++k)
                            s += w[(co * cin + ci) * K + k] * xb[ci * L + l + k];
                    row[co * lout + l] = s;
                }
            double *ob = out + b * cout * (out == x ? L : lout);
            const int64_t ostride = (out == x) ? L : lout;
            for (int64_t co = 0; co < cout; ++co)
                memcpy(ob + co * ostride, row + co * lout,
                       sizeof(double) * (size_t)lout);
        }
        free(row);
    }
}

static uint64_t splitmix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

double bko_uniform(uint64_t seed, uint64_t idx) {
    const uint64_t h = splitmix64(seed ^ (idx * 0xD1B54A32D192ED03ull));
    return (double)(h >> 11) * (1.0 / 9007199254740992.0);
}
