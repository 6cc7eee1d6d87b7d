/*
 * CPU oracle for the two BKMA hot paths (advection, conv1d).
 *
 * TEST INFRASTRUCTURE ONLY: this library is the checker. It is loaded by
 * tests/, by __graft_entry__.smoke() and by bench.py's cpu_baseline / reference
 * arm. The product path (libbkma_gb300.so) never links or calls it.
 *
 * Every function restates, in plain C, the arithmetic of the reference
 * (Maison-de-la-Simulation/parallel-advection) in the same operation order so
 * that an FP64 run is bit-identical to the reference compiled with
 * -ffp-contract=off. The citation on each function names the reference
 * file:line it follows.
 *
 * Parity status: pinned. tests/golden/ holds vectors produced by the
 * reference's own AdvectionSolver / ConvSolver / ConfigMap compiled on the CPU
 * (oracle/build_ref.sh); tests/test_oracle_golden.py checks this restatement
 * against them bit-for-bit.
 */
#ifndef BKMA_ORACLE_H
#define BKMA_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Mirror of ADVParams (src/config/AdvectionParams.hpp:10-57). */
typedef struct bko_adv_params {
    int64_t n0, n1, n2;
    double dt;
    double minX, maxX, minVx, maxVx;
    /* derived by bko_adv_update_deltas */
    double width, dx, dvx, inv_dx;
} bko_adv_params;

/* ADVParams::update_deltas (src/config/AdvectionParams.cpp:96-103). */
void bko_adv_update_deltas(bko_adv_params *p);

/* AdvectionSolver::coord (src/solvers/AdvectionSolver.hpp:23-26). */
double bko_coord(int i, double min_value, double delta);

/* AdvectionSolver::lag_basis (src/solvers/AdvectionSolver.hpp:31-51):
 * the reference's 6-point "degree 5" weights at px in [2,3). */
void bko_lag_basis_ref5(double px, double coef[6]);

/* Textbook Lagrange weights on nodes 0..npts-1 evaluated at px (product
 * formula). The reference has no form for degrees 3 and 9; this is the
 * standard centred Lagrange basis used for those degrees. */
void bko_lag_basis_textbook(int npts, double px, double *coef);

/* AdvectionSolver::displ (src/solvers/AdvectionSolver.hpp:56-66), with the
 * line velocity passed explicitly (the reference derives it from i0 with
 * coord(i0, minRealVx, dvx)). */
double bko_displ_v(const bko_adv_params *p, int i1, double vx);

/* Velocity of line i0 by the reference law coord(i0, minRealVx, dvx). */
double bko_line_velocity(const bko_adv_params *p, int64_t i0);

/* The departure cell of point (i1) on a line of velocity vx, as computed in
 * AdvectionSolver::operator() (src/solvers/AdvectionSolver.hpp:76-85):
 * returns leftNode and writes the fractional coordinate d = LAG_OFFSET +
 * inv_dx*(foot - coord(leftNode)) to *d_out. */
int bko_departure(const bko_adv_params *p, int i1, double vx, double *d_out);

/* One advection time step over the whole field data[n0][n1][n2] (FP64,
 * in place), following the AdaptiveWg schedule (src/core/AdaptiveWg.hpp:
 * 111-134): every (i0,i2) line is computed into a scratch line first, then
 * written back. degree 5 with ref_weights=1 is the reference solver
 * (AdvectionSolver.hpp:71-99); degree 3/5/9 with ref_weights=0 uses the
 * textbook basis with taps leftNode-(npts/2-1) .. leftNode+npts/2.
 * velocity: NULL for the reference law, else one value per i0 line.
 * i0_offset shifts the global line index (sharded n0).
 * nthreads <= 0 uses the OpenMP default. */
void bko_adv_step(const bko_adv_params *p, double *data, int64_t n0_local,
                  int64_t i0_offset, const double *velocity, int degree,
                  int ref_weights, int nthreads);

/* fill_buffer_adv (src/tools/init.hpp:31-46): data = sin(4*pi*x). */
void bko_fill_adv(const bko_adv_params *p, double *data);

/* validate_result_adv (src/tools/validation.hpp:9-80): max over i2 of the
 * mean L1 error against sin(4*pi*(x - v*t)), t = max_iter*dt. */
double bko_validate_adv(const bko_adv_params *p, const double *data,
                        int64_t max_iter);

/* Reference-semantics conv1d step (ConvSolver, src/solvers/ConvSolver.hpp:
 * 20-44, driven by AdaptiveWg with window()=K, src/core/AdaptiveWg.hpp:82-83,
 * 123-134). data[n0][n1][n2] with n1 = C*L; weight[K][Cin][Cout]; bias[Cout].
 * In place: data[:, 0:n1-K+1, :] receives the packed outputs. */
void bko_conv_ref_step(double *data, int64_t n0, int64_t n1, int64_t n2,
                       const double *weight, const double *bias, int64_t K,
                       int64_t cin, int64_t length, int nthreads);

/* PyTorch-semantics conv1d (cross-correlation, stride 1, no padding), FP64:
 * out[b][co][l] = bias[co] + sum_ci sum_k w[co][ci][k] * x[b][ci][l+k] for
 * l < L-K+1. Accumulation order: bias, then ci outer, k inner. out may alias
 * x (in place, Cin == Cout): row b is read fully before it is written. */
void bko_conv_torch(const double *x, double *out, int64_t B, int64_t cin,
                    int64_t cout, int64_t L, int64_t K, const double *w,
                    const double *bias, int nthreads);

/* Counter-based uniform generator shared with the device init kernels:
 * splitmix64(seed ^ (idx * golden)) -> [0,1) with 53 random bits. */
double bko_uniform(uint64_t seed, uint64_t idx);

#ifdef __cplusplus
}
#endif
#endif
