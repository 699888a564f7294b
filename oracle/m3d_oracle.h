/* C restatement of the reference's octree-FV forward + adjoint solve.
 * ORACLE / TEST INFRASTRUCTURE ONLY -- see m3d_oracle.c. Complex arrays are
 * interleaved (re, im) doubles. */
#ifndef M3D_ORACLE_H
#define M3D_ORACLE_H

#include "m3d_case.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct m3d_oracle m3d_oracle;

/* ForwardSolverFV::setup + set_sigma (staggered grid and operators built here) */
m3d_oracle* m3d_oracle_create(const m3d_case* cs);
void m3d_oracle_destroy(m3d_oracle* S);
int m3d_oracle_sizes(const m3d_oracle* S, int* ne, int* nf, int* nc, int* nn);
int m3d_oracle_set_sigma(m3d_oracle* S, const double* sigma);
int m3d_oracle_set_tol_override(m3d_oracle* S, double tol);
/* compute_single_frequency: both polarisations, Z_out [ns][4] complex (xx, xy, yx, yy) */
int m3d_oracle_solve_frequency(m3d_oracle* S, double freq, double* Z_out);
int m3d_oracle_factorize(m3d_oracle* S, double freq);
int m3d_oracle_release(m3d_oracle* S);
int m3d_oracle_get_E(const m3d_oracle* S, int pol, double* out);
int m3d_oracle_set_E(m3d_oracle* S, const double* E1, const double* E2);
int m3d_oracle_adjoint_rhs(m3d_oracle* S, const double* wr, double* rhs1, double* rhs2);
int m3d_oracle_adjoint_solve(m3d_oracle* S, const double* rhs, double* lam);
int m3d_oracle_sensitivity(m3d_oracle* S, const double* E, const double* lam, double* g);
int m3d_oracle_perturbation_rhs(m3d_oracle* S, int pol, const double* dsig, double* out);
int m3d_oracle_delta_impedance(m3d_oracle* S, const double* dE, int pol, double* dZ);
int m3d_oracle_last_iters(const m3d_oracle* S, int* out, int cap);
int m3d_oracle_station_cells(const m3d_oracle* S, int* out);
int m3d_oracle_matrix_nnz(const m3d_oracle* S);
int m3d_oracle_get_matrix(const m3d_oracle* S, int* ptr, int* idx, double* val);
int m3d_oracle_get_edges(const m3d_oracle* S, double* xyz, double* len, int* dir, double* adual,
                         int* dead, int* node1, int* node2);
int m3d_oracle_gradient(m3d_oracle* S, const double* freqs, int nf, const double* obs_Z,
                        const double* obs_err, double* Z_out, double* grad);
/* CPU-baseline sample: seconds for exactly n_iter SSOR-BiCGStab iterations on
 * the assembled, BC-eliminated system of `freq` (setup time in *setup_s). */
double m3d_oracle_time_iterations(m3d_oracle* S, double freq, int n_iter, double* setup_s);

/* octree regularisation (src/inversion/regularization_octree.cpp) on the
 * oracle's mesh: setup, W^T W x, diag(W^T W), CmCm^T x, objective and
 * gradient (params = ln sigma per cell, ref per active cell or NULL). */
typedef struct m3d_oracle_reg m3d_oracle_reg;
m3d_oracle_reg* m3d_oracle_reg_create(const m3d_oracle* S, double alpha_s, double alpha_x, double alpha_y,
                                      double alpha_z, int n_smooth);
void m3d_oracle_reg_destroy(m3d_oracle_reg* R);
int m3d_oracle_reg_num_active(const m3d_oracle_reg* R);
void m3d_oracle_reg_active_to_global(const m3d_oracle_reg* R, int* a2g);
void m3d_oracle_reg_apply_wtw(const m3d_oracle_reg* R, const double* x, double* y);
void m3d_oracle_reg_diagonal(const m3d_oracle_reg* R, double* d);
void m3d_oracle_reg_apply_cmcmt(const m3d_oracle_reg* R, const double* x, double* y);
double m3d_oracle_reg_evaluate(const m3d_oracle_reg* R, const double* params, const double* ref, double* grad);

#ifdef __cplusplus
}
#endif

#endif
