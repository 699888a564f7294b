/* Test-oracle case description shared by the two CPU checkers:
 *   oracle/_ref  - the reference's own solver sources compiled against shims
 *   oracle/m3d_oracle.c - the C restatement of the same path
 * ORACLE / TEST INFRASTRUCTURE ONLY: the product never includes this file.
 *
 * All arrays are caller-owned, little-endian host memory; complex values are
 * interleaved (re, im) doubles.
 */
#ifndef M3D_CASE_H
#define M3D_CASE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct m3d_case {
    /* leaf list of the octree (the mesh input of the solve) */
    double domain[6];          /* x_min x_max y_min y_max z_min z_max (m) */
    int min_level, max_level;
    int n_cells;
    const int* level;          /* [n_cells] */
    const double* cx;          /* [n_cells] cell centres */
    const double* cy;
    const double* cz;
    const int* cell_type;      /* [n_cells] 0 earth, 1 air, 2 ocean */
    /* model */
    const double* sigma;       /* [n_cells] S/m */
    double sigma_bg;           /* background sigma of the 1-D primary field */
    /* survey */
    int n_stations;
    const double* station_xyz; /* [n_stations*3] */
    int n_freqs;
    const double* freqs;       /* [n_freqs] Hz */
    /* ForwardParamsFV (include/maple3dmt/forward/forward_solver_fv.h:31-69) */
    double bicgstab_tol;
    int bicgstab_maxiter;
    int scattered_field;
    double air_z_threshold;
    int div_correction;
    int div_corr_iters;
    double div_corr_tol;
    int divcorr_outer_max;
    int divcorr_iter_per_dc;
    /* observed impedances for the gradient: [n_stations][n_freqs][4] complex,
       errors [n_stations][n_freqs][4]; weight is 1 where error > 0 */
    const double* obs_Z;
    const double* obs_err;
} m3d_case;

#ifdef __cplusplus
}
#endif

#endif
