/* m3d_gb300.h -- C ABI of the GB300 forward + adjoint octree-FV EM solver.
 *
 * This is the drop-in boundary under the reference's forward-solver interface
 * maple3dmt::forward::IForwardSolver (include/maple3dmt/forward/iforward_solver.h:31-115)
 * and its octree implementation ForwardSolverFV
 * (include/maple3dmt/forward/forward_solver_fv.h:77-253).  Every entry point
 * names the reference member it replaces.
 *
 * Conventions
 *  - Plain pointers and sizes only; all buffers are caller-owned host
 *    memory, except for m3d_dot_batched and m3d_dot_batched_noalloc, whose
 *    vectors are device pointers; complex vectors are interleaved (re, im)
 *    doubles.
 *  - Edge vectors use the reference's edge numbering (StaggeredGrid edge ids,
 *    src/octree/staggered_grid.cpp:82-121); cell vectors the leaf order;
 *    impedances are [station][4] in the order Zxx, Zxy, Zyx, Zyy.
 *  - Every function returns M3D_OK (0) or one M3D_ERR_* code and, except
 *    m3d_dot_batched_noalloc (stream-ordered), has synchronised the device
 *    before it returns; m3d_last_error() gives the message of the last
 *    failure on that handle.
 *  - A solver handle is single-threaded, like the reference (not re-entrant).
 *    Different handles may be driven from different host threads at the
 *    same time (each owns its CUDA streams); m3d_group_station_gradients
 *    does exactly that for per-frequency meshes.
 *  - Solver state follows the reference's ordering rules: a frequency must be
 *    solved (m3d_compute_single_frequency) or factorised before the adjoint,
 *    sensitivity and J.v calls of that frequency
 *    (src/inversion/inversion_fv.cpp:250-291); M3D_ERR_STATE otherwise.
 */
#ifndef M3D_GB300_H
#define M3D_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define M3D_OK 0
#define M3D_ERR_ARG 1         /* null pointer, bad size or value out of range */
#define M3D_ERR_STATE 2       /* call out of order (e.g. adjoint before forward) */
#define M3D_ERR_CUDA 3        /* CUDA runtime error */
#define M3D_ERR_OOM 4         /* host or device allocation failed */
#define M3D_ERR_NO_DEVICE 5   /* no usable CUDA device */
#define M3D_ERR_TOO_LARGE 6   /* size beyond a fixed limit of the entry point */
#define M3D_ERR_NUMERIC 7     /* non-finite values met in a solve */

/* Per-right-hand-side solve status (m3d_stats.status). */
#define M3D_SOLVE_CONVERGED 1
#define M3D_SOLVE_BREAKDOWN 2
#define M3D_SOLVE_MAXITER 3
#define M3D_SOLVE_STAGNATED 4
#define M3D_SOLVE_DIVERGED 5

/* ---------------------------------------------------------------------- */
/* Mesh input: the finished octree leaf list.                              */
/* Replaces the octree::OctreeMesh& argument of ForwardSolverFV::setup     */
/* (include/maple3dmt/forward/forward_solver_fv.h:82-83), read through     */
/* OctreeMesh::cell_center / cell_level / cell_type / params               */
/* (include/maple3dmt/octree/octree_mesh.h:124-177).                        */
/* ---------------------------------------------------------------------- */
typedef struct m3d_leaves {
    double domain[6];      /* x_min x_max y_min y_max z_min z_max (m) */
    int min_level;
    int max_level;         /* <= 14 */
    int n_cells;
    const int* level;      /* [n_cells] */
    const double* cx;      /* [n_cells] cell centres (m) */
    const double* cy;
    const double* cz;
    const int* cell_type;  /* [n_cells] 0 earth, 1 air, 2 ocean */
} m3d_leaves;

/* ---------------------------------------------------------------------- */
/* Layout introspection (host only, no device needed).                     */
/* StaggeredGrid::build + DiscreteOperators::build                          */
/* (src/octree/staggered_grid.cpp:70-409, src/octree/operators.cpp:19-170). */
/* ---------------------------------------------------------------------- */
typedef struct m3d_layout m3d_layout;

int m3d_layout_build(const m3d_leaves* leaves, m3d_layout** out);
void m3d_layout_destroy(m3d_layout* L);
/* nnz = stiffness pattern size (including the diagonal of every edge). */
int m3d_layout_sizes(const m3d_layout* L, int* n_edges, int* n_faces, int* n_cells, int* n_nodes,
                     int* nnz, int* n_hanging);
/* Any pointer may be NULL. xyz [ne][3]; node1/node2: edge end-point node ids. */
int m3d_layout_edges(const m3d_layout* L, double* xyz, double* length, int* direction,
                     double* dual_area, int* dead, int* node1, int* node2);
/* S = Ce^T Mf^-1 Ce (real): rowptr [ne+1], col [nnz], val [nnz]. */
int m3d_layout_stiffness(const m3d_layout* L, int* rowptr, int* col, double* val);
/* hanging pairs [n_hanging][3]: coarse, child1, child2. */
int m3d_layout_hanging(const m3d_layout* L, int* pairs);

/* ---------------------------------------------------------------------- */
/* Solver                                                                   */
/* ---------------------------------------------------------------------- */

/* Mirrors ForwardParamsFV (include/maple3dmt/forward/forward_solver_fv.h:31-69)
 * plus the GPU's own knobs. m3d_params_default() fills the reference defaults
 * (bicgstab_maxiter 2000, tol 1e-7, ...). */
typedef struct m3d_params {
    double bicgstab_tol;
    int bicgstab_maxiter;
    int scattered_field;      /* 1: solve for E_sec, E = E_pri + E_sec */
    double air_z_threshold;   /* m */
    int div_correction;
    int div_corr_iters;
    double div_corr_tol;
    int divcorr_outer_max;
    int divcorr_iter_per_dc;
    double sigma_bg;          /* background sigma of the 1-D primary field (RefinementParams::sigma_bg) */
    /* GPU */
    int precision;            /* 0: complex128 Krylov; 1: complex64 Krylov inside FP64 refinement */
    int true_residual_check;  /* 1: confirm ||b - A x|| / ||b|| <= tol in FP64 and refine until met */
    int max_refinements;      /* FP64 refinement steps allowed on top of the Krylov solve */
    int print_level;
    int forward_interleaved;  /* 0: forward as the reference (full BiCGStab, then divergence
                                 correction, forward_solver_fv.cpp:346-367); 1: forward solved
                                 with interleaved divergence correction like the adjoint (:778-888) */
    int row_kernels;          /* SpMV / SSOR row kernels: 0 CSR rows read by the lanes,
                                 1 32-row slices bulk-copied to shared memory */
    int divcorr_precond;      /* divergence-correction PCG preconditioner: 0 Jacobi (the
                                 reference's), 1 aggregation multigrid V-cycle */
    int ssor_form;            /* mixed-precision inner solve: 0 right-preconditioned SSOR-BiCGStab
                                 as the reference, 1 Eisenstat split form (staged rows) for batches
                                 without a right-hand side that gets the gradient-space term (those
                                 always run the right-preconditioned form) */
    int gradcorr;             /* 1: the mixed-precision inner solve adds a gradient-space term
                                 G (i omega L)^-1 G^T (one multigrid V-cycle on the divergence-
                                 correction Laplacian L) to the SSOR preconditioner of the
                                 right-hand sides with f <= gradcorr_fmax; needs div_correction.
                                 Batches with such a right-hand side run the right-preconditioned
                                 form.  0: SSOR alone (the reference's preconditioner) */
    double gradcorr_fmax;     /* Hz */
    int gradcorr_presmooth;   /* V-cycle of the gradient-space term: 1 V(1,1), 0 V(0,1) */
    int divcorr_mixed;        /* 1 (with precision 1, divcorr_precond 1): the divergence-correction Poisson solve runs as
                                 complex-FP32 PCG (FP32 multigrid V(1,1) preconditioner) inside FP64
                                 iterative refinement, stopped by the FP64 true residual at the
                                 reference's 1e-10 |divJ|; 0: FP64 PCG */
    double inner_tol_floor;   /* smallest relative residual asked of one complex-FP32 inner solve (3e-5),
                                 when residual_replacement is 0 */
    int residual_replacement; /* 1: the complex-FP32 inner solve (right-preconditioned form) runs to the
                                 final tolerance, its residual replaced by the FP64 true residual of the
                                 accumulated solution each time it falls 1000x (no Krylov restart).
                                 0 (default): restart per FP64 refinement, measured faster on C2 */
    int gradcorr_overlap;     /* 1: the V-cycles of the gradient-space term run on a second CUDA stream,
                                 overlapping the forward SSOR sweep (same arithmetic); 0: one stream */
    int krylov;               /* inner solve of the mixed-precision path: 0 BiCGStab (default), 1 flexible
                                 GMRES (restart fgmres_m) with the SSOR / gradient-space preconditioner */
    int fgmres_m;             /* FGMRES restart length (20) */
    int learned_period;       /* with krylov = 1 and a trained network (m3d_learn_*): every learned_period-th
                                 FGMRES direction comes from the network instead of SSOR (0: never; 2) */
    int sweep_rows;           /* SSOR ordering (super-block, colour) with super-blocks of about sweep_rows
                                 edges, so a sweep's gathers stay in L2; 0: colour order over the mesh */
    int coop_sweep;           /* 1: each staged SSOR sweep is one cooperative launch over all its groups
                                 (bounded grid barriers between groups); 0: one launch per group */
    int cuda_graphs;          /* 1: the mixed-precision inner solve captures its 10-iteration chunk (every
                                 launch of ten BiCGStab iterations, both streams) in a CUDA graph once per
                                 batch shape and refinement step, from the shape's third chunk on, and
                                 replays it; 0 (default): launches issued one by one (measured as fast on
                                 C2 and faster with several meshes at once) */
    double ssor_relax;        /* relaxation factor omega of the SSOR sweeps of the mixed-precision inner
                                 solve, 0 < omega < 2 (1: the reference's symmetric Gauss-Seidel,
                                 ssor.h:58-78); the FP64 path always uses 1 */
} m3d_params;

typedef struct m3d_solver m3d_solver;

/* Counters of the last solving call (all right-hand sides of that call). */
typedef struct m3d_stats {
    int n_rhs;                 /* m3d_gradient_batch: forward then adjoint RHS of each frequency group */
    int iterations[64];        /* Krylov iterations per RHS (first 64) */
    int status[64];            /* M3D_SOLVE_* per RHS */
    double true_residual[64];  /* ||b - A x||_2 / ||b||_2 in FP64, before divergence correction */
    int total_iterations;
    int refinements;
    double seconds;
    long long kernel_launches;
    int divcorr_calls;         /* divcorr_poisson_ calls (forward_solver_fv.cpp:623-722) */
    int divcorr_outer;         /* Poisson rounds inside them */
    long long divcorr_cg_iterations;  /* Jacobi-PCG iterations, summed over rhs */
    long long forward_iterations;     /* Krylov iterations of the forward phase, summed over rhs */
    long long adjoint_iterations;     /* ... of the adjoint phase */
    long long divcorr_cg_sweeps;      /* batched PCG iterations run (each serves every rhs of a batch) */
    double divcorr_setup_ms;          /* host time of the last multigrid setup of the PCG */
    int replacements;                 /* residual replacements of the inner solves */
    int graphs_failed;                /* 1: a chunk capture failed, chunks run as direct launches */
    long long graph_replays;          /* CUDA-graph chunk replays since the handle was created */
} m3d_stats;

void m3d_params_default(m3d_params* p);

/* Handle creation binds to CUDA device `device` (no device work yet). */
int m3d_solver_create(int device, m3d_solver** out);
void m3d_solver_destroy(m3d_solver* s);
const char* m3d_last_error(const m3d_solver* s);

/* ForwardSolverFV::setup (forward_solver_fv.cpp:28-47): layout + device upload. */
int m3d_solver_setup(m3d_solver* s, const m3d_leaves* leaves, const m3d_params* params);
int m3d_solver_sizes(const m3d_solver* s, int* n_edges, int* n_cells, int* n_nodes, int* n_colours);
/* ForwardSolverFV::set_sigma (:49-51) / update_sigma (:53-58). */
int m3d_set_sigma(m3d_solver* s, const double* sigma, int n_cells);
/* Station positions (x, y, z) [n][3]; mapped to cells as find_stations_ (:1393-1485). */
int m3d_set_stations(m3d_solver* s, const double* xyz, int n_stations);
/* set_solver_tolerance_override (forward_solver_fv.h:181); 0 restores. */
int m3d_set_tolerance_override(m3d_solver* s, double tol);
/* current_omega (forward_solver_fv.h:104); 0 before any frequency. */
int m3d_current_omega(const m3d_solver* s, double* omega);

/* compute_single_frequency (:1732-1738): assemble, solve both polarisations,
 * divergence correction, impedances. Z_out [n_stations][4] complex, may be NULL. */
int m3d_compute_single_frequency(m3d_solver* s, double freq_hz, double* Z_out);
/* factorize_frequency (:1743-1750): assemble only. */
int m3d_factorize_frequency(m3d_solver* s, double freq_hz);
/* release_factorization (:1755-1757). */
int m3d_release_factorization(m3d_solver* s);
/* background_E (forward_solver_fv.h:132-134): pol 0 or 1, E_out [n_edges] complex. */
int m3d_background_E(m3d_solver* s, int pol, double* E_out);
/* set_background_fields_complex (:1762-1765). */
int m3d_set_background_fields(m3d_solver* s, const double* E1, const double* E2);

/* build_adjoint_rhs_from_residual (:1804-2013): wr [n_stations][4] complex. */
int m3d_build_adjoint_rhs(m3d_solver* s, const double* wr, double* rhs1, double* rhs2);
/* adjoint_solve_complex (:1770-1773 -> :914-924). */
int m3d_adjoint_solve(m3d_solver* s, const double* rhs, double* lambda);
/* solve_rhs_complex (:1796-1799 -> :930-940). */
int m3d_solve_rhs(m3d_solver* s, const double* rhs, double* x);
/* n_rhs right-hand sides at the factorised frequency, each solved as
 * adjoint_solve / solve_rhs does (solve_with_divcorr_, :778-888), batched 16
 * per launch: the reference's loop over many adjoint sources (e.g. one per
 * station and polarisation) as multi-RHS solves.  rhs, out [n_rhs][n_edges]
 * complex; stats cover every right-hand side (first 64). */
int m3d_solve_rhs_batch(m3d_solver* s, const double* rhs, int n_rhs, double* out);
/* Gradients of n_src residual sources at the solved single frequency
 * (m3d_compute_single_frequency first), one per source: for source j,
 * build_adjoint_rhs_from_residual (:1804-2013) of wr[j], both adjoint solves
 * (adjoint_solve_complex, :914-924) and compute_sensitivity_complex
 * (:989-1059) of each polarisation, summed over the two polarisations as
 * InversionFV::compute_gradient_ sums them (src/inversion/inversion_fv.cpp:
 * 280-290).  With wr[j] non-zero at one station, g[j] is that station's row
 * of J^T W^2 r.  Built, solved (eight sources, sixteen right-hand sides per
 * batched solve) and reduced on the device.  wr [n_src][n_stations][4]
 * complex, g [n_src][n_cells]; stats cover every right-hand side (first 64). */
int m3d_station_gradients(m3d_solver* s, const double* wr, int n_src, double* g);
/* Per-frequency meshes of uneven size (one handle per frequency mesh, each
 * set up, with conductivity and stations, all on one device), run
 * concurrently: one host thread per handle, each on its handle's own CUDA
 * stream, started in decreasing order of stiffness entries, at most
 * max_concurrent at once
 * (0: all).  For mesh m: m3d_compute_single_frequency(freqs[m]) -> Z_out[m]
 * [n_stations][4] (Z_out or Z_out[m] nullable), then
 * m3d_station_gradients(wr[m], n_src[m]) -> g_out[m] [n_src[m]][n_cells(m)].
 * The GPU counterpart of the reference's per-frequency loop
 * (src/inversion/inversion_fv.cpp:250-291) and of its frequency-parallel
 * manager (src/utils/freq_parallel.cpp:99-195) on one device.  status[m]
 * gets mesh m's return code (m3d_last_error(handles[m]) its message); the
 * call returns the first non-zero status in mesh order, M3D_OK if none.
 * The handles must be distinct and must not be used by other threads
 * during the call. */
int m3d_group_station_gradients(m3d_solver* const* handles, int n_meshes, const double* freqs,
                                const double* const* wr, const int* n_src, double* const* Z_out,
                                double* const* g_out, int max_concurrent, int* status);
/* compute_sensitivity_complex (:1778-1782 -> :989-1059): g [n_cells]. */
int m3d_compute_sensitivity(m3d_solver* s, const double* E, const double* lambda, double* g);
/* build_perturbation_rhs_complex (:1787-1791 -> :945-984): pol 1 or 2. */
int m3d_build_perturbation_rhs(m3d_solver* s, int pol, const double* delta_sigma, double* rhs);
/* extract_delta_impedance_complex (:2018-2065): pol 1 or 2, dZ [n_stations][4]. */
int m3d_extract_delta_impedance(m3d_solver* s, const double* dE, int pol, double* dZ);

/* ---------------------------------------------------------------------- */
/* Batched entry points: every frequency of an inversion iteration in one   */
/* multi-right-hand-side solve (the GPU counterpart of the frequency loop   */
/* in compute_responses :63-79 and InversionFV::compute_gradient_           */
/* src/inversion/inversion_fv.cpp:230-312).                                 */
/* ---------------------------------------------------------------------- */

/* All frequencies, both polarisations: Z_out [n_freqs][n_stations][4];
 * E_out (nullable) [n_freqs][2][n_edges]. Fields stay on the device for
 * m3d_gradient_batch's adjoint phase. */
int m3d_forward_batch(m3d_solver* s, const double* freqs, int n_freqs, double* Z_out, double* E_out);

/* Forward + weighted residual + adjoint + sensitivity for all frequencies:
 * obs_Z [n_stations][n_freqs][4] complex, obs_err [n_stations][n_freqs][4]
 * (components with err <= 0 carry no weight). grad [n_cells] = sum over
 * frequencies and polarisations; Z_out nullable [n_freqs][n_stations][4]. */
int m3d_gradient_batch(m3d_solver* s, const double* freqs, int n_freqs, const double* obs_Z,
                       const double* obs_err, double* Z_out, double* grad);

/* ---------------------------------------------------------------------- */
/* Octree model regularisation (RegularizationOctree,                      */
/* src/inversion/regularization_octree.cpp) on the solver's mesh.          */
/* ---------------------------------------------------------------------- */

/* RegParamsOctree (include/maple3dmt/inversion/regularization_octree.h:25-32);
 * alpha_r (reference damping) is not used by the operators below. */
typedef struct m3d_reg_params {
    double alpha_s, alpha_x, alpha_y, alpha_z;
    int n_smooth;
} m3d_reg_params;

/* RegularizationOctree::setup (:24-172): active (earth) cells, W^T W from
 * face adjacency, neighbour lists, unit average diagonal.  Host setup once
 * per mesh, operators on the GPU.  After m3d_solver_setup. */
int m3d_reg_setup(m3d_solver* s, const m3d_reg_params* p);
/* n_active (); active_to_global [n_active] */
int m3d_reg_num_active(const m3d_solver* s, int* n_active);
int m3d_reg_active_to_global(const m3d_solver* s, int* a2g);
/* apply_WtW (:229-231), apply_CmCmT (:251-281), diagonal_WtW (:236-246):
 * active-space vectors [n_active] */
int m3d_reg_apply_wtw(m3d_solver* s, const double* x, double* y);
int m3d_reg_apply_cmcmt(m3d_solver* s, const double* x, double* y);
int m3d_reg_diagonal_wtw(m3d_solver* s, double* d);
/* evaluate (:183-201) and gradient (:206-224): params = ln(sigma) per cell
 * [n_cells], ref [n_active] (nullable: zero reference model); value
 * nullable; grad nullable [n_cells] */
int m3d_reg_evaluate(m3d_solver* s, const double* params, const double* ref, double* value, double* grad);

/* GN-CG product out = J^T W^2 J dsigma for all frequencies in two batched
 * solves: the data term of ImplicitJtJOperatorFV::Mult
 * (src/inversion/implicit_jtj_fv.cpp:78-192); the regularisation term
 * lambda W^T W x and the log-sigma / active-cell mapping stay with the caller.
 * Per frequency f and polarisation p: build_perturbation_rhs(p+1, dsigma) on
 * the background field, solve_rhs, extract_delta_impedance(p+1), weighting by
 * w^2 = 1/err^2 (0 where err <= 0), build_adjoint_rhs_from_residual (source
 * of polarisation p), adjoint_solve, compute_sensitivity with the background
 * field, summed.  Inner solves stop at relative residual inner_tol (the
 * reference uses 1e-4, implicit_jtj_fv.cpp:113).  The background fields are
 * those the last m3d_forward_batch left on the device (the reference's
 * cache_background_fields, :37-56): freqs must be the same n_freqs <= 8
 * frequencies, else M3D_ERR_STATE.  dsigma, out [n_cells]; obs_err
 * [n_stations][n_freqs][4]. */
int m3d_jtjv_batch(m3d_solver* s, const double* freqs, int n_freqs, const double* dsigma,
                   const double* obs_err, double inner_tol, double* out);

/* Batched Hermitian inner products out[k] = sum_i conj(x[i][k]) * y[i][k] of
 * K interleaved complex-FP64 DEVICE vectors x, y ([n][K] complex; K in
 * {1, 2, 4, 8, 16}); out is a device pointer to K complex values.  The
 * reduction of BiCGStabSolver::dot (include/maple3dmt/forward/bicgstab.h:68-73)
 * for K systems in one pass, exposed for callers that keep their own vectors
 * on the device (misfit and model norms of an inversion).  Runs on the
 * solver's stream with the reduction scratch of m3d_solver_setup (required
 * first) and synchronises before returning. */
int m3d_dot_batched(m3d_solver* s, const double* x, const double* y, long long n, int K, double* out);

/* Allocation-free m3d_dot_batched (no counterpart in the reference): same
 * kernel and result, but no solver handle and no device allocation, for
 * callers that own all device memory and may not allocate.  Its reduction
 * scratch is a fixed 256 KiB static device array per device (K <= 16
 * right-hand sides x 1024 blocks); K > 16 returns M3D_ERR_TOO_LARGE, n is
 * unlimited.  x, y, out are device pointers on the current device; the call
 * enqueues on `stream` (a cudaStream_t; NULL = legacy default stream) and
 * returns without synchronising.  The first call on each device looks up the
 * scratch address (set-up); make it before latency-critical work.  Calls on
 * the same device share the scratch: calls in flight at the same time (two
 * streams, or two host threads without a lock) race and give wrong results,
 * so issue them on one stream or serialise them. */
int m3d_dot_batched_noalloc(const double* x, const double* y, long long n, int K, double* out, void* stream);

int m3d_get_stats(const m3d_solver* s, m3d_stats* out);

/* ---------------------------------------------------------------------- */
/* Measurement (no counterpart in the reference, which times with wall     */
/* clocks in its drivers): CUDA events on the solver's own stream.         */
/* ---------------------------------------------------------------------- */

/* Record a start / stop event; stop synchronises and returns elapsed ms. */
int m3d_timer_start(m3d_solver* s);
int m3d_timer_stop(m3d_solver* s, double* ms);

/* Kernel classes: 0 SpMV, 1 SSOR apply (all colour sweeps), 2 Krylov vector
 * updates, 3 divergence correction (one interval per call, its bytes counted
 * from the call's PCG sweeps), 4 gradient-space term of the preconditioner,
 * 5 J^T r sensitivity.  bytes = algorithmic bytes (matrix entries, diagonals
 * and vector streams each counted once). */
typedef struct m3d_kernel_times {
    long long launches[6];
    double ms[6];
    double bytes[6];
    /* the same split by batch width: [class][K = 2, 4, 8, 16, other] */
    long long launches_k[6][5];
    double ms_k[6][5];
    double bytes_k[6][5];
} m3d_kernel_times;

int m3d_set_kernel_timing(m3d_solver* s, int on);   /* also resets the totals */
int m3d_get_kernel_times(m3d_solver* s, m3d_kernel_times* out);

/* ---------------------------------------------------------------------- */
/* Autotuner (no counterpart in the reference, which runs one serial      */
/* solve): row-kernel layout and right-hand-side block size of the        */
/* batched FP32 inner solve, measured on this mesh and GPU.               */
/* ---------------------------------------------------------------------- */

typedef struct m3d_tune_entry {
    int row_kernels;          /* 0 CSR rows read by the lanes, 1 slice-staged rows */
    int K;                    /* right-hand sides per batch (2, 4, 8, 16) */
    double ms_per_iter;       /* one FP32 BiCGStab iteration of the batch */
    double ms_per_rhs_iter;   /* the same per right-hand side */
} m3d_tune_entry;

/* Times `reps` FP32 inner-solve iterations at frequency freq for both
 * layouts and K = 2 .. max_K (at most 8 entries into table, *n_entries set),
 * then applies the layout fastest at max_K (m3d_params.row_kernels) and the
 * K with the least time per right-hand side as the batch of
 * m3d_solve_rhs_batch (*row_kernels, *rhs_block report them).  Results are
 * cached per (edges, stiffness entries, max_K, gradient-space term) for the
 * process: a repeated call applies the cached choice without timing
 * (*cached = 1) unless force != 0.  Drops the factorisation and the resident
 * fields; call after m3d_set_sigma, before the solves. */
int m3d_autotune(m3d_solver* s, double freq, int max_K, int reps, int force, m3d_tune_entry* table,
                 int* n_entries, int* row_kernels, int* rhs_block, int* cached);

/* ---------------------------------------------------------------------- */
/* Learned preconditioner network (no counterpart in the reference, whose */
/* solve has no learned part): a 3-D convolutional network, 3x3x3 kernels, */
/* ReLU between layers, BF16 weights and activations with FP32            */
/* accumulation on the tcgen05 tensor cores.  These entry points take     */
/* host arrays, for checking the kernels; the solver drives the same      */
/* network on device data (m3d_learn_*).                                  */
/* ---------------------------------------------------------------------- */

typedef struct m3d_cnn m3d_cnn;

/* layers >= 2; c_in, hidden, c_out in 1..32; He-initialised from seed. */
int m3d_cnn_create(int device, int layers, int c_in, int hidden, int c_out, unsigned seed, m3d_cnn** out);
void m3d_cnn_destroy(m3d_cnn* c);
const char* m3d_cnn_last_error(const m3d_cnn* c);
/* w [layers][27][32 c_out][32 c_in] (zero-padded), b [layers][32], FP32;
 * tap t = (dz + 1) 9 + (dy + 1) 3 + (dx + 1) */
int m3d_cnn_get_weights(m3d_cnn* c, float* w, float* b);
int m3d_cnn_set_weights(m3d_cnn* c, const float* w, const float* b);
/* x [n][D][H][W][c_in] -> y [n][D][H][W][c_out]; W in {16, 32, 64, 128}, H a
 * multiple of 128 / W; zero padding at the grid boundary */
int m3d_cnn_forward(m3d_cnn* c, const float* x, int n, int D, int H, int W, float* y);
/* gradients of sum(dy * network(x)): dw, db as in get_weights, dx like x
 * (may be null) */
int m3d_cnn_backward(m3d_cnn* c, const float* x, const float* dy, int n, int D, int H, int W, float* dw, float* db,
                     float* dx);
/* one Adam step on 0.5 mean |network(x) - target|^2 (mean over voxels and
 * samples, summed over channels); the loss before the step into *loss */
int m3d_cnn_train_step(m3d_cnn* c, const float* x, const float* target, int n, int D, int H, int W, float lr,
                       double* loss);

/* The network as the solver's learned preconditioner.  A dense grid of
 * (2^grid_level)^3 cells over the mesh's unit cube carries each right-hand
 * side's field to the network (per cell and direction means, unit RMS, plus
 * conductivity and frequency channels) and the network's output back to the
 * edges.  Training pairs are recorded from the plain FP64 SSOR-BiCGStab
 * forward solves of m3d_learn_collect (residual r_k -> error x* - x_k, at
 * every poll of the solve).  With m3d_params.krylov = 1 the mixed-precision
 * solve runs flexible GMRES and, once m3d_learn_train has run, takes every
 * learned_period-th direction from the network: the network's coarse
 * correction c (scaled per right-hand side by least squares) followed by one
 * SSOR / gradient-space application to the rest, z = a c + B (v - a A c).
 * The FP64 true residual remains the stopping test. */
int m3d_learn_setup(m3d_solver* s, int grid_level, int layers, int hidden, unsigned seed, long long max_samples);
/* the inner solve between calls: m3d_params.krylov, fgmres_m, learned_period */
int m3d_set_krylov(m3d_solver* s, int krylov, int fgmres_m, int learned_period);
/* plain FP64 forward solves of freqs at the current conductivity, recording
 * pairs until max_samples are held; *n_samples = pairs held */
int m3d_learn_collect(m3d_solver* s, const double* freqs, int nf, long long* n_samples);
/* Adam (learning rate lr, minibatch <= 16) over the first (1 - val_frac) of
 * the pairs; mean loss per epoch into epoch_loss[epochs] (may be null), the
 * held-out pairs' loss into *val_loss (may be null) */
int m3d_learn_train(m3d_solver* s, int epochs, float lr, int batch, unsigned seed, double val_frac,
                    double* epoch_loss, double* val_loss);

/* ---------------------------------------------------------------------- */
/* Test hook (no counterpart in the reference).                           */
/* ---------------------------------------------------------------------- */

/* on != 0: every slice-staged kernel of this solver polls its copy barrier
 * once without blocking and takes its timeout path when the copy has not
 * landed (the block skips its slices and waits, bounded, for the copy in
 * flight); the next solve then fails with M3D_ERR_CUDA.  on = 0 restores
 * the bounded waits.  For testing the error path only. */
int m3d_test_set_consume_no_wait(m3d_solver* s, int on);

#ifdef __cplusplus
}
#endif

#endif /* M3D_GB300_H */
