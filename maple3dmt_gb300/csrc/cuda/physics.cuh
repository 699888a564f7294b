// Device data of one mesh and the non-Krylov kernels of the solve path:
// system diagonal (assembly), primary field and boundary lift, hanging-edge
// interpolation, divergence correction, station impedances, adjoint source,
// sensitivity and the J.v pieces.  Each launcher cites the reference code it
// restates.
#pragma once

#include <cuda_runtime.h>

#include "common.cuh"
#include "krylov.cuh"

namespace m3d {

struct GcDev;   // FP32 node multigrid (gradcorr.cuh)

// Row flags (permuted edge rows).
enum : unsigned char {
    kFlagConstrained = 1,   // identity row in A (solve BC or dead)   forward_solver_fv.cpp:214-217
    kFlagBc = 2,            // Dirichlet edge of the solve            :166-194
    kFlagDead = 4,          // dead coarse hanging edge               :206-208
    kFlagDcBc = 8,          // BC edge of compute_bc_flags_           :559-569
    kFlagSensFixed = 16,    // skipped by compute_sensitivity         :1019-1029
    kFlagPad = 32,          // padding row of the sliced layout
};

struct MeshDev {
    int ne, n_pad, nc, nn, n_slices;
    int* perm;          // [n_pad] permuted row -> reference edge id (-1 padding)
    int* iperm;         // [ne] reference edge id -> permuted row
    unsigned char* flags;  // [n_pad]
    signed char* dir;   // [n_pad] edge direction
    double* ez;         // [n_pad] edge midpoint z
    double* s_diag;     // [n_pad] S_ii
    double* me_geom;    // [n_pad] A_dual * L
    double* adual;      // [n_pad]
    double* elen;       // [n_pad]
    int* nadj;          // [n_pad] number of adjacent cells
    int* adj_ptr;       // [n_pad + 1] adjacency of permuted rows (reference cell order)
    int* adj_cell;
    int* lift_ptr;      // [n_pad + 1] free row -> BC columns (reference column order)
    int* lift_col;
    double* lift_val;
    int nhp;
    int* hp;            // [nhp][3] coarse, child1, child2 (permuted rows)
    // nodes
    int* inc_ptr;       // [nn + 1] node -> incident edges, reference edge order
    int* inc_edge;      // permuted edge row
    int* inc_other;     // other node
    double* inc_gv;     // G[e, v]
    double* inc_gw;     // G[e, other]
    unsigned char* node_bc;  // [nn]
    int* e_node;        // [n_pad][2] node ids in G's column order (pads: 0)
    double* e_g;        // [n_pad][2] G values
    // cells
    int* cell_ptr;      // [nc + 1] cell -> edges (StaggeredGrid::cell_edges order), permuted rows
    int* cell_edge;
    double* sens_w;     // [n_pad] A_dual * L / n_adj of rows the sensitivity sums, 0 for the others
};

// Per station data, built by the host at m3d_set_stations.
struct StationDev {
    int ns;
    int* cell;          // [ns] station cell (-1 none)
    double* geom;       // [ns][6] cx cy cz cdx cdy cdz
    int* e_ptr;         // [ns + 1]
    int* e_row;         // permuted rows of the cell's edges, cell_edges order
    unsigned char* e_code;  // bit0-1 direction, bit2 top (z > cz), bit3 +x (x > cx), bit4 +y (y > cy)
    double* sigma_cell; // [ns] sigma of the station cell (1-D fallback)
};

// Cached H / Z of a station at one frequency (StationHCache, forward_solver_fv.h:216-223).
struct HCache {
    double2 Hx1, Hy1, Hx2, Hy2, det, Zxx, Zxy, Zyx, Zyy;
    double cdx, cdy, cdz, pad_;
};

// Vector of K right-hand sides, [n_pad][K] complex double.
struct VecK {
    double2* p;
    int K;
};

// Per right-hand side data of a batch.
struct RhsInfo {
    int K;
    int f[dev::kMaxRhs];         // frequency slot of the diagonal arrays
    int pol[dev::kMaxRhs];       // source polarisation 0 (Ex) / 1 (Ey), -1 none
    double2 ik[dev::kMaxRhs];    // sqrt(i omega mu0 sigma_bg) (forward_solver_fv.cpp:121)
    double omega[dev::kMaxRhs];
};

namespace phys {

// build_edge_mass (operators.cpp:481-518) and me_sigma of
// build_div_laplacian / compute_div_sigma_E (:956-973, :1030-1048).
void edge_mass(const MeshDev& m, const double* sigma, double* Me, double* me_dc, cudaStream_t s);
// Frequency-independent diagonal pairs (S_ii, Me_i) of A on free rows, (1, 0)
// on constrained / padding rows (operators.cpp:607-616, forward_solver_fv.cpp:224-234);
// d_f = S_ii + i omega_f Me_i and its SSOR inverse (ssor.h:37-44) are formed
// by the kernels that need them.
void diag_coeffs(const MeshDev& m, const double* Me, double2* sm, float2* sm32, cudaStream_t s);
// E_primary on edges of direction pol for each rhs (forward_solver_fv.cpp:121-136, :318-323);
void primary_field(const MeshDev& m, VecK out, const RhsInfo& info, bool bc_only, cudaStream_t s);
// rhs_total of build_rhs (:244-255) from the BC values in `ebc`.
void lift_rhs(const MeshDev& m, VecK ebc, VecK rhs, cudaStream_t s);
// out = a - b (elementwise, all rhs).
void vsub(long n, const double2* a, const double2* b, double2* out, cudaStream_t s);
// interpolate_hanging (:258-261) on every rhs of x.
void interpolate_hanging(const MeshDev& m, VecK x, bool sequential, cudaStream_t s);
// E = E_pri + E_sec; E_bc on BC rows (:357-361).
void combine_total(const MeshDev& m, VecK epri, VecK esec, VecK ebc, VecK e, cudaStream_t s);
// gather / scatter between reference order (host layout [K][ne]) and permuted [n_pad][K]
void to_permuted(const MeshDev& m, const double2* ref, int K, int k, VecK dst, cudaStream_t s);
void from_permuted(const MeshDev& m, VecK src, int k, double2* ref, cudaStream_t s);
void fill_zero(VecK v, long n_pad, cudaStream_t s);

// ---- divergence correction (forward_solver_fv.cpp:623-722) ----
struct DcState {
    double div0, dn, rn;
    double2 rz, alpha, beta;
    int outer;      // outer iterations done
    int done;       // outer loop finished for this rhs
    int cg_run;     // PCG still iterating
    int cg_iter;
    int active;     // rhs takes part
    int pad_;
};
struct DcWork {
    double2 *divJ, *phi, *r, *z, *p, *Ap, *phi0;  // [nn][K]
    double* lap_diag;   // [nn] L_vv (1 on BC nodes)
    double* lap_off;    // [inc] off-diagonal per incidence entry (0 on BC rows / columns)
    double* jac_inv;    // [nn] inverse Jacobi diagonal (1 where L has no usable diagonal)
    DcState* st;        // [K]
    // L's off-diagonal part as 32-node slice segments (staged.cuh format, FP64
    // values, columns fixed per mesh, values rewritten with lap_off)
    unsigned char* lap_seg;
    const int4* lap_work;   // [n_node_slices]
    const int* lap_qpos;    // [inc] index, in doubles into lap_seg, of incidence q's value
    int lap_stage;          // bytes of the largest node segment
    int n_node_slices;
    unsigned* seg_err;
};

// Laplacian values for the current sigma (build_div_laplacian + Dirichlet rows/cols, :581-606).
void dc_build_laplacian(const MeshDev& m, const double* me_dc, DcWork w, cudaStream_t s);
// phi0 = G^T rhs / (i omega) (compute_phi0 :893-908) for every rhs.
void dc_phi0(const MeshDev& m, VecK rhs, const RhsInfo& info, DcWork w, cudaStream_t s);
// One full divcorr_poisson_ call on every active rhs of E; phi0 optional.
// Returns the number of kernel launches. Iteration caps: outer <= max_outer,
// PCG <= max(500, nn) per outer (the reference's caps).
struct DcCounters { int calls = 0, outer = 0; long long cg_iterations = 0, cg_sweeps = 0; };
// Multigrid V-cycle preconditioner of the node-Laplacian PCG (host setup in
// host/amg.cpp).  Level 0 is L itself, applied through the node slice
// segments of DcWork; levels 1.. are CSR Galerkin operators, linked by
// piecewise-constant aggregation; the coarsest level is solved by a dense
// inverse.  Work vectors are [n_l][K] complex.
constexpr int kAmgMaxLevels = 8;
struct AmgLevelDev {
    int n;
    const int *ptr, *col;          // A_l (levels >= 1)
    const double* val;
    const double* dinv;            // Jacobi smoother scale
    const int* agg;                // [n] aggregate in level l+1 (-1: none)
    const int *rptr, *rcol;        // members of each aggregate of level l+1
    double2 *b, *x, *y, *r;        // right side, pre-smoothed iterate, post-smoothed iterate, residual
};
struct AmgDev {
    int n_levels = 0;
    AmgLevelDev lv[kAmgMaxLevels];
    int n_coarse = 0;
    const double* coarse_inv = nullptr;   // [n_coarse][n_coarse]
    double omega = 2.0 / 3.0;             // smoother damping
};

// With `mixed` set, the Poisson solve of each round is the mixed-precision
// one of gradcorr.cuh (FP32 PCG inside FP64 refinement, same stopping rule).
long long divcorr(const MeshDev& m, const double* me_dc, VecK E, bool use_phi0, DcWork w,
                  int max_outer, double tol, const int* active_host, dev::RedScratch red,
                  cudaStream_t s, int cg_chunk, DcCounters* counters = nullptr, const AmgDev* amg = nullptr,
                  const GcDev* mixed = nullptr);

// ---- GN-CG J^T W^2 J v pieces (implicit_jtj_fv.cpp:78-192) ----
// w^2 dZ of lane 2f + p into wr_p[f] (err [ns][nf][4], dz [2 nf][ns][4], wr_p [nf][ns][4]).
void jtj_weight(int ns, int nf, const double* err, const double2* dz, double2* wr0, double2* wr1, cudaStream_t s);
// out = lane 2f of a, lane 2f + 1 of b ([n_pad][K]).
void pick_pol_lanes(long n_pad, int K, const double2* a, const double2* b, double2* out, cudaStream_t s);

// ---- stations (forward_solver_fv.cpp:1490-1727, :1804-2065) ----
// Z and H cache per (frequency f, station); E1 = rhs 2f, E2 = rhs 2f+1 of E.
void station_impedance(const StationDev& st, VecK E, const double* omegas, int nf, HCache* hc,
                       double2* Z, cudaStream_t s);
// weighted residual wr = w^2 conj(obs - pred), w = 1/err (inversion_fv.cpp:258-271);
// obs/err layout [ns][nf_total][4] with frequency offset f0.
void weighted_residual(int ns, int nf, int nf_total, int f0, const double2* obs, const double* err,
                       const double2* Z, double2* wr, cudaStream_t s);
// adjoint source for every frequency: rhs 2f <- pol1, 2f+1 <- pol2 (must be zeroed first).
void adjoint_rhs(const StationDev& st, const MeshDev& m, const double2* wr, const HCache* hc,
                 const double* omegas, int nf, VecK out, cudaStream_t s);
// adjoint sources of n_src station residuals at one frequency: wr [n_src][ns][4],
// one station cache hc [ns] and omega[0]; rhs 2j <- pol1, 2j+1 <- pol2 of
// source j (must be zeroed first).
void adjoint_rhs_sources(const StationDev& st, const double2* wr, const HCache* hc, const double* omega, int n_src,
                         VecK out, cudaStream_t s);
// g[j][c] = sum_p Re(i omega sum_e lambda_e E_e dMe), lambda rhs 2j+p against
// E rhs e0+p, for n_src <= 8 sources at one frequency (g [n_src][nc], written).
void sensitivity_sources(const MeshDev& m, const double* sigma, VecK E, int e0, VecK lam, const double* omega,
                         int n_src, double* g, cudaStream_t s);
// g[c] (+)= sum_f Re(i omega_f sum_e lambda_e E_e dMe) over both polarisations
// (compute_sensitivity :989-1059 summed as in inversion_fv.cpp:282-288).
// E rhs 2f+p pairs with lambda rhs 2f+p; npol = 1 uses rhs f only.
void sensitivity(const MeshDev& m, const double* sigma, VecK E, VecK lam, const double* omegas,
                 int nf, int npol, double* g, cudaStream_t s);
// build_perturbation_rhs (:945-984) for one rhs.
void perturbation_rhs(const MeshDev& m, const double* sigma, const double* dsigma, VecK E, int kE,
                      double omega, VecK out, int kout, cudaStream_t s);
// extract_delta_impedance_complex (:2018-2065).
void delta_impedance(const StationDev& st, VecK dE, int kE, const HCache* hc, int pol, double2* dZ,
                     cudaStream_t s);

}  // namespace phys
}  // namespace m3d
