// Gradient-space correction of the SSOR preconditioner (auxiliary nodal
// space) for the complex-FP32 inner solve.
//
// At low frequency A = C^T Mf^-1 C + i omega Me is nearly singular on
// discrete gradients: C G = 0, so for a gradient g = G phi on the free edges
// A g = i omega Me g, and G~^T A G~ = i omega L, where G~ is the edge-node
// gradient of build_gradient (src/octree/operators.cpp) restricted to free
// edges (rows that are not identity rows of the eliminated system) and to
// the nodes that are not Dirichlet nodes of the divergence correction, and L
// is exactly the Poisson operator of divcorr_poisson_
// (src/forward/forward_solver_fv.cpp:623-722, build_div_laplacian
// src/octree/operators.cpp:952-1019) with its Dirichlet rows.  SSOR damps
// the curl part of the error but barely moves the gradient part, which is
// why the reference interleaves divergence corrections between BiCGStab
// bursts.  Here the preconditioner itself gets the gradient-space term:
//
//     B r = M_ssor^-1 r + G~ (i omega L)^-1 G~^T r,
//
// the additive two-level form of Hiptmair's hybrid smoother, with (L)^-1
// replaced by one V-cycle of the aggregation multigrid that already
// preconditions the divergence-correction PCG (host/amg.cpp).  B is a
// different preconditioner for the same system, so the converged solution
// and the FP64 true-residual test are unchanged; only the iteration count
// drops (at 0.01 Hz about five-fold on the 1.7 M-edge mesh).
//
// The V-cycle (V(0,1) by default: post-smoothing only) runs in FP32 on
// [n][K] complex node vectors.  Level 0 is read from a packed FP32 copy of the
// divergence-correction Laplacian's incidence lists (gc_pack_level0, redone
// whenever the Laplacian is rebuilt); the coarser levels read the FP64 CSR
// operators of the device hierarchy, which a conductivity update refreshes in
// place.  The same cycle, run as V(1,1), preconditions the FP32 PCG of the
// mixed-precision divergence correction (dc_poisson_mixed_k).
#pragma once

#include <cuda_runtime.h>

#include "krylov.cuh"
#include "physics.cuh"

namespace m3d {

struct GcLevel {
    int n = 0;
    const int *ptr = nullptr, *col = nullptr;   // A_l in CSR (levels >= 1)
    const double* val = nullptr;
    const double* dinv = nullptr;               // Jacobi scale 1 / a_ii
    float* dinv32 = nullptr;                    // its FP32 copy (level 0, refreshed with the Laplacian)
    const int* agg = nullptr;                   // [n] aggregate in level l+1 (-1: none)
    const int *rptr = nullptr, *rcol = nullptr; // members of each aggregate of level l+1
    float2 *b = nullptr, *x = nullptr, *y = nullptr;   // [n][kMaxRhs] right side, pre-smoothed, scratch / post-smoothed
};

// Per right-hand side state of the FP32 PCG of the mixed-precision
// divergence-correction solve.
struct GcPcgState {
    double rho, tol, rz, alpha, beta;
    int run, iter, ref, pad_;
};

struct GcDev {
    int n_levels = 0;          // 0: correction unavailable
    int nn = 0;
    // level 0 = the divergence-correction Laplacian in incidence form
    const int *inc_ptr = nullptr, *inc_other = nullptr;
    const double *lap_off = nullptr, *lap_diag = nullptr;
    // FP32 copy read by the V-cycle and the FP32 PCG: (other node, value bits)
    // per incidence entry, and the diagonal; refreshed with the Laplacian
    int2* lap_pk = nullptr;
    float* lap_diag32 = nullptr;
    // restriction G~^T (per incidence entry) and prolongation G~ (per
    // permuted edge row, two entries), zero on masked edges / nodes
    const int* inc_edge = nullptr;
    const float* inc_g = nullptr;
    const int* e_node = nullptr;
    const float* e_g = nullptr;
    float2* out0 = nullptr;               // [nn][kMaxRhs] V-cycle result of the current half iteration
    GcLevel lv[phys::kAmgMaxLevels];
    int n_coarse = 0;
    const double* coarse_inv = nullptr;   // [n_coarse][n_coarse]
    float omega = 2.0f / 3.0f;            // smoother damping
    int presmooth = 0;                    // 1: V(1,1) cycle; 0: V(0,1) (post-smoothing only)
    double omega_max = 0.0;               // lanes with angular frequency <= omega_max are corrected
    long inc_entries = 0;                 // incidence entries (algorithmic bytes)
    // FP32 PCG work of the mixed-precision divergence-correction solve, [nn][kMaxRhs]
    float2 *dc_x = nullptr, *dc_r = nullptr, *dc_z = nullptr, *dc_p = nullptr, *dc_ap = nullptr;
    GcPcgState* dc_st = nullptr;          // [kMaxRhs]
};

// Masked FP32 restriction / prolongation weights (once per mesh).
void gc_weights(const MeshDev& m, float* inc_g, float* e_g, cudaStream_t s);
// FP32 level-0 copy (lap_pk, lap_diag32) of the current Laplacian.
void gc_pack_level0(const GcDev& g, cudaStream_t s);

// g.out0 = V(G~^T in), one V-cycle on every lane; in is
// [n_pad][K] complex FP32.  The term G~ out0 / (i omega) is added per row by
// the backward SSOR sweep (GcRowTerm).
template <int K>
void gc_apply_k(const GcDev& g, int n_rows, const float2* in, cudaStream_t s, long long* launches,
                KernelTimer* timer);

// Solves L phi = divJ for the right-hand sides of w with cg_run set (the
// PCG stage of divcorr_poisson_, forward_solver_fv.cpp:668-710): FP64
// iterative refinement around FP32 PCG solves preconditioned by the FP32
// V(1,1) cycle, until |divJ - L phi| < 1e-10 |divJ| in FP64.  Leaves phi in
// w.phi, clears cg_run, adds the FP32 iterations to each cg_iter and the
// batched iterations to *sweeps.  Returns the kernel launches.
template <int K>
long long dc_poisson_mixed_k(const GcDev& g, int nn, phys::DcWork w, dev::RedScratch red, cudaStream_t s,
                             long long* sweeps);

// Row term over g.out0 for the lanes k of B with 0 < omega_k <= g.omega_max.
GcRowTerm gc_row_term(const GcDev& g, const BatchView& B);

}  // namespace m3d
