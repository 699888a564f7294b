// Aggregation algebraic multigrid hierarchy for the node Laplacian
// of the divergence correction (the Poisson operator of divcorr_poisson_,
// src/forward/forward_solver_fv.cpp:623-722, built by build_div_laplacian,
// src/octree/operators.cpp:952-1019).  Host-side setup only; the V-cycle runs
// on the GPU (mg_apply in cuda/physics.cu).  The solver builds it with
// piecewise-constant prolongation (omega_p = 0); the smoothed prolongator of
// the option is kept for the setup tests.  The reference preconditions this PCG with
// Jacobi; the multigrid V-cycle is a stronger symmetric positive-definite
// preconditioner for the same system and the same stopping rule.
#pragma once

#include <vector>

namespace m3d {

struct CsrReal {
    int n_rows = 0, n_cols = 0;
    std::vector<int> ptr, col;
    std::vector<double> val;
};

struct AmgLevel {
    CsrReal A;                  // level operator, diagonal included
    std::vector<double> dinv;   // Jacobi smoother scale: 1 / a_ii (1 where a_ii is absent)
    CsrReal P;                  // prolongator to this level from the next (n_rows x n_next)
    CsrReal R;                  // restriction P^T
};

struct AmgHierarchy {
    std::vector<AmgLevel> levels;   // levels[0] is the fine operator
    std::vector<std::vector<int>> aggregates;   // per level l: row -> aggregate of level l+1 (-1: none)
    int n_coarse = 0;               // rows of the coarsest level
    std::vector<double> coarse_inv; // dense inverse of the coarsest operator, row-major
};

struct AmgOptions {
    double theta = 0.08;      // strength threshold |a_ij| >= theta sqrt(a_ii a_jj)
    double omega_p = 2.0 / 3.0; // prolongator smoothing weight (times D^-1 A)
    int max_coarse = 200;     // stop coarsening at or below this many rows
    int max_levels = 8;
};

// Builds the hierarchy of the symmetric operator A (CSR with the diagonal
// included).  Rows without strong off-diagonal connections (Dirichlet rows)
// are left out of every aggregate: the smoother alone handles them.
void amg_build(const CsrReal& A, const AmgOptions& opt, AmgHierarchy& H);

// Rebuilds the operators of a hierarchy for new values of the same sparsity
// pattern (a new conductivity on the same mesh), keeping the aggregates of
// `H` (the costly part of the setup).  Only for piecewise-constant
// prolongation (omega_p = 0).
void amg_refresh(const CsrReal& A, const AmgOptions& opt, AmgHierarchy& H);
// The same with the new values already written into H.levels[0].A.
void amg_refresh_values(const AmgOptions& opt, AmgHierarchy& H);

}  // namespace m3d
