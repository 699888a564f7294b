// Batched multi-right-hand-side SSOR-preconditioned BiCGStab on the edge
// system, and the sliced-ELL operator it runs on.
//
// Restates BiCGStabSolver::solve (src/forward/bicgstab.cpp:15-166; Hermitian
// dots include/maple3dmt/forward/bicgstab.h:68-73) and
// SSORPreconditioner::apply (include/maple3dmt/forward/ssor.h:53-78, omega = 1)
// for K right-hand sides at once.  Differences from the reference, by design:
//  * Gauss-Seidel order is colour by colour (a graph colouring of A), so each
//    sweep is K parallel launches instead of a serial loop; within a colour
//    the original edge order is kept.  This is SSOR on the colour-permuted
//    matrix, a different (equally valid) preconditioner, so iterates differ
//    while converged solutions agree.
//  * A's off-diagonal part is real and shared by every frequency; each right-
//    hand side r carries its own complex diagonal d_f(r) (frequency f(r)).
//  * Scalars (rho, alpha, omega, norms) stay on the device; every reduction is
//    a deterministic grid reduction whose last block also runs the scalar
//    recurrences and the per-RHS stopping / breakdown tests.
#pragma once

#include <cuda_runtime.h>
#include <vector>

#include "common.cuh"

namespace m3d {

// Per right-hand side state of one BiCGStab solve (device memory).
struct BicgState {
    double2 rho, rho_old, alpha, omega, beta;
    double bnorm, rnorm, snorm, res, tol, true_res;
    int status;      // kRunning, kConverged, kBreakdown, kMaxIter, kInactive
    int iter, maxiter;
    int pend_x;      // x += alpha * p_hat still to apply this iteration
    int breakdown;   // 1 rho, 2 (r0,v), 3 (t,t), 4 omega
    int pad_;
};

enum : int { kRunning = 0, kConverged = 1, kBreakdown = 2, kMaxIter = 3, kInactive = 9 };

// Sliced ELL storage of the off-diagonal part, rows in colour order, each row
// holding its "lower" entries (earlier colours) then its "upper" entries.
template <class R>
struct EllView {
    const int* slice_off;
    const int* slice_wl;
    const int* slice_wu;
    const int* col;
    const R* val;
    int n_slices;
};

template <class R>
struct DiagView {
    const dev::cplx<R>* d;     // [n_freq][n_pad] diagonal of A
    const dev::cplx<R>* dinv;  // [n_freq][n_pad] 1 / diagonal (ssor.h:37-44)
    int n_pad;
};

// Frequency index of each right-hand side of the batch.
struct BatchView {
    int K;
    int fmap[dev::kMaxRhs];
};

// Everything one launch of the batched solver needs.
template <class R>
struct KrylovCtx {
    EllView<R> A;
    DiagView<R> D;
    BatchView B;
    std::vector<int> colour_slices;  // [n_colours + 1] slice ranges per colour
    int n_pad;
    int grid_vec;     // blocks for vector kernels with reductions
    int grid_spmv;    // blocks for SpMV kernels with reductions
    dev::RedScratch red;
    cudaStream_t stream;
    long long* launches;   // host counter of kernel launches
};

// Work vectors of one batched solve, each [n_pad][K] complex of type R.
template <class R>
struct KrylovVecs {
    dev::cplx<R> *x, *b, *r, *r0, *p, *v, *s, *t, *ph, *sh, *y;
};

enum SpmvMode : int {
    kSpmvPlain = 0,    // y = A x
    kSpmvAp = 1,       // v = A p_hat, (r0, v) -> alpha
    kSpmvAs = 2,       // t = A s_hat, (t, t), (t, s) -> omega
    kSpmvInit = 3,     // r = b - A x, r0 = r, |b|, |r|, (r0, r) -> start
    kSpmvTrueRes = 4,  // y = b - A x, |y| / |b| -> true_res
};

// Host launchers (explicit instantiations for R in {double, float}).
template <class R>
void spmv(const KrylovCtx<R>& c, int mode, const dev::cplx<R>* x, dev::cplx<R>* y,
          const dev::cplx<R>* aux, dev::cplx<R>* aux_out, BicgState* st);
template <class R>
void ssor_apply(const KrylovCtx<R>& c, const dev::cplx<R>* in, dev::cplx<R>* y, dev::cplx<R>* out);
template <class R>
void bicg_init(const KrylovCtx<R>& c, const KrylovVecs<R>& v, BicgState* st);
template <class R>
void bicg_iteration(const KrylovCtx<R>& c, const KrylovVecs<R>& v, BicgState* st);

}  // namespace m3d
