// Batched multi-right-hand-side SSOR-preconditioned BiCGStab on the edge
// system, and the split-CSR operator it runs on.
//
// Restates BiCGStabSolver::solve (src/forward/bicgstab.cpp:15-166; Hermitian
// dots include/maple3dmt/forward/bicgstab.h:68-73) and
// SSORPreconditioner::apply (include/maple3dmt/forward/ssor.h:53-78, omega = 1)
// for K right-hand sides at once.  Differences from the reference, by design:
//  * Gauss-Seidel order is colour by colour (a graph colouring of A), so each
//    sweep is one parallel launch per colour instead of a serial loop; within
//    a colour the original edge order is kept.  This is SSOR on the colour-
//    permuted matrix, a different (equally valid) preconditioner, so iterates
//    differ while converged solutions agree.
//  * Lanes run over right-hand sides: lane l of a warp works on rhs l % K of
//    row (warp row base + l / K), so each neighbour gather of K complex values
//    is one contiguous, coalesced segment and each matrix entry is a
//    broadcast load shared by the K lanes of its row.
//  * A's off-diagonal part is real and shared by every frequency; each right-
//    hand side r carries its own complex diagonal d_f(r) (frequency f(r)).
//  * Scalars (rho, alpha, omega, norms) stay on the device; every reduction is
//    a deterministic grid reduction whose last block also runs the scalar
//    recurrences and the per-RHS stopping / breakdown tests.
#pragma once

#include <cuda_runtime.h>
#include <vector>

#include "common.cuh"
#include "staged.cuh"

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

// Off-diagonal part in "split CSR": rows in the solver's permuted order, each
// row holding its lower entries (columns in earlier colours) in
// [rp[i], rs[i]) and its upper entries in [rs[i], rp[i+1]).
template <class R>
struct OpView {
    const int* rp;     // [n_pad + 1]
    const int* rs;     // [n_pad]
    const int* col;
    const R* val;
    int n_pad;
};

// Diagonal of A for every frequency from one frequency-independent pair per
// row: sm[row] = (S_ii, Me_i) on free rows and (1, 0) on constrained or padding
// rows, so d_f = S_ii + i omega_f Me_i (operators.cpp:607-616) and the SSOR
// inverse (ssor.h:37-44) are formed in registers.
template <class R>
struct DiagView {
    const dev::cplx<R>* sm;
};

// Frequency index of each right-hand side of the batch.
struct BatchView {
    int K;
    int fmap[dev::kMaxRhs];
    double omega[dev::kMaxRhs];   // angular frequency of each right-hand side
    double relax = 1.0;           // SSOR relaxation factor of the sweeps (1: the reference's symmetric GS)
};

// Per-row gradient-space term of the right-preconditioned FP32 iteration
// (gradcorr.cuh): with y the node vector of one multigrid V-cycle, the
// preconditioned vector gets c = G~ y / (i omega) added by the backward SSOR
// sweep as it writes each row; G~ y at permuted row i =
// e_g[2i] y[e_node[2i]] + e_g[2i+1] y[e_node[2i+1]].
struct GcRowTerm {
    const float2* ya = nullptr;   // V-cycle output (null: no term)
    const int* e_node = nullptr;
    const float* e_g = nullptr;
    float s[dev::kMaxRhs] = {};   // 1 / omega of each lane; 0: no term on that lane
};

__device__ __forceinline__ float2 gc_grad_row(const GcRowTerm& t, const float2* __restrict__ y, int row, int rhs,
                                              int K) {
    const float g0 = __ldg(&t.e_g[2 * row]), g1 = __ldg(&t.e_g[2 * row + 1]);
    if (g0 == 0.0f && g1 == 0.0f) return make_float2(0.0f, 0.0f);
    const float2 a = y[(size_t)__ldg(&t.e_node[2 * row]) * K + rhs];
    const float2 b = y[(size_t)__ldg(&t.e_node[2 * row + 1]) * K + rhs];
    return make_float2(g0 * a.x + g1 * b.x, g0 * a.y + g1 * b.y);
}

// Optional CUDA-event timing of kernel classes on the solver's stream.
enum KernelClass : int {
    kClsSpmv = 0, kClsSsor = 1, kClsVec = 2, kClsDivcorr = 3, kClsGradcorr = 4, kClsSens = 5, kNumCls = 6
};
struct KernelTimer {
    bool on = false;
    cudaStream_t stream = nullptr;
    std::vector<cudaEvent_t> pool;
    struct Pair { int cls; int kb; cudaEvent_t a, b; double bytes; };
    std::vector<Pair> open;
    long long launches[kNumCls] = {};
    double ms[kNumCls] = {};
    double bytes[kNumCls] = {};
    static constexpr int kNumKBins = 5;   // K = 2, 4, 8, 16, other
    long long launches_k[kNumCls][kNumKBins] = {};
    double ms_k[kNumCls][kNumKBins] = {};
    double bytes_k[kNumCls][kNumKBins] = {};
    cudaEvent_t get();
    // events on the timer's stream, or on `s` for work launched on another
    // stream that the timer's stream joins before collect()
    int begin(int cls, double algorithmic_bytes, int K = 0, cudaStream_t s = nullptr);   // handle or -1
    void end(int handle, cudaStream_t s = nullptr);
    // algorithmic bytes of an interval whose work is only known after its
    // launches were issued (the PCG sweeps of a divergence correction)
    void set_bytes(int handle, double algorithmic_bytes);
    void collect();   // synchronises and folds finished pairs into the totals
    void reset();
    // pairs recorded inside a CUDA-graph capture: taken out of the open list
    // (they belong to the graph), folded into the totals after every replay
    // has finished, and their events returned when the graph is destroyed
    std::vector<Pair> take(size_t from);
    void fold(const std::vector<Pair>& ps);
    void release(std::vector<Pair>& ps);
    ~KernelTimer();
};

struct GcDev;   // gradient-space correction of the preconditioner (gradcorr.cuh)

// Everything one launch of the batched solver needs.
template <class R>
struct KrylovCtx {
    OpView<R> A;
    DiagView<R> D;
    BatchView B;
    std::vector<int> colour_ptr;     // [n_colours + 1] ranges of colour_list per colour
    const int* colour_list;          // device: 32-row slice ids grouped by colour, memory order inside
    int n_pad;
    int grid_vec;     // blocks for vector kernels with reductions
    int grid_spmv;    // blocks for SpMV kernels with reductions
    dev::RedScratch red;
    cudaStream_t stream;
    long long* launches;   // host counter of kernel launches
    KernelTimer* timer;    // may be null
    long nnz;              // true off-diagonal entries (algorithmic bytes)
    int n_rows;            // real edge rows
    int n_freq;            // distinct diagonals in use
    // slice-staged copy of A's off-diagonal part (see staged.cuh) and which
    // row kernels run: kRowsDirect (CSR rows read by the lanes) or
    // kRowsStaged (segments bulk-copied to shared memory)
    dev::SegView<R> seg;
    int row_kernels;
    // Eisenstat form of SSOR-BiCGStab (staged rows only): per-colour block
    // partial sums of the sweeps' dot products, summed by one reduction kernel
    double2* eis_partial = nullptr;   // [eis_slots][kMaxQ * kMaxRhs]
    int eis_slots = 0;
    // right-preconditioned form only (complex FP32): when set, each SSOR
    // apply is followed by the gradient-space term of the preconditioner
    const GcDev* gc = nullptr;
    // when set, the V-cycle runs on gc_stream, forked after the p / s update
    // and joined before the backward sweep, overlapping the forward sweep
    cudaStream_t gc_stream = nullptr;
    cudaEvent_t gc_fork = nullptr, gc_join = nullptr;
    // staged rows: each SSOR sweep as one cooperative launch over all sweep
    // groups (grid barriers between groups) instead of one launch per group
    int coop = 0;
    const int* colour_ptr_d = nullptr;   // device copy of colour_ptr
    unsigned* gridbar = nullptr;         // [2] barrier counter and generation
};

enum RowKernels : int { kRowsDirect = 0, kRowsStaged = 1 };

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
// SSOR apply plus the gradient-space term of c (if attached): out = B in
template <class R>
void precond_apply(const KrylovCtx<R>& c, const dev::cplx<R>* in, dev::cplx<R>* y, dev::cplx<R>* out);
template <class R>
void bicg_init(const KrylovCtx<R>& c, const KrylovVecs<R>& v, BicgState* st);
template <class R>
void bicg_iteration(const KrylovCtx<R>& c, const KrylovVecs<R>& v, BicgState* st);

// BiCGStab on the split-preconditioned operator A_hat = M1^-1 A M2^-1 of the
// SSOR splitting M = (D + L) D^-1 (D + U), M1 = (D + L) D^-1, M2 = D + U
// (S. C. Eisenstat, "Efficient implementation of a class of preconditioned
// conjugate gradient methods", SIAM J. Sci. Stat. Comput. 2 (1981)):
//   A_hat z = D (w + (D + L)^-1 (z - D w)),  w = (D + U)^-1 z,
// one backward and one forward sweep per application and no separate SpMV.
// eis_init: r = b_hat = D (D + L)^-1 b, r0 = r, x_hat = 0 (x must be zero);
// eis_iteration: one BiCGStab step on A_hat (x holds x_hat);
// eis_finish: out = M2^-1 x_hat = (D + U)^-1 x_hat, the correction in x-space.
template <class R>
void eis_init(const KrylovCtx<R>& c, const KrylovVecs<R>& v, BicgState* st);
template <class R>
void eis_iteration(const KrylovCtx<R>& c, const KrylovVecs<R>& v, BicgState* st);
template <class R>
void eis_finish(const KrylovCtx<R>& c, const KrylovVecs<R>& v, dev::cplx<R>* out);

}  // namespace m3d
