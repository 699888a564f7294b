// GpuSolver: host orchestration of the GB300 forward + adjoint solve behind
// the C ABI of include/m3d_gb300.h.
#pragma once

#include <cuda_runtime.h>

#include <complex>
#include <memory>
#include <functional>
#include <string>
#include <vector>

#include "m3d_gb300.h"
#include "host/amg.hpp"
#include "host/regularization.hpp"
#include "host/layout.hpp"
#include "cuda/krylov.cuh"
#include "cuda/physics.cuh"
#include "cuda/gradcorr.cuh"
#include "cuda/regularization.cuh"
#include "cuda/learned.cuh"

namespace m3d {

// One measured configuration of the autotuner: row-kernel layout, batch
// width K, milliseconds per FP32 BiCGStab iteration of the batch and per
// right-hand side.
struct TuneEntry {
    int row_kernels;
    int K;
    double ms_per_iter;
    double ms_per_rhs_iter;
};

struct BatchResult {
    int K = 0;
    std::vector<int> iters, status;
    std::vector<double> res, true_res;
};

class GpuSolver {
public:
    explicit GpuSolver(int device);
    ~GpuSolver();

    int device;
    std::string err;
    m3d_params P;
    bool ready = false;

    // ---- setup ----
    void setup(const m3d_leaves* leaves, const m3d_params* params);
    void set_sigma(const double* sigma, int n);
    void set_stations(const double* xyz, int n);

    // ---- per-frequency interface (IForwardSolver) ----
    void factorize(const std::vector<double>& freqs);
    void compute_single_frequency(double freq, double* Z_out);
    void background_E(int pol, double* out);
    void set_test_consume_no_wait(bool on);   // test hook of the staged kernels' error path
    // times the FP32 inner solve for each row-kernel layout and batch width
    // (<= max_K) at frequency freq and applies the fastest; drops the
    // factorisation and the resident fields
    std::vector<TuneEntry> autotune(double freq, int max_K, int reps);
    int rhs_block = 16;   // right-hand sides per batched solve of solve_rhs_batch

    // ---- learned preconditioner (no counterpart in the reference) ----
    // dense grid of 2^grid_level cells per axis, a `layers`-deep network of
    // `hidden` channels, room for max_samples training pairs
    void learn_setup(int grid_level, int layers, int hidden, unsigned seed, long max_samples);
    // plain FP64 SSOR-BiCGStab forward solves of freqs (current sigma),
    // recording training pairs; returns the pairs held
    long learn_collect(const double* freqs, int nf);
    // Adam epochs over the first (1 - val_frac) of the pairs; mean loss per
    // epoch, the held-out pairs' loss to *val_loss
    std::vector<double> learn_train(int epochs, float lr, int batch, unsigned seed, double val_frac,
                                    double* val_loss);
    long learn_samples() const { return ds_n; }
    bool learn_trained() const { return net_trained; }
    learn::Cnn* learn_net() { return net.get(); }
    void set_background(const double* E1, const double* E2);
    void build_adjoint_rhs(const double* wr, double* rhs1, double* rhs2);
    void adjoint_solve(const double* rhs, double* lam, bool perturbation);
    void sensitivity(const double* E, const double* lam, double* g);
    void perturbation_rhs(int pol, const double* dsig, double* out);
    void delta_impedance(const double* dE, int pol, double* dZ);
    void release();

    // ---- batched ----
    void forward_batch(const double* freqs, int nf, double* Z_out, double* E_out);
    void jtjv_batch(const double* freqs, int nf, const double* dsigma, const double* err, double inner_tol,
                    double* out);
    void solve_rhs_batch(const double* rhs, int n_rhs, double* out);
    void station_gradients(const double* wr, int n_src, double* g);
    // octree model regularisation (RegularizationOctree) on this mesh
    RegHost reg_host;
    RegDev reg{};
    bool reg_ok = false;
    std::vector<void*> reg_mem;
    double *d_reg_in = nullptr, *d_reg_out = nullptr, *d_reg_ref = nullptr;
    void reg_setup(const RegParams& p);
    void reg_free();
    void reg_apply(int op, const double* x, double* y);   // op 0: W^T W, 1: CmCm^T, 2: diagonal (x unused)
    void reg_evaluate(const double* params, const double* ref, double* value, double* grad);
    double2 *d_jtj_rhs = nullptr, *d_jtj_dE = nullptr, *d_jtj_a = nullptr, *d_jtj_b = nullptr;
    double2 *d_jtj_dz = nullptr, *d_jtj_wr0 = nullptr, *d_jtj_wr1 = nullptr;
    double* d_jtj_ds = nullptr;
    double* d_jtj_err = nullptr;
    void gradient_batch(const double* freqs, int nf, const double* obs, const double* err, double* Z_out,
                        double* grad);
    // batched Hermitian dot of caller-owned device vectors on the solver's
    // stream, with the reduction scratch allocated by setup
    void dot_batched(const double2* x, const double2* y, long long n, int K, double2* out);

    m3d_stats stats{};
    KernelTimer timer;
    // CUDA graphs of the mixed-precision inner solve's 10-iteration chunk, one
    // per batch shape of the running refinement step (destroyed at its end)
    struct ChunkGraph {
        int K = 0;
        const void* x = nullptr;   // the vector set the batch runs in
        bool eis = false, gc = false;
        cudaGraphExec_t exec = nullptr;
        long long launches = 0;    // kernel launches one replay issues
        std::vector<KernelTimer::Pair> pairs;
    };
    std::vector<ChunkGraph> chunk_graphs;
    bool graphs_failed = false;    // a capture failed: chunks run as direct launches from then on
    std::string graphs_error;
    long long graph_replays = 0;
    int chunk_graph(int K, const void* x, bool eis, bool gc, const std::function<void()>& body);
    void graphs_clear();
    cudaEvent_t ev_start = nullptr, ev_stop = nullptr;
    void timer_start();
    void begin_call();
    void end_call();
    double timer_stop();
    double tol_override = 0.0;
    double current_omega = 0.0;

    int n_edges() const { return L.ne; }
    int n_cells() const { return L.nc; }
    int n_stations() const { return sd.ns; }
    long nnz_off = 0;       // off-diagonal stiffness entries
    int n_nodes() const { return L.nn; }
    int n_colours() const { return (int)colour_ptr.size() - 1; }

private:
    HostLayout L;
    cudaStream_t stream = nullptr;
    long long launches = 0;

    // host-side structure
    std::vector<int> perm, iperm, colour_ptr, colour_list;
    int* d_colour_list = nullptr;
    int* d_colour_ptr = nullptr;        // device copy of colour_ptr (cooperative sweeps)
    unsigned* d_gridbar = nullptr;      // grid barrier of the cooperative sweeps
    std::vector<unsigned char> flags_ref;  // reference order
    int n_pad = 0, n_slices = 0;
    bool hp_sequential = false;

    // device mesh
    MeshDev md{};
    int *d_op_rp = nullptr, *d_op_rs = nullptr, *d_col = nullptr;
    double* d_val = nullptr;
    float* d_val32 = nullptr;
    // slice-staged segments of the same operator (staged.cuh), per precision
    unsigned char *d_seg64 = nullptr, *d_seg32 = nullptr;
    int4 *d_work64 = nullptr, *d_work32 = nullptr;   // [n_slices] natural order, then colour order
    dev::SegView<double> seg64{};
    dev::SegView<float> seg32{};
    unsigned* d_seg_err = nullptr;
    int4* d_lap_work = nullptr;   // node-Laplacian slice work items (dc.lap_work)
    // multigrid preconditioner of the divergence-correction PCG (rebuilt per sigma)
    std::vector<int> h_inc_ptr, h_inc_other;
    phys::AmgDev amg{};
    bool amg_ok = false;
    AmgHierarchy amg_host;          // kept between conductivity updates: aggregates are reused
    double* h_lap_pinned = nullptr; // pinned staging of the Laplacian read back for the host setup
    std::vector<int> a0_pos_q, a0_pos_d;   // incidence / diagonal -> position in the level-0 operator values
    CsrReal amg_pending_A0;         // level-0 operator waiting for a full build
    double amg_setup_ms = 0.0;      // host time of the last multigrid setup
    std::vector<void*> amg_mem;
    void build_amg();
    void free_amg();
    const phys::AmgDev* amg_or_null() const { return (amg_ok && P.divcorr_precond == 1) ? &amg : nullptr; }
    // gradient-space term of the FP32 inner solve's preconditioner, on the
    // same hierarchy (FP32 work vectors, masked transfer weights)
    GcDev gc{};
    bool gc_ok = false;
    std::vector<void*> gc_mem;
    void build_gc();
    cudaStream_t gc_stream = nullptr;
    cudaEvent_t gc_fork = nullptr, gc_join = nullptr;
    void attach_gc(KrylovCtx<float>& c);
    bool want_amg() const {
        return P.divcorr_precond == 1 || (P.precision == 1 && (P.gradcorr == 1 || P.divcorr_mixed == 1));
    }
    const GcDev* mixed_or_null() const {
        return (gc_ok && P.divcorr_mixed == 1 && P.divcorr_precond == 1 && P.precision == 1 && gc.dc_st) ? &gc
                                                                                                     : nullptr;
    }
    int* d_lap_qpos = nullptr;    // incidence -> value slot in dc.lap_seg
    void build_segments(const std::vector<int>& op_rp, const std::vector<int>& op_rs, const std::vector<int>& ecol,
                        const std::vector<double>& eval);
    void check_seg_err();

    // sigma
    std::vector<double> sigma_h;
    double *d_sigma = nullptr, *d_Me = nullptr, *d_me_dc = nullptr;
    bool have_sigma = false, lap_built = false;

    // factorised frequencies (diagonals)
    std::vector<double> fz_freqs;
    int diag_cap = 0;
    double2* d_diag = nullptr;    // [n_pad] (S_ii, Me_i) pairs, see phys::diag_coeffs
    float2* d_diag32 = nullptr;
    double* d_omegas = nullptr;

    // reductions
    dev::RedScratch red{};

    // Krylov work vectors for batches of up to 16 right-hand sides
    KrylovVecs<double> kv{};
    int kv_K = 0;
    KrylovVecs<float> kv32{};     // complex-FP32 inner solve of the mixed-precision path
    int kv32_K = 0;
    KrylovVecs<float> kv32b{};    // second set for repacking the batch to fewer lanes
    int kv32b_K = 0;
    int *d_lane_map = nullptr, *d_lane_add = nullptr, *d_lane_sel = nullptr;   // [16] lane maps
    double2* d_eis_partial = nullptr;   // block partial sums of the Eisenstat sweeps
    int eis_slots = 0;
    void ensure_vecs32b(int K);
    double* d_scale = nullptr;    // [16] per-rhs residual norms of the refinement step
    // fields of the last forward solve: [n_pad][Kf], rhs 2f+p
    double2* d_E = nullptr;
    int E_K = 0, E_nf = 0;
    double2 *d_Epri = nullptr, *d_Ebc = nullptr, *d_rhs = nullptr, *d_tmp = nullptr;
    double2* d_lam = nullptr;     // adjoint solutions
    double2* d_adj = nullptr;     // adjoint sources
    int fwd_cap = 0;
    int E_cap = 0;       // capacity (lanes) of d_E, grown only by its writers
    int jtj_ns = -1;     // station count the jtjv_batch station buffers were sized for
    double2* d_src_wr = nullptr;   // [8][ns][4] residuals of one batch of station sources
    double* d_src_g = nullptr;     // [8][nc] their gradients
    int src_ns = -1;               // station count d_src_wr was sized for

    // divergence correction
    phys::DcWork dc{};
    int dc_K = 0;

    // stations
    StationDev sd{};
    std::vector<int> st_cell;
    bool stations_set = false;
    HCache* d_hc = nullptr;
    double2 *d_Z = nullptr, *d_wr = nullptr, *d_obs = nullptr;
    double* d_err = nullptr;
    int hc_cap = 0, obs_cap = 0;
    double* d_grad = nullptr;
    double2* d_host_stage = nullptr;   // [ne] staging of host vectors
    double* d_stage_real = nullptr;    // [max(nc, ne)]
    BicgState* d_states = nullptr;     // [16] Krylov scalars of the running batch
    BicgState* d_states2 = nullptr;    // [16] true-residual checks of the outer loop

    // helpers
    void free_all();
    void upload_mesh();
    void ensure_sigma_device();
    void ensure_vecs(int K);
    void ensure_fields(int K);
    void ensure_E(int K);
    double divcorr_bytes(const phys::DcCounters& before, const phys::DcCounters& after, int K) const;
    double sens_bytes(int lanes) const;
    void ensure_dc(int K);
    void ensure_hc(int nf);
    KrylovCtx<double> kctx(int K, const int* fmap) const;
    KrylovCtx<float> kctx32(int K, const int* fmap) const;
    void ensure_vecs32(int K);
    // FP32 BiCGStab on the residual equation inside FP64 refinement
    BatchResult solve_batch_mixed(int K, const int* fmap, double2* b, double2* x, const std::vector<int>& active,
                                  double tol, int maxiter);
    // dispatch on P.precision
    BatchResult solve_any(int K, const int* fmap, double2* b, double2* x, const std::vector<int>& active,
                          double tol, int maxiter);
    RhsInfo rhs_info(int K, const std::vector<int>& f, const std::vector<int>& pol,
                     const std::vector<double>& freqs) const;
    BatchResult solve_batch(int K, const int* fmap, double2* b, double2* x, const std::vector<int>& active,
                            double tol, int maxiter);
    void run_forward(const std::vector<double>& freqs, double* Z_out);
    void run_adjoint(int K, const int* fmap, const RhsInfo& info, double2* rhs, double2* x,
                     const std::vector<int>& active);
    // solve_with_divcorr_ (forward_solver_fv.cpp:778-888) on a batch; fills
    // per-rhs iterations / status / true residual
    void solve_divcorr(int K, const int* fmap, const RhsInfo& info, double2* rhs, double2* x,
                       const std::vector<int>& active, double tol, std::vector<int>& iters,
                       std::vector<int>& status, std::vector<double>& tres);
    phys::DcCounters dcc;   // divergence-correction counters of the current call
    // learned preconditioner state (learned_solver.cu)
    std::unique_ptr<learn::Cnn> net;
    learn::GridMap gm{};
    int learn_level = 0;
    __nv_bfloat16* ds_feat = nullptr;   // [ds_cap][G^3][8] network inputs
    float* ds_tgt = nullptr;            // [ds_cap][G^3][6] targets
    long ds_n = 0, ds_cap = 0;
    float* lw_work = nullptr;           // grid means scratch [16][G^3][6] + 16
    double* d_lane_freq = nullptr;
    int* d_snap_lane = nullptr;
    long* d_snap_slot = nullptr;
    float* tr_target = nullptr;
    bool net_trained = false;
    bool collecting = false;
    struct Snap { int lane; long slot; };
    std::vector<Snap> pending;
    float2 *fg_V = nullptr, *fg_Z = nullptr, *fg_w = nullptr;
    double2 *fg_part = nullptr, *fg_h = nullptr;
    double *fg_inv = nullptr, *fg_scale = nullptr;
    int fg_cap_K = 0, fg_cap_m = 0;
    void learn_free();
    void learn_sigma_changed();
    void collect_snapshot(const double2* x, const double2* r, int K, const std::vector<BicgState>& hs,
                          const int* fmap);
    void collect_finish(const double2* x, int K);
    void net_apply(const KrylovCtx<float>& c32, const float2* v, float2* z, int K, const int* fmap);
    void ensure_fgmres(int K, int m);
    void fg_mdot(const float2* V, int nv, const float2* w, int K, std::vector<std::complex<double>>& h,
                 bool with_self = false);
    BatchResult solve_batch_fgmres(int K, const int* fmap, double2* b, double2* x, const std::vector<int>& active,
                                   double tol, int maxiter);
    void sync();
};

}  // namespace m3d
