// extern "C" boundary of include/m3d_gb300.h over GpuSolver.  Every entry
// point catches exceptions, maps them to an M3D_ERR_* code, records the
// message on the handle and synchronises before returning.
#include <cuda_runtime.h>

#include <cstring>
#include <algorithm>
#include <atomic>
#include <new>
#include <stdexcept>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "m3d_gb300.h"
#include "solver.hpp"

struct m3d_solver {
    m3d::GpuSolver* s = nullptr;
    std::string err;
};

namespace {

int fail(m3d_solver* h, int code, const std::string& msg) {
    if (h) h->err = msg;
    return code;
}

template <class F>
int guarded(m3d_solver* h, F&& f) {
    if (!h || !h->s) return M3D_ERR_ARG;
    try {
        f(*h->s);
        h->err.clear();
        return M3D_OK;
    } catch (const std::bad_alloc&) {
        cudaGetLastError();
        return fail(h, M3D_ERR_OOM, "allocation failed");
    } catch (const std::invalid_argument& e) {
        return fail(h, M3D_ERR_ARG, e.what());
    } catch (const std::logic_error& e) {
        return fail(h, M3D_ERR_STATE, e.what());
    } catch (const std::runtime_error& e) {
        return fail(h, M3D_ERR_CUDA, e.what());
    } catch (...) {
        return fail(h, M3D_ERR_CUDA, "unknown failure");
    }
}

bool ready(const m3d_solver* h) { return h && h->s && h->s->ready; }

// Inputs that enter a solve are checked on the host: a NaN or Inf in a
// right-hand side, field or data vector fails the call with M3D_ERR_NUMERIC
// before anything is launched (the reference would iterate on it to maxiter).
bool all_finite(const double* v, size_t n) {
    for (size_t i = 0; i < n; ++i)
        if (!std::isfinite(v[i])) return false;
    return true;
}

size_t edge_doubles(const m3d_solver* h) { return 2 * (size_t)h->s->n_edges(); }

}  // namespace

namespace m3d {
bool leaves_valid(const m3d_leaves* lv);
}

extern "C" void m3d_params_default(m3d_params* p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    // ForwardParamsFV defaults (include/maple3dmt/forward/forward_solver_fv.h:36-64)
    p->bicgstab_tol = 1e-7;
    p->bicgstab_maxiter = 2000;
    p->scattered_field = 1;
    p->air_z_threshold = 1.0;
    p->div_correction = 1;
    p->div_corr_iters = 10;
    p->div_corr_tol = 2e-3;
    p->divcorr_outer_max = 20;
    p->divcorr_iter_per_dc = 500;
    p->sigma_bg = 0.01;
    p->precision = 0;
    p->true_residual_check = 1;
    p->max_refinements = 3;
    p->print_level = 0;
    p->forward_interleaved = 0;
    p->row_kernels = 1;
    p->divcorr_precond = 1;
    p->ssor_form = 1;
    p->gradcorr = 1;
    p->gradcorr_fmax = 1e30;
    p->gradcorr_presmooth = 0;
    p->divcorr_mixed = 1;
    p->inner_tol_floor = 3e-5;
    p->residual_replacement = 0;
    p->gradcorr_overlap = 1;
    p->krylov = 0;
    p->fgmres_m = 20;
    p->learned_period = 2;
    p->sweep_rows = 0;
    p->coop_sweep = 0;
    p->cuda_graphs = 0;
    p->ssor_relax = 1.0;
}

extern "C" int m3d_solver_create(int device, m3d_solver** out) {
    if (!out) return M3D_ERR_ARG;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) {
        cudaGetLastError();
        return M3D_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= n) return M3D_ERR_ARG;
    auto* h = new (std::nothrow) m3d_solver;
    if (!h) return M3D_ERR_OOM;
    h->s = new (std::nothrow) m3d::GpuSolver(device);
    if (!h->s) { delete h; return M3D_ERR_OOM; }
    *out = h;
    return M3D_OK;
}

extern "C" void m3d_solver_destroy(m3d_solver* h) {
    if (!h) return;
    delete h->s;
    delete h;
}

extern "C" const char* m3d_last_error(const m3d_solver* h) { return h ? h->err.c_str() : "null handle"; }

extern "C" int m3d_solver_setup(m3d_solver* h, const m3d_leaves* leaves, const m3d_params* params) {
    if (!h || !m3d::leaves_valid(leaves) || !params) return fail(h, M3D_ERR_ARG, "invalid leaves or params");
    if (params->bicgstab_tol <= 0 || params->bicgstab_maxiter < 1 || params->divcorr_iter_per_dc < 1 ||
        params->sigma_bg <= 0 || params->precision < 0 || params->precision > 1 || params->row_kernels < 0 ||
        params->row_kernels > 1 || params->divcorr_precond < 0 || params->divcorr_precond > 1 ||
        params->ssor_form < 0 || params->ssor_form > 1 || params->gradcorr < 0 || params->gradcorr > 1 ||
        !(params->gradcorr_fmax >= 0.0) || params->gradcorr_presmooth < 0 || params->gradcorr_presmooth > 1 ||
        params->divcorr_mixed < 0 || params->divcorr_mixed > 1 || !(params->inner_tol_floor > 0.0) ||
        params->inner_tol_floor >= 1.0 || params->residual_replacement < 0 || params->residual_replacement > 1 ||
        params->gradcorr_overlap < 0 || params->gradcorr_overlap > 1 || params->krylov < 0 ||
        params->krylov > 1 || params->fgmres_m < 2 || params->fgmres_m > 47 || params->learned_period < 0 || params->sweep_rows < 0 ||
        params->coop_sweep < 0 || params->coop_sweep > 1 || params->cuda_graphs < 0 || params->cuda_graphs > 1 ||
        !(params->ssor_relax > 0.0 && params->ssor_relax < 2.0))
        return fail(h, M3D_ERR_ARG, "invalid solver parameters");
    return guarded(h, [&](m3d::GpuSolver& s) { s.setup(leaves, params); });
}

extern "C" int m3d_set_krylov(m3d_solver* h, int krylov, int fgmres_m, int learned_period) {
    if (!ready(h)) return fail(h, M3D_ERR_STATE, "solver not set up");
    if (krylov < 0 || krylov > 1 || fgmres_m < 2 || fgmres_m > 47 || learned_period < 0)
        return fail(h, M3D_ERR_ARG, "invalid Krylov settings");
    h->s->P.krylov = krylov;
    h->s->P.fgmres_m = fgmres_m;
    h->s->P.learned_period = learned_period;
    return M3D_OK;
}

extern "C" int m3d_solver_sizes(const m3d_solver* h, int* ne, int* nc, int* nn, int* ncol) {
    if (!ready(h)) return M3D_ERR_STATE;
    if (ne) *ne = h->s->n_edges();
    if (nc) *nc = h->s->n_cells();
    if (nn) *nn = h->s->n_nodes();
    if (ncol) *ncol = h->s->n_colours();
    return M3D_OK;
}

extern "C" int m3d_set_sigma(m3d_solver* h, const double* sigma, int n) {
    if (!ready(h)) return fail(h, M3D_ERR_STATE, "solver not set up");
    if (!sigma || n != h->s->n_cells()) return fail(h, M3D_ERR_ARG, "sigma must have n_cells entries");
    for (int i = 0; i < n; ++i)
        if (!(sigma[i] > 0.0) || !std::isfinite(sigma[i])) return fail(h, M3D_ERR_ARG, "sigma must be finite and > 0");
    return guarded(h, [&](m3d::GpuSolver& s) { s.set_sigma(sigma, n); });
}

extern "C" int m3d_set_stations(m3d_solver* h, const double* xyz, int n) {
    if (!ready(h)) return fail(h, M3D_ERR_STATE, "solver not set up");
    if (n < 1 || !xyz) return fail(h, M3D_ERR_ARG, "need at least one station");
    return guarded(h, [&](m3d::GpuSolver& s) { s.set_stations(xyz, n); });
}

extern "C" int m3d_set_tolerance_override(m3d_solver* h, double tol) {
    if (!ready(h)) return fail(h, M3D_ERR_STATE, "solver not set up");
    if (tol < 0) return fail(h, M3D_ERR_ARG, "tolerance must be >= 0");
    h->s->tol_override = tol;
    return M3D_OK;
}

extern "C" int m3d_current_omega(const m3d_solver* h, double* omega) {
    if (!h || !h->s || !omega) return M3D_ERR_ARG;
    *omega = h->s->current_omega;
    return M3D_OK;
}

extern "C" int m3d_compute_single_frequency(m3d_solver* h, double freq, double* Z_out) {
    if (!ready(h)) return fail(h, M3D_ERR_STATE, "solver not set up");
    if (!(freq > 0)) return fail(h, M3D_ERR_ARG, "frequency must be > 0");
    return guarded(h, [&](m3d::GpuSolver& s) { s.compute_single_frequency(freq, Z_out); });
}

extern "C" int m3d_factorize_frequency(m3d_solver* h, double freq) {
    if (!ready(h)) return fail(h, M3D_ERR_STATE, "solver not set up");
    if (!(freq > 0)) return fail(h, M3D_ERR_ARG, "frequency must be > 0");
    return guarded(h, [&](m3d::GpuSolver& s) { s.factorize(std::vector<double>{freq}); });
}

extern "C" int m3d_release_factorization(m3d_solver* h) {
    if (!ready(h)) return fail(h, M3D_ERR_STATE, "solver not set up");
    return guarded(h, [&](m3d::GpuSolver& s) { s.release(); });
}

extern "C" int m3d_background_E(m3d_solver* h, int pol, double* E_out) {
    if (!ready(h)) return fail(h, M3D_ERR_STATE, "solver not set up");
    if ((pol != 0 && pol != 1) || !E_out) return fail(h, M3D_ERR_ARG, "pol must be 0 or 1");
    return guarded(h, [&](m3d::GpuSolver& s) { s.background_E(pol, E_out); });
}

extern "C" int m3d_set_background_fields(m3d_solver* h, const double* E1, const double* E2) {
    if (!ready(h)) return fail(h, M3D_ERR_STATE, "solver not set up");
    if (!E1 || !E2) return fail(h, M3D_ERR_ARG, "null field");
    if (!all_finite(E1, edge_doubles(h)) || !all_finite(E2, edge_doubles(h)))
        return fail(h, M3D_ERR_NUMERIC, "non-finite value in a background field");
    return guarded(h, [&](m3d::GpuSolver& s) { s.set_background(E1, E2); });
}

extern "C" int m3d_build_adjoint_rhs(m3d_solver* h, const double* wr, double* rhs1, double* rhs2) {
    if (!ready(h)) return fail(h, M3D_ERR_STATE, "solver not set up");
    if (!wr || !rhs1 || !rhs2) return fail(h, M3D_ERR_ARG, "null buffer");
    if (!all_finite(wr, 8 * (size_t)h->s->n_stations()))
        return fail(h, M3D_ERR_NUMERIC, "non-finite value in the weighted residual");
    return guarded(h, [&](m3d::GpuSolver& s) { s.build_adjoint_rhs(wr, rhs1, rhs2); });
}

extern "C" int m3d_adjoint_solve(m3d_solver* h, const double* rhs, double* lambda) {
    if (!ready(h)) return fail(h, M3D_ERR_STATE, "solver not set up");
    if (!rhs || !lambda) return fail(h, M3D_ERR_ARG, "null buffer");
    if (!all_finite(rhs, edge_doubles(h))) return fail(h, M3D_ERR_NUMERIC, "non-finite value in the right-hand side");
    return guarded(h, [&](m3d::GpuSolver& s) { s.adjoint_solve(rhs, lambda, false); });
}

extern "C" int m3d_solve_rhs_batch(m3d_solver* h, const double* rhs, int n_rhs, double* out) {
    if (!ready(h)) return fail(h, M3D_ERR_STATE, "solver not set up");
    if (!rhs || !out || n_rhs < 1) return fail(h, M3D_ERR_ARG, "null buffer or no right-hand side");
    if (!all_finite(rhs, edge_doubles(h) * (size_t)n_rhs))
        return fail(h, M3D_ERR_NUMERIC, "non-finite value in a right-hand side");
    return guarded(h, [&](m3d::GpuSolver& s) { s.solve_rhs_batch(rhs, n_rhs, out); });
}

extern "C" int m3d_station_gradients(m3d_solver* h, const double* wr, int n_src, double* g) {
    if (!ready(h)) return fail(h, M3D_ERR_STATE, "solver not set up");
    if (n_src < 0 || (n_src > 0 && (!wr || !g))) return fail(h, M3D_ERR_ARG, "null buffer or n_src < 0");
    if (n_src > 0 && !all_finite(wr, (size_t)n_src * h->s->n_stations() * 8))
        return fail(h, M3D_ERR_NUMERIC, "non-finite value in a residual source");
    return guarded(h, [&](m3d::GpuSolver& s) { s.station_gradients(wr, n_src, g); });
}

extern "C" int m3d_group_station_gradients(m3d_solver* const* handles, int n_meshes, const double* freqs,
                                           const double* const* wr, const int* n_src, double* const* Z_out,
                                           double* const* g_out, int max_concurrent, int* status) {
    if (!handles || n_meshes < 1 || !freqs || !wr || !n_src || !g_out || !status) return M3D_ERR_ARG;
    for (int m = 0; m < n_meshes; ++m) status[m] = M3D_OK;
    for (int m = 0; m < n_meshes; ++m) {
        if (!ready(handles[m])) status[m] = fail(handles[m], M3D_ERR_STATE, "solver not set up");
        for (int q = 0; q < m; ++q)
            if (handles[q] == handles[m]) status[m] = fail(handles[m], M3D_ERR_ARG, "handle repeated in the group");
    }
    for (int m = 0; m < n_meshes; ++m)
        if (status[m] != M3D_OK) return status[m];
    // most stiffness entries first, so the long solves start early and the
    // small ones fill in behind them
    std::vector<int> order(n_meshes);
    for (int m = 0; m < n_meshes; ++m) order[m] = m;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        return handles[a]->s->nnz_off > handles[b]->s->nnz_off;
    });
    std::atomic<int> next{0};
    auto worker = [&]() {
        for (;;) {
            const int i = next.fetch_add(1);
            if (i >= n_meshes) return;
            const int m = order[i];
            m3d_solver* h = handles[m];
            if (cudaSetDevice(h->s->device) != cudaSuccess) {
                cudaGetLastError();
                status[m] = fail(h, M3D_ERR_CUDA, "cudaSetDevice failed");
                continue;
            }
            std::vector<double> z;
            double* zp = Z_out ? Z_out[m] : nullptr;
            if (!zp) {
                z.resize((size_t)std::max(1, h->s->n_stations()) * 8);
                zp = z.data();
            }
            int rc = m3d_compute_single_frequency(h, freqs[m], zp);
            if (rc == M3D_OK) rc = m3d_station_gradients(h, wr[m], n_src[m], g_out[m]);
            status[m] = rc;
        }
    };
    const int nw = max_concurrent > 0 ? std::min(max_concurrent, n_meshes) : n_meshes;
    std::vector<std::thread> pool;
    try {
        for (int w = 1; w < nw; ++w) pool.emplace_back(worker);
    } catch (...) {
        // fewer threads than asked: the ones started and this one share the work
    }
    worker();
    for (auto& t : pool) t.join();
    for (int m = 0; m < n_meshes; ++m)
        if (status[m] != M3D_OK) return status[m];
    return M3D_OK;
}

extern "C" int m3d_solve_rhs(m3d_solver* h, const double* rhs, double* x) {
    if (!ready(h)) return fail(h, M3D_ERR_STATE, "solver not set up");
    if (!rhs || !x) return fail(h, M3D_ERR_ARG, "null buffer");
    if (!all_finite(rhs, edge_doubles(h))) return fail(h, M3D_ERR_NUMERIC, "non-finite value in the right-hand side");
    return guarded(h, [&](m3d::GpuSolver& s) { s.adjoint_solve(rhs, x, true); });
}

extern "C" int m3d_compute_sensitivity(m3d_solver* h, const double* E, const double* lambda, double* g) {
    if (!ready(h)) return fail(h, M3D_ERR_STATE, "solver not set up");
    if (!E || !lambda || !g) return fail(h, M3D_ERR_ARG, "null buffer");
    if (!all_finite(E, edge_doubles(h)) || !all_finite(lambda, edge_doubles(h)))
        return fail(h, M3D_ERR_NUMERIC, "non-finite value in a field");
    return guarded(h, [&](m3d::GpuSolver& s) { s.sensitivity(E, lambda, g); });
}

extern "C" int m3d_build_perturbation_rhs(m3d_solver* h, int pol, const double* dsig, double* rhs) {
    if (!ready(h)) return fail(h, M3D_ERR_STATE, "solver not set up");
    if ((pol != 1 && pol != 2) || !dsig || !rhs) return fail(h, M3D_ERR_ARG, "pol must be 1 or 2");
    if (!all_finite(dsig, (size_t)h->s->n_cells())) return fail(h, M3D_ERR_NUMERIC, "non-finite value in dsigma");
    return guarded(h, [&](m3d::GpuSolver& s) { s.perturbation_rhs(pol, dsig, rhs); });
}

extern "C" int m3d_extract_delta_impedance(m3d_solver* h, const double* dE, int pol, double* dZ) {
    if (!ready(h)) return fail(h, M3D_ERR_STATE, "solver not set up");
    if ((pol != 1 && pol != 2) || !dE || !dZ) return fail(h, M3D_ERR_ARG, "pol must be 1 or 2");
    if (!all_finite(dE, edge_doubles(h))) return fail(h, M3D_ERR_NUMERIC, "non-finite value in dE");
    return guarded(h, [&](m3d::GpuSolver& s) { s.delta_impedance(dE, pol, dZ); });
}

extern "C" int m3d_forward_batch(m3d_solver* h, const double* freqs, int nf, double* Z_out, double* E_out) {
    if (!ready(h)) return fail(h, M3D_ERR_STATE, "solver not set up");
    if (!freqs || nf < 1) return fail(h, M3D_ERR_ARG, "need frequencies");
    for (int f = 0; f < nf; ++f) if (!(freqs[f] > 0)) return fail(h, M3D_ERR_ARG, "frequencies must be > 0");
    return guarded(h, [&](m3d::GpuSolver& s) { s.forward_batch(freqs, nf, Z_out, E_out); });
}

extern "C" int m3d_reg_setup(m3d_solver* h, const m3d_reg_params* p) {
    if (!ready(h)) return fail(h, M3D_ERR_STATE, "solver not set up");
    if (!p || p->n_smooth < 0) return fail(h, M3D_ERR_ARG, "invalid regularisation parameters");
    m3d::RegParams q;
    q.alpha_s = p->alpha_s; q.alpha_x = p->alpha_x; q.alpha_y = p->alpha_y; q.alpha_z = p->alpha_z;
    q.n_smooth = p->n_smooth;
    return guarded(h, [&](m3d::GpuSolver& s) { s.reg_setup(q); });
}

extern "C" int m3d_reg_num_active(const m3d_solver* h, int* n) {
    if (!ready(h) || !h->s->reg_ok) return M3D_ERR_STATE;
    if (!n) return M3D_ERR_ARG;
    *n = h->s->reg.na;
    return M3D_OK;
}

extern "C" int m3d_reg_active_to_global(const m3d_solver* h, int* a2g) {
    if (!ready(h) || !h->s->reg_ok) return M3D_ERR_STATE;
    if (!a2g) return M3D_ERR_ARG;
    const auto& v = h->s->reg_host.a2g;
    std::copy(v.begin(), v.end(), a2g);
    return M3D_OK;
}

extern "C" int m3d_reg_apply_wtw(m3d_solver* h, const double* x, double* y) {
    if (!ready(h)) return fail(h, M3D_ERR_STATE, "solver not set up");
    if (!x || !y) return fail(h, M3D_ERR_ARG, "null buffer");
    return guarded(h, [&](m3d::GpuSolver& s) { s.reg_apply(0, x, y); });
}

extern "C" int m3d_reg_apply_cmcmt(m3d_solver* h, const double* x, double* y) {
    if (!ready(h)) return fail(h, M3D_ERR_STATE, "solver not set up");
    if (!x || !y) return fail(h, M3D_ERR_ARG, "null buffer");
    return guarded(h, [&](m3d::GpuSolver& s) { s.reg_apply(1, x, y); });
}

extern "C" int m3d_reg_diagonal_wtw(m3d_solver* h, double* d) {
    if (!ready(h)) return fail(h, M3D_ERR_STATE, "solver not set up");
    if (!d) return fail(h, M3D_ERR_ARG, "null buffer");
    return guarded(h, [&](m3d::GpuSolver& s) { s.reg_apply(2, nullptr, d); });
}

extern "C" int m3d_reg_evaluate(m3d_solver* h, const double* params, const double* ref, double* value,
                                double* grad) {
    if (!ready(h)) return fail(h, M3D_ERR_STATE, "solver not set up");
    if (!params) return fail(h, M3D_ERR_ARG, "null buffer");
    return guarded(h, [&](m3d::GpuSolver& s) { s.reg_evaluate(params, ref, value, grad); });
}

extern "C" int m3d_jtjv_batch(m3d_solver* h, const double* freqs, int nf, const double* dsigma,
                              const double* obs_err, double inner_tol, double* out) {
    if (!ready(h)) return fail(h, M3D_ERR_STATE, "solver not set up");
    if (!freqs || nf < 1 || !dsigma || !obs_err || !out) return fail(h, M3D_ERR_ARG, "null buffer");
    if (nf > 8) return fail(h, M3D_ERR_ARG, "at most 8 frequencies per call");
    if (!(inner_tol > 0.0) || inner_tol >= 1.0) return fail(h, M3D_ERR_ARG, "inner_tol must be in (0, 1)");
    for (int f = 0; f < nf; ++f) if (!(freqs[f] > 0)) return fail(h, M3D_ERR_ARG, "frequencies must be > 0");
    if (!all_finite(dsigma, (size_t)h->s->n_cells()) || !all_finite(obs_err, 4 * (size_t)h->s->n_stations() * nf))
        return fail(h, M3D_ERR_NUMERIC, "non-finite value in dsigma or the data errors");
    return guarded(h, [&](m3d::GpuSolver& s) { s.jtjv_batch(freqs, nf, dsigma, obs_err, inner_tol, out); });
}

extern "C" int m3d_gradient_batch(m3d_solver* h, const double* freqs, int nf, const double* obs_Z,
                                  const double* obs_err, double* Z_out, double* grad) {
    if (!ready(h)) return fail(h, M3D_ERR_STATE, "solver not set up");
    if (!freqs || nf < 1 || !obs_Z || !obs_err || !grad) return fail(h, M3D_ERR_ARG, "null buffer");
    for (int f = 0; f < nf; ++f) if (!(freqs[f] > 0)) return fail(h, M3D_ERR_ARG, "frequencies must be > 0");
    const size_t nd = 4 * (size_t)h->s->n_stations() * nf;
    if (!all_finite(obs_Z, 2 * nd) || !all_finite(obs_err, nd))
        return fail(h, M3D_ERR_NUMERIC, "non-finite value in the observed data or errors");
    return guarded(h, [&](m3d::GpuSolver& s) { s.gradient_batch(freqs, nf, obs_Z, obs_err, Z_out, grad); });
}

extern "C" int m3d_dot_batched(m3d_solver* h, const double* x, const double* y, long long n, int K,
                               double* out) {
    if (!ready(h)) return fail(h, M3D_ERR_STATE, "solver not set up");
    if (K != 1 && K != 2 && K != 4 && K != 8 && K != 16)
        return fail(h, M3D_ERR_ARG, "K must be 1, 2, 4, 8 or 16");
    if (n < 0 || !out || (n > 0 && (!x || !y))) return fail(h, M3D_ERR_ARG, "invalid vectors");
    return guarded(h, [&](m3d::GpuSolver& s) {
        s.dot_batched(reinterpret_cast<const double2*>(x), reinterpret_cast<const double2*>(y), n, K,
                      reinterpret_cast<double2*>(out));
    });
}

extern "C" int m3d_get_stats(const m3d_solver* h, m3d_stats* out) {
    if (!h || !h->s || !out) return M3D_ERR_ARG;
    *out = h->s->stats;
    return M3D_OK;
}

extern "C" int m3d_timer_start(m3d_solver* h) {
    if (!ready(h)) return fail(h, M3D_ERR_STATE, "solver not set up");
    return guarded(h, [&](m3d::GpuSolver& s) { s.timer_start(); });
}

extern "C" int m3d_timer_stop(m3d_solver* h, double* ms) {
    if (!ready(h)) return fail(h, M3D_ERR_STATE, "solver not set up");
    if (!ms) return fail(h, M3D_ERR_ARG, "null output");
    return guarded(h, [&](m3d::GpuSolver& s) { *ms = s.timer_stop(); });
}

extern "C" int m3d_set_kernel_timing(m3d_solver* h, int on) {
    if (!ready(h)) return fail(h, M3D_ERR_STATE, "solver not set up");
    return guarded(h, [&](m3d::GpuSolver& s) { s.timer.reset(); s.timer.on = on != 0; });
}

namespace {
struct TuneKey {
    int ne;
    long long nnz;
    int max_K, gradcorr, device;
    bool operator<(const TuneKey& o) const {
        return std::tie(ne, nnz, max_K, gradcorr, device) < std::tie(o.ne, o.nnz, o.max_K, o.gradcorr, o.device);
    }
};
struct TuneChoice {
    std::vector<m3d::TuneEntry> table;
    int row_kernels, rhs_block;
};
std::mutex g_tune_mu;
std::map<TuneKey, TuneChoice> g_tune_cache;
}  // namespace

extern "C" int m3d_autotune(m3d_solver* h, double freq, int max_K, int reps, int force, m3d_tune_entry* table,
                            int* n_entries, int* row_kernels, int* rhs_block, int* cached) {
    if (!ready(h)) return fail(h, M3D_ERR_STATE, "solver not set up");
    if (!(freq > 0) || max_K < 2 || max_K > 16 || reps < 1) return fail(h, M3D_ERR_ARG, "invalid tuning arguments");
    return guarded(h, [&](m3d::GpuSolver& s) {
        const TuneKey key{s.n_edges(), s.nnz_off, max_K, s.P.gradcorr, s.device};
        TuneChoice ch;
        bool hit = false;
        {
            std::lock_guard<std::mutex> lock(g_tune_mu);
            auto it = g_tune_cache.find(key);
            if (it != g_tune_cache.end() && !force) { ch = it->second; hit = true; }
        }
        if (hit) {
            s.P.row_kernels = ch.row_kernels;
            s.rhs_block = ch.rhs_block;
        } else {
            ch.table = s.autotune(freq, max_K, reps);
            ch.row_kernels = s.P.row_kernels;
            ch.rhs_block = s.rhs_block;
            std::lock_guard<std::mutex> lock(g_tune_mu);
            g_tune_cache[key] = ch;
        }
        const int n = std::min<int>((int)ch.table.size(), 8);
        for (int i = 0; i < n && table; ++i)
            table[i] = m3d_tune_entry{ch.table[i].row_kernels, ch.table[i].K, ch.table[i].ms_per_iter,
                                      ch.table[i].ms_per_rhs_iter};
        if (n_entries) *n_entries = n;
        if (row_kernels) *row_kernels = ch.row_kernels;
        if (rhs_block) *rhs_block = ch.rhs_block;
        if (cached) *cached = hit ? 1 : 0;
    });
}

extern "C" int m3d_learn_setup(m3d_solver* h, int grid_level, int layers, int hidden, unsigned seed,
                               long long max_samples) {
    if (!ready(h)) return fail(h, M3D_ERR_STATE, "solver not set up");
    if (layers < 2 || hidden < 1 || hidden > 32 || max_samples < 1) return fail(h, M3D_ERR_ARG, "invalid network");
    return guarded(h, [&](m3d::GpuSolver& s) { s.learn_setup(grid_level, layers, hidden, seed, (long)max_samples); });
}

extern "C" int m3d_learn_collect(m3d_solver* h, const double* freqs, int nf, long long* n_samples) {
    if (!ready(h)) return fail(h, M3D_ERR_STATE, "solver not set up");
    if (!freqs || nf < 1) return fail(h, M3D_ERR_ARG, "need frequencies");
    for (int f = 0; f < nf; ++f) if (!(freqs[f] > 0)) return fail(h, M3D_ERR_ARG, "frequencies must be > 0");
    return guarded(h, [&](m3d::GpuSolver& s) {
        const long n = s.learn_collect(freqs, nf);
        if (n_samples) *n_samples = n;
    });
}

extern "C" int m3d_learn_train(m3d_solver* h, int epochs, float lr, int batch, unsigned seed, double val_frac,
                               double* epoch_loss, double* val_loss) {
    if (!ready(h)) return fail(h, M3D_ERR_STATE, "solver not set up");
    if (epochs < 1 || !(lr > 0.0f) || batch < 1 || val_frac < 0.0 || val_frac >= 1.0)
        return fail(h, M3D_ERR_ARG, "invalid training arguments");
    return guarded(h, [&](m3d::GpuSolver& s) {
        const std::vector<double> hist = s.learn_train(epochs, lr, batch, seed, val_frac, val_loss);
        if (epoch_loss) std::copy(hist.begin(), hist.end(), epoch_loss);
    });
}

extern "C" int m3d_test_set_consume_no_wait(m3d_solver* h, int on) {
    if (!ready(h)) return fail(h, M3D_ERR_STATE, "solver not set up");
    return guarded(h, [&](m3d::GpuSolver& s) { s.set_test_consume_no_wait(on != 0); });
}

extern "C" int m3d_get_kernel_times(m3d_solver* h, m3d_kernel_times* out) {
    if (!ready(h)) return fail(h, M3D_ERR_STATE, "solver not set up");
    if (!out) return fail(h, M3D_ERR_ARG, "null output");
    return guarded(h, [&](m3d::GpuSolver& s) {
        s.timer.collect();
        for (int i = 0; i < m3d::kNumCls; ++i) {
            out->launches[i] = s.timer.launches[i];
            out->ms[i] = s.timer.ms[i];
            out->bytes[i] = s.timer.bytes[i];
            for (int j = 0; j < 5; ++j) {
                out->launches_k[i][j] = s.timer.launches_k[i][j];
                out->ms_k[i][j] = s.timer.ms_k[i][j];
                out->bytes_k[i][j] = s.timer.bytes_k[i][j];
            }
        }
    });
}
