// C++ host face of the GB300 solver with the method set of the reference's
// maple3dmt::forward::IForwardSolver (include/maple3dmt/forward/iforward_solver.h:31-115)
// and the concrete setup / set_sigma of ForwardSolverFV
// (include/maple3dmt/forward/forward_solver_fv.h:82-86), implemented over the C ABI
// of m3d_gb300.h.  Header-only; link against libm3d_gb300.so.
//
// Types follow the reference: ComplexVec = std::vector<std::complex<double>>,
// RealVec = std::vector<double>, per-station residual / delta-Z arrays of
// std::array<Complex, 4> ordered xx, xy, yx, yy; polarisation index 0/1 for
// background_E and 1/2 for the perturbation calls (forward_solver_fv.cpp:952,2049).
//
// Error behaviour: the reference logs failures and returns; this class throws
// m3d::SolverError carrying the M3D_ERR_* code and message instead, because a
// device failure must not be mistaken for a converged solve.  Non-convergence
// is reported through last_stats(), as the reference's BiCGStabResult is.
#pragma once

#include <array>
#include <complex>
#include <stdexcept>
#include <string>
#include <vector>

#include "m3d_gb300.h"

namespace m3d {

using Complex = std::complex<double>;
using ComplexVec = std::vector<Complex>;
using RealVec = std::vector<double>;

class SolverError : public std::runtime_error {
public:
    SolverError(int code, const std::string& msg) : std::runtime_error(msg), code(code) {}
    int code;
};

class GpuForwardSolverFV {
public:
    explicit GpuForwardSolverFV(int device = 0) {
        check(m3d_solver_create(device, &h_), "m3d_solver_create");
    }
    ~GpuForwardSolverFV() { m3d_solver_destroy(h_); }
    GpuForwardSolverFV(const GpuForwardSolverFV&) = delete;
    GpuForwardSolverFV& operator=(const GpuForwardSolverFV&) = delete;

    // ForwardSolverFV::setup(mesh, params): the mesh as its finished leaf list.
    void setup(const m3d_leaves& leaves, const m3d_params& params) {
        check(m3d_solver_setup(h_, &leaves, &params), "setup");
        check(m3d_solver_sizes(h_, &ne_, &nc_, nullptr, nullptr), "sizes");
    }
    void set_sigma(const RealVec& sigma) { check(m3d_set_sigma(h_, sigma.data(), (int)sigma.size()), "set_sigma"); }
    // find_stations_ input (station x, y, z of the observed data)
    void set_stations(const std::vector<std::array<double, 3>>& xyz) {
        ns_ = (int)xyz.size();
        check(m3d_set_stations(h_, &xyz[0][0], ns_), "set_stations");
    }

    // ---- IForwardSolver ----
    // compute_single_frequency: returns Z [station] {xx, xy, yx, yy}
    std::vector<std::array<Complex, 4>> compute_single_frequency(double freq_hz) {
        std::vector<std::array<Complex, 4>> Z(ns_);
        check(m3d_compute_single_frequency(h_, freq_hz, reinterpret_cast<double*>(Z.data())), "forward");
        return Z;
    }
    // compute_responses: every frequency, Z [freq][station]
    std::vector<std::vector<std::array<Complex, 4>>> compute_responses(const RealVec& freqs) {
        std::vector<std::array<Complex, 4>> flat(freqs.size() * ns_);
        check(m3d_forward_batch(h_, freqs.data(), (int)freqs.size(), reinterpret_cast<double*>(flat.data()), nullptr),
              "forward_batch");
        std::vector<std::vector<std::array<Complex, 4>>> Z(freqs.size());
        for (size_t f = 0; f < freqs.size(); ++f) Z[f].assign(flat.begin() + f * ns_, flat.begin() + (f + 1) * ns_);
        return Z;
    }
    void factorize_frequency(double freq_hz) { check(m3d_factorize_frequency(h_, freq_hz), "factorize"); }
    void release_factorization() { check(m3d_release_factorization(h_), "release"); }
    int num_elements() const { return nc_; }
    double current_omega() const {
        double w = 0;
        m3d_current_omega(h_, &w);
        return w;
    }
    void build_adjoint_rhs_from_residual(const std::vector<std::array<Complex, 4>>& wr, ComplexVec& rhs1,
                                         ComplexVec& rhs2) {
        rhs1.assign(ne_, Complex(0, 0));
        rhs2.assign(ne_, Complex(0, 0));
        check(m3d_build_adjoint_rhs(h_, reinterpret_cast<const double*>(wr.data()), d(rhs1), d(rhs2)), "adjoint rhs");
    }
    void adjoint_solve_complex(const ComplexVec& rhs, ComplexVec& lambda) {
        lambda.assign(ne_, Complex(0, 0));
        check(m3d_adjoint_solve(h_, cd(rhs), d(lambda)), "adjoint solve");
    }
    void compute_sensitivity_complex(const ComplexVec& E, const ComplexVec& lambda, RealVec& g) {
        g.assign(nc_, 0.0);
        check(m3d_compute_sensitivity(h_, cd(E), cd(lambda), g.data()), "sensitivity");
    }
    void build_perturbation_rhs_complex(int pol, const RealVec& delta_sigma, ComplexVec& rhs) {
        rhs.assign(ne_, Complex(0, 0));
        check(m3d_build_perturbation_rhs(h_, pol, delta_sigma.data(), d(rhs)), "perturbation rhs");
    }
    void solve_rhs_complex(const ComplexVec& rhs, ComplexVec& x) {
        x.assign(ne_, Complex(0, 0));
        check(m3d_solve_rhs(h_, cd(rhs), d(x)), "solve rhs");
    }
    void extract_delta_impedance_complex(const ComplexVec& dE, int pol, std::vector<std::array<Complex, 4>>& dZ) {
        dZ.assign(ns_, {});
        check(m3d_extract_delta_impedance(h_, cd(dE), pol, reinterpret_cast<double*>(dZ.data())), "delta Z");
    }
    ComplexVec background_E(int pol) const {
        ComplexVec E(ne_);
        check(m3d_background_E(h_, pol, reinterpret_cast<double*>(E.data())), "background_E");
        return E;
    }
    void set_background_fields_complex(const ComplexVec& E1, const ComplexVec& E2) {
        check(m3d_set_background_fields(h_, cd(E1), cd(E2)), "set_background_fields");
    }
    void set_solver_tolerance_override(double tol) { check(m3d_set_tolerance_override(h_, tol), "tol override"); }

    // ---- batched gradient (InversionFV::compute_gradient_ for all frequencies) ----
    // obs / err: [station][freq][4]; returns the gradient over cells
    RealVec gradient(const RealVec& freqs, const std::vector<Complex>& obs, const RealVec& err,
                     std::vector<std::array<Complex, 4>>* Z_out = nullptr) {
        RealVec g(nc_, 0.0);
        std::vector<std::array<Complex, 4>> Z(freqs.size() * ns_);
        check(m3d_gradient_batch(h_, freqs.data(), (int)freqs.size(), cd(obs), err.data(),
                                 reinterpret_cast<double*>(Z.data()), g.data()), "gradient");
        if (Z_out) *Z_out = std::move(Z);
        return g;
    }

    // ---- per-source gradients at the solved frequency (one row of J^T W^2 r per station source) ----
    // wr: [source][station] residual weights; returns [source][cell]
    std::vector<RealVec> station_gradients(const std::vector<std::vector<std::array<Complex, 4>>>& wr) {
        const int n = (int)wr.size();
        std::vector<std::array<Complex, 4>> flat;
        flat.reserve((size_t)n * ns_);
        for (const auto& w : wr) {
            if ((int)w.size() != ns_) throw SolverError(M3D_ERR_ARG, "station_gradients: one entry per station");
            flat.insert(flat.end(), w.begin(), w.end());
        }
        RealVec g((size_t)n * nc_, 0.0);
        check(m3d_station_gradients(h_, reinterpret_cast<const double*>(flat.data()), n, g.data()),
              "station_gradients");
        std::vector<RealVec> out(n);
        for (int j = 0; j < n; ++j) out[j].assign(g.begin() + (size_t)j * nc_, g.begin() + (size_t)(j + 1) * nc_);
        return out;
    }

    // ---- GN-CG J^T W^2 J v (ImplicitJtJOperatorFV::Mult, data term) ----
    // after forward_batch(freqs) (the cached background fields); err: [station][freq][4]
    RealVec jtjv(const RealVec& freqs, const RealVec& dsigma, const RealVec& err, double inner_tol = 1e-4) {
        RealVec y(nc_, 0.0);
        check(m3d_jtjv_batch(h_, freqs.data(), (int)freqs.size(), dsigma.data(), err.data(), inner_tol, y.data()),
              "jtjv");
        return y;
    }

    // ---- octree regularisation (RegularizationOctree) ----
    int reg_setup(double alpha_s, double alpha_x, double alpha_y, double alpha_z, int n_smooth) {
        m3d_reg_params p{alpha_s, alpha_x, alpha_y, alpha_z, n_smooth};
        check(m3d_reg_setup(h_, &p), "reg_setup");
        int n = 0;
        check(m3d_reg_num_active(h_, &n), "reg_num_active");
        n_active_ = n;
        return n;
    }
    RealVec reg_apply_WtW(const RealVec& x) {
        RealVec y(n_active_, 0.0);
        check(m3d_reg_apply_wtw(h_, x.data(), y.data()), "reg_apply_wtw");
        return y;
    }
    RealVec reg_apply_CmCmT(const RealVec& x) {
        RealVec y(n_active_, 0.0);
        check(m3d_reg_apply_cmcmt(h_, x.data(), y.data()), "reg_apply_cmcmt");
        return y;
    }
    // ln(sigma) per cell; ref per active cell (empty: zero); returns the objective, fills grad [n_cells]
    double reg_evaluate(const RealVec& log_sigma, const RealVec& ref, RealVec* grad = nullptr) {
        double v = 0.0;
        if (grad) grad->assign(nc_, 0.0);
        check(m3d_reg_evaluate(h_, log_sigma.data(), ref.empty() ? nullptr : ref.data(), &v,
                               grad ? grad->data() : nullptr), "reg_evaluate");
        return v;
    }

    m3d_stats last_stats() const {
        m3d_stats s{};
        m3d_get_stats(h_, &s);
        return s;
    }
    int num_edges() const { return ne_; }

private:
    m3d_solver* h_ = nullptr;
    int ne_ = 0, nc_ = 0, ns_ = 0, n_active_ = 0;
    static double* d(ComplexVec& v) { return reinterpret_cast<double*>(v.data()); }
    static const double* cd(const ComplexVec& v) { return reinterpret_cast<const double*>(v.data()); }
    void check(int rc, const char* what) const {
        if (rc != M3D_OK) throw SolverError(rc, std::string(what) + ": " + m3d_last_error(h_));
    }
};

}  // namespace m3d
