// Oracle driver around the reference's OWN solver sources (compiled
// unmodified from the reference tree by oracle/build_ref.sh into oracle/_ref).
// TEST INFRASTRUCTURE ONLY: it generates golden vectors and pins the C
// restatement in oracle/m3d_oracle.c; nothing in the product links it.
//
// The driver follows the caller sequence of the reference:
//   ForwardSolverFV::setup / set_sigma          (src/forward/forward_solver_fv.cpp:28-51)
//   compute_single_frequency per frequency      (:1732-1738)
//   weighted residual, adjoint RHS, 2 adjoint solves, 2 sensitivities, sum
//                                               (src/inversion/inversion_fv.cpp:250-291)
// and dumps the staggered grid / operator layout, A (before BC elimination),
// E1/E2, Z, the adjoint RHS, lambda and the gradient as named arrays.
#include "maple3dmt/octree/octree_mesh.h"
#include "maple3dmt/octree/staggered_grid.h"
#include "maple3dmt/octree/operators.h"
#include "maple3dmt/forward/forward_solver_fv.h"
#include "maple3dmt/inversion/regularization_octree.h"
#include "maple3dmt/data/mt_data.h"
#include "maple3dmt/utils/logger.h"

#include "m3d_case.h"

#include <cstdio>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

using namespace maple3dmt;

namespace maple3dmt {
namespace octree {

OctreeMesh::OctreeMesh() = default;
OctreeMesh::~OctreeMesh() = default;

void OctreeMesh::load_leaves(const RefinementParams& params, int n_cells,
                             const int* level, const Real* cx, const Real* cy,
                             const Real* cz, const int* cell_type) {
    params_ = params;
    num_cells_ = n_cells;
    cx_.assign(cx, cx + n_cells);
    cy_.assign(cy, cy + n_cells);
    cz_.assign(cz, cz + n_cells);
    level_.assign(level, level + n_cells);
    type_.resize(n_cells);
    for (int i = 0; i < n_cells; ++i) type_[i] = static_cast<CellType>(cell_type[i]);
}

// octree_mesh.cpp:560 (cell_sizes_ = h_unit * min(dx, dy, dz)) and :577-590
Real OctreeMesh::cell_size(int local_id) const {
    Real dx = params_.domain_x_max - params_.domain_x_min;
    Real dy = params_.domain_y_max - params_.domain_y_min;
    Real dz = params_.domain_z_max - params_.domain_z_min;
    Real h_unit = (Real)(1 << (19 - level_[local_id])) / (Real)(1 << 19);
    return h_unit * std::min({dx, dy, dz});
}

void OctreeMesh::cell_size_xyz(int local_id, Real& dx, Real& dy, Real& dz) const {
    int level = level_[local_id];
    Real h_unit = 1.0 / (1 << level);
    dx = h_unit * (params_.domain_x_max - params_.domain_x_min);
    dy = h_unit * (params_.domain_y_max - params_.domain_y_min);
    dz = h_unit * (params_.domain_z_max - params_.domain_z_min);
}

void OctreeMesh::build_staggered_grid() {
    staggered_ = std::make_unique<StaggeredGrid>();
    staggered_->build(*this);
}

}  // namespace octree
}  // namespace maple3dmt

namespace {

struct Writer {
    FILE* f = nullptr;
    explicit Writer(const char* path) {
        f = std::fopen(path, "wb");
        if (f) std::fwrite("M3DA1\0\0\0", 1, 8, f);
    }
    ~Writer() { if (f) std::fclose(f); }
    void put(const std::string& name, char dt, const void* data, uint64_t count, size_t esz) {
        uint32_t n = (uint32_t)name.size();
        std::fwrite(&n, 4, 1, f);
        std::fwrite(name.data(), 1, n, f);
        std::fwrite(&dt, 1, 1, f);
        std::fwrite(&count, 8, 1, f);
        if (count) std::fwrite(data, esz, count, f);
    }
    void d(const std::string& n, const std::vector<double>& v) { put(n, 'f', v.data(), v.size(), 8); }
    void i(const std::string& n, const std::vector<int>& v) { put(n, 'i', v.data(), v.size(), 4); }
    void c(const std::string& n, const std::vector<Complex>& v) { put(n, 'c', v.data(), v.size(), 16); }
};

}  // namespace

extern "C" int ref_run(const m3d_case* cs, const char* out_path, int flags, int log_level) {
    utils::Logger::instance().set_level(static_cast<utils::LogLevel>(log_level));

    octree::RefinementParams rp;
    rp.domain_x_min = cs->domain[0]; rp.domain_x_max = cs->domain[1];
    rp.domain_y_min = cs->domain[2]; rp.domain_y_max = cs->domain[3];
    rp.domain_z_min = cs->domain[4]; rp.domain_z_max = cs->domain[5];
    rp.min_level = cs->min_level;
    rp.max_level = cs->max_level;
    rp.sigma_bg = cs->sigma_bg;

    octree::OctreeMesh mesh;
    mesh.load_leaves(rp, cs->n_cells, cs->level, cs->cx, cs->cy, cs->cz, cs->cell_type);
    mesh.build_staggered_grid();

    Writer w(out_path);
    if (!w.f) return 1;

    if (flags & 8) {
        // RegularizationOctree (src/inversion/regularization_octree.cpp:24-286) with
        // fixed parameters: alpha_s 1.5, alpha_x 1.0, alpha_y 0.8, alpha_z 0.5,
        // n_smooth 2; test vector x_j = sin(0.37 j) + j / n_active; model
        // params = ln(sigma), reference model ln(0.01) on every active cell.
        inversion::RegParamsOctree rg;
        rg.alpha_s = 1.5; rg.alpha_x = 1.0; rg.alpha_y = 0.8; rg.alpha_z = 0.5; rg.n_smooth = 2;
        inversion::RegularizationOctree reg;
        reg.setup(mesh, rg);
        const int na = reg.n_active();
        std::vector<int> a2g(reg.active_to_global().begin(), reg.active_to_global().end());
        RealVec x(na), wx, cx, dg;
        for (int j = 0; j < na; ++j) x[j] = std::sin(0.37 * j) + (double)j / na;
        reg.apply_WtW(x, wx);
        reg.apply_CmCmT(x, cx);
        reg.diagonal_WtW(dg);
        model::ConductivityModel m;
        m.init_3d(cs->n_cells, cs->sigma_bg);
        for (int c = 0; c < cs->n_cells; ++c) m.params()[c] = std::log(cs->sigma[c]);
        reg.set_reference_model(RealVec(na, std::log(0.01)));
        RealVec gr;
        reg.gradient(m, gr);
        w.i("reg_a2g", a2g); w.d("reg_x", x); w.d("reg_wtw_x", wx); w.d("reg_cmcm_x", cx);
        w.d("reg_diag", dg); w.d("reg_eval", std::vector<double>{reg.evaluate(m)}); w.d("reg_grad", gr);
        if (!(flags & 7)) return 0;
    }

    forward::ForwardParamsFV fp;
    fp.bicgstab_tol = cs->bicgstab_tol;
    fp.bicgstab_maxiter = cs->bicgstab_maxiter;
    fp.print_level = 1;
    fp.scattered_field = cs->scattered_field != 0;
    fp.air_z_threshold = cs->air_z_threshold;
    fp.div_correction = cs->div_correction != 0;
    fp.div_corr_iters = cs->div_corr_iters;
    fp.div_corr_tol = cs->div_corr_tol;
    fp.divcorr_outer_max = cs->divcorr_outer_max;
    fp.divcorr_iter_per_dc = cs->divcorr_iter_per_dc;

    forward::ForwardSolverFV fwd;
    fwd.setup(mesh, fp);
    RealVec sigma(cs->sigma, cs->sigma + cs->n_cells);
    fwd.set_sigma(sigma);

    const auto& sg = mesh.staggered();
    const int ne = sg.num_edges();
    const int nc = sg.num_cells();

    if (flags & 1) {
        // Staggered grid and operator layout.
        std::vector<double> exyz(3 * ne), elen(ne);
        std::vector<int> edir(ne), eadj_ptr(ne + 1, 0), eadj;
        for (int e = 0; e < ne; ++e) {
            const auto& ei = sg.edge(e);
            exyz[3 * e] = ei.x; exyz[3 * e + 1] = ei.y; exyz[3 * e + 2] = ei.z;
            elen[e] = ei.length; edir[e] = ei.direction;
            for (int c : ei.adj_cells) eadj.push_back(c);
            eadj_ptr[e + 1] = (int)eadj.size();
        }
        w.d("edge_xyz", exyz); w.d("edge_len", elen); w.i("edge_dir", edir);
        w.i("edge_adj_ptr", eadj_ptr); w.i("edge_adj", eadj);
        const int nf = sg.num_faces();
        std::vector<double> fxyz(3 * nf), farea(nf);
        std::vector<int> fnorm(nf), fcm(nf), fcp(nf), fe_ptr(nf + 1, 0), fe;
        for (int f = 0; f < nf; ++f) {
            const auto& fi = sg.face(f);
            fxyz[3 * f] = fi.x; fxyz[3 * f + 1] = fi.y; fxyz[3 * f + 2] = fi.z;
            farea[f] = fi.area; fnorm[f] = fi.normal; fcm[f] = fi.cell_minus; fcp[f] = fi.cell_plus;
            for (int e : fi.edges) fe.push_back(e);
            fe_ptr[f + 1] = (int)fe.size();
        }
        w.d("face_xyz", fxyz); w.d("face_area", farea); w.i("face_normal", fnorm);
        w.i("face_cm", fcm); w.i("face_cp", fcp); w.i("face_edges_ptr", fe_ptr); w.i("face_edges", fe);
        std::vector<int> hf, he;
        for (const auto& h : sg.hanging_faces()) {
            hf.push_back(h.coarse_face);
            for (int k = 0; k < 4; ++k) hf.push_back(h.fine_faces[k]);
        }
        for (const auto& h : sg.hanging_edges()) {
            he.push_back(h.coarse_edge); he.push_back(h.fine_edges[0]); he.push_back(h.fine_edges[1]);
        }
        w.i("hanging_faces", hf); w.i("hanging_edges", he);
        std::vector<int> ce_ptr(nc + 1, 0), ce_id;
        std::vector<double> ce_frac;
        for (int c = 0; c < nc; ++c) {
            for (const auto& x : sg.cell_edges()[c]) { ce_id.push_back(x.edge_id); ce_frac.push_back(x.volume_fraction); }
            ce_ptr[c + 1] = (int)ce_id.size();
        }
        w.i("cell_edges_ptr", ce_ptr); w.i("cell_edges", ce_id); w.d("cell_edges_frac", ce_frac);

        octree::DiscreteOperators ops;
        ops.build(sg);
        const auto& Ce = ops.curl_e2f();
        w.i("Ce_rowptr", Ce.rowptr); w.i("Ce_colidx", Ce.colidx); w.d("Ce_values", Ce.values);
        const auto& G = ops.gradient_node();
        w.i("G_rowptr", G.rowptr); w.i("G_colidx", G.colidx); w.d("G_values", G.values);
        std::vector<double> adual(ne);
        std::vector<int> dead(ne);
        for (int e = 0; e < ne; ++e) { adual[e] = ops.edge_dual_area(e); dead[e] = ops.is_dead_edge(e); }
        w.d("edge_dual_area", adual); w.i("dead_edge", dead);
        std::vector<int> deadf(nf);
        for (int f = 0; f < nf; ++f) deadf[f] = ops.is_dead_face(f);
        w.i("dead_face", deadf);
        std::vector<int> nn{ops.num_nodes()};
        w.i("num_nodes", nn);
        DiagMatR Me, Mfi;
        ops.build_edge_mass(sigma, Me);
        ops.build_face_mass_inv(Mfi);
        w.d("Me", Me.diag); w.d("Mf_inv", Mfi.diag);
        if (cs->n_freqs > 0) {
            SparseMatC A;
            const Real omega = constants::TWOPI * cs->freqs[0];
            ops.assemble_system(omega, sigma, A);   // first call: map path
            SparseMatC A2;
            ops.assemble_system(omega, sigma, A2);  // second call: cached-pattern path
            w.i("A_rowptr", A.rowptr); w.i("A_colidx", A.colidx); w.c("A_values", A.values);
            w.c("A_values_cached", A2.values);
            SparseMatR L;
            ops.build_div_laplacian(sigma, L);
            w.i("L_rowptr", L.rowptr); w.i("L_colidx", L.colidx); w.d("L_values", L.values);
        }
    }

    if (flags & 2) {
        const int ns = cs->n_stations;
        const int nfq = cs->n_freqs;
        data::MTData obs;
        for (int s = 0; s < ns; ++s) {
            data::Station st;
            st.name = "S" + std::to_string(s);
            st.x = cs->station_xyz[3 * s]; st.y = cs->station_xyz[3 * s + 1]; st.z = cs->station_xyz[3 * s + 2];
            obs.add_station(st);
        }
        obs.set_frequencies(RealVec(cs->freqs, cs->freqs + nfq));
        if (cs->obs_Z) {
            for (int s = 0; s < ns; ++s)
                for (int f = 0; f < nfq; ++f) {
                    data::MTResponse r;
                    data::Datum* d[4] = {&r.Zxx, &r.Zxy, &r.Zyx, &r.Zyy};
                    for (int k = 0; k < 4; ++k) {
                        size_t o = ((size_t)s * nfq + f) * 4 + k;
                        d[k]->value = Complex(cs->obs_Z[2 * o], cs->obs_Z[2 * o + 1]);
                        d[k]->error = cs->obs_err[o];
                        d[k]->weight = cs->obs_err[o] > 0 ? 1.0 : 0.0;
                    }
                    obs.set_observed(s, f, r);
                }
        }
        std::vector<Complex> E1all, E2all, Zall, rhs1all, rhs2all, lam1all, lam2all;
        RealVec grad(nc, 0.0), gper;
        for (int f = 0; f < nfq; ++f) {
            fwd.compute_single_frequency(f, obs, obs);
            const auto& E1 = fwd.background_E(0);
            const auto& E2 = fwd.background_E(1);
            E1all.insert(E1all.end(), E1.begin(), E1.end());
            E2all.insert(E2all.end(), E2.begin(), E2.end());
            for (int s = 0; s < ns; ++s) {
                const auto& p = obs.predicted(s, f);
                Zall.push_back(p.Zxx.value); Zall.push_back(p.Zxy.value);
                Zall.push_back(p.Zyx.value); Zall.push_back(p.Zyy.value);
            }
            if ((flags & 4) && cs->obs_Z) {
                // src/inversion/inversion_fv.cpp:258-288
                std::vector<std::array<Complex, 4>> wr(ns);
                for (int s = 0; s < ns; ++s) {
                    const auto& o = obs.observed(s, f);
                    const auto& p = obs.predicted(s, f);
                    auto w_res = [](const data::Datum& od, const data::Datum& pd) -> Complex {
                        if (od.weight <= 0.0 || od.error <= 0.0) return Complex(0, 0);
                        Real wt = 1.0 / od.error;
                        return wt * wt * std::conj(od.value - pd.value);
                    };
                    wr[s][0] = w_res(o.Zxx, p.Zxx); wr[s][1] = w_res(o.Zxy, p.Zxy);
                    wr[s][2] = w_res(o.Zyx, p.Zyx); wr[s][3] = w_res(o.Zyy, p.Zyy);
                }
                ComplexVec a1, a2, l1, l2;
                fwd.build_adjoint_rhs_from_residual(f, wr, a1, a2);
                fwd.adjoint_solve_complex(a1, l1);
                fwd.adjoint_solve_complex(a2, l2);
                RealVec g1(nc, 0.0), g2(nc, 0.0);
                fwd.compute_sensitivity_complex(fwd.background_E(0), l1, g1);
                fwd.compute_sensitivity_complex(fwd.background_E(1), l2, g2);
                for (int c = 0; c < nc; ++c) grad[c] += g1[c] + g2[c];
                rhs1all.insert(rhs1all.end(), a1.begin(), a1.end());
                rhs2all.insert(rhs2all.end(), a2.begin(), a2.end());
                lam1all.insert(lam1all.end(), l1.begin(), l1.end());
                lam2all.insert(lam2all.end(), l2.begin(), l2.end());
                gper.insert(gper.end(), g1.begin(), g1.end());
                gper.insert(gper.end(), g2.begin(), g2.end());
            }
            fwd.release_factorization();
        }
        w.c("E1", E1all); w.c("E2", E2all); w.c("Z", Zall);
        if ((flags & 4) && cs->obs_Z) {
            w.c("adj_rhs1", rhs1all); w.c("adj_rhs2", rhs2all);
            w.c("lambda1", lam1all); w.c("lambda2", lam2all);
            w.d("grad", grad); w.d("grad_per_pol", gper);
        }
    }
    return 0;
}
