// Layout introspection C ABI (include/m3d_gb300.h, m3d_layout_*): host only.
#include "m3d_gb300.h"
#include "layout.hpp"

#include <new>
#include <stdexcept>

struct m3d_layout {
    m3d::HostLayout L;
};

namespace m3d {
bool leaves_valid(const m3d_leaves* lv) {
    return lv && lv->n_cells > 0 && lv->level && lv->cx && lv->cy && lv->cz && lv->cell_type &&
           lv->max_level >= lv->min_level && lv->min_level >= 0 && lv->max_level <= 14 &&
           lv->domain[1] > lv->domain[0] && lv->domain[3] > lv->domain[2] && lv->domain[5] > lv->domain[4];
}
LeafInput to_leaf_input(const m3d_leaves* lv) {
    LeafInput in;
    for (int i = 0; i < 6; ++i) in.domain[i] = lv->domain[i];
    in.min_level = lv->min_level;
    in.max_level = lv->max_level;
    in.nc = lv->n_cells;
    in.level = lv->level;
    in.cx = lv->cx; in.cy = lv->cy; in.cz = lv->cz;
    in.type = lv->cell_type;
    return in;
}
}  // namespace m3d

extern "C" int m3d_layout_build(const m3d_leaves* leaves, m3d_layout** out) {
    if (!out || !m3d::leaves_valid(leaves)) return M3D_ERR_ARG;
    auto* h = new (std::nothrow) m3d_layout;
    if (!h) return M3D_ERR_OOM;
    try {
        m3d::build_layout(m3d::to_leaf_input(leaves), h->L);
    } catch (const std::bad_alloc&) {
        delete h;
        return M3D_ERR_OOM;
    } catch (const std::exception&) {
        delete h;
        return M3D_ERR_ARG;
    }
    *out = h;
    return M3D_OK;
}

extern "C" void m3d_layout_destroy(m3d_layout* L) { delete L; }

extern "C" int m3d_layout_sizes(const m3d_layout* h, int* ne, int* nf, int* nc, int* nn, int* nnz,
                                int* nh) {
    if (!h) return M3D_ERR_ARG;
    const auto& L = h->L;
    if (ne) *ne = L.ne;
    if (nf) *nf = L.nf;
    if (nc) *nc = L.nc;
    if (nn) *nn = L.nn;
    if (nnz) *nnz = (int)L.s_idx.size();
    if (nh) *nh = (int)L.hp.size();
    return M3D_OK;
}

extern "C" int m3d_layout_edges(const m3d_layout* h, double* xyz, double* len, int* dir, double* adual,
                                int* dead, int* node1, int* node2) {
    if (!h) return M3D_ERR_ARG;
    const auto& L = h->L;
    for (int e = 0; e < L.ne; ++e) {
        if (xyz) { xyz[3 * e] = L.ex[e]; xyz[3 * e + 1] = L.ey[e]; xyz[3 * e + 2] = L.ez[e]; }
        if (len) len[e] = L.elen[e];
        if (dir) dir[e] = L.edir[e];
        if (adual) adual[e] = L.adual[e];
        if (dead) dead[e] = L.dead[e];
        if (node1) node1[e] = L.n1[e];
        if (node2) node2[e] = L.n2[e];
    }
    return M3D_OK;
}

extern "C" int m3d_layout_stiffness(const m3d_layout* h, int* ptr, int* idx, double* val) {
    if (!h) return M3D_ERR_ARG;
    const auto& L = h->L;
    for (int i = 0; i <= L.ne; ++i) if (ptr) ptr[i] = L.s_ptr[i];
    for (size_t k = 0; k < L.s_idx.size(); ++k) {
        if (idx) idx[k] = L.s_idx[k];
        if (val) val[k] = L.s_val[k];
    }
    return M3D_OK;
}

extern "C" int m3d_layout_hanging(const m3d_layout* h, int* pairs) {
    if (!h || !pairs) return M3D_ERR_ARG;
    const auto& L = h->L;
    for (size_t i = 0; i < L.hp.size(); ++i)
        for (int k = 0; k < 3; ++k) pairs[3 * i + k] = L.hp[i][k];
    return M3D_OK;
}
