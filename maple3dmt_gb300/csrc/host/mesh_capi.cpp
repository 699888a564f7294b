// C ABI of the octree leaf builder (include/m3d_mesh.h).
#include "m3d_mesh.h"
#include "m3d_gb300.h"
#include "octree_build.hpp"

#include <new>

struct m3d_octree {
    m3d::OctreeLeaves leaves;
};

extern "C" int m3d_octree_build(const m3d_mesh_params* p, const double* stations, int n_stations,
                                const double* freqs, int n_freqs, m3d_octree** out) {
    if (!p || !out || n_stations < 0 || n_freqs < 0) return M3D_ERR_ARG;
    if ((n_stations > 0 && !stations) || (n_freqs > 0 && !freqs)) return M3D_ERR_ARG;
    if (p->min_level < 0 || p->max_level < p->min_level || p->max_level > 16) return M3D_ERR_ARG;
    if (!(p->domain[1] > p->domain[0] && p->domain[3] > p->domain[2] && p->domain[5] > p->domain[4]))
        return M3D_ERR_ARG;
    m3d::MeshParams mp;
    mp.x_min = p->domain[0]; mp.x_max = p->domain[1];
    mp.y_min = p->domain[2]; mp.y_max = p->domain[3];
    mp.z_min = p->domain[4]; mp.z_max = p->domain[5];
    mp.min_level = p->min_level;
    mp.max_level = p->max_level;
    mp.station_refine_radius = p->station_refine_radius;
    mp.station_refine_level = p->station_refine_level;
    mp.sigma_bg = p->sigma_bg;
    mp.max_interest_depth = p->max_interest_depth;
    mp.air_surface_thickness = p->air_surface_thickness;
    mp.air_mid_thickness = p->air_mid_thickness;
    mp.air_upper_thickness = p->air_upper_thickness;
    mp.transition_padding = p->transition_padding;
    mp.station_x_min = p->station_bbox[0]; mp.station_x_max = p->station_bbox[1];
    mp.station_y_min = p->station_bbox[2]; mp.station_y_max = p->station_bbox[3];
    for (int r = 0; r < p->n_regions; ++r) {
        const double* g = p->regions + 8 * r;
        mp.regions.push_back({g[0], g[1], g[2], g[3], g[4], g[5], (int)g[6], g[7]});
    }
    std::vector<std::array<double, 3>> st(n_stations);
    for (int s = 0; s < n_stations; ++s) st[s] = {stations[3 * s], stations[3 * s + 1], stations[3 * s + 2]};
    std::vector<double> fr(freqs, freqs + n_freqs);
    auto* t = new (std::nothrow) m3d_octree;
    if (!t) return M3D_ERR_OOM;
    try {
        t->leaves = m3d::build_octree(mp, st, fr);
    } catch (...) {
        delete t;
        return M3D_ERR_OOM;
    }
    *out = t;
    return M3D_OK;
}

extern "C" int m3d_octree_num_cells(const m3d_octree* t) {
    return t ? (int)t->leaves.quads.size() : -1;
}

extern "C" int m3d_octree_get(const m3d_octree* t, int* level, int* qxyz, double* cx, double* cy,
                              double* cz, int* cell_type) {
    if (!t) return M3D_ERR_ARG;
    const auto& L = t->leaves;
    for (size_t i = 0; i < L.quads.size(); ++i) {
        if (level) level[i] = L.level[i];
        if (qxyz) { qxyz[3 * i] = L.quads[i].x; qxyz[3 * i + 1] = L.quads[i].y; qxyz[3 * i + 2] = L.quads[i].z; }
        if (cx) cx[i] = L.cx[i];
        if (cy) cy[i] = L.cy[i];
        if (cz) cz[i] = L.cz[i];
        if (cell_type) cell_type[i] = L.type[i];
    }
    return M3D_OK;
}

extern "C" int m3d_octree_is_balanced(const m3d_octree* t) {
    return t ? (m3d::octree_is_face_balanced(t->leaves) ? 1 : 0) : 0;
}

extern "C" void m3d_octree_destroy(m3d_octree* t) { delete t; }
