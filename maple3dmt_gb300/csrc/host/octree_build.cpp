// Octree leaf builder (p4est stand-in).  See octree_build.hpp for scope.
#include "octree_build.hpp"

#include <algorithm>
#include <cmath>
#include <unordered_set>

namespace m3d {

namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr double kMu0 = 4.0e-7 * kPi;
constexpr double kTwoPi = 2.0 * kPi;

inline int32_t qlen(int level) { return kRootLen >> level; }

// Morton key of the lower corner, x in the lowest bit (p4est z-order).
inline uint64_t morton(const Quad& q) {
    uint64_t k = 0;
    for (int b = 0; b < kMaxLevel; ++b) {
        k |= (uint64_t)((q.x >> b) & 1) << (3 * b);
        k |= (uint64_t)((q.y >> b) & 1) << (3 * b + 1);
        k |= (uint64_t)((q.z >> b) & 1) << (3 * b + 2);
    }
    return k;
}

inline uint64_t okey(int level, int32_t x, int32_t y, int32_t z) {
    const int s = kMaxLevel - level;
    return ((uint64_t)level << 57) | ((uint64_t)(x >> s) << 38) |
           ((uint64_t)(y >> s) << 19) | (uint64_t)(z >> s);
}

struct Box {
    double x0, y0, z0, x1, y1, z1;
};

// Physical box of a quadrant, with the arithmetic of the refine callbacks
// (octree_mesh.cpp:139-160, :220-232, :285-297).
inline Box quad_box(const MeshParams& p, const Quad& q) {
    const double rl = (double)kRootLen;
    const int32_t ql = qlen(q.level);
    const double Lx = p.x_max - p.x_min, Ly = p.y_max - p.y_min, Lz = p.z_max - p.z_min;
    Box b;
    b.x0 = p.x_min + (double)q.x / rl * Lx;
    b.y0 = p.y_min + (double)q.y / rl * Ly;
    b.z0 = p.z_min + (double)q.z / rl * Lz;
    b.x1 = p.x_min + (double)(q.x + ql) / rl * Lx;
    b.y1 = p.y_min + (double)(q.y + ql) / rl * Ly;
    b.z1 = p.z_min + (double)(q.z + ql) / rl * Lz;
    return b;
}

inline double box_point_dist2(double px, double py, double pz, const Box& b) {
    auto cd = [](double v, double lo, double hi) {
        if (v < lo) return lo - v;
        if (v > hi) return v - hi;
        return 0.0;
    };
    const double dx = cd(px, b.x0, b.x1), dy = cd(py, b.y0, b.y1), dz = cd(pz, b.z0, b.z1);
    return dx * dx + dy * dy + dz * dz;
}

// One non-recursive refinement pass (p8est_refine with recursive = 0):
// every current leaf is offered to the callback once; children replace it in
// Morton order and are not revisited in the same pass.
template <class Fn>
bool refine_pass(std::vector<Quad>& quads, Fn&& fn) {
    std::vector<Quad> out;
    out.reserve(quads.size() * 2);
    bool changed = false;
    for (const Quad& q : quads) {
        if (q.level < kMaxLevel - 1 && fn(q)) {
            const int32_t h = qlen(q.level + 1);
            for (int c = 0; c < 8; ++c) {
                Quad ch;
                ch.x = q.x + ((c & 1) ? h : 0);
                ch.y = q.y + ((c & 2) ? h : 0);
                ch.z = q.z + ((c & 4) ? h : 0);
                ch.level = (int8_t)(q.level + 1);
                out.push_back(ch);
            }
            changed = true;
        } else {
            out.push_back(q);
        }
    }
    quads.swap(out);
    return changed;
}

void sort_morton(std::vector<Quad>& quads) {
    std::vector<std::pair<uint64_t, Quad>> tmp(quads.size());
    for (size_t i = 0; i < quads.size(); ++i) tmp[i] = {morton(quads[i]), quads[i]};
    std::sort(tmp.begin(), tmp.end(),
              [](const auto& a, const auto& b) { return a.first < b.first; });
    for (size_t i = 0; i < quads.size(); ++i) quads[i] = tmp[i].second;
}

std::unordered_set<uint64_t> internal_set(const std::vector<Quad>& quads) {
    std::unordered_set<uint64_t> s;
    s.reserve(quads.size());
    for (const Quad& q : quads) {
        int32_t x = q.x, y = q.y, z = q.z;
        for (int l = q.level - 1; l >= 0; --l) {
            const int32_t m = ~(qlen(l) - 1);
            x &= m; y &= m; z &= m;
            if (!s.insert(okey(l, x, y, z)).second) break;  // ancestors already present
        }
    }
    return s;
}

// A leaf must split if the same-size cube across one of its faces is split
// and one of that cube's four children touching the shared face is split too
// (then a leaf two or more levels finer touches this face).
bool needs_split(const Quad& q, const std::unordered_set<uint64_t>& internal) {
    const int32_t h = qlen(q.level);
    const int32_t h2 = h >> 1;
    const int32_t base[3] = {q.x, q.y, q.z};
    for (int axis = 0; axis < 3; ++axis) {
        for (int s = -1; s <= 1; s += 2) {
            int32_t n[3] = {base[0], base[1], base[2]};
            n[axis] += s * h;
            if (n[axis] < 0 || n[axis] >= kRootLen) continue;
            if (!internal.count(okey(q.level, n[0], n[1], n[2]))) continue;
            const int32_t face_c = (s > 0) ? n[axis] : n[axis] + h2;
            const int a1 = (axis + 1) % 3, a2 = (axis + 2) % 3;
            for (int i = 0; i < 2; ++i)
                for (int j = 0; j < 2; ++j) {
                    int32_t c[3];
                    c[axis] = face_c;
                    c[a1] = n[a1] + i * h2;
                    c[a2] = n[a2] + j * h2;
                    if (internal.count(okey(q.level + 1, c[0], c[1], c[2]))) return true;
                }
        }
    }
    return false;
}

// 2:1 face balance (p8est_balance with P8EST_CONNECT_FACE): forced splits are
// applied until none is left, which yields the coarsest balanced refinement.
void balance_face(std::vector<Quad>& quads) {
    for (;;) {
        auto internal = internal_set(quads);
        bool any = false;
        std::vector<char> split(quads.size(), 0);
        for (size_t i = 0; i < quads.size(); ++i)
            if (needs_split(quads[i], internal)) { split[i] = 1; any = true; }
        if (!any) break;
        size_t idx = 0;
        refine_pass(quads, [&](const Quad&) { return split[idx++] != 0; });
    }
    sort_morton(quads);
}

}  // namespace

OctreeLeaves build_octree(const MeshParams& p,
                          const std::vector<std::array<double, 3>>& stations,
                          const std::vector<double>& freqs) {
    OctreeLeaves t;
    t.params = p;
    std::vector<Quad>& quads = t.quads;

    // Uniform forest at min_level (p8est_new_ext, octree_mesh.cpp:40-42).
    {
        const int32_t n = 1 << p.min_level;
        const int32_t h = qlen(p.min_level);
        for (int32_t k = 0; k < n; ++k)
            for (int32_t j = 0; j < n; ++j)
                for (int32_t i = 0; i < n; ++i)
                    quads.push_back(Quad{i * h, j * h, k * h, (int8_t)p.min_level});
        sort_morton(quads);
    }

    const double Lx = p.x_max - p.x_min, Ly = p.y_max - p.y_min, Lz = p.z_max - p.z_min;

    // Station refinement (octree_mesh.cpp:129-200).
    if (!stations.empty()) {
        const double domain_diag = std::max({Lx, Ly, Lz});
        const double h_finest = domain_diag / (1 << p.station_refine_level);
        const double air_max_z = 2.0 * h_finest;
        const double r2 = p.station_refine_radius * p.station_refine_radius;
        auto fn = [&](const Quad& q) {
            if (q.level >= p.station_refine_level) return false;
            const Box b = quad_box(p, q);
            for (const auto& st : stations) {
                if (b.z0 > st[2] + air_max_z) continue;
                if (box_point_dist2(st[0], st[1], st[2], b) < r2) return true;
            }
            return false;
        };
        for (int pass = 0; pass < p.max_level - p.min_level; ++pass) refine_pass(quads, fn);
    }

    // Region refinement (octree_mesh.cpp:211-261).
    for (const RefineRegion& reg : p.regions) {
        auto fn = [&](const Quad& q) {
            if (q.level >= reg.level) return false;
            const Box b = quad_box(p, q);
            const double pad = reg.padding;
            if (b.x1 < reg.x_min - pad || b.x0 > reg.x_max + pad) return false;
            if (b.y1 < reg.y_min - pad || b.y0 > reg.y_max + pad) return false;
            if (b.z1 < reg.z_min - pad || b.z0 > reg.z_max + pad) return false;
            return true;
        };
        for (int pass = 0; pass < reg.level - p.min_level; ++pass) refine_pass(quads, fn);
    }

    // Skin-depth layers (octree_mesh.cpp:316-493).
    if (!freqs.empty()) {
        const double f_min = *std::min_element(freqs.begin(), freqs.end());
        const double delta_max = std::sqrt(2.0 / (kTwoPi * f_min * kMu0 * p.sigma_bg));
        const double pad_h = 0.5 * delta_max + p.transition_padding;
        double rx0, rx1, ry0, ry1;
        if (p.station_x_max > p.station_x_min) {
            rx0 = p.station_x_min - pad_h; rx1 = p.station_x_max + pad_h;
            ry0 = p.station_y_min - pad_h; ry1 = p.station_y_max + pad_h;
        } else {
            const double hx = (p.x_max - p.x_min) * 0.2, hy = (p.y_max - p.y_min) * 0.2;
            rx0 = -hx - pad_h; rx1 = hx + pad_h;
            ry0 = -hy - pad_h; ry1 = hy + pad_h;
        }
        rx0 = std::max(rx0, p.x_min); rx1 = std::min(rx1, p.x_max);
        ry0 = std::max(ry0, p.y_min); ry1 = std::min(ry1, p.y_max);

        const int off = (p.max_level >= 9) ? 2 : 1;
        const int L1 = std::max(p.min_level + 1, p.max_level - off);
        const int L2 = std::max(p.min_level + 1, p.max_level - off - 1);
        const int L3 = std::max(p.min_level, p.max_level - off - 2);
        struct Layer { double z_top, z_bot; int level; };
        std::vector<Layer> layers;
        double z_interest_bot = -3.0 * delta_max;
        if (p.max_interest_depth > 0) z_interest_bot = -p.max_interest_depth;
        const double z_l1_bot = std::max(-0.5 * delta_max, z_interest_bot);
        if (z_l1_bot < 0) layers.push_back({0.0, z_l1_bot, L1});
        const double z_l2_top = -0.5 * delta_max;
        const double z_l2_bot = std::max(-1.5 * delta_max, z_interest_bot);
        if (z_l2_top > z_interest_bot && z_l2_bot < z_l2_top) layers.push_back({z_l2_top, z_l2_bot, L2});
        const double z_l3_top = -1.5 * delta_max;
        const double z_l3_bot = std::max(-3.0 * delta_max, z_interest_bot);
        if (z_l3_top > z_interest_bot && z_l3_bot < z_l3_top && L3 > p.min_level)
            layers.push_back({z_l3_top, z_l3_bot, L3});
        const int L_deep = p.min_level + 1;
        if (z_interest_bot > p.z_min && L_deep > p.min_level)
            layers.push_back({z_interest_bot, p.z_min, L_deep});
        const int L_as = std::max(p.min_level + 1, L1 - 1);
        const int L_am = std::max(p.min_level, L_as - 1);
        const int L_au = std::max(p.min_level, L_am - 1);
        const double za1 = p.air_surface_thickness;
        const double za2 = za1 + p.air_mid_thickness;
        const double za3 = za2 + p.air_upper_thickness;
        layers.push_back({za1, 0.0, L_as});
        layers.push_back({za2, za1, L_am});
        layers.push_back({za3, za2, L_au});

        auto fn = [&](const Quad& q) {
            const Box b = quad_box(p, q);
            if (b.x1 < rx0 || b.x0 > rx1) return false;
            if (b.y1 < ry0 || b.y0 > ry1) return false;
            int target = p.min_level;
            for (const Layer& l : layers)
                if (b.z1 > l.z_bot && b.z0 < l.z_top) target = std::max(target, l.level);
            return q.level < target;
        };
        for (int pass = 0; pass < p.max_level - p.min_level; ++pass)
            if (!refine_pass(quads, fn)) break;
    }

    balance_face(quads);

    // Cell data (octree_mesh.cpp:523-566) and flat-terrain classification
    // (octree_mesh.cpp:667-694 with terrain z = 0).
    const size_t nc = quads.size();
    t.cx.resize(nc); t.cy.resize(nc); t.cz.resize(nc);
    t.level.resize(nc); t.type.resize(nc);
    const double rl = (double)kRootLen;
    for (size_t i = 0; i < nc; ++i) {
        const Quad& q = quads[i];
        const int32_t ql = qlen(q.level);
        const double cxu = (q.x + ql / 2.0) / rl;
        const double cyu = (q.y + ql / 2.0) / rl;
        const double czu = (q.z + ql / 2.0) / rl;
        t.cx[i] = p.x_min + cxu * Lx;
        t.cy[i] = p.y_min + cyu * Ly;
        t.cz[i] = p.z_min + czu * Lz;
        t.level[i] = q.level;
        const double h = (1.0 / (1 << q.level)) * Lz;
        const double terrain_z = 0.0;
        int ty;
        if (t.cz[i] + h / 2.0 < terrain_z) ty = kEarth;
        else if (t.cz[i] - h / 2.0 > terrain_z) ty = kAir;
        else {
            double ef = (terrain_z - (t.cz[i] - h / 2.0)) / h;
            ef = std::min(1.0, std::max(0.0, ef));
            ty = (ef > 0.5) ? kEarth : kAir;
        }
        t.type[i] = ty;
    }
    return t;
}

bool octree_is_face_balanced(const OctreeLeaves& t) {
    auto internal = internal_set(t.quads);
    for (const Quad& q : t.quads)
        if (needs_split(q, internal)) return false;
    return true;
}

}  // namespace m3d
