// Host layout producer.  See layout.hpp for what it restates.
#include "layout.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <stdexcept>

namespace m3d {

namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr double kMu0 = 4.0e-7 * kPi;

// Open-addressing map from a 3 x int64 key to an int id.
class KeyMap {
public:
    explicit KeyMap(size_t expect) {
        size_t c = 16;
        while (c < 2 * expect + 16) c <<= 1;
        keys_.assign(c * 3, 0);
        vals_.assign(c, -1);
        mask_ = c - 1;
    }
    // Returns the slot value reference; `inserted` is true if the key was new.
    int& get(const int64_t* k, bool& inserted) {
        if (2 * (n_ + 1) > vals_.size()) grow();
        size_t i = hash(k) & mask_;
        for (;;) {
            if (vals_[i] == -1) {
                keys_[3 * i] = k[0]; keys_[3 * i + 1] = k[1]; keys_[3 * i + 2] = k[2];
                vals_[i] = -2;  // reserved; caller assigns
                ++n_;
                inserted = true;
                return vals_[i];
            }
            if (keys_[3 * i] == k[0] && keys_[3 * i + 1] == k[1] && keys_[3 * i + 2] == k[2]) {
                inserted = false;
                return vals_[i];
            }
            i = (i + 1) & mask_;
        }
    }
    int find(const int64_t* k) const {
        size_t i = hash(k) & mask_;
        for (;;) {
            if (vals_[i] == -1) return -1;
            if (keys_[3 * i] == k[0] && keys_[3 * i + 1] == k[1] && keys_[3 * i + 2] == k[2]) return vals_[i];
            i = (i + 1) & mask_;
        }
    }

private:
    std::vector<int64_t> keys_;
    std::vector<int> vals_;
    size_t mask_ = 0, n_ = 0;
    static size_t hash(const int64_t* k) {
        uint64_t h = 1469598103934665603ull;
        for (int i = 0; i < 3; ++i) {
            uint64_t x = (uint64_t)k[i];
            x ^= x >> 33; x *= 0xff51afd7ed558ccdull; x ^= x >> 33;
            h = (h ^ x) * 1099511628211ull;
        }
        return (size_t)h;
    }
    void grow() {
        std::vector<int64_t> ok = std::move(keys_);
        std::vector<int> ov = std::move(vals_);
        size_t c = ov.size() * 2;
        keys_.assign(c * 3, 0);
        vals_.assign(c, -1);
        mask_ = c - 1;
        n_ = 0;
        for (size_t i = 0; i < ov.size(); ++i)
            if (ov[i] != -1) { bool ins; get(&ok[3 * i], ins) = ov[i]; }
    }
};

struct GridCtx {
    double dx, dy, dz, x0, y0, z0, quant;
    // staggered_grid.cpp:31-36 (direction folded into the z key)
    void key(double px, double py, double pz, int dir, int64_t* k) const {
        k[0] = (int64_t)std::llround((px - x0) / dx * quant);
        k[1] = (int64_t)std::llround((py - y0) / dy * quant);
        k[2] = (int64_t)std::llround((pz - z0) / dz * quant) * 4 + dir;
    }
};

}  // namespace

void build_layout(const LeafInput& in, HostLayout& L) {
    if (in.nc <= 0 || !in.level || !in.cx || !in.cy || !in.cz || !in.type)
        throw std::runtime_error("build_layout: empty or null leaf list");
    if (in.max_level > 14 || in.min_level < 0 || in.min_level > in.max_level)
        throw std::runtime_error("build_layout: levels out of range (0 <= min <= max <= 14)");
    const int nc = in.nc;
    L = HostLayout();
    std::memcpy(L.domain, in.domain, sizeof(L.domain));
    L.min_level = in.min_level;
    L.max_level = in.max_level;
    L.nc = nc;
    L.ccx.assign(in.cx, in.cx + nc);
    L.ccy.assign(in.cy, in.cy + nc);
    L.ccz.assign(in.cz, in.cz + nc);
    L.clevel.assign(in.level, in.level + nc);
    L.ctype.assign(in.type, in.type + nc);
    for (int c = 0; c < nc; ++c)
        if (in.level[c] < 0 || in.level[c] > in.max_level)
            throw std::runtime_error("build_layout: cell level outside [0, max_level]");

    GridCtx g;
    g.dx = in.domain[1] - in.domain[0];
    g.dy = in.domain[3] - in.domain[2];
    g.dz = in.domain[5] - in.domain[4];
    g.x0 = in.domain[0]; g.y0 = in.domain[2]; g.z0 = in.domain[4];
    g.quant = (double)(1 << (in.max_level + 2));
    {
        const double mn = std::min({g.dx, g.dy, g.dz});
        const double h = (double)(1 << (19 - in.level[0])) / (double)(1 << 19);
        L.cell_size0 = h * mn;  // octree_mesh.cpp:560
    }
    auto half = [&](int c, double* ch) {  // staggered_grid.cpp:58-67
        ch[0] = in.cx[c]; ch[1] = in.cy[c]; ch[2] = in.cz[c];
        const double h = 1.0 / (1 << in.level[c]);
        ch[3] = h * g.dx / 2.0; ch[4] = h * g.dy / 2.0; ch[5] = h * g.dz / 2.0;
    };

    // ---- edges (staggered_grid.cpp:78-122) ----
    std::vector<std::vector<int>> adj;
    KeyMap em((size_t)nc * 4);
    auto add_edge = [&](double x, double y, double z, int dir, double len, int c) {
        int64_t k[3];
        g.key(x, y, z, dir, k);
        bool ins;
        int& slot = em.get(k, ins);
        if (ins) {
            slot = (int)L.ex.size();
            L.ex.push_back(x); L.ey.push_back(y); L.ez.push_back(z);
            L.edir.push_back(dir); L.elen.push_back(len);
            adj.emplace_back();
        }
        adj[slot].push_back(c);
    };
    for (int c = 0; c < nc; ++c) {
        double ch[6];
        half(c, ch);
        const double cx = ch[0], cy = ch[1], cz = ch[2], hx = ch[3], hy = ch[4], hz = ch[5];
        const double ey[4] = {cy - hy, cy - hy, cy + hy, cy + hy};
        const double ez[4] = {cz - hz, cz + hz, cz - hz, cz + hz};
        for (int i = 0; i < 4; ++i) add_edge(cx, ey[i], ez[i], 0, 2.0 * hx, c);
        const double ex[4] = {cx - hx, cx - hx, cx + hx, cx + hx};
        for (int i = 0; i < 4; ++i) add_edge(ex[i], cy, ez[i], 1, 2.0 * hy, c);
        const double ex3[4] = {cx - hx, cx + hx, cx - hx, cx + hx};
        const double ey3[4] = {cy - hy, cy - hy, cy + hy, cy + hy};
        for (int i = 0; i < 4; ++i) add_edge(ex3[i], ey3[i], cz, 2, 2.0 * hz, c);
    }
    const int ne = (int)L.ex.size();
    L.ne = ne;

    // ---- faces (staggered_grid.cpp:128-224) ----
    std::vector<double> fx, fy, fz;
    std::vector<int>& fnorm = L.fnorm;
    std::vector<int>& fcm = L.fcm;
    std::vector<int>& fcp = L.fcp;
    fnorm.clear(); fcm.clear(); fcp.clear();
    std::vector<std::array<int, 4>> fedge;
    std::vector<int> fnedge;
    KeyMap fm((size_t)nc * 4);
    for (int c = 0; c < nc; ++c) {
        double ch[6];
        half(c, ch);
        const double cx = ch[0], cy = ch[1], cz = ch[2], hx = ch[3], hy = ch[4], hz = ch[5];
        struct ERef { double x, y, z; int d; };
        struct FDef { double x, y, z; int n; double a; ERef e[4]; };
        const FDef fd[6] = {
            {cx + hx, cy, cz, 0, 4 * hy * hz,
             {{cx + hx, cy, cz - hz, 1}, {cx + hx, cy, cz + hz, 1}, {cx + hx, cy - hy, cz, 2}, {cx + hx, cy + hy, cz, 2}}},
            {cx - hx, cy, cz, 0, 4 * hy * hz,
             {{cx - hx, cy, cz - hz, 1}, {cx - hx, cy, cz + hz, 1}, {cx - hx, cy - hy, cz, 2}, {cx - hx, cy + hy, cz, 2}}},
            {cx, cy + hy, cz, 1, 4 * hx * hz,
             {{cx, cy + hy, cz - hz, 0}, {cx, cy + hy, cz + hz, 0}, {cx - hx, cy + hy, cz, 2}, {cx + hx, cy + hy, cz, 2}}},
            {cx, cy - hy, cz, 1, 4 * hx * hz,
             {{cx, cy - hy, cz - hz, 0}, {cx, cy - hy, cz + hz, 0}, {cx - hx, cy - hy, cz, 2}, {cx + hx, cy - hy, cz, 2}}},
            {cx, cy, cz + hz, 2, 4 * hx * hy,
             {{cx, cy - hy, cz + hz, 0}, {cx, cy + hy, cz + hz, 0}, {cx - hx, cy, cz + hz, 1}, {cx + hx, cy, cz + hz, 1}}},
            {cx, cy, cz - hz, 2, 4 * hx * hy,
             {{cx, cy - hy, cz - hz, 0}, {cx, cy + hy, cz - hz, 0}, {cx - hx, cy, cz - hz, 1}, {cx + hx, cy, cz - hz, 1}}},
        };
        for (int f = 0; f < 6; ++f) {
            int64_t k[3];
            g.key(fd[f].x, fd[f].y, fd[f].z, fd[f].n, k);
            bool ins;
            int& slot = fm.get(k, ins);
            if (ins) {
                slot = (int)fx.size();
                std::array<int, 4> el{-1, -1, -1, -1};
                int cnt = 0;
                for (int e = 0; e < 4; ++e) {
                    int64_t ek[3];
                    g.key(fd[f].e[e].x, fd[f].e[e].y, fd[f].e[e].z, fd[f].e[e].d, ek);
                    const int id = em.find(ek);
                    if (id >= 0) el[cnt++] = id;
                }
                fx.push_back(fd[f].x); fy.push_back(fd[f].y); fz.push_back(fd[f].z);
                fnorm.push_back(fd[f].n); L.farea.push_back(fd[f].a);
                fcm.push_back(-1); fcp.push_back(-1);
                fedge.push_back(el); fnedge.push_back(cnt);
            }
            const int fid = slot;
            if (f == 0 || f == 2 || f == 4) fcm[fid] = c; else fcp[fid] = c;
        }
    }
    const int nf = (int)fx.size();
    L.nf = nf;

    // ---- hanging faces / edges (staggered_grid.cpp:241-391) ----
    std::vector<std::array<int, 5>> hfaces;
    if (in.min_level < in.max_level) {
        const double mh = std::min({g.dx / (1 << in.max_level), g.dy / (1 << in.max_level),
                                    g.dz / (1 << in.max_level)});
        const double btol = mh * 0.01;
        KeyMap flk((size_t)nf), elk((size_t)ne);
        for (int f = 0; f < nf; ++f) {
            int64_t k[3]; bool ins;
            g.key(fx[f], fy[f], fz[f], fnorm[f], k);
            flk.get(k, ins) = f;
        }
        for (int e = 0; e < ne; ++e) {
            int64_t k[3]; bool ins;
            g.key(L.ex[e], L.ey[e], L.ez[e], L.edir[e], k);
            elk.get(k, ins) = e;
        }
        std::vector<char> fdone(nf, 0), ehang(ne, 0);
        for (int f = 0; f < nf; ++f) {
            if (fdone[f]) continue;
            if (fcm[f] >= 0 && fcp[f] >= 0) continue;
            if (fcm[f] < 0 && fcp[f] < 0) continue;
            const int n = fnorm[f];
            bool on_bnd = false;
            if (n == 0) on_bnd = fx[f] < in.domain[0] + btol || fx[f] > in.domain[1] - btol;
            if (n == 1) on_bnd = fy[f] < in.domain[2] + btol || fy[f] > in.domain[3] - btol;
            if (n == 2) on_bnd = fz[f] < in.domain[4] + btol || fz[f] > in.domain[5] - btol;
            if (on_bnd) continue;
            const int ccell = fcm[f] >= 0 ? fcm[f] : fcp[f];
            double ch[6];
            half(ccell, ch);
            const double fhx = ch[3] / 2, fhy = ch[4] / 2, fhz = ch[5] / 2;
            bool all = true;
            std::array<int, 4> subs{};
            int idx = 0;
            for (int s1 = -1; s1 <= 1 && all; s1 += 2)
                for (int s2 = -1; s2 <= 1; s2 += 2) {
                    double sx = fx[f], sy = fy[f], sz = fz[f];
                    if (n == 0) { sy += s1 * fhy; sz += s2 * fhz; }
                    else if (n == 1) { sx += s1 * fhx; sz += s2 * fhz; }
                    else { sx += s1 * fhx; sy += s2 * fhy; }
                    int64_t k[3];
                    g.key(sx, sy, sz, n, k);
                    const int id = flk.find(k);
                    if (id < 0 || fdone[id]) { all = false; break; }
                    subs[idx++] = id;
                }
            if (!all) continue;
            for (int q = 0; q < 4; ++q)
                if (fcm[subs[q]] >= 0 && fcp[subs[q]] >= 0) { all = false; break; }
            if (!all) continue;
            hfaces.push_back({f, subs[0], subs[1], subs[2], subs[3]});
            fdone[f] = 1;
            for (int q = 0; q < 4; ++q) fdone[subs[q]] = 1;
            for (int q = 0; q < 4; ++q) {
                const int ff = subs[q];
                if (fcm[ff] < 0) fcm[ff] = ccell;
                else if (fcp[ff] < 0) fcp[ff] = ccell;
            }
            fcm[f] = -1; fcp[f] = -1;
            for (int q = 0; q < 4; ++q) {
                const int ff = subs[q];
                for (int t = 0; t < fnedge[ff]; ++t) {
                    const int eid = fedge[ff][t];
                    if (eid < 0) continue;
                    auto& a = adj[eid];
                    if (std::find(a.begin(), a.end(), ccell) == a.end()) a.push_back(ccell);
                }
            }
            for (int t = 0; t < fnedge[f]; ++t) {
                const int eid = fedge[f][t];
                if (eid < 0 || ehang[eid]) continue;
                const int d = L.edir[eid];
                const double ql = L.elen[eid] / 4.0;
                double a1[3] = {L.ex[eid], L.ey[eid], L.ez[eid]};
                double a2[3] = {L.ex[eid], L.ey[eid], L.ez[eid]};
                a1[d] -= ql; a2[d] += ql;
                int64_t k1[3], k2[3];
                g.key(a1[0], a1[1], a1[2], d, k1);
                g.key(a2[0], a2[1], a2[2], d, k2);
                const int i1 = elk.find(k1), i2 = elk.find(k2);
                if (i1 >= 0 && i2 >= 0) {
                    L.hp.push_back({eid, i1, i2});
                    ehang[eid] = 1;
                }
            }
        }
    }

    // ---- flatten adjacency; cell -> edges (staggered_grid.cpp:393-409) ----
    L.adj_ptr.assign(ne + 1, 0);
    for (int e = 0; e < ne; ++e) L.adj_ptr[e + 1] = L.adj_ptr[e] + (int)adj[e].size();
    L.adj.resize(L.adj_ptr[ne]);
    for (int e = 0; e < ne; ++e) std::copy(adj[e].begin(), adj[e].end(), L.adj.begin() + L.adj_ptr[e]);
    {
        std::vector<int> cnt(nc + 1, 0);
        for (int e = 0; e < ne; ++e)
            for (int c : adj[e]) if (c >= 0 && c < nc) cnt[c + 1]++;
        L.cell_ptr.assign(nc + 1, 0);
        for (int c = 0; c < nc; ++c) L.cell_ptr[c + 1] = L.cell_ptr[c] + cnt[c + 1];
        L.cell_edge.resize(L.cell_ptr[nc]);
        std::vector<int> pos(L.cell_ptr.begin(), L.cell_ptr.end() - 1);
        for (int e = 0; e < ne; ++e)
            for (int c : adj[e]) if (c >= 0 && c < nc) L.cell_edge[pos[c]++] = e;
    }

    // ---- operators: centres, half extents, dual lengths / areas (operators.cpp:62-157) ----
    {
        std::vector<double> ccx(nc, 0.0), ccy(nc, 0.0), ccz(nc, 0.0);
        std::vector<double> chx(nc, 0.0), chy(nc, 0.0), chz(nc, 0.0);
        std::vector<int> cnt(nc, 0);
        for (int e = 0; e < ne; ++e)
            for (int c : adj[e])
                if (c >= 0 && c < nc) { ccx[c] += L.ex[e]; ccy[c] += L.ey[e]; ccz[c] += L.ez[e]; cnt[c]++; }
        for (int c = 0; c < nc; ++c)
            if (cnt[c] > 0) { ccx[c] /= cnt[c]; ccy[c] /= cnt[c]; ccz[c] /= cnt[c]; }
        for (int e = 0; e < ne; ++e) {
            const int d = L.edir[e];
            const double hl = L.elen[e] / 2.0;
            for (int c : adj[e]) {
                if (c < 0 || c >= nc) continue;
                if (d == 0 && hl > chx[c]) chx[c] = hl;
                if (d == 1 && hl > chy[c]) chy[c] = hl;
                if (d == 2 && hl > chz[c]) chz[c] = hl;
            }
        }
        L.fdual.resize(nf);
        for (int f = 0; f < nf; ++f) {
            const int n = fnorm[f], cm = fcm[f], cp = fcp[f];
            double v;
            if (cm >= 0 && cp >= 0) {
                const double a = n == 0 ? ccx[cm] : n == 1 ? ccy[cm] : ccz[cm];
                const double b = n == 0 ? ccx[cp] : n == 1 ? ccy[cp] : ccz[cp];
                v = std::abs(b - a);
            } else {
                const int c = cm >= 0 ? cm : cp;
                if (c >= 0) v = n == 0 ? chx[c] : n == 1 ? chy[c] : chz[c];
                else v = std::sqrt(L.farea[f]);
            }
            if (v < 1e-20) v = std::sqrt(L.farea[f]);
            L.fdual[f] = v;
        }
        L.adual.resize(ne);
        for (int e = 0; e < ne; ++e) {
            const int d = L.edir[e];
            if (adj[e].empty()) { L.adual[e] = L.elen[e] * L.elen[e]; continue; }
            double s = 0; int count = 0;
            for (int c : adj[e]) {
                if (c < 0 || c >= nc) continue;
                double h1, h2;
                if (d == 0) { h1 = chy[c]; h2 = chz[c]; }
                else if (d == 1) { h1 = chx[c]; h2 = chz[c]; }
                else { h1 = chx[c]; h2 = chy[c]; }
                s += h1 * h2;
                ++count;
            }
            L.adual[e] = count > 0 ? s : L.elen[e] * L.elen[e];
        }
    }

    // ---- curl with right-hand-rule signs (operators.cpp:192-244) ----
    struct Ent { int row, col; double val; };
    std::vector<Ent> ent;
    ent.reserve((size_t)nf * 4);
    for (int f = 0; f < nf; ++f)
        for (int t = 0; t < fnedge[f]; ++t) {
            const int eid = fedge[f][t];
            if (eid < 0 || eid >= ne) continue;
            const int n = fnorm[f], d = L.edir[eid];
            double sign = 0.0;
            if (n == 0) {
                if (d == 1) sign = (L.ez[eid] < fz[f]) ? 1.0 : -1.0;
                else if (d == 2) sign = (L.ey[eid] < fy[f]) ? -1.0 : 1.0;
            } else if (n == 1) {
                if (d == 2) sign = (L.ex[eid] < fx[f]) ? 1.0 : -1.0;
                else if (d == 0) sign = (L.ez[eid] < fz[f]) ? -1.0 : 1.0;
            } else {
                if (d == 0) sign = (L.ey[eid] < fy[f]) ? 1.0 : -1.0;
                else if (d == 1) sign = (L.ex[eid] < fx[f]) ? -1.0 : 1.0;
            }
            if (std::abs(sign) > 0.5) ent.push_back({f, eid, sign * L.elen[eid]});
        }

    // ---- hanging faces: dead rows dropped, dead edges split 1/2 (operators.cpp:344-466) ----
    L.dead.assign(ne, 0);
    L.dead_f.assign(nf, 0);
    if (!hfaces.empty()) {
        std::vector<int> ch1(ne, -1), ch2(ne, -1);
        for (const auto& h : L.hp) { L.dead[h[0]] = 1; ch1[h[0]] = h[1]; ch2[h[0]] = h[2]; }
        for (const auto& h : hfaces) L.dead_f[h[0]] = 1;
        std::vector<Ent> e2;
        e2.reserve(ent.size() + L.hp.size() * 4);
        for (const Ent& x : ent) {
            if (L.dead_f[x.row]) continue;
            if (std::abs(x.val) < 1e-30) continue;
            if (L.dead[x.col]) {
                e2.push_back({x.row, ch1[x.col], 0.5 * x.val});
                e2.push_back({x.row, ch2[x.col], 0.5 * x.val});
            } else {
                e2.push_back(x);
            }
        }
        // merge equal (row, col) in insertion order, output sorted (std::map semantics)
        std::stable_sort(e2.begin(), e2.end(), [](const Ent& a, const Ent& b) {
            return a.row != b.row ? a.row < b.row : a.col < b.col;
        });
        ent.clear();
        for (size_t k = 0; k < e2.size();) {
            const int r = e2[k].row, c = e2[k].col;
            double s = 0.0;
            while (k < e2.size() && e2[k].row == r && e2[k].col == c) s += e2[k++].val;
            if (std::abs(s) > 1e-30) ent.push_back({r, c, s});
        }
    }
    L.ce_ptr.assign(nf + 1, 0);
    for (const Ent& x : ent) L.ce_ptr[x.row + 1]++;
    for (int f = 0; f < nf; ++f) L.ce_ptr[f + 1] += L.ce_ptr[f];
    L.ce_idx.resize(ent.size());
    L.ce_val.resize(ent.size());
    {
        std::vector<int> pos(L.ce_ptr.begin(), L.ce_ptr.end() - 1);
        for (const Ent& x : ent) { const int p = pos[x.row]++; L.ce_idx[p] = x.col; L.ce_val[p] = x.val; }
    }

    // ---- face mass inverse (operators.cpp:539-551) ----
    std::vector<double> mfi(nf);
    for (int f = 0; f < nf; ++f) {
        if (L.dead_f[f]) { mfi[f] = 0.0; continue; }
        const double mf = kMu0 * L.farea[f] / L.fdual[f];
        mfi[f] = mf > 1e-30 ? 1.0 / mf : 0.0;
    }

    // ---- S = Ce^T Mf^-1 Ce: pattern of operators.cpp:631-651, values of :586-604 ----
    // Row i visits the faces through edge i in increasing face order, so each
    // (i, j) accumulates its face terms in the reference's order.
    {
        std::vector<int> tptr(ne + 1, 0), tidx(L.ce_idx.size());
        std::vector<double> tval(L.ce_idx.size());
        for (int k = 0; k < (int)L.ce_idx.size(); ++k) tptr[L.ce_idx[k] + 1]++;
        for (int e = 0; e < ne; ++e) tptr[e + 1] += tptr[e];
        {
            std::vector<int> pos(tptr.begin(), tptr.end() - 1);
            for (int f = 0; f < nf; ++f)
                for (int k = L.ce_ptr[f]; k < L.ce_ptr[f + 1]; ++k) {
                    const int p = pos[L.ce_idx[k]]++;
                    tidx[p] = f; tval[p] = L.ce_val[k];
                }
        }
        L.s_ptr.assign(ne + 1, 0);
        L.s_idx.clear(); L.s_val.clear();
        L.s_idx.reserve((size_t)ne * 20); L.s_val.reserve((size_t)ne * 20);
        std::vector<std::pair<int, double>> row;
        for (int i = 0; i < ne; ++i) {
            row.clear();
            row.push_back({i, 0.0});
            for (int t = tptr[i]; t < tptr[i + 1]; ++t) {
                const int f = tidx[t];
                const double cfi = tval[t];
                const double m = mfi[f];
                for (int k = L.ce_ptr[f]; k < L.ce_ptr[f + 1]; ++k) {
                    const int j = L.ce_idx[k];
                    const double v = cfi * m * L.ce_val[k];
                    auto it = std::find_if(row.begin(), row.end(), [j](const auto& p) { return p.first == j; });
                    if (it == row.end()) row.push_back({j, v});
                    else it->second += v;
                }
            }
            std::sort(row.begin(), row.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
            for (const auto& p : row) { L.s_idx.push_back(p.first); L.s_val.push_back(p.second); }
            L.s_ptr[i + 1] = (int)L.s_idx.size();
        }
    }

    // ---- node gradient (operators.cpp:849-944) ----
    {
        double minL = 1e30;
        for (int e = 0; e < ne; ++e) if (L.elen[e] > 1e-10) minL = std::min(minL, L.elen[e]);
        const double tol = minL * 0.01;
        KeyMap nm((size_t)ne);
        L.n1.resize(ne); L.n2.resize(ne);
        int nn = 0;
        for (int e = 0; e < ne; ++e) {
            const int d = L.edir[e];
            const double hl = L.elen[e] * 0.5;
            double p1[3] = {L.ex[e], L.ey[e], L.ez[e]};
            double p2[3] = {L.ex[e], L.ey[e], L.ez[e]};
            p1[d] -= hl; p2[d] += hl;
            for (int s = 0; s < 2; ++s) {
                const double* p = s ? p2 : p1;
                const int64_t k[3] = {(int64_t)std::llround(p[0] / tol), (int64_t)std::llround(p[1] / tol),
                                      (int64_t)std::llround(p[2] / tol)};
                bool ins;
                int& slot = nm.get(k, ins);
                if (ins) slot = nn++;
                (s ? L.n2 : L.n1)[e] = slot;
            }
        }
        L.nn = nn;
    }
}

}  // namespace m3d
