// RegularizationOctree::setup restated on the host layout (see regularization.hpp).
#include "host/regularization.hpp"

#include <algorithm>
#include <cmath>
#include <tuple>

namespace m3d {

void reg_build(const HostLayout& L, const RegParams& p, RegHost& R) {
    R = RegHost{};
    R.p = p;
    const int nc = L.nc;
    R.nc = nc;
    R.g2a.assign(nc, -1);
    for (int c = 0; c < nc; ++c)
        if (L.ctype[c] == 0) { R.g2a[c] = (int)R.a2g.size(); R.a2g.push_back(c); }
    const int na = (int)R.a2g.size();
    R.na = na;
    // cell volumes from the level (OctreeMesh::cell_size_xyz)
    std::vector<double> vol(nc);
    for (int c = 0; c < nc; ++c) {
        const double h = 1.0 / (double)(1 << L.clevel[c]);
        const double dx = h * (L.domain[1] - L.domain[0]), dy = h * (L.domain[3] - L.domain[2]),
                     dz = h * (L.domain[5] - L.domain[4]);
        vol[c] = dx * dy * dz;
    }
    struct Entry { int row, col, ord; double val; };
    std::vector<Entry> q;
    std::vector<std::tuple<int, int, double>> faces;   // (a, b, w) in face order
    R.diagw.assign(na, 0.0);
    const int nf = (int)L.fcm.size();
    for (int f = 0; f < nf; ++f) {
        const int cm = L.fcm[f], cp = L.fcp[f];
        if (cm < 0 || cp < 0 || cm >= nc || cp >= nc) continue;
        const int am = R.g2a[cm], ap = R.g2a[cp];
        if (am < 0 || ap < 0) continue;
        const int n = L.fnorm[f];
        const double al = n == 0 ? p.alpha_x : n == 1 ? p.alpha_y : n == 2 ? p.alpha_z : 1.0;
        const double ddx = L.ccx[cm] - L.ccx[cp], ddy = L.ccy[cm] - L.ccy[cp], ddz = L.ccz[cm] - L.ccz[cp];
        const double dist = std::sqrt(ddx * ddx + ddy * ddy + ddz * ddz);
        if (dist < 1e-10) continue;
        const double vgm = std::pow(vol[cm] * vol[cp], 1.0 / 6.0);
        const double w = al * L.farea[f] / (dist * vgm);
        const int o = (int)q.size();
        q.push_back({am, am, o, w});
        q.push_back({am, ap, o + 1, -w});
        q.push_back({ap, ap, o + 2, w});
        q.push_back({ap, am, o + 3, -w});
        faces.emplace_back(am, ap, w);
        R.diagw[am] += w;
        R.diagw[ap] += w;
    }
    // entries summed per (row, col) in face order, as the map accumulation does
    std::sort(q.begin(), q.end(), [](const Entry& a, const Entry& b) {
        return std::tie(a.row, a.col, a.ord) < std::tie(b.row, b.col, b.ord);
    });
    R.ptr.assign(na + 1, 0);
    for (size_t t = 0; t < q.size();) {
        const int r = q[t].row, c = q[t].col;
        double s = 0.0;
        for (; t < q.size() && q[t].row == r && q[t].col == c; ++t) {
            if (q[t].val < 0) s -= -q[t].val;
            else s += q[t].val;
        }
        R.idx.push_back(c);
        R.val.push_back(s);
        R.ptr[r + 1]++;
    }
    for (int i = 0; i < na; ++i) R.ptr[i + 1] += R.ptr[i];
    std::vector<int> cnt(na, 0);
    for (const auto& f : faces) { cnt[std::get<0>(f)]++; cnt[std::get<1>(f)]++; }
    R.aptr.assign(na + 1, 0);
    for (int i = 0; i < na; ++i) R.aptr[i + 1] = R.aptr[i] + cnt[i];
    R.aidx.assign(R.aptr[na], 0);
    R.aw.assign(R.aptr[na], 0.0);
    std::vector<int> fill(na, 0);
    for (const auto& f : faces) {
        const int a = std::get<0>(f), b = std::get<1>(f);
        const double w = std::get<2>(f);
        R.aidx[R.aptr[a] + fill[a]] = b; R.aw[R.aptr[a] + fill[a]] = w; fill[a]++;
        R.aidx[R.aptr[b] + fill[b]] = a; R.aw[R.aptr[b] + fill[b]] = w; fill[b]++;
    }
    // unit average diagonal (:146-160)
    double dsum = 0.0;
    for (int i = 0; i < na; ++i) dsum += R.diagw[i];
    const double davg = na > 0 ? dsum / na : 1.0;
    if (davg > 1e-30) {
        const double sc = 1.0 / davg;
        for (double& v : R.val) v *= sc;
        for (double& d : R.diagw) d *= sc;
        for (double& w : R.aw) w *= sc;
    }
}

}  // namespace m3d
