// Aggregation AMG setup (see amg.hpp).  Aggregation follows Vanek,
// Mandel and Brezina, "Algebraic multigrid by smoothed aggregation for second
// and fourth order elliptic problems", Computing 56 (1996): strength of
// connection |a_ij| >= theta sqrt(a_ii a_jj), greedy aggregates around roots
// whose strong neighbourhood is still free, leftovers attached to the
// aggregate they are most strongly tied to; tentative prolongator piecewise
// constant, optionally smoothed by one damped Jacobi step (omega_p > 0);
// Galerkin coarse operators.
#include "host/amg.hpp"

#include <algorithm>
#include <cmath>
#include <stdexcept>
#include <thread>

namespace m3d {

namespace {

std::vector<double> diagonal(const CsrReal& A) {
    std::vector<double> d(A.n_rows, 0.0);
    for (int i = 0; i < A.n_rows; ++i)
        for (int k = A.ptr[i]; k < A.ptr[i + 1]; ++k)
            if (A.col[k] == i) d[i] += A.val[k];
    return d;
}

// Strong off-diagonal neighbours of every row.
void strength(const CsrReal& A, const std::vector<double>& d, double theta, std::vector<int>& sptr,
              std::vector<int>& scol, std::vector<double>& sw) {
    const int n = A.n_rows;
    sptr.assign(n + 1, 0);
    scol.clear();
    sw.clear();
    for (int i = 0; i < n; ++i) {
        for (int k = A.ptr[i]; k < A.ptr[i + 1]; ++k) {
            const int j = A.col[k];
            if (j == i) continue;
            const double a = std::fabs(A.val[k]);
            if (a == 0.0 || d[i] <= 0.0 || d[j] <= 0.0) continue;
            if (a >= theta * std::sqrt(d[i] * d[j])) {
                scol.push_back(j);
                sw.push_back(a);
            }
        }
        sptr[i + 1] = (int)scol.size();
    }
}

int aggregate(const CsrReal& A, const std::vector<double>& d, double theta, std::vector<int>& agg) {
    const int n = A.n_rows;
    std::vector<int> sptr, scol;
    std::vector<double> sw;
    strength(A, d, theta, sptr, scol, sw);
    agg.assign(n, -1);
    int na = 0;
    // 1: roots with an entirely free strong neighbourhood
    for (int i = 0; i < n; ++i) {
        if (agg[i] != -1 || sptr[i] == sptr[i + 1]) continue;
        bool free_nb = true;
        for (int k = sptr[i]; k < sptr[i + 1] && free_nb; ++k) free_nb = agg[scol[k]] == -1;
        if (!free_nb) continue;
        agg[i] = na;
        for (int k = sptr[i]; k < sptr[i + 1]; ++k) agg[scol[k]] = na;
        ++na;
    }
    // 2: attach free nodes to the aggregate of their strongest aggregated neighbour
    std::vector<int> agg2 = agg;
    for (int i = 0; i < n; ++i) {
        if (agg[i] != -1) continue;
        double best = -1.0;
        for (int k = sptr[i]; k < sptr[i + 1]; ++k) {
            const int j = scol[k];
            if (agg[j] != -1 && sw[k] > best) {
                best = sw[k];
                agg2[i] = agg[j];
            }
        }
    }
    agg.swap(agg2);
    // 3: what is left (strong neighbours all free) forms new aggregates
    for (int i = 0; i < n; ++i) {
        if (agg[i] != -1 || sptr[i] == sptr[i + 1]) continue;
        agg[i] = na;
        for (int k = sptr[i]; k < sptr[i + 1]; ++k)
            if (agg[scol[k]] == -1) agg[scol[k]] = na;
        ++na;
    }
    return na;
}

// P = (I - omega D^-1 A) P0, P0 the piecewise-constant aggregate indicator.
void smoothed_prolongator(const CsrReal& A, const std::vector<double>& d, const std::vector<int>& agg, int na,
                          double omega, CsrReal& P) {
    const int n = A.n_rows;
    P.n_rows = n;
    P.n_cols = na;
    P.ptr.assign(n + 1, 0);
    P.col.clear();
    P.val.clear();
    std::vector<double> acc(na, 0.0);
    std::vector<int> mark(na, -1), touched;
    for (int i = 0; i < n; ++i) {
        touched.clear();
        auto add = [&](int J, double v) {
            if (mark[J] != i) {
                mark[J] = i;
                acc[J] = 0.0;
                touched.push_back(J);
            }
            acc[J] += v;
        };
        if (agg[i] >= 0) add(agg[i], 1.0);
        if (d[i] > 0.0) {
            const double s = omega / d[i];
            for (int k = A.ptr[i]; k < A.ptr[i + 1]; ++k) {
                const int J = agg[A.col[k]];
                if (J >= 0) add(J, -s * A.val[k]);
            }
        }
        std::sort(touched.begin(), touched.end());
        for (int J : touched) {
            if (acc[J] == 0.0) continue;
            P.col.push_back(J);
            P.val.push_back(acc[J]);
        }
        P.ptr[i + 1] = (int)P.col.size();
    }
}

void transpose(const CsrReal& P, CsrReal& R) {
    R.n_rows = P.n_cols;
    R.n_cols = P.n_rows;
    R.ptr.assign(R.n_rows + 1, 0);
    for (int c : P.col) R.ptr[c + 1]++;
    for (int i = 0; i < R.n_rows; ++i) R.ptr[i + 1] += R.ptr[i];
    R.col.assign(P.col.size(), 0);
    R.val.assign(P.val.size(), 0.0);
    std::vector<int> pos(R.ptr.begin(), R.ptr.end() - 1);
    for (int i = 0; i < P.n_rows; ++i)
        for (int k = P.ptr[i]; k < P.ptr[i + 1]; ++k) {
            const int q = pos[P.col[k]]++;
            R.col[q] = i;
            R.val[q] = P.val[k];
        }
}

// C = A B (CSR), columns sorted within each row.
void spgemm(const CsrReal& A, const CsrReal& B, CsrReal& C) {
    C.n_rows = A.n_rows;
    C.n_cols = B.n_cols;
    C.ptr.assign(A.n_rows + 1, 0);
    C.col.clear();
    C.val.clear();
    std::vector<double> acc(B.n_cols, 0.0);
    std::vector<int> mark(B.n_cols, -1), touched;
    for (int i = 0; i < A.n_rows; ++i) {
        touched.clear();
        for (int k = A.ptr[i]; k < A.ptr[i + 1]; ++k) {
            const int j = A.col[k];
            const double a = A.val[k];
            for (int q = B.ptr[j]; q < B.ptr[j + 1]; ++q) {
                const int c = B.col[q];
                if (mark[c] != i) {
                    mark[c] = i;
                    acc[c] = 0.0;
                    touched.push_back(c);
                }
                acc[c] += a * B.val[q];
            }
        }
        std::sort(touched.begin(), touched.end());
        for (int c : touched) {
            C.col.push_back(c);
            C.val.push_back(acc[c]);
        }
        C.ptr[i + 1] = (int)C.col.size();
    }
}

// Dense inverse by Gauss-Jordan elimination with partial pivoting; a pivot
// that vanishes (a row the operator does not reach) is replaced by 1.
void dense_inverse(const CsrReal& A, std::vector<double>& inv) {
    const int n = A.n_rows;
    std::vector<double> a((size_t)n * n, 0.0);
    inv.assign((size_t)n * n, 0.0);
    double scale = 0.0;
    for (int i = 0; i < n; ++i) {
        inv[(size_t)i * n + i] = 1.0;
        for (int k = A.ptr[i]; k < A.ptr[i + 1]; ++k) {
            a[(size_t)i * n + A.col[k]] += A.val[k];
            scale = std::max(scale, std::fabs(A.val[k]));
        }
    }
    const double tiny = 1e-14 * (scale > 0.0 ? scale : 1.0);
    for (int c = 0; c < n; ++c) {
        int p = c;
        for (int r = c + 1; r < n; ++r)
            if (std::fabs(a[(size_t)r * n + c]) > std::fabs(a[(size_t)p * n + c])) p = r;
        if (std::fabs(a[(size_t)p * n + c]) < tiny) {
            // unreachable direction: identity on it
            for (int k = 0; k < n; ++k) { a[(size_t)c * n + k] = 0.0; a[(size_t)k * n + c] = 0.0; }
            a[(size_t)c * n + c] = 1.0;
            for (int k = 0; k < n; ++k) { inv[(size_t)c * n + k] = 0.0; }
            inv[(size_t)c * n + c] = 1.0;
            p = c;
        }
        if (p != c)
            for (int k = 0; k < n; ++k) {
                std::swap(a[(size_t)p * n + k], a[(size_t)c * n + k]);
                std::swap(inv[(size_t)p * n + k], inv[(size_t)c * n + k]);
            }
        const double piv = a[(size_t)c * n + c];
        for (int k = 0; k < n; ++k) {
            a[(size_t)c * n + k] /= piv;
            inv[(size_t)c * n + k] /= piv;
        }
        for (int r = 0; r < n; ++r) {
            if (r == c) continue;
            const double f = a[(size_t)r * n + c];
            if (f == 0.0) continue;
            for (int k = 0; k < n; ++k) {
                a[(size_t)r * n + k] -= f * a[(size_t)c * n + k];
                inv[(size_t)r * n + k] -= f * inv[(size_t)c * n + k];
            }
        }
    }
}

}  // namespace

void amg_build(const CsrReal& A0, const AmgOptions& opt, AmgHierarchy& H) {
    H.levels.clear();
    H.aggregates.clear();
    H.levels.emplace_back();
    H.levels[0].A = A0;
    for (int l = 0;; ++l) {
        AmgLevel& L = H.levels[l];
        const std::vector<double> d = diagonal(L.A);
        L.dinv.assign(L.A.n_rows, 1.0);
        for (int i = 0; i < L.A.n_rows; ++i)
            if (std::fabs(d[i]) > 1e-300) L.dinv[i] = 1.0 / d[i];
        if (L.A.n_rows <= opt.max_coarse || l + 1 >= opt.max_levels) break;
        std::vector<int> agg;
        const int na = aggregate(L.A, d, opt.theta, agg);
        if (na == 0 || na > 0.85 * L.A.n_rows) break;   // coarsening stalled
        smoothed_prolongator(L.A, d, agg, na, opt.omega_p, L.P);
        H.aggregates.push_back(agg);
        transpose(L.P, L.R);
        CsrReal AP;
        spgemm(L.A, L.P, AP);
        AmgLevel next;
        spgemm(L.R, AP, next.A);
        H.levels.push_back(std::move(next));
    }
    const AmgLevel& C = H.levels.back();
    if (C.A.n_rows > 4096) throw std::runtime_error("multigrid coarsening left too large a coarse level");
    H.n_coarse = C.A.n_rows;
    dense_inverse(C.A, H.coarse_inv);
}

void amg_refresh(const CsrReal& A0, const AmgOptions& opt, AmgHierarchy& H) {
    if (H.levels.empty()) throw std::runtime_error("no hierarchy to refresh");
    H.levels[0].A = A0;
    amg_refresh_values(opt, H);
}

void amg_refresh_values(const AmgOptions& opt, AmgHierarchy& H) {
    if (opt.omega_p != 0.0) throw std::runtime_error("multigrid refresh needs piecewise-constant prolongation");
    const int nl = (int)H.levels.size();
    if (nl < 1 || (int)H.aggregates.size() != nl - 1) throw std::runtime_error("no hierarchy to refresh");
    for (int l = 0; l < nl; ++l) {
        AmgLevel& L = H.levels[l];
        const std::vector<double> d = diagonal(L.A);
        L.dinv.assign(L.A.n_rows, 1.0);
        for (int i = 0; i < L.A.n_rows; ++i)
            if (std::fabs(d[i]) > 1e-300) L.dinv[i] = 1.0 / d[i];
        if (l + 1 == nl) break;
        const std::vector<int>& agg = H.aggregates[l];
        if ((int)agg.size() != L.A.n_rows) throw std::runtime_error("hierarchy does not match the operator");
        // A_{l+1}[I][J] = sum of a_ij over i in I, j in J (P0^T A P0), with the
        // pattern of the previous coarse operator
        AmgLevel& C = H.levels[l + 1];
        std::fill(C.A.val.begin(), C.A.val.end(), 0.0);
        // coarse rows are independent (each entry is summed by one thread in
        // the same order), so they are split across host threads
        const int nI = C.A.n_rows;
        const int nt = std::max(1, std::min<int>(16, (int)std::thread::hardware_concurrency()));
        std::vector<char> bad(nt, 0);
        auto rows = [&](int t) {
            std::vector<int> pos(nI, -1);
            for (int I = (int)((long)nI * t / nt); I < (int)((long)nI * (t + 1) / nt); ++I) {
                for (int k = C.A.ptr[I]; k < C.A.ptr[I + 1]; ++k) pos[C.A.col[k]] = k;
                for (int q = L.R.ptr[I]; q < L.R.ptr[I + 1]; ++q) {
                    const int i = L.R.col[q];
                    for (int k = L.A.ptr[i]; k < L.A.ptr[i + 1]; ++k) {
                        const int J = agg[L.A.col[k]];
                        if (J < 0) continue;
                        if (pos[J] < C.A.ptr[I]) { bad[t] = 1; return; }
                        C.A.val[pos[J]] += L.A.val[k];
                    }
                }
            }
        };
        if (nt == 1 || nI < 4096) {
            for (int t = 0; t < nt; ++t) rows(t);
        } else {
            std::vector<std::thread> th;
            for (int t = 0; t < nt; ++t) th.emplace_back(rows, t);
            for (auto& x : th) x.join();
        }
        for (char b : bad)
            if (b) throw std::runtime_error("coarse pattern changed");
    }
    const AmgLevel& Cl = H.levels.back();
    H.n_coarse = Cl.A.n_rows;
    dense_inverse(Cl.A, H.coarse_inv);
}

}  // namespace m3d
