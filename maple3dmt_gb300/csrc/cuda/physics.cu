// Non-Krylov kernels of the solve path.  See physics.cuh for the reference
// code each launcher restates.
#include "physics.cuh"
#include "gradcorr.cuh"
#include "staged.cuh"

#include <algorithm>
#include <stdexcept>
#include <vector>

namespace m3d {
namespace phys {

using namespace dev;

namespace {

constexpr double kMu0 = 4.0e-7 * 3.14159265358979323846;

inline void ck() {
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) throw std::runtime_error(cudaGetErrorString(e));
}

inline int grid1(long n, int cap = 65536) {
    long b = (n + kBlock - 1) / kBlock;
    if (b < 1) b = 1;
    if (b > cap) b = cap;
    return (int)b;
}

__device__ __forceinline__ double2 zero2() { return make_double2(0.0, 0.0); }

// principal square root (Kahan's formulation of the half-angle formula)
__device__ double2 csqrt_d(double2 z) {
    const double r = hypot(z.x, z.y);
    if (r == 0.0) return zero2();
    const double t = sqrt((r + fabs(z.x)) * 0.5);
    if (z.x >= 0.0) return make_double2(t, z.y / (2.0 * t));
    return make_double2(fabs(z.y) / (2.0 * t), copysign(t, z.y));
}

// exp(a + ib) = e^a (cos b, sin b)
__device__ double2 cexp_d(double2 z) {
    double s, c;
    sincos(z.y, &s, &c);
    const double e = exp(z.x);
    return make_double2(e * c, e * s);
}

// ---------------------------------------------------------------------------
// assembly
// ---------------------------------------------------------------------------

__global__ void k_edge_mass(MeshDev m, const double* __restrict__ sigma, double* __restrict__ Me,
                            double* __restrict__ me_dc) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= m.n_pad) return;
    const unsigned char fl = m.flags[row];
    if (fl & kFlagPad) { Me[row] = 0.0; me_dc[row] = 0.0; return; }
    const int a0 = m.adj_ptr[row], a1 = m.adj_ptr[row + 1];
    double sum = 0.0;
    int count = 0;
    for (int k = a0; k < a1; ++k) { sum += sigma[m.adj_cell[k]]; ++count; }
    const double sa = count > 0 ? sum / count : 1e-8;
    const bool dead = (fl & kFlagDead) != 0;
    Me[row] = (dead || a1 == a0) ? 0.0 : sa * m.me_geom[row];      // operators.cpp:494-517
    me_dc[row] = dead ? 0.0 : sa * m.adual[row] * m.elen[row];      // operators.cpp:958-972
}

// (S_ii, Me_i) on free rows and (1, 0) on constrained / padding rows: the
// frequency-independent pair from which the batched kernels form
// d_f = S_ii + i omega_f Me_i.
__global__ void k_diag_coeffs(MeshDev m, const double* __restrict__ Me, double2* sm, float2* sm32) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= m.n_pad) return;
    double2 v;
    if (m.flags[row] & (kFlagConstrained | kFlagPad)) v = make_double2(1.0, 0.0);
    else v = make_double2(m.s_diag[row], Me[row]);
    sm[row] = v;
    sm32[row] = make_float2((float)v.x, (float)v.y);
}

// ---------------------------------------------------------------------------
// right-hand sides and post-processing
// ---------------------------------------------------------------------------

__global__ void k_primary(MeshDev m, VecK out, RhsInfo info, int bc_only) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int K = out.K;
    if (i >= (long)m.n_pad * K) return;
    const int row = (int)(i / K), k = (int)(i % K);
    const unsigned char fl = m.flags[row];
    double2 v = zero2();
    const int pol = info.pol[k];
    if (!(fl & kFlagPad) && pol >= 0 && m.dir[row] == pol && (!bc_only || (fl & kFlagBc))) {
        const double z = m.ez[row];
        const double2 ik = info.ik[k];
        if (z >= 0.0) v = make_double2(1.0 + ik.x * z, ik.y * z);
        else v = cexp_d(make_double2(ik.x * z, ik.y * z));
    }
    out.p[i] = v;
}

__global__ void k_lift(MeshDev m, VecK ebc, VecK rhs) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int K = rhs.K;
    if (i >= (long)m.n_pad * K) return;
    const int row = (int)(i / K), k = (int)(i % K);
    const unsigned char fl = m.flags[row];
    double2 v = zero2();
    if (fl & kFlagPad) {
    } else if (fl & kFlagBc) {
        v = ebc.p[i];
    } else if (!(fl & kFlagConstrained)) {
        for (int q = m.lift_ptr[row]; q < m.lift_ptr[row + 1]; ++q) {
            const double a = m.lift_val[q];
            const double2 e = ebc.p[(size_t)m.lift_col[q] * K + k];
            v.x -= a * e.x;
            v.y -= a * e.y;
        }
    }
    rhs.p[i] = v;
}

__global__ void k_vsub(long n, const double2* __restrict__ a, const double2* __restrict__ b, double2* out) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = csub(a[i], b[i]);
}

__global__ void k_hanging(MeshDev m, VecK x) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int K = x.K;
    if (i >= (long)m.nhp * K) return;
    const int h = (int)(i / K), k = (int)(i % K);
    const int c = m.hp[3 * h], c1 = m.hp[3 * h + 1], c2 = m.hp[3 * h + 2];
    const double2 a = x.p[(size_t)c1 * K + k], b = x.p[(size_t)c2 * K + k];
    x.p[(size_t)c * K + k] = make_double2(0.5 * (a.x + b.x), 0.5 * (a.y + b.y));
}

// list order matters when a child is itself a coarse edge: one thread per rhs
__global__ void k_hanging_seq(MeshDev m, VecK x) {
    const int k = threadIdx.x;
    if (k >= x.K) return;
    const int K = x.K;
    for (int h = 0; h < m.nhp; ++h) {
        const int c = m.hp[3 * h], c1 = m.hp[3 * h + 1], c2 = m.hp[3 * h + 2];
        const double2 a = x.p[(size_t)c1 * K + k], b = x.p[(size_t)c2 * K + k];
        x.p[(size_t)c * K + k] = make_double2(0.5 * (a.x + b.x), 0.5 * (a.y + b.y));
    }
}

__global__ void k_combine(MeshDev m, VecK epri, VecK esec, VecK ebc, VecK e) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int K = e.K;
    if (i >= (long)m.n_pad * K) return;
    const int row = (int)(i / K);
    const unsigned char fl = m.flags[row];
    e.p[i] = (fl & kFlagBc) ? ebc.p[i] : cadd(epri.p[i], esec.p[i]);
}

__global__ void k_to_perm(MeshDev m, const double2* __restrict__ ref, VecK dst, int k) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < m.ne) dst.p[(size_t)m.iperm[e] * dst.K + k] = ref[e];
}

__global__ void k_from_perm(MeshDev m, VecK src, int k, double2* __restrict__ ref) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < m.ne) ref[e] = src.p[(size_t)m.iperm[e] * src.K + k];
}

// ---------------------------------------------------------------------------
// divergence correction
// ---------------------------------------------------------------------------

__global__ void k_dc_lap(MeshDev m, const double* __restrict__ me, DcWork w) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= m.nn) return;
    const int a = m.inc_ptr[v], b = m.inc_ptr[v + 1];
    if (m.node_bc[v]) {
        w.lap_diag[v] = 1.0;
        w.jac_inv[v] = 1.0;
        for (int q = a; q < b; ++q) {
            w.lap_off[q] = 0.0;
            reinterpret_cast<double*>(w.lap_seg)[w.lap_qpos[q]] = 0.0;
        }
        return;
    }
    double diag = 0.0;
    bool any = false;
    for (int q = a; q < b; ++q) {
        const int e = m.inc_edge[q];
        const double we = me[e];
        double off = 0.0;
        if (we >= 1e-30) {
            const double gv = m.inc_gv[q], gw = m.inc_gw[q];
            diag += gv * we * gv;
            any = true;
            if (!m.node_bc[m.inc_other[q]]) off = gv * we * gw;
        }
        w.lap_off[q] = off;
        reinterpret_cast<double*>(w.lap_seg)[w.lap_qpos[q]] = off;
    }
    w.lap_diag[v] = diag;
    // Jacobi preconditioner z = r / diag (r where the diagonal is absent or
    // below 1e-30), stored as its inverse so the PCG multiplies
    w.jac_inv[v] = (any && fabs(diag) > 1e-30) ? 1.0 / diag : 1.0;
}

// phi0_v = sum_e G[e,v] rhs_e / (i omega)
__global__ void k_dc_phi0(MeshDev m, VecK rhs, RhsInfo info, DcWork w) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int K = rhs.K;
    if (i >= (long)m.nn * K) return;
    const int v = (int)(i / K), k = (int)(i % K);
    double2 acc = zero2();
    for (int q = m.inc_ptr[v]; q < m.inc_ptr[v + 1]; ++q) {
        const int e = m.inc_edge[q];
        if (m.flags[e] & kFlagDead) continue;
        const double2 r = rhs.p[(size_t)e * K + k];
        acc.x += m.inc_gv[q] * r.x;
        acc.y += m.inc_gv[q] * r.y;
    }
    w.phi0[i] = cdiv(acc, make_double2(0.0, info.omega[k]));
}

// divJ = G^T (me E) - phi0, zero on BC nodes; |divJ| -> outer-loop test
template <int K>
__global__ void __launch_bounds__(kBlock) k_dc_divj(MeshDev m, const double* __restrict__ me, VecK E,
                                                    int use_phi0, DcWork w, double tol, RedScratch rs) {
    const long n = (long)m.nn * K;
    const long i0 = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const long stride = (long)gridDim.x * blockDim.x;
    const int k = (int)(i0 % K);
    const bool act = w.st[k].active && !w.st[k].done;
    double2 acc[1] = {zero2()};
    for (long i = i0; i < n && act; i += stride) {
        const int v = (int)(i / K);
        double2 d = zero2();
        if (!m.node_bc[v]) {
            for (int q = m.inc_ptr[v]; q < m.inc_ptr[v + 1]; ++q) {
                const int e = m.inc_edge[q];
                const double we = me[e];
                if (m.flags[e] & kFlagDead) continue;
                const double2 ev = E.p[(size_t)e * K + k];
                const double2 wev = make_double2(we * ev.x, we * ev.y);
                d.x += m.inc_gv[q] * wev.x;
                d.y += m.inc_gv[q] * wev.y;
            }
            if (use_phi0) d = csub(d, w.phi0[i]);
        }
        w.divJ[i] = d;
        acc[0].x += d.x * d.x + d.y * d.y;
    }
    __shared__ double2 out[K];
    if (grid_reduce_lanes<1, K>(acc, rs, out)) {
        if (threadIdx.x < K) {
            DcState S = w.st[threadIdx.x];
            if (S.active && !S.done) {
                const double dn = sqrt(out[threadIdx.x].x);
                S.dn = dn;
                if (S.outer == 0) S.div0 = dn;
                const double rel = (S.div0 > 1e-30) ? dn / S.div0 : 0.0;
                if ((rel < tol && S.outer > 0) || dn < 1e-12) {
                    S.done = 1;
                    S.cg_run = 0;
                } else {
                    S.cg_run = 1;
                    S.cg_iter = 0;
                }
            }
            w.st[threadIdx.x] = S;
        }
    }
}

__device__ __forceinline__ double2 jac_apply(double2 r, double dinv) {
    return make_double2(r.x * dinv, r.y * dinv);
}

// The node Laplacian is real symmetric and the Jacobi preconditioner real
// positive, so (r, z) = sum |r|^2 / d and (p, L p) are real: the PCG scalars
// alpha, beta and (r, z) are carried as reals (imaginary parts zero), which
// is the reference's complex recurrence (forward_solver_fv.cpp:681-710)
// without its rounding-level imaginary parts, at a third of the FP64 work.

// phi = 0, r = divJ, z = r / diag, p = z, rz = (r, z)
template <int K>
__global__ void __launch_bounds__(kBlock) k_dc_cg_init(int nn, DcWork w, RedScratch rs) {
    const long n = (long)nn * K;
    const long i0 = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const long stride = (long)gridDim.x * blockDim.x;
    const int k = (int)(i0 % K);
    const bool run = w.st[k].cg_run;
    double2 acc[1] = {zero2()};
    for (long i = i0; i < n && run; i += stride) {
        const int v = (int)(i / K);
        const double2 r = w.divJ[i];
        const double2 z = jac_apply(r, w.jac_inv[v]);
        w.phi[i] = zero2();
        w.r[i] = r;
        w.z[i] = z;
        w.p[i] = z;
        acc[0].x += r.x * z.x + r.y * z.y;
    }
    __shared__ double2 out[K];
    if (grid_reduce_lanes<1, K>(acc, rs, out)) {
        if (threadIdx.x < K && w.st[threadIdx.x].cg_run) w.st[threadIdx.x].rz = make_double2(out[threadIdx.x].x, 0.0);
    }
}

// Ap = L p, (p, Ap) -> alpha   (forward_solver_fv.cpp:681-692), over
// 32-node slice segments of L's off-diagonal part staged in shared memory by
// bulk copies (staged.cuh): off-diagonal sum, then the diagonal term.
// Right-hand sides whose PCG has stopped do no work.
template <int K>
__global__ void __launch_bounds__(StagedShape<K>::NT, StagedMinBlocks<double, K>::v)
    k_dc_cg_ap_st(int nn, DcWork w, RedScratch rs) {
    using Sh = StagedShape<K>;
    constexpr int RPW = 32 / K;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int rhs = lane % K;
    const int lr0 = warp * RPW + lane / K;
    const bool run = w.st[rhs].cg_run;
    double2 acc[1] = {zero2()};
    slice_pipeline<1>(w.lap_seg, w.lap_work, w.n_node_slices, w.lap_stage, w.seg_err,
                      [&](const SegItem& it, const unsigned char* base) {
        SegRows<double> L;
        L.bind(base);
#pragma unroll
        for (int ps = 0; ps < Sh::PASSES; ++ps) {
            const int lr = ps * Sh::ROWS_PER_PASS + lr0;
            const int v = it.slice * kSlice + lr;
            if (v >= nn || !run) continue;
            const size_t i = (size_t)v * K + rhs;
            const double2 pv = w.p[i];
            const double dg = w.lap_diag[v];
            double2 s = seg_row_dot<double, K>(L.col, L.val, L.begin_of(lr), L.end[lr], w.p, rhs, zero2());
            s.x += dg * pv.x;
            s.y += dg * pv.y;
            w.Ap[i] = s;
            acc[0].x += pv.x * s.x + pv.y * s.y;
        }
    });
    __shared__ double2 out[K];
    if (grid_reduce_lanes<1, K, Sh::NT>(acc, rs, out)) {
        if (threadIdx.x < K) {
            DcState S = w.st[threadIdx.x];
            if (S.cg_run) {
                const double pAp = out[threadIdx.x].x;
                if (fabs(pAp) < 1e-30) S.cg_run = 0;
                else S.alpha = make_double2(S.rz.x / pAp, 0.0);
            }
            w.st[threadIdx.x] = S;
        }
    }
}

// phi += alpha p, r -= alpha Ap, |r| test, z = r / diag, beta   (:693-710)
template <int K>
__global__ void __launch_bounds__(kBlock) k_dc_cg_update(int nn, int cg_max, DcWork w, RedScratch rs) {
    const long n = (long)nn * K;
    const long i0 = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const long stride = (long)gridDim.x * blockDim.x;
    const int k = (int)(i0 % K);
    const DcState S0 = w.st[k];
    const bool run = S0.cg_run;
    const double al = S0.alpha.x;
    double2 acc[2] = {zero2(), zero2()};
    for (long i = i0; i < n && run; i += stride) {
        const int v = (int)(i / K);
        const double2 pv = w.p[i], apv = w.Ap[i];
        double2 ph = w.phi[i];
        ph.x += al * pv.x;
        ph.y += al * pv.y;
        w.phi[i] = ph;
        double2 r = w.r[i];
        r.x -= al * apv.x;
        r.y -= al * apv.y;
        w.r[i] = r;
        const double2 z = jac_apply(r, w.jac_inv[v]);
        w.z[i] = z;
        acc[0].x += r.x * r.x + r.y * r.y;
        acc[1].x += r.x * z.x + r.y * z.y;
    }
    __shared__ double2 out[2 * K];
    if (grid_reduce_lanes<2, K>(acc, rs, out)) {
        if (threadIdx.x < K) {
            DcState S = w.st[threadIdx.x];
            if (S.cg_run) {
                S.rn = out[threadIdx.x].x;
                S.cg_iter += 1;
                if (sqrt(S.rn) < 1e-10 * S.dn) {
                    S.cg_run = 0;
                } else {
                    const double rzn = out[K + threadIdx.x].x;
                    S.beta = make_double2(rzn / (S.rz.x + 1e-30), 0.0);
                    S.rz = make_double2(rzn, 0.0);
                    if (S.cg_iter >= cg_max) S.cg_run = 0;
                }
            }
            w.st[threadIdx.x] = S;
        }
    }
}

// p = z + beta p
template <int K>
__global__ void __launch_bounds__(kBlock) k_dc_cg_p(int nn, DcWork w) {
    const long n = (long)nn * K;
    const long i0 = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const long stride = (long)gridDim.x * blockDim.x;
    if (i0 >= n) return;
    const int k = (int)(i0 % K);
    if (!w.st[k].cg_run) return;
    const double be = w.st[k].beta.x;
    for (long i = i0; i < n; i += stride) {
        const double2 z = w.z[i];
        double2 pv = w.p[i];
        pv.x = z.x + be * pv.x;
        pv.y = z.y + be * pv.y;
        w.p[i] = pv;
    }
}

// ---------------------------------------------------------------------------
// Multigrid-preconditioned PCG (AmgDev).  Same recurrence as the Jacobi PCG
// above with z = M^-1 r from one V-cycle: one damped-Jacobi pre-smoothing
// step from zero, residual, restriction to the aggregates, the coarse
// correction, prolongation, one damped-Jacobi post-smoothing step -- a
// symmetric positive-definite preconditioner, so CG's recurrence and its
// stopping rule (|r| < 1e-10 |divJ|) are unchanged.
// ---------------------------------------------------------------------------

// phi = 0, r = divJ   (forward_solver_fv.cpp:668-679 without the Jacobi step)
template <int K>
__global__ void __launch_bounds__(kBlock) k_mg_cg_init(int nn, DcWork w) {
    const long n = (long)nn * K;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        if (!w.st[i % K].cg_run) continue;
        w.phi[i] = zero2();
        w.r[i] = w.divJ[i];
    }
}

// phi += alpha p, r -= alpha Ap, |r| test   (:693-704)
template <int K>
__global__ void __launch_bounds__(kBlock) k_mg_cg_update(int nn, int cg_max, DcWork w, RedScratch rs) {
    const long n = (long)nn * K;
    const long i0 = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const long stride = (long)gridDim.x * blockDim.x;
    const DcState S0 = w.st[i0 % K];
    const bool run = S0.cg_run;
    const double al = S0.alpha.x;
    double2 acc[1] = {zero2()};
    for (long i = i0; i < n && run; i += stride) {
        const double2 pv = w.p[i], apv = w.Ap[i];
        double2 ph = w.phi[i];
        ph.x += al * pv.x;
        ph.y += al * pv.y;
        w.phi[i] = ph;
        double2 r = w.r[i];
        r.x -= al * apv.x;
        r.y -= al * apv.y;
        w.r[i] = r;
        acc[0].x += r.x * r.x + r.y * r.y;
    }
    __shared__ double2 out[K];
    if (grid_reduce_lanes<1, K>(acc, rs, out)) {
        if (threadIdx.x < K) {
            DcState S = w.st[threadIdx.x];
            if (S.cg_run) {
                S.rn = out[threadIdx.x].x;
                S.cg_iter += 1;
                if (sqrt(S.rn) < 1e-10 * S.dn || S.cg_iter >= cg_max) S.cg_run = 0;
            }
            w.st[threadIdx.x] = S;
        }
    }
}

// x = omega dinv b   (pre-smoothing from a zero iterate)
template <int K>
__global__ void __launch_bounds__(kBlock) k_mg_pre(AmgLevelDev L, const double2* __restrict__ b,
                                                   double2* __restrict__ x, double omega, const DcState* st) {
    const long n = (long)L.n * K;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        if (!st[i % K].cg_run) continue;
        const double s = omega * L.dinv[i / K];
        const double2 bv = b[i];
        x[i] = make_double2(s * bv.x, s * bv.y);
    }
}

// (A_l x)_i for one row of a CSR level (levels >= 1), eight gathers in flight
template <int K>
__device__ __forceinline__ double2 mg_row(const AmgLevelDev& L, int row, const double2* __restrict__ x, int k) {
    double2 s = zero2();
    const int q0 = __ldg(&L.ptr[row]), q1 = __ldg(&L.ptr[row + 1]);
    for (int q = q0; q < q1; q += 8) {
        double a[8];
        double2 xv[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const bool ok = q + u < q1;
            const int c = ok ? __ldg(&L.col[q + u]) : 0;
            a[u] = ok ? __ldg(&L.val[q + u]) : 0.0;
            xv[u] = ok ? x[(size_t)c * K + k] : zero2();
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            s.x += a[u] * xv[u].x;
            s.y += a[u] * xv[u].y;
        }
    }
    return s;
}

// r = b - A_l x   (levels >= 1)
template <int K>
__global__ void __launch_bounds__(kBlock) k_mg_resid(AmgLevelDev L, const DcState* st) {
    const long n = (long)L.n * K;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int k = (int)(i % K);
        if (!st[k].cg_run) continue;
        const double2 ax = mg_row<K>(L, (int)(i / K), L.x, k);
        const double2 bv = L.b[i];
        L.r[i] = make_double2(bv.x - ax.x, bv.y - ax.y);
    }
}

// y = x + omega dinv (b - A_l x)   (post-smoothing, levels >= 1)
template <int K>
__global__ void __launch_bounds__(kBlock) k_mg_post(AmgLevelDev L, double omega, const DcState* st) {
    const long n = (long)L.n * K;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int k = (int)(i % K);
        if (!st[k].cg_run) continue;
        const int row = (int)(i / K);
        const double2 ax = mg_row<K>(L, row, L.x, k);
        const double2 bv = L.b[i], xv = L.x[i];
        const double s = omega * L.dinv[row];
        L.y[i] = make_double2(xv.x + s * (bv.x - ax.x), xv.y + s * (bv.y - ax.y));
    }
}

// b_next[I] = sum over the members i of aggregate I of r[i]
template <int K>
__global__ void __launch_bounds__(kBlock) k_mg_restrict(AmgLevelDev L, int n_next, const double2* __restrict__ r,
                                                        double2* __restrict__ b_next, const DcState* st) {
    const long n = (long)n_next * K;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int k = (int)(i % K);
        if (!st[k].cg_run) continue;
        const int I = (int)(i / K);
        double2 s = zero2();
        for (int q = L.rptr[I]; q < L.rptr[I + 1]; ++q) {
            const double2 v = r[(size_t)L.rcol[q] * K + k];
            s.x += v.x;
            s.y += v.y;
        }
        b_next[i] = s;
    }
}

// x[i] += x_next[agg[i]]
template <int K>
__global__ void __launch_bounds__(kBlock) k_mg_prolong(AmgLevelDev L, const double2* __restrict__ x_next,
                                                       double2* __restrict__ x, const DcState* st) {
    const long n = (long)L.n * K;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int k = (int)(i % K);
        if (!st[k].cg_run) continue;
        const int a = L.agg[i / K];
        if (a < 0) continue;
        const double2 v = x_next[(size_t)a * K + k];
        double2 xv = x[i];
        xv.x += v.x;
        xv.y += v.y;
        x[i] = xv;
    }
}

// coarsest level: x = A_c^-1 b (dense)
template <int K>
__global__ void __launch_bounds__(kBlock) k_mg_coarse(int nc, const double* __restrict__ inv,
                                                      const double2* __restrict__ b, double2* __restrict__ x,
                                                      const DcState* st) {
    const long n = (long)nc * K;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int k = (int)(i % K);
        if (!st[k].cg_run) continue;
        const int row = (int)(i / K);
        double2 s = zero2();
        for (int j = 0; j < nc; ++j) {
            const double a = __ldg(&inv[(size_t)row * nc + j]);
            const double2 v = b[(size_t)j * K + k];
            s.x += a * v.x;
            s.y += a * v.y;
        }
        x[i] = s;
    }
}

// Level-0 residual r0 = b - L x over the node slice segments.
template <int K>
__global__ void __launch_bounds__(StagedShape<K>::NT, StagedMinBlocks<double, K>::v)
    k_mg0_resid_st(int nn, DcWork w, const double2* __restrict__ b, const double2* __restrict__ x,
                   double2* __restrict__ r) {
    using Sh = StagedShape<K>;
    constexpr int RPW = 32 / K;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int rhs = lane % K;
    const int lr0 = warp * RPW + lane / K;
    const bool run = w.st[rhs].cg_run;
    slice_pipeline<1>(w.lap_seg, w.lap_work, w.n_node_slices, w.lap_stage, w.seg_err,
                      [&](const SegItem& it, const unsigned char* base) {
        SegRows<double> L;
        L.bind(base);
#pragma unroll
        for (int ps = 0; ps < Sh::PASSES; ++ps) {
            const int lr = ps * Sh::ROWS_PER_PASS + lr0;
            const int v = it.slice * kSlice + lr;
            if (v >= nn || !run) continue;
            const size_t i = (size_t)v * K + rhs;
            const double2 xv = x[i], bv = b[i];
            const double dg = w.lap_diag[v];
            double2 s = seg_row_dot<double, K>(L.col, L.val, L.begin_of(lr), L.end[lr], x, rhs, zero2());
            s.x += dg * xv.x;
            s.y += dg * xv.y;
            r[i] = make_double2(bv.x - s.x, bv.y - s.y);
        }
    });
}

// Level-0 post-smoothing z = x + omega dinv (r - L x), then (r, z) -> beta
// (:705-710): the last kernel of the preconditioner application.
template <int K>
__global__ void __launch_bounds__(StagedShape<K>::NT, StagedMinBlocks<double, K>::v)
    k_mg0_post_st(int nn, DcWork w, const double* __restrict__ dinv, double omega, const double2* __restrict__ x,
                  RedScratch rs) {
    using Sh = StagedShape<K>;
    constexpr int RPW = 32 / K;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int rhs = lane % K;
    const int lr0 = warp * RPW + lane / K;
    const bool run = w.st[rhs].cg_run;
    double2 acc[1] = {zero2()};
    slice_pipeline<1>(w.lap_seg, w.lap_work, w.n_node_slices, w.lap_stage, w.seg_err,
                      [&](const SegItem& it, const unsigned char* base) {
        SegRows<double> L;
        L.bind(base);
#pragma unroll
        for (int ps = 0; ps < Sh::PASSES; ++ps) {
            const int lr = ps * Sh::ROWS_PER_PASS + lr0;
            const int v = it.slice * kSlice + lr;
            if (v >= nn || !run) continue;
            const size_t i = (size_t)v * K + rhs;
            const double2 xv = x[i], rv = w.r[i];
            const double dg = w.lap_diag[v];
            double2 s = seg_row_dot<double, K>(L.col, L.val, L.begin_of(lr), L.end[lr], x, rhs, zero2());
            s.x += dg * xv.x;
            s.y += dg * xv.y;
            const double sc = omega * dinv[v];
            const double2 z = make_double2(xv.x + sc * (rv.x - s.x), xv.y + sc * (rv.y - s.y));
            w.z[i] = z;
            acc[0].x += rv.x * z.x + rv.y * z.y;
        }
    });
    __shared__ double2 out[K];
    if (grid_reduce_lanes<1, K, Sh::NT>(acc, rs, out)) {
        if (threadIdx.x < K) {
            DcState S = w.st[threadIdx.x];
            if (S.cg_run) {
                const double rzn = out[threadIdx.x].x;
                S.beta = make_double2(S.cg_iter == 0 ? 0.0 : rzn / (S.rz.x + 1e-30), 0.0);
                S.rz = make_double2(rzn, 0.0);
            }
            w.st[threadIdx.x] = S;
        }
    }
}

// One V-cycle: z = M^-1 r for every running right-hand side.  Returns launches.
template <int K>
long long mg_apply(const MeshDev& m, DcWork w, const AmgDev& A, RedScratch red, int cap, cudaStream_t s) {
    long long launches = 0;
    auto grid = [&](long n) {
        long g = (n + kBlock - 1) / kBlock;
        return (int)std::max(1L, std::min(g, (long)8 * 152 * 4));
    };
    const int nl = A.n_levels;
    // level 0: b = r; pre-smoothed iterate in lv[0].x
    const AmgLevelDev& L0 = A.lv[0];
    k_mg_pre<K><<<grid((long)m.nn * K), kBlock, 0, s>>>(L0, w.r, L0.x, A.omega, w.st);
    ++launches;
    if (nl > 1) {
        launch_staged(k_mg0_resid_st<K>, StagedShape<K>::NT, w.lap_stage, w.n_node_slices, 1 << 20, s, m.nn, w,
                      (const double2*)w.r, (const double2*)L0.x, L0.r);
        k_mg_restrict<K><<<grid((long)A.lv[1].n * K), kBlock, 0, s>>>(L0, A.lv[1].n, L0.r, A.lv[1].b, w.st);
        launches += 2;
        // down
        for (int l = 1; l < nl - 1; ++l) {
            const AmgLevelDev& L = A.lv[l];
            k_mg_pre<K><<<grid((long)L.n * K), kBlock, 0, s>>>(L, L.b, L.x, A.omega, w.st);
            k_mg_resid<K><<<grid((long)L.n * K), kBlock, 0, s>>>(L, w.st);
            k_mg_restrict<K><<<grid((long)A.lv[l + 1].n * K), kBlock, 0, s>>>(L, A.lv[l + 1].n, L.r, A.lv[l + 1].b,
                                                                              w.st);
            launches += 3;
        }
        // coarsest
        const AmgLevelDev& C = A.lv[nl - 1];
        k_mg_coarse<K><<<grid((long)C.n * K), kBlock, 0, s>>>(A.n_coarse, A.coarse_inv, C.b, C.x, w.st);
        ++launches;
        // up: prolong the finished iterate of level l+1 into level l, post-smooth
        for (int l = nl - 2; l >= 1; --l) {
            const AmgLevelDev& L = A.lv[l];
            const double2* xn = (l + 1 == nl - 1) ? A.lv[l + 1].x : A.lv[l + 1].y;
            k_mg_prolong<K><<<grid((long)L.n * K), kBlock, 0, s>>>(L, xn, L.x, w.st);
            k_mg_post<K><<<grid((long)L.n * K), kBlock, 0, s>>>(L, A.omega, w.st);
            launches += 2;
        }
        const double2* x1 = (nl - 1 == 1) ? A.lv[1].x : A.lv[1].y;
        k_mg_prolong<K><<<grid((long)m.nn * K), kBlock, 0, s>>>(L0, x1, L0.x, w.st);
        ++launches;
    }
    launch_staged(k_mg0_post_st<K>, StagedShape<K>::NT, w.lap_stage, w.n_node_slices, cap, s, m.nn, w, L0.dinv,
                  A.omega, (const double2*)L0.x, red);
    ++launches;
    return launches;
}

// E -= G phi on edges that are not BC (:714-720), for rhs still in the outer loop
__global__ void k_dc_grad(MeshDev m, VecK E, DcWork w) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int K = E.K;
    if (i >= (long)m.n_pad * K) return;
    const int row = (int)(i / K), k = (int)(i % K);
    const DcState& S = w.st[k];
    if (!S.active || S.done) return;
    const unsigned char fl = m.flags[row];
    if (fl & (kFlagPad | kFlagDcBc)) return;
    const int n0 = m.e_node[2 * row], n1 = m.e_node[2 * row + 1];
    const double g0 = m.e_g[2 * row], g1 = m.e_g[2 * row + 1];
    const double2 a = w.phi[(size_t)n0 * K + k], b = w.phi[(size_t)n1 * K + k];
    const double2 gr = make_double2(g0 * a.x + g1 * b.x, g0 * a.y + g1 * b.y);
    E.p[i] = csub(E.p[i], gr);
}

__global__ void k_dc_outer_done(int K, DcWork w) {
    const int k = threadIdx.x;
    if (k < K) {
        DcState S = w.st[k];
        if (S.active && !S.done) S.outer += 1;
        w.st[k] = S;
    }
}

// ---------------------------------------------------------------------------
// stations
// ---------------------------------------------------------------------------

__device__ __forceinline__ double2 cdivn(double2 a, int n) { return cdiv(a, make_double2((double)n, 0.0)); }
__device__ __forceinline__ double2 chalf(double2 a, double2 b) {
    return cmul(cadd(a, b), make_double2(0.5, 0.0));
}

__global__ void k_station_z(StationDev st, VecK E, const double* __restrict__ omegas, int nf,
                            HCache* hc, double2* Z) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nf * st.ns) return;
    const int f = i / st.ns, s = i % st.ns;
    const int K = E.K;
    HCache H;
    H.Hx1 = H.Hy1 = H.Hx2 = H.Hy2 = H.det = H.Zxx = H.Zxy = H.Zyx = H.Zyy = zero2();
    H.cdx = H.cdy = H.cdz = 0.0; H.pad_ = 0.0;
    double2* zo = Z + (size_t)i * 4;
    const int cell = st.cell[s];
    if (cell < 0) {
        hc[i] = H;
        zo[0] = zo[1] = zo[2] = zo[3] = zero2();
        return;
    }
    const double omega = omegas[f];
    const double2 iwmu = make_double2(0.0, omega * kMu0);
    const double cdx = st.geom[6 * s + 3], cdy = st.geom[6 * s + 4], cdz = st.geom[6 * s + 5];
    double2 Ex1t = zero2(), Ex1b = zero2(), Ex2t = zero2(), Ex2b = zero2();
    double2 Ey1t = zero2(), Ey1b = zero2(), Ey2t = zero2(), Ey2b = zero2();
    double2 Ez1px = zero2(), Ez1mx = zero2(), Ez2px = zero2(), Ez2mx = zero2();
    double2 Ez1py = zero2(), Ez1my = zero2(), Ez2py = zero2(), Ez2my = zero2();
    int nxt = 0, nxb = 0, nyt = 0, nyb = 0, npx = 0, nmx = 0, npy = 0, nmy = 0;
    for (int q = st.e_ptr[s]; q < st.e_ptr[s + 1]; ++q) {
        const int row = st.e_row[q];
        const unsigned char code = st.e_code[q];
        const int d = code & 3;
        const double2 e1 = E.p[(size_t)row * K + 2 * f], e2 = E.p[(size_t)row * K + 2 * f + 1];
        if (d == 0) {
            if (code & 4) { Ex1t = cadd(Ex1t, e1); Ex2t = cadd(Ex2t, e2); ++nxt; }
            else { Ex1b = cadd(Ex1b, e1); Ex2b = cadd(Ex2b, e2); ++nxb; }
        } else if (d == 1) {
            if (code & 4) { Ey1t = cadd(Ey1t, e1); Ey2t = cadd(Ey2t, e2); ++nyt; }
            else { Ey1b = cadd(Ey1b, e1); Ey2b = cadd(Ey2b, e2); ++nyb; }
        } else {
            if (code & 8) { Ez1px = cadd(Ez1px, e1); Ez2px = cadd(Ez2px, e2); ++npx; }
            else { Ez1mx = cadd(Ez1mx, e1); Ez2mx = cadd(Ez2mx, e2); ++nmx; }
            if (code & 16) { Ez1py = cadd(Ez1py, e1); Ez2py = cadd(Ez2py, e2); ++npy; }
            else { Ez1my = cadd(Ez1my, e1); Ez2my = cadd(Ez2my, e2); ++nmy; }
        }
    }
    if (nxt > 0) { Ex1t = cdivn(Ex1t, nxt); Ex2t = cdivn(Ex2t, nxt); }
    if (nxb > 0) { Ex1b = cdivn(Ex1b, nxb); Ex2b = cdivn(Ex2b, nxb); }
    if (nyt > 0) { Ey1t = cdivn(Ey1t, nyt); Ey2t = cdivn(Ey2t, nyt); }
    if (nyb > 0) { Ey1b = cdivn(Ey1b, nyb); Ey2b = cdivn(Ey2b, nyb); }
    if (npx > 0) { Ez1px = cdivn(Ez1px, npx); Ez2px = cdivn(Ez2px, npx); }
    if (nmx > 0) { Ez1mx = cdivn(Ez1mx, nmx); Ez2mx = cdivn(Ez2mx, nmx); }
    if (npy > 0) { Ez1py = cdivn(Ez1py, npy); Ez2py = cdivn(Ez2py, npy); }
    if (nmy > 0) { Ez1my = cdivn(Ez1my, nmy); Ez2my = cdivn(Ez2my, nmy); }
    const bool bx = nxt > 0 && nxb > 0, by = nyt > 0 && nyb > 0;
    const double2 Ex1 = bx ? chalf(Ex1t, Ex1b) : (nxt > 0 ? Ex1t : Ex1b);
    const double2 Ey1 = by ? chalf(Ey1t, Ey1b) : (nyt > 0 ? Ey1t : Ey1b);
    const double2 Ex2 = bx ? chalf(Ex2t, Ex2b) : (nxt > 0 ? Ex2t : Ex2b);
    const double2 Ey2 = by ? chalf(Ey2t, Ey2b) : (nyt > 0 ? Ey2t : Ey2b);
    double2 dEx1 = zero2(), dEx2 = zero2(), dEy1 = zero2(), dEy2 = zero2();
    if (bx) { dEx1 = cscale(csub(Ex1t, Ex1b), 1.0 / 1.0); dEx1 = make_double2(dEx1.x / cdz, dEx1.y / cdz);
              dEx2 = csub(Ex2t, Ex2b); dEx2 = make_double2(dEx2.x / cdz, dEx2.y / cdz); }
    if (by) { dEy1 = csub(Ey1t, Ey1b); dEy1 = make_double2(dEy1.x / cdz, dEy1.y / cdz);
              dEy2 = csub(Ey2t, Ey2b); dEy2 = make_double2(dEy2.x / cdz, dEy2.y / cdz); }
    double2 dEz1x = zero2(), dEz2x = zero2(), dEz1y = zero2(), dEz2y = zero2();
    if (npx > 0 && nmx > 0) {
        dEz1x = csub(Ez1px, Ez1mx); dEz1x = make_double2(dEz1x.x / cdx, dEz1x.y / cdx);
        dEz2x = csub(Ez2px, Ez2mx); dEz2x = make_double2(dEz2x.x / cdx, dEz2x.y / cdx);
    }
    if (npy > 0 && nmy > 0) {
        dEz1y = csub(Ez1py, Ez1my); dEz1y = make_double2(dEz1y.x / cdy, dEz1y.y / cdy);
        dEz2y = csub(Ez2py, Ez2my); dEz2y = make_double2(dEz2y.x / cdy, dEz2y.y / cdy);
    }
    const double2 Hx1 = cdiv(csub(dEz1y, dEy1), iwmu);
    const double2 Hy1 = cdiv(csub(dEx1, dEz1x), iwmu);
    const double2 Hx2 = cdiv(csub(dEz2y, dEy2), iwmu);
    const double2 Hy2 = cdiv(csub(dEx2, dEz2x), iwmu);
    const double2 det = csub(cmul(Hx1, Hy2), cmul(Hx2, Hy1));
    H.Hx1 = Hx1; H.Hy1 = Hy1; H.Hx2 = Hx2; H.Hy2 = Hy2; H.det = det;
    H.cdx = cdx; H.cdy = cdy; H.cdz = cdz;
    double2 Zxx, Zxy, Zyx, Zyy;
    if (hypot(det.x, det.y) > 1e-30) {
        Zxx = cdiv(csub(cmul(Ex1, Hy2), cmul(Ex2, Hy1)), det);
        Zxy = cdiv(csub(cmul(Ex2, Hx1), cmul(Ex1, Hx2)), det);
        Zyx = cdiv(csub(cmul(Ey1, Hy2), cmul(Ey2, Hy1)), det);
        Zyy = cdiv(csub(cmul(Ey2, Hx1), cmul(Ey1, Hx2)), det);
    } else {
        const double2 z1 = csqrt_d(cdiv(iwmu, make_double2(st.sigma_cell[s], 0.0)));
        Zxx = zero2(); Zxy = z1; Zyx = cneg(z1); Zyy = zero2();
    }
    H.Zxx = Zxx; H.Zxy = Zxy; H.Zyx = Zyx; H.Zyy = Zyy;
    hc[i] = H;
    zo[0] = Zxx; zo[1] = Zxy; zo[2] = Zyx; zo[3] = Zyy;
}

__global__ void k_wr(int ns, int nf, int nf_total, int f0, const double2* __restrict__ obs,
                     const double* __restrict__ err, const double2* __restrict__ Z, double2* wr) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nf * ns * 4) return;
    const int f = i / (ns * 4), s = (i / 4) % ns, c = i % 4;
    const size_t o = ((size_t)s * nf_total + f0 + f) * 4 + c;
    const double e = err[o];
    double2 v = zero2();
    if (e > 0.0) {
        const double w = 1.0 / e;
        const double2 d = csub(obs[o], Z[((size_t)f * ns + s) * 4 + c]);
        v = make_double2(w * w * d.x, -(w * w * d.y));
    }
    wr[((size_t)f * ns + s) * 4 + c] = v;
}

// forward_solver_fv.cpp:1837-2010, one thread per frequency (stations may share edges)
// Thread f builds source f: wr[f] [ns][4], the station cache hcs[f * hc_stride]
// and omegas[f * om_stride] (strides ns and 1 over frequencies, 0 and 0 for
// many sources at one frequency), into lanes 2f and 2f + 1.
__global__ void k_adjoint_rhs(StationDev st, const double2* __restrict__ wr, const HCache* __restrict__ hcs,
                              const double* __restrict__ omegas, int nf, int hc_stride, int om_stride, VecK out) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    const int K = out.K;
    const double2 iwmu = make_double2(0.0, omegas[(size_t)f * om_stride] * kMu0);
    for (int s = 0; s < st.ns; ++s) {
        if (st.cell[s] < 0) continue;
        const double2* w = wr + ((size_t)f * st.ns + s) * 4;
        const HCache hc = hcs[(size_t)f * hc_stride + s];
        if (hypot(hc.det.x, hc.det.y) < 1e-30) continue;
        const double2 sx1 = cdiv(csub(cmul(w[0], hc.Hy2), cmul(w[1], hc.Hx2)), hc.det);
        const double2 sy1 = cdiv(csub(cmul(w[2], hc.Hy2), cmul(w[3], hc.Hx2)), hc.det);
        const double2 sx2 = cdiv(cadd(cmul(cneg(w[0]), hc.Hy1), cmul(w[1], hc.Hx1)), hc.det);
        const double2 sy2 = cdiv(cadd(cmul(cneg(w[2]), hc.Hy1), cmul(w[3], hc.Hx1)), hc.det);
        const double2 aHx1 = cneg(cadd(cmul(hc.Zxx, sx1), cmul(hc.Zyx, sy1)));
        const double2 aHy1 = cneg(cadd(cmul(hc.Zxy, sx1), cmul(hc.Zyy, sy1)));
        const double2 aHx2 = cneg(cadd(cmul(hc.Zxx, sx2), cmul(hc.Zyx, sy2)));
        const double2 aHy2 = cneg(cadd(cmul(hc.Zxy, sx2), cmul(hc.Zyy, sy2)));
        int nxt = 0, nxb = 0, nyt = 0, nyb = 0, npx = 0, nmx = 0, npy = 0, nmy = 0;
        for (int q = st.e_ptr[s]; q < st.e_ptr[s + 1]; ++q) {
            const unsigned char code = st.e_code[q];
            const int d = code & 3;
            if (d == 0) { if (code & 4) ++nxt; else ++nxb; }
            else if (d == 1) { if (code & 4) ++nyt; else ++nyb; }
            else { if (code & 8) ++npx; else ++nmx; if (code & 16) ++npy; else ++nmy; }
        }
        double wxt = nxt > 0 ? 0.5 / nxt : 0.0, wxb = nxb > 0 ? 0.5 / nxb : 0.0;
        double wyt = nyt > 0 ? 0.5 / nyt : 0.0, wyb = nyb > 0 ? 0.5 / nyb : 0.0;
        if (nxt == 0) wxb = nxb > 0 ? 1.0 / nxb : 0.0;
        if (nxb == 0) wxt = nxt > 0 ? 1.0 / nxt : 0.0;
        if (nyt == 0) wyb = nyb > 0 ? 1.0 / nyb : 0.0;
        if (nyb == 0) wyt = nyt > 0 ? 1.0 / nyt : 0.0;
        const double2 icdz = cdiv(make_double2(1.0, 0.0), make_double2(iwmu.x * hc.cdz, iwmu.y * hc.cdz));
        const double2 icdx = cdiv(make_double2(1.0, 0.0), make_double2(iwmu.x * hc.cdx, iwmu.y * hc.cdx));
        const double2 icdy = cdiv(make_double2(1.0, 0.0), make_double2(iwmu.x * hc.cdy, iwmu.y * hc.cdy));
        for (int q = st.e_ptr[s]; q < st.e_ptr[s + 1]; ++q) {
            const int row = st.e_row[q];
            const unsigned char code = st.e_code[q];
            const int d = code & 3;
            double2* a1 = out.p + (size_t)row * K + 2 * f;
            double2* a2 = a1 + 1;
            if (d == 0) {
                const bool top = code & 4;
                const double we = top ? wxt : wxb;
                *a1 = cadd(*a1, cscale(sx1, we));
                *a2 = cadd(*a2, cscale(sx2, we));
                if (top && nxt > 0) {
                    const double2 wh = make_double2(icdz.x / nxt, icdz.y / nxt);
                    *a1 = cadd(*a1, cmul(aHy1, wh)); *a2 = cadd(*a2, cmul(aHy2, wh));
                } else if (!top && nxb > 0) {
                    const double2 wh = make_double2(-icdz.x / nxb, -icdz.y / nxb);
                    *a1 = cadd(*a1, cmul(aHy1, wh)); *a2 = cadd(*a2, cmul(aHy2, wh));
                }
            } else if (d == 1) {
                const bool top = code & 4;
                const double we = top ? wyt : wyb;
                *a1 = cadd(*a1, cscale(sy1, we));
                *a2 = cadd(*a2, cscale(sy2, we));
                if (top && nyt > 0) {
                    const double2 wh = make_double2(-icdz.x / nyt, -icdz.y / nyt);
                    *a1 = cadd(*a1, cmul(aHx1, wh)); *a2 = cadd(*a2, cmul(aHx2, wh));
                } else if (!top && nyb > 0) {
                    const double2 wh = make_double2(icdz.x / nyb, icdz.y / nyb);
                    *a1 = cadd(*a1, cmul(aHx1, wh)); *a2 = cadd(*a2, cmul(aHx2, wh));
                }
            } else {
                const bool py = code & 16;
                if (py && npy > 0) {
                    const double2 wh = make_double2(icdy.x / npy, icdy.y / npy);
                    *a1 = cadd(*a1, cmul(aHx1, wh)); *a2 = cadd(*a2, cmul(aHx2, wh));
                } else if (!py && nmy > 0) {
                    const double2 wh = make_double2(-icdy.x / nmy, -icdy.y / nmy);
                    *a1 = cadd(*a1, cmul(aHx1, wh)); *a2 = cadd(*a2, cmul(aHx2, wh));
                }
                const bool px = code & 8;
                if (px && npx > 0) {
                    const double2 wh = make_double2(-icdx.x / npx, -icdx.y / npx);
                    *a1 = cadd(*a1, cmul(aHy1, wh)); *a2 = cadd(*a2, cmul(aHy2, wh));
                } else if (!px && nmx > 0) {
                    const double2 wh = make_double2(icdx.x / nmx, icdx.y / nmx);
                    *a1 = cadd(*a1, cmul(aHy1, wh)); *a2 = cadd(*a2, cmul(aHy2, wh));
                }
            }
        }
    }
}

// sum over cell c's edges of Im(lambda_e E_e) * w_e (w_e = A_dual L / n_adj,
// 0 for skipped edges) for one lane pair; the edges go four at a time with
// all their loads issued before the first product, so a thread has twelve
// independent loads in flight instead of a chain per edge.  Edge order of
// the sums is the cell's edge order.
__device__ __forceinline__ double cell_im_sum(const MeshDev& m, int c, const VecK& lam, int kl, const VecK& E,
                                              int kE) {
    const int q0 = m.cell_ptr[c], q1 = m.cell_ptr[c + 1];
    double sy = 0.0;
    for (int q = q0; q < q1; q += 4) {
        int e[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) e[u] = q + u < q1 ? m.cell_edge[q + u] : -1;
        double w[4];
        double2 l[4], f[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            if (e[u] >= 0) {
                w[u] = m.sens_w[e[u]];
                l[u] = lam.p[(size_t)e[u] * lam.K + kl];
                f[u] = E.p[(size_t)e[u] * E.K + kE];
            } else {
                w[u] = 0.0;
                l[u] = f[u] = zero2();
            }
        }
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (w[u] != 0.0) sy += cmul(l[u], f[u]).y * w[u];
    }
    return sy;
}

// G consecutive threads per cell (G a power of two >= nf * npol, so a group
// never straddles a warp), thread k of the group on lane k = npol * f + p:
// each edge row of E and lambda (K lanes, interleaved) is read as one
// contiguous segment, and the per-edge data are broadcast within the
// group.  The group's lane terms -omega_f sigma_c Im(sum_e lambda_e E_e w_e)
// are summed by a fixed shuffle tree, so the result is deterministic.
// compute_sensitivity, forward_solver_fv.cpp:989-1059.
template <int G>
__global__ void k_sensitivity(MeshDev m, const double* __restrict__ sigma, VecK E, VecK lam,
                              const double* __restrict__ omegas, int nf, int npol, double* g) {
    const long total = ((long)m.nc * G + 31) / 32 * 32;
    const long stride = (long)gridDim.x * blockDim.x;
    const int nl = nf * npol;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += stride) {
        const int c = (int)(t / G);
        const int k = (int)(t % G);
        const bool live = c < m.nc;
        double v = 0.0;
        if (live && k < nl) v = -omegas[k / npol] * (sigma[c] * cell_im_sum(m, c, lam, k, E, k));   // Re(i omega s)
        for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o, G);
        if (live && k == 0) g[c] += v;
    }
}

// Per-source sensitivities: lambda lanes 2j + p (source j, polarisation p)
// against the forward field's lanes e0 + p at one frequency; g[j][c] is the
// sum over the two polarisations of Re(i omega sum_e lambda_e E_e dMe)
// (compute_sensitivity, forward_solver_fv.cpp:989-1059, per polarisation,
// summed as inversion_fv.cpp:280-290 sums them).  Same thread layout as
// k_sensitivity; a source's two lanes are neighbours in the group.
template <int G>
__global__ void k_sensitivity_src(MeshDev m, const double* __restrict__ sigma, VecK E, int e0, VecK lam,
                                  const double* __restrict__ omega, int n_src, double* __restrict__ g) {
    const long total = ((long)m.nc * G + 31) / 32 * 32;
    const long stride = (long)gridDim.x * blockDim.x;
    const int nl = 2 * n_src;
    const double om = omega[0];
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += stride) {
        const int c = (int)(t / G);
        const int k = (int)(t % G);
        const bool live = c < m.nc && k < nl;
        double v = 0.0;
        if (live) v = -om * (sigma[c] * cell_im_sum(m, c, lam, k, E, e0 + (k & 1)));
        const double w = __shfl_xor_sync(0xffffffffu, v, 1, G);
        if (live && (k & 1) == 0) g[(size_t)(k >> 1) * m.nc + c] = v + w;
    }
}

__global__ void k_pert_rhs(MeshDev m, const double* __restrict__ sigma, const double* __restrict__ dsig,
                           VecK E, int kE, double omega, VecK out, int kout) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= m.n_pad) return;
    double2 acc = zero2();
    if (!(m.flags[row] & kFlagPad)) {
        const int a0 = m.adj_ptr[row], a1 = m.adj_ptr[row + 1];
        const double L = m.elen[row];
        const double vol = L * L * L;
        double si = 0.0;
        int na = 0;
        for (int k = a0; k < a1; ++k) {
            const double sg = sigma[m.adj_cell[k]];
            if (sg > 1e-30) { si += 1.0 / sg; ++na; }
        }
        const double sa = (na > 0 && si > 1e-30) ? na / si : 1e-8;
        const double2 ev = E.p[(size_t)row * E.K + kE];
        for (int k = a0; k < a1; ++k) {
            const int c = m.adj_cell[k];
            const double ds = dsig[c];
            if (fabs(ds) < 1e-30) continue;
            const double sc = sigma[c];
            const double dMe = vol * sa * sa / (na * sc * sc);
            const double2 t = cmul(make_double2(0.0, omega * (ds * dMe)), ev);
            acc = csub(acc, t);
        }
    }
    out.p[(size_t)row * out.K + kout] = acc;
}

__global__ void k_delta_z(StationDev st, VecK dE, int kE, const HCache* __restrict__ hcs, int pol, double2* dZ) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= st.ns) return;
    double2* o = dZ + (size_t)s * 4;
    o[0] = o[1] = o[2] = o[3] = zero2();
    if (st.cell[s] < 0) return;
    double2 dEx = zero2(), dEy = zero2();
    int nx = 0, ny = 0;
    for (int q = st.e_ptr[s]; q < st.e_ptr[s + 1]; ++q) {
        const int d = st.e_code[q] & 3;
        const double2 v = dE.p[(size_t)st.e_row[q] * dE.K + kE];
        if (d == 0) { dEx = cadd(dEx, v); ++nx; }
        else if (d == 1) { dEy = cadd(dEy, v); ++ny; }
    }
    if (nx > 0) dEx = cdivn(dEx, nx);
    if (ny > 0) dEy = cdivn(dEy, ny);
    const HCache hc = hcs[s];
    if (hypot(hc.det.x, hc.det.y) < 1e-30) return;
    const double2 id = cdiv(make_double2(1.0, 0.0), hc.det);
    if (pol == 1) {
        o[0] = cmul(cmul(dEx, hc.Hy2), id); o[1] = cmul(cmul(dEx, cneg(hc.Hx2)), id);
        o[2] = cmul(cmul(dEy, hc.Hy2), id); o[3] = cmul(cmul(dEy, cneg(hc.Hx2)), id);
    } else {
        o[0] = cmul(cmul(dEx, cneg(hc.Hy1)), id); o[1] = cmul(cmul(dEx, hc.Hx1), id);
        o[2] = cmul(cmul(dEy, cneg(hc.Hy1)), id); o[3] = cmul(cmul(dEy, hc.Hx1), id);
    }
}

}  // namespace

void edge_mass(const MeshDev& m, const double* sigma, double* Me, double* me_dc, cudaStream_t s) {
    k_edge_mass<<<grid1(m.n_pad), kBlock, 0, s>>>(m, sigma, Me, me_dc);
    ck();
}

void diag_coeffs(const MeshDev& m, const double* Me, double2* sm, float2* sm32, cudaStream_t s) {
    k_diag_coeffs<<<grid1(m.n_pad), kBlock, 0, s>>>(m, Me, sm, sm32);
    ck();
}

void primary_field(const MeshDev& m, VecK out, const RhsInfo& info, bool bc_only, cudaStream_t s) {
    const long n = (long)m.n_pad * out.K;
    k_primary<<<(int)((n + kBlock - 1) / kBlock), kBlock, 0, s>>>(m, out, info, bc_only ? 1 : 0);
    ck();
}

void lift_rhs(const MeshDev& m, VecK ebc, VecK rhs, cudaStream_t s) {
    const long n = (long)m.n_pad * rhs.K;
    k_lift<<<(int)((n + kBlock - 1) / kBlock), kBlock, 0, s>>>(m, ebc, rhs);
    ck();
}

void vsub(long n, const double2* a, const double2* b, double2* out, cudaStream_t s) {
    k_vsub<<<(int)((n + kBlock - 1) / kBlock), kBlock, 0, s>>>(n, a, b, out);
    ck();
}

void interpolate_hanging(const MeshDev& m, VecK x, bool sequential, cudaStream_t s) {
    if (m.nhp == 0) return;
    if (sequential) {
        k_hanging_seq<<<1, 32, 0, s>>>(m, x);
    } else {
        const long n = (long)m.nhp * x.K;
        k_hanging<<<(int)((n + kBlock - 1) / kBlock), kBlock, 0, s>>>(m, x);
    }
    ck();
}

void combine_total(const MeshDev& m, VecK epri, VecK esec, VecK ebc, VecK e, cudaStream_t s) {
    const long n = (long)m.n_pad * e.K;
    k_combine<<<(int)((n + kBlock - 1) / kBlock), kBlock, 0, s>>>(m, epri, esec, ebc, e);
    ck();
}

void to_permuted(const MeshDev& m, const double2* ref, int K, int k, VecK dst, cudaStream_t s) {
    (void)K;
    k_to_perm<<<grid1(m.ne), kBlock, 0, s>>>(m, ref, dst, k);
    ck();
}

void from_permuted(const MeshDev& m, VecK src, int k, double2* ref, cudaStream_t s) {
    k_from_perm<<<grid1(m.ne), kBlock, 0, s>>>(m, src, k, ref);
    ck();
}

void fill_zero(VecK v, long n_pad, cudaStream_t s) {
    cudaMemsetAsync(v.p, 0, sizeof(double2) * (size_t)n_pad * v.K, s);
    ck();
}

void dc_build_laplacian(const MeshDev& m, const double* me_dc, DcWork w, cudaStream_t s) {
    k_dc_lap<<<grid1(m.nn), kBlock, 0, s>>>(m, me_dc, w);
    ck();
}

void dc_phi0(const MeshDev& m, VecK rhs, const RhsInfo& info, DcWork w, cudaStream_t s) {
    const long n = (long)m.nn * rhs.K;
    k_dc_phi0<<<(int)((n + kBlock - 1) / kBlock), kBlock, 0, s>>>(m, rhs, info, w);
    ck();
}

template <int K>
long long divcorr_k(const MeshDev& m, const double* me_dc, VecK E, bool use_phi0, DcWork w, int max_outer,
                    double tol, const int* active_host, RedScratch red, cudaStream_t s, int cg_chunk,
                    DcCounters* counters, const AmgDev* amg, const GcDev* mixed) {
    if (counters) counters->calls += 1;
    long long launches = 0;
    std::vector<DcState> hs(K);
    for (int k = 0; k < K; ++k) {
        DcState S{};
        S.active = active_host[k] ? 1 : 0;
        S.done = S.active ? 0 : 1;
        hs[k] = S;
    }
    cudaMemcpyAsync(w.st, hs.data(), sizeof(DcState) * K, cudaMemcpyHostToDevice, s);
    const int cap = red.max_blocks;
    const int g_divj = wave_grid(k_dc_divj<K>, cap), g_init = wave_grid(k_dc_cg_init<K>, cap);
    const int g_up = wave_grid(k_dc_cg_update<K>, cap);
    const int g_p = wave_grid(k_dc_cg_p<K>, 1 << 20);
    const int cg_max = m.nn > 500 ? m.nn : 500;
    const int ge = (int)(((long)m.n_pad * K + kBlock - 1) / kBlock);
    for (int outer = 0; outer < max_outer; ++outer) {
        k_dc_divj<K><<<g_divj, kBlock, 0, s>>>(m, me_dc, E, use_phi0 ? 1 : 0, w, tol, red);
        ck(); ++launches;
        cudaMemcpyAsync(hs.data(), w.st, sizeof(DcState) * K, cudaMemcpyDeviceToHost, s);
        cudaStreamSynchronize(s);
        bool any = false;
        for (int k = 0; k < K; ++k) any |= (hs[k].active && !hs[k].done);
        if (!any) break;
        if (mixed) {
            long long sweeps = 0;
            launches += dc_poisson_mixed_k<K>(*mixed, m.nn, w, red, s, &sweeps);
            cudaMemcpyAsync(hs.data(), w.st, sizeof(DcState) * K, cudaMemcpyDeviceToHost, s);
            cudaStreamSynchronize(s);
            if (counters) {
                counters->outer += 1;
                counters->cg_sweeps += sweeps;
                for (int k = 0; k < K; ++k) if (hs[k].active && !hs[k].done) counters->cg_iterations += hs[k].cg_iter;
            }
            k_dc_grad<<<ge, kBlock, 0, s>>>(m, E, w);
            k_dc_outer_done<<<1, 32, 0, s>>>(K, w);
            ck(); launches += 2;
            continue;
        }
        if (amg) {
            // z = M^-1 divJ, rz, p = z
            k_mg_cg_init<K><<<g_p, kBlock, 0, s>>>(m.nn, w);
            launches += 1 + mg_apply<K>(m, w, *amg, red, cap, s);
            k_dc_cg_p<K><<<g_p, kBlock, 0, s>>>(m.nn, w);
            ++launches;
        } else {
            k_dc_cg_init<K><<<g_init, kBlock, 0, s>>>(m.nn, w, red);
            ++launches;
        }
        ck();
        int chunk = amg ? std::max(1, cg_chunk / 4) : cg_chunk;
        int it = 0;
        for (; it < cg_max;) {
            const int n_it = (cg_max - it) < chunk ? (cg_max - it) : chunk;
            for (int j = 0; j < n_it; ++j) {
                launch_staged(k_dc_cg_ap_st<K>, StagedShape<K>::NT, w.lap_stage, w.n_node_slices, cap, s, m.nn,
                              w, red);
                if (amg) {
                    k_mg_cg_update<K><<<g_up, kBlock, 0, s>>>(m.nn, cg_max, w, red);
                    launches += 2 + mg_apply<K>(m, w, *amg, red, cap, s);
                } else {
                    k_dc_cg_update<K><<<g_up, kBlock, 0, s>>>(m.nn, cg_max, w, red);
                    launches += 2;
                }
                k_dc_cg_p<K><<<g_p, kBlock, 0, s>>>(m.nn, w);
                ++launches;
            }
            ck();
            it += n_it;
            cudaMemcpyAsync(hs.data(), w.st, sizeof(DcState) * K, cudaMemcpyDeviceToHost, s);
            cudaStreamSynchronize(s);
            bool run = false;
            for (int k = 0; k < K; ++k) run |= hs[k].cg_run != 0;
            if (!run) break;
            chunk = chunk < 200 ? 2 * chunk : chunk;   // polls grow sparser as PCG runs on
        }
        if (counters) {
            counters->outer += 1;
            counters->cg_sweeps += it;
            for (int k = 0; k < K; ++k) if (hs[k].active && !hs[k].done) counters->cg_iterations += hs[k].cg_iter;
        }
        k_dc_grad<<<ge, kBlock, 0, s>>>(m, E, w);
        k_dc_outer_done<<<1, 32, 0, s>>>(K, w);
        ck(); launches += 2;
    }
    return launches;
}

long long divcorr(const MeshDev& m, const double* me_dc, VecK E, bool use_phi0, DcWork w, int max_outer,
                  double tol, const int* active_host, RedScratch red, cudaStream_t s, int cg_chunk,
                  DcCounters* counters, const AmgDev* amg, const GcDev* mixed) {
    switch (E.K) {
        case 2: return divcorr_k<2>(m, me_dc, E, use_phi0, w, max_outer, tol, active_host, red, s, cg_chunk, counters, amg, mixed);
        case 4: return divcorr_k<4>(m, me_dc, E, use_phi0, w, max_outer, tol, active_host, red, s, cg_chunk, counters, amg, mixed);
        case 8: return divcorr_k<8>(m, me_dc, E, use_phi0, w, max_outer, tol, active_host, red, s, cg_chunk, counters, amg, mixed);
        case 16: return divcorr_k<16>(m, me_dc, E, use_phi0, w, max_outer, tol, active_host, red, s, cg_chunk, counters, amg, mixed);
        default: throw std::runtime_error("divergence correction batch must be 2, 4, 8 or 16");
    }
}

void station_impedance(const StationDev& st, VecK E, const double* omegas, int nf, HCache* hc, double2* Z,
                       cudaStream_t s) {
    const int n = nf * st.ns;
    if (n == 0) return;
    k_station_z<<<(n + 127) / 128, 128, 0, s>>>(st, E, omegas, nf, hc, Z);
    ck();
}

void weighted_residual(int ns, int nf, int nf_total, int f0, const double2* obs, const double* err,
                       const double2* Z, double2* wr, cudaStream_t s) {
    const int n = nf * ns * 4;
    if (n == 0) return;
    k_wr<<<(n + kBlock - 1) / kBlock, kBlock, 0, s>>>(ns, nf, nf_total, f0, obs, err, Z, wr);
    ck();
}

// JtJ.v weighting (ImplicitJtJOperatorFV::Mult, implicit_jtj_fv.cpp:137-150):
// lane k = 2f + p of dZ ([K][ns][4]) times w^2, w = 1 / err (0 where err <= 0),
// into wr_p[f] ([nf][ns][4], not conjugated, as the reference passes it).
__global__ void k_jtj_weight(int ns, int nf, const double* __restrict__ err, const double2* __restrict__ dz,
                             double2* __restrict__ wr0, double2* __restrict__ wr1) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 2 * nf * ns * 4) return;
    const int k = i / (ns * 4), s = (i / 4) % ns, c = i % 4;
    const int f = k / 2, p = k % 2;
    const double e = err[((size_t)s * nf + f) * 4 + c];
    double2 v = zero2();
    if (e > 0.0) {
        const double w2 = 1.0 / (e * e);
        const double2 d = dz[((size_t)k * ns + s) * 4 + c];
        v = make_double2(w2 * d.x, w2 * d.y);
    }
    (p == 0 ? wr0 : wr1)[((size_t)f * ns + s) * 4 + c] = v;
}

// out lane 2f from a (pol 1 source of wr_0), lane 2f + 1 from b (pol 2 source of wr_1)
__global__ void k_pick_pol_lanes(long n, int K, const double2* __restrict__ a, const double2* __restrict__ b,
                                 double2* __restrict__ out) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = ((i % K) % 2 == 0) ? a[i] : b[i];
}

void jtj_weight(int ns, int nf, const double* err, const double2* dz, double2* wr0, double2* wr1, cudaStream_t s) {
    const int n = 2 * nf * ns * 4;
    if (n == 0) return;
    k_jtj_weight<<<(n + kBlock - 1) / kBlock, kBlock, 0, s>>>(ns, nf, err, dz, wr0, wr1);
    ck();
}

void pick_pol_lanes(long n_pad, int K, const double2* a, const double2* b, double2* out, cudaStream_t s) {
    const long n = n_pad * K;
    k_pick_pol_lanes<<<(int)((n + kBlock - 1) / kBlock), kBlock, 0, s>>>(n, K, a, b, out);
    ck();
}

void adjoint_rhs(const StationDev& st, const MeshDev& m, const double2* wr, const HCache* hc,
                 const double* omegas, int nf, VecK out, cudaStream_t s) {
    (void)m;
    k_adjoint_rhs<<<1, 32, 0, s>>>(st, wr, hc, omegas, nf, st.ns, 1, out);
    ck();
}

void adjoint_rhs_sources(const StationDev& st, const double2* wr, const HCache* hc, const double* omega, int n_src,
                         VecK out, cudaStream_t s) {
    if (n_src < 1 || 2 * n_src > out.K) throw std::invalid_argument("adjoint sources: 1 .. K/2");
    k_adjoint_rhs<<<1, 32, 0, s>>>(st, wr, hc, omega, n_src, 0, 0, out);
    ck();
}

void sensitivity(const MeshDev& m, const double* sigma, VecK E, VecK lam, const double* omegas, int nf,
                 int npol, double* g, cudaStream_t s) {
    const int nl = nf * npol;
    if (nl < 1 || nl > dev::kMaxRhs) throw std::invalid_argument("sensitivity: 1..16 lanes");
    const long n = (long)m.nc * 16;
    if (nl == 1) k_sensitivity<1><<<grid1(n / 16), kBlock, 0, s>>>(m, sigma, E, lam, omegas, nf, npol, g);
    else if (nl == 2) k_sensitivity<2><<<grid1(n / 8), kBlock, 0, s>>>(m, sigma, E, lam, omegas, nf, npol, g);
    else if (nl <= 4) k_sensitivity<4><<<grid1(n / 4), kBlock, 0, s>>>(m, sigma, E, lam, omegas, nf, npol, g);
    else if (nl <= 8) k_sensitivity<8><<<grid1(n / 2), kBlock, 0, s>>>(m, sigma, E, lam, omegas, nf, npol, g);
    else k_sensitivity<16><<<grid1(n), kBlock, 0, s>>>(m, sigma, E, lam, omegas, nf, npol, g);
    ck();
}

void sensitivity_sources(const MeshDev& m, const double* sigma, VecK E, int e0, VecK lam, const double* omega,
                         int n_src, double* g, cudaStream_t s) {
    if (n_src < 1 || 2 * n_src > dev::kMaxRhs) throw std::invalid_argument("sensitivity: 1 .. 8 sources");
    const long n = (long)m.nc * 16;
    if (n_src == 1) k_sensitivity_src<2><<<grid1(n / 8), kBlock, 0, s>>>(m, sigma, E, e0, lam, omega, n_src, g);
    else if (n_src == 2) k_sensitivity_src<4><<<grid1(n / 4), kBlock, 0, s>>>(m, sigma, E, e0, lam, omega, n_src, g);
    else if (n_src <= 4) k_sensitivity_src<8><<<grid1(n / 2), kBlock, 0, s>>>(m, sigma, E, e0, lam, omega, n_src, g);
    else k_sensitivity_src<16><<<grid1(n), kBlock, 0, s>>>(m, sigma, E, e0, lam, omega, n_src, g);
    ck();
}

void perturbation_rhs(const MeshDev& m, const double* sigma, const double* dsigma, VecK E, int kE, double omega,
                      VecK out, int kout, cudaStream_t s) {
    k_pert_rhs<<<grid1(m.n_pad), kBlock, 0, s>>>(m, sigma, dsigma, E, kE, omega, out, kout);
    ck();
}

void delta_impedance(const StationDev& st, VecK dE, int kE, const HCache* hc, int pol, double2* dZ,
                     cudaStream_t s) {
    if (st.ns == 0) return;
    k_delta_z<<<(st.ns + 127) / 128, 128, 0, s>>>(st, dE, kE, hc, pol, dZ);
    ck();
}

}  // namespace phys
}  // namespace m3d
