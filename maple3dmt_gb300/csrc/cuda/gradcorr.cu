// Gradient-space correction kernels (see gradcorr.cuh).
#include "gradcorr.cuh"

#include <algorithm>
#include <stdexcept>
#include <vector>

namespace m3d {

using namespace dev;

namespace {

constexpr int kGcBlock = 256;

int gc_grid(long work) {
    long b = (work + kGcBlock - 1) / kGcBlock;
    return (int)std::max(1L, std::min(b, (long)1 << 20));
}

void gc_check(long long* launches) {
    if (launches) ++*launches;
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) throw std::runtime_error(cudaGetErrorString(e));
}

__device__ __forceinline__ float2 f2(float x, float y) { return make_float2(x, y); }

// inc_g[q] = G[e, v] unless v is a Dirichlet node or e is an identity /
// padding row; e_g likewise per edge end.
__global__ void k_gc_weights(MeshDev m, float* __restrict__ inc_g, float* __restrict__ e_g) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned char masked = kFlagConstrained | kFlagPad;
    if (i < m.nn) {
        const int v = (int)i;
        for (int q = m.inc_ptr[v]; q < m.inc_ptr[v + 1]; ++q) {
            const int e = m.inc_edge[q];
            const bool off = m.node_bc[v] || (m.flags[e] & masked);
            inc_g[q] = off ? 0.0f : (float)m.inc_gv[q];
        }
    }
    if (i < m.n_pad) {
        const int r = (int)i;
        for (int j = 0; j < 2; ++j) {
            const int v = m.e_node[2 * r + j];
            const bool off = (m.flags[r] & masked) || m.node_bc[v];
            e_g[2 * r + j] = off ? 0.0f : (float)m.e_g[2 * r + j];
        }
    }
}

__global__ void k_gc_pack0(GcDev g) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= g.nn) return;
    g.lap_diag32[v] = (float)g.lap_diag[v];
    g.lv[0].dinv32[v] = (float)g.lv[0].dinv[v];
    for (int q = g.inc_ptr[v]; q < g.inc_ptr[v + 1]; ++q)
        g.lap_pk[q] = make_int2(g.inc_other[q], __float_as_int((float)g.lap_off[q]));
}

// x~_j of the up-sweep: level iterate plus the prolonged coarse correction
struct XPlain {
    const float2* x;
    __device__ __forceinline__ float2 operator()(int j, int k, int K) const { return x[(size_t)j * K + k]; }
};
struct XProlonged {
    const float2* x;     // null: the level was not pre-smoothed (x = 0)
    const int* agg;
    const float2* xc;
    __device__ __forceinline__ float2 operator()(int j, int k, int K) const {
        float2 v = x ? x[(size_t)j * K + k] : f2(0.0f, 0.0f);
        const int a = __ldg(&agg[j]);
        if (a >= 0) {
            const float2 c = xc[(size_t)a * K + k];
            v.x += c.x;
            v.y += c.y;
        }
        return v;
    }
};

// (A_l x~)_row; level 0 through the incidence form of the node Laplacian
template <int K, bool L0, class XF>
__device__ __forceinline__ float2 level_row(const GcDev& g, const GcLevel& L, int row, const XF& xf, int k) {
    float2 s = f2(0.0f, 0.0f);
    if (L0) {
        const float dg = __ldg(&g.lap_diag32[row]);
        const float2 xr = xf(row, k, K);
        s.x = dg * xr.x;
        s.y = dg * xr.y;
        const int q0 = __ldg(&g.inc_ptr[row]), q1 = __ldg(&g.inc_ptr[row + 1]);
        for (int q = q0; q < q1; q += 4) {
            float a[4];
            float2 xv[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int2 e = q + u < q1 ? __ldg(&g.lap_pk[q + u]) : make_int2(0, 0);
                a[u] = __int_as_float(e.y);
                xv[u] = a[u] != 0.0f ? xf(e.x, k, K) : f2(0.0f, 0.0f);
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                s.x += a[u] * xv[u].x;
                s.y += a[u] * xv[u].y;
            }
        }
    } else {
        const int q0 = __ldg(&L.ptr[row]), q1 = __ldg(&L.ptr[row + 1]);
        for (int q = q0; q < q1; q += 4) {
            float a[4];
            float2 xv[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const bool ok = q + u < q1;
                a[u] = ok ? (float)__ldg(&L.val[q + u]) : 0.0f;
                xv[u] = ok ? xf(__ldg(&L.col[q + u]), k, K) : f2(0.0f, 0.0f);
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                s.x += a[u] * xv[u].x;
                s.y += a[u] * xv[u].y;
            }
        }
    }
    return s;
}

// b0 = G~^T in; x0 = omega D^-1 b0 (pre-smoothing from zero) when level 0
// is not the coarsest
template <int K>
__global__ void __launch_bounds__(kGcBlock) k_gc_restrict_edges(GcDev g, const float2* __restrict__ in, int presmooth) {
    const GcLevel& L = g.lv[0];
    const long n = (long)g.nn * K;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int v = (int)(i / K), k = (int)(i % K);
        float2 acc = f2(0.0f, 0.0f);
        const int q0 = __ldg(&g.inc_ptr[v]), q1 = __ldg(&g.inc_ptr[v + 1]);
        for (int q = q0; q < q1; q += 4) {
            float w[4];
            float2 e[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                w[u] = q + u < q1 ? __ldg(&g.inc_g[q + u]) : 0.0f;
                e[u] = w[u] != 0.0f ? in[(size_t)__ldg(&g.inc_edge[q + u]) * K + k] : f2(0.0f, 0.0f);
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                acc.x += w[u] * e[u].x;
                acc.y += w[u] * e[u].y;
            }
        }
        L.b[i] = acc;
        if (presmooth) {
            const float sc = g.omega * (float)__ldg(&L.dinv[v]);
            L.x[i] = f2(sc * acc.x, sc * acc.y);
        }
    }
}

// r_l = b - A_l x, written to y (free until the up-sweep)
template <int K, bool L0>
__global__ void __launch_bounds__(kGcBlock) k_gc_resid(GcDev g, GcLevel L) {
    const long n = (long)L.n * K;
    const XPlain xf{L.x};
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int row = (int)(i / K), k = (int)(i % K);
        const float2 ax = level_row<K, L0>(g, L, row, xf, k);
        const float2 bv = L.b[i];
        L.y[i] = f2(bv.x - ax.x, bv.y - ax.y);
    }
}

// b_{l+1}[I] = sum of the level-l residual src over the members of aggregate
// I (src = b_l when level l is not pre-smoothed), and the pre-smoothed
// x_{l+1} = omega D^-1 b_{l+1} when level l+1 is
template <int K>
__global__ void __launch_bounds__(kGcBlock) k_gc_restrict(GcDev g, GcLevel L, GcLevel N, const float2* __restrict__ src,
                                                          int presmooth) {
    const long n = (long)N.n * K;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int I = (int)(i / K), k = (int)(i % K);
        float2 acc = f2(0.0f, 0.0f);
        const int m0 = __ldg(&L.rptr[I]), m1 = __ldg(&L.rptr[I + 1]);
        for (int m = m0; m < m1; m += 4) {
            float2 r[4];
#pragma unroll
            for (int u = 0; u < 4; ++u)
                r[u] = m + u < m1 ? src[(size_t)__ldg(&L.rcol[m + u]) * K + k] : f2(0.0f, 0.0f);
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                acc.x += r[u].x;
                acc.y += r[u].y;
            }
        }
        N.b[i] = acc;
        if (presmooth) {
            const float sc = g.omega * (float)__ldg(&N.dinv[I]);
            N.x[i] = f2(sc * acc.x, sc * acc.y);
        }
    }
}

// coarsest level: x = A_c^-1 b (dense); one block per row, thread t on
// lane t % K and columns j = t / K (mod kGcBlock / K), summed in shared memory
template <int K>
__global__ void __launch_bounds__(kGcBlock) k_gc_coarse(int nc, const double* __restrict__ inv,
                                                        const float2* __restrict__ b, float2* __restrict__ x) {
    constexpr int G = kGcBlock / K;
    __shared__ float2 part[kGcBlock];
    const int k = threadIdx.x % K, grp = threadIdx.x / K;
    for (int row = blockIdx.x; row < nc; row += gridDim.x) {
        float2 s = f2(0.0f, 0.0f);
        for (int j = grp; j < nc; j += G) {
            const float a = (float)__ldg(&inv[(size_t)row * nc + j]);
            const float2 v = b[(size_t)j * K + k];
            s.x += a * v.x;
            s.y += a * v.y;
        }
        part[threadIdx.x] = s;
        __syncthreads();
        if (grp == 0) {
            float2 t = f2(0.0f, 0.0f);
            for (int q = 0; q < G; ++q) {
                const float2 p = part[q * K + k];
                t.x += p.x;
                t.y += p.y;
            }
            x[(size_t)row * K + k] = t;
        }
        __syncthreads();
    }
}

// y_l = x~ + omega D^-1 (b - A_l x~), x~ = x_l + P xc (prolongation fused)
template <int K, bool L0>
__global__ void __launch_bounds__(kGcBlock) k_gc_up(GcDev g, GcLevel L, const float2* __restrict__ xc,
                                                    float2* __restrict__ out, int presmoothed) {
    const long n = (long)L.n * K;
    const XProlonged xf{presmoothed ? L.x : nullptr, L.agg, xc};
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int row = (int)(i / K), k = (int)(i % K);
        const float2 ax = level_row<K, L0>(g, L, row, xf, k);
        const float2 xt = xf(row, k, K);
        const float2 bv = L.b[i];
        const float sc = g.omega * (float)__ldg(&L.dinv[row]);
        out[i] = f2(xt.x + sc * (bv.x - ax.x), xt.y + sc * (bv.y - ax.y));
    }
}

// t = x + P xc (x optional): the level-0 iterate after the coarse
// correction, written out so the smoothing step gathers it directly
template <int K>
__global__ void __launch_bounds__(kGcBlock) k_gc_prolong0(GcDev g, const float2* __restrict__ xc,
                                                          float2* __restrict__ t, int presmoothed) {
    const GcLevel& L = g.lv[0];
    const XProlonged xf{presmoothed ? L.x : nullptr, L.agg, xc};
    const long n = (long)g.nn * K;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        t[i] = xf((int)(i / K), (int)(i % K), K);
}

// y0 = t + omega D^-1 (b0 - L t)
template <int K>
__global__ void __launch_bounds__(kGcBlock) k_gc_smooth0(GcDev g, const float2* __restrict__ t,
                                                         float2* __restrict__ out) {
    const GcLevel& L = g.lv[0];
    const XPlain xf{t};
    const long n = (long)g.nn * K;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int row = (int)(i / K), k = (int)(i % K);
        const float2 ax = level_row<K, true>(g, L, row, xf, k);
        const float2 xt = t[i];
        const float2 bv = L.b[i];
        const float sc = g.omega * __ldg(&L.dinv32[row]);
        out[i] = f2(xt.x + sc * (bv.x - ax.x), xt.y + sc * (bv.y - ax.y));
    }
}

// x0 = omega D^-1 b0 (pre-smoothing from zero, node-vector input)
template <int K>
__global__ void __launch_bounds__(kGcBlock) k_gc_pre0(GcDev g) {
    const GcLevel& L = g.lv[0];
    const long n = (long)g.nn * K;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const float sc = g.omega * (float)__ldg(&L.dinv[i / K]);
        const float2 b = L.b[i];
        L.x[i] = f2(sc * b.x, sc * b.y);
    }
}

// V-cycle from level 0 with g.lv[0].b set (and g.lv[0].x when pre): result in out
template <int K>
void vcycle_k(const GcDev& g, int pre, float2* out, cudaStream_t s, long long* launches) {
    const int nl = g.n_levels;
    if (nl == 1) {
        k_gc_coarse<K><<<std::max(1, g.n_coarse), kGcBlock, 0, s>>>(g.n_coarse, g.coarse_inv, g.lv[0].b, out);
        gc_check(launches);
        return;
    }
    for (int l = 0; l + 1 < nl; ++l) {
        const int pre_next = (pre && l + 1 < nl - 1) ? 1 : 0;
        const long rw = (long)g.lv[l].n * K;
        const float2* src = g.lv[l].b;
        if (pre) {   // residual of the pre-smoothed iterate, in y
            if (l == 0) k_gc_resid<K, true><<<gc_grid(rw), kGcBlock, 0, s>>>(g, g.lv[l]);
            else k_gc_resid<K, false><<<gc_grid(rw), kGcBlock, 0, s>>>(g, g.lv[l]);
            gc_check(launches);
            src = g.lv[l].y;
        }
        k_gc_restrict<K><<<gc_grid((long)g.lv[l + 1].n * K), kGcBlock, 0, s>>>(g, g.lv[l], g.lv[l + 1], src,
                                                                                pre_next);
        gc_check(launches);
    }
    const GcLevel& C = g.lv[nl - 1];
    k_gc_coarse<K><<<std::max(1, g.n_coarse), kGcBlock, 0, s>>>(g.n_coarse, g.coarse_inv, C.b, C.x);
    gc_check(launches);
    for (int l = nl - 2; l >= 0; --l) {
        const float2* xc = (l + 1 == nl - 1) ? g.lv[l + 1].x : g.lv[l + 1].y;
        float2* dst = l == 0 ? out : g.lv[l].y;
        const long work = (long)g.lv[l].n * K;
        if (l == 0) {
            // level 0 in two passes: prolongation into y (the level's scratch),
            // then the smoothing step gathers it directly
            k_gc_prolong0<K><<<gc_grid(work), kGcBlock, 0, s>>>(g, xc, g.lv[0].y, pre);
            gc_check(launches);
            k_gc_smooth0<K><<<gc_grid(work), kGcBlock, 0, s>>>(g, g.lv[0].y, dst);
        } else {
            k_gc_up<K, false><<<gc_grid(work), kGcBlock, 0, s>>>(g, g.lv[l], xc, dst, pre);
        }
        gc_check(launches);
    }
}

}  // namespace

void gc_weights(const MeshDev& m, float* inc_g, float* e_g, cudaStream_t s) {
    const long n = std::max<long>(m.nn, m.n_pad);
    k_gc_weights<<<gc_grid(n), kGcBlock, 0, s>>>(m, inc_g, e_g);
    gc_check(nullptr);
}

void gc_pack_level0(const GcDev& g, cudaStream_t s) {
    if (g.n_levels < 1 || !g.lap_pk) return;
    k_gc_pack0<<<(g.nn + kGcBlock - 1) / kGcBlock, kGcBlock, 0, s>>>(g);
    gc_check(nullptr);
}

GcRowTerm gc_row_term(const GcDev& g, const BatchView& B) {
    GcRowTerm t;
    t.ya = g.out0;
    t.e_node = g.e_node;
    t.e_g = g.e_g;
    for (int k = 0; k < kMaxRhs; ++k) {
        const double om = k < B.K ? B.omega[k] : 0.0;
        t.s[k] = (om > 0.0 && om <= g.omega_max) ? (float)(1.0 / om) : 0.0f;
    }
    return t;
}

template <int K>
void gc_apply_k(const GcDev& g, int n_rows, const float2* in, cudaStream_t s, long long* launches,
                KernelTimer* timer) {
    const int nl = g.n_levels;
    if (nl < 1) return;
    float2* out = g.out0;
    // the edge vector gathered once; level-0 node vectors b, x (written, read
    // back), the scratch residual (written, read by the restriction), the
    // result (written); the Laplacian's incidence entries (value + column)
    // twice; the restriction weights once
    const double eb = (double)n_rows * K * sizeof(float2), nb = (double)g.nn * K * sizeof(float2);
    const double bytes = eb + 7 * nb + 2.0 * g.inc_entries * 12 + (double)g.inc_entries * 8;
    const int th = timer ? timer->begin(kClsGradcorr, bytes, K, s) : -1;
    const int pre = g.presmooth && nl > 1 ? 1 : 0;   // V(1,1) or V(0,1)
    k_gc_restrict_edges<K><<<gc_grid((long)g.nn * K), kGcBlock, 0, s>>>(g, in, pre);
    gc_check(launches);
    vcycle_k<K>(g, pre, out, s, launches);
    if (timer) timer->end(th, s);
}

// ---------------------------------------------------------------------------
// Mixed-precision solve of the divergence-correction Poisson system
// (divcorr_poisson_, forward_solver_fv.cpp:623-722): FP64 iterative
// refinement around complex-FP32 PCG solves preconditioned by the FP32
// V(1,1) cycle (symmetric: Jacobi pre- and post-smoothing, R = P^T, exact
// coarse solve).  A right-hand side stops when its FP64 true residual
// |divJ - L phi| falls below 1e-10 |divJ|, the reference's PCG stopping rule.
// ---------------------------------------------------------------------------
namespace {

using phys::DcWork;
using phys::DcState;

// phi = 0, r = divJ on the running right-hand sides
template <int K>
__global__ void __launch_bounds__(kGcBlock) k_dcm_init64(int nn, DcWork w) {
    const long n = (long)nn * K;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        if (!w.st[i % K].cg_run) continue;
        w.phi[i] = make_double2(0.0, 0.0);
        w.r[i] = w.divJ[i];
    }
}

// |r|^2 of the FP64 residual; right-hand sides at 1e-10 |divJ| (or out of
// refinements) stop, the others get rho = |r| and the FP32 tolerance
template <int K>
__global__ void __launch_bounds__(kGcBlock) k_dcm_norm(int nn, DcWork w, GcDev g, int max_ref, RedScratch rs) {
    const long n = (long)nn * K;
    const long i0 = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const long stride = (long)gridDim.x * blockDim.x;
    const bool run = w.st[i0 % K].cg_run;
    double2 acc[1] = {make_double2(0.0, 0.0)};
    for (long i = i0; i < n && run; i += stride) {
        const double2 r = w.r[i];
        acc[0].x += r.x * r.x + r.y * r.y;
    }
    __shared__ double2 out[K];
    if (grid_reduce_lanes<1, K, kGcBlock>(acc, rs, out)) {
        if (threadIdx.x < K) {
            DcState S = w.st[threadIdx.x];
            GcPcgState T = g.dc_st[threadIdx.x];
            T.run = 0;
            if (S.cg_run) {
                S.rn = out[threadIdx.x].x;
                const double rho = sqrt(S.rn);
                if (rho < 1e-10 * S.dn || T.ref >= max_ref) {
                    S.cg_run = 0;
                } else {
                    T.rho = rho;
                    T.tol = fmax(0.5e-10 * S.dn / rho, 1e-5);
                    T.run = 1;
                    T.iter = 0;
                    T.ref += 1;
                }
            }
            w.st[threadIdx.x] = S;
            g.dc_st[threadIdx.x] = T;
        }
    }
}

// r32 = r / rho, x32 = 0
template <int K>
__global__ void __launch_bounds__(kGcBlock) k_dcm_start(int nn, DcWork w, GcDev g) {
    const long n = (long)nn * K;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const GcPcgState& T = g.dc_st[i % K];
        float2 b = f2(0.0f, 0.0f);
        if (T.run) {
            const double2 r = w.r[i];
            const double sc = 1.0 / T.rho;
            b = f2((float)(r.x * sc), (float)(r.y * sc));
        }
        g.dc_r[i] = b;
        g.dc_x[i] = f2(0.0f, 0.0f);
    }
}

// p = z, rz = (r, z) (real: L and the V-cycle are real symmetric)
template <int K>
__global__ void __launch_bounds__(kGcBlock) k_dcm_first(int nn, GcDev g, RedScratch rs) {
    const long n = (long)nn * K;
    const long i0 = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const long stride = (long)gridDim.x * blockDim.x;
    const bool run = g.dc_st[i0 % K].run;
    double2 acc[1] = {make_double2(0.0, 0.0)};
    for (long i = i0; i < n && run; i += stride) {
        const float2 r = g.dc_r[i], z = g.dc_z[i];
        g.dc_p[i] = z;
        acc[0].x += (double)(r.x * z.x + r.y * z.y);
    }
    __shared__ double2 out[K];
    if (grid_reduce_lanes<1, K, kGcBlock>(acc, rs, out)) {
        if (threadIdx.x < K && g.dc_st[threadIdx.x].run) g.dc_st[threadIdx.x].rz = out[threadIdx.x].x;
    }
}

// Ap = L p (FP32, incidence form), (p, Ap) -> alpha
template <int K>
__global__ void __launch_bounds__(kGcBlock) k_dcm_ap(int nn, GcDev g, RedScratch rs) {
    const long n = (long)nn * K;
    const long i0 = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const long stride = (long)gridDim.x * blockDim.x;
    const bool run = g.dc_st[i0 % K].run;
    const XPlain xf{g.dc_p};
    double2 acc[1] = {make_double2(0.0, 0.0)};
    for (long i = i0; i < n && run; i += stride) {
        const int v = (int)(i / K), k = (int)(i % K);
        const float2 ap = level_row<K, true>(g, g.lv[0], v, xf, k);
        const float2 p = g.dc_p[i];
        g.dc_ap[i] = ap;
        acc[0].x += (double)(p.x * ap.x + p.y * ap.y);
    }
    __shared__ double2 out[K];
    if (grid_reduce_lanes<1, K, kGcBlock>(acc, rs, out)) {
        if (threadIdx.x < K) {
            GcPcgState T = g.dc_st[threadIdx.x];
            if (T.run) {
                const double pap = out[threadIdx.x].x;
                if (!(fabs(pap) > 1e-30)) T.run = 0;
                else T.alpha = T.rz / pap;
            }
            g.dc_st[threadIdx.x] = T;
        }
    }
}

// x += alpha p, r -= alpha Ap, |r| <= tol (|b| = 1) or the iteration cap stops
template <int K>
__global__ void __launch_bounds__(kGcBlock) k_dcm_update(int nn, GcDev g, int cap, RedScratch rs) {
    const long n = (long)nn * K;
    const long i0 = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const long stride = (long)gridDim.x * blockDim.x;
    const GcPcgState T0 = g.dc_st[i0 % K];
    const float al = (float)T0.alpha;
    double2 acc[1] = {make_double2(0.0, 0.0)};
    for (long i = i0; i < n && T0.run; i += stride) {
        const float2 p = g.dc_p[i], ap = g.dc_ap[i];
        float2 x = g.dc_x[i], r = g.dc_r[i];
        x.x += al * p.x;
        x.y += al * p.y;
        r.x -= al * ap.x;
        r.y -= al * ap.y;
        g.dc_x[i] = x;
        g.dc_r[i] = r;
        acc[0].x += (double)(r.x * r.x + r.y * r.y);
    }
    __shared__ double2 out[K];
    if (grid_reduce_lanes<1, K, kGcBlock>(acc, rs, out)) {
        if (threadIdx.x < K) {
            GcPcgState T = g.dc_st[threadIdx.x];
            if (T.run) {
                T.iter += 1;
                if (sqrt(out[threadIdx.x].x) <= T.tol || T.iter >= cap) T.run = 0;
            }
            g.dc_st[threadIdx.x] = T;
        }
    }
}

// (r, z) -> beta
template <int K>
__global__ void __launch_bounds__(kGcBlock) k_dcm_rz(int nn, GcDev g, RedScratch rs) {
    const long n = (long)nn * K;
    const long i0 = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const long stride = (long)gridDim.x * blockDim.x;
    const bool run = g.dc_st[i0 % K].run;
    double2 acc[1] = {make_double2(0.0, 0.0)};
    for (long i = i0; i < n && run; i += stride) {
        const float2 r = g.dc_r[i], z = g.dc_z[i];
        acc[0].x += (double)(r.x * z.x + r.y * z.y);
    }
    __shared__ double2 out[K];
    if (grid_reduce_lanes<1, K, kGcBlock>(acc, rs, out)) {
        if (threadIdx.x < K) {
            GcPcgState T = g.dc_st[threadIdx.x];
            if (T.run) {
                const double rzn = out[threadIdx.x].x;
                T.beta = rzn / (T.rz + 1e-300);
                T.rz = rzn;
            }
            g.dc_st[threadIdx.x] = T;
        }
    }
}

// p = z + beta p
template <int K>
__global__ void __launch_bounds__(kGcBlock) k_dcm_p(int nn, GcDev g) {
    const long n = (long)nn * K;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const GcPcgState& T = g.dc_st[i % K];
        if (!T.run) continue;
        const float be = (float)T.beta;
        const float2 z = g.dc_z[i];
        float2 p = g.dc_p[i];
        p.x = z.x + be * p.x;
        p.y = z.y + be * p.y;
        g.dc_p[i] = p;
    }
}

// phi += rho x (FP64), then r = divJ - L phi in FP64 (incidence form)
template <int K>
__global__ void __launch_bounds__(kGcBlock) k_dcm_back(int nn, DcWork w, GcDev g) {
    const long n = (long)nn * K;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        if (!w.st[i % K].cg_run) continue;
        const double rho = g.dc_st[i % K].rho;
        const float2 x = g.dc_x[i];
        double2 ph = w.phi[i];
        ph.x += rho * (double)x.x;
        ph.y += rho * (double)x.y;
        w.phi[i] = ph;
    }
}

template <int K>
__global__ void __launch_bounds__(kGcBlock) k_dcm_resid64(int nn, DcWork w, GcDev g) {
    const long n = (long)nn * K;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int v = (int)(i / K), k = (int)(i % K);
        if (!w.st[k].cg_run) continue;
        const double2 pv = w.phi[i];
        const double dg = __ldg(&g.lap_diag[v]);
        double sx = dg * pv.x, sy = dg * pv.y;
        const int q0 = __ldg(&g.inc_ptr[v]), q1 = __ldg(&g.inc_ptr[v + 1]);
        for (int q = q0; q < q1; q += 4) {
            double a[4];
            double2 xv[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const bool ok = q + u < q1;
                a[u] = ok ? __ldg(&g.lap_off[q + u]) : 0.0;
                xv[u] = (ok && a[u] != 0.0) ? w.phi[(size_t)__ldg(&g.inc_other[q + u]) * K + k] : make_double2(0.0, 0.0);
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                sx += a[u] * xv[u].x;
                sy += a[u] * xv[u].y;
            }
        }
        const double2 d = w.divJ[i];
        w.r[i] = make_double2(d.x - sx, d.y - sy);
    }
}

// per right-hand side: the FP32 PCG iterations into cg_iter, the refinement
// counter reset for the next call
template <int K>
__global__ void k_dcm_count(DcWork w, GcDev g, int reset) {
    const int k = threadIdx.x;
    if (k >= K) return;
    GcPcgState T = g.dc_st[k];
    if (reset) {
        T.ref = 0;
        T.run = 0;
    } else {
        DcState S = w.st[k];
        S.cg_iter += T.iter;
        w.st[k] = S;
    }
    g.dc_st[k] = T;
}

}  // namespace

template <int K>
long long dc_poisson_mixed_k(const GcDev& g, int nn, DcWork w, RedScratch red, cudaStream_t s,
                             long long* sweeps) {
    long long launches = 0;
    const int cap = red.max_blocks;
    const int g_n = gc_grid((long)nn * K);
    const int g_norm = wave_grid(k_dcm_norm<K>, cap, kGcBlock), g_first = wave_grid(k_dcm_first<K>, cap, kGcBlock);
    const int g_ap = wave_grid(k_dcm_ap<K>, cap, kGcBlock), g_up = wave_grid(k_dcm_update<K>, cap, kGcBlock);
    const int g_rz = wave_grid(k_dcm_rz<K>, cap, kGcBlock);
    constexpr int kMaxRef = 8, kCap = 400, kPoll = 8;
    // V(1,1) cycle on the FP32 residual, into z
    GcDev gv = g;
    gv.lv[0].b = g.dc_r;
    auto precondition = [&]() {
        k_gc_pre0<K><<<g_n, kGcBlock, 0, s>>>(gv);
        gc_check(&launches);
        vcycle_k<K>(gv, gv.n_levels > 1 ? 1 : 0, g.dc_z, s, &launches);
    };
    k_dcm_count<K><<<1, 32, 0, s>>>(w, g, 1);
    k_dcm_init64<K><<<g_n, kGcBlock, 0, s>>>(nn, w);
    gc_check(&launches);
    launches += 1;
    std::vector<GcPcgState> hs(K);
    for (int ref = 0; ref <= kMaxRef; ++ref) {
        k_dcm_norm<K><<<g_norm, kGcBlock, 0, s>>>(nn, w, g, kMaxRef, red);
        gc_check(&launches);
        cudaMemcpyAsync(hs.data(), g.dc_st, sizeof(GcPcgState) * K, cudaMemcpyDeviceToHost, s);
        cudaStreamSynchronize(s);
        bool any = false;
        for (int k = 0; k < K; ++k) any |= hs[k].run != 0;
        if (!any) break;
        k_dcm_start<K><<<g_n, kGcBlock, 0, s>>>(nn, w, g);
        gc_check(&launches);
        precondition();
        k_dcm_first<K><<<g_first, kGcBlock, 0, s>>>(nn, g, red);
        gc_check(&launches);
        for (int it = 0; it < kCap; it += kPoll) {
            for (int j = 0; j < kPoll; ++j) {
                k_dcm_ap<K><<<g_ap, kGcBlock, 0, s>>>(nn, g, red);
                gc_check(&launches);
                k_dcm_update<K><<<g_up, kGcBlock, 0, s>>>(nn, g, kCap, red);
                gc_check(&launches);
                precondition();
                k_dcm_rz<K><<<g_rz, kGcBlock, 0, s>>>(nn, g, red);
                gc_check(&launches);
                k_dcm_p<K><<<g_n, kGcBlock, 0, s>>>(nn, g);
                gc_check(&launches);
            }
            if (sweeps) *sweeps += kPoll;
            cudaMemcpyAsync(hs.data(), g.dc_st, sizeof(GcPcgState) * K, cudaMemcpyDeviceToHost, s);
            cudaStreamSynchronize(s);
            bool run = false;
            for (int k = 0; k < K; ++k) run |= hs[k].run != 0;
            if (!run) break;
        }
        k_dcm_count<K><<<1, 32, 0, s>>>(w, g, 0);
        k_dcm_back<K><<<g_n, kGcBlock, 0, s>>>(nn, w, g);
        k_dcm_resid64<K><<<g_n, kGcBlock, 0, s>>>(nn, w, g);
        gc_check(&launches);
        launches += 2;
    }
    return launches;
}

template long long dc_poisson_mixed_k<2>(const GcDev&, int, DcWork, RedScratch, cudaStream_t, long long*);
template long long dc_poisson_mixed_k<4>(const GcDev&, int, DcWork, RedScratch, cudaStream_t, long long*);
template long long dc_poisson_mixed_k<8>(const GcDev&, int, DcWork, RedScratch, cudaStream_t, long long*);
template long long dc_poisson_mixed_k<16>(const GcDev&, int, DcWork, RedScratch, cudaStream_t, long long*);

template void gc_apply_k<2>(const GcDev&, int, const float2*, cudaStream_t, long long*, KernelTimer*);
template void gc_apply_k<4>(const GcDev&, int, const float2*, cudaStream_t, long long*, KernelTimer*);
template void gc_apply_k<8>(const GcDev&, int, const float2*, cudaStream_t, long long*, KernelTimer*);
template void gc_apply_k<16>(const GcDev&, int, const float2*, cudaStream_t, long long*, KernelTimer*);

}  // namespace m3d
