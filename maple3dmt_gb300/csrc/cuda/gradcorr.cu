// Gradient-space correction kernels (see gradcorr.cuh).
#include "gradcorr.cuh"

#include <algorithm>
#include <stdexcept>

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
        const float dg = (float)__ldg(&g.lap_diag[row]);
        const float2 xr = xf(row, k, K);
        s.x = dg * xr.x;
        s.y = dg * xr.y;
        const int q0 = __ldg(&g.inc_ptr[row]), q1 = __ldg(&g.inc_ptr[row + 1]);
        for (int q = q0; q < q1; q += 4) {
            float a[4];
            float2 xv[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const bool ok = q + u < q1;
                a[u] = ok ? (float)__ldg(&g.lap_off[q + u]) : 0.0f;
                xv[u] = (ok && a[u] != 0.0f) ? xf(__ldg(&g.inc_other[q + u]), k, K) : f2(0.0f, 0.0f);
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

}  // namespace

void gc_weights(const MeshDev& m, float* inc_g, float* e_g, cudaStream_t s) {
    const long n = std::max<long>(m.nn, m.n_pad);
    k_gc_weights<<<gc_grid(n), kGcBlock, 0, s>>>(m, inc_g, e_g);
    gc_check(nullptr);
}

GcRowTerm gc_row_term(const GcDev& g, const BatchView& B, int which) {
    GcRowTerm t;
    t.ya = g.out0[which];
    t.e_node = g.e_node;
    t.e_g = g.e_g;
    for (int k = 0; k < kMaxRhs; ++k) {
        const double om = k < B.K ? B.omega[k] : 0.0;
        t.s[k] = (om > 0.0 && om <= g.omega_max) ? (float)(1.0 / om) : 0.0f;
    }
    return t;
}

template <int K>
void gc_apply_k(const GcDev& g, int n_rows, const float2* in, int which, cudaStream_t s, long long* launches,
                KernelTimer* timer) {
    const int nl = g.n_levels;
    if (nl < 1) return;
    float2* out = g.out0[which];
    // the edge vector gathered once; level-0 node vectors b, x (written, read
    // back), the scratch residual (written, read by the restriction), the
    // result (written); the Laplacian's incidence entries (value + column)
    // twice; the restriction weights once
    const double eb = (double)n_rows * K * sizeof(float2), nb = (double)g.nn * K * sizeof(float2);
    const double bytes = eb + 7 * nb + 2.0 * g.inc_entries * 12 + (double)g.inc_entries * 8;
    const int th = timer ? timer->begin(kClsGradcorr, bytes, K) : -1;
    const int pre = g.presmooth && nl > 1 ? 1 : 0;   // V(1,1) or V(0,1)
    k_gc_restrict_edges<K><<<gc_grid((long)g.nn * K), kGcBlock, 0, s>>>(g, in, pre);
    gc_check(launches);
    if (nl == 1) {
        k_gc_coarse<K><<<std::max(1, g.n_coarse), kGcBlock, 0, s>>>(g.n_coarse, g.coarse_inv, g.lv[0].b, out);
        gc_check(launches);
    } else {
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
            if (l == 0) k_gc_up<K, true><<<gc_grid(work), kGcBlock, 0, s>>>(g, g.lv[l], xc, dst, pre);
            else k_gc_up<K, false><<<gc_grid(work), kGcBlock, 0, s>>>(g, g.lv[l], xc, dst, pre);
            gc_check(launches);
        }
    }
    if (timer) timer->end(th);
}

template void gc_apply_k<2>(const GcDev&, int, const float2*, int, cudaStream_t, long long*, KernelTimer*);
template void gc_apply_k<4>(const GcDev&, int, const float2*, int, cudaStream_t, long long*, KernelTimer*);
template void gc_apply_k<8>(const GcDev&, int, const float2*, int, cudaStream_t, long long*, KernelTimer*);
template void gc_apply_k<16>(const GcDev&, int, const float2*, int, cudaStream_t, long long*, KernelTimer*);

}  // namespace m3d
