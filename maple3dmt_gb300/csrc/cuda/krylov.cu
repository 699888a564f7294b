// Batched SSOR-BiCGStab kernels.  See krylov.cuh for what they restate.
#include "krylov.cuh"

#include "gradcorr.cuh"

#include <algorithm>
#include <map>
#include <mutex>
#include <stdexcept>
#include <string>
#include <tuple>
#include <type_traits>
#include <utility>

namespace m3d {

namespace dev {

int resident_blocks(const void* kernel, int threads, int smem) {
    static std::mutex mu;
    static std::map<std::tuple<int, const void*, int, int>, int> cache;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lock(mu);
    const auto key = std::make_tuple(dev, kernel, threads, smem);
    const auto it = cache.find(key);
    if (it != cache.end()) return it->second;
    int sms = 0, nb = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, threads, (size_t)smem);
    const int g = std::max(1, nb) * std::max(1, sms);
    cache[key] = g;
    return g;
}

}  // namespace dev

using namespace dev;

cudaEvent_t KernelTimer::get() {
    if (!pool.empty()) {
        cudaEvent_t e = pool.back();
        pool.pop_back();
        return e;
    }
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) throw std::runtime_error("cudaEventCreate failed");
    return e;
}

// Inside a stream capture a plain event record only marks a dependency; the
// timer's records become event-record nodes of the graph (re-recorded at
// every replay) with cudaEventRecordExternal.
static void timer_record(cudaEvent_t e, cudaStream_t s) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cs) == cudaSuccess && cs == cudaStreamCaptureStatusActive)
        cudaEventRecordWithFlags(e, s, cudaEventRecordExternal);
    else
        cudaEventRecord(e, s);
}

int KernelTimer::begin(int cls, double algorithmic_bytes, int K, cudaStream_t s) {
    if (!on) return -1;
    const int kb = K == 2 ? 0 : K == 4 ? 1 : K == 8 ? 2 : K == 16 ? 3 : 4;
    Pair p{cls, kb, get(), get(), algorithmic_bytes};
    timer_record(p.a, s ? s : stream);
    open.push_back(p);
    return (int)open.size() - 1;
}

void KernelTimer::end(int h, cudaStream_t s) {
    if (h < 0) return;
    timer_record(open[h].b, s ? s : stream);
}

void KernelTimer::set_bytes(int h, double algorithmic_bytes) {
    if (h < 0) return;
    open[h].bytes = algorithmic_bytes;
}

void KernelTimer::collect() {
    if (open.empty()) return;
    cudaStreamSynchronize(stream);
    for (const Pair& p : open) {
        float t = 0.f;
        if (cudaEventElapsedTime(&t, p.a, p.b) == cudaSuccess) {
            ms[p.cls] += t;
            bytes[p.cls] += p.bytes;
            launches[p.cls] += 1;
            ms_k[p.cls][p.kb] += t;
            bytes_k[p.cls][p.kb] += p.bytes;
            launches_k[p.cls][p.kb] += 1;
        }
        pool.push_back(p.a);
        pool.push_back(p.b);
    }
    open.clear();
    cudaGetLastError();
}

std::vector<KernelTimer::Pair> KernelTimer::take(size_t from) {
    std::vector<Pair> ps;
    if (from < open.size()) {
        ps.assign(open.begin() + (long)from, open.end());
        open.resize(from);
    }
    return ps;
}

void KernelTimer::fold(const std::vector<Pair>& ps) {
    for (const Pair& p : ps) {
        float t = 0.f;
        if (cudaEventElapsedTime(&t, p.a, p.b) == cudaSuccess) {
            ms[p.cls] += t;
            bytes[p.cls] += p.bytes;
            launches[p.cls] += 1;
            ms_k[p.cls][p.kb] += t;
            bytes_k[p.cls][p.kb] += p.bytes;
            launches_k[p.cls][p.kb] += 1;
        }
    }
    cudaGetLastError();
}

void KernelTimer::release(std::vector<Pair>& ps) {
    for (const Pair& p : ps) {
        pool.push_back(p.a);
        pool.push_back(p.b);
    }
    ps.clear();
}

void KernelTimer::reset() {
    collect();
    for (int i = 0; i < kNumCls; ++i) {
        launches[i] = 0; ms[i] = 0; bytes[i] = 0;
        for (int j = 0; j < kNumKBins; ++j) { launches_k[i][j] = 0; ms_k[i][j] = 0; bytes_k[i][j] = 0; }
    }
}

KernelTimer::~KernelTimer() {
    for (auto& p : open) { cudaEventDestroy(p.a); cudaEventDestroy(p.b); }
    for (auto e : pool) cudaEventDestroy(e);
}

namespace {

// Rows per warp when lane l works on rhs l % K.
template <int K> struct Rpw { static constexpr int v = 32 / K; };

template <class R>
__device__ __forceinline__ cplx<R> diag_of(const DiagView<R>& D, int row, R om) {
    const cplx<R> a = D.sm[row];
    return cm<R>(a.x, om * a.y);
}
// 1 / d: Smith's division in FP64 (as the assembly of the reference system),
// conj(d) / |d|^2 in FP32
__device__ __forceinline__ double2 inv_c(double2 d) { return cdiv(make_double2(1.0, 0.0), d); }
__device__ __forceinline__ float2 inv_c(float2 d) {
    const float n = d.x * d.x + d.y * d.y;
    return make_float2(d.x / n, -d.y / n);
}

// ---------------------------------------------------------------------------
// Scalar recurrences of BiCGStabSolver::solve (src/forward/bicgstab.cpp),
// run by thread k < K of the last block of each reduction.
// ---------------------------------------------------------------------------

__device__ __forceinline__ double cabs_(double2 z) { return hypot(z.x, z.y); }

// r = b - A x0; r0 = r: |b|^2, |r|^2, (r0, r)   (bicgstab.cpp:24-41, :51)
__device__ void ep_init(BicgState& S, const double2* out, int k, int K) {
    if (S.status == kInactive) return;
    double bn = sqrt(out[0 * K + k].x);
    if (bn < 1e-30) bn = 1.0;
    S.bnorm = bn;
    S.rnorm = sqrt(out[1 * K + k].x);
    S.iter = 0;
    S.pend_x = 0;
    S.breakdown = 0;
    S.res = S.rnorm / bn;
    if (S.res < S.tol) { S.status = kConverged; return; }
    S.status = kRunning;
    S.rho = out[2 * K + k];
    S.rho_old = make_double2(1.0, 0.0);
    S.alpha = make_double2(1.0, 0.0);
    S.omega = make_double2(1.0, 0.0);
    if (cabs_(S.rho) < 1e-30) { S.status = kBreakdown; S.breakdown = 1; S.iter = 1; }
}

// (r0, v) -> alpha   (bicgstab.cpp:79-87)
__device__ void ep_r0v(BicgState& S, const double2* out, int k, int K) {
    if (S.status != kRunning) return;
    const double2 r0v = out[k];
    if (cabs_(r0v) < 1e-30) {
        S.status = kBreakdown; S.breakdown = 2; S.iter += 1; S.res = S.rnorm / S.bnorm;
        return;
    }
    S.alpha = cdiv(S.rho, r0v);
}

// |s| -> early exit   (bicgstab.cpp:89-103)
__device__ void ep_s(BicgState& S, const double2* out, int k, int K) {
    if (S.status != kRunning) return;
    S.snorm = sqrt(out[k].x);
    if (S.snorm / S.bnorm < S.tol) {
        S.status = kConverged; S.pend_x = 1; S.iter += 1; S.res = S.snorm / S.bnorm;
    }
}

// (t, t), (t, s) -> omega   (bicgstab.cpp:116-125)
__device__ void ep_omega(BicgState& S, const double2* out, int k, int K) {
    if (S.status != kRunning) return;
    const double2 tt = out[0 * K + k], ts = out[1 * K + k];
    if (cabs_(tt) < 1e-30) {
        S.status = kBreakdown; S.breakdown = 3; S.pend_x = 1; S.iter += 1; S.res = S.snorm / S.bnorm;
        return;
    }
    S.omega = cdiv(ts, tt);
}

// |r|, (r0, r) -> stop tests, next rho and beta   (bicgstab.cpp:127-160, :51-62)
__device__ void ep_xr(BicgState& S, const double2* out, int k, int K) {
    if (S.pend_x) { S.pend_x = 0; return; }
    if (S.status != kRunning) return;
    S.iter += 1;
    S.rnorm = sqrt(out[0 * K + k].x);
    const double rel = S.rnorm / S.bnorm;
    S.res = rel;
    if (rel < S.tol) { S.status = kConverged; return; }
    if (cabs_(S.omega) < 1e-30) { S.status = kBreakdown; S.breakdown = 4; return; }
    S.rho_old = S.rho;
    S.rho = out[1 * K + k];
    if (S.iter >= S.maxiter) { S.status = kMaxIter; return; }
    if (cabs_(S.rho) < 1e-30) { S.status = kBreakdown; S.breakdown = 1; return; }
    S.beta = cmul(cdiv(S.rho, S.rho_old), cdiv(S.alpha, S.omega));
}

// |b - A x| / |b|
__device__ void ep_trueres(BicgState& S, const double2* out, int k, int K) {
    if (S.status == kInactive) return;
    double bn = sqrt(out[1 * K + k].x);
    if (bn < 1e-30) bn = 1.0;
    S.rnorm = sqrt(out[0 * K + k].x);
    S.bnorm = bn;
    S.true_res = S.rnorm / bn;
}

// ---------------------------------------------------------------------------
// Row products: entries [k0, k1) of one row against one right-hand side
// (this lane's), unrolled four deep so four independent gathers are in
// flight per lane; the K lanes of the row read the same entry (broadcast)
// and neighbouring complex values of the same vector row (coalesced).
// ---------------------------------------------------------------------------
template <class R, int K>
__device__ __forceinline__ cplx<R> row_dot(const OpView<R>& A, int k0, int k1, const cplx<R>* v, int rhs) {
    using C = cplx<R>;
    C s = cm<R>(0, 0);
    int k = k0;
    for (; k + 4 <= k1; k += 4) {
        int c[4];
        R a[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) { c[u] = __ldg(&A.col[k + u]); a[u] = __ldg(&A.val[k + u]); }
        C xv[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) xv[u] = v[(size_t)c[u] * K + rhs];
#pragma unroll
        for (int u = 0; u < 4; ++u) { s.x += a[u] * xv[u].x; s.y += a[u] * xv[u].y; }
    }
    for (; k < k1; ++k) {
        const int c = __ldg(&A.col[k]);
        const R a = __ldg(&A.val[k]);
        const C xv = v[(size_t)c * K + rhs];
        s.x += a * xv.x;
        s.y += a * xv.y;
    }
    return s;
}

// ---------------------------------------------------------------------------
// SpMV y = A x with fused reductions; warp task = Rpw<K> consecutive rows.
// ---------------------------------------------------------------------------
template <class R, int K, int MODE>
__global__ void __launch_bounds__(kBlock) k_spmv(OpView<R> A, DiagView<R> D, BatchView B,
                                                 const cplx<R>* __restrict__ x, cplx<R>* __restrict__ y,
                                                 const cplx<R>* __restrict__ aux,
                                                 cplx<R>* __restrict__ aux_out, BicgState* st,
                                                 RedScratch rs) {
    using C = cplx<R>;
    constexpr int RPW = Rpw<K>::v;
    constexpr int NQ = (MODE == kSpmvAp) ? 1 : (MODE == kSpmvAs || MODE == kSpmvTrueRes) ? 2 : 3;
    constexpr bool REDUCE = MODE != kSpmvPlain;
    const int lane = threadIdx.x & 31;
    const int rhs = lane % K, sub = lane / K;
    const long wg = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long W = ((long)gridDim.x * blockDim.x) >> 5;
    const R om = (R)B.omega[rhs];
    C accR[NQ];   // per-thread partial sums in the working precision
#pragma unroll
    for (int q = 0; q < NQ; ++q) accR[q] = cm<R>(0, 0);
    const long groups = A.n_pad / RPW;
    for (long t = wg; t < groups; t += W) {
        const int row = (int)(t * RPW) + sub;
        const C s = row_dot<R, K>(A, A.rp[row], A.rp[row + 1], x, rhs);
        const size_t i = (size_t)row * K + rhs;
        const C d = diag_of(D, row, om);
        const C yv = cadd(s, cmul(d, x[i]));
        if (MODE == kSpmvPlain) {
            y[i] = yv;
        } else if (MODE == kSpmvAp) {
            y[i] = yv;
            accR[0] = cadd(accR[0], cjmul(aux[i], yv));
        } else if (MODE == kSpmvAs) {
            y[i] = yv;
            accR[0].x += yv.x * yv.x + yv.y * yv.y;
            accR[1] = cadd(accR[1], cjmul(yv, aux[i]));
        } else if (MODE == kSpmvInit) {
            const C bv = aux[i];
            const C rv = csub(bv, yv);
            y[i] = rv;
            aux_out[i] = rv;
            accR[0].x += bv.x * bv.x + bv.y * bv.y;
            accR[1].x += rv.x * rv.x + rv.y * rv.y;
            accR[2] = cadd(accR[2], cjmul(rv, rv));
        } else {  // kSpmvTrueRes
            const C bv = aux[i];
            const C rv = csub(bv, yv);
            y[i] = rv;
            accR[0].x += rv.x * rv.x + rv.y * rv.y;
            accR[1].x += bv.x * bv.x + bv.y * bv.y;
        }
    }
    if (!REDUCE) return;
    double2 acc[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) acc[q] = to_d(accR[q]);
    __shared__ double2 out[NQ * K];
    if (grid_reduce_lanes<NQ, K>(acc, rs, out)) {
        if (threadIdx.x < K) {
            BicgState S = st[threadIdx.x];
            if (MODE == kSpmvAp) ep_r0v(S, out, threadIdx.x, K);
            else if (MODE == kSpmvAs) ep_omega(S, out, threadIdx.x, K);
            else if (MODE == kSpmvInit) ep_init(S, out, threadIdx.x, K);
            else ep_trueres(S, out, threadIdx.x, K);
            st[threadIdx.x] = S;
        }
    }
}

// SSOR forward sweep over the 32-row slices of one colour (list[0..count)):
//   y_i = (in_i - sum_{j in earlier colours} a_ij y_j) / d_i      (ssor.h:58-66)
// Gathered rows belong to other colours, which this launch does not write.
template <class R, int K>
__global__ void __launch_bounds__(kBlock) k_ssor_fwd(OpView<R> A, DiagView<R> D, BatchView B,
                                                     const int* __restrict__ list, int count,
                                                     const cplx<R>* __restrict__ in, cplx<R>* y) {
    using C = cplx<R>;
    constexpr int RPW = Rpw<K>::v;
    constexpr int GPS = kSlice / RPW;   // row groups per slice
    const int lane = threadIdx.x & 31;
    const int rhs = lane % K, sub = lane / K;
    const long wg = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long W = ((long)gridDim.x * blockDim.x) >> 5;
    const long tasks = (long)count * GPS;
    const R om = (R)B.omega[rhs];
    for (long t = wg; t < tasks; t += W) {
        const int row = list[t / GPS] * kSlice + (int)(t % GPS) * RPW + sub;
        const C s = row_dot<R, K>(A, A.rp[row], A.rs[row], y, rhs);
        const size_t i = (size_t)row * K + rhs;
        y[i] = cmul(csub(in[i], s), cscale(inv_c(diag_of(D, row, om)), (R)B.relax));
    }
}

// SSOR backward sweep over the slices of one colour:
//   out_i = y_i - (sum_{j in later colours} a_ij out_j) / d_i      (ssor.h:69-78)
template <class R, int K>
__global__ void __launch_bounds__(kBlock) k_ssor_bwd(OpView<R> A, DiagView<R> D, BatchView B,
                                                     const int* __restrict__ list, int count,
                                                     const cplx<R>* __restrict__ y, cplx<R>* out) {
    using C = cplx<R>;
    constexpr int RPW = Rpw<K>::v;
    constexpr int GPS = kSlice / RPW;
    const int lane = threadIdx.x & 31;
    const int rhs = lane % K, sub = lane / K;
    const long wg = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long W = ((long)gridDim.x * blockDim.x) >> 5;
    const long tasks = (long)count * GPS;
    const R om = (R)B.omega[rhs];
    for (long t = wg; t < tasks; t += W) {
        const int row = list[t / GPS] * kSlice + (int)(t % GPS) * RPW + sub;
        const C s = row_dot<R, K>(A, A.rs[row], A.rp[row + 1], out, rhs);
        const size_t i = (size_t)row * K + rhs;
        out[i] = csub(y[i], cmul(s, cscale(inv_c(diag_of(D, row, om)), (R)B.relax)));
    }
}

// ---------------------------------------------------------------------------
// Slice-staged row kernels (segments of staged.cuh in shared memory).
// ---------------------------------------------------------------------------

// SpMV over slice-staged rows, same modes and reductions as k_spmv.
template <class R, int K, int MODE>
__global__ void __launch_bounds__(StagedShape<K>::NT, StagedMinBlocks<R, K>::v) k_spmv_st(SegView<R> S, long n_slices, DiagView<R> D,
                                                                BatchView B, const cplx<R>* __restrict__ x,
                                                                cplx<R>* __restrict__ y,
                                                                const cplx<R>* __restrict__ aux,
                                                                cplx<R>* __restrict__ aux_out, BicgState* st,
                                                                RedScratch rs) {
    using C = cplx<R>;
    using Sh = StagedShape<K>;
    constexpr int RPW = Rpw<K>::v;
    constexpr int NQ = (MODE == kSpmvAp) ? 1 : (MODE == kSpmvAs || MODE == kSpmvTrueRes) ? 2 : 3;
    constexpr bool REDUCE = MODE != kSpmvPlain;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int rhs = lane % K;
    const int lr0 = warp * RPW + lane / K;
    const R om = (R)B.omega[rhs];
    C accR[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) accR[q] = cm<R>(0, 0);
    slice_pipeline<3>(S.seg, S.work_nat, n_slices, S.stage_spmv, S.err, [&](const SegItem& it, const unsigned char* base) {
        SegRows<R> lo, up;
        lo.bind(base);
        up.bind(base + (size_t)it.lo_len * 16);
#pragma unroll
        for (int ps = 0; ps < Sh::PASSES; ++ps) {
            const int lr = ps * Sh::ROWS_PER_PASS + lr0;
            const int row = it.slice * kSlice + lr;
            const size_t i = (size_t)row * K + rhs;
            const C xi = x[i];
            const C av = (MODE != kSpmvPlain) ? aux[i] : cm<R>(0, 0);
            const C d = diag_of(D, row, om);
            const C s = seg_row_dot_lu<R, K>(lo, up, lr, x, rhs);
            const C yv = cadd(s, cmul(d, xi));
            if (MODE == kSpmvPlain) {
                y[i] = yv;
            } else if (MODE == kSpmvAp) {
                y[i] = yv;
                accR[0] = cadd(accR[0], cjmul(av, yv));
            } else if (MODE == kSpmvAs) {
                y[i] = yv;
                accR[0].x += yv.x * yv.x + yv.y * yv.y;
                accR[1] = cadd(accR[1], cjmul(yv, av));
            } else if (MODE == kSpmvInit) {
                const C rv = csub(av, yv);
                y[i] = rv;
                aux_out[i] = rv;
                accR[0].x += av.x * av.x + av.y * av.y;
                accR[1].x += rv.x * rv.x + rv.y * rv.y;
                accR[2] = cadd(accR[2], cjmul(rv, rv));
            } else {  // kSpmvTrueRes
                const C rv = csub(av, yv);
                y[i] = rv;
                accR[0].x += rv.x * rv.x + rv.y * rv.y;
                accR[1].x += av.x * av.x + av.y * av.y;
            }
        }
    });
    if (!REDUCE) return;
    double2 acc[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) acc[q] = to_d(accR[q]);
    __shared__ double2 out[NQ * K];
    if (grid_reduce_lanes<NQ, K, Sh::NT>(acc, rs, out)) {
        if (threadIdx.x < K) {
            BicgState T = st[threadIdx.x];
            if (MODE == kSpmvAp) ep_r0v(T, out, threadIdx.x, K);
            else if (MODE == kSpmvAs) ep_omega(T, out, threadIdx.x, K);
            else if (MODE == kSpmvInit) ep_init(T, out, threadIdx.x, K);
            else ep_trueres(T, out, threadIdx.x, K);
            st[threadIdx.x] = T;
        }
    }
}

// SSOR forward sweep of one colour over slice-staged lower parts
// (ssor.h:58-66); items work_col[0..count) of the colour.
template <class R, int K>
__device__ __forceinline__ void ssor_fwd_rows(const SegItem& it, const unsigned char* base, const DiagView<R>& D,
                                              R om, R rx, int rhs, int lr0, const cplx<R>* __restrict__ in,
                                              cplx<R>* y) {
    using C = cplx<R>;
    using Sh = StagedShape<K>;
    SegRows<R> lo;
    lo.bind(base);
    // one pass's gathers at a time: at 46 registers the forward sweep keeps
    // more resident blocks than with both passes' heads held (69 registers),
    // which measured faster for its short lower rows
#pragma unroll
    for (int ps = 0; ps < Sh::PASSES; ++ps) {
        const int lr = ps * Sh::ROWS_PER_PASS + lr0;
        const int row = it.slice * kSlice + lr;
        const size_t i = (size_t)row * K + rhs;
        const C iv = in[i];
        const C d = diag_of(D, row, om);
        const C s = seg_row_dot<R, K>(lo.col, lo.val, lo.begin_of(lr), lo.end[lr], y, rhs, cm<R>(0, 0));
        y[i] = cmul(csub(iv, s), cscale(inv_c(d), rx));
    }
}

// SSOR forward sweep of one colour over slice-staged lower parts (ssor.h:58-66).
template <class R, int K>
__global__ void __launch_bounds__(StagedShape<K>::NT, StagedMinBlocks<R, K>::v) k_ssor_fwd_st(SegView<R> S, const int4* __restrict__ work,
                                                                    int count, DiagView<R> D, BatchView B,
                                                                    const cplx<R>* __restrict__ in, cplx<R>* y) {
    constexpr int RPW = Rpw<K>::v;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int rhs = lane % K;
    const int lr0 = warp * RPW + lane / K;
    const R om = (R)B.omega[rhs];
    slice_pipeline<1>(S.seg, work, count, S.stage_lo, S.err, [&](const SegItem& it, const unsigned char* base) {
        ssor_fwd_rows<R, K>(it, base, D, om, (R)B.relax, rhs, lr0, in, y);
    });
}

// The backward rows of one staged slice (ssor.h:69-78).  GC: the
// preconditioner's gradient-space term c = G~ y0 / (i omega) is added to the
// written row, out_i = w_i + c_i; the sweep then keeps w in y (in place of the
// forward result, read once per row before it is replaced) and gathers the
// later colours' w from there.
template <class R, int K, bool GC>
__device__ __forceinline__ void ssor_bwd_rows(const SegItem& it, const unsigned char* base, const DiagView<R>& D,
                                              R om, R rx, int rhs, int lr0, cplx<R>* y, cplx<R>* out,
                                              const GcRowTerm& gt) {
    using C = cplx<R>;
    using Sh = StagedShape<K>;
    constexpr int NP = Sh::PASSES;
    SegRows<R> up;
    up.bind(base);
    // every pass's loads (the term's node indices first, the row gathers, then
    // the node values) are issued before the first row is written
    int n0[NP], n1[NP];
    if (GC) {
#pragma unroll
        for (int ps = 0; ps < NP; ++ps) {
            const int row = it.slice * kSlice + ps * Sh::ROWS_PER_PASS + lr0;
            n0[ps] = __ldg(&gt.e_node[2 * row]);
            n1[ps] = __ldg(&gt.e_node[2 * row + 1]);
        }
    }
    RowHead<R, K> h[NP];
    C yv[NP], dv[NP];
#pragma unroll
    for (int ps = 0; ps < NP; ++ps) {
        const int lr = ps * Sh::ROWS_PER_PASS + lr0;
        const int row = it.slice * kSlice + lr;
        yv[ps] = y[(size_t)row * K + rhs];
        dv[ps] = diag_of(D, row, om);
        h[ps].load(up.col, up.val, up.begin_of(lr), up.end[lr], GC ? y : out, rhs);
    }
    float g0[NP], g1[NP];
    float2 ya[NP], yb[NP];
#pragma unroll
    for (int ps = 0; ps < NP; ++ps) {
        g0[ps] = g1[ps] = 0.0f;
        ya[ps] = yb[ps] = make_float2(0.0f, 0.0f);
        if (GC) {
            const int row = it.slice * kSlice + ps * Sh::ROWS_PER_PASS + lr0;
            g0[ps] = __ldg(&gt.e_g[2 * row]);
            g1[ps] = __ldg(&gt.e_g[2 * row + 1]);
            ya[ps] = gt.ya[(size_t)n0[ps] * K + rhs];
            yb[ps] = gt.ya[(size_t)n1[ps] * K + rhs];
        }
    }
#pragma unroll
    for (int ps = 0; ps < NP; ++ps) {
        const int lr = ps * Sh::ROWS_PER_PASS + lr0;
        const int row = it.slice * kSlice + lr;
        const size_t i = (size_t)row * K + rhs;
        C s = h[ps].sum(cm<R>(0, 0));
        const int b = up.begin_of(lr) + 8, e = up.end[lr];
        if (b < e) s = seg_row_dot<R, K>(up.col, up.val, b, e, GC ? y : out, rhs, s);
        const C w = csub(yv[ps], cmul(s, cscale(inv_c(dv[ps]), rx)));
        if (GC) {
            y[i] = w;
            const float sc = gt.s[rhs];
            const float gx = g0[ps] * ya[ps].x + g1[ps] * yb[ps].x, gy = g0[ps] * ya[ps].y + g1[ps] * yb[ps].y;
            out[i] = cm<R>(w.x + (R)(sc * gy), w.y - (R)(sc * gx));
        } else {
            out[i] = w;
        }
    }
}

// SSOR backward sweep of one colour over slice-staged upper parts.
template <class R, int K, bool GC>
__global__ void __launch_bounds__(StagedShape<K>::NT, StagedMinBlocks<R, K>::v) k_ssor_bwd_st(SegView<R> S, const int4* __restrict__ work,
                                                                    int count, DiagView<R> D, BatchView B,
                                                                    cplx<R>* y, cplx<R>* out, GcRowTerm gt) {
    constexpr int RPW = Rpw<K>::v;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int rhs = lane % K;
    const int lr0 = warp * RPW + lane / K;
    const R om = (R)B.omega[rhs];
    slice_pipeline<2>(S.seg, work, count, S.stage_up, S.err, [&](const SegItem& it, const unsigned char* base) {
        ssor_bwd_rows<R, K, GC>(it, base, D, om, (R)B.relax, rhs, lr0, y, out, gt);
    });
}

// Whole sweeps in one cooperative launch: the sweep groups (colours, or
// (super-block, colour) pairs) one after another, a grid barrier between
// groups in place of a kernel boundary.  gptr: device copy of the groups'
// slice ranges; bar: the barrier's counter and generation.
template <class R, int K>
__global__ void __launch_bounds__(StagedShape<K>::NT, StagedMinBlocks<R, K>::v) k_ssor_fwd_coop(
    SegView<R> S, const int4* __restrict__ work, const int* __restrict__ gptr, int n_groups, DiagView<R> D,
    BatchView B, const cplx<R>* __restrict__ in, cplx<R>* y, unsigned* bar) {
    constexpr int RPW = Rpw<K>::v;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int rhs = lane % K;
    const int lr0 = warp * RPW + lane / K;
    const R om = (R)B.omega[rhs];
    for (int g = 0; g < n_groups; ++g) {
        if (g > 0) grid_barrier(bar, bar + 1, S.err);
        const int s0 = gptr[g], s1 = gptr[g + 1];
        slice_pipeline<1>(S.seg, work + s0, s1 - s0, S.stage_lo, S.err,
                          [&](const SegItem& it, const unsigned char* base) {
                              ssor_fwd_rows<R, K>(it, base, D, om, (R)B.relax, rhs, lr0, in, y);
                          });
    }
}

template <class R, int K, bool GC>
__global__ void __launch_bounds__(StagedShape<K>::NT, StagedMinBlocks<R, K>::v) k_ssor_bwd_coop(
    SegView<R> S, const int4* __restrict__ work, const int* __restrict__ gptr, int n_groups, DiagView<R> D,
    BatchView B, cplx<R>* y, cplx<R>* out, GcRowTerm gt, unsigned* bar) {
    constexpr int RPW = Rpw<K>::v;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int rhs = lane % K;
    const int lr0 = warp * RPW + lane / K;
    const R om = (R)B.omega[rhs];
    for (int g = n_groups - 1; g >= 0; --g) {
        if (g < n_groups - 1) grid_barrier(bar, bar + 1, S.err);
        const int s0 = gptr[g], s1 = gptr[g + 1];
        slice_pipeline<2>(S.seg, work + s0, s1 - s0, S.stage_up, S.err,
                          [&](const SegItem& it, const unsigned char* base) {
                              ssor_bwd_rows<R, K, GC>(it, base, D, om, (R)B.relax, rhs, lr0, y, out, gt);
                          });
    }
}

// ---------------------------------------------------------------------------
// Vector updates (thread per element (row, rhs); rhs = element % K is fixed
// per thread because the grid stride is a multiple of K).
// ---------------------------------------------------------------------------

// p = r (first iteration) or r + beta (p - omega v)   (bicgstab.cpp:60-67)
template <class R, int K>
__global__ void __launch_bounds__(kBlock) k_update_p(long n, const cplx<R>* __restrict__ r,
                                                     cplx<R>* __restrict__ p, const cplx<R>* __restrict__ v,
                                                     const BicgState* __restrict__ st) {
    using C = cplx<R>;
    const long i0 = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const long stride = (long)gridDim.x * blockDim.x;
    if (i0 >= n) return;
    const BicgState S = st[i0 % K];
    const bool run = S.status == kRunning;
    const bool first = S.iter == 0;
    const C beta = from_d<C>(S.beta), om = from_d<C>(S.omega);
    for (long i = i0; i < n; i += stride) {
        if (!run) { p[i] = cm<R>(0, 0); continue; }
        if (first) { p[i] = r[i]; continue; }
        p[i] = cadd(r[i], cmul(beta, csub(p[i], cmul(om, v[i]))));
    }
}

// s = r - alpha v, |s|^2   (bicgstab.cpp:89-94)
template <class R, int K>
__global__ void __launch_bounds__(kBlock) k_update_s(long n, const cplx<R>* __restrict__ r,
                                                     const cplx<R>* __restrict__ v, cplx<R>* __restrict__ s,
                                                     BicgState* st, RedScratch rs) {
    using C = cplx<R>;
    const long i0 = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const long stride = (long)gridDim.x * blockDim.x;
    const int rhs = (int)(i0 % K);
    const BicgState S = st[rhs];
    const bool run = S.status == kRunning;
    const C al = from_d<C>(S.alpha);
    R ss = 0;
    for (long i = i0; i < n; i += stride) {
        if (!run) { s[i] = cm<R>(0, 0); continue; }
        const C sv = csub(r[i], cmul(al, v[i]));
        s[i] = sv;
        ss += sv.x * sv.x + sv.y * sv.y;
    }
    double2 acc[1] = {make_double2((double)ss, 0.0)};
    __shared__ double2 out[K];
    if (grid_reduce_lanes<1, K>(acc, rs, out)) {
        if (threadIdx.x < K) {
            BicgState T = st[threadIdx.x];
            ep_s(T, out, threadIdx.x, K);
            st[threadIdx.x] = T;
        }
    }
}

// x += alpha p_hat + omega s_hat; r = s - omega t; |r|^2, (r0, r)
// (bicgstab.cpp:127-133); right-hand sides that stopped at the s test or at
// a (t, t) breakdown take x += alpha p_hat only (:96, :123).
template <class R, int K>
__global__ void __launch_bounds__(kBlock) k_update_xr(long n, cplx<R>* __restrict__ x, cplx<R>* __restrict__ r,
                                                      const cplx<R>* __restrict__ r0,
                                                      const cplx<R>* __restrict__ ph,
                                                      const cplx<R>* __restrict__ sh,
                                                      const cplx<R>* __restrict__ s,
                                                      const cplx<R>* __restrict__ t, BicgState* st,
                                                      RedScratch rs) {
    using C = cplx<R>;
    const long i0 = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const long stride = (long)gridDim.x * blockDim.x;
    const int rhs = (int)(i0 % K);
    const BicgState S = st[rhs];
    const bool run = S.status == kRunning;
    const bool pend = S.pend_x != 0;
    const C al = from_d<C>(S.alpha), om = from_d<C>(S.omega);
    R rr = 0;
    C r0r = cm<R>(0, 0);
    for (long i = i0; i < n; i += stride) {
        if (pend) { x[i] = cadd(x[i], cmul(al, ph[i])); continue; }
        if (!run) continue;
        x[i] = cadd(x[i], cadd(cmul(al, ph[i]), cmul(om, sh[i])));
        const C rv = csub(s[i], cmul(om, t[i]));
        r[i] = rv;
        rr += rv.x * rv.x + rv.y * rv.y;
        r0r = cadd(r0r, cjmul(r0[i], rv));
    }
    double2 acc[2] = {make_double2((double)rr, 0.0), to_d(r0r)};
    __shared__ double2 out[2 * K];
    if (grid_reduce_lanes<2, K>(acc, rs, out)) {
        if (threadIdx.x < K) {
            BicgState T = st[threadIdx.x];
            ep_xr(T, out, threadIdx.x, K);
            st[threadIdx.x] = T;
        }
    }
}

inline void check_launch(long long* counter) {
    if (counter) ++*counter;
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) throw std::runtime_error(cudaGetErrorString(e));
}

inline int blocks_for(long work, int per_block, int cap) {
    long b = (work + per_block - 1) / per_block;
    if (b < 1) b = 1;
    if (b > cap) b = cap;
    return (int)b;
}

// Algorithmic bytes of one matrix pass: off-diagonal entries (value +
// column), one row pointer and one (S_ii, Me_i) diagonal pair per row,
//   M = nnz_off (b_r + 4) + 4 (n + 1) + n b_c,
// the diagonals of every frequency being formed from the pair on the fly.
// Vector streams are added by the callers, each counted once per pass
// (gathers included once).
template <class R>
double matrix_bytes(const KrylovCtx<R>& c) {
    return (double)c.nnz * (sizeof(R) + 4) + 4.0 * ((double)c.n_rows + 1) + (double)c.n_rows * sizeof(cplx<R>);
}

template <class R, int K>
void spmv_staged(const KrylovCtx<R>& c, int mode, const cplx<R>* x, cplx<R>* y, const cplx<R>* aux,
                 cplx<R>* aux_out, BicgState* st) {
    constexpr int NT = StagedShape<K>::NT;
    const long ns = c.n_pad / kSlice;
    const int sb = c.seg.stage_spmv;
    // reducing modes: every block must reach the reduction, so the grid stays
    // within the partial-sum scratch
    const int cap = (mode == kSpmvPlain) ? (1 << 20) : c.red.max_blocks;
    switch (mode) {
        case kSpmvPlain:
            launch_staged(k_spmv_st<R, K, kSpmvPlain>, NT, sb, ns, cap, c.stream, c.seg, ns, c.D, c.B, x, y, aux,
                          aux_out, st, c.red);
            break;
        case kSpmvAp:
            launch_staged(k_spmv_st<R, K, kSpmvAp>, NT, sb, ns, cap, c.stream, c.seg, ns, c.D, c.B, x, y, aux,
                          aux_out, st, c.red);
            break;
        case kSpmvAs:
            launch_staged(k_spmv_st<R, K, kSpmvAs>, NT, sb, ns, cap, c.stream, c.seg, ns, c.D, c.B, x, y, aux,
                          aux_out, st, c.red);
            break;
        case kSpmvInit:
            launch_staged(k_spmv_st<R, K, kSpmvInit>, NT, sb, ns, cap, c.stream, c.seg, ns, c.D, c.B, x, y, aux,
                          aux_out, st, c.red);
            break;
        default:
            launch_staged(k_spmv_st<R, K, kSpmvTrueRes>, NT, sb, ns, cap, c.stream, c.seg, ns, c.D, c.B, x, y, aux,
                          aux_out, st, c.red);
            break;
    }
}

template <class R, int K>
void spmv_k(const KrylovCtx<R>& c, int mode, const cplx<R>* x, cplx<R>* y, const cplx<R>* aux,
            cplx<R>* aux_out, BicgState* st) {
    const long warps = (long)c.A.n_pad / Rpw<K>::v;
    int grid;
    if (mode == kSpmvPlain) {
        grid = blocks_for(warps, kWarpsPerBlock, 1 << 20);
    } else {
        grid = c.grid_spmv;
    }
    const int streams = 2 + (aux ? 1 : 0) + (aux_out ? 1 : 0);
    const int th = c.timer ? c.timer->begin(kClsSpmv, matrix_bytes(c) +
                                            (double)c.n_rows * K * sizeof(cplx<R>) * streams, K) : -1;
    const int cap = c.red.max_blocks;
    if (c.row_kernels == kRowsStaged) {
        spmv_staged<R, K>(c, mode, x, y, aux, aux_out, st);
        check_launch(c.launches);
        if (c.timer) c.timer->end(th);
        return;
    }
    switch (mode) {
        case kSpmvPlain:
            k_spmv<R, K, kSpmvPlain><<<grid, kBlock, 0, c.stream>>>(c.A, c.D, c.B, x, y, aux, aux_out, st, c.red);
            break;
        case kSpmvAp: {
            auto kf = k_spmv<R, K, kSpmvAp>;
            kf<<<wave_grid(kf, cap), kBlock, 0, c.stream>>>(c.A, c.D, c.B, x, y, aux, aux_out, st, c.red);
            break;
        }
        case kSpmvAs: {
            auto kf = k_spmv<R, K, kSpmvAs>;
            kf<<<wave_grid(kf, cap), kBlock, 0, c.stream>>>(c.A, c.D, c.B, x, y, aux, aux_out, st, c.red);
            break;
        }
        case kSpmvInit: {
            auto kf = k_spmv<R, K, kSpmvInit>;
            kf<<<wave_grid(kf, cap), kBlock, 0, c.stream>>>(c.A, c.D, c.B, x, y, aux, aux_out, st, c.red);
            break;
        }
        default: {
            auto kf = k_spmv<R, K, kSpmvTrueRes>;
            kf<<<wave_grid(kf, cap), kBlock, 0, c.stream>>>(c.A, c.D, c.B, x, y, aux, aux_out, st, c.red);
            break;
        }
    }
    check_launch(c.launches);
    if (c.timer) c.timer->end(th);
}

// out_i += G~ y0 / (i omega) = s (g.y, -g.x) on the lanes with s != 0
template <class R, int K>
__global__ void __launch_bounds__(kBlock) k_add_gc_term(long n, cplx<R>* __restrict__ out, GcRowTerm gt) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int rhs = (int)(i % K);
    const float sc = gt.s[rhs];
    if (sc == 0.0f) return;
    const float2 g = gc_grad_row(gt, gt.ya, (int)(i / K), rhs, K);
    cplx<R> o = out[i];
    o.x += (R)(sc * g.y);
    o.y -= (R)(sc * g.x);
    out[i] = o;
}

// Blocks of a cooperative launch: every block resident at once (the
// occupancy of the kernel at this shared memory on every SM), less a quarter
// when another stream's kernels should run beside it.
inline int coop_grid(const void* kernel, int nt, int smem, bool share) {
    if (smem > 48 * 1024) cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, nt, smem);
    const int full = std::max(1, per_sm) * std::max(1, sms);
    return share ? std::max(sms, full - full / 4) : full;
}

inline void cuda_check_launch(cudaError_t e, long long* launches) {
    if (e != cudaSuccess) {
        cudaGetLastError();
        throw std::runtime_error(std::string("cooperative sweep launch failed: ") + cudaGetErrorString(e));
    }
    if (launches) ++*launches;
}

template <class R, int K>
void ssor_k(const KrylovCtx<R>& c, const cplx<R>* in, cplx<R>* y, cplx<R>* out, const GcRowTerm& gt = GcRowTerm{}) {
    constexpr int G = kSlice / Rpw<K>::v;   // row-group tasks per slice
    const int nc = (int)c.colour_ptr.size() - 1;
    // whole apply: matrix once (lower forward, upper backward), vectors in,
    // y (written, read back), out; with the gradient-space term y written
    // back once more and two node indices and weights per row
    const double gcb = gt.ya ? (double)c.n_rows * (K * sizeof(cplx<R>) + 16) : 0.0;
    int th = c.timer ? c.timer->begin(kClsSsor, matrix_bytes(c) + gcb +
                                      (double)c.n_rows * K * sizeof(cplx<R>) * 4, K) : -1;
    // the V-cycle of the term runs on the side stream; the backward sweep
    // waits for it, and the wait is kept out of the timed interval (the
    // apply is timed as two intervals, the bytes all counted with the first)
    const bool join = gt.ya && c.gc_stream;
    auto wait_join = [&]() {
        if (!join) return;
        if (c.timer) c.timer->end(th);
        cudaStreamWaitEvent(c.stream, c.gc_join, 0);
        th = c.timer ? c.timer->begin(kClsSsor, 0.0, K) : -1;
    };
    if (c.row_kernels == kRowsStaged && c.coop && c.colour_ptr_d && c.gridbar && nc > 1) {
        constexpr int NT = StagedShape<K>::NT;
        // with the gradient-space V-cycle running beside the forward sweep,
        // a quarter of the resident blocks is left to it
        const bool share = gt.ya && c.gc_stream;
        {
            auto kf = k_ssor_fwd_coop<R, K>;
            const int smem = 2 * c.seg.stage_lo;
            const int grid = coop_grid(reinterpret_cast<const void*>(kf), NT, smem, share);
            cudaMemsetAsync(c.gridbar, 0, sizeof(unsigned), c.stream);
            void* args[] = {(void*)&c.seg, (void*)&c.seg.work_col, (void*)&c.colour_ptr_d, (void*)&nc,
                            (void*)&c.D, (void*)&c.B, (void*)&in, (void*)&y, (void*)&c.gridbar};
            cuda_check_launch(cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(kf), grid, NT, args, smem,
                                                          c.stream), c.launches);
        }
        wait_join();
        {
            const int smem = 2 * c.seg.stage_up;
            cudaMemsetAsync(c.gridbar, 0, sizeof(unsigned), c.stream);
            if (gt.ya) {
                auto kf = k_ssor_bwd_coop<R, K, true>;
                const int grid = coop_grid(reinterpret_cast<const void*>(kf), NT, smem, false);
                void* args[] = {(void*)&c.seg, (void*)&c.seg.work_col, (void*)&c.colour_ptr_d, (void*)&nc,
                                (void*)&c.D, (void*)&c.B, (void*)&y, (void*)&out, (void*)&gt, (void*)&c.gridbar};
                cuda_check_launch(cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(kf), grid, NT, args,
                                                              smem, c.stream), c.launches);
            } else {
                auto kf = k_ssor_bwd_coop<R, K, false>;
                const int grid = coop_grid(reinterpret_cast<const void*>(kf), NT, smem, false);
                void* args[] = {(void*)&c.seg, (void*)&c.seg.work_col, (void*)&c.colour_ptr_d, (void*)&nc,
                                (void*)&c.D, (void*)&c.B, (void*)&y, (void*)&out, (void*)&gt, (void*)&c.gridbar};
                cuda_check_launch(cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(kf), grid, NT, args,
                                                              smem, c.stream), c.launches);
            }
        }
        if (c.timer) c.timer->end(th);
        return;
    }
    if (c.row_kernels == kRowsStaged) {
        constexpr int NT = StagedShape<K>::NT;
        for (int col = 0; col < nc; ++col) {
            const int s0 = c.colour_ptr[col], s1 = c.colour_ptr[col + 1];
            if (s1 <= s0) continue;
            launch_staged(k_ssor_fwd_st<R, K>, NT, c.seg.stage_lo, s1 - s0, 1 << 20, c.stream, c.seg,
                          c.seg.work_col + s0, s1 - s0, c.D, c.B, in, y);
            check_launch(c.launches);
        }
        wait_join();
        for (int col = nc - 1; col >= 0; --col) {
            const int s0 = c.colour_ptr[col], s1 = c.colour_ptr[col + 1];
            if (s1 <= s0) continue;
            if (gt.ya)
                launch_staged(k_ssor_bwd_st<R, K, true>, NT, c.seg.stage_up, s1 - s0, 1 << 20, c.stream, c.seg,
                              c.seg.work_col + s0, s1 - s0, c.D, c.B, y, out, gt);
            else
                launch_staged(k_ssor_bwd_st<R, K, false>, NT, c.seg.stage_up, s1 - s0, 1 << 20, c.stream, c.seg,
                              c.seg.work_col + s0, s1 - s0, c.D, c.B, y, out, gt);
            check_launch(c.launches);
        }
        if (c.timer) c.timer->end(th);
        return;
    }
    for (int col = 0; col < nc; ++col) {
        const int s0 = c.colour_ptr[col], s1 = c.colour_ptr[col + 1];
        if (s1 <= s0) continue;
        const int grid = blocks_for((long)(s1 - s0) * G, kWarpsPerBlock, 1 << 20);
        k_ssor_fwd<R, K><<<grid, kBlock, 0, c.stream>>>(c.A, c.D, c.B, c.colour_list + s0, s1 - s0, in, y);
        check_launch(c.launches);
    }
    wait_join();
    for (int col = nc - 1; col >= 0; --col) {
        const int s0 = c.colour_ptr[col], s1 = c.colour_ptr[col + 1];
        if (s1 <= s0) continue;
        const int grid = blocks_for((long)(s1 - s0) * G, kWarpsPerBlock, 1 << 20);
        k_ssor_bwd<R, K><<<grid, kBlock, 0, c.stream>>>(c.A, c.D, c.B, c.colour_list + s0, s1 - s0, y, out);
        check_launch(c.launches);
    }
    if (gt.ya) {   // CSR rows: the gradient-space term in a pass of its own
        const long n = (long)c.n_pad * K;
        k_add_gc_term<R, K><<<blocks_for(n, kBlock, 1 << 20), kBlock, 0, c.stream>>>(n, out, gt);
        check_launch(c.launches);
    }
    if (c.timer) c.timer->end(th);
}

// One V-cycle of the gradient-space term on G~^T in (complex FP32 only),
// output in the node buffer g.out0; the backward SSOR sweep adds the term
// per row (GcRowTerm).
template <class R, int K>
void gc_term(const KrylovCtx<R>& c, const cplx<R>* in) {
    if constexpr (std::is_same<R, float>::value) {
        if (!c.gc) return;
        if (c.gc_stream) {
            cudaEventRecord(c.gc_fork, c.stream);
            cudaStreamWaitEvent(c.gc_stream, c.gc_fork, 0);
            gc_apply_k<K>(*c.gc, c.n_rows, in, c.gc_stream, c.launches, c.timer);
            cudaEventRecord(c.gc_join, c.gc_stream);
        } else {
            gc_apply_k<K>(*c.gc, c.n_rows, in, c.stream, c.launches, c.timer);
        }
    }
}

template <class R, int K>
void iteration_k(const KrylovCtx<R>& c, const KrylovVecs<R>& v, BicgState* st) {
    const long n = (long)c.n_pad * K;
    const int gv = c.grid_vec;
    const double vb = (double)c.n_rows * K * sizeof(cplx<R>);
    int th = c.timer ? c.timer->begin(kClsVec, 4 * vb, K) : -1;
    k_update_p<R, K><<<gv, kBlock, 0, c.stream>>>(n, v.r, v.p, v.v, st);
    check_launch(c.launches);
    if (c.timer) c.timer->end(th);
    // the gradient-space term: V-cycle first, added to the preconditioned
    // vector by the backward sweep
    GcRowTerm gt;
    if (c.gc) gt = gc_row_term(*c.gc, c.B);
    gc_term<R, K>(c, v.p);
    ssor_k<R, K>(c, v.p, v.y, v.ph, gt);
    spmv_k<R, K>(c, kSpmvAp, v.ph, v.v, v.r0, nullptr, st);
    th = c.timer ? c.timer->begin(kClsVec, 3 * vb, K) : -1;
    k_update_s<R, K><<<wave_grid(k_update_s<R, K>, gv), kBlock, 0, c.stream>>>(n, v.r, v.v, v.s, st, c.red);
    check_launch(c.launches);
    if (c.timer) c.timer->end(th);
    gc_term<R, K>(c, v.s);
    ssor_k<R, K>(c, v.s, v.y, v.sh, gt);
    spmv_k<R, K>(c, kSpmvAs, v.sh, v.t, v.s, nullptr, st);
    th = c.timer ? c.timer->begin(kClsVec, 8 * vb, K) : -1;
    k_update_xr<R, K><<<wave_grid(k_update_xr<R, K>, gv), kBlock, 0, c.stream>>>(n, v.x, v.r, v.r0, v.ph, v.sh, v.s, v.t, st, c.red);
    check_launch(c.launches);
    if (c.timer) c.timer->end(th);
}

// ---------------------------------------------------------------------------
// Eisenstat form of SSOR-BiCGStab (see krylov.cuh): sweeps over the staged
// lower / upper segments, the BiCGStab p-update fused into the backward
// sweep, the dot products of the forward sweep summed per colour launch and
// block, then once in block order by k_eis_reduce.
// ---------------------------------------------------------------------------

// Mode of the forward sweep and reduction for t = A_hat s whose |s|^2 comes
// from the fused backward sweep (quantities |s|^2, (t, t), (t, s)).
constexpr int kEisAsS = 5;

// Per-block partial sums of NQ quantities per right-hand side (lane l on
// rhs l % K): shuffle tree over the lanes of a right-hand side, warps in order;
// written to dst[q * K + k].
template <int NQ, int K, int NT>
__device__ __forceinline__ void block_partial_lanes(double2 (&acc)[NQ], double2* __restrict__ dst) {
    constexpr int PK = NQ * K, NW = NT / 32;
    __shared__ double2 sm[NW][PK];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int off = 16; off >= K; off >>= 1)
#pragma unroll
        for (int q = 0; q < NQ; ++q) acc[q] = cadd(acc[q], shfl_xor(acc[q], off));
    if (lane < K)
#pragma unroll
        for (int q = 0; q < NQ; ++q) sm[warp][q * K + lane] = acc[q];
    __syncthreads();
    if (threadIdx.x < PK) {
        double2 t = make_double2(0.0, 0.0);
        for (int w = 0; w < NW; ++w) t = cadd(t, sm[w][threadIdx.x]);
        dst[threadIdx.x] = t;
    }
}

// Backward sweep of one colour: w_i = (z_i - sum_{upper} a_ij w_j) / d_i.
// FUSE 0: z = z_in.  FUSE 1: z is the new search direction, p = r + beta
// (p - omega v) (r on the first iteration, 0 for right-hand sides not
// running), written back to p (bicgstab.cpp:60-67).  FUSE 2: z = s = r - alpha v
// (0 when not running), written to `p`, and this block's partial |s|^2 in
// slot q = 0 of a 3-quantity partial block (:89-94).
template <class R, int K, int FUSE>
__global__ void __launch_bounds__(StagedShape<K>::NT, StagedMinBlocks<R, K>::v)
    k_eis_bwd_st(SegView<R> S, const int4* __restrict__ work, int count, DiagView<R> D, BatchView B,
                 const cplx<R>* __restrict__ z_in, cplx<R>* p, const cplx<R>* __restrict__ r,
                 const cplx<R>* __restrict__ vv, const BicgState* __restrict__ st, cplx<R>* w,
                 double2* __restrict__ partial) {
    using C = cplx<R>;
    using Sh = StagedShape<K>;
    constexpr int RPW = Rpw<K>::v;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int rhs = lane % K;
    const int lr0 = warp * RPW + lane / K;
    const R om = (R)B.omega[rhs];
    bool run = true, first = false;
    C be = cm<R>(0, 0), omg = cm<R>(0, 0), al = cm<R>(0, 0);
    if (FUSE != 0) {
        const BicgState T = st[rhs];
        run = T.status == kRunning;
        first = T.iter == 0;
        be = from_d<C>(T.beta);
        omg = from_d<C>(T.omega);
        al = from_d<C>(T.alpha);
    }
    R ss = 0;
    slice_pipeline<2>(S.seg, work, count, S.stage_up, S.err, [&](const SegItem& it, const unsigned char* base) {
        SegRows<R> up;
        up.bind(base);
#pragma unroll
        for (int ps = 0; ps < Sh::PASSES; ++ps) {
            const int lr = ps * Sh::ROWS_PER_PASS + lr0;
            const int row = it.slice * kSlice + lr;
            const size_t i = (size_t)row * K + rhs;
            C z;
            if (FUSE == 1) {
                if (!run) z = cm<R>(0, 0);
                else if (first) z = r[i];
                else z = cadd(r[i], cmul(be, csub(p[i], cmul(omg, vv[i]))));
                p[i] = z;
            } else if (FUSE == 2) {
                z = run ? csub(r[i], cmul(al, vv[i])) : cm<R>(0, 0);
                p[i] = z;
                ss += z.x * z.x + z.y * z.y;
            } else {
                z = z_in[i];
            }
            const C d = diag_of(D, row, om);
            const C s = seg_row_dot<R, K>(up.col, up.val, up.begin_of(lr), up.end[lr], w, rhs, cm<R>(0, 0));
            w[i] = cmul(csub(z, s), inv_c(d));
        }
    });
    if (FUSE == 2) {
        double2 acc[3] = {make_double2((double)ss, 0.0), make_double2(0.0, 0.0), make_double2(0.0, 0.0)};
        block_partial_lanes<3, K, Sh::NT>(acc, partial + (size_t)blockIdx.x * 3 * K);
    }
}

// Forward sweep of one colour: y_i = ((z_i - d_i w_i) - sum_{lower} a_ij y_j) / d_i,
// out_i = d_i (w_i + y_i) = (A_hat z)_i, with this block's partial dot
// products of out: (aux, out) (MODE Ap) or (out, out), (out, aux) (MODE As).
template <class R, int K, int MODE>
__global__ void __launch_bounds__(StagedShape<K>::NT, StagedMinBlocks<R, K>::v)
    k_eis_fwd_st(SegView<R> S, const int4* __restrict__ work, int count, DiagView<R> D, BatchView B,
                 const cplx<R>* __restrict__ z, const cplx<R>* __restrict__ w, cplx<R>* y,
                 cplx<R>* __restrict__ out, const cplx<R>* __restrict__ aux, double2* __restrict__ partial) {
    using C = cplx<R>;
    using Sh = StagedShape<K>;
    constexpr int RPW = Rpw<K>::v;
    constexpr int NQ = (MODE == kSpmvAp) ? 1 : 2;
    constexpr int NQW = (MODE == kEisAsS) ? 3 : NQ;   // quantities per partial block written
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int rhs = lane % K;
    const int lr0 = warp * RPW + lane / K;
    const R om = (R)B.omega[rhs];
    C accR[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) accR[q] = cm<R>(0, 0);
    slice_pipeline<1>(S.seg, work, count, S.stage_lo, S.err, [&](const SegItem& it, const unsigned char* base) {
        SegRows<R> lo;
        lo.bind(base);
#pragma unroll
        for (int ps = 0; ps < Sh::PASSES; ++ps) {
            const int lr = ps * Sh::ROWS_PER_PASS + lr0;
            const int row = it.slice * kSlice + lr;
            const size_t i = (size_t)row * K + rhs;
            const C zv = z[i], wv = w[i];
            const C d = diag_of(D, row, om);
            const C t = csub(zv, cmul(d, wv));
            const C s = seg_row_dot<R, K>(lo.col, lo.val, lo.begin_of(lr), lo.end[lr], y, rhs, cm<R>(0, 0));
            const C yv = cmul(csub(t, s), inv_c(d));
            y[i] = yv;
            const C ov = cmul(d, cadd(wv, yv));
            out[i] = ov;
            if (MODE == kSpmvAp) {
                accR[0] = cadd(accR[0], cjmul(aux[i], ov));
            } else {
                accR[0].x += ov.x * ov.x + ov.y * ov.y;
                accR[1] = cadd(accR[1], cjmul(ov, aux[i]));
            }
        }
    });
    double2 acc[NQW];
    acc[0] = make_double2(0.0, 0.0);
#pragma unroll
    for (int q = 0; q < NQ; ++q) acc[NQW - NQ + q] = to_d(accR[q]);
    block_partial_lanes<NQW, K, Sh::NT>(acc, partial + (size_t)blockIdx.x * NQW * K);
}

// Sums the block partials of all colour launches and runs the scalar step:
// alpha (MODE Ap, bicgstab.cpp:79-87) or omega (MODE As, :116-125).  Block b
// sums slots [b * kEisSlotsPerBlock, ...) in a fixed order, the last block to
// finish sums the block results in block order: deterministic, and no single
// block walks thousands of slots.
constexpr int kEisSlotsPerBlock = 64;

template <int K, int MODE>
__global__ void __launch_bounds__(kBlock) k_eis_reduce(const double2* __restrict__ partial, int slots,
                                                       BicgState* st, RedScratch rs) {
    constexpr int NQ = (MODE == kSpmvAp) ? 1 : (MODE == kEisAsS) ? 3 : 2;
    constexpr int PK = NQ * K;
    constexpr int CH = kBlock / PK;
    __shared__ double2 chunk[kBlock];
    __shared__ double2 out[PK];
    __shared__ bool am_last;
    const int p = threadIdx.x % PK, j = threadIdx.x / PK;
    const int s0 = blockIdx.x * kEisSlotsPerBlock;
    const int s1 = min(slots, s0 + kEisSlotsPerBlock);
    double2 s = make_double2(0.0, 0.0);
    if (j < CH)
        for (int b = s0 + j; b < s1; b += CH) s = cadd(s, __ldcg(&partial[(size_t)b * PK + p]));
    chunk[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x < PK) {
        double2 t = make_double2(0.0, 0.0);
        for (int jj = 0; jj < CH; ++jj) t = cadd(t, chunk[jj * PK + threadIdx.x]);
        __stcg(&rs.partial[(size_t)blockIdx.x * PK + threadIdx.x], t);
        __threadfence();
    }
    __syncthreads();
    if (threadIdx.x == 0) am_last = atomicAdd(rs.counter, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!am_last) return;
    __threadfence();
    s = make_double2(0.0, 0.0);
    if (j < CH)
        for (int b = j; b < (int)gridDim.x; b += CH) s = cadd(s, __ldcg(&rs.partial[(size_t)b * PK + p]));
    chunk[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x < PK) {
        double2 t = make_double2(0.0, 0.0);
        for (int jj = 0; jj < CH; ++jj) t = cadd(t, chunk[jj * PK + threadIdx.x]);
        out[threadIdx.x] = t;
    }
    __syncthreads();
    if (threadIdx.x < K) {
        BicgState T = st[threadIdx.x];
        if (MODE == kSpmvAp) {
            ep_r0v(T, out, threadIdx.x, K);
        } else if (MODE == kEisAsS) {
            ep_s(T, out, threadIdx.x, K);
            ep_omega(T, out + K, threadIdx.x, K);
        } else {
            ep_omega(T, out, threadIdx.x, K);
        }
        st[threadIdx.x] = T;
    }
    if (threadIdx.x == 0) *rs.counter = 0u;
}

// r = r0 = D y (the split right side b_hat = D (D + L)^-1 b), |b_hat|, (r0, r) -> start
template <class R, int K>
__global__ void __launch_bounds__(kBlock) k_eis_init(long n, DiagView<R> D, BatchView B,
                                                     const cplx<R>* __restrict__ y, cplx<R>* __restrict__ r,
                                                     cplx<R>* __restrict__ r0, BicgState* st, RedScratch rs) {
    using C = cplx<R>;
    const long i0 = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const long stride = (long)gridDim.x * blockDim.x;
    const int rhs = (int)(i0 % K);
    const R om = (R)B.omega[rhs];
    R bb = 0;
    C rr = cm<R>(0, 0);
    for (long i = i0; i < n; i += stride) {
        const C rv = cmul(diag_of(D, (int)(i / K), om), y[i]);
        r[i] = rv;
        r0[i] = rv;
        bb += rv.x * rv.x + rv.y * rv.y;
        rr = cadd(rr, cjmul(rv, rv));
    }
    double2 acc[3] = {make_double2((double)bb, 0.0), make_double2((double)bb, 0.0), to_d(rr)};
    __shared__ double2 out[3 * K];
    if (grid_reduce_lanes<3, K>(acc, rs, out)) {
        if (threadIdx.x < K) {
            BicgState T = st[threadIdx.x];
            ep_init(T, out, threadIdx.x, K);
            st[threadIdx.x] = T;
        }
    }
}

// Blocks of one staged launch (as launch_staged chooses them).
template <class F>
int staged_grid(F* kernel, int nt, int stage_bytes, long items, int cap) {
    const int smem = 2 * stage_bytes;
    if (smem > 48 * 1024)
        cudaFuncSetAttribute(reinterpret_cast<const void*>(kernel), cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    return (int)std::min<long>((long)wave_grid(kernel, cap, nt, smem), std::max<long>(items, 1));
}

// out = A_hat z over every colour.  FUSE 1: z is the updated p; FUSE 2: z
// is s = r - alpha v, stored in `p`, with |s|^2 reduced alongside (MODE
// kEisAsS); see k_eis_bwd_st.  The backward sweeps of FUSE 2 take the first
// partial slots, the forward sweeps the next; one reduction sums them all.
template <class R, int K, int FUSE, int MODE>
void eis_apply_k(const KrylovCtx<R>& c, const cplx<R>* z, cplx<R>* p, const cplx<R>* r, const cplx<R>* vv,
                 BicgState* st, cplx<R>* w, cplx<R>* y, cplx<R>* out, const cplx<R>* aux) {
    constexpr int NT = StagedShape<K>::NT;
    constexpr int NQW = (MODE == kSpmvAp) ? 1 : (MODE == kEisAsS) ? 3 : 2;
    const int nc = (int)c.colour_ptr.size() - 1;
    int slot = 0;
    for (int col = nc - 1; col >= 0; --col) {
        const int s0 = c.colour_ptr[col], s1 = c.colour_ptr[col + 1];
        if (s1 <= s0) continue;
        auto kb = k_eis_bwd_st<R, K, FUSE>;
        const int g = staged_grid(kb, NT, c.seg.stage_up, s1 - s0, 1 << 20);
        if (FUSE == 2 && slot + g > c.eis_slots) throw std::runtime_error("Eisenstat partial-sum scratch too small");
        kb<<<g, NT, 2 * c.seg.stage_up, c.stream>>>(c.seg, c.seg.work_col + s0, s1 - s0, c.D, c.B, z, p, r, vv,
                                                      (const BicgState*)st, w,
                                                      c.eis_partial + (size_t)slot * NQW * K);
        check_launch(c.launches);
        if (FUSE == 2) slot += g;
    }
    const cplx<R>* zz = FUSE != 0 ? (const cplx<R>*)p : z;
    for (int col = 0; col < nc; ++col) {
        const int s0 = c.colour_ptr[col], s1 = c.colour_ptr[col + 1];
        if (s1 <= s0) continue;
        auto kf = k_eis_fwd_st<R, K, MODE>;
        const int g = staged_grid(kf, NT, c.seg.stage_lo, s1 - s0, 1 << 20);
        if (slot + g > c.eis_slots) throw std::runtime_error("Eisenstat partial-sum scratch too small");
        kf<<<g, NT, 2 * c.seg.stage_lo, c.stream>>>(c.seg, c.seg.work_col + s0, s1 - s0, c.D, c.B, zz,
                                                      (const cplx<R>*)w, y, out, aux,
                                                      c.eis_partial + (size_t)slot * NQW * K);
        check_launch(c.launches);
        slot += g;
    }
    const int gr = std::max(1, (slot + kEisSlotsPerBlock - 1) / kEisSlotsPerBlock);
    if (gr > c.red.max_blocks) throw std::runtime_error("Eisenstat reduction grid beyond the reduction scratch");
    k_eis_reduce<K, MODE><<<gr, kBlock, 0, c.stream>>>(c.eis_partial, slot, st, c.red);
    check_launch(c.launches);
}

template <class R, int K>
void eis_init_k(const KrylovCtx<R>& c, const KrylovVecs<R>& v, BicgState* st) {
    constexpr int NT = StagedShape<K>::NT;
    const int nc = (int)c.colour_ptr.size() - 1;
    for (int col = 0; col < nc; ++col) {
        const int s0 = c.colour_ptr[col], s1 = c.colour_ptr[col + 1];
        if (s1 <= s0) continue;
        launch_staged(k_ssor_fwd_st<R, K>, NT, c.seg.stage_lo, s1 - s0, 1 << 20, c.stream, c.seg,
                      c.seg.work_col + s0, s1 - s0, c.D, c.B, (const cplx<R>*)v.b, v.y);
        check_launch(c.launches);
    }
    const long n = (long)c.n_pad * K;
    k_eis_init<R, K><<<wave_grid(k_eis_init<R, K>, c.grid_vec), kBlock, 0, c.stream>>>(n, c.D, c.B, v.y, v.r, v.r0,
                                                                                    st, c.red);
    check_launch(c.launches);
}

template <class R, int K>
void eis_iteration_k(const KrylovCtx<R>& c, const KrylovVecs<R>& v, BicgState* st) {
    const long n = (long)c.n_pad * K;
    const int gv = c.grid_vec;
    const double vb = (double)c.n_rows * K * sizeof(cplx<R>);
    // p update + v = A_hat p: matrix once, r, p (read, write), v (read, write), w (write, read), y
    int th = c.timer ? c.timer->begin(kClsSsor, matrix_bytes(c) + 9 * vb, K) : -1;
    eis_apply_k<R, K, 1, kSpmvAp>(c, nullptr, v.p, v.r, v.v, st, v.ph, v.y, v.v, v.r0);
    if (c.timer) c.timer->end(th);
    // s = r - alpha v with |s|^2, and t = A_hat s: matrix once, r, v, s (write,
    // read twice), w (write, read), y, t
    th = c.timer ? c.timer->begin(kClsSsor, matrix_bytes(c) + 9 * vb, K) : -1;
    eis_apply_k<R, K, 2, kEisAsS>(c, nullptr, v.s, v.r, v.v, st, v.ph, v.y, v.t, v.s);
    if (c.timer) c.timer->end(th);
    th = c.timer ? c.timer->begin(kClsVec, 8 * vb, K) : -1;
    k_update_xr<R, K><<<wave_grid(k_update_xr<R, K>, gv), kBlock, 0, c.stream>>>(n, v.x, v.r, v.r0, v.p, v.s, v.s,
                                                                              v.t, st, c.red);
    check_launch(c.launches);
    if (c.timer) c.timer->end(th);
}

template <class R, int K>
void eis_finish_k(const KrylovCtx<R>& c, const KrylovVecs<R>& v, cplx<R>* out) {
    constexpr int NT = StagedShape<K>::NT;
    const int nc = (int)c.colour_ptr.size() - 1;
    for (int col = nc - 1; col >= 0; --col) {
        const int s0 = c.colour_ptr[col], s1 = c.colour_ptr[col + 1];
        if (s1 <= s0) continue;
        launch_staged(k_eis_bwd_st<R, K, 0>, NT, c.seg.stage_up, s1 - s0, 1 << 20, c.stream, c.seg,
                      c.seg.work_col + s0, s1 - s0, c.D, c.B, (const cplx<R>*)v.x, (cplx<R>*)nullptr,
                      (const cplx<R>*)nullptr, (const cplx<R>*)nullptr, (const BicgState*)nullptr, out,
                      (double2*)nullptr);
        check_launch(c.launches);
    }
}

}  // namespace

#define M3D_DISPATCH_K(K_, CALL)                                    \
    switch (K_) {                                                   \
        case 2: CALL(2); break;                                     \
        case 4: CALL(4); break;                                     \
        case 8: CALL(8); break;                                     \
        case 16: CALL(16); break;                                   \
        default: throw std::runtime_error("batch size must be 2, 4, 8 or 16"); \
    }

template <class R>
void spmv(const KrylovCtx<R>& c, int mode, const cplx<R>* x, cplx<R>* y, const cplx<R>* aux,
          cplx<R>* aux_out, BicgState* st) {
#define CALL(K) spmv_k<R, K>(c, mode, x, y, aux, aux_out, st)
    M3D_DISPATCH_K(c.B.K, CALL)
#undef CALL
}

template <class R>
void ssor_apply(const KrylovCtx<R>& c, const cplx<R>* in, cplx<R>* y, cplx<R>* out) {
#define CALL(K) ssor_k<R, K>(c, in, y, out)
    M3D_DISPATCH_K(c.B.K, CALL)
#undef CALL
}

// out = B in: the SSOR apply plus, when the context carries it, the
// gradient-space term (V-cycle on the side stream, added by the backward
// sweep) -- the right preconditioner of one half iteration of iteration_k.
template <class R>
void precond_apply(const KrylovCtx<R>& c, const cplx<R>* in, cplx<R>* y, cplx<R>* out) {
#define CALL(K)                                  \
    {                                            \
        GcRowTerm gt;                            \
        if (c.gc) gt = gc_row_term(*c.gc, c.B);  \
        gc_term<R, K>(c, in);                    \
        ssor_k<R, K>(c, in, y, out, gt);         \
    }
    M3D_DISPATCH_K(c.B.K, CALL)
#undef CALL
}

template <class R>
void bicg_init(const KrylovCtx<R>& c, const KrylovVecs<R>& v, BicgState* st) {
    spmv(c, kSpmvInit, v.x, v.r, v.b, v.r0, st);
}

template <class R>
void bicg_iteration(const KrylovCtx<R>& c, const KrylovVecs<R>& v, BicgState* st) {
#define CALL(K) iteration_k<R, K>(c, v, st)
    M3D_DISPATCH_K(c.B.K, CALL)
#undef CALL
}

template <class R>
void eis_init(const KrylovCtx<R>& c, const KrylovVecs<R>& v, BicgState* st) {
    if (c.row_kernels != kRowsStaged) throw std::logic_error("Eisenstat form needs the staged row kernels");
#define CALL(K) eis_init_k<R, K>(c, v, st)
    M3D_DISPATCH_K(c.B.K, CALL)
#undef CALL
}

template <class R>
void eis_iteration(const KrylovCtx<R>& c, const KrylovVecs<R>& v, BicgState* st) {
#define CALL(K) eis_iteration_k<R, K>(c, v, st)
    M3D_DISPATCH_K(c.B.K, CALL)
#undef CALL
}

template <class R>
void eis_finish(const KrylovCtx<R>& c, const KrylovVecs<R>& v, cplx<R>* out) {
#define CALL(K) eis_finish_k<R, K>(c, v, out)
    M3D_DISPATCH_K(c.B.K, CALL)
#undef CALL
}

template void spmv<double>(const KrylovCtx<double>&, int, const double2*, double2*, const double2*, double2*, BicgState*);
template void spmv<float>(const KrylovCtx<float>&, int, const float2*, float2*, const float2*, float2*, BicgState*);
template void ssor_apply<double>(const KrylovCtx<double>&, const double2*, double2*, double2*);
template void ssor_apply<float>(const KrylovCtx<float>&, const float2*, float2*, float2*);
template void precond_apply<float>(const KrylovCtx<float>&, const float2*, float2*, float2*);
template void bicg_init<double>(const KrylovCtx<double>&, const KrylovVecs<double>&, BicgState*);
template void bicg_init<float>(const KrylovCtx<float>&, const KrylovVecs<float>&, BicgState*);
template void bicg_iteration<double>(const KrylovCtx<double>&, const KrylovVecs<double>&, BicgState*);
template void bicg_iteration<float>(const KrylovCtx<float>&, const KrylovVecs<float>&, BicgState*);

template void eis_init<float>(const KrylovCtx<float>&, const KrylovVecs<float>&, BicgState*);
template void eis_iteration<float>(const KrylovCtx<float>&, const KrylovVecs<float>&, BicgState*);
template void eis_finish<float>(const KrylovCtx<float>&, const KrylovVecs<float>&, float2*);

}  // namespace m3d
