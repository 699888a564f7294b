// GpuSolver: the learned preconditioner and the flexible GMRES inner solve
// that uses it.  No counterpart in the reference, whose inner solve is
// SSOR-BiCGStab (src/forward/bicgstab.cpp:15-166); the hook is the same place,
// the solve of one right-hand side batch inside solve_frequency
// (forward_solver_fv.cpp:266-285), and the judge of convergence stays the
// FP64 true residual of the mixed-precision refinement.
//
// Learned part:
//   * a dense grid of G^3 cells over the octree's unit cube (G = 2^level);
//     an edge field enters the network as per (cell, direction) means of its
//     values, scaled to unit RMS per right-hand side, plus a conductivity
//     channel and a frequency channel; the network's 6 output channels (the
//     error's real and imaginary parts per direction) are prolonged back to
//     the edges piecewise constant;
//   * training pairs come from the plain FP64 SSOR-BiCGStab solve itself:
//     at every host poll of a forward solve the iterate x_k and the residual
//     r_k = b - A x_k of each running right-hand side are recorded on the
//     grid; once the solve has converged, the target of snapshot k is the
//     error x* - x_k on the grid, normalised to unit RMS (FGMRES only needs
//     its direction);
//   * the network (learned.cu, BF16 tcgen05 kernels) is trained with Adam on
//     the GPU;
//   * FGMRES takes every learned_period-th direction from the network
//     (z = P N(R v)) and the others from the SSOR / gradient-space
//     preconditioner; the least-squares step weighs them, so a poor network
//     costs an iteration, not convergence.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstring>
#include <numeric>
#include <random>
#include <stdexcept>

#include "solver.hpp"
#include "cuda/learned.cuh"

namespace m3d {

using namespace dev;

namespace {

constexpr double kPi = 3.14159265358979323846;

void lck(cudaError_t e, const char* what) {
    if (e != cudaSuccess) {
        cudaGetLastError();
        throw std::runtime_error(std::string("learned: ") + what + ": " + cudaGetErrorString(e));
    }
}

template <class T>
T* lalloc(size_t n) {
    void* p = nullptr;
    if (cudaMalloc(&p, (n ? n : 1) * sizeof(T)) != cudaSuccess) {
        cudaGetLastError();
        throw std::bad_alloc();
    }
    return static_cast<T*>(p);
}

template <class T>
T* lupload(const std::vector<T>& h, cudaStream_t s) {
    T* p = lalloc<T>(h.size());
    if (!h.empty()) lck(cudaMemcpyAsync(p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s), "upload");
    return p;
}

template <class T>
void lfree(T*& p) {
    if (p) cudaFree(p);
    p = nullptr;
}

// ---- FGMRES vector kernels ([n_pad][K] complex FP32, lane k = i % K) ----

// b32[i] = y64[i] / scale[k] (0 where scale is 0)
__global__ void k_fg_to32(const double2* __restrict__ y, float2* __restrict__ b, int K, const double* __restrict__ scale,
                          long n) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double s = scale[i % K];
    const double2 w = y[i];
    b[i] = s > 0.0 ? make_float2((float)(w.x / s), (float)(w.y / s)) : make_float2(0.f, 0.f);
}

// x64[i] += d32[i] * scale[k]
__global__ void k_fg_add64(double2* __restrict__ x, const float2* __restrict__ d, int K,
                           const double* __restrict__ scale, long n) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double s = scale[i % K];
    if (s == 0.0) return;
    const float2 v = d[i];
    double2 xv = x[i];
    xv.x += (double)v.x * s;
    xv.y += (double)v.y * s;
    x[i] = xv;
}

// part[q][block][k] = sum over this block's elements of conj(V_q) w, q < nv
// (V_q at V + q * ld), and for q = nv (with_self) of conj(w) w.  Each thread
// sums its strided elements (about n / 262144, all of one lane) in FP32, the
// precision of the vectors, and the block reduces the threads' sums in FP64
// in a fixed tree: FP64 arithmetic runs at a small fraction of FP32 on this
// GPU and would bound the pass otherwise.
constexpr int kFgMaxV = 48;
__global__ void __launch_bounds__(256) k_fg_mdot(const float2* __restrict__ V, long ld, int nv, int with_self,
                                                 const float2* __restrict__ w, int K, long n,
                                                 double2* __restrict__ part) {
    __shared__ double2 sh[256];
    const int nb = gridDim.x;
    for (int q = 0; q < nv + with_self; ++q) {
        float2 acc = make_float2(0.0f, 0.0f);
        const float2* vq = q < nv ? V + (size_t)q * ld : w;
        for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)nb * blockDim.x) {
            const float2 a = vq[i], b = w[i];
            acc.x += a.x * b.x + a.y * b.y;
            acc.y += a.x * b.y - a.y * b.x;
        }
        sh[threadIdx.x] = make_double2((double)acc.x, (double)acc.y);
        __syncthreads();
        // threads t and t + s hold the same lane when K divides s
        for (int s = 128; s >= K; s >>= 1) {
            if (threadIdx.x < s) {
                sh[threadIdx.x].x += sh[threadIdx.x + s].x;
                sh[threadIdx.x].y += sh[threadIdx.x + s].y;
            }
            __syncthreads();
        }
        if (threadIdx.x < K) part[((size_t)q * nb + blockIdx.x) * K + threadIdx.x] = sh[threadIdx.x];
        __syncthreads();
    }
}

__global__ void k_fg_mdot_final(const double2* __restrict__ part, int nv, int nb, int K, double2* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv * K) return;
    const int q = i / K, k = i % K;
    double2 s = make_double2(0.0, 0.0);
    for (int b = 0; b < nb; ++b) {
        const double2 p = part[((size_t)q * nb + b) * K + k];
        s.x += p.x;
        s.y += p.y;
    }
    out[i] = s;
}

// w[i] += sign * sum_q c[q][k] V_q[i]
__global__ void k_fg_maxpy(const float2* __restrict__ V, long ld, int nv, const double2* __restrict__ c, int K,
                           long n, float2* __restrict__ w, float sign) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int k = (int)(i % K);
    float2 acc = w[i];
    for (int q = 0; q < nv; ++q) {
        const double2 cq = c[(size_t)q * K + k];
        const float2 v = V[(size_t)q * ld + i];
        const float cr = (float)cq.x * sign, ci = (float)cq.y * sign;
        acc.x += cr * v.x - ci * v.y;
        acc.y += cr * v.y + ci * v.x;
    }
    w[i] = acc;
}

// v[i] = w[i] * inv[k]
__global__ void k_fg_scale(const float2* __restrict__ w, float2* __restrict__ v, const double* __restrict__ inv, int K,
                           long n) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float s = (float)inv[i % K];
    const float2 a = w[i];
    v[i] = make_float2(a.x * s, a.y * s);
}

// ---- dataset kernels ----

// ds_feat[slot[j]][c][0..8) = in[lane[j]][c][0..8)
__global__ void k_pack_feat(const __nv_bfloat16* __restrict__ in, int n_cells, const int* __restrict__ lane,
                            const long* __restrict__ slot, int nj, __nv_bfloat16* __restrict__ ds) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)nj * n_cells) return;
    const int j = (int)(i / n_cells), c = (int)(i % n_cells);
    const __nv_bfloat16* s = in + ((size_t)lane[j] * n_cells + c) * learn::kCh;
    __nv_bfloat16* d = ds + ((size_t)slot[j] * n_cells + c) * learn::kInCh;
    *reinterpret_cast<uint4*>(d) = *reinterpret_cast<const uint4*>(s);
}

// ds_tgt[slot[j]] = means[lane[j]]  (FP32 [n_cells][6])
__global__ void k_pack_tgt(const float* __restrict__ m, int n_cells, const int* __restrict__ lane,
                           const long* __restrict__ slot, int nj, float* __restrict__ ds) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long per = (long long)n_cells * learn::kOutCh;
    if (i >= (long long)nj * per) return;
    const int j = (int)(i / per);
    const long long r = i % per;
    ds[(size_t)slot[j] * per + r] = m[(size_t)lane[j] * per + r];
}

// target of snapshot j: (means(x*) of its lane - stored means(x_k)) / RMS;
// one block per snapshot
__global__ void k_finish_tgt(const float* __restrict__ m, int n_cells, const int* __restrict__ lane,
                             const long* __restrict__ slot, float* __restrict__ ds) {
    __shared__ double sh[256];
    const int j = blockIdx.x;
    const long long per = (long long)n_cells * learn::kOutCh;
    float* t = ds + (size_t)slot[j] * per;
    const float* a = m + (size_t)lane[j] * per;
    double acc = 0.0;
    for (long long r = threadIdx.x; r < per; r += blockDim.x) {
        const float e = a[r] - t[r];
        t[r] = e;
        acc += (double)e * e;
    }
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    const double rms = sqrt(sh[0] / (double)per);
    const float inv = rms > 0.0 ? (float)(1.0 / rms) : 0.0f;
    for (long long r = threadIdx.x; r < per; r += blockDim.x) t[r] *= inv;
}

// network input [n][c][32] from samples idx[j] of ds_feat ([.][c][8])
__global__ void k_unpack_feat(const __nv_bfloat16* __restrict__ ds, const long* __restrict__ idx, int nj, int n_cells,
                              __nv_bfloat16* __restrict__ in) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)nj * n_cells) return;
    const int j = (int)(i / n_cells), c = (int)(i % n_cells);
    const uint4 v = *reinterpret_cast<const uint4*>(ds + ((size_t)idx[j] * n_cells + c) * learn::kInCh);
    uint4* o = reinterpret_cast<uint4*>(in + ((size_t)j * n_cells + c) * learn::kCh);
    o[0] = v;
    o[1] = make_uint4(0, 0, 0, 0);
    o[2] = make_uint4(0, 0, 0, 0);
    o[3] = make_uint4(0, 0, 0, 0);
}

__global__ void k_unpack_tgt(const float* __restrict__ ds, const long* __restrict__ idx, int nj, int n_cells,
                             float* __restrict__ t) {
    const long long per = (long long)n_cells * learn::kOutCh;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)nj * per) return;
    const int j = (int)(i / per);
    t[i] = ds[(size_t)idx[j] * per + i % per];
}

inline unsigned blocks(long long n) { return (unsigned)((n + 255) / 256); }

}  // namespace

// ---------------------------------------------------------------------------
// set-up: dense grid of the mesh, network, dataset
// ---------------------------------------------------------------------------

void GpuSolver::learn_free() {
    lfree(gm.cd_ptr); lfree(gm.cd_row); lfree(gm.row_cell); lfree(gm.row_dir);
    lfree(gm.sig_ptr); lfree(gm.sig_leaf); lfree(gm.sig_feat);
    lfree(ds_feat); lfree(ds_tgt); lfree(lw_work); lfree(d_lane_freq); lfree(d_snap_lane); lfree(d_snap_slot);
    lfree(fg_V); lfree(fg_Z); lfree(fg_w); lfree(fg_part); lfree(fg_h); lfree(fg_inv); lfree(fg_scale);
    lfree(tr_target);
    fg_cap_K = 0; fg_cap_m = 0;
    net.reset();
    gm = learn::GridMap{};
    ds_n = ds_cap = 0;
    net_trained = false;
}

void GpuSolver::learn_setup(int grid_level, int layers, int hidden, unsigned seed, long max_samples) {
    if (!ready) throw std::logic_error("solver not set up");
    if (grid_level < 4 || grid_level > 7) throw std::invalid_argument("grid level must be 4 .. 7");
    if (max_samples < 1) throw std::invalid_argument("max_samples must be >= 1");
    learn_free();
    const int G = 1 << grid_level;
    const int nc = G * G * G;
    const double* dm = L.domain;
    const double ext[3] = {dm[1] - dm[0], dm[3] - dm[2], dm[5] - dm[4]};
    auto cell_of = [&](double x, double y, double z) {
        int ix = (int)std::floor((x - dm[0]) / ext[0] * G);
        int iy = (int)std::floor((y - dm[2]) / ext[1] * G);
        int iz = (int)std::floor((z - dm[4]) / ext[2] * G);
        ix = std::min(std::max(ix, 0), G - 1);
        iy = std::min(std::max(iy, 0), G - 1);
        iz = std::min(std::max(iz, 0), G - 1);
        return (iz * G + iy) * G + ix;
    };
    // rows of every (cell, direction): free edges only (identity rows keep 0)
    std::vector<int> cnt(3 * (size_t)nc + 1, 0), row_cell(n_pad, -1);
    std::vector<signed char> row_dir(n_pad, 0);
    for (int e = 0; e < L.ne; ++e) {
        if (flags_ref[e] & kFlagConstrained) continue;
        const int c = cell_of(L.ex[e], L.ey[e], L.ez[e]);
        const int row = iperm[e];
        row_cell[row] = c;
        row_dir[row] = (signed char)L.edir[e];
        ++cnt[3 * (size_t)c + L.edir[e] + 1];
    }
    for (size_t i = 1; i < cnt.size(); ++i) cnt[i] += cnt[i - 1];
    std::vector<int> cd_row(cnt.back()), fill(cnt.begin(), cnt.end() - 1);
    for (int e = 0; e < L.ne; ++e) {
        if (flags_ref[e] & kFlagConstrained) continue;
        const int c = cell_of(L.ex[e], L.ey[e], L.ez[e]);
        cd_row[fill[3 * (size_t)c + L.edir[e]]++] = iperm[e];
    }
    // leaves of every cell: a leaf at or below the grid level lies in one
    // cell, a coarser leaf covers a block of cells
    std::vector<std::vector<int>> lists(nc);
    for (int c = 0; c < L.nc; ++c) {
        const int lv = L.clevel[c];
        if (lv >= grid_level) {
            lists[cell_of(L.ccx[c], L.ccy[c], L.ccz[c])].push_back(c);
        } else {
            const int span = 1 << (grid_level - lv);
            const double h[3] = {ext[0] / (1 << lv), ext[1] / (1 << lv), ext[2] / (1 << lv)};
            const int c0 = cell_of(L.ccx[c] - 0.5 * h[0] + 1e-9 * ext[0], L.ccy[c] - 0.5 * h[1] + 1e-9 * ext[1],
                                   L.ccz[c] - 0.5 * h[2] + 1e-9 * ext[2]);
            const int x0 = c0 % G, y0 = (c0 / G) % G, z0 = c0 / (G * G);
            for (int dz = 0; dz < span; ++dz)
                for (int dy = 0; dy < span; ++dy)
                    for (int dx = 0; dx < span; ++dx) {
                        const int x = x0 + dx, y = y0 + dy, z = z0 + dz;
                        if (x < G && y < G && z < G) lists[(z * G + y) * G + x].push_back(c);
                    }
        }
    }
    std::vector<int> sig_ptr(nc + 1, 0), sig_leaf;
    for (int c = 0; c < nc; ++c) {
        sig_leaf.insert(sig_leaf.end(), lists[c].begin(), lists[c].end());
        sig_ptr[c + 1] = (int)sig_leaf.size();
    }
    gm.G = G;
    gm.n_cells = nc;
    gm.n_pad = n_pad;
    gm.cd_ptr = lupload(cnt, stream);
    gm.cd_row = lupload(cd_row, stream);
    gm.row_cell = lupload(row_cell, stream);
    gm.row_dir = lupload(row_dir, stream);
    gm.sig_ptr = lupload(sig_ptr, stream);
    gm.sig_leaf = lupload(sig_leaf, stream);
    gm.sig_feat = lalloc<float>(nc);
    learn_level = grid_level;
    net.reset(new learn::Cnn(device, layers, learn::kInCh, hidden, learn::kOutCh, seed));
    net->set_stream(stream);
    net->ensure(kMaxRhs, G, G, G);
    ds_cap = max_samples;
    ds_feat = lalloc<__nv_bfloat16>((size_t)ds_cap * nc * learn::kInCh);
    ds_tgt = lalloc<float>((size_t)ds_cap * nc * learn::kOutCh);
    lw_work = lalloc<float>((size_t)kMaxRhs * nc * learn::kOutCh + kMaxRhs);
    d_lane_freq = lalloc<double>(kMaxRhs);
    d_snap_lane = lalloc<int>(kMaxRhs);
    d_snap_slot = lalloc<long>(kMaxRhs);
    ds_n = 0;
    if (have_sigma) learn::grid_sigma_feature(gm, d_sigma, stream);
    sync();
}

// the conductivity channel follows every set_sigma
void GpuSolver::learn_sigma_changed() {
    if (gm.sig_feat) learn::grid_sigma_feature(gm, d_sigma, stream);
}

// ---------------------------------------------------------------------------
// training pairs from the plain FP64 solve
// ---------------------------------------------------------------------------

// Called by solve_batch at every host poll while collecting: records the
// grid view of r_k (network input) and of x_k for each running lane.
void GpuSolver::collect_snapshot(const double2* x, const double2* r, int K, const std::vector<BicgState>& hs,
                                 const int* fmap) {
    std::vector<int> lanes;
    for (int k = 0; k < K; ++k)
        if (hs[k].status == kRunning && hs[k].iter > 0 && ds_n + (long)lanes.size() < ds_cap) lanes.push_back(k);
    if (lanes.empty()) return;
    std::vector<double> fq(kMaxRhs, 0.0);
    for (int k = 0; k < K; ++k) fq[k] = fz_freqs[fmap[k]];
    lck(cudaMemcpyAsync(d_lane_freq, fq.data(), sizeof(double) * kMaxRhs, cudaMemcpyHostToDevice, stream), "freq");
    std::vector<long> slots(lanes.size());
    for (size_t j = 0; j < lanes.size(); ++j) slots[j] = ds_n + (long)j;
    lck(cudaMemcpyAsync(d_snap_lane, lanes.data(), sizeof(int) * lanes.size(), cudaMemcpyHostToDevice, stream), "lane");
    lck(cudaMemcpyAsync(d_snap_slot, slots.data(), sizeof(long) * slots.size(), cudaMemcpyHostToDevice, stream),
        "slot");
    const int nj = (int)lanes.size();
    learn::grid_features(gm, r, K, d_lane_freq, net->input(), lw_work, stream);
    k_pack_feat<<<blocks((long long)nj * gm.n_cells), 256, 0, stream>>>(net->input(), gm.n_cells, d_snap_lane,
                                                                       d_snap_slot, nj, ds_feat);
    learn::grid_means(gm, x, K, lw_work, stream);
    k_pack_tgt<<<blocks((long long)nj * gm.n_cells * learn::kOutCh), 256, 0, stream>>>(
        lw_work, gm.n_cells, d_snap_lane, d_snap_slot, nj, ds_tgt);
    lck(cudaGetLastError(), "snapshot");
    sync();   // the lane and slot lists are reused by the next poll
    for (size_t j = 0; j < lanes.size(); ++j) pending.push_back({lanes[j], ds_n + (long)j});
    ds_n += nj;
}

// After the solve: target of every pending snapshot = grid(x*) - grid(x_k),
// normalised to unit RMS.
void GpuSolver::collect_finish(const double2* x, int K) {
    if (pending.empty()) return;
    learn::grid_means(gm, x, K, lw_work, stream);
    for (size_t j0 = 0; j0 < pending.size(); j0 += kMaxRhs) {
        const int nj = (int)std::min<size_t>(kMaxRhs, pending.size() - j0);
        std::vector<int> lanes(nj);
        std::vector<long> slots(nj);
        for (int j = 0; j < nj; ++j) { lanes[j] = pending[j0 + j].lane; slots[j] = pending[j0 + j].slot; }
        lck(cudaMemcpyAsync(d_snap_lane, lanes.data(), sizeof(int) * nj, cudaMemcpyHostToDevice, stream), "lane");
        lck(cudaMemcpyAsync(d_snap_slot, slots.data(), sizeof(long) * nj, cudaMemcpyHostToDevice, stream), "slot");
        k_finish_tgt<<<nj, 256, 0, stream>>>(lw_work, gm.n_cells, d_snap_lane, d_snap_slot, ds_tgt);
        lck(cudaGetLastError(), "finish");
        sync();
    }
    pending.clear();
}

long GpuSolver::learn_collect(const double* freqs, int nf) {
    if (!net) throw std::logic_error("learned preconditioner not set up (m3d_learn_setup)");
    const m3d_params saved = P;
    P.precision = 0;           // the plain FP64 SSOR-BiCGStab
    P.forward_interleaved = 0;
    P.div_correction = 0;      // the divergence correction is not part of the Krylov solve
    collecting = true;
    try {
        for (int f0 = 0; f0 < nf; f0 += 8) {
            const int g = std::min(8, nf - f0);
            run_forward(std::vector<double>(freqs + f0, freqs + f0 + g), nullptr);
        }
    } catch (...) {
        collecting = false;
        pending.clear();
        P = saved;
        throw;
    }
    collecting = false;
    P = saved;
    return ds_n;
}

// ---------------------------------------------------------------------------
// training
// ---------------------------------------------------------------------------

std::vector<double> GpuSolver::learn_train(int epochs, float lr, int batch, unsigned seed, double val_frac,
                                           double* val_loss) {
    if (!net) throw std::logic_error("learned preconditioner not set up (m3d_learn_setup)");
    if (ds_n < 2) throw std::logic_error("no training pairs collected (m3d_learn_collect)");
    batch = std::max(1, std::min(batch, kMaxRhs));
    const long n_val = std::min<long>(ds_n - 1, std::max<long>(0, (long)std::floor(val_frac * ds_n)));
    const long n_tr = ds_n - n_val;
    if (!tr_target) tr_target = lalloc<float>((size_t)kMaxRhs * gm.n_cells * learn::kOutCh);
    long* d_idx = lalloc<long>(kMaxRhs);
    std::vector<long> order(n_tr);
    std::iota(order.begin(), order.end(), 0L);
    std::mt19937 rng(seed);
    std::vector<double> hist;
    auto run_batch = [&](const long* idx, int nj, bool step) {
        lck(cudaMemcpyAsync(d_idx, idx, sizeof(long) * nj, cudaMemcpyHostToDevice, stream), "idx");
        k_unpack_feat<<<blocks((long long)nj * gm.n_cells), 256, 0, stream>>>(ds_feat, d_idx, nj, gm.n_cells,
                                                                             net->input());
        k_unpack_tgt<<<blocks((long long)nj * gm.n_cells * learn::kOutCh), 256, 0, stream>>>(ds_tgt, d_idx, nj,
                                                                                            gm.n_cells, tr_target);
        lck(cudaGetLastError(), "batch");
        net->forward(nj);
        const double l = net->loss_backward(nj, tr_target);
        if (step) net->adam_step(lr);
        return l;
    };
    try {
        for (int ep = 0; ep < epochs; ++ep) {
            std::shuffle(order.begin(), order.end(), rng);
            double sum = 0.0;
            long nb = 0;
            for (long b0 = 0; b0 + batch <= n_tr; b0 += batch) {
                sum += run_batch(order.data() + b0, batch, true);
                ++nb;
            }
            hist.push_back(nb ? sum / nb : 0.0);
        }
        if (val_loss) {
            double sum = 0.0;
            long nb = 0;
            std::vector<long> vi;
            for (long i = n_tr; i < ds_n; ++i) vi.push_back(i);
            for (size_t b0 = 0; b0 < vi.size(); b0 += batch) {
                const int nj = (int)std::min<size_t>(batch, vi.size() - b0);
                sum += run_batch(vi.data() + b0, nj, false) * nj;
                nb += nj;
            }
            *val_loss = nb ? sum / nb : 0.0;
        }
    } catch (...) {
        cudaFree(d_idx);
        throw;
    }
    cudaFree(d_idx);
    if (net->error_flag()) throw std::runtime_error("learned: a tensor-core kernel's barrier wait timed out");
    net_trained = true;
    return hist;
}

// The learned direction for K lanes (FP32): the network's coarse correction
// c = P N(R v), scaled per lane by the alpha minimising |v - alpha A c|, then
// one application of the SSOR / gradient-space preconditioner B to what is
// left: z = alpha c + B (v - alpha A c) -- a two-level step whose coarse
// solve is the network.
void GpuSolver::net_apply(const KrylovCtx<float>& c32, const float2* v, float2* z, int K, const int* fmap) {
    std::vector<double> fq(kMaxRhs, 0.0);
    for (int k = 0; k < K; ++k) fq[k] = fz_freqs[fmap[k]];
    lck(cudaMemcpyAsync(d_lane_freq, fq.data(), sizeof(double) * kMaxRhs, cudaMemcpyHostToDevice, stream), "freq");
    learn::grid_features(gm, v, K, d_lane_freq, net->input(), lw_work, stream);
    const float* out = net->forward(K);
    float2* cvec = kv32.t;
    float2* acv = kv32.v;
    float2* rest = kv32.s;
    learn::grid_prolong(gm, out, K, cvec, stream);
    spmv(c32, kSpmvPlain, cvec, acv, nullptr, nullptr, nullptr);
    launches += 3 + 2 * (long long)net->layers();
    std::vector<std::complex<double>> d1, d2;
    fg_mdot(acv, 1, v, K, d1);      // (Ac, v)
    fg_mdot(acv, 1, acv, K, d2);    // (Ac, Ac)
    std::vector<double2> alpha(kMaxRhs, make_double2(0.0, 0.0));
    for (int k = 0; k < K; ++k) {
        const double den = d2[k].real();
        const std::complex<double> a = den > 0.0 ? d1[k] / den : std::complex<double>(0.0);
        alpha[k] = make_double2(a.real(), a.imag());
    }
    const long n = (long)n_pad * K;
    lck(cudaMemcpyAsync(fg_h, alpha.data(), sizeof(double2) * kMaxRhs, cudaMemcpyHostToDevice, stream), "alpha");
    lck(cudaMemcpyAsync(rest, v, sizeof(float2) * n, cudaMemcpyDeviceToDevice, stream), "copy");
    k_fg_maxpy<<<blocks(n), 256, 0, stream>>>(acv, n, 1, fg_h, K, n, rest, -1.0f);
    precond_apply(c32, rest, kv32.y, z);
    k_fg_maxpy<<<blocks(n), 256, 0, stream>>>(cvec, n, 1, fg_h, K, n, z, 1.0f);
    lck(cudaGetLastError(), "learned direction");
    launches += 2;
}

// ---------------------------------------------------------------------------
// flexible GMRES inner solve inside the FP64 refinement
// ---------------------------------------------------------------------------

void GpuSolver::ensure_fgmres(int K, int m) {
    if (fg_cap_K >= K && fg_cap_m >= m) return;
    lfree(fg_V); lfree(fg_Z); lfree(fg_w); lfree(fg_part); lfree(fg_h); lfree(fg_inv); lfree(fg_scale);
    const size_t n = (size_t)n_pad * K;
    fg_V = lalloc<float2>(n * (m + 1));
    fg_Z = lalloc<float2>(n * m);
    fg_w = lalloc<float2>(n);
    fg_part = lalloc<double2>((size_t)1024 * kFgMaxV * kMaxRhs);
    fg_h = lalloc<double2>((size_t)kFgMaxV * kMaxRhs);
    fg_inv = lalloc<double>(kMaxRhs);
    fg_scale = lalloc<double>(kMaxRhs);
    fg_cap_K = K;
    fg_cap_m = m;
}

// h[q][k] = (V_q, w)_k for q < nv, and (w, w)_k as q = nv when with_self,
// into host h (the first nv also left in fg_h)
void GpuSolver::fg_mdot(const float2* V, int nv, const float2* w, int K, std::vector<std::complex<double>>& h,
                        bool with_self) {
    const long n = (long)n_pad * K;
    const int nb = (int)std::min<long>(1024, (n + 255) / 256);
    const int nq = nv + (with_self ? 1 : 0);
    k_fg_mdot<<<nb, 256, 0, stream>>>(V, n, nv, with_self ? 1 : 0, w, K, n, fg_part);
    k_fg_mdot_final<<<(nq * K + 255) / 256, 256, 0, stream>>>(fg_part, nq, nb, K, fg_h);
    lck(cudaGetLastError(), "mdot");
    launches += 2;
    std::vector<double2> t((size_t)nq * K);
    lck(cudaMemcpyAsync(t.data(), fg_h, sizeof(double2) * t.size(), cudaMemcpyDeviceToHost, stream), "h");
    sync();
    h.resize(t.size());
    for (size_t i = 0; i < t.size(); ++i) h[i] = {t[i].x, t[i].y};
}

BatchResult GpuSolver::solve_batch_fgmres(int K, const int* fmap, double2* b, double2* x,
                                          const std::vector<int>& active, double tol, int maxiter) {
    using cd = std::complex<double>;
    const int m = std::max(2, std::min(P.fgmres_m > 0 ? P.fgmres_m : 20, kFgMaxV - 1));
    ensure_vecs(K);
    ensure_vecs32(K);
    ensure_fgmres(K, m);
    const KrylovCtx<double> c64 = kctx(K, fmap);
    KrylovCtx<float> c32 = kctx32(K, fmap);
    bool use_gc = false;
    if (gc_ok && P.gradcorr == 1 && gc.omega_max > 0.0)
        for (int k = 0; k < K; ++k)
            if (active[k]) {
                const double om = 2.0 * kPi * fz_freqs[fmap[k]];
                use_gc |= om > 0.0 && om <= gc.omega_max;
            }
    if (use_gc) attach_gc(c32);
    const bool learned = P.learned_period > 0 && net && net_trained;
    const long n = (long)n_pad * K;
    const long ld = n;
    BatchResult R;
    R.K = K;
    R.iters.assign(K, 0); R.status.assign(K, kInactive); R.res.assign(K, 0.0); R.true_res.assign(K, 0.0);
    std::vector<int> run = active;
    std::vector<double> prev(K, 1e300);
    std::vector<BicgState> hs(K);
    const int max_steps = 2 + std::max(0, P.max_refinements) * 4;
    for (int step = 0; step <= max_steps; ++step) {
        for (int k = 0; k < K; ++k) {
            std::memset(&hs[k], 0, sizeof(BicgState));
            hs[k].status = active[k] ? kConverged : kInactive;
        }
        lck(cudaMemcpyAsync(d_states, hs.data(), sizeof(BicgState) * K, cudaMemcpyHostToDevice, stream), "states");
        spmv(c64, kSpmvTrueRes, x, kv.y, b, nullptr, d_states);
        lck(cudaMemcpyAsync(hs.data(), d_states, sizeof(BicgState) * K, cudaMemcpyDeviceToHost, stream), "states");
        sync();
        std::vector<int> lane_on(K, 0);
        std::vector<double> scale(kMaxRhs, 0.0), itol(K, 0.0);
        bool any = false;
        for (int k = 0; k < K; ++k) {
            if (!active[k]) continue;
            const double rel = hs[k].true_res;
            R.true_res[k] = rel;
            R.res[k] = rel;
            if (!run[k]) continue;
            if (rel <= tol) { run[k] = 0; R.status[k] = kConverged; continue; }
            if (!std::isfinite(rel)) { run[k] = 0; R.status[k] = kBreakdown; continue; }
            if (rel > 0.9 * prev[k] || R.iters[k] >= maxiter || step == max_steps) {
                run[k] = 0;
                if (R.status[k] == kInactive || R.status[k] == kConverged) R.status[k] = kMaxIter;
                continue;
            }
            prev[k] = rel;
            scale[k] = hs[k].rnorm;
            itol[k] = std::min(0.5, std::max(tol / rel, P.inner_tol_floor));
            lane_on[k] = 1;
            any = true;
        }
        if (!any) break;
        // v_0 = r / |r| per lane (FP32), beta = |v_0|
        lck(cudaMemcpyAsync(fg_scale, scale.data(), sizeof(double) * kMaxRhs, cudaMemcpyHostToDevice, stream), "scale");
        k_fg_to32<<<blocks(n), 256, 0, stream>>>(kv.y, fg_V, K, fg_scale, n);
        launches += 1;
        std::vector<cd> hv;
        fg_mdot(fg_V, 1, fg_V, K, hv);
        std::vector<double> beta(K, 0.0), inv(kMaxRhs, 0.0);
        for (int k = 0; k < K; ++k) {
            beta[k] = lane_on[k] ? std::sqrt(std::max(0.0, hv[k].real())) : 0.0;
            inv[k] = beta[k] > 0.0 ? 1.0 / beta[k] : 0.0;
            if (beta[k] == 0.0) lane_on[k] = 0;
        }
        lck(cudaMemcpyAsync(fg_inv, inv.data(), sizeof(double) * kMaxRhs, cudaMemcpyHostToDevice, stream), "inv");
        k_fg_scale<<<blocks(n), 256, 0, stream>>>(fg_V, fg_V, fg_inv, K, n);
        // Arnoldi with per-lane Givens rotations (host, FP64)
        std::vector<std::vector<cd>> H(K, std::vector<cd>((size_t)(m + 1) * m, cd(0.0)));
        std::vector<std::vector<cd>> cs(K, std::vector<cd>(m)), sn(K, std::vector<cd>(m));
        std::vector<std::vector<cd>> g(K, std::vector<cd>(m + 1, cd(0.0)));
        std::vector<int> steps(K, 0), live = lane_on;
        for (int k = 0; k < K; ++k) g[k][0] = beta[k];
        int j = 0;
        for (; j < m; ++j) {
            bool any_live = false;
            for (int k = 0; k < K; ++k) any_live |= live[k] != 0;
            if (!any_live) break;
            const float2* vj = fg_V + (size_t)j * ld;
            float2* zj = fg_Z + (size_t)j * ld;
            if (learned && (j % P.learned_period) == P.learned_period - 1) net_apply(c32, vj, zj, K, fmap);
            else precond_apply(c32, vj, kv32.y, zj);
            spmv(c32, kSpmvPlain, zj, fg_w, nullptr, nullptr, nullptr);
            // classical Gram-Schmidt with the norm of w in the same reduction:
            // |w - V h|^2 = |w|^2 - |h|^2 (V orthonormal); a second pass only
            // where that cancels below half of |w|^2 (DGKS criterion)
            std::vector<cd> h1, h2;
            fg_mdot(fg_V, j + 1, fg_w, K, h1, true);
            k_fg_maxpy<<<blocks(n), 256, 0, stream>>>(fg_V, ld, j + 1, fg_h, K, n, fg_w, -1.0f);
            launches += 3;
            std::vector<double> nrm2(K, 0.0);
            bool again = false;
            for (int k = 0; k < K; ++k) {
                if (!live[k]) continue;
                double hh = 0.0;
                for (int q = 0; q <= j; ++q) hh += std::norm(h1[(size_t)q * K + k]);
                const double ww = h1[(size_t)(j + 1) * K + k].real();
                nrm2[k] = ww - hh;
                again |= nrm2[k] < 0.5 * ww;
            }
            if (again) {
                fg_mdot(fg_V, j + 1, fg_w, K, h2, true);
                k_fg_maxpy<<<blocks(n), 256, 0, stream>>>(fg_V, ld, j + 1, fg_h, K, n, fg_w, -1.0f);
                launches += 3;
                for (int k = 0; k < K; ++k) {
                    if (!live[k]) continue;
                    double hh = 0.0;
                    for (int q = 0; q <= j; ++q) hh += std::norm(h2[(size_t)q * K + k]);
                    nrm2[k] = h2[(size_t)(j + 1) * K + k].real() - hh;
                }
            }
            for (int k = 0; k < K; ++k) {
                inv[k] = 0.0;
                if (!live[k]) continue;
                std::vector<cd>& Hk = H[k];
                for (int q = 0; q <= j; ++q)
                    Hk[(size_t)q * m + j] = h1[(size_t)q * K + k] + (again ? h2[(size_t)q * K + k] : cd(0.0));
                const double hn = std::sqrt(std::max(0.0, nrm2[k]));
                Hk[(size_t)(j + 1) * m + j] = hn;
                inv[k] = hn > 1e-30 * beta[k] ? 1.0 / hn : 0.0;
                // previous rotations on column j
                for (int q = 0; q < j; ++q) {
                    const cd a = Hk[(size_t)q * m + j], bq = Hk[(size_t)(q + 1) * m + j];
                    Hk[(size_t)q * m + j] = std::conj(cs[k][q]) * a + std::conj(sn[k][q]) * bq;
                    Hk[(size_t)(q + 1) * m + j] = -sn[k][q] * a + cs[k][q] * bq;
                }
                const cd a = Hk[(size_t)j * m + j], bb = Hk[(size_t)(j + 1) * m + j];
                const double r = std::sqrt(std::norm(a) + std::norm(bb));
                if (r == 0.0) { cs[k][j] = 1.0; sn[k][j] = 0.0; }
                else { cs[k][j] = a / r; sn[k][j] = bb / r; }
                Hk[(size_t)j * m + j] = r;
                Hk[(size_t)(j + 1) * m + j] = 0.0;
                g[k][j + 1] = -sn[k][j] * g[k][j];
                g[k][j] = std::conj(cs[k][j]) * g[k][j];
                steps[k] = j + 1;
                const double res = std::abs(g[k][j + 1]) / beta[k];
                if (res <= itol[k] || inv[k] == 0.0 || R.iters[k] + steps[k] >= maxiter) live[k] = 0;
            }
            lck(cudaMemcpyAsync(fg_inv, inv.data(), sizeof(double) * kMaxRhs, cudaMemcpyHostToDevice, stream), "inv");
            k_fg_scale<<<blocks(n), 256, 0, stream>>>(fg_w, fg_V + (size_t)(j + 1) * ld, fg_inv, K, n);
            ++launches;
        }
        // y = H^-1 g per lane, d = Z y, x64 += scale * d
        const int ncols = std::max(1, j);
        std::vector<double2> y((size_t)ncols * K, make_double2(0.0, 0.0));
        for (int k = 0; k < K; ++k) {
            const int s = steps[k];
            std::vector<cd> yk(s);
            for (int q = s - 1; q >= 0; --q) {
                cd acc = g[k][q];
                for (int p = q + 1; p < s; ++p) acc -= H[k][(size_t)q * m + p] * yk[p];
                const cd d = H[k][(size_t)q * m + q];
                yk[q] = std::abs(d) > 0.0 ? acc / d : cd(0.0);
            }
            for (int q = 0; q < s; ++q) y[(size_t)q * K + k] = make_double2(yk[q].real(), yk[q].imag());
            R.iters[k] += s;
        }
        lck(cudaMemsetAsync(kv32.x, 0, sizeof(float2) * n, stream), "memset");
        lck(cudaMemcpyAsync(fg_h, y.data(), sizeof(double2) * y.size(), cudaMemcpyHostToDevice, stream), "y");
        k_fg_maxpy<<<blocks(n), 256, 0, stream>>>(fg_Z, ld, ncols, fg_h, K, n, kv32.x, 1.0f);
        k_fg_add64<<<blocks(n), 256, 0, stream>>>(x, kv32.x, K, fg_scale, n);
        launches += 2;
        lck(cudaGetLastError(), "fgmres");
        if (step > 0) ++stats.refinements;
    }
    check_seg_err();
    timer.collect();
    return R;
}

}  // namespace m3d
