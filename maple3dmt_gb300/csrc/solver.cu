// GpuSolver implementation: see solver.hpp.
#include "solver.hpp"

#include "cuda/dot.cuh"
#include "host/amg.hpp"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstring>
#include <stdexcept>

namespace m3d {

namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr double kMu0 = 4.0e-7 * kPi;

void cuda_ok(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

template <class T>
T* dalloc(size_t n) {
    T* p = nullptr;
    if (n == 0) n = 1;
    const cudaError_t e = cudaMalloc(&p, n * sizeof(T));
    if (e != cudaSuccess) throw std::bad_alloc();
    return p;
}

template <class T>
T* dupload(const std::vector<T>& v, cudaStream_t s) {
    T* p = dalloc<T>(v.size());
    if (!v.empty()) cuda_ok(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s), "upload");
    return p;
}

// Krylov work vectors start zeroed: staged row kernels read padding entries
// (value 0) on the row itself, and 0 * x must never meet uninitialised bits.
template <class T>
T* dalloc_zero(size_t n, cudaStream_t s) {
    T* p = dalloc<T>(n);
    cuda_ok(cudaMemsetAsync(p, 0, (n ? n : 1) * sizeof(T), s), "memset");
    return p;
}

template <class T>
void dfree(T*& p) {
    if (p) cudaFree(p);
    p = nullptr;
}

int pow2_at_least(int k) {
    int K = 2;
    while (K < k) K *= 2;
    return K;
}

__global__ void k_zero_col(double2* x, int K, int k, int n_pad) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < n_pad) x[(size_t)r * K + k] = make_double2(0.0, 0.0);
}

// b32 = y64 / scale[k] (scale 0: column left at zero)
__global__ void k_to_f32_scaled(const double2* __restrict__ y, float2* __restrict__ b,
                                const double* __restrict__ scale, int K, long n) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double s = scale[i % K];
    const double inv = s > 0.0 ? 1.0 / s : 0.0;
    const double2 v = y[i];
    b[i] = make_float2((float)(v.x * inv), (float)(v.y * inv));
}

// x64 += d32 * scale[k]
__global__ void k_add_f32_scaled(double2* __restrict__ x, const float2* __restrict__ d,
                                 const double* __restrict__ scale, int K, long n) {
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


// Residual replacement (reliable updating, van der Vorst and Ye 2000) of the
// inner solve: on lanes with rep[j] set, r32 = y64[map[j]] / scale[j] (the
// FP64 true residual of the accumulated FP64 solution, in the lane's
// scaling) and x32 = 0 (its correction having been added to x64); rho =
// (r0, r), beta and |r| are recomputed from the new residual so the
// BiCGStab recurrence continues without a restart.
template <int Kc>
__global__ void __launch_bounds__(256) k_replace_lanes(const double2* __restrict__ y, int K, float2* __restrict__ r,
                                                       float2* __restrict__ x, const float2* __restrict__ r0,
                                                       const int* __restrict__ map, const int* __restrict__ rep,
                                                       const double* __restrict__ scale, long n_rows, BicgState* st,
                                                       dev::RedScratch rs) {
    const long n = n_rows * Kc;
    const long i0 = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const long stride = (long)gridDim.x * blockDim.x;
    const int j = (int)(i0 % Kc), m = map[j];
    const bool on = m >= 0 && rep[j] && scale[j] > 0.0;
    const double inv = on ? 1.0 / scale[j] : 0.0;
    double2 acc[2] = {make_double2(0.0, 0.0), make_double2(0.0, 0.0)};
    for (long i = i0; i < n && on; i += stride) {
        const double2 w = y[(i / Kc) * K + m];
        const float2 v = make_float2((float)(w.x * inv), (float)(w.y * inv));
        r[i] = v;
        x[i] = make_float2(0.0f, 0.0f);
        const float2 a = r0[i];
        acc[0].x += (double)a.x * v.x + (double)a.y * v.y;
        acc[0].y += (double)a.x * v.y - (double)a.y * v.x;
        acc[1].x += (double)v.x * v.x + (double)v.y * v.y;
    }
    __shared__ double2 out[2 * Kc];
    if (dev::grid_reduce_lanes<2, Kc, 256>(acc, rs, out)) {
        const int jj = threadIdx.x;
        if (jj < Kc && map[jj] >= 0 && rep[jj] && scale[jj] > 0.0) {
            BicgState S = st[jj];
            if (S.status == kRunning) {
                S.rnorm = sqrt(out[Kc + jj].x);
                S.res = S.rnorm / S.bnorm;
                S.rho = out[jj];
                if (S.res < S.tol) S.status = kConverged;
                else S.beta = dev::cmul(dev::cdiv(S.rho, S.rho_old), dev::cdiv(S.alpha, S.omega));
                st[jj] = S;
            }
        }
    }
}

// Compact layout of the mixed-precision inner solve: lane j of a K_c-wide
// batch works on right-hand side map[j] of the K-wide FP64 batch (-1: padding).

// b32[row][j] = y64[row][map[j]] / scale[j]   (0 on padding lanes)
__global__ void k_to_f32_lanes(const double2* __restrict__ y, int K, float2* __restrict__ b, int Kc,
                               const int* __restrict__ map, const double* __restrict__ scale, long n_rows) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_rows * Kc) return;
    const long row = i / Kc;
    const int j = (int)(i % Kc), m = map[j];
    const double s = scale[j];
    float2 v = make_float2(0.f, 0.f);
    if (m >= 0 && s > 0.0) {
        const double2 w = y[row * K + m];
        v = make_float2((float)(w.x / s), (float)(w.y / s));
    }
    b[i] = v;
}

// x64[row][map[j]] += x32[row][j] * scale[j] for lanes with add[j] set
__global__ void k_add_f32_lanes(double2* __restrict__ x, int K, const float2* __restrict__ d, int Kc,
                                const int* __restrict__ map, const int* __restrict__ add,
                                const double* __restrict__ scale, long n_rows) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_rows * Kc) return;
    const long row = i / Kc;
    const int j = (int)(i % Kc), m = map[j];
    if (m < 0 || !add[j] || scale[j] == 0.0) return;
    const float2 v = d[i];
    double2 xv = x[row * K + m];
    xv.x += (double)v.x * scale[j];
    xv.y += (double)v.y * scale[j];
    x[row * K + m] = xv;
}

// Repacks up to five K_s-wide FP32 vectors into K_d-wide ones:
// dst[row][j] = src[row][sel[j]] (0 where sel[j] < 0).
struct LaneMove {
    const float2* src[5];
    float2* dst[5];
    int nvec;
};
__global__ void k_gather_lanes(LaneMove mv, int Ks, int Kd, const int* __restrict__ sel, long n_rows) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_rows * Kd) return;
    const long row = i / Kd;
    const int j = (int)(i % Kd), sj = sel[j];
    for (int v = 0; v < mv.nvec; ++v)
        mv.dst[v][i] = sj >= 0 ? mv.src[v][row * Ks + sj] : make_float2(0.f, 0.f);
}

}  // namespace

GpuSolver::GpuSolver(int dev_) : device(dev_) {
    m3d_params_default(&P);
    std::memset(&stats, 0, sizeof(stats));
}

GpuSolver::~GpuSolver() {
    free_all();
    if (ev_start) cudaEventDestroy(ev_start);
    if (ev_stop) cudaEventDestroy(ev_stop);
}

void GpuSolver::free_all() {
    if (stream) cudaStreamSynchronize(stream);
    graphs_clear();
    learn_free();
    dfree(md.perm); dfree(md.iperm); dfree(md.flags); dfree(md.dir); dfree(md.ez); dfree(md.s_diag);
    dfree(md.me_geom); dfree(md.adual); dfree(md.elen); dfree(md.nadj); dfree(md.adj_ptr); dfree(md.adj_cell);
    dfree(md.lift_ptr); dfree(md.lift_col); dfree(md.lift_val); dfree(md.hp); dfree(md.sens_w);
    dfree(md.inc_ptr); dfree(md.inc_edge); dfree(md.inc_other); dfree(md.inc_gv); dfree(md.inc_gw);
    dfree(md.node_bc); dfree(md.e_node); dfree(md.e_g); dfree(md.cell_ptr); dfree(md.cell_edge);
    dfree(d_op_rp); dfree(d_op_rs); dfree(d_col); dfree(d_val); dfree(d_val32);
    dfree(d_seg64); dfree(d_seg32); dfree(d_work64); dfree(d_work32); dfree(d_seg_err);
    seg64 = dev::SegView<double>{}; seg32 = dev::SegView<float>{};
    dfree(d_colour_list); dfree(d_colour_ptr); dfree(d_gridbar);
    dfree(d_src_wr); dfree(d_src_g); src_ns = -1;
    dfree(d_sigma); dfree(d_Me); dfree(d_me_dc);
    dfree(d_diag); dfree(d_diag32); dfree(d_omegas);
    dfree(red.partial); dfree(red.final_); dfree(red.counter);
    dfree(kv.x); dfree(kv.b); dfree(kv.r); dfree(kv.r0); dfree(kv.p); dfree(kv.v); dfree(kv.s); dfree(kv.t);
    dfree(kv.ph); dfree(kv.sh); dfree(kv.y);
    dfree(kv32.x); dfree(kv32.b); dfree(kv32.r); dfree(kv32.r0); dfree(kv32.p); dfree(kv32.v); dfree(kv32.s);
    dfree(kv32.t); dfree(kv32.ph); dfree(kv32.sh); dfree(kv32.y); dfree(d_scale);
    kv32_K = 0;
    dfree(kv32b.x); dfree(kv32b.b); dfree(kv32b.r); dfree(kv32b.r0); dfree(kv32b.p); dfree(kv32b.v);
    dfree(kv32b.s); dfree(kv32b.t); dfree(kv32b.ph); dfree(kv32b.sh); dfree(kv32b.y);
    dfree(d_lane_map); dfree(d_lane_add); dfree(d_lane_sel); dfree(d_eis_partial);
    kv32b_K = 0;
    eis_slots = 0;
    dfree(d_E); dfree(d_Epri); dfree(d_Ebc); dfree(d_rhs); dfree(d_tmp); dfree(d_lam); dfree(d_adj);
    dfree(dc.divJ); dfree(dc.phi); dfree(dc.r); dfree(dc.z); dfree(dc.p); dfree(dc.Ap); dfree(dc.phi0);
    dfree(dc.lap_diag); dfree(dc.lap_off); dfree(dc.jac_inv); dfree(dc.st);
    dfree(dc.lap_seg); dfree(d_lap_work); dfree(d_lap_qpos);
    free_amg();
    amg_host = AmgHierarchy{};
    a0_pos_q.clear();
    a0_pos_d.clear();
    if (h_lap_pinned) { cudaFreeHost(h_lap_pinned); h_lap_pinned = nullptr; }
    reg_free();
    dc.lap_work = nullptr; dc.lap_qpos = nullptr;
    dfree(sd.cell); dfree(sd.geom); dfree(sd.e_ptr); dfree(sd.e_row); dfree(sd.e_code); dfree(sd.sigma_cell);
    dfree(d_hc); dfree(d_Z); dfree(d_wr); dfree(d_obs); dfree(d_err); dfree(d_grad);
    dfree(d_jtj_rhs); dfree(d_jtj_dE); dfree(d_jtj_a); dfree(d_jtj_b); dfree(d_jtj_dz); dfree(d_jtj_wr0);
    dfree(d_jtj_wr1); dfree(d_jtj_ds); dfree(d_jtj_err);
    dfree(d_host_stage); dfree(d_stage_real); dfree(d_states); dfree(d_states2);
    if (gc_stream) { cudaStreamDestroy(gc_stream); gc_stream = nullptr; }
    if (gc_fork) { cudaEventDestroy(gc_fork); gc_fork = nullptr; }
    if (gc_join) { cudaEventDestroy(gc_join); gc_join = nullptr; }
    if (stream) { cudaStreamDestroy(stream); stream = nullptr; }
    kv_K = 0; fwd_cap = 0; E_cap = 0; E_nf = 0; E_K = 0; dc_K = 0; hc_cap = 0; obs_cap = 0; diag_cap = 0;
    jtj_ns = -1;
    ready = false; have_sigma = false; lap_built = false; stations_set = false;
}

void GpuSolver::sync() { cuda_ok(cudaStreamSynchronize(stream), "stream sync"); }

// ---------------------------------------------------------------------------
// setup: layout, boundary sets, colouring, sliced-ELL permutation, upload
// ---------------------------------------------------------------------------

void GpuSolver::setup(const m3d_leaves* lv, const m3d_params* params) {
    free_all();
    if (params) P = *params;
    cuda_ok(cudaSetDevice(device), "cudaSetDevice");
    cuda_ok(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "stream");
    timer.stream = stream;
    if (!ev_start) { cuda_ok(cudaEventCreate(&ev_start), "event"); cuda_ok(cudaEventCreate(&ev_stop), "event"); }

    LeafInput in;
    for (int i = 0; i < 6; ++i) in.domain[i] = lv->domain[i];
    in.min_level = lv->min_level; in.max_level = lv->max_level; in.nc = lv->n_cells;
    in.level = lv->level; in.cx = lv->cx; in.cy = lv->cy; in.cz = lv->cz; in.type = lv->cell_type;
    build_layout(in, L);
    const int ne = L.ne;
    const double* dm = L.domain;

    // Boundary sets (forward_solver_fv.cpp:117, :166-217; :556-569; :1012-1029)
    flags_ref.assign(ne, 0);
    const double bt = L.cell_size0 * 0.1;
    const double air = P.air_z_threshold;
    for (int e = 0; e < ne; ++e) {
        const double x = L.ex[e], y = L.ey[e], z = L.ez[e];
        const bool onb = x <= dm[0] + bt || x >= dm[1] - bt || y <= dm[2] + bt || y >= dm[3] - bt ||
                         z <= dm[4] + bt || z >= dm[5] - bt;
        const bool is_bc = onb || z > air;
        const bool dead = L.dead[e] != 0;
        const bool on1 = x <= dm[0] + 1.0 || x >= dm[1] - 1.0 || y <= dm[2] + 1.0 || y >= dm[3] - 1.0 ||
                         z <= dm[4] + 1.0 || z >= dm[5] - 1.0 || z > air;
        unsigned char f = 0;
        if (is_bc) f |= kFlagBc;
        if (dead) f |= kFlagDead;
        if (is_bc || dead) f |= kFlagConstrained;
        if (!dead && on1) f |= kFlagDcBc;
        if (dead || on1) f |= kFlagSensFixed;
        flags_ref[e] = f;
    }
    auto free_row = [&](int e) { return !(flags_ref[e] & kFlagConstrained); };

    // Greedy colouring of the free-free coupling graph in reference order.
    std::vector<int> colour(ne, 0);
    {
        std::vector<int> mark(64, -1);
        for (int i = 0; i < ne; ++i) {
            if (!free_row(i)) { colour[i] = 0; continue; }
            for (int k = L.s_ptr[i]; k < L.s_ptr[i + 1]; ++k) {
                const int j = L.s_idx[k];
                if (j >= i || !free_row(j)) continue;
                const int c = colour[j];
                if (c >= (int)mark.size()) mark.resize(c + 1, -1);
                mark[c] = i;
            }
            int c = 0;
            while (c < (int)mark.size() && mark[c] == i) ++c;
            colour[i] = c;
        }
    }
    // later neighbours are coloured afterwards; greedy above only looked at
    // j < i, which is exactly the constraint set of sequential greedy.
    //
    // Small colours (under 1 % of the free rows; greedy leaves a few, each a
    // launch per sweep and mostly padding slices): each of their rows moves
    // to the lowest large colour that none of its neighbours has; colours
    // left empty disappear and the rest are renumbered in order.
    {
        int nc0 = *std::max_element(colour.begin(), colour.end()) + 1;
        std::vector<long> cnt(nc0, 0);
        long nfree = 0;
        for (int i = 0; i < ne; ++i)
            if (free_row(i)) { ++cnt[colour[i]]; ++nfree; }
        std::vector<char> small(nc0, 0);
        for (int c = 0; c < nc0; ++c) small[c] = cnt[c] > 0 && cnt[c] < nfree / 100;
        std::vector<int> mark(nc0, -1);
        for (int i = 0; i < ne; ++i) {
            if (!free_row(i) || !small[colour[i]]) continue;
            for (int k = L.s_ptr[i]; k < L.s_ptr[i + 1]; ++k) {
                const int j = L.s_idx[k];
                if (j != i && free_row(j)) mark[colour[j]] = i;
            }
            for (int c = 0; c < nc0; ++c)
                if (!small[c] && mark[c] != i) {
                    --cnt[colour[i]];
                    ++cnt[c];
                    colour[i] = c;
                    break;
                }
        }
        std::vector<int> remap(nc0, -1);
        int next = 0;
        for (int c = 0; c < nc0; ++c)
            if (cnt[c] > 0 || c == 0) remap[c] = next++;
        for (int i = 0; i < ne; ++i) colour[i] = remap[colour[i]];
    }
    const int n_col = *std::max_element(colour.begin(), colour.end()) + 1;

    // Permutation: the reference order (cell by cell along the Morton curve)
    // is cut into blocks of kRowBlock edges; inside a block rows are grouped by
    // colour (reference order kept within a group) and each group is padded to
    // whole slices.  A row's neighbours then sit in the same block or the next
    // one, so gathers stay inside a small, cache-resident window, while each
    // SSOR colour sweep walks its slice list across all blocks.
    //
    // Sweep groups: with sweep_rows > 0 the reference order is also cut into
    // super-blocks of about sweep_rows edges, and the SSOR ordering becomes
    // (super-block, colour): a sweep runs every colour of one super-block
    // before the next one, so the rows it gathers stay in L2 while the
    // super-block is swept.  A group (super-block, colour) is what a colour
    // was: independent rows, one sweep step.  sweep_rows = 0: one super-block.
    constexpr int kRowBlock = 16384;
    const int blocks_per_sb = P.sweep_rows > 0 ? std::max(1, P.sweep_rows / kRowBlock) : (1 << 30);
    const int n_sb = (int)(((long)(ne + kRowBlock - 1) / kRowBlock + blocks_per_sb - 1) / blocks_per_sb);
    auto group_of = [&](int e) { return (e / kRowBlock / blocks_per_sb) * n_col + colour[e]; };
    const int n_grp = n_sb * n_col;
    perm.clear();
    std::vector<std::vector<int>> slices_of(n_grp);
    {
        std::vector<std::vector<int>> byc(n_col);
        for (int b0 = 0; b0 < ne; b0 += kRowBlock) {
            for (auto& v : byc) v.clear();
            for (int e = b0; e < std::min(ne, b0 + kRowBlock); ++e) byc[colour[e]].push_back(e);
            const int g0 = (b0 / kRowBlock / blocks_per_sb) * n_col;
            for (int c = 0; c < n_col; ++c) {
                if (byc[c].empty()) continue;
                const int s0 = (int)(perm.size() / dev::kSlice);
                for (int e : byc[c]) perm.push_back(e);
                while (perm.size() % dev::kSlice) perm.push_back(-1);
                const int s1 = (int)(perm.size() / dev::kSlice);
                for (int s = s0; s < s1; ++s) slices_of[g0 + c].push_back(s);
            }
        }
    }
    colour_ptr.assign(1, 0);
    colour_list.clear();
    for (int g = 0; g < n_grp; ++g) {
        if (slices_of[g].empty()) continue;
        colour_list.insert(colour_list.end(), slices_of[g].begin(), slices_of[g].end());
        colour_ptr.push_back((int)colour_list.size());
    }
    n_pad = (int)perm.size();
    n_slices = n_pad / dev::kSlice;
    iperm.assign(ne, -1);
    for (int r = 0; r < n_pad; ++r) if (perm[r] >= 0) iperm[perm[r]] = r;

    // Split CSR of the free-free off-diagonal part in permuted row order:
    // lower (earlier sweep group) entries, then upper, each in reference
    // column order.
    std::vector<int> op_rp(n_pad + 1, 0), op_rs(n_pad, 0), ecol;
    std::vector<double> eval;
    {
        ecol.reserve((size_t)L.s_idx.size());
        eval.reserve((size_t)L.s_idx.size());
        std::vector<int> up_c;
        std::vector<double> up_v;
        for (int r = 0; r < n_pad; ++r) {
            const int e = perm[r];
            up_c.clear(); up_v.clear();
            if (e >= 0 && free_row(e))
                for (int k = L.s_ptr[e]; k < L.s_ptr[e + 1]; ++k) {
                    const int j = L.s_idx[k];
                    if (j == e || !free_row(j)) continue;
                    if (group_of(j) < group_of(e)) { ecol.push_back(iperm[j]); eval.push_back(L.s_val[k]); }
                    else { up_c.push_back(iperm[j]); up_v.push_back(L.s_val[k]); }
                }
            op_rs[r] = (int)ecol.size();
            ecol.insert(ecol.end(), up_c.begin(), up_c.end());
            eval.insert(eval.end(), up_v.begin(), up_v.end());
            op_rp[r + 1] = (int)ecol.size();
            if (ecol.size() > 2000000000UL) throw std::runtime_error("mesh too large for 32-bit row pointers");
        }
        nnz_off = (long)ecol.size();
    }

    // Per permuted row data.
    std::vector<unsigned char> flags(n_pad, kFlagPad);
    std::vector<signed char> dir(n_pad, 0);
    std::vector<double> ez(n_pad, 0.0), sdiag(n_pad, 1.0), megeom(n_pad, 0.0), adual(n_pad, 0.0), elen(n_pad, 1.0);
    std::vector<int> nadj(n_pad, 0), adj_ptr(n_pad + 1, 0), adj_cell;
    std::vector<int> lift_ptr(n_pad + 1, 0), lift_col;
    std::vector<double> lift_val;
    for (int r = 0; r < n_pad; ++r) {
        const int e = perm[r];
        if (e >= 0) {
            flags[r] = flags_ref[e];
            dir[r] = (signed char)L.edir[e];
            ez[r] = L.ez[e];
            for (int k = L.s_ptr[e]; k < L.s_ptr[e + 1]; ++k) if (L.s_idx[k] == e) sdiag[r] = L.s_val[k];
            megeom[r] = L.adual[e] * L.elen[e];
            adual[r] = L.adual[e];
            elen[r] = L.elen[e];
            nadj[r] = L.adj_ptr[e + 1] - L.adj_ptr[e];
            for (int k = L.adj_ptr[e]; k < L.adj_ptr[e + 1]; ++k) adj_cell.push_back(L.adj[k]);
            if (free_row(e))
                for (int k = L.s_ptr[e]; k < L.s_ptr[e + 1]; ++k) {
                    const int j = L.s_idx[k];
                    if (j != e && (flags_ref[j] & kFlagBc)) { lift_col.push_back(iperm[j]); lift_val.push_back(L.s_val[k]); }
                }
        }
        adj_ptr[r + 1] = (int)adj_cell.size();
        lift_ptr[r + 1] = (int)lift_col.size();
    }
    std::vector<int> hp(3 * L.hp.size());
    {
        std::vector<char> coarse(ne, 0);
        for (const auto& h : L.hp) coarse[h[0]] = 1;
        hp_sequential = false;
        for (size_t i = 0; i < L.hp.size(); ++i) {
            for (int k = 0; k < 3; ++k) hp[3 * i + k] = iperm[L.hp[i][k]];
            if (coarse[L.hp[i][1]] || coarse[L.hp[i][2]]) hp_sequential = true;
        }
    }
    // node incidence in reference edge order; G[e, n1] = -1/L, G[e, n2] = +1/L
    const int nn = L.nn;
    std::vector<int> inc_ptr(nn + 1, 0), inc_edge(2 * ne), inc_other(2 * ne);
    std::vector<double> inc_gv(2 * ne), inc_gw(2 * ne);
    std::vector<unsigned char> node_bc(nn, 0);
    std::vector<int> e_node(2 * n_pad, 0);
    std::vector<double> e_g(2 * n_pad, 0.0);
    for (int e = 0; e < ne; ++e) { inc_ptr[L.n1[e] + 1]++; inc_ptr[L.n2[e] + 1]++; }
    for (int v = 0; v < nn; ++v) inc_ptr[v + 1] += inc_ptr[v];
    {
        std::vector<int> pos(inc_ptr.begin(), inc_ptr.end() - 1);
        for (int e = 0; e < ne; ++e) {
            const double inv = 1.0 / L.elen[e];
            const int a = L.n1[e], b = L.n2[e];
            int q = pos[a]++;
            inc_edge[q] = iperm[e]; inc_other[q] = b; inc_gv[q] = -inv; inc_gw[q] = +inv;
            q = pos[b]++;
            inc_edge[q] = iperm[e]; inc_other[q] = a; inc_gv[q] = +inv; inc_gw[q] = -inv;
            if (flags_ref[e] & kFlagDcBc) { node_bc[a] = 1; node_bc[b] = 1; }
            const int r = iperm[e];
            if (a < b) { e_node[2 * r] = a; e_g[2 * r] = -inv; e_node[2 * r + 1] = b; e_g[2 * r + 1] = +inv; }
            else { e_node[2 * r] = b; e_g[2 * r] = +inv; e_node[2 * r + 1] = a; e_g[2 * r + 1] = -inv; }
        }
    }
    std::vector<int> cell_edge(L.cell_edge.size());
    for (size_t q = 0; q < cell_edge.size(); ++q) cell_edge[q] = iperm[L.cell_edge[q]];

    // node Laplacian off-diagonal pattern as 32-node slice segments (values
    // are written by k_dc_lap through lap_qpos at every conductivity update)
    {
        const int nsl = (nn + dev::kSlice - 1) / dev::kSlice;
        std::vector<unsigned char> seg;
        std::vector<int4> work(nsl);
        std::vector<int> qpos(inc_other.size(), 0);
        int stage = 0;
        for (int sl = 0; sl < nsl; ++sl) {
            const long off = (long)seg.size();
            uint16_t end[dev::kSlice];
            std::vector<int> cols;
            std::vector<long> qs;   // incidence of each entry, -1 for padding
            for (int r = 0; r < dev::kSlice; ++r) {
                const int v = sl * dev::kSlice + r;
                if (v < nn)
                    for (int q = inc_ptr[v]; q < inc_ptr[v + 1]; ++q) { cols.push_back(inc_other[q]); qs.push_back(q); }
                while (cols.size() % 4) { cols.push_back(v); qs.push_back(-1); }
                if (cols.size() > 65535) throw std::runtime_error("node slice segment too large");
                end[r] = (uint16_t)cols.size();
            }
            const size_t n = cols.size();
            const size_t bytes = dev::kSegHeader + 4 * n + 8 * n;
            seg.resize(off + bytes, 0);
            std::memcpy(seg.data() + off, end, sizeof(end));
            std::memcpy(seg.data() + off + dev::kSegHeader, cols.data(), 4 * n);
            const long vbase = (off + dev::kSegHeader + 4 * (long)n) / 8;
            for (size_t j = 0; j < n; ++j)
                if (qs[j] >= 0) qpos[qs[j]] = (int)(vbase + (long)j);
            if (off / 16 > 2000000000L || (long)(bytes / 16) > 65535) throw std::runtime_error("node segment too large");
            work[sl] = make_int4(sl, (int)(off / 16), 0, (int)((bytes / 16) << 16));
            stage = std::max(stage, (int)bytes);
        }
        if (seg.size() / 8 > 2000000000UL) throw std::runtime_error("node segments too large");
        dc.lap_seg = dupload(seg, stream);
        dc.lap_work = d_lap_work = dupload(work, stream);
        dc.lap_qpos = d_lap_qpos = dupload(qpos, stream);
        dc.lap_stage = stage;
        dc.n_node_slices = nsl;
    }
    h_inc_ptr = inc_ptr;
    h_inc_other = inc_other;

    // upload
    md.ne = ne; md.n_pad = n_pad; md.nc = L.nc; md.nn = nn; md.n_slices = n_slices;
    md.perm = dupload(perm, stream); md.iperm = dupload(iperm, stream);
    md.flags = dupload(flags, stream); md.dir = dupload(dir, stream); md.ez = dupload(ez, stream);
    md.s_diag = dupload(sdiag, stream); md.me_geom = dupload(megeom, stream);
    md.adual = dupload(adual, stream); md.elen = dupload(elen, stream); md.nadj = dupload(nadj, stream);
    md.adj_ptr = dupload(adj_ptr, stream); md.adj_cell = dupload(adj_cell, stream);
    md.lift_ptr = dupload(lift_ptr, stream); md.lift_col = dupload(lift_col, stream);
    md.lift_val = dupload(lift_val, stream);
    md.nhp = (int)L.hp.size(); md.hp = dupload(hp, stream);
    md.inc_ptr = dupload(inc_ptr, stream); md.inc_edge = dupload(inc_edge, stream);
    md.inc_other = dupload(inc_other, stream); md.inc_gv = dupload(inc_gv, stream);
    md.inc_gw = dupload(inc_gw, stream); md.node_bc = dupload(node_bc, stream);
    md.e_node = dupload(e_node, stream); md.e_g = dupload(e_g, stream);
    md.cell_ptr = dupload(L.cell_ptr, stream); md.cell_edge = dupload(cell_edge, stream);
    {
        // per-edge factor of dMe/dsigma_c (compute_sensitivity,
        // forward_solver_fv.cpp:1010-1030): constrained edges and edges
        // without adjacent cells are skipped there and weigh 0 here
        std::vector<double> sens_w(n_pad, 0.0);
        for (int r = 0; r < n_pad; ++r)
            if (!(flags[r] & kFlagSensFixed) && nadj[r] > 0) sens_w[r] = adual[r] * elen[r] / nadj[r];
        md.sens_w = dupload(sens_w, stream);
    }
    d_op_rp = dupload(op_rp, stream); d_op_rs = dupload(op_rs, stream);
    d_col = dupload(ecol, stream); d_val = dupload(eval, stream);
    d_colour_list = dupload(colour_list, stream);
    d_colour_ptr = dupload(colour_ptr, stream);
    d_gridbar = dalloc_zero<unsigned>(2, stream);
    build_segments(op_rp, op_rs, ecol, eval);
    {
        std::vector<float> ev32(eval.begin(), eval.end());
        d_val32 = dupload(ev32, stream);
    }
    // reduction scratch: enough blocks for two waves on every SM
    int sms = 0;
    cuda_ok(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device), "sm count");
    red.max_blocks = std::max(2, 8 * sms);
    red.max_blocks += red.max_blocks & 1;
    red.partial = dalloc<double2>((size_t)red.max_blocks * dev::kMaxQ * dev::kMaxRhs);
    red.final_ = dalloc<double2>(dev::kMaxQ * dev::kMaxRhs);
    red.counter = dalloc<unsigned int>(1);
    cuda_ok(cudaMemsetAsync(red.counter, 0, sizeof(unsigned int), stream), "memset");
    d_sigma = dalloc<double>(L.nc);
    d_Me = dalloc<double>(n_pad);
    d_diag = dalloc<double2>(n_pad);
    d_diag32 = dalloc<float2>(n_pad);
    d_me_dc = dalloc<double>(n_pad);
    d_host_stage = dalloc<double2>(std::max(ne, 1));
    d_stage_real = dalloc<double>(std::max(ne, L.nc));
    d_grad = dalloc<double>(L.nc);
    d_states = dalloc<BicgState>(dev::kMaxRhs);
    d_states2 = dalloc<BicgState>(dev::kMaxRhs);
    sigma_h.assign(L.nc, 0.0);
    sync();
    ready = true;
}

void GpuSolver::set_sigma(const double* sigma, int n) {
    if (n != L.nc) throw std::invalid_argument("sigma size != number of cells");
    sigma_h.assign(sigma, sigma + n);
    cuda_ok(cudaMemcpyAsync(d_sigma, sigma, sizeof(double) * n, cudaMemcpyHostToDevice, stream), "sigma");
    phys::edge_mass(md, d_sigma, d_Me, d_me_dc, stream);
    phys::diag_coeffs(md, d_Me, d_diag, d_diag32, stream);
    learn_sigma_changed();
    launches += 2;
    have_sigma = true;
    lap_built = false;
    if (stations_set) {
        std::vector<double> sc(st_cell.size(), 0.0);
        for (size_t s = 0; s < st_cell.size(); ++s) if (st_cell[s] >= 0) sc[s] = sigma_h[st_cell[s]];
        cuda_ok(cudaMemcpyAsync(sd.sigma_cell, sc.data(), sizeof(double) * sc.size(), cudaMemcpyHostToDevice, stream), "sc");
    }
    sync();
}

// find_stations_ (forward_solver_fv.cpp:1393-1485) on the leaf geometry
void GpuSolver::set_stations(const double* xyz, int n) {
    const double* dm = L.domain;
    const double DX = dm[1] - dm[0], DY = dm[3] - dm[2], DZ = dm[5] - dm[4];
    st_cell.assign(n, -1);
    for (int si = 0; si < n; ++si) {
        const double sx = xyz[3 * si], sy = xyz[3 * si + 1], sz = 0.0;
        int best = -1, fb = -1;
        double bcz = 1e30, fbd = 1e30;
        for (int c = 0; c < L.nc; ++c) {
            if (L.ctype[c] == 1) continue;
            const double cx = L.ccx[c], cy = L.ccy[c], cz = L.ccz[c];
            const double h = 1.0 / (1 << L.clevel[c]);
            const double hdx = h * DX, hdy = h * DY;
            const bool inx = (sx >= cx - hdx / 2 - 1.0) && (sx <= cx + hdx / 2 + 1.0);
            const bool iny = (sy >= cy - hdy / 2 - 1.0) && (sy <= cy + hdy / 2 + 1.0);
            if (inx && iny && cz < 0 && std::abs(cz) < bcz) { bcz = std::abs(cz); best = c; }
            const double d = std::sqrt((cx - sx) * (cx - sx) + (cy - sy) * (cy - sy) + (cz - sz) * (cz - sz));
            if (d < fbd) { fbd = d; fb = c; }
        }
        if (best < 0) best = fb;
        st_cell[si] = best;
    }
    std::vector<double> geom(6 * (size_t)n, 0.0), sc(n, 0.0);
    std::vector<int> eptr(n + 1, 0), erow;
    std::vector<unsigned char> ecode;
    for (int s = 0; s < n; ++s) {
        const int c = st_cell[s];
        if (c >= 0) {
            const double h = 1.0 / (1 << L.clevel[c]);
            const double cx = L.ccx[c], cy = L.ccy[c], cz = L.ccz[c];
            geom[6 * s] = cx; geom[6 * s + 1] = cy; geom[6 * s + 2] = cz;
            geom[6 * s + 3] = h * DX; geom[6 * s + 4] = h * DY; geom[6 * s + 5] = h * DZ;
            sc[s] = have_sigma ? sigma_h[c] : 0.0;
            for (int q = L.cell_ptr[c]; q < L.cell_ptr[c + 1]; ++q) {
                const int e = L.cell_edge[q];
                unsigned char code = (unsigned char)L.edir[e];
                if (L.ez[e] > cz) code |= 4;
                if (L.ex[e] > cx) code |= 8;
                if (L.ey[e] > cy) code |= 16;
                erow.push_back(iperm[e]);
                ecode.push_back(code);
            }
        }
        eptr[s + 1] = (int)erow.size();
    }
    dfree(sd.cell); dfree(sd.geom); dfree(sd.e_ptr); dfree(sd.e_row); dfree(sd.e_code); dfree(sd.sigma_cell);
    sd.ns = n;
    sd.cell = dupload(st_cell, stream);
    sd.geom = dupload(geom, stream);
    sd.e_ptr = dupload(eptr, stream);
    sd.e_row = dupload(erow, stream);
    sd.e_code = dupload(ecode, stream);
    sd.sigma_cell = dupload(sc, stream);
    stations_set = true;
    hc_cap = 0;
    dfree(d_hc); dfree(d_Z); dfree(d_wr);
    // every buffer sized by the station count goes with the old stations:
    // observed data and errors of gradient_batch, the weighted dZ and
    // residual buffers of jtjv_batch
    dfree(d_obs); dfree(d_err);
    obs_cap = 0;
    dfree(d_jtj_dz); dfree(d_jtj_wr0); dfree(d_jtj_wr1); dfree(d_jtj_err);
    jtj_ns = -1;
    sync();
}

// ---------------------------------------------------------------------------
// buffers
// ---------------------------------------------------------------------------

void GpuSolver::ensure_vecs(int K) {
    if (kv_K >= K) return;
    dfree(kv.x); dfree(kv.b); dfree(kv.r); dfree(kv.r0); dfree(kv.p); dfree(kv.v); dfree(kv.s); dfree(kv.t);
    dfree(kv.ph); dfree(kv.sh); dfree(kv.y);
    const size_t n = (size_t)n_pad * K;
    for (double2** q : {&kv.x, &kv.b, &kv.r, &kv.r0, &kv.p, &kv.v, &kv.s, &kv.t, &kv.ph, &kv.sh, &kv.y})
        *q = dalloc_zero<double2>(n, stream);
    kv_K = K;
}

// Work vectors of the forward / adjoint calls.  The resident background
// field d_E is not among them: a call that only needs wider scratch (e.g.
// solve_rhs_batch with 16 right-hand sides after a 2-frequency forward) must
// not drop the field that jtjv_batch, perturbation_rhs and background_E read.
void GpuSolver::ensure_fields(int K) {
    if (fwd_cap >= K) return;
    dfree(d_Epri); dfree(d_Ebc); dfree(d_rhs); dfree(d_tmp); dfree(d_lam); dfree(d_adj);
    const size_t n = (size_t)n_pad * K;
    d_Epri = dalloc<double2>(n); d_Ebc = dalloc<double2>(n);
    d_rhs = dalloc<double2>(n); d_tmp = dalloc<double2>(n); d_lam = dalloc<double2>(n); d_adj = dalloc<double2>(n);
    fwd_cap = K;
}

// The resident background field, [n_pad][K] with the writer's K as stride.
// Only its writers (run_forward, set_background) grow it; a regrow discards
// the old field, so the resident-field state is reset with it.
void GpuSolver::ensure_E(int K) {
    if (E_cap >= K) return;
    dfree(d_E);
    d_E = dalloc<double2>((size_t)n_pad * K);
    E_cap = K;
    E_nf = 0;
    E_K = 0;
}

void GpuSolver::ensure_dc(int K) {
    if (!dc.lap_diag) {
        dc.lap_diag = dalloc<double>(L.nn);
        dc.jac_inv = dalloc<double>(L.nn);
        dc.lap_off = dalloc<double>(2 * (size_t)L.ne);
        dc.st = dalloc<phys::DcState>(dev::kMaxRhs);
    }
    if (dc_K >= K) return;
    dfree(dc.divJ); dfree(dc.phi); dfree(dc.r); dfree(dc.z); dfree(dc.p); dfree(dc.Ap); dfree(dc.phi0);
    const size_t n = (size_t)L.nn * K;
    for (double2** q : {&dc.divJ, &dc.phi, &dc.r, &dc.z, &dc.p, &dc.Ap, &dc.phi0}) *q = dalloc_zero<double2>(n, stream);
    dc_K = K;
}

void GpuSolver::ensure_hc(int nf) {
    if (hc_cap >= nf) return;
    dfree(d_hc); dfree(d_Z); dfree(d_wr);
    const size_t n = (size_t)std::max(1, sd.ns) * nf;
    d_hc = dalloc<HCache>(n);
    d_Z = dalloc<double2>(4 * n);
    d_wr = dalloc<double2>(4 * n);
    hc_cap = nf;
}

void GpuSolver::ensure_sigma_device() {
    if (!have_sigma) throw std::logic_error("conductivity not set (m3d_set_sigma)");
    if (P.div_correction && !lap_built) {
        ensure_dc(2);
        phys::dc_build_laplacian(md, d_me_dc, dc, stream);
        ++launches;
        lap_built = true;
        if (want_amg()) build_amg();
    }
}

void GpuSolver::free_amg() {
    if (stream) cudaStreamSynchronize(stream);
    for (void* p : amg_mem) cudaFree(p);
    amg_mem.clear();
    amg = phys::AmgDev{};
    amg_ok = false;
    for (void* p : gc_mem) cudaFree(p);
    gc_mem.clear();
    gc = GcDev{};
    gc_ok = false;
}

// Gradient-space correction over the device hierarchy just built: level 0
// reads the divergence-correction Laplacian through the node incidence, the
// coarser levels the hierarchy's CSR operators (both refreshed in place for
// a new conductivity); FP32 work vectors for up to 16 right-hand sides.
void GpuSolver::build_gc() {
    if (!amg_ok || P.precision != 1 || (P.gradcorr != 1 && P.divcorr_mixed != 1)) return;
    auto zeros2 = [&](size_t n) {
        float2* p = dalloc_zero<float2>(n, stream);
        gc_mem.push_back((void*)p);
        return p;
    };
    const long n_inc = (long)h_inc_other.size();
    float* inc_g = dalloc<float>((size_t)std::max<long>(1, n_inc));
    gc_mem.push_back((void*)inc_g);
    float* e_g = dalloc<float>(2 * (size_t)n_pad);
    gc_mem.push_back((void*)e_g);
    gc_weights(md, inc_g, e_g, stream);
    ++launches;
    gc.n_levels = amg.n_levels;
    gc.nn = L.nn;
    gc.inc_ptr = md.inc_ptr;
    gc.inc_other = md.inc_other;
    gc.inc_edge = md.inc_edge;
    gc.lap_off = dc.lap_off;
    gc.lap_diag = dc.lap_diag;
    gc.inc_g = inc_g;
    int2* pk = dalloc<int2>((size_t)std::max<long>(1, n_inc));
    gc_mem.push_back((void*)pk);
    float* d32 = dalloc<float>((size_t)L.nn);
    gc_mem.push_back((void*)d32);
    gc.lap_pk = pk;
    gc.lap_diag32 = d32;
    float* dv32 = dalloc<float>((size_t)L.nn);
    gc_mem.push_back((void*)dv32);
    gc.e_node = md.e_node;
    gc.e_g = e_g;
    for (int l = 0; l < amg.n_levels; ++l) {
        const phys::AmgLevelDev& a = amg.lv[l];
        GcLevel& g = gc.lv[l];
        g.n = a.n;
        g.ptr = a.ptr;
        g.col = a.col;
        g.val = a.val;
        g.dinv = a.dinv;
        if (l == 0) g.dinv32 = dv32;
        g.agg = a.agg;
        g.rptr = a.rptr;
        g.rcol = a.rcol;
        const size_t n = (size_t)a.n * dev::kMaxRhs;
        g.b = zeros2(n);
        g.x = zeros2(n);
        g.y = zeros2(n);
    }
    gc.out0 = zeros2((size_t)L.nn * dev::kMaxRhs);
    if (P.divcorr_mixed == 1) {
        for (float2** q : {&gc.dc_x, &gc.dc_r, &gc.dc_z, &gc.dc_p, &gc.dc_ap}) *q = zeros2((size_t)L.nn * dev::kMaxRhs);
        GcPcgState* st = dalloc_zero<GcPcgState>(dev::kMaxRhs, stream);
        gc_mem.push_back((void*)st);
        gc.dc_st = st;
    }
    gc.n_coarse = amg.n_coarse;
    gc.coarse_inv = amg.coarse_inv;
    gc.omega = (float)amg.omega;
    gc.presmooth = P.gradcorr_presmooth;
    gc.omega_max = P.gradcorr == 1 ? 2.0 * kPi * P.gradcorr_fmax : 0.0;
    gc.inc_entries = n_inc;
    gc_pack_level0(gc, stream);
    ++launches;
    if (!gc_stream) {
        cuda_ok(cudaStreamCreateWithFlags(&gc_stream, cudaStreamNonBlocking), "stream");
        cuda_ok(cudaEventCreateWithFlags(&gc_fork, cudaEventDisableTiming), "event");
        cuda_ok(cudaEventCreateWithFlags(&gc_join, cudaEventDisableTiming), "event");
    }
    sync();
    gc_ok = true;
}

// The gradient-space term on a FP32 batch context; with gradcorr_overlap its
// V-cycles run on the side stream, overlapping the forward SSOR sweeps.
void GpuSolver::attach_gc(KrylovCtx<float>& c) {
    c.gc = &gc;
    if (P.gradcorr_overlap == 1) {
        c.gc_stream = gc_stream;
        c.gc_fork = gc_fork;
        c.gc_join = gc_join;
    }
}

// Aggregation multigrid hierarchy of the node Laplacian just built on the
// device (host setup, host/amg.cpp); falls back to the Jacobi PCG when the
// coarsening does not reach a small coarse level.
void GpuSolver::build_amg() {
    const auto t0 = std::chrono::steady_clock::now();
    const int nn = L.nn;
    const size_t n_inc = h_inc_other.size();
    // the Laplacian read back through a pinned staging buffer
    if (!h_lap_pinned) cuda_ok(cudaMallocHost(&h_lap_pinned, sizeof(double) * (nn + n_inc + 1)), "pinned");
    double* diag = h_lap_pinned;
    double* off = h_lap_pinned + nn;
    cuda_ok(cudaMemcpyAsync(diag, dc.lap_diag, sizeof(double) * nn, cudaMemcpyDeviceToHost, stream), "lap");
    cuda_ok(cudaMemcpyAsync(off, dc.lap_off, sizeof(double) * n_inc, cudaMemcpyDeviceToHost, stream), "lap");
    sync();
    AmgOptions opt;
    opt.omega_p = 0.0;   // piecewise-constant prolongation (the kernels assume it)
    AmgHierarchy& H = amg_host;
    bool built = false;
    // same mesh and zero pattern: write level 0's values in place and refresh
    // the coarse operators on the kept aggregates
    if (!H.levels.empty() && H.levels[0].A.n_rows == nn && a0_pos_q.size() == n_inc && (int)a0_pos_d.size() == nn) {
        bool same = true;
        std::vector<double>& val = H.levels[0].A.val;
        for (int v = 0; v < nn && same; ++v) {
            for (int q = h_inc_ptr[v]; q < h_inc_ptr[v + 1]; ++q) {
                const int p = a0_pos_q[q];
                if ((off[q] != 0.0) != (p >= 0)) { same = false; break; }
                if (p >= 0) val[p] = off[q];
            }
            val[a0_pos_d[v]] = diag[v];
        }
        if (same) {
            try {
                amg_refresh_values(opt, H);
                built = true;
            } catch (const std::exception&) {
                built = false;
            }
        }
    }
    if (!built) {
        CsrReal A0;
        A0.n_rows = A0.n_cols = nn;
        A0.ptr.assign(nn + 1, 0);
        a0_pos_q.assign(n_inc, -1);
        a0_pos_d.assign(nn, -1);
        for (int v = 0; v < nn; ++v) {
            for (int q = h_inc_ptr[v]; q < h_inc_ptr[v + 1]; ++q)
                if (off[q] != 0.0) {
                    a0_pos_q[q] = (int)A0.col.size();
                    A0.col.push_back(h_inc_other[q]);
                    A0.val.push_back(off[q]);
                }
            a0_pos_d[v] = (int)A0.col.size();
            A0.col.push_back(v);
            A0.val.push_back(diag[v]);
            A0.ptr[v + 1] = (int)A0.col.size();
        }
        if (!H.levels.empty() && H.levels[0].A.n_rows == nn) {
            try {
                amg_refresh(A0, opt, H);   // same mesh: keep the aggregates
                built = true;
            } catch (const std::exception&) {
                built = false;
            }
        }
        if (!built) amg_pending_A0 = std::move(A0);
    }
    const int nl_dev = amg_ok ? amg.n_levels : 0;
    if (built && nl_dev == (int)H.levels.size()) {
        // same hierarchy on the device: refresh the values in place
        for (int l = 0; l < nl_dev; ++l) {
            const AmgLevel& Lv = H.levels[l];
            phys::AmgLevelDev& d = amg.lv[l];
            if (l > 0)
                cuda_ok(cudaMemcpyAsync(const_cast<double*>(d.val), Lv.A.val.data(), sizeof(double) * Lv.A.val.size(),
                                        cudaMemcpyHostToDevice, stream), "mg values");
            cuda_ok(cudaMemcpyAsync(const_cast<double*>(d.dinv), Lv.dinv.data(), sizeof(double) * Lv.dinv.size(),
                                    cudaMemcpyHostToDevice, stream), "mg values");
        }
        cuda_ok(cudaMemcpyAsync(const_cast<double*>(amg.coarse_inv), H.coarse_inv.data(),
                                sizeof(double) * H.coarse_inv.size(), cudaMemcpyHostToDevice, stream), "mg values");
        if (gc_ok) {
            gc_pack_level0(gc, stream);
            ++launches;
        }
        sync();
        amg_setup_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        return;
    }
    free_amg();
    if (!built) {
        try {
            amg_build(amg_pending_A0, opt, H);
            amg_pending_A0 = CsrReal{};
        } catch (const std::exception&) {
            H = AmgHierarchy{};
            return;   // Jacobi PCG
        }
    }
    const int nl = (int)H.levels.size();
    // a single level (tiny meshes) or a large coarse level: keep the Jacobi PCG
    if (nl < 2 || nl > phys::kAmgMaxLevels || H.n_coarse > 2048) return;
    auto up = [&](const auto& v) {
        auto* p = dupload(v, stream);
        amg_mem.push_back((void*)p);
        return p;
    };
    auto zeros = [&](size_t n) {
        double2* p = dalloc_zero<double2>(n, stream);
        amg_mem.push_back((void*)p);
        return p;
    };
    amg.n_levels = nl;
    for (int l = 0; l < nl; ++l) {
        const AmgLevel& Lv = H.levels[l];
        phys::AmgLevelDev& d = amg.lv[l];
        d.n = Lv.A.n_rows;
        if (l > 0) {
            d.ptr = up(Lv.A.ptr);
            d.col = up(Lv.A.col);
            d.val = up(Lv.A.val);
        }
        d.dinv = up(Lv.dinv);
        if (l + 1 < nl) {
            std::vector<int> agg(d.n, -1);
            for (int i = 0; i < d.n; ++i)
                if (Lv.P.ptr[i + 1] > Lv.P.ptr[i]) agg[i] = Lv.P.col[Lv.P.ptr[i]];
            d.agg = up(agg);
            d.rptr = up(Lv.R.ptr);
            d.rcol = up(Lv.R.col);
        }
        const size_t n = (size_t)d.n * dev::kMaxRhs;
        d.b = zeros(n);
        d.x = zeros(n);
        d.y = zeros(n);
        d.r = zeros(n);
    }
    amg.n_coarse = H.n_coarse;
    amg.coarse_inv = up(H.coarse_inv);
    amg_ok = true;
    sync();
    build_gc();
    amg_setup_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

KrylovCtx<double> GpuSolver::kctx(int K, const int* fmap) const {
    KrylovCtx<double> c;
    c.A = OpView<double>{d_op_rp, d_op_rs, d_col, d_val, n_pad};
    c.D = DiagView<double>{d_diag};
    c.B.K = K;
    for (int k = 0; k < dev::kMaxRhs; ++k) {
        c.B.fmap[k] = (k < K) ? fmap[k] : 0;
        c.B.omega[k] = (k < K && c.B.fmap[k] < (int)fz_freqs.size()) ? 2.0 * kPi * fz_freqs[c.B.fmap[k]] : 0.0;
    }
    c.colour_ptr = colour_ptr;
    c.colour_list = d_colour_list;
    c.n_pad = n_pad;
    c.grid_vec = red.max_blocks;
    c.grid_spmv = std::max(2, red.max_blocks / 2);
    c.red = red;
    c.stream = stream;
    c.launches = const_cast<long long*>(&launches);
    c.timer = timer.on ? const_cast<KernelTimer*>(&timer) : nullptr;
    c.nnz = nnz_off;
    c.n_rows = L.ne;
    std::vector<int> fs(fmap, fmap + K);
    std::sort(fs.begin(), fs.end());
    c.n_freq = (int)(std::unique(fs.begin(), fs.end()) - fs.begin());
    c.seg = seg64;
    c.row_kernels = P.row_kernels;
    c.coop = P.coop_sweep;
    c.colour_ptr_d = d_colour_ptr;
    c.gridbar = d_gridbar;
    return c;
}

RhsInfo GpuSolver::rhs_info(int K, const std::vector<int>& f, const std::vector<int>& pol,
                            const std::vector<double>& freqs) const {
    RhsInfo info;
    std::memset(&info, 0, sizeof(info));
    info.K = K;
    for (int k = 0; k < K; ++k) {
        info.f[k] = f[k];
        info.pol[k] = pol[k];
        const double om = 2.0 * kPi * freqs[f[k]];
        info.omega[k] = om;
        const std::complex<double> ik = std::sqrt(std::complex<double>(0.0, om * kMu0 * P.sigma_bg));
        info.ik[k] = make_double2(ik.real(), ik.imag());
    }
    return info;
}

// ---------------------------------------------------------------------------
// factorisation (assembly of the per-frequency diagonals)
// ---------------------------------------------------------------------------

void GpuSolver::factorize(const std::vector<double>& freqs) {
    ensure_sigma_device();
    const int nf = (int)freqs.size();
    if (diag_cap < nf) {
        dfree(d_omegas);
        d_omegas = dalloc<double>(nf);
        diag_cap = nf;
    }
    std::vector<double> om(nf);
    for (int f = 0; f < nf; ++f) om[f] = 2.0 * kPi * freqs[f];
    cuda_ok(cudaMemcpyAsync(d_omegas, om.data(), sizeof(double) * nf, cudaMemcpyHostToDevice, stream), "omegas");
    fz_freqs = freqs;
    current_omega = om.back();
}

// ---------------------------------------------------------------------------
// batched BiCGStab (device-resident scalars, host polls every chunk)
// ---------------------------------------------------------------------------

BatchResult GpuSolver::solve_batch(int K, const int* fmap, double2* b, double2* x, const std::vector<int>& active,
                                   double tol, int maxiter) {
    ensure_vecs(K);
    KrylovCtx<double> c = kctx(K, fmap);
    KrylovVecs<double> v = kv;
    v.b = b;
    v.x = x;
    BatchResult R;
    R.K = K;
    R.iters.assign(K, 0); R.status.assign(K, kInactive); R.res.assign(K, 0.0); R.true_res.assign(K, 0.0);
    std::vector<BicgState> hs(K);
    std::vector<int> run_set = active;
    const int chunk = 10;
    // pass 0 is the solve; passes 1.. restart from x (r = b - A x recomputed
    // in FP64) for right-hand sides whose recursive residual met tol while
    // the true residual did not.
    const int passes = 1 + (P.true_residual_check ? std::max(0, P.max_refinements) : 0);
    for (int pass = 0; pass < passes; ++pass) {
        bool any = false;
        for (int k = 0; k < K; ++k) any |= run_set[k] != 0;
        if (!any) break;
        for (int k = 0; k < K; ++k) {
            std::memset(&hs[k], 0, sizeof(BicgState));
            hs[k].tol = tol;
            hs[k].maxiter = std::max(1, maxiter - R.iters[k]);
            hs[k].status = run_set[k] ? kRunning : kInactive;
        }
        cuda_ok(cudaMemcpyAsync(d_states, hs.data(), sizeof(BicgState) * K, cudaMemcpyHostToDevice, stream), "states");
        bicg_init(c, v, d_states);
        int it = 0;
        for (;;) {
            cuda_ok(cudaMemcpyAsync(hs.data(), d_states, sizeof(BicgState) * K, cudaMemcpyDeviceToHost, stream), "states");
            sync();
            bool run = false;
            for (int k = 0; k < K; ++k) run |= hs[k].status == kRunning;
            if (collecting && net && run) collect_snapshot(v.x, v.r, K, hs, fmap);   // training pairs
            if (!run || it >= maxiter) break;
            for (int i = 0; i < chunk && it < maxiter; ++i, ++it) bicg_iteration(c, v, d_states);
        }
        for (int k = 0; k < K; ++k) {
            if (!run_set[k]) continue;
            R.iters[k] += hs[k].iter;
            R.status[k] = hs[k].status == kRunning ? kMaxIter : hs[k].status;   // stopped by the host's cap
            R.res[k] = hs[k].res;
        }
        // FP64 true residual || b - A x || / || b || of every active rhs
        for (int k = 0; k < K; ++k) {
            std::memset(&hs[k], 0, sizeof(BicgState));
            hs[k].status = active[k] ? kConverged : kInactive;
        }
        cuda_ok(cudaMemcpyAsync(d_states, hs.data(), sizeof(BicgState) * K, cudaMemcpyHostToDevice, stream), "states");
        spmv(c, kSpmvTrueRes, x, kv.y, b, nullptr, d_states);
        cuda_ok(cudaMemcpyAsync(hs.data(), d_states, sizeof(BicgState) * K, cudaMemcpyDeviceToHost, stream), "states");
        sync();
        for (int k = 0; k < K; ++k) {
            if (active[k]) R.true_res[k] = hs[k].true_res;
            // non-finite values reached the iterate: report a breakdown
            if (active[k] && !std::isfinite(R.true_res[k])) R.status[k] = kBreakdown;
            const bool again = run_set[k] && R.status[k] == kConverged && R.true_res[k] > tol &&
                               R.iters[k] < maxiter;
            run_set[k] = again ? 1 : 0;
            if (again && pass + 1 < passes) ++stats.refinements;
        }
    }
    if (collecting && net) collect_finish(x, K);
    timer.collect();
    return R;
}

void GpuSolver::ensure_vecs32(int K) {
    if (kv32_K >= K) return;
    dfree(kv32.x); dfree(kv32.b); dfree(kv32.r); dfree(kv32.r0); dfree(kv32.p); dfree(kv32.v); dfree(kv32.s);
    dfree(kv32.t); dfree(kv32.ph); dfree(kv32.sh); dfree(kv32.y);
    const size_t n = (size_t)n_pad * K;
    for (float2** q : {&kv32.x, &kv32.b, &kv32.r, &kv32.r0, &kv32.p, &kv32.v, &kv32.s, &kv32.t, &kv32.ph, &kv32.sh,
                       &kv32.y})
        *q = dalloc_zero<float2>(n, stream);
    if (!d_scale) d_scale = dalloc<double>(dev::kMaxRhs);
    kv32_K = K;
}

void GpuSolver::ensure_vecs32b(int K) {
    if (kv32b_K >= K) return;
    KrylovVecs<float>& v = kv32b;
    dfree(v.x); dfree(v.b); dfree(v.r); dfree(v.r0); dfree(v.p); dfree(v.v); dfree(v.s);
    dfree(v.t); dfree(v.ph); dfree(v.sh); dfree(v.y);
    const size_t n = (size_t)n_pad * K;
    for (float2** q : {&v.x, &v.b, &v.r, &v.r0, &v.p, &v.v, &v.s, &v.t, &v.ph, &v.sh, &v.y})
        *q = dalloc_zero<float2>(n, stream);
    if (!d_lane_map) {
        d_lane_map = dalloc<int>(dev::kMaxRhs);
        d_lane_add = dalloc<int>(dev::kMaxRhs);
        d_lane_sel = dalloc<int>(dev::kMaxRhs);
    }
    if (!d_eis_partial) {
        // one slot per block of every backward and forward colour launch of
        // an operator application: 2 x colours x (32 resident blocks per SM)
        int sms = 0;
        cuda_ok(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device), "sm count");
        eis_slots = 2 * std::max(1, n_colours()) * 32 * std::max(1, sms);
        d_eis_partial = dalloc<double2>((size_t)eis_slots * dev::kMaxQ * dev::kMaxRhs);
    }
    kv32b_K = K;
}

KrylovCtx<float> GpuSolver::kctx32(int K, const int* fmap) const {
    const KrylovCtx<double> c = kctx(K, fmap);
    KrylovCtx<float> f;
    f.A = OpView<float>{d_op_rp, d_op_rs, d_col, d_val32, n_pad};
    f.D = DiagView<float>{d_diag32};
    f.B = c.B;
    f.B.relax = P.ssor_relax;   // the FP64 context keeps the reference's 1
    f.colour_ptr = c.colour_ptr;
    f.colour_list = c.colour_list;
    f.n_pad = c.n_pad;
    f.grid_vec = c.grid_vec;
    f.grid_spmv = c.grid_spmv;
    f.red = c.red;
    f.stream = c.stream;
    f.launches = c.launches;
    f.timer = c.timer;
    f.nnz = c.nnz;
    f.n_rows = c.n_rows;
    f.n_freq = c.n_freq;
    f.seg = seg32;
    f.row_kernels = c.row_kernels;
    f.eis_partial = d_eis_partial;
    f.eis_slots = eis_slots;
    f.coop = c.coop;
    f.colour_ptr_d = c.colour_ptr_d;
    f.gridbar = c.gridbar;
    return f;
}

BatchResult GpuSolver::solve_any(int K, const int* fmap, double2* b, double2* x, const std::vector<int>& active,
                                 double tol, int maxiter) {
    BatchResult R = (P.precision == 1 && P.krylov == 1) ? solve_batch_fgmres(K, fmap, b, x, active, tol, maxiter)
                    : (P.precision == 1)                 ? solve_batch_mixed(K, fmap, b, x, active, tol, maxiter)
                                                         : solve_batch(K, fmap, b, x, active, tol, maxiter);
    check_seg_err();
    return R;
}

// A staged kernel whose barrier wait timed out skipped its slices: the
// call's results are invalid and the call fails with M3D_ERR_CUDA.  The error
// bit is cleared (a test-hook bit is kept) so that the next call starts clean.
void GpuSolver::check_seg_err() {
    if (!d_seg_err) return;
    unsigned e = 0;
    cuda_ok(cudaMemcpyAsync(&e, d_seg_err, sizeof(unsigned), cudaMemcpyDeviceToHost, stream), "seg err");
    sync();
    if (e & dev::kErrCopyTimeout) {
        const unsigned keep = e & dev::kTestConsumeNoWait;
        cuda_ok(cudaMemcpyAsync(d_seg_err, &keep, sizeof(unsigned), cudaMemcpyHostToDevice, stream), "seg err");
        sync();
        throw std::runtime_error("slice-staged copy did not complete (barrier wait timed out)");
    }
}

void GpuSolver::set_test_consume_no_wait(bool on) {
    if (!d_seg_err) throw std::logic_error("solver not set up");
    const unsigned v = on ? dev::kTestConsumeNoWait : 0u;
    cuda_ok(cudaMemcpyAsync(d_seg_err, &v, sizeof(unsigned), cudaMemcpyHostToDevice, stream), "seg err");
    sync();
}

// Slice segments (staged.cuh) of the split operator for both precisions:
// per 32-row slice a lower and an upper segment, each [uint16 row ends]
// [int32 columns] [values], every row padded to a multiple of four entries,
// 16-byte aligned, and one work item per slice in natural and in
// colour-sweep order.
void GpuSolver::build_segments(const std::vector<int>& op_rp, const std::vector<int>& op_rs,
                               const std::vector<int>& ecol, const std::vector<double>& eval) {
    const int ns = n_slices;
    auto build = [&](auto tag, std::vector<unsigned char>& buf, std::vector<int4>& work, int& st_lo, int& st_up,
                     int& st_spmv) {
        using R = decltype(tag);
        buf.clear();
        work.assign((size_t)ns, make_int4(0, 0, 0, 0));
        st_lo = st_up = st_spmv = 0;
        auto put = [&](int s, bool upper) -> std::pair<long, int> {
            const long off = (long)buf.size();
            uint16_t end[dev::kSlice];
            std::vector<int> cols;
            std::vector<R> vals;
            for (int r = 0; r < dev::kSlice; ++r) {
                const int row = s * dev::kSlice + r;
                const int b = upper ? op_rs[row] : op_rp[row];
                const int e = upper ? op_rp[row + 1] : op_rs[row];
                for (int k = b; k < e; ++k) { cols.push_back(ecol[k]); vals.push_back((R)eval[k]); }
                // pad the row to whole groups of four with zero entries on the
                // row itself (a finite value times zero)
                while (cols.size() % 4) { cols.push_back(row); vals.push_back((R)0); }
                if (cols.size() > 65535) throw std::runtime_error("slice segment too large");
                end[r] = (uint16_t)cols.size();
            }
            const size_t n = cols.size();
            const size_t n4 = (n + 3) & ~(size_t)3;
            const size_t per = 16 / sizeof(R);
            const size_t nv = (n + per - 1) / per * per;
            const size_t bytes = dev::kSegHeader + 4 * n4 + sizeof(R) * nv;
            buf.resize(off + bytes, 0);
            std::memcpy(buf.data() + off, end, sizeof(end));
            std::memcpy(buf.data() + off + dev::kSegHeader, cols.data(), 4 * n);
            std::memcpy(buf.data() + off + dev::kSegHeader + 4 * n4, vals.data(), sizeof(R) * n);
            if ((long)(bytes / 16) > 65535) throw std::runtime_error("slice segment too large");
            return {off / 16, (int)(bytes / 16)};
        };
        for (int s = 0; s < ns; ++s) {
            const auto lo = put(s, false);
            const auto up = put(s, true);
            if (lo.first > 2000000000L || up.first > 2000000000L) throw std::runtime_error("mesh too large for segments");
            work[s] = make_int4(s, (int)lo.first, (int)up.first, (lo.second << 16) | up.second);
            st_lo = std::max(st_lo, lo.second * 16);
            st_up = std::max(st_up, up.second * 16);
            st_spmv = std::max(st_spmv, (lo.second + up.second) * 16);
        }
        std::vector<int4> wc(colour_list.size());
        for (size_t i = 0; i < colour_list.size(); ++i) wc[i] = work[colour_list[i]];
        work.insert(work.end(), wc.begin(), wc.end());
    };
    std::vector<unsigned char> b64, b32;
    std::vector<int4> w64, w32;
    int l64, u64, s64, l32, u32, s32;
    build(double(0), b64, w64, l64, u64, s64);
    build(float(0), b32, w32, l32, u32, s32);
    d_seg64 = dupload(b64, stream);
    d_seg32 = dupload(b32, stream);
    d_work64 = dupload(w64, stream);
    d_work32 = dupload(w32, stream);
    d_seg_err = dalloc<unsigned>(1);
    cuda_ok(cudaMemsetAsync(d_seg_err, 0, sizeof(unsigned), stream), "memset");
    seg64 = dev::SegView<double>{d_seg64, d_work64, d_work64 + ns, s64, l64, u64, d_seg_err};
    seg32 = dev::SegView<float>{d_seg32, d_work32, d_work32 + ns, s32, l32, u32, d_seg_err};
    dc.seg_err = d_seg_err;
}

// Mixed precision: each step computes r = b - A x in FP64, solves A d = r
// with the complex-FP32 batched BiCGStab (scaled to unit norm, relative
// tolerance max(tol / ||r||_rel, inner_tol_floor)), and adds d to x in FP64.  Steps repeat
// until the FP64 true residual meets tol, the iteration budget is spent or a
// step fails to reduce the residual by 10 %.
//
// The FP32 solve runs only the right-hand sides that still need it, packed
// into the narrowest power-of-two batch (>= 2 lanes); whenever at most half of
// the lanes are still iterating, the survivors' x, r, r0, p, v and Krylov
// scalars are repacked into a batch half as wide (or narrower), after the
// finished lanes' corrections have been added to the FP64 x.  Converged
// systems then stop costing vector traffic; the matrix stream is shared by
// whatever remains.
// The graph of one 10-iteration chunk for the batch shape (K lanes in vector
// set x, form, gradient-space term): captured from the chunk's launches on
// first use, both streams included (the V-cycle branch joins the capture
// through its fork and join events), instantiated and kept until the end of
// the refinement step.  Every kernel argument of the chunk is fixed for a
// shape within a step (vectors, Krylov scalars and lane data stay where they
// are; a compaction changes the shape).  Returns the graph's index, or -1 if
// the capture failed, in which case nothing ran and chunks are launched
// directly from then on.
int GpuSolver::chunk_graph(int K, const void* x, bool eis, bool gc, const std::function<void()>& body) {
    for (size_t i = 0; i < chunk_graphs.size(); ++i) {
        const ChunkGraph& g = chunk_graphs[i];
        if (g.K == K && g.x == x && g.eis == eis && g.gc == gc) return (int)i;
    }
    const size_t t0 = timer.open.size();
    const long long l0 = launches;
    if (cudaStreamBeginCapture(stream, cudaStreamCaptureModeRelaxed) != cudaSuccess) {
        graphs_error = cudaGetErrorString(cudaGetLastError());
        graphs_failed = true;
        return -1;
    }
    std::string what;
    try {
        body();
    } catch (const std::exception& e) {
        what = e.what();
    }
    cudaGraph_t graph = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(stream, &graph);
    std::vector<KernelTimer::Pair> pairs = timer.take(t0);
    const long long nl = launches - l0;
    launches = l0;
    cudaGraphExec_t exec = nullptr;
    cudaError_t ei = cudaErrorUnknown;
    if (what.empty() && ec == cudaSuccess && graph) ei = cudaGraphInstantiate(&exec, graph, 0ULL);
    if (graph) cudaGraphDestroy(graph);
    if (!what.empty() || ec != cudaSuccess || ei != cudaSuccess) {
        graphs_error = !what.empty() ? what : cudaGetErrorString(ec != cudaSuccess ? ec : ei);
        cudaGetLastError();
        if (exec) cudaGraphExecDestroy(exec);
        timer.release(pairs);
        graphs_failed = true;
        return -1;
    }
    ChunkGraph g;
    g.K = K;
    g.x = x;
    g.eis = eis;
    g.gc = gc;
    g.exec = exec;
    g.launches = nl;
    g.pairs = std::move(pairs);
    chunk_graphs.push_back(std::move(g));
    return (int)chunk_graphs.size() - 1;
}

void GpuSolver::graphs_clear() {
    for (ChunkGraph& g : chunk_graphs) {
        if (g.exec) cudaGraphExecDestroy(g.exec);
        timer.release(g.pairs);
    }
    chunk_graphs.clear();
}

BatchResult GpuSolver::solve_batch_mixed(int K, const int* fmap, double2* b, double2* x,
                                         const std::vector<int>& active, double tol, int maxiter) {
    graphs_clear();   // graphs hold the arguments of the step that captured them
    ensure_vecs(K);
    ensure_vecs32(K);
    ensure_vecs32b(std::max(2, K / 2));
    const KrylovCtx<double> c64 = kctx(K, fmap);
    BatchResult R;
    R.K = K;
    R.iters.assign(K, 0); R.status.assign(K, kInactive); R.res.assign(K, 0.0); R.true_res.assign(K, 0.0);
    std::vector<int> run = active;
    std::vector<double> prev(K, 1e300), scale(K, 0.0);
    std::vector<BicgState> hs(K);
    const int chunk = 10;
    const int max_steps = 2 + std::max(0, P.max_refinements) * 4;
    auto pow2_at_least = [](int n) { int k = 2; while (k < n) k *= 2; return k; };
    auto launch_grid = [](long n) { return (int)((n + 255) / 256); };
    for (int step = 0; step <= max_steps; ++step) {
        // FP64 true residual y = b - A x
        for (int k = 0; k < K; ++k) {
            std::memset(&hs[k], 0, sizeof(BicgState));
            hs[k].status = active[k] ? kConverged : kInactive;
        }
        cuda_ok(cudaMemcpyAsync(d_states, hs.data(), sizeof(BicgState) * K, cudaMemcpyHostToDevice, stream), "states");
        spmv(c64, kSpmvTrueRes, x, kv.y, b, nullptr, d_states);
        cuda_ok(cudaMemcpyAsync(hs.data(), d_states, sizeof(BicgState) * K, cudaMemcpyDeviceToHost, stream), "states");
        sync();
        std::vector<int> lanes;   // current lane -> right-hand side of the FP64 batch
        for (int k = 0; k < K; ++k) {
            if (!active[k]) continue;
            const double rel = hs[k].true_res;
            R.true_res[k] = rel;
            R.res[k] = rel;
            if (!run[k]) continue;
            if (rel <= tol) { run[k] = 0; R.status[k] = kConverged; continue; }
            if (!std::isfinite(rel)) {   // non-finite values reached the iterate: report, stop this lane
                run[k] = 0;
                R.status[k] = kBreakdown;
                continue;
            }
            if (rel > 0.9 * prev[k] || R.iters[k] >= maxiter || step == max_steps) {
                run[k] = 0;
                if (R.status[k] == kInactive || R.status[k] == kConverged) R.status[k] = kMaxIter;
                continue;
            }
            prev[k] = rel;
            scale[k] = hs[k].rnorm;
            lanes.push_back(k);
        }
        if (lanes.empty()) break;
        int Kc = pow2_at_least((int)lanes.size());
        lanes.resize(Kc, -1);
        KrylovVecs<float> cur = kv32, other = kv32b;
        int cur_cap = kv32_K, other_cap = kv32b_K;
        if (Kc > other_cap) { /* start in the wide set */ } else { std::swap(cur, other); std::swap(cur_cap, other_cap); }
        // per-lane maps, scales and frequencies of the packed batch
        std::vector<int> map(dev::kMaxRhs, -1), add(dev::kMaxRhs, 0), fm(dev::kMaxRhs, 0);
        std::vector<double> sc(dev::kMaxRhs, 0.0);
        auto upload_lanes = [&](int Kn) {
            for (int j = 0; j < dev::kMaxRhs; ++j) {
                map[j] = (j < Kn) ? lanes[j] : -1;
                sc[j] = (j < Kn && lanes[j] >= 0) ? scale[lanes[j]] : 0.0;
                fm[j] = (j < Kn && lanes[j] >= 0) ? fmap[lanes[j]] : fmap[lanes[0] >= 0 ? lanes[0] : 0];
            }
            cuda_ok(cudaMemcpyAsync(d_lane_map, map.data(), sizeof(int) * dev::kMaxRhs, cudaMemcpyHostToDevice, stream), "map");
            cuda_ok(cudaMemcpyAsync(d_scale, sc.data(), sizeof(double) * dev::kMaxRhs, cudaMemcpyHostToDevice, stream), "scale");
        };
        // the gradient-space term needs the right-preconditioned form: a
        // batch with a corrected right-hand side runs that form throughout
        bool use_gc = false;
        if (gc_ok && P.gradcorr == 1 && gc.omega_max > 0.0)
            for (int j = 0; j < Kc; ++j)
                if (lanes[j] >= 0) {
                    const double om = 2.0 * kPi * fz_freqs[fmap[lanes[j]]];
                    use_gc |= om > 0.0 && om <= gc.omega_max;
                }
        const bool eis = !use_gc && P.ssor_form == 1 && P.row_kernels == kRowsStaged && P.ssor_relax == 1.0;
        // residual replacement needs the untransformed residual of the
        // right-preconditioned form
        const bool replace = P.residual_replacement == 1 && !eis;
        std::vector<double> rep_level(dev::kMaxRhs, 1.0);
        // flushes lanes with add[j] set: x64 += scale * d32, d32 the x-space
        // correction (x_hat mapped back by (D + U)^-1 in the Eisenstat form)
        auto flush = [&](const KrylovCtx<float>& cc, const KrylovVecs<float>& v, int Kn) {
            const float2* d = v.x;
            if (eis) {
                eis_finish(cc, v, v.sh);
                d = v.sh;
            }
            cuda_ok(cudaMemcpyAsync(d_lane_add, add.data(), sizeof(int) * dev::kMaxRhs, cudaMemcpyHostToDevice, stream), "add");
            k_add_f32_lanes<<<launch_grid((long)n_pad * Kn), 256, 0, stream>>>(x, K, d, Kn, d_lane_map, d_lane_add,
                                                                           d_scale, (long)n_pad);
            ++launches;
        };
        auto replace_lanes = [&](int Kn, const KrylovVecs<float>& v) {
            // d_lane_add holds the replaced lanes (uploaded by the flush)
#define M3D_REPLACE(KC)                                                                                        \
    {                                                                                                          \
        auto kf = k_replace_lanes<KC>;                                                                         \
        kf<<<wave_grid(kf, red.max_blocks, 256), 256, 0, stream>>>(kv.y, K, v.r, v.x, v.r0, d_lane_map,        \
                                                                   d_lane_add, d_scale, (long)n_pad, d_states, \
                                                                   red);                                       \
    }
            switch (Kn) {
                case 2: M3D_REPLACE(2) break;
                case 4: M3D_REPLACE(4) break;
                case 8: M3D_REPLACE(8) break;
                default: M3D_REPLACE(16) break;
            }
#undef M3D_REPLACE
            cuda_ok(cudaGetLastError(), "replace");
            ++launches;
        };
        upload_lanes(Kc);
        k_to_f32_lanes<<<launch_grid((long)n_pad * Kc), 256, 0, stream>>>(kv.y, K, cur.b, Kc, d_lane_map, d_scale,
                                                                      (long)n_pad);
        cuda_ok(cudaMemsetAsync(cur.x, 0, sizeof(float2) * (size_t)n_pad * Kc, stream), "memset");
        launches += 2;
        std::vector<BicgState> ls(Kc);
        for (int j = 0; j < Kc; ++j) {
            std::memset(&ls[j], 0, sizeof(BicgState));
            const int k = lanes[j];
            if (k < 0) { ls[j].status = kInactive; continue; }
            // with residual replacement the inner solve runs to the final
            // tolerance; without, to what complex FP32 reaches reliably
            ls[j].tol = std::min(0.5, std::max(tol / R.true_res[k], replace ? 0.25 * tol / R.true_res[k]
                                                                                    : P.inner_tol_floor));
            ls[j].maxiter = std::max(1, maxiter - R.iters[k]);
            ls[j].status = kRunning;
        }
        cuda_ok(cudaMemcpyAsync(d_states, ls.data(), sizeof(BicgState) * Kc, cudaMemcpyHostToDevice, stream), "states");
        KrylovCtx<float> c32 = kctx32(Kc, fm.data());
        if (use_gc) attach_gc(c32);
        if (eis) eis_init(c32, cur, d_states);
        else bicg_init(c32, cur, d_states);
        int it = 0;
        auto record = [&](int j) {   // lane j leaves the batch
            const int k = lanes[j];
            if (k < 0) return;
            R.iters[k] += ls[j].iter;
            if (ls[j].status == kBreakdown) R.status[k] = kBreakdown;
        };
        int pending_graph = -1;   // replayed graph whose timer pairs wait for this poll
        int chunks_of_shape = 0;  // chunks run since the batch shape last changed
        for (;;) {
            cuda_ok(cudaMemcpyAsync(ls.data(), d_states, sizeof(BicgState) * Kc, cudaMemcpyDeviceToHost, stream), "states");
            sync();
            if (pending_graph >= 0) {
                if (timer.on) timer.fold(chunk_graphs[pending_graph].pairs);
                pending_graph = -1;
            }
            int nrun = 0;
            for (int j = 0; j < Kc; ++j) nrun += (lanes[j] >= 0 && ls[j].status == kRunning);
            if (nrun == 0 || it >= maxiter) break;
            if (replace) {
                // lanes whose recursive residual fell 1000x since the last
                // replacement: flush x, FP64 true residual, replace r
                std::vector<int> rep(dev::kMaxRhs, 0);
                bool anyrep = false;
                for (int j = 0; j < Kc; ++j)
                    if (lanes[j] >= 0 && ls[j].status == kRunning && ls[j].res < 1e-3 * rep_level[j]) {
                        rep[j] = 1;
                        anyrep = true;
                    }
                if (anyrep) {
                    add = rep;
                    flush(c32, cur, Kc);
                    std::vector<BicgState> ts(K);
                    for (int k = 0; k < K; ++k) {
                        std::memset(&ts[k], 0, sizeof(BicgState));
                        ts[k].status = kInactive;
                    }
                    for (int j = 0; j < Kc; ++j)
                        if (rep[j]) ts[lanes[j]].status = kConverged;
                    cuda_ok(cudaMemcpyAsync(d_states2, ts.data(), sizeof(BicgState) * K, cudaMemcpyHostToDevice,
                                            stream), "states");
                    spmv(c64, kSpmvTrueRes, x, kv.y, b, nullptr, d_states2);
                    replace_lanes(Kc, cur);
                    for (int j = 0; j < Kc; ++j)
                        if (rep[j]) rep_level[j] = ls[j].res;
                    ++stats.replacements;
                    continue;   // re-read the states
                }
            }
            const int Kn = pow2_at_least(nrun);
            if (Kn < Kc && Kn <= other_cap) {
                // finished lanes: add their corrections and record them
                for (int j = 0; j < dev::kMaxRhs; ++j)
                    add[j] = (j < Kc && lanes[j] >= 0 && ls[j].status != kRunning) ? 1 : 0;
                flush(c32, cur, Kc);
                std::vector<int> sel(dev::kMaxRhs, -1), nl(Kn, -1);
                std::vector<BicgState> ns(Kn);
                int q = 0;
                for (int j = 0; j < Kc; ++j) {
                    if (lanes[j] < 0) continue;
                    if (ls[j].status == kRunning) { sel[q] = j; nl[q] = lanes[j]; ns[q] = ls[j]; ++q; }
                    else record(j);
                }
                for (; q < Kn; ++q) { std::memset(&ns[q], 0, sizeof(BicgState)); ns[q].status = kInactive; }
                cuda_ok(cudaMemcpyAsync(d_lane_sel, sel.data(), sizeof(int) * dev::kMaxRhs, cudaMemcpyHostToDevice, stream), "sel");
                LaneMove mv{};
                mv.nvec = 5;
                const float2* srcs[5] = {cur.x, cur.r, cur.r0, cur.p, cur.v};
                float2* dsts[5] = {other.x, other.r, other.r0, other.p, other.v};
                for (int v = 0; v < 5; ++v) { mv.src[v] = srcs[v]; mv.dst[v] = dsts[v]; }
                k_gather_lanes<<<launch_grid((long)n_pad * Kn), 256, 0, stream>>>(mv, Kc, Kn, d_lane_sel, (long)n_pad);
                ++launches;
                lanes = nl;
                ls = ns;
                cuda_ok(cudaMemcpyAsync(d_states, ls.data(), sizeof(BicgState) * Kn, cudaMemcpyHostToDevice, stream), "states");
                upload_lanes(Kn);
                std::swap(cur, other);
                std::swap(cur_cap, other_cap);
                Kc = Kn;
                c32 = kctx32(Kc, fm.data());
                if (use_gc) attach_gc(c32);
                chunks_of_shape = 0;
            }
            auto body = [&]() {
                for (int i = 0; i < chunk; ++i) {
                    if (eis) eis_iteration(c32, cur, d_states);
                    else bicg_iteration(c32, cur, d_states);
                }
            };
            // a shape is captured at its third chunk: short bursts (a few chunks
            // between divergence corrections) would not repay the capture
            ++chunks_of_shape;
            const int gi = (P.cuda_graphs && !graphs_failed && maxiter - it >= chunk && chunks_of_shape >= 3)
                               ? chunk_graph(Kc, cur.x, eis, use_gc, body) : -1;
            if (gi >= 0) {
                cuda_ok(cudaGraphLaunch(chunk_graphs[gi].exec, stream), "graph launch");
                launches += chunk_graphs[gi].launches;
                ++graph_replays;
                pending_graph = gi;
                it += chunk;
            } else {
                for (int i = 0; i < chunk && it < maxiter; ++i, ++it) {
                    if (eis) eis_iteration(c32, cur, d_states);
                    else bicg_iteration(c32, cur, d_states);
                }
            }
        }
        for (int j = 0; j < dev::kMaxRhs; ++j) add[j] = (j < Kc && lanes[j] >= 0) ? 1 : 0;
        flush(c32, cur, Kc);
        for (int j = 0; j < Kc; ++j) record(j);
        if (step > 0) ++stats.refinements;
        graphs_clear();
    }
    timer.collect();
    return R;
}

void GpuSolver::begin_call() {
    stats.forward_iterations = 0;
    stats.adjoint_iterations = 0;
    stats.refinements = 0;
    stats.replacements = 0;
    dcc = phys::DcCounters();
}

void GpuSolver::end_call() {
    stats.graphs_failed = graphs_failed ? 1 : 0;
    stats.graph_replays = graph_replays;
    stats.divcorr_calls = dcc.calls;
    stats.divcorr_outer = dcc.outer;
    stats.divcorr_cg_iterations = dcc.cg_iterations;
    stats.divcorr_cg_sweeps = dcc.cg_sweeps;
    stats.divcorr_setup_ms = amg_setup_ms;
    stats.kernel_launches = launches;
}

void GpuSolver::timer_start() { cuda_ok(cudaEventRecord(ev_start, stream), "event"); }

double GpuSolver::timer_stop() {
    cuda_ok(cudaEventRecord(ev_stop, stream), "event");
    cuda_ok(cudaEventSynchronize(ev_stop), "event");
    float ms = 0.f;
    cuda_ok(cudaEventElapsedTime(&ms, ev_start, ev_stop), "event");
    return ms;
}

// Algorithmic bytes of one divergence-correction call, from its counters:
// per outer round the divergence div(sigma E) (E read, edge mass, two
// incidence entries per edge, divJ written) and the update E -= G phi (E read
// and written, phi gathered); per PCG sweep of the Poisson solve the
// Laplacian product and the vector streams -- FP32 vectors and the packed
// 8-byte Laplacian entries (read by the product and twice by the level-0
// smoothing) in the mixed-precision solve, FP64 vectors with 12-byte CSR
// entries in the FP64 PCG.  Coarse multigrid levels are not counted.
double GpuSolver::divcorr_bytes(const phys::DcCounters& before, const phys::DcCounters& after, int K) const {
    const double n = L.ne, nn = L.nn, q = 2.0 * L.ne;
    const double outer = (double)(after.outer - before.outer);
    const double sweeps = (double)(after.cg_sweeps - before.cg_sweeps);
    const double round = (n * K * 16 + n * 8 + q * 12 + nn * K * 16) + (2 * n * K * 16 + q * 12 + nn * K * 16);
    const double sweep = P.divcorr_mixed && P.divcorr_precond ? 10.0 * nn * K * 8 + 3.0 * 8 * q
                                                              : 8.0 * nn * K * 16 + q * 12 + nn * 8;
    return outer * round + sweeps * sweep;
}

// Algorithmic bytes of one sensitivity launch over `lanes` (E, lambda) pairs:
// both fields once, the cell->edge map (about 12 index + weight entries per
// cell), sigma read and the gradient read and written.
double GpuSolver::sens_bytes(int lanes) const {
    return 2.0 * L.ne * 16.0 * lanes + (double)L.nc * (12.0 * 12.0) + 24.0 * L.nc;
}

// ---------------------------------------------------------------------------
// forward: solve_frequency (forward_solver_fv.cpp:84-531) for nf frequencies
// ---------------------------------------------------------------------------

void GpuSolver::run_forward(const std::vector<double>& freqs, double* Z_out) {
    if (!stations_set) throw std::logic_error("stations not set (m3d_set_stations)");
    const int nf = (int)freqs.size();
    const int Kreal = 2 * nf;
    if (Kreal > dev::kMaxRhs) throw std::invalid_argument("at most 8 frequencies per forward group");
    const int K = pow2_at_least(Kreal);
    const auto t0 = std::chrono::steady_clock::now();
    factorize(freqs);
    ensure_vecs(K);
    ensure_fields(K);
    ensure_E(K);
    ensure_hc(nf);
    std::vector<int> fmap(K, 0), pol(K, -1), active(K, 0);
    for (int k = 0; k < Kreal; ++k) { fmap[k] = k / 2; pol[k] = k % 2; active[k] = 1; }
    const RhsInfo info = rhs_info(K, fmap, pol, freqs);
    const KrylovCtx<double> c = kctx(K, fmap.data());
    const VecK Ebc{d_Ebc, K}, Epri{d_Epri, K}, rhs{d_rhs, K}, tmp{d_tmp, K}, E{d_E, K}, X{kv.x, K};
    phys::primary_field(md, Ebc, info, true, stream);
    phys::lift_rhs(md, Ebc, rhs, stream);
    phys::primary_field(md, Epri, info, false, stream);
    spmv(c, kSpmvPlain, d_Epri, d_tmp, nullptr, nullptr, nullptr);
    phys::vsub((long)n_pad * K, d_rhs, d_tmp, kv.b, stream);
    cuda_ok(cudaMemsetAsync(kv.x, 0, sizeof(double2) * (size_t)n_pad * K, stream), "memset");
    launches += 5;
    BatchResult R;
    if (P.forward_interleaved && P.div_correction) {
        // the forward system solved like the adjoint one (ModEM-style bursts
        // with divergence correction, source divergence G^T rhs_sec / (i omega))
        R.K = K;
        R.iters.assign(K, 0); R.status.assign(K, 0); R.res.assign(K, 0.0); R.true_res.assign(K, 0.0);
        solve_divcorr(K, fmap.data(), info, kv.b, kv.x, active, P.bicgstab_tol, R.iters, R.status, R.true_res);
        for (int k = 0; k < K; ++k) if (R.status[k] == M3D_SOLVE_CONVERGED) R.status[k] = kConverged;
    } else {
        R = solve_any(K, fmap.data(), kv.b, kv.x, active, P.bicgstab_tol, P.bicgstab_maxiter);
    }
    phys::interpolate_hanging(md, X, hp_sequential, stream);
    phys::combine_total(md, Epri, X, Ebc, E, stream);
    launches += 2;
    if (P.div_correction) {
        ensure_dc(K);
        const int th = timer.on ? timer.begin(kClsDivcorr, 0.0, K) : -1;
        const phys::DcCounters dc0 = dcc;
        launches += phys::divcorr(md, d_me_dc, E, false, dc, P.div_corr_iters, P.div_corr_tol, active.data(),
                                  red, stream, 25, &dcc, amg_or_null(), mixed_or_null());
        timer.end(th);
        timer.set_bytes(th, divcorr_bytes(dc0, dcc, K));
    }
    phys::station_impedance(sd, E, d_omegas, nf, d_hc, d_Z, stream);
    ++launches;
    if (Z_out)
        cuda_ok(cudaMemcpyAsync(Z_out, d_Z, sizeof(double2) * 4 * (size_t)sd.ns * nf, cudaMemcpyDeviceToHost, stream), "Z");
    sync();
    E_K = K;
    E_nf = nf;
    stats.n_rhs = Kreal;
    stats.total_iterations = 0;
    for (int k = 0; k < Kreal; ++k) stats.forward_iterations += R.iters[k];
    for (int k = 0; k < Kreal && k < 64; ++k) {
        stats.iterations[k] = R.iters[k];
        stats.status[k] = R.status[k];
        stats.true_residual[k] = R.true_res[k];
        stats.total_iterations += R.iters[k];
    }
    stats.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    stats.kernel_launches = launches;
}

void GpuSolver::compute_single_frequency(double freq, double* Z_out) {
    begin_call();
    run_forward(std::vector<double>{freq}, Z_out);
    end_call();
}

void GpuSolver::background_E(int pol, double* out) {
    if (!d_E || E_nf < 1) throw std::logic_error("no forward solution");
    const int k = 2 * (E_nf - 1) + pol;
    phys::from_permuted(md, VecK{d_E, E_K}, k, d_host_stage, stream);
    cuda_ok(cudaMemcpyAsync(out, d_host_stage, sizeof(double2) * L.ne, cudaMemcpyDeviceToHost, stream), "E");
    sync();
}

void GpuSolver::set_background(const double* E1, const double* E2) {
    ensure_fields(2);
    ensure_E(2);
    cuda_ok(cudaMemsetAsync(d_E, 0, sizeof(double2) * (size_t)n_pad * 2, stream), "memset");
    for (int p = 0; p < 2; ++p) {
        cuda_ok(cudaMemcpyAsync(d_host_stage, p == 0 ? E1 : E2, sizeof(double2) * L.ne, cudaMemcpyHostToDevice, stream), "E");
        phys::to_permuted(md, d_host_stage, 2, p, VecK{d_E, 2}, stream);
    }
    E_K = 2;
    E_nf = 1;
    sync();
}

void GpuSolver::build_adjoint_rhs(const double* wr, double* rhs1, double* rhs2) {
    if (E_nf != 1 || !d_hc) throw std::logic_error("adjoint source needs a solved single frequency");
    ensure_fields(2);
    cuda_ok(cudaMemcpyAsync(d_wr, wr, sizeof(double2) * 4 * (size_t)sd.ns, cudaMemcpyHostToDevice, stream), "wr");
    cuda_ok(cudaMemsetAsync(d_adj, 0, sizeof(double2) * (size_t)n_pad * 2, stream), "memset");
    phys::adjoint_rhs(sd, md, d_wr, d_hc, d_omegas + (fz_freqs.size() - 1), 1, VecK{d_adj, 2}, stream);
    for (int p = 0; p < 2; ++p) {
        phys::from_permuted(md, VecK{d_adj, 2}, p, d_host_stage, stream);
        cuda_ok(cudaMemcpyAsync(p == 0 ? rhs1 : rhs2, d_host_stage, sizeof(double2) * L.ne, cudaMemcpyDeviceToHost, stream), "rhs");
        sync();
    }
}

// solve_with_divcorr_ (forward_solver_fv.cpp:778-888) for every active rhs:
// initial correction with phi0 = G^T rhs / (i omega), then bursts of at most
// divcorr_iter_per_dc BiCGStab iterations, each followed by a correction and
// an FP64 true-residual test, with the reference's divergence (res > 1 ->
// zero) and stagnation (> 0.95 of the previous residual) exits.
void GpuSolver::solve_divcorr(int K, const int* fmap, const RhsInfo& info, double2* rhs, double2* x,
                              const std::vector<int>& active, double tol, std::vector<int>& iters,
                              std::vector<int>& status, std::vector<double>& tres) {
    const KrylovCtx<double> c = kctx(K, fmap);
    ensure_dc(K);
    ensure_vecs(K);
    phys::dc_phi0(md, VecK{rhs, K}, info, dc, stream);
    ++launches;
    int th = timer.on ? timer.begin(kClsDivcorr, 0.0, K) : -1;
    {
        const phys::DcCounters dc0 = dcc;
        launches += phys::divcorr(md, d_me_dc, VecK{x, K}, true, dc, P.div_corr_iters, P.div_corr_tol,
                                  active.data(), red, stream, 25, &dcc, amg_or_null(), mixed_or_null());
        timer.end(th);
        timer.set_bytes(th, divcorr_bytes(dc0, dcc, K));
    }
    std::vector<int> done(K, 0);
    std::vector<double> prev(K, 1e30);
    for (int k = 0; k < K; ++k) done[k] = !active[k];
    for (int outer = 0; outer < P.divcorr_outer_max; ++outer) {
        std::vector<int> act(K, 0);
        bool any = false;
        for (int k = 0; k < K; ++k) { act[k] = !done[k]; any |= act[k] != 0; }
        if (!any) break;
        BatchResult R = solve_any(K, fmap, rhs, x, act, tol, P.divcorr_iter_per_dc);
        std::vector<int> dca(K, 0);
        for (int k = 0; k < K; ++k) {
            if (!act[k]) continue;
            iters[k] += R.iters[k];
            tres[k] = R.true_res[k];
            status[k] = R.status[k];
            if (R.res[k] > 1.0) {
                k_zero_col<<<(n_pad + 255) / 256, 256, 0, stream>>>(x, K, k, n_pad);
                ++launches;
                status[k] = M3D_SOLVE_DIVERGED;
                done[k] = 1;
            } else if (R.status[k] == kConverged) {
                done[k] = 1;
            } else {
                dca[k] = 1;
            }
        }
        bool anyd = false;
        for (int k = 0; k < K; ++k) anyd |= dca[k] != 0;
        if (!anyd) break;
        th = timer.on ? timer.begin(kClsDivcorr, 0.0, K) : -1;
        const phys::DcCounters dc0 = dcc;
        launches += phys::divcorr(md, d_me_dc, VecK{x, K}, true, dc, P.div_corr_iters, P.div_corr_tol,
                                  dca.data(), red, stream, 25, &dcc, amg_or_null(), mixed_or_null());
        timer.end(th);
        timer.set_bytes(th, divcorr_bytes(dc0, dcc, K));
        std::vector<BicgState> hs(K);
        for (int k = 0; k < K; ++k) {
            std::memset(&hs[k], 0, sizeof(BicgState));
            hs[k].status = dca[k] ? kConverged : kInactive;
        }
        cuda_ok(cudaMemcpyAsync(d_states2, hs.data(), sizeof(BicgState) * K, cudaMemcpyHostToDevice, stream), "st");
        spmv(c, kSpmvTrueRes, x, kv.y, rhs, nullptr, d_states2);
        cuda_ok(cudaMemcpyAsync(hs.data(), d_states2, sizeof(BicgState) * K, cudaMemcpyDeviceToHost, stream), "st");
        sync();
        for (int k = 0; k < K; ++k) {
            if (!dca[k]) continue;
            const double rel = hs[k].true_res;
            tres[k] = rel;
            if (rel < tol) { done[k] = 1; status[k] = M3D_SOLVE_CONVERGED; }
            else if (outer > 0 && rel > 0.95 * prev[k]) { done[k] = 1; status[k] = M3D_SOLVE_STAGNATED; }
            prev[k] = rel;
        }
    }
    timer.collect();
}

// adjoint_solve / solve_rhs (forward_solver_fv.cpp:914-940): solve_with_divcorr_
// when divergence correction is on, else solve_system_ (:727-759)
void GpuSolver::run_adjoint(int K, const int* fmap, const RhsInfo& info, double2* rhs, double2* x,
                            const std::vector<int>& active) {
    const double tol = tol_override > 0 ? tol_override : P.bicgstab_tol;
    cuda_ok(cudaMemsetAsync(x, 0, sizeof(double2) * (size_t)n_pad * K, stream), "memset");
    stats.n_rhs = 0;
    stats.total_iterations = 0;
    std::vector<int> iters(K, 0), status(K, 0);
    std::vector<double> tres(K, 0.0);
    if (P.div_correction && current_omega > 0) {
        solve_divcorr(K, fmap, info, rhs, x, active, tol, iters, status, tres);
    } else {
        BatchResult R = solve_any(K, fmap, rhs, x, active, tol, P.bicgstab_maxiter);
        for (int k = 0; k < K; ++k) {
            if (!active[k]) continue;
            iters[k] = R.iters[k]; status[k] = R.status[k]; tres[k] = R.true_res[k];
            if (R.status[k] != kConverged && R.res[k] > 1.0) {
                k_zero_col<<<(n_pad + 255) / 256, 256, 0, stream>>>(x, K, k, n_pad);
                ++launches;
                status[k] = M3D_SOLVE_DIVERGED;
            }
        }
    }
    sync();
    int nr = 0;
    for (int k = 0; k < K; ++k) {
        if (!active[k]) continue;
        if (nr < 64) { stats.iterations[nr] = iters[k]; stats.status[nr] = status[k]; stats.true_residual[nr] = tres[k]; }
        stats.total_iterations += iters[k];
        ++nr;
    }
    stats.n_rhs = nr;
    stats.adjoint_iterations += stats.total_iterations;
    stats.kernel_launches = launches;
}

void GpuSolver::adjoint_solve(const double* rhs_h, double* out, bool perturbation) {
    (void)perturbation;
    if (fz_freqs.empty()) throw std::logic_error("no factorised frequency");
    const auto t0 = std::chrono::steady_clock::now();
    begin_call();
    ensure_fields(2);
    ensure_vecs(2);
    const int K = 2;
    // use the last factorised frequency (diag slot)
    const int fslot = (int)fz_freqs.size() - 1;
    std::vector<int> fmap(K, fslot), pol(K, -1), active{1, 0};
    RhsInfo info = rhs_info(K, fmap, pol, fz_freqs);
    cuda_ok(cudaMemsetAsync(d_adj, 0, sizeof(double2) * (size_t)n_pad * K, stream), "memset");
    cuda_ok(cudaMemcpyAsync(d_host_stage, rhs_h, sizeof(double2) * L.ne, cudaMemcpyHostToDevice, stream), "rhs");
    phys::to_permuted(md, d_host_stage, K, 0, VecK{d_adj, K}, stream);
    run_adjoint(K, fmap.data(), info, d_adj, d_lam, active);
    phys::from_permuted(md, VecK{d_lam, K}, 0, d_host_stage, stream);
    cuda_ok(cudaMemcpyAsync(out, d_host_stage, sizeof(double2) * L.ne, cudaMemcpyDeviceToHost, stream), "lam");
    sync();
    end_call();
    stats.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

// Many right-hand sides at the factorised frequency, 16 lanes per batched
// solve_with_divcorr_ (the per-RHS path of adjoint_solve / solve_rhs).
void GpuSolver::solve_rhs_batch(const double* rhs_h, int n_rhs, double* out) {
    if (fz_freqs.empty()) throw std::logic_error("no factorised frequency");
    const auto t0 = std::chrono::steady_clock::now();
    begin_call();
    const int fslot = (int)fz_freqs.size() - 1;
    std::vector<int> all_it, all_st;
    std::vector<double> all_tr;
    long long it_total = 0;
    const int blk = std::max(2, std::min(dev::kMaxRhs, rhs_block));
    for (int r0 = 0; r0 < n_rhs; r0 += blk) {
        const int g = std::min(blk, n_rhs - r0);
        const int K = pow2_at_least(std::max(2, g));
        ensure_fields(K);
        ensure_vecs(K);
        std::vector<int> fmap(K, fslot), pol(K, -1), active(K, 0);
        for (int k = 0; k < g; ++k) active[k] = 1;
        RhsInfo info = rhs_info(K, fmap, pol, fz_freqs);
        cuda_ok(cudaMemsetAsync(d_adj, 0, sizeof(double2) * (size_t)n_pad * K, stream), "memset");
        for (int k = 0; k < g; ++k) {
            cuda_ok(cudaMemcpyAsync(d_host_stage, rhs_h + (size_t)(r0 + k) * 2 * L.ne, sizeof(double2) * L.ne,
                                    cudaMemcpyHostToDevice, stream), "rhs");
            phys::to_permuted(md, d_host_stage, K, k, VecK{d_adj, K}, stream);
        }
        run_adjoint(K, fmap.data(), info, d_adj, d_lam, active);
        it_total += stats.total_iterations;
        for (int k = 0; k < stats.n_rhs && k < 64; ++k) {
            all_it.push_back(stats.iterations[k]);
            all_st.push_back(stats.status[k]);
            all_tr.push_back(stats.true_residual[k]);
        }
        for (int k = 0; k < g; ++k) {
            phys::from_permuted(md, VecK{d_lam, K}, k, d_host_stage, stream);
            cuda_ok(cudaMemcpyAsync(out + (size_t)(r0 + k) * 2 * L.ne, d_host_stage, sizeof(double2) * L.ne,
                                    cudaMemcpyDeviceToHost, stream), "out");
            sync();   // the staging buffer is reused by the next lane
        }
    }
    stats.total_iterations = (int)it_total;
    stats.n_rhs = (int)all_it.size();
    for (size_t k = 0; k < all_it.size() && k < 64; ++k) {
        stats.iterations[k] = all_it[k];
        stats.status[k] = all_st[k];
        stats.true_residual[k] = all_tr[k];
    }
    stats.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    end_call();
}

// Gradients of many residual sources at the solved single frequency, one per
// source: for source j, build_adjoint_rhs_from_residual(wr_j)
// (forward_solver_fv.cpp:1804-2013), both polarisations' adjoint solves
// (adjoint_solve_complex -> solve_with_divcorr_, :914-924) and
// compute_sensitivity_complex (:989-1059) of each, summed over the two
// polarisations as InversionFV::compute_gradient_ sums them
// (inversion_fv.cpp:280-290).  With wr_j non-zero at one station this is
// that station's row of J^T W^2 r.  Eight sources (sixteen right-hand sides)
// per batch, built, solved and reduced on the device: only wr goes in and g
// comes out.  wr [n_src][ns][4] complex, g [n_src][nc].
void GpuSolver::station_gradients(const double* wr_h, int n_src, double* g_out) {
    if (E_nf != 1 || !d_hc || fz_freqs.empty())
        throw std::logic_error("station gradients need a solved single frequency");
    if (n_src < 0) throw std::invalid_argument("n_src < 0");
    const auto t0 = std::chrono::steady_clock::now();
    begin_call();
    const int ns = sd.ns;
    const int fslot = (int)fz_freqs.size() - 1;
    if (src_ns != ns) {
        dfree(d_src_wr); dfree(d_src_g);
        d_src_wr = dalloc<double2>((size_t)8 * std::max(1, ns) * 4);
        d_src_g = dalloc<double>((size_t)8 * L.nc);
        src_ns = ns;
    }
    std::vector<int> all_it, all_st;
    std::vector<double> all_tr;
    long long it_total = 0;
    for (int j0 = 0; j0 < n_src; j0 += 8) {
        const int g = std::min(8, n_src - j0);
        const int K = pow2_at_least(2 * g);
        ensure_fields(K);
        ensure_vecs(K);
        cuda_ok(cudaMemcpyAsync(d_src_wr, wr_h + (size_t)j0 * ns * 8, sizeof(double2) * (size_t)g * ns * 4,
                                cudaMemcpyHostToDevice, stream), "wr");
        cuda_ok(cudaMemsetAsync(d_adj, 0, sizeof(double2) * (size_t)n_pad * K, stream), "memset");
        phys::adjoint_rhs_sources(sd, d_src_wr, d_hc, d_omegas + fslot, g, VecK{d_adj, K}, stream);
        ++launches;
        std::vector<int> fmap(K, fslot), pol(K, -1), active(K, 0);
        for (int k = 0; k < 2 * g; ++k) active[k] = 1;
        RhsInfo info = rhs_info(K, fmap, pol, fz_freqs);
        run_adjoint(K, fmap.data(), info, d_adj, d_lam, active);
        it_total += stats.total_iterations;
        for (int k = 0; k < stats.n_rhs; ++k) {
            all_it.push_back(stats.iterations[k]);
            all_st.push_back(stats.status[k]);
            all_tr.push_back(stats.true_residual[k]);
        }
        {
            const int ts = timer.on ? timer.begin(kClsSens, sens_bytes(2 * g), K) : -1;
            phys::sensitivity_sources(md, d_sigma, VecK{d_E, E_K}, 0, VecK{d_lam, K}, d_omegas + fslot, g, d_src_g,
                                      stream);
            timer.end(ts);
        }
        ++launches;
        cuda_ok(cudaMemcpyAsync(g_out + (size_t)j0 * L.nc, d_src_g, sizeof(double) * (size_t)g * L.nc,
                                cudaMemcpyDeviceToHost, stream), "g");
        sync();
    }
    stats.total_iterations = (int)it_total;
    stats.n_rhs = (int)all_it.size();
    for (size_t k = 0; k < all_it.size() && k < 64; ++k) {
        stats.iterations[k] = all_it[k];
        stats.status[k] = all_st[k];
        stats.true_residual[k] = all_tr[k];
    }
    stats.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    end_call();
}

void GpuSolver::sensitivity(const double* E_h, const double* lam_h, double* g) {
    ensure_fields(2);
    cuda_ok(cudaMemsetAsync(d_tmp, 0, sizeof(double2) * (size_t)n_pad * 2, stream), "memset");
    cuda_ok(cudaMemcpyAsync(d_host_stage, E_h, sizeof(double2) * L.ne, cudaMemcpyHostToDevice, stream), "E");
    phys::to_permuted(md, d_host_stage, 2, 0, VecK{d_tmp, 2}, stream);
    cuda_ok(cudaMemcpyAsync(d_host_stage, lam_h, sizeof(double2) * L.ne, cudaMemcpyHostToDevice, stream), "lam");
    phys::to_permuted(md, d_host_stage, 2, 1, VecK{d_tmp, 2}, stream);
    // lambda sits in column 1: view it through a shifted pointer with the same stride
    cuda_ok(cudaMemsetAsync(d_grad, 0, sizeof(double) * L.nc, stream), "memset");
    double om = current_omega;
    cuda_ok(cudaMemcpyAsync(d_stage_real, &om, sizeof(double), cudaMemcpyHostToDevice, stream), "om");
    phys::sensitivity(md, d_sigma, VecK{d_tmp, 2}, VecK{d_tmp + 1, 2}, d_stage_real, 1, 1, d_grad, stream);
    cuda_ok(cudaMemcpyAsync(g, d_grad, sizeof(double) * L.nc, cudaMemcpyDeviceToHost, stream), "g");
    sync();
}

void GpuSolver::perturbation_rhs(int pol, const double* dsig, double* out) {
    if (E_nf < 1) throw std::logic_error("no background field");
    ensure_fields(2);
    cuda_ok(cudaMemcpyAsync(d_stage_real, dsig, sizeof(double) * L.nc, cudaMemcpyHostToDevice, stream), "dsig");
    const int kE = 2 * (E_nf - 1) + (pol == 1 ? 0 : 1);
    phys::perturbation_rhs(md, d_sigma, d_stage_real, VecK{d_E, E_K}, kE, current_omega, VecK{d_tmp, 2}, 0, stream);
    phys::from_permuted(md, VecK{d_tmp, 2}, 0, d_host_stage, stream);
    cuda_ok(cudaMemcpyAsync(out, d_host_stage, sizeof(double2) * L.ne, cudaMemcpyDeviceToHost, stream), "out");
    sync();
}

void GpuSolver::delta_impedance(const double* dE, int pol, double* dZ) {
    if (E_nf != 1 || !d_hc) throw std::logic_error("delta impedance needs a solved single frequency");
    ensure_fields(2);
    cuda_ok(cudaMemsetAsync(d_tmp, 0, sizeof(double2) * (size_t)n_pad * 2, stream), "memset");
    cuda_ok(cudaMemcpyAsync(d_host_stage, dE, sizeof(double2) * L.ne, cudaMemcpyHostToDevice, stream), "dE");
    phys::to_permuted(md, d_host_stage, 2, 0, VecK{d_tmp, 2}, stream);
    phys::delta_impedance(sd, VecK{d_tmp, 2}, 0, d_hc, pol, d_wr, stream);
    cuda_ok(cudaMemcpyAsync(dZ, d_wr, sizeof(double2) * 4 * (size_t)sd.ns, cudaMemcpyDeviceToHost, stream), "dZ");
    sync();
}

void GpuSolver::release() {
    fz_freqs.clear();
    E_nf = 0;
}

void GpuSolver::dot_batched(const double2* x, const double2* y, long long n, int K, double2* out) {
    cuda_ok(cudaSetDevice(device), "cudaSetDevice");
    const int cap = std::min(dev::kDotMaxBlocks, red.max_blocks);
    cuda_ok(dev::launch_dot_batched(x, y, n, K, cap, red, out, stream), "dot launch");
    ++launches;
    sync();
}

// ---------------------------------------------------------------------------
// batched entry points
// ---------------------------------------------------------------------------

void GpuSolver::forward_batch(const double* freqs, int nf, double* Z_out, double* E_out) {
    if (nf < 1) throw std::invalid_argument("no frequencies");
    const auto t0 = std::chrono::steady_clock::now();
    begin_call();
    long long it_total = 0;
    for (int f0 = 0; f0 < nf; f0 += 8) {
        const int g = std::min(8, nf - f0);
        std::vector<double> fr(freqs + f0, freqs + f0 + g);
        run_forward(fr, Z_out ? Z_out + (size_t)f0 * sd.ns * 8 : nullptr);
        it_total += stats.total_iterations;
        if (E_out) {
            for (int k = 0; k < 2 * g; ++k) {
                phys::from_permuted(md, VecK{d_E, E_K}, k, d_host_stage, stream);
                cuda_ok(cudaMemcpyAsync(E_out + ((size_t)(f0 * 2 + k)) * L.ne * 2, d_host_stage,
                                        sizeof(double2) * L.ne, cudaMemcpyDeviceToHost, stream), "E");
            }
            sync();
        }
    }
    stats.total_iterations = (int)it_total;
    stats.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    end_call();
}

// ImplicitJtJOperatorFV::Mult (implicit_jtj_fv.cpp:78-192) without the
// regularisation term, for the frequencies whose background fields are
// resident: every perturbation solve of the product in one batched solve and
// every adjoint solve in a second, at the relaxed tolerance of :113.
void GpuSolver::jtjv_batch(const double* freqs, int nf, const double* dsigma, const double* err, double inner_tol,
                           double* out) {
    if (E_nf != nf || (int)fz_freqs.size() != nf || E_K < 2 * nf || !d_hc)
        throw std::logic_error("no resident background fields for these frequencies (m3d_forward_batch first)");
    for (int f = 0; f < nf; ++f)
        if (fz_freqs[f] != freqs[f])
            throw std::logic_error("no resident background fields for these frequencies (m3d_forward_batch first)");
    const auto t0 = std::chrono::steady_clock::now();
    begin_call();
    const int ns = sd.ns;
    const int K = E_K;
    const size_t nv = (size_t)n_pad * dev::kMaxRhs;
    if (!d_jtj_rhs) {
        d_jtj_rhs = dalloc<double2>(nv); d_jtj_dE = dalloc<double2>(nv);
        d_jtj_a = dalloc<double2>(nv); d_jtj_b = dalloc<double2>(nv);
        d_jtj_ds = dalloc<double>((size_t)L.nc);
    }
    if (jtj_ns != ns) {   // station-sized buffers follow the current station set
        dfree(d_jtj_dz); dfree(d_jtj_wr0); dfree(d_jtj_wr1); dfree(d_jtj_err);
        d_jtj_dz = dalloc<double2>((size_t)dev::kMaxRhs * std::max(1, ns) * 4);
        d_jtj_wr0 = dalloc<double2>((size_t)8 * std::max(1, ns) * 4);
        d_jtj_wr1 = dalloc<double2>((size_t)8 * std::max(1, ns) * 4);
        d_jtj_err = dalloc<double>((size_t)8 * std::max(1, ns) * 4);
        jtj_ns = ns;
    }
    ensure_fields(K);
    cuda_ok(cudaMemcpyAsync(d_jtj_ds, dsigma, sizeof(double) * L.nc, cudaMemcpyHostToDevice, stream), "dsigma");
    cuda_ok(cudaMemcpyAsync(d_jtj_err, err, sizeof(double) * (size_t)ns * nf * 4, cudaMemcpyHostToDevice, stream),
            "err");
    cuda_ok(cudaMemsetAsync(d_grad, 0, sizeof(double) * L.nc, stream), "memset");
    const double tol_saved = tol_override;
    tol_override = inner_tol;
    struct Restore {
        double& t;
        double v;
        ~Restore() { t = v; }
    } restore{tol_override, tol_saved};
    std::vector<int> fmap(K, 0), pol(K, -1), active(K, 0);
    for (int k = 0; k < 2 * nf; ++k) { fmap[k] = k / 2; active[k] = 1; }
    std::vector<double> fr(freqs, freqs + nf);
    RhsInfo info = rhs_info(K, fmap, pol, fr);
    current_omega = 2.0 * kPi * fr[0];
    long long it_total = 0;
    std::vector<int> all_it, all_st;
    std::vector<double> all_tr;
    auto keep = [&]() {
        for (int k = 0; k < stats.n_rhs && k < 64; ++k) {
            all_it.push_back(stats.iterations[k]);
            all_st.push_back(stats.status[k]);
            all_tr.push_back(stats.true_residual[k]);
        }
    };
    // J.v: perturbation right-hand sides (:127-130) and their solves (:133)
    cuda_ok(cudaMemsetAsync(d_jtj_rhs, 0, sizeof(double2) * (size_t)n_pad * K, stream), "memset");
    for (int k = 0; k < 2 * nf; ++k)
        phys::perturbation_rhs(md, d_sigma, d_jtj_ds, VecK{d_E, E_K}, k, 2.0 * kPi * fr[k / 2],
                               VecK{d_jtj_rhs, K}, k, stream);
    launches += 2 * nf;
    run_adjoint(K, fmap.data(), info, d_jtj_rhs, d_jtj_dE, active);
    it_total += stats.total_iterations;
    keep();
    // delta Z (:136) and its weighting (:139-150)
    for (int k = 0; k < 2 * nf; ++k)
        phys::delta_impedance(sd, VecK{d_jtj_dE, K}, k, d_hc + (size_t)(k / 2) * ns, k % 2 + 1,
                              d_jtj_dz + (size_t)k * ns * 4, stream);
    phys::jtj_weight(ns, nf, d_jtj_err, d_jtj_dz, d_jtj_wr0, d_jtj_wr1, stream);
    launches += 2 * nf + 1;
    // J^T: adjoint source of polarisation p from the weighted dZ of
    // perturbation p (:154-164), adjoint solve, sensitivity (:167-175)
    cuda_ok(cudaMemsetAsync(d_jtj_a, 0, sizeof(double2) * (size_t)n_pad * K, stream), "memset");
    cuda_ok(cudaMemsetAsync(d_jtj_b, 0, sizeof(double2) * (size_t)n_pad * K, stream), "memset");
    phys::adjoint_rhs(sd, md, d_jtj_wr0, d_hc, d_omegas, nf, VecK{d_jtj_a, K}, stream);
    phys::adjoint_rhs(sd, md, d_jtj_wr1, d_hc, d_omegas, nf, VecK{d_jtj_b, K}, stream);
    phys::pick_pol_lanes(n_pad, K, d_jtj_a, d_jtj_b, d_adj, stream);
    launches += 3;
    run_adjoint(K, fmap.data(), info, d_adj, d_lam, active);
    it_total += stats.total_iterations;
    keep();
    {
        const int ts = timer.on ? timer.begin(kClsSens, sens_bytes(2 * nf), K) : -1;
        phys::sensitivity(md, d_sigma, VecK{d_E, K}, VecK{d_lam, K}, d_omegas, nf, 2, d_grad, stream);
        timer.end(ts);
    }
    ++launches;
    cuda_ok(cudaMemcpyAsync(out, d_grad, sizeof(double) * L.nc, cudaMemcpyDeviceToHost, stream), "out");
    sync();
    stats.total_iterations = (int)it_total;
    stats.n_rhs = (int)all_it.size();
    for (size_t k = 0; k < all_it.size() && k < 64; ++k) {
        stats.iterations[k] = all_it[k];
        stats.status[k] = all_st[k];
        stats.true_residual[k] = all_tr[k];
    }
    stats.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    end_call();
}

// ---------------------------------------------------------------------------
// octree model regularisation (regularization_octree.cpp)
// ---------------------------------------------------------------------------

void GpuSolver::reg_free() {
    if (stream) cudaStreamSynchronize(stream);
    for (void* p : reg_mem) cudaFree(p);
    reg_mem.clear();
    reg = RegDev{};
    reg_ok = false;
    d_reg_in = d_reg_out = d_reg_ref = nullptr;
}

void GpuSolver::reg_setup(const RegParams& p) {
    if (!ready) throw std::logic_error("solver not set up");
    reg_free();
    reg_build(L, p, reg_host);
    const RegHost& R = reg_host;
    auto up = [&](const auto& v) {
        auto* q = dupload(v, stream);
        reg_mem.push_back((void*)q);
        return q;
    };
    auto scratch = [&](size_t n) {
        double* q = dalloc<double>(std::max<size_t>(1, n));
        reg_mem.push_back((void*)q);
        return q;
    };
    reg.nc = R.nc;
    reg.na = R.na;
    reg.n_smooth = p.n_smooth;
    reg.alpha_s = p.alpha_s;
    reg.a2g = up(R.a2g);
    reg.ptr = up(R.ptr);
    reg.idx = up(R.idx);
    reg.val = up(R.val);
    reg.aptr = up(R.aptr);
    reg.aidx = up(R.aidx);
    reg.aw = up(R.aw);
    reg.diagw = up(R.diagw);
    reg.t0 = scratch(R.na);
    reg.t1 = scratch(R.na);
    reg.t2 = scratch(R.na);
    reg.dot = scratch(1);
    const size_t nio = (size_t)std::max(R.na, R.nc);
    d_reg_in = scratch(nio);
    d_reg_out = scratch(nio);
    d_reg_ref = scratch(R.na);
    sync();
    reg_ok = true;
}

void GpuSolver::reg_apply(int op, const double* x, double* y) {
    if (!reg_ok) throw std::logic_error("regularisation not set up (m3d_reg_setup)");
    const size_t nb = sizeof(double) * (size_t)reg.na;
    if (op != 2) cuda_ok(cudaMemcpyAsync(d_reg_in, x, nb, cudaMemcpyHostToDevice, stream), "x");
    if (op == 0) reg_apply_wtw(reg, d_reg_in, d_reg_out, stream);
    else if (op == 1) reg_apply_cmcmt(reg, d_reg_in, d_reg_out, stream);
    else reg_diagonal(reg, d_reg_out, stream);
    ++launches;
    cuda_ok(cudaMemcpyAsync(y, d_reg_out, nb, cudaMemcpyDeviceToHost, stream), "y");
    sync();
}

void GpuSolver::reg_evaluate(const double* params, const double* ref, double* value, double* grad) {
    if (!reg_ok) throw std::logic_error("regularisation not set up (m3d_reg_setup)");
    cuda_ok(cudaMemcpyAsync(d_reg_in, params, sizeof(double) * (size_t)reg.nc, cudaMemcpyHostToDevice, stream),
            "params");
    if (ref)
        cuda_ok(cudaMemcpyAsync(d_reg_ref, ref, sizeof(double) * (size_t)reg.na, cudaMemcpyHostToDevice, stream),
                "ref");
    m3d::reg_evaluate(reg, d_reg_in, ref ? d_reg_ref : nullptr, grad ? d_reg_out : nullptr, stream);
    launches += 3;
    if (value) cuda_ok(cudaMemcpyAsync(value, reg.dot, sizeof(double), cudaMemcpyDeviceToHost, stream), "value");
    if (grad)
        cuda_ok(cudaMemcpyAsync(grad, d_reg_out, sizeof(double) * (size_t)reg.nc, cudaMemcpyDeviceToHost, stream),
                "grad");
    sync();
}

void GpuSolver::gradient_batch(const double* freqs, int nf, const double* obs, const double* err, double* Z_out,
                               double* grad) {
    if (nf < 1) throw std::invalid_argument("no frequencies");
    const auto t0 = std::chrono::steady_clock::now();
    begin_call();
    const int ns = sd.ns;
    if (obs_cap < nf) {
        dfree(d_obs); dfree(d_err);
        d_obs = dalloc<double2>((size_t)ns * nf * 4 + 1);
        d_err = dalloc<double>((size_t)ns * nf * 4 + 1);
        obs_cap = nf;
    }
    cuda_ok(cudaMemcpyAsync(d_obs, obs, sizeof(double2) * (size_t)ns * nf * 4, cudaMemcpyHostToDevice, stream), "obs");
    cuda_ok(cudaMemcpyAsync(d_err, err, sizeof(double) * (size_t)ns * nf * 4, cudaMemcpyHostToDevice, stream), "err");
    cuda_ok(cudaMemsetAsync(d_grad, 0, sizeof(double) * L.nc, stream), "memset");
    long long it_total = 0;
    // per right-hand side counters of every solve of the call: forward then
    // adjoint of each frequency group
    std::vector<int> all_it, all_st;
    std::vector<double> all_tr;
    auto keep = [&]() {
        for (int k = 0; k < stats.n_rhs && k < 64; ++k) {
            all_it.push_back(stats.iterations[k]);
            all_st.push_back(stats.status[k]);
            all_tr.push_back(stats.true_residual[k]);
        }
    };
    for (int f0 = 0; f0 < nf; f0 += 8) {
        const int g = std::min(8, nf - f0);
        std::vector<double> fr(freqs + f0, freqs + f0 + g);
        run_forward(fr, Z_out ? Z_out + (size_t)f0 * ns * 8 : nullptr);
        it_total += stats.total_iterations;
        keep();
        const int K = E_K;
        phys::weighted_residual(ns, g, nf, f0, d_obs, d_err, d_Z, d_wr, stream);
        cuda_ok(cudaMemsetAsync(d_adj, 0, sizeof(double2) * (size_t)n_pad * K, stream), "memset");
        phys::adjoint_rhs(sd, md, d_wr, d_hc, d_omegas, g, VecK{d_adj, K}, stream);
        launches += 2;
        std::vector<int> fmap(K, 0), pol(K, -1), active(K, 0);
        for (int k = 0; k < 2 * g; ++k) { fmap[k] = k / 2; active[k] = 1; }
        RhsInfo info = rhs_info(K, fmap, pol, fr);
        current_omega = 2.0 * kPi * fr[0];
        run_adjoint(K, fmap.data(), info, d_adj, d_lam, active);
        it_total += stats.total_iterations;
        keep();
        const int ts = timer.on ? timer.begin(kClsSens, sens_bytes(2 * g), K) : -1;
        phys::sensitivity(md, d_sigma, VecK{d_E, K}, VecK{d_lam, K}, d_omegas, g, 2, d_grad, stream);
        timer.end(ts);
        ++launches;
    }
    cuda_ok(cudaMemcpyAsync(grad, d_grad, sizeof(double) * L.nc, cudaMemcpyDeviceToHost, stream), "grad");
    sync();
    stats.total_iterations = (int)it_total;
    stats.n_rhs = (int)all_it.size();
    for (size_t k = 0; k < all_it.size() && k < 64; ++k) {
        stats.iterations[k] = all_it[k];
        stats.status[k] = all_st[k];
        stats.true_residual[k] = all_tr[k];
    }
    stats.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    end_call();
}

// ---------------------------------------------------------------------------
// autotuner of the batched FP32 inner solve (no counterpart in the reference,
// which has one serial solve)
// ---------------------------------------------------------------------------

// For each row-kernel layout (CSR rows read by the lanes, slice-staged rows)
// and each batch width K <= max_K (right-hand sides sharing one matrix
// stream), runs `reps` iterations of the FP32 BiCGStab inner solve -- with
// the gradient-space term when the solver would use it at this frequency --
// on a constant right-hand side with tolerance 0, timed with CUDA events on
// the solver's stream.  The layout that is fastest at the widest batch and
// the batch width with the least time per right-hand side are applied
// (row_kernels, rhs_block).  The factorisation and the resident fields are
// dropped: call after set_sigma, before the solves.
std::vector<TuneEntry> GpuSolver::autotune(double freq, int max_K, int reps) {
    if (!(freq > 0.0)) throw std::invalid_argument("frequency must be > 0");
    if (reps < 1) throw std::invalid_argument("reps must be >= 1");
    max_K = std::max(2, std::min(dev::kMaxRhs, max_K));
    factorize(std::vector<double>{freq});
    ensure_vecs32(max_K);
    const double om = 2.0 * kPi * freq;
    const bool use_gc = gc_ok && P.gradcorr == 1 && gc.omega_max > 0.0 && om <= gc.omega_max;
    const int rk_saved = P.row_kernels;
    std::vector<TuneEntry> out;
    cudaEvent_t e0, e1;
    cuda_ok(cudaEventCreate(&e0), "event");
    cuda_ok(cudaEventCreate(&e1), "event");
    const bool timer_on = timer.on;
    timer.on = false;
    try {
        for (int rk : {kRowsDirect, kRowsStaged}) {
            P.row_kernels = rk;
            for (int K = 2; K <= max_K; K *= 2) {
                std::vector<int> fmap(K, 0);
                const size_t n = (size_t)n_pad * K;
                // b = 1 + 1i on every row (bit pattern of 1.0f), x = 0
                const std::vector<float2> ones(n, make_float2(1.0f, 1.0f));
                cuda_ok(cudaMemcpyAsync(kv32.b, ones.data(), sizeof(float2) * n, cudaMemcpyHostToDevice, stream),
                        "b");
                cuda_ok(cudaMemsetAsync(kv32.x, 0, sizeof(float2) * n, stream), "memset");
                std::vector<BicgState> st(K);
                for (int k = 0; k < K; ++k) {
                    std::memset(&st[k], 0, sizeof(BicgState));
                    st[k].tol = 0.0;
                    st[k].maxiter = 1 << 30;
                    st[k].status = kRunning;
                }
                cuda_ok(cudaMemcpyAsync(d_states, st.data(), sizeof(BicgState) * K, cudaMemcpyHostToDevice, stream),
                        "states");
                KrylovCtx<float> c32 = kctx32(K, fmap.data());
                if (use_gc) attach_gc(c32);
                bicg_init(c32, kv32, d_states);
                for (int i = 0; i < 2; ++i) bicg_iteration(c32, kv32, d_states);   // warm-up
                cuda_ok(cudaEventRecord(e0, stream), "event");
                for (int i = 0; i < reps; ++i) bicg_iteration(c32, kv32, d_states);
                cuda_ok(cudaEventRecord(e1, stream), "event");
                cuda_ok(cudaEventSynchronize(e1), "event");
                float ms = 0.f;
                cuda_ok(cudaEventElapsedTime(&ms, e0, e1), "event");
                check_seg_err();
                out.push_back(TuneEntry{rk, K, ms / reps, ms / reps / K});
            }
        }
    } catch (...) {
        P.row_kernels = rk_saved;
        timer.on = timer_on;
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        throw;
    }
    timer.on = timer_on;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    // layout: fastest at the widest batch; batch width: least time per rhs
    int best_rk = rk_saved;
    double best_t = 1e300;
    for (const TuneEntry& t : out)
        if (t.K == max_K && t.ms_per_iter < best_t) { best_t = t.ms_per_iter; best_rk = t.row_kernels; }
    int best_K = max_K;
    double best_r = 1e300;
    for (const TuneEntry& t : out)
        if (t.row_kernels == best_rk && t.ms_per_rhs_iter < best_r) { best_r = t.ms_per_rhs_iter; best_K = t.K; }
    P.row_kernels = best_rk;
    rhs_block = best_K;
    release();
    E_nf = 0;
    E_K = 0;
    return out;
}

}  // namespace m3d
