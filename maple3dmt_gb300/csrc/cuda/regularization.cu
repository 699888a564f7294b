// Octree regularisation kernels (see regularization.cuh).
#include "regularization.cuh"

#include <stdexcept>

namespace m3d {

namespace {

constexpr int kRegBlock = 256;

int reg_grid(long n) { return (int)((n + kRegBlock - 1) / kRegBlock > 0 ? (n + kRegBlock - 1) / kRegBlock : 1); }

void reg_check() {
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) throw std::runtime_error(cudaGetErrorString(e));
}

// CSRMatrix::matvec (include/maple3dmt/common.h:52-61)
__global__ void k_reg_wtw(RegDev r, const double* __restrict__ x, double* __restrict__ y) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= r.na) return;
    double s = 0.0;
    for (int k = r.ptr[i]; k < r.ptr[i + 1]; ++k) s = __dadd_rn(s, __dmul_rn(r.val[k], x[r.idx[k]]));
    y[i] = s;
}

__global__ void k_reg_diag(RegDev r, double* __restrict__ d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= r.na) return;
    double v = 0.0;
    for (int k = r.ptr[i]; k < r.ptr[i + 1]; ++k)
        if (r.idx[k] == i) { v = r.val[k]; break; }
    d[i] = v;
}

// one pass y_i = (x_i + sum_j w_ij / d_i x_j) / (1 + sum_j w_ij / d_i)
__global__ void k_reg_diffuse(RegDev r, const double* __restrict__ x, double* __restrict__ y) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= r.na) return;
    double sum = x[i], wt = 1.0;
    const double dg = r.diagw[i] > 0 ? r.diagw[i] : 1.0;
    for (int k = r.aptr[i]; k < r.aptr[i + 1]; ++k) {
        const double wn = __ddiv_rn(r.aw[k], dg);
        sum = __dadd_rn(sum, __dmul_rn(wn, x[r.aidx[k]]));
        wt = __dadd_rn(wt, wn);
    }
    y[i] = __ddiv_rn(sum, wt);
}

__global__ void k_reg_dm(RegDev r, const double* __restrict__ params, const double* __restrict__ ref,
                         double* __restrict__ dm) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= r.na) return;
    dm[j] = __dsub_rn(params[r.a2g[j]], ref ? ref[j] : 0.0);
}

// alpha_s sum_j dm_j wd_j: one block, fixed strides, fixed tree
__global__ void __launch_bounds__(1024) k_reg_dot(RegDev r, const double* __restrict__ a, const double* __restrict__ b) {
    __shared__ double part[1024];
    double s = 0.0;
    for (int j = threadIdx.x; j < r.na; j += blockDim.x) s = __dadd_rn(s, __dmul_rn(a[j], b[j]));
    part[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) part[threadIdx.x] = __dadd_rn(part[threadIdx.x], part[threadIdx.x + w]);
        __syncthreads();
    }
    if (threadIdx.x == 0) *r.dot = __dmul_rn(r.alpha_s, part[0]);
}

__global__ void k_reg_zero(int n, double* __restrict__ g) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < n) g[c] = 0.0;
}

__global__ void k_reg_grad(RegDev r, const double* __restrict__ wd, double* __restrict__ g) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= r.na) return;
    g[r.a2g[j]] = __dmul_rn(__dmul_rn(2.0, r.alpha_s), wd[j]);
}

}  // namespace

void reg_apply_wtw(const RegDev& r, const double* x, double* y, cudaStream_t s) {
    k_reg_wtw<<<reg_grid(r.na), kRegBlock, 0, s>>>(r, x, y);
    reg_check();
}

void reg_diagonal(const RegDev& r, double* d, cudaStream_t s) {
    k_reg_diag<<<reg_grid(r.na), kRegBlock, 0, s>>>(r, d);
    reg_check();
}

void reg_apply_cmcmt(const RegDev& r, const double* x, double* y, cudaStream_t s) {
    const int passes = 2 * r.n_smooth;
    if (passes <= 0) {
        cudaMemcpyAsync(y, x, sizeof(double) * (size_t)r.na, cudaMemcpyDeviceToDevice, s);
        reg_check();
        return;
    }
    const double* cur = x;
    for (int p = 0; p < passes; ++p) {
        double* dst = (p == passes - 1) ? y : (p % 2 == 0 ? r.t0 : r.t1);
        k_reg_diffuse<<<reg_grid(r.na), kRegBlock, 0, s>>>(r, cur, dst);
        reg_check();
        cur = dst;
    }
}

void reg_evaluate(const RegDev& r, const double* params, const double* ref, double* grad, cudaStream_t s) {
    k_reg_dm<<<reg_grid(r.na), kRegBlock, 0, s>>>(r, params, ref, r.t0);
    k_reg_wtw<<<reg_grid(r.na), kRegBlock, 0, s>>>(r, r.t0, r.t1);
    k_reg_dot<<<1, 1024, 0, s>>>(r, r.t0, r.t1);
    reg_check();
    if (grad) {
        k_reg_zero<<<reg_grid(r.nc), kRegBlock, 0, s>>>(r.nc, grad);
        k_reg_grad<<<reg_grid(r.na), kRegBlock, 0, s>>>(r, r.t1, grad);
        reg_check();
    }
}

}  // namespace m3d
