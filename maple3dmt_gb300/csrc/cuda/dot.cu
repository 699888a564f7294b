// Batched Hermitian dot kernel (see dot.cuh).
#include "dot.cuh"

namespace m3d {
namespace dev {

namespace {

// Thread t of the grid owns the (row, rhs) pairs t, t + stride, ...; the grid
// stride is a multiple of 256 and hence of K, so lane l always accumulates
// right-hand side l % K, which is what grid_reduce_lanes expects.
template <int K>
__global__ void __launch_bounds__(kBlock) k_dot_batched(const double2* __restrict__ x,
                                                        const double2* __restrict__ y, long long n,
                                                        RedScratch rs, double2* __restrict__ out) {
    __shared__ double2 tot[K];
    double2 acc[1] = {make_double2(0.0, 0.0)};
    const long long total = n * K;
    const long long stride = (long long)gridDim.x * blockDim.x;
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    // two independent loads in flight per thread before the dependent adds
    for (; t + stride < total; t += 2 * stride) {
        const double2 x0 = __ldg(x + t), y0 = __ldg(y + t);
        const double2 x1 = __ldg(x + t + stride), y1 = __ldg(y + t + stride);
        acc[0] = cadd(acc[0], cadd(cjmul(x0, y0), cjmul(x1, y1)));
    }
    if (t < total) acc[0] = cadd(acc[0], cjmul(__ldg(x + t), __ldg(y + t)));
    if (grid_reduce_lanes<1, K>(acc, rs, tot) && threadIdx.x < K) out[threadIdx.x] = tot[threadIdx.x];
}

}  // namespace

int dot_blocks(long long n, int K, int cap) {
    const long long work = n * (long long)K;
    long long b = (work + kBlock - 1) / kBlock;
    if (b < 1) b = 1;
    if (b > cap) b = cap;
    return (int)b;
}

cudaError_t launch_dot_batched(const double2* x, const double2* y, long long n, int K, int cap, RedScratch rs,
                               double2* out, cudaStream_t st) {
    const int g = dot_blocks(n, K, cap);
    switch (K) {
        case 1: k_dot_batched<1><<<g, kBlock, 0, st>>>(x, y, n, rs, out); break;
        case 2: k_dot_batched<2><<<g, kBlock, 0, st>>>(x, y, n, rs, out); break;
        case 4: k_dot_batched<4><<<g, kBlock, 0, st>>>(x, y, n, rs, out); break;
        case 8: k_dot_batched<8><<<g, kBlock, 0, st>>>(x, y, n, rs, out); break;
        case 16: k_dot_batched<16><<<g, kBlock, 0, st>>>(x, y, n, rs, out); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace dev
}  // namespace m3d
