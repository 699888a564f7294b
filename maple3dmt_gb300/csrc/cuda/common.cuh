// Device helpers shared by the solver kernels: complex arithmetic on
// double2 / float2, warp and block reductions, and a deterministic grid
// reduction (per-block partials summed in block order by the last block).
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

namespace m3d {
namespace dev {

constexpr int kWarp = 32;
constexpr int kBlock = 256;               // threads per block for every kernel here
constexpr int kWarpsPerBlock = kBlock / kWarp;
constexpr int kSlice = 32;                // sliced-ELL slice height (rows per warp)
constexpr int kMaxRhs = 16;               // right-hand sides per batched launch
constexpr int kMaxQ = 3;                  // reduced quantities per kernel

template <class R> struct CTraits;
template <> struct CTraits<double> { using C = double2; };
template <> struct CTraits<float> { using C = float2; };
template <class R> using cplx = typename CTraits<R>::C;

template <class R> __host__ __device__ __forceinline__ cplx<R> cm(R a, R b) {
    cplx<R> z; z.x = a; z.y = b; return z;
}
template <class C> __host__ __device__ __forceinline__ C cadd(C a, C b) { a.x += b.x; a.y += b.y; return a; }
template <class C> __host__ __device__ __forceinline__ C csub(C a, C b) { a.x -= b.x; a.y -= b.y; return a; }
template <class C> __host__ __device__ __forceinline__ C cneg(C a) { a.x = -a.x; a.y = -a.y; return a; }
template <class C> __host__ __device__ __forceinline__ C cmul(C a, C b) {
    C z; z.x = a.x * b.x - a.y * b.y; z.y = a.x * b.y + a.y * b.x; return z;
}
// conj(a) * b
template <class C> __host__ __device__ __forceinline__ C cjmul(C a, C b) {
    C z; z.x = a.x * b.x + a.y * b.y; z.y = a.x * b.y - a.y * b.x; return z;
}
template <class C, class R> __host__ __device__ __forceinline__ C cscale(C a, R s) { a.x *= s; a.y *= s; return a; }
template <class C> __host__ __device__ __forceinline__ double cabs2(C a) { return (double)a.x * a.x + (double)a.y * a.y; }
__host__ __device__ __forceinline__ double cabsd(double2 a) { return hypot(a.x, a.y); }
// Smith's algorithm for a / b (R. L. Smith, CACM 5(8), 1962).
__host__ __device__ __forceinline__ double2 cdiv(double2 a, double2 b) {
    double2 z;
    if (fabs(b.x) >= fabs(b.y)) {
        const double r = b.y / b.x, d = b.x + b.y * r;
        z.x = (a.x + a.y * r) / d; z.y = (a.y - a.x * r) / d;
    } else {
        const double r = b.x / b.y, d = b.x * r + b.y;
        z.x = (a.x * r + a.y) / d; z.y = (a.y * r - a.x) / d;
    }
    return z;
}
__host__ __device__ __forceinline__ double2 to_d(double2 a) { return a; }
__host__ __device__ __forceinline__ double2 to_d(float2 a) { return make_double2(a.x, a.y); }
template <class C> __host__ __device__ __forceinline__ C from_d(double2 a);
template <> __host__ __device__ __forceinline__ double2 from_d<double2>(double2 a) { return a; }
template <> __host__ __device__ __forceinline__ float2 from_d<float2>(double2 a) {
    return make_float2((float)a.x, (float)a.y);
}

__device__ __forceinline__ double shfl_xor(double v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }
__device__ __forceinline__ double2 shfl_xor(double2 v, int m) {
    v.x = __shfl_xor_sync(0xffffffffu, v.x, m);
    v.y = __shfl_xor_sync(0xffffffffu, v.y, m);
    return v;
}

// Blocks of `threads` threads with `smem` bytes of dynamic shared memory of
// `kernel` that are resident on the current device at once (occupancy API x
// SM count); cached per (device, kernel, threads, smem).
int resident_blocks(const void* kernel, int threads = kBlock, int smem = 0);

// One resident wave of `kernel`, at most `cap` blocks.
template <class F>
inline int wave_grid(F* kernel, int cap, int threads = kBlock, int smem = 0) {
    const int g = resident_blocks(reinterpret_cast<const void*>(kernel), threads, smem);
    return g < cap ? g : cap;
}

// Scratch for grid reductions: partial[block][kMaxQ * kMaxRhs] and a counter
// that the last block resets.
struct RedScratch {
    double2* partial;
    double2* final_;      // [kMaxQ * kMaxRhs], result of the last reduction
    unsigned int* counter;
    int max_blocks;
};

// Sums, over the grid, NQ complex quantities for each of K right-hand sides.
// `acc[kt][q]` is this thread's contribution for right-hand side rhs0 + kt.
// Lanes are combined through shared memory in lane order, warps in warp
// order and blocks in block order by the last block to arrive, so the result
// is deterministic for a fixed launch shape.  Returns true in the last block;
// then `out[q * K + k]` (shared memory, NQ*K entries) holds the totals.
template <int NQ, int K, int KT>
__device__ bool grid_reduce(const double2 (&acc)[KT][NQ], int rhs0, RedScratch rs, double2* out) {
    __shared__ double2 sm[kWarpsPerBlock][NQ][K];
    __shared__ bool am_last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < kWarpsPerBlock * NQ * K; i += blockDim.x)
        (&sm[0][0][0])[i] = make_double2(0.0, 0.0);
    __syncthreads();
    for (int l = 0; l < 32; ++l) {
        if (lane == l) {
#pragma unroll
            for (int kt = 0; kt < KT; ++kt)
#pragma unroll
                for (int q = 0; q < NQ; ++q)
                    sm[warp][q][rhs0 + kt] = cadd(sm[warp][q][rhs0 + kt], acc[kt][q]);
        }
        __syncwarp();
    }
    __syncthreads();
    if (threadIdx.x < NQ * K) {
        const int q = threadIdx.x / K, k = threadIdx.x % K;
        double2 s = make_double2(0.0, 0.0);
        for (int w = 0; w < kWarpsPerBlock; ++w) s = cadd(s, sm[w][q][k]);
        __stcg(&rs.partial[(size_t)blockIdx.x * (NQ * K) + threadIdx.x], s);
        __threadfence();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned t = atomicAdd(rs.counter, 1u);
        am_last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!am_last) return false;
    __threadfence();
    // Last block: for each of the NQ*K totals, thread t sums blocks t, t+256, ...
    // then a fixed-shape tree over the 256 threads; deterministic and short.
    __shared__ double2 red[kBlock];
    for (int qk = 0; qk < NQ * K; ++qk) {
        double2 s = make_double2(0.0, 0.0);
        for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x)
            s = cadd(s, __ldcg(&rs.partial[(size_t)b * (NQ * K) + qk]));
        red[threadIdx.x] = s;
        __syncthreads();
        for (int w = blockDim.x / 2; w > 0; w >>= 1) {
            if ((int)threadIdx.x < w) red[threadIdx.x] = cadd(red[threadIdx.x], red[threadIdx.x + w]);
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            out[qk] = red[0];
            rs.final_[qk] = red[0];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) *rs.counter = 0u;
    __syncthreads();
    return true;
}

// Grid reduction for kernels whose lane l always works on right-hand side
// l % K (K a power of two <= 32, blockDim a multiple of 32): a shuffle tree
// over the lanes that share a right-hand side, warps combined in warp order,
// blocks in block order by the last block to arrive (each of the NQ*K totals
// summed by a fixed set of threads, then in a fixed order).  Deterministic
// for a fixed launch shape.  Returns true in the last block, where
// out[q * K + k] (shared, NQ*K entries) holds the totals.
template <int NQ, int K, int NT = kBlock>
__device__ bool grid_reduce_lanes(double2 (&acc)[NQ], RedScratch rs, double2* out) {
    static_assert(K >= 1 && K <= 32 && (K & (K - 1)) == 0, "K must be a power of two <= 32");
    static_assert(NT % 32 == 0 && NT >= 32, "block size must be whole warps");
    constexpr int PK = NQ * K;
    constexpr int NW = NT / 32;
    __shared__ double2 sm[NW][PK];
    __shared__ double2 chunk[NT];
    __shared__ bool am_last;
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
        double2 s = make_double2(0.0, 0.0);
        for (int w = 0; w < NW; ++w) s = cadd(s, sm[w][threadIdx.x]);
        __stcg(&rs.partial[(size_t)blockIdx.x * PK + threadIdx.x], s);
        __threadfence();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned t = atomicAdd(rs.counter, 1u);
        am_last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!am_last) return false;
    __threadfence();
    constexpr int CH = NT / PK > 0 ? NT / PK : 1;   // threads per total
    const int p = threadIdx.x % PK, j = threadIdx.x / PK;
    double2 s = make_double2(0.0, 0.0);
    if (j < CH)
        for (int b = j; b < (int)gridDim.x; b += CH) s = cadd(s, __ldcg(&rs.partial[(size_t)b * PK + p]));
    chunk[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x < PK) {
        double2 t = make_double2(0.0, 0.0);
        for (int jj = 0; jj < CH; ++jj) t = cadd(t, chunk[jj * PK + threadIdx.x]);
        out[threadIdx.x] = t;
        rs.final_[threadIdx.x] = t;
    }
    if (threadIdx.x == 0) *rs.counter = 0u;
    __syncthreads();
    return true;
}

}  // namespace dev
}  // namespace m3d
