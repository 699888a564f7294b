// Learned preconditioner network (learned.cuh): BF16 implicit-GEMM 3-D
// convolutions on tcgen05 tensor cores, their backward passes and Adam.
//
// Forward (and, with transposed weights, the input gradient): one CTA of 128
// threads computes a tile of 128 output voxels x 32 channels.
//   warp 0 / lane 0  TMA producer: the 27 taps' weights once (2 KB each),
//                    then for every tap the 128-voxel input box shifted by
//                    (dz, dy, dx) -- out-of-range rows arrive as zeros, the
//                    convolution's zero padding -- into a 4-stage ring;
//   warp 1           allocates 32 TMEM columns; lane 0 issues per tap two
//                    tcgen05.mma (K = 16 each, M = 128, N = 32) into the FP32
//                    accumulator and frees the stage with tcgen05.commit;
//   all 4 warps      epilogue: tcgen05.ld of their 32 TMEM lanes, bias,
//                    ReLU or the ReLU mask of the backward pass, BF16 store.
// Grids up to 64 voxels wide use k_conv3d_halo instead: each tile's input
// and its border arrive once per x shift and the taps are line offsets into
// those boxes (see the kernel's comment).
// GEMM view: M = voxels, N = output channels, K = 27 taps x 32 channels.
// Weight gradient: dW[t] = sum_v dY[v]^T X[v + off_t] as one GEMM with
// M = 27 x 32 (tap, input channel) rows padded to 896, N = 32 output channels,
// K = every voxel of the batch, both operands K-major (the shifted inputs
// gathered once per layer, the output gradient transposed), split over K
// across CTAs and summed in a fixed order.
//
// Every barrier wait is bounded; a timeout sets an error flag that the host
// turns into an error, the CTA waits (bounded) for its copies and MMAs in
// flight and frees its tensor memory before it exits.
#include "learned.cuh"

#include <cmath>
#include <cstring>
#include <mutex>
#include <random>
#include <stdexcept>
#include <string>

#include "tc.cuh"

namespace m3d {
namespace learn {

namespace {

constexpr int kStages = 4;
constexpr int kTileA = 128 * 64;      // bytes of a 128-row, 64-byte-row operand tile
constexpr int kTapB = 32 * 64;        // bytes of one tap's 32 x 32 weights
constexpr int kConvSmem = kTaps * kTapB + kStages * kTileA + 1024;
constexpr int kGemmStage = kTileA + kTapB;
constexpr int kGemmSmem = kStages * kGemmStage + 1024;
constexpr int kMPad = 896;            // 27 x 32 weight-gradient rows padded to 7 x 128

void ck(cudaError_t e, const char* what) {
    if (e != cudaSuccess) {
        cudaGetLastError();
        throw std::runtime_error(std::string("cnn: ") + what + ": " + cudaGetErrorString(e));
    }
}

struct ConvArgs {
    int D, H, W, bw, bh, tiles_h;
    int n_tiles;                  // tiles of the launch
    const float* bias;            // [32] or null
    int relu;
    const __nv_bfloat16* mask;    // keep where mask > 0 (null: keep all)
    __nv_bfloat16* out;           // [.][32]
    float* out32;                 // [.][n32] or null
    int n32;
    unsigned* err;
};

__global__ void __launch_bounds__(128, 1) k_conv3d_tc(const __grid_constant__ CUtensorMap xmap,
                                                      const __grid_constant__ CUtensorMap wmap, ConvArgs a) {
    extern __shared__ unsigned char smem_raw[];
    unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                                           ~static_cast<uintptr_t>(1023));
    unsigned char* sB = base;
    unsigned char* sA = base + kTaps * kTapB;
    __shared__ __align__(8) uint64_t full[kStages], empty[kStages], wbar, done;
    __shared__ uint32_t tmem_base;
    __shared__ int fail;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int per_n = a.D * a.tiles_h;
    const int n = blockIdx.x / per_n, rem = blockIdx.x % per_n;
    const int z = rem / a.tiles_h, y0 = (rem % a.tiles_h) * a.bh;
    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; ++s) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], 1);
        }
        tc::mbar_init(&wbar, 1);
        tc::mbar_init(&done, 1);
        tc::fence_barrier_init();
        fail = 0;
    }
    if (warp == 1) {
        tc::tmem_alloc(&tmem_base, 32);
        tc::tmem_relinquish();
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = tmem_base;
    if (warp == 0 && lane == 0) {
        // producer
        tc::mbar_expect_tx(&wbar, kTaps * kTapB);
        for (int t = 0; t < kTaps; ++t) tc::tma_load_2d(sB + t * kTapB, &wmap, &wbar, 0, t * kCh);
        int issued = 0;
        for (int t = 0; t < kTaps; ++t) {
            const int s = t % kStages;
            if (t >= kStages && !tc::mbar_wait(&empty[s], (unsigned)((t / kStages) - 1) & 1u)) {
                atomicOr(a.err, tc::kErrWait);
                fail = 1;
                break;
            }
            const int dz = t / 9 - 1, dy = (t / 3) % 3 - 1, dx = t % 3 - 1;
            tc::mbar_expect_tx(&full[s], kTileA);
            tc::tma_load_5d(sA + s * kTileA, &xmap, &full[s], 0, dx, y0 + dy, z + dz, n);
            ++issued;
        }
        // every issued copy has landed before the CTA can leave
        tc::mbar_wait(&wbar, 0);
        for (int t = issued - 1; t >= 0 && t >= issued - kStages; --t)
            tc::mbar_wait(&full[t % kStages], (unsigned)(t / kStages) & 1u);
    } else if (warp == 1 && lane == 0) {
        // MMA issuer
        constexpr uint32_t idesc = tc::idesc_bf16(128, 32);
        bool ok = tc::mbar_wait(&wbar, 0);
        for (int t = 0; t < kTaps && ok; ++t) {
            const int s = t % kStages;
            if (!tc::mbar_wait(&full[s], (unsigned)(t / kStages) & 1u)) {
                ok = false;
                break;
            }
            tc::tc_fence_after();
            const uint64_t ad = tc::sdesc_sw64(sA + s * kTileA);
            const uint64_t bd = tc::sdesc_sw64(sB + t * kTapB);
            tc::mma_bf16(tmem, ad, bd, idesc, t > 0 ? 1u : 0u);
            tc::mma_bf16(tmem, ad + 2, bd + 2, idesc, 1u);   // second half of the 64-byte rows (+32 B)
            tc::mma_commit(&empty[s]);
        }
        if (!ok) {
            atomicOr(a.err, tc::kErrWait);
            fail = 1;
        }
        tc::mma_commit(&done);
    }
    __syncwarp();
    const bool got = tc::mbar_wait(&done, 0);
    tc::tc_fence_after();
    if (!got) atomicOr(a.err, tc::kErrWait);
    float acc[32];
    tc::tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16), acc);
    __syncthreads();   // `fail` is final here
    if (got && !fail) {
        const int m = warp * 32 + lane;
        const int yy = y0 + m / a.bw, xx = m % a.bw;
        const size_t v = (((size_t)n * a.D + z) * a.H + yy) * a.W + xx;
        float keep[32];
#pragma unroll
        for (int c = 0; c < 32; ++c) keep[c] = 1.0f;
        if (a.mask) {
            const uint4* mp = reinterpret_cast<const uint4*>(a.mask + v * kCh);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const uint4 u = mp[q];
                const __nv_bfloat16* h = reinterpret_cast<const __nv_bfloat16*>(&u);
#pragma unroll
                for (int j = 0; j < 8; ++j) keep[8 * q + j] = __bfloat162float(h[j]) > 0.0f ? 1.0f : 0.0f;
            }
        }
#pragma unroll
        for (int c = 0; c < 32; ++c) {
            float x = acc[c] + (a.bias ? a.bias[c] : 0.0f);
            if (a.relu) x = fmaxf(x, 0.0f);
            acc[c] = x * keep[c];
        }
        if (a.out) {
            uint4* op = reinterpret_cast<uint4*>(a.out + v * kCh);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                uint4 u;
                __nv_bfloat16* h = reinterpret_cast<__nv_bfloat16*>(&u);
#pragma unroll
                for (int j = 0; j < 8; ++j) h[j] = __float2bfloat16_rn(acc[8 * q + j]);
                op[q] = u;
            }
        }
        if (a.out32) {
#pragma unroll
            for (int c = 0; c < 32; ++c)
                if (c < a.n32) a.out32[v * a.n32 + c] = acc[c];
        }
    }
    if (!got) tc::mbar_wait(&done, 0);   // MMAs still in flight: let them finish before freeing TMEM
    tc::tc_fence_before();
    __syncthreads();
    if (warp == 1) tc::tmem_dealloc(tmem, 32);
}

// Halo form of the forward / input-gradient convolution, for grids up to 64
// voxels wide (one tile = 128 voxels = 128 / W lines of W voxels): instead
// of one 8 KB copy per tap, a tile's input comes in as three boxes, one per
// x shift (dx = -1, 0, 1), each holding the tile's lines with a one-voxel
// border in y and z.  The 27 taps' A operands are then line offsets into
// these boxes (tap (dz, dy) of box dx starts at line dz (bh + 2) + dy; the
// 128 rows are contiguous and 1 KB aligned, so the SWIZZLE_64B descriptor
// stays valid), and each input byte crosses from L2 three times per tile
// instead of twenty-seven.  Persistent CTAs of six warps, one per SM:
//   warp 4 / lane 0  TMA producer: the weights once, then per tile the three
//                    boxes, each reused as soon as its nine taps' MMAs are done;
//   warp 5           allocates 64 TMEM columns (two accumulators); lane 0
//                    issues the 54 MMAs of a tile into one accumulator while
//                    the epilogue drains the other;
//   warps 0-3        epilogue: tcgen05.ld of their 32 lanes, release of the
//                    accumulator, bias / ReLU / mask, BF16 store.
// Every wait is bounded; a timeout flags an error and every role stops.
constexpr int kHaloMaxW = 64;
__host__ __device__ constexpr int halo_box_bytes(int W) { return (128 + 2 * W) * 3 * 64; }
constexpr int halo_smem(int W) { return kTaps * kTapB + 3 * halo_box_bytes(W) + 1024; }

__global__ void __launch_bounds__(192, 1) k_conv3d_halo(const __grid_constant__ CUtensorMap hmap,
                                                        const __grid_constant__ CUtensorMap wmap, ConvArgs a) {
    extern __shared__ unsigned char smem_raw[];
    unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                                           ~static_cast<uintptr_t>(1023));
    unsigned char* sB = base;
    unsigned char* sX = base + kTaps * kTapB;
    const int box_bytes = halo_box_bytes(a.W);
    __shared__ __align__(8) uint64_t bfull[3], bempty[3], tfull[2], tempty[2], wbar, mdone;
    __shared__ uint32_t tmem_base;
    __shared__ volatile int fail;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int per_n = a.D * a.tiles_h;
    const int box_lines_y = a.bh + 2;
    if (threadIdx.x == 0) {
        for (int d = 0; d < 3; ++d) {
            tc::mbar_init(&bfull[d], 1);
            tc::mbar_init(&bempty[d], 1);
        }
        for (int b = 0; b < 2; ++b) {
            tc::mbar_init(&tfull[b], 1);
            tc::mbar_init(&tempty[b], 128);
        }
        tc::mbar_init(&wbar, 1);
        tc::mbar_init(&mdone, 1);
        tc::fence_barrier_init();
        fail = 0;
    }
    if (warp == 5) {
        tc::tmem_alloc(&tmem_base, 64);
        tc::tmem_relinquish();
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = tmem_base;
    int last_issue[3] = {-1, -1, -1};   // producer: the tile each box was last loaded for
    if (warp == 4) {
        if (lane == 0) {
            tc::mbar_expect_tx(&wbar, kTaps * kTapB);
            for (int t = 0; t < kTaps; ++t) tc::tma_load_2d(sB + t * kTapB, &wmap, &wbar, 0, t * kCh);
            int it = 0;
            for (int tile = blockIdx.x; tile < a.n_tiles && !fail; tile += gridDim.x, ++it) {
                const int n = tile / per_n, rem = tile % per_n;
                const int z = rem / a.tiles_h, y0 = (rem % a.tiles_h) * a.bh;
                for (int d = 0; d < 3; ++d) {
                    if (it > 0 && !tc::mbar_wait(&bempty[d], (unsigned)(it - 1) & 1u)) {
                        atomicOr(a.err, tc::kErrWait);
                        fail = 1;
                        break;
                    }
                    tc::mbar_expect_tx(&bfull[d], box_bytes);
                    tc::tma_load_5d(sX + d * box_bytes, &hmap, &bfull[d], 0, d - 1, y0 - 1, z - 1, n);
                    last_issue[d] = it;
                }
            }
        }
    } else if (warp == 5) {
        if (lane == 0) {
            constexpr uint32_t idesc = tc::idesc_bf16(128, 32);
            bool ok = tc::mbar_wait(&wbar, 0);
            int it = 0;
            for (int tile = blockIdx.x; tile < a.n_tiles && ok && !fail; tile += gridDim.x, ++it) {
                const int b = it & 1;
                if (it >= 2 && !tc::mbar_wait(&tempty[b], (unsigned)((it >> 1) - 1) & 1u)) {
                    ok = false;
                    break;
                }
                tc::tc_fence_after();
                const uint32_t dt = tmem + 32u * (uint32_t)b;
                bool first = true;
                for (int d = 0; d < 3 && ok; ++d) {
                    if (!tc::mbar_wait(&bfull[d], (unsigned)it & 1u)) {
                        ok = false;
                        break;
                    }
                    tc::tc_fence_after();
                    for (int dz = 0; dz < 3; ++dz)
                        for (int dy = 0; dy < 3; ++dy) {
                            const int t = dz * 9 + dy * 3 + d;
                            const int line = dz * box_lines_y + dy;
                            const uint64_t ad = tc::sdesc_sw64(sX + d * box_bytes + line * a.bw * 64);
                            const uint64_t bd = tc::sdesc_sw64(sB + t * kTapB);
                            tc::mma_bf16(dt, ad, bd, idesc, first ? 0u : 1u);
                            tc::mma_bf16(dt, ad + 2, bd + 2, idesc, 1u);   // second half of the 64-byte rows
                            first = false;
                        }
                    tc::mma_commit(&bempty[d]);
                }
                if (!ok) break;
                tc::mma_commit(&tfull[b]);
            }
            if (!ok) {
                atomicOr(a.err, tc::kErrWait);
                fail = 1;
            }
        }
    } else {
        int it = 0;
        for (int tile = blockIdx.x; tile < a.n_tiles; tile += gridDim.x, ++it) {
            const int b = it & 1;
            const bool got = tc::mbar_wait(&tfull[b], (unsigned)(it >> 1) & 1u);
            // the TMEM load is warp-collective: the warp decides together
            if (!__all_sync(0xffffffffu, (got && !fail) ? 1 : 0)) {
                if (lane == 0) {
                    atomicOr(a.err, tc::kErrWait);
                    fail = 1;
                }
                break;
            }
            tc::tc_fence_after();
            float acc[32];
            tc::tmem_ld32(tmem + 32u * (uint32_t)b + ((uint32_t)(warp * 32) << 16), acc);
            tc::tc_fence_before();
            tc::mbar_arrive(&tempty[b]);
            const int n = tile / per_n, rem = tile % per_n;
            const int z = rem / a.tiles_h, y0 = (rem % a.tiles_h) * a.bh;
            const int m = warp * 32 + lane;
            const int yy = y0 + m / a.bw, xx = m % a.bw;
            const size_t v = (((size_t)n * a.D + z) * a.H + yy) * a.W + xx;
            float keep[32];
#pragma unroll
            for (int c = 0; c < 32; ++c) keep[c] = 1.0f;
            if (a.mask) {
                const uint4* mp = reinterpret_cast<const uint4*>(a.mask + v * kCh);
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const uint4 u = mp[q];
                    const __nv_bfloat16* h = reinterpret_cast<const __nv_bfloat16*>(&u);
#pragma unroll
                    for (int j = 0; j < 8; ++j) keep[8 * q + j] = __bfloat162float(h[j]) > 0.0f ? 1.0f : 0.0f;
                }
            }
#pragma unroll
            for (int c = 0; c < 32; ++c) {
                float x = acc[c] + (a.bias ? a.bias[c] : 0.0f);
                if (a.relu) x = fmaxf(x, 0.0f);
                acc[c] = x * keep[c];
            }
            if (a.out) {
                uint4* op = reinterpret_cast<uint4*>(a.out + v * kCh);
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    uint4 u;
                    __nv_bfloat16* h = reinterpret_cast<__nv_bfloat16*>(&u);
#pragma unroll
                    for (int j = 0; j < 8; ++j) h[j] = __float2bfloat16_rn(acc[8 * q + j]);
                    op[q] = u;
                }
            }
            if (a.out32) {
#pragma unroll
                for (int c = 0; c < 32; ++c)
                    if (c < a.n32) a.out32[v * a.n32 + c] = acc[c];
            }
        }
    }
    __syncthreads();
    if (warp == 4 && lane == 0) {
        // every issued copy lands before the CTA leaves
        tc::mbar_wait(&wbar, 0);
        for (int d = 0; d < 3; ++d)
            if (last_issue[d] >= 0) tc::mbar_wait(&bfull[d], (unsigned)last_issue[d] & 1u);
    }
    if (warp == 5 && lane == 0) {
        // every issued MMA completes before the accumulators are freed
        tc::mma_commit(&mdone);
        tc::mbar_wait(&mdone, 0);
    }
    tc::tc_fence_before();
    __syncthreads();
    if (warp == 5) tc::tmem_dealloc(tmem, 64);
}

struct GemmArgs {
    int k_steps;        // 32-element K steps per split
    float* ws;          // [splits][kMPad][32]
    unsigned* err;
};

// D[896 x 32] partial = A[896 x K] B[32 x K]^T over this CTA's K range;
// blockIdx.x = 128-row M tile, blockIdx.y = K split.
__global__ void __launch_bounds__(128, 1) k_gemm_tn_tc(const __grid_constant__ CUtensorMap amap,
                                                       const __grid_constant__ CUtensorMap bmap, GemmArgs a) {
    extern __shared__ unsigned char smem_raw[];
    unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                                           ~static_cast<uintptr_t>(1023));
    __shared__ __align__(8) uint64_t full[kStages], empty[kStages], done;
    __shared__ uint32_t tmem_base;
    __shared__ int fail;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int mt = blockIdx.x, split = blockIdx.y;
    const int k0 = split * a.k_steps;
    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; ++s) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], 1);
        }
        tc::mbar_init(&done, 1);
        tc::fence_barrier_init();
        fail = 0;
    }
    if (warp == 1) {
        tc::tmem_alloc(&tmem_base, 32);
        tc::tmem_relinquish();
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = tmem_base;
    if (warp == 0 && lane == 0) {
        int issued = 0;
        for (int j = 0; j < a.k_steps; ++j) {
            const int s = j % kStages;
            if (j >= kStages && !tc::mbar_wait(&empty[s], (unsigned)((j / kStages) - 1) & 1u)) {
                atomicOr(a.err, tc::kErrWait);
                fail = 1;
                break;
            }
            unsigned char* st = base + s * kGemmStage;
            tc::mbar_expect_tx(&full[s], kGemmStage);
            tc::tma_load_2d(st, &amap, &full[s], (k0 + j) * 32, mt * 128);
            tc::tma_load_2d(st + kTileA, &bmap, &full[s], (k0 + j) * 32, 0);
            ++issued;
        }
        for (int j = issued - 1; j >= 0 && j >= issued - kStages; --j)
            tc::mbar_wait(&full[j % kStages], (unsigned)(j / kStages) & 1u);
    } else if (warp == 1 && lane == 0) {
        constexpr uint32_t idesc = tc::idesc_bf16(128, 32);
        bool ok = true;
        for (int j = 0; j < a.k_steps; ++j) {
            const int s = j % kStages;
            if (!tc::mbar_wait(&full[s], (unsigned)(j / kStages) & 1u)) {
                ok = false;
                break;
            }
            tc::tc_fence_after();
            unsigned char* st = base + s * kGemmStage;
            const uint64_t ad = tc::sdesc_sw64(st), bd = tc::sdesc_sw64(st + kTileA);
            tc::mma_bf16(tmem, ad, bd, idesc, j > 0 ? 1u : 0u);
            tc::mma_bf16(tmem, ad + 2, bd + 2, idesc, 1u);
            tc::mma_commit(&empty[s]);
        }
        if (!ok) {
            atomicOr(a.err, tc::kErrWait);
            fail = 1;
        }
        tc::mma_commit(&done);
    }
    __syncwarp();
    const bool got = tc::mbar_wait(&done, 0);
    tc::tc_fence_after();
    if (!got) atomicOr(a.err, tc::kErrWait);
    float acc[32];
    tc::tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16), acc);
    __syncthreads();
    const int m = mt * 128 + warp * 32 + lane;
    float* o = a.ws + ((size_t)split * kMPad + m) * 32;
#pragma unroll
    for (int c = 0; c < 32; ++c) o[c] = (got && !fail && a.k_steps > 0) ? acc[c] : 0.0f;
    if (!got) tc::mbar_wait(&done, 0);
    tc::tc_fence_before();
    __syncthreads();
    if (warp == 1) tc::tmem_dealloc(tmem, 32);
}

// xcol[t * 32 + c][g] = x[n][z + dz][y + dy][x + dx][c] (zero outside),
// g = n V + voxel < G, rows `ld` long; one thread per (voxel, tap).
__global__ void k_im2col_t(const __nv_bfloat16* __restrict__ x, __nv_bfloat16* __restrict__ xcol, int D, int H,
                           int W, long long G, long long ld) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= G * kTaps) return;
    const int t = (int)(i / G);
    const long long g = i % G;
    const int V = D * H * W;
    const int s = (int)(g / V), v = (int)(g % V);
    const int xx = v % W, yy = (v / W) % H, zz = v / (W * H);
    const int dz = t / 9 - 1, dy = (t / 3) % 3 - 1, dx = t % 3 - 1;
    const int z2 = zz + dz, y2 = yy + dy, x2 = xx + dx;
    __nv_bfloat16 vals[32];
    if (z2 >= 0 && z2 < D && y2 >= 0 && y2 < H && x2 >= 0 && x2 < W) {
        const uint4* p = reinterpret_cast<const uint4*>(x + (((size_t)s * D + z2) * H * W + (size_t)y2 * W + x2) * kCh);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const uint4 u = p[q];
            const __nv_bfloat16* h = reinterpret_cast<const __nv_bfloat16*>(&u);
#pragma unroll
            for (int j = 0; j < 8; ++j) vals[8 * q + j] = h[j];
        }
    } else {
#pragma unroll
        for (int c = 0; c < 32; ++c) vals[c] = __float2bfloat16_rn(0.0f);
    }
#pragma unroll
    for (int c = 0; c < 32; ++c) xcol[(size_t)(t * kCh + c) * ld + g] = vals[c];
}

// dyt[c][g] = d[g][c], g < G, rows `ld` long
__global__ void k_transpose_ch(const __nv_bfloat16* __restrict__ d, __nv_bfloat16* __restrict__ dyt, long long G,
                               long long ld) {
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= G) return;
    const uint4* p = reinterpret_cast<const uint4*>(d + g * kCh);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const uint4 u = p[q];
        const __nv_bfloat16* h = reinterpret_cast<const __nv_bfloat16*>(&u);
#pragma unroll
        for (int j = 0; j < 8; ++j) dyt[(size_t)(8 * q + j) * ld + g] = h[j];
    }
}

// dW[t][co][ci] = sum over splits of ws[s][t * 32 + ci][co] (fixed order)
__global__ void k_wgrad_reduce(const float* __restrict__ ws, int splits, float* __restrict__ gw) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kWElems) return;
    const int t = i / (kCh * kCh), co = (i / kCh) % kCh, ci = i % kCh;
    float s = 0.0f;
    for (int p = 0; p < splits; ++p) s += ws[((size_t)p * kMPad + t * kCh + ci) * kCh + co];
    gw[i] = s;
}

// db[c] = sum_g d[g][c]: per-block partials (double) then one block sums them
__global__ void k_bias_partial(const __nv_bfloat16* __restrict__ d, long long G, double* __restrict__ part) {
    __shared__ double sh[256];
    const int c = threadIdx.x & 31, r = threadIdx.x >> 5;   // 8 rows of 32 channels per pass
    double acc = 0.0;
    for (long long g = (long long)blockIdx.x * 8 + r; g < G; g += (long long)gridDim.x * 8)
        acc += (double)__bfloat162float(d[g * kCh + c]);
    sh[threadIdx.x] = acc;
    __syncthreads();
    if (r == 0) {
        double s = 0.0;
        for (int k = 0; k < 8; ++k) s += sh[k * 32 + c];
        part[(size_t)blockIdx.x * kCh + c] = s;
    }
}

__global__ void k_bias_final(const double* __restrict__ part, int nb, float* __restrict__ gb) {
    const int c = threadIdx.x;
    if (c >= kCh) return;
    double s = 0.0;
    for (int b = 0; b < nb; ++b) s += part[(size_t)b * kCh + c];
    gb[c] = (float)s;
}

// delta = dout (FP32 [G][c_out]) as BF16 [G][32]
__global__ void k_dout_to_delta(const float* __restrict__ dout, int c_out, long long G, __nv_bfloat16* __restrict__ d) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= G * kCh) return;
    const long long g = i / kCh;
    const int c = (int)(i % kCh);
    d[i] = __float2bfloat16_rn(c < c_out ? dout[g * c_out + c] : 0.0f);
}

// MSE loss: dout = (out - target) / (G), partial sums of (out - target)^2
__global__ void k_mse(const float* __restrict__ out, const float* __restrict__ target, long long n_el, double inv,
                      float* __restrict__ dout, double* __restrict__ part) {
    __shared__ double sh[256];
    double acc = 0.0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n_el; i += (long long)gridDim.x * blockDim.x) {
        const float df = out[i] - target[i];
        dout[i] = (float)(df * inv);
        acc += (double)df * df;
    }
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

// Adam on the FP32 masters of layer-padded weights and biases; entries
// outside a layer's channel block stay zero.  Then the BF16 forward copy and
// the transposed, tap-reversed copy of the input-gradient pass.
struct AdamArgs {
    float lr, b1, b2, eps, c1, c2;   // c1 = 1 / (1 - b1^t), c2 = 1 / (1 - b2^t)
};

__global__ void k_adam(float* __restrict__ w, float* __restrict__ m, float* __restrict__ v,
                       const float* __restrict__ g, long long n, AdamArgs a) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = a.b1 * m[i] + (1.0f - a.b1) * gi;
    const float vi = a.b2 * v[i] + (1.0f - a.b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= a.lr * (mi * a.c1) / (sqrtf(vi * a.c2) + a.eps);
}

__global__ void k_weights_bf16(const float* __restrict__ w32, const int* __restrict__ ci, const int* __restrict__ co,
                               int L, __nv_bfloat16* __restrict__ wbf, __nv_bfloat16* __restrict__ wtbf) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)L * kWElems) return;
    const int l = (int)(i / kWElems), r = (int)(i % kWElems);
    const int t = r / (kCh * kCh), o = (r / kCh) % kCh, c = r % kCh;
    const float x = (o < co[l] && c < ci[l]) ? w32[i] : 0.0f;
    wbf[i] = __float2bfloat16_rn(x);
    // transposed, reversed taps: wt[26 - t][c][o] = w[t][o][c]
    wtbf[(size_t)l * kWElems + ((size_t)(kTaps - 1 - t) * kCh + c) * kCh + o] = __float2bfloat16_rn(x);
}

// ---- tensor maps ----
using EncodeFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                              const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                              CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeFn encoder() {
    static EncodeFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, []() {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeFn>(p);
        cudaGetLastError();
    });
    if (!fn) throw std::runtime_error("cnn: cuTensorMapEncodeTiled not available");
    return fn;
}

}  // namespace

// box (32 channels, bw, bh, 1, 1); with halo = 1 (32, bw, bh + 2, 3, 1)
void encode_act_map(CUtensorMap* m, const void* base, int n, int D, int H, int W, int bw, int bh, int halo) {
    const cuuint64_t dims[5] = {(cuuint64_t)kCh, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)D, (cuuint64_t)n};
    const cuuint64_t strides[4] = {(cuuint64_t)kCh * 2, (cuuint64_t)W * kCh * 2, (cuuint64_t)H * W * kCh * 2,
                                   (cuuint64_t)D * H * W * kCh * 2};
    const cuuint32_t box[5] = {(cuuint32_t)kCh, (cuuint32_t)bw, (cuuint32_t)(bh + 2 * halo),
                               (cuuint32_t)(1 + 2 * halo), 1};
    const cuuint32_t es[5] = {1, 1, 1, 1, 1};
    const CUresult r = encoder()(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<void*>(base), dims, strides, box,
                                 es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
                                 CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) throw std::runtime_error("cnn: activation tensor map encode failed");
}

// rows x cols BF16, row-major (cols contiguous, a multiple of 32); box 32 x box_rows
void encode_2d_map(CUtensorMap* m, const void* base, long long cols, int rows, int box_rows) {
    const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)cols * 2};
    const cuuint32_t box[2] = {32, (cuuint32_t)box_rows};
    const cuuint32_t es[2] = {1, 1};
    const CUresult r = encoder()(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box,
                                 es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
                                 CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) throw std::runtime_error("cnn: 2-D tensor map encode failed");
}

// ---------------------------------------------------------------------------
// Cnn
// ---------------------------------------------------------------------------

template <class T>
static T* dmalloc(size_t n) {
    void* p = nullptr;
    if (n == 0) n = 1;
    if (cudaMalloc(&p, n * sizeof(T)) != cudaSuccess) {
        cudaGetLastError();
        throw std::bad_alloc();
    }
    return static_cast<T*>(p);
}

template <class T>
static void dfree(T*& p) {
    if (p) cudaFree(p);
    p = nullptr;
}

Cnn::Cnn(int device, int layers, int c_in, int hidden, int c_out, unsigned seed)
    : dev(device), L(layers), cin(c_in), hid(hidden), cout(c_out) {
    if (L < 2 || cin < 1 || cin > kCh || cout < 1 || cout > kCh || hid < 1 || hid > kCh)
        throw std::invalid_argument("cnn: layers >= 2, channels 1..32");
    ck(cudaSetDevice(dev), "cudaSetDevice");
    ck(cudaStreamCreateWithFlags(&own_st, cudaStreamNonBlocking), "stream");
    st = own_st;
    ci.assign(L, hid);
    co.assign(L, hid);
    ci[0] = cin;
    co[L - 1] = cout;
    const size_t nw = (size_t)L * kWElems, nb = (size_t)L * kCh;
    w32 = dmalloc<float>(nw); mw = dmalloc<float>(nw); vw = dmalloc<float>(nw); gw = dmalloc<float>(nw);
    b32 = dmalloc<float>(nb); mb = dmalloc<float>(nb); vb = dmalloc<float>(nb); gb = dmalloc<float>(nb);
    wbf = dmalloc<__nv_bfloat16>(nw);
    wtbf = dmalloc<__nv_bfloat16>(nw);
    err = dmalloc<unsigned>(1);
    ck(cudaMemset(err, 0, sizeof(unsigned)), "memset");
    dch = dmalloc<int>(2 * L);
    {
        std::vector<int> h(2 * L);
        for (int l = 0; l < L; ++l) { h[l] = ci[l]; h[L + l] = co[l]; }
        ck(cudaMemcpy(dch, h.data(), sizeof(int) * 2 * L, cudaMemcpyHostToDevice), "channels");
    }
    for (float* p : {mw, vw, gw}) ck(cudaMemset(p, 0, nw * sizeof(float)), "memset");
    for (float* p : {mb, vb, gb}) ck(cudaMemset(p, 0, nb * sizeof(float)), "memset");
    // He initialisation (normal, std sqrt(2 / fan_in)), zero biases
    std::mt19937 rng(seed);
    std::vector<float> hw(nw, 0.0f), hb(nb, 0.0f);
    for (int l = 0; l < L; ++l) {
        std::normal_distribution<float> nd(0.0f, std::sqrt(2.0f / (kTaps * ci[l])));
        for (int t = 0; t < kTaps; ++t)
            for (int o = 0; o < co[l]; ++o)
                for (int c = 0; c < ci[l]; ++c) hw[(size_t)l * kWElems + ((size_t)t * kCh + o) * kCh + c] = nd(rng);
    }
    set_weights(hw.data(), hb.data());
    w_map.resize(L);
    wt_map.resize(L);
    for (int l = 0; l < L; ++l) {
        encode_2d_map(&w_map[l], wbf + (size_t)l * kWElems, kCh, kTaps * kCh, kCh);
        encode_2d_map(&wt_map[l], wtbf + (size_t)l * kWElems, kCh, kTaps * kCh, kCh);
    }
}

Cnn::~Cnn() {
    cudaSetDevice(dev);
    free_grid();
    for (float** p : {&w32, &mw, &vw, &gw, &b32, &mb, &vb, &gb}) dfree(*p);
    dfree(wbf);
    dfree(wtbf);
    dfree(err);
    dfree(dch);
    if (own_st) cudaStreamDestroy(own_st);   // never a caller's stream (set_stream)
}

void Cnn::free_grid() {
    for (auto*& p : act) dfree(p);
    act.clear();
    dfree(delta[0]);
    dfree(delta[1]);
    dfree(out32);
    dfree(dout32);
    dfree(xcol);
    dfree(dyt);
    dfree(ws);
    dfree(red);
    n_cap = 0;
}

void Cnn::upload_bf16() {
    const long long n = (long long)L * kWElems;
    k_weights_bf16<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(w32, dch, dch + L, L, wbf, wtbf);
    ck(cudaGetLastError(), "weights");
    ck(cudaStreamSynchronize(st), "sync");
}

void Cnn::set_weights(const float* w, const float* b) {
    ck(cudaSetDevice(dev), "cudaSetDevice");
    const size_t nw = (size_t)L * kWElems, nb = (size_t)L * kCh;
    std::vector<float> hw(w, w + nw), hb(b, b + nb);
    for (int l = 0; l < L; ++l) {   // keep the padding zero
        for (int t = 0; t < kTaps; ++t)
            for (int o = 0; o < kCh; ++o)
                for (int c = 0; c < kCh; ++c)
                    if (o >= co[l] || c >= ci[l]) hw[(size_t)l * kWElems + ((size_t)t * kCh + o) * kCh + c] = 0.0f;
        for (int o = co[l]; o < kCh; ++o) hb[(size_t)l * kCh + o] = 0.0f;
    }
    ck(cudaMemcpyAsync(w32, hw.data(), nw * sizeof(float), cudaMemcpyHostToDevice, st), "w");
    ck(cudaMemcpyAsync(b32, hb.data(), nb * sizeof(float), cudaMemcpyHostToDevice, st), "b");
    upload_bf16();
}

void Cnn::get_weights(float* w, float* b) const {
    ck(cudaMemcpy(w, w32, (size_t)L * kWElems * sizeof(float), cudaMemcpyDeviceToHost), "w");
    ck(cudaMemcpy(b, b32, (size_t)L * kCh * sizeof(float), cudaMemcpyDeviceToHost), "b");
}

void Cnn::get_grads(float* dw, float* db) const {
    ck(cudaStreamSynchronize(st), "sync");
    ck(cudaMemcpy(dw, gw, (size_t)L * kWElems * sizeof(float), cudaMemcpyDeviceToHost), "dw");
    ck(cudaMemcpy(db, gb, (size_t)L * kCh * sizeof(float), cudaMemcpyDeviceToHost), "db");
}

unsigned Cnn::error_flag() {
    unsigned e = 0;
    ck(cudaMemcpyAsync(&e, err, sizeof(unsigned), cudaMemcpyDeviceToHost, st), "err");
    ck(cudaStreamSynchronize(st), "sync");
    if (e) {
        const unsigned z = 0;
        ck(cudaMemcpyAsync(err, &z, sizeof(unsigned), cudaMemcpyHostToDevice, st), "err");
        ck(cudaStreamSynchronize(st), "sync");
    }
    return e;
}

void Cnn::ensure(int n, int D_, int H_, int W_) {
    if (W_ != 16 && W_ != 32 && W_ != 64 && W_ != 128)
        throw std::invalid_argument("cnn: grid W must be 16, 32, 64 or 128");
    const int bw_ = W_, bh_ = 128 / W_;
    if (H_ % bh_ != 0 || D_ < 1 || n < 1) throw std::invalid_argument("cnn: grid H must be a multiple of 128 / W");
    if (n <= n_cap && D_ == D && H_ == H && W_ == W) return;
    ck(cudaSetDevice(dev), "cudaSetDevice");
    free_grid();
    D = D_; H = H_; W = W_; V = D * H * W; bw = bw_; bh = bh_;
    n_cap = n;
    const size_t G = (size_t)n * V;
    act.assign(L + 1, nullptr);
    for (auto*& p : act) {
        p = dmalloc<__nv_bfloat16>(G * kCh);
        ck(cudaMemsetAsync(p, 0, G * kCh * 2, st), "memset");
    }
    for (auto*& p : delta) p = dmalloc<__nv_bfloat16>(G * kCh);
    out32 = dmalloc<float>(G * cout);
    dout32 = dmalloc<float>(G * cout);
    xcol = dmalloc<__nv_bfloat16>((size_t)kMPad * G);
    ck(cudaMemsetAsync(xcol, 0, (size_t)kMPad * G * 2, st), "memset");   // rows 864.. stay zero
    dyt = dmalloc<__nv_bfloat16>((size_t)kCh * G);
    const long long ksteps = (long long)G / 32;
    splits = (int)std::max<long long>(1, std::min<long long>(64, ksteps / 8));
    ws = dmalloc<float>((size_t)splits * kMPad * kCh);
    red = dmalloc<double>(4096 * kCh);
    act_map.resize(L + 1);
    for (int l = 0; l <= L; ++l) encode_act_map(&act_map[l], act[l], n, D, H, W, bw, bh);
    delta_map.resize(2);
    for (int k = 0; k < 2; ++k) encode_act_map(&delta_map[k], delta[k], n, D, H, W, bw, bh);
    act_hmap.assign(L + 1, CUtensorMap{});
    delta_hmap.assign(2, CUtensorMap{});
    if (W <= kHaloMaxW) {
        for (int l = 0; l <= L; ++l) encode_act_map(&act_hmap[l], act[l], n, D, H, W, bw, bh, 1);
        for (int k = 0; k < 2; ++k) encode_act_map(&delta_hmap[k], delta[k], n, D, H, W, bw, bh, 1);
    }
    encode_2d_map(&xcol_map, xcol, (long long)G, kMPad, 128);
    encode_2d_map(&dyt_map, dyt, (long long)G, kCh, kCh);
    ck(cudaStreamSynchronize(st), "sync");
}

void Cnn::conv(int l, bool transposed, const CUtensorMap& in_map, const CUtensorMap& in_hmap,
               const __nv_bfloat16* mask, __nv_bfloat16* out, float* o32, int n32, int n) {
    static bool attr = false;
    if (!attr) {
        ck(cudaFuncSetAttribute(k_conv3d_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kConvSmem), "attr");
        ck(cudaFuncSetAttribute(k_conv3d_halo, cudaFuncAttributeMaxDynamicSharedMemorySize, halo_smem(kHaloMaxW)),
           "attr");
        attr = true;
    }
    ConvArgs a{};
    a.D = D; a.H = H; a.W = W; a.bw = bw; a.bh = bh; a.tiles_h = H / bh;
    a.bias = transposed ? nullptr : b32 + (size_t)l * kCh;
    a.relu = (!transposed && l < L - 1) ? 1 : 0;
    a.mask = mask;
    a.out = out;
    a.out32 = o32;
    a.n32 = n32;
    a.err = err;
    a.n_tiles = n * D * (H / bh);
    if (W <= kHaloMaxW) {
        // persistent CTAs, one per SM (up to 198 KB of shared memory each)
        static int sms = 0;
        if (!sms) ck(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count");
        const int grid = std::max(1, std::min(a.n_tiles, sms));
        k_conv3d_halo<<<grid, 192, halo_smem(W), st>>>(in_hmap, transposed ? wt_map[l] : w_map[l], a);
    } else {
        k_conv3d_tc<<<a.n_tiles, 128, kConvSmem, st>>>(in_map, transposed ? wt_map[l] : w_map[l], a);
    }
    ck(cudaGetLastError(), "conv launch");
}

const float* Cnn::forward(int n) {
    if (n > n_cap) throw std::invalid_argument("cnn: more samples than ensure() sized");
    ck(cudaSetDevice(dev), "cudaSetDevice");
    for (int l = 0; l < L; ++l)
        conv(l, false, act_map[l], act_hmap[l], nullptr, act[l + 1], l == L - 1 ? out32 : nullptr, cout, n);
    return out32;
}

void Cnn::wgrad(int l, const __nv_bfloat16* x, const __nv_bfloat16* d, int n) {
    static bool attr = false;
    if (!attr) {
        ck(cudaFuncSetAttribute(k_gemm_tn_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kGemmSmem), "attr");
        attr = true;
    }
    const long long G = (long long)n * V;
    const long long Gcap = (long long)n_cap * V;
    // the operand rows are n_cap samples long (the tensor maps' extent);
    // only this call's first G columns are written and read
    k_im2col_t<<<(unsigned)((G * kTaps + 255) / 256), 256, 0, st>>>(x, xcol, D, H, W, G, Gcap);
    k_transpose_ch<<<(unsigned)((G + 255) / 256), 256, 0, st>>>(d, dyt, G, Gcap);
    ck(cudaGetLastError(), "im2col");
    // K split over CTAs: the largest divisor of the 32-voxel step count
    // not above `splits`
    const long long ksteps = G / 32;
    int sp = (int)std::max<long long>(1, std::min<long long>(splits, ksteps));
    while (ksteps % sp) --sp;
    GemmArgs a{(int)(ksteps / sp), ws, err};
    k_gemm_tn_tc<<<dim3(kMPad / 128, sp), 128, kGemmSmem, st>>>(xcol_map, dyt_map, a);
    ck(cudaGetLastError(), "gemm launch");
    k_wgrad_reduce<<<(kWElems + 255) / 256, 256, 0, st>>>(ws, sp, gw + (size_t)l * kWElems);
    const int nb = (int)std::min<long long>(4096, (G + 7) / 8);
    k_bias_partial<<<nb, 256, 0, st>>>(d, G, red);
    k_bias_final<<<1, 32, 0, st>>>(red, nb, gb + (size_t)l * kCh);
    ck(cudaGetLastError(), "wgrad");
}

void Cnn::backward(int n, const float* dout, float* dx) {
    ck(cudaSetDevice(dev), "cudaSetDevice");
    const long long G = (long long)n * V;
    k_dout_to_delta<<<(unsigned)((G * kCh + 255) / 256), 256, 0, st>>>(dout, cout, G, delta[0]);
    ck(cudaGetLastError(), "delta");
    int cur = 0;
    for (int l = L - 1; l >= 0; --l) {
        wgrad(l, act[l], delta[cur], n);
        if (l > 0 || dx) {
            // input gradient; for l > 0 masked by ReLU'(act[l]) into the next delta
            conv(l, true, delta_map[cur], delta_hmap[cur], l > 0 ? act[l] : nullptr, delta[cur ^ 1],
                 (l == 0 && dx) ? dx : nullptr, kCh, n);
            cur ^= 1;
        }
    }
}

double Cnn::loss_backward(int n, const float* target) {
    const long long G = (long long)n * V;
    const long long n_el = G * cout;
    const int nb = 1024;
    k_mse<<<nb, 256, 0, st>>>(out32, target, n_el, 1.0 / (double)G, dout32, red);
    ck(cudaGetLastError(), "mse");
    std::vector<double> h(nb);
    ck(cudaMemcpyAsync(h.data(), red, nb * sizeof(double), cudaMemcpyDeviceToHost, st), "loss");
    backward(n, dout32, nullptr);
    ck(cudaStreamSynchronize(st), "sync");
    double s = 0.0;
    for (double v : h) s += v;
    return 0.5 * s / (double)G;
}

void Cnn::adam_step(float lr, float beta1, float beta2, float eps) {
    ++adam_t;
    AdamArgs a{lr, beta1, beta2, eps, (float)(1.0 / (1.0 - std::pow((double)beta1, (double)adam_t))),
               (float)(1.0 / (1.0 - std::pow((double)beta2, (double)adam_t)))};
    const long long nw = (long long)L * kWElems, nb = (long long)L * kCh;
    k_adam<<<(unsigned)((nw + 255) / 256), 256, 0, st>>>(w32, mw, vw, gw, nw, a);
    k_adam<<<(unsigned)((nb + 255) / 256), 256, 0, st>>>(b32, mb, vb, gb, nb, a);
    ck(cudaGetLastError(), "adam");
    upload_bf16();
}

// ---------------------------------------------------------------------------
// dense-grid view of edge fields
// ---------------------------------------------------------------------------

namespace {

__global__ void k_sigma_feature(GridMap g, const double* __restrict__ sigma) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.n_cells) return;
    double s = 0.0;
    const int b = g.sig_ptr[c], e = g.sig_ptr[c + 1];
    for (int q = b; q < e; ++q) s += log10(sigma[g.sig_leaf[q]]);
    g.sig_feat[c] = e > b ? (float)((s / (e - b) + 2.0) / 3.0) : 0.0f;
}

// means[k][c][2 d + (re, im)] over the rows of (c, d); one thread per (c, k)
template <class C>
__global__ void k_grid_means(GridMap g, const C* __restrict__ v, int K, float* __restrict__ out) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)g.n_cells * K) return;
    const int c = (int)(i / K), k = (int)(i % K);
    float* o = out + ((size_t)k * g.n_cells + c) * kOutCh;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const int b = g.cd_ptr[3 * c + d], e = g.cd_ptr[3 * c + d + 1];
        double re = 0.0, im = 0.0;
        for (int q = b; q < e; ++q) {
            const C x = v[(size_t)g.cd_row[q] * K + k];
            re += (double)x.x;
            im += (double)x.y;
        }
        const double inv = e > b ? 1.0 / (e - b) : 0.0;
        o[2 * d] = (float)(re * inv);
        o[2 * d + 1] = (float)(im * inv);
    }
}

// per-lane sum of squares of the means: one block per lane, fixed order
__global__ void k_lane_rms(const float* __restrict__ m, int n, float* __restrict__ rms) {
    __shared__ double sh[256];
    const int k = blockIdx.x;
    const float* p = m + (size_t)k * n;
    double acc = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) acc += (double)p[i] * p[i];
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) rms[k] = (float)sqrt(sh[0] / n);
}

__global__ void k_grid_input(GridMap g, const float* __restrict__ m, const float* __restrict__ rms, int K,
                             const double* __restrict__ freq, __nv_bfloat16* __restrict__ in) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)g.n_cells * K) return;
    const int k = (int)(i / g.n_cells), c = (int)(i % g.n_cells);
    const float sc = rms[k] > 0.0f ? 1.0f / rms[k] : 0.0f;
    const float* p = m + ((size_t)k * g.n_cells + c) * kOutCh;
    __nv_bfloat16 vals[kCh];
#pragma unroll
    for (int j = 0; j < kCh; ++j) vals[j] = __float2bfloat16_rn(0.0f);
#pragma unroll
    for (int j = 0; j < kOutCh; ++j) vals[j] = __float2bfloat16_rn(p[j] * sc);
    vals[6] = __float2bfloat16_rn(g.sig_feat[c]);
    vals[7] = __float2bfloat16_rn(freq[k] > 0.0 ? (float)(log10(freq[k]) / 3.0) : 0.0f);
    uint4* o = reinterpret_cast<uint4*>(in + ((size_t)k * g.n_cells + c) * kCh);
#pragma unroll
    for (int q = 0; q < 4; ++q) o[q] = reinterpret_cast<const uint4*>(vals)[q];
}

__global__ void k_grid_prolong(GridMap g, const float* __restrict__ out, int K, float2* __restrict__ z) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)g.n_pad * K) return;
    const int row = (int)(i / K), k = (int)(i % K);
    const int c = g.row_cell[row];
    float2 r = make_float2(0.0f, 0.0f);
    if (c >= 0) {
        const int d = g.row_dir[row];
        const float* p = out + ((size_t)k * g.n_cells + c) * kOutCh;
        r = make_float2(p[2 * d], p[2 * d + 1]);
    }
    z[i] = r;
}

template <class C>
void features_impl(const GridMap& g, const C* v, int K, const double* freq, __nv_bfloat16* in, float* work,
                   cudaStream_t s) {
    const long long n = (long long)g.n_cells * K;
    k_grid_means<C><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(g, v, K, work);
    float* rms = work + (size_t)K * g.n_cells * kOutCh;
    k_lane_rms<<<K, 256, 0, s>>>(work, g.n_cells * kOutCh, rms);
    k_grid_input<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(g, work, rms, K, freq, in);
    ck(cudaGetLastError(), "grid features");
}

}  // namespace

void grid_sigma_feature(const GridMap& g, const double* sigma, cudaStream_t s) {
    k_sigma_feature<<<(g.n_cells + 255) / 256, 256, 0, s>>>(g, sigma);
    ck(cudaGetLastError(), "sigma feature");
}

void grid_features(const GridMap& g, const double2* v, int K, const double* freq, __nv_bfloat16* in, float* work,
                   cudaStream_t s) {
    features_impl(g, v, K, freq, in, work, s);
}

void grid_features(const GridMap& g, const float2* v, int K, const double* freq, __nv_bfloat16* in, float* work,
                   cudaStream_t s) {
    features_impl(g, v, K, freq, in, work, s);
}

void grid_means(const GridMap& g, const double2* v, int K, float* out, cudaStream_t s) {
    const long long n = (long long)g.n_cells * K;
    k_grid_means<double2><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(g, v, K, out);
    ck(cudaGetLastError(), "grid means");
}

void grid_prolong(const GridMap& g, const float* out, int K, float2* z, cudaStream_t s) {
    const long long n = (long long)g.n_pad * K;
    k_grid_prolong<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(g, out, K, z);
    ck(cudaGetLastError(), "grid prolong");
}

}  // namespace learn
}  // namespace m3d
