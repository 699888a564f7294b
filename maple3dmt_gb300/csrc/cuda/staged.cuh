// Slice-staged operator rows: the off-diagonal matrix, split into its lower
// (earlier colour) and upper parts, is stored per 32-row slice as a
// contiguous segment that one bulk asynchronous copy (cp.async.bulk, the
// TMA engine's 1-D mode) moves into shared memory:
//
//   segment = [uint16 end[32]]                 row r owns entries [end[r-1], end[r])
//             [int32 col[n]]
//             [R val[n]]
//
// with every row padded to a multiple of four entries (padding entries point
// at the row itself with value 0), so rows start on 16-byte boundaries and
// are read four entries at a time, and every segment starts and ends on a
// 16-byte boundary.  A slice's work item
// (int4) is {slice, lower offset, upper offset, (lower length << 16) | upper
// length}, offsets and lengths in 16-byte units.  Kernels keep two segments in
// flight per block (double buffering on two mbarriers): the next slice's
// matrix stream arrives while the current slice's gathers run.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "common.cuh"

namespace m3d {
namespace dev {

constexpr int kSegHeader = 64;                  // bytes of the row-end table
constexpr long long kWaitCycles = 4000000000LL;  // bound of every barrier wait (~2 s)
constexpr unsigned kErrCopyTimeout = 1u;
// Test hook, set by the host in the same flag word: with this bit set, the
// consume wait of every staged kernel polls its barrier once without
// blocking and takes the timeout path if the copy has not landed; the drain
// wait for a copy in flight keeps its full bound.
constexpr unsigned kTestConsumeNoWait = 1u << 31;

template <class R>
struct SegView {
    const unsigned char* seg;   // all segments of one precision
    const int4* work_nat;       // [n_slices] natural slice order (SpMV)
    const int4* work_col;       // colour sweep order (slices of colour c at colour_ptr[c])
    int stage_spmv;             // bytes of the largest lower + upper segment pair
    int stage_lo;               // bytes of the largest lower segment
    int stage_up;               // bytes of the largest upper segment
    unsigned* err;              // device flag, kErrCopyTimeout on a barrier timeout
};

__device__ __forceinline__ unsigned smem_addr(const void* p) {
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_inval(uint64_t* bar) {
    asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// orders this thread's generic-proxy shared-memory accesses before later
// async-proxy (bulk copy) accesses
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

// global -> shared bulk copy; dst, src 16-byte aligned, bytes a multiple of 16
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Non-blocking test of phase `parity` of `bar`.
__device__ __forceinline__ bool mbar_test_wait(uint64_t* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Waits for phase `parity` of `bar` for at most kWaitCycles; false on timeout.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity) {
    if (mbar_try_wait(bar, parity)) return true;
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity))
        if (clock64() - t0 > kWaitCycles) return false;
    return true;
}

// Unpacked work item.
struct SegItem {
    int slice;
    int lo_off, up_off;   // 16-byte units
    int lo_len, up_len;   // 16-byte units
};

__device__ __forceinline__ SegItem unpack(int4 w) {
    SegItem it;
    it.slice = w.x;
    it.lo_off = w.y;
    it.up_off = w.z;
    it.lo_len = (int)((unsigned)w.w >> 16);
    it.up_len = (int)((unsigned)w.w & 0xffffu);
    return it;
}

// Row r's entry range of a staged segment and its column / value arrays.
template <class R>
struct SegRows {
    const uint16_t* end;
    const int* col;
    const R* val;
    __device__ __forceinline__ void bind(const unsigned char* base) {
        end = reinterpret_cast<const uint16_t*>(base);
        const int n = end[kSlice - 1];
        col = reinterpret_cast<const int*>(base + kSegHeader);
        val = reinterpret_cast<const R*>(base + kSegHeader + 4 * n);
    }
    __device__ __forceinline__ int begin_of(int r) const { return r ? end[r - 1] : 0; }
};


// Threads per block of the staged kernels and passes over a 32-row slice:
// K lanes per row, so a slice is 32 K lane-rows; up to 256 threads per block.
template <int K> struct StagedShape {
    static constexpr int NT = (32 * K < 256) ? 32 * K : 256;
    static constexpr int PASSES = 32 * K / NT;
    static constexpr int ROWS_PER_PASS = 32 / PASSES;
};

// Persistent slice pipeline of one block: work items i = blockIdx.x,
// blockIdx.x + gridDim.x, ... < n_items; item i's lower (PARTS & 1) and upper
// (PARTS & 2) segments are bulk-copied into stage k & 1 one item ahead of
// use, so the next slice's matrix stream is in flight while body() runs.
// Every thread waits (bounded) on the stage's barrier itself; the one block
// barrier per item also ORs the threads' outcomes, so the whole block takes
// the same branch: on a timeout it sets kErrCopyTimeout in *err, skips the
// stage, waits (bounded) for the late copy and stops.  The call's results
// are then invalid and the host reports the error.
template <int PARTS, class Body>
__device__ __forceinline__ void slice_pipeline(const unsigned char* __restrict__ seg, const int4* __restrict__ work,
                                               long n_items, int stage_bytes, unsigned* err, Body body) {
    extern __shared__ __align__(128) unsigned char dsm[];
    __shared__ __align__(8) uint64_t bar[2];
    __shared__ int4 wk[2];
    __shared__ int no_wait;
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_mbar_init();
        no_wait = (*reinterpret_cast<volatile unsigned*>(err) & kTestConsumeNoWait) != 0;
    }
    __syncthreads();
    auto issue = [&](long i, int stg) {   // thread 0 only
        const int4 w = __ldg(&work[i]);
        wk[stg] = w;
        const SegItem it = unpack(w);
        unsigned bytes = 0;
        if (PARTS & 1) bytes += (unsigned)it.lo_len * 16u;
        if (PARTS & 2) bytes += (unsigned)it.up_len * 16u;
        unsigned char* dst = dsm + (size_t)stg * stage_bytes;
        mbar_expect_tx(&bar[stg], bytes);
        if (PARTS & 1) {
            bulk_g2s(dst, seg + (size_t)it.lo_off * 16, (unsigned)it.lo_len * 16u, &bar[stg]);
            dst += (size_t)it.lo_len * 16;
        }
        if (PARTS & 2) bulk_g2s(dst, seg + (size_t)it.up_off * 16, (unsigned)it.up_len * 16u, &bar[stg]);
    };
    auto wait_stage = [&](int stg, unsigned parity) {
        return no_wait ? mbar_test_wait(&bar[stg], parity) : mbar_wait_bounded(&bar[stg], parity);
    };
    // every exit leaves the barriers invalidated, so that a kernel may run
    // the pipeline again (one sweep group after another)
    auto finish = [&]() {
        __syncthreads();
        if (threadIdx.x == 0) {
            mbar_inval(&bar[0]);
            mbar_inval(&bar[1]);
        }
        __syncthreads();
    };
    long i = blockIdx.x;
    if (i >= n_items) {   // uniform: the whole block has no item
        finish();
        return;
    }
    if (threadIdx.x == 0) issue(i, 0);
    // outcome of the wait for the item about to be consumed, block-uniform
    bool fail = __syncthreads_or(!wait_stage(0, 0u)) != 0;
    int k = 0;
    for (;;) {
        const int stg = k & 1;
        if (fail) {
            // never consume a stage that did not arrive; let the late copy
            // land (bounded) before the block leaves
            if (threadIdx.x == 0) {
                atomicOr(err, kErrCopyTimeout);
                mbar_wait_bounded(&bar[stg], (unsigned)(k >> 1) & 1u);
            }
            finish();
            return;
        }
        const long next = i + gridDim.x;
        if (threadIdx.x == 0 && next < n_items) {
            fence_proxy_async_smem();
            issue(next, stg ^ 1);
        }
        body(unpack(wk[stg]), dsm + (size_t)stg * stage_bytes);
        if (next >= n_items) {
            finish();
            return;
        }
        // wait for the next item's stage; the same barrier ends this item
        fail = __syncthreads_or(!wait_stage(stg ^ 1, (unsigned)((k + 1) >> 1) & 1u)) != 0;
        i = next;
        ++k;
    }
}

// Barrier over all blocks of a cooperative launch (every block resident):
// an arrival counter and a generation word in global memory, the wait
// bounded by kWaitCycles; a timeout sets kErrCopyTimeout in *err and lets the
// block go on (the call's results are then invalid).  The last block to
// arrive resets the counter before it moves the generation on.
__device__ __forceinline__ void grid_barrier(unsigned* count, unsigned* gen, unsigned* err) {
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned* vgen = gen;
        const unsigned g = *vgen;
        __threadfence();
        const unsigned nb = gridDim.x * gridDim.y * gridDim.z;
        if (atomicAdd(count, 1u) == nb - 1) {
            *reinterpret_cast<volatile unsigned*>(count) = 0u;
            __threadfence();
            atomicAdd(gen, 1u);
        } else {
            const long long t0 = clock64();
            while (*vgen == g)
                if (clock64() - t0 > kWaitCycles) {
                    atomicOr(err, kErrCopyTimeout);
                    break;
                }
        }
        __threadfence();
    }
    __syncthreads();
}

// Four values of a staged row from shared memory.
__device__ __forceinline__ void lds4(const float* p, float (&a)[4]) {
    const float4 q = *reinterpret_cast<const float4*>(p);
    a[0] = q.x; a[1] = q.y; a[2] = q.z; a[3] = q.w;
}
__device__ __forceinline__ void lds4(const double* p, double (&a)[4]) {
    const double2 q0 = *reinterpret_cast<const double2*>(p);
    const double2 q1 = *reinterpret_cast<const double2*>(p + 2);
    a[0] = q0.x; a[1] = q0.y; a[2] = q1.x; a[3] = q1.y;
}

// The first eight entries of one staged row [b, e) (b, e multiples of 4):
// values read from shared memory and the gathers v[c_j][rhs] issued, summed
// later by sum() in entry order (entries past e are zero).  A sweep loads the
// heads of all its passes' rows before it writes the first one, so the
// gathers of every pass are in flight together; the rows of one colour are
// independent, which makes the early loads exact.
template <class R, int K>
struct RowHead {
    R a[8];
    cplx<R> x[8];
    __device__ __forceinline__ void load(const int* __restrict__ col, const R* __restrict__ val, int b, int e,
                                         const cplx<R>* v, int rhs) {
#pragma unroll
        for (int g = 0; g < 2; ++g) {
            const int k = b + 4 * g;
            if (k < e) {
                const int4 c = *reinterpret_cast<const int4*>(col + k);
                R q[4];
                lds4(val + k, q);
#pragma unroll
                for (int u = 0; u < 4; ++u) a[4 * g + u] = q[u];
                x[4 * g + 0] = v[(size_t)c.x * K + rhs];
                x[4 * g + 1] = v[(size_t)c.y * K + rhs];
                x[4 * g + 2] = v[(size_t)c.z * K + rhs];
                x[4 * g + 3] = v[(size_t)c.w * K + rhs];
            } else {
#pragma unroll
                for (int u = 0; u < 4; ++u) { a[4 * g + u] = (R)0; x[4 * g + u] = cm<R>(0, 0); }
            }
        }
    }
    __device__ __forceinline__ cplx<R> sum(cplx<R> s) const {
#pragma unroll
        for (int u = 0; u < 8; ++u) { s.x += a[u] * x[u].x; s.y += a[u] * x[u].y; }
        return s;
    }
};

// s + sum over one staged row's entries [b, e) (b, e multiples of 4) of
// a_j * v[c_j][rhs]: 16-byte shared-memory reads, eight gathers in flight,
// sums in entry order.
template <class R, int K>
__device__ __forceinline__ cplx<R> seg_row_dot(const int* __restrict__ col, const R* __restrict__ val, int b, int e,
                                               const cplx<R>* __restrict__ v, int rhs, cplx<R> s) {
    using C = cplx<R>;
    for (int k = b; k < e; k += 8) {
        const bool two = k + 4 < e;
        const int4 c0 = *reinterpret_cast<const int4*>(col + k);
        R a0[4], a1[4] = {0, 0, 0, 0};
        lds4(val + k, a0);
        C x[8];
        x[0] = v[(size_t)c0.x * K + rhs];
        x[1] = v[(size_t)c0.y * K + rhs];
        x[2] = v[(size_t)c0.z * K + rhs];
        x[3] = v[(size_t)c0.w * K + rhs];
        if (two) {
            const int4 c1 = *reinterpret_cast<const int4*>(col + k + 4);
            lds4(val + k + 4, a1);
            x[4] = v[(size_t)c1.x * K + rhs];
            x[5] = v[(size_t)c1.y * K + rhs];
            x[6] = v[(size_t)c1.z * K + rhs];
            x[7] = v[(size_t)c1.w * K + rhs];
        } else {
#pragma unroll
            for (int u = 4; u < 8; ++u) x[u] = cm<R>(0, 0);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) { s.x += a0[u] * x[u].x; s.y += a0[u] * x[u].y; }
#pragma unroll
        for (int u = 0; u < 4; ++u) { s.x += a1[u] * x[4 + u].x; s.y += a1[u] * x[4 + u].y; }
    }
    return s;
}

// Lower and upper parts of one staged row: the first (up to) eight entries of
// each part are gathered in one round, longer rows continue part by part.
template <class R, int K>
__device__ __forceinline__ cplx<R> seg_row_dot_lu(const SegRows<R>& lo, const SegRows<R>& up, int r,
                                                  const cplx<R>* __restrict__ v, int rhs) {
    using C = cplx<R>;
    const int bl = lo.begin_of(r), el = lo.end[r];
    const int bu = up.begin_of(r), eu = up.end[r];
    const bool on[4] = {bl < el, bl + 4 < el, bu < eu, bu + 4 < eu};
    const int at[4] = {bl, bl + 4, bu, bu + 4};
    R a[4][4];
    C x[16];
#pragma unroll
    for (int g = 0; g < 4; ++g) {
        const SegRows<R>& P = g < 2 ? lo : up;
        if (on[g]) {
            const int4 c = *reinterpret_cast<const int4*>(P.col + at[g]);
            lds4(P.val + at[g], a[g]);
            x[4 * g + 0] = v[(size_t)c.x * K + rhs];
            x[4 * g + 1] = v[(size_t)c.y * K + rhs];
            x[4 * g + 2] = v[(size_t)c.z * K + rhs];
            x[4 * g + 3] = v[(size_t)c.w * K + rhs];
        } else {
#pragma unroll
            for (int u = 0; u < 4; ++u) { a[g][u] = (R)0; x[4 * g + u] = cm<R>(0, 0); }
        }
    }
    C s = cm<R>(0, 0);
#pragma unroll
    for (int g = 0; g < 2; ++g)
#pragma unroll
        for (int u = 0; u < 4; ++u) { s.x += a[g][u] * x[4 * g + u].x; s.y += a[g][u] * x[4 * g + u].y; }
    if (bl + 8 < el) s = seg_row_dot<R, K>(lo.col, lo.val, bl + 8, el, v, rhs, s);
#pragma unroll
    for (int g = 2; g < 4; ++g)
#pragma unroll
        for (int u = 0; u < 4; ++u) { s.x += a[g][u] * x[4 * g + u].x; s.y += a[g][u] * x[4 * g + u].y; }
    if (bu + 8 < eu) s = seg_row_dot<R, K>(up.col, up.val, bu + 8, eu, v, rhs, s);
    return s;
}

// Register cap of the staged kernels: 768 resident threads per SM for
// complex FP32, 512 for complex FP64 (sixteen gathers in flight per thread).
template <class R, int K> struct StagedMinBlocks {
    static constexpr int t = (sizeof(R) == 8 ? 512 : 768) / StagedShape<K>::NT;
    static constexpr int v = t > 0 ? t : 1;
};

// Launches one staged kernel: at most one resident wave of blocks (of
// StagedShape<K>::NT threads with two stages of dynamic shared memory), no
// more than there are work items, no more than `cap`.
template <class F, class... Args>
inline void launch_staged(F* kernel, int nt, int stage_bytes, long items, int cap, cudaStream_t st, Args... args) {
    const int smem = 2 * stage_bytes;
    if (smem > 48 * 1024)
        cudaFuncSetAttribute(reinterpret_cast<const void*>(kernel), cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    long g = std::min<long>((long)wave_grid(kernel, cap, nt, smem), std::max<long>(items, 1));
    kernel<<<(int)g, nt, smem, st>>>(args...);
}

}  // namespace dev
}  // namespace m3d
