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
#include <cstdint>

#include "common.cuh"

namespace m3d {
namespace dev {

constexpr int kSegHeader = 64;                  // bytes of the row-end table
constexpr long long kWaitCycles = 4000000000LL;  // bound of every barrier wait (~2 s)
constexpr unsigned kErrCopyTimeout = 1u;

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

}  // namespace dev
}  // namespace m3d
