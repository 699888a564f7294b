// Batched Hermitian inner products of K interleaved complex-FP64 vectors,
//   out[k] = sum_i conj(x[i][k]) * y[i][k],   x, y laid out [n][K],
// the reduction of BiCGStabSolver::dot (include/maple3dmt/forward/bicgstab.h:68-73)
// for K systems in one HBM pass.  The grid is a pure function of (n, K, cap),
// so results are bit-reproducible for a fixed cap.
#pragma once

#include <cuda_runtime.h>

#include "common.cuh"

namespace m3d {
namespace dev {

constexpr int kDotMaxBlocks = 1024;   // largest grid of the dot kernel

// Blocks of the dot launch: one thread per (row, rhs) pair up to `cap` blocks
// (grid-stride beyond), at least one block so that n == 0 writes zeros.
int dot_blocks(long long n, int K, int cap);

// Enqueues the batched dot on `st`.  `rs.partial` holds >= dot_blocks(...) * K
// entries, `rs.final_` >= K, `*rs.counter` is zero on entry and zero again
// when the kernel ends.  K in {1, 2, 4, 8, 16}; `out` is a device pointer to K
// complex values.
cudaError_t launch_dot_batched(const double2* x, const double2* y, long long n, int K, int cap, RedScratch rs,
                               double2* out, cudaStream_t st);

}  // namespace dev
}  // namespace m3d
