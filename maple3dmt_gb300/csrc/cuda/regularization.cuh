// Octree model regularisation on the GPU: the operators of
// RegularizationOctree (src/inversion/regularization_octree.cpp:177-286) over
// the host-built W^T W and neighbour lists (host/regularization.hpp).
// Products and sums are rounded one operation at a time (no fused
// multiply-add), in the reference's order, so W^T W x, diag(W^T W), CmCm^T x
// and the gradient equal the reference's bit for bit; the objective's dot
// product is a deterministic block reduction.
#pragma once

#include <cuda_runtime.h>

namespace m3d {

struct RegDev {
    int nc = 0, na = 0, n_smooth = 2;
    double alpha_s = 1.0;
    const int *a2g = nullptr, *ptr = nullptr, *idx = nullptr, *aptr = nullptr, *aidx = nullptr;
    const double *val = nullptr, *aw = nullptr, *diagw = nullptr;
    double *t0 = nullptr, *t1 = nullptr, *t2 = nullptr;   // [na] scratch
    double* dot = nullptr;                                // [1]
};

// y = W^T W x (apply_WtW, :229-231); x, y device [na]
void reg_apply_wtw(const RegDev& r, const double* x, double* y, cudaStream_t s);
// diag(W^T W) (diagonal_WtW, :236-246)
void reg_diagonal(const RegDev& r, double* d, cudaStream_t s);
// y = CmCm^T x, 2 n_smooth diffusion passes (apply_CmCmT, :251-281)
void reg_apply_cmcmt(const RegDev& r, const double* x, double* y, cudaStream_t s);
// alpha_s dm^T W^T W dm into r.dot (evaluate, :183-201) and, when grad is not
// null, the gradient 2 alpha_s W^T W dm on the active cells of grad [nc]
// (gradient, :206-224); dm = params[a2g] - ref (ref null: 0)
void reg_evaluate(const RegDev& r, const double* params, const double* ref, double* grad, cudaStream_t s);

}  // namespace m3d
