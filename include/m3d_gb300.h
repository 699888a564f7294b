/* m3d_gb300.h -- C ABI of the GB300 forward + adjoint octree-FV EM solver.
 *
 * This is the drop-in boundary under the reference's forward-solver interface
 * maple3dmt::forward::IForwardSolver (include/maple3dmt/forward/iforward_solver.h:31-115)
 * and its octree implementation ForwardSolverFV
 * (include/maple3dmt/forward/forward_solver_fv.h:77-253).  Every entry point
 * below names the reference member it replaces.
 *
 * Conventions
 *  - Plain host pointers and sizes only; all buffers are caller-owned host
 *    memory; complex vectors are interleaved (re, im) doubles.
 *  - Edge vectors use the reference's edge numbering (StaggeredGrid edge ids,
 *    src/octree/staggered_grid.cpp:82-121); cell vectors the leaf order.
 *  - Every function returns M3D_OK (0) or one M3D_ERR_* code and synchronises
 *    the device before returning; m3d_last_error() gives the message.
 *  - A solver handle is single-threaded, like the reference (not re-entrant).
 */
#ifndef M3D_GB300_H
#define M3D_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define M3D_OK 0
#define M3D_ERR_ARG 1         /* null pointer, bad size or value out of range */
#define M3D_ERR_STATE 2       /* call out of order (e.g. adjoint before forward) */
#define M3D_ERR_CUDA 3        /* CUDA runtime error */
#define M3D_ERR_OOM 4         /* host or device allocation failed */
#define M3D_ERR_NO_DEVICE 5   /* no usable CUDA device */
#define M3D_ERR_TOO_LARGE 6   /* size beyond a fixed limit of the entry point */
#define M3D_ERR_NUMERIC 7     /* non-finite values met in a solve */

#ifdef __cplusplus
}
#endif

#endif /* M3D_GB300_H */
