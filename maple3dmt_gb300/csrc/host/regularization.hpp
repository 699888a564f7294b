// Octree model regularisation, host setup: RegularizationOctree::setup
// (src/inversion/regularization_octree.cpp:24-172) on the solver's layout.
// Active cells are the earth cells; each face between two active cells adds
// w = alpha_dir * area / (dist * (V_minus V_plus)^(1/6)) to W^T W (diagonal
// +w, off-diagonal -w, summed in face order) and to the neighbour lists of
// the CmCm^T diffusion; everything is scaled to a unit average diagonal.
// The operators run on the GPU (cuda/regularization.cu).
#pragma once

#include <vector>

#include "host/layout.hpp"

namespace m3d {

struct RegParams {
    double alpha_s = 1.0, alpha_x = 1.0, alpha_y = 1.0, alpha_z = 1.0;
    int n_smooth = 2;
};

struct RegHost {
    int nc = 0, na = 0;
    std::vector<int> a2g, g2a;
    std::vector<int> ptr, idx;      // W^T W, columns sorted
    std::vector<double> val;
    std::vector<int> aptr, aidx;    // neighbours of each active cell, face order
    std::vector<double> aw;
    std::vector<double> diagw;
    RegParams p;
};

void reg_build(const HostLayout& L, const RegParams& p, RegHost& R);

}  // namespace m3d
