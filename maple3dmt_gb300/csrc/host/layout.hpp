// Host layout producer: from the octree leaf list to the edge system the GPU
// solves.  Runs once per mesh.
//
// It restates, with hash tables instead of std::map and in the same edge /
// face / node numbering and floating-point operation order, the reference's
//   StaggeredGrid::build          src/octree/staggered_grid.cpp:70-409
//   DiscreteOperators::build      src/octree/operators.cpp:19-170, 176-466, 849-944
//   stiffness pattern and values  src/octree/operators.cpp:556-622, 624-836
// so that the GPU starts from the reference's system bit for bit.  The key
// structural fact used downstream: S = Ce^T diag(Mf^-1) Ce depends only on
// the geometry, so A(sigma, omega) = S + i*omega*diag(Me(sigma)) differs
// between frequencies and models only on its diagonal.
#pragma once
#include <array>
#include <cstdint>
#include <vector>

namespace m3d {

struct LeafInput {
    double domain[6];
    int min_level, max_level;
    int nc;
    const int* level;
    const double *cx, *cy, *cz;
    const int* type;
};

struct HostLayout {
    int ne = 0, nf = 0, nc = 0, nn = 0;
    double domain[6];
    int min_level = 0, max_level = 0;
    // cells (leaf order)
    std::vector<double> ccx, ccy, ccz;   // geometric centres from the leaves
    std::vector<int> clevel, ctype;
    double cell_size0 = 0;               // OctreeMesh::cell_size(0)
    // edges (reference numbering)
    std::vector<double> ex, ey, ez, elen;
    std::vector<int> edir;
    std::vector<int> adj_ptr, adj;       // edge -> adjacent cells (after hanging fix-up)
    std::vector<double> adual;           // edge dual area
    std::vector<char> dead;              // dead (coarse hanging) edges
    std::vector<std::array<int, 3>> hp;  // hanging pairs: coarse, child1, child2
    // faces
    std::vector<double> farea, fdual;
    std::vector<int> fnorm, fcm, fcp;    // normal direction, minus / plus cell (after the hanging fix-up)
    std::vector<char> dead_f;
    // curl after hanging-face handling: faces x edges
    std::vector<int> ce_ptr, ce_idx;
    std::vector<double> ce_val;
    // S = Ce^T Mf^-1 Ce on the reference pattern (diagonal always present)
    std::vector<int> s_ptr, s_idx;
    std::vector<double> s_val;
    // node gradient: edge -> (minus node, plus node)
    std::vector<int> n1, n2;
    // cell -> edges (StaggeredGrid::cell_edges order)
    std::vector<int> cell_ptr, cell_edge;
};

// Throws std::runtime_error on malformed input.
void build_layout(const LeafInput& in, HostLayout& L);

}  // namespace m3d
