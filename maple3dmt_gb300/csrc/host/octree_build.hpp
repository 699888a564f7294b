// Octree leaf builder: a p4est-free stand-in for the mesh producer that sits
// in front of the forward solve.
//
// The reference builds its octree with p8est (src/octree/octree_mesh.cpp:25-63):
// a uniform forest at min_level, non-recursive refinement passes around
// stations (:129-200), inside refine regions (:211-261) and in skin-depth
// layers (:279-493), then a 2:1 FACE balance (:507-518) and extraction of
// cell centres / levels (:523-566) and an earth/air classification
// (:656-709).  p4est is not available here, so this file restates those
// refinement rules over an explicit leaf set with p4est's integer quadrant
// coordinates (root length 2^19) and Morton leaf order (child id = x + 2y + 4z).
//
// The mesh is an INPUT of the solve path (the solver receives the leaf list);
// this builder only exists so that tests and benchmarks can make the meshes
// the reference's drivers would make.
#pragma once
#include <cstdint>
#include <vector>
#include <array>

namespace m3d {

constexpr int kMaxLevel = 19;                 // P8EST_MAXLEVEL
constexpr int32_t kRootLen = 1 << kMaxLevel;  // P8EST_ROOT_LEN

struct RefineRegion {
    double x_min, x_max, y_min, y_max, z_min, z_max;
    int level;
    double padding;
};

// Mirrors octree::RefinementParams (include/maple3dmt/octree/octree_mesh.h:37-90).
struct MeshParams {
    double x_min = -50000, x_max = 50000;
    double y_min = -50000, y_max = 50000;
    double z_min = -50000, z_max = 50000;
    int min_level = 3;
    int max_level = 8;
    double station_refine_radius = 5000.0;
    int station_refine_level = 7;
    std::vector<RefineRegion> regions;
    double sigma_bg = 0.01;
    double max_interest_depth = 0.0;
    double air_surface_thickness = 2000.0;
    double air_mid_thickness = 8000.0;
    double air_upper_thickness = 20000.0;
    double transition_padding = 0.0;
    double station_x_min = 0, station_x_max = 0;
    double station_y_min = 0, station_y_max = 0;
};

struct Quad {
    int32_t x, y, z;   // lower corner, integer coordinates in [0, kRootLen)
    int8_t level;
};

enum CellType : int { kEarth = 0, kAir = 1, kOcean = 2 };

struct OctreeLeaves {
    MeshParams params;
    std::vector<Quad> quads;         // Morton order
    std::vector<double> cx, cy, cz;  // cell centres (octree_mesh.cpp:549-557)
    std::vector<int> level;
    std::vector<int> type;           // CellType
};

// Build the leaf set for the given parameters, stations (x,y,z) and frequencies.
// Flat terrain at z = 0 (the configs here are flat-earth).
OctreeLeaves build_octree(const MeshParams& p,
                          const std::vector<std::array<double, 3>>& stations,
                          const std::vector<double>& freqs);

// True if every pair of face-adjacent leaves differs by at most one level.
bool octree_is_face_balanced(const OctreeLeaves& t);

}  // namespace m3d
