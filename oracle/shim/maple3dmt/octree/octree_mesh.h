// Shim for the reference's octree mesh header, used ONLY to compile the
// reference's own forward-solver sources as a test oracle (oracle/_ref).
//
// The reference's OctreeMesh (include/maple3dmt/octree/octree_mesh.h:105-216)
// wraps p8est, which is not installed here.  The solve path only reads a
// finished leaf set through num_cells_local / cell_center / cell_size /
// cell_size_xyz / cell_level / cell_type / params / staggered, so this shim
// keeps that public surface and is filled from an explicit leaf list (levels
// and centres) produced elsewhere.  The accessor arithmetic follows
// src/octree/octree_mesh.cpp:571-594.
#pragma once

#include "maple3dmt/common.h"

#ifdef MAPLE3DMT_USE_OCTREE

#include <functional>
#include <array>

namespace maple3dmt {

namespace data { struct Station; }

namespace octree {

class StaggeredGrid;

struct RefineRegion {
    Real x_min, x_max, y_min, y_max, z_min, z_max;
    int level;
    Real padding;
};

struct RefinementParams {
    Real domain_x_min, domain_x_max;
    Real domain_y_min, domain_y_max;
    Real domain_z_min, domain_z_max;
    int  min_level = 3;
    int  max_level = 8;
    Real h_min     = 50.0;
    Real h_max     = 10000.0;
    Real station_refine_radius = 5000.0;
    int  station_refine_level  = 7;
    std::vector<RefineRegion> refine_regions;
    int  terrain_refine_level  = 6;
    int  skin_depth_levels     = 2;
    Real sigma_bg              = 0.01;
    Real max_interest_depth    = 0.0;
    Real air_surface_thickness = 2000.0;
    Real air_mid_thickness     = 8000.0;
    Real air_upper_thickness   = 20000.0;
    Real transition_padding    = 0.0;
    Real station_x_min = 0, station_x_max = 0;
    Real station_y_min = 0, station_y_max = 0;
    bool replicate_mesh        = false;
};

enum class CellType : int { EARTH = 0, AIR = 1, OCEAN = 2 };

class OctreeMesh {
public:
    OctreeMesh();
    ~OctreeMesh();
    OctreeMesh(const OctreeMesh&) = delete;
    OctreeMesh& operator=(const OctreeMesh&) = delete;

    /// Fill from a finished leaf list (replaces setup + set_terrain).
    void load_leaves(const RefinementParams& params, int n_cells,
                     const int* level, const Real* cx, const Real* cy,
                     const Real* cz, const int* cell_type);

    int num_cells_local() const { return num_cells_; }
    int num_cells_global() const { return num_cells_; }

    void cell_center(int local_id, Real& x, Real& y, Real& z) const {
        x = cx_[local_id]; y = cy_[local_id]; z = cz_[local_id];
    }
    Real cell_size(int local_id) const;
    void cell_size_xyz(int local_id, Real& dx, Real& dy, Real& dz) const;
    int  cell_level(int local_id) const { return level_[local_id]; }
    CellType cell_type(int local_id) const { return type_[local_id]; }

    const StaggeredGrid& staggered() const { return *staggered_; }
    StaggeredGrid& staggered() { return *staggered_; }
    void build_staggered_grid();

    const RefinementParams& params() const { return params_; }

private:
    RefinementParams params_;
    int num_cells_ = 0;
    std::vector<Real> cx_, cy_, cz_;
    std::vector<int> level_;
    std::vector<CellType> type_;
    std::unique_ptr<StaggeredGrid> staggered_;
};

}  // namespace octree
}  // namespace maple3dmt

#endif  // MAPLE3DMT_USE_OCTREE
