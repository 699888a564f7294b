/* Octree leaf builder: C ABI of the p4est stand-in that produces the mesh the
 * forward solve consumes.
 *
 * Replaces, for this image where p4est is absent, the mesh construction the
 * reference performs in octree::OctreeMesh::setup + set_terrain
 * (include/maple3dmt/octree/octree_mesh.h:115-121; src/octree/octree_mesh.cpp:25-78).
 * It is not part of the solve path: the solver takes the leaf list as input
 * (m3d_solver_setup in m3d_gb300.h).
 *
 * All functions return 0 on success and a nonzero M3D_ERR_* code otherwise.
 */
#ifndef M3D_MESH_H
#define M3D_MESH_H

#ifdef __cplusplus
extern "C" {
#endif

/* Mirrors octree::RefinementParams (include/maple3dmt/octree/octree_mesh.h:37-90). */
typedef struct m3d_mesh_params {
    double domain[6];              /* x_min x_max y_min y_max z_min z_max (m) */
    int min_level;
    int max_level;
    double station_refine_radius;  /* m */
    int station_refine_level;
    double sigma_bg;               /* S/m, sets the skin-depth layers */
    double max_interest_depth;     /* m, 0 = 3 skin depths */
    double air_surface_thickness;  /* m */
    double air_mid_thickness;
    double air_upper_thickness;
    double transition_padding;
    double station_bbox[4];        /* x_min x_max y_min y_max of the station array */
    int n_regions;
    const double* regions;         /* [n_regions][8]: x0 x1 y0 y1 z0 z1 level padding */
} m3d_mesh_params;

typedef struct m3d_octree m3d_octree;

/* Build the leaf set: uniform min_level forest, station / region / skin-depth
 * refinement passes, 2:1 face balance, Morton order, flat-terrain earth/air
 * classification. stations: [n_stations][3] (x, y, z) in m. */
int m3d_octree_build(const m3d_mesh_params* params, const double* stations, int n_stations,
                     const double* freqs, int n_freqs, m3d_octree** out);

int m3d_octree_num_cells(const m3d_octree* t);

/* Copy out the leaf list. Any pointer may be NULL. qxyz: [n_cells][3] integer
 * lower corners at root length 2^19. cell_type: 0 earth, 1 air. */
int m3d_octree_get(const m3d_octree* t, int* level, int* qxyz, double* cx, double* cy,
                   double* cz, int* cell_type);

/* 1 if every pair of face-adjacent leaves differs by at most one level. */
int m3d_octree_is_balanced(const m3d_octree* t);

void m3d_octree_destroy(m3d_octree* t);

#ifdef __cplusplus
}
#endif

#endif /* M3D_MESH_H */
