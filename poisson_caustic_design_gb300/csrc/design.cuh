// design.cuh -- device state of one Caustic_design instance (internal).
//
// Mirrors the members of class Caustic_design (caustic_design.h:16-43) and
// Mesh (mesh.h:51-58) that the iterations touch, resident in device memory:
// target points as double2 (x, y; the target z stays 0), source heights z
// (the source x, y never move), per-vertex fields, and res_x x res_y grids.
#pragma once

#include "common.cuh"

struct pcd_ctx;

namespace pcd {

struct Design {
    pcd_ctx *ctx = nullptr;
    pcd_design_params p{};
    bool initialized = false;

    // per vertex (mesh_res_x * mesh_res_y)
    double2 *tp = nullptr;       // target points (x, y)
    double2 *src_xy = nullptr;   // source points (x, y), the undeformed grid
    double2 *inv = nullptr;      // inverted transport map
    double2 *tp_cells = nullptr; // target points the last dual cells were built from
    double *sz = nullptr;        // source heights
    double *target_areas = nullptr, *areas = nullptr, *errors = nullptr;
    double *vgx = nullptr, *vgy = nullptr;      // vertex gradients
    double *nrm_x = nullptr, *nrm_y = nullptr;  // refractive slopes
    double *hv = nullptr;                       // sampled heights
    double *pts_out = nullptr;                  // n x 3 staging for the getters
    // per grid cell (res_x * res_y)
    double *pixels = nullptr, *raster = nullptr, *phi = nullptr, *h = nullptr;
    double *norm_x = nullptr, *norm_y = nullptr, *div = nullptr;
    unsigned int *owner = nullptr;  // point-location owner per query
    double *qc = nullptr;           // query coordinates: raster sample x, y; shrunk source vertex x, y
    double *grad = nullptr;         // 2 grids: the gradient of phi, allocated on the first request
    // reductions
    double *scratch = nullptr;
    unsigned int *counter = nullptr;
    unsigned long long *small = nullptr;
    unsigned long long *small_host = nullptr;

    int alloc();
    void release();
    int initialize(const double *image_host);
    int transport_iteration(double *step_out, pcd_solve_stats *stats);
    int height_iteration(int itr, double *update_out, pcd_solve_stats *stats);
    // The iterations in two halves around their Poisson solve (raster into
    // phi; div into h), for batches that solve many designs' grids at once.
    int transport_pre(double *step_out);
    int transport_post(double *step_out);
    int height_pre();
    int height_post(double *update_out);
    int get_grid(int which, double *out);
    int get_vertices(int which, double *out);
    int smooth_target(double f);
    int count_folds(long long *folds);
    int set_target_points(const double *pts3);

   private:
    int locate(const double2 *pts, int mode, int qx, int qy, cudaStream_t s);
    int raster_values(const double2 *pts, const double *va, const double *vb, double *oa, double *ob,
                      cudaStream_t s, unsigned int *misses_host);
};

}  // namespace pcd

struct pcd_design {
    pcd::Design d;
};

namespace pcd {
// Releases the device state of every design of ctx and detaches them; their
// handles stay valid until pcd_design_destroy, and every other call on them
// returns PCD_BAD_ARG.
void design_detach_all(pcd_ctx *ctx);
}  // namespace pcd
