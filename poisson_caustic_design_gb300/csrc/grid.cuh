// grid.cuh -- per-cell grid kernels (internal).
#pragma once

#include "common.cuh"

namespace pcd {

// Reduction scratch of the grid kernels (mean and count at buf[0..1], per-block
// partials after them).
struct GridScratch {
    double *buf = nullptr;
    unsigned int *counter = nullptr;
    int reserve();
    void release();
};

int subtract_average(GridScratch &sc, double *g, long n, cudaStream_t s);
int gradient(const double *g, double *gx, double *gy, int W, int H, cudaStream_t s);
int divergence(const double *nx, const double *ny, double *div, int W, int H, cudaStream_t s);
int resize_nearest(const double *in, int ow, int oh, int ild, double *out, int nw, int nh, int old, cudaStream_t s);

}  // namespace pcd
