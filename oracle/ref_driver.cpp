// ref_driver.cpp -- C entry points over the reference's own compiled sources.
//
// TEST INFRASTRUCTURE ONLY.  oracle/Makefile compiles this file together with
// the reference's unmodified src/*.cpp (read in place, never copied) into
// oracle/_ref/libpcd_ref.so.  It exists to pin the CPU restatement in
// pcd_oracle.c and to generate the golden fixtures under tests/golden/.
//
// The design entry points replay main.cpp:216-269 without the PNG loader:
// the caller passes the already-resized gray grid.
#include <vector>
#include <string>
#include <cstring>
#include <cmath>

#include "solver.h"
#include "utils.h"
#include "mesh.h"
#include "caustic_design.h"

// Defined with external linkage in caustic_design.cpp:156 but not declared in
// any header.
double bilinearInterpolation(const std::vector<std::vector<double>> &image, double x, double y);

namespace {
std::vector<std::vector<double>> to_grid(const double *p, int w, int h)
{
    std::vector<std::vector<double>> g(h, std::vector<double>(w));
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) g[y][x] = p[(long)y * w + x];
    return g;
}
void from_grid(const std::vector<std::vector<double>> &g, double *p)
{
    long k = 0;
    for (auto &row : g)
        for (double v : row) p[k++] = v;
}
}  // namespace

extern "C" {

// poisson_solver, solver.cpp:70 (in place on phi).
void ref_poisson_solver(const double *b, double *phi, int w, int h, int max_iter, double tol, int threads)
{
    auto B = to_grid(b, w, h);
    auto P = to_grid(phi, w, h);
    poisson_solver(B, P, w, h, max_iter, tol, threads);
    from_grid(P, phi);
}

void ref_subtract_average(double *g, int w, int h)
{
    auto G = to_grid(g, w, h);
    subtractAverage(G);
    from_grid(G, g);
}

void ref_gradient(const double *g, int w, int h, double *gx, double *gy)
{
    auto G = calculate_gradient(to_grid(g, w, h));
    from_grid(G[0], gx);
    from_grid(G[1], gy);
}

void ref_divergence(const double *nx, const double *ny, int w, int h, double *div)
{
    auto D = calculate_divergence(to_grid(nx, w, h), to_grid(ny, w, h), w, h);
    from_grid(D, div);
}

double ref_bilinear(const double *g, int w, int h, double x, double y)
{
    return bilinearInterpolation(to_grid(g, w, h), x, y);
}

void ref_scale_proportional(const double *g, int w, int h, double lo, double hi, double *out)
{
    from_grid(scale_matrix_proportional(to_grid(g, w, h), lo, hi), out);
}

// ---- Caustic_design replay (main.cpp:224-262) ----
void *ref_design_create(int mesh_res_x, int mesh_res_y, int res_x, int res_y, double width,
                        double height, double focal_l, double thickness, int threads)
{
    auto *d = new Caustic_design();
    d->set_mesh_resolution(mesh_res_x, mesh_res_y);
    d->set_domain_resolution(res_x, res_y);
    d->set_mesh_size(width, height);
    d->set_lens_focal_length(focal_l);
    d->set_lens_thickness(thickness);
    d->set_solver_max_threads(threads);
    return d;
}

void ref_design_initialize(void *h, const double *image)
{
    auto *d = static_cast<Caustic_design *>(h);
    d->initialize_solvers(to_grid(image, d->resolution_x, d->resolution_y));
}

double ref_design_transport(void *h) { return static_cast<Caustic_design *>(h)->perform_transport_iteration(); }

void ref_design_height(void *h, int itr) { static_cast<Caustic_design *>(h)->perform_height_map_iteration(itr); }

// which: 0 phi, 1 h, 2 raster, 3 divergence, 4 norm_x, 5 norm_y (grids);
// 10 target_points, 11 source_points (n x 3); 12 target_areas, 13 errors,
// 14 normals x, 15 normals y, 16 vertex_gradient x, 17 vertex_gradient y.
int ref_design_get(void *h, int which, double *out)
{
    auto *d = static_cast<Caustic_design *>(h);
    switch (which) {
    case 0: from_grid(d->phi, out); return 0;
    case 1: from_grid(d->h, out); return 0;
    case 2: from_grid(d->raster, out); return 0;
    case 3: from_grid(d->divergence, out); return 0;
    case 4: from_grid(d->norm_x, out); return 0;
    case 5: from_grid(d->norm_y, out); return 0;
    case 10: from_grid(d->mesh->target_points, out); return 0;
    case 11: from_grid(d->mesh->source_points, out); return 0;
    case 12: std::memcpy(out, d->target_areas.data(), d->target_areas.size() * sizeof(double)); return 0;
    case 13: std::memcpy(out, d->errors.data(), d->errors.size() * sizeof(double)); return 0;
    case 14: std::memcpy(out, d->normals[0].data(), d->normals[0].size() * sizeof(double)); return 0;
    case 15: std::memcpy(out, d->normals[1].data(), d->normals[1].size() * sizeof(double)); return 0;
    case 16: std::memcpy(out, d->vertex_gradient[0].data(), d->vertex_gradient[0].size() * sizeof(double)); return 0;
    case 17: std::memcpy(out, d->vertex_gradient[1].data(), d->vertex_gradient[1].size() * sizeof(double)); return 0;
    }
    return -1;
}

// save_solid_obj, utils.cpp:198-260, on the structured mesh's triangles
// (generate_structured_mesh, mesh.cpp:45-64: two per quad, {i, i+1, i+nx} and
// {i+nx, i+1, i+nx+1}); front / back are nx*ny x 3 points.
void ref_save_solid_obj(const double *front, const double *back, int nx, int ny, double thickness, double width,
                        double height, const char *filename)
{
    std::vector<std::vector<double>> F, B;
    for (int i = 0; i < nx * ny; i++) {
        F.push_back({front[3 * i], front[3 * i + 1], front[3 * i + 2]});
        B.push_back({back[3 * i], back[3 * i + 1], back[3 * i + 2]});
    }
    std::vector<std::vector<int>> tri;
    for (int y = 0; y < ny - 1; y++)
        for (int x = 0; x < nx - 1; x++) {
            const int i = y * nx + x;
            tri.push_back({i, i + 1, i + nx});
            tri.push_back({i + nx, i + 1, i + nx + 1});
        }
    save_solid_obj(F, B, tri, thickness, width, height, nx, ny, std::string(filename));
}

// export_grid_to_svg, utils.cpp:262-307; points are nx*ny x 3.
void ref_export_grid_svg(const double *pts, int nx, int ny, double width, double height, const char *filename,
                         double stroke_width)
{
    std::vector<std::vector<double>> P;
    for (int i = 0; i < nx * ny; i++) P.push_back({pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]});
    export_grid_to_svg(P, width, height, nx, ny, std::string(filename), stroke_width);
}

// Mesh::laplacian_smoothing, mesh.cpp:534-606 (public member), in place on
// an nx*ny x 3 point set.
void ref_laplacian_smoothing(double *pts, int nx, int ny, double width, double height, double factor)
{
    Mesh m(width, height, nx, ny);
    std::vector<point_t> P;
    for (int i = 0; i < nx * ny; i++) P.push_back({pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]});
    m.laplacian_smoothing(P, factor);
    for (int i = 0; i < nx * ny; i++)
        for (int c = 0; c < 3; c++) pts[3 * i + c] = P[i][c];
}

void ref_design_destroy(void *h)
{
    auto *d = static_cast<Caustic_design *>(h);
    delete d->mesh;
    delete d;
}

}  // extern "C"
