// pcd_legacy.hpp -- the reference's C++ signatures over libpcd_gb300's C ABI.
//
// Header-only.  A program written against dylanmsu/poisson_caustic_design's
// src/solver.h and src/caustic_design.h compiles against this header instead
// and links libpcd_gb300.so; the solve and the per-iteration mesh/grid steps
// then run on the GPU.
//
//   poisson_solver(...)      src/solver.h:8        (solver.cpp:70-148)
//   solver_progress          src/solver.h:10       (never updated, as in the reference)
//   class Caustic_design     src/caustic_design.h:7-66
//   struct Mesh (members read by callers: target_points, source_points,
//                width, height, res_x, res_y)   src/mesh.h:51-58
//
// Differences a caller can observe (all stated in the header of pcd.h):
//   * max_threads / set_solver_max_threads are accepted and ignored;
//   * a raster miss throws std::runtime_error instead of calling exit(0)
//     (mesh.cpp:277-279);
//   * the public members are host copies refreshed after every
//     initialize_solvers / perform_*_iteration call.
#ifndef PCD_LEGACY_HPP
#define PCD_LEGACY_HPP

#include <stdexcept>
#include <string>
#include <vector>

#include "pcd.h"

inline double solver_progress = 0.0;

inline void poisson_solver(std::vector<std::vector<double>> &input, std::vector<std::vector<double>> &output,
                           int width, int height, int max_iterations, double convergence_threshold,
                           int max_threads)
{
    std::vector<double> b((size_t)width * height), phi((size_t)width * height);
    for (int y = 0; y < height; y++)
        for (int x = 0; x < width; x++) {
            b[(size_t)y * width + x] = input[y][x];
            phi[(size_t)y * width + x] = output[y][x];
        }
    int st = pcd_poisson_solver(b.data(), phi.data(), width, height, max_iterations, convergence_threshold,
                                max_threads);
    if (st != PCD_OK && st != PCD_NOT_CONVERGED)
        throw std::runtime_error(std::string("pcd_poisson_solver: ") + pcd_last_error());
    for (int y = 0; y < height; y++)
        for (int x = 0; x < width; x++) output[y][x] = phi[(size_t)y * width + x];
}

namespace pcd_legacy {

inline void check(int st, const char *where)
{
    if (st != PCD_OK && st != PCD_NOT_CONVERGED)
        throw std::runtime_error(std::string(where) + ": " + pcd_status_string(st) + ": " + pcd_last_error());
}

inline std::vector<std::vector<double>> to_rows(const std::vector<double> &flat, int w, int h)
{
    std::vector<std::vector<double>> g(h, std::vector<double>(w));
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) g[y][x] = flat[(size_t)y * w + x];
    return g;
}

}  // namespace pcd_legacy

// Host view of the mesh state (mesh.h:51-58).
struct Mesh {
    std::vector<std::vector<double>> source_points;
    std::vector<std::vector<double>> target_points;
    double width = 0.0, height = 0.0;
    int res_x = 0, res_y = 0;
};

class Caustic_design {
   public:
    Caustic_design() { pcd_legacy::check(pcd_ctx_create(-1, &ctx_), "pcd_ctx_create"); }
    ~Caustic_design()
    {
        if (d_) pcd_design_destroy(d_);
        if (ctx_) pcd_ctx_destroy(ctx_);
        delete mesh;
    }
    Caustic_design(const Caustic_design &) = delete;
    Caustic_design &operator=(const Caustic_design &) = delete;

    Mesh *mesh = nullptr;
    std::vector<std::vector<double>> phi;
    std::vector<double> errors;
    std::vector<double> target_areas;
    std::vector<std::vector<double>> raster;
    std::vector<std::vector<double>> h;
    std::vector<std::vector<double>> divergence;
    std::vector<std::vector<double>> norm_x;
    std::vector<std::vector<double>> norm_y;
    std::vector<std::vector<double>> vertex_gradient;
    std::vector<std::vector<double>> normals;

    int mesh_res_x = 0, mesh_res_y = 0;
    int resolution_x = 0, resolution_y = 0;
    double width = 0.0, height = 0.0;
    double focal_l = 0.0, thickness = 0.0;
    int nthreads = 0;

    void set_mesh_resolution(int w, int hgt) { mesh_res_x = w; mesh_res_y = hgt; }
    void set_domain_resolution(int w, int hgt) { resolution_x = w; resolution_y = hgt; }
    void set_mesh_size(double w, double hgt) { width = w; height = hgt; }
    void set_lens_focal_length(double f) { focal_l = f; }
    void set_lens_thickness(double t) { thickness = t; }
    void set_solver_max_threads(int n) { nthreads = n; }

    void initialize_solvers(std::vector<std::vector<double>> image)
    {
        if (d_) { pcd_design_destroy(d_); d_ = nullptr; }
        pcd_design_params p;
        pcd_design_params_default(&p);
        p.mesh_res_x = mesh_res_x; p.mesh_res_y = mesh_res_y;
        p.res_x = resolution_x; p.res_y = resolution_y;
        p.width = width; p.height = height;
        p.focal_l = focal_l; p.thickness = thickness;
        pcd_legacy::check(pcd_design_create(ctx_, &p, &d_), "pcd_design_create");
        std::vector<double> img((size_t)resolution_x * resolution_y);
        for (int y = 0; y < resolution_y; y++)
            for (int x = 0; x < resolution_x; x++) img[(size_t)y * resolution_x + x] = image[y][x];
        pcd_legacy::check(pcd_design_initialize(d_, img.data()), "pcd_design_initialize");
        delete mesh;
        mesh = new Mesh();
        mesh->width = width; mesh->height = height;
        mesh->res_x = mesh_res_x; mesh->res_y = mesh_res_y;
        refresh();
    }

    double perform_transport_iteration()
    {
        double step = 0.0;
        pcd_legacy::check(pcd_design_transport_iteration(d_, &step, nullptr), "perform_transport_iteration");
        refresh();
        return step;
    }

    void perform_height_map_iteration(int itr)
    {
        double upd = 0.0;
        pcd_legacy::check(pcd_design_height_iteration(d_, itr, &upd, nullptr), "perform_height_map_iteration");
        refresh();
    }

    // output files (caustic_design.cpp:20-26,55-61)
    void save_solid_obj_target(const std::string &filename)
    {
        pcd_legacy::check(pcd_design_save_solid_obj(d_, 1, filename.c_str()), "save_solid_obj_target");
    }
    void save_solid_obj_source(const std::string &filename)
    {
        pcd_legacy::check(pcd_design_save_solid_obj(d_, 0, filename.c_str()), "save_solid_obj_source");
    }
    void export_paramererization_to_svg(const std::string &filename, double line_width)
    {
        pcd_legacy::check(pcd_design_export_parameterization_svg(d_, filename.c_str(), line_width),
                          "export_paramererization_to_svg");
    }
    void export_inverted_transport_map(std::string filename, double stroke_width)
    {
        pcd_legacy::check(pcd_design_export_inverted_transport_map_svg(d_, filename.c_str(), stroke_width),
                          "export_inverted_transport_map");
    }

   private:
    pcd_ctx *ctx_ = nullptr;
    pcd_design *d_ = nullptr;

    std::vector<std::vector<double>> grid(int which)
    {
        std::vector<double> flat((size_t)resolution_x * resolution_y);
        pcd_legacy::check(pcd_design_get_grid(d_, which, flat.data()), "pcd_design_get_grid");
        return pcd_legacy::to_rows(flat, resolution_x, resolution_y);
    }

    std::vector<double> verts(int which)
    {
        std::vector<double> v((size_t)mesh_res_x * mesh_res_y);
        pcd_legacy::check(pcd_design_get_vertices(d_, which, v.data()), "pcd_design_get_vertices");
        return v;
    }

    std::vector<std::vector<double>> points(int which)
    {
        std::vector<double> flat((size_t)mesh_res_x * mesh_res_y * 3);
        pcd_legacy::check(pcd_design_get_vertices(d_, which, flat.data()), "pcd_design_get_vertices");
        return pcd_legacy::to_rows(flat, 3, mesh_res_x * mesh_res_y);
    }

    void refresh()
    {
        phi = grid(PCD_GRID_PHI);
        h = grid(PCD_GRID_H);
        raster = grid(PCD_GRID_RASTER);
        divergence = grid(PCD_GRID_DIVERGENCE);
        norm_x = grid(PCD_GRID_NORM_X);
        norm_y = grid(PCD_GRID_NORM_Y);
        errors = verts(PCD_VERT_ERRORS);
        target_areas = verts(PCD_VERT_TARGET_AREAS);
        vertex_gradient = {verts(PCD_VERT_GRADIENT_X), verts(PCD_VERT_GRADIENT_Y)};
        normals = {verts(PCD_VERT_NORMALS_X), verts(PCD_VERT_NORMALS_Y)};
        mesh->target_points = points(PCD_VERT_TARGET_POINTS);
        mesh->source_points = points(PCD_VERT_SOURCE_POINTS);
    }
};

// main.cpp:29-109 (the PNG loader; see pcd_image_to_grid)
inline void image_to_grid(const std::string &filename, std::vector<std::vector<double>> &image_grid)
{
    int w = 0, h = 0;
    if (pcd_image_to_grid(filename.c_str(), &w, &h, nullptr) != PCD_OK)
        throw std::runtime_error("Failed to open PNG file.");
    std::vector<double> flat((size_t)w * h);
    if (pcd_image_to_grid(filename.c_str(), &w, &h, flat.data()) != PCD_OK)
        throw std::runtime_error("Error during PNG read.");
    image_grid = pcd_legacy::to_rows(flat, w, h);
}

// main.cpp:13-27
inline void resize_image(const std::vector<std::vector<double>> &input_image,
                         std::vector<std::vector<double>> &output_image, int new_width, int new_height)
{
    const int oh = (int)input_image.size(), ow = oh ? (int)input_image[0].size() : 0;
    std::vector<double> in((size_t)ow * oh), out((size_t)new_width * new_height);
    for (int y = 0; y < oh; y++)
        for (int x = 0; x < ow; x++) in[(size_t)y * ow + x] = input_image[y][x];
    pcd_legacy::check(pcd_resize_image(in.data(), ow, oh, out.data(), new_width, new_height), "resize_image");
    output_image = pcd_legacy::to_rows(out, new_width, new_height);
}

// main.cpp:111-135
inline void save_heightmap_as_json(const std::vector<std::vector<double>> &heightmap, const std::string &filename)
{
    const int h = (int)heightmap.size(), w = h ? (int)heightmap[0].size() : 0;
    std::vector<double> flat((size_t)w * h);
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) flat[(size_t)y * w + x] = heightmap[y][x];
    if (pcd_write_heightmap_json(flat.data(), w, h, filename.c_str()) != PCD_OK)
        throw std::runtime_error("Failed to open output file.");
}

#endif  // PCD_LEGACY_HPP
