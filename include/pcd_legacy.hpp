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
// The state lives on the GPU.  The public members keep the reference's names
// and types (each converts implicitly to it, and indexing, size() and range
// for work on it directly): a member's host copy is fetched from the device on
// its first use after initialize_solvers / perform_*_iteration, so an
// iteration call copies nothing back and a caller pays only for what it reads.
//
// Differences a caller can observe (all stated in the header of pcd.h):
//   * max_threads / set_solver_max_threads are accepted and ignored;
//   * a raster miss throws std::runtime_error instead of calling exit(0)
//     (mesh.cpp:277-279);
//   * a host copy a caller changes is not written back to the device (the
//     next iteration replaces it with the device's state);
//   * target_cells lists each vertex's quads in the library's fixed triangle
//     order (the reference walks an unordered_set); first_target_cells stays
//     empty, as in the reference, which never fills it.
#ifndef PCD_LEGACY_HPP
#define PCD_LEGACY_HPP

#include <functional>
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

typedef std::vector<double> point_t;      // mesh.h:17
typedef std::vector<point_t> polygon_t;   // mesh.h:18

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

// A public member backed by device state: the host copy is fetched on the
// first use after invalidate().  Converts to T&, and forwards indexing,
// size() and iteration, so code written for the plain member compiles.
template <typename T>
class lazy {
   public:
    using value_type = typename T::value_type;
    lazy() = default;
    explicit lazy(std::function<void(T &)> fetch) : fetch_(std::move(fetch)) {}
    lazy(const lazy &) = delete;
    lazy &operator=(const lazy &) = delete;
    lazy &operator=(const T &v)
    {
        v_ = v;
        stale_ = false;
        return *this;
    }
    T &get()
    {
        if (stale_) {
            if (fetch_) fetch_(v_);
            stale_ = false;
        }
        return v_;
    }
    const T &get() const { return const_cast<lazy *>(this)->get(); }
    operator T &() { return get(); }
    operator const T &() const { return get(); }
    value_type &operator[](size_t i) { return get()[i]; }
    const value_type &operator[](size_t i) const { return get()[i]; }
    size_t size() const { return get().size(); }
    bool empty() const { return get().empty(); }
    typename T::iterator begin() { return get().begin(); }
    typename T::iterator end() { return get().end(); }
    typename T::const_iterator begin() const { return get().begin(); }
    typename T::const_iterator end() const { return get().end(); }
    void invalidate() { stale_ = true; }

   private:
    std::function<void(T &)> fetch_;
    bool stale_ = true;
    T v_;
};

using grid_t = std::vector<std::vector<double>>;

// The barycentric dual cells of the structured mesh from its points
// (Mesh::build_target_partitioned_dual_cells, mesh.cpp:174-231, with
// edge_centroid / triangle_centroid of mesh.cpp:154-172), in the library's
// triangle order around each vertex.
inline std::vector<std::vector<polygon_t>> dual_cells(const std::vector<double> &p3, int nx, int ny)
{
    std::vector<std::vector<polygon_t>> cells((size_t)nx * ny);
    const int cx = nx - 1;
    auto pt = [&](int v) { return point_t{p3[3 * (size_t)v], p3[3 * (size_t)v + 1], p3[3 * (size_t)v + 2]}; };
    for (int i = 0; i < ny; i++)
        for (int j = 0; j < nx; j++) {
            int tri[6], pos[6], m = 0;
            if (i < ny - 1 && j < nx - 1) { tri[m] = 2 * (i * cx + j); pos[m++] = 0; }
            if (i < ny - 1 && j > 0) {
                tri[m] = 2 * (i * cx + j - 1); pos[m++] = 1;
                tri[m] = 2 * (i * cx + j - 1) + 1; pos[m++] = 1;
            }
            if (i > 0 && j < nx - 1) {
                tri[m] = 2 * ((i - 1) * cx + j); pos[m++] = 2;
                tri[m] = 2 * ((i - 1) * cx + j) + 1; pos[m++] = 0;
            }
            if (i > 0 && j > 0) { tri[m] = 2 * ((i - 1) * cx + j - 1) + 1; pos[m++] = 2; }
            std::vector<polygon_t> &cell = cells[(size_t)i * nx + j];
            for (int q = 0; q < m; q++) {
                const int c = tri[q] >> 1, base = (c / cx) * nx + c % cx;
                int v[3];
                if ((tri[q] & 1) == 0) { v[0] = base; v[1] = base + 1; v[2] = base + nx; }
                else { v[0] = base + nx; v[1] = base + 1; v[2] = base + nx + 1; }
                const point_t a = pt(v[pos[q]]), b = pt(v[(pos[q] + 1) % 3]), d = pt(v[(pos[q] + 2) % 3]);
                polygon_t quad(4, point_t(3));
                for (int k = 0; k < 3; k++) {
                    quad[0][k] = a[k];
                    quad[1][k] = (a[k] + b[k]) / 2.0;
                    quad[2][k] = (a[k] + b[k] + d[k]) / 3.0;
                    quad[3][k] = (a[k] + d[k]) / 2.0;
                }
                cell.push_back(quad);
            }
        }
    return cells;
}

}  // namespace pcd_legacy

// Host view of the mesh state (mesh.h:51-58); the point sets are fetched
// from the device on first use after each iteration.
struct Mesh {
    pcd_legacy::lazy<std::vector<point_t>> source_points;
    pcd_legacy::lazy<std::vector<point_t>> target_points;
    double width = 0.0, height = 0.0;
    int res_x = 0, res_y = 0;

    Mesh(std::function<void(std::vector<point_t> &)> src, std::function<void(std::vector<point_t> &)> tgt)
        : source_points(std::move(src)), target_points(std::move(tgt))
    {
    }
};

class Caustic_design {
   public:
    Caustic_design()
        : phi([this](grid_t &v) { v = grid(PCD_GRID_PHI); }),
          errors([this](std::vector<double> &v) { v = verts(PCD_VERT_ERRORS); }),
          target_cells([this](std::vector<std::vector<polygon_t>> &v) {
              v = pcd_legacy::dual_cells(flat_points(PCD_VERT_CELL_POINTS), mesh_res_x, mesh_res_y);
          }),
          target_areas([this](std::vector<double> &v) { v = verts(PCD_VERT_TARGET_AREAS); }),
          pixels([this](grid_t &v) { v = grid(PCD_GRID_PIXELS); }),
          raster([this](grid_t &v) { v = grid(PCD_GRID_RASTER); }),
          gradient([this](std::vector<grid_t> &v) { v = {grid(PCD_GRID_GRADIENT_X), grid(PCD_GRID_GRADIENT_Y)}; }),
          h([this](grid_t &v) { v = grid(PCD_GRID_H); }),
          divergence([this](grid_t &v) { v = grid(PCD_GRID_DIVERGENCE); }),
          norm_x([this](grid_t &v) { v = grid(PCD_GRID_NORM_X); }),
          norm_y([this](grid_t &v) { v = grid(PCD_GRID_NORM_Y); }),
          vertex_gradient([this](grid_t &v) { v = {verts(PCD_VERT_GRADIENT_X), verts(PCD_VERT_GRADIENT_Y)}; }),
          normals([this](grid_t &v) { v = {verts(PCD_VERT_NORMALS_X), verts(PCD_VERT_NORMALS_Y)}; })
    {
        pcd_legacy::check(pcd_ctx_create(-1, &ctx_), "pcd_ctx_create");
    }
    ~Caustic_design()
    {
        if (d_) pcd_design_destroy(d_);
        if (ctx_) pcd_ctx_destroy(ctx_);
        delete mesh;
    }
    Caustic_design(const Caustic_design &) = delete;
    Caustic_design &operator=(const Caustic_design &) = delete;

    using grid_t = pcd_legacy::grid_t;

    Mesh *mesh = nullptr;
    pcd_legacy::lazy<grid_t> phi;
    pcd_legacy::lazy<std::vector<double>> errors;
    pcd_legacy::lazy<std::vector<std::vector<polygon_t>>> target_cells;
    std::vector<std::vector<polygon_t>> first_target_cells;
    pcd_legacy::lazy<std::vector<double>> target_areas;
    pcd_legacy::lazy<grid_t> pixels;
    pcd_legacy::lazy<grid_t> raster;
    pcd_legacy::lazy<std::vector<grid_t>> gradient;
    pcd_legacy::lazy<grid_t> h;
    pcd_legacy::lazy<grid_t> divergence;
    pcd_legacy::lazy<grid_t> norm_x;
    pcd_legacy::lazy<grid_t> norm_y;
    pcd_legacy::lazy<grid_t> vertex_gradient;
    pcd_legacy::lazy<grid_t> normals;

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
        mesh = new Mesh([this](std::vector<point_t> &v) { v = points(PCD_VERT_SOURCE_POINTS); },
                        [this](std::vector<point_t> &v) { v = points(PCD_VERT_TARGET_POINTS); });
        mesh->width = width; mesh->height = height;
        mesh->res_x = mesh_res_x; mesh->res_y = mesh_res_y;
        invalidate();
    }

    double perform_transport_iteration()
    {
        double step = 0.0;
        pcd_legacy::check(pcd_design_transport_iteration(d_, &step, nullptr), "perform_transport_iteration");
        invalidate();
        return step;
    }

    void perform_height_map_iteration(int itr)
    {
        double upd = 0.0;
        pcd_legacy::check(pcd_design_height_iteration(d_, itr, &upd, nullptr), "perform_height_map_iteration");
        invalidate();
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

    grid_t grid(int which)
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

    std::vector<double> flat_points(int which)
    {
        std::vector<double> flat((size_t)mesh_res_x * mesh_res_y * 3);
        pcd_legacy::check(pcd_design_get_vertices(d_, which, flat.data()), "pcd_design_get_vertices");
        return flat;
    }

    std::vector<point_t> points(int which) { return pcd_legacy::to_rows(flat_points(which), 3, mesh_res_x * mesh_res_y); }

    void invalidate()
    {
        phi.invalidate(); errors.invalidate(); target_cells.invalidate(); target_areas.invalidate();
        pixels.invalidate(); raster.invalidate(); gradient.invalidate(); h.invalidate();
        divergence.invalidate(); norm_x.invalidate(); norm_y.invalidate(); vertex_gradient.invalidate();
        normals.invalidate();
        if (mesh) {
            mesh->target_points.invalidate();
            mesh->source_points.invalidate();
        }
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
