// writers.cu -- the reference's output files, written from host arrays or
// from a design's device state (host code).
//
// The text matches the reference's writers byte for byte: numbers go through
// the formats its streams use (operator<< on a double with the default
// precision is printf "%g"; std::to_string(double) is "%f"), vertex and face
// order follow it, including the second SVG loop's use of res_x as its
// bound (utils.cpp:292).  Files are written in full or not at all: a file
// that cannot be opened returns PCD_BAD_ARG (the reference prints to cerr).
#include <cstdio>
#include <string>
#include <vector>

#include "api_internal.cuh"
#include "design.cuh"

namespace pcd {

namespace {

std::string g(double v)
{
    char buf[64];
    std::snprintf(buf, sizeof(buf), "%g", v);
    return buf;
}

std::string f(double v)
{
    char buf[384];
    std::snprintf(buf, sizeof(buf), "%f", v);
    return buf;
}

int write_file(const char *filename, const std::string &text)
{
    if (!filename) return PCD_BAD_ARG;
    FILE *fp = std::fopen(filename, "wb");
    if (!fp) {
        set_error(std::string("cannot open ") + filename + " for writing");
        return PCD_BAD_ARG;
    }
    const size_t n = std::fwrite(text.data(), 1, text.size(), fp);
    const int rc = std::fclose(fp);
    if (n != text.size() || rc != 0) {
        set_error(std::string("short write to ") + filename);
        return PCD_BAD_ARG;
    }
    return PCD_OK;
}

// perimeter of the structured mesh, clockwise from vertex 0 (utils.cpp:173-195)
std::vector<int> perimeter(int nx, int ny)
{
    std::vector<int> p;
    for (int i = 0; i < nx; ++i) p.push_back(i);
    for (int i = nx - 1; i < nx * ny; i += nx) p.push_back(i);
    for (int i = nx * (ny - 1) + nx - 1; i > nx * (ny - 1) - 1; --i) p.push_back(i);
    for (int i = nx * (ny - 1) - nx; i > nx - 1; i -= nx) p.push_back(i);
    return p;
}

}  // namespace

int write_solid_obj(const double *front, const double *back, int nx, int ny, double thickness, double width,
                    double height, const char *filename)
{
    if (!front || !back || nx < 2 || ny < 2) {
        set_error("pcd_write_solid_obj: bad arguments");
        return PCD_BAD_ARG;
    }
    const int n = nx * ny;
    double min_h = 0.0;
    for (int i = 0; i < n; i++)
        if (min_h > front[3 * i + 2]) min_h = front[3 * i + 2];
    std::string t;
    t.reserve((size_t)n * 80);
    t += "# Generated by the software algorithm written by Dylan Missuwe\n";
    t += "# The algorithm used to create the lens is based on the paper "
         "\"Poisson-Based Continuous Surface Generation for Goal-Based Caustics\" by Yue et al (2014)\n";
    for (int i = 0; i < n; i++)
        t += "v " + g(width - front[3 * i]) + " " + g(height - front[3 * i + 1]) + " " + g(-(front[3 * i + 2])) + "\n";
    for (int i = 0; i < n; i++)
        t += "v " + g(width - back[3 * i]) + " " + g(height - back[3 * i + 1]) + " " + g(-thickness - min_h) + "\n";
    // structured-mesh triangles (mesh.cpp:57-63), then the same reversed for the back
    auto face = [&](int a, int b, int c) {
        t += "f " + std::to_string(a) + " " + std::to_string(b) + " " + std::to_string(c) + "\n";
    };
    for (int y = 0; y < ny - 1; y++)
        for (int x = 0; x < nx - 1; x++) {
            const int i = y * nx + x;
            face(i + 1, i + 2, i + nx + 1);
            face(i + nx + 1, i + 2, i + nx + 2);
        }
    for (int y = 0; y < ny - 1; y++)
        for (int x = 0; x < nx - 1; x++) {
            const int i = y * nx + x;
            face(i + n + 1, i + nx + n + 1, i + 1 + n + 1);
            face(i + nx + n + 1, i + nx + 1 + n + 1, i + 1 + n + 1);
        }
    // side wall between the front and back perimeters (utils.cpp:243-256)
    const std::vector<int> per = perimeter(nx, ny);
    for (size_t k = 0; k < per.size(); ++k) {
        const int top = per[k], bottom = per[k] + n;
        const int next_top = per[(k + 1) % per.size()], next_bottom = next_top + n;
        face(top + 1, bottom + 1, next_bottom + 1);
        face(top + 1, next_bottom + 1, next_top + 1);
    }
    return write_file(filename, t);
}

int write_grid_svg(const double *pts, int nx, int ny, double width, double height, const char *filename,
                   double stroke_width)
{
    if (!pts || nx < 1 || ny < 1 || !(width > 0.0)) {
        set_error("pcd_write_grid_svg: bad arguments");
        return PCD_BAD_ARG;
    }
    const double aspect = height / width;
    std::string t;
    t += "<?xml version=\"1.0\" encoding=\"UTF-8\" ?>\n";
    t += "<svg width=\"1000\" height=\"" + g(1000.0f * aspect) +
         "\" xmlns=\"http://www.w3.org/2000/svg\" xmlns:xlink=\"http://www.w3.org/1999/xlink\">\n";
    t += "<rect width=\"100%\" height=\"100%\" fill=\"white\"/>\n";
    auto coord = [&](int idx) {
        return f((pts[3 * idx] / width) * 1000.0f) + "," + f((pts[3 * idx + 1] / height) * 1000.0f * aspect);
    };
    const std::string tail = "\" fill=\"none\" stroke=\"black\" stroke-width=\"" + g(stroke_width) + "\"/>\n";
    for (int j = 0; j < ny; j++) {
        std::string path = "M";
        for (int i = 0; i < nx; i++) {
            path += coord(i + j * nx);
            if (i < nx - 1) path += "L";
        }
        t += "<path d=\"" + path + tail;
    }
    for (int j = 0; j < nx; j++) {
        std::string path = "M";
        for (int i = 0; i < ny; i++) {
            path += coord(j + i * nx);
            if (i < nx - 1) path += "L";  // the reference bounds this loop's separators by res_x
        }
        t += "<path d=\"" + path + tail;
    }
    t += "</svg>\n";
    return write_file(filename, t);
}

int write_heightmap_json(const double *h, int width, int height, const char *filename)
{
    if (!h || width < 0 || height < 0) {
        set_error("pcd_write_heightmap_json: bad arguments");
        return PCD_BAD_ARG;
    }
    std::string t = "[\n";
    for (int i = 0; i < height; ++i) {
        t += "  [";
        for (int j = 0; j < width; ++j) {
            t += g(h[(size_t)i * width + j]);
            if (j < width - 1) t += ", ";
        }
        t += "]";
        t += i < height - 1 ? ",\n" : "\n";
    }
    t += "]\n";
    return write_file(filename, t);
}

}  // namespace pcd

using namespace pcd;

extern "C" {

int pcd_write_solid_obj(const double *front_points, const double *back_points, int mesh_res_x, int mesh_res_y,
                        double thickness, double width, double height, const char *filename)
{
    return write_solid_obj(front_points, back_points, mesh_res_x, mesh_res_y, thickness, width, height, filename);
}

int pcd_write_grid_svg(const double *points, int mesh_res_x, int mesh_res_y, double width, double height,
                       const char *filename, double stroke_width)
{
    return write_grid_svg(points, mesh_res_x, mesh_res_y, width, height, filename, stroke_width);
}

int pcd_write_heightmap_json(const double *h, int width, int height, const char *filename)
{
    return write_heightmap_json(h, width, height, filename);
}

int pcd_design_save_solid_obj(pcd_design *d, int which, const char *filename)
{
    if (!d || (which != 0 && which != 1)) return PCD_BAD_ARG;
    const pcd_design_params &p = d->d.p;
    const size_t n = (size_t)p.mesh_res_x * p.mesh_res_y;
    std::vector<double> src(3 * n), front;
    PCD_TRY(pcd_design_get_vertices(d, PCD_VERT_SOURCE_POINTS, src.data()));
    if (which == 1) {
        front.resize(3 * n);
        PCD_TRY(pcd_design_get_vertices(d, PCD_VERT_TARGET_POINTS, front.data()));
    }
    return write_solid_obj(which == 1 ? front.data() : src.data(), src.data(), p.mesh_res_x, p.mesh_res_y,
                           p.thickness, p.width, p.height, filename);
}

int pcd_design_export_parameterization_svg(pcd_design *d, const char *filename, double stroke_width)
{
    if (!d) return PCD_BAD_ARG;
    const pcd_design_params &p = d->d.p;
    std::vector<double> tgt(3 * (size_t)p.mesh_res_x * p.mesh_res_y);
    PCD_TRY(pcd_design_get_vertices(d, PCD_VERT_TARGET_POINTS, tgt.data()));
    return write_grid_svg(tgt.data(), p.mesh_res_x, p.mesh_res_y, p.width, p.height, filename, stroke_width);
}

int pcd_design_export_inverted_transport_map_svg(pcd_design *d, const char *filename, double stroke_width)
{
    if (!d) return PCD_BAD_ARG;
    const pcd_design_params &p = d->d.p;
    std::vector<double> inv(3 * (size_t)p.mesh_res_x * p.mesh_res_y);
    PCD_TRY(pcd_design_get_vertices(d, PCD_VERT_INVERTED_MAP, inv.data()));
    return write_grid_svg(inv.data(), p.mesh_res_x, p.mesh_res_y, p.width, p.height, filename, stroke_width);
}

int pcd_design_save_heightmap_json(pcd_design *d, const char *filename)
{
    if (!d) return PCD_BAD_ARG;
    const pcd_design_params &p = d->d.p;
    std::vector<double> h((size_t)p.res_x * p.res_y);
    PCD_TRY(pcd_design_get_grid(d, PCD_GRID_H, h.data()));
    return write_heightmap_json(h.data(), p.res_x, p.res_y, filename);
}

}  // extern "C"
