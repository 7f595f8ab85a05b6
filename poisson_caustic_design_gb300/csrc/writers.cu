// writers.cu -- the reference's output files, written from host arrays or
// from a design's device state (host code).
//
// The text matches the reference's writers byte for byte: numbers go through
// the formats its streams use (operator<< on a double with the default
// precision is printf "%g"; std::to_string(double) is "%f"), vertex and face
// order follow it, including the second SVG loop's use of res_x as its
// bound (utils.cpp:292).  Files are written in full or not at all: a file
// that cannot be opened returns PCD_BAD_ARG (the reference prints to cerr).
#include <algorithm>
#include <cstdio>
#include <string>
#include <thread>
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

// number formats appended in place (no temporaries)
void app_g(std::string &t, double v)
{
    char buf[64];
    const int k = std::snprintf(buf, sizeof(buf), "%g", v);
    t.append(buf, (size_t)k);
}

void app_f(std::string &t, double v)
{
    char buf[384];
    const int k = std::snprintf(buf, sizeof(buf), "%f", v);
    t.append(buf, (size_t)k);
}

void app_i(std::string &t, int v)
{
    char buf[16];
    const int k = std::snprintf(buf, sizeof(buf), "%d", v);
    t.append(buf, (size_t)k);
}

// Appends emit(i, text) for i = 0 .. count-1 to t, in order: ranges of at
// least `grain` items formatted on up to 16 host threads into separate
// buffers, then concatenated (the bytes do not depend on the thread count).
template <class Emit>
void parallel_text(std::string &t, long count, long grain, Emit emit)
{
    const long hw = std::max(1u, std::thread::hardware_concurrency());
    const long T = std::max(1L, std::min({hw, 16L, count / std::max(1L, grain)}));
    if (T == 1) {
        for (long i = 0; i < count; i++) emit(i, t);
        return;
    }
    std::vector<std::string> part((size_t)T);
    std::vector<std::thread> th;
    for (long k = 0; k < T; k++)
        th.emplace_back([&, k] {
            const long a = count * k / T, b = count * (k + 1) / T;
            for (long i = a; i < b; i++) emit(i, part[(size_t)k]);
        });
    for (auto &x : th) x.join();
    size_t total = t.size();
    for (auto &p : part) total += p.size();
    t.reserve(total);
    for (auto &p : part) t += p;
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
    auto vert = [](std::string &s, double a, double b, double c) {
        s += "v ";
        app_g(s, a);
        s += ' ';
        app_g(s, b);
        s += ' ';
        app_g(s, c);
        s += '\n';
    };
    parallel_text(t, n, 4096, [&](long i, std::string &s) {
        vert(s, width - front[3 * i], height - front[3 * i + 1], -(front[3 * i + 2]));
    });
    parallel_text(t, n, 4096, [&](long i, std::string &s) {
        vert(s, width - back[3 * i], height - back[3 * i + 1], -thickness - min_h);
    });
    // structured-mesh triangles (mesh.cpp:57-63), then the same reversed for the back
    auto face_to = [](std::string &s, int a, int b, int c) {
        s += "f ";
        app_i(s, a);
        s += ' ';
        app_i(s, b);
        s += ' ';
        app_i(s, c);
        s += '\n';
    };
    const long cells = (long)(nx - 1) * (ny - 1);
    parallel_text(t, cells, 4096, [&](long k, std::string &s) {
        const int y = (int)(k / (nx - 1)), x = (int)(k - (long)y * (nx - 1)), i = y * nx + x;
        face_to(s, i + 1, i + 2, i + nx + 1);
        face_to(s, i + nx + 1, i + 2, i + nx + 2);
    });
    parallel_text(t, cells, 4096, [&](long k, std::string &s) {
        const int y = (int)(k / (nx - 1)), x = (int)(k - (long)y * (nx - 1)), i = y * nx + x;
        face_to(s, i + n + 1, i + nx + n + 1, i + 1 + n + 1);
        face_to(s, i + nx + n + 1, i + nx + 1 + n + 1, i + 1 + n + 1);
    });
    auto face = [&](int a, int b, int c) { face_to(t, a, b, c); };
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
    auto coord = [&](std::string &s, int idx) {
        app_f(s, (pts[3 * idx] / width) * 1000.0f);
        s += ',';
        app_f(s, (pts[3 * idx + 1] / height) * 1000.0f * aspect);
    };
    const std::string tail = "\" fill=\"none\" stroke=\"black\" stroke-width=\"" + g(stroke_width) + "\"/>\n";
    // one path a row, then one a column, each formatted on its own
    parallel_text(t, ny, 8, [&](long j, std::string &s) {
        s += "<path d=\"M";
        for (int i = 0; i < nx; i++) {
            coord(s, i + (int)j * nx);
            if (i < nx - 1) s += 'L';
        }
        s += tail;
    });
    parallel_text(t, nx, 8, [&](long j, std::string &s) {
        s += "<path d=\"M";
        for (int i = 0; i < ny; i++) {
            coord(s, (int)j + i * nx);
            if (i < nx - 1) s += 'L';  // the reference bounds this loop's separators by res_x
        }
        s += tail;
    });
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
    parallel_text(t, height, 8, [&](long i, std::string &s) {
        s += "  [";
        for (int j = 0; j < width; ++j) {
            app_g(s, h[(size_t)i * width + j]);
            if (j < width - 1) s += ", ";
        }
        s += "]";
        s += i < height - 1 ? ",\n" : "\n";
    });
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
