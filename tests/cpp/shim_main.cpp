// Replays main.cpp:216-262 of the reference (without the PNG loader) against
// include/pcd_legacy.hpp, i.e. the reference's C++ signatures backed by
// libpcd_gb300.  Usage: shim_main <res> <image.f64> <out.f64>
//   image.f64: (4res)^2 doubles, row-major; out.f64 receives the transport
//   step sizes (50 slots, NaN after the last), the final target points
//   (n x 3), source points (n x 3) and h ((4res)^2).
// Timing mode: shim_main time <res> <image.f64> prints the wall time (ms) of
// the first transport iteration through Caustic_design (the shim) and through
// the C ABI directly, after an untimed warm-up, and the two step sizes.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "pcd_legacy.hpp"

static double ms_since(std::chrono::steady_clock::time_point t)
{
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t).count();
}

static double abi_iteration(int res, const std::vector<double> &flat, double *step)
{
    pcd_ctx *ctx = nullptr;
    pcd_design *d = nullptr;
    pcd_ctx_create(-1, &ctx);
    pcd_design_params p;
    pcd_design_params_default(&p);
    p.mesh_res_x = p.mesh_res_y = res;
    p.res_x = p.res_y = 4 * res;
    p.width = p.height = 0.5;
    p.focal_l = 1.5;
    p.thickness = 0.1;
    pcd_design_create(ctx, &p, &d);
    pcd_design_initialize(d, flat.data());
    const auto t = std::chrono::steady_clock::now();
    pcd_design_transport_iteration(d, step, nullptr);
    const double ms = ms_since(t);
    pcd_design_destroy(d);
    pcd_ctx_destroy(ctx);
    return ms;
}

static int timing(int res, const char *image)
{
    const int n = 4 * res;
    std::vector<double> flat((size_t)n * n);
    FILE *f = std::fopen(image, "rb");
    if (!f || std::fread(flat.data(), sizeof(double), flat.size(), f) != flat.size()) return 3;
    std::fclose(f);
    std::vector<std::vector<double>> img = pcd_legacy::to_rows(flat, n, n);
    double s0 = 0, s1 = 0, s2 = 0;
    abi_iteration(res, flat, &s0);  // warm-up
    double shim_ms;
    {
        Caustic_design cd;
        cd.set_mesh_resolution(res, res);
        cd.set_domain_resolution(n, n);
        cd.set_mesh_size(0.5, 0.5);
        cd.set_lens_focal_length(1.5);
        cd.set_lens_thickness(0.1);
        cd.initialize_solvers(img);
        const auto t = std::chrono::steady_clock::now();
        s1 = cd.perform_transport_iteration();
        shim_ms = ms_since(t);
    }
    const double abi_ms = abi_iteration(res, flat, &s2);
    std::printf("%.3f %.3f %.17g %.17g\n", shim_ms, abi_ms, s1, s2);
    return 0;
}

int main(int argc, char **argv)
{
    if (argc == 4 && std::strcmp(argv[1], "time") == 0) return timing(std::atoi(argv[2]), argv[3]);
    if (argc != 4) return 2;
    const int res = std::atoi(argv[1]);
    const int n = 4 * res;
    std::vector<std::vector<double>> img(n, std::vector<double>(n));
    FILE *f = std::fopen(argv[2], "rb");
    if (!f) return 3;
    for (auto &row : img)
        if (std::fread(row.data(), sizeof(double), n, f) != (size_t)n) return 4;
    std::fclose(f);

    // a single-tile lexicographic check of the free function first
    std::vector<std::vector<double>> D(8, std::vector<double>(8, 0.0)), phi(8, std::vector<double>(8, 0.0));
    D[2][3] = 1.0;
    D[5][6] = -1.0;
    poisson_solver(D, phi, 8, 8, 100000, 1e-10, 4);
    if (!(std::fabs(phi[2][3] - phi[5][6]) > 0.1)) return 5;

    Caustic_design cd;
    cd.set_mesh_resolution(res, res);
    cd.set_domain_resolution(n, n);
    cd.set_mesh_size(0.5, 0.5);
    cd.set_lens_focal_length(1.5);
    cd.set_lens_thickness(0.1);
    cd.set_solver_max_threads(1);
    cd.initialize_solvers(img);
    std::vector<double> steps(50, NAN);
    for (int itr = 0; itr < 50; itr++) {
        double s = cd.perform_transport_iteration();
        steps[itr] = s;
        if (s < 0.01) break;
    }
    for (int itr = 0; itr < 3; itr++) cd.perform_height_map_iteration(itr);

    FILE *o = std::fopen(argv[3], "wb");
    if (!o) return 6;
    std::fwrite(steps.data(), sizeof(double), steps.size(), o);
    for (auto &p : cd.mesh->target_points) std::fwrite(p.data(), sizeof(double), 3, o);
    for (auto &p : cd.mesh->source_points) std::fwrite(p.data(), sizeof(double), 3, o);
    for (auto &row : cd.h) std::fwrite(row.data(), sizeof(double), row.size(), o);
    std::fclose(o);
    return 0;
}
