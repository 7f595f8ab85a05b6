// Replays main.cpp:216-262 of the reference (without the PNG loader) against
// include/pcd_legacy.hpp, i.e. the reference's C++ signatures backed by
// libpcd_gb300.  Usage: shim_main <res> <image.f64> <out.f64>
//   image.f64: (4res)^2 doubles, row-major; out.f64 receives the transport
//   step sizes (50 slots, NaN after the last), the final target points
//   (n x 3), source points (n x 3) and h ((4res)^2).
#include <cmath>
#include <cstdio>
#include <vector>

#include "pcd_legacy.hpp"

int main(int argc, char **argv)
{
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
