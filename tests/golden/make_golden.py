"""Write the golden fixtures in this folder from the reference's own compiled
sources (oracle/_ref/libpcd_ref.so, built by oracle/Makefile from the mounted
reference tree).  Run from the repository root:

    python tests/golden/make_golden.py

Fixtures (all float64, seeded inputs, the reference run with max_threads=1):

* solver_cases.npz  -- poisson_solver (solver.cpp:70-148) on small grids:
  zero and warm starts, ragged sizes, a NaN hole, an iteration cap.
* utils_cases.npz   -- calculate_gradient / calculate_divergence /
  subtractAverage / scale_matrix_proportional / bilinearInterpolation.
* writer_cases.npz -- save_solid_obj (utils.cpp:198-260) and
  export_grid_to_svg (utils.cpp:262-307) output files (bytes) of the
  reference on seeded point sets: ragged and square meshes, negative heights,
  %g exponents, the non-square SVG whose second loop uses res_x as bound.
* mesh_cases.npz -- Mesh::laplacian_smoothing (mesh.cpp:534-606) with the
  factor 0.1f of caustic_design.cpp:216 on perturbed meshes (one folded).
* pipeline_r{16,32,64}.npz -- Caustic_design replay of main.cpp:216-262 at
  mesh resolution r (grid 4r): per-iteration step sizes, target areas, the
  first iteration's errors/raster, final phi / target points, and after the
  three height iterations h and the source points.
* pipeline_r128.npz -- the same replay at the full-pipeline workload's own
  size (mesh 128 x 128, 512 x 512 grids, width 0.5, focal length 1.5,
  thickness 0.1, conv 0.01), kept compact: step sizes, target areas, the first
  iteration's errors, the final target and source points (the vertex heights
  are the source points' z) and the final h sampled every 4th cell.  About
  five minutes of single-threaded CPU:

      python tests/golden/make_golden.py --r128
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), "..", ".."))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle as O  # noqa: E402
from poisson_caustic_design_gb300 import inputs  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def solver_cases(R: O.Ref):
    cases = {}
    rng = np.random.default_rng(20241203)

    def add(name, b, phi0, max_iter, tol):
        phi = phi0.copy()
        R.poisson_solver(b, phi, max_iter, tol, 1)
        cases[f"{name}/b"] = b
        cases[f"{name}/phi0"] = phi0
        cases[f"{name}/phi"] = phi
        cases[f"{name}/params"] = np.array([max_iter, tol])

    b = rng.standard_normal((5, 7)); b -= b.mean()
    add("rand_7x5", b, np.zeros_like(b), 100000, 1e-9)
    b = rng.standard_normal((17, 33)); b -= b.mean()
    add("warm_33x17", b, rng.standard_normal((17, 33)), 100000, 1e-7)
    add("gauss_64", inputs.poisson_rhs(64, 1, "gaussian"), np.zeros((64, 64)), 100000, 1e-7)
    add("binary_96x80", inputs.poisson_rhs(96, 2, "binary", m=80), np.zeros((80, 96)), 100000, 1e-7)
    add("gauss_128", inputs.poisson_rhs(128, 3, "gaussian"), np.zeros((128, 128)), 100000, 1e-7)
    b = inputs.poisson_rhs(48, 4, "gaussian", m=40)
    b[10:14, 20:27] = np.nan
    b[0, 0] = np.nan
    b = R.subtract_average(b)   # consistent again on the non-NaN cells (utils.cpp:60-86)
    add("nanhole_48x40", b, np.zeros_like(b), 100000, 1e-8)
    add("capped_64", inputs.poisson_rhs(64, 5, "binary"), np.zeros((64, 64)), 50, 1e-12)
    b = rng.standard_normal((1, 16)); b -= b.mean()
    add("single_row_16x1", b, np.zeros((1, 16)), 3000, 1e-9)
    np.savez_compressed(os.path.join(OUT, "solver_cases.npz"), **cases)


def utils_cases(R: O.Ref):
    rng = np.random.default_rng(7)
    g = rng.standard_normal((19, 23))
    g2 = rng.standard_normal((19, 23))
    gx, gy = R.gradient(g)
    pts = np.array([[-0.5, -0.5], [3.25, 2.75], [22.5, 18.5], [0.0, 0.0], [21.999, 17.2], [10.0, 5.5]])
    gn = g.copy(); gn[3, 4] = np.nan
    np.savez_compressed(
        os.path.join(OUT, "utils_cases.npz"),
        g=g, g2=g2, gx=gx, gy=gy, div=R.divergence(g, g2), sub=R.subtract_average(gn), gn=gn,
        scaled=R.scale_proportional(g * 3.0 + 1.0, 0.0, 1.0), pts=pts,
        bil=np.array([R.bilinear(g, x, y) for x, y in pts]),
    )


def pipeline(R: O.Ref, res: int, seed: int, width=0.5, focal=1.5, thickness=0.1, conv=0.01):
    img = inputs.pipeline_image(res, seed)
    d = O.RefDesign(R, res, res, 4 * res, 4 * res, width, width, focal, thickness, 1)
    d.initialize(img)
    out = {"image": img, "params": np.array([res, width, focal, thickness, conv, seed]),
           "target_areas": d.get("target_areas")}
    steps = []
    for itr in range(50):
        s = d.transport_iteration()
        steps.append(s)
        if itr == 0:
            out["errors_0"] = d.get("errors")
            out["raster_0"] = d.get("raster")
            out["phi_0"] = d.get("phi")
            out["target_points_0"] = d.get("target_points")
        if s < conv:
            break
    out["steps"] = np.array(steps)
    out["phi"] = d.get("phi")
    out["target_points"] = d.get("target_points")
    for itr in range(3):
        d.height_iteration(itr)
        if itr == 0:
            out["normals_x_0"] = d.get("normals_x")
            out["normals_y_0"] = d.get("normals_y")
            out["divergence_0"] = d.get("divergence")
            out["h_0"] = d.get("h")
            out["source_points_0"] = d.get("source_points")
    out["h"] = d.get("h")
    out["source_points"] = d.get("source_points")
    d.close()
    np.savez_compressed(os.path.join(OUT, f"pipeline_r{res}.npz"), **out)
    return len(steps)


def pipeline_compact(R: O.Ref, res: int, seed: int, width=0.5, focal=1.5, thickness=0.1, conv=0.01):
    img = inputs.pipeline_image(res, seed)
    d = O.RefDesign(R, res, res, 4 * res, 4 * res, width, width, focal, thickness, 1)
    d.initialize(img)
    out = {"params": np.array([res, width, focal, thickness, conv, seed]), "target_areas": d.get("target_areas")}
    steps = []
    for itr in range(50):
        s = d.transport_iteration()
        steps.append(s)
        if itr == 0:
            out["errors_0"] = d.get("errors")
        if s < conv:
            break
    out["steps"] = np.array(steps)
    out["target_points"] = d.get("target_points")
    for itr in range(3):
        d.height_iteration(itr)
    out["h_sub4"] = np.ascontiguousarray(d.get("h")[::4, ::4])
    out["source_points"] = d.get("source_points")
    d.close()
    np.savez_compressed(os.path.join(OUT, f"pipeline_r{res}.npz"), **out)
    return len(steps)


def writer_cases(R: O.Ref):
    import tempfile

    rng = np.random.default_rng(77)
    cases = {}

    def pts(nx, ny, w, h, zlo, zhi, jitter=True):
        y, x = np.meshgrid(np.arange(ny) * h / (ny - 1), np.arange(nx) * w / (nx - 1), indexing="ij")
        p = np.stack([x.ravel(), y.ravel(), rng.uniform(zlo, zhi, nx * ny)], axis=1)
        if jitter:
            p[:, :2] += rng.normal(0, 0.01 * w, (nx * ny, 2))
        return p

    with tempfile.TemporaryDirectory() as td:
        fn = os.path.join(td, "out")
        obj = [("obj_a", 7, 5, 0.5, 0.35, 0.1, pts(7, 5, 0.5, 0.35, -0.03, 0.02), pts(7, 5, 0.5, 0.35, 0, 0, False)),
               ("obj_b", 4, 4, 1.0, 1.0, 0.2, pts(4, 4, 1.0, 1.0, 0.0, 0.0), pts(4, 4, 1.0, 1.0, 0.0, 0.02, False)),
               ("obj_c", 3, 6, 12345.678, 0.001, 1e-7,
                pts(3, 6, 12345.678, 0.001, -1e-5, 3e4), pts(3, 6, 12345.678, 0.001, -2.0, 2.0))]
        for name, nx, ny, w, h, th, front, back in obj:
            R.save_solid_obj(front, back, nx, ny, th, w, h, fn)
            cases[f"{name}/front"], cases[f"{name}/back"] = front, back
            cases[f"{name}/params"] = np.array([nx, ny, w, h, th])
            cases[f"{name}/text"] = np.frombuffer(open(fn, "rb").read(), dtype=np.uint8)
        svg = [("svg_a", 7, 5, 0.5, 0.35, 0.5), ("svg_b", 5, 7, 0.35, 0.5, 1.0), ("svg_c", 6, 6, 0.5, 0.5, 1.0)]
        for name, nx, ny, w, h, sw in svg:
            p = pts(nx, ny, w, h, 0.0, 0.0)
            R.export_grid_svg(p, nx, ny, w, h, fn, sw)
            cases[f"{name}/points"] = p
            cases[f"{name}/params"] = np.array([nx, ny, w, h, sw])
            cases[f"{name}/text"] = np.frombuffer(open(fn, "rb").read(), dtype=np.uint8)
    np.savez_compressed(os.path.join(OUT, "writer_cases.npz"), **cases)


def mesh_cases(R: O.Ref):
    rng = np.random.default_rng(31)
    cases = {}
    f = float(np.float32(0.1))
    for name, nx, ny, w, h, sig in (("smooth_a", 9, 7, 0.5, 0.35, 0.02), ("smooth_b", 16, 16, 0.5, 0.5, 0.06)):
        y, x = np.meshgrid(np.arange(ny) * h / (ny - 1), np.arange(nx) * w / (nx - 1), indexing="ij")
        p = np.stack([x.ravel(), y.ravel(), np.zeros(nx * ny)], axis=1)
        p[:, :2] += rng.normal(0, sig * w / nx, (nx * ny, 2))
        cases[f"{name}/points"] = p
        cases[f"{name}/params"] = np.array([nx, ny, w, h, f])
        cases[f"{name}/smoothed"] = R.laplacian_smoothing(p, nx, ny, w, h, f)
    np.savez_compressed(os.path.join(OUT, "mesh_cases.npz"), **cases)


def main():
    O.build(ref=True)
    R = O.Ref()
    if "--r128" in sys.argv[1:]:
        n = pipeline_compact(R, 128, 47)
        print(f"pipeline r128: {n} transport iterations")
        return
    solver_cases(R)
    utils_cases(R)
    writer_cases(R)
    mesh_cases(R)
    for res, seed in ((16, 3), (32, 11), (64, 29)):
        n = pipeline(R, res, seed)
        print(f"pipeline r{res}: {n} transport iterations")


if __name__ == "__main__":
    main()
