"""CPU checkers for the Poisson caustic-design hot path.

TEST INFRASTRUCTURE ONLY: tests/, ``__graft_entry__.smoke()`` and bench.py's
CPU-baseline leg use this module as the checker.  The product
(``poisson_caustic_design_gb300``) never imports it.

Three checkers live here:

* ``Port``: ctypes over ``_build/libpcd_oracle.so``, our C restatement of the
  reference's solver and per-iteration mesh/grid steps (pcd_oracle.c, each
  function citing the reference file:line).  Built on every machine.
* ``Ref``: ctypes over ``_ref/libpcd_ref.so``, the reference's own
  src/*.cpp compiled in place (oracle/Makefile).  Only present where the
  reference tree is mounted; used to pin ``Port`` and to write the golden
  fixtures.
* ``dct_solve``: the exact FP64 solve of the reference operator by a DCT-II
  diagonalisation (scipy), the "oracle solved to 1e-12".
* ``PortDesign``: the Caustic_design iteration sequence
  (caustic_design.cpp:190-364) composed from ``Port`` primitives.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "libpcd_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libpcd_ref.so")
# the reference tree: $PCD_REFERENCE when set, else where this container mounts it
REF_TREE = os.environ.get("PCD_REFERENCE", "/root/reference")

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")


def build(ref: bool | None = None) -> None:
    """Compile the port (always) and the reference library (when its tree exists)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    if ref is None:
        ref = os.path.isdir(os.path.join(REF_TREE, "src"))
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={REF_TREE}"], check=True)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class Port:
    """Our C restatement (pcd_oracle.c)."""

    def __init__(self, path: str = PORT_SO):
        if not os.path.exists(path):
            build(ref=False)
        L = C.CDLL(path)
        self.L = L
        L.pcdo_poisson_solver.argtypes = [_dp, _dp, C.c_int, C.c_int, C.c_int, C.c_double, C.POINTER(C.c_double)]
        L.pcdo_poisson_solver.restype = C.c_int
        L.pcdo_poisson_solver_threads.argtypes = [_dp, _dp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int,
                                                  C.c_int, C.c_double, C.POINTER(C.c_double)]
        L.pcdo_poisson_solver_threads.restype = C.c_int
        L.pcdo_sor_sweeps.argtypes = [_dp, _dp, C.c_int, C.c_int, C.c_int, C.c_double]
        L.pcdo_sor_sweeps.restype = C.c_double
        L.pcdo_residual.argtypes = [_dp, _dp, C.c_int, C.c_int, C.c_void_p, _dp]
        L.pcdo_subtract_average.argtypes = [_dp, C.c_long]
        L.pcdo_gradient.argtypes = [_dp, C.c_int, C.c_int, _dp, _dp]
        L.pcdo_divergence.argtypes = [_dp, _dp, C.c_int, C.c_int, _dp]
        L.pcdo_scale_proportional.argtypes = [_dp, C.c_long, C.c_double, C.c_double, _dp]
        L.pcdo_resize_nearest.argtypes = [_dp, C.c_int, C.c_int, _dp, C.c_int, C.c_int]
        L.pcdo_bilinear.argtypes = [_dp, C.c_int, C.c_int, C.c_double, C.c_double]
        L.pcdo_bilinear.restype = C.c_double
        L.pcdo_mesh_points.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, _dp]
        L.pcdo_dual_cell_areas.argtypes = [_dp, C.c_int, C.c_int, _dp]
        L.pcdo_target_areas.argtypes = [_dp, C.c_int, C.c_int, C.c_double, C.c_double, _dp, C.c_int, C.c_int, _dp]
        L.pcdo_raster.argtypes = [_dp, _dp, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int, C.c_int, _dp]
        L.pcdo_raster.restype = C.c_int
        L.pcdo_inverted_map.argtypes = [_dp, _dp, C.c_int, C.c_int, C.c_double, C.c_double, _dp]
        L.pcdo_inverted_map.restype = C.c_int
        L.pcdo_refractive_normals.argtypes = [_dp, _dp, C.c_long, C.c_double, C.c_double, _dp, _dp]
        L.pcdo_step_grid.argtypes = [_dp, _dp, _dp, C.c_int, C.c_int, C.c_double, C.c_double]
        L.pcdo_step_grid.restype = C.c_double
        L.pcdo_sample_vertices.argtypes = [_dp, C.c_int, C.c_int, _dp, C.c_long, C.c_double, C.c_double, _dp]
        L.pcdo_set_source_heights.argtypes = [_dp, _dp, C.c_long]
        L.pcdo_set_source_heights.restype = C.c_double
        L.pcdo_laplacian_smoothing.argtypes = [_dp, C.c_int, C.c_int, C.c_double]
        L.pcdo_count_folds.argtypes = [_dp, C.c_int, C.c_int]
        L.pcdo_count_folds.restype = C.c_long

    # solver.cpp:70-148 with one tile (max_threads <= 3)
    def poisson_solver(self, D, phi, max_iterations=100000, tol=1e-7):
        """In place on ``phi`` (float64, C-contiguous).  Returns (sweeps, last max|delta|)."""
        D = _f64(D)
        assert phi.dtype == np.float64 and phi.flags.c_contiguous
        h, w = D.shape
        mu = C.c_double(0)
        n = self.L.pcdo_poisson_solver(D, phi, w, h, int(max_iterations), float(tol), C.byref(mu))
        return n, mu.value

    def poisson_solver_threads(self, D, phi, max_iterations=100000, tol=1e-7, max_threads=1, omega=0.0):
        """solver.cpp:70-148 with the reference's tile threading (hardware
        threads = os.cpu_count()).  Returns (sweeps, last max|delta|)."""
        D = _f64(D)
        assert phi.dtype == np.float64 and phi.flags.c_contiguous
        h, w = D.shape
        mu = C.c_double(0)
        n = self.L.pcdo_poisson_solver_threads(D, phi, w, h, int(max_iterations), float(tol), int(max_threads),
                                               int(os.cpu_count() or 1), float(omega), C.byref(mu))
        return n, mu.value

    def sor_sweeps(self, D, phi, sweeps, omega=None):
        h, w = D.shape
        if omega is None:
            omega = 2.0 / (1.0 + 3.14159265 / w)
        return self.L.pcdo_sor_sweeps(_f64(D), phi, w, h, int(sweeps), float(omega))

    def residual(self, D, phi):
        """(r, ||r||2, ||b||2, max|r|) for the Neumann operator of solver.cpp:29-47."""
        D = _f64(D)
        h, w = D.shape
        r = np.empty_like(D)
        out = np.zeros(3)
        self.L.pcdo_residual(D, _f64(phi), w, h, r.ctypes.data, out)
        return r, out[0], out[1], out[2]

    def subtract_average(self, g):
        g = _f64(g).copy()
        self.L.pcdo_subtract_average(g, g.size)
        return g

    def gradient(self, g):
        g = _f64(g)
        h, w = g.shape
        gx, gy = np.empty_like(g), np.empty_like(g)
        self.L.pcdo_gradient(g, w, h, gx, gy)
        return gx, gy

    def divergence(self, nx, ny):
        nx, ny = _f64(nx), _f64(ny)
        h, w = nx.shape
        d = np.empty_like(nx)
        self.L.pcdo_divergence(nx, ny, w, h, d)
        return d

    def scale_proportional(self, g, lo=0.0, hi=1.0):
        g = _f64(g)
        out = np.empty_like(g)
        self.L.pcdo_scale_proportional(g, g.size, lo, hi, out)
        return out

    def resize_nearest(self, g, nw, nh):
        g = _f64(g)
        out = np.empty((nh, nw))
        self.L.pcdo_resize_nearest(g, g.shape[1], g.shape[0], out, nw, nh)
        return out

    def bilinear(self, g, x, y):
        g = _f64(g)
        return self.L.pcdo_bilinear(g, g.shape[1], g.shape[0], float(x), float(y))

    def mesh_points(self, nx, ny, width, height):
        p = np.empty((nx * ny, 3))
        self.L.pcdo_mesh_points(nx, ny, width, height, p)
        return p

    def dual_cell_areas(self, pts, nx, ny):
        a = np.empty(nx * ny)
        self.L.pcdo_dual_cell_areas(_f64(pts), nx, ny, a)
        return a

    def target_areas(self, pixels, width, height, pts, nx, ny):
        pixels = _f64(pixels)
        out = np.empty(nx * ny)
        self.L.pcdo_target_areas(pixels, pixels.shape[1], pixels.shape[0], width, height, _f64(pts), nx, ny, out)
        return out

    def raster(self, pts, vals, nx, ny, width, height, rx, ry):
        out = np.empty((ry, rx))
        miss = self.L.pcdo_raster(_f64(pts), _f64(vals), nx, ny, width, height, rx, ry, out)
        return out, miss

    def inverted_map(self, tgt, src, nx, ny, width, height):
        inv = np.empty((nx * ny, 2))
        miss = self.L.pcdo_inverted_map(_f64(tgt), _f64(src), nx, ny, width, height, inv)
        return inv, miss

    def refractive_normals(self, inv, src, focal, ri=1.49):
        n = src.shape[0]
        nx, ny = np.empty(n), np.empty(n)
        self.L.pcdo_refractive_normals(_f64(inv), _f64(src), n, focal, ri, nx, ny)
        return nx, ny

    def laplacian_smoothing(self, pts, nx, ny, factor):
        """Mesh::laplacian_smoothing, mesh.cpp:534-606 (returns a smoothed copy)."""
        p = _f64(pts).copy()
        self.L.pcdo_laplacian_smoothing(p, int(nx), int(ny), float(factor))
        return p

    def count_folds(self, pts, nx, ny):
        return int(self.L.pcdo_count_folds(_f64(pts), int(nx), int(ny)))

    def step_grid(self, tgt, vgx, vgy, nx, ny, width, step):
        return self.L.pcdo_step_grid(tgt, _f64(vgx), _f64(vgy), nx, ny, width, step)

    def sample_vertices(self, grid, pts, width, height):
        grid = _f64(grid)
        out = np.empty(pts.shape[0])
        self.L.pcdo_sample_vertices(grid, grid.shape[1], grid.shape[0], _f64(pts), pts.shape[0], width, height, out)
        return out

    def set_source_heights(self, src, hv):
        hv = _f64(hv).copy()
        return self.L.pcdo_set_source_heights(src, hv, hv.size)


class PortDesign:
    """Caustic_design iteration sequence composed from Port primitives.

    initialize_solvers caustic_design.cpp:334-364, perform_transport_iteration
    :190-266, perform_height_map_iteration :269-332.  The Poisson solves use the
    one-tile SOR of solver.cpp (bit-identical to the reference at max_threads=1).
    """

    def __init__(self, port: Port, mesh_res_x, mesh_res_y, res_x, res_y, width, height, focal_l, thickness):
        self.p = port
        self.nx, self.ny = mesh_res_x, mesh_res_y
        self.rx, self.ry = res_x, res_y
        self.width, self.height = width, height
        self.focal_l, self.thickness = focal_l, thickness

    def initialize(self, image):
        p = self.p
        self.pixels = p.scale_proportional(image, 0.0, 1.0)
        self.target_points = p.mesh_points(self.nx, self.ny, self.width, self.height)
        self.source_points = self.target_points.copy()
        self.target_areas = p.target_areas(self.pixels, self.width, self.height, self.target_points, self.nx, self.ny)
        self.phi = np.zeros((self.ry, self.rx))
        self.h = np.zeros((self.ry, self.rx))

    def transport_iteration(self, tol=1e-7, max_iterations=100000):
        p = self
        areas = self.p.dual_cell_areas(self.target_points, self.nx, self.ny)
        self.errors = (self.target_areas - areas) / areas
        raster, miss = self.p.raster(self.target_points, self.errors, self.nx, self.ny, self.width, self.height, self.rx, self.ry)
        if miss:
            raise RuntimeError(f"raster miss at {miss} samples")
        self.raster = self.p.subtract_average(raster)
        self.sweeps = self.p.poisson_solver(self.raster, self.phi, max_iterations, tol)[0]
        gx, gy = self.p.gradient(self.phi)
        self.vgx = self.p.sample_vertices(gx, self.target_points, self.width, self.height)
        self.vgy = self.p.sample_vertices(gy, self.target_points, self.width, self.height)
        # step_size is the float literal 0.05f (caustic_design.cpp:250)
        return self.p.step_grid(self.target_points, self.vgx, self.vgy, self.nx, self.ny, self.width,
                                float(np.float32(0.05)))

    def height_iteration(self, tol=1e-8, max_iterations=100000):
        inv, miss = self.p.inverted_map(self.target_points, self.source_points, self.nx, self.ny, self.width, self.height)
        if miss:
            raise RuntimeError(f"inverse map miss at {miss} vertices")
        focal = self.rx / self.width * self.focal_l          # caustic_design.cpp:271
        nxv, nyv = self.p.refractive_normals(inv, self.source_points, focal, 1.49)
        self.normals = (nxv, nyv)
        self.norm_x, m1 = self.p.raster(self.source_points, nxv, self.nx, self.ny, self.width, self.height, self.rx, self.ry)
        self.norm_y, m2 = self.p.raster(self.source_points, nyv, self.nx, self.ny, self.width, self.height, self.rx, self.ry)
        self.divergence = self.p.subtract_average(self.p.divergence(self.norm_x, self.norm_y))
        self.sweeps = self.p.poisson_solver(self.divergence, self.h, max_iterations, tol)[0]
        hv = self.p.sample_vertices(self.h, self.source_points, self.width, self.height)
        return self.p.set_source_heights(self.source_points, hv)


class Ref:
    """The reference's own compiled sources (oracle/_ref/libpcd_ref.so)."""

    def __init__(self, path: str = REF_SO):
        if not os.path.exists(path):
            build(ref=True)
        L = C.CDLL(path)
        self.L = L
        L.ref_poisson_solver.argtypes = [_dp, _dp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int]
        L.ref_subtract_average.argtypes = [_dp, C.c_int, C.c_int]
        L.ref_gradient.argtypes = [_dp, C.c_int, C.c_int, _dp, _dp]
        L.ref_divergence.argtypes = [_dp, _dp, C.c_int, C.c_int, _dp]
        L.ref_bilinear.argtypes = [_dp, C.c_int, C.c_int, C.c_double, C.c_double]
        L.ref_bilinear.restype = C.c_double
        L.ref_scale_proportional.argtypes = [_dp, C.c_int, C.c_int, C.c_double, C.c_double, _dp]
        L.ref_design_create.argtypes = [C.c_int] * 4 + [C.c_double] * 4 + [C.c_int]
        L.ref_design_create.restype = C.c_void_p
        L.ref_design_initialize.argtypes = [C.c_void_p, _dp]
        L.ref_design_transport.argtypes = [C.c_void_p]
        L.ref_design_transport.restype = C.c_double
        L.ref_design_height.argtypes = [C.c_void_p, C.c_int]
        L.ref_design_get.argtypes = [C.c_void_p, C.c_int, _dp]
        L.ref_design_get.restype = C.c_int
        L.ref_design_destroy.argtypes = [C.c_void_p]
        L.ref_save_solid_obj.argtypes = [_dp, _dp, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_char_p]
        L.ref_export_grid_svg.argtypes = [_dp, C.c_int, C.c_int, C.c_double, C.c_double, C.c_char_p, C.c_double]
        L.ref_laplacian_smoothing.argtypes = [_dp, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double]

    @staticmethod
    def available() -> bool:
        return os.path.exists(REF_SO) or os.path.isdir(os.path.join(REF_TREE, "src"))

    def save_solid_obj(self, front, back, nx, ny, thickness, width, height, filename):
        """save_solid_obj (utils.cpp:198-260) on the structured mesh's triangles."""
        self.L.ref_save_solid_obj(_f64(front), _f64(back), int(nx), int(ny), float(thickness), float(width),
                                  float(height), filename.encode())

    def laplacian_smoothing(self, pts, nx, ny, width, height, factor):
        """Mesh::laplacian_smoothing (mesh.cpp:534-606) of the reference (a smoothed copy)."""
        p = _f64(pts).copy()
        self.L.ref_laplacian_smoothing(p, int(nx), int(ny), float(width), float(height), float(factor))
        return p

    def export_grid_svg(self, pts, nx, ny, width, height, filename, stroke_width):
        """export_grid_to_svg (utils.cpp:262-307)."""
        self.L.ref_export_grid_svg(_f64(pts), int(nx), int(ny), float(width), float(height), filename.encode(),
                                   float(stroke_width))

    def poisson_solver(self, D, phi, max_iterations=100000, tol=1e-7, threads=1):
        h, w = D.shape
        self.L.ref_poisson_solver(_f64(D), phi, w, h, int(max_iterations), float(tol), int(threads))

    def subtract_average(self, g):
        g = _f64(g).copy()
        self.L.ref_subtract_average(g, g.shape[1], g.shape[0])
        return g

    def gradient(self, g):
        g = _f64(g)
        gx, gy = np.empty_like(g), np.empty_like(g)
        self.L.ref_gradient(g, g.shape[1], g.shape[0], gx, gy)
        return gx, gy

    def divergence(self, nx, ny):
        nx = _f64(nx)
        d = np.empty_like(nx)
        self.L.ref_divergence(nx, _f64(ny), nx.shape[1], nx.shape[0], d)
        return d

    def bilinear(self, g, x, y):
        g = _f64(g)
        return self.L.ref_bilinear(g, g.shape[1], g.shape[0], float(x), float(y))

    def scale_proportional(self, g, lo=0.0, hi=1.0):
        g = _f64(g)
        out = np.empty_like(g)
        self.L.ref_scale_proportional(g, g.shape[1], g.shape[0], lo, hi, out)
        return out


class RefDesign:
    """Caustic_design from the reference's compiled sources."""

    GRIDS = {"phi": 0, "h": 1, "raster": 2, "divergence": 3, "norm_x": 4, "norm_y": 5}
    VERTS = {"target_points": 10, "source_points": 11, "target_areas": 12, "errors": 13,
             "normals_x": 14, "normals_y": 15, "vertex_gradient_x": 16, "vertex_gradient_y": 17}

    def __init__(self, ref: Ref, mesh_res_x, mesh_res_y, res_x, res_y, width, height, focal_l, thickness, threads=1):
        self.r = ref
        self.nx, self.ny, self.rx, self.ry = mesh_res_x, mesh_res_y, res_x, res_y
        self.h = ref.L.ref_design_create(mesh_res_x, mesh_res_y, res_x, res_y, width, height, focal_l, thickness, threads)

    def initialize(self, image):
        self.r.L.ref_design_initialize(self.h, _f64(image))

    def transport_iteration(self):
        return self.r.L.ref_design_transport(self.h)

    def height_iteration(self, itr):
        self.r.L.ref_design_height(self.h, itr)

    def get(self, name):
        if name in self.GRIDS:
            out = np.empty((self.ry, self.rx))
            self.r.L.ref_design_get(self.h, self.GRIDS[name], out)
            return out
        n = self.nx * self.ny
        out = np.empty((n, 3)) if name.endswith("points") else np.empty(n)
        self.r.L.ref_design_get(self.h, self.VERTS[name], out)
        return out

    def close(self):
        if self.h:
            self.r.L.ref_design_destroy(self.h)
            self.h = None


def dct_solve(b: np.ndarray) -> np.ndarray:
    """Exact solve of  sum_nbr phi - cnt*phi = b  (Neumann graph Laplacian of
    solver.cpp:29-47, no NaN cells) by DCT-II diagonalisation; returns the
    mean-zero solution.  Eigenvalues 2cos(pi k/W) + 2cos(pi l/H) - 4."""
    from scipy.fft import dctn, idctn

    b = np.asarray(b, dtype=np.float64)
    h, w = b.shape
    bh = dctn(b - b.mean(), type=2, norm="ortho")
    lx = 2.0 * np.cos(np.pi * np.arange(w) / w) - 2.0
    ly = 2.0 * np.cos(np.pi * np.arange(h) / h) - 2.0
    lam = ly[:, None] + lx[None, :]
    lam[0, 0] = 1.0
    ph = bh / lam
    ph[0, 0] = 0.0
    return idctn(ph, type=2, norm="ortho")


def rel_err_mod_const(x: np.ndarray, ref: np.ndarray):
    """(relative L2, relative max) error of x against ref, both mean-removed."""
    x = np.asarray(x, np.float64) - np.mean(x)
    ref = np.asarray(ref, np.float64) - np.mean(ref)
    d = x - ref
    nr = np.linalg.norm(ref)
    return float(np.linalg.norm(d) / nr), float(np.abs(d).max() / np.abs(ref).max())


def heightmap_json_text(h) -> str:
    """save_heightmap_as_json, main.cpp:111-135 (main.cpp does not compile
    here: no png.h).  operator<< on a double with the stream's default
    precision prints like printf "%g" -- the same formatting the reference's
    compiled save_solid_obj uses for its vertices, which pins it."""
    h = np.asarray(h, dtype=np.float64)
    rows = []
    for i in range(h.shape[0]):
        rows.append("  [" + ", ".join("%g" % v for v in h[i]) + "]")
    return "[\n" + ",\n".join(rows) + ("\n" if rows else "") + "]\n"
