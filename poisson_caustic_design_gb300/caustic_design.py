"""Host mirror of ``class Caustic_design`` (src/caustic_design.h:7-66).

Method names, argument meaning and call order follow the reference:

    d = CausticDesign()
    d.set_mesh_resolution(res, res)            # caustic_design.cpp:28-31
    d.set_domain_resolution(4*res, 4*res)      # :33-36
    d.set_mesh_size(width, height)             # :38-41
    d.set_lens_focal_length(focal)             # :43-45
    d.set_lens_thickness(thickness)            # :47-49
    d.set_solver_max_threads(n)                # :51-53 (accepted, ignored)
    d.initialize_solvers(image)                # :334-364
    step = d.perform_transport_iteration()     # :190-266
    d.perform_height_map_iteration(itr)        # :269-332

The state lives on the GPU (libpcd_gb300); the reference's public members
(``phi``, ``h``, ``raster``, ``errors``, ``mesh->target_points`` ...) are
read through properties that copy them to host arrays on access.  A raster
miss raises ``PCDError`` with status PCD_RASTER_MISS (the reference calls
exit(0), mesh.cpp:277-279).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import check
from .solver import Context, SolveOptions

GRID = {"phi": 0, "h": 1, "raster": 2, "divergence": 3, "norm_x": 4, "norm_y": 5, "pixels": 6, "gradient_x": 7,
        "gradient_y": 8}
VERT = {"target_points": 10, "source_points": 11, "target_areas": 12, "errors": 13, "normals_x": 14,
        "normals_y": 15, "vertex_gradient_x": 16, "vertex_gradient_y": 17, "inverted_map": 18, "cell_points": 19}


def dual_cells(points, nx, ny):
    """The barycentric dual cell of every vertex of the structured mesh
    (Mesh::build_target_partitioned_dual_cells, mesh.cpp:174-231): for each
    triangle around the vertex, the quad (v, mid(v, j), centroid(v, j, k),
    mid(v, k)) with j, k the triangle's next vertices (edge_centroid and
    triangle_centroid, mesh.cpp:154-172).  Triangles in the library's fixed
    order (the reference walks an unordered_set).  Returns one list of 4 x 3
    quads per vertex."""
    p = np.asarray(points, dtype=np.float64)
    cells = []
    cx = nx - 1
    for i in range(ny):
        for j in range(nx):
            tris = []
            if i < ny - 1 and j < nx - 1:
                tris.append((2 * (i * cx + j), 0))
            if i < ny - 1 and j > 0:
                tris += [(2 * (i * cx + j - 1), 1), (2 * (i * cx + j - 1) + 1, 1)]
            if i > 0 and j < nx - 1:
                tris += [(2 * ((i - 1) * cx + j), 2), (2 * ((i - 1) * cx + j) + 1, 0)]
            if i > 0 and j > 0:
                tris.append((2 * ((i - 1) * cx + j - 1) + 1, 2))
            quads = []
            for t, pos in tris:
                c = t >> 1
                base = (c // cx) * nx + c % cx
                v = (base, base + 1, base + nx) if t % 2 == 0 else (base + nx, base + 1, base + nx + 1)
                a, b, d = p[v[pos]], p[v[(pos + 1) % 3]], p[v[(pos + 2) % 3]]
                quads.append(np.array([a, (a + b) / 2.0, (a + b + d) / 3.0, (a + d) / 2.0]))
            cells.append(quads)
    return cells


class CausticDesign:
    def __init__(self, ctx: Context | None = None, transport: SolveOptions | None = None,
                 height_solve: SolveOptions | None = None, raster_miss_policy: int = 0):
        self._L = _lib.load()
        self._ctx = ctx or Context()
        self._own_ctx = ctx is None
        self._h = None
        self.mesh_res_x = self.mesh_res_y = 0
        self.resolution_x = self.resolution_y = 0
        self.width = self.height = 0.0
        self.focal_l = self.thickness = 0.0
        self.nthreads = 0
        self.transport_opts = transport or SolveOptions(tol=1e-7)      # caustic_design.cpp:222
        self.height_opts = height_solve or SolveOptions(tol=1e-8)      # caustic_design.cpp:311
        self.last_solve_stats = None
        # 0: a raster miss raises PCDError (PCD_RASTER_MISS; the reference
        # exits); 1: the target mesh is smoothed and the iteration returns NaN
        self.raster_miss_policy = int(raster_miss_policy)
        self.last_status = None

    # ---- setters (caustic_design.cpp:28-53) ----
    def set_mesh_resolution(self, width: int, height: int):
        self.mesh_res_x, self.mesh_res_y = int(width), int(height)

    def set_domain_resolution(self, width: int, height: int):
        self.resolution_x, self.resolution_y = int(width), int(height)

    def set_mesh_size(self, width: float, height: float):
        self.width, self.height = float(width), float(height)

    def set_lens_focal_length(self, focal_length: float):
        self.focal_l = float(focal_length)

    def set_lens_thickness(self, thickness: float):
        self.thickness = float(thickness)

    def set_solver_max_threads(self, n_threads: int):
        self.nthreads = int(n_threads)

    # ---- iterations ----
    def initialize_solvers(self, image):
        img = self._create(image)
        check(self._L.pcd_design_initialize(self._h, img.ctypes.data), "pcd_design_initialize")

    def _create(self, image):
        """The device design for the current settings (before initialisation);
        returns the image as a contiguous float64 array."""
        img = np.ascontiguousarray(image, dtype=np.float64)
        if img.shape != (self.resolution_y, self.resolution_x):
            raise ValueError(f"image must be resolution_y x resolution_x = {(self.resolution_y, self.resolution_x)}")
        self.close()
        p = _lib.DesignParams()
        self._L.pcd_design_params_default(C.byref(p))
        p.mesh_res_x, p.mesh_res_y = self.mesh_res_x, self.mesh_res_y
        p.res_x, p.res_y = self.resolution_x, self.resolution_y
        p.width, p.height = self.width, self.height
        p.focal_l, p.thickness = self.focal_l, self.thickness
        p.transport = self.transport_opts.to_c()
        p.height_solve = self.height_opts.to_c()
        p.raster_miss_policy = self.raster_miss_policy
        h = C.c_void_p()
        check(self._L.pcd_design_create(self._ctx.handle, C.byref(p), C.byref(h)), "pcd_design_create")
        self._h = h
        return img

    def perform_transport_iteration(self) -> float:
        """Returns the step size; NaN when a raster miss was handled by
        smoothing the target mesh (raster_miss_policy 1, status in
        ``last_status``), as caustic_design.cpp:214-217 intends."""
        step = C.c_double(0)
        st = _lib.SolveStats()
        self.last_status = check(self._L.pcd_design_transport_iteration(self._h, C.byref(step), C.byref(st)),
                                 "pcd_design_transport_iteration", (_lib.PCD_OK, _lib.PCD_MESH_SMOOTHED))
        self.last_solve_stats = st.as_dict()
        return step.value

    # ---- fold handling ----
    def smooth_target_mesh(self, smoothing_factor: float):
        """Mesh::laplacian_smoothing (mesh.cpp:534-606) of the target mesh."""
        check(self._L.pcd_design_smooth_target_mesh(self._h, float(smoothing_factor)), "smooth_target_mesh")

    def count_folds(self) -> int:
        """Triangles of the target mesh with non-positive signed area."""
        n = C.c_longlong(0)
        check(self._L.pcd_design_count_folds(self._h, C.byref(n)), "count_folds")
        return n.value

    def set_target_points(self, points):
        p = np.ascontiguousarray(points, dtype=np.float64)
        if p.shape != (self.mesh_res_x * self.mesh_res_y, 3):
            raise ValueError("points must be mesh_res_x * mesh_res_y x 3")
        check(self._L.pcd_design_set_target_points(self._h, p.ctypes.data_as(C.POINTER(C.c_double))),
              "set_target_points")

    def perform_height_map_iteration(self, itr: int = 0) -> float:
        upd = C.c_double(0)
        st = _lib.SolveStats()
        check(self._L.pcd_design_height_iteration(self._h, int(itr), C.byref(upd), C.byref(st)),
              "pcd_design_height_iteration")
        self.last_solve_stats = st.as_dict()
        return upd.value

    # ---- output files (caustic_design.cpp:20-26,55-61) ----
    def save_solid_obj_target(self, filename: str):
        check(self._L.pcd_design_save_solid_obj(self._h, 1, filename.encode()), "save_solid_obj_target")

    def save_solid_obj_source(self, filename: str):
        check(self._L.pcd_design_save_solid_obj(self._h, 0, filename.encode()), "save_solid_obj_source")

    def export_paramererization_to_svg(self, filename: str, line_width: float):
        check(self._L.pcd_design_export_parameterization_svg(self._h, filename.encode(), float(line_width)),
              "export_paramererization_to_svg")

    def export_inverted_transport_map(self, filename: str, stroke_width: float):
        check(self._L.pcd_design_export_inverted_transport_map_svg(self._h, filename.encode(), float(stroke_width)),
              "export_inverted_transport_map")

    # ---- public members (caustic_design.h:16-30, mesh.h:51-52) ----
    def _grid(self, name):
        out = np.empty((self.resolution_y, self.resolution_x))
        check(self._L.pcd_design_get_grid(self._h, GRID[name], out.ctypes.data), "pcd_design_get_grid")
        return out

    _POINT_FIELDS = ("target_points", "source_points", "inverted_map", "cell_points")  # n x 3

    def _vert(self, name):
        n = self.mesh_res_x * self.mesh_res_y
        out = np.empty((n, 3)) if name in self._POINT_FIELDS else np.empty(n)
        check(self._L.pcd_design_get_vertices(self._h, VERT[name], out.ctypes.data), "pcd_design_get_vertices")
        return out

    phi = property(lambda self: self._grid("phi"))
    h = property(lambda self: self._grid("h"))
    raster = property(lambda self: self._grid("raster"))
    divergence = property(lambda self: self._grid("divergence"))
    norm_x = property(lambda self: self._grid("norm_x"))
    norm_y = property(lambda self: self._grid("norm_y"))
    errors = property(lambda self: self._vert("errors"))
    target_areas = property(lambda self: self._vert("target_areas"))

    @property
    def vertex_gradient(self):
        return [self._vert("vertex_gradient_x"), self._vert("vertex_gradient_y")]

    @property
    def normals(self):
        return [self._vert("normals_x"), self._vert("normals_y")]

    pixels = property(lambda self: self._grid("pixels"))

    @property
    def gradient(self):
        """calculate_gradient(phi) (caustic_design.cpp:225): [d/dx, d/dy] grids."""
        return [self._grid("gradient_x"), self._grid("gradient_y")]

    def target_cells(self):
        """The dual cells of the target mesh that the last transport iteration
        (or the initialisation) built (caustic_design.cpp:195-196,343-344)."""
        return dual_cells(self._vert("cell_points"), self.mesh_res_x, self.mesh_res_y)

    # never filled by the reference (caustic_design.cpp reads it only in
    # commented-out code): an empty list, as there
    first_target_cells = property(lambda self: [])

    def target_points(self):
        return self._vert("target_points")

    def source_points(self):
        return self._vert("source_points")

    def inverted_map(self):
        """The inverted transport map of the current target mesh (mesh.cpp:348-409), n x 3 with z = 0."""
        return self._vert("inverted_map")

    def close(self):
        if self._h:
            self._L.pcd_design_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
            if self._own_ctx:
                self._ctx.close()
        except Exception:
            pass


# ---- writers from host arrays (utils.cpp:198-307, main.cpp:111-135) ----
def _pts(a, n):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if a.shape != (n, 3):
        raise ValueError(f"points must be {n} x 3")
    return a


def save_solid_obj(front_points, back_points, res_x: int, res_y: int, thickness: float, width: float, height: float,
                   filename: str) -> None:
    """save_solid_obj (utils.cpp:198-260) on the structured mesh's triangles."""
    n = int(res_x) * int(res_y)
    f, b = _pts(front_points, n), _pts(back_points, n)
    L = _lib.load()
    check(L.pcd_write_solid_obj(f.ctypes.data_as(C.POINTER(C.c_double)), b.ctypes.data_as(C.POINTER(C.c_double)),
                                int(res_x), int(res_y), float(thickness), float(width), float(height),
                                filename.encode()), "pcd_write_solid_obj")


def export_grid_to_svg(points, width: float, height: float, res_x: int, res_y: int, filename: str,
                       stroke_width: float) -> None:
    """export_grid_to_svg (utils.cpp:262-307)."""
    p = _pts(points, int(res_x) * int(res_y))
    L = _lib.load()
    check(L.pcd_write_grid_svg(p.ctypes.data_as(C.POINTER(C.c_double)), int(res_x), int(res_y), float(width),
                               float(height), filename.encode(), float(stroke_width)), "pcd_write_grid_svg")


def save_heightmap_as_json(heightmap, filename: str) -> None:
    """save_heightmap_as_json (main.cpp:111-135)."""
    h = np.ascontiguousarray(heightmap, dtype=np.float64)
    if h.ndim != 2:
        raise ValueError("heightmap must be 2-D")
    L = _lib.load()
    check(L.pcd_write_heightmap_json(h.ctypes.data_as(C.POINTER(C.c_double)), h.shape[1], h.shape[0],
                                     filename.encode()), "pcd_write_heightmap_json")


# ---- batched designs (no counterpart in the reference) ----------------------
# The same step on many designs at once: each design runs on a host thread of
# its own inside the library and its work stays on its context's stream, so
# designs created on distinct contexts overlap on the GPU.

def _handles(designs):
    return (C.c_void_p * len(designs))(*[d._h.value for d in designs])


def initialize_batch(designs, images):
    """initialize_solvers on every design at once (images[i] for designs[i])."""
    imgs = [d._create(im) for d, im in zip(designs, images)]
    n = len(designs)
    ptrs = (C.c_void_p * n)(*[im.ctypes.data for im in imgs])
    L = _lib.load()
    check(L.pcd_design_initialize_batch(_handles(designs), n, ptrs, (C.c_int * n)()), "pcd_design_initialize_batch")


def transport_iteration_batch(designs):
    """perform_transport_iteration on every design at once; returns the step
    sizes (each design's solve statistics go to its ``last_solve_stats``)."""
    n = len(designs)
    steps = np.zeros(n)
    st = (_lib.SolveStats * n)()
    codes = (C.c_int * n)()
    L = _lib.load()
    check(L.pcd_design_transport_iteration_batch(_handles(designs), n, steps.ctypes.data_as(_lib._dp), st, codes),
          "pcd_design_transport_iteration_batch")
    for d, s, c in zip(designs, st, codes):
        d.last_solve_stats = s.as_dict()
        d.last_status = int(c)
    return steps


def height_iteration_batch(designs, itr: int):
    """perform_height_map_iteration(itr) on every design at once; returns the
    height updates."""
    n = len(designs)
    upd = np.zeros(n)
    st = (_lib.SolveStats * n)()
    codes = (C.c_int * n)()
    L = _lib.load()
    check(L.pcd_design_height_iteration_batch(_handles(designs), n, int(itr), upd.ctypes.data_as(_lib._dp), st,
                                              codes), "pcd_design_height_iteration_batch")
    for d, s, c in zip(designs, st, codes):
        d.last_solve_stats = s.as_dict()
        d.last_status = int(c)
    return upd
