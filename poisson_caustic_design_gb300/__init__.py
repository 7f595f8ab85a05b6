"""GB300-native (sm_103a) Poisson caustic design.

The hot path of dylanmsu/poisson_caustic_design -- the grid Poisson solve and
the per-iteration mesh/grid steps of Caustic_design -- as hand-written CUDA
kernels behind a C ABI (include/pcd.h, libpcd_gb300.so), with host mirrors of
the reference's interfaces:

* ``poisson_solver`` -- src/solver.h:8
* ``CausticDesign`` -- class Caustic_design, src/caustic_design.h:7-66
"""
from . import inputs  # noqa: F401
from ._lib import PCDError  # noqa: F401
from .solver import (PREC_FP64, PREC_MIXED, SCHED_AUTO, SCHED_CLUSTER, SCHED_LAUNCHES,  # noqa: F401
                     SCHED_PERSISTENT, SCHED_STREAM, SCHED_STRIPES, SCHED_TILES, SCHED_BLOCKS,
                     STOP_MAX_UPDATE, STOP_REL_RESIDUAL, Context, SolveOptions, batch_solve, poisson_solver,
                     solver_progress)
from .caustic_design import (CausticDesign, export_grid_to_svg, height_iteration_batch,  # noqa: F401
                             initialize_batch, save_heightmap_as_json, save_solid_obj, transport_iteration_batch)
