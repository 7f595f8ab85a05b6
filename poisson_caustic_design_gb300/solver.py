"""Host-side mirror of the reference's Poisson solver interface.

``poisson_solver(D, phi, width, height, max_iterations, convergence_threshold,
max_threads)`` keeps the signature and in-place semantics of
``poisson_solver`` in src/solver.h:8 (src/solver.cpp:70-148): ``phi`` is the
initial guess and is overwritten; the solve stops when one sweep's max |delta|
drops below ``convergence_threshold`` or after ``max_iterations`` sweeps.
``Context`` exposes the library's explicit options (relative-residual stop,
mixed precision) on host arrays or on CUDA tensors.

Every call runs the CUDA kernels of libpcd_gb300; nothing here computes on the
CPU.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import (PREC_FP64, PREC_MIXED, SCHED_AUTO, SCHED_CLUSTER, SCHED_LAUNCHES, SCHED_PERSISTENT, SCHED_STREAM,
                   SCHED_STRIPES, SCHED_TILES, SCHED_BLOCKS, STOP_MAX_UPDATE,
                   STOP_REL_RESIDUAL, check)

__all__ = ["poisson_solver", "batch_solve", "solver_progress", "Context", "SolveOptions", "PREC_FP64", "PREC_MIXED",
           "STOP_MAX_UPDATE", "STOP_REL_RESIDUAL", "SCHED_AUTO", "SCHED_LAUNCHES", "SCHED_PERSISTENT",
           "SCHED_CLUSTER", "SCHED_STRIPES", "SCHED_STREAM", "SCHED_TILES", "SCHED_BLOCKS"]

# solver.h:10 declares `extern double solver_progress`; the reference never
# updates it (solver.cpp:9,63-68), so neither does this mirror.
solver_progress = 0.0


@dataclass
class SolveOptions:
    max_iterations: int = 100000
    tol: float = 1e-7
    stop: int = STOP_MAX_UPDATE
    precision: int = PREC_FP64
    omega: float = 0.0
    check_every: int = 0
    refine_every: int = 0
    warm_start: int = 1      # 0 zero, 1 phi is the initial guess, 2 learned prediction
    schedule: int = 0
    refine_drop: float = 0.0
    block_sweeps: int = 0

    def to_c(self) -> _lib.SolveOpts:
        o = _lib.SolveOpts()
        o.max_iterations = int(self.max_iterations)
        o.tol = float(self.tol)
        o.stop = int(self.stop)
        o.precision = int(self.precision)
        o.omega = float(self.omega)
        o.check_every = int(self.check_every)
        o.refine_every = int(self.refine_every)
        o.warm_start = int(self.warm_start)
        o.schedule = int(self.schedule)
        o.refine_drop = float(self.refine_drop)
        o.block_sweeps = int(self.block_sweeps)
        return o


def _as_grid(a, name):
    if not isinstance(a, np.ndarray) or a.dtype != np.float64 or a.ndim != 2 or not a.flags.c_contiguous:
        raise TypeError(f"{name} must be a C-contiguous 2-D float64 numpy array")
    return a


class Context:
    """A device context (stream + workspace) of libpcd_gb300."""

    def __init__(self, device: int = -1):
        L = _lib.load()
        h = C.c_void_p()
        check(L.pcd_ctx_create(int(device), C.byref(h)), "pcd_ctx_create")
        self._h = h
        self._L = L

    @property
    def handle(self):
        return self._h

    @property
    def stream(self) -> int:
        return int(self._L.pcd_ctx_stream(self._h) or 0)

    def close(self):
        if self._h:
            self._L.pcd_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_autotune(self, enable: bool = True) -> None:
        """Turn the context's autotuner on or off (pcd_ctx_set_autotune)."""
        check(self._L.pcd_ctx_set_autotune(self._h, 1 if enable else 0), "pcd_ctx_set_autotune")

    def autotune_info(self) -> dict:
        """Shapes tuned so far and trial solves run (pcd_ctx_autotune_info)."""
        e, t = C.c_int(0), C.c_longlong(0)
        check(self._L.pcd_ctx_autotune_info(self._h, C.byref(e), C.byref(t)), "pcd_ctx_autotune_info")
        return {"entries": e.value, "trials": t.value}

    def solve(self, b: np.ndarray, phi: np.ndarray, opts: SolveOptions | None = None, allow_not_converged=True):
        """Solve L phi = b on host arrays, in place on phi.  Returns stats dict."""
        _as_grid(b, "b")
        _as_grid(phi, "phi")
        if b.shape != phi.shape:
            raise ValueError("b and phi shapes differ")
        h, w = b.shape
        o = (opts or SolveOptions()).to_c()
        st = _lib.SolveStats()
        ok = (_lib.PCD_OK, _lib.PCD_NOT_CONVERGED) if allow_not_converged else (_lib.PCD_OK,)
        s = check(self._L.pcd_poisson_solve(self._h, b.ctypes.data, phi.ctypes.data, w, h, C.byref(o), C.byref(st)),
                  "pcd_poisson_solve", ok)
        d = st.as_dict()
        d["status"] = s
        return d

    def solve_device(self, b, phi, opts: SolveOptions | None = None, stream=None, allow_not_converged=True):
        """Solve on CUDA tensors (float64, 2-D, unit column stride), in place on phi."""
        import torch

        for t, n in ((b, "b"), (phi, "phi")):
            if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == torch.float64 and t.dim() == 2
                    and t.stride(1) == 1):
                raise TypeError(f"{n} must be a 2-D float64 CUDA tensor with unit column stride")
        if b.shape != phi.shape or b.stride(0) != phi.stride(0):
            raise ValueError("b and phi must share shape and row stride")
        h, w = b.shape
        o = (opts or SolveOptions()).to_c()
        st = _lib.SolveStats()
        if stream is None:
            stream = torch.cuda.current_stream(b.device).cuda_stream
        ok = (_lib.PCD_OK, _lib.PCD_NOT_CONVERGED) if allow_not_converged else (_lib.PCD_OK,)
        s = check(self._L.pcd_poisson_solve_device(self._h, b.data_ptr(), phi.data_ptr(), w, h, b.stride(0),
                                                   C.byref(o), C.byref(st), C.c_void_p(int(stream))),
                  "pcd_poisson_solve_device", ok)
        d = st.as_dict()
        d["status"] = s
        return d


def batch_solve(ctx: Context, bs, phis, opts: SolveOptions | None = None, stream=None):
    """Solve many independent grids (CUDA float64 tensors, 2-D, unit column
    stride, of any sizes) in one persistent launch.  Returns (per-instance
    stats, batch stats)."""
    import torch

    if len(bs) != len(phis) or not bs:
        raise ValueError("need equally many right-hand sides and solutions")
    arr = (_lib.Instance * len(bs))()
    for i, (b, p) in enumerate(zip(bs, phis)):
        if not (isinstance(b, torch.Tensor) and b.is_cuda and b.dtype == torch.float64 and b.dim() == 2
                and b.stride(1) == 1 and p.shape == b.shape and p.stride() == b.stride()):
            raise TypeError("instances must be 2-D float64 CUDA tensors with unit column stride, b and phi alike")
        arr[i].width, arr[i].height, arr[i].ld = b.shape[1], b.shape[0], b.stride(0)
        arr[i].b, arr[i].phi = b.data_ptr(), p.data_ptr()
    o = (opts or SolveOptions(stop=STOP_REL_RESIDUAL, tol=1e-6, omega=-1.0)).to_c()
    st = (_lib.InstanceStats * len(bs))()
    bst = _lib.BatchStats()
    if stream is None:
        stream = torch.cuda.current_stream(bs[0].device).cuda_stream
    L = _lib.load()
    s = check(L.pcd_batch_solve_device(ctx.handle, arr, len(bs), C.byref(o), st, C.byref(bst),
                                       C.c_void_p(int(stream))), "pcd_batch_solve_device",
              (_lib.PCD_OK, _lib.PCD_NOT_CONVERGED))
    per = [{k: getattr(x, k) for k, _ in x._fields_} for x in st]
    return per, {**{k: getattr(bst, k) for k, _ in bst._fields_}, "status": s}


def poisson_solver(D, phi, width: int, height: int, max_iterations: int, convergence_threshold: float,
                   max_threads: int = 1) -> None:
    """Drop-in for ``poisson_solver`` (src/solver.h:8).

    ``D`` and ``phi`` are height x width float64 arrays (``phi`` C-contiguous,
    updated in place).  ``max_threads`` is accepted and ignored.  Returns None
    like the reference; non-convergence is silent.
    """
    D = np.ascontiguousarray(D, dtype=np.float64)
    _as_grid(phi, "phi")
    if D.shape != (height, width) or phi.shape != (height, width):
        raise ValueError("D and phi must be height x width")
    L = _lib.load()
    check(L.pcd_poisson_solver(D.ctypes.data, phi.ctypes.data, int(width), int(height), int(max_iterations),
                               float(convergence_threshold), int(max_threads)),
          "pcd_poisson_solver", (_lib.PCD_OK, _lib.PCD_NOT_CONVERGED))
