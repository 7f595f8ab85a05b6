"""Benchmark of the GB300 Poisson solve (the caustic-design hot path).

Workload (the single-solve configuration): one 512 x 512 Poisson solve of the
reference's Neumann operator, b = seeded target density - 1 (16-Gaussian
mixtures and binary disk/rectangle fields alternating, mean removed in FP64),
to a relative FP64 residual ||b - L phi|| / ||b|| <= 1e-6.  A step is one
such solve of one instance.  The headline form is the learned warm start
(the committed 64^2 U-Net weights) + FP32 sweeps with FP64 defect correction;
the mixed form from a zero guess and the plain FP64 form are timed beside it.
The context's autotuner picks each form's settings during the warm-up.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--no-cpu-baseline] [--no-batch] [--headline-only] [--no-autotune]

Prints one JSON line.  `value` = wall time per solve (ms, lower is better)
with b resident in HBM, measured with CUDA events on the launching stream;
the L2 is flushed (a 512 MiB write) before every timed solve.  `e2e` = the
same metric through the host-array C ABI (pcd_poisson_solve: pinned host b in,
host phi out, copies inside the timed region).  `--impl reference` times the
reference's CPU solver (its tile-threaded SOR schedule, restated in C under
oracle/ because the reference tree is not present on the GPU host) on all host
cores for the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_GRID = 512
TOL = 1e-6
METRIC = "OT solve wall-time to residual 1e-6 at 512²: learned+mixed vs plain GPU"
UNIT = "ms/solve"
SEEDS = [(s, "gaussian" if s % 2 == 0 else "binary") for s in range(8)]
# DRAM bytes (read + write) of one k_sor_cluster_rr launch of the autotuned
# headline solve, ncu (profiles/k_sor_cluster_rr_512_autotuned.md)
CLUSTER_DRAM_BYTES_PER_LAUNCH = 2.183e6
# FP64 operations per cell-sweep of the block schedule's update and the
# measured FP64 FMA rate of this part (dependent-free FMA loop, all SMs)
FP64_OPS_PER_CELL = 5
FP64_OPS_PER_S = 0.60e12


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cpu-budget-s", type=float, default=20.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-pipelines", action="store_true",
                    help="skip the full-pipeline sections (mesh 128 and mesh 1024 designs)")
    ap.add_argument("--headline-only", action="store_true",
                    help="time only the headline form (skips the other forms, the accuracy and end-to-end "
                         "sections, the batch and the 4096^2 sections): for profiling the headline step")
    ap.add_argument("--no-autotune", action="store_true", help="solve with the schedules' default settings")
    ap.add_argument("--stream-only", action="store_true",
                    help="only the 4096^2 sweep-roofline section (for profiling the stream kernel)")
    ap.add_argument("--batch-only", action="store_true",
                    help="one solve of the 64-grid batch and nothing else (for profiling the batched kernels)")
    ap.add_argument("--config4", action="store_true",
                    help="instead of the headline: the full caustic pipeline at a 1024^2 mesh on 4096^2 grids "
                         "(transport and height iterations, plain FP64 and mixed), one JSON line")
    ap.add_argument("--pipeline-profile", action="store_true",
                    help="one caustic design at the 1024^2-mesh / 4096^2-grid size: initialisation, one transport "
                         "and one height iteration with the solves capped at 8 sweeps (for profiling the "
                         "pipeline kernels), per-step device times as one JSON line")
    ap.add_argument("--cpu-sample", type=float, default=None, metavar="BUDGET_S",
                    help="internal: time the reference's CPU solver on the eight densities in this fresh process "
                         "(per-solve budget BUDGET_S) and print one JSON object")
    ap.add_argument("--cpu-omega", choices=["reference", "neumann"], default="reference",
                    help="internal, with --cpu-sample: the reference's omega or the Neumann-optimal one")
    ap.add_argument("--cpu-what", choices=["solve", "config0", "config4"], default="solve",
                    help="internal, with --cpu-sample: the single solves, the full-pipeline workload's first "
                         "transport iteration, or the 4096^2 per-sweep time")
    return ap.parse_args()


def dist_setup(n):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
        pg = dist
    return rank, world, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def max_over_ranks(pg, x):
    if pg is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None
        self.th = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        self.th = threading.Thread(target=self._read, daemon=True)
        self.th.start()

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.th:
            self.th.join(timeout=2)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                smax = float(r[2])
                for k, name in enumerate(names):
                    if r[5 + k].lower().startswith("active"):
                        reasons.add(name)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def instances():
    from poisson_caustic_design_gb300 import inputs

    return [inputs.poisson_rhs(N_GRID, s, k) for s, k in SEEDS]


# ---------------------------------------------------------------------------
def exact_solve(b):
    """The FP64 solution of the reference operator (Neumann graph Laplacian,
    solver.cpp:29-47) to machine precision: DCT-II diagonalisation with the
    eigenvalues 2 cos(pi k / W) + 2 cos(pi l / H) - 4, mean-zero (the accuracy
    yardstick of every timed form, computed on the host outside the timed
    region)."""
    from scipy.fft import dctn, idctn

    h, w = b.shape
    bh = dctn(b - b.mean(), type=2, norm="ortho")
    lam = (2.0 * np.cos(np.pi * np.arange(h) / h) - 2.0)[:, None] + (2.0 * np.cos(np.pi * np.arange(w) / w) - 2.0)
    lam[0, 0] = 1.0
    ph = bh / lam
    ph[0, 0] = 0.0
    return idctn(ph, type=2, norm="ortho")


def err_mod_const(x, ref):
    """(relative L2, relative max) error of x against ref, both mean-removed."""
    x = x - x.mean()
    ref = ref - ref.mean()
    d = x - ref
    return float(np.linalg.norm(d) / np.linalg.norm(ref)), float(np.abs(d).max() / np.abs(ref).max())


def neumann_omega(n):
    """The optimal SOR factor of the Neumann operator on an n x n grid (the
    GPU forms' omega): 2 / (1 + sin t) with cos t = (1 + cos(pi / n)) / 2."""
    mu = 0.5 * (1.0 + np.cos(np.pi / n))
    return 2.0 / (1.0 + np.sqrt(1.0 - mu * mu))


def cpu_reference_solve(port, b, threads, budget_s, chunk=25, omega=0.0):
    """The reference's solver on the host: chunks of `chunk` sweeps of its
    tile-threaded SOR (poisson_solver(b, phi, W, H, chunk, 0.0, T) warm-started
    in place; omega 0 = the reference's 2/(1+pi/W)), relative residual checked
    between chunks outside the timed region.  Returns (ms to tolerance or
    extrapolated, sweeps, rel, extrapolated)."""
    phi = np.zeros_like(b)
    t_solve = 0.0
    sweeps = 0
    rel = 1.0
    hist = []
    while True:
        t = time.perf_counter()
        port.poisson_solver_threads(b, phi, chunk, 0.0, threads, omega)
        t_solve += time.perf_counter() - t
        sweeps += chunk
        _, rn, bn, _ = port.residual(b, phi)
        rel = rn / bn
        hist.append((sweeps, rel, t_solve))
        if rel <= TOL:
            return t_solve * 1e3, sweeps, rel, False
        if t_solve > budget_s and len(hist) >= 4:
            # extrapolate with the last chunks' geometric rate
            (s0, r0, t0), (s1, r1, t1) = hist[len(hist) // 2], hist[-1]
            rate = (np.log(r1) - np.log(r0)) / (s1 - s0)
            more = (np.log(TOL) - np.log(r1)) / rate if rate < 0 else float("inf")
            per_sweep = (t1 - t0) / (s1 - s0)
            return (t_solve + more * per_sweep) * 1e3, sweeps + int(more), rel, True


def cpu_sample(budget_s, omega_kind="reference", seeds=None):
    """The reference's threaded CPU solver on the workload's densities (all
    eight by default), one solve each, in the calling process: mean ms per
    solve, sweeps per solve, and whether a solve was extrapolated."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    oracle.build(ref=False)
    port = oracle.Port()
    threads = os.cpu_count() or 1
    seg = int(np.floor(np.sqrt(threads)))
    omega = neumann_omega(N_GRID) if omega_kind == "neumann" else 0.0
    bs = instances()
    per = []
    for k in (seeds if seeds is not None else range(len(bs))):
        ms, sweeps, rel, ex = cpu_reference_solve(port, bs[k], threads, budget_s, omega=omega)
        per.append({"seed": SEEDS[k][0], "kind": SEEDS[k][1], "ms": ms, "sweeps": sweeps, "extrapolated": ex})
    return {"ms": float(np.mean([p["ms"] for p in per])), "sweeps": float(np.mean([p["sweeps"] for p in per])),
            "extrapolated": any(p["extrapolated"] for p in per), "threads": seg * seg, "omega": omega_kind,
            "per_solve": per}


def cpu_pipeline_sample(what):
    """The reference's pipeline on the host with its threaded solver: config0
    = initialisation and first transport iteration of the 128^2-mesh design
    (the C port of caustic_design.cpp:190-266,334-364; the reference's own
    1e-7 max-update solve on all host threads); config4 = the threaded SOR's
    time per sweep on a 4096^2 grid."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    from poisson_caustic_design_gb300 import inputs

    oracle.build(ref=False)
    port = oracle.Port()
    threads = os.cpu_count() or 1
    seg = int(np.floor(np.sqrt(threads)))
    if what == "config4":
        b = inputs.poisson_rhs(4096, 3, "gaussian")
        phi = np.zeros_like(b)
        port.poisson_solver_threads(b, phi, 2, 0.0, threads)
        t = time.perf_counter()
        port.poisson_solver_threads(b, phi, 6, 0.0, threads)
        return {"per_sweep_ms": (time.perf_counter() - t) / 6 * 1e3, "threads": seg * seg}

    class Threaded(oracle.Port):
        def poisson_solver(self, D, phi, max_iterations=100000, tol=1e-7):
            return self.poisson_solver_threads(D, phi, max_iterations, tol, threads)

    d = oracle.PortDesign(Threaded(), 128, 128, 512, 512, 0.5, 0.5, 1.5, 0.1)
    t = time.perf_counter()
    d.initialize(inputs.pipeline_image(128, 47))
    t_init = time.perf_counter() - t
    t = time.perf_counter()
    step = d.transport_iteration()
    return {"init_ms": t_init * 1e3, "first_transport_ms": (time.perf_counter() - t) * 1e3, "step": step,
            "sweeps": d.sweeps, "threads": seg * seg}


def cpu_sample_subprocess(budget_s, omega_kind="reference", what="solve"):
    """cpu_sample (or cpu_pipeline_sample) in a fresh interpreter: no CUDA
    context and no runtime threads of this process compete with the solver's
    fork-join threads."""
    env = {**os.environ, "WORLD_SIZE": "1", "RANK": "0"}
    r = subprocess.run([sys.executable, os.path.abspath(__file__), "--cpu-sample", str(budget_s), "--cpu-omega",
                        omega_kind, "--cpu-what", what], capture_output=True, text=True, env=env)
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    if r.returncode != 0 or not lines:
        raise RuntimeError(f"CPU baseline subprocess failed ({r.returncode}): {r.stderr[-500:]}")
    return json.loads(lines[-1])


def run_reference(args, rank, world, pg):
    """--impl reference: rank 0 times the reference's CPU solver."""
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    oracle.build(ref=False)
    port = oracle.Port()
    threads = os.cpu_count() or 1
    seg = int(np.floor(np.sqrt(threads)))
    bs = instances()
    budget = max(2.0, min(args.cpu_budget_s, 150.0 / max(1, args.steps + args.warmup)))
    for w in range(args.warmup):
        cpu_reference_solve(port, bs[w % len(bs)], threads, budget)
    times, sweeps_l, extrap = [], [], False
    for k in range(args.steps):
        ms, sweeps, rel, ex = cpu_reference_solve(port, bs[k % len(bs)], threads, budget)
        times.append(ms)
        sweeps_l.append(sweeps)
        extrap |= ex
    v = float(np.mean(times))
    # the same solver with the Neumann-optimal omega that the GPU forms use:
    # splits the GPU/CPU ratio into the omega (algorithm) and the hardware
    neu = cpu_sample(budget, "neumann")
    sample = (f"{args.steps} solves of 512x512 (Gaussian/binary RHS) to rel residual 1e-6, tile-threaded "
              f"lexicographic SOR with the reference's omega on {seg * seg} tile threads; chunks of 25 sweeps, "
              f"residual checks outside the timed region" + ("; slow solves extrapolated from the chunk rate"
                                                            if extrap else ""))
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": v, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded densities)",
        "config": {"workload": "single 512x512 Neumann Poisson solve to rel residual 1e-6", "grid": N_GRID,
                   "tol": TOL, "l2": "host CPU run"},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": seg * seg, "kind": "port", "sample": sample},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "sweeps_per_solve": float(np.mean(sweeps_l)),
        "neumann_omega_variant": {"ms_per_solve": neu["ms"], "sweeps_per_solve": neu["sweeps"],
                                  "extrapolated": neu["extrapolated"],
                                  "note": "the same CPU solver on the eight densities with the Neumann-optimal "
                                          "omega of the GPU forms (not the reference's own omega)"},
    }
    print(json.dumps(line), flush=True)


def batch_instances(pcd):
    """The 64-grid batch: sides drawn from {64, 96, 128, 256, 512, 1024}
    (seed 2024), seeded Gaussian densities, on the current CUDA device."""
    rs = np.random.default_rng(2024)
    sizes = [int(rs.choice([64, 96, 128, 256, 512, 1024])) for _ in range(64)]
    return sizes, [pcd.inputs.poisson_rhs_torch(n_, [5000 + i])[0].contiguous() for i, n_ in enumerate(sizes)]


def stream_section(ctx, stream, peak):
    """Sweep rates on 4096^2, 256 sweeps per solve: FP32 stream passes and
    FP32 register-resident tile passes (12 B algorithmic per cell-sweep; the
    tile passes move about a quarter of that per sweep, four sweeps per pass),
    FP64 in-place stripes (24 B)."""
    import torch

    import poisson_caustic_design_gb300 as pcd

    n4 = 4096
    b4 = pcd.inputs.poisson_rhs_torch(n4, [77])[0].contiguous()
    p4 = torch.zeros_like(b4)
    out = {}
    for prec, bpc, nm, sch in ((pcd.PREC_MIXED, 12, "fp32_sweeps", pcd.SCHED_STREAM),
                               (pcd.PREC_MIXED, 12, "fp32_tiles", pcd.SCHED_TILES),
                               (pcd.PREC_FP64, 24, "fp64_sweeps", pcd.SCHED_STRIPES)):
        o4 = pcd.SolveOptions(stop=pcd.STOP_REL_RESIDUAL, tol=0.0, max_iterations=256, omega=-1.0, precision=prec,
                              warm_start=0, schedule=sch, refine_every=256)
        ctx.solve_device(b4, p4, o4, stream=stream.cuda_stream)
        st4 = ctx.solve_device(b4, p4, o4, stream=stream.cuda_stream)
        per_sweep = st4["sweep_ms"] * 1e-3 / st4["sweeps"]
        ach = bpc * n4 * n4 / per_sweep / 1e9
        out[nm] = {"us_per_sweep": per_sweep * 1e6, "achieved_gbs": ach, "frac_hbm": ach / peak,
                   "schedule": int(st4["schedule_used"])}
    return out


def _design(pcd, ctx, R, N, transport=None, height=None):
    d = pcd.CausticDesign(ctx, transport=transport, height_solve=height)
    d.set_mesh_resolution(R, R)
    d.set_domain_resolution(N, N)
    d.set_mesh_size(0.5, 0.5)
    d.set_lens_focal_length(1.5)
    d.set_lens_thickness(0.1)
    return d


def config0_section(pcd, ctx, device, batch=16):
    """The full-pipeline workload: mesh 128^2 on 512^2 grids, width 0.5,
    focal length 1.5, thickness 0.1, conv 0.01 (the reference's main.cpp
    sequence: transport iterations until the step falls below conv, then 3
    height iterations) on the seeded target of the committed reference golden
    (tests/golden/pipeline_r128.npz, written by the reference's own compiled
    Caustic_design).  Plain FP64 with the reference's solves (max |delta| <
    1e-7 / 1e-8, its omega) and mixed precision with the same stops; the plain
    form's final points and heights against the reference's; then `batch`
    designs of different targets as one batch of contexts."""
    import torch

    z = np.load(os.path.join(ROOT, "tests", "golden", "pipeline_r128.npz"))
    R, conv, seed = int(z["params"][0]), float(z["params"][4]), int(z["params"][5])
    N = 4 * R
    out = {"mesh": R, "grid": N, "conv": conv, "forms": {}}
    for name, prec in (("plain_fp64", pcd.PREC_FP64), ("mixed", pcd.PREC_MIXED)):
        d = _design(pcd, ctx, R, N, pcd.SolveOptions(tol=1e-7, precision=prec),
                    pcd.SolveOptions(tol=1e-8, precision=prec))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        d.initialize_solvers(pcd.inputs.pipeline_image(R, seed))
        t1 = time.perf_counter()
        steps, sweeps, first = [], 0, None
        for _ in range(50):
            steps.append(d.perform_transport_iteration())
            sweeps += d.last_solve_stats["sweeps"]
            if first is None:
                torch.cuda.synchronize()
                first = (time.perf_counter() - t1) * 1e3
            if steps[-1] < conv:
                break
        t2 = time.perf_counter()
        for itr in range(3):
            d.perform_height_map_iteration(itr)
        torch.cuda.synchronize()
        t3 = time.perf_counter()
        tp, sp = d.target_points(), d.source_points()
        zr, zt = z["source_points"][:, 2], z["target_points"]
        rec = {"total_ms": (t3 - t0) * 1e3, "init_ms": (t1 - t0) * 1e3, "transport_ms": (t2 - t1) * 1e3,
               "height_ms": (t3 - t2) * 1e3, "first_transport_ms": first, "transport_iterations": len(steps),
               "reference_transport_iterations": len(z["steps"]), "transport_sweeps": sweeps,
               "target_points_rel_l2_vs_reference": float(np.linalg.norm(tp - zt) / np.linalg.norm(zt)),
               "target_points_max_abs_vs_reference": float(np.abs(tp - zt).max()),
               "vertex_heights_rel_l2_vs_reference": float(np.linalg.norm(sp[:, 2] - zr) / np.linalg.norm(zr))}
        out["forms"][name] = rec
        d.close()
    # `batch` targets (seeds 0..batch-1) through the whole pipeline as
    # lock-step batches (one context; each step's solves of all targets in one
    # batched solve) against the same targets one after the other, both with
    # mixed-precision relative-residual solves (1e-9 transport, 1e-10 height:
    # the accuracy the reference's own stop reaches at this size)
    tr = pcd.SolveOptions(stop=pcd.STOP_REL_RESIDUAL, tol=1e-9, precision=pcd.PREC_MIXED, omega=-1.0,
                          max_iterations=200000)
    hs = pcd.SolveOptions(stop=pcd.STOP_REL_RESIDUAL, tol=1e-10, precision=pcd.PREC_MIXED, omega=-1.0,
                          max_iterations=200000)
    imgs = [pcd.inputs.pipeline_image(R, s) for s in range(batch)]

    def run(ds, batched):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rounds = 0
        if batched:
            pcd.initialize_batch(ds, imgs)
            live = list(ds)
            while live and rounds < 50:
                st = pcd.transport_iteration_batch(live)
                rounds += 1
                live = [d for d, x in zip(live, st) if not x < conv]
            for itr in range(3):
                pcd.height_iteration_batch(ds, itr)
        else:
            for d, im in zip(ds, imgs):
                d.initialize_solvers(im)
                for _ in range(50):
                    rounds += 1
                    if d.perform_transport_iteration() < conv:
                        break
                for itr in range(3):
                    d.perform_height_map_iteration(itr)
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) * 1e3, rounds

    shared = pcd.Context(device)
    ds = [_design(pcd, shared, R, N, tr, hs) for _ in range(batch)]
    one = [_design(pcd, ctx, R, N, tr, hs) for _ in range(batch)]
    ms_b, rounds = run(ds, True)
    ms_s, its = run(one, False)
    diff = max(float(np.abs(a.target_points() - b.target_points()).max()) for a, b in zip(ds, one))
    out["batched"] = {"targets": batch, "form": "mixed, relative residual 1e-9 / 1e-10, lock-step batches",
                      "wall_ms": ms_b, "ms_per_target": ms_b / batch, "rounds_of_transport_iterations": rounds,
                      "sequential_wall_ms": ms_s, "sequential_transport_iterations": its,
                      "speedup_over_sequential": ms_s / ms_b, "max_abs_target_point_diff_vs_sequential": diff}
    for d in ds + one:
        d.close()
    shared.close()
    return out


def config3_section(pcd, ctx, net, train_steps=12):
    """The learned warm start on the held-out seeds (900000-900007, Gaussian
    and binary densities): each solved to relative residual 1e-6 at 256^2 and
    512^2 by the mixed form from a zero guess and from the network's judged
    prediction (train_unet.evaluate), and the CUDA-event time of a training
    step at the network's 64^2 grid and batch 32 (seeded random inputs)."""
    import torch

    from poisson_caustic_design_gb300 import learned as _learned
    from poisson_caustic_design_gb300 import train_unet as _train

    rows = _train.evaluate(ctx, net)
    summ = _train.summarize(rows)
    tnet = _learned.UNet(ctx, resolution=64, max_batch=32, seed=1)
    g = torch.Generator(device="cpu").manual_seed(64)
    x = torch.randn(32, 64, 64, generator=g).cuda()
    t = torch.randn(32, 64, 64, generator=g).cuda()
    tnet.train_step(x, t, 1e-4)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(train_steps):
        tnet.train_step(x, t, 1e-4)
    e1.record()
    e1.synchronize()
    tnet.close()
    net.attach(ctx)
    return {"held_out_seeds": [900000, 900007], "sizes": [256, 512], "tol": 1e-6,
            "mean_sweep_ratio": summ["mean_sweep_ratio"], "mean_time_ratio": summ["mean_time_ratio"],
            "accepted": summ["accepted"], "evaluated": summ["evaluated"],
            "mean_ms": {str(n): {"zero_start": float(np.mean([r["ms_0"] for r in rows if r["n"] == n])),
                                 "learned_start": float(np.mean([r["ms_2"] for r in rows if r["n"] == n]))}
                        for n in (256, 512)},
            "train_step_ms_64x32": e0.elapsed_time(e1) / train_steps,
            "note": "ratios are learned + mixed over mixed from a zero guess; the network runs on the density "
                    "area-averaged to 64^2 (BF16, tcgen05 tensor cores)"}


def config4_section(pcd, ctx, device, batch=16):
    """The largest workload: mesh 1024^2 on 4096^2 grids.  `batch` targets
    (seeds 0..batch-1) initialised and taken through their first transport
    iteration (the costliest: phi starts at 0) as one batch of contexts, mixed
    precision with the reference's stop (max |delta| < 1e-7, Neumann-optimal
    omega); the conv 0.001 loop would take minutes per target, so this is a
    bounded sample of it."""
    import torch

    R, N = 1024, 4096
    ctxs = [pcd.Context(device) for _ in range(batch)]
    tr = pcd.SolveOptions(tol=1e-7, precision=pcd.PREC_MIXED, omega=-1.0, max_iterations=200000)
    ds = [_design(pcd, c, R, N, tr, tr) for c in ctxs]
    imgs = [pcd.inputs.pipeline_image(R, s) for s in range(batch)]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    pcd.initialize_batch(ds, imgs)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    steps = pcd.transport_iteration_batch(ds)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    sweeps = [d.last_solve_stats["sweeps"] for d in ds]
    out = {"mesh": R, "grid": N, "targets": batch, "form": "mixed", "init_ms": (t1 - t0) * 1e3,
           "first_transport_ms": (t2 - t1) * 1e3, "ms_per_target_transport": (t2 - t1) * 1e3 / batch,
           "sweeps_mean": float(np.mean(sweeps)), "steps_finite": bool(np.all(np.isfinite(steps)))}
    for d in ds:
        d.close()
    for c in ctxs:
        c.close()
    return out


def measured_hbm_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


# ---------------------------------------------------------------------------
def run_ours(args, rank, world, local, pg):
    import torch

    import poisson_caustic_design_gb300 as pcd
    from poisson_caustic_design_gb300 import _lib

    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    ctx = pcd.Context(local)
    # the context's autotuner picks each form's settings during the warm-up
    # (trial solves on the first call of a shape, outside the timed region)
    ctx.set_autotune(not args.no_autotune)
    L = _lib.load()
    if args.batch_only:
        import torch

        sizes, bb = batch_instances(pcd)
        pp = [torch.zeros_like(x) for x in bb]
        bopts = pcd.SolveOptions(stop=pcd.STOP_REL_RESIDUAL, tol=TOL, max_iterations=200000, omega=-1.0,
                                 warm_start=0)
        per, bst = pcd.batch_solve(ctx, bb, pp, bopts)
        torch.cuda.synchronize(dev)
        print(json.dumps({"batch_only": {"device_ms": bst["device_ms"], "clusters": bst["clusters"],
                                         "all_converged": bool(all(x["converged"] for x in per))}}), flush=True)
        ctx.close()
        return
    if args.stream_only:
        peak, src = measured_hbm_peak()
        print(json.dumps({"roofline_stream_4096": stream_section(ctx, torch.cuda.current_stream(dev), peak),
                          "peak_gbs": peak, "peak_source": src}), flush=True)
        ctx.close()
        return
    bs_host = instances()
    bs = [torch.from_numpy(b).to(dev) for b in bs_host]
    phi = torch.zeros((N_GRID, N_GRID), dtype=torch.float64, device=dev)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)

    forms = {
        "mixed": pcd.SolveOptions(stop=pcd.STOP_REL_RESIDUAL, tol=TOL, max_iterations=200000,
                                  precision=pcd.PREC_MIXED, omega=-1.0, warm_start=0),
        "plain_fp64": pcd.SolveOptions(stop=pcd.STOP_REL_RESIDUAL, tol=TOL, max_iterations=200000,
                                       precision=pcd.PREC_FP64, omega=-1.0, warm_start=0),
    }
    from poisson_caustic_design_gb300 import learned as _learned

    wpath = _learned.default_weights_path(64)
    net = None
    if os.path.exists(wpath):
        net = _learned.UNet(ctx, resolution=64, max_batch=1)
        net.load(wpath)
        net.attach(ctx)
        forms = {"learned_mixed": pcd.SolveOptions(stop=pcd.STOP_REL_RESIDUAL, tol=TOL, max_iterations=200000,
                                                   precision=pcd.PREC_MIXED, omega=-1.0, warm_start=2), **forms}
    headline = "learned_mixed" if net is not None else "mixed"
    if args.headline_only:
        forms = {headline: forms[headline]}

    def timed(opts, k):
        b = bs[k % len(bs)]
        flush.zero_()                      # evict the L2 (512 MiB > 129 MB) before each solve
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        st = ctx.solve_device(b, phi, opts, stream=stream.cuda_stream)
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1), st

    results = {}
    launches_before = L.pcd_kernel_launches()
    # clocks sampled across all timed regions (the forms and the end-to-end runs)
    sampler = ClockSampler(local)
    sampler.start()
    for name, opts in forms.items():
        for w in range(args.warmup):
            timed(opts, w)
        torch.cuda.synchronize()
        barrier(pg)
        if name == headline:
            launches_before = L.pcd_kernel_launches()
        ms, sweeps, sweep_ms, rels, warm, checks = [], [], [], [], [], []
        for k in range(args.steps):
            t, st = timed(opts, k)
            ms.append(t)
            sweeps.append(st["sweeps"])
            sweep_ms.append(st["sweep_ms"])
            rels.append(st["rel_residual"])
            warm.append(st["warm_used"])
            checks.append(st["residual_checks"])
        torch.cuda.synchronize()
        barrier(pg)
        if name == headline:
            launches = L.pcd_kernel_launches() - launches_before
        results[name] = {"ms": max_over_ranks(pg, float(np.sum(ms))) / args.steps, "sweeps": float(np.mean(sweeps)),
                         "sweep_ms": float(np.mean(sweep_ms)), "max_rel_residual": float(np.max(rels)),
                         "residual_checks": float(np.mean(checks)),
                         "schedule": int(st["schedule_used"]),
                         "tuned": {"check_every": st["check_every_used"], "refine_every": st["refine_every_used"],
                                   "refine_drop": st["refine_drop_used"]}}
        if name == "learned_mixed":
            results[name]["warm_accepted"] = int(sum(w == 2 for w in warm))

    acc, e2e, e2e_ms = {}, None, []
    if not args.headline_only:
        # accuracy of every form on every one of the eight densities against
        # the exact FP64 solve (DCT, residual ~1e-13), outside the timed region
        exact = [exact_solve(b) for b in bs_host]
        for name, opts in forms.items():
            per = []
            for k, b in enumerate(bs):
                out = torch.zeros_like(phi)
                ctx.solve_device(b, out, opts, stream=stream.cuda_stream)
                torch.cuda.synchronize()
                per.append(err_mod_const(out.cpu().numpy(), exact[k]))
            acc[name] = {"l2_mean": float(np.mean([p[0] for p in per])), "l2_max": float(max(p[0] for p in per)),
                         "max_mean": float(np.mean([p[1] for p in per])), "max_max": float(max(p[1] for p in per)),
                         "instances": len(per), "reference": "exact FP64 DCT solve of the same b"}

        # end to end through the host-array C ABI: pinned b in, phi out
        hopts = forms[headline]
        hb = [torch.from_numpy(b).pin_memory() for b in bs_host]
        hphi = torch.zeros((N_GRID, N_GRID), dtype=torch.float64).pin_memory()
        for w in range(args.warmup):
            ctx.solve(hb[w % len(hb)].numpy(), hphi.numpy(), hopts)
        barrier(pg)
        # host-timed, so a single stall of the host (the clock sampler's
        # nvidia-smi queries the driver meanwhile) moves a short mean: three
        # samples per step, all of them averaged
        for k in range(3 * args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            t = time.perf_counter()
            ctx.solve(hb[k % len(hb)].numpy(), hphi.numpy(), hopts)
            e2e_ms.append((time.perf_counter() - t) * 1e3)
        barrier(pg)
        e2e = max_over_ranks(pg, float(np.mean(e2e_ms)))
    clocks = sampler.stop()
    if e2e_ms:
        print("e2e samples (ms): " + " ".join(f"{t:.2f}" for t in e2e_ms), file=sys.stderr, flush=True)

    # roofline of the dominant kernel of the headline step: the FP32 cluster
    # sweep kernel (k_sor_cluster_rr, one launch per FP32 cycle).  Algorithmic
    # bytes per cell-sweep: 12 (read e, read r32, write e in FP32); a launch
    # runs sweeps / cycles sweeps (cycles = FP64 residual evaluations - 1 on
    # the cluster schedule), over the sweep kernels' device time (CUDA events
    # on the context stream around the cycle loop).
    hm = results[headline]
    cells = N_GRID * N_GRID
    alg_bytes = 12.0 * cells * hm["sweeps"]
    achieved = alg_bytes / (hm["sweep_ms"] * 1e-3) / 1e9
    peak, peak_src = measured_hbm_peak()
    cycles = max(1.0, hm["residual_checks"] - 1.0)
    # DRAM bytes per k_sor_cluster_rr launch of the autotuned headline
    # configuration, from one ncu capture: the band load of e and r32 only --
    # the grid stays on the cluster for the whole launch
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": CLUSTER_DRAM_BYTES_PER_LAUNCH, "traffic_unit": "bytes per launch (ncu)",
            "alg_bytes_per_launch": alg_bytes / cycles, "sweeps_per_launch": hm["sweeps"] / cycles,
            "peak_source": peak_src, "kernel": "k_sor_cluster_rr (FP32 sweeps)", "alg_bytes_per_solve": alg_bytes,
            "note": "the 512^2 working set stays on one 16-CTA cluster for a whole FP32 cycle (e in registers, "
                    "r32 in shared memory): the kernel is bound by FP32 issue, block and cluster barriers, not "
                    "HBM; DRAM traffic per launch is the band load and store (ncu summary under profiles/)"}
    # the plain FP64 form's sweep kernel (the block schedule at 512^2) is bound
    # by the FP64 pipe: reported against the measured FP64 FMA rate of this part
    if "plain_fp64" in results:
        pf = results["plain_fp64"]
        us = 1e3 * pf["sweep_ms"] / max(1.0, pf["sweeps"])
        roof["plain_fp64_sweep"] = {"us_per_sweep": us, "schedule": pf["schedule"],
                                    "alg_gbs": 24.0 * cells / (us * 1e-6) / 1e9,
                                    "fp64_issue_bound_us": FP64_OPS_PER_CELL * cells / FP64_OPS_PER_S * 1e6,
                                    "note": "5 FP64 operations per cell-sweep over the measured 0.60 TFMA/s "
                                            "FP64 rate of this part"}

    # batched configuration: 64 instances, sizes uniform in {64..1024}^2,
    # batched tile passes or the cluster form (CUDA graphs, the autotuner
    # picks); FP32 sweeps, FP64 residuals
    batched = None
    if not args.no_batch and not args.headline_only:
        sizes, bb = batch_instances(pcd)
        pp = [torch.zeros_like(x) for x in bb]
        bopts = pcd.SolveOptions(stop=pcd.STOP_REL_RESIDUAL, tol=TOL, max_iterations=200000, omega=-1.0, warm_start=0)
        for w in range(max(1, args.warmup // 2)):
            pcd.batch_solve(ctx, bb, pp, bopts)
        bt = []
        for k in range(max(2, args.steps // 2)):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            per, bst = pcd.batch_solve(ctx, bb, pp, bopts, stream=stream.cuda_stream)
            e1.record(stream)
            e1.synchronize()
            bt.append(e0.elapsed_time(e1))
        bms = float(np.mean(bt))
        batched = {"instances": 64, "sizes": {str(n_): sizes.count(n_) for n_ in sorted(set(sizes))},
                   "ms_per_batch": bms, "solves_per_s": 64 / (bms * 1e-3),
                   "alg_gbs": 12.0 * bst["cell_sweeps"] / (bms * 1e-3) / 1e9,
                   "all_converged": bool(all(x["converged"] for x in per)),
                   "max_rel_residual": float(max(x["rel_residual"] for x in per)),
                   "form": "tiles" if bst["clusters"] == 0 else "clusters",
                   "clusters": bst["clusters"], "cluster_size": bst["cluster_size"],
                   "check_every": bst["check_every"], "refine_drop": bst["refine_drop"], "autotuned": bool(bst["tuned"])}
        del bb, pp

    stream_roof = None
    if not args.no_batch and not args.headline_only:
        stream_roof = stream_section(ctx, stream, peak)

    # the full-pipeline workloads (mesh 128 and mesh 1024), with the CPU
    # reference's matching sample timed in a fresh process
    config0 = config4 = None
    if not args.no_pipelines and not args.headline_only:
        config0 = config0_section(pcd, ctx, local)
        config4 = config4_section(pcd, ctx, local)
        if rank == 0 and not args.no_cpu_baseline:
            c0 = cpu_sample_subprocess(0.0, what="config0")
            config0["cpu_reference_first_transport"] = {
                **c0, "gpu_plain_fp64_first_transport_ms": config0["forms"]["plain_fp64"]["first_transport_ms"],
                "note": "initialisation and first transport iteration of the same design on the host cores "
                        "(the C port of the reference's steps, its threaded solver)"}
            c4 = cpu_sample_subprocess(0.0, what="config4")
            config4["cpu_reference"] = {**c4, "first_transport_ms_extrapolated": c4["per_sweep_ms"] *
                                        config4["sweeps_mean"],
                                        "note": "per-sweep time of the reference's threaded SOR at 4096^2 times "
                                                "the GPU's mean sweep count (one transport solve takes minutes)"}

    # config 3: the learned warm start on held-out seeds at 256^2 and 512^2
    # (learned + mixed against mixed from a zero guess, same tolerance), and
    # one training step of the network at its training batch
    config3 = None
    if net is not None and not args.no_pipelines and not args.headline_only:
        config3 = config3_section(pcd, ctx, net)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline and not args.headline_only:
        # the reference's threaded solver on the same eight densities as the
        # reference arm, in a fresh process (no CUDA context, no runtime threads
        # of this one competing with its fork-join threads), 3 s per solve at
        # most (slower solves extrapolated from their chunk rate)
        cs = cpu_sample_subprocess(3.0)
        cpu = {"value": cs["ms"], "unit": UNIT, "cores": cs["threads"], "kind": "port",
               "sweeps_per_solve": cs["sweeps"],
               "sample": (f"one solve of each of the eight 512x512 densities (Gaussian/binary) to rel residual 1e-6 "
                          f"({cs['sweeps']:.0f} sweeps on average" + (", slow solves extrapolated from the chunk "
                                                                       "rate" if cs["extrapolated"] else "")
                          + f") of the reference's tile-threaded SOR schedule on {cs['threads']} threads, in a "
                          "separate process")}

    line = {
        "metric": METRIC, "value": hm["ms"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": hm["ms"], "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 sweeps + f64 residual/update", "data": "synthetic (seeded densities)",
        "config": {"workload": "single 512x512 Neumann Poisson solve to rel residual 1e-6 (" +
                               ("learned U-Net warm start + " if headline == "learned_mixed" else "") +
                               "FP32 sweeps + FP64 defect correction)", "grid": N_GRID, "tol": TOL,
                   "omega": "neumann-optimal",
                   "l2": "flushed before every solve (512 MiB write)", "instances": len(SEEDS),
                   "autotuned": not args.no_autotune,
                   "schedule": {1: "launches", 2: "persistent", 3: "cluster", 4: "stripes",
                                5: "stream"}.get(hm["schedule"], "?")},
        "forms": {k: {**v, "err_vs_exact_fp64": acc.get(k)} for k, v in results.items()},
        "speedup_plain_over_mixed": (results["plain_fp64"]["ms"] / results["mixed"]["ms"]
                                     if "plain_fp64" in results else None),
        "speedup_plain_over_headline": (results["plain_fp64"]["ms"] / hm["ms"] if "plain_fp64" in results else None),
        "headline_form": headline,
        "batched": batched,
        "config0_pipeline": config0,
        "config4_pipeline_batched": config4,
        "config3_learned": config3,
        "roofline_stream_4096": stream_roof,
        "roofline": roof,
        "cpu_baseline": cpu,
        "e2e": ({"value": e2e, "unit": UNIT, "h2d_bytes_per_step": cells * 8, "d2h_bytes_per_step": cells * 8,
                 "samples": len(e2e_ms), "median": float(np.median(e2e_ms))}
                if e2e is not None else None),
        "gpu_launches": int(launches),
        "gpu_launches_per_step": int(launches) / args.steps,
        "clocks": clocks,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()


def run_pipeline_profile(local):
    """The pipeline kernels at the 1024^2-mesh / 4096^2-grid size (fields of
    128 MiB, beyond the L2): one design's initialisation, one transport and
    one height iteration in mixed precision with each Poisson solve capped at 8
    sweeps, so that a launch list of this run is the pipeline's own kernels."""
    import torch

    import poisson_caustic_design_gb300 as pcd

    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    ctx = pcd.Context(local)
    R, N = 1024, 4096
    cap = pcd.SolveOptions(tol=1e-7, precision=pcd.PREC_MIXED, omega=-1.0, max_iterations=8)
    d = pcd.CausticDesign(ctx, transport=cap, height_solve=cap)
    d.set_mesh_resolution(R, R)
    d.set_domain_resolution(N, N)
    d.set_mesh_size(0.5, 0.5)
    d.set_lens_focal_length(1.5)
    d.set_lens_thickness(0.1)
    img = pcd.inputs.pipeline_image(R, seed=4)
    out = {"mesh": R, "grid": N}
    for name, fn in (("init", lambda: d.initialize_solvers(img)), ("transport", d.perform_transport_iteration),
                     ("height", lambda: d.perform_height_map_iteration(0))):
        torch.cuda.synchronize()
        t = time.perf_counter()
        fn()
        torch.cuda.synchronize()
        out[name + "_ms"] = (time.perf_counter() - t) * 1e3
        if name != "init":
            out[name + "_solve_ms"] = d.last_solve_stats["device_ms"]
    # the steps around the solve at the same size: image ingest (a 1024^2
    # 8-bit PNG decoded, resized to the 4096^2 grid on the GPU), fold handling
    # (one Laplacian smoothing of the target mesh, the fold count), the
    # output files (the target solid as OBJ, the parameterisation as SVG)
    import tempfile

    from poisson_caustic_design_gb300 import image as _image

    png = _gray_png(np.clip(np.round(_image.resize_image(img, R, R)), 0, 255).astype(np.uint8))
    steps = {"png_decode_1024": lambda: _image.png_decode(png),
             "resize_1024_to_4096": lambda: _image.resize_image(img[::4, ::4], N, N),
             "smooth_target_mesh": lambda: d.smooth_target_mesh(0.5),
             "count_folds": d.count_folds}
    with tempfile.TemporaryDirectory() as td:
        steps["save_solid_obj_target"] = lambda: d.save_solid_obj_target(os.path.join(td, "target.obj"))
        steps["export_parameterization_svg"] = lambda: d.export_paramererization_to_svg(os.path.join(td, "p.svg"),
                                                                                         0.5)
        for name, fn in steps.items():
            fn()  # first use (allocations, page cache)
            torch.cuda.synchronize()
            t = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            out[name + "_ms"] = (time.perf_counter() - t) * 1e3
    out["png_bytes"] = len(png)
    print(json.dumps({"pipeline_profile": out}), flush=True)
    d.close()
    ctx.close()


def _gray_png(u8):
    """An 8-bit grayscale PNG of a 2-D uint8 array (filter 0 rows, zlib),
    written here so that the decoder is timed on an independent encoding."""
    import struct
    import zlib

    h, w = u8.shape
    raw = b"".join(b"\x00" + u8[y].tobytes() for y in range(h))

    def chunk(kind, data):
        return struct.pack(">I", len(data)) + kind + data + struct.pack(">I", zlib.crc32(kind + data) & 0xFFFFFFFF)

    return (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 0, 0, 0, 0)) +
            chunk(b"IDAT", zlib.compress(raw, 6)) + chunk(b"IEND", b""))


def run_config4(args, local):
    """Full pipeline at mesh 1024^2 / grid 4096^2 on one target: target-area
    initialisation, two transport iterations and one height iteration, with the
    reference's stop rule (max |delta| < 1e-7 transport, 1e-8 height; the
    Neumann-optimal omega) in plain FP64 and in mixed precision.  The CPU
    figure is the reference's tile-threaded SOR per-sweep time at 4096^2 on
    the host cores times the GPU plain form's sweep count (extrapolated: a
    full CPU iteration takes hours)."""
    import torch

    import poisson_caustic_design_gb300 as pcd

    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    ctx = pcd.Context(local)
    R, N = 1024, 4096
    img = pcd.inputs.pipeline_image(R, seed=4)
    out = {"mesh": R, "grid": N, "width": 0.5, "focal_l": 1.5, "thickness": 0.1, "forms": {}}
    for name, prec in (("plain_fp64", pcd.PREC_FP64), ("mixed", pcd.PREC_MIXED)):
        tr = pcd.SolveOptions(tol=1e-7, precision=prec, omega=-1.0, max_iterations=200000)
        hs = pcd.SolveOptions(tol=1e-8, precision=prec, omega=-1.0, max_iterations=200000)
        d = pcd.CausticDesign(ctx, transport=tr, height_solve=hs)
        d.set_mesh_resolution(R, R)
        d.set_domain_resolution(N, N)
        d.set_mesh_size(0.5, 0.5)
        d.set_lens_focal_length(1.5)
        d.set_lens_thickness(0.1)
        torch.cuda.synchronize()
        t = time.perf_counter()
        d.initialize_solvers(img)
        torch.cuda.synchronize()
        rec = {"init_ms": (time.perf_counter() - t) * 1e3, "transport": []}
        for it in range(2):
            t = time.perf_counter()
            step = d.perform_transport_iteration()
            torch.cuda.synchronize()
            st = d.last_solve_stats
            rec["transport"].append({"ms": (time.perf_counter() - t) * 1e3, "step": step, "sweeps": st["sweeps"],
                                     "solve_ms": st["device_ms"], "schedule": st["schedule_used"]})
        t = time.perf_counter()
        upd = d.perform_height_map_iteration(0)
        torch.cuda.synchronize()
        st = d.last_solve_stats
        rec["height"] = {"ms": (time.perf_counter() - t) * 1e3, "update": upd, "sweeps": st["sweeps"],
                         "solve_ms": st["device_ms"]}
        out["forms"][name] = rec
        d.close()
    # CPU: per-sweep time of the reference's threaded schedule at 4096^2
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    oracle.build(ref=False)
    port = oracle.Port()
    threads = os.cpu_count() or 1
    b = pcd.inputs.poisson_rhs(N, 3, "gaussian")
    phi = np.zeros_like(b)
    port.poisson_solver_threads(b, phi, 2, 0.0, threads)
    t = time.perf_counter()
    port.poisson_solver_threads(b, phi, 6, 0.0, threads)
    per_sweep = (time.perf_counter() - t) / 6
    plain = out["forms"]["plain_fp64"]
    cpu_ms = [per_sweep * x["sweeps"] * 1e3 for x in plain["transport"]]
    seg = int(np.floor(np.sqrt(threads)))
    out["cpu_reference"] = {"per_sweep_ms": per_sweep * 1e3, "threads": seg * seg,
                            "transport_ms_extrapolated": cpu_ms,
                            "note": "per-sweep time x the GPU plain form's sweep count"}
    print(json.dumps({"config4": out}), flush=True)
    ctx.close()


def main():
    args = parse()
    if args.cpu_sample is not None:
        out = (cpu_sample(args.cpu_sample, args.cpu_omega) if args.cpu_what == "solve"
               else cpu_pipeline_sample(args.cpu_what))
        print(json.dumps(out), flush=True)
        return
    rank, world, local, pg = dist_setup(args.gpus)
    if args.impl == "reference":
        run_reference(args, rank, world, pg)
    elif args.config4:
        if rank == 0:
            run_config4(args, local)
    elif args.pipeline_profile:
        if rank == 0:
            run_pipeline_profile(local)
    else:
        run_ours(args, rank, world, local, pg)
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
