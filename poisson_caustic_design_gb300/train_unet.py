"""Train the learned warm start and measure what it gains.

    python -m poisson_caustic_design_gb300.train_unet --out weights.npz \\
        [--pairs 20000] [--data-resolution 256] [--resolution 64] [--epochs 30] [--batch 32]

Training pairs come from the library's batched GPU solver (FP32 sweeps, FP64
defect correction, relative residual 1e-7) on seeded 256^2 densities:
Gaussian mixtures for even seeds, binary disk/rectangle fields for odd seeds.
The network runs on the pairs area-averaged to 64^2: there a 4-level U-Net's
receptive field (about 90 cells) spans the whole grid, which the Poisson
inverse needs (at 256^2 it spans a third of it); the library averages a
solve's right-hand side to the network grid and interpolates the prediction
back.  Seeds
from 900000 on are held out for the evaluation, which solves each held-out
density at 256^2 and 512^2 to relative residual 1e-6 from a zero guess and
from the network's prediction and reports sweeps and wall time.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np


def evaluate(ctx, net, sizes=(256, 512), seeds=range(900000, 900008)):
    import torch

    import poisson_caustic_design_gb300 as pcd
    from poisson_caustic_design_gb300 import inputs

    net.attach(ctx)
    rows = []
    for n in sizes:
        for s in seeds:
            b = inputs.poisson_rhs_torch(n, [s])[0].contiguous()
            rec = {"n": n, "seed": s}
            for warm in (0, 2):
                phi = torch.zeros_like(b)
                opts = pcd.SolveOptions(stop=pcd.STOP_REL_RESIDUAL, tol=1e-6, precision=pcd.PREC_MIXED, omega=-1.0,
                                        warm_start=warm)
                ctx.solve_device(b, phi, opts)  # warm-up of graphs / clusters
                phi.zero_()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                st = ctx.solve_device(b, phi, opts)
                e1.record()
                e1.synchronize()
                rec[f"sweeps_{warm}"] = st["sweeps"]
                rec[f"ms_{warm}"] = e0.elapsed_time(e1)
                if warm == 2:
                    rec["warm_used"] = st["warm_used"]
                    rec["warm_rel"] = st["warm_rel_residual"]
            rows.append(rec)
    return rows


def summarize(rows):
    """Mean sweep and time ratios (learned start / zero start) per grid size."""
    return {
        "mean_sweep_ratio": {str(n): float(np.mean([r["sweeps_2"] / r["sweeps_0"] for r in rows if r["n"] == n]))
                             for n in (256, 512)},
        "mean_time_ratio": {str(n): float(np.mean([r["ms_2"] / r["ms_0"] for r in rows if r["n"] == n]))
                            for n in (256, 512)},
        "accepted": int(sum(r["warm_used"] == 2 for r in rows)), "evaluated": len(rows),
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=None, help="where to write the trained weights (required unless --evaluate-only)")
    ap.add_argument("--pairs", type=int, default=20000)
    ap.add_argument("--resolution", type=int, default=64, help="network grid")
    ap.add_argument("--data-resolution", type=int, default=256, help="grid of the training solves")
    ap.add_argument("--epochs", type=int, default=30)
    ap.add_argument("--batch", type=int, default=32)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--report", default=None)
    ap.add_argument("--time-budget-s", type=float, default=None)
    ap.add_argument("--half", action="store_true", help="store the weights as float16")
    ap.add_argument("--evaluate-only", default=None, metavar="WEIGHTS",
                    help="skip training: evaluate these weights on the held-out seeds")
    args = ap.parse_args()
    if not args.evaluate_only and not args.out:
        ap.error("--out is required unless --evaluate-only is given")

    import torch

    import poisson_caustic_design_gb300 as pcd
    from poisson_caustic_design_gb300 import learned

    ctx = pcd.Context(0)
    if args.evaluate_only:
        net = learned.UNet(ctx, resolution=args.resolution, max_batch=1)
        net.load(args.evaluate_only)
        rows = evaluate(ctx, net)
        for r in rows:
            print(json.dumps(r), flush=True)
        summ = summarize(rows)
        print(json.dumps(summ), flush=True)
        if args.report:
            with open(args.report, "w") as f:
                json.dump({"summary": summ, "rows": rows}, f, indent=1)
        return
    t0 = time.time()
    x, t = learned.make_pairs(ctx, range(args.pairs), args.data_resolution, tol=1e-7, net_res=args.resolution)
    torch.cuda.synchronize()
    t_data = time.time() - t0
    print(f"pairs: {x.shape[0]} solved at {args.data_resolution}^2, network grid {args.resolution}^2, "
          f"in {t_data:.1f} s", flush=True)
    net = learned.UNet(ctx, resolution=args.resolution, max_batch=args.batch, seed=0)
    t0 = time.time()
    hist = learned.train(net, x, t, epochs=args.epochs, batch=args.batch, lr=args.lr, log=lambda m: print(m, flush=True),
                         time_budget_s=args.time_budget_s)
    torch.cuda.synchronize()
    t_train = time.time() - t0
    net.save(args.out, half=args.half)
    del x, t
    rows = evaluate(ctx, net)
    for r in rows:
        print(json.dumps(r), flush=True)
    summ = {
        "pairs": args.pairs, "resolution": args.resolution, "data_resolution": args.data_resolution,
        "epochs": args.epochs, "batch": args.batch,
        "data_s": t_data, "train_s": t_train, "loss": hist, **summarize(rows),
    }
    print(json.dumps(summ), flush=True)
    if args.report:
        with open(args.report, "w") as f:
            json.dump({"summary": summ, "rows": rows}, f, indent=1)


if __name__ == "__main__":
    main()
