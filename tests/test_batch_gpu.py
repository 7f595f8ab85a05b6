"""The batched solve (many grids of uneven sizes in one persistent cluster
launch) against the exact DCT solve and against the single-grid solver."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SIZES = [(64, 64), (96, 96), (128, 128), (256, 256), (512, 512), (1024, 1024), (300, 200), (97, 33), (640, 480),
         (64, 700)]


def test_batch_matches_exact_and_single_solves(ctx):
    import torch

    import oracle
    import poisson_caustic_design_gb300 as pcd

    rhs = [pcd.inputs.poisson_rhs(w, 40 + i, "gaussian" if i % 2 else "binary", m=h) for i, (w, h) in enumerate(SIZES)]
    bs = [torch.from_numpy(b).cuda() for b in rhs]
    phis = [torch.full_like(b, 7.0) for b in bs]           # garbage: warm_start=False must ignore it
    opts = pcd.SolveOptions(stop=pcd.STOP_REL_RESIDUAL, tol=1e-8, max_iterations=200000, omega=-1.0,
                            warm_start=False)
    per, bst = pcd.batch_solve(ctx, bs, phis, opts)
    torch.cuda.synchronize()
    assert bst["status"] == 0 and bst["clusters"] >= 1
    port = oracle.Port()
    for i, (b, p) in enumerate(zip(rhs, phis)):
        assert per[i]["converged"] == 1, (SIZES[i], per[i])
        phi = p.cpu().numpy()
        _, rn, bn, _ = port.residual(b, phi)
        assert rn / bn <= 1.05e-8, (SIZES[i], rn / bn, per[i])
        assert abs(rn / bn - per[i]["rel_residual"]) <= 1e-3 * per[i]["rel_residual"] + 1e-15
        e2, _ = oracle.rel_err_mod_const(phi, oracle.dct_solve(b))
        assert e2 < 1e-6, (SIZES[i], e2)
    # the same grid through the single-grid solver agrees to the tolerance
    single = np.zeros_like(rhs[4])
    ctx.solve(rhs[4], single, pcd.SolveOptions(stop=pcd.STOP_REL_RESIDUAL, tol=1e-8, omega=-1.0,
                                               precision=pcd.PREC_MIXED))
    assert oracle.rel_err_mod_const(phis[4].cpu().numpy(), single)[0] < 1e-6


def test_batch_graph_replay_is_repeatable(ctx):
    import torch

    import poisson_caustic_design_gb300 as pcd

    bs = [torch.from_numpy(pcd.inputs.poisson_rhs(n, n, "gaussian")).cuda() for n in (64, 128, 256)]
    phis = [torch.zeros_like(b) for b in bs]
    opts = pcd.SolveOptions(stop=pcd.STOP_REL_RESIDUAL, tol=1e-6, omega=-1.0, warm_start=False)
    per1, _ = pcd.batch_solve(ctx, bs, phis, opts)
    first = [p.clone() for p in phis]
    per2, _ = pcd.batch_solve(ctx, bs, phis, opts)
    for a, b in zip(first, phis):
        assert torch.equal(a, b)       # same schedule per cluster: deterministic per instance
    assert [x["sweeps"] for x in per1] == [x["sweeps"] for x in per2]


def test_batch_graphs_survive_buffer_growth():
    """A cached batch graph holds the addresses of the context's scratch and
    descriptor buffers: a later batch that needs more of either reallocates
    them and drops the cached graphs, so replaying the first batch's
    signature captures it again (same results as on a fresh context)."""
    import torch

    import poisson_caustic_design_gb300 as pcd

    opts = pcd.SolveOptions(stop=pcd.STOP_REL_RESIDUAL, tol=1e-6, max_iterations=200000, omega=-1.0,
                            warm_start=False)
    small = [torch.from_numpy(pcd.inputs.poisson_rhs(1024, 61, "gaussian", m=512)).cuda()]
    large = [torch.from_numpy(pcd.inputs.poisson_rhs(1024, 62 + i, "gaussian")).cuda() for i in range(3)]
    large += [torch.from_numpy(pcd.inputs.poisson_rhs(64, 70 + i, "binary")).cuda() for i in range(40)]

    def run(c, bs):
        ps = [torch.zeros_like(b) for b in bs]
        per, bst = pcd.batch_solve(c, bs, ps, opts)
        torch.cuda.synchronize()
        assert bst["status"] == 0 and all(x["converged"] for x in per)
        return [p.cpu() for p in ps]

    ctx = pcd.Context(0)
    first = run(ctx, small)
    run(ctx, large)          # more global scratch and more descriptors
    again = run(ctx, small)  # the first signature again
    ctx.close()
    fresh_ctx = pcd.Context(0)
    fresh = run(fresh_ctx, small)
    fresh_ctx.close()
    assert torch.equal(first[0], again[0]) and torch.equal(first[0], fresh[0])


def test_batch_rejects_bad_instances(ctx):
    import torch

    import poisson_caustic_design_gb300 as pcd

    # 16 rows: below the cluster form's floor of 2 x 16 CTAs (the tile form,
    # which takes such grids, is not used for a width that is not a multiple of 8)
    b = torch.zeros((16, 18), dtype=torch.float64, device="cuda")
    with pytest.raises(pcd.PCDError):
        pcd.batch_solve(ctx, [b], [torch.zeros_like(b)])
    # the same through the cluster form explicitly
    b = torch.zeros((16, 16), dtype=torch.float64, device="cuda")
    with pytest.raises(pcd.PCDError):
        pcd.batch_solve(ctx, [b], [torch.zeros_like(b)], pcd.SolveOptions(stop=pcd.STOP_REL_RESIDUAL, tol=1e-6,
                                                                          schedule=pcd.SCHED_CLUSTER))
    # the relative-residual stop is required
    b = torch.zeros((64, 64), dtype=torch.float64, device="cuda")
    with pytest.raises(pcd.PCDError):
        pcd.batch_solve(ctx, [b], [torch.zeros_like(b)], pcd.SolveOptions(stop=pcd.STOP_MAX_UPDATE, tol=1e-6))


TILE_SIZES = [(64, 64), (96, 64), (128, 128), (256, 200), (512, 512), (1024, 1024), (504, 33), (1024, 300)]


def test_batch_tile_form_matches_cluster_form(ctx):
    """Grids whose widths are multiples of 8 run on batched tile passes (every
    grid's tiles in one launch per pass, FP64 refreshes batched per chunk):
    each converges to the tolerance against the exact solve, as on the
    cluster form (schedule CLUSTER), with a similar sweep count."""
    import torch

    import oracle
    import poisson_caustic_design_gb300 as pcd

    rhs = [pcd.inputs.poisson_rhs(w, 80 + i, "binary" if i % 2 else "gaussian", m=h)
           for i, (w, h) in enumerate(TILE_SIZES)]
    bs = [torch.from_numpy(b).cuda() for b in rhs]
    res = {}
    for sched in (0, 3):
        phis = [torch.full_like(b, 3.0) for b in bs]
        opts = pcd.SolveOptions(stop=pcd.STOP_REL_RESIDUAL, tol=1e-8, max_iterations=200000, omega=-1.0,
                                warm_start=False, schedule=sched)
        per, bst = pcd.batch_solve(ctx, bs, phis, opts)
        torch.cuda.synchronize()
        assert bst["status"] == 0
        assert (bst["clusters"] == 0) if sched == 0 else (bst["clusters"] >= 1)
        port = oracle.Port()
        for i, (b, p) in enumerate(zip(rhs, phis)):
            assert per[i]["converged"] == 1, (TILE_SIZES[i], per[i])
            phi = p.cpu().numpy()
            _, rn, bn, _ = port.residual(b, phi)
            assert rn / bn <= 1.05e-8, (TILE_SIZES[i], rn / bn, per[i])
            assert abs(rn / bn - per[i]["rel_residual"]) <= 1e-3 * per[i]["rel_residual"] + 1e-15
            assert oracle.rel_err_mod_const(phi, oracle.dct_solve(b))[0] < 1e-6, TILE_SIZES[i]
        res[sched] = [x["sweeps"] for x in per]
    for (w, h), st, sc in zip(TILE_SIZES, res[0], res[3]):
        assert st <= 1.3 * sc + 64, ((w, h), st, sc)


def test_batch_tile_form_padded_rows_and_sweep_cap(ctx):
    """Batched tile passes on padded rows (ld a multiple of 4 above the width)
    stop every grid at max_iterations exactly, with the iterate of the
    single-grid tile schedule (the same FP64 refreshes every 64 sweeps)."""
    import torch

    import poisson_caustic_design_gb300 as pcd

    shapes = [(256, 100, 260), (128, 70, 132), (512, 40, 520)]
    bs, phis = [], []
    for i, (w, h, ld) in enumerate(shapes):
        full = torch.zeros((h, ld), dtype=torch.float64, device="cuda")
        full[:, :w] = torch.from_numpy(pcd.inputs.poisson_rhs(w, 90 + i, "gaussian", m=h)).cuda()
        bs.append(full[:, :w])
        phis.append(torch.zeros((h, ld), dtype=torch.float64, device="cuda")[:, :w])
    opts = pcd.SolveOptions(stop=pcd.STOP_REL_RESIDUAL, tol=1e-14, max_iterations=101, omega=-1.0,
                            warm_start=False, refine_every=64)
    per, bst = pcd.batch_solve(ctx, bs, phis, opts)
    torch.cuda.synchronize()
    assert bst["clusters"] == 0 and bst["status"] == 1
    for (w, h, ld), b, p, x in zip(shapes, bs, phis, per):
        assert x["sweeps"] == 101 and x["converged"] == 0, x
        single = torch.zeros((h, ld), dtype=torch.float64, device="cuda")[:, :w]
        st = ctx.solve_device(b, single, pcd.SolveOptions(stop=pcd.STOP_REL_RESIDUAL, tol=1e-14, max_iterations=101,
                                                          omega=-1.0, precision=pcd.PREC_MIXED, schedule=6,
                                                          refine_every=64, warm_start=0))
        assert st["sweeps"] == 101 and st["schedule_used"] == 6
        ref = single.cpu().numpy()
        err = np.abs(p.cpu().numpy() - ref).max() / np.abs(ref).max()
        assert err < 1e-6, ((w, h), err)


def test_batch_tile_form_takes_short_and_wide_grids(ctx):
    """The batched tile form has neither the cluster form's height floor
    (2 x the cluster size) nor its 4096-column ceiling: a batch with a 16-row
    grid and a 4104-column grid goes to the tile passes and every grid reaches
    the tolerance against the exact solve."""
    import torch

    import oracle
    import poisson_caustic_design_gb300 as pcd

    shapes = [(64, 16), (4104, 40), (128, 128)]
    rhs = [pcd.inputs.poisson_rhs(w, 70 + i, "gaussian", m=h) for i, (w, h) in enumerate(shapes)]
    bs = [torch.from_numpy(b).cuda() for b in rhs]
    phis = [torch.zeros_like(b) for b in bs]
    opts = pcd.SolveOptions(stop=pcd.STOP_REL_RESIDUAL, tol=1e-8, max_iterations=400000, omega=-1.0,
                            warm_start=False)
    per, bst = pcd.batch_solve(ctx, bs, phis, opts)
    torch.cuda.synchronize()
    assert bst["status"] == 0 and bst["clusters"] == 0     # the tile form ran
    for i, (b, p) in enumerate(zip(rhs, phis)):
        assert per[i]["converged"] == 1, (shapes[i], per[i])
        e2, _ = oracle.rel_err_mod_const(p.cpu().numpy(), oracle.dct_solve(b))
        assert e2 < 1e-6, (shapes[i], e2)
