"""The context autotuner: the first AUTO solve of a shape (and the first batch
of a size signature) times candidate settings on the caller's data, keeps the
fastest that converged and reuses it; the returned solution is the winner's,
solved from the caller's own starting phi, so it meets the same tolerance as
an untuned solve and agrees with the exact (DCT) solution."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture()
def tctx():
    import poisson_caustic_design_gb300 as pcd

    c = pcd.Context(0)
    c.set_autotune(True)
    yield c
    c.close()


@pytest.mark.parametrize("prec", [0, 1])
def test_autotuned_solve_is_correct_and_cached(tctx, prec):
    import oracle
    import poisson_caustic_design_gb300 as pcd

    b = pcd.inputs.poisson_rhs(256, 21, "binary")
    exact = oracle.dct_solve(b)
    o = pcd.SolveOptions(stop=pcd.STOP_REL_RESIDUAL, tol=1e-8, max_iterations=200000, precision=prec, omega=-1.0,
                         warm_start=0)
    phi = np.full_like(b, 7.0)  # garbage in phi: a zero start must ignore it in every trial
    st = tctx.solve(b, phi, o)
    info = tctx.autotune_info()
    assert st["tuned"] == 1 and info["entries"] == 1 and info["trials"] >= 3
    assert st["converged"] and st["rel_residual"] <= 1e-8
    assert oracle.rel_err_mod_const(phi, exact)[0] < 1e-6
    # second call of the shape: reuses the kept settings, no new trials
    phi2 = np.zeros_like(b)
    st2 = tctx.solve(b, phi2, o)
    assert st2["tuned"] == 1 and tctx.autotune_info()["trials"] == info["trials"]
    assert (st2["check_every_used"], st2["refine_every_used"], st2["refine_drop_used"]) == \
        (st["check_every_used"], st["refine_every_used"], st["refine_drop_used"])
    assert st2["converged"] and oracle.rel_err_mod_const(phi2, exact)[0] < 1e-6


def test_autotuner_restores_the_warm_start(tctx):
    """Trials run from a snapshot of the caller's phi: a warm-started tuned
    solve ends where an untuned warm-started solve ends (same tolerance)."""
    import oracle
    import poisson_caustic_design_gb300 as pcd

    b = pcd.inputs.poisson_rhs(192, 8, "gaussian", m=160)
    exact = oracle.dct_solve(b)
    start = exact + 1e-2 * np.abs(exact).max() * np.sin(np.linspace(0, 9, b.size)).reshape(b.shape)
    o = pcd.SolveOptions(stop=pcd.STOP_REL_RESIDUAL, tol=1e-9, max_iterations=200000, precision=1, omega=-1.0,
                         warm_start=1)
    phi = start.copy()
    st = tctx.solve(b, phi, o)
    assert st["tuned"] == 1 and st["converged"]
    assert oracle.rel_err_mod_const(phi, exact)[0] < 1e-7


def test_pinned_settings_bypass_the_tuner(tctx):
    import poisson_caustic_design_gb300 as pcd

    b = pcd.inputs.poisson_rhs(96, 3, "gaussian")
    phi = np.zeros_like(b)
    st = tctx.solve(b, phi, pcd.SolveOptions(stop=pcd.STOP_REL_RESIDUAL, tol=1e-7, precision=1, omega=-1.0,
                                             warm_start=0, check_every=16))
    assert st["tuned"] == 0 and st["check_every_used"] == 16
    assert tctx.autotune_info()["trials"] == 0


def test_autotuned_batch(tctx):
    import torch

    import poisson_caustic_design_gb300 as pcd

    sizes = [64, 96, 128, 256, 64, 128]
    bs = [torch.from_numpy(pcd.inputs.poisson_rhs(n, 40 + i, "gaussian")).cuda() for i, n in enumerate(sizes)]
    ps = [torch.zeros_like(b) for b in bs]
    o = pcd.SolveOptions(stop=pcd.STOP_REL_RESIDUAL, tol=1e-6, omega=-1.0, warm_start=0)
    per, bst = pcd.batch_solve(tctx, bs, ps, o)
    # 16- or 8-CTA clusters, or (cluster size 0) the batched tile passes
    assert bst["tuned"] == 1 and bst["cluster_size"] in (0, 8, 16)
    assert all(x["converged"] and x["rel_residual"] <= 1e-6 for x in per)
    trials = tctx.autotune_info()["trials"]
    assert trials >= 2
    per2, bst2 = pcd.batch_solve(tctx, bs, ps, o)
    assert bst2["tuned"] == 1 and tctx.autotune_info()["trials"] == trials
    assert (bst2["cluster_size"], bst2["check_every"]) == (bst["cluster_size"], bst["check_every"])
    assert all(x["converged"] for x in per2)
