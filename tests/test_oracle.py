"""The CPU oracle pinned against the reference's own outputs (golden fixtures
written by tests/golden/make_golden.py from the reference's compiled sources),
plus oracle self-consistency (DCT exact solve).  CPU only."""
import numpy as np
import pytest

from conftest import load_golden, solver_case_names


@pytest.mark.parametrize("name", solver_case_names())
def test_port_solver_bit_exact_vs_reference(port, name):
    z = load_golden("solver_cases.npz")
    b, phi0, ref = z[f"{name}/b"], z[f"{name}/phi0"], z[f"{name}/phi"]
    max_iter, tol = z[f"{name}/params"]
    if b.size > 100_000:
        pytest.skip("large case covered on GPU tests")
    phi = phi0.copy()
    port.poisson_solver(b, phi, int(max_iter), float(tol))
    # one-tile lexicographic SOR in the same operation order: identical bits
    assert np.array_equal(np.isnan(phi), np.isnan(ref))
    m = ~np.isnan(ref)
    assert np.array_equal(phi[m], ref[m])


def test_port_utils_bit_exact_vs_reference(port):
    z = load_golden("utils_cases.npz")
    gx, gy = port.gradient(z["g"])
    assert np.array_equal(gx, z["gx"]) and np.array_equal(gy, z["gy"])
    assert np.array_equal(port.divergence(z["g"], z["g2"]), z["div"])
    sub = port.subtract_average(z["gn"])
    assert np.array_equal(np.isnan(sub), np.isnan(z["sub"]))
    m = ~np.isnan(sub)
    assert np.array_equal(sub[m], z["sub"][m])
    assert np.array_equal(port.scale_proportional(z["g"] * 3.0 + 1.0), z["scaled"])
    for (x, y), v in zip(z["pts"], z["bil"]):
        assert port.bilinear(z["g"], x, y) == v


@pytest.mark.parametrize("res", [16, 32])
def test_port_pipeline_vs_reference(port, res):
    """Caustic_design replay: the port matches the reference to rounding."""
    import oracle

    z = load_golden(f"pipeline_r{res}.npz")
    r, width, focal, thickness, conv, seed = z["params"]
    r = int(r)
    d = oracle.PortDesign(port, r, r, 4 * r, 4 * r, width, width, focal, thickness)
    d.initialize(z["image"])
    np.testing.assert_allclose(d.target_areas, z["target_areas"], rtol=1e-12, atol=1e-18)
    steps = []
    for itr in range(50):
        s = d.transport_iteration()
        steps.append(s)
        if s < conv:
            break
    assert len(steps) == len(z["steps"])
    np.testing.assert_allclose(steps, z["steps"], rtol=1e-9)
    tp = z["target_points"]
    assert np.abs(d.target_points - tp).max() < 1e-12
    for itr in range(3):
        d.height_iteration()
    sp = z["source_points"]
    assert np.linalg.norm(d.source_points[:, 2] - sp[:, 2]) / np.linalg.norm(sp[:, 2]) < 1e-10
    e = oracle.rel_err_mod_const(d.h, z["h"])[0]
    assert e < 1e-10


def test_dct_exact_solve_matches_reference_operator(port):
    """The DCT solution satisfies the reference operator to rounding."""
    import oracle
    from poisson_caustic_design_gb300 import inputs

    for n, m in ((64, 64), (96, 40)):
        b = inputs.poisson_rhs(n, 5, "gaussian", m=m)
        phi = oracle.dct_solve(b)
        r, rn, bn, rmax = port.residual(b, phi)
        assert rn / bn < 1e-12


def test_reference_solution_close_to_dct():
    """The reference's own converged output (tol 1e-7) is the DCT solution to ~1e-8."""
    import oracle

    z = load_golden("solver_cases.npz")
    for name in ("gauss_64", "gauss_128", "binary_96x80"):
        e2, emax = oracle.rel_err_mod_const(z[f"{name}/phi"], oracle.dct_solve(z[f"{name}/b"]))
        assert e2 < 1e-7, (name, e2)


def test_cosine_mode_known_answer():
    """b = cos(pi k (x+1/2)/W) cos(pi l (y+1/2)/H) is an eigenvector of the
    Neumann operator with eigenvalue 2cos(pi k/W)+2cos(pi l/H)-4."""
    import oracle

    W, H, k, l = 48, 32, 3, 2
    x = (np.arange(W) + 0.5) / W
    y = (np.arange(H) + 0.5) / H
    b = np.cos(np.pi * l * y)[:, None] * np.cos(np.pi * k * x)[None, :]
    lam = 2 * np.cos(np.pi * k / W) + 2 * np.cos(np.pi * l / H) - 4
    np.testing.assert_allclose(oracle.dct_solve(b), b / lam, atol=1e-12)


@pytest.mark.parametrize("res", [16, 32])
def test_reference_height_accuracy_is_bounded(port, res):
    """The reference's h (max|delta| < 1e-8 stop) lies within 5e-5 of the exact
    solve of its final divergence; GPU parity on h is judged against this."""
    import oracle

    z = load_golden(f"pipeline_r{res}.npz")
    r, width, focal, thickness, conv, seed = z["params"]
    r = int(r)
    d = oracle.PortDesign(port, r, r, 4 * r, 4 * r, width, width, focal, thickness)
    d.initialize(z["image"])
    for _ in range(len(z["steps"])):
        d.transport_iteration()
    for _ in range(3):
        d.height_iteration()
    e_ref = oracle.rel_err_mod_const(z["h"], oracle.dct_solve(d.divergence))[0]
    assert 1e-6 < e_ref < 5e-5


def test_threaded_port_matches_reference_schedule(port):
    """The port's tile-threaded solver (solver.cpp:80-129): one tile for
    max_threads < 4 is the golden result bit for bit; more tiles (chaotic, as
    in the reference) converge to the same solution."""
    import oracle

    z = load_golden("solver_cases.npz")
    b, ref = z["binary_96x80/b"], z["binary_96x80/phi"]
    phi = np.zeros_like(b)
    port.poisson_solver_threads(b, phi, 100000, 1e-7, 3)
    assert np.array_equal(phi, ref)
    phi = np.zeros_like(b)
    port.poisson_solver_threads(b, phi, 100000, 1e-7, 16)
    assert oracle.rel_err_mod_const(phi, ref)[0] < 1e-7


@pytest.mark.parametrize("name", ["smooth_a", "smooth_b"])
def test_laplacian_smoothing_port_matches_reference(port, name):
    """Mesh::laplacian_smoothing (mesh.cpp:534-606), factor 0.1f: the port is
    bit-identical to the reference's compiled function (golden)."""
    z = load_golden("mesh_cases.npz")
    nx, ny, w, h, f = z[f"{name}/params"]
    out = port.laplacian_smoothing(z[f"{name}/points"], int(nx), int(ny), f)
    assert np.array_equal(out, z[f"{name}/smoothed"])


def test_fold_count_port(port):
    nx = ny = 8
    y, x = np.meshgrid(np.arange(ny) / (ny - 1), np.arange(nx) / (nx - 1), indexing="ij")
    p = np.stack([x.ravel(), y.ravel(), np.zeros(nx * ny)], axis=1)
    assert port.count_folds(p, nx, ny) == 0
    p[3 * nx + 3, 0] += 1.6 / (nx - 1)   # past its right neighbour: its fan inverts
    assert port.count_folds(p, nx, ny) > 0
