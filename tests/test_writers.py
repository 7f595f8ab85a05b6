"""The output files (row f3): the library's host writers produce the
reference's files byte for byte on the same inputs.  OBJ and SVG golden files
were written by the reference's own compiled utils.cpp (save_solid_obj,
export_grid_to_svg); the heightmap JSON writer of main.cpp (which does not
compile here) is checked against its restatement in the oracle, whose %g
number format the reference's OBJ files pin.  Host code only: no GPU."""
import numpy as np
import pytest

from conftest import load_golden


def _read(path):
    with open(path, "rb") as f:
        return f.read()


@pytest.mark.parametrize("name", ["obj_a", "obj_b", "obj_c"])
def test_solid_obj_matches_reference_bytes(tmp_path, name):
    import poisson_caustic_design_gb300 as pcd

    z = load_golden("writer_cases.npz")
    nx, ny, w, h, th = z[f"{name}/params"]
    out = str(tmp_path / "out.obj")
    pcd.save_solid_obj(z[f"{name}/front"], z[f"{name}/back"], int(nx), int(ny), th, w, h, out)
    assert _read(out) == bytes(z[f"{name}/text"])


@pytest.mark.parametrize("name", ["svg_a", "svg_b", "svg_c"])
def test_grid_svg_matches_reference_bytes(tmp_path, name):
    import poisson_caustic_design_gb300 as pcd

    z = load_golden("writer_cases.npz")
    nx, ny, w, h, sw = z[f"{name}/params"]
    out = str(tmp_path / "out.svg")
    pcd.export_grid_to_svg(z[f"{name}/points"], w, h, int(nx), int(ny), out, sw)
    assert _read(out) == bytes(z[f"{name}/text"])


def test_heightmap_json_matches_restatement(tmp_path):
    import oracle
    import poisson_caustic_design_gb300 as pcd

    rng = np.random.default_rng(5)
    h = rng.normal(0, 0.02, (5, 7))
    h[0, 0], h[1, 2], h[2, 3], h[4, 6] = 0.0, -0.0, 1.5e-7, 12345678.9
    out = str(tmp_path / "h.json")
    pcd.save_heightmap_as_json(h, out)
    assert _read(out).decode() == oracle.heightmap_json_text(h)


def test_writer_rejects_bad_path_and_shapes(tmp_path):
    import poisson_caustic_design_gb300 as pcd

    p = np.zeros((12, 3))
    with pytest.raises(pcd.PCDError):
        pcd.save_solid_obj(p, p, 4, 3, 0.1, 1.0, 1.0, str(tmp_path / "no_such_dir" / "x.obj"))
    with pytest.raises(ValueError):
        pcd.save_solid_obj(p, p, 5, 3, 0.1, 1.0, 1.0, str(tmp_path / "x.obj"))


def test_threaded_writers_match_reference_bytes_on_a_large_mesh(tmp_path):
    """At sizes where the writers format in several threads (ordered chunks
    of at least 4096 vertices or cells, 8 rows or paths), the files are still
    the reference's byte for byte: OBJ and SVG against the reference's own
    compiled writers (utils.cpp:198-307), the heightmap JSON against the
    oracle's restatement of main.cpp:111-135."""
    import oracle
    import poisson_caustic_design_gb300 as pcd

    if not oracle.Ref.available():
        pytest.skip("the reference's sources are not on this machine")
    ref = oracle.Ref()
    nx, ny, w, h, th = 150, 120, 0.5, 0.4, 0.1
    rng = np.random.default_rng(11)
    front = np.column_stack([rng.random(nx * ny) * w, rng.random(nx * ny) * h, rng.normal(0, 0.01, nx * ny)])
    back = np.column_stack([rng.random(nx * ny) * w, rng.random(nx * ny) * h, np.zeros(nx * ny)])
    a, b = str(tmp_path / "a.obj"), str(tmp_path / "b.obj")
    pcd.save_solid_obj(front, back, nx, ny, th, w, h, a)
    ref.save_solid_obj(front, back, nx, ny, th, w, h, b)
    assert _read(a) == _read(b)
    c, d = str(tmp_path / "c.svg"), str(tmp_path / "d.svg")
    pcd.export_grid_to_svg(front, w, h, nx, ny, c, 0.5)
    ref.export_grid_svg(front, nx, ny, w, h, d, 0.5)
    assert _read(c) == _read(d)
    hm = rng.normal(0, 0.02, (300, 200))
    e = str(tmp_path / "h.json")
    pcd.save_heightmap_as_json(hm, e)
    assert _read(e).decode() == oracle.heightmap_json_text(hm)
