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
