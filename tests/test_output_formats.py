"""The result writers against the files the reference's own writers make
(tests/golden/ref_output.npz: InversionBase::result2text, result2vtk,
output_obs_data, output_obs_data_vtk on a refined mesh with seeded values):
byte for byte."""
from pathlib import Path

import numpy as np
import pytest

from graada3d_gb300 import output

GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module")
def ref():
    return np.load(GOLDEN / "ref_output.npz")


def _same(path: Path, ref, name: str):
    want = bytes(ref["file:" + name])
    got = path.read_bytes()
    assert got == want, name


def test_model_txt(ref, tmp_path):
    output.write_model_txt(tmp_path / "model.txt", ref["leaf"], ref["m"])
    _same(tmp_path / "model.txt", ref, "model.txt")


def test_model_vtk_and_points(ref, tmp_path):
    params = [("model", ref["m"]), ("m0", ref["m0"]), ("m0s", ref["m0s"])]
    output.write_model_vtk(tmp_path / "model.vtk", ref["leaf"], params)
    output.write_model_vtk_points(tmp_path / "model_points.vtk", ref["leaf"], params)
    _same(tmp_path / "model.vtk", ref, "model.vtk")
    _same(tmp_path / "model_points.vtk", ref, "model_points.vtk")


def test_data_text_and_vtk(ref, tmp_path):
    files = output.write_data(str(tmp_path / "dobs"), ref["obs"], ref["dobs"], int(ref["mask"]))
    assert [Path(f).name for f in files] == ["dobs_g_z", "dobs_T_zz", "dobs_T_xz", "dobs_T_yz",
                                            "dobs_T_xx", "dobs_T_xy"]
    for f in files:
        _same(Path(f), ref, Path(f).name)
    output.write_data_vtk(tmp_path / "dobs.vtk", ref["obs"], ref["dobs"], int(ref["mask"]))
    _same(tmp_path / "dobs.vtk", ref, "dobs.vtk")


def test_vtk_vertices_shared_between_cells(ref):
    """Every cell corner maps to one point; neighbours share theirs (the
    refined mesh's 281 cells have 555 distinct corners, the reference's count)."""
    verts, ids = output._vertex_ids(np.asarray(ref["leaf"]))
    text = bytes(ref["file:model.vtk"]).decode()
    assert f"POINTS\t{verts.shape[0]}\tdouble" in text
    c = np.asarray(ref["leaf"])
    np.testing.assert_array_equal(verts[ids[:, 0]], c[:, [0, 2, 4]])
    np.testing.assert_array_equal(verts[ids[:, 6]], c[:, [1, 3, 5]])


def test_size_errors(ref, tmp_path):
    with pytest.raises(ValueError):
        output.write_model_txt(tmp_path / "x.txt", ref["leaf"], ref["m"][:-1])
    with pytest.raises(ValueError):
        output.write_data(str(tmp_path / "d"), ref["obs"], ref["dobs"][:-1], int(ref["mask"]))
