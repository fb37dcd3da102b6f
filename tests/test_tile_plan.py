"""The assembly tile plan (build_tile_plan in assemble.cu, host code) on CPU:
every cell exactly once and every face the walk takes over shared exactly, for
regular, odd-sized, shuffled, tall and refined meshes.  A small C++ checker
(tests/tile_plan_check.cpp) is built against the in-tree library."""
import shutil
import subprocess

import numpy as np
import pytest

from conftest import REPO

pytestmark = pytest.mark.skipif(shutil.which("g++") is None, reason="no C++ compiler")


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    from graada3d_gb300.build import build_library

    lib = build_library()
    exe = tmp_path_factory.mktemp("plan") / "tile_plan_check"
    subprocess.run(["g++", "-O2", "-std=c++17", str(REPO / "tests" / "tile_plan_check.cpp"),
                    "-o", str(exe), f"-L{lib.parent}", "-lgrada_gpu", f"-Wl,-rpath,{lib.parent}"],
                   check=True)
    return exe


def _run(checker, tmp_path, cells):
    path = tmp_path / "cells.bin"
    with open(path, "wb") as f:
        np.array([len(cells)], np.int64).tofile(f)
        np.ascontiguousarray(cells, np.float64).tofile(f)
    res = subprocess.run([str(checker), str(path)], capture_output=True, text=True)
    assert res.returncode == 0, res.stdout + res.stderr
    v = res.stdout.split()
    return {"tiles": int(v[3]), "z": float(v[7]), "y": float(v[9]), "x": float(v[11])}


def _refined(levels):
    from graada3d_gb300 import mesh
    from graada3d_gb300.fwd import split_cells

    cells = mesh.regular_mesh((0.0, 10000.0), 16, (0.0, 10000.0), 16, (0.0, 5000.0), 8)
    box = [2500, 3500, 1000, 9000, 500, 3500]
    for _ in range(levels):
        inter = ((cells[:, 0] < box[1]) & (cells[:, 1] > box[0]) & (cells[:, 2] < box[3]) &
                 (cells[:, 3] > box[2]) & (cells[:, 4] < box[5]) & (cells[:, 5] > box[4]))
        inside = ((cells[:, 0] >= box[0]) & (cells[:, 1] <= box[1]) & (cells[:, 2] >= box[2]) &
                  (cells[:, 3] <= box[3]) & (cells[:, 4] >= box[4]) & (cells[:, 5] <= box[5]))
        idx = np.nonzero(inter & ~inside)[0]
        kids = split_cells(cells[idx])
        keep = np.ones(len(cells), bool)
        keep[idx] = False
        cells = np.vstack([cells[keep], kids.reshape(-1, 6)])
    return cells


def test_regular_mesh_tiles_are_2x4(checker, tmp_path):
    from graada3d_gb300 import mesh

    s = _run(checker, tmp_path, mesh.regular_mesh((0, 3000.), 24, (0, 2500.), 20, (0, 1500.), 12))
    assert s["tiles"] == 60  # 12 x-pairs x 5 y-quads, 12 levels
    # shares printed to 4 decimals
    assert s["z"] == pytest.approx(11 / 12, abs=1e-4) and s["y"] == pytest.approx(0.75, abs=1e-4)
    assert s["x"] == pytest.approx(0.5, abs=1e-4)


@pytest.mark.parametrize("shape", ["odd_shuffled", "tall", "refined_shuffled"])
def test_irregular_meshes(checker, tmp_path, shape):
    from graada3d_gb300 import mesh

    rng = np.random.default_rng(3)
    if shape == "odd_shuffled":
        cells = mesh.regular_mesh((0, 1300.), 13, (0, 1100.), 11, (0, 700.), 7)
        cells = cells[rng.permutation(len(cells))]
    elif shape == "tall":
        cells = mesh.regular_mesh((0, 50.), 3, (0, 50.), 1, (0, 1300.), 130)
    else:
        cells = _refined(2)
        cells = cells[rng.permutation(len(cells))]
    s = _run(checker, tmp_path, cells)
    assert s["z"] > 0.8
    if shape != "tall":
        assert s["y"] > 0.5 and s["x"] > 0.3
