"""Pin the CPU oracle against the reference's own golden data (no GPU).

* forward_models.npz: the reference's committed noise-free forward fields
  (Examples/Forward_modelling/*/result/data_no_noise, 15 significant digits).
* ref_fields.npz: G blocks from the reference kernels compiled from source.
"""
import numpy as np
import pytest

from graada3d_gb300 import mesh
from oracle import prism


def _model(g, name):
    R = g[f"{name}_region"]
    nx, ny, nz = (int(v) for v in g[f"{name}_n"])
    prisms = mesh.regular_mesh((R[0], R[1]), nx, (R[2], R[3]), ny, (R[4], R[5]), nz)
    rho = mesh.set_boxes(prisms, g[f"{name}_boxes"])
    return prisms, rho


@pytest.mark.parametrize("name", ["model1", "model2", "model3", "test_compute"])
def test_oracle_reproduces_reference_forward_fields(golden, name):
    g = golden("forward_models.npz")
    prisms, rho = _model(g, name)
    nz = rho != 0
    obs = g[f"{name}_obs"]
    want = g[f"{name}_fields"]
    got = prism.forward_field(prisms[nz], rho[nz], obs, int(g[f"{name}_mask"]))
    scale = np.abs(want).max(axis=0)
    err = np.abs(got - want).max(axis=0) / scale
    # the files carry 15 significant digits
    assert err.max() < 5e-14, err


@pytest.mark.parametrize("case", ["random", "coincident", "far", "edges"])
def test_oracle_matches_compiled_reference_kernels(golden, case):
    g = golden("ref_fields.npz")
    pr, ob, G = g[f"{case}_prisms"], g[f"{case}_obs"], g[f"{case}_G"]
    got = prism.compute_G(pr, ob, 0x3FF)
    n = ob.shape[0]
    for k in range(10):
        blk_want = G[k * n:(k + 1) * n]
        blk_got = got[k * n:(k + 1) * n]
        scale = np.abs(blk_want).max()
        assert np.abs(blk_got - blk_want).max() <= 1e-14 * scale, (case, k)


def test_mesh_helpers_follow_reference_order():
    p = mesh.regular_mesh((0.0, 2.0), 2, (0.0, 3.0), 3, (0.0, 1.0), 2)
    # id = i*(ny*nz) + j*nz + k  (Mesh.cpp:830-847)
    assert p.shape == (12, 6)
    np.testing.assert_array_equal(p[1], [0, 1, 0, 1, 0.5, 1.0])
    np.testing.assert_array_equal(p[2], [0, 1, 1, 2, 0.0, 0.5])
    np.testing.assert_array_equal(p[6], [1, 2, 0, 1, 0.0, 0.5])
    ob = mesh.observation_grid(3, 0, 100, 2, 0, 50, -0.1)
    np.testing.assert_array_equal(ob[:4, :2], [[0, 0], [50, 0], [100, 0], [0, 50]])
