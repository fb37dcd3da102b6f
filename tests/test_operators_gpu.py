"""Regularisation operators built on the device (grada_build_operators) from
the face table, against the compiled reference's operators on a refined mesh
(tests/golden/ref_operators.npz) and against the host construction."""
from pathlib import Path

import numpy as np
import pytest
import scipy.sparse as sp

from graada3d_gb300 import GradaError, mesh
from graada3d_gb300 import regularization as reg
from graada3d_gb300.inversion import GaussNewtonInversion

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
# Z = 1 / |zp - zc|^(beta/2): the device's pow and the host C library's may
# differ by two ulps; every other operation is the reference's, in its order
RTOL = 6e-16 * 4


def _ref_csr(f, key):
    n = f["leaf"].shape[0]
    return sp.csr_matrix((f[key + "_data"], f[key + "_indices"], f[key + "_indptr"]), shape=(n, n))


def _close_csr(got, want, rtol):
    got, want = sp.csr_matrix(got), sp.csr_matrix(want)
    want.sort_indices()
    want.eliminate_zeros()
    assert np.array_equal(got.indptr, want.indptr)
    assert np.array_equal(got.indices, want.indices)
    np.testing.assert_allclose(got.data, want.data, rtol=rtol, atol=0)


def test_device_operators_match_reference_on_refined_mesh(gpu_ctx):
    f = np.load(GOLDEN / "ref_operators.npz")
    leaf = f["leaf"]
    inv = GaussNewtonInversion(leaf, f["obs"], 0x002, ctx=gpu_ctx)
    inv.build_operators(reg.face_table(leaf), float(f["beta"]), 0, f["alphas"])
    for key in ("Ws", "Wx", "Wy", "Wz"):
        _close_csr(inv.get_operator(key), _ref_csr(f, key), RTOL)


def _refined_mesh():
    box = [1100.0, 2600.0, 1400.0, 2900.0, 300.0, 1300.0]
    o = mesh.Octree.regular((0.0, 4000.0), 8, (0.0, 4000.0), 8, (0.0, 2000.0), 4)
    for _ in range(2):
        c = o.leaves()
        cross = ((c[:, 0] < box[1]) & (c[:, 1] > box[0]) & (c[:, 2] < box[3]) & (c[:, 3] > box[2])
                 & (c[:, 4] < box[5]) & (c[:, 5] > box[4]))
        o.refine(np.nonzero(cross)[0])
    return o.leaves(), box


def test_device_operators_match_host_and_solve_alike(gpu_ctx):
    """Device-built and host-built operators: the same rows to a few ulps, and
    tolerance-stopped CG solves with either agree (the transposes included)."""
    prisms, box = _refined_mesh()
    obs = mesh.observation_grid(16, 0.0, 4000.0, 16, 0.0, 4000.0, -20.0)
    inv = GaussNewtonInversion(prisms, obs, 0x012, ctx=gpu_ctx)
    alphas = (1.0, 1.3, 0.7, 1.1)
    host = reg.mesh_operators(prisms, obs, 1.5, a_s=alphas[0], a_z=alphas[1], a_x=alphas[2],
                              a_y=alphas[3])
    inv.compute_G("fp64")
    G = inv.get_G()
    rng = np.random.default_rng(7)
    rho = mesh.set_boxes(prisms, [box + [300.0]])
    d = G @ rho
    dobs = d + 0.02 * np.abs(d) * rng.standard_normal(d.size)
    wd = reg.data_weights(dobs, [0.02, 0.02], [1e-3, 1e-2], obs.shape[0])
    inv.set_cross_gradient(False)
    inv.set_dobs(dobs, wd)
    mk = rng.uniform(-100, 100, inv.Nm)
    P = reg.p_diag(mk, -1000.0, 1000.0)
    inv.build_operators(reg.face_table(prisms), 1.5, 0, alphas)
    for key in ("Ws", "Wx", "Wy", "Wz"):
        _close_csr(inv.get_operator(key), host[key], RTOL)
    dev = [inv.solve_cg(1e-4, 400, lam, mk, np.zeros(inv.Nm), P) for lam in (10.0, 0.1)]
    inv.set_operators(host)
    for key in ("Ws", "Wx", "Wy", "Wz"):
        _close_csr(inv.get_operator(key), host[key], 0.0)
    for (dx, err, it), lam in zip(dev, (10.0, 0.1)):
        dxh, errh, ith = inv.solve_cg(1e-4, 400, lam, mk, np.zeros(inv.Nm), P)
        assert it == ith and it < 400
        assert np.abs(dx - dxh).max() <= 1e-10 * np.abs(dxh).max()


def test_device_operators_with_sensitivity_depth_weighting(gpu_ctx):
    """depth_flag 1: Z_ii = sqrt(||G(:, i)|| / Nd) from the device's G."""
    prisms = mesh.regular_mesh((0.0, 2000.0), 6, (0.0, 1500.0), 5, (0.0, 1000.0), 4)
    obs = mesh.observation_grid(7, 0.0, 2000.0, 6, 0.0, 1500.0, -30.0)
    inv = GaussNewtonInversion(prisms, obs, 0x012, ctx=gpu_ctx)
    with pytest.raises(GradaError):  # needs G
        inv.build_operators(reg.face_table(prisms), 1.5, 1)
    inv.compute_G("fp64")
    G = inv.get_G()
    Z = np.sqrt(np.linalg.norm(G, axis=0) / G.shape[0])
    inv.build_operators(reg.face_table(prisms), 1.5, 1)
    host = reg.regular_mesh_operators((6, 5, 4), prisms, obs, 1.5)
    V = host["V"]
    for key, D in (("Ws", sp.identity(inv.Nm, format="csr")), ("Wx", host["Dx"]),
                   ("Wy", host["Dy"]), ("Wz", host["Dz"])):
        want = sp.csr_matrix((sp.diags(V) @ D) @ sp.diags(Z))
        _close_csr(inv.get_operator(key), want, 1e-13)


def test_build_operators_rejects_bad_tables(gpu_ctx):
    prisms = mesh.regular_mesh((0.0, 300.0), 3, (0.0, 200.0), 2, (0.0, 200.0), 2)
    obs = mesh.observation_grid(3, 0.0, 300.0, 2, 0.0, 200.0, -5.0)
    inv = GaussNewtonInversion(prisms, obs, 0x002, ctx=gpu_ctx)
    good = reg.face_table(prisms)
    inv.build_operators(good, 2.0)
    for mutate in (lambda t: t.__setitem__((0, 0, 1), 12),     # neighbour out of range
                   lambda t: t.__setitem__((0, 0, 1), 0),      # itself
                   lambda t: t.__setitem__((1, 1, 0), 2),      # side not in {-1, 0, 1}
                   lambda t: t.__setitem__((2, 2, 3), 5)):     # one neighbour and a stray one
        bad = good.copy()
        mutate(bad)
        with pytest.raises(GradaError):
            inv.build_operators(bad, 2.0)
    with pytest.raises(GradaError):
        inv.build_operators(good, 2.0, depth_flag=2)
    with pytest.raises(ValueError):
        inv.build_operators(good[:-1], 2.0)
