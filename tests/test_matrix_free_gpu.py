"""Matrix-free mode (G larger than HBM): every product re-evaluates the prism
kernels in FP64.  It must agree with the stored FP64 G, product for product
and through a full inversion."""
import numpy as np
import pytest

from graada3d_gb300 import mesh
from graada3d_gb300 import regularization as reg
from graada3d_gb300.inversion import GaussNewtonInversion

pytestmark = pytest.mark.gpu


def _problem(mask=0x012):
    prisms = mesh.regular_mesh((0.0, 3000.0), 12, (0.0, 3000.0), 12, (0.0, 1500.0), 6)
    obs = mesh.observation_grid(15, 0.0, 3000.0, 15, 0.0, 3000.0, -30.0)
    rho = mesh.set_boxes(prisms, [[750, 1750, 1000, 2000, 250, 1000, 250.0]])
    return prisms, obs, rho, (12, 12, 6), mask


@pytest.mark.parametrize("mask", [0x012, 0x3FE, 0x3FF])
def test_matrix_free_products_match_stored_G(gpu_ctx, mask):
    prisms, obs, rho, n, _ = _problem()
    inv = GaussNewtonInversion(prisms, obs, mask, ctx=gpu_ctx)
    inv.compute_G("fp64")
    rng = np.random.default_rng(3)
    x = rng.standard_normal(inv.Nm)
    y = rng.standard_normal(inv.Nd)
    d, r = inv.G_vec_mul(x), inv.GT_vec_mul(y)
    inv.compute_G("matrix_free")
    d_mf, r_mf = inv.G_vec_mul(x), inv.GT_vec_mul(y)
    assert np.abs(d_mf - d).max() <= 1e-12 * np.abs(d).max()
    assert np.abs(r_mf - r).max() <= 1e-12 * np.abs(r).max()


def test_matrix_free_inversion_matches_stored_G(gpu_ctx):
    prisms, obs, rho, n, mask = _problem()
    inv = GaussNewtonInversion(prisms, obs, mask, ctx=gpu_ctx)
    inv.compute_G("fp64")
    d = inv.G_vec_mul(rho)
    dobs = d + 0.02 * np.abs(d) * np.random.default_rng(4).standard_normal(d.size)
    wd = reg.data_weights(dobs, [0.02, 0.02], [1e-3, 1e-2], obs.shape[0])
    inv.set_cross_gradient(False)
    inv.set_operators(reg.regular_mesh_operators(n, prisms, obs, 1.5))
    inv.set_dobs(dobs, wd)
    prm = dict(max_lambda=1e-1, n_lambda=10, rate=0.6, target=1.0, stag=0.02, cg_tol=1e-6,
               cg_factor=40, gn_iter=2, lp=[2, 2, 2, 2, 2], eps2=1e-9)
    nm = inv.Nm
    args = (np.zeros(nm), np.full(nm, -1000.0), np.full(nm, 1000.0))
    m64, rep64 = inv.invert(prm, *args)
    t64 = inv.trials()
    inv.compute_G("matrix_free")
    mmf, repmf = inv.invert(prm, *args, fp64_refinement=True)
    tmf = inv.trials()
    assert repmf["fp64_refinements"] == 0  # the products are FP64 already
    first = t64[:, 0] == 1
    assert tmf.shape == t64.shape
    np.testing.assert_allclose(tmf[first, 1:3], t64[first, 1:3], rtol=1e-6)
    np.testing.assert_allclose(tmf[:, 2], t64[:, 2], rtol=1e-3)
    assert np.linalg.norm(mmf - m64) <= 1e-3 * np.linalg.norm(m64)


def test_matrix_free_expand_then_products(gpu_ctx):
    prisms, obs, rho, n, mask = _problem()
    inv = GaussNewtonInversion(prisms, obs, mask, ctx=gpu_ctx)
    inv.compute_G("matrix_free")
    inv.expand_G([5, 40, 863])
    x = np.random.default_rng(5).standard_normal(inv.Nm)
    d_mf = inv.G_vec_mul(x)
    ref = GaussNewtonInversion(inv.prisms, obs, mask)
    ref.compute_G("fp64")
    d = ref.G_vec_mul(x)
    assert np.abs(d_mf - d).max() <= 1e-12 * np.abs(d).max()
    ref.ctx.close()


def test_matrix_free_joint_constraint_inversion(gpu_ctx):
    """The constraint mix of the large matrix-free case at a small size: L1
    IRLS, cross-gradient coupling to a smooth structure model and a reference
    model.  The first Gauss-Newton iteration's trials equal the stored-FP64
    run's (every product is FP64 either way); later ones are chaotic under
    L1 IRLS and are only required to stay close."""
    prisms, obs, rho, n, mask = _problem()
    inv = GaussNewtonInversion(prisms, obs, mask, ctx=gpu_ctx)
    inv.compute_G("fp64")
    d = inv.G_vec_mul(rho)
    dobs = d + 0.02 * np.abs(d) * np.random.default_rng(8).standard_normal(d.size)
    wd = reg.data_weights(dobs, [0.02, 0.02], [1e-3, 1e-2], obs.shape[0])
    ops = reg.regular_mesh_operators(n, prisms, obs, 1.5)
    c = prisms.reshape(-1, 6)
    xc, yc, zc = (c[:, 0] + c[:, 1]) / 2, (c[:, 2] + c[:, 3]) / 2, (c[:, 4] + c[:, 5]) / 2
    m0s = 200.0 * np.exp(-((xc - 1500) ** 2 + (yc - 1500) ** 2 + (zc - 600) ** 2) / 2000.0 ** 2)
    m0 = 0.5 * m0s
    ops.update(reg.cross_gradient_operators(n, prisms, m0s, ops))
    inv.set_operators(ops)
    inv.set_cross_gradient(True, 1.0)
    inv.set_dobs(dobs, wd)
    prm = dict(max_lambda=1e-1, n_lambda=6, rate=0.6, target=1.0, stag=0.02, cg_tol=1e-6,
               cg_factor=30, gn_iter=2, lp=[1, 1, 1, 1, 2], eps2=1e-9)
    nm = inv.Nm
    args = (np.zeros(nm), np.full(nm, -1000.0), np.full(nm, 1000.0), m0)
    m64, rep64 = inv.invert(prm, *args)
    t64 = inv.trials()
    inv.compute_G("matrix_free")
    mmf, repmf = inv.invert(prm, *args)
    tmf = inv.trials()
    first = (t64[:, 0] == 1) & (np.arange(len(t64)) < 3)
    np.testing.assert_allclose(tmf[: first.sum(), 1:3], t64[first, 1:3], rtol=1e-6)
    assert abs(repmf["final_misfit"] - rep64["final_misfit"]) <= 0.05 * rep64["final_misfit"]
    inv.set_cross_gradient(False)
