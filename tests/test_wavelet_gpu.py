"""The wavelet-compressed G on the device (grada_compute_G_wavelet) against
the oracle's restatement of Fwd::compute_G_wavelet and the wavelet products,
on the device's own FP64 G: the same kept coefficients, bitwise, and bitwise
products (the oracle reproduces the device's summation orders)."""
import numpy as np
import pytest

from graada3d_gb300 import GradaError, mesh
from graada3d_gb300 import regularization as reg
from graada3d_gb300.inversion import GaussNewtonInversion
from oracle import inversion as oinv
from oracle import wavelet as wv

pytestmark = pytest.mark.gpu


def _regular():
    o = mesh.Octree.regular((0.0, 3000.0), 12, (0.0, 2500.0), 10, (0.0, 1500.0), 6)
    obs = mesh.observation_grid(15, 0.0, 3000.0, 12, 0.0, 2500.0, -25.0)
    return o, obs


def _refined():
    box = [1100.0, 2600.0, 1400.0, 2900.0, 300.0, 1300.0]
    o = mesh.Octree.regular((0.0, 4000.0), 8, (0.0, 4000.0), 8, (0.0, 2000.0), 4)
    for _ in range(2):
        c = o.leaves()
        cross = ((c[:, 0] < box[1]) & (c[:, 1] > box[0]) & (c[:, 2] < box[3]) & (c[:, 3] > box[2])
                 & (c[:, 4] < box[5]) & (c[:, 5] > box[4]))
        o.refine(np.nonzero(cross)[0])
    obs = mesh.observation_grid(12, 0.0, 4000.0, 12, 0.0, 4000.0, -20.0)
    return o, obs


@pytest.mark.parametrize("case,rel,batch,values", [
    ("regular", 5e-4, None, "fp64"), ("regular", 0.0, None, "fp64"),
    ("refined", 5e-4, None, "fp64"), ("refined", 1e-2, None, "fp64"),
    ("regular", 5e-4, 7, "fp64"), ("refined", 5e-4, 50, "fp64"),
    ("regular", 5e-4, None, "fp32"), ("refined", 5e-4, 9, "fp32")])
def test_wavelet_rows_and_products_match_oracle(gpu_ctx, monkeypatch, case, rel, batch, values):
    """batch: observation points per assembly batch of the compression (the
    rows of a batch interleave with other batches' in G's row order); values:
    the kept coefficients' storage."""
    if batch is not None:
        monkeypatch.setenv("GRADA_WAVELET_BATCH_POINTS", str(batch))
    o, obs = _regular() if case == "regular" else _refined()
    prisms, order = o.leaves(), o.wavelet_order()
    inv = GaussNewtonInversion(prisms, obs, 0x012, ctx=gpu_ctx)
    inv.compute_G("fp64")
    Gd = inv.get_G()
    comp = wv.compress(Gd, order, rel, fp32=values == "fp32")
    inv.compute_G_wavelet(order, rel, values)
    n_dy, rp, cols, vals = inv.get_wavelet_G()
    assert n_dy == comp[0]
    np.testing.assert_array_equal(rp, comp[1])
    np.testing.assert_array_equal(cols, comp[2])
    np.testing.assert_array_equal(vals.view(np.uint64), comp[3].view(np.uint64))
    rng = np.random.default_rng(11)
    x, y = rng.standard_normal(inv.Nm), rng.standard_normal(inv.Nd)
    np.testing.assert_array_equal(inv.G_vec_mul(x), wv.G_vec_mul(comp, order, x))
    np.testing.assert_array_equal(inv.GT_vec_mul(y), wv.GT_vec_mul(comp, order, y))
    if rel == 0.0:  # nothing dropped: the dense products to rounding
        np.testing.assert_allclose(inv.G_vec_mul(x), Gd @ x, rtol=0,
                                   atol=1e-12 * np.abs(Gd @ x).max())
        np.testing.assert_allclose(inv.GT_vec_mul(y), Gd.T @ y, rtol=0,
                                   atol=1e-12 * np.abs(Gd.T @ y).max())
    else:
        assert cols.size < Gd.shape[0] * n_dy
        err = np.linalg.norm(inv.G_vec_mul(x) - Gd @ x) / np.linalg.norm(Gd @ x)
        assert err < 50 * rel


class _WaveletOp:
    """G @ x and G.T @ y through the oracle's compressed rows."""

    def __init__(self, comp, order, transpose=False):
        self.comp, self.order, self.t = comp, order, transpose

    @property
    def T(self):
        return _WaveletOp(self.comp, self.order, not self.t)

    def __matmul__(self, v):
        if self.t:
            return wv.GT_vec_mul(self.comp, self.order, v)
        return wv.G_vec_mul(self.comp, self.order, v)


def test_solve_cg_with_wavelet_G_matches_oracle(gpu_ctx):
    """solve_cg on the compressed rows (the reference's method_id 2) against the
    oracle's solve_cg driving the oracle's compressed products."""
    o, obs = _refined()
    prisms, order = o.leaves(), o.wavelet_order()
    inv = GaussNewtonInversion(prisms, obs, 0x012, ctx=gpu_ctx)
    inv.compute_G("fp64")
    Gd = inv.get_G()
    rho = mesh.set_boxes(prisms, [[1100.0, 2600.0, 1400.0, 2900.0, 300.0, 1300.0, 300.0]])
    rng = np.random.default_rng(12)
    d = Gd @ rho
    dobs = d + 0.02 * np.abs(d) * rng.standard_normal(d.size)
    wd = reg.data_weights(dobs, [0.02, 0.02], [1e-3, 1e-2], obs.shape[0])
    ops = reg.mesh_operators(prisms, obs, 1.5)
    comp = wv.compress(Gd, order, 5e-4)
    inv.compute_G_wavelet(order, 5e-4)
    inv.set_cross_gradient(False)
    inv.set_operators(ops)
    inv.set_dobs(dobs, wd)
    mk = rng.uniform(-100, 100, inv.Nm)
    P = reg.p_diag(mk, -1000.0, 1000.0)
    op = _WaveletOp(comp, order)
    for lam in (10.0, 0.1):
        dx, err, it = inv.solve_cg(1e-4, 400, lam, mk, np.zeros(inv.Nm), P)
        dxo, erro, ito = oinv.solve_cg(1e-4, 400, lam, mk, np.zeros(inv.Nm), wd, dobs, P, op,
                                       ops["Ws"], ops["Wx"], ops["Wy"], ops["Wz"])
        assert it == ito and it < 400
        assert np.abs(dx - dxo).max() <= 1e-8 * np.abs(dxo).max()


def test_wavelet_G_errors(gpu_ctx):
    o, obs = _regular()
    prisms, order = o.leaves(), o.wavelet_order()
    inv = GaussNewtonInversion(prisms, obs, 0x002, ctx=gpu_ctx)
    bad = order.copy()
    bad[3] = bad[4]
    with pytest.raises(GradaError):
        inv.compute_G_wavelet(bad, 1e-3)
    with pytest.raises(GradaError):
        inv.compute_G_wavelet(order, -1.0)
    with pytest.raises(GradaError):  # not compressed yet
        inv.get_wavelet_G()
    inv.compute_G_wavelet(order, 1e-3)
    with pytest.raises(GradaError):  # the dense G is gone, as in the reference
        inv.get_G()
    inv.compute_G("fp32")  # back to a stored G
    assert inv.get_G().shape == (inv.Nd, inv.Nm)
