"""FP64 G kept beside a reduced-precision G (grada_keep_fp64_G): the reduced
entries are bitwise those of the direct assembly, and mixed-precision
inversions predict the data with FP64 products of the kept G."""
import numpy as np
import pytest

from graada3d_gb300 import mesh
from graada3d_gb300 import regularization as reg
from graada3d_gb300.inversion import GaussNewtonInversion

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("storage", ["fp32", "bf16", "fp16"])
def test_reduced_entries_from_kept_fp64_are_bitwise_the_direct_ones(gpu_ctx, storage):
    prisms = mesh.regular_mesh((0.0, 3000.0), 14, (0.0, 2500.0), 11, (0.0, 1500.0), 7)
    obs = mesh.observation_grid(13, 0.0, 3000.0, 12, 0.0, 2500.0, -30.0)
    inv = GaussNewtonInversion(prisms, obs, 0x3FE, ctx=gpu_ctx)
    inv.compute_G(storage)
    direct = inv.get_G()
    x = np.random.default_rng(1).standard_normal(inv.Nm)
    y_direct = inv.G_vec_mul(x)
    inv.compute_G(storage, keep_fp64=True)
    kept = inv.get_G()
    assert np.array_equal(direct.view(np.uint64), kept.view(np.uint64))
    assert np.array_equal(y_direct, inv.G_vec_mul(x))


def _problem(ctx, n=(16, 16, 8), nobs=(20, 20), mask=0x072, seed=21):
    prisms = mesh.regular_mesh((0.0, 4000.0), n[0], (0.0, 4000.0), n[1], (0.0, 2000.0), n[2])
    obs = mesh.observation_grid(nobs[0], 0.0, 4000.0, nobs[1], 0.0, 4000.0, -20.0)
    rho = mesh.set_boxes(prisms, [[1000, 2000, 1250, 2500, 500, 1250, 300.0],
                                  [2500, 3500, 500, 1500, 250, 1000, -200.0]])
    inv = GaussNewtonInversion(prisms, obs, mask, ctx=ctx)
    inv.compute_G("fp64")
    G64 = inv.get_G()
    rng = np.random.default_rng(seed)
    d = G64 @ rho
    dobs = d + 0.02 * np.abs(d) * rng.standard_normal(d.size)
    nf = bin(mask).count("1")
    wd = reg.data_weights(dobs, [0.02] * nf, [1e-3] + [1e-2] * (nf - 1), obs.shape[0])
    inv.set_cross_gradient(False)
    inv.set_operators(reg.regular_mesh_operators(n, prisms, obs, 1.5))
    inv.set_dobs(dobs, wd)
    return inv, G64, dobs, wd


def _misfit(G64, m, dobs, wd):
    return float(np.sqrt(np.mean((wd * (dobs - G64 @ m)) ** 2)))


@pytest.mark.parametrize("storage,p", [("fp32", 2), ("fp32", 1), ("bf16", 2)])
def test_inversion_with_kept_fp64_predicts_in_fp64(gpu_ctx, storage, p):
    """The reported misfits are FP64 misfits of the reduced-precision run's own
    models (to rounding), every prediction being an FP64 product; the model
    stays as close to the all-FP64 run as the reference-form mixed run."""
    inv, G64, dobs, wd = _problem(gpu_ctx)
    prm = dict(max_lambda=1e-1, n_lambda=12, rate=0.6, target=1.0, stag=0.02, cg_tol=1e-6,
               cg_factor=50, gn_iter=3, lp=[p, p, p, p, 2], eps2=1e-9)
    nm = inv.Nm
    args = (np.zeros(nm), np.full(nm, -1000.0), np.full(nm, 1000.0))
    m64, rep64 = inv.invert(prm, *args)
    f_model = 0.0  # spread of the FP64 run under rounding-level data perturbations
    for s in range(2):
        inv.set_dobs(dobs * (1 + 4e-16 * np.random.default_rng(400 + s).standard_normal(dobs.size)),
                     wd)
        mp, _ = inv.invert(prm, *args)
        f_model = max(f_model, np.linalg.norm(mp - m64) / np.linalg.norm(m64))
    inv.set_dobs(dobs, wd)
    inv.compute_G(storage, keep_fp64=True)
    m, rep = inv.invert(prm, *args, fp64_refinement=True)
    trials = inv.trials()
    # one FP64 product for the start misfit, one per CG right-hand side and one
    # per trial misfit
    assert rep["fp64_refinements"] == 1 + 2 * rep["n_trials"]
    np.testing.assert_allclose(rep["final_misfit"], _misfit(G64, m, dobs, wd), rtol=1e-12)
    assert trials.shape[0] == rep["n_trials"]
    tol = {2: 0.01, 1: 0.05}[p] if storage == "fp32" else 0.05
    rel = np.linalg.norm(m - m64) / np.linalg.norm(m64)
    assert rel < max(tol, 3 * f_model), (rel, f_model)


def test_sweep_with_kept_fp64_matches_fixed_lambda_inversions(gpu_ctx):
    """Columns of the sweep equal grada_invert with the same lambda, both
    predicting with the kept FP64 G: first-trial misfits agree to the CG's
    rounding (block vs single products), the first trial's lambda exactly."""
    inv, G64, dobs, wd = _problem(gpu_ctx, mask=0x012)
    inv.compute_G("fp32", keep_fp64=True)
    prm = dict(max_lambda=1e-1, n_lambda=1, rate=0.6, target=1.0, stag=0.02, cg_tol=1e-6,
               cg_factor=40, gn_iter=3, lp=[2] * 5, eps2=1e-9)
    nm = inv.Nm
    args = (np.zeros(nm), np.full(nm, -1000.0), np.full(nm, 1000.0))
    lam = np.logspace(-1, 1, 16)
    models, reps = inv.lambda_sweep(prm, lam, *args, fp64_refinement=True)
    for c in [0, 8, 15]:
        m1, rep1 = inv.invert(dict(prm, max_lambda=float(lam[c])), *args, fp64_refinement=True)
        t1, tb = inv.trials(), inv.sweep_trials(c)
        assert tb[0, 1] == t1[0, 1]
        np.testing.assert_allclose(tb[0, 2], t1[0, 2], rtol=1e-5)
        assert reps[c]["fp64_refinements"] > 0
        np.testing.assert_allclose(reps[c]["final_misfit"], _misfit(G64, models[:, c], dobs, wd),
                                   rtol=1e-10)
