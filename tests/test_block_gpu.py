"""Blocks of right-hand sides on one G: the block products (tensor cores for
FP32 / 16-bit G, FP64 pipe for FP64 G, one prism evaluation per pair for
matrix-free G), the block CG solve and the fixed-lambda sweep, each checked
column by column against the single-vector entry points that reproduce the
reference (Fwd::G_vec_mul / GT_vec_mul, solve_cg, invert_with_own_CG)."""
import numpy as np
import pytest

from graada3d_gb300 import mesh
from graada3d_gb300 import regularization as reg
from graada3d_gb300.inversion import GaussNewtonInversion

pytestmark = pytest.mark.gpu

# Block product vs the single-vector product of the same stored G, relative
# to max |result|.  Both accumulate in FP32 over hundreds of terms (~sqrt(n)
# * 2^-24 of the result each), so FP32 G agrees to ~1e-5: 3xTF32 on both
# operands vs FP32 CUDA-core products.  16-bit G: the right-hand side split
# into two 16-bit parts (~22 bits for fp16, ~16 for bf16) vs FP32.
TOL_BLOCK = {"fp64": 1e-13, "fp32": 2e-5, "fp16": 2e-5, "bf16": 1e-4, "matrix_free": 1e-12}


def _geometry(n=(12, 10, 6), nobs=(15, 13), mask=0x012):
    prisms = mesh.regular_mesh((0.0, 3000.0), n[0], (0.0, 2500.0), n[1], (0.0, 1500.0), n[2])
    obs = mesh.observation_grid(nobs[0], 0.0, 3000.0, nobs[1], 0.0, 2500.0, -30.0)
    return prisms, obs, n, mask


@pytest.mark.parametrize("storage", ["fp64", "fp32", "bf16", "fp16", "matrix_free"])
@pytest.mark.parametrize("mask", [0x012, 0x3FE])
@pytest.mark.parametrize("nrhs", [16, 5, 21])
def test_block_products_match_single_products(gpu_ctx, storage, mask, nrhs):
    if storage == "matrix_free" and nrhs == 21 and mask == 0x3FE:
        pytest.skip("covered by the 16- and 5-column cases")
    prisms, obs, n, _ = _geometry(mask=mask)
    inv = GaussNewtonInversion(prisms, obs, mask, ctx=gpu_ctx)
    inv.compute_G(storage)
    rng = np.random.default_rng(7 + nrhs)
    X = rng.standard_normal((inv.Nm, nrhs)) * rng.uniform(0.1, 100.0, nrhs)
    Y = rng.standard_normal((inv.Nd, nrhs)) * rng.uniform(0.1, 100.0, nrhs)
    GX = inv.G_mat_mul(X)
    GTY = inv.GT_mat_mul(Y)
    tol = TOL_BLOCK[storage]
    for c in range(nrhs):
        y1 = inv.G_vec_mul(X[:, c])
        x1 = inv.GT_vec_mul(Y[:, c])
        assert np.abs(GX[:, c] - y1).max() <= tol * np.abs(y1).max(), (storage, c)
        assert np.abs(GTY[:, c] - x1).max() <= tol * np.abs(x1).max(), (storage, c)


@pytest.mark.parametrize("storage", ["fp32", "bf16", "fp16"])
def test_tensor_core_products_against_fp64_G(gpu_ctx, storage):
    """Absolute quality: the block product of a low-precision G against the
    FP64 product, within the storage's own rounding."""
    prisms, obs, n, mask = _geometry(n=(20, 18, 9), nobs=(23, 21))
    inv = GaussNewtonInversion(prisms, obs, mask, ctx=gpu_ctx)
    inv.compute_G("fp64")
    rng = np.random.default_rng(11)
    X = rng.standard_normal((inv.Nm, 16))
    Y = rng.standard_normal((inv.Nd, 16))
    ref_gx, ref_gty = inv.G_mat_mul(X), inv.GT_mat_mul(Y)
    inv.compute_G(storage)
    gx, gty = inv.G_mat_mul(X), inv.GT_mat_mul(Y)
    tol = {"fp32": 1e-5, "fp16": 2e-3, "bf16": 1e-2}[storage]
    assert np.abs(gx - ref_gx).max() <= tol * np.abs(ref_gx).max()
    assert np.abs(gty - ref_gty).max() <= tol * np.abs(ref_gty).max()


def _inversion_problem(ctx, storage="fp64", mask=0x012, n=(12, 12, 6), nobs=(15, 15)):
    prisms = mesh.regular_mesh((0.0, 3000.0), n[0], (0.0, 3000.0), n[1], (0.0, 1500.0), n[2])
    obs = mesh.observation_grid(nobs[0], 0.0, 3000.0, nobs[1], 0.0, 3000.0, -30.0)
    rho = mesh.set_boxes(prisms, [[750, 1750, 1000, 2000, 250, 1000, 250.0],
                                  [2000, 2750, 250, 1250, 250, 750, -150.0]])
    inv = GaussNewtonInversion(prisms, obs, mask, ctx=ctx)
    inv.compute_G("fp64")
    d = inv.G_vec_mul(rho)
    dobs = d + 0.02 * np.abs(d) * np.random.default_rng(4).standard_normal(d.size)
    wd = reg.data_weights(dobs, [0.02, 0.02], [1e-3, 1e-2], obs.shape[0])
    if storage != "fp64":
        inv.compute_G(storage)
    inv.set_cross_gradient(False)
    inv.set_operators(reg.regular_mesh_operators(n, prisms, obs, 1.5))
    inv.set_dobs(dobs, wd)
    return inv, rho


@pytest.mark.parametrize("storage", ["fp64", "fp32"])
def test_solve_cg_block_matches_single_solves(gpu_ctx, storage):
    inv, rho = _inversion_problem(gpu_ctx, storage)
    nm = inv.Nm
    rng = np.random.default_rng(5)
    ncol = 16
    lam = np.logspace(-3, 1, ncol)
    mk = rng.uniform(-50, 50, (nm, ncol))
    P = rng.uniform(100, 500, (nm, ncol))
    WL = {k: rng.uniform(0.5, 2.0, (nm, ncol)) for k in ["s", "x", "z"]}
    WL["y"] = None
    mref = rng.uniform(-10, 10, nm)
    dx, err, it = inv.solve_cg_block(1e-6, 40, lam, mk, mref, P, WL)
    for c in range(ncol):
        wl1 = {k: (None if v is None else v[:, c]) for k, v in WL.items()}
        dx1, err1, it1 = inv.solve_cg(1e-6, 40, lam[c], mk[:, c], mref, P[:, c], wl1)
        if storage == "fp64":
            assert it[c] == it1
            assert np.abs(dx[:, c] - dx1).max() <= 1e-8 * np.abs(dx1).max()
            assert abs(err[c] - err1) <= 1e-6 * err1
        else:  # different summation order in FP32: the iterates drift slowly
            assert abs(it[c] - it1) <= 2
            assert np.linalg.norm(dx[:, c] - dx1) <= 1e-3 * np.linalg.norm(dx1)


def test_solve_cg_block_zero_rhs_column(gpu_ctx):
    """A column whose right-hand side vanishes (no data signal, m at the
    reference) is solved by dx = 0 while the others iterate."""
    prisms, obs, n, mask = _geometry(n=(10, 10, 5), nobs=(12, 12))
    inv = GaussNewtonInversion(prisms, obs, mask, ctx=gpu_ctx)
    inv.compute_G("fp64")
    inv.set_cross_gradient(False)
    inv.set_operators(reg.regular_mesh_operators(n, prisms, obs, 1.5))
    inv.set_dobs(np.zeros(inv.Nd), np.ones(inv.Nd))
    nm = inv.Nm
    mk = np.zeros((nm, 3))
    mk[:, 1] = np.random.default_rng(2).uniform(-20, 20, nm)
    dx, err, it = inv.solve_cg_block(1e-8, 30, [0.1, 0.1, 1.0], mk, np.zeros(nm),
                                     np.full((nm, 3), 200.0))
    assert np.all(dx[:, 0] == 0.0) and it[0] == 0
    assert np.all(dx[:, 2] == 0.0) and it[2] == 0
    assert it[1] > 0 and np.abs(dx[:, 1]).max() > 0


def _prm(lp, gn=4):
    return dict(max_lambda=1e-1, n_lambda=1, rate=0.6, target=1.0, stag=0.02, cg_tol=1e-6,
                cg_factor=40, gn_iter=gn, lp=[lp] * 5, eps2=1e-9)


def _rounding_floor(inv, prm, args, m1, rep1, t1, n=3):
    """How far the single inversion itself moves when the data are perturbed at
    the rounding level (4e-16 relative): relative change of the first-trial
    misfit, of every trial misfit, of the final misfit and of the model (max
    over n perturbations).  Where the CG stops at its iteration cap on a weakly
    regularised system the iterates carry the rounding differences amplified
    many orders of magnitude; a different summation order (block vs single
    products) is a perturbation of the same kind."""
    d0, w0 = inv.dobs.copy(), inv.wd.copy()
    first = trials = final = model = 0.0
    for s in range(n):
        inv.set_dobs(d0 * (1 + 4e-16 * np.random.default_rng(100 + s).standard_normal(d0.size)), w0)
        m, rep = inv.invert(prm, *args)
        t = inv.trials()
        first = max(first, abs(t[0, 2] / t1[0, 2] - 1))
        if t.shape == t1.shape:
            trials = max(trials, (np.abs(t[:, 2] / t1[:, 2] - 1)).max())
        else:
            trials = np.inf
        final = max(final, abs(rep["final_misfit"] / rep1["final_misfit"] - 1))
        model = max(model, np.linalg.norm(m - m1) / max(np.linalg.norm(m1), 1.0))
    inv.set_dobs(d0, w0)
    return first, trials, final, model


@pytest.mark.parametrize("lp", [2, 1])
def test_lambda_sweep_matches_fixed_lambda_inversions(gpu_ctx, lp):
    """Column c of the sweep is grada_invert with n_lambda = 1 and max_lambda =
    lambda_c.  The block and the single products sum in different orders
    (1e-16 relative).  Where the CG converges the two agree to 1e-7; on the
    weakly regularised column (lambda = 1e-3) the CG stops at its 40-step cap
    and the difference is amplified like any rounding-level perturbation, so
    there it is bounded by 20 times the single inversion's own spread under
    data perturbed by 4e-16 (measured).  L1 IRLS weights ((Wm)^2 + 1e-9)^(-1/4)
    amplify it further in later Gauss-Newton iterations, so later trials are
    compared loosely for p = 1."""
    inv, rho = _inversion_problem(gpu_ctx, "fp64")
    nm = inv.Nm
    lam = np.logspace(-3, 1, 16)
    args = (np.zeros(nm), np.full(nm, -1000.0), np.full(nm, 1000.0))
    models, reps = inv.lambda_sweep(_prm(lp), lam, *args)
    cap = _prm(lp)["cg_factor"]
    for c in [0, 5, 10, 15]:
        prm = dict(_prm(lp), max_lambda=float(lam[c]))
        m1, rep1 = inv.invert(prm, *args)
        t1 = inv.trials()
        tb = inv.sweep_trials(c)
        np.testing.assert_allclose(tb[0, 1], t1[0, 1], rtol=0, atol=0)  # lambda
        assert tb[0, 3] == t1[0, 3]  # CG iterations of the first trial
        if t1[0, 3] < cap:
            f_first, f_trials, f_final, f_model = 0.0, 0.0, 0.0, 0.0
        else:
            f_first, f_trials, f_final, f_model = _rounding_floor(inv, prm, args, m1, rep1, t1)
            assert f_first < 1e-3  # the problem stays meaningful
        np.testing.assert_allclose(tb[0, 2], t1[0, 2], rtol=max(1e-7, 20 * f_first))
        assert reps[c]["final_lambda"] == rep1["final_lambda"]
        if lp == 2:
            assert reps[c]["gn_iterations"] == rep1["gn_iterations"]
            assert tb.shape == t1.shape
            np.testing.assert_allclose(tb[:, 2], t1[:, 2], rtol=max(1e-6, 20 * f_trials))
            assert abs(reps[c]["final_misfit"] - rep1["final_misfit"]) <= \
                max(1e-6, 20 * f_final) * rep1["final_misfit"]
            assert np.linalg.norm(models[:, c] - m1) <= \
                max(1e-5, 20 * f_model) * max(np.linalg.norm(m1), 1.0)
        else:
            assert abs(reps[c]["gn_iterations"] - rep1["gn_iterations"]) <= 1
            assert abs(reps[c]["final_misfit"] - rep1["final_misfit"]) <= 0.1 * rep1["final_misfit"]


def test_lambda_sweep_more_than_sixteen_and_mixed_precision(gpu_ctx):
    inv, rho = _inversion_problem(gpu_ctx, "fp32")
    nm = inv.Nm
    lam = np.logspace(-3, 1, 18)
    args = (np.zeros(nm), np.full(nm, -1000.0), np.full(nm, 1000.0))
    models, reps = inv.lambda_sweep(_prm(2, gn=3), lam, *args, fp64_refinement=True)
    assert models.shape == (nm, 18)
    assert all(r["fp64_refinements"] >= 1 for r in reps)
    for c in [3, 17]:
        m1, rep1 = inv.invert(dict(_prm(2, gn=3), max_lambda=float(lam[c])), *args,
                              fp64_refinement=True)
        assert abs(reps[c]["final_misfit"] - rep1["final_misfit"]) <= 1e-3 * rep1["final_misfit"]
        assert np.linalg.norm(models[:, c] - m1) <= 1e-3 * max(np.linalg.norm(m1), 1.0)


def test_lambda_sweep_matrix_free_matches_stored(gpu_ctx):
    inv, rho = _inversion_problem(gpu_ctx, "fp64", n=(10, 10, 5), nobs=(12, 12))
    nm = inv.Nm
    lam = np.logspace(-2, 0, 4)
    args = (np.zeros(nm), np.full(nm, -1000.0), np.full(nm, 1000.0))
    m64, r64 = inv.lambda_sweep(_prm(2, gn=2), lam, *args)
    inv.compute_G("matrix_free")
    mmf, rmf = inv.lambda_sweep(_prm(2, gn=2), lam, *args)
    for c in range(4):
        assert abs(rmf[c]["final_misfit"] - r64[c]["final_misfit"]) <= 1e-8 * r64[c]["final_misfit"]
        assert np.linalg.norm(mmf[:, c] - m64[:, c]) <= 1e-8 * max(np.linalg.norm(m64[:, c]), 1.0)


@pytest.mark.parametrize("storage", ["fp64", "fp32", "bf16", "fp16", "matrix_free"])
def test_block_products_tiny_problem(gpu_ctx, storage):
    """3 cells, 2 points: one tensor-core tile mostly out of bounds (zero-filled),
    a single assembly tile, 3 right-hand sides."""
    prisms = mesh.regular_mesh((0.0, 300.0), 3, (0.0, 100.0), 1, (0.0, 100.0), 1)
    obs = np.array([[50.0, 50.0, -10.0], [250.0, 40.0, -20.0]])
    inv = GaussNewtonInversion(prisms, obs, 0x3FE, ctx=gpu_ctx)
    inv.compute_G(storage)
    rng = np.random.default_rng(2)
    X = rng.standard_normal((inv.Nm, 3))
    Y = rng.standard_normal((inv.Nd, 3))
    GX, GTY = inv.G_mat_mul(X), inv.GT_mat_mul(Y)
    tol = TOL_BLOCK[storage]
    for c in range(3):
        y1, x1 = inv.G_vec_mul(X[:, c]), inv.GT_vec_mul(Y[:, c])
        assert np.abs(GX[:, c] - y1).max() <= tol * np.abs(y1).max()
        assert np.abs(GTY[:, c] - x1).max() <= tol * np.abs(x1).max()
