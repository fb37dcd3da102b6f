"""Parity of the GPU inversion path (solve_cg, invert_with_own_CG) with the
reference compiled from source (fixtures) and with the NumPy oracle, through
the C ABI."""
import numpy as np
import pytest

import inversion_fixtures as fx
from graada3d_gb300 import GradaError, mesh
from graada3d_gb300 import regularization as reg
from graada3d_gb300.inversion import GaussNewtonInversion
from oracle import inversion as oinv
from test_inversion_oracle import check_invert_against_reference

pytestmark = pytest.mark.gpu


def _setup(f, ctx, storage="fp64"):
    inv = GaussNewtonInversion(fx.prisms(f), f["obs"], int(f["mask"]), ctx=ctx)
    inv.compute_G(storage)
    ops = {k: fx.csr(f, k) for k in ["Ws", "Wx", "Wy", "Wz"]}
    if fx.has_crg(f):
        ops.update({k: fx.csr(f, k) for k in ["Tx", "Ty", "Tz"]})
        inv.set_cross_gradient(True, float(f["alphas"][4]))
    else:
        inv.set_cross_gradient(False)
    inv.set_operators(ops)
    inv.set_dobs(f["dobs"], f["Wd"])
    return inv


@pytest.mark.parametrize("name", fx.CASES)
def test_gpu_G_matches_reference_G(gpu_ctx, name):
    f = fx.load(name)
    inv = _setup(f, gpu_ctx)
    G = inv.get_G()
    n = f["obs"].shape[0]
    for k in range(G.shape[0] // n):
        blk = slice(k * n, (k + 1) * n)
        assert np.abs(G[blk] - f["G"][blk]).max() <= 1e-9 * np.abs(f["G"][blk]).max()


@pytest.mark.parametrize("name", fx.CASES)
def test_solve_cg_matches_reference(gpu_ctx, name):
    f = fx.load(name)
    inv = _setup(f, gpu_ctx)
    dx, err, it = inv.solve_cg(float(f["solve_tol"]), int(f["solve_maxit"]), float(f["solve_lambda"]),
                               f["solve_mk"], f["solve_mref"], f["solve_P"], fx.wl_dict(f))
    assert it == int(f["cg_iters"])
    ref = f["cg_dx"]
    assert np.abs(dx - ref).max() <= 1e-7 * np.abs(ref).max()
    assert abs(err - float(f["cg_err"])) <= 1e-5 * abs(float(f["cg_err"]))


@pytest.mark.parametrize("name", fx.CASES)
def test_invert_matches_reference(gpu_ctx, name):
    f = fx.load(name)
    inv = _setup(f, gpu_ctx)
    nm = inv.Nm
    mmin, mmax, mini = f["bounds"]
    m0 = f["m0"] if "m0" in f.files else None
    m, rep = inv.invert(fx.prm(f), np.full(nm, mini), np.full(nm, mmin), np.full(nm, mmax), m0)
    trials = [tuple(r) for r in inv.trials()]
    iters = [tuple(r) for r in inv.iterations()]
    assert rep["n_trials"] == len(trials)
    check_invert_against_reference(f, m, rep["final_misfit"], trials, iters)


def _l2_problem(n=(16, 16, 8), nobs=(20, 20), mask=0x012, seed=21):
    prisms = mesh.regular_mesh((0.0, 4000.0), n[0], (0.0, 4000.0), n[1], (0.0, 2000.0), n[2])
    obs = mesh.observation_grid(nobs[0], 0.0, 4000.0, nobs[1], 0.0, 4000.0, -20.0)
    rho = mesh.set_boxes(prisms, [[1000, 2000, 1250, 2500, 500, 1250, 300.0],
                                  [2500, 3500, 500, 1500, 250, 1000, -200.0]])
    return prisms, obs, rho, n, mask, np.random.default_rng(seed)


def test_solve_cg_stops_on_tolerance_like_oracle(gpu_ctx):
    prisms, obs, rho, n, mask, rng = _l2_problem()
    inv = GaussNewtonInversion(prisms, obs, mask, ctx=gpu_ctx)
    inv.compute_G("fp64")
    G = inv.get_G()
    d = G @ rho
    dobs = d + 0.02 * np.abs(d) * rng.standard_normal(d.size)
    wd = reg.data_weights(dobs, [0.02, 0.02], [1e-3, 1e-2], obs.shape[0])
    ops = reg.regular_mesh_operators(n, prisms, obs, 1.5)
    inv.set_cross_gradient(False)
    inv.set_operators(ops)
    inv.set_dobs(dobs, wd)
    mk = rng.uniform(-100, 100, inv.Nm)
    P = reg.p_diag(mk, -1000.0, 1000.0)
    for lam in (10.0, 0.1):
        dx, err, it = inv.solve_cg(1e-4, 200, lam, mk, np.zeros(inv.Nm), P)
        dxo, erro, ito = oinv.solve_cg(1e-4, 200, lam, mk, np.zeros(inv.Nm), wd, dobs, P, G,
                                       ops["Ws"], ops["Wx"], ops["Wy"], ops["Wz"])
        assert it == ito and it < 200
        assert np.abs(dx - dxo).max() <= 1e-8 * np.abs(dxo).max()


def test_invert_l2_matches_oracle_at_2048_cells(gpu_ctx):
    prisms, obs, rho, n, mask, rng = _l2_problem()
    inv = GaussNewtonInversion(prisms, obs, mask, ctx=gpu_ctx)
    inv.compute_G("fp64")
    G = inv.get_G()
    d = G @ rho
    dobs = d + 0.02 * np.abs(d) * rng.standard_normal(d.size)
    wd = reg.data_weights(dobs, [0.02, 0.02], [1e-3, 1e-2], obs.shape[0])
    ops = reg.regular_mesh_operators(n, prisms, obs, 1.5)
    inv.set_cross_gradient(False)
    inv.set_operators(ops)
    inv.set_dobs(dobs, wd)
    prm = dict(max_lambda=1e-1, n_lambda=12, rate=0.6, target=1.0, stag=0.02, cg_tol=1e-6,
               cg_factor=50, gn_iter=3, lp=[2, 2, 2, 2, 2], eps2=1e-9)
    nm = inv.Nm
    m, rep = inv.invert(prm, np.zeros(nm), np.full(nm, -1000.0), np.full(nm, 1000.0))
    mo, misfit_o, lam_o, trials_o, iters_o = oinv.invert(
        G, dobs, wd, ops["Ws"], ops["Wx"], ops["Wy"], ops["Wz"], prm, np.zeros(nm),
        np.full(nm, -1000.0), np.full(nm, 1000.0))
    tr = inv.trials()
    to = np.array(trials_o)
    assert tr.shape[0] == to.shape[0]
    # Gauss-Newton iteration 1 starts both runs from the same model: its trials
    # agree to 1e-6.  Later iterations start from models that carry the
    # rounding differences of 50 unconverged CG steps on an ill-conditioned
    # system (the GPU and NumPy reduce in different orders), amplified by the
    # lambda search; there the agreement is 1e-3.
    first = tr[:, 0] == 1
    np.testing.assert_allclose(tr[first, 1:3], to[first, 1:3], rtol=1e-6)
    np.testing.assert_array_equal(tr[first, 3], to[first, 3])
    np.testing.assert_allclose(tr[:, 1:3], to[:, 1:3], rtol=1e-3)
    assert abs(rep["final_misfit"] - misfit_o) <= 1e-3 * misfit_o
    assert np.linalg.norm(m - mo) <= 1e-3 * np.linalg.norm(mo)


@pytest.mark.parametrize("storage,p,tol", [("fp32", 2, 0.01), ("fp16", 2, 0.02), ("bf16", 2, 0.05),
                                           ("fp32", 1, 0.05), ("fp16", 1, 0.08), ("bf16", 1, 0.10)])
def test_mixed_precision_inversion_close_to_fp64(gpu_ctx, storage, p, tol):
    """Reduced-precision G (with one FP64 matrix-free residual per Gauss-Newton
    iteration) against the all-FP64 run: relative model difference below 1 %
    (FP32) / 5 % (bf16) for L2.  L1 IRLS amplifies any perturbation of the
    CG iterates (weights up to eps^-1/2 ~ 180; the FP64 reference itself
    changes its trial sequence with the OpenMP thread count), so there the
    bounds are 5 % / 10 %.  Every trial of this configuration stops its CG at
    the 50-step cap, and near the target misfit the discrete lambda search
    makes even the all-FP64 run move by ~1 % (model) and ~3 % (final misfit)
    when the data are perturbed at the rounding level (4e-16 relative), so the
    bounds are at least 3 times that measured spread.  A 16-bit G perturbs the
    iterates far more than rounding (bf16 entries carry 2^-9 relative error), and
    the discrete lambda steps (rate 0.6) can then end the search one trial over,
    so the L2 final-misfit bound is also at least the storage's model bound."""
    prisms, obs, rho, n, mask, rng = _l2_problem(mask=0x072)
    inv = GaussNewtonInversion(prisms, obs, mask, ctx=gpu_ctx)
    inv.compute_G("fp64")
    G = inv.get_G()
    d = G @ rho
    dobs = d + 0.02 * np.abs(d) * rng.standard_normal(d.size)
    wd = reg.data_weights(dobs, [0.02] * 4, [1e-3, 1e-2, 1e-2, 1e-2], obs.shape[0])
    ops = reg.regular_mesh_operators(n, prisms, obs, 1.5)
    inv.set_cross_gradient(False)
    inv.set_operators(ops)
    inv.set_dobs(dobs, wd)
    prm = dict(max_lambda=1e-1, n_lambda=12, rate=0.6, target=1.0, stag=0.02, cg_tol=1e-6,
               cg_factor=50, gn_iter=3, lp=[p, p, p, p, 2], eps2=1e-9)
    nm = inv.Nm
    args = (np.zeros(nm), np.full(nm, -1000.0), np.full(nm, 1000.0))
    m64, rep64 = inv.invert(prm, *args)
    f_model = f_misfit = 0.0  # spread of the FP64 run under rounding-level data perturbations
    for s in range(2):
        inv.set_dobs(dobs * (1 + 4e-16 * np.random.default_rng(200 + s).standard_normal(d.size)), wd)
        mp, repp = inv.invert(prm, *args)
        f_model = max(f_model, np.linalg.norm(mp - m64) / np.linalg.norm(m64))
        f_misfit = max(f_misfit, abs(repp["final_misfit"] / rep64["final_misfit"] - 1))
    inv.set_dobs(dobs, wd)
    assert f_model < 0.05 and f_misfit < 0.1  # the comparison stays meaningful
    inv.compute_G(storage)
    mlp, replp = inv.invert(prm, *args, fp64_refinement=True)
    assert replp["fp64_refinements"] >= 1
    rel = np.linalg.norm(mlp - m64) / np.linalg.norm(m64)
    assert rel < max(tol, 3 * f_model), (rel, f_model)
    if p == 2:
        assert abs(replp["final_misfit"] - rep64["final_misfit"]) <= \
            max(0.02, tol, 3 * f_misfit) * rep64["final_misfit"], f_misfit
    else:  # the perturbed L1 run may well end lower; it must not end higher
        assert replp["final_misfit"] <= max(1.05, 1 + 3 * f_misfit) * rep64["final_misfit"]


def test_inversion_error_paths(gpu_ctx):
    prisms, obs, rho, n, mask, rng = _l2_problem(n=(4, 4, 2), nobs=(5, 5))
    inv = GaussNewtonInversion(prisms, obs, mask, ctx=gpu_ctx)
    nm = inv.Nm
    with pytest.raises(GradaError):  # G not assembled
        inv.solve_cg(1e-6, 10, 1.0, np.zeros(nm), np.zeros(nm), np.ones(nm))
    inv.compute_G("fp64")
    with pytest.raises(GradaError):  # no data yet
        inv.solve_cg(1e-6, 10, 1.0, np.zeros(nm), np.zeros(nm), np.ones(nm))
    bad = np.ones(inv.Nd)
    bad[3] = np.nan
    with pytest.raises(GradaError):
        inv.set_dobs(bad, np.ones(inv.Nd))
    # a column index outside the matrix is rejected before any upload
    from graada3d_gb300.fwd import _ptr
    from graada3d_gb300.inversion import _iptr
    rp = np.arange(nm + 1, dtype=np.int32)
    ci = np.arange(nm, dtype=np.int32)
    ci[0] = nm + 5
    v = np.ones(nm)
    st = inv.ctx.lib.grada_set_operator(inv.ctx.handle, 0, nm, nm, _iptr(rp), _iptr(ci), _ptr(v))
    assert st == -1


def _refined_problem(mask=0x012, seed=31):
    """8 x 8 x 4 base over [0, 4 km]^2 x [0, 2 km] refined twice at the boundary
    of a +300 kg/m^3 box (face-balance cascades included), 16 x 16 points."""
    box = [1100.0, 2600.0, 1400.0, 2900.0, 300.0, 1300.0]
    o = mesh.Octree.regular((0.0, 4000.0), 8, (0.0, 4000.0), 8, (0.0, 2000.0), 4)
    for _ in range(2):
        c = o.leaves()
        cross = ((c[:, 0] < box[1]) & (c[:, 1] > box[0]) & (c[:, 2] < box[3]) & (c[:, 3] > box[2])
                 & (c[:, 4] < box[5]) & (c[:, 5] > box[4]))
        inside = ((c[:, 0] >= box[0]) & (c[:, 1] <= box[1]) & (c[:, 2] >= box[2])
                  & (c[:, 3] <= box[3]) & (c[:, 4] >= box[4]) & (c[:, 5] <= box[5]))
        o.refine(np.nonzero(cross & ~inside)[0])
    prisms = o.leaves()
    obs = mesh.observation_grid(16, 0.0, 4000.0, 16, 0.0, 4000.0, -20.0)
    rho = mesh.set_boxes(prisms, [box + [300.0]])
    return prisms, obs, rho, mask, np.random.default_rng(seed)


def _refined_setup(ctx, p_mask=0x012):
    prisms, obs, rho, mask, rng = _refined_problem(mask=p_mask)
    assert np.unique(prisms[:, 1] - prisms[:, 0]).size == 3
    inv = GaussNewtonInversion(prisms, obs, mask, ctx=ctx)
    inv.compute_G("fp64")
    G = inv.get_G()
    d = G @ rho
    dobs = d + 0.02 * np.abs(d) * rng.standard_normal(d.size)
    nf = bin(mask).count("1")
    wd = reg.data_weights(dobs, [0.02] * nf, [1e-3] + [1e-2] * (nf - 1), obs.shape[0])
    ops = reg.mesh_operators(prisms, obs, 1.5)
    assert (np.diff(ops["Wx"].indptr) == 5).any()
    inv.set_cross_gradient(False)
    inv.set_operators(ops)
    inv.set_dobs(dobs, wd)
    return inv, G, dobs, wd, ops, rng


def test_solve_cg_on_refined_mesh_matches_oracle(gpu_ctx):
    """An octree-refined mesh (three cell sizes, faces with four finer
    neighbours): G assembled on the device for its leaves, operators from the
    leaves' geometry; CG solves that stop on their tolerance agree with the
    oracle's to 1e-8."""
    inv, G, dobs, wd, ops, rng = _refined_setup(gpu_ctx)
    mk = rng.uniform(-100, 100, inv.Nm)
    P = reg.p_diag(mk, -1000.0, 1000.0)
    for lam in (10.0, 0.1):
        dx, err, it = inv.solve_cg(1e-4, 400, lam, mk, np.zeros(inv.Nm), P)
        dxo, erro, ito = oinv.solve_cg(1e-4, 400, lam, mk, np.zeros(inv.Nm), wd, dobs, P, G,
                                       ops["Ws"], ops["Wx"], ops["Wy"], ops["Wz"])
        assert it == ito and it < 400
        assert np.abs(dx - dxo).max() <= 1e-8 * np.abs(dxo).max()


@pytest.mark.parametrize("p", [2, 1])
def test_invert_on_refined_mesh_matches_oracle(gpu_ctx, p):
    """The whole inversion on the refined mesh against the oracle's with the
    same operators.  Its CG runs stop at the 50-step cap on a system more
    ill-conditioned than the regular meshes' (cell sizes 125-500 m), so the
    first Gauss-Newton iteration's trial misfits are held to 1e-6 or to three
    times the spread of the GPU run under rounding-level (4e-16) data
    perturbations, whichever is larger."""
    inv, G, dobs, wd, ops, rng = _refined_setup(gpu_ctx)
    prm = dict(max_lambda=1e-1, n_lambda=12, rate=0.6, target=1.0, stag=0.02, cg_tol=1e-6,
               cg_factor=50, gn_iter=3, lp=[p, p, p, p, 2], eps2=1e-9)
    nm = inv.Nm
    args = (np.zeros(nm), np.full(nm, -1000.0), np.full(nm, 1000.0))
    m, rep = inv.invert(prm, *args)
    tr = inv.trials()
    first_g = tr[:, 0] == 1
    spread = 0.0
    for s in range(2):
        inv.set_dobs(dobs * (1 + 4e-16 * np.random.default_rng(300 + s).standard_normal(dobs.size)),
                     wd)
        inv.invert(prm, *args)
        tp = inv.trials()
        k = min(first_g.sum(), (tp[:, 0] == 1).sum())
        spread = max(spread, float(np.max(np.abs(tp[:k, 2] / tr[:k, 2] - 1))))
    mo, misfit_o, lam_o, trials_o, iters_o = oinv.invert(
        G, dobs, wd, ops["Ws"], ops["Wx"], ops["Wy"], ops["Wz"], prm, *args)
    to = np.array(trials_o)
    first_o = to[:, 0] == 1
    k = min(first_g.sum(), first_o.sum())
    np.testing.assert_array_equal(tr[:k, 1], to[:k, 1])  # the same lambdas
    np.testing.assert_allclose(tr[:k, 2], to[:k, 2], rtol=max(1e-6, 3 * spread))
    assert spread < 0.01  # the comparison stays meaningful
    assert rep["final_misfit"] <= 1.1 * misfit_o


def test_result_writers_take_device_results(gpu_ctx, tmp_path):
    """result2text / result2vtk / output_*_data after an inversion on the
    refined mesh: the files carry the inverted model and the device G m in
    the reference's formats (the formats themselves are pinned byte for byte
    on the CPU)."""
    from graada3d_gb300 import output

    inv, G, dobs, wd, ops, rng = _refined_setup(gpu_ctx)
    prm = dict(max_lambda=1e-1, n_lambda=3, rate=0.6, target=1.0, stag=0.02, cg_tol=1e-6,
               cg_factor=20, gn_iter=1, lp=[2] * 5, eps2=1e-9)
    nm = inv.Nm
    m, rep = inv.invert(prm, np.zeros(nm), np.full(nm, -1000.0), np.full(nm, 1000.0))
    base = str(tmp_path / "result")
    inv.result2text(base)
    inv.result2vtk(base)
    inv.output_obs_data(str(tmp_path / "dobs"))
    inv.output_predicted_data(str(tmp_path / "dpre"))
    inv.output_predicted_data_vtk(str(tmp_path / "dpre.vtk"))
    txt = np.loadtxt(base + ".txt", comments="#")
    np.testing.assert_allclose(txt[:, 9], m, rtol=1e-13, atol=1e-300)
    np.testing.assert_allclose(txt[:, :6], inv.prisms, rtol=1e-15, atol=0)
    d = (G @ m).reshape(2, -1)
    for k, name in enumerate(["g_z", "T_zz"]):
        dpre = np.loadtxt(tmp_path / f"dpre_{name}")
        np.testing.assert_allclose(dpre[:, 3], d[k], rtol=1e-12, atol=1e-12 * np.abs(d[k]).max())
    np.testing.assert_allclose(dpre[:, :3], inv.obs, rtol=1e-15, atol=0)
    assert (tmp_path / "dobs_T_zz").read_bytes() == _written(output.write_data, tmp_path, inv.obs,
                                                            dobs, inv.field_flag)
    vtk = (tmp_path / "result.vtk").read_text()
    assert vtk.count("SCALARS ") == 3 and f"CELL_TYPES\t{nm}" in vtk
    assert (tmp_path / "dpre.vtk").read_text().count("SCALARS g_z double 1") == 2


def _written(writer, tmp_path, obs, d, mask):
    writer(str(tmp_path / "again"), obs, d, mask)
    return (tmp_path / "again_T_zz").read_bytes()
