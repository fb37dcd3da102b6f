"""Pin the NumPy inversion oracle and the host-side helpers against the
reference compiled from source (fixtures in tests/golden/ref_inversion_*.npz).
No GPU."""
import numpy as np
import pytest

import inversion_fixtures as fx
from oracle import inversion as oinv
from oracle import prism


@pytest.mark.parametrize("name", fx.CASES)
def test_reference_G_matches_oracle_kernels(name):
    f = fx.load(name)
    G = prism.compute_G(fx.prisms(f), f["obs"], int(f["mask"]))
    assert np.abs(G - f["G"]).max() <= 1e-13 * np.abs(f["G"]).max()


@pytest.mark.parametrize("name", fx.CASES)
def test_solve_cg_oracle_matches_reference(name):
    f = fx.load(name)
    T = (fx.csr(f, "Tx"), fx.csr(f, "Ty"), fx.csr(f, "Tz")) if fx.has_crg(f) else None
    dx, err, it = oinv.solve_cg(float(f["solve_tol"]), int(f["solve_maxit"]), float(f["solve_lambda"]),
                                f["solve_mk"], f["solve_mref"], f["Wd"], f["dobs"], f["solve_P"],
                                f["G"], fx.csr(f, "Ws"), fx.csr(f, "Wx"), fx.csr(f, "Wy"),
                                fx.csr(f, "Wz"), T, float(f["alphas"][4]), None, fx.wl_dict(f))
    assert it == int(f["cg_iters"])
    ref = f["cg_dx"]
    assert np.abs(dx - ref).max() <= 1e-7 * np.abs(ref).max()
    assert abs(err - float(f["cg_err"])) <= 1e-5 * abs(float(f["cg_err"]))


@pytest.mark.parametrize("name", fx.CASES)
def test_invert_oracle_matches_reference(name):
    f = fx.load(name)
    T = (fx.csr(f, "Tx"), fx.csr(f, "Ty"), fx.csr(f, "Tz")) if fx.has_crg(f) else None
    nm = f["G"].shape[1]
    mmin, mmax, mini = f["bounds"]
    m0 = f["m0"] if "m0" in f.files else None
    m, misfit, lam, trials, iters = oinv.invert(
        f["G"], f["dobs"], f["Wd"], fx.csr(f, "Ws"), fx.csr(f, "Wx"), fx.csr(f, "Wy"),
        fx.csr(f, "Wz"), fx.prm(f), np.full(nm, mini), np.full(nm, mmin), np.full(nm, mmax), m0, T,
        float(f["alphas"][4]))
    check_invert_against_reference(f, m, misfit, trials, iters)


def check_invert_against_reference(f, m, misfit, trials, iters):
    """L2: the whole run matches (lambda sequence, every trial misfit, the
    final model).  p < 2: the IRLS weights (v^2 + eps^2)^((p-2)/4) with
    eps^2 = 1e-9 reach eps^-1/2 ~ 180 (L1) and eps^-1 ~ 3e4 (L0) times the
    others, so rounding differences grow from trial to trial; the reference
    itself gives different trial sequences from the 7th trial on when only
    its OpenMP thread count changes (1, 3 or 8 threads).  There the first
    six trials (before any reweighted system has been solved twice) must
    match, and the run must end in the same state: misfit below target, or
    the same stopping misfit within 50 %."""
    ref_trials = f["inv_trials"]
    got = np.array([[t[1], t[2]] for t in trials])
    l2 = all(int(p) == 2 for p in f["lp"])
    if l2:
        assert len(trials) == ref_trials.shape[0]
        np.testing.assert_allclose(got, ref_trials, rtol=1e-6)
        np.testing.assert_allclose([it[2] for it in iters], f["inv_iterations"][:, 2], rtol=1e-6)
        assert abs(misfit - float(f["inv_misfit"])) <= 1e-6 * float(f["inv_misfit"])
        assert np.abs(m - f["inv_m"]).max() <= 1e-5 * np.abs(f["inv_m"]).max()
        return
    k = min(6, len(trials), ref_trials.shape[0])
    np.testing.assert_allclose(got[:k], ref_trials[:k], rtol=1e-5)
    ref_misfit = float(f["inv_misfit"])
    target = float(f["target"])
    if ref_misfit < target:
        assert misfit < target * 1.5
    else:
        assert abs(misfit - ref_misfit) <= 0.5 * ref_misfit


@pytest.mark.parametrize("name", fx.CASES)
def test_host_operators_match_reference(name):
    """The host-side operator builder for regular meshes reproduces the
    reference's Ws/Wx/Wy/Wz (and T) matrices."""
    from graada3d_gb300 import regularization as reg

    f = fx.load(name)
    pr = fx.prisms(f)
    a = f["alphas"]
    ops = reg.regular_mesh_operators(tuple(int(v) for v in f["n"]), pr, f["obs"], float(f["beta"]),
                                     a_s=a[0], a_z=a[1], a_x=a[2], a_y=a[3])
    for key in ["Ws", "Wx", "Wy", "Wz"]:
        want = fx.csr(f, key).toarray()
        got = ops[key].toarray()
        assert np.abs(got - want).max() <= 1e-14 * np.abs(want).max(), key
    if fx.has_crg(f):
        T = reg.cross_gradient_operators(tuple(int(v) for v in f["n"]), pr, f["m0s"], ops)
        for key in ["Tx", "Ty", "Tz"]:
            want = fx.csr(f, key).toarray()
            assert np.abs(T[key].toarray() - want).max() <= 1e-12 * np.abs(want).max(), key
    wd = reg.data_weights(f["dobs"], f["rel"], f["abs"], f["obs"].shape[0])
    np.testing.assert_array_equal(wd, f["Wd"])
