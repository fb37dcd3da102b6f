"""The first Gauss-Newton iteration of the reference's adaptive inversions
(ref_adaptive_*_inversion fixtures, oracle/refdrv/ref_inversion.cpp mode 3),
before any refinement, restated on the CPU: the C oracle's G, the host-built
operators (regularization.mesh_operators, bitwise the reference's on these
meshes), the structure model's T operators, and the NumPy restatement of
invert_with_own_CG (oracle/inversion.py) with one Gauss-Newton iteration.
Its lambda sequence equals the reference's, its first trials agree to 1e-6,
and the iteration's misfit to 1e-6 (plain, cross-gradient) or 1e-4 where the
run starts from the reference model (GaussNewtonInversion.cpp:752-765): there
the later trials' CG solves at small lambda spread at 1e-5 between any two
summation orders."""
import numpy as np
import pytest

from oracle import inversion as oinv
from oracle import prism


@pytest.mark.parametrize("variant", ["", "crg", "pet"])
def test_first_iteration_of_adaptive_fixtures_matches_reference(golden, variant):
    from graada3d_gb300 import mesh
    from graada3d_gb300 import regularization as reg

    f = golden(f"ref_adaptive_{variant}_inversion.npz" if variant else "ref_adaptive_inversion.npz")
    nx, ny, nz = (int(v) for v in f["n"])
    prisms = mesh.regular_mesh(tuple(f["xl"]), nx, tuple(f["yl"]), ny, tuple(f["zl"]), nz)
    mask = int(f["mask"])
    G = prism.compute_G(prisms, f["obs"], mask)
    beta = float(f["beta"])
    alphas = tuple(float(v) for v in f["alphas"][:4])
    ops = reg.mesh_operators(prisms, f["obs"], beta, *alphas)
    wd = reg.data_weights(f["dobs"], f["rel"], f["abs"], f["obs"].shape[0])
    m0s = f["m0s"] if "m0s" in f.files else None
    m0 = f["m0"] if "m0" in f.files else None
    T = None
    if m0s is not None:
        t = reg.cross_gradient_operators(None, prisms, m0s, ops)
        T = (t["Tx"], t["Ty"], t["Tz"])
    prm = {"max_lambda": float(f["max_lambda"]), "n_lambda": int(f["n_lambda"]),
           "rate": float(f["rate"]), "target": float(f["target"]), "stag": float(f["stag"]),
           "cg_tol": float(f["cg_tol"]), "cg_factor": float(f["cg_factor"]), "gn_iter": 1,
           "lp": [int(v) for v in f["lp"]], "eps2": float(f["eps2"]),
           "start_from_reference": m0 is not None}
    nm = prisms.shape[0]
    mmin, mmax, mini = f["bounds"]
    _, _, _, trials, iters = oinv.invert(
        G, f["dobs"], wd, ops["Ws"], ops["Wx"], ops["Wy"], ops["Wz"], prm, np.full(nm, mini),
        np.full(nm, mmin), np.full(nm, mmax), m0, T, float(f["alphas"][4]))
    ref_its, ref_trials = f["ref_iterations"], f["ref_trials"]
    n1 = int(ref_its[0, 1])
    got = np.array([[t[1], t[2]] for t in trials])
    assert len(iters) == 1 and int(iters[0][1]) == n1 and got.shape[0] == n1
    np.testing.assert_allclose(got[:, 0], ref_trials[:n1, 0], rtol=1e-12, atol=0)
    np.testing.assert_allclose(got[:4, 1], ref_trials[:4, 1], rtol=1e-6, atol=0)
    tol = 1e-6 if m0 is None else 1e-4
    np.testing.assert_allclose(got[:, 1], ref_trials[:n1, 1], rtol=tol, atol=0)
    np.testing.assert_allclose(iters[0][2], ref_its[0, 2], rtol=tol, atol=0)
