"""Concurrent batches of independent problems (many contexts, one host thread
and one stream each) give exactly what the single calls give."""
import numpy as np
import pytest

from graada3d_gb300 import Context, mesh
from graada3d_gb300 import regularization as reg
from graada3d_gb300.inversion import GaussNewtonInversion, compute_G_batch, invert_batch

pytestmark = pytest.mark.gpu


def _problems(n=5, seed=30):
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        nx = int(rng.integers(6, 14))
        nz = max(2, nx // 2)
        no = int(rng.integers(8, 16))
        prisms = mesh.regular_mesh((0.0, 2000.0), nx, (0.0, 2000.0), nx, (0.0, 1000.0), nz)
        obs = mesh.observation_grid(no, 0.0, 2000.0, no, 0.0, 2000.0, -20.0)
        x0, y0 = rng.uniform(200, 1000, 2)
        rho = mesh.set_boxes(prisms, [[x0, x0 + 800, y0, y0 + 800, 0, 1000, rng.uniform(100, 400)]])
        assert np.any(rho != 0)
        out.append((prisms, obs, rho, (nx, nx, nz)))
    return out


def test_batched_inversions_equal_single_runs():
    probs = _problems()
    prm = dict(max_lambda=1e-1, n_lambda=8, rate=0.6, target=1.0, stag=0.02, cg_tol=1e-6,
               cg_factor=30, gn_iter=2, lp=[2, 2, 2, 2, 2], eps2=1e-9)
    invs, args = [], []
    for prisms, obs, rho, n in probs:
        inv = GaussNewtonInversion(prisms, obs, 0x012, ctx=Context(0))
        inv.compute_G("fp64")
        d = inv.G_vec_mul(rho)
        dobs = d * (1 + 0.02 * np.random.default_rng(obs.shape[0]).standard_normal(d.size))
        inv.set_cross_gradient(False)
        inv.set_operators(reg.regular_mesh_operators(n, prisms, obs, 1.5))
        inv.set_dobs(dobs, reg.data_weights(dobs, [0.02, 0.02], [1e-3, 1e-2], obs.shape[0]))
        invs.append(inv)
        nm = inv.Nm
        args.append((np.zeros(nm), np.full(nm, -1000.0), np.full(nm, 1000.0)))
    single = [inv.invert(prm, *a) for inv, a in zip(invs, args)]
    compute_G_batch(invs, "fp64")  # re-assemble all at once: same G
    batch = invert_batch(invs, [prm] * len(invs), [a[0] for a in args], [a[1] for a in args],
                         [a[2] for a in args], max_threads=3)
    for (m1, r1), (m2, r2) in zip(single, batch):
        assert np.array_equal(m1, m2)
        assert r1["final_misfit"] == r2["final_misfit"] and r1["n_trials"] == r2["n_trials"]
    for inv in invs:
        inv.ctx.close()
