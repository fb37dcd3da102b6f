"""Batched inversions in one persistent launch (grada_invert_batch_persistent):
each problem's whole invert_with_own_CG (GaussNewtonInversion.cpp:657-1103)
runs on a team of CTAs from a device queue, and its model, report and
lambda/misfit record are bitwise those of grada_invert on its own -- for L2,
L1 with the cross-gradient and reference-model terms, and L0 problems, FP64 G
or FP32 G with the FP64 G kept, any team size and the one-team-per-problem
layout (the single runs take the
persistent CG loop too, GRADA_CG_FUSED=1)."""
import numpy as np
import pytest

import inversion_fixtures as fx
from conftest import cg_path
from graada3d_gb300 import Context, GradaError, mesh
from graada3d_gb300 import regularization as reg
from graada3d_gb300.inversion import GaussNewtonInversion, invert_batch_persistent

pytestmark = pytest.mark.gpu

PRM = dict(max_lambda=1e-1, n_lambda=8, rate=0.6, target=1.0, stag=0.02, cg_tol=1e-6,
           cg_factor=30, gn_iter=3, lp=[2, 2, 2, 2, 2], eps2=1e-9)


def _regular(k, storage):
    rng = np.random.default_rng(40 + k)
    nx = int(rng.integers(6, 16))
    nz = max(2, nx // 2)
    no = int(rng.integers(8, 18))
    prisms = mesh.regular_mesh((0.0, 2000.0), nx, (0.0, 2000.0), nx, (0.0, 1000.0), nz)
    obs = mesh.observation_grid(no, 0.0, 2000.0, no, 0.0, 2000.0, -20.0)
    x0, y0 = rng.uniform(200, 1000, 2)
    rho = mesh.set_boxes(prisms, [[x0, x0 + 800, y0, y0 + 800, 0, 1000, rng.uniform(100, 400)]])
    inv = GaussNewtonInversion(prisms, obs, 0x012, ctx=Context(0))
    inv.compute_G("fp64")
    d = inv.G_vec_mul(rho)
    dobs = d * (1 + 0.02 * np.random.default_rng(obs.shape[0]).standard_normal(d.size))
    inv.set_cross_gradient(False)
    inv.set_operators(reg.regular_mesh_operators((nx, nx, nz), prisms, obs, 1.5))
    inv.set_dobs(dobs, reg.data_weights(dobs, [0.02, 0.02], [1e-3, 1e-2], obs.shape[0]))
    _store(inv, storage)
    nm = inv.Nm
    return inv, dict(PRM), (np.zeros(nm), np.full(nm, -1000.0), np.full(nm, 1000.0), None)


def _fixture(name, storage):
    f = fx.load(name)
    inv = GaussNewtonInversion(fx.prisms(f), f["obs"], int(f["mask"]), ctx=Context(0))
    ops = {k: fx.csr(f, k) for k in ["Ws", "Wx", "Wy", "Wz"]}
    if fx.has_crg(f):
        ops.update({k: fx.csr(f, k) for k in ["Tx", "Ty", "Tz"]})
        inv.set_cross_gradient(True, float(f["alphas"][4]))
    else:
        inv.set_cross_gradient(False)
    inv.set_operators(ops)
    inv.set_dobs(f["dobs"], f["Wd"])
    _store(inv, storage)
    nm = inv.Nm
    mmin, mmax, mini = f["bounds"]
    m0 = f["m0"] if "m0" in f.files else None
    return inv, fx.prm(f), (np.full(nm, mini), np.full(nm, mmin), np.full(nm, mmax), m0)


def _store(inv, storage):
    if storage == "fp64":
        inv.compute_G("fp64")
    else:
        inv.compute_G(storage, keep_fp64=True)


def _problems(storage):
    probs = [_regular(k, storage) for k in range(4)]
    probs += [_fixture(name, storage) for name in fx.CASES]
    return probs


def _singles(probs, mixed):
    # the batch runs the persistent CG loop for every storage, FP64 included
    out = []
    with cg_path("1"):
        for inv, prm, (mi, lo, hi, m0) in probs:
            m, rep = inv.invert(prm, mi, lo, hi, m0, fp64_refinement=mixed)
            out.append((m, rep, inv.trials(), inv.iterations()))
    return out


def _batch(probs, mixed, team):
    invs = [p[0] for p in probs]
    res, shape = invert_batch_persistent(invs, [p[1] for p in probs], [p[2][0] for p in probs],
                                         [p[2][1] for p in probs], [p[2][2] for p in probs],
                                         [p[2][3] for p in probs], fp64_refinement=mixed,
                                         team_ctas=team)
    return res, shape


@pytest.mark.parametrize("storage", ["fp64", "fp32"])
def test_persistent_batch_equals_single_inversions(storage):
    mixed = storage != "fp64"
    probs = _problems(storage)
    single = _singles(probs, mixed)
    for team in (1, 3, 16, -1):  # -1: one team per problem, sized by its G
        res, (teams, per) = _batch(probs, mixed, team)
        assert per == team and teams >= 1
        if team < 0:
            assert teams == len(probs)
        for k, ((m, rep), (m1, rep1, tr1, it1)) in enumerate(zip(res, single)):
            assert np.array_equal(m, m1), (storage, team, k)
            assert rep == rep1, (storage, team, k)
            assert np.array_equal(probs[k][0].trials(), tr1), (storage, team, k)
            assert np.array_equal(probs[k][0].iterations(), it1), (storage, team, k)
    for inv, *_ in probs:
        inv.ctx.close()


def test_persistent_batch_rejects_storage_without_fp64_predictions():
    inv, prm, (mi, lo, hi, m0) = _regular(0, "fp64")
    inv.compute_G("fp32")  # no kept FP64 G
    with pytest.raises(GradaError) as e:
        invert_batch_persistent([inv], [prm], [mi], [lo], [hi], [m0], fp64_refinement=True)
    assert e.value.status == -4 and "FP64" in str(e.value)
    inv.ctx.close()


def test_persistent_batch_barrier_expiry_reported_then_recovers():
    probs = [_regular(k, "fp64") for k in range(3)]
    first, _ = _batch(probs, False, 4)
    ctx0 = probs[0][0].ctx
    ctx0.check(ctx0.lib.grada_inject_fault(ctx0.handle, 3))  # zero wait limit on the next launch
    with pytest.raises(GradaError) as e:
        _batch(probs, False, 4)
    assert e.value.status == -2 and "barrier" in str(e.value)
    again, _ = _batch(probs, False, 4)
    for (m1, r1), (m2, r2) in zip(first, again):
        assert np.array_equal(m1, m2) and r1 == r2
    for inv, *_ in probs:
        inv.ctx.close()
