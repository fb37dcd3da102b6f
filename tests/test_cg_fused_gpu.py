"""The persistent CG solve (one cooperative launch per solve_cg, cg_fused.cu)
against the graph-replayed iteration it replaces: both run the same blocks with
the same summation orders, so dx, the iteration count and err are bitwise
equal, for every stored G; and whole inversions (invert_with_own_CG,
GaussNewtonInversion.cpp:657-1103, which calls solve_cg per lambda trial)
give bitwise the same model and lambda/misfit record.  Also: a real
device-side wait expiry of a grid barrier, and the context afterwards."""
import os

import numpy as np
import pytest

import inversion_fixtures as fx
from graada3d_gb300 import GradaError
from graada3d_gb300.inversion import GaussNewtonInversion

pytestmark = pytest.mark.gpu


class graph_path:
    """Selects the graph-replayed CG path (GRADA_CG_FUSED=0) inside the block."""

    def __enter__(self):
        self.old = os.environ.get("GRADA_CG_FUSED")
        os.environ["GRADA_CG_FUSED"] = "0"

    def __exit__(self, *exc):
        if self.old is None:
            os.environ.pop("GRADA_CG_FUSED", None)
        else:
            os.environ["GRADA_CG_FUSED"] = self.old


def _setup(f, ctx, storage):
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


def _solve(inv, f):
    return inv.solve_cg(float(f["solve_tol"]), int(f["solve_maxit"]), float(f["solve_lambda"]),
                        f["solve_mk"], f["solve_mref"], f["solve_P"], fx.wl_dict(f))


@pytest.mark.parametrize("storage", ["fp64", "fp32", "bf16", "fp16"])
@pytest.mark.parametrize("name", fx.CASES)
def test_fused_solve_cg_bitwise_equal_to_graph_path(gpu_ctx, name, storage):
    f = fx.load(name)
    inv = _setup(f, gpu_ctx, storage)
    dx, err, it = _solve(inv, f)
    with graph_path():
        dx_g, err_g, it_g = _solve(inv, f)
    assert it == it_g
    assert err == err_g
    assert np.array_equal(dx, dx_g)
    if storage == "fp64":  # and the reference's own solve (same check as the graph path's test)
        assert it == int(f["cg_iters"])
        assert np.abs(dx - f["cg_dx"]).max() <= 1e-7 * np.abs(f["cg_dx"]).max()


@pytest.mark.parametrize("storage", ["fp64", "fp32"])
@pytest.mark.parametrize("name", fx.CASES)
def test_fused_invert_bitwise_equal_to_graph_path(gpu_ctx, name, storage):
    f = fx.load(name)
    inv = _setup(f, gpu_ctx, storage)
    nm = inv.Nm
    mmin, mmax, mini = f["bounds"]
    m0 = f["m0"] if "m0" in f.files else None
    args = (fx.prm(f), np.full(nm, mini), np.full(nm, mmin), np.full(nm, mmax), m0)
    m, rep = inv.invert(*args, fp64_refinement=storage != "fp64")
    trials = inv.trials()
    with graph_path():
        m_g, rep_g = inv.invert(*args, fp64_refinement=storage != "fp64")
    assert np.array_equal(m, m_g)
    assert np.array_equal(trials, inv.trials())
    assert rep["cg_iterations"] == rep_g["cg_iterations"]


def test_fused_barrier_wait_expiry_is_reported_and_context_recovers(gpu_ctx):
    f = fx.load("l2")
    inv = _setup(f, gpu_ctx, "fp32")
    dx, err, it = _solve(inv, f)
    FAULT_CG_WAIT = 3  # the next solve's barrier waits have a zero limit
    inv.ctx.check(inv.ctx.lib.grada_inject_fault(inv.ctx.handle, FAULT_CG_WAIT))
    with pytest.raises(GradaError) as e:
        _solve(inv, f)
    assert e.value.status == -2 and "barrier" in str(e.value)
    dx2, err2, it2 = _solve(inv, f)  # same context, normal limits
    assert it2 == it and err2 == err and np.array_equal(dx2, dx)
