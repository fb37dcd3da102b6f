"""The persistent CG solve (one cooperative launch per solve_cg, cg_fused.cu)
against the reference's solve_cg (GaussNewtonInversion.cpp:1417-1698, the
compiled reference's fixtures), against its phases run as a graph of four
kernels per iteration (cg_phases.cu, the default for stored G: bitwise the same
solve) and against the generic graph-replayed iteration.  The two device paths sum the dot products and G p's column ranges
in different (each fixed) orders, so they agree to rounding: FP64 to 1e-9 of
max|dx|, reduced-precision G to 1e-4, iteration counts within one (whole L2
inversions: FP64 trial misfits to 1e-6, FP32 to 1e-3).  The
persistent solve is deterministic: repeated solves are bitwise equal.  Also: a
real device-side wait expiry of a grid barrier, and the context afterwards."""
import numpy as np
import pytest

import inversion_fixtures as fx
from conftest import cg_path
from graada3d_gb300 import GradaError
from graada3d_gb300.inversion import GaussNewtonInversion

pytestmark = pytest.mark.gpu


def graph_path():
    return cg_path("0")


def fused_path():
    return cg_path("1")


def phase_path():
    return cg_path("2")


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


def _solve(inv, f, maxit=None):
    maxit = int(f["solve_maxit"]) if maxit is None else maxit
    return inv.solve_cg(float(f["solve_tol"]), maxit, float(f["solve_lambda"]),
                        f["solve_mk"], f["solve_mref"], f["solve_P"], fx.wl_dict(f))


@pytest.mark.parametrize("storage", ["fp64", "fp32", "bf16", "fp16"])
@pytest.mark.parametrize("name", fx.CASES)
def test_phase_kernels_give_the_persistent_solve_bitwise(gpu_ctx, name, storage):
    f = fx.load(name)
    inv = _setup(f, gpu_ctx, storage)
    # the fixture's limit, one that ends inside the first graph replay (odd:
    # the graph then holds maxit iterations) and one past a replay boundary
    for maxit in (None, 5, 17):
        with fused_path():
            dx, err, it = _solve(inv, f, maxit)
        with phase_path():
            dx2, err2, it2 = _solve(inv, f, maxit)
        assert it2 == it and err2 == err and np.array_equal(dx2, dx), maxit


@pytest.mark.parametrize("storage", ["fp64", "fp32", "bf16", "fp16"])
@pytest.mark.parametrize("name", fx.CASES)
def test_fused_solve_cg_matches_graph_path_and_reference(gpu_ctx, name, storage):
    f = fx.load(name)
    inv = _setup(f, gpu_ctx, storage)
    with fused_path():
        dx, err, it = _solve(inv, f)
        dx2, err2, it2 = _solve(inv, f)
    assert it2 == it and err2 == err and np.array_equal(dx2, dx)  # deterministic
    with graph_path():
        dx_g, err_g, it_g = _solve(inv, f)
    assert abs(it - it_g) <= 1
    tol = 1e-9 if storage == "fp64" else 1e-4
    if it == it_g:
        assert np.abs(dx - dx_g).max() <= tol * np.abs(dx_g).max()
    if storage == "fp64":  # the reference's own solve, as the graph path's test checks it
        assert it == int(f["cg_iters"])
        assert np.abs(dx - f["cg_dx"]).max() <= 1e-7 * np.abs(f["cg_dx"]).max()
        assert abs(err - float(f["cg_err"])) <= 1e-5 * abs(float(f["cg_err"]))


@pytest.mark.parametrize("storage", ["fp64", "fp32"])
def test_fused_l2_invert_matches_graph_path(gpu_ctx, storage):
    f = fx.load("l2")
    inv = _setup(f, gpu_ctx, storage)
    nm = inv.Nm
    mmin, mmax, mini = f["bounds"]
    args = (fx.prm(f), np.full(nm, mini), np.full(nm, mmin), np.full(nm, mmax), None)
    with fused_path():
        m, rep = inv.invert(*args, fp64_refinement=storage != "fp64")
    trials = inv.trials()
    with graph_path():
        m_g, rep_g = inv.invert(*args, fp64_refinement=storage != "fp64")
    # FP32 products summed in other orders differ at FP32 rounding, which the
    # lambda search carries on; FP64 ones at FP64 rounding
    rt, mt = (1e-6, 1e-5) if storage == "fp64" else (1e-3, 1e-2)
    assert rep["n_trials"] == rep_g["n_trials"]
    assert np.allclose(trials[:, 2], inv.trials()[:, 2], rtol=rt, atol=0)
    assert np.abs(m - m_g).max() <= mt * np.abs(m_g).max()


def test_fused_barrier_wait_expiry_is_reported_and_context_recovers(gpu_ctx):
    f = fx.load("l2")
    inv = _setup(f, gpu_ctx, "fp32")
    with fused_path():
        dx, err, it = _solve(inv, f)
        FAULT_CG_WAIT = 3  # the next persistent solve's barrier waits have a zero limit
        inv.ctx.check(inv.ctx.lib.grada_inject_fault(inv.ctx.handle, FAULT_CG_WAIT))
        with pytest.raises(GradaError) as e:
            _solve(inv, f)
        assert e.value.status == -2 and "barrier" in str(e.value)
        dx2, err2, it2 = _solve(inv, f)  # same context, normal limits
    assert it2 == it and err2 == err and np.array_equal(dx2, dx)
