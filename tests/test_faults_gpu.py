"""Failure handling without a GPU fault: faults are injected on the host
(grada_inject_fault) and every call reports a status and leaves the context
usable -- a failed device allocation, the expiry flag of a tensor-core wait, a
real expiry of the tensor-core kernels' bounded mbarrier waits (their main-loop
limit set to nothing, the drains kept), non-finite input, empty or malformed
geometry."""
import numpy as np
import pytest

from graada3d_gb300 import GradaError, mesh
from graada3d_gb300.inversion import GaussNewtonInversion

pytestmark = pytest.mark.gpu

FAULT_ALLOC, FAULT_TC_TIMEOUT, FAULT_TC_WAIT = 1, 2, 4
ERR_CUDA, ERR_OOM, ERR_NONFINITE, ERR_INVALID = -2, -3, -5, -1


def _inv(ctx):
    prisms = mesh.regular_mesh((0.0, 2000.0), 8, (0.0, 2000.0), 8, (0.0, 1000.0), 4)
    obs = mesh.observation_grid(10, 0.0, 2000.0, 10, 0.0, 2000.0, -20.0)
    return GaussNewtonInversion(prisms, obs, 0x012, ctx=ctx)


def _status(exc):
    return exc.value.status


def test_injected_allocation_failure_then_recovery():
    from graada3d_gb300 import Context

    ctx = Context(0)  # a fresh context: its first allocation is the one that fails
    try:
        ctx.check(ctx.lib.grada_inject_fault(ctx.handle, FAULT_ALLOC))
        with pytest.raises(GradaError) as e:
            _inv(ctx)
        assert _status(e) == ERR_OOM and "injected" in str(e.value)
        inv = _inv(ctx)  # the next allocation succeeds
        inv.compute_G("fp32")
        assert np.isfinite(inv.G_vec_mul(np.ones(inv.Nm))).all()
    finally:
        ctx.close()


def test_tensor_core_wait_expiry_is_reported_and_cleared(gpu_ctx):
    inv = _inv(gpu_ctx)
    inv.compute_G("bf16")
    X = np.random.default_rng(1).standard_normal((inv.Nm, 16))
    good = inv.G_mat_mul(X)
    gpu_ctx.check(gpu_ctx.lib.grada_inject_fault(gpu_ctx.handle, FAULT_TC_TIMEOUT))
    with pytest.raises(GradaError) as e:
        inv.G_mat_mul(X)
    assert _status(e) == ERR_CUDA and "bounded wait" in str(e.value)
    np.testing.assert_array_equal(inv.G_mat_mul(X), good)  # context usable, same result


@pytest.mark.parametrize("storage", ["bf16", "fp32"])
def test_tensor_core_real_wait_expiry_then_same_product(gpu_ctx, storage):
    inv = _inv(gpu_ctx)
    inv.compute_G(storage)
    X = np.random.default_rng(2).standard_normal((inv.Nm, 16))
    Y = np.random.default_rng(3).standard_normal((inv.Nd, 16))
    good = inv.G_mat_mul(X)
    good_t = inv.GT_mat_mul(Y)
    gpu_ctx.check(gpu_ctx.lib.grada_inject_fault(gpu_ctx.handle, FAULT_TC_WAIT))
    with pytest.raises(GradaError) as e:
        inv.G_mat_mul(X)
    assert _status(e) == ERR_CUDA and "bounded wait" in str(e.value)
    np.testing.assert_array_equal(inv.G_mat_mul(X), good)  # TMEM freed, context usable
    np.testing.assert_array_equal(inv.GT_mat_mul(Y), good_t)


def test_nonfinite_and_malformed_inputs(gpu_ctx):
    inv = _inv(gpu_ctx)
    inv.compute_G("fp64")
    d = np.ones(inv.Nd)
    d[3] = np.nan
    with pytest.raises(GradaError) as e:
        inv.set_dobs(d, np.ones(inv.Nd))
    assert _status(e) == ERR_NONFINITE
    bad = mesh.regular_mesh((0.0, 2000.0), 2, (0.0, 2000.0), 2, (0.0, 1000.0), 2)
    bad[0, 0], bad[0, 1] = bad[0, 1], bad[0, 0]  # x0 > x1
    with pytest.raises(GradaError) as e:
        GaussNewtonInversion(bad, inv.obs, 0x012, ctx=gpu_ctx)
    assert _status(e) == ERR_INVALID
    with pytest.raises(GradaError) as e:
        gpu_ctx.check(gpu_ctx.lib.grada_inject_fault(gpu_ctx.handle, 99))
    assert _status(e) == ERR_INVALID


def test_pending_allocation_fault_can_be_cleared():
    from graada3d_gb300 import Context

    ctx = Context(0)
    try:
        ctx.check(ctx.lib.grada_inject_fault(ctx.handle, FAULT_ALLOC))
        ctx.check(ctx.lib.grada_inject_fault(ctx.handle, 0))  # cleared
        _inv(ctx).compute_G("fp32")
    finally:
        ctx.close()
