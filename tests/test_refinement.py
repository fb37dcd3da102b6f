"""Refinement indicator (AdaptiveInversion::indicator_calculator, AdaptiveInversion.cpp:
108-204) on a mesh refined at six cells: the CPU restatement and the device
kernel against the compiled reference (tests/golden/ref_indicator.npz), bitwise."""
import numpy as np
import pytest

from oracle import refinement


def test_restated_indicator_equals_reference(golden):
    r = golden("ref_indicator.npz")
    got = refinement.indicator(r["m"], r["rowptr"], r["neighbour"], r["area"])
    np.testing.assert_array_equal(got, r["indicator"])


@pytest.mark.gpu
def test_device_indicator_equals_reference(gpu_ctx, golden):
    from graada3d_gb300.inversion import GaussNewtonInversion

    r = golden("ref_indicator.npz")
    obs = np.array([[300.0, 250.0, -1.0]])
    inv = GaussNewtonInversion(r["leaf"], obs, 0x002, ctx=gpu_ctx)
    got = inv.indicator_calculator(r["m"], r["rowptr"], r["neighbour"], r["area"])
    np.testing.assert_array_equal(got, r["indicator"])
