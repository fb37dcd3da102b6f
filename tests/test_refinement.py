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


def test_indicator_pairs_from_geometry_equal_reference(golden):
    """regularization.indicator_pairs builds the reference's (neighbour, area)
    list from the cells alone, in its order, bitwise."""
    from graada3d_gb300 import regularization as reg

    r = golden("ref_indicator.npz")
    rp, nb, ar = reg.indicator_pairs(r["leaf"])
    np.testing.assert_array_equal(rp, r["rowptr"])
    np.testing.assert_array_equal(nb, r["neighbour"])
    np.testing.assert_array_equal(ar.view(np.uint64), r["area"].view(np.uint64))


def test_refine_mesh_steps_equal_reference(golden):
    """One AdaptiveInversion::refine_mesh of the reference (ref_adapt.npz): the
    indicator over the geometric pairs, the marks (fraction, minimum sizes), the
    octree split and the model the children inherit all equal the reference's."""
    from graada3d_gb300 import mesh
    from graada3d_gb300 import regularization as reg
    from graada3d_gb300.adaptive import refinement_marks

    f = golden("ref_adapt.npz")
    o = mesh.Octree.regular((0.0, 600.0), 6, (0.0, 500.0), 5, (0.0, 400.0), 4)
    pts, c = f["pre_points"], o.leaves()
    inside = ((pts[None, :, 0] > c[:, None, 0]) & (pts[None, :, 0] < c[:, None, 1])
              & (pts[None, :, 1] > c[:, None, 2]) & (pts[None, :, 1] < c[:, None, 3])
              & (pts[None, :, 2] > c[:, None, 4]) & (pts[None, :, 2] < c[:, None, 5]))
    o.refine(np.nonzero(inside.any(1))[0])
    assert np.array_equal(o.leaves().view(np.uint64), f["leaf0"].view(np.uint64))
    ind = refinement.indicator(f["m0"], *reg.indicator_pairs(f["leaf0"]))
    np.testing.assert_array_equal(ind, f["indicator"])
    marks = refinement_marks(ind, f["leaf0"], float(f["fraction"]), f["min_size"])
    assert marks.size > 0
    n0 = f["leaf0"].shape[0]
    split = o.refine(marks)
    assert np.array_equal(o.leaves().view(np.uint64), f["leaf1"].view(np.uint64))
    np.testing.assert_array_equal(f["m0"][o.parent_leaf(split, n0)], f["m1"])
    # nothing to do for a fraction below one cell
    assert refinement_marks(ind, f["leaf0"], 0.1 / n0, f["min_size"]).size == 0
    assert refinement_marks(ind, f["leaf0"], -1.0, f["min_size"]).size == 0


@pytest.mark.gpu
def test_device_refine_mesh_step(gpu_ctx, golden):
    """adaptive.refine_mesh on the device: the same leaves and inherited model
    as the reference's refine_mesh, G expanded to the re-assembled G of the new
    cells, the operators rebuilt to the host construction's."""
    from graada3d_gb300 import adaptive, mesh
    from graada3d_gb300 import regularization as reg
    from graada3d_gb300.inversion import GaussNewtonInversion

    f = golden("ref_adapt.npz")
    o = mesh.Octree.regular((0.0, 600.0), 6, (0.0, 500.0), 5, (0.0, 400.0), 4)
    pts, c = f["pre_points"], o.leaves()
    inside = ((pts[None, :, 0] > c[:, None, 0]) & (pts[None, :, 0] < c[:, None, 1])
              & (pts[None, :, 1] > c[:, None, 2]) & (pts[None, :, 1] < c[:, None, 3])
              & (pts[None, :, 2] > c[:, None, 4]) & (pts[None, :, 2] < c[:, None, 5]))
    o.refine(np.nonzero(inside.any(1))[0])
    obs = np.array([[300.0, 250.0, -10.0], [120.0, 400.0, -15.0]])
    inv = GaussNewtonInversion(o.leaves(), obs, 0x012, ctx=gpu_ctx)
    inv.compute_G("fp64")
    m1, = adaptive.refine_mesh(inv, o, f["m0"], float(f["fraction"]), f["min_size"], 1.5)
    assert np.array_equal(inv.prisms.view(np.uint64), f["leaf1"].view(np.uint64))
    np.testing.assert_array_equal(m1, f["m1"])
    G_exp = inv.get_G()
    inv.compute_G("fp64")
    np.testing.assert_array_equal(G_exp, inv.get_G())
    host = reg.mesh_operators(inv.prisms, obs, 1.5)
    for key in ("Ws", "Wx", "Wy", "Wz"):
        got, want = inv.get_operator(key), host[key]
        assert np.array_equal(got.indices, want.indices)
        np.testing.assert_allclose(got.data, want.data, rtol=2.4e-15, atol=0)


def test_refinement_marks_rules():
    """refine_mesh's rule (AdaptiveInversion.cpp:639-683): strictly above the
    int(fraction Nm)-th largest indicator; a cell any of whose sizes is at (to
    1e-7) or below the minimum is never split."""
    from graada3d_gb300.adaptive import refinement_marks

    cells = np.array([[0, 10, 0, 10, 0, 10], [10, 20, 0, 10, 0, 10], [20, 25, 0, 5, 0, 5],
                      [25, 30, 0, 5, 0, 5], [30, 40, 0, 10, 0, 10.00000005]], dtype=float)
    ind = np.array([5.0, 4.0, 9.0, 1.0, 8.0])
    # fraction 0.4 of 5 cells: tol = 3rd largest = 5.0, so indicators 9 and 8 qualify
    np.testing.assert_array_equal(refinement_marks(ind, cells, 0.4, (1.0, 1.0, 1.0)), [2, 4])
    # minimum 5: cell 2 (5 m) is at the minimum
    np.testing.assert_array_equal(refinement_marks(ind, cells, 0.4, (5.0, 5.0, 5.0)), [4])
    # minimum 10.00000005 in z: cell 4 is within 1e-7 of it
    np.testing.assert_array_equal(refinement_marks(ind, cells, 0.4, (1.0, 1.0, 10.00000005)), [])
    # ties at the threshold are not split
    np.testing.assert_array_equal(refinement_marks(np.ones(5), cells, 0.4, (1, 1, 1)), [])


def test_parent_leaf_maps_children_into_their_parents():
    from graada3d_gb300 import mesh

    rng = np.random.default_rng(5)
    o = mesh.Octree.regular((0.0, 400.0), 4, (0.0, 300.0), 3, (0.0, 200.0), 2)
    for _ in range(3):
        old = o.leaves()
        split = o.refine(rng.choice(old.shape[0], size=old.shape[0] // 5, replace=False))
        new = o.leaves()
        parent = o.parent_leaf(split, old.shape[0])
        assert parent.size == new.shape[0] == old.shape[0] + 7 * split.size
        p = old[parent]
        assert np.all(new[:, 0::2] >= p[:, 0::2]) and np.all(new[:, 1::2] <= p[:, 1::2])
        kept = np.setdiff1d(np.arange(old.shape[0]), split)
        assert np.isin(kept, parent).all()


def _lcg_model(n, seed):
    """The fixture drivers' seeded model: s <- s * 6364136223846793005 +
    1442695040888963407 (mod 2^64), m = (((s >> 11) % 200001) - 100000) / 137."""
    out, s, mask = np.empty(n), seed, (1 << 64) - 1
    for i in range(n):
        s = (s * 6364136223846793005 + 1442695040888963407) & mask
        out[i] = (float((s >> 11) % 200001) - 100000.0) / 137.0
    return out


def test_structure_model_interpolation_and_crg_refinement_equal_reference(golden):
    """mesh.Multilinear is the reference's gridded-model interpolator bitwise
    (probes inside, on grid points and beyond every side; the cell-centre values
    invert_with_own_CG gives the leaves), and a refine_mesh(0.25, interpolator,
    "crg") gives the same leaves and the same structure model, the children
    interpolated at their centres (ref_interp.npz)."""
    from graada3d_gb300 import mesh
    from graada3d_gb300 import regularization as reg
    from graada3d_gb300.adaptive import carry_over, refinement_marks

    f = golden("ref_interp.npz")
    interp = mesh.Multilinear(f["grid_x"], f["grid_y"], f["grid_z"], f["values"])
    np.testing.assert_array_equal(interp(f["probes"]), f["probe_values"])
    o = mesh.Octree.regular((0.0, 600.0), 6, (0.0, 500.0), 5, (0.0, 400.0), 4)
    pts, c = f["pre_points"], o.leaves()
    inside = ((pts[None, :, 0] > c[:, None, 0]) & (pts[None, :, 0] < c[:, None, 1])
              & (pts[None, :, 1] > c[:, None, 2]) & (pts[None, :, 1] < c[:, None, 3])
              & (pts[None, :, 2] > c[:, None, 4]) & (pts[None, :, 2] < c[:, None, 5]))
    o.refine(np.nonzero(inside.any(1))[0])
    leaf0 = o.leaves()
    m0s = interp(mesh.cell_centres(leaf0))
    np.testing.assert_array_equal(m0s, f["m0s0"])
    m = _lcg_model(leaf0.shape[0], 99)
    ind = refinement.indicator(m, *reg.indicator_pairs(leaf0))
    marks = refinement_marks(ind, leaf0, float(f["fraction"]), (1.0, 1.0, 1.0))
    split = o.refine(marks)
    assert np.array_equal(o.leaves().view(np.uint64), f["leaf1"].view(np.uint64))
    parent = o.parent_leaf(split, leaf0.shape[0])
    np.testing.assert_array_equal(carry_over(m0s, parent, split, o.leaves(), interp), f["m0s1"])
