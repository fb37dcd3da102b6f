"""AdaptiveInversion::expand_G on the device: the spliced G equals the G of
the refined cell list, column for column (AdaptiveInversion.cpp:23-106)."""
import numpy as np
import pytest

from graada3d_gb300 import Fwd, GradaError, mesh
from graada3d_gb300.fwd import split_cells


def test_children_follow_reference_order():
    """Mesh::refinement makes children x outer, y, z inner at the centre
    (Mesh.cpp:1579-1600): the same order as a 2x2x2 regular mesh of the cell."""
    cell = np.array([[10.0, 30.0, -5.0, 15.0, 100.0, 140.0]])
    want = mesh.regular_mesh((10.0, 30.0), 2, (-5.0, 15.0), 2, (100.0, 140.0), 2)
    np.testing.assert_array_equal(split_cells(cell)[0], want)


@pytest.mark.gpu
@pytest.mark.parametrize("storage", ["fp64", "fp32"])
def test_expand_G_equals_assembly_of_refined_mesh(gpu_ctx, storage):
    prisms = mesh.regular_mesh((0.0, 600.0), 6, (0.0, 500.0), 5, (0.0, 400.0), 4)
    obs = mesh.observation_grid(8, -50.0, 650.0, 5, -50.0, 550.0, -5.0)
    mask = 0x3FE
    f = Fwd(prisms, obs, mask, ctx=gpu_ctx)
    f.compute_G(storage)
    parents = np.array([0, 3, 17, 18, 50, 119])
    f.expand_G(parents)
    assert f.Nm == prisms.shape[0] + 7 * parents.size
    got = f.get_G()
    # the refined leaf list: each parent replaced in place by its 8 children
    refined = []
    kids = split_cells(prisms[parents])
    pk = dict(zip(parents.tolist(), range(parents.size)))
    for j in range(prisms.shape[0]):
        if j in pk:
            refined.extend(kids[pk[j]])
        else:
            refined.append(prisms[j])
    refined = np.array(refined)
    np.testing.assert_array_equal(f.prisms, refined)
    g2 = Fwd(refined, obs, mask)
    g2.compute_G(storage)
    want = g2.get_G()
    assert np.array_equal(got, want)
    x = np.random.default_rng(1).standard_normal(f.Nm)
    np.testing.assert_allclose(f.G_vec_mul(x), want @ x, rtol=0,
                               atol=1e-5 * np.abs(want).sum(1).max())
    g2.ctx.close()


@pytest.mark.gpu
def test_expand_G_rejects_bad_input(gpu_ctx):
    prisms = mesh.regular_mesh((0.0, 100.0), 2, (0.0, 100.0), 2, (0.0, 100.0), 2)
    obs = np.array([[50.0, 50.0, -1.0]])
    f = Fwd(prisms, obs, 0x2, ctx=gpu_ctx)
    f.compute_G("fp64")
    with pytest.raises(GradaError):
        f.expand_G([3, 1])  # not ascending
    with pytest.raises(GradaError):
        f.expand_G([8])  # out of range
    f.compute_G("bf16")
    with pytest.raises(GradaError):
        f.expand_G([1])


# ---- pinned to the reference's own refinement path --------------------------
# tests/golden/ref_expand.npz: Mesh::refinement of six cells of a 6 x 5 x 4 mesh,
# Mesh::rearrange_id and AdaptiveInversion::expand_G run by the compiled
# reference (oracle/refdrv/ref_expand.cpp).

def _ref_expand(golden):
    return golden("ref_expand.npz")


def test_children_and_leaf_order_match_reference(golden):
    r = _ref_expand(golden)
    np.testing.assert_array_equal(r["split_index"], r["parents"])
    np.testing.assert_array_equal(split_cells(r["prisms"][r["parents"]]), r["children"])
    refined = []
    pk = {int(p): k for k, p in enumerate(r["parents"])}
    for j in range(r["prisms"].shape[0]):
        refined.extend(r["children"][pk[j]] if j in pk else [r["prisms"][j]])
    np.testing.assert_array_equal(np.array(refined), r["leaf"])


@pytest.mark.gpu
def test_expand_G_matches_reference_expand_G(gpu_ctx, golden):
    r = _ref_expand(golden)
    f = Fwd(r["prisms"], r["obs"], int(r["mask"]), ctx=gpu_ctx)
    f.compute_G("fp64")
    f.expand_G(r["parents"], r["children"])
    np.testing.assert_array_equal(f.prisms, r["leaf"])
    G = f.get_G()[: f.Nd]
    ref = r["G"]
    assert G.shape == ref.shape
    n = r["obs"].shape[0]
    for k in range(ref.shape[0] // n):  # per component, relative to its largest entry
        blk = slice(k * n, (k + 1) * n)
        assert np.abs(G[blk] - ref[blk]).max() <= 1e-10 * np.abs(ref[blk]).max(), k
