"""Host-side mesh refinement and regularisation operators on octree-refined
meshes against the compiled reference (tests/golden/ref_operators.npz:
Mesh::refinement with its face-balance cascade, then
InversionBase::set_difference_matrix, set_Vmatrix, set_depth_weighting,
set_Tmatrix and GaussNewtonInversion.cpp:711-714)."""
from pathlib import Path

import numpy as np
import pytest
import scipy.sparse as sp

from graada3d_gb300 import mesh
from graada3d_gb300 import regularization as reg

GOLDEN = Path(__file__).resolve().parent / "golden"


def _load():
    return np.load(GOLDEN / "ref_operators.npz")


def _csr(f, key):
    n = f["leaf"].shape[0]
    return sp.csr_matrix((f[key + "_data"], f[key + "_indices"], f[key + "_indptr"]), shape=(n, n))


def _same_csr(a, b):
    """Equal sparsity pattern and bitwise-equal values."""
    a, b = sp.csr_matrix(a), sp.csr_matrix(b)
    a.sort_indices()
    b.sort_indices()
    a.eliminate_zeros()
    b.eliminate_zeros()
    return (np.array_equal(a.indptr, b.indptr) and np.array_equal(a.indices, b.indices)
            and np.array_equal(a.data.view(np.uint64), b.data.view(np.uint64)))


def _octree_of(f):
    n = f["n"]
    lim = f["limits"]
    o = mesh.Octree.regular(lim[0:2], int(n[0]), lim[2:4], int(n[1]), lim[4:6], int(n[2]))
    for r in f["passes"]:
        pts = r[~np.isnan(r[:, 0])]
        cells = o.leaves()
        inside = ((pts[None, :, 0] > cells[:, None, 0]) & (pts[None, :, 0] < cells[:, None, 1]) &
                  (pts[None, :, 1] > cells[:, None, 2]) & (pts[None, :, 1] < cells[:, None, 3]) &
                  (pts[None, :, 2] > cells[:, None, 4]) & (pts[None, :, 2] < cells[:, None, 5]))
        o.refine(np.nonzero(inside.any(1))[0])
    return o


def test_octree_refinement_matches_reference_leaves():
    """Same leaves, bitwise, in the same order, at the same levels, cascades
    included (the fixture's passes split level-1 and level-2 cells next to
    coarser ones)."""
    f = _load()
    o = _octree_of(f)
    assert np.array_equal(o.leaves().view(np.uint64), f["leaf"].view(np.uint64))
    assert np.array_equal(o.levels(), f["level"])
    assert f["level"].max() == 3


def test_wavelet_order_matches_reference():
    """Octree.wavelet_order is Mesh::get_reordered_id after the reference's
    refinements (the sequence the wavelet-compressed G runs along)."""
    f = _load()
    np.testing.assert_array_equal(_octree_of(f).wavelet_order(), f["reordered_id"])
    # unrefined: the z snake over (x, y) lines
    o = mesh.Octree.regular((0, 1), 2, (0, 1), 2, (0, 1), 3)
    np.testing.assert_array_equal(o.wavelet_order(), [0, 1, 2, 5, 4, 3, 6, 7, 8, 11, 10, 9])


def test_difference_matrices_match_reference():
    f = _load()
    Dx, Dy, Dz = reg.difference_matrices(f["leaf"])
    for key, D in (("Dx", Dx), ("Dy", Dy), ("Dz", Dz)):
        assert _same_csr(D, _csr(f, key)), key
    # the fixture holds every face case: four finer neighbours on the +side
    # and, at a boundary, on the -side
    assert (np.diff(_csr(f, "Dx").indptr) == 5).sum() > 0
    assert (np.diff(_csr(f, "Dz").indptr) == 5).sum() > 0


def test_face_table_matches_the_reference_faces():
    """The geometric face table equals the one the drop-in reads from the
    reference's own Face objects (dropin/FaceTable_gb300.cpp run on the
    reference's refined mesh): the same side, neighbours and child-face order
    for every cell and axis, so either feeds grada_build_operators alike."""
    f = _load()
    t = reg.face_table(f["leaf"])
    np.testing.assert_array_equal(t, f["face_table"])
    assert (t[:, :, 0] == -1).any() and (t[:, :, 2] >= 0).any()


def test_mesh_operators_match_reference():
    f = _load()
    a = f["alphas"]
    ops = reg.mesh_operators(f["leaf"], f["obs"], float(f["beta"]), a_s=a[0], a_z=a[1], a_x=a[2],
                             a_y=a[3])
    np.testing.assert_array_equal(ops["V"], f["V"])
    # Z = 1 / |zp - zc|^(beta/2): numpy's power and the C library's pow may
    # round the last bit differently
    np.testing.assert_allclose(ops["Z"], f["Z"], rtol=4e-16, atol=0)
    for key in ["Ws", "Wx", "Wy", "Wz"]:
        want = _csr(f, key).toarray()
        got = ops[key].toarray()
        assert np.abs(got - want).max() <= 1e-14 * np.abs(want).max(), key
    T = reg.cross_gradient_operators(None, f["leaf"], f["m0s"], ops)
    for key in ["Tx", "Ty", "Tz"]:
        want = _csr(f, key).toarray()
        assert np.abs(T[key].toarray() - want).max() <= 1e-12 * np.abs(want).max(), key


def test_difference_matrices_equal_regular_builder():
    """On unrefined meshes, uniform and with uneven spacing, the geometric
    builder gives the regular one's matrices bit for bit."""
    xs = np.array([0.0, 40.0, 100.0, 180.0, 300.0])
    ys = np.array([-50.0, 0.0, 70.0, 90.0])
    zs = np.array([0.0, 25.0, 60.0, 120.0, 250.0, 400.0])
    for pr, n in ((mesh.regular_mesh((0, 3000), 7, (0, 2000), 5, (0, 1500), 4), (7, 5, 4)),
                  (mesh.prisms_from_points(xs, ys, zs), (4, 3, 5)),
                  (mesh.regular_mesh((0, 300), 3, (0, 200), 2, (0, 100), 1), (3, 2, 1))):
        obs = mesh.observation_grid(3, 0, 100, 3, 0, 100, -5.0)
        want = reg.regular_mesh_operators(n, pr, obs, 1.5)
        got = reg.mesh_operators(pr, obs, 1.5)
        for key in ("Dx", "Dy", "Dz", "Ws", "Wx", "Wy", "Wz"):
            assert _same_csr(got[key], want[key]), (n, key)


def test_unbalanced_mesh_is_rejected():
    """Splitting one child of a split cell without the cascade leaves a face
    between cells two levels apart: no reference mesh has one."""
    from graada3d_gb300.fwd import split_cells

    base = mesh.regular_mesh((0, 400), 4, (0, 400), 4, (0, 400), 4)
    kids = split_cells(base[21:22]).reshape(8, 6)
    grand = split_cells(kids[0:1]).reshape(8, 6)
    cells = np.vstack([base[:21], grand, kids[1:], base[22:]])
    with pytest.raises(ValueError, match="face-balanced"):
        reg.difference_matrices(cells)
    with pytest.raises(ValueError, match="overlap"):
        reg.difference_matrices(np.vstack([cells, cells[:1]]))


def test_dyke_mesh_is_face_balanced():
    """The refined two-dyke benchmark mesh is the Octree's (cascades included):
    its operators build, every cell has a row in each direction and rows sum
    to zero (differences of a constant vanish)."""
    import bench

    cells = bench.refined_dyke_mesh(levels=2)
    D = reg.difference_matrices(cells)
    for M in D:
        assert (np.diff(M.indptr) >= 2).all()
        s = np.abs(M @ np.ones(cells.shape[0]))
        assert s.max() <= 1e-15 * np.abs(M).max()


def test_octree_random_refinements_stay_face_balanced():
    """Random passes of splits (cascades included) keep every face between
    cells at most one level apart, tile the domain, and give a wavelet order
    that is a permutation of the leaves."""
    rng = np.random.default_rng(17)
    o = mesh.Octree.regular((0.0, 800.0), 4, (0.0, 600.0), 3, (0.0, 400.0), 2)
    for _ in range(4):
        n = len(o.leaf_keys())
        o.refine(rng.choice(n, size=max(1, n // 10), replace=False))
    cells = o.leaves()
    vol = np.prod(cells[:, 1::2] - cells[:, 0::2], axis=1).sum()
    assert abs(vol - 800.0 * 600.0 * 400.0) <= 1e-9 * vol
    reg.face_table(cells)  # raises on a face between cells two levels apart
    w = o.wavelet_order()
    np.testing.assert_array_equal(np.sort(w), np.arange(cells.shape[0]))
    assert o.levels().max() >= 3


def test_padded_mesh_matches_reference_leaves():
    """mesh.padded_mesh is Mesh::generate_regular_mesh_with_padding bit for bit
    (tests/golden/ref_padded.npz: 6 x 5 x 4 cells of interest, 4 padding cells
    on each x / y side and 3 below, stretch 1.8); its operators build."""
    f = np.load(GOLDEN / "ref_padded.npz")
    pr = mesh.padded_mesh((0.0, 3000.0), 6, (0.0, 3000.0), 5, (0.0, 1500.0), 4, 4, 1.8, 4, 1.8, 3,
                          1.8)
    assert np.array_equal(pr.view(np.uint64), f["leaf"].view(np.uint64))
    xs, ys, zs = mesh.padded_mesh_points((0.0, 3000.0), 6, (0.0, 3000.0), 5, (0.0, 1500.0), 4, 4,
                                         1.8, 4, 1.8, 3, 1.8)
    obs = mesh.observation_grid(3, 0.0, 3000.0, 3, 0.0, 3000.0, -10.0)
    n = (len(xs) - 1, len(ys) - 1, len(zs) - 1)
    want = reg.regular_mesh_operators(n, pr, obs, 1.5)
    got = reg.mesh_operators(pr, obs, 1.5)
    for key in ("Dx", "Dy", "Dz", "Wx", "Wy", "Wz"):
        assert _same_csr(got[key], want[key]), key
