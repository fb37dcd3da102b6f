"""The wavelet oracle (restated periodic Daubechies-4 pyramid and the
reference's row compression) against the transform's own properties.  GSL,
whose transform the reference calls, is absent: parity with it is unpinned."""
import numpy as np

from oracle import wavelet as wv


def test_filters_are_orthonormal_with_two_vanishing_moments():
    h, g = wv.H, wv.G
    assert abs(np.dot(h, h) - 1) < 1e-15 and abs(np.dot(g, g) - 1) < 1e-15
    assert abs(np.dot(h, g)) < 1e-16
    assert abs(h.sum() - np.sqrt(2)) < 1e-15
    k = np.arange(4)
    assert abs(g.sum()) < 1e-15 and abs(np.dot(k, g)) < 1e-15


def test_transform_is_orthogonal_and_inverts():
    rng = np.random.default_rng(3)
    for n in (2, 4, 8, 64, 1024):
        x = rng.standard_normal((5, n))
        c = wv.forward(x)
        np.testing.assert_allclose(np.linalg.norm(c, axis=1), np.linalg.norm(x, axis=1), rtol=1e-14)
        np.testing.assert_allclose(wv.inverse(c), x, rtol=0, atol=2e-14 * np.abs(x).max())


def test_constant_signal_has_one_coefficient():
    c = wv.forward(np.full(256, 3.0))
    assert abs(c[0] - 3.0 * 16.0) < 1e-12
    assert np.abs(c[1:]).max() < 1e-13


def test_padding_length():
    assert [wv.padded_length(n) for n in (2, 3, 4, 5, 1000, 1024, 1025)] == \
        [2, 4, 4, 8, 1024, 1024, 2048]


def test_compressed_products_without_threshold_equal_dense():
    rng = np.random.default_rng(5)
    nd, nm = 30, 300
    Gd = np.cumsum(rng.standard_normal((nd, nm)), axis=1)
    order = rng.permutation(nm)
    comp = wv.compress(Gd, order, 0.0)
    assert comp[2].size == nd * comp[0]  # every coefficient kept, zeros included
    x, y = rng.standard_normal(nm), rng.standard_normal(nd)
    np.testing.assert_allclose(wv.G_vec_mul(comp, order, x), Gd @ x, rtol=0,
                               atol=1e-13 * np.abs(Gd @ x).max())
    np.testing.assert_allclose(wv.GT_vec_mul(comp, order, y), Gd.T @ y, rtol=0,
                               atol=1e-13 * np.abs(Gd.T @ y).max())


def test_threshold_keeps_the_largest_coefficients():
    rng = np.random.default_rng(6)
    Gd = np.cumsum(np.cumsum(rng.standard_normal((8, 500)), axis=1), axis=1)  # smooth rows
    order = np.arange(500)
    full = wv.forward(np.pad(Gd, ((0, 0), (0, 12))))
    sizes = []
    for rel in (1e-6, 1e-4, 1e-2):
        n_dy, rp, cols, vals = wv.compress(Gd, order, rel)
        sizes.append(cols.size)
        for r in range(8):
            kept = cols[rp[r]:rp[r + 1]]
            thr = rel * np.abs(full[r]).max()
            assert np.all(np.abs(full[r, kept]) >= thr - 1e-15)
            dropped = np.setdiff1d(np.arange(n_dy), kept)
            assert np.all(np.abs(full[r, dropped]) < thr)
            np.testing.assert_array_equal(vals[rp[r]:rp[r + 1]], full[r, kept])
    assert sizes[0] > sizes[1] > sizes[2]
