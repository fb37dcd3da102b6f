"""Test oracle (test infrastructure only): the reference's wavelet-compressed
sensitivity matrix restated in NumPy.

Follows Fwd::compute_G_wavelet (src/Forward_modelling/Fwd.cpp:148-219),
Fwd::compress_vec (:298-358), Fwd::wavelet_transform_vec /
inverse_wavelet_transform_vec (:257-296, :360-402) and the wavelet branches of
Fwd::G_vec_mul / GT_vec_mul (:80-146).  The reference takes its transform from
GSL (gsl_wavelet_daubechies, member 4, gsl_wavelet_transform_forward /
_inverse, GSL 2.x), which is absent here; this restates the published
periodic Daubechies-4 pyramid algorithm GSL implements: the four-tap scaling
filter h of Daubechies (1988), the wavelet filter g_k = (-1)^k h_{3-k}, no
offset, levels n = n_dy, n_dy / 2, ..., 2 (forward) with the approximations of
a level in entries [0, n/2) and its details in [n/2, n), every sum accumulated
in index order from zero.  The products sum in the device's fixed parallel
orders (documented at G_vec_mul / GT_vec_mul), which differ from the
reference's sequential sums at the rounding level.  Parity with GSL itself is
unpinned; the device path
is checked against this restatement, and the restatement against the
transform's own properties (orthogonality, exact reconstruction, vanishing
moments).
"""
from __future__ import annotations

import numpy as np

# (1 + sqrt 3, 3 + sqrt 3, 3 - sqrt 3, 1 - sqrt 3) / (4 sqrt 2), correctly rounded
H = np.array([0.48296291314453416, 0.8365163037378079, 0.2241438680420134, -0.12940952255126037])
G = np.array([H[3], -H[2], H[1], -H[0]])


def padded_length(n: int) -> int:
    """n when it is a power of two, else the next power of two (Fwd.cpp:302-312)."""
    p = 1
    while p < n:
        p *= 2
    return p


def forward(data: np.ndarray) -> np.ndarray:
    """Forward transform along the last axis (a power-of-two length)."""
    a = np.array(data, dtype=np.float64, copy=True)
    n = a.shape[-1]
    while n >= 2:
        nh = n // 2
        ii = np.arange(nh)
        h = np.zeros(a.shape[:-1] + (nh,))
        g = np.zeros(a.shape[:-1] + (nh,))
        for k in range(4):
            v = a[..., (2 * ii + k) & (n - 1)]
            h = h + H[k] * v
            g = g + G[k] * v
        a[..., :nh] = h
        a[..., nh:n] = g
        n = nh
    return a


def inverse(coef: np.ndarray) -> np.ndarray:
    """Inverse transform along the last axis: levels n = 2, 4, ..., each output
    accumulating its contributions in the order the pyramid visits them."""
    a = np.array(coef, dtype=np.float64, copy=True)
    total = a.shape[-1]
    n = 2
    while n <= total:
        nh = n // 2
        out = np.zeros(a.shape[:-1] + (n,))
        for i in range(nh):
            ai = a[..., i]
            ai1 = a[..., i + nh]
            for k in range(4):
                jf = (2 * i + k) & (n - 1)
                out[..., jf] = out[..., jf] + (H[k] * ai + G[k] * ai1)
        a[..., :n] = out
        n *= 2
    return a


def compress(Gd: np.ndarray, order: np.ndarray, rel: float, fp32: bool = False):
    """Rows of the dense G (Nd x Nm), cells in `order` (Mesh::get_reordered_id),
    transformed and thresholded: (n_dy, rowptr, cols, vals); fp32: the kept
    values rounded to FP32 (the device's optional value storage)."""
    nd, nm = Gd.shape
    n_dy = padded_length(nm)
    data = np.zeros((nd, n_dy))
    data[:, :nm] = Gd[:, order]
    c = forward(data)
    rowptr = [0]
    cols, vals = [], []
    for r in range(nd):
        a = np.abs(c[r])
        thr = rel * a.max()
        keep = np.nonzero((a > thr) | (np.abs(a - thr) < 1e-15))[0]
        cols.append(keep)
        vals.append(c[r, keep])
        rowptr.append(rowptr[-1] + keep.size)
    vals = np.concatenate(vals)
    if fp32:
        vals = vals.astype(np.float32).astype(np.float64)
    return n_dy, np.array(rowptr, dtype=np.int64), np.concatenate(cols), vals


GT_BLOCKS = 304  # row blocks of the device's G^T y


def _warp_sum(p: np.ndarray) -> float:
    """The device's row sum: lane l adds entries l, l + 32, ... in order from
    zero, then lanes combine by a butterfly (xor 16, 8, 4, 2, 1)."""
    lanes = np.zeros(32)
    for l in range(min(32, p.size)):
        lanes[l] = np.cumsum(p[l::32])[-1]
    for off in (16, 8, 4, 2, 1):
        lanes = lanes + lanes[np.arange(32) ^ off]
    return float(lanes[0])


def G_vec_mul(comp, order: np.ndarray, x: np.ndarray) -> np.ndarray:
    """Fwd::G_vec_mul's wavelet branch (Fwd.cpp:113-140): x reordered, padded
    and transformed, each row's kept coefficients dotted with it (summed in the
    device's fixed order instead of the reference's sequential one)."""
    n_dy, rowptr, cols, vals = comp
    w = np.zeros(n_dy)
    w[:order.size] = x[order]
    w = forward(w)
    y = np.empty(rowptr.size - 1)
    for r in range(y.size):
        s = slice(rowptr[r], rowptr[r + 1])
        y[r] = _warp_sum(vals[s] * w[cols[s]])
    return y


def GT_vec_mul(comp, order: np.ndarray, y: np.ndarray) -> np.ndarray:
    """Fwd::GT_vec_mul's wavelet branch (Fwd.cpp:80-112): the kept coefficients
    times y added per coefficient index -- the rows in consecutive blocks of
    ceil(Nd / 304), each block's rows in order into its own partial vector, the
    partials in block order -- then the inverse transform and the cell order."""
    n_dy, rowptr, cols, vals = comp
    nd = rowptr.size - 1
    R = max(1, -(-nd // GT_BLOCKS))
    pw = np.zeros(n_dy)
    for b0 in range(0, nd, R):
        part = np.zeros(n_dy)
        for r in range(b0, min(nd, b0 + R)):
            s = slice(rowptr[r], rowptr[r + 1])
            part[cols[s]] = part[cols[s]] + vals[s] * y[r]
        pw = pw + part
    pw = inverse(pw)
    x = np.empty(order.size)
    x[order] = pw[:order.size]
    return x
