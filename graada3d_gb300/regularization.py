"""Host-side construction of the inversion operators for regular meshes.

In the reference these operators are built on the host by InversionBase and
GaussNewtonInversion and only *applied* in the hot path; the GPU library takes
them as CSR matrices (grada_set_operator).  This module restates their
construction for an unrefined regular mesh (leaf order x outer, z inner) so
that the Python side can drive the library without the reference's Mesh
classes:

* V_ii = sqrt(cell volume)                 InversionBase::set_Vmatrix, InversionBase.cpp:452-466
* Z_ii = |zp - zc|^(-beta/2), zp = mean observation z
                                           InversionBase::set_depth_weighting, :497-519
* D_s = I; D_x1, D_y1, D_z1: forward difference to the +axis neighbour,
  backward difference for the last cell of a line, no row if the axis has
  one cell (z only)                        InversionBase::set_difference_matrix, :189-434
* W_* = a_* S_* V D_* Z with S_* = I      GaussNewtonInversion.cpp:711-714
* T_z = V (diag(D_y m0s) D_x - diag(D_x m0s) D_y), T_x, T_y cyclic
                                           InversionBase::set_Tmatrix, :468-495
* Wd_ii = 1 / (rel_f |d_i| + abs_f)        InversionBase::set_dobs, :561-579
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp


def _difference(nx: int, ny: int, nz: int, sizes: np.ndarray, axis: int) -> sp.csr_matrix:
    n = nx * ny * nz
    strides = (ny * nz, nz, 1)
    counts = (nx, ny, nz)
    stride = strides[axis]
    idx = np.arange(n)
    pos = (idx // strides[axis]) % counts[axis]
    rows, cols, vals = [], [], []
    h = sizes[:, axis]
    fwd = pos < counts[axis] - 1
    i = idx[fwd]
    w = -1.0 / (0.5 * (h[i] + h[i + stride]))
    rows += [i, i]
    cols += [i, i + stride]
    vals += [w, -w]
    bwd = (~fwd) & (pos > 0)
    i = idx[bwd]
    w = 1.0 / (0.5 * (h[i] + h[i - stride]))
    rows += [i, i]
    cols += [i, i - stride]
    vals += [w, -w]
    D = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                      shape=(n, n))
    D.sort_indices()
    return D


def regular_mesh_operators(n, prisms, obs, beta: float, a_s=1.0, a_z=1.0, a_x=1.0, a_y=1.0):
    """Ws, Wx, Wy, Wz (CSR) plus V, Z, D_x, D_y, D_z for a regular mesh."""
    nx, ny, nz = n
    pr = np.asarray(prisms, dtype=np.float64)
    sizes = np.abs(np.stack([pr[:, 1] - pr[:, 0], pr[:, 3] - pr[:, 2], pr[:, 5] - pr[:, 4]], 1))
    vol = sizes[:, 0] * sizes[:, 1] * sizes[:, 2]
    V = np.sqrt(vol)
    zp = np.asarray(obs, dtype=np.float64)[:, 2].sum() / obs.shape[0]
    zc = 0.5 * (pr[:, 4] + pr[:, 5])
    Z = 1.0 / np.abs(zp - zc) ** (beta * 0.5)
    Dx = _difference(nx, ny, nz, sizes, 0)
    Dy = _difference(nx, ny, nz, sizes, 1)
    Dz = _difference(nx, ny, nz, sizes, 2)
    Ds = sp.identity(pr.shape[0], format="csr")

    def W(a, D):
        M = (sp.diags(a * V) @ D) @ sp.diags(Z)
        M = sp.csr_matrix(M)
        M.sort_indices()
        return M

    return {"Ws": W(a_s, Ds), "Wx": W(a_x, Dx), "Wy": W(a_y, Dy), "Wz": W(a_z, Dz),
            "V": V, "Z": Z, "Dx": Dx, "Dy": Dy, "Dz": Dz}


def cross_gradient_operators(n, prisms, m0s, ops) -> dict:
    """T_x, T_y, T_z of set_Tmatrix from the structure model m0s."""
    Dx, Dy, Dz, V = ops["Dx"], ops["Dy"], ops["Dz"], ops["V"]
    dzs, dxs, dys = Dz @ m0s, Dx @ m0s, Dy @ m0s
    Vd = sp.diags(V)

    def T(a, Da, b, Db):
        M = sp.csr_matrix(Vd @ (sp.diags(a) @ Da - sp.diags(b) @ Db))
        M.sort_indices()
        return M

    return {"Tz": T(dys, Dx, dxs, Dy), "Tx": T(dzs, Dy, dys, Dz), "Ty": T(dxs, Dz, dzs, Dx)}


def data_weights(dobs, rel, absf, n_obs: int) -> np.ndarray:
    d = np.asarray(dobs, dtype=np.float64)
    out = np.empty_like(d)
    for k in range(len(rel)):
        blk = slice(k * n_obs, (k + 1) * n_obs)
        out[blk] = 1.0 / (rel[k] * np.abs(d[blk]) + absf[k])
    return out


def p_diag(m, mmin, mmax):
    """P_ii = (mmax - m)(m - mmin)/(mmax - mmin), GaussNewtonInversion.cpp:856-861."""
    return (mmax - m) * (m - mmin) / (mmax - mmin)
