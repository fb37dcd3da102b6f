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
  On a refined (face-balanced) mesh the neighbour across a face is a cell of
  the same size, a coarser cell, or four finer cells that each take a
  quarter of the off-diagonal weight (``difference_matrices``).
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


def _axis_lattice(lo: np.ndarray, hi: np.ndarray):
    """Distinct bound coordinates of one axis (values closer than 1e-9 of the
    extent merged) and each cell's [first, last) interval index range."""
    v = np.unique(np.concatenate([lo, hi]))
    tol = 1e-9 * max(float(v[-1] - v[0]), 1e-300)
    v = v[np.concatenate([[True], np.diff(v) > tol])]
    i0 = np.searchsorted(v, lo - tol)
    i1 = np.searchsorted(v, hi - tol)
    return v, i0, i1


def _leaf_owner(pr: np.ndarray):
    """Cell id of every interval box of the lattice the cells' bounds span.
    Raises if the cells overlap or leave holes in their bounding box."""
    lat = [_axis_lattice(pr[:, 2 * a], pr[:, 2 * a + 1]) for a in range(3)]
    shape = tuple(len(l[0]) - 1 for l in lat)
    if np.prod(shape, dtype=np.float64) > 2.0 ** 31:
        raise ValueError(f"lattice of {shape} interval boxes is too large")
    owner = np.full(shape, -1, dtype=np.int64)
    lo = np.stack([l[1] for l in lat], 1)
    span = np.stack([l[2] - l[1] for l in lat], 1)
    if (span <= 0).any():
        raise ValueError("cell with zero extent")
    if int(np.prod(span, axis=1).sum()) != int(np.prod(shape)):
        raise ValueError("cells overlap or do not fill their bounding box")
    groups = {}
    for c, s in enumerate(map(tuple, span)):
        groups.setdefault(s, []).append(c)
    for s, ids in groups.items():
        ids = np.asarray(ids)
        ox, oy, oz = (np.arange(s[a]) for a in range(3))
        owner[(lo[ids, 0][:, None, None, None] + ox[None, :, None, None]),
              (lo[ids, 1][:, None, None, None] + oy[None, None, :, None]),
              (lo[ids, 2][:, None, None, None] + oz[None, None, None, :])] = ids[:, None, None, None]
    if (owner < 0).any():
        raise ValueError("cells overlap or do not fill their bounding box")
    return owner, [l[0] for l in lat], lo, lo + span


def _face_neighbours(pr, owner, lat, lo, hi, axis: int, side: int):
    """Cells across each cell's face on `side` (+1 / -1) of `axis`, probed at
    four points of the face at 0.3 / 0.7 of its two extents: (n, 4) ids, -1 on
    the bounding box's boundary.  Four equal ids: one cell of the same or a
    coarser level; four distinct ids: four finer cells, in the order of
    Mesh::refinement's child faces (first transverse axis outer)."""
    n = pr.shape[0]
    t = [b for b in range(3) if b != axis]
    ia = hi[:, axis] if side > 0 else lo[:, axis] - 1
    inside = (ia >= 0) & (ia < owner.shape[axis])
    out = np.full((n, 4), -1, dtype=np.int64)
    probes = []
    for b in t:
        p0, p1 = pr[:, 2 * b], pr[:, 2 * b + 1]
        probes.append([np.searchsorted(lat[b], p0 + f * (p1 - p0), side="right") - 1
                       for f in (0.3, 0.7)])
    q = 0
    for u in range(2):
        for w in range(2):
            idx = [None, None, None]
            idx[axis] = ia[inside]
            idx[t[0]] = probes[0][u][inside]
            idx[t[1]] = probes[1][w][inside]
            out[inside, q] = owner[idx[0], idx[1], idx[2]]
            q += 1
    return out


def face_table(prisms) -> np.ndarray:
    """Per cell and axis the face InversionBase::set_difference_matrix
    (InversionBase.cpp:189-434) differences against, from the leaf cells'
    bounds alone (regular, padded and octree-refined meshes): an (n, 3, 5)
    int32 table of [side, c0, c1, c2, c3].

    * side +1: the +axis face has cells across it (:208-220, :251-263);
    * side -1: the +axis face is on the boundary, the -axis face has cells
      across it (:223-249);
    * side 0: both faces on the boundary, no row (:389 for z; the
      reference's x and y rows need two cells).

    c0..c3: one neighbour of the same or a coarser level (c1 = c2 = c3 = -1)
    or four finer neighbours in the order of the reference's child faces.
    Raises if a face has a neighbour pattern a face-balanced octree cannot
    have (two levels apart, or finer in one transverse direction only)."""
    pr = np.asarray(prisms, dtype=np.float64)
    n = pr.shape[0]
    sizes = np.abs(pr[:, 1::2] - pr[:, 0::2])
    owner, lat, lo, hi = _leaf_owner(pr)
    table = np.full((n, 3, 5), -1, dtype=np.int32)
    table[:, :, 0] = 0
    for axis in range(3):
        t = [b for b in range(3) if b != axis]
        done = np.zeros(n, dtype=bool)
        for side in (1, -1):
            nb = _face_neighbours(pr, owner, lat, lo, hi, axis, side)
            has = (nb[:, 0] >= 0) & ~done
            one = has & (nb == nb[:, :1]).all(1)
            four = has & ~one
            if four.any():
                k = nb[four]
                if not all(len(set(r)) == 4 for r in k.tolist()):
                    raise ValueError("face neighbours are not face-balanced")
                half = sizes[four][:, t] * 0.5
                for q in range(4):
                    if not np.allclose(sizes[k[:, q]][:, t], half, rtol=1e-9, atol=0.0):
                        raise ValueError("face neighbours are not face-balanced")
            if one.any():
                big = sizes[nb[one, 0]][:, t]
                mine = sizes[one][:, t]
                ok = np.isclose(big, mine, rtol=1e-9) | np.isclose(big, 2 * mine, rtol=1e-9)
                if not ok.all():
                    raise ValueError("face neighbours are not face-balanced")
            table[one, axis, 0] = side
            table[one, axis, 1] = nb[one, 0]
            table[four, axis, 0] = side
            table[four, axis, 1:] = nb[four]
            done |= has
    return table


def indicator_pairs(prisms):
    """The (neighbour, face area) list AdaptiveInversion::indicator_calculator
    (AdaptiveInversion.cpp:108-204) sums over, from the leaf cells' bounds: for
    each cell, for side j = -, + the x, y and z faces; a face with one cell
    across it (same or coarser level) gives that cell and the cell's own face
    area, a face with four finer cells across gives them in the reference's
    child-face order with their face areas, a boundary face nothing.  Returns
    (rowptr (Nm + 1), neighbour, area), the arguments of
    grada_refinement_indicator."""
    pr = np.asarray(prisms, dtype=np.float64)
    n = pr.shape[0]
    sizes = np.abs(pr[:, 1::2] - pr[:, 0::2])
    owner, lat, lo, hi = _leaf_owner(pr)
    blocks = []  # (count, neighbours, areas) per (side, axis), each (n, 4)
    for side in (-1, 1):
        for axis in range(3):
            t = [b for b in range(3) if b != axis]
            nb = _face_neighbours(pr, owner, lat, lo, hi, axis, side)
            has = nb[:, 0] >= 0
            one = has & (nb == nb[:, :1]).all(1)
            cnt = np.where(one, 1, np.where(has, 4, 0))
            own = sizes[:, t[0]] * sizes[:, t[1]]
            kid = np.where(nb >= 0, sizes[np.maximum(nb, 0), t[0]] * sizes[np.maximum(nb, 0), t[1]],
                           0.0)
            area = np.where(one[:, None], own[:, None], kid)
            blocks.append((cnt, nb, area))
    counts = np.stack([b[0] for b in blocks], 1)  # (n, 6)
    rowptr = np.zeros(n + 1, dtype=np.int64)
    rowptr[1:] = np.cumsum(counts.sum(1))
    total = int(rowptr[-1])
    neighbour = np.empty(total, dtype=np.int64)
    area = np.empty(total)
    pos = rowptr[:-1].copy()
    for cnt, nb, ar in blocks:
        for q in range(4):
            sel = cnt > q
            neighbour[pos[sel]] = nb[sel, q]
            area[pos[sel]] = ar[sel, q]
            pos[sel] += 1
    return rowptr, neighbour, area


def difference_matrices(prisms, table=None) -> tuple:
    """D_x1, D_y1, D_z1 (CSR) of InversionBase::set_difference_matrix from the
    face table (``face_table`` of the cells unless given), with h the cells'
    sizes along the axis and w = 1 / (0.5 (h0 + h1)), h1 that of c0:
    -side w on the diagonal and side w to one neighbour, or side w / 4 to each
    of four finer ones (:208-263, :223-249 for side -1)."""
    pr = np.asarray(prisms, dtype=np.float64)
    n = pr.shape[0]
    sizes = np.abs(pr[:, 1::2] - pr[:, 0::2])
    tab = face_table(pr) if table is None else np.asarray(table)
    mats = []
    for axis in range(3):
        f = tab[:, axis]
        side = f[:, 0].astype(np.float64)
        rowsel = f[:, 0] != 0
        one = rowsel & (f[:, 2] < 0)
        four = rowsel & (f[:, 2] >= 0)
        i = np.nonzero(rowsel)[0]
        h1 = sizes[f[i, 1], axis]
        w = np.zeros(n)
        w[i] = 1.0 / (0.5 * (sizes[i, axis] + h1))
        rows, cols, vals = [i], [i], [-side[i] * w[i]]
        j = np.nonzero(one)[0]
        rows.append(j)
        cols.append(f[j, 1])
        vals.append(side[j] * w[j])
        j = np.nonzero(four)[0]
        for q in range(4):
            rows.append(j)
            cols.append(f[j, 1 + q])
            vals.append(side[j] * w[j] * 0.25)
        D = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                          shape=(n, n))
        D.sort_indices()
        mats.append(D)
    return tuple(mats)


def _operators(pr, obs, beta, D, a_s, a_z, a_x, a_y):
    sizes = np.abs(np.stack([pr[:, 1] - pr[:, 0], pr[:, 3] - pr[:, 2], pr[:, 5] - pr[:, 4]], 1))
    vol = sizes[:, 0] * sizes[:, 1] * sizes[:, 2]
    V = np.sqrt(vol)
    # summed in order, as InversionBase.cpp:505-510 does
    zp = np.cumsum(np.asarray(obs, dtype=np.float64)[:, 2])[-1] / obs.shape[0]
    zc = 0.5 * (pr[:, 4] + pr[:, 5])
    Z = 1.0 / np.abs(zp - zc) ** (beta * 0.5)
    Dx, Dy, Dz = D
    Ds = sp.identity(pr.shape[0], format="csr")

    def W(a, D):
        M = (sp.diags(a * V) @ D) @ sp.diags(Z)
        M = sp.csr_matrix(M)
        M.sort_indices()
        return M

    return {"Ws": W(a_s, Ds), "Wx": W(a_x, Dx), "Wy": W(a_y, Dy), "Wz": W(a_z, Dz),
            "V": V, "Z": Z, "Dx": Dx, "Dy": Dy, "Dz": Dz}


def regular_mesh_operators(n, prisms, obs, beta: float, a_s=1.0, a_z=1.0, a_x=1.0, a_y=1.0):
    """Ws, Wx, Wy, Wz (CSR) plus V, Z, D_x, D_y, D_z for a regular mesh."""
    nx, ny, nz = n
    pr = np.asarray(prisms, dtype=np.float64)
    sizes = np.abs(np.stack([pr[:, 1] - pr[:, 0], pr[:, 3] - pr[:, 2], pr[:, 5] - pr[:, 4]], 1))
    D = tuple(_difference(nx, ny, nz, sizes, a) for a in range(3))
    return _operators(pr, obs, beta, D, a_s, a_z, a_x, a_y)


def mesh_operators(prisms, obs, beta: float, a_s=1.0, a_z=1.0, a_x=1.0, a_y=1.0, table=None):
    """Ws, Wx, Wy, Wz (CSR) plus V, Z, D_x, D_y, D_z for any leaf-cell list
    (regular, padded or octree-refined), the differences from the cells'
    bounds (``difference_matrices``; ``table``: a face table already built by
    ``face_table``)."""
    pr = np.asarray(prisms, dtype=np.float64)
    return _operators(pr, obs, beta, difference_matrices(pr, table), a_s, a_z, a_x, a_y)


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
