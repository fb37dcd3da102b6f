"""Host-side mesh and observation helpers with the reference's conventions.

Mesh construction and refinement stay on the host in the reference; these
helpers build the same regular meshes and observation grids as
``Mesh::generate_regular_mesh`` and ``Observation::generate`` so that tests
and benchmarks can feed the GPU path the cell order and coordinates the
reference would produce.

* ``regular_mesh`` -- Mesh.cpp:500-514 (grid points from Eigen's LinSpaced)
  and Mesh.cpp:830-847 (leaf order: x outermost, then y, z innermost).
* ``padded_mesh`` -- Mesh::generate_regular_mesh_with_padding, Mesh.cpp:516-587.
* ``set_boxes`` -- Mesh::set_parameter_in_a_region, Mesh.cpp:1079-1107: a
  cell takes a box's value when it lies entirely inside the box (1e-10
  tolerance); later boxes overwrite earlier ones.
* ``observation_grid`` -- Observation::generate, Observation.cpp:48-77
* ``Octree`` -- Mesh::refinement, Mesh.cpp:1462-1942: octant splits kept
  face-balanced, leaves in the reference's leaf order.
* ``Multilinear`` -- the gridded-model interpolation of
  InversionBase::create_crg_model_from_data / create_ref_model_from_data.
  (x fastest).
"""
from __future__ import annotations

import numpy as np


def linspaced(low: float, high: float, n: int) -> np.ndarray:
    """Eigen::VectorXd::LinSpaced(n, low, high) for n >= 2 (NullaryFunctors.h)."""
    low = float(low)
    high = float(high)
    size1 = n - 1
    step = (high - low) / float(size1)
    i = np.arange(n, dtype=np.float64)
    if abs(high) < abs(low):
        v = high - (size1 - i) * step
        v[0] = low
    else:
        v = low + i * step
        v[-1] = high
    return v


def regular_mesh_points(xlim, nx, ylim, ny, zlim, nz):
    return linspaced(*xlim, nx + 1), linspaced(*ylim, ny + 1), linspaced(*zlim, nz + 1)


def prisms_from_points(xs, ys, zs) -> np.ndarray:
    """(nx*ny*nz, 6) cells x0 x1 y0 y1 z0 z1 in the reference leaf order."""
    nx, ny, nz = len(xs) - 1, len(ys) - 1, len(zs) - 1
    I, J, K = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    I, J, K = I.ravel(), J.ravel(), K.ravel()
    return np.stack([xs[I], xs[I + 1], ys[J], ys[J + 1], zs[K], zs[K + 1]], axis=1)


def regular_mesh(xlim, nx, ylim, ny, zlim, nz) -> np.ndarray:
    return prisms_from_points(*regular_mesh_points(xlim, nx, ylim, ny, zlim, nz))


def padded_mesh_points(xlim, nx, ylim, ny, zlim, nz, npx, sx, npy, sy, npz, sz):
    """Mesh::generate_regular_mesh_with_padding (Mesh.cpp:516-587): the regular
    points of the area of interest, then npx / npy padding cells on both x / y
    sides and npz below, each one `s` times wider than the one inside it
    (starting from the first interior spacing)."""
    xi, yi, zi = regular_mesh_points(xlim, nx, ylim, ny, zlim, nz)

    def pad(inner, n, stretch, both):
        lo = n if both else 0
        pts = np.empty(inner.size + (2 * n if both else n))
        pts[lo:lo + inner.size] = inner
        d = inner[1] - inner[0]
        top = lo + inner.size - 1
        for i in range(n):
            d *= stretch
            pts[top + 1 + i] = pts[top + i] + d
            if both:
                pts[lo - 1 - i] = pts[lo - i] - d
        return pts

    return pad(xi, npx, sx, True), pad(yi, npy, sy, True), pad(zi, npz, sz, False)


def padded_mesh(xlim, nx, ylim, ny, zlim, nz, npx, sx, npy, sy, npz, sz) -> np.ndarray:
    return prisms_from_points(*padded_mesh_points(xlim, nx, ylim, ny, zlim, nz, npx, sx, npy, sy,
                                                  npz, sz))


def set_boxes(prisms: np.ndarray, boxes, values: np.ndarray | None = None) -> np.ndarray:
    """Density per cell from boxes (x0 x1 y0 y1 z0 z1 value), whole cells only."""
    p = np.asarray(prisms, dtype=np.float64)
    rho = np.zeros(p.shape[0]) if values is None else np.array(values, dtype=np.float64)

    def ge(a, b):
        return (a > b) | (np.abs(a - b) < 1e-10)

    def le(a, b):
        return (a < b) | (np.abs(a - b) < 1e-10)

    for b in boxes:
        x0, x1, y0, y1, z0, z1, v = b
        inside = (ge(p[:, 4], z0) & le(p[:, 5], z1) & ge(p[:, 0], x0) & le(p[:, 1], x1)
                  & ge(p[:, 2], y0) & le(p[:, 3], y1))
        rho[inside] = v
    return rho


def observation_grid(nx, x0, x1, ny, y0, y1, z0) -> np.ndarray:
    """(nx*ny, 3) points, x fastest, as Observation::generate."""
    xs = 0.0
    ys = 0.0
    if nx > 1:
        xs = (x1 - x0) / (nx - 1)
    if ny > 1:
        ys = (y1 - y0) / (ny - 1)
    iy, ix = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    return np.stack([x0 + ix.ravel() * xs, y0 + iy.ravel() * ys, np.full(nx * ny, float(z0))], 1)


def _halves(lo: float, hi: float, bit: int):
    mid = 0.5 * (hi + lo)  # RectPrism::get_center, RectPrism.cpp:45-50
    return (lo, mid) if bit == 0 else (mid, hi)


class Octree:
    """A regular base mesh refined by splitting leaf cells into octants the way
    Mesh::refinement does it (Mesh.cpp:1462-1942).

    * Face balance (Mesh.cpp:1474-1551): before a cell of level L splits, each
      face neighbour of level L - 1 is split first, recursively, so that cells
      sharing a face differ by one level at most.  Boundary faces impose
      nothing.  The set of leaves this gives does not depend on the order of
      the cascaded splits: it is the smallest face-balanced refinement that
      splits every requested cell.
    * Children (Mesh.cpp:1562-1600): split at the centre 0.5 (hi + lo), x
      outermost, then y, z innermost.
    * Leaf order (Mesh.cpp:830-847 for the base, 1930-1942 for a split): the
      base cells x outermost, z innermost, each split cell replaced in place
      by its eight children, i.e. a depth-first walk.

    Cells are keyed (level, i, j, k) with i, j, k indices on the level's grid
    of (nx, ny, nz) * 2**level cells.
    """

    def __init__(self, xs, ys, zs):
        self.pts = [np.asarray(v, dtype=np.float64) for v in (xs, ys, zs)]
        self.n = tuple(len(v) - 1 for v in self.pts)
        self.split_cells: set = set()
        self._bounds: dict = {}
        self._leaves = None

    @classmethod
    def regular(cls, xlim, nx, ylim, ny, zlim, nz) -> "Octree":
        return cls(*regular_mesh_points(xlim, nx, ylim, ny, zlim, nz))

    def bounds(self, key) -> tuple:
        """x0 x1 y0 y1 z0 z1 of a cell."""
        L, i, j, k = key
        if L == 0:
            xs, ys, zs = self.pts
            return (xs[i], xs[i + 1], ys[j], ys[j + 1], zs[k], zs[k + 1])
        b = self._bounds.get(key)
        if b is None:
            p = self.bounds((L - 1, i >> 1, j >> 1, k >> 1))
            b = (*_halves(p[0], p[1], i & 1), *_halves(p[2], p[3], j & 1),
                 *_halves(p[4], p[5], k & 1))
            self._bounds[key] = b
        return b

    def exists(self, key) -> bool:
        L, i, j, k = key
        if L == 0:
            return 0 <= i < self.n[0] and 0 <= j < self.n[1] and 0 <= k < self.n[2]
        return (L - 1, i >> 1, j >> 1, k >> 1) in self.split_cells

    def is_leaf(self, key) -> bool:
        return self.exists(key) and key not in self.split_cells

    def _split(self, key) -> None:
        L, i, j, k = key
        if L > 0:
            for a in range(3):
                for step in (-1, 1):
                    c = [i, j, k]
                    c[a] += step
                    if not 0 <= c[a] < (self.n[a] << L):
                        continue  # boundary face
                    nb = (L, c[0], c[1], c[2])
                    if not self.exists(nb):
                        coarse = (L - 1, c[0] >> 1, c[1] >> 1, c[2] >> 1)
                        if self.is_leaf(coarse):
                            self._split(coarse)
        self.split_cells.add(key)
        self._leaves = None

    def refine(self, leaf_indices) -> np.ndarray:
        """Split the given leaves (indices into the current ``leaf_keys()``) in
        ascending order, skipping those a cascade already split.  Returns the
        indices, in the old leaf order and ascending, of every leaf split
        (requested or cascaded): the parents AdaptiveInversion::expand_G
        replaces by their children."""
        keys = self.leaf_keys()
        before = set(self.split_cells)
        for t in sorted(int(v) for v in np.asarray(leaf_indices).ravel()):
            if self.is_leaf(keys[t]):
                self._split(keys[t])
        new = self.split_cells - before
        return np.array([t for t, k in enumerate(keys) if k in new], dtype=np.int64)

    def parent_leaf(self, split: np.ndarray, n_old: int) -> np.ndarray:
        """For each current leaf, the index of the old leaf it lies in, after a
        refine() that split the old leaves `split` (children inherit their
        parent's values, Mesh.cpp:1575-1590)."""
        out, prev = [], 0
        for j in np.asarray(split, dtype=np.int64):
            out.extend(range(prev, int(j)))
            out.extend([int(j)] * 8)
            prev = int(j) + 1
        out.extend(range(prev, n_old))
        return np.array(out, dtype=np.int64)

    def leaf_keys(self) -> list:
        if self._leaves is None:
            out = []
            nx, ny, nz = self.n
            for i in range(nx):
                for j in range(ny):
                    for k in range(nz):
                        stack = [(0, i, j, k)]
                        while stack:
                            key = stack.pop()
                            if key in self.split_cells:
                                L, a, b, c = key
                                for o in range(7, -1, -1):
                                    stack.append((L + 1, 2 * a + (o >> 2), 2 * b + ((o >> 1) & 1),
                                                  2 * c + (o & 1)))
                            else:
                                out.append(key)
            self._leaves = out
        return self._leaves

    def wavelet_order(self) -> np.ndarray:
        """Mesh::get_reordered_id for every position: the leaf index of the
        i-th cell in the sequence the wavelet compression runs along
        (ro_leaf_cells).  Base cells: x outermost, then y, with z running
        forward and backward on alternate (x, y) lines (Mesh.cpp:855-892); a
        split cell is replaced by its children in the order 0 2 6 4 5 7 3 1
        when its line runs forward, 1 3 7 5 4 6 2 0 otherwise, the children
        keeping the parent's direction (Mesh.cpp:1605, 1946-1960)."""
        index = {k: t for t, k in enumerate(self.leaf_keys())}
        fwd_kids = (0, 2, 6, 4, 5, 7, 3, 1)
        bwd_kids = (1, 3, 7, 5, 4, 6, 2, 0)
        out = []
        nx, ny, nz = self.n
        for i in range(nx):
            for j in range(ny):
                forward = (i * ny + j) % 2 == 0
                kids = fwd_kids if forward else bwd_kids
                for kk in range(nz):
                    k = kk if forward else nz - 1 - kk
                    stack = [(0, i, j, k)]
                    while stack:
                        key = stack.pop()
                        if key in self.split_cells:
                            L, a, b, c = key
                            for o in reversed(kids):
                                stack.append((L + 1, 2 * a + (o >> 2), 2 * b + ((o >> 1) & 1),
                                              2 * c + (o & 1)))
                        else:
                            out.append(index[key])
        return np.array(out, dtype=np.int64)

    def leaves(self) -> np.ndarray:
        """(n, 6) leaf cells x0 x1 y0 y1 z0 z1 in leaf order."""
        return np.array([self.bounds(k) for k in self.leaf_keys()], dtype=np.float64).reshape(-1, 6)

    def levels(self) -> np.ndarray:
        return np.array([k[0] for k in self.leaf_keys()], dtype=np.int64)


class Multilinear:
    """Multilinear interpolation of values on a rectilinear x, y, z grid, the
    interpolator the reference builds from a gridded constraint model
    (InversionBase.cpp:1305-1307, the vendored Linterp InterpMultilinear):

    * per axis the cell is found by an upper bound in the grid; a coordinate
      below the first grid point takes the first point's values, one at or
      beyond the last takes the last's (no extrapolation), and inside the
      fraction (x - g_c) / (g_c+1 - g_c) is clamped to [0, 1];
    * the eight corner values are combined x first: lower + t_x (upper -
      lower), each side combining y then z the same way.

    values: (nx, ny, nz), x outermost."""

    def __init__(self, grid_x, grid_y, grid_z, values):
        self.grids = [np.asarray(g, dtype=np.float64) for g in (grid_x, grid_y, grid_z)]
        self.values = np.asarray(values, dtype=np.float64).reshape([g.size for g in self.grids])
        for g in self.grids:
            if g.size < 1 or np.any(np.diff(g) <= 0):
                raise ValueError("grid coordinates must increase")

    def __call__(self, points) -> np.ndarray:
        p = np.asarray(points, dtype=np.float64).reshape(-1, 3)
        lo, hi, t = [], [], []
        for d, g in enumerate(self.grids):
            x = p[:, d]
            n = g.size
            c = np.searchsorted(g, x, side="right") - 1
            c = np.where(x < g[0], -1, np.where(x >= g[-1], n - 1, c))
            inner = (c >= 0) & (c < n - 1)
            ci = np.clip(c, 0, max(n - 2, 0))
            y = np.zeros(x.size)
            if n >= 2:
                with np.errstate(invalid="ignore", divide="ignore"):
                    yy = (x - g[ci]) / (g[np.minimum(ci + 1, n - 1)] - g[ci])
                y = np.where(inner, np.clip(yy, 0.0, 1.0), y)
            y = np.where(c == -1, 1.0, y)
            lo.append(np.where(c < 0, 0, np.where(c >= n - 1, n - 1, c)))
            hi.append(np.where(c < 0, 0, np.where(c >= n - 1, n - 1, c + 1)))
            t.append(y)
        f = self.values

        def corner(bx, by, bz):
            return f[(hi[0] if bx else lo[0]), (hi[1] if by else lo[1]), (hi[2] if bz else lo[2])]

        def along_z(bx, by):
            a, b = corner(bx, by, 0), corner(bx, by, 1)
            return a + t[2] * (b - a)

        def along_y(bx):
            a, b = along_z(bx, 0), along_z(bx, 1)
            return a + t[1] * (b - a)

        a, b = along_y(0), along_y(1)
        return a + t[0] * (b - a)


def cell_centres(cells) -> np.ndarray:
    """RectPrism::get_center of each cell (RectPrism.cpp:45-50)."""
    c = np.asarray(cells, dtype=np.float64).reshape(-1, 6)
    return np.stack([0.5 * (c[:, 1] + c[:, 0]), 0.5 * (c[:, 3] + c[:, 2]),
                     0.5 * (c[:, 5] + c[:, 4])], 1)
