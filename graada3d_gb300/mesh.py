"""Host-side mesh and observation helpers with the reference's conventions.

Mesh construction and refinement stay on the host in the reference; these
helpers build the same regular meshes and observation grids as
``Mesh::generate_regular_mesh`` and ``Observation::generate`` so that tests
and benchmarks can feed the GPU path the cell order and coordinates the
reference would produce.

* ``regular_mesh`` -- Mesh.cpp:500-514 (grid points from Eigen's LinSpaced)
  and Mesh.cpp:830-847 (leaf order: x outermost, then y, z innermost).
* ``set_boxes`` -- Mesh::set_parameter_in_a_region, Mesh.cpp:1079-1107: a
  cell takes a box's value when it lies entirely inside the box (1e-10
  tolerance); later boxes overwrite earlier ones.
* ``observation_grid`` -- Observation::generate, Observation.cpp:48-77
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
