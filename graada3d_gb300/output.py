"""Result writers in the reference's text and VTK formats.

The reference writes its results on the host (GraAda3D.cpp:792-806); these
writers take device results (the inverted model, the observed and the
predicted data) and produce the same files byte for byte:

* ``write_model_txt``        -- Mesh::out_model_txt, Mesh.cpp:1416-1460
* ``write_model_vtk``        -- Mesh::out_model_vtk, Mesh.cpp:1160-1287
* ``write_model_vtk_points`` -- Mesh::out_model_vtk_points, Mesh.cpp:1289-1415
* ``write_data``             -- InversionBase::out_data, InversionBase.cpp:743-784
* ``write_data_vtk``         -- InversionBase::out_data_vtk, InversionBase.cpp:798-880

Number formats are those of the C++ streams the reference uses: a bare
``<<`` of a double prints ``%.6g``; ``scientific`` with ``setprecision(p)``
and ``setw(w) << left`` prints ``%-w.pe``.  VTK point ids follow the order of
a ``std::set<Point>``: coordinates compared lexicographically (x, then y,
then z), points whose coordinate differences sum to less than 3e-12 being one
point (Point::operator== / operator<, Point.cpp:111-142, TOL from gs.h:19).
"""
from __future__ import annotations

import numpy as np

COMPONENT_NAMES = ["V", "g_z", "g_x", "g_y", "T_zz", "T_xz", "T_yz", "T_xx", "T_xy", "T_yy"]
_POINT_EQ = 3 * 1.0e-12


def _g(v) -> str:
    return "%.6g" % v


def _cells(cells) -> np.ndarray:
    c = np.asarray(cells, dtype=np.float64).reshape(-1, 6)
    return c


def _centers(c: np.ndarray) -> np.ndarray:
    # RectPrism::get_center, RectPrism.cpp:45-50
    return np.stack([0.5 * (c[:, 1] + c[:, 0]), 0.5 * (c[:, 3] + c[:, 2]),
                     0.5 * (c[:, 5] + c[:, 4])], 1)


def component_names(mask: int) -> list:
    return [COMPONENT_NAMES[b] for b in range(10) if (int(mask) >> b) & 1]


def write_model_txt(path, cells, values) -> None:
    c = _cells(cells)
    v = np.asarray(values, dtype=np.float64).ravel()
    if v.size != c.shape[0]:
        raise ValueError("one value per cell expected")
    ctr = _centers(c)
    labels = ["#x0(m)", "x1(m)", "#y0(m)", "y1(m)", "#z0(m)", "z1(m)", "xc(m)", "yc(m)", "zc(m)",
              "value"]
    rows = np.column_stack([c, ctr, v])
    fmt = "%-22.14e" * 10 + "\n"
    with open(path, "w") as fh:
        fh.write("#The first 6 parameters give the dimensions of a cell. The 7-9 parameters are "
                 "the cell center. The 10th parameter is the value within the cell.\n")
        fh.write("".join("%-22s" % s for s in labels) + "\n")
        fh.write("".join(fmt % tuple(r) for r in rows.tolist()))


def _vertex_ids(c: np.ndarray):
    """Unique vertices in std::set<Point> order and each cell's 8 vertex ids in
    the reference's corner order (x1y1z1, x2y1z1, x2y2z1, x1y2z1, then z2)."""
    x1, x2, y1, y2, z1, z2 = (c[:, k] for k in range(6))
    corners = [(x1, y1, z1), (x2, y1, z1), (x2, y2, z1), (x1, y2, z1),
               (x1, y1, z2), (x2, y1, z2), (x2, y2, z2), (x1, y2, z2)]
    pts = np.stack([np.stack(v, 1) for v in corners], 1).reshape(-1, 3)  # cell-major
    order = np.lexsort((pts[:, 2], pts[:, 1], pts[:, 0]))
    sp = pts[order]
    new = np.ones(sp.shape[0], dtype=bool)
    new[1:] = np.abs(np.diff(sp, axis=0)).sum(1) >= _POINT_EQ
    group = np.cumsum(new) - 1
    starts = np.nonzero(new)[0]
    # a set keeps the first point inserted of those it holds as equal
    first = np.minimum.reduceat(order, starts)
    ids = np.empty(pts.shape[0], dtype=np.int64)
    ids[order] = group
    return pts[first], ids.reshape(-1, 8)


def _cell_data(fh, n: int, params) -> None:
    for j, (name, vals) in enumerate(params):
        v = np.asarray(vals, dtype=np.float64).ravel()
        if v.size != n:
            raise ValueError(f"{name}: {n} values expected")
        fh.write(f"SCALARS {name} double 1\nLOOKUP_TABLE table{j}\n")
        fh.write("".join(_g(x) + "\n" for x in v.tolist()))


def _params(params):
    if isinstance(params, dict):
        return list(params.items())
    return list(params)


def write_model_vtk(path, cells, params) -> None:
    """``params``: (name, values) pairs or a dict, one value per cell each."""
    c = _cells(cells)
    params = _params(params)
    verts, ids = _vertex_ids(c)
    n = c.shape[0]
    with open(path, "w") as fh:
        fh.write("# vtk DataFile Version 3.0\nGravity inversion using rectangular prisms\nASCII\n"
                 "DATASET UNSTRUCTURED_GRID\n")
        fh.write(f"\nPOINTS\t{verts.shape[0]}\tdouble\n")
        fh.write("".join(f"{_g(x)}\t{_g(y)}\t{_g(z)}\n" for x, y, z in verts.tolist()))
        fh.write(f"\nCELLS\t{n}\t{n * 9}\n")
        fh.write("".join("8\t" + "".join(f"{k}\t" for k in row) + "\n" for row in ids.tolist()))
        fh.write(f"\nCELL_TYPES\t{n}\n")
        fh.write("12\n" * n)
        fh.write(f"\nCELL_DATA\t{n}\n")
        _cell_data(fh, n, params)
        fh.write("\n")


def write_model_vtk_points(path, cells, params) -> None:
    c = _cells(cells)
    params = _params(params)
    n = c.shape[0]
    ctr = _centers(c)
    with open(path, "w") as fh:
        fh.write("# vtk DataFile Version 3.0\nGravity inversion using rectangular prisms\nASCII\n"
                 "DATASET UNSTRUCTURED_GRID\n")
        fh.write(f"\nPOINTS\t{n}\tdouble\n")
        fh.write("".join(f"{_g(x)}\t{_g(y)}\t{_g(z)}\n" for x, y, z in ctr.tolist()))
        fh.write(f"\nCELLS\t{n}\t{n * 2}\n")
        fh.write("".join(f"1\t{i}\n" for i in range(n)))
        fh.write(f"\nCELL_TYPES\t{n}\n")
        fh.write("1\n" * n)
        fh.write(f"\nCELL_DATA\t{n}\n")
        _cell_data(fh, n, params)
        fh.write(f"\nPOINT_DATA\t{n}\n")
        _cell_data(fh, n, params)
        fh.write("\n")


def _split_data(obs, d, mask):
    o = np.asarray(obs, dtype=np.float64).reshape(-1, 3)
    names = component_names(mask)
    v = np.asarray(d, dtype=np.float64).ravel()
    if v.size != o.shape[0] * len(names):
        raise ValueError("data size is not points x components")
    return o, names, v.reshape(len(names), o.shape[0])


def write_data(out_name, obs, d, mask) -> list:
    """One file per component, ``<out_name>_<component>``; returns their names."""
    o, names, v = _split_data(obs, d, mask)
    fmt = "%-30.15e" * 4 + "\n"
    files = []
    for j, name in enumerate(names):
        fn = f"{out_name}_{name}"
        with open(fn, "w") as fh:
            fh.write("".join(fmt % (p[0], p[1], p[2], x) for p, x in zip(o.tolist(), v[j].tolist())))
        files.append(fn)
    return files


def write_data_vtk(path, obs, d, mask) -> None:
    o, names, v = _split_data(obs, d, mask)
    n = o.shape[0]
    params = list(zip(names, v))
    with open(path, "w") as fh:
        fh.write("# vtk DataFile Version 3.0\nGravity effects\nASCII\nDATASET UNSTRUCTURED_GRID\n")
        fh.write(f"\nPOINTS\t{n}\tdouble\n")
        fh.write("".join(f"{_g(x)}\t{_g(y)}\t{_g(z)}\n" for x, y, z in o.tolist()))
        fh.write(f"\nCELLS\t{n}\t{n * 2}\n")
        fh.write("".join(f"1\t{i}\n" for i in range(n)))
        fh.write(f"\nCELL_TYPES\t{n}\n")
        fh.write("1\n" * n)
        fh.write(f"\nCELL_DATA\t{n}\n")
        _cell_data(fh, n, params)
        fh.write(f"\nPOINT_DATA\t{n}\n")
        _cell_data(fh, n, params)
        fh.write("\n")
