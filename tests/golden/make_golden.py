"""Generate the golden fixtures under tests/golden/ from the reference.

Run in a checkout that has the reference tree (the one ``make -C oracle -s refdir``
names, or GRADA_REFERENCE) after ``make -C oracle all ref``:

    python tests/golden/make_golden.py [--ref REFERENCE_TREE] [--only NAME]

Fixtures written (all .npz):
  forward_models.npz  the reference's committed noise-free forward fields
                      (Examples/Forward_modelling/{model1,model2,model3}/result/
                      data_no_noise and tests/test_compute/result_no_noise) with
                      the observation points read from the same files and the
                      density model rebuilt from the anomaly lists the
                      examples' makeModel calls use.
  ref_fields.npz      G blocks (all ten components) from the reference's own
                      GravFormula, compiled from its sources into
                      oracle/_ref/ref_fields, on seeded geometries including
                      degenerate ones (points on cell-face planes and above
                      vertical edges, far-away cells).
  ref_operators.npz   regularisation operators on an octree-refined mesh
                      (oracle/_ref/ref_operators).
  ref_output.npz      the files the reference's result writers produce, with
                      their inputs (oracle/_ref/ref_output).
  ref_adapt.npz       one AdaptiveInversion::refine_mesh of the reference
                      (oracle/_ref/ref_adapt).
  ref_interp.npz      the structure-model interpolation and a "crg" refinement
                      (oracle/_ref/ref_interp).
  ref_inversion_*.npz regular-mesh inversion problems with the reference's
                      G, host-built operators, one solve_cg call and a full
                      invert_with_own_CG run (oracle/_ref/ref_inversion).
  ref_adaptive_inversion.npz  the adaptive inversion (invert_with_own_CG with
                      two mesh refinements): final leaves, model, records and
                      the cells split per refinement (oracle/_ref/ref_inversion).
  ref_adaptive_{crg,pet}_inversion.npz  the same with a gridded constraint
                      model: the structure model (cross-gradient, T rebuilt at
                      each refinement) or the reference model, interpolated
                      onto the children (oracle/_ref/ref_inversion).
"""
from __future__ import annotations

import argparse
import os
import re
import struct
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
REF_BIN = REPO / "oracle" / "_ref"

# ---------------------------------------------------------------------------
# forward models from Examples/Forward_modelling
# ---------------------------------------------------------------------------

FIELD_BIT = {"V": 0, "gz": 1, "gx": 2, "gy": 3, "Tzz": 4, "Txz": 5, "Tyz": 6, "Txx": 7, "Txy": 8,
             "Tyy": 9}
HEADER_FIELD = {"g_z": "gz", "g_x": "gx", "g_y": "gy", "T_zz": "Tzz", "T_xz": "Txz",
                "T_yz": "Tyz", "T_xx": "Txx", "T_xy": "Txy", "T_yy": "Tyy", "V": "V"}


def parse_make_model(script: str):
    """-R x0/x1/y0/y1/z0/z1 --nx --ny --nz and -a boxes of the first makeModel line."""
    for line in script.splitlines():
        line = line.split("#", 1)[0]
        if "makeModel" not in line:
            continue
        R = re.search(r"-R\s+(\S+)", line).group(1).split("/")
        nx = int(re.search(r"--nx\s+(\d+)", line).group(1))
        ny = int(re.search(r"--ny\s+(\d+)", line).group(1))
        nz = int(re.search(r"--nz\s+(\d+)", line).group(1))
        boxes = [list(map(float, a.split("/"))) for a in re.findall(r"-a\s+(\S+)", line)]
        afile = re.search(r"-A\s+(\S+)", line)
        return [float(v) for v in R], (nx, ny, nz), boxes, (afile.group(1) if afile else None)
    raise ValueError("no makeModel line")


def read_anomaly_file(path: Path):
    boxes = []
    for line in path.read_text().splitlines():
        line = line.split("#", 1)[0].strip()
        if line:
            boxes.append([float(v) for v in line.split()[:7]])
    return boxes


def read_data_file(path: Path):
    lines = path.read_text().splitlines()
    header = lines[0]
    names = [HEADER_FIELD[m] for m in re.findall(r"([gT]_[xyz]{1,2}|V) \(", header)]
    arr = np.array([[float(v) for v in l.split()] for l in lines[1:] if l.strip()])
    return names, arr[:, :3], arr[:, 3:]


def forward_models(ref: Path) -> None:
    ex = ref / "Examples" / "Forward_modelling"
    cases = {
        "model1": (ex / "model1" / "build_density_model2.sh", ex / "model1" / "result" / "data_no_noise"),
        "model2": (ex / "model2" / "build_density_model.sh", ex / "model2" / "result" / "data_no_noise"),
        "model3": (ex / "model3" / "build_density_model.sh", ex / "model3" / "result" / "data_no_noise"),
        "test_compute": (ex / "tests" / "test_make_model" / "build.sh",
                         ex / "tests" / "test_compute" / "result_no_noise"),
    }
    out = {}
    for name, (script, data) in cases.items():
        R, n, boxes, afile = parse_make_model(script.read_text())
        if afile:
            boxes = read_anomaly_file(script.parent / afile)
        names, obs, fields = read_data_file(data)
        mask = 0
        for f in names:
            mask |= 1 << FIELD_BIT[f]
        # the file lists components in the order compute.cpp writes them, which is
        # ascending field-bit order
        assert [FIELD_BIT[f] for f in names] == sorted(FIELD_BIT[f] for f in names)
        out[f"{name}_region"] = np.array(R)
        out[f"{name}_n"] = np.array(n, dtype=np.int64)
        out[f"{name}_boxes"] = np.array(boxes)
        out[f"{name}_obs"] = obs
        out[f"{name}_fields"] = fields
        out[f"{name}_mask"] = np.array(mask, dtype=np.int64)
        print(f"{name}: {len(boxes)} boxes, {obs.shape[0]} points, fields {names}")
    out["cases"] = np.array(list(cases))
    np.savez_compressed(HERE / "forward_models.npz", **out)


# ---------------------------------------------------------------------------
# G blocks from the compiled reference kernels
# ---------------------------------------------------------------------------


def run_ref_fields(prisms: np.ndarray, obs: np.ndarray, mask: int) -> np.ndarray:
    exe = REF_BIN / "ref_fields"
    with tempfile.TemporaryDirectory() as td:
        fin, fout = Path(td) / "in.bin", Path(td) / "out.bin"
        with open(fin, "wb") as f:
            f.write(struct.pack("<qqI", prisms.shape[0], obs.shape[0], mask))
            f.write(np.ascontiguousarray(prisms, dtype="<f8").tobytes())
            f.write(np.ascontiguousarray(obs, dtype="<f8").tobytes())
        subprocess.run([str(exe), str(fin), str(fout)], check=True)
        nf = bin(mask).count("1")
        G = np.fromfile(fout, dtype="<f8").reshape(prisms.shape[0], nf * obs.shape[0]).T
    return np.asfortranarray(G)


def regular_prisms(xl, yl, zl, nx, ny, nz):
    """Cells of Mesh::generate_regular_mesh in leaf order (x outer, z inner)."""
    def pts(a, b, n):
        step = (b - a) / n
        v = a + step * np.arange(n + 1)
        v[-1] = b
        return v
    xs, ys, zs = pts(*xl, nx), pts(*yl, ny), pts(*zl, nz)
    out = np.empty((nx * ny * nz, 6))
    idx = 0
    for i in range(nx):
        for j in range(ny):
            for k in range(nz):
                out[idx] = [xs[i], xs[i + 1], ys[j], ys[j + 1], zs[k], zs[k + 1]]
                idx += 1
    return out


def exact_field(ob, pr):
    """Closed-form corner sums of 1/r's antiderivatives (see prism.cuh) in
    40-digit arithmetic: an independent, cancellation-free value of all ten
    components for one (point, prism) pair."""
    import mpmath as mp

    mp.mp.dps = 40
    g0 = mp.mpf("6.673e-11")
    px, py, pz = (mp.mpf(float(v)) for v in ob)
    X = [mp.mpf(float(pr[0])) - px, mp.mpf(float(pr[1])) - px]
    Y = [mp.mpf(float(pr[2])) - py, mp.mpf(float(pr[3])) - py]
    Z = [mp.mpf(float(pr[4])) - pz, mp.mpf(float(pr[5])) - pz]
    acc = [mp.mpf(0)] * 10

    def at(b, a):  # atan(b/a); a == 0 terms cancel between the faces they touch
        return mp.mpf(0) if a == 0 else mp.atan(b / a)

    def ln(v):  # only reached with v > 0 for points outside the prism
        return mp.log(v) if v > 0 else mp.mpf(0)

    for i in range(2):
        for j in range(2):
            for k in range(2):
                x, y, z = X[i], Y[j], Z[k]
                s = (-1) ** (i + j + k + 1)
                r = mp.sqrt(x * x + y * y + z * z)
                lx, ly, lz = ln(x + r), ln(y + r), ln(z + r)
                ax, ay, az = at(y * z, x * r), at(x * z, y * r), at(x * y, z * r)
                v = [x * y * lz + y * z * lx + z * x * ly - x * x * ax / 2 - y * y * ay / 2 - z * z * az / 2,
                     -(x * ly + y * lx - z * az), -(y * lz + z * ly - x * ax), -(z * lx + x * lz - y * ay),
                     -az, ly, lx, -ax, lz, -ay]
                for c in range(10):
                    acc[c] += s * v[c]
    sc = [g0] + [g0 * 100000] * 3 + [g0 * 1000000000] * 6
    return np.array([float(acc[c] * sc[c]) for c in range(10)])


def exact_G(prisms, obs):
    n = obs.shape[0]
    E = np.zeros((10 * n, prisms.shape[0]), order="F")
    for i in range(n):
        for j in range(prisms.shape[0]):
            e = exact_field(obs[i], prisms[j])
            for k in range(10):
                E[i + k * n, j] = e[k]
    return E


def ref_fields() -> None:
    rng = np.random.default_rng(20240601)
    cases = {}
    # (a) random prisms, random points above them
    n = 64
    x0 = rng.uniform(-2000, 2000, n); dx = rng.uniform(20, 600, n)
    y0 = rng.uniform(-2000, 2000, n); dy = rng.uniform(20, 600, n)
    z0 = rng.uniform(0, 1500, n); dz = rng.uniform(20, 600, n)
    pr = np.stack([x0, x0 + dx, y0, y0 + dy, z0, z0 + dz], 1)
    ob = np.stack([rng.uniform(-2500, 2500, 48), rng.uniform(-2500, 2500, 48),
                   -rng.uniform(0.05, 300, 48)], 1)
    cases["random"] = (pr, ob)
    # (b) regular mesh with points on the cell-face planes (x, y multiples of the cell size)
    pr = regular_prisms((0.0, 400.0), (0.0, 300.0), (0.0, 200.0), 4, 3, 2)
    gx, gy = np.meshgrid(np.arange(-100.0, 501.0, 100.0), np.arange(-100.0, 401.0, 50.0), indexing="xy")
    ob = np.stack([gx.ravel(), gy.ravel(), np.full(gx.size, -0.1)], 1)
    cases["coincident"] = (pr, ob)
    # (c) far field: 50 m cells seen from 20-60 km away
    pr = regular_prisms((0.0, 100.0), (0.0, 100.0), (0.0, 100.0), 2, 2, 2)
    ang = rng.uniform(0, 2 * np.pi, 24); dist = rng.uniform(2e4, 6e4, 24)
    ob = np.stack([dist * np.cos(ang), dist * np.sin(ang), -rng.uniform(1, 500, 24)], 1)
    cases["far"] = (pr, ob)
    # (d) points above vertical edges and above the centre of a cell
    pr = np.array([[0.0, 100.0, 0.0, 80.0, 10.0, 60.0], [100.0, 250.0, 0.0, 80.0, 10.0, 60.0]])
    ob = np.array([[0.0, 0.0, -5.0], [100.0, 80.0, -0.1], [50.0, 40.0, -1.0], [250.0, 0.0, -20.0],
                   [100.0, 40.0, -0.5], [175.0, 0.0, -3.0]])
    cases["edges"] = (pr, ob)
    out = {}
    for name, (pr, ob) in cases.items():
        G = run_ref_fields(pr, ob, 0x3FF)
        out[f"{name}_prisms"] = pr
        out[f"{name}_obs"] = ob
        out[f"{name}_G"] = G
        out[f"{name}_exact"] = exact_G(pr, ob)
        print(f"ref_fields {name}: G {G.shape}")
    out["cases"] = np.array(list(cases))
    np.savez_compressed(HERE / "ref_fields.npz", **out)


def ref_expand() -> None:
    """ref_expand.npz: the reference's own refinement path on a 6 x 5 x 4 regular mesh
    (Fwd::compute_G, Mesh::refinement of six cells, Mesh::rearrange_id,
    AdaptiveInversion::expand_G, run by oracle/_ref/ref_expand): the expanded G
    (nine components at 6 x 4 points), the refined leaf list and each split
    parent's children in Cell::child_cells order."""
    from graada3d_gb300 import mesh as gm

    exe = REF_BIN / "ref_expand"
    nx, ny, nz = 6, 5, 4
    xl, yl, zl = (0.0, 600.0), (0.0, 500.0), (0.0, 400.0)
    obs = gm.observation_grid(6, -50.0, 650.0, 4, -50.0, 550.0, -5.0)
    mask = 0x3FE
    parents = np.array([0, 3, 17, 18, 50, 119], dtype=np.int64)
    with tempfile.TemporaryDirectory() as td:
        fin, fout = Path(td) / "in.bin", Path(td) / "out.bin"
        with open(fin, "wb") as fh:
            np.array([nx, ny, nz], dtype=np.int64).tofile(fh)
            np.array([*xl, *yl, *zl], dtype=np.float64).tofile(fh)
            np.array([obs.shape[0]], dtype=np.int64).tofile(fh)
            obs.astype(np.float64).tofile(fh)
            np.array([mask], dtype=np.uint32).tofile(fh)
            np.array([parents.size], dtype=np.int64).tofile(fh)
            parents.tofile(fh)
        subprocess.run([str(exe), str(fin), str(fout)], check=True, cwd=td)
        raw = np.fromfile(fout, dtype=np.uint8)
    off = 0

    def take(n, dt):
        nonlocal off
        a = raw[off:off + n * np.dtype(dt).itemsize].view(dt)
        off += n * np.dtype(dt).itemsize
        return a

    rows, cols = take(2, np.int64)
    G = take(rows * cols, np.float64).reshape(cols, rows).T
    n_leaf = int(take(1, np.int64)[0])
    leaf = take(6 * n_leaf, np.float64).reshape(n_leaf, 6)
    n_split = int(take(1, np.int64)[0])
    idx, kids = [], []
    for _ in range(n_split):
        idx.append(int(take(1, np.int64)[0]))
        kids.append(take(48, np.float64).reshape(8, 6))
    prisms = gm.regular_mesh(xl, nx, yl, ny, zl, nz)
    np.savez_compressed(HERE / "ref_expand.npz", prisms=prisms, obs=obs, mask=np.int64(mask),
                        parents=parents, G=G, leaf=leaf, split_index=np.array(idx),
                        children=np.array(kids))


def ref_padded() -> None:
    """ref_padded.npz: the reference's padded mesh (Mesh::generate_regular_mesh_with_padding:
    6 x 5 x 4 cells of interest over [0, 3 km]^2 x [0, 1.5 km] with 4 padding cells on each
    x/y side and 3 below, stretch 1.8) and its Fwd::compute_G for nine components at 5 x 4
    points, run by oracle/_ref/ref_padded.  Stored compactly: the leaf cells, a seeded
    density model with the reference's G rho, and twelve whole columns of G (cells of
    interest and the largest, farthest padding cells)."""
    exe = REF_BIN / "ref_padded"
    from graada3d_gb300 import mesh as gm

    obs = gm.observation_grid(5, -500.0, 3500.0, 4, -500.0, 3500.0, -10.0)
    mask = 0x3FE
    with tempfile.TemporaryDirectory() as td:
        fin, fout = Path(td) / "in.bin", Path(td) / "out.bin"
        with open(fin, "wb") as fh:
            np.array([6, 5, 4], dtype=np.int64).tofile(fh)
            np.array([0.0, 3000.0, 0.0, 3000.0, 0.0, 1500.0], dtype=np.float64).tofile(fh)
            np.array([4, 4, 3], dtype=np.int64).tofile(fh)
            np.array([1.8, 1.8, 1.8], dtype=np.float64).tofile(fh)
            np.array([obs.shape[0]], dtype=np.int64).tofile(fh)
            obs.astype(np.float64).tofile(fh)
            np.array([mask], dtype=np.uint32).tofile(fh)
        subprocess.run([str(exe), str(fin), str(fout)], check=True, cwd=td)
        raw = np.fromfile(fout, dtype=np.uint8)
    n_leaf = int(raw[:8].view(np.int64)[0])
    leaf = raw[8:8 + 48 * n_leaf].view(np.float64).reshape(n_leaf, 6)
    off = 8 + 48 * n_leaf
    rows, cols = raw[off:off + 16].view(np.int64)
    G = raw[off + 16:off + 16 + 8 * rows * cols].view(np.float64).reshape(cols, rows).T
    rng = np.random.default_rng(31)
    rho = rng.uniform(-300.0, 300.0, n_leaf)
    vol = (leaf[:, 1] - leaf[:, 0]) * (leaf[:, 3] - leaf[:, 2]) * (leaf[:, 5] - leaf[:, 4])
    cols_pick = np.unique(np.concatenate([np.argsort(vol)[-6:], np.argsort(vol)[:3],
                                          [0, n_leaf // 2, n_leaf - 1]]))
    np.savez_compressed(HERE / "ref_padded.npz", leaf=leaf, obs=obs, mask=np.int64(mask),
                        rho=rho, d=G @ rho, cols=cols_pick, G_cols=G[:, cols_pick])


def ref_indicator() -> None:
    """ref_indicator.npz: the reference's refinement indicator
    (AdaptiveInversion::indicator_calculator) on a 6 x 5 x 4 mesh refined at six cells,
    for a seeded model, with the (neighbour, face area) list of every cell in the
    order the reference adds them (oracle/_ref/ref_indicator)."""
    exe = REF_BIN / "ref_indicator"
    parents = np.array([0, 3, 17, 18, 50, 119], dtype=np.int64)
    with tempfile.TemporaryDirectory() as td:
        fin, fout = Path(td) / "in.bin", Path(td) / "out.bin"
        with open(fin, "wb") as fh:
            np.array([6, 5, 4], dtype=np.int64).tofile(fh)
            np.array([0.0, 600.0, 0.0, 500.0, 0.0, 400.0], dtype=np.float64).tofile(fh)
            np.array([parents.size], dtype=np.int64).tofile(fh)
            parents.tofile(fh)
            np.array([12345], dtype=np.uint64).tofile(fh)
        subprocess.run([str(exe), str(fin), str(fout)], check=True, cwd=td)
        raw = np.fromfile(fout, dtype=np.uint8)
    off = 0

    def take(cnt, dt):
        nonlocal off
        a = raw[off:off + cnt * np.dtype(dt).itemsize].view(dt)
        off += cnt * np.dtype(dt).itemsize
        return a

    n = int(take(1, np.int64)[0])
    leaf = take(6 * n, np.float64).reshape(n, 6)
    m = take(n, np.float64)
    ind = take(n, np.float64)
    nnz = int(take(1, np.int64)[0])
    rowptr = take(n + 1, np.int64)
    nb = take(nnz, np.int64)
    area = take(nnz, np.float64)
    np.savez_compressed(HERE / "ref_indicator.npz", leaf=leaf, m=m, indicator=ind,
                        rowptr=rowptr, neighbour=nb, area=area)


REFINE_PASSES = [
    # first refinement pass: base cells, one at the +x and one at the +z boundary
    [(150.0, 250.0, 150.0), (450.0, 250.0, 150.0), (250.0, 250.0, 250.0), (550.0, 50.0, 350.0)],
    # second pass: level-1 cells against unrefined neighbours (face-balance cascades)
    [(110.0, 210.0, 110.0), (590.0, 60.0, 390.0), (240.0, 240.0, 210.0)],
    # third pass: a level-2 cell whose neighbours are level 1 (cascade of two levels)
    [(101.0, 201.0, 101.0), (595.0, 55.0, 395.0)],
]


def ref_operators() -> None:
    """ref_operators.npz: the reference's regularisation operators on a 6 x 5 x 4
    mesh refined in three passes by Mesh::refinement (cascades included): leaf
    cells and levels, D_x1/D_y1/D_z1, V, Z, Ws/Wx/Wy/Wz, for a seeded
    structure model T_x/T_y/T_z, the face table the drop-in reads from the
    reference's Face objects and Mesh::get_reordered_id of every position
    (oracle/_ref/ref_operators)."""
    exe = REF_BIN / "ref_operators"
    obs = np.array([[120.0, 80.0, -20.0], [300.0, 260.0, -35.0], [520.0, 430.0, -10.0],
                    [80.0, 470.0, -25.0]])
    alphas = np.array([1.0, 1.3, 0.7, 1.1])  # a_s, a_z, a_x, a_y
    beta = 1.5
    with tempfile.TemporaryDirectory() as td:
        fin, fout = Path(td) / "in.bin", Path(td) / "out.bin"
        with open(fin, "wb") as fh:
            np.array([6, 5, 4], dtype=np.int64).tofile(fh)
            np.array([0.0, 600.0, 0.0, 500.0, 0.0, 400.0], dtype=np.float64).tofile(fh)
            np.array([len(REFINE_PASSES)], dtype=np.int64).tofile(fh)
            for r in REFINE_PASSES:
                np.array([len(r)], dtype=np.int64).tofile(fh)
                np.array(r, dtype=np.float64).tofile(fh)
            np.array([obs.shape[0]], dtype=np.int64).tofile(fh)
            obs.tofile(fh)
            np.array([beta], dtype=np.float64).tofile(fh)
            alphas.tofile(fh)
            np.array([777], dtype=np.uint64).tofile(fh)
        subprocess.run([str(exe), str(fin), str(fout)], check=True, cwd=td)
        raw = np.fromfile(fout, dtype=np.uint8)
    off = 0

    def take(cnt, dt):
        nonlocal off
        a = raw[off:off + cnt * np.dtype(dt).itemsize].view(dt)
        off += cnt * np.dtype(dt).itemsize
        return a

    out = {}

    def csr(key):
        n = int(take(1, np.int64)[0])
        nnz = int(take(1, np.int64)[0])
        out[key + "_indptr"] = take(n + 1, np.int64)
        out[key + "_indices"] = take(nnz, np.int64)
        out[key + "_data"] = take(nnz, np.float64)

    n = int(take(1, np.int64)[0])
    out["leaf"] = take(6 * n, np.float64).reshape(n, 6)
    out["level"] = take(n, np.int64)
    for key in ("Dx", "Dy", "Dz"):
        csr(key)
    out["V"] = take(n, np.float64)
    out["Z"] = take(n, np.float64)
    for key in ("Ws", "Wx", "Wy", "Wz"):
        csr(key)
    out["m0s"] = take(n, np.float64)
    for key in ("Tx", "Ty", "Tz"):
        csr(key)
    out["face_table"] = take(15 * n, np.int32).reshape(n, 3, 5)
    out["reordered_id"] = take(n, np.int64)
    assert off == raw.size
    passes = np.full((len(REFINE_PASSES), max(map(len, REFINE_PASSES)), 3), np.nan)
    for k, r in enumerate(REFINE_PASSES):
        passes[k, :len(r)] = r
    np.savez_compressed(HERE / "ref_operators.npz", n=np.array([6, 5, 4]),
                        limits=np.array([0.0, 600.0, 0.0, 500.0, 0.0, 400.0]), passes=passes,
                        obs=obs, beta=beta, alphas=alphas, **out)


OUTPUT_FILES = ["model.txt", "model.vtk", "model_points.vtk", "dobs.vtk"] + \
    [f"dobs_{c}" for c in ["g_z", "T_zz", "T_xz", "T_yz", "T_xx", "T_xy"]]


def ref_output() -> None:
    """ref_output.npz: the files the reference's own writers make (result2text,
    result2vtk, output_obs_data, output_obs_data_vtk) for the refined mesh of
    ref_operators.npz, seeded models m, m0, m0s and data for six components
    (oracle/_ref/ref_output), with those inputs."""
    exe = REF_BIN / "ref_output"
    obs = np.array([[120.0, 80.0, -20.0], [300.0, 260.0, -35.0], [520.0, 430.0, -10.0],
                    [80.0, 470.0, -25.5], [0.125, 1e-3, -1234.5678]])
    mask = 0x1F2  # gz, Tzz, Txz, Tyz, Txx, Txy
    with tempfile.TemporaryDirectory() as td:
        fin, fout = Path(td) / "in.bin", Path(td) / "out.bin"
        with open(fin, "wb") as fh:
            np.array([6, 5, 4], dtype=np.int64).tofile(fh)
            np.array([0.0, 600.0, 0.0, 500.0, 0.0, 400.0], dtype=np.float64).tofile(fh)
            np.array([len(REFINE_PASSES)], dtype=np.int64).tofile(fh)
            for r in REFINE_PASSES:
                np.array([len(r)], dtype=np.int64).tofile(fh)
                np.array(r, dtype=np.float64).tofile(fh)
            np.array([obs.shape[0]], dtype=np.int64).tofile(fh)
            obs.tofile(fh)
            np.array([mask], dtype=np.uint32).tofile(fh)
            np.array([99], dtype=np.uint64).tofile(fh)
        subprocess.run([str(exe), str(fin), str(fout)], check=True, cwd=td,
                       stdout=subprocess.DEVNULL)
        raw = np.fromfile(fout, dtype=np.uint8)
        files = {f"file:{name}": np.frombuffer((Path(td) / name).read_bytes(), dtype=np.uint8)
                 for name in OUTPUT_FILES}
    off = 0

    def take(cnt, dt):
        nonlocal off
        a = raw[off:off + cnt * np.dtype(dt).itemsize].view(dt)
        off += cnt * np.dtype(dt).itemsize
        return a

    n = int(take(1, np.int64)[0])
    leaf = take(6 * n, np.float64).reshape(n, 6)
    m = take(n, np.float64)
    m0 = take(n, np.float64)
    m0s = take(n, np.float64)
    nd = int(take(1, np.int64)[0])
    dobs = take(nd, np.float64)
    assert off == raw.size
    np.savez_compressed(HERE / "ref_output.npz", leaf=leaf, obs=obs, mask=np.int64(mask), m=m,
                        m0=m0, m0s=m0s, dobs=dobs, **files)


def ref_adapt() -> None:
    """ref_adapt.npz: one AdaptiveInversion::refine_mesh(0.25) of the reference on a
    6 x 5 x 4 mesh first refined at four cells (levels mixed), a seeded model and
    minimum cell sizes of 20 m (level-2 cells still split, with face-balance
    cascades): the leaves and model before, the indicator, the leaves and the
    inherited model after (oracle/_ref/ref_adapt)."""
    exe = REF_BIN / "ref_adapt"
    pts = np.array(REFINE_PASSES[0], dtype=np.float64)
    frac, min_size = 0.25, (20.0, 20.0, 20.0)
    with tempfile.TemporaryDirectory() as td:
        fin, fout = Path(td) / "in.bin", Path(td) / "out.bin"
        with open(fin, "wb") as fh:
            np.array([6, 5, 4], dtype=np.int64).tofile(fh)
            np.array([0.0, 600.0, 0.0, 500.0, 0.0, 400.0], dtype=np.float64).tofile(fh)
            np.array([pts.shape[0]], dtype=np.int64).tofile(fh)
            pts.tofile(fh)
            np.array([frac, *min_size], dtype=np.float64).tofile(fh)
            np.array([2024], dtype=np.uint64).tofile(fh)
        subprocess.run([str(exe), str(fin), str(fout)], check=True, cwd=td,
                       stdout=subprocess.DEVNULL)
        raw = np.fromfile(fout, dtype=np.uint8)
    off = 0

    def take(cnt, dt):
        nonlocal off
        a = raw[off:off + cnt * np.dtype(dt).itemsize].view(dt)
        off += cnt * np.dtype(dt).itemsize
        return a

    n0 = int(take(1, np.int64)[0])
    leaf0 = take(6 * n0, np.float64).reshape(n0, 6)
    m0 = take(n0, np.float64)
    ind = take(n0, np.float64)
    n1 = int(take(1, np.int64)[0])
    leaf1 = take(6 * n1, np.float64).reshape(n1, 6)
    m1 = take(n1, np.float64)
    assert off == raw.size
    np.savez_compressed(HERE / "ref_adapt.npz", pre_points=pts, fraction=frac,
                        min_size=np.array(min_size), leaf0=leaf0, m0=m0, indicator=ind,
                        leaf1=leaf1, m1=m1)


def ref_interp() -> None:
    """ref_interp.npz: the cross-gradient structure model read from a seeded
    gridded file (InversionBase::create_crg_model_from_data, Linterp's
    InterpMultilinear) on a 6 x 5 x 4 mesh first refined at four cells: its
    cell-centre values, its values at probe points (inside, on grid points and
    outside the grid on every side), and one refine_mesh(0.25, interpolator,
    "crg") whose children take interpolated values (oracle/_ref/ref_interp)."""
    exe = REF_BIN / "ref_interp"
    rng = np.random.default_rng(77)
    pts = np.array(REFINE_PASSES[0], dtype=np.float64)
    grids = [np.sort(np.concatenate([[40.0, 560.0], rng.uniform(40.0, 560.0, 9)])),
             np.sort(np.concatenate([[-20.0, 470.0], rng.uniform(-20.0, 470.0, 7)])),
             np.sort(np.concatenate([[30.0, 390.0], rng.uniform(30.0, 390.0, 5)]))]
    vals = rng.uniform(-300.0, 300.0, (grids[0].size, grids[1].size, grids[2].size))
    probes = np.vstack([rng.uniform([-100, -100, -100], [700, 600, 500], (40, 3)),
                        np.stack(np.meshgrid(grids[0][[0, 4, -1]], grids[1][[0, 3, -1]],
                                             grids[2][[0, 2, -1]], indexing="ij"), -1).reshape(-1, 3)])
    with tempfile.TemporaryDirectory() as td:
        fin, fout = Path(td) / "in.bin", Path(td) / "out.bin"
        with open(fin, "wb") as fh:
            np.array([6, 5, 4], dtype=np.int64).tofile(fh)
            np.array([0.0, 600.0, 0.0, 500.0, 0.0, 400.0], dtype=np.float64).tofile(fh)
            np.array([pts.shape[0]], dtype=np.int64).tofile(fh)
            pts.tofile(fh)
            for g in grids:
                np.array([g.size], dtype=np.int64).tofile(fh)
                g.tofile(fh)
            vals.tofile(fh)
            np.array([probes.shape[0]], dtype=np.int64).tofile(fh)
            probes.tofile(fh)
            np.array([0.25], dtype=np.float64).tofile(fh)
            np.array([99], dtype=np.uint64).tofile(fh)
        subprocess.run([str(exe), str(fin), str(fout)], check=True, cwd=td,
                       stdout=subprocess.DEVNULL)
        raw = np.fromfile(fout, dtype=np.uint8)
    off = 0

    def take(cnt, dt):
        nonlocal off
        a = raw[off:off + cnt * np.dtype(dt).itemsize].view(dt)
        off += cnt * np.dtype(dt).itemsize
        return a

    n0 = int(take(1, np.int64)[0])
    m0s0 = take(n0, np.float64)
    probe_vals = take(probes.shape[0], np.float64)
    n1 = int(take(1, np.int64)[0])
    leaf1 = take(6 * n1, np.float64).reshape(n1, 6)
    m0s1 = take(n1, np.float64)
    assert off == raw.size
    np.savez_compressed(HERE / "ref_interp.npz", pre_points=pts, grid_x=grids[0], grid_y=grids[1],
                        grid_z=grids[2], values=vals, probes=probes, probe_values=probe_vals,
                        m0s0=m0s0, leaf1=leaf1, m0s1=m0s1, fraction=0.25)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=None, help="reference tree (default: the oracle recipe's)")
    ap.add_argument("--only", default=None)
    a = ap.parse_args()
    if a.ref:
        ref = Path(a.ref)
    else:
        sys.path.insert(0, str(HERE.parent.parent))
        from oracle import reference_dir

        ref = reference_dir()
        if ref is None:
            sys.exit("reference tree not found: pass --ref or set GRADA_REFERENCE")
    jobs = {"forward_models": lambda: forward_models(ref), "ref_fields": ref_fields,
            "ref_expand": ref_expand, "ref_padded": ref_padded,
            "ref_indicator": ref_indicator, "ref_operators": ref_operators,
            "ref_output": ref_output, "ref_adapt": ref_adapt, "ref_interp": ref_interp}
    try:
        from inversion_cases import adaptive_fixture, inversion_fixtures  # noqa: E402
        jobs["ref_inversion"] = inversion_fixtures
        jobs["ref_adaptive_inversion"] = adaptive_fixture
        for v in ("crg", "pet"):
            jobs[f"ref_adaptive_{v}_inversion"] = (lambda v=v: adaptive_fixture(v))
    except ImportError:
        pass
    for name, fn in jobs.items():
        if a.only and a.only != name:
            continue
        fn()


if __name__ == "__main__":
    sys.path.insert(0, str(HERE))
    sys.path.insert(0, str(REPO))
    main()
