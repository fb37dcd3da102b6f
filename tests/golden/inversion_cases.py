"""Inversion fixtures from the reference compiled into oracle/_ref/ref_inversion.

Each case sets up GaussNewtonInversion on a small regular mesh the way
GraAdaInv::start_inversion does and records: the reference's G, the
host-built operators (Ws, Wx, Wy, Wz and, with the cross-gradient constraint,
T_x, T_y, T_z), Wd, one solve_cg call with non-trivial WL weights, and a full
invert_with_own_CG run (final model, misfit, lambda, and the
lambda_misfit_GN / Iteration_misfit_GN records).  Imported by make_golden.py.
"""
from __future__ import annotations

import os
import struct
import subprocess
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
EXE = REPO / "oracle" / "_ref" / "ref_inversion"


def _read_csr(buf, off):
    n, nnz = struct.unpack_from("<qq", buf, off)
    off += 16
    rp = np.frombuffer(buf, "<i8", n + 1, off).astype(np.int32)
    off += 8 * (n + 1)
    ci = np.frombuffer(buf, "<i8", nnz, off).astype(np.int32)
    off += 8 * nnz
    v = np.frombuffer(buf, "<f8", nnz, off).copy()
    off += 8 * nnz
    return (rp, ci, v), off


def _parse_table(path: Path):
    rows = []
    for line in path.read_text().splitlines()[1:]:
        if line.strip():
            rows.append([float(t) for t in line.split()])
    return np.array(rows)


def run_case(c: dict, solve: dict | None, full: bool, exe: Path = EXE, threads: int = 1):
    """Runs the fixture driver `exe` (the reference's ref_inversion, or the same
    driver linked with the drop-ins) on case c; raises CalledProcessError when
    the driver fails."""
    nx, ny, nz = c["n"]
    nm = nx * ny * nz
    obs = c["obs"]
    mask = c["mask"]
    nf = bin(mask).count("1")
    nd = nf * obs.shape[0]
    out = {}
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        for mode in ([1] if solve else []) + ([2] if full else []):
            b = bytearray()
            b += struct.pack("<qqq", nx, ny, nz)
            b += struct.pack("<6d", *c["xl"], *c["yl"], *c["zl"])
            b += struct.pack("<q", obs.shape[0]) + obs.astype("<f8").tobytes()
            b += struct.pack("<I", mask)
            b += c["dobs"].astype("<f8").tobytes()
            b += np.asarray(c["rel"], "<f8").tobytes() + np.asarray(c["abs"], "<f8").tobytes()
            b += struct.pack("<d", c["beta"])
            b += struct.pack("<5d", *c["alphas"])
            b += struct.pack("<dqd", c["max_lambda"], c["n_lambda"], c["rate"])
            b += struct.pack("<4d", c["target"], c["stag"], c["cg_tol"], c["cg_factor"])
            b += struct.pack("<q", c["gn_iter"])
            b += struct.pack("<5q", *c["lp"])
            b += struct.pack("<d", c["eps2"])
            b += struct.pack("<3d", c["m_min"], c["m_max"], c["m_ini"])
            b += struct.pack("<q", 1 if c.get("m0s") is not None else 0)
            if c.get("m0s") is not None:
                b += c["m0s"].astype("<f8").tobytes()
            b += struct.pack("<q", 1 if c.get("m0") is not None else 0)
            if c.get("m0") is not None:
                b += c["m0"].astype("<f8").tobytes()
            b += struct.pack("<q", mode)
            if mode == 1:
                b += struct.pack("<ddq", solve["lambda"], solve["tol"], solve["maxit"])
                for v in [solve["mk"], solve["mref"], solve["P"]] + list(solve["WL"]):
                    b += np.asarray(v, "<f8").tobytes()
            wd = td / f"run{mode}"
            wd.mkdir()
            (wd / "in.bin").write_bytes(bytes(b))
            # one OpenMP thread: the reference's reductions are then reproducible
            env = dict(os.environ, OMP_NUM_THREADS=str(threads))
            subprocess.run([str(exe), "in.bin", "out.bin"], cwd=wd, check=True,
                           stdout=subprocess.DEVNULL, stderr=subprocess.PIPE, env=env)
            buf = (wd / "out.bin").read_bytes()
            off = 0
            rows, cols = struct.unpack_from("<qq", buf, off)
            off += 16
            G = np.frombuffer(buf, "<f8", rows * cols, off).reshape(cols, rows).T.copy()
            off += 8 * rows * cols
            ops = {}
            for name in ["Ws", "Wx", "Wy", "Wz"]:
                ops[name], off = _read_csr(buf, off)
            (use_crg,) = struct.unpack_from("<q", buf, off)
            off += 8
            if use_crg:
                for name in ["Tx", "Ty", "Tz"]:
                    ops[name], off = _read_csr(buf, off)
                out["S_crg"] = np.frombuffer(buf, "<f8", nm, off).copy()
                off += 8 * nm
            wdiag = np.frombuffer(buf, "<f8", nd, off).copy()
            off += 8 * nd
            out["G"] = G
            out["Wd"] = wdiag
            for name, (rp, ci, v) in ops.items():
                out[f"{name}_rowptr"], out[f"{name}_col"], out[f"{name}_val"] = rp, ci, v
            if mode == 1:
                out["cg_dx"] = np.frombuffer(buf, "<f8", nm, off).copy()
                off += 8 * nm
                out["cg_err"], out["cg_iters"] = struct.unpack_from("<dq", buf, off)
            else:
                out["inv_m"] = np.frombuffer(buf, "<f8", nm, off).copy()
                off += 8 * nm
                out["inv_misfit"], out["inv_lambda"] = struct.unpack_from("<dd", buf, off)
                out["inv_trials"] = _parse_table(wd / "lambda_misfit_GN")
                out["inv_iterations"] = _parse_table(wd / "Iteration_misfit_GN")
    return out


def make_case(name: str, seed: int):
    from graada3d_gb300 import mesh as gm
    from oracle import prism as oracle_prism

    rng = np.random.default_rng(seed)
    if name == "l2":
        n, lp, mask, crg, ref = (8, 8, 4), (2, 2, 2, 2, 2), 0x012, False, False
    elif name == "l1_crg":
        n, lp, mask, crg, ref = (6, 7, 5), (1, 1, 1, 1, 1), 0x072, True, True
    else:  # l0
        n, lp, mask, crg, ref = (7, 6, 4), (0, 0, 0, 0, 2), 0x002, False, False
    nx, ny, nz = n
    xl, yl, zl = (0.0, 1000.0), (0.0, 900.0), (0.0, 500.0)
    prisms = gm.regular_mesh(xl, nx, yl, ny, zl, nz)
    obs = gm.observation_grid(9, 0.0, 1000.0, 8, 0.0, 900.0, -10.0)
    boxes = [[250, 500, 200, 450, 100, 300, 300.0], [600, 850, 500, 800, 150, 400, -200.0]]
    rho = gm.set_boxes(prisms, boxes)
    G = oracle_prism.compute_G(prisms, obs, mask)
    d = G @ rho
    dobs = d + 0.02 * np.abs(d) * rng.standard_normal(d.size)
    nf = bin(mask).count("1")
    c = dict(n=n, xl=xl, yl=yl, zl=zl, obs=obs, mask=mask, dobs=dobs, rel=[0.02] * nf,
             abs=[1e-3 if (mask >> 1) & 1 and k == 0 else 1e-2 for k in range(nf)], beta=1.5,
             alphas=(1.0, 1.0, 1.0, 1.0, 1.0 if crg else 0.0), max_lambda=1e-1, n_lambda=8,
             rate=0.6, target=1.0, stag=0.02, cg_tol=1e-6, cg_factor=30, gn_iter=3, lp=lp,
             eps2=1e-9, m_min=-1000.0, m_max=1000.0, m_ini=0.0)
    if crg:
        xc = 0.5 * (prisms[:, 0] + prisms[:, 1])
        zc = 0.5 * (prisms[:, 4] + prisms[:, 5])
        c["m0s"] = np.sin(xc / 300.0) + 0.5 * np.cos(zc / 200.0)
    if ref:
        c["m0"] = 50.0 * np.sin(xc / 400.0) * np.cos(zc / 250.0)
    nm = nx * ny * nz
    mk = rng.uniform(-300, 300, nm)
    P = (c["m_max"] - mk) * (mk - c["m_min"]) / (c["m_max"] - c["m_min"])
    WL = [rng.uniform(0.5, 2.0, nm) for _ in range(7)]
    solve = {"lambda": 0.05, "tol": 1e-9, "maxit": 40, "mk": mk,
             "mref": c.get("m0", np.zeros(nm)), "P": P, "WL": WL}
    return c, solve


def inversion_fixtures() -> None:
    for name, seed in [("l2", 11), ("l1_crg", 12), ("l0", 13)]:
        c, solve = make_case(name, seed)
        res = run_case(c, solve, full=True)
        out = {
            "n": np.array(c["n"]), "xl": np.array(c["xl"]), "yl": np.array(c["yl"]),
            "zl": np.array(c["zl"]), "obs": c["obs"], "mask": np.array(c["mask"]),
            "dobs": c["dobs"], "rel": np.array(c["rel"]), "abs": np.array(c["abs"]),
            "beta": np.array(c["beta"]), "alphas": np.array(c["alphas"]),
            "max_lambda": np.array(c["max_lambda"]), "n_lambda": np.array(c["n_lambda"]),
            "rate": np.array(c["rate"]), "target": np.array(c["target"]),
            "stag": np.array(c["stag"]), "cg_tol": np.array(c["cg_tol"]),
            "cg_factor": np.array(c["cg_factor"]), "gn_iter": np.array(c["gn_iter"]),
            "lp": np.array(c["lp"]), "eps2": np.array(c["eps2"]),
            "bounds": np.array([c["m_min"], c["m_max"], c["m_ini"]]),
            "solve_lambda": np.array(solve["lambda"]), "solve_tol": np.array(solve["tol"]),
            "solve_maxit": np.array(solve["maxit"]), "solve_mk": solve["mk"],
            "solve_mref": solve["mref"], "solve_P": solve["P"], "solve_WL": np.array(solve["WL"]),
        }
        if c.get("m0s") is not None:
            out["m0s"] = c["m0s"]
        if c.get("m0") is not None:
            out["m0"] = c["m0"]
        for k, v in res.items():
            out[k] = np.asarray(v)
        np.savez_compressed(HERE / f"ref_inversion_{name}.npz", **out)
        print(f"ref_inversion {name}: Nm={np.prod(c['n'])} Nd={res['G'].shape[0]} "
              f"cg_iters={res['cg_iters']} final misfit={res['inv_misfit']:.4f} "
              f"trials={len(res['inv_trials'])}")


def pack_input(c: dict, mode: int, adaptive: dict | None = None) -> bytes:
    """The ref_inversion driver's input for case c (modes 2 and 3)."""
    nx, ny, nz = c["n"]
    obs = c["obs"]
    b = bytearray()
    b += struct.pack("<qqq", nx, ny, nz)
    b += struct.pack("<6d", *c["xl"], *c["yl"], *c["zl"])
    b += struct.pack("<q", obs.shape[0]) + obs.astype("<f8").tobytes()
    b += struct.pack("<I", c["mask"])
    b += c["dobs"].astype("<f8").tobytes()
    b += np.asarray(c["rel"], "<f8").tobytes() + np.asarray(c["abs"], "<f8").tobytes()
    b += struct.pack("<d", c["beta"])
    b += struct.pack("<5d", *c["alphas"])
    b += struct.pack("<dqd", c["max_lambda"], c["n_lambda"], c["rate"])
    b += struct.pack("<4d", c["target"], c["stag"], c["cg_tol"], c["cg_factor"])
    b += struct.pack("<q", c["gn_iter"])
    b += struct.pack("<5q", *c["lp"])
    b += struct.pack("<d", c["eps2"])
    b += struct.pack("<3d", c["m_min"], c["m_max"], c["m_ini"])
    b += struct.pack("<q", 1 if c.get("m0s") is not None else 0)
    if c.get("m0s") is not None:
        b += c["m0s"].astype("<f8").tobytes()
    b += struct.pack("<q", 1 if c.get("m0") is not None else 0)
    if c.get("m0") is not None:
        b += c["m0"].astype("<f8").tobytes()
    b += struct.pack("<q", mode)
    if mode == 3:
        b += struct.pack("<qqd3d", adaptive["max_refinements"], adaptive["interval"],
                         adaptive["fraction"], *adaptive["min_size"])
    return bytes(b)


def make_adaptive_case(seed: int = 21):
    """A small L2 inversion (8 x 8 x 4 cells, gz + Tzz at 9 x 8 points) with two
    refinements of 10 % of the cells, one per Gauss-Newton iteration, down to a
    quarter of the base cell size."""
    c, _ = make_case("l2", seed)
    c["gn_iter"] = 5
    c["stag"] = 0.005
    adaptive = {"max_refinements": 2, "interval": 1, "fraction": 0.1,
                "min_size": (1000.0 / 8 / 4, 900.0 / 8 / 4, 500.0 / 4 / 4)}
    return c, adaptive


def make_adaptive_crg_case(seed: int = 23, crg: bool = True, ref: bool = False):
    """The adaptive case with gridded constraint models on the 8 x 8 x 4 cells:
    the structure model of the l1_crg case (crg: the cross-gradient constraint,
    a_crg 1) and / or its reference model (ref), each read by the reference from
    a grid at the cell centres.  The reference then refines with refine_mesh(a,
    interpolator, "crg"), (a, interpolator, "pet") or (a, interp_m0s, interp_m0).
    L2 on every term."""
    from graada3d_gb300 import mesh as gm

    c, adaptive = make_adaptive_case(seed)
    prisms = gm.regular_mesh(c["xl"], c["n"][0], c["yl"], c["n"][1], c["zl"], c["n"][2])
    xc = 0.5 * (prisms[:, 0] + prisms[:, 1])
    zc = 0.5 * (prisms[:, 4] + prisms[:, 5])
    if crg:
        c["m0s"] = np.sin(xc / 300.0) + 0.5 * np.cos(zc / 200.0)
        c["alphas"] = (1.0, 1.0, 1.0, 1.0, 1.0)
    if ref:
        c["m0"] = 50.0 * np.sin(xc / 400.0) * np.cos(zc / 250.0)
    return c, adaptive


def run_adaptive(c: dict, adaptive: dict, exe: Path = EXE):
    """The reference's adaptive inversion on case c: final leaves, model, misfit,
    lambda, the lambda/misfit and iteration records, and the number of cells
    split at each refinement (the reference prints it)."""
    import re

    with tempfile.TemporaryDirectory() as td:
        wd = Path(td)
        (wd / "in.bin").write_bytes(pack_input(c, 3, adaptive))
        env = dict(os.environ, OMP_NUM_THREADS="1")
        res = subprocess.run([str(exe), "in.bin", "out.bin"], cwd=wd, check=True,
                             capture_output=True, text=True, env=env)
        buf = (wd / "out.bin").read_bytes()
        # skip the set-up dump (G, operators, Wd) that precedes the mode's output
        rows, cols = struct.unpack_from("<qq", buf, 0)
        off = 16 + 8 * rows * cols
        for _ in range(4):
            _, off = _read_csr(buf, off)
        (use_crg,) = struct.unpack_from("<q", buf, off)
        off += 8
        if use_crg:
            for _ in range(3):
                _, off = _read_csr(buf, off)
            off += 8 * cols
        off += 8 * rows
        (n,) = struct.unpack_from("<q", buf, off)
        off += 8
        leaves = np.frombuffer(buf, "<f8", 6 * n, off).reshape(n, 6).copy()
        off += 48 * n
        m = np.frombuffer(buf, "<f8", n, off).copy()
        off += 8 * n
        misfit, lam = struct.unpack_from("<dd", buf, off)
        splits = [int(v) for v in re.findall(r"(\d+) elements are refined", res.stdout)]
        return {"leaves": leaves, "m": m, "misfit": misfit, "lambda": lam, "splits": np.array(splits),
                "trials": _parse_table(wd / "lambda_misfit_GN"),
                "iterations": _parse_table(wd / "Iteration_misfit_GN")}


def adaptive_fixture(variant: str = "") -> None:
    """variant "": the plain adaptive inversion; "crg", "pet", "crg_pet": with the
    structure model, the reference model, or both."""
    if variant:
        c, ad = make_adaptive_crg_case(crg="crg" in variant, ref="pet" in variant)
    else:
        c, ad = make_adaptive_case()
    res = run_adaptive(c, ad)
    out = {"n": np.array(c["n"]), "xl": np.array(c["xl"]), "yl": np.array(c["yl"]),
           "zl": np.array(c["zl"]), "obs": c["obs"], "mask": np.array(c["mask"]),
           "dobs": c["dobs"], "rel": np.array(c["rel"]), "abs": np.array(c["abs"]),
           "beta": np.array(c["beta"]), "alphas": np.array(c["alphas"]),
           "max_lambda": np.array(c["max_lambda"]), "n_lambda": np.array(c["n_lambda"]),
           "rate": np.array(c["rate"]), "target": np.array(c["target"]), "stag": np.array(c["stag"]),
           "cg_tol": np.array(c["cg_tol"]), "cg_factor": np.array(c["cg_factor"]),
           "gn_iter": np.array(c["gn_iter"]), "lp": np.array(c["lp"]), "eps2": np.array(c["eps2"]),
           "bounds": np.array([c["m_min"], c["m_max"], c["m_ini"]]),
           "max_refinements": np.array(ad["max_refinements"]), "interval": np.array(ad["interval"]),
           "fraction": np.array(ad["fraction"]), "min_size": np.array(ad["min_size"])}
    for k in ("m0s", "m0"):
        if c.get(k) is not None:
            out[k] = c[k]
    for k, v in res.items():
        out["ref_" + k] = np.asarray(v)
    name = f"ref_adaptive_{variant}_inversion" if variant else "ref_adaptive_inversion"
    np.savez_compressed(HERE / f"{name}.npz", **out)
    print(f"{name}: leaves {res['leaves'].shape[0]} splits {res['splits']} "
          f"misfit {res['misfit']:.4f} trials {len(res['trials'])}")
