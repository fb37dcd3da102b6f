"""Loading helpers for the ref_inversion_*.npz fixtures (shared by the CPU and
GPU inversion tests)."""
import numpy as np
import scipy.sparse as sp

from conftest import GOLDEN

CASES = ["l2", "l1_crg", "l0"]


def load(name):
    return np.load(GOLDEN / f"ref_inversion_{name}.npz", allow_pickle=False)


def csr(f, key):
    rp, ci, v = f[f"{key}_rowptr"], f[f"{key}_col"], f[f"{key}_val"]
    n = rp.size - 1
    return sp.csr_matrix((v, ci, rp), shape=(n, n))


def has_crg(f):
    return "Tx_rowptr" in f.files


def prm(f):
    return {
        "max_lambda": float(f["max_lambda"]), "n_lambda": int(f["n_lambda"]),
        "rate": float(f["rate"]), "target": float(f["target"]), "stag": float(f["stag"]),
        "cg_tol": float(f["cg_tol"]), "cg_factor": float(f["cg_factor"]),
        "gn_iter": int(f["gn_iter"]), "lp": [int(v) for v in f["lp"]], "eps2": float(f["eps2"]),
        "start_from_reference": "m0" in f.files,
    }


def wl_dict(f):
    WL = f["solve_WL"]
    return dict(zip(["s", "x", "y", "z", "tx", "ty", "tz"], WL))


def prisms(f):
    from graada3d_gb300 import mesh

    nx, ny, nz = (int(v) for v in f["n"])
    return mesh.regular_mesh(tuple(f["xl"]), nx, tuple(f["yl"]), ny, tuple(f["zl"]), nz)
