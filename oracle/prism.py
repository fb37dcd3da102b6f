"""ctypes binding of ``liboracle.so`` (prism_oracle.c) -- TEST INFRASTRUCTURE ONLY.

The C file restates the reference algorithm (face integrals of
src/Forward_modelling/Integral.cpp driven by GravFormula.cpp); see its header.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
_lib = None

_dp = ctypes.POINTER(ctypes.c_double)


def build(force: bool = False) -> Path:
    """Compile liboracle.so with gcc (OpenMP, no FP contraction)."""
    src = HERE / "prism_oracle.c"
    if force or not LIB.exists() or LIB.stat().st_mtime < src.stat().st_mtime:
        tmp = LIB.with_suffix(".so.tmp")
        subprocess.run(
            ["gcc", "-O2", "-fPIC", "-fopenmp", "-ffp-contract=off", "-shared", "-o", str(tmp),
             str(src), "-lm"],
            check=True,
        )
        os.replace(tmp, LIB)
    return LIB


def load():
    global _lib
    if _lib is None:
        build()
        lib = ctypes.CDLL(str(LIB))
        lib.oracle_prism_field.argtypes = [_dp, _dp, ctypes.c_double, ctypes.c_uint32, _dp]
        lib.oracle_compute_G.argtypes = [_dp, ctypes.c_int64, _dp, ctypes.c_int64, ctypes.c_uint32,
                                         _dp, ctypes.c_int64]
        lib.oracle_forward_field.argtypes = [_dp, _dp, ctypes.c_int64, _dp, ctypes.c_int64,
                                             ctypes.c_uint32, _dp]
        lib.oracle_num_threads.restype = ctypes.c_int
        _lib = lib
    return _lib


def _p(a):
    return a.ctypes.data_as(_dp)


def n_fields(mask: int) -> int:
    return bin(int(mask) & 0x3FF).count("1")


def prism_field(obs, prism, rho: float = 1.0, mask: int = 0x3FF) -> np.ndarray:
    """GravFormula::field_caused_by_single_prism: 10-vector in field-bit order."""
    lib = load()
    o = np.ascontiguousarray(obs, dtype=np.float64)
    p = np.ascontiguousarray(prism, dtype=np.float64)
    out = np.zeros(10)
    lib.oracle_prism_field(_p(o), _p(p), float(rho), int(mask), _p(out))
    return out


def compute_G(prisms, obs, mask: int) -> np.ndarray:
    """Fwd::compute_G: (Nd, Nm) float64, column-major."""
    lib = load()
    pr = np.ascontiguousarray(prisms, dtype=np.float64).reshape(-1, 6)
    ob = np.ascontiguousarray(obs, dtype=np.float64).reshape(-1, 3)
    nd = n_fields(mask) * ob.shape[0]
    G = np.zeros((nd, pr.shape[0]), dtype=np.float64, order="F")
    lib.oracle_compute_G(_p(pr), pr.shape[0], _p(ob), ob.shape[0], int(mask), _p(G), nd)
    return G


def forward_field(prisms, rho, obs, mask: int) -> np.ndarray:
    """compute.cpp field sum: (N_obs, n_fields)."""
    lib = load()
    pr = np.ascontiguousarray(prisms, dtype=np.float64).reshape(-1, 6)
    r = np.ascontiguousarray(rho, dtype=np.float64)
    ob = np.ascontiguousarray(obs, dtype=np.float64).reshape(-1, 3)
    out = np.zeros((ob.shape[0], n_fields(mask)))
    lib.oracle_forward_field(_p(pr), _p(r), pr.shape[0], _p(ob), ob.shape[0], int(mask), _p(out))
    return out


def num_threads() -> int:
    return int(load().oracle_num_threads())
