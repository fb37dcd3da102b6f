"""Python view of the reference's ``GaussNewtonInversion`` over the C ABI.

Mirrors the members the hot path uses (src/Inversion/GaussNewtonInversion.h,
InversionBase.h): ``set_dobs`` (data and Wd), the host-built regularisation
operators, ``solve_cg`` and ``invert`` (invert_with_own_CG on a fixed mesh),
plus the records the reference writes to lambda_misfit_GN and
Iteration_misfit_GN.  The forward part (``compute_G``, products) is inherited
from :class:`graada3d_gb300.fwd.Fwd`, as GaussNewtonInversion inherits Fwd.
"""
from __future__ import annotations

import ctypes

import numpy as np
import scipy.sparse as sp

from . import output
from ._lib import InvertParams, InvertReport
from .fwd import Fwd, _ptr

OP_SLOTS = {"Ws": 0, "Wx": 1, "Wy": 2, "Wz": 3, "Tx": 4, "Ty": 5, "Tz": 6}
WL_ORDER = ["s", "x", "y", "z", "tx", "ty", "tz"]


def _iptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))


class GaussNewtonInversion(Fwd):
    """GPU-backed counterpart of the reference GaussNewtonInversion."""

    def set_dobs(self, dobs, wd) -> None:
        """Observed data (Nd) and the diagonal of Wd (InversionBase::set_dobs)."""
        self.dobs = np.ascontiguousarray(dobs, dtype=np.float64)
        self.wd = np.ascontiguousarray(wd, dtype=np.float64)
        if self.dobs.shape != (self.Nd,) or self.wd.shape != (self.Nd,):
            raise ValueError(f"expected {self.Nd} data and weights")
        self.ctx.check(self.ctx.lib.grada_set_data(self.ctx.handle, _ptr(self.dobs), _ptr(self.wd)))

    def set_operator(self, name: str, A) -> None:
        A = sp.csr_matrix(A)
        A.sort_indices()
        rp = np.ascontiguousarray(A.indptr, dtype=np.int32)
        ci = np.ascontiguousarray(A.indices, dtype=np.int32)
        v = np.ascontiguousarray(A.data, dtype=np.float64)
        self.ctx.check(self.ctx.lib.grada_set_operator(self.ctx.handle, OP_SLOTS[name], A.shape[0],
                                                       v.size, _iptr(rp), _iptr(ci), _ptr(v)))

    def set_operators(self, ops: dict) -> None:
        for name in ["Ws", "Wx", "Wy", "Wz", "Tx", "Ty", "Tz"]:
            if name in ops and ops[name] is not None:
                self.set_operator(name, ops[name])

    def build_operators(self, faces, beta: float = 2.0, depth_flag: int = 0,
                        alphas=(1.0, 1.0, 1.0, 1.0)) -> None:
        """Ws, Wx, Wy, Wz built on the device from the face table
        (``regularization.face_table``); alphas = (a_s, a_z, a_x, a_y)."""
        f = np.ascontiguousarray(faces, dtype=np.int32)
        if f.shape != (self.Nm, 3, 5):
            raise ValueError(f"face table of shape ({self.Nm}, 3, 5) expected")
        a = np.ascontiguousarray(alphas, dtype=np.float64)
        if a.shape != (4,):
            raise ValueError("four weights expected")
        self.ctx.check(self.ctx.lib.grada_build_operators(
            self.ctx.handle, f.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), float(beta),
            int(depth_flag), _ptr(a)))

    def get_operator(self, name: str) -> sp.csr_matrix:
        """An operator as the device holds it."""
        nnz = ctypes.c_int64()
        self.ctx.check(self.ctx.lib.grada_get_operator(self.ctx.handle, OP_SLOTS[name],
                                                       ctypes.byref(nnz), None, None, None))
        rp = np.empty(self.Nm + 1, dtype=np.int32)
        ci = np.empty(max(nnz.value, 1), dtype=np.int32)
        v = np.empty(max(nnz.value, 1))
        self.ctx.check(self.ctx.lib.grada_get_operator(
            self.ctx.handle, OP_SLOTS[name], ctypes.byref(nnz), _iptr(rp), _iptr(ci), _ptr(v)))
        return sp.csr_matrix((v[:nnz.value], ci[:nnz.value], rp), shape=(self.Nm, self.Nm))

    def set_cross_gradient(self, enabled: bool, a_crg: float = 1.0, S_crg=None) -> None:
        S = None
        if S_crg is not None:
            self._s_crg = np.ascontiguousarray(S_crg, dtype=np.float64)
            S = _ptr(self._s_crg)
        self.ctx.check(self.ctx.lib.grada_set_cross_gradient(self.ctx.handle, int(bool(enabled)),
                                                             float(a_crg), S))

    def solve_cg(self, tol, maxit, lam, mk, mref, P, WL=None):
        """GaussNewtonInversion::solve_cg; WL dict keyed s,x,y,z,tx,ty,tz (None = I).
        Returns (dx, err, iterations)."""
        vec = [np.ascontiguousarray(v, dtype=np.float64) for v in (mk, mref, P)]
        wl_arrays = []
        arr = (ctypes.POINTER(ctypes.c_double) * 7)()
        for k, key in enumerate(WL_ORDER):
            w = None if WL is None else WL.get(key)
            if w is None:
                arr[k] = ctypes.POINTER(ctypes.c_double)()
            else:
                w = np.ascontiguousarray(w, dtype=np.float64)
                wl_arrays.append(w)
                arr[k] = _ptr(w)
        dx = np.empty(self.Nm)
        err = ctypes.c_double()
        it = ctypes.c_int()
        self.ctx.check(self.ctx.lib.grada_solve_cg(
            self.ctx.handle, float(tol), int(maxit), float(lam), _ptr(vec[0]), _ptr(vec[1]),
            _ptr(vec[2]), arr, _ptr(dx), ctypes.byref(err), ctypes.byref(it)))
        return dx, err.value, it.value

    def cg_phase_times(self):
        """Mean ns per CG iteration of the persistent loop's four phases (G p,
        finish and regulariser rows, step, G^T s and adjoint) over the persistent
        solves since the last invert, and their iteration count."""
        out = np.zeros(4)
        n = ctypes.c_int64()
        self.ctx.check(self.ctx.lib.grada_cg_phase_times(self.ctx.handle, _ptr(out), ctypes.byref(n)))
        return out, n.value

    def cg_loop_time(self):
        """(loop seconds, graph-building seconds, CG iterations) of the CG loops
        since the last invert: the loops alone, without the set-up, predictions
        and lambda control around them (grada_cg_loop_time)."""
        out = np.zeros(2)
        n = ctypes.c_int64()
        self.ctx.check(self.ctx.lib.grada_cg_loop_time(self.ctx.handle, _ptr(out), ctypes.byref(n)))
        return float(out[0]), float(out[1]), n.value

    def invert(self, prm: dict, m_ini, m_min, m_max, m0=None, fp64_refinement: bool = False):
        """invert_with_own_CG on the current G.  prm keys as oracle.inversion.invert
        (max_lambda, n_lambda, rate, target, stag, cg_tol, cg_factor, gn_iter,
        lp[5], eps2, start_from_reference).  Returns (m, report)."""
        p = _params(prm, fp64_refinement)
        vecs = [np.ascontiguousarray(v, dtype=np.float64) for v in (m_ini, m_min, m_max)]
        m0a = None if m0 is None else np.ascontiguousarray(m0, dtype=np.float64)
        out = np.empty(self.Nm)
        rep = InvertReport()
        self.ctx.check(self.ctx.lib.grada_invert(
            self.ctx.handle, ctypes.byref(p), _ptr(vecs[0]), _ptr(vecs[1]), _ptr(vecs[2]),
            None if m0a is None else _ptr(m0a), _ptr(out), ctypes.byref(rep)))
        self.m = out
        self.m0 = m0a
        return out, {f: getattr(rep, f) for f, _ in InvertReport._fields_}

    # -- result writers (GraAda3D.cpp:792-806); the files are the reference's
    #    byte for byte (graada3d_gb300.output)

    def _model(self, m):
        v = getattr(self, "m", None) if m is None else m
        if v is None:
            raise ValueError("no model: run invert() or pass m")
        return np.asarray(v, dtype=np.float64)

    def get_predicted_field(self, m=None) -> np.ndarray:
        """G m on the device (InversionBase::get_predicted_field, InversionBase.cpp:696-708)."""
        return self.G_vec_mul(self._model(m))

    def result2text(self, filename: str, m=None) -> None:
        """<filename>.txt (InversionBase::result2text, InversionBase.cpp:883-887)."""
        output.write_model_txt(filename + ".txt", self.prisms, self._model(m))

    def result2vtk(self, filename: str, m=None, m0=None, m0s=None) -> None:
        """<filename>.vtk and <filename>_points.vtk with the model, the reference
        model and the structure model (zero when not given, as the reference
        initialises them; InversionBase::result2vtk, InversionBase.cpp:888-896)."""
        zero = np.zeros(self.Nm)
        m0 = getattr(self, "m0", None) if m0 is None else m0
        params = [("model", self._model(m)), ("m0", zero if m0 is None else m0),
                  ("m0s", zero if m0s is None else m0s)]
        output.write_model_vtk(filename + ".vtk", self.prisms, params)
        output.write_model_vtk_points(filename + "_points.vtk", self.prisms, params)

    def output_obs_data(self, out_name: str) -> None:
        output.write_data(out_name, self.obs, self.dobs, self.field_flag)

    def output_predicted_data(self, out_name: str, m=None) -> None:
        output.write_data(out_name, self.obs, self.get_predicted_field(m), self.field_flag)

    def output_obs_data_vtk(self, filename: str) -> None:
        output.write_data_vtk(filename, self.obs, self.dobs, self.field_flag)

    def output_predicted_data_vtk(self, filename: str, m=None) -> None:
        output.write_data_vtk(filename, self.obs, self.get_predicted_field(m), self.field_flag)

    def solve_cg_block(self, tol, maxit, lambdas, mk, mref, P, WL=None):
        """Several solve_cg systems at once (grada_solve_cg_block): column c has
        lambdas[c], mk[:, c], P[:, c] and WL[key][:, c] (Nm x n arrays; a WL entry
        may also be None).  Returns (dx (Nm x n), err (n), iterations (n))."""
        lam = np.ascontiguousarray(lambdas, dtype=np.float64)
        n = lam.size
        blk = lambda a: np.asfortranarray(np.broadcast_to(
            np.asarray(a, dtype=np.float64).reshape(self.Nm, -1), (self.Nm, n)))
        mk_b, P_b = blk(mk), blk(P)
        mref_v = np.ascontiguousarray(mref, dtype=np.float64)
        arr = (ctypes.POINTER(ctypes.c_double) * 7)()
        keep = []
        for k, key in enumerate(WL_ORDER):
            w = None if WL is None else WL.get(key)
            if w is None:
                arr[k] = ctypes.POINTER(ctypes.c_double)()
            else:
                wb = blk(w)
                keep.append(wb)
                arr[k] = _ptr(wb)
        dx = np.empty((self.Nm, n), order="F")
        err = np.empty(n)
        it = (ctypes.c_int * n)()
        self.ctx.check(self.ctx.lib.grada_solve_cg_block(
            self.ctx.handle, float(tol), int(maxit), n, _ptr(lam), _ptr(mk_b), _ptr(mref_v),
            _ptr(P_b), arr, _ptr(dx), _ptr(err), it))
        return dx, err, np.array(it[:], dtype=int)

    def lambda_sweep(self, prm: dict, lambdas, m_ini, m_min, m_max, m0=None,
                     fp64_refinement: bool = False):
        """grada_lambda_sweep: for each lambda the fixed-lambda Gauss-Newton run
        (invert with n_lambda = 1, max_lambda = lambda), all lambdas advancing
        together with block CG solves.  Returns (models (Nm x n), [report])."""
        lam = np.ascontiguousarray(lambdas, dtype=np.float64)
        n = lam.size
        p = _params(dict(prm, max_lambda=float(lam[0]), n_lambda=1), fp64_refinement)
        vecs = [np.ascontiguousarray(v, dtype=np.float64) for v in (m_ini, m_min, m_max)]
        m0a = None if m0 is None else np.ascontiguousarray(m0, dtype=np.float64)
        out = np.empty((self.Nm, n), order="F")
        reps = (InvertReport * n)()
        self.ctx.check(self.ctx.lib.grada_lambda_sweep(
            self.ctx.handle, ctypes.byref(p), n, _ptr(lam), _ptr(vecs[0]), _ptr(vecs[1]),
            _ptr(vecs[2]), None if m0a is None else _ptr(m0a), _ptr(out), reps))
        return out, [{f: getattr(reps[k], f) for f, _ in InvertReport._fields_} for k in range(n)]

    def sweep_trials(self, column: int) -> np.ndarray:
        """(n, 5) trial records of one column of the last lambda_sweep."""
        n = ctypes.c_int64()
        self.ctx.check(self.ctx.lib.grada_get_sweep_trials(self.ctx.handle, int(column), None, 0,
                                                           ctypes.byref(n)))
        out = np.empty((n.value, 5))
        self.ctx.check(self.ctx.lib.grada_get_sweep_trials(self.ctx.handle, int(column),
                                                           _ptr(out), n.value, ctypes.byref(n)))
        return out

    def indicator_calculator(self, m, rowptr, neighbour, area) -> np.ndarray:
        """AdaptiveInversion::indicator_calculator on the device: per cell the sum
        of (m[neighbour] - m[cell])^2 * area over its (neighbour, area) list (CSR,
        in the reference's face order)."""
        mv = np.ascontiguousarray(m, dtype=np.float64)
        rp = np.ascontiguousarray(rowptr, dtype=np.int64)
        nb = np.ascontiguousarray(neighbour, dtype=np.int64)
        ar = np.ascontiguousarray(area, dtype=np.float64)
        out = np.empty(self.Nm)
        p64 = ctypes.POINTER(ctypes.c_int64)
        self.ctx.check(self.ctx.lib.grada_refinement_indicator(
            self.ctx.handle, _ptr(mv), rp.ctypes.data_as(p64), nb.ctypes.data_as(p64), _ptr(ar),
            _ptr(out)))
        return out

    def trials(self) -> np.ndarray:
        """(n, 5): gn_iteration, lambda, misfit, cg_iterations, cg_error."""
        n = ctypes.c_int64()
        self.ctx.check(self.ctx.lib.grada_get_trials(self.ctx.handle, None, 0, ctypes.byref(n)))
        out = np.empty((n.value, 5))
        self.ctx.check(self.ctx.lib.grada_get_trials(self.ctx.handle, _ptr(out), n.value,
                                                     ctypes.byref(n)))
        return out

    def iterations(self) -> np.ndarray:
        """(n, 3): gn_iteration, n_trials, misfit."""
        n = ctypes.c_int64()
        self.ctx.check(self.ctx.lib.grada_get_iterations(self.ctx.handle, None, 0, ctypes.byref(n)))
        out = np.empty((n.value, 3))
        self.ctx.check(self.ctx.lib.grada_get_iterations(self.ctx.handle, _ptr(out), n.value,
                                                         ctypes.byref(n)))
        return out


def _params(prm: dict, fp64_refinement: bool) -> InvertParams:
    p = InvertParams()
    p.max_lambda = prm["max_lambda"]
    p.n_lambda = prm["n_lambda"]
    p.lambda_decreasing_rate = prm["rate"]
    p.target_misfit = prm["target"]
    p.stag_tol = prm["stag"]
    p.cg_tol = prm["cg_tol"]
    p.cg_iteration_factor = prm["cg_factor"]
    p.gn_iterations = prm["gn_iter"]
    p.lp_s, p.lp_x, p.lp_y, p.lp_z, p.lp_t = (int(v) for v in prm["lp"])
    p.epsilon2 = prm["eps2"]
    p.start_from_reference = int(bool(prm.get("start_from_reference", False)))
    p.fp64_refinement = int(bool(fp64_refinement))
    return p


def compute_G_batch(invs, storage="fp64", max_threads: int = 0, keep_fp64: bool = False) -> None:
    """grada_compute_G_batch over the contexts of several Fwd/GaussNewtonInversion objects
    (keep_fp64: as Fwd.compute_G)."""
    from .fwd import STORAGE

    lib = invs[0].ctx.lib
    n = len(invs)
    for i in invs:
        i.ctx.check(lib.grada_keep_fp64_G(i.ctx.handle, int(bool(keep_fp64))))
    ctxs = (ctypes.c_void_p * n)(*[i.ctx.handle.value for i in invs])
    st = (ctypes.c_int * n)()
    s = STORAGE[storage] if isinstance(storage, str) else int(storage)
    rc = lib.grada_compute_G_batch(n, ctxs, s, int(max_threads), st)
    if rc != 0:
        bad = [k for k in range(n) if st[k] != 0]
        invs[bad[0]].ctx.check(st[bad[0]])


def invert_batch(invs, prms, m_inis, m_mins, m_maxs, m0s=None, fp64_refinement=False,
                 max_threads: int = 0):
    """grada_invert_batch: the inversions of several GaussNewtonInversion objects run
    concurrently.  Returns [(m, report)] in input order."""
    lib = invs[0].ctx.lib
    n = len(invs)
    dp = ctypes.POINTER(ctypes.c_double)
    ctxs = (ctypes.c_void_p * n)(*[i.ctx.handle.value for i in invs])
    params = (InvertParams * n)(*[_params(p, fp64_refinement) for p in prms])
    keep = []

    def arr(vs):
        out = (dp * n)()
        for k, v in enumerate(vs):
            if v is None:
                out[k] = dp()
            else:
                a = np.ascontiguousarray(v, dtype=np.float64)
                keep.append(a)
                out[k] = _ptr(a)
        return out

    outs = [np.empty(i.Nm) for i in invs]
    reports = (InvertReport * n)()
    st = (ctypes.c_int * n)()
    rc = lib.grada_invert_batch(n, ctxs, params, arr(m_inis), arr(m_mins), arr(m_maxs),
                                arr(m0s if m0s is not None else [None] * n), arr(outs), reports,
                                int(max_threads), st)
    if rc != 0:
        bad = [k for k in range(n) if st[k] != 0]
        invs[bad[0]].ctx.check(st[bad[0]])
    return [(outs[k], {f: getattr(reports[k], f) for f, _ in InvertReport._fields_})
            for k in range(n)]


def invert_batch_persistent(invs, prms, m_inis, m_mins, m_maxs, m0s=None, fp64_refinement=False,
                            team_ctas: int = 0):
    """grada_invert_batch_persistent: the inversions of several GaussNewtonInversion
    objects (one device, the same G storage) in one persistent cooperative launch,
    a team of CTAs per problem.  team_ctas: > 0 teams of that size taking problems
    from a device queue, -1 one team per problem sized by its G, 0 the tuning
    table's choice.  Returns ([(m, report)] in input order, (teams, CTAs per team
    or -1))."""
    lib = invs[0].ctx.lib
    n = len(invs)
    dp = ctypes.POINTER(ctypes.c_double)
    ctxs = (ctypes.c_void_p * n)(*[i.ctx.handle.value for i in invs])
    params = (InvertParams * n)(*[_params(p, fp64_refinement) for p in prms])
    keep = []

    def arr(vs):
        out = (dp * n)()
        for k, v in enumerate(vs):
            if v is None:
                out[k] = dp()
            else:
                a = np.ascontiguousarray(v, dtype=np.float64)
                keep.append(a)
                out[k] = _ptr(a)
        return out

    outs = [np.empty(i.Nm) for i in invs]
    reports = (InvertReport * n)()
    st = (ctypes.c_int * n)()
    rc = lib.grada_invert_batch_persistent(n, ctxs, params, arr(m_inis), arr(m_mins), arr(m_maxs),
                                           arr(m0s if m0s is not None else [None] * n), arr(outs),
                                           reports, int(team_ctas), st)
    invs[0].ctx.check(rc)
    for k in range(n):
        invs[k].m = outs[k]
    teams, per = ctypes.c_int(), ctypes.c_int()
    invs[0].ctx.check(lib.grada_batch_shape(invs[0].ctx.handle, ctypes.byref(teams), ctypes.byref(per)))
    return ([(outs[k], {f: getattr(reports[k], f) for f, _ in InvertReport._fields_})
             for k in range(n)], (teams.value, per.value))


def load_batch_tuning(path) -> None:
    """Loads a team-size table for invert_batch_persistent (grada_load_batch_tuning)."""
    from . import _lib

    lib = _lib.load()
    rc = lib.grada_load_batch_tuning(str(path).encode())
    if rc != 0:
        raise _lib.GradaError(rc, f"cannot load the batch tuning table {path}")
