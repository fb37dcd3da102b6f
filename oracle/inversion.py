"""NumPy restatement of the reference inversion -- TEST INFRASTRUCTURE ONLY.

Follows src/Inversion/GaussNewtonInversion.cpp:
  solve_cg            :1417-1698  (CGLS on the stacked system, with the
                                   reference's operator choices)
  invert_with_own_CG  :657-1103   (lambda search, IRLS, bound transform;
                                   no mesh refinement)
Operators are scipy.sparse CSR matrices built on the host; G is a dense
(Nd, Nm) array.  Used to check the GPU path at sizes the compiled reference
is not run on, and pinned itself against the reference's outputs
(tests/golden/ref_inversion_*.npz).
"""
from __future__ import annotations

import math

import numpy as np
import scipy.sparse as sp


def solve_cg(tol, maxit, lam, mk, mref, Wd, dobs, P, G, Ws, Wx, Wy, Wz, T=None, a_crg=1.0,
             S_crg=None, WL=None):
    """One solve_cg call.  WL: dict with keys s,x,y,z,tx,ty,tz of diagonals
    (None = ones).  T: (Tx, Ty, Tz) from set_Tmatrix or None.  Returns
    (dx, err, iterations)."""
    nm = mk.size
    nd = dobs.size
    ones = np.ones(nm)
    W = {k: (ones if WL is None or WL.get(k) is None else WL[k]) for k in
         ["s", "x", "y", "z", "tx", "ty", "tz"]}
    sl = math.sqrt(lam)
    crg = T is not None
    if crg:
        sc = a_crg * (np.ones(nm) if S_crg is None else S_crg)
        Tx = sp.diags(sc) @ T[0]
        Ty = sp.diags(sc) @ T[1]
        Tz = sp.diags(sc) @ T[2]
    # b (:1458-1472)
    b0 = Wd * (dobs - G @ mk)
    bs = [-sl * W["s"] * (Ws @ (mk - mref)), -sl * W["z"] * (Wz @ mk), -sl * W["x"] * (Wx @ mk),
          -sl * W["y"] * (Wy @ mk)]
    if crg:
        bs += [-W["tz"] * (Tz @ mk), -W["tx"] * (Tx @ mk), -W["ty"] * (Ty @ mk)]
    s0 = -b0
    ss = [-v for v in bs]
    ops = [Ws, Wz, Wx, Wy] + ([Tz, Tx, Ty] if crg else [])
    c = [sl, sl, sl, sl] + ([1.0, 1.0, 1.0] if crg else [])
    adj_wl = [W["s"], W["z"], W["x"], W["y"]] + ([W["tz"], W["tx"], W["ty"]] if crg else [])
    adj_wl0 = list(adj_wl)
    if crg:
        adj_wl0[6] = W["y"]  # :1508
    fwd_wl = [ones, W["z"], W["x"], W["y"]] + ([W["z"], W["x"], W["y"]] if crg else [])

    def adjoint(d_seg, segs, wls):
        r = P * (G.T @ (Wd * d_seg))
        for A, ci, wl, sv in zip(ops, c, wls, segs):
            r = r + ci * P * (A.T @ (wl * sv))
        return r

    r = adjoint(s0, ss, adj_wl0)
    ATb = adjoint(b0, bs, adj_wl)
    ATb2 = float(ATb @ ATb)
    dx = np.zeros(nm)
    p = np.zeros(nm)
    beta = 0.0
    err = 0.0
    r2 = float(r @ r)
    it = maxit
    for i in range(maxit):
        p = -r + beta * p
        Pp = P * p
        t0 = Wd * (G @ Pp)
        ts = [ci * wl * (A @ Pp) for A, ci, wl in zip(ops, c, fwd_wl)]
        t2 = float(t0 @ t0) + sum(float(v @ v) for v in ts)
        alpha = r2 / t2
        s0 = s0 + alpha * t0
        ss = [sv + alpha * tv for sv, tv in zip(ss, ts)]
        dx = dx + alpha * p
        r = adjoint(s0, ss, adj_wl)
        rlast2 = r2
        r2 = float(r @ r)
        beta = r2 / rlast2
        err = r2 / ATb2
        if err < tol:
            it = i + 1
            break
    return dx, err, it


def bound_update(m, dx, mmin, mmax, mt_prev):
    """:877-911, sequential in cell order like the reference loop."""
    mt = mt_prev.copy()
    with np.errstate(over="ignore", invalid="ignore"):
        for i in range(m.size):
            try:
                temp = math.exp(dx[i])
            except OverflowError:
                temp = math.inf
            temp2 = mmin[i] * (mmax[i] - m[i]) + mmax[i] * (m[i] - mmin[i]) * temp
            temp3 = (mmax[i] - m[i]) + (m[i] - mmin[i]) * temp
            if math.isinf(temp) or math.isinf(temp2):
                mt[i] = (mmax[i] - 1e-6 + mt[i]) / 2.0
                mt[i] = 0.5 * (mt[i] + (mt[i + 1] if i == 0 else mt[i - 1]))
            elif abs(temp3) < 1e-10:
                mt[i] = (mmin[i] + 1e-6 + mt[i]) / 2.0
                mt[i] = 0.5 * (mt[i] + (mt[i + 1] if i == 0 else mt[i - 1]))
            else:
                mt[i] = temp2 / temp3
    return mt


def invert(G, dobs, Wd, Ws, Wx, Wy, Wz, prm, m_ini, mmin, mmax, m0=None, T=None, a_crg=1.0):
    """invert_with_own_CG on a fixed mesh.  prm keys: max_lambda, n_lambda,
    rate, target, stag, cg_tol, cg_factor, gn_iter, lp (5), eps2,
    start_from_reference.  Returns (m, misfit, lambda, trials, iterations)."""
    nm = m_ini.size
    nd = dobs.size
    m0 = np.zeros(nm) if m0 is None else m0
    m = (m0 if prm.get("start_from_reference") else m_ini).astype(float).copy()
    for i in range(nm):
        if prm.get("start_from_reference"):
            if m[i] > mmax[i] or abs(m[i] - mmax[i]) < 1e-7:
                m[i] = mmax[i] - 0.01
            if m[i] < mmin[i] or abs(m[i] - mmin[i]) < 1e-7:
                m[i] = mmin[i] + 0.01
        else:
            if m[i] > mmax[i] or abs(m[i] - mmax[i]) < 1e-7:
                m[i] = 0.5 * (mmax[i] + mmin[i])
            if m[i] < mmin[i] or abs(m[i] - mmin[i]) < 1e-7:
                m[i] = 0.5 * (mmax[i] + mmin[i])

    def misfit_of(v):
        e = Wd * (G @ v - dobs)
        return math.sqrt(float(e @ e) / nd)

    misfit = misfit_of(m)
    lam = prm["max_lambda"]
    lam_opt = lam
    misfit_opt = misfit
    m_opt = m.copy()
    rate = prm["rate"]
    lp = prm["lp"]
    expo = [-(2 - p) / 4.0 for p in lp]
    WL = {k: np.ones(nm) for k in ["s", "x", "y", "z", "tx", "ty", "tz"]}
    trials, iters = [], []
    crg = T is not None
    for i in range(prm["gn_iter"]):
        m_trial = m.copy()
        last1, last2 = 10 * misfit, 100 * misfit
        misfit_last_it = misfit
        if i == 0 or prm["n_lambda"] == 1 or abs(rate - 1) < 1e-6:
            lam = prm["max_lambda"]
        else:
            lam = lam_opt * (1 / rate) ** min(3, prm["n_lambda"] - 2)
            if lam < min(prm["max_lambda"] * rate ** 20, 1.0e-5):
                lam = 1.0
        cg_maxit = int(prm["cg_factor"] * nm) if prm["cg_factor"] < 1 else int(prm["cg_factor"])
        P = (mmax - m) * (m - mmin) / (mmax - mmin)
        j = 0
        while j < prm["n_lambda"]:
            dx, err, it = solve_cg(prm["cg_tol"], cg_maxit, lam, m, m0, Wd, dobs, P, G, Ws, Wx, Wy,
                                   Wz, T, a_crg, None, WL)
            m_trial = bound_update(m, dx, mmin, mmax, m_trial)
            last2, last1 = last1, misfit
            misfit = misfit_of(m_trial)
            trials.append((i + 1, lam, misfit, it, err))
            if j == 0 or misfit < misfit_opt:
                misfit_opt = misfit
                m_opt = m_trial.copy()
                if i > 0:
                    m = m_opt.copy()
                lam_opt = lam
            if (abs(misfit - last1) / min(misfit, last1) < prm["stag"]
                    and abs(last1 - last2) / min(last1, last2) < prm["stag"] and j > 1):
                break
            if misfit > last1 and last1 > last2 and j > 1:
                break
            lam = lam * rate
            for key, A, k in [("s", Ws, 0), ("x", Wx, 1), ("y", Wy, 2), ("z", Wz, 3)]:
                if lp[k] != 2:
                    v = A @ (m_opt - m0) if key == "s" else A @ m_opt
                    WL[key] = (v * v + prm["eps2"]) ** expo[k]
            if lp[4] != 2 and crg:
                for key, A in [("tx", T[0]), ("ty", T[1]), ("tz", T[2])]:
                    v = A @ m_opt
                    WL[key] = (v * v + prm["eps2"]) ** expo[4]
            if misfit < prm["target"]:
                break
            j += 1
        else:
            j = prm["n_lambda"]
        m = m_opt.copy()
        misfit = misfit_opt
        iters.append((i + 1, prm["n_lambda"] if j == prm["n_lambda"] else j + 1, misfit))
        if misfit < prm["target"] or i == prm["gn_iter"] - 1:
            break
        if abs(misfit - misfit_last_it) / min(misfit, misfit_last_it) < prm["stag"]:
            break
    return m, misfit, lam, trials, iters
