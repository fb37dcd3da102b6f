"""One mesh refinement of the adaptive inversion, the reference's
AdaptiveInversion::refine_mesh (src/Inversion/AdaptiveInversion.cpp:637-735)
without the constraint-model re-interpolation:

1. the refinement indicator of every leaf for the current model, on the
   device (grada_refinement_indicator), over the (neighbour, area) list built
   from the cells (``regularization.indicator_pairs``);
2. the cells to split (``refinement_marks``, on the host);
3. the split, face balance included (``mesh.Octree.refine``, on the host);
4. G expanded in place on the device (grada_expand_G), the model inherited by
   the children, and the regularisation operators rebuilt on the device
   (grada_build_operators).
"""
from __future__ import annotations

import numpy as np

from . import mesh
from . import regularization as reg


def refinement_marks(indicator, prisms, fraction: float, min_size) -> np.ndarray:
    """The leaves refine_mesh splits (AdaptiveInversion.cpp:639-683): none when
    fraction < 0 or fraction x Nm < 1; else those whose indicator exceeds the
    int(fraction x Nm)-th largest (0-based) and whose sizes are all above the
    minimum (a size within 1e-7 of it counts as at the minimum).  Ascending.
    fraction x Nm must stay below Nm (fraction < 1): the reference reads past
    the end of its sorted indicator there, so this raises ValueError instead."""
    ind = np.asarray(indicator, dtype=np.float64)
    nm = ind.size
    if fraction < 0 or abs(fraction * nm) < 1:
        return np.zeros(0, dtype=np.int64)
    if int(fraction * nm) >= nm:
        raise ValueError(f"refinement fraction {fraction} selects index {int(fraction * nm)} "
                         f"of {nm} indicator values; it must satisfy int(fraction * Nm) < Nm")
    tol = np.sort(ind)[::-1][int(fraction * nm)]
    pr = np.asarray(prisms, dtype=np.float64)
    size = np.abs(pr[:, 1::2] - pr[:, 0::2])
    mn = np.asarray(min_size, dtype=np.float64)
    small = ((size < mn) | (np.abs(size - mn) < 1e-7)).any(1)
    return np.nonzero((ind > tol) & ~small)[0].astype(np.int64)


def carry_over(values, parent, split, new_cells, interpolator=None) -> np.ndarray:
    """A per-cell vector on the refined cells: children take their parent's
    value (Cell's constructor copies the parent's parameters, Mesh.cpp:1575-1590)
    or, with an interpolator, its value at their centre -- what the
    constrained refine_mesh variants do for the structure (cross-gradient) and
    reference models (AdaptiveInversion.cpp:333-375); other cells keep theirs."""
    out = np.asarray(values, dtype=np.float64)[parent].copy()
    if interpolator is not None:
        child = np.isin(parent, split)
        out[child] = interpolator(mesh.cell_centres(np.asarray(new_cells)[child]))
    return out


def refine_mesh(inv, octree, m, fraction: float, min_size, beta: float,
                alphas=(1.0, 1.0, 1.0, 1.0), extra=()):
    """One refinement of `inv` (a GaussNewtonInversion whose cells are
    ``octree.leaves()``) for the model m.  Splits the marked cells, expands G
    and rebuilds Ws/Wx/Wy/Wz on the device.  Returns the model on the new
    cells and the vectors of `extra` on them: each entry a per-cell vector
    (children take the parent's value) or a (vector, interpolator) pair
    (children take the interpolator's value at their centre, as the
    constrained refine_mesh variants do).  Nothing changes when no cell is
    marked."""
    prisms = octree.leaves()
    indicator = inv.indicator_calculator(m, *reg.indicator_pairs(prisms))
    marks = refinement_marks(indicator, prisms, fraction, min_size)
    if marks.size == 0:
        return (np.asarray(m), *(v[0] if isinstance(v, tuple) else v for v in extra))
    n_old = prisms.shape[0]
    split = octree.refine(marks)
    parent = octree.parent_leaf(split, n_old)
    inv.expand_G(split)
    if not np.array_equal(inv.prisms.view(np.uint64), octree.leaves().view(np.uint64)):
        raise RuntimeError("expanded cells differ from the refined mesh")
    inv.build_operators(reg.face_table(inv.prisms), beta, 0, alphas)
    out = [np.asarray(m)[parent]]
    for v in extra:
        vec, interp = v if isinstance(v, tuple) else (v, None)
        out.append(carry_over(vec, parent, split, inv.prisms, interp))
    return tuple(out)


def invert_adaptive(inv, octree, prm: dict, m_ini, m_min, m_max, m0=None, *,
                    max_refinements: int, interval: int, fraction: float, min_size, beta: float,
                    alphas=(1.0, 1.0, 1.0, 1.0), fp64_refinement: bool = False,
                    m0s=None, m0s_interpolator=None, m0_interpolator=None):
    """The adaptive inversion (invert_with_own_CG with its refinement branch,
    GaussNewtonInversion.cpp:1098-1294) through grada_invert_adaptive: the
    Gauss-Newton loop, lambda search and CG run in the library; at each
    refinement the library calls back here, and refine_mesh splits the marked
    cells of `octree` (on the host), expands G and rebuilds Ws/Wx/Wy/Wz (on the
    device), and the model, bounds and reference model follow the children.
    With the cross-gradient constraint (m0s: the structure model on the
    current cells, T_x, T_y, T_z set from it and the constraint enabled),
    children take m0s_interpolator's value at their centre (refine_mesh(a,
    interpolator, "crg"), AdaptiveInversion.cpp:206-386; children take their
    parent's value without an interpolator) and T_x, T_y, T_z are rebuilt from
    the new structure model (set_Tmatrix, GaussNewtonInversion.cpp:1266-1268).
    With m0_interpolator the reference model's children likewise take its value
    at their centre (refine_mesh(a, interpolator, "pet") and, with both models,
    refine_mesh(a, interp_m0s, interp_m0), AdaptiveInversion.cpp:206-386, 388-534).
    `inv` must hold G for octree.leaves() with its data and operators set.
    Returns (model on the final cells, report)."""
    import ctypes

    from . import _lib
    from .inversion import _params, _ptr

    lib = inv.ctx.lib
    nm = inv.Nm
    state = {"mmin": np.asarray(m_min, dtype=np.float64).copy(),
             "mmax": np.asarray(m_max, dtype=np.float64).copy(),
             "m0": np.zeros(nm) if m0 is None else np.asarray(m0, dtype=np.float64).copy(),
             "m0s": None if m0s is None else np.asarray(m0s, dtype=np.float64).copy()}
    errors = []

    def on_refine(user, ctx_handle, m_ptr, n):
        try:
            m = np.ctypeslib.as_array(m_ptr, shape=(n,)).copy()
            extra = [state["mmin"], state["mmax"],
                     state["m0"] if m0_interpolator is None else (state["m0"], m0_interpolator)]
            if state["m0s"] is not None:
                extra.append((state["m0s"], m0s_interpolator))
            new_m, mmin, mmax, m0v, *rest = refine_mesh(inv, octree, m, fraction, min_size, beta,
                                                        alphas, extra=tuple(extra))
            state.update(mmin=np.ascontiguousarray(mmin), mmax=np.ascontiguousarray(mmax),
                         m0=np.ascontiguousarray(m0v))
            if state["m0s"] is not None and rest[0].shape[0] != state["m0s"].shape[0]:
                state["m0s"] = np.ascontiguousarray(rest[0])
                ops = reg.mesh_operators(inv.prisms, inv.obs, beta, *alphas)
                inv.set_operators(reg.cross_gradient_operators(None, inv.prisms, state["m0s"], ops))
            new_m = np.ascontiguousarray(new_m)
            return lib.grada_set_inversion_model(inv.ctx.handle, _ptr(new_m), _ptr(state["mmin"]),
                                                 _ptr(state["mmax"]), _ptr(state["m0"]))
        except BaseException as e:  # reported after the call returns
            errors.append(e)
            return -1

    callback = _lib.REFINE_FN(on_refine)
    ap = _lib.AdaptiveParams(int(max_refinements), int(interval),
                             ctypes.cast(callback, ctypes.c_void_p), None)
    p = _params(prm, fp64_refinement)
    vecs = [np.ascontiguousarray(v, dtype=np.float64) for v in (m_ini, m_min, m_max)]
    m0a = None if m0 is None else np.ascontiguousarray(m0, dtype=np.float64)
    rep = _lib.InvertReport()
    rc = lib.grada_invert_adaptive(inv.ctx.handle, ctypes.byref(p), ctypes.byref(ap),
                                   _ptr(vecs[0]), _ptr(vecs[1]), _ptr(vecs[2]),
                                   None if m0a is None else _ptr(m0a), ctypes.byref(rep))
    if errors:
        raise errors[0]
    inv.ctx.check(rc)
    out = np.empty(inv.Nm)
    inv.ctx.check(lib.grada_get_model(inv.ctx.handle, _ptr(out)))
    inv.m = out
    return out, {f: getattr(rep, f) for f, _ in _lib.InvertReport._fields_}
