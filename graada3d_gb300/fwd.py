"""Python view of the reference's ``Fwd`` interface over the C ABI.

Mirrors ``Fwd`` (src/Forward_modelling/Fwd.h:14-94): bind a mesh (prisms in
leaf order) and observation points with a field flag, ``compute_G``,
``G_vec_mul``, ``GT_vec_mul``, ``get_G``.  All arithmetic happens in
``libgrada_gpu.so`` on the GPU; this module only moves NumPy arrays across
the ABI.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import GradaError

# Field bits of GS::ComputationOptions (gs.h:46-57).
FIELD_BITS = {
    "V": 0x001, "gz": 0x002, "gx": 0x004, "gy": 0x008, "Tzz": 0x010,
    "Txz": 0x020, "Tyz": 0x040, "Txx": 0x080, "Txy": 0x100, "Tyy": 0x200,
}
FIELD_ORDER = ["V", "gz", "gx", "gy", "Tzz", "Txz", "Tyz", "Txx", "Txy", "Tyy"]

G_FP64, G_FP32, G_BF16_ROWSCALE, G_FP16_ROWSCALE, G_MATRIX_FREE, G_WAVELET = 0, 1, 2, 3, 4, 5
STORAGE = {"fp64": G_FP64, "fp32": G_FP32, "bf16": G_BF16_ROWSCALE, "fp16": G_FP16_ROWSCALE,
           "matrix_free": G_MATRIX_FREE}


def field_mask(names) -> int:
    m = 0
    for n in names:
        m |= FIELD_BITS[n]
    return m


def mask_fields(mask: int) -> list[str]:
    return [n for b, n in enumerate(FIELD_ORDER) if mask & (1 << b)]


def split_cells(cells) -> np.ndarray:
    """Children of each cell as Mesh::refinement makes them (Mesh.cpp:1562-1600):
    split at the centre, x outermost, then y, z innermost.  (n, 8, 6)."""
    c = np.asarray(cells, dtype=np.float64).reshape(-1, 6)
    out = np.empty((c.shape[0], 8, 6))
    mids = [0.5 * (c[:, 1] + c[:, 0]), 0.5 * (c[:, 3] + c[:, 2]), 0.5 * (c[:, 5] + c[:, 4])]
    lo = [c[:, 0], c[:, 2], c[:, 4]]
    hi = [c[:, 1], c[:, 3], c[:, 5]]
    idx = 0
    for i in range(2):
        for j in range(2):
            for k in range(2):
                for a, s in enumerate((i, j, k)):
                    out[:, idx, 2 * a] = lo[a] if s == 0 else mids[a]
                    out[:, idx, 2 * a + 1] = mids[a] if s == 0 else hi[a]
                idx += 1
    return out


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class Context:
    """One library context (one CUDA stream, owned device buffers)."""

    def __init__(self, device: int = 0):
        self.lib = _lib.load()
        h = ctypes.c_void_p()
        st = self.lib.grada_ctx_create(int(device), ctypes.byref(h))
        if st != 0:
            raise GradaError(st, f"grada_ctx_create(device={device}) failed")
        self.handle = h

    def check(self, status: int) -> None:
        if status != 0:
            msg = self.lib.grada_last_error(self.handle)
            raise GradaError(status, msg.decode() if msg else "")

    @property
    def stream(self) -> int:
        return int(self.lib.grada_ctx_stream(self.handle) or 0)

    def sync(self) -> None:
        self.check(self.lib.grada_sync(self.handle))

    def device_bytes(self) -> int:
        return int(self.lib.grada_ctx_device_bytes(self.handle))

    def fp64_peak(self) -> float:
        out = ctypes.c_double()
        self.check(self.lib.grada_measure_fp64_peak(self.handle, ctypes.byref(out)))
        return out.value

    def close(self) -> None:
        if getattr(self, "handle", None):
            self.lib.grada_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class Fwd:
    """GPU-backed counterpart of the reference ``Fwd`` class."""

    def __init__(self, prisms, obs, field_flag, ctx: Context | None = None):
        self.ctx = ctx or Context()
        self.set_geometry(prisms, obs, field_flag)

    # Fwd::set_mesh / set_observation / set_field_flag
    def set_geometry(self, prisms, obs, field_flag) -> None:
        if not isinstance(field_flag, (int, np.integer)):
            field_flag = field_mask(field_flag)
        self.prisms = np.ascontiguousarray(prisms, dtype=np.float64).reshape(-1, 6)
        self.obs = np.ascontiguousarray(obs, dtype=np.float64).reshape(-1, 3)
        self.field_flag = int(field_flag)
        self.ctx.check(
            self.ctx.lib.grada_set_geometry(
                self.ctx.handle, _ptr(self.prisms), self.prisms.shape[0], _ptr(self.obs),
                self.obs.shape[0], self.field_flag,
            )
        )
        self._dims()

    def _dims(self) -> None:
        nc, no, nd, ld = (ctypes.c_int64() for _ in range(4))
        nf = ctypes.c_int()
        self.ctx.check(
            self.ctx.lib.grada_get_dims(
                self.ctx.handle, ctypes.byref(nc), ctypes.byref(no), ctypes.byref(nf),
                ctypes.byref(nd), ctypes.byref(ld),
            )
        )
        self.Nm, self.N_obs, self.n_fields, self.Nd, self.ld = nc.value, no.value, nf.value, nd.value, ld.value

    def get_n_fields(self) -> int:
        return self.n_fields

    def compute_G(self, storage: str | int = "fp64", keep_fp64: bool = False) -> None:
        """Fwd::compute_G in the given storage.  keep_fp64: with a reduced
        storage also keep the FP64 G, from which the reduced entries are
        rounded and which mixed-precision inversions then predict with
        (grada_keep_fp64_G)."""
        s = STORAGE[storage] if isinstance(storage, str) else int(storage)
        self.ctx.check(self.ctx.lib.grada_keep_fp64_G(self.ctx.handle, int(bool(keep_fp64))))
        self.ctx.check(self.ctx.lib.grada_compute_G(self.ctx.handle, s))

    def compute_G_wavelet(self, order, relative_threshold: float, values: str = "fp64") -> None:
        """Fwd::compute_G_wavelet: rows of G along ``order`` (Mesh::get_reordered_id,
        e.g. ``mesh.Octree.wavelet_order()``) Daubechies-4 transformed and
        thresholded; the products then use the compressed rows.  values: "fp64"
        (the reference's) or "fp32" (kept coefficients rounded to FP32)."""
        o = np.ascontiguousarray(order, dtype=np.int64)
        if o.shape != (self.Nm,):
            raise ValueError(f"expected an order of {self.Nm} cells")
        self.ctx.check(self.ctx.lib.grada_compute_G_wavelet_ex(
            self.ctx.handle, o.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
            float(relative_threshold), STORAGE[values]))

    def get_wavelet_G(self):
        """(n_dy, rowptr, cols, vals) of the compressed rows."""
        n_dy, nnz = ctypes.c_int64(), ctypes.c_int64()
        self.ctx.check(self.ctx.lib.grada_get_wavelet_G(self.ctx.handle, ctypes.byref(n_dy),
                                                        ctypes.byref(nnz), None, None, None))
        rp = np.empty(self.Nd + 1, dtype=np.int64)
        ci = np.empty(max(nnz.value, 1), dtype=np.int32)
        v = np.empty(max(nnz.value, 1))
        self.ctx.check(self.ctx.lib.grada_get_wavelet_G(
            self.ctx.handle, ctypes.byref(n_dy), ctypes.byref(nnz),
            rp.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
            ci.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), _ptr(v)))
        return n_dy.value, rp, ci[:nnz.value].astype(np.int64), v[:nnz.value]

    def get_G(self) -> np.ndarray:
        """G as an (Nd, Nm) float64 array in column-major (Fortran) order."""
        out = np.empty((self.ld, self.Nm), dtype=np.float64, order="F")
        self.ctx.check(self.ctx.lib.grada_get_G(self.ctx.handle, _ptr(out), self.ld))
        return out[: self.Nd, :]

    def get_G_rows(self, rows) -> np.ndarray:
        """Rows of the stored G, (len(rows), Nm) float64 (grada_get_G_rows)."""
        idx = np.ascontiguousarray(rows, dtype=np.int64)
        out = np.empty((idx.size, self.Nm), dtype=np.float64)
        self.ctx.check(self.ctx.lib.grada_get_G_rows(
            self.ctx.handle, idx.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), idx.size, _ptr(out)))
        return out

    def G_column_norms(self) -> np.ndarray:
        """||G(:, j)||_2 for every cell j (grada_G_column_norms), the quantity
        InversionBase::set_depth_weighting(beta, 1) takes from G's columns."""
        out = np.empty(self.Nm, dtype=np.float64)
        self.ctx.check(self.ctx.lib.grada_G_column_norms(self.ctx.handle, _ptr(out)))
        return out

    def G_vec_mul(self, vec) -> np.ndarray:
        x = np.ascontiguousarray(vec, dtype=np.float64)
        if x.shape != (self.Nm,):
            raise ValueError(f"expected a vector of {self.Nm} cells")
        y = np.empty(self.Nd, dtype=np.float64)
        self.ctx.check(self.ctx.lib.grada_G_vec_mul(self.ctx.handle, _ptr(x), _ptr(y)))
        return y

    def GT_vec_mul(self, vec) -> np.ndarray:
        y = np.ascontiguousarray(vec, dtype=np.float64)
        if y.shape != (self.Nd,):
            raise ValueError(f"expected a vector of {self.Nd} data")
        x = np.empty(self.Nm, dtype=np.float64)
        self.ctx.check(self.ctx.lib.grada_GT_vec_mul(self.ctx.handle, _ptr(y), _ptr(x)))
        return x

    def G_mat_mul(self, X) -> np.ndarray:
        """Y = G X for a block of right-hand sides X (Nm x n); n x G_vec_mul."""
        X = np.asfortranarray(np.asarray(X, dtype=np.float64).reshape(self.Nm, -1))
        Y = np.empty((self.Nd, X.shape[1]), dtype=np.float64, order="F")
        self.ctx.check(self.ctx.lib.grada_G_mat_mul(self.ctx.handle, X.shape[1], _ptr(X), _ptr(Y)))
        return Y

    def GT_mat_mul(self, Y) -> np.ndarray:
        """X = G^T Y for a block Y (Nd x n); n x GT_vec_mul."""
        Y = np.asfortranarray(np.asarray(Y, dtype=np.float64).reshape(self.Nd, -1))
        X = np.empty((self.Nm, Y.shape[1]), dtype=np.float64, order="F")
        self.ctx.check(self.ctx.lib.grada_GT_mat_mul(self.ctx.handle, Y.shape[1], _ptr(Y), _ptr(X)))
        return X

    def expand_G(self, parent_index, children=None) -> None:
        """AdaptiveInversion::expand_G: replace each listed cell (ascending
        indices) by its 8 children (x outer, y, z inner; split at the centre when
        children is None) in G and in the cell list."""
        idx = np.ascontiguousarray(parent_index, dtype=np.int64)
        kids = None
        if children is not None:
            kids = np.ascontiguousarray(children, dtype=np.float64).reshape(idx.size, 8, 6)
        self.ctx.check(self.ctx.lib.grada_expand_G(
            self.ctx.handle, idx.size, idx.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
            None if kids is None else _ptr(kids)))
        if kids is None:
            kids = split_cells(self.prisms[idx])
        parts, prev = [], 0
        for k, j in enumerate(idx):
            parts.append(self.prisms[prev:j])
            parts.append(kids[k].reshape(8, 6))
            prev = j + 1
        parts.append(self.prisms[prev:])
        self.prisms = np.ascontiguousarray(np.vstack(parts))
        self._dims()

    def forward_field(self, rho) -> np.ndarray:
        """compute.cpp field sum: (N_obs, n_fields) array, components in bit order."""
        r = np.ascontiguousarray(rho, dtype=np.float64)
        if r.shape != (self.Nm,):
            raise ValueError(f"expected a density per cell ({self.Nm})")
        out = np.empty((self.N_obs, self.n_fields), dtype=np.float64)
        self.ctx.check(self.ctx.lib.grada_forward_field(self.ctx.handle, _ptr(r), _ptr(out)))
        return out
