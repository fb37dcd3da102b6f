"""Padded meshes (Mesh::generate_regular_mesh_with_padding, Mesh.cpp:516-795):
cells of very different sizes, the largest far outside the area of interest.
G and the field sum of the reference's own padded mesh (tests/golden/
ref_padded.npz, from the compiled reference) against the GPU, stored and
matrix-free."""
import numpy as np
import pytest

from graada3d_gb300 import Fwd

pytestmark = pytest.mark.gpu

TOL = 1e-10  # relative to each component's largest |value|


def _per_component(a, ref, n):
    for k in range(ref.shape[0] // n):
        blk = slice(k * n, (k + 1) * n)
        scale = np.abs(ref[blk]).max()
        assert np.abs(a[blk] - ref[blk]).max() <= TOL * scale, k


@pytest.mark.parametrize("storage", ["fp64", "matrix_free"])
def test_padded_mesh_matches_reference(gpu_ctx, golden, storage):
    r = golden("ref_padded.npz")
    f = Fwd(r["leaf"], r["obs"], int(r["mask"]), ctx=gpu_ctx)
    n = r["obs"].shape[0]
    f.compute_G(storage)
    d = f.G_vec_mul(r["rho"])
    _per_component(d, r["d"], n)
    if storage == "fp64":
        G = f.get_G()[: f.Nd]
        _per_component(G[:, r["cols"]], r["G_cols"], n)
