"""grada_G_vec_mul_noalloc: the product for callers that cannot allocate
device memory (inside another library's stream capture, under their own
device-memory budget, or where an allocation's device-wide synchronisation is
not acceptable).  It must give what the context-based product gives, call
after call, while its scratch lives in a fixed array inside the library.

Kept in a file that pytest collects last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_G_vec_mul_noalloc_matches_context_product():
    import torch

    from graada3d_gb300 import Fwd, _lib, mesh

    lib = _lib.load()
    prisms = mesh.regular_mesh((0.0, 3000.0), 12, (0.0, 2500.0), 10, (0.0, 1500.0), 6)
    obs = mesh.observation_grid(23, -200.0, 3200.0, 19, -200.0, 2700.0, -15.0)
    f = Fwd(prisms, obs, 0x3FE)
    f.compute_G("fp64")
    G = f.get_G()
    nd, nm, ld = f.Nd, f.Nm, f.ld
    padded = np.zeros((ld, nm), order="F")
    padded[:nd] = G
    dev = torch.device("cuda", 0)
    d_G = torch.from_numpy(np.ascontiguousarray(padded.ravel(order="F"))).to(dev)
    d_y = torch.empty(nd, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    tol = 1e-12 * np.abs(G).sum(axis=1).max()
    rng = np.random.default_rng(8)
    for call in range(2):  # two calls in a row share the scratch array
        x = rng.uniform(-500.0, 500.0, nm)
        want = f.G_vec_mul(x)  # the existing entry point
        d_x = torch.from_numpy(x).to(dev)
        d_y.fill_(np.nan)
        st = lib.grada_G_vec_mul_noalloc(ctypes.c_void_p(d_G.data_ptr()), nd, nm, ld,
                                         ctypes.c_void_p(d_x.data_ptr()),
                                         ctypes.c_void_p(d_y.data_ptr()),
                                         ctypes.c_void_p(stream.cuda_stream))
        assert st == 0, f"call {call}: status {st}"
        torch.cuda.synchronize(dev)
        got = d_y.cpu().numpy()
        assert np.abs(got - want).max() <= tol, f"call {call}"
    # a G taller than the fixed scratch is refused before anything runs
    st = lib.grada_G_vec_mul_noalloc(ctypes.c_void_p(d_G.data_ptr()), (1 << 20) + 2, nm,
                                     (1 << 20) + 2, ctypes.c_void_p(d_y.data_ptr()),
                                     ctypes.c_void_p(d_y.data_ptr()), None)
    assert st == -7
    f.ctx.close()
