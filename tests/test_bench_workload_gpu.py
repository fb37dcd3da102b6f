"""Parity at the benchmarked size: the nine-component FP64 G of the 64 x 64 x 32
mesh (131,072 cells over 20 x 20 x 8 km) for observation points of the
101 x 101 grid at 50 m height, over all cells, against the oracle
(Fwd::compute_G, src/Forward_modelling/Fwd.cpp:47-78, restated in C).

The points include the 25 that lie on cell-face planes (x, y in {0, 5, 10, 15,
20} km), the coincident geometry the reference's face integrals branch on, and
the full-size tile plan (eight 32-level runs per tile) is the one the benchmark
uses.  Tolerance: 1e-10 of max|component| over the checked rows.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_benchmark_workload_rows_match_oracle():
    import bench
    from graada3d_gb300 import Fwd
    from oracle import prism as oracle_prism

    prisms, obs, _ = bench.build_problem()
    idx = bench.parity_points()
    sub = obs[idx]
    f = Fwd(prisms, sub, bench.MASK)
    f.compute_G("fp64")
    G = f.get_G()
    oracle_prism.build()
    want = oracle_prism.compute_G(prisms, sub, bench.MASK)
    n = idx.size
    for k, name in enumerate(bench.COMPONENTS):
        blk = slice(k * n, (k + 1) * n)
        err = np.abs(G[blk] - want[blk]).max() / np.abs(want[blk]).max()
        assert err <= bench.PARITY_TOL, f"{name}: {err:.3e}"
    # the row gather returns the same rows as the whole-matrix copy
    rows = np.array([0, 5, n + 3, 8 * n + n - 1], dtype=np.int64)
    assert np.array_equal(f.get_G_rows(rows), G[rows])
    f.ctx.close()
