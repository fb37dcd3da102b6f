"""Autotuner of the batched persistent inversion's team size.

grada_invert_batch_persistent splits the GPU's resident CTAs into teams; a team
takes one problem at a time from a device queue.  Small teams keep many
problems in flight but give each one little bandwidth; large teams finish a
problem sooner but leave CTAs idle on small problems and lengthen the tail.
A third layout gives each problem its own team, sized in proportion to its G, and
starts them all at once (-1).  The best choice depends on the problem sizes, so it is
measured: for each class
of synthetic batches (uniform meshes, gz + Tzz, the batch's spread of cell and
point counts) the batch is run with every candidate team size under shortened
inversion settings (the team-size effect is per CG iteration), and the fastest
wins.  The table row is "<largest G of the class, entries> <CTAs per team>";
the library reads tuning/batch_teams.tsv beside itself on first use.  A row's team size
may be -1, the proportional layout.

    python -m graada3d_gb300.autotune [--out PATH] [--storage fp32+fp64|fp64]

Needs a GPU.
"""
from __future__ import annotations

import argparse
import json
import time
from pathlib import Path

import numpy as np

from . import Context, mesh
from . import regularization as reg
from .inversion import GaussNewtonInversion, invert_batch_persistent

TABLE = Path(__file__).resolve().parent / "tuning" / "batch_teams.tsv"

# (name, problems, cells range, points range): the middle class is the
# 64-problem batch of uneven size (4k-60k cells, 400-5,000 points)
CLASSES = [
    ("small", 64, (4000, 15000), (400, 1500)),
    ("uneven-64", 64, (4000, 60000), (400, 5000)),
    ("large", 8, (60000, 100000), (3000, 6000)),
]
# team sizes tried; -1 is one team per problem sized by its G, all problems at once
CANDIDATES = (-1, 2, 4, 8, 16, 32, 64)
SHORT = dict(max_lambda=1e-1, n_lambda=3, rate=0.6, target=1e-9, stag=0.0, cg_tol=1e-30,
             cg_factor=20, gn_iter=1, lp=[2, 2, 2, 2, 2], eps2=1e-9)


def synthetic_batch(n: int, cells: tuple, points: tuple, seed: int, storage: str, device: int = 0):
    """n seeded problems: uniform meshes nx = ny, nz = nx/2 over 10 x 10 x 5 km,
    square point grids 100 m above, gz + Tzz of two boxes with 2 % noise, L2
    operators.  Returns (inversions, per-problem (m_ini, m_min, m_max))."""
    invs, args = [], []
    for k in range(n):
        rng = np.random.default_rng(seed + k)
        nc = int(rng.integers(cells[0], cells[1] + 1))
        nx = max(4, int(round((2 * nc) ** (1 / 3))))
        nz = max(2, nx // 2)
        no = max(2, int(round(int(rng.integers(points[0], points[1] + 1)) ** 0.5)))
        L = 10000.0
        prisms = mesh.regular_mesh((0.0, L), nx, (0.0, L), nx, (0.0, L / 2), nz)
        obs = mesh.observation_grid(no, 0.0, L, no, 0.0, L, -100.0)
        boxes = []
        for v in (300.0, -200.0):
            s_ = rng.uniform(1000, 3000, 3)
            x0, y0 = rng.uniform(0, L - s_[0]), rng.uniform(0, L - s_[1])
            z0 = rng.uniform(0, L / 2 - s_[2])
            boxes.append([x0, x0 + s_[0], y0, y0 + s_[1], z0, z0 + s_[2], v])
        rho = mesh.set_boxes(prisms, boxes)
        inv = GaussNewtonInversion(prisms, obs, 0x012, ctx=Context(device))
        inv.compute_G("fp64")
        d = inv.G_vec_mul(rho)
        dobs = d + 0.02 * np.abs(d) * rng.standard_normal(d.size)
        inv.set_cross_gradient(False)
        inv.set_operators(reg.regular_mesh_operators((nx, nx, nz), prisms, obs, 1.5))
        inv.set_dobs(dobs, reg.data_weights(dobs, [0.02, 0.02], [1e-3, 1e-2], obs.shape[0]))
        if storage != "fp64":
            inv.compute_G(storage.split("+")[0], keep_fp64=True)
        invs.append(inv)
        nm = inv.Nm
        args.append((np.zeros(nm), np.full(nm, -1000.0), np.full(nm, 1000.0)))
    return invs, args


def time_batch(invs, args, team: int, storage: str, prm=None, reps: int = 2) -> float:
    import torch

    prm = prm or SHORT
    best = float("inf")
    for _ in range(reps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        invert_batch_persistent(invs, [prm] * len(invs), [a[0] for a in args],
                                [a[1] for a in args], [a[2] for a in args],
                                fp64_refinement=storage != "fp64", team_ctas=team)
        torch.cuda.synchronize()
        best = min(best, time.perf_counter() - t0)
    return best


def tune(storage: str = "fp32+fp64", classes=CLASSES, candidates=CANDIDATES):
    rows, report = [], {}
    for name, n, cells, points in classes:
        invs, args = synthetic_batch(n, cells, points, 500, storage)
        bound = max(i.Nd * i.Nm for i in invs)
        times = {t: time_batch(invs, args, t, storage) for t in candidates}
        best = min(times, key=times.get)
        rows.append((float(bound), int(best)))
        report[name] = {"largest_G_entries": int(bound), "seconds": times, "team": int(best)}
        for inv in invs:
            inv.ctx.close()
    rows.sort()
    return rows, report


def write_table(rows, path: Path, note: str) -> None:
    path.parent.mkdir(parents=True, exist_ok=True)
    lines = ["# team size of grada_invert_batch_persistent by the batch's largest G",
             f"# {note}", "# largest_G_entries  ctas_per_team"]
    lines += [f"{b:.6g} {t}" for b, t in rows]
    path.write_text("\n".join(lines) + "\n")


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=str(TABLE))
    ap.add_argument("--storage", default="fp32+fp64", choices=["fp32+fp64", "fp64"])
    a = ap.parse_args()
    rows, report = tune(a.storage)
    write_table(rows, Path(a.out), f"measured with {a.storage} G, shortened inversions "
                                   f"(1 Gauss-Newton iteration, 3 lambdas, 20 CG iterations)")
    print(json.dumps(report))


if __name__ == "__main__":
    main()
