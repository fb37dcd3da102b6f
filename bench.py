"""Benchmark: FP64 sensitivity assembly (G entries/s) on one GB300.

Workload (the reference's nine-component FP64 forward at scale): uniform
64 x 64 x 32 = 131,072 prism cells over x, y in [0, 20 km], z in [0, 8 km];
101 x 101 = 10,201 observation points on [0, 20 km]^2 at 50 m height;
components gz, gx, gy, Txx, Txy, Txz, Tyy, Tyz, Tzz (field flag 0x3FE), so G
is 91,809 x 131,072 = 1.2034e10 entries (96.3 GB in FP64).  One step is one
full assembly of G (Fwd::compute_G).  The inputs are the geometry only
(synthetic, built the way the reference's Mesh/Observation classes build
them); the output (96 GB) is far larger than L2.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

--impl reference times the reference algorithm on the host cores instead
(the CPU oracle restating the reference's face-integral kernels, OpenMP over
all host threads) on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import csv
import io
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO))

WORKLOAD = {
    "workload": "fp64 sensitivity assembly, 9 components",
    "cells": [64, 64, 32],
    "domain_m": [20000.0, 20000.0, 8000.0],
    "obs": [101, 101],
    "obs_height_m": 50.0,
    "field_flag": "0x3FE",
    "rows": 91809,
    "cols": 131072,
    "storage": "fp64",
}
MASK = 0x3FE
METRIC = "G entries/s"
UNIT = "entries/s"

# Algorithmic FP64 work per (observation, cell) pair for the nine-component
# flag, frozen once: the corner-grouped closed form evaluated cell by cell with
# only the faces of a vertical column shared, counted by ncu (DFMA = 2,
# DADD/DMUL = 1 from the executed-instruction counters) on a 1,024-point x
# 4,096-cell case (bench.py --case profile).  roofline.achieved is
# this figure x pairs/s.
FP64_FLOPS_PER_PAIR = 767.4

# FP64 work the current kernel executes per pair on the same case (faces shared
# with the cells above, before in y and before in x; seeded reciprocal and
# square root; 193-bin log and pi/128 rotation tables): 128.74 DFMA + 53.35 DADD
# + 122.19 DMUL.  Re-measured whenever the kernel changes; reported beside the
# algorithmic figure.
FP64_FLOPS_EXECUTED_PER_PAIR = 433.0

# DRAM bytes (read + write) of one assembly launch on this workload, from one ncu
# capture (dram__bytes_read.sum + dram__bytes_write.sum, one pass) of the full-size
# launch.  The algorithmic G write is 96.3 GB.
ASSEMBLY_DRAM_BYTES_PER_LAUNCH = 4_873_539_072 + 98_284_599_040


def build_problem():
    from graada3d_gb300 import mesh

    prisms = mesh.regular_mesh((0.0, 20000.0), 64, (0.0, 20000.0), 64, (0.0, 8000.0), 32)
    obs = mesh.observation_grid(101, 0.0, 20000.0, 101, 0.0, 20000.0, -50.0)
    rng = np.random.default_rng(3)
    boxes = []
    for _ in range(20):
        x0, y0 = rng.uniform(0, 20000, 2)
        z0 = rng.uniform(0, 8000)
        sx, sy, sz = rng.uniform(500, 4000, 3)
        boxes.append([x0, x0 + sx, y0, y0 + sy, z0, z0 + sz, rng.uniform(-500, 500)])
    rho = mesh.set_boxes(prisms, boxes)
    return prisms, obs, rho


# Output rows of the nine-component flag, in G's row order (ascending field bit).
COMPONENTS = ["gz", "gx", "gy", "Tzz", "Txz", "Tyz", "Txx", "Txy", "Tyy"]
PARITY_TOL = 1e-10  # FP64 path: |G - oracle| <= 1e-10 x max|component|


def parity_points(n_random: int = 39, seed: int = 11) -> np.ndarray:
    """Observation indices whose rows of the benchmarked G are checked against the
    oracle: the 25 points on x, y in {0, 5, 10, 15, 20} km, which lie on cell-face
    planes of the 312.5 m mesh (the coincident case), and n_random seeded others."""
    plane = [25 * iy * 101 + 25 * ix for iy in range(5) for ix in range(5)]
    rest = np.setdiff1d(np.arange(101 * 101), plane)
    pick = np.random.default_rng(seed).choice(rest, n_random, replace=False)
    return np.concatenate([np.array(plane, dtype=np.int64), np.sort(pick).astype(np.int64)])


def bench_parity(f, prisms, obs) -> dict:
    """Rows of the G that the timed steps assembled, read back from the device
    (grada_get_G_rows), against the oracle's G for the same points over all cells."""
    from oracle import prism as oracle_prism

    idx = parity_points()
    n_obs = obs.shape[0]
    rows = (idx[None, :] + n_obs * np.arange(len(COMPONENTS))[:, None]).ravel()
    got = f.get_G_rows(rows)
    oracle_prism.build()
    t0 = time.perf_counter()
    want = oracle_prism.compute_G(prisms, obs[idx], MASK)
    t_oracle = time.perf_counter() - t0
    n = idx.size
    errs = {}
    for k, name in enumerate(COMPONENTS):
        blk = slice(k * n, (k + 1) * n)
        errs[name] = float(np.abs(got[blk] - want[blk]).max() / np.abs(want[blk]).max())
    worst = max(errs.values())
    return {"points": int(n), "face_plane_points": 25, "rows": int(rows.size), "cells": int(prisms.shape[0]),
            "max_rel_err": errs, "worst": worst, "tol": PARITY_TOL, "pass": bool(worst <= PARITY_TOL),
            "against": "oracle (Fwd::compute_G restated in C) on the same points, all cells",
            "oracle_s": t_oracle}


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        out, _ = self.proc.communicate(timeout=10)
        rows = [r for r in csv.reader(io.StringIO(out)) if len(r) >= 9]
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                smax = float(r[2])
            except ValueError:
                continue
            for name, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(name)
        load = [s for s in sm if smax and s > 0.3 * smax] or sm
        return {"sm_mhz": statistics.median(load) if load else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_sample(prisms, obs, target_s: float = 12.0):
    """Reference algorithm (CPU oracle) on a bounded observation subset."""
    from oracle import prism as oracle_prism

    oracle_prism.build()
    threads = oracle_prism.num_threads()
    n = 2
    t0 = time.perf_counter()
    oracle_prism.compute_G(prisms, obs[:n], MASK)
    dt = time.perf_counter() - t0
    n_obs = int(min(obs.shape[0], max(n, round(n * target_s / max(dt, 1e-3)))))
    t0 = time.perf_counter()
    oracle_prism.compute_G(prisms, obs[:n_obs], MASK)
    dt = time.perf_counter() - t0
    entries = 9 * n_obs * prisms.shape[0]
    return {
        "value": entries / dt,
        "unit": UNIT,
        "cores": threads,
        "kind": "port",
        "sample": f"Fwd::compute_G restated in C (oracle/prism_oracle.c), {n_obs} observation points x "
                  f"{prisms.shape[0]} cells x 9 components = {entries:.3e} entries in {dt:.2f} s",
        "seconds": dt,
    }


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group(backend="gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(world, v: float) -> float:
    if world <= 1:
        return v
    import torch
    import torch.distributed as dist

    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def shard_units(n: int, world: int, rank: int) -> list[int]:
    """Indices of the independent units (problems, lambda values) this rank runs
    when replicas share a batch: round-robin, disjoint, covering 0..n-1."""
    return list(range(rank, n, world))


def run_reference(args):
    world, rank, _ = dist_init()
    if rank != 0:
        return
    prisms, obs, _ = build_problem()
    for _ in range(max(0, min(args.warmup, 1))):
        cpu_sample(prisms, obs, target_s=2.0)
    times = []
    samples = []
    for _ in range(args.steps):
        s = cpu_sample(prisms, obs, target_s=args.ref_seconds)
        samples.append(s)
        times.append(s["seconds"])
    value = float(np.median([s["value"] for s in samples]))
    entries_full = 9 * obs.shape[0] * prisms.shape[0]
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * entries_full / value,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic",
        "config": dict(WORKLOAD, sample="bounded observation subset per step, extrapolated by entries/s"),
        "cpu_baseline": {k: samples[-1][k] for k in ("value", "unit", "cores", "kind", "sample")},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    line["cpu_baseline"]["value"] = value
    print(json.dumps(line))


def run_gpu(args):
    world, rank, local = dist_init()
    import torch

    from graada3d_gb300 import Context, Fwd

    torch.cuda.set_device(local)
    prisms, obs, rho = build_problem()
    ctx = Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", local))
    fp64_peak = ctx.fp64_peak()
    f = Fwd(prisms, obs, MASK, ctx=ctx)
    entries = f.Nd * f.Nm
    pairs = f.N_obs * f.Nm

    # ---- device-resident assembly (value) ---------------------------------
    for _ in range(args.warmup):
        f.compute_G("fp64")
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    clocks = ClockSampler(local)
    barrier(world)
    torch.cuda.synchronize()
    clocks.start()
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    t_start.record(stream)
    for k in range(args.steps):
        ev[k][0].record(stream)
        f.compute_G("fp64")
        ev[k][1].record(stream)
    t_end.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    clk = clocks.stop()
    total_ms = t_start.elapsed_time(t_end)
    per_launch_ms = [a.elapsed_time(b) for a, b in ev]
    total_ms = max_over_ranks(world, total_ms)
    ms_per_step = total_ms / args.steps
    value = world * entries * args.steps / (total_ms * 1e-3)

    # ---- end to end through the C ABI with host buffers (e2e) --------------
    h2d = prisms.nbytes + obs.nbytes + rho.nbytes
    d2h = f.Nd * 8
    e2e_steps = max(1, min(args.steps, 3))
    f.set_geometry(prisms, obs, MASK)
    f.compute_G("fp64")
    f.G_vec_mul(rho)
    barrier(world)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        f.set_geometry(prisms, obs, MASK)  # H2D of the geometry
        f.compute_G("fp64")
        d = f.G_vec_mul(rho)  # predicted field back to the host
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(world, (time.perf_counter() - t0) / e2e_steps)
    assert np.isfinite(d).all()
    e2e_value = world * entries / e2e_s
    # parity of the benchmarked G itself (after the timed region)
    parity = bench_parity(f, prisms, obs) if rank == 0 else None

    roofline = None
    per_launch = statistics.median(per_launch_ms) * 1e-3
    if FP64_FLOPS_PER_PAIR:
        achieved = FP64_FLOPS_PER_PAIR * pairs / per_launch
        roofline = {"bound": "fp64", "achieved": achieved / 1e12, "peak": fp64_peak / 1e12,
                    "unit": "TFLOP/s", "frac": achieved / fp64_peak,
                    "traffic": ASSEMBLY_DRAM_BYTES_PER_LAUNCH,
                    "traffic_unit": "bytes per launch (ncu, full-size launch)",
                    "algorithmic_flops_per_pair": FP64_FLOPS_PER_PAIR,
                    "executed_flops_per_pair": FP64_FLOPS_EXECUTED_PER_PAIR,
                    "executed_tflops": FP64_FLOPS_EXECUTED_PER_PAIR * pairs / per_launch / 1e12,
                    "executed_frac": FP64_FLOPS_EXECUTED_PER_PAIR * pairs / per_launch / fp64_peak,
                    "note": "algorithmic work is the frozen per-cell figure; the kernel shares "
                            "faces between neighbouring cells and executes less, so frac can "
                            "exceed 1 while executed_frac stays below it",
                    "peak_source": "DFMA loop measured in this run (grada_measure_fp64_peak)"}
    else:
        roofline = {"bound": "fp64", "achieved": None, "peak": fp64_peak / 1e12, "unit": "TFLOP/s",
                    "frac": None, "traffic": None,
                    "peak_source": "DFMA loop measured in this run (grada_measure_fp64_peak)"}
    g_bytes = entries * 8
    hbm = {"write_GBps": g_bytes / per_launch / 1e9}
    try:
        peaks = json.loads((REPO / "MEASURED_PEAKS.json").read_text())
        hbm["peak_GBps"] = peaks.get("hbm_gbs")
        hbm["frac"] = hbm["write_GBps"] / peaks["hbm_gbs"]
    except Exception:
        pass

    if rank == 0:
        line = {
            "metric": METRIC,
            "value": value,
            "unit": UNIT,
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": ms_per_step,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f64",
            "data": "synthetic",
            "config": dict(WORKLOAD, l2="output per step (96 GB) is larger than L2; inputs are 6.5 MB of geometry",
                           parallelism="replicas" if world > 1 else "single GPU"),
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "steps": e2e_steps,
                    "includes": "grada_set_geometry (H2D) + grada_compute_G + grada_G_vec_mul (host rho -> host field)"},
            "gpu_launches": args.steps,
            "kernel_ms": {"median": statistics.median(per_launch_ms), "min": min(per_launch_ms),
                          "max": max(per_launch_ms)},
            "roofline": roofline,
            "parity": parity,
            "hbm_write": hbm,
            "clocks": clk,
        }
        if world == 1 and not args.no_block:
            line["block_products"] = block_products_summary()
        if world == 1 and not args.no_inversion:
            # second half of the metric: inversion time to chi^2 = N, mixed precision vs
            # all-FP64 -- the 16,384-cell L2 problem and the L1 problem on the
            # 236,226-leaf refined dyke mesh (gz, Tzz, Txz, Tyz at 101 x 101 points)
            line["inversion"] = run_inversion("l2_16k")
            if not args.no_refined_inversion:
                line["inversion_refined"] = run_inversion(
                    "l1_refined_chi2", ("fp64", "fp32+fp64", "bf16+fp64", "fp16+fp64"))
        if world == 1 and not args.no_cpu_baseline:
            cb = cpu_sample(prisms, obs, target_s=args.ref_seconds)
            cb.pop("seconds", None)
            line["cpu_baseline"] = cb
        print(json.dumps(line))
    ctx.close()


INVERSION_CASES = {
    # 32 x 32 x 16 cells over [0,10 km]^2 x [0,5 km], gz + Tzz at
    # 41 x 41 points 100 m above, L2, lambda0 = 0.1, 30 lambdas, rate 0.6, CG max 50
    "l2_16k": dict(cells=(32, 32, 16), domain=(10000.0, 10000.0, 5000.0), obs=(41, 41), height=100.0,
                 mask=0x012, lp=[2, 2, 2, 2, 2], eps2=1e-9, boxes="two_boxes", gn_iter=10),
    # L1 IRLS on a uniform mesh of about the refined one's size: 196,608 cells (64 x 64 x 48 over the
    # same domain; the reference refines to ~200k leaves on the host): gz, Tzz, Txz, Tyz at
    # 101 x 101 points 100 m above, two dykes of +400 kg/m^3, L1 IRLS
    "l1_196k": dict(cells=(64, 64, 48), domain=(10000.0, 10000.0, 5000.0), obs=(101, 101),
                 height=100.0, mask=0x072, lp=[1, 1, 1, 1, 2], eps2=1e-10, boxes="dykes",
                 gn_iter=10),
    # the same L1 problem on the 32 x 32 x 16 base refined 3 levels at the dyke boundaries
    # with the reference's face-balance cascade (236,226 leaves), operators from the
    # leaves' geometry
    "l1_refined": dict(cells="dyke_refined", domain=(10000.0, 10000.0, 5000.0), obs=(101, 101),
                       height=100.0, mask=0x072, lp=[1, 1, 1, 1, 2], eps2=1e-10, boxes="dykes",
                       gn_iter=10),
    # the same refined problem with a schedule under which the runs reach chi^2 = N:
    # lambda_0 = 1e-4 halved per trial, up to 200 CG iterations per solve and a
    # 0.5 % stagnation test (with at most 50 CG iterations every format stops on
    # stagnation at a misfit near 1.5; schedules with lambda_0 = 0.1, 1e-3 and
    # rates 0.3-0.6 reach it with 5,200-7,600 CG iterations, this one with the fewest)
    "l1_refined_chi2": dict(cells="dyke_refined", domain=(10000.0, 10000.0, 5000.0),
                            obs=(101, 101), height=100.0, mask=0x072, lp=[1, 1, 1, 1, 2],
                            eps2=1e-10, boxes="dykes", gn_iter=10,
                            prm=dict(max_lambda=1e-4, rate=0.5, cg_factor=200, stag=0.005)),
}


def inversion_problem(name: str):
    from graada3d_gb300 import mesh
    from graada3d_gb300 import regularization as reg

    c = INVERSION_CASES[name]
    Lx, Ly, Lz = c["domain"]
    if c["cells"] == "dyke_refined":
        prisms = refined_dyke_mesh(3)
    else:
        nx, ny, nz = c["cells"]
        prisms = mesh.regular_mesh((0.0, Lx), nx, (0.0, Ly), ny, (0.0, Lz), nz)
    obs = mesh.observation_grid(c["obs"][0], 0.0, Lx, c["obs"][1], 0.0, Ly, -c["height"])
    rng = np.random.default_rng(1 if c["boxes"] == "two_boxes" else 4)
    if c["boxes"] == "two_boxes":
        boxes = []
        for v in (300.0, -200.0):
            sx, sy, sz = rng.uniform(1000, 3000, 3)
            x0, y0 = rng.uniform(0, Lx - sx), rng.uniform(0, Ly - sy)
            z0 = rng.uniform(0, Lz - sz)
            boxes.append([x0, x0 + sx, y0, y0 + sy, z0, z0 + sz, v])
    else:
        boxes = [[2500, 3500, 1000, 9000, 500, 3500, 400.0], [6000, 7000, 1000, 9000, 500, 3500, 400.0]]
    rho = mesh.set_boxes(prisms, boxes)
    nf = bin(c["mask"]).count("1")
    rel = [0.02] * nf
    absf = [1e-3 if (c["mask"] & 2) and k == 0 else 1e-2 for k in range(nf)]
    if c["cells"] == "dyke_refined":
        ops = reg.mesh_operators(prisms, obs, 1.5)
    else:
        ops = reg.regular_mesh_operators((nx, ny, nz), prisms, obs, 1.5)
    return c, prisms, obs, rho, rel, absf, ops, rng


def run_inversion(name: str, storages=("fp64", "fp32", "fp16", "bf16", "fp32+fp64", "fp16+fp64")):
    """Inversion to chi^2 = N (misfit < 1) on the GPU: all-FP64 vs reduced-precision
    G with one FP64 residual refinement per Gauss-Newton iteration; "X+fp64" keeps
    the FP64 G beside the X one and predicts every trial with it (grada_keep_fp64_G)."""
    import torch

    from graada3d_gb300 import regularization as reg
    from graada3d_gb300.inversion import GaussNewtonInversion

    c, prisms, obs, rho, rel, absf, ops, rng = inversion_problem(name)
    inv = GaussNewtonInversion(prisms, obs, c["mask"])
    inv.compute_G("fp64")
    d = inv.G_vec_mul(rho)
    dobs = d + 0.02 * np.abs(d) * np.random.default_rng(2 if name == "l2_16k" else 5).standard_normal(d.size)
    wd = reg.data_weights(dobs, rel, absf, obs.shape[0])
    inv.set_cross_gradient(False)
    inv.set_operators(ops)
    inv.set_dobs(dobs, wd)
    nm = inv.Nm
    prm = dict(max_lambda=1e-1, n_lambda=30, rate=0.6, target=1.0, stag=0.02, cg_tol=1e-6,
               cg_factor=50, gn_iter=c["gn_iter"], lp=c["lp"], eps2=c["eps2"])
    prm.update(c.get("prm", {}))
    args = (np.zeros(nm), np.full(nm, -1000.0), np.full(nm, 1000.0))
    out = {"case": name, "cells": nm, "data": inv.Nd, "lp": c["lp"][0],
           "schedule": {k: prm[k] for k in ("max_lambda", "n_lambda", "rate", "stag", "cg_tol",
                                             "cg_factor", "gn_iter", "target")}}
    m64 = None
    for st in storages:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        inv.compute_G(st.split("+")[0], keep_fp64=st.endswith("+fp64"))
        torch.cuda.synchronize()
        t_asm = time.perf_counter() - t0
        t0 = time.perf_counter()
        m, rep = inv.invert(prm, *args, fp64_refinement=(st != "fp64"))
        t_inv = time.perf_counter() - t0
        r = {"assemble_s": t_asm, "invert_s": t_inv, "total_s": t_asm + t_inv,
             "misfit": rep["final_misfit"], "chi2_reached": rep["final_misfit"] < 1.0,
             "gn_iterations": rep["gn_iterations"], "trials": rep["n_trials"],
             "cg_iterations": int(rep["cg_iterations"]),
             "ms_per_cg_iteration": 1e3 * t_inv / max(1, rep["cg_iterations"]),
             "gn_misfits": [float(v) for v in inv.iterations()[:, 2]]}
        loop_s, graph_s, n_loop = inv.cg_loop_time()
        if n_loop:  # the CG loops alone (set-up, predictions and lambda control excluded)
            r["cg_loop_ms_per_iteration"] = 1e3 * loop_s / n_loop
            r["cg_graph_build_s"] = graph_s
        ph, n_ph = inv.cg_phase_times()
        if n_ph:  # the persistent CG loop ran: its phases' mean time per iteration
            r["cg_phase_us"] = {"gp": ph[0] / 1e3, "finish_rows": ph[1] / 1e3, "step": ph[2] / 1e3,
                                "gts_adjoint": ph[3] / 1e3}
        if st == "fp64":
            m64 = m
        else:
            if m64 is not None:
                r["model_rel_diff_vs_fp64"] = float(np.linalg.norm(m - m64) / np.linalg.norm(m64))
            r["fp64_refinements"] = int(rep["fp64_refinements"])
        out[st] = r
    if "fp64" in out:
        for st in storages:
            if st != "fp64":
                out[st]["invert_speedup_vs_fp64"] = out["fp64"]["invert_s"] / out[st]["invert_s"]
                out[st]["wall_speedup_vs_fp64"] = out["fp64"]["total_s"] / out[st]["total_s"]
    inv.ctx.close()
    return out


def run_matrix_free_1m():
    """One matrix-free G x and G^T y with 128 x 128 x 64 =
    1,048,576 cells over [0, 20 km]^2 x [0, 8 km], gz + Tzz at 201 x 201 points
    50 m above (G would be 80,802 x 1,048,576 = 678 GB in FP64, beyond HBM)."""
    import torch

    from graada3d_gb300 import mesh
    from graada3d_gb300.inversion import GaussNewtonInversion

    prisms = mesh.regular_mesh((0.0, 20000.0), 128, (0.0, 20000.0), 128, (0.0, 8000.0), 64)
    obs = mesh.observation_grid(201, 0.0, 20000.0, 201, 0.0, 20000.0, -50.0)
    inv = GaussNewtonInversion(prisms, obs, 0x012)
    inv.compute_G("matrix_free")
    lib, h = inv.ctx.lib, inv.ctx.handle
    import ctypes

    dev = torch.device("cuda")
    x = torch.randn(inv.Nm, dtype=torch.float64, device=dev)
    y = torch.randn(inv.ld, dtype=torch.float64, device=dev)
    dout = torch.empty(inv.ld, dtype=torch.float64, device=dev)
    xout = torch.empty(inv.Nm, dtype=torch.float64, device=dev)
    stream = torch.cuda.ExternalStream(inv.ctx.stream)
    out = {"case": "matrix-free-1m", "cells": inv.Nm, "points": inv.N_obs, "rows": inv.Nd,
           "pairs_per_product": inv.N_obs * inv.Nm}
    for name, fn, a, b in (("G_x", lib.grada_G_vec_mul_dev, x, dout),
                           ("GT_y", lib.grada_GT_vec_mul_dev, y, xout)):
        fn(h, ctypes.c_void_p(a.data_ptr()), ctypes.c_void_p(b.data_ptr()))  # warm-up
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn(h, ctypes.c_void_p(a.data_ptr()), ctypes.c_void_p(b.data_ptr()))
        e1.record(stream)
        torch.cuda.synchronize()
        s = e0.elapsed_time(e1) * 1e-3
        out[name] = {"s": s, "pairs_per_s": out["pairs_per_product"] / s,
                     "G_entries_per_s": inv.Nd * inv.Nm / s}
    out["cg_iteration_s"] = out["G_x"]["s"] + out["GT_y"]["s"]
    inv.ctx.close()
    return out


def run_gemv_case():
    """G x and G^T y alone with a 40,804 x 196,608 G (4 components at 101 x 101 points over 196,608 cells), every
    storage kind: 3 warm-up + 10 timed calls each, CUDA events on the context
    stream; G (16-64 GB) is far larger than L2."""
    import ctypes

    import torch

    from graada3d_gb300 import Fwd, mesh

    prisms = mesh.regular_mesh((0.0, 10000.0), 64, (0.0, 10000.0), 64, (0.0, 5000.0), 48)
    obs = mesh.observation_grid(101, 0.0, 10000.0, 101, 0.0, 10000.0, -100.0)
    f = Fwd(prisms, obs, 0x072)
    lib, h = f.ctx.lib, f.ctx.handle
    stream = torch.cuda.ExternalStream(f.ctx.stream)
    dev = torch.device("cuda")
    x = torch.randn(f.Nm, dtype=torch.float64, device=dev)
    y = torch.randn(f.ld, dtype=torch.float64, device=dev)
    ox = torch.empty(f.Nm, dtype=torch.float64, device=dev)
    oy = torch.empty(f.ld, dtype=torch.float64, device=dev)
    peak = json.loads((REPO / "MEASURED_PEAKS.json").read_text()).get("hbm_gbs") \
        if (REPO / "MEASURED_PEAKS.json").exists() else None
    res = {"case": "gemv", "rows": f.Nd, "cols": f.Nm, "hbm_peak_GBps": peak}
    for st, bpe in (("fp64", 8), ("fp32", 4), ("fp16", 2), ("bf16", 2)):
        f.compute_G(st)
        gbytes = f.Nd * f.Nm * bpe + 8 * (f.Nd + f.Nm)
        for name, fn, a, b in (("G_x", lib.grada_G_vec_mul_dev, x, oy),
                               ("GT_y", lib.grada_GT_vec_mul_dev, y, ox)):
            for _ in range(3):
                fn(h, ctypes.c_void_p(a.data_ptr()), ctypes.c_void_p(b.data_ptr()))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(stream)
            for _ in range(10):
                fn(h, ctypes.c_void_p(a.data_ptr()), ctypes.c_void_p(b.data_ptr()))
            e1.record(stream)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / 10
            r = {"ms": ms, "GBps": gbytes / ms / 1e6}
            if peak:
                r["frac_of_hbm"] = r["GBps"] / peak
            res[f"{st}_{name}"] = r
    f.ctx.close()
    return res


def run_batched_64(n_problems: int = 64):
    """Independent inversions of uneven size (uniform
    meshes nx = ny, nz = nx/2 with 4k-60k cells, square point grids of 400-5,000
    points, gz + Tzz, seeded models, seeds 100..163), run one after the other and
    then as one concurrent batch (one context, host thread and stream each).
    Under torchrun the problems are sharded over the ranks (replicas, one GPU
    each); times are the max over ranks."""
    import torch

    from graada3d_gb300 import Context, mesh
    from graada3d_gb300 import regularization as reg
    from graada3d_gb300.inversion import (GaussNewtonInversion, compute_G_batch, invert_batch,
                                          invert_batch_persistent)

    world, rank, local = dist_init()
    if torch.cuda.is_available():
        torch.cuda.set_device(local)
    prm = dict(max_lambda=1e-1, n_lambda=30, rate=0.6, target=1.0, stag=0.02, cg_tol=1e-6,
               cg_factor=50, gn_iter=10, lp=[2, 2, 2, 2, 2], eps2=1e-9)
    invs, args, sizes = [], [], []
    mine = shard_units(n_problems, world, rank)
    for k in mine:
        rng = np.random.default_rng(100 + k)
        cells = int(rng.integers(4000, 60001))
        nx = max(4, int(round((2 * cells) ** (1 / 3))))
        nz = max(2, nx // 2)
        pts = int(rng.integers(400, 5001))
        no = max(2, int(round(pts ** 0.5)))
        L = 10000.0
        prisms = mesh.regular_mesh((0.0, L), nx, (0.0, L), nx, (0.0, L / 2), nz)
        obs = mesh.observation_grid(no, 0.0, L, no, 0.0, L, -100.0)
        boxes = []
        for v in (300.0, -200.0):
            s_ = rng.uniform(1000, 3000, 3)
            x0, y0, z0 = rng.uniform(0, L - s_[0]), rng.uniform(0, L - s_[1]), rng.uniform(0, L / 2 - s_[2])
            boxes.append([x0, x0 + s_[0], y0, y0 + s_[1], z0, z0 + s_[2], v])
        rho = mesh.set_boxes(prisms, boxes)
        inv = GaussNewtonInversion(prisms, obs, 0x012, ctx=Context(local))
        inv.compute_G("fp64")
        d = inv.G_vec_mul(rho)
        dobs = d + 0.02 * np.abs(d) * rng.standard_normal(d.size)
        inv.set_cross_gradient(False)
        inv.set_operators(reg.regular_mesh_operators((nx, nx, nz), prisms, obs, 1.5))
        inv.set_dobs(dobs, reg.data_weights(dobs, [0.02, 0.02], [1e-3, 1e-2], obs.shape[0]))
        invs.append(inv)
        nm = inv.Nm
        args.append((np.zeros(nm), np.full(nm, -1000.0), np.full(nm, 1000.0)))
        sizes.append((nm, obs.shape[0]))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for inv in invs:
        inv.compute_G("fp64")
    seq = [inv.invert(prm, *a) for inv, a in zip(invs, args)]
    torch.cuda.synchronize()
    t_seq = time.perf_counter() - t0
    t0 = time.perf_counter()
    compute_G_batch(invs, "fp64")
    bat = invert_batch(invs, [prm] * len(invs), [a[0] for a in args], [a[1] for a in args],
                       [a[2] for a in args])
    torch.cuda.synchronize()
    t_bat = time.perf_counter() - t0
    same = all(np.array_equal(a[0], b[0]) for a, b in zip(seq, bat))
    reached = sum(1 for _, r in bat if r["final_misfit"] < 1.0)
    # the same batch in one persistent launch (a team of CTAs per problem from a
    # device queue; team size from the tuning table)
    t0 = time.perf_counter()
    compute_G_batch(invs, "fp64")
    per, shape = invert_batch_persistent(invs, [prm] * len(invs), [a[0] for a in args],
                                         [a[1] for a in args], [a[2] for a in args])
    torch.cuda.synchronize()
    t_per = time.perf_counter() - t0
    # the single runs take the CG loop's phase kernels, the batch the same
    # phases in one persistent launch: the same sums in the same order
    per_diff = max(float(np.linalg.norm(a[0] - b[0]) / max(np.linalg.norm(a[0]), 1e-30))
                   for a, b in zip(seq, per))
    per_same = all(np.array_equal(a[0], b[0]) for a, b in zip(seq, per))
    # the same batch with FP32 G (HBM-bound products) and the FP64 G kept for
    # every prediction
    t0 = time.perf_counter()
    compute_G_batch(invs, "fp32", keep_fp64=True)
    mix = invert_batch(invs, [prm] * len(invs), [a[0] for a in args], [a[1] for a in args],
                       [a[2] for a in args], fp64_refinement=True)
    torch.cuda.synchronize()
    t_mix = time.perf_counter() - t0
    mix_diff = [float(np.linalg.norm(a[0] - b[0]) / max(np.linalg.norm(b[0]), 1e-30))
                for a, b in zip(mix, bat)]
    mix_reached = sum(1 for _, r in mix if r["final_misfit"] < 1.0)
    t0 = time.perf_counter()
    compute_G_batch(invs, "fp32", keep_fp64=True)
    mix_per, mix_shape = invert_batch_persistent(invs, [prm] * len(invs), [a[0] for a in args],
                                                 [a[1] for a in args], [a[2] for a in args],
                                                 fp64_refinement=True)
    torch.cuda.synchronize()
    t_mix_per = time.perf_counter() - t0
    mix_per_same = all(np.array_equal(a[0], b[0]) for a, b in zip(mix, mix_per))
    # G bytes the CG products stream (two reads of G per CG iteration), the
    # bulk of the batch's HBM traffic; over the whole wall time (assembly,
    # predictions and set-up included) a lower bound on the products' rate
    entries = [inv.ld * inv.Nm for inv in invs]

    def cg_bytes(results, esize):
        return float(sum(2 * r["cg_iterations"] * e * esize for (_, r), e in zip(results, entries)))

    b64, b64_per = cg_bytes(bat, 8), cg_bytes(per, 8)
    b32, b32_per = cg_bytes(mix, 4), cg_bytes(mix_per, 4)
    for inv in invs:
        inv.ctx.close()
    t_seq, t_bat = max_over_ranks(world, t_seq), max_over_ranks(world, t_bat)
    t_mix = max_over_ranks(world, t_mix)
    t_per, t_mix_per = max_over_ranks(world, t_per), max_over_ranks(world, t_mix_per)
    return {"case": "batched-64", "problems": n_problems, "ranks": world,
            "problems_per_rank": len(mine),
            "cells_range": [min(s[0] for s in sizes), max(s[0] for s in sizes)],
            "points_range": [min(s[1] for s in sizes), max(s[1] for s in sizes)],
            "sequential_s": t_seq, "batched_s": t_bat, "speedup": t_seq / t_bat,
            "identical_models": same, "chi2_reached_rank0": reached,
            "persistent": {"launches": 1, "teams": shape[0], "ctas_per_team": shape[1],
                           "s": t_per, "speedup_vs_sequential": t_seq / t_per,
                           "speedup_vs_concurrent": t_bat / t_per,
                           "identical_models_to_single_runs": per_same,
                           "max_model_rel_diff_vs_single_runs": per_diff},
            "cg_iterations_rank0": int(sum(r["cg_iterations"] for _, r in bat)),
            "cg_G_bytes_rank0": {"fp64": b64, "fp32": b32},
            "cg_G_TB_per_s_rank0": {"fp64_concurrent": b64 / t_bat / 1e12,
                                    "fp64_persistent": b64_per / t_per / 1e12,
                                    "fp32_concurrent": b32 / t_mix / 1e12,
                                    "fp32_persistent": b32_per / t_mix_per / 1e12},
            "fp32_kept_fp64": {"batched_s": t_mix, "speedup_vs_fp64_batch": t_bat / t_mix,
                               "persistent": {"launches": 1, "teams": mix_shape[0],
                                              "ctas_per_team": mix_shape[1], "s": t_mix_per,
                                              "speedup_vs_concurrent": t_mix / t_mix_per,
                                              "speedup_vs_fp64_persistent": t_per / t_mix_per,
                                              "identical_models_to_single_runs": mix_per_same},
                               "model_rel_diff_vs_fp64": {"median": float(np.median(mix_diff)),
                                                          "max": float(np.max(mix_diff))},
                               "chi2_reached_rank0": mix_reached}}


def sweep_problem():
    """The 64 x 64 x 32 mesh of the assembly benchmark (64 x 64 x 32 =
    131,072 cells over [0, 20 km]^2 x [0, 8 km]) and points (101 x 101 at 50 m),
    the gz + Tzz rows of its G (20,402 x 131,072), its 20-box model, data with 2 %
    seeded noise."""
    from graada3d_gb300 import regularization as reg

    prisms, obs, rho = build_problem()
    ops = reg.regular_mesh_operators((64, 64, 32), prisms, obs, 1.5)
    return prisms, obs, rho, ops


def _peak_gbs():
    p = REPO / "MEASURED_PEAKS.json"
    return json.loads(p.read_text()).get("hbm_gbs") if p.exists() else None


def run_block_gemm_case():
    """The 16-column block products G X and G^T Y against sixteen single products,
    on the 20,402 x 131,072 gz + Tzz G of the assembly benchmark's geometry, each storage:
    3 warm-up + 10 timed calls, CUDA events on the context stream.  G (5-21 GB)
    is far larger than L2."""
    import ctypes

    import torch

    from graada3d_gb300 import Fwd

    prisms, obs, rho, _ = sweep_problem()
    f = Fwd(prisms, obs, 0x012)
    lib, h = f.ctx.lib, f.ctx.handle
    stream = torch.cuda.ExternalStream(f.ctx.stream)
    dev = torch.device("cuda")
    X = torch.randn(f.Nm * 16, dtype=torch.float64, device=dev)
    Y = torch.randn(f.ld * 16, dtype=torch.float64, device=dev)
    oX = torch.empty(f.Nm * 16, dtype=torch.float64, device=dev)
    oY = torch.empty(f.ld * 16, dtype=torch.float64, device=dev)
    x1 = torch.randn(f.Nm, dtype=torch.float64, device=dev)
    y1 = torch.randn(f.ld, dtype=torch.float64, device=dev)
    o1 = torch.empty(max(f.Nm, f.ld), dtype=torch.float64, device=dev)
    peak = _peak_gbs()
    res = {"case": "block-gemm", "rows": f.Nd, "cols": f.Nm, "rhs": 16, "hbm_peak_GBps": peak}

    def timed(fn, a, b, reps=10):
        for _ in range(3):
            f.ctx.check(fn(h, ctypes.c_void_p(a.data_ptr()), ctypes.c_void_p(b.data_ptr())))
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn(h, ctypes.c_void_p(a.data_ptr()), ctypes.c_void_p(b.data_ptr()))
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    for st, bpe in (("fp32", 4), ("bf16", 2), ("fp16", 2), ("fp64", 8)):
        f.compute_G(st)
        gbytes = f.Nd * f.Nm * bpe
        flops = 2.0 * f.Nd * f.Nm * 16
        for name, fb, a, b, fs, a1 in (("G_X", lib.grada_G_block_mul_dev, X, oY, lib.grada_G_vec_mul_dev, x1),
                                        ("GT_Y", lib.grada_GT_block_mul_dev, Y, oX, lib.grada_GT_vec_mul_dev, y1)):
            ms = timed(fb, a, b, reps=10 if st != "fp64" else 3)
            ms1 = timed(fs, a1, o1)
            r = {"ms": ms, "GBps": gbytes / ms / 1e6, "TFLOPs": flops / ms / 1e9,
                 "single_product_ms": ms1, "speedup_vs_16_single": 16 * ms1 / ms}
            if peak:
                r["frac_of_hbm"] = r["GBps"] / peak
            res[f"{st}_{name}"] = r
    f.ctx.close()
    return res


def run_block_gemm_profile():
    """Fixed small case for ncu captures of the tensor-core block products:
    gz + Tzz rows of a 32 x 32 x 32 = 32,768-cell mesh under the 101 x 101
    points (20,402 x 32,768; FP32 G 2.7 GB, larger than L2), FP32 then bf16,
    two G X and two G^T Y calls each."""
    import ctypes

    import torch

    from graada3d_gb300 import Fwd, mesh

    prisms = mesh.regular_mesh((0.0, 20000.0), 32, (0.0, 20000.0), 32, (0.0, 8000.0), 32)
    obs = mesh.observation_grid(101, 0.0, 20000.0, 101, 0.0, 20000.0, -50.0)
    f = Fwd(prisms, obs, 0x012)
    lib, h = f.ctx.lib, f.ctx.handle
    dev = torch.device("cuda")
    X = torch.randn(f.Nm * 16, dtype=torch.float64, device=dev)
    Y = torch.randn(f.ld * 16, dtype=torch.float64, device=dev)
    oX = torch.empty(f.Nm * 16, dtype=torch.float64, device=dev)
    oY = torch.empty(f.ld * 16, dtype=torch.float64, device=dev)
    for st in ("fp32", "bf16"):
        f.compute_G(st)
        for _ in range(2):
            f.ctx.check(lib.grada_G_block_mul_dev(h, ctypes.c_void_p(X.data_ptr()), ctypes.c_void_p(oY.data_ptr())))
            f.ctx.check(lib.grada_GT_block_mul_dev(h, ctypes.c_void_p(Y.data_ptr()), ctypes.c_void_p(oX.data_ptr())))
        torch.cuda.synchronize()
    f.ctx.close()
    print(json.dumps({"case": "block-gemm-profile", "rows": f.Nd, "cols": f.Nm}))


def block_products_summary():
    """Tensor-core block products (16 right-hand sides) on the gz + Tzz rows of the
    bench geometry (20,402 x 131,072), FP32 (3xTF32) and bf16 G: ms per product
    (3 warm-up + 10 timed, CUDA events) and the fraction of the measured HBM copy
    peak the algorithmic bytes (Nd x Nm x bytes/entry) reach."""
    import ctypes

    import torch

    from graada3d_gb300 import Fwd

    prisms, obs, _ = build_problem()
    f = Fwd(prisms, obs, 0x012)
    lib, h = f.ctx.lib, f.ctx.handle
    stream = torch.cuda.ExternalStream(f.ctx.stream)
    dev = torch.device("cuda")
    X = torch.randn(f.Nm * 16, dtype=torch.float64, device=dev)
    Y = torch.randn(f.ld * 16, dtype=torch.float64, device=dev)
    oX = torch.empty(f.Nm * 16, dtype=torch.float64, device=dev)
    oY = torch.empty(f.ld * 16, dtype=torch.float64, device=dev)
    peak = _peak_gbs()
    out = {"rows": f.Nd, "cols": f.Nm, "rhs": 16}
    for st, bpe in (("fp32", 4), ("bf16", 2)):
        f.compute_G(st)
        for name, fn, a, b in (("G_X", lib.grada_G_block_mul_dev, X, oY),
                               ("GT_Y", lib.grada_GT_block_mul_dev, Y, oX)):
            for _ in range(3):
                f.ctx.check(fn(h, ctypes.c_void_p(a.data_ptr()), ctypes.c_void_p(b.data_ptr())))
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(10):
                fn(h, ctypes.c_void_p(a.data_ptr()), ctypes.c_void_p(b.data_ptr()))
            e1.record(stream)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / 10
            r = {"ms": round(ms, 4), "GBps": round(f.Nd * f.Nm * bpe / ms / 1e6, 1)}
            if peak:
                r["frac_of_hbm"] = round(r["GBps"] / peak, 3)
            out[f"{st}_{name}"] = r
    f.ctx.close()
    return out


def run_lambda_sweep_16(n_lambda: int = 16, gn_iter: int = 5,
                        storages=("fp64", "fp32", "bf16", "fp32+fp64", "bf16+fp64"),
                        sequential: bool = True):
    """A 16-value regularisation sweep (lambda
    log-spaced 1e-3 .. 1e1) on the shared gz + Tzz G of the assembly benchmark's geometry,
    each lambda a fixed-lambda Gauss-Newton run (L2, CG <= 50, up to gn_iter
    iterations), run as one block (block CG, tensor-core products) and, for
    comparison, as 16 separate inversions.  "X+fp64" keeps the FP64 G beside the X
    one and predicts with it (grada_keep_fp64_G)."""
    import torch

    from graada3d_gb300 import regularization as reg
    from graada3d_gb300.inversion import GaussNewtonInversion

    prisms, obs, rho, ops = sweep_problem()
    inv = GaussNewtonInversion(prisms, obs, 0x012)
    inv.compute_G("fp64")
    d = inv.G_vec_mul(rho)
    dobs = d + 0.02 * np.abs(d) * np.random.default_rng(3).standard_normal(d.size)
    wd = reg.data_weights(dobs, [0.02, 0.02], [1e-3, 1e-2], obs.shape[0])
    inv.set_cross_gradient(False)
    inv.set_operators(ops)
    inv.set_dobs(dobs, wd)
    nm = inv.Nm
    lam = np.logspace(-3, 1, n_lambda)
    prm = dict(max_lambda=1e-1, n_lambda=1, rate=0.6, target=1.0, stag=0.02, cg_tol=1e-6,
               cg_factor=50, gn_iter=gn_iter, lp=[2, 2, 2, 2, 2], eps2=1e-9)
    args = (np.zeros(nm), np.full(nm, -1000.0), np.full(nm, 1000.0))
    out = {"case": "lambda-sweep-16", "cells": nm, "data": inv.Nd, "lambdas": n_lambda,
           "gn_iter_max": gn_iter}
    models = {}
    for st in storages:
        inv.compute_G(st.split("+")[0], keep_fp64=st.endswith("+fp64"))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        m, reps = inv.lambda_sweep(prm, lam, *args, fp64_refinement=(st != "fp64"))
        torch.cuda.synchronize()
        t = time.perf_counter() - t0
        models[st] = m
        r = {"block_s": t, "misfits": [round(x["final_misfit"], 4) for x in reps],
             "cg_iterations": int(sum(x["cg_iterations"] for x in reps)),
             "gn_iterations": [int(x["gn_iterations"]) for x in reps]}
        if st != "fp64" and "fp64" in models:
            rel = [float(np.linalg.norm(m[:, c] - models["fp64"][:, c]) /
                         max(np.linalg.norm(models["fp64"][:, c]), 1e-30)) for c in range(n_lambda)]
            r["model_rel_diff_vs_fp64_max"] = max(rel)
        if st != "fp64" and sequential:
            t0 = time.perf_counter()
            for c in range(n_lambda):
                inv.invert(dict(prm, max_lambda=float(lam[c])), *args, fp64_refinement=True)
            torch.cuda.synchronize()
            r["sequential_s"] = time.perf_counter() - t0
            r["speedup_block_vs_sequential"] = r["sequential_s"] / t
        out[st] = r
    inv.ctx.close()
    return out


def run_mf_profile():
    """Fixed small case for ncu captures of the matrix-free field sum and the
    FP64 assembly with two components: 32 x 32 x 32 = 32,768 cells, gz + Tzz at
    51 x 51 points (50 m over 20 km x 20 km); one FP64 assembly, one
    matrix-free G x."""
    from graada3d_gb300 import Fwd, mesh

    prisms = mesh.regular_mesh((0.0, 20000.0), 32, (0.0, 20000.0), 32, (0.0, 8000.0), 32)
    obs = mesh.observation_grid(51, 0.0, 20000.0, 51, 0.0, 20000.0, -50.0)
    f = Fwd(prisms, obs, 0x012)
    f.compute_G("fp64")
    x = np.ones(f.Nm)
    y64 = f.G_vec_mul(x)
    f.compute_G("matrix_free")
    y = f.G_vec_mul(x)
    assert np.abs(y - y64).max() <= 1e-12 * np.abs(y64).max()
    print(json.dumps({"case": "mf-profile", "pairs": f.N_obs * f.Nm}))
    f.ctx.close()


DYKES = [[2500, 3500, 1000, 9000, 500, 3500], [6000, 7000, 1000, 9000, 500, 3500]]


def refined_dyke_mesh(levels: int = 3):
    """32 x 32 x 16 cells over [0, 10 km]^2 x [0, 5 km], refined `levels` times at the
    leaves that cross the boundary of one of two +400 kg/m^3 dykes, with the
    reference's face-balance cascade and leaf order (mesh.Octree, Mesh::refinement
    + rearrange_id).  Three levels give 236,226 leaves."""
    from graada3d_gb300 import mesh

    o = mesh.Octree.regular((0.0, 10000.0), 32, (0.0, 10000.0), 32, (0.0, 5000.0), 16)
    for _ in range(levels):
        cells = o.leaves()
        mark = np.zeros(len(cells), bool)
        for b in DYKES:
            inter = ((cells[:, 0] < b[1]) & (cells[:, 1] > b[0]) & (cells[:, 2] < b[3]) &
                     (cells[:, 3] > b[2]) & (cells[:, 4] < b[5]) & (cells[:, 5] > b[4]))
            inside = ((cells[:, 0] >= b[0]) & (cells[:, 1] <= b[1]) & (cells[:, 2] >= b[2]) &
                      (cells[:, 3] <= b[3]) & (cells[:, 4] >= b[4]) & (cells[:, 5] <= b[5]))
            mark |= inter & ~inside
        o.refine(np.nonzero(mark)[0])
    return o.leaves()


def run_assembly_refined():
    """FP64 assembly of gz, Tzz, Txz, Tyz at 101 x 101 points 100 m above
    [0, 10 km]^2 on the adaptively refined 236,226-leaf dyke mesh and on the
    uniform 196,608-cell (64 x 64 x 48) mesh over the same domain: 3 warm-up and
    5 timed assemblies each (CUDA events).  On the refined mesh fewer cells
    share faces with a neighbour run in the assembly tiles."""
    import torch

    from graada3d_gb300 import Fwd, mesh

    obs = mesh.observation_grid(101, 0.0, 10000.0, 101, 0.0, 10000.0, -100.0)
    out = {"case": "assembly-refined", "points": obs.shape[0], "components": 4}
    for name, cells in (("refined", refined_dyke_mesh()),
                        ("uniform", mesh.regular_mesh((0.0, 10000.0), 64, (0.0, 10000.0), 64,
                                                      (0.0, 5000.0), 48))):
        f = Fwd(cells, obs, 0x072)
        stream = torch.cuda.ExternalStream(f.ctx.stream)
        for _ in range(3):
            f.compute_G("fp64")
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(5):
            f.compute_G("fp64")
        e1.record(stream)
        torch.cuda.synchronize()
        s = e0.elapsed_time(e1) / 5 * 1e-3
        out[name] = {"cells": f.Nm, "s": s, "G_entries_per_s": f.Nd * f.Nm / s,
                     "pairs_per_s": f.N_obs * f.Nm / s}
        f.ctx.close()
    return out


def run_operators_refined():
    """Rebuild of the regularisation operators after a refinement on the
    236,226-leaf dyke mesh: the face table from the leaves' geometry (host),
    then Ws/Wx/Wy/Wz with their transposes either built on the host and
    uploaded (grada_set_operator) or built on the device from the table
    (grada_build_operators).  Host wall clock, 1 warm-up + 3 timed runs each."""
    from graada3d_gb300 import mesh
    from graada3d_gb300 import regularization as reg
    from graada3d_gb300.inversion import GaussNewtonInversion

    cells = refined_dyke_mesh(3)
    obs = mesh.observation_grid(101, 0.0, 10000.0, 101, 0.0, 10000.0, -100.0)
    inv = GaussNewtonInversion(cells, obs, 0x072)

    def timed(fn, k=3):
        fn()
        t0 = time.perf_counter()
        for _ in range(k):
            out = fn()
        return (time.perf_counter() - t0) / k, out

    t_table, table = timed(lambda: reg.face_table(cells))
    t_host, ops = timed(lambda: reg.mesh_operators(cells, obs, 1.5, table=table))
    t_upload, _ = timed(lambda: inv.set_operators(ops))
    t_dev, _ = timed(lambda: inv.build_operators(table, 1.5))
    worst = 0.0
    for key in ("Ws", "Wx", "Wy", "Wz"):
        a, b = inv.get_operator(key), ops[key]
        worst = max(worst, float(np.max(np.abs(a.data - b.data) / np.abs(b.data))))
    out = {"case": "operators-refined", "cells": int(cells.shape[0]),
           "nnz_W": int(sum(ops[k].nnz for k in ("Ws", "Wx", "Wy", "Wz"))),
           "face_table_host_s": t_table, "W_host_build_s": t_host, "W_upload_s": t_upload,
           "W_device_build_s": t_dev, "max_rel_diff_device_vs_host": worst}
    inv.ctx.close()
    return out


def run_wavelet_case(rel: float = 5e-4):
    """The reference's method_id 2 at the 32 x 32 x 16-cell size (16,384 cells over
    [0, 10 km]^2 x [0, 5 km], gz + Tzz at 41 x 41 points 100 m above): FP64
    assembly plus Daubechies-4 compression of every row at the relative threshold
    of the reference's example configurations (5e-4), then G x and G^T y on the
    compressed rows against the dense FP64 ones (CUDA events, 20 runs each), the
    relative error of G x on the two-box model, and an L2 inversion to the
    target misfit on each."""
    import torch

    from graada3d_gb300 import mesh
    from graada3d_gb300 import regularization as reg
    from graada3d_gb300.inversion import GaussNewtonInversion

    c, prisms, obs, rho, rel_e, absf, ops, rng = inversion_problem("l2_16k")
    o = mesh.Octree.regular((0.0, 10000.0), 32, (0.0, 10000.0), 32, (0.0, 5000.0), 16)
    order = o.wavelet_order()
    import ctypes

    inv = GaussNewtonInversion(prisms, obs, c["mask"])
    lib, h = inv.ctx.lib, inv.ctx.handle
    stream = torch.cuda.ExternalStream(inv.ctx.stream)
    x = torch.from_numpy(rho).cuda()
    y = torch.empty(inv.ld, dtype=torch.float64, device="cuda")
    r = torch.zeros(inv.ld, dtype=torch.float64, device="cuda")
    r[:inv.Nd] = torch.from_numpy(np.random.default_rng(3).standard_normal(inv.Nd))
    g = torch.empty(inv.Nm, dtype=torch.float64, device="cuda")

    def products():
        out = []
        for fn, a, b in ((lib.grada_G_vec_mul_dev, x, y), (lib.grada_GT_vec_mul_dev, r, g)):
            for _ in range(3):
                inv.ctx.check(fn(h, ctypes.c_void_p(a.data_ptr()), ctypes.c_void_p(b.data_ptr())))
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(20):
                fn(h, ctypes.c_void_p(a.data_ptr()), ctypes.c_void_p(b.data_ptr()))
            e1.record(stream)
            torch.cuda.synchronize()
            out.append(e0.elapsed_time(e1) / 20)
        return out

    t0 = time.perf_counter()
    inv.compute_G("fp64")
    torch.cuda.synchronize()
    t_dense = time.perf_counter() - t0
    d_dense = inv.G_vec_mul(rho)
    ms_dense = products()
    dobs = d_dense + 0.02 * np.abs(d_dense) * np.random.default_rng(2).standard_normal(d_dense.size)
    wd = reg.data_weights(dobs, rel_e, absf, obs.shape[0])
    inv.set_cross_gradient(False)
    inv.set_operators(ops)
    inv.set_dobs(dobs, wd)
    nm = inv.Nm
    prm = dict(max_lambda=1e-1, n_lambda=30, rate=0.6, target=1.0, stag=0.02, cg_tol=1e-6,
               cg_factor=50, gn_iter=c["gn_iter"], lp=c["lp"], eps2=c["eps2"])
    args = (np.zeros(nm), np.full(nm, -1000.0), np.full(nm, 1000.0))
    t0 = time.perf_counter()
    m64, rep64 = inv.invert(prm, *args)
    t_inv64 = time.perf_counter() - t0
    t0 = time.perf_counter()
    inv.compute_G_wavelet(order, rel)
    torch.cuda.synchronize()
    t_wv = time.perf_counter() - t0
    n_dy, rp, cols, vals = inv.get_wavelet_G()
    d_wv = inv.G_vec_mul(rho)
    ms_wv = products()
    t0 = time.perf_counter()
    mw, repw = inv.invert(prm, *args)
    t_invw = time.perf_counter() - t0
    out = {"case": "wavelet", "cells": nm, "data": inv.Nd, "threshold": rel, "n_dy": n_dy,
           "kept": int(cols.size), "compression_ratio": inv.Nd * nm / cols.size,
           "dense_assemble_s": t_dense, "wavelet_assemble_compress_s": t_wv,
           "G_x_ms": {"dense_fp64": ms_dense[0], "wavelet": ms_wv[0]},
           "GT_y_ms": {"dense_fp64": ms_dense[1], "wavelet": ms_wv[1]},
           "G_x_rel_error": float(np.linalg.norm(d_wv - d_dense) / np.linalg.norm(d_dense)),
           "invert": {"dense_fp64": {"s": t_inv64, "misfit": rep64["final_misfit"],
                                     "trials": rep64["n_trials"]},
                      "wavelet": {"s": t_invw, "misfit": repw["final_misfit"],
                                  "trials": repw["n_trials"],
                                  "model_rel_diff": float(np.linalg.norm(mw - m64)
                                                          / np.linalg.norm(m64))}}}
    inv.ctx.close()
    return out


def run_wavelet_1m(variants=((5e-4, "fp64"), (5e-5, "fp64"), (5e-6, "fp64"), (5e-6, "fp32"))):
    """The wavelet-compressed G at the matrix-free case's size: 128 x 128 x 64 =
    1,048,576 cells over [0, 20 km]^2 x [0, 8 km], gz + Tzz at 201 x 201 points 50 m
    above (the FP64 G would be 678 GB).  Compression at the reference's example
    threshold (5e-4) and two lower ones (values in FP64, and in FP32 at 5e-6), in
    batches of points, never holding the dense G; then G x and G^T y on the
    compressed rows (CUDA events, 5 runs each) against one matrix-free FP64
    product of each, and the relative error of the compressed G x on a two-box
    model."""
    import ctypes

    import torch

    from graada3d_gb300 import mesh
    from graada3d_gb300.inversion import GaussNewtonInversion

    o = mesh.Octree.regular((0.0, 20000.0), 128, (0.0, 20000.0), 128, (0.0, 8000.0), 64)
    prisms = mesh.regular_mesh((0.0, 20000.0), 128, (0.0, 20000.0), 128, (0.0, 8000.0), 64)
    order = o.wavelet_order()
    obs = mesh.observation_grid(201, 0.0, 20000.0, 201, 0.0, 20000.0, -50.0)
    rho = mesh.set_boxes(prisms, [[5000, 9000, 6000, 12000, 1000, 3000, 300.0],
                                  [12000, 16000, 4000, 8000, 2000, 5000, -200.0]])
    inv = GaussNewtonInversion(prisms, obs, 0x012)
    lib, h = inv.ctx.lib, inv.ctx.handle
    stream = torch.cuda.ExternalStream(inv.ctx.stream)
    x = torch.from_numpy(rho).cuda()
    y = torch.empty(inv.ld, dtype=torch.float64, device="cuda")
    r = torch.zeros(inv.ld, dtype=torch.float64, device="cuda")
    r[:inv.Nd] = torch.from_numpy(np.random.default_rng(3).standard_normal(inv.Nd))
    g = torch.empty(inv.Nm, dtype=torch.float64, device="cuda")

    def timed(fn, a, b, k):
        inv.ctx.check(fn(h, ctypes.c_void_p(a.data_ptr()), ctypes.c_void_p(b.data_ptr())))
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(k):
            fn(h, ctypes.c_void_p(a.data_ptr()), ctypes.c_void_p(b.data_ptr()))
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / k * 1e-3

    out = {"case": "wavelet-1m", "cells": inv.Nm, "data": inv.Nd}
    inv.compute_G("matrix_free")
    out["matrix_free_s"] = {"G_x": timed(lib.grada_G_vec_mul_dev, x, y, 1),
                            "GT_y": timed(lib.grada_GT_vec_mul_dev, r, g, 1)}
    d_exact = y[:inv.Nd].cpu().numpy().copy()
    out["matrix_free_s"]["cg_iteration"] = sum(out["matrix_free_s"].values())
    for rel, values in variants:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        inv.compute_G_wavelet(order, rel, values)
        torch.cuda.synchronize()
        res = {"compress_s": time.perf_counter() - t0}
        nnz = ctypes.c_int64()
        n_dy = ctypes.c_int64()
        inv.ctx.check(lib.grada_get_wavelet_G(h, ctypes.byref(n_dy), ctypes.byref(nnz), None,
                                              None, None))
        res["kept"] = nnz.value
        res["compression_ratio"] = inv.Nd * n_dy.value / nnz.value
        res["stored_GB"] = nnz.value * (12 if values == "fp64" else 8) / 1e9
        res["G_x_s"] = timed(lib.grada_G_vec_mul_dev, x, y, 5)
        res["GT_y_s"] = timed(lib.grada_GT_vec_mul_dev, r, g, 5)
        res["cg_iteration_s"] = res["G_x_s"] + res["GT_y_s"]
        d_wv = y[:inv.Nd].cpu().numpy()
        res["G_x_rel_error"] = float(np.linalg.norm(d_wv - d_exact) / np.linalg.norm(d_exact))
        out[f"threshold_{rel:g}_{values}"] = res
    inv.ctx.close()
    return out


def run_wavelet_inversion_1m(rel: float = 5e-6):
    """The joint-constraint inversion of the matrix-free case's size on the
    wavelet-compressed G: 128 x 128 x 64 = 1,048,576 cells, gz + Tzz at 201 x 201
    points 50 m above, three seeded boxes, 2 % noise; L1 IRLS on Ws/Wx/Wy/Wz,
    cross-gradient coupling to a seeded Gaussian-correlated structure model
    (2 km correlation length) that is also the reference model.  The CG runs on
    the compressed rows (threshold 5e-6); one exact FP64 residual per
    Gauss-Newton iteration (the matrix-free evaluation) keeps the data term
    exact.  The data and the final misfit come from the FP64 field sum."""
    from scipy.ndimage import gaussian_filter

    import torch

    from graada3d_gb300 import mesh
    from graada3d_gb300 import regularization as reg
    from graada3d_gb300.inversion import GaussNewtonInversion

    n = (128, 128, 64)
    L = (20000.0, 20000.0, 8000.0)
    t0 = time.perf_counter()
    o = mesh.Octree.regular((0.0, L[0]), n[0], (0.0, L[1]), n[1], (0.0, L[2]), n[2])
    prisms = mesh.regular_mesh((0.0, L[0]), n[0], (0.0, L[1]), n[1], (0.0, L[2]), n[2])
    obs = mesh.observation_grid(201, 0.0, L[0], 201, 0.0, L[1], -50.0)
    rho = mesh.set_boxes(prisms, [[5000, 9000, 6000, 12000, 1000, 3000, 300.0],
                                  [12000, 16000, 4000, 8000, 2000, 5000, -200.0],
                                  [8000, 14000, 13000, 17000, 500, 1500, 150.0]])
    rng = np.random.default_rng(41)
    field = gaussian_filter(rng.standard_normal(n), sigma=[2000.0 / (L[a] / n[a]) for a in range(3)],
                            mode="wrap")
    m0s = (200.0 * field / np.abs(field).max()).ravel()  # leaf order: x outer, z inner
    ops = reg.regular_mesh_operators(n, prisms, obs, 1.5)
    ops.update(reg.cross_gradient_operators(n, prisms, m0s, ops))
    t_host = time.perf_counter() - t0

    inv = GaussNewtonInversion(prisms, obs, 0x012)
    t0 = time.perf_counter()
    d = inv.forward_field(rho).T.ravel()
    t_exact = time.perf_counter() - t0
    dobs = d + 0.02 * np.abs(d) * np.random.default_rng(42).standard_normal(d.size)
    wd = reg.data_weights(dobs, [0.02, 0.02], [1e-3, 1e-2], obs.shape[0])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    inv.compute_G_wavelet(o.wavelet_order(), rel)
    torch.cuda.synchronize()
    t_comp = time.perf_counter() - t0
    inv.set_operators(ops)
    inv.set_cross_gradient(True, 1.0)
    inv.set_dobs(dobs, wd)
    prm = dict(max_lambda=1e-1, n_lambda=10, rate=0.6, target=1.0, stag=0.02, cg_tol=1e-6,
               cg_factor=50, gn_iter=3, lp=[1, 1, 1, 1, 2], eps2=1e-10)
    nm = inv.Nm
    t0 = time.perf_counter()
    m, rep = inv.invert(prm, np.zeros(nm), np.full(nm, -1000.0), np.full(nm, 1000.0), m0s,
                        fp64_refinement=True)
    t_inv = time.perf_counter() - t0
    d_fin = inv.forward_field(m).T.ravel()
    exact_misfit = float(np.sqrt(np.mean((wd * (dobs - d_fin)) ** 2)))
    out = {"case": "wavelet-inversion-1m", "cells": nm, "data": inv.Nd, "threshold": rel,
           "host_setup_s": t_host, "exact_data_s": t_exact, "compress_s": t_comp,
           "invert_s": t_inv, "gn_iterations": rep["gn_iterations"], "trials": rep["n_trials"],
           "cg_iterations": int(rep["cg_iterations"]),
           "ms_per_cg_iteration": 1e3 * t_inv / max(1, rep["cg_iterations"]),
           "fp64_residuals": int(rep["fp64_refinements"]),
           "gn_misfits": [float(v) for v in inv.iterations()[:, 2]],
           "final_misfit_reported": rep["final_misfit"], "final_misfit_exact_fp64": exact_misfit,
           "matrix_free_cg_iteration_s_for_comparison": 29.4}
    inv.ctx.close()
    return out


def run_cg_tall(storages=("fp64", "fp32", "bf16")):
    """The CG loop on a tall G with the rows of the refined dyke inversion: gz,
    Tzz, Txz, Tyz at 101 x 101 points 100 m above [0, 10 km]^2 (40,804 rows) over
    40 x 40 x 20 = 32,000 cells to 5 km depth (G 2.6 GB in bf16, 5.2 GB in
    FP32, 10.4 GB in FP64: small enough for ncu, the same row count as the
    refined inversion).  Three solves of 100 CG iterations each (tolerance 0,
    so every solve runs to its cap) on an L2 problem; the loop's host time per
    iteration (grada_cg_loop_time) against two reads of G at the copy rate."""
    import torch

    from graada3d_gb300 import mesh
    from graada3d_gb300 import regularization as reg
    from graada3d_gb300.inversion import GaussNewtonInversion

    n = (40, 40, 20)
    prisms = mesh.regular_mesh((0.0, 10000.0), n[0], (0.0, 10000.0), n[1], (0.0, 5000.0), n[2])
    obs = mesh.observation_grid(101, 0.0, 10000.0, 101, 0.0, 10000.0, -100.0)
    rng = np.random.default_rng(11)
    rho = mesh.set_boxes(prisms, [[2500, 3500, 1000, 9000, 500, 3500, 400.0],
                                  [6000, 7000, 1000, 9000, 500, 3500, 400.0]])
    inv = GaussNewtonInversion(prisms, obs, 0x072)
    ops = reg.regular_mesh_operators(n, prisms, obs, 1.5)
    peak = _peak_gbs()
    out = {"case": "cg-tall", "rows": inv.Nd, "cells": inv.Nm, "solves": 3, "iterations_per_solve": 100}
    d = None
    for st in storages:
        inv.compute_G(st)
        if d is None:
            d = inv.G_vec_mul(rho)
            dobs = d + 0.02 * np.abs(d) * rng.standard_normal(d.size)
            wd = reg.data_weights(dobs, [0.02] * 4, [1e-3, 1e-2, 1e-2, 1e-2], obs.shape[0])
            inv.set_cross_gradient(False)
            inv.set_operators(ops)
            inv.set_dobs(dobs, wd)
        nm = inv.Nm
        mk, mref, P = np.zeros(nm), np.zeros(nm), np.ones(nm)
        inv.solve_cg(0.0, 20, 1e-3, mk, mref, P)  # warm-up (graph built)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        base = inv.cg_loop_time()
        for _ in range(3):
            inv.solve_cg(0.0, 100, 1e-3, mk, mref, P)
        wall = time.perf_counter() - t0
        loop_s, _, iters = (a - b for a, b in zip(inv.cg_loop_time(), base))
        bpe = {"fp64": 8, "fp32": 4, "bf16": 2, "fp16": 2}[st]
        gbytes = 2.0 * inv.ld * nm * bpe
        r = {"iterations": int(iters), "loop_ms_per_iteration": 1e3 * loop_s / max(1, iters),
             "solve_ms_per_iteration": 1e3 * wall / max(1, iters),
             "G_bytes_per_iteration": gbytes}
        r["loop_TBps"] = gbytes / (loop_s / max(1, iters)) / 1e12
        if peak:
            r["loop_frac_of_hbm"] = r["loop_TBps"] * 1e3 / peak
        out[st] = r
    inv.ctx.close()
    return out


def run_profile_case(args):
    """The fixed small case profiles are taken on: 1,024 points (32 x 32 at
    50 m height over 20 km x 20 km) x 4,096 cells (16 x 16 x 16 over the
    benchmark domain), nine components, one FP64 assembly, then the dense
    products on it."""
    from graada3d_gb300 import Fwd, mesh

    prisms = mesh.regular_mesh((0.0, 20000.0), 16, (0.0, 20000.0), 16, (0.0, 8000.0), 16)
    obs = mesh.observation_grid(32, 0.0, 20000.0, 32, 0.0, 20000.0, -50.0)
    f = Fwd(prisms, obs, MASK)
    t0 = time.perf_counter()
    f.compute_G("fp64")
    dt = time.perf_counter() - t0
    x = np.ones(f.Nm)
    y = f.G_vec_mul(x)
    z = f.GT_vec_mul(y)
    assert np.isfinite(z).all()
    print(json.dumps({"case": "profile", "pairs": f.N_obs * f.Nm, "entries": f.Nd * f.Nm,
                      "assemble_s": dt}))
    f.ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--case", default="bench", choices=["bench", "profile", "inversion-l2-16k",
                                                         "inversion-l1-196k", "inversion-l1-refined",
                                                         "inversion-l1-refined-chi2",
                                                         "matrix-free-1m",
                                                         "gemv", "batched-64", "block-gemm",
                                                         "lambda-sweep-16", "block-gemm-profile",
                                                         "mf-profile", "assembly-refined", "cg-tall",
                                                         "operators-refined", "wavelet",
                                                         "wavelet-1m", "wavelet-inversion-1m"])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--ref-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-inversion", action="store_true")
    ap.add_argument("--no-refined-inversion", action="store_true",
                    help="skip the refined-mesh L1 inversion (about five minutes)")
    ap.add_argument("--no-block", action="store_true")
    ap.add_argument("--sweep-storages", default="fp64,fp32,bf16,fp32+fp64,bf16+fp64")
    ap.add_argument("--no-sequential", action="store_true")
    ap.add_argument("--storages", default=None,
                    help="G storages of an --case inversion-* run, e.g. fp64,fp32+fp64")
    args = ap.parse_args()
    if args.case == "profile":
        run_profile_case(args)
    elif args.case == "block-gemm":
        print(json.dumps(run_block_gemm_case()))
    elif args.case == "cg-tall":
        st = tuple(args.storages.split(",")) if args.storages else ("fp64", "fp32", "bf16")
        print(json.dumps(run_cg_tall(st)))
    elif args.case == "assembly-refined":
        print(json.dumps(run_assembly_refined()))
    elif args.case == "operators-refined":
        print(json.dumps(run_operators_refined()))
    elif args.case == "wavelet":
        print(json.dumps(run_wavelet_case()))
    elif args.case == "wavelet-1m":
        print(json.dumps(run_wavelet_1m()))
    elif args.case == "wavelet-inversion-1m":
        print(json.dumps(run_wavelet_inversion_1m()))
    elif args.case == "mf-profile":
        run_mf_profile()
    elif args.case == "block-gemm-profile":
        run_block_gemm_profile()
    elif args.case == "lambda-sweep-16":
        print(json.dumps(run_lambda_sweep_16(storages=tuple(args.sweep_storages.split(",")),
                                        sequential=not args.no_sequential)))
    elif args.case == "batched-64":
        res = run_batched_64()
        if int(os.environ.get("RANK", "0")) == 0:
            print(json.dumps(res))
    elif args.case == "gemv":
        print(json.dumps(run_gemv_case()))
    elif args.case == "matrix-free-1m":
        print(json.dumps(run_matrix_free_1m()))
    elif args.case.startswith("inversion-"):
        name = args.case.split("-", 1)[1].replace("-", "_")
        st = tuple(args.storages.split(",")) if args.storages else None
        print(json.dumps(run_inversion(name, st) if st else run_inversion(name)))
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
