"""Batched ensemble of independent HD channel instances on one GPU.

Each instance is its own plan and solver (uneven grids are allowed).  Two ways to run them:

* batch (default): ``api.Batch`` records one RK step of every FP32-bulk solver and replays it
  as batched launches -- the i-th kernel of every instance's step runs as one launch per FFT
  length class over the tiles of all the instances in that class -- captured as one CUDA graph
  per RK step (a few dozen launches a step for the whole ensemble);
* graph: the solvers are autotuned per plan and one RK step of all of them is captured as one
  CUDA graph whose branches are the instances' own kernel chains (several hundred kernels).

    python -m specter_gb300.ensemble --instances 64 --steps 200 [--mode graph] [--seq-sample K]

Instance draw (seeded, numpy PCG64): nx, ny in {32, 48, 64, 96}, nz (physical) in {33, 65, 97}
(+25 FC-Gram points), z in [0, 2], nu log-uniform in [2e-4, 2e-3], RK2, dt = 1e-4, and the
channel initial field of specter_gb300.initial (Poiseuille + solenoidal perturbation, |k| <= 8,
amplitude 0.05) with its own seed.  The comparison runs the same instances one after another
through the plain FP64 form (no graph), optionally on a sample of them.  Prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import math
import time

import numpy as np

GRID_XY = (32, 48, 64, 96)
GRID_Z = (33, 65, 97)


def draw(n, seed):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        out.append(dict(nx=int(rng.choice(GRID_XY)), ny=int(rng.choice(GRID_XY)), nzp=int(rng.choice(GRID_Z)),
                        nu=float(math.exp(rng.uniform(math.log(2e-4), math.log(2e-3)))), seed=int(seed) * 1000 + i,
                        Lz=2.0, dt=1e-4, ord=2, amp=0.05, kmax=8))
    return out


def make(api, initial, inst, precision):
    plan = api.Plan((inst["nx"], inst["ny"], inst["nzp"] + 25), (0, 0, 25), (0, 0, 5), (1.0, 1.0, inst["Lz"]),
                    precision=precision)
    s = api.Solver(plan, api.HD, ord=inst["ord"], dt=inst["dt"], nu=inst["nu"])
    v = initial.channel_velocity(plan, seed=inst["seed"], amp=inst["amp"], kmax=inst["kmax"])
    for f, sp in zip((s.vx, s.vy, s.vz), initial.to_spectral(plan, v)):
        f.copy_from(sp)
    s.pr.zero()
    plan.synchronize()
    return plan, s


def rel_l2(a, b):
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / nb) if nb > 0 else float(np.linalg.norm(a))


def run(instances=64, steps=200, seed=20261203, seq_sample=None, autotune=True, graph_steps=1, mode="batch"):
    from specter_gb300 import api, initial
    insts = draw(instances, seed)
    t0 = time.perf_counter()
    built = [make(api, initial, x, api.FP32) for x in insts]
    t_build = time.perf_counter() - t0
    caps = []
    t0 = time.perf_counter()
    solvers = [s for _, s in built]
    if mode == "batch":
        runner = api.Batch(solvers)
        kernels = runner.kernels
    else:
        for _, s in built:
            caps.append(s.autotune() if autotune else None)
        if steps % graph_steps:
            raise ValueError("steps must be a multiple of graph_steps")
        runner = api.Graph(solvers, nsteps=graph_steps)
        kernels = runner.kernels // graph_steps
    t_prep = time.perf_counter() - t0
    for p, _ in built:
        p.synchronize()
    t0 = time.perf_counter()
    if mode == "batch":
        runner.step(steps)
    else:
        for _ in range(steps // graph_steps):
            runner.launch()
    runner.synchronize()
    t_run = time.perf_counter() - t0
    for s in solvers:
        s.check()
    solves_per_s = instances / t_run
    pts = sum(x["nx"] * x["ny"] * x["nzp"] * x["ord"] for x in insts) * steps
    result = {"instances": instances, "steps": steps, "seed": seed, "precision": "fp32-bulk", "mode": mode,
              "kernels_per_step": kernels, "seconds": round(t_run, 4),
              "solves_per_s": round(solves_per_s, 3), "mpts_stages_per_s": round(pts / t_run / 1e6, 2),
              "build_s": round(t_build, 2), "prepare_s": round(t_prep, 2), "caps": caps or None}
    graph = runner
    # sequential plain FP64 on a sample (first k instances): time per solve, error of the ensemble
    k = instances if seq_sample is None else min(seq_sample, instances)
    if k > 0:
        t_seq, errs = 0.0, []
        for i in range(k):
            p64, s64 = make(api, initial, insts[i], api.FP64)
            t0 = time.perf_counter()
            s64.step(steps)
            p64.synchronize()
            t_seq += time.perf_counter() - t0
            s64.check()
            s32 = solvers[i]
            # relative L2 on the physical grid (c2r of both states in FP64, rows z < nzp)
            fc, fr = p64.field(api.COMPLEX), p64.field(api.REAL)

            def phys(data):
                fc.upload(np.ascontiguousarray(data, dtype=np.complex128))
                api.fftp3d_complex_to_real(p64, fc, fr)
                return fr.download()[: p64.nzp]

            e = max(rel_l2(phys(a.download()), phys(b.download()))
                    for a, b in zip((s32.vx, s32.vy, s32.vz), (s64.vx, s64.vy, s64.vz)))
            errs.append(e)
            fc.close()
            fr.close()
            s64.close()
            p64.close()
        seq_solves = k / t_seq
        result.update({"sequential_fp64": {"sample": k, "seconds": round(t_seq, 3),
                                           "solves_per_s": round(seq_solves, 4)},
                       "speedup_vs_sequential_fp64": round(solves_per_s / seq_solves, 2),
                       "fp32_vs_fp64_rel_l2_max": max(errs), "fp32_vs_fp64_rel_l2_median": float(np.median(errs)),
                       "error_metric": "relative L2 of vx, vy, vz on the physical grid (max over components)"})
    graph.close()
    return result, insts, built


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--instances", type=int, default=64)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--seed", type=int, default=20261203)
    ap.add_argument("--seq-sample", type=int, default=None,
                    help="instances run through sequential FP64 (default: all of them)")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--graph-steps", type=int, default=1, help="RK steps captured per graph launch (mode graph)")
    ap.add_argument("--mode", default="batch", choices=("batch", "graph"))
    args = ap.parse_args(argv)
    res, _, _ = run(args.instances, args.steps, args.seed, args.seq_sample, not args.no_autotune, args.graph_steps,
                    args.mode)
    print(json.dumps(res), flush=True)
    return res


if __name__ == "__main__":
    main()
