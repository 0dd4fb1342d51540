"""Served stream of channel and convection solves with continuous batching on one GPU.

Requests arrive as a Poisson process (default mean rate 50/s).  Each asks for an HD channel or
a BOUSS convection solve on a grid drawn from nx, ny in {64, 128, 256} and nz (physical) in
{65, 129, 257} (+25 FC-Gram points), for a step count drawn uniformly from [100, 2000], with
the parameters and seeded initial fields of the channel case (RK2, dt 1e-4, nu 1e-3, z in
[0, 2], Poiseuille + perturbation) or the convection case (RK2, dt 1e-5, nu = kappa = 1e-4,
z in [0, 1], theta' noise, v = 0).

The server keeps the state of every admitted simulation resident in HBM and admits waiting
requests in arrival order while the device memory they need fits the budget.  Each admitted
simulation runs on its own plan stream from a captured one-step CUDA graph, launched in chunks of
steps whenever its previous chunk has finished, so the kernels of different simulations overlap
on the device and new requests start while others are running (continuous batching).  Among the
admitted simulations, chunks go to those with the least remaining work (grid points x stages
left) until the running set holds `fill_points` grid points, so short requests are not held
behind long ones (policy "srpt"; policy "all" runs every admitted simulation).  A simulation's
memory is released as soon as its result is out.  Time-to-result of a request is its completion
time minus its arrival time.

    python -m specter_gb300.serve --requests 32 --rate 50 --budget-gb 120

Prints one JSON line: solves/s, p50 / p99 time-to-result, and the plain-FP64 sequential
comparison (per-grid FP64 step times measured here, times the requests' step counts).
"""
from __future__ import annotations

import argparse
import collections
import json
import time
from dataclasses import dataclass, field

import numpy as np

GRID_XY = (64, 128, 256)
GRID_Z = (65, 129, 257)
KINDS = ("HD", "BOUSS")


@dataclass
class Request:
    rid: int
    arrival: float
    kind: str
    nx: int
    ny: int
    nzp: int
    steps: int
    seed: int
    admitted: float = -1.0
    done: float = -1.0
    result: list = field(default_factory=list)


def draw_requests(n, rate=50.0, seed=20261203, steps=(100, 2000), grid_xy=GRID_XY, grid_z=GRID_Z, kinds=KINDS):
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    for i in range(n):
        t += float(rng.exponential(1.0 / rate))
        out.append(Request(i, t, str(rng.choice(kinds)), int(rng.choice(grid_xy)), int(rng.choice(grid_xy)),
                           int(rng.choice(grid_z)), int(rng.integers(steps[0], steps[1] + 1)), int(seed) * 1000 + i))
    return out


def case(req):
    if req.kind == "HD":
        return dict(solver="HD", Lz=2.0, ord=2, dt=1e-4, nu=1e-3, kappa=0.0)
    return dict(solver="BOUSS", Lz=1.0, ord=2, dt=1e-5, nu=1e-4, kappa=1e-4)


def make(api, initial, req, precision):
    c = case(req)
    plan = api.Plan((req.nx, req.ny, req.nzp + 25), (0, 0, 25), (0, 0, 5), (1.0, 1.0, c["Lz"]), precision=precision)
    bouss = c["solver"] == "BOUSS"
    s = api.Solver(plan, api.BOUSS if bouss else api.HD, ord=c["ord"], dt=c["dt"], nu=c["nu"], kappa=c["kappa"])
    if bouss:
        th = initial.convection_theta(plan, seed=req.seed, amp=1e-3)
        s.th.copy_from(initial.to_spectral(plan, [th])[0])
        for f in (s.vx, s.vy, s.vz, s.pr):
            f.zero()
    else:
        v = initial.channel_velocity(plan, seed=req.seed, amp=0.05, kmax=8)
        for f, sp in zip((s.vx, s.vy, s.vz), initial.to_spectral(plan, v)):
            f.copy_from(sp)
        s.pr.zero()
    return plan, s


def field_bytes(req, precision):
    es = 16 if precision == 0 else 8
    ldx = ((req.nx // 2 + 1) + 7) // 8 * 8
    return ldx * req.ny * (req.nzp + 25) * es


class Server:
    """Continuous-batching request loop (see the module docstring)."""

    def __init__(self, budget_bytes, chunk=25, precision=1, keep_results=False, autotune=False, policy="srpt",
                 fill_points=16_000_000):
        from specter_gb300 import api, initial
        self.api, self.initial = api, initial
        self.budget = int(budget_bytes)
        self.chunk = int(chunk)
        self.precision = precision
        self.keep = keep_results
        self.autotune = autotune
        self.policy = policy
        self.fill_points = fill_points
        self.per_field = {}  # solver kind -> device bytes per field-sized unit, measured

    def _estimate(self, req):
        return int(self.per_field.get(req.kind, 48.0) * field_bytes(req, self.precision))

    def _start(self, req, now):
        plan, s = make(self.api, self.initial, req, self.precision)
        if self.autotune:
            s.autotune()
        g = self.api.Graph([s], nsteps=1)
        used = self.api.solver_memory(s)
        self.per_field[req.kind] = max(self.per_field.get(req.kind, 0.0), used / field_bytes(req, self.precision))
        req.admitted = now
        return {"req": req, "plan": plan, "solver": s, "graph": g, "remaining": req.steps, "inflight": 0,
                "bytes": used, "points": req.nx * req.ny * req.nzp}

    def _running_set(self, active):
        if self.policy == "all":
            return active
        chosen, pts = [], 0
        for e in sorted(active, key=lambda e: e["remaining"] * e["points"]):
            if chosen and pts + e["points"] > self.fill_points:
                break
            chosen.append(e)
            pts += e["points"]
        return chosen

    def _launch(self, e):
        k = min(self.chunk, e["remaining"])
        for _ in range(k):
            e["graph"].launch()
        e["inflight"] = k

    def run(self, requests):
        pending = collections.deque(sorted(requests, key=lambda r: r.arrival))
        waiting, active = collections.deque(), []
        used, peak_used, peak_active, peak_running = 0, 0, 0, 0
        t0 = time.perf_counter()
        while pending or waiting or active:
            now = time.perf_counter() - t0
            while pending and pending[0].arrival <= now:
                waiting.append(pending.popleft())
            while waiting and (used + self._estimate(waiting[0]) <= self.budget or not active):
                e = self._start(waiting.popleft(), time.perf_counter() - t0)
                used += e["bytes"]
                active.append(e)
            peak_used, peak_active = max(peak_used, used), max(peak_active, len(active))
            progressed = False
            for e in list(active):
                if e["inflight"] and e["graph"].done():
                    progressed = True
                    e["remaining"] -= e["inflight"]
                    e["inflight"] = 0
                    if e["remaining"] == 0:
                        req = e["req"]
                        req.done = time.perf_counter() - t0
                        e["solver"].check()
                        if self.keep:
                            req.result = [f.download() for f in e["solver"].state]
                        e["graph"].close()
                        e["solver"].close()
                        e["plan"].close()
                        used -= e["bytes"]
                        active.remove(e)
            running = self._running_set(active)
            peak_running = max(peak_running, len(running))
            for e in running:
                if not e["inflight"]:
                    self._launch(e)
                    progressed = True
            if not progressed:
                time.sleep(2e-4)
        makespan = time.perf_counter() - t0
        ttr = np.array([r.done - r.arrival for r in requests])
        return {"requests": len(requests), "makespan_s": round(makespan, 3),
                "solves_per_s": round(len(requests) / makespan, 4),
                "ttr_p50_s": round(float(np.percentile(ttr, 50)), 3), "ttr_p99_s": round(float(np.percentile(ttr, 99)), 3),
                "ttr_max_s": round(float(ttr.max()), 3), "ttr_mean_s": round(float(ttr.mean()), 3),
                "peak_active": peak_active, "peak_running": peak_running, "policy": self.policy,
                "peak_bytes": int(peak_used), "budget_bytes": self.budget}


def sequential_fp64_estimate(requests, probe_steps=3):
    """Time of running the requests one after another through the plain FP64 form: the FP64 step
    time of each distinct (kind, grid) is measured here (probe_steps after one warm-up step) and
    multiplied by the requests' step counts."""
    from specter_gb300 import api, initial
    per_step = {}
    for r in requests:
        key = (r.kind, r.nx, r.ny, r.nzp)
        if key in per_step:
            continue
        plan, s = make(api, initial, r, api.FP64)
        s.step(1)
        plan.synchronize()
        t0 = time.perf_counter()
        s.step(probe_steps)
        plan.synchronize()
        per_step[key] = (time.perf_counter() - t0) / probe_steps
        s.close()
        plan.close()
    total = sum(per_step[(r.kind, r.nx, r.ny, r.nzp)] * r.steps for r in requests)
    return total, per_step


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--requests", type=int, default=32)
    ap.add_argument("--rate", type=float, default=50.0)
    ap.add_argument("--seed", type=int, default=20261203)
    ap.add_argument("--budget-gb", type=float, default=None, help="default: 80%% of the free device memory")
    ap.add_argument("--chunk", type=int, default=25)
    ap.add_argument("--max-steps", type=int, default=2000)
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--policy", default="srpt", choices=("srpt", "all"))
    ap.add_argument("--fill-points", type=float, default=16e6)
    args = ap.parse_args(argv)
    from specter_gb300 import api
    free, total = api.device_memory()
    budget = int(args.budget_gb * 1e9) if args.budget_gb else int(0.8 * free)
    reqs = draw_requests(args.requests, args.rate, args.seed, steps=(100, args.max_steps))
    srv = Server(budget, chunk=args.chunk, policy=args.policy, fill_points=int(args.fill_points))
    res = srv.run(reqs)
    res.update({"rate_per_s": args.rate, "seed": args.seed, "precision": "fp32-bulk", "chunk_steps": args.chunk,
                "step_range": [100, args.max_steps]})
    if not args.no_fp64:
        t_seq, per_step = sequential_fp64_estimate(reqs)
        res["sequential_fp64"] = {"seconds": round(t_seq, 2), "solves_per_s": round(len(reqs) / t_seq, 5),
                                  "how": "measured FP64 step time per grid x requested steps"}
        res["speedup_vs_sequential_fp64"] = round(res["solves_per_s"] / (len(reqs) / t_seq), 2)
    print(json.dumps(res), flush=True)
    return res


if __name__ == "__main__":
    main()
