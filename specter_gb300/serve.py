"""Served stream of channel and convection solves with continuous batching on one GPU.

Requests arrive as a Poisson process (default mean rate 50/s).  Each asks for an HD channel or
a BOUSS convection solve on a grid drawn from nx, ny in {64, 128, 256} and nz (physical) in
{65, 129, 257} (+25 FC-Gram points), for a step count drawn uniformly from [100, 2000], with
the parameters and seeded initial fields of the channel case (RK2, dt 1e-4, nu 1e-3, z in
[0, 2], Poiseuille + perturbation) or the convection case (RK2, dt 1e-5, nu = kappa = 1e-4,
z in [0, 1], theta' noise, v = 0).

The server keeps the state of every admitted simulation resident in HBM and admits waiting
requests in arrival order while the device memory they need fits the budget.  Setting a
simulation up (plan, state allocation, initial field, graph capture) runs on a setup thread, so
arrivals never stall the dispatch loop that keeps the running simulations fed.  Each admitted
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
comparison: a seeded sample of the requests run to completion one after another through the
plain FP64 form (measured), and the per-grid FP64 step times times all requests' step counts.
"""
from __future__ import annotations

import argparse
import collections
import json
import queue
import threading
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
        t_setup = time.perf_counter()
        plan, s = make(self.api, self.initial, req, self.precision)
        if self.autotune:
            s.autotune()
        g = self.api.Graph([s], nsteps=1)
        used = self.api.solver_memory(s)
        self.per_field[req.kind] = max(self.per_field.get(req.kind, 0.0), used / field_bytes(req, self.precision))
        req.admitted = now
        return {"req": req, "plan": plan, "solver": s, "graph": g, "remaining": req.steps, "inflight": 0,
                "bytes": used, "points": req.nx * req.ny * req.nzp, "setup_s": time.perf_counter() - t_setup}

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

    def _setup_worker(self, todo, ready, t0):
        """Setup thread: builds the admitted requests' simulations in admission order."""
        while True:
            req = todo.get()
            if req is None:
                return
            try:
                ready.put(self._start(req, time.perf_counter() - t0))
            except Exception as exc:  # re-raised by the dispatch loop
                ready.put({"req": req, "error": exc})

    def run(self, requests):
        pending = collections.deque(sorted(requests, key=lambda r: r.arrival))
        waiting, active = collections.deque(), []
        todo, ready = queue.Queue(), queue.Queue()
        used, peak_used, peak_active, peak_running, in_setup = 0, 0, 0, 0, 0
        reserved = {}  # request id -> bytes reserved at admission, until its setup reports
        setup_s = []
        t0 = time.perf_counter()
        worker = threading.Thread(target=self._setup_worker, args=(todo, ready, t0), daemon=True)
        worker.start()
        try:
            while pending or waiting or active or in_setup:
                now = time.perf_counter() - t0
                while pending and pending[0].arrival <= now:
                    waiting.append(pending.popleft())
                # admission by memory budget: reserve the estimate, build on the setup thread
                while waiting and (used + self._estimate(waiting[0]) <= self.budget or not (active or in_setup)):
                    req = waiting.popleft()
                    reserved[req.rid] = self._estimate(req)
                    used += reserved[req.rid]
                    in_setup += 1
                    todo.put(req)
                progressed = False
                while True:
                    try:
                        e = ready.get_nowait()
                    except queue.Empty:
                        break
                    in_setup -= 1
                    if "error" in e:
                        raise e["error"]
                    used += e["bytes"] - reserved.pop(e["req"].rid)
                    setup_s.append(e["setup_s"])
                    active.append(e)
                    progressed = True
                peak_used, peak_active = max(peak_used, used), max(peak_active, len(active))
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
        finally:
            todo.put(None)
            worker.join()
        makespan = time.perf_counter() - t0
        ttr = np.array([r.done - r.arrival for r in requests])
        return {"requests": len(requests), "makespan_s": round(makespan, 3),
                "solves_per_s": round(len(requests) / makespan, 4),
                "ttr_p50_s": round(float(np.percentile(ttr, 50)), 3), "ttr_p99_s": round(float(np.percentile(ttr, 99)), 3),
                "ttr_max_s": round(float(ttr.max()), 3), "ttr_mean_s": round(float(ttr.mean()), 3),
                "setup_s_mean": round(float(np.mean(setup_s)), 3) if setup_s else None,
                "peak_active": peak_active, "peak_running": peak_running, "policy": self.policy,
                "peak_bytes": int(peak_used), "budget_bytes": self.budget}


def sequential_fp64_sample(requests, k, seed=1):
    """A seeded sample of k requests run one after another to completion through the plain FP64
    form (measured, not estimated): (seconds, the sampled request indices)."""
    from specter_gb300 import api, initial
    rng = np.random.default_rng(seed)
    idx = sorted(rng.choice(len(requests), size=min(k, len(requests)), replace=False).tolist())
    total = 0.0
    for i in idx:
        r = requests[i]
        plan, s = make(api, initial, r, api.FP64)
        plan.synchronize()
        t0 = time.perf_counter()
        s.step(r.steps)
        plan.synchronize()
        total += time.perf_counter() - t0
        s.check()
        s.close()
        plan.close()
    return total, idx


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
    ap.add_argument("--seq-sample", type=int, default=4, help="requests run sequentially in plain FP64 (0: estimate only)")
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
        t_est, per_step = sequential_fp64_estimate(reqs)
        res["sequential_fp64_estimate"] = {"seconds": round(t_est, 2), "solves_per_s": round(len(reqs) / t_est, 5),
                                           "how": "measured FP64 step time per grid x requested steps"}
        if args.seq_sample > 0:
            t_run, idx = sequential_fp64_sample(reqs, args.seq_sample)
            est_sample = sum(per_step[(reqs[i].kind, reqs[i].nx, reqs[i].ny, reqs[i].nzp)] * reqs[i].steps for i in idx)
            res["sequential_fp64"] = {"sample_requests": idx, "seconds": round(t_run, 2),
                                      "solves_per_s": round(len(idx) / t_run, 5),
                                      "estimate_seconds_same_sample": round(est_sample, 2),
                                      "how": "the sampled requests run to completion one after another, plain FP64"}
            res["speedup_vs_sequential_fp64"] = round(res["solves_per_s"] / (len(idx) / t_run), 2)
        res["speedup_vs_sequential_fp64_estimate"] = round(res["solves_per_s"] / (len(reqs) / t_est), 2)
    print(json.dumps(res), flush=True)
    return res


if __name__ == "__main__":
    main()
