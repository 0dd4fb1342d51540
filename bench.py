"""Benchmark of SPECTER's per-RK-stage hot path on GB300.

Workload (one "step" = one RK2 step = 2 RK stages over the whole grid): the Boussinesq
Rayleigh-Benard case, nx = ny = 512 (periodic, Lx = Ly = 2*pi), nz = 513 physical points
(+ Cz = 25 FC-Gram continuation points, NZ = 538) on z in [0, 1], d = 5, Pr = 1,
nu = kappa = 1e-4, RK order 2, dt = 1e-5; seeded synthetic initial field
(theta' = 1e-3 * U(-1,1) * z(1 - z), v = 0).  Each field is 566 MB (FP32) or 1.13 GB (FP64
words), far larger than the 129 MB L2, so no L2 flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--form nl32|fp32|fp64] [--impl reference]

The headline form (--form nl32, the default) is the precision form that keeps within 1e-5
relative L2 of plain FP64 after 1000 steps: the nonlinear term in FP32, the state and every
operation that carries it through a z transform in float-float (FP32 pairs).  Beside it the line
reports plain FP64 (`fp64`), FP32-bulk (`fp32_bulk`, faster, but outside the 1e-5 gate) and
`precision`: each form against plain FP64 after 10 steps in this run, with the committed
1000-step record of profiles/precision_bouss512.md.

Prints one JSON line (rank 0).  `value` is grid points x RK stages per second with the state
resident in HBM; `e2e` is the same metric through the C ABI with the state uploaded from
pinned host memory and downloaded back every step (steps / total time).  `--impl reference`
times the FP64 CPU restatement of the reference algorithm (the oracle; the Fortran reference
cannot be built here) on a bounded sample of the same workload on the host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "RK-stage Mpts/s FP32-bulk vs FP64 at ≤1e-5 rel err; ensemble solves/s, p99 lat"
UNIT = "Mpts*stages/s"
CFG = dict(nx=512, ny=512, nzp=513, cz=25, oz=5, Lx=1.0, Ly=1.0, Lz=1.0,
           solver="BOUSS", ord=2, dt=1e-5, nu=1e-4, kappa=1e-4, seed=20261203)
# CPU sample: same z grid and physics, 128 x 128 in (x, y), one RK2 step per timed step
CPU_SAMPLE = dict(CFG, nx=128, ny=128)


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu, self.rows, self.proc = gpu, [], None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) == 7:
                self.rows.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def build_solver(api, initial, cfg, precision, fused=True, nl_fp32=False):
    nz = cfg["nzp"] + cfg["cz"]
    plan = api.Plan((cfg["nx"], cfg["ny"], nz), (0, 0, cfg["cz"]), (0, 0, cfg["oz"]),
                    (cfg["Lx"], cfg["Ly"], cfg["Lz"]), precision=precision)
    s = api.Solver(plan, api.BOUSS, ord=cfg["ord"], dt=cfg["dt"], nu=cfg["nu"], kappa=cfg["kappa"], fused=fused,
                   nl_fp32=nl_fp32)
    th = initial.convection_theta(plan, seed=cfg["seed"], amp=1e-3)
    fth = initial.to_spectral(plan, [th])[0]
    s.th.copy_from(fth)
    for f in (s.vx, s.vy, s.vz, s.pr):
        f.zero()
    plan.synchronize()
    return plan, s


def dominant_roofline(report, hbm_peak, traffic_table):
    name, (n, ms, b) = max(report.items(), key=lambda kv: kv[1][1])
    per_ms = ms / n
    per_bytes = b / n
    achieved = per_bytes / (per_ms * 1e-3) / 1e9
    traffic = traffic_table.get(name)
    return {"kernel": name, "bound": "hbm", "achieved": round(achieved, 1), "peak": hbm_peak, "unit": "GB/s",
            "frac": round(achieved / hbm_peak, 4), "traffic": traffic,
            "algorithmic_bytes_per_launch": per_bytes, "avg_launch_ms": round(per_ms, 4),
            "launches": n, "share": round(ms / sum(v[1] for v in report.values()), 4)}


def fft_flops_per_stage(cfg, z_engine):
    """Model FFT operation count of one fused BOUSS RK stage (the secondary figure): 5 L log2 L
    per complex length-L transform, Bluestein counted at its padded length L (two length-L
    transforms plus the chirp and filter multiplies), 2.5 nx log2 nx per real x transform.
    Transforms per column, counted from the kernels: z 23 = z_inverse 4 fields x (value, d/dz)
    + fused_vcomp 3 x (NL forward, round trip inverse + forward) + fused_vproj 1 (pressure)
    + fused_theta 5; y 16 = 12 inverse (value, d/dy, d/dz of 4 fields) + 4 forward (NL);
    x 19 = 15 c2r + 4 r2c (x_nonlinear)."""
    import math
    nx, ny, nzp = cfg["nx"], cfg["ny"], cfg["nzp"]
    nz, nxh = nzp + cfg["cz"], cfg["nx"] // 2 + 1

    def cfft(L):
        return 5.0 * L * math.log2(L)
    L = z_engine["L"]
    z_col = 2 * cfft(L) + 6.0 * (2 * nz + L) if z_engine["bluestein"] else cfft(nz)
    return 23 * nxh * ny * z_col + 16 * nxh * nzp * cfft(ny) + 19 * ny * nzp * 2.5 * nx * math.log2(nx)


def fp64_gemm_tflops(device):
    """Measured FP64 peak: torch.matmul (cuBLAS DGEMM) of 8192^3, best of 3."""
    import torch
    a = torch.randn(8192, 8192, dtype=torch.float64, device=device)
    b = torch.randn(8192, 8192, dtype=torch.float64, device=device)
    torch.matmul(a, b)
    best = 1e30
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1) * 1e-3)
    return 2.0 * 8192 ** 3 / best / 1e12


def load_traffic(form="fp32"):
    """Per-launch DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of each kernel from
    the committed ncu summary of this workload and form: the rows
    '| kernel | launches | bytes per launch |' of profiles/dram_traffic_bouss512.md (FP32-bulk)
    or profiles/dram_traffic_bouss512_nl32.md (the precision form)."""
    name = "dram_traffic_bouss512.md" if form == "fp32" else f"dram_traffic_bouss512_{form}.md"
    path = os.path.join(ROOT, "profiles", name)
    out = {}
    try:
        for ln in open(path):
            cells = [c.strip() for c in ln.strip().strip("|").split("|")]
            if len(cells) >= 3 and cells[2].replace(".", "").replace("e", "").replace("+", "").isdigit():
                out[cells[0]] = float(cells[2])
    except OSError:
        pass
    return out


def cpu_baseline(steps, warmup, threads=None):
    """The oracle (FP64 CPU restatement) on the bounded sample; returns (value, cores, sample)."""
    import numpy as np
    from oracle import oracle as O
    O.build()
    threads = threads or os.cpu_count()
    O.set_threads(threads)
    c = CPU_SAMPLE
    g = O.Grid(c["nx"], c["ny"], c["nzp"] + c["cz"], c["cz"], c["oz"], c["Lx"], c["Ly"], c["Lz"])
    rng = np.random.default_rng(c["seed"])
    th = np.zeros(g.rshape)
    z = g.z[: c["nzp"]]
    th[: c["nzp"]] = 1e-3 * rng.uniform(-1, 1, (c["nzp"], c["ny"], c["nx"])) * (z * (c["Lz"] - z))[:, None, None]
    tht = g.fftp3d_real_to_complex(th)
    zero = np.zeros(g.sshape, complex)
    p = g.params(dt=c["dt"], nu=c["nu"], ord=c["ord"], kappa=c["kappa"])
    state = (zero, zero, zero, tht, zero)
    for _ in range(warmup):
        out = g.run(p, 1, *state[:3], state[4], th=state[3])
        state = (out[0], out[1], out[2], out[3], out[4])
    t0 = time.perf_counter()
    for _ in range(steps):
        out = g.run(p, 1, *state[:3], state[4], th=state[3])
        state = (out[0], out[1], out[2], out[3], out[4])
    dt = time.perf_counter() - t0
    pts = c["nx"] * c["ny"] * c["nzp"] * c["ord"] * steps
    sample = (f"{c['nx']}x{c['ny']}x{c['nzp']} (+{c['cz']}) BOUSS RK2, {steps} step(s) of the FP64 oracle, "
              f"{threads} threads")
    return pts / dt / 1e6, threads, sample


def max_over_ranks(v: float, dist=None, device="cpu") -> float:
    """The largest v over all ranks (the job's time is its slowest replica's)."""
    if dist is None:
        return float(v)
    import torch
    t = torch.tensor([float(v)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(world, pts, stages, seconds):
    """Whole-job Mpts*stages/s: every replica advances its own grid of `pts` points by `stages`
    RK stages; the job takes the slowest replica's `seconds`."""
    return world * pts * stages / seconds / 1e6


def run_reference(args):
    """--impl reference: the CPU restatement of the reference algorithm on the host cores."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    steps = max(1, min(args.steps, 3))
    warmup = 1 if args.warmup > 0 else 0
    value, cores, sample = cpu_baseline(steps, warmup)
    line = {"metric": METRIC, "value": round(value, 4), "unit": UNIT, "impl": "reference",
            "n_gpus": args.gpus, "steps": steps, "warmup": warmup, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "BOUSS Rayleigh-Benard 512x512x513 (+25 FC-Gram), RK2, dt=1e-5; "
                                   "timed on the bounded sample", "sample_grid": "128x128x513",
                       "parallelism": "host threads"},
            "cpu_baseline": {"value": round(value, 4), "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": round(value, 4), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def time_steps(plan, s, K, local):
    """K RK steps (one solver call) bracketed by CUDA events on the plan stream; returns ms."""
    import torch
    stream = torch.cuda.ExternalStream(plan.stream, device=torch.device("cuda", local))
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(stream)
    s.step(K)
    ev1.record(stream)
    ev1.synchronize()
    torch.cuda.synchronize()
    return ev0.elapsed_time(ev1)


def physical_errors(api, p64, a, b, names):
    """Relative L2 of each state field of solver a against solver b on the physical grid (FP64
    c2r of both states, rows z < nzp)."""
    import numpy as np
    fc, fr = p64.field(api.COMPLEX), p64.field(api.REAL)

    def phys(data):
        fc.upload(np.ascontiguousarray(data, dtype=np.complex128))
        api.fftp3d_complex_to_real(p64, fc, fr)
        return fr.download()[: p64.nzp]
    out = {}
    for name, fa, fb in zip(names, (a.vx, a.vy, a.vz, a.th), (b.vx, b.vy, b.vz, b.th)):
        ra, rb = phys(fa.download()), phys(fb.download())
        nb = float(np.linalg.norm(rb))
        out[name] = float(np.linalg.norm(ra - rb) / nb) if nb > 0 else float(np.linalg.norm(ra))
    fc.close()
    fr.close()
    return out


def committed_precision():
    """The committed 1000-step record of the precision study (profiles/precision_bouss512.md,
    its line starting with 'RESULT ')."""
    path = os.path.join(ROOT, "profiles", "precision_bouss512.md")
    try:
        for ln in open(path):
            if ln.startswith("RESULT "):
                return json.loads(ln[len("RESULT "):])
    except (OSError, ValueError):
        pass
    return None


FORMS = {
    "nl32": "precision form: FP32 nonlinear term, float-float (FP32-pair) state and column kernels",
    "fp32": "FP32-bulk (FP32 transforms and products; FP64 continuation arithmetic, wall solve, reductions)",
    "fp64": "plain FP64",
}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300")
    ap.add_argument("--refseq", action="store_true", help="time the reference call sequence instead of the fused stages")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--grid", default=None, help="NX,NY,NZP: another grid of the same case (profiling, sweeps)")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default tile widths")
    ap.add_argument("--caps", default=None, help="Z,Y,X,FUSED,SPLIT: set these instead of autotuning")
    ap.add_argument("--ff", default=None, help="PAIR_PROJ,PAIR_COLS: block shapes of the float-float column kernels "
                                                 "(with --caps; 0 = one 576-thread block per SM, 1 = two of 288)")
    ap.add_argument("--form", default="nl32", choices=sorted(FORMS),
                    help="the timed form: nl32 (the precision form, default), fp32 (FP32-bulk), fp64 (plain)")
    ap.add_argument("--fp64", action="store_true", help="same as --form fp64")
    ap.add_argument("--no-extra", action="store_true",
                    help="time the chosen form only (no FP64 / FP32-bulk lines, no in-run precision check)")
    args = ap.parse_args()
    if args.fp64:
        args.form = "fp64"
    if args.impl == "reference":
        return run_reference(args)

    import torch
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    from specter_gb300 import api, initial
    api.set_device(local)
    K, W = args.steps, max(args.warmup, 3)

    cfg = dict(CFG)
    if args.grid:
        cfg["nx"], cfg["ny"], cfg["nzp"] = (int(v) for v in args.grid.split(","))
    form = args.form
    prec = api.FP32 if form == "fp32" else api.FP64
    plan, s = build_solver(api, initial, cfg, prec, fused=not args.refseq, nl_fp32=form == "nl32")
    # tile widths of each kernel family picked by timing RK steps (state restored afterwards)
    if form == "fp64":
        caps = None
    elif args.caps:
        caps = [int(v) for v in args.caps.split(",")]
        api.set_tile_caps(plan, caps[:4])
        api.set_option(plan, "velocity_split", caps[4])
        if args.ff:
            for name, v in zip(("ff_pair_proj", "ff_pair_cols"), args.ff.split(",")):
                api.set_option(plan, name, int(v))
    else:
        caps = s.autotune() if not args.no_autotune else None
    ff_opts = {n: api.get_option(plan, n) for n in ("ff_engine", "ff_pair_proj", "ff_pair_cols")} if form == "nl32" else None
    for _ in range(W):
        s.step(1)
    plan.synchronize()
    if dist:
        dist.barrier()
    plan.profile(True)
    n0 = plan.launch_count
    with ClockSampler(local) as clocks:
        ms = time_steps(plan, s, K, local)
    launches = plan.launch_count - n0
    report = plan.profile_report()
    plan.profile(False)
    s.check()
    ms = max_over_ranks(ms, dist, f"cuda:{local}")
    pts = cfg["nx"] * cfg["ny"] * cfg["nzp"]
    value = job_throughput(world, pts, cfg["ord"] * K, ms * 1e-3)

    # end to end through the C ABI: the state uploaded from pinned host memory (reference layout)
    # and downloaded back every step; value = steps / total time (the mean step)
    fields = [f for f in (s.vx, s.vy, s.vz, s.th, s.pr)]
    host = [torch.empty(f.nbytes, dtype=torch.uint8, pin_memory=True) for f in fields]
    ptrs = [h.data_ptr() for h in host]
    # one untimed round trip creates the staging buffers and the copy stream
    api.fields_download(fields, ptrs)
    api.fields_upload(fields, ptrs)
    Ke = max(5, K // 2)
    plan.synchronize()
    if dist:
        dist.barrier()
    tsteps = []
    for _ in range(Ke):
        t0 = time.perf_counter()
        api.fields_upload(fields, ptrs)     # pinned host -> device, conversions overlapped
        s.step(1)
        api.fields_download(fields, ptrs)   # device -> pinned host, returns with the data on the host
        plan.synchronize()
        tsteps.append(time.perf_counter() - t0)
    te = max_over_ranks(sum(tsteps) / len(tsteps), dist, f"cuda:{local}")
    e2e = job_throughput(world, pts, cfg["ord"], te)
    nbytes = sum(f.nbytes for f in fields)

    line = None
    if rank == 0:
        field_mb = (cfg["nx"] // 2 + 1) * cfg["ny"] * (cfg["nzp"] + cfg["cz"]) * (16 if form != "fp32" else 8) / 1e6
        peak, peak_kind = peaks()
        roof = dominant_roofline(report, peak, load_traffic(form))
        roof["peak_kind"] = peak_kind
        # stage-level model of the frozen measurement definition: B = 128 * N * s per BOUSS stage,
        # s the word size of the state (FP64-sized words for the FP64 and precision forms)
        N = cfg["nx"] * cfg["ny"] * (cfg["nzp"] + cfg["cz"])
        es = 4 if form == "fp32" else 8
        model_gbs = 128 * N * es * cfg["ord"] * K / (ms * 1e-3) / 1e9
        line = {"metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": world, "steps": K,
                "warmup": W, "ms_per_step": round(ms / K, 4), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None,
                "dtype": {"nl32": "f32 (nonlinear) + f32x2 float-float (state, column kernels)", "fp32": "f32",
                          "fp64": "f64"}[form],
                "data": "synthetic",
                "config": {"workload": f"BOUSS Rayleigh-Benard {cfg['nx']}x{cfg['ny']}x{cfg['nzp']} (+{cfg['cz']} FC-Gram, "
                                       f"NZ={cfg['nzp'] + cfg['cz']}), RK2, dt=1e-5",
                           "form": form, "form_detail": FORMS[form],
                           "path": "reference-sequence" if args.refseq else "fused",
                           "autotune_caps_z_y_x_fused_split": list(caps) if caps else None,
                           "ff_column_kernels": ff_opts,
                           "l2": f"inputs larger than L2 ({field_mb:.0f} MB per field), no flush",
                           "parallelism": f"replicas x{world}" if world > 1 else "single GPU"},
                "roofline": roof,
                "stage_model": {"bytes_per_stage": 128 * N * es, "achieved_gbs": round(model_gbs, 1),
                                "frac": round(model_gbs / peak, 4)},
                "kernels": {k: {"launches": v[0], "ms": round(v[1], 3),
                                "gbs": round(v[2] / (v[1] * 1e-3) / 1e9, 1) if v[1] > 0 else None}
                            for k, v in sorted(report.items(), key=lambda kv: -kv[1][1])},
                "clocks": clocks.summary(),
                "e2e": {"value": round(e2e, 2), "unit": UNIT, "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
                        "steps": Ke, "mean_ms_per_step": round(1e3 * statistics.mean(tsteps), 3),
                        "median_ms_per_step": round(1e3 * statistics.median(tsteps), 3),
                        "ms_per_step_each": [round(1e3 * t, 1) for t in tsteps]},
                "gpu_launches": launches}
        if not args.no_extra and world == 1 and not args.grid:
            extra_forms(api, initial, cfg, local, form, line, peak, caps)
        if not args.no_cpu and world == 1:
            v, cores, sample = cpu_baseline(1, 0)
            line["cpu_baseline"] = {"value": round(v, 4), "unit": UNIT, "cores": cores, "kind": "port", "sample": sample}
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


def extra_forms(api, initial, cfg, local, form, line, peak, caps):
    """The other forms of the same workload, beside the headline: plain FP64 (the reference's
    own precision, with its roofline against HBM and against the measured FP64 peak) and
    FP32-bulk; and the precision check: each form against plain FP64 after 10 steps from the
    same initial field (in run), with the committed 1000-step record."""
    names = ["vx", "vy", "vz", "th"]
    pts = cfg["nx"] * cfg["ny"] * cfg["nzp"]
    N = cfg["nx"] * cfg["ny"] * (cfg["nzp"] + cfg["cz"])
    # plain FP64: 2 timed steps
    p64, s64 = build_solver(api, initial, cfg, api.FP64, fused=True)
    s64.step(1)
    p64.profile(True)
    ms64 = time_steps(p64, s64, 2, local)
    rep64 = p64.profile_report()
    p64.profile(False)
    v64 = pts * cfg["ord"] * 2 / (ms64 * 1e-3) / 1e6
    fpeak = fp64_gemm_tflops(f"cuda:{local}")
    flops64 = fft_flops_per_stage(cfg, p64.engines["z"]) * cfg["ord"] * 2 / (ms64 * 1e-3) / 1e12
    model64 = 128 * N * 8 * cfg["ord"] * 2 / (ms64 * 1e-3) / 1e9
    line["fp64"] = {"value": round(v64, 2), "unit": UNIT, "ms_per_step": round(ms64 / 2, 3), "steps": 2,
                    "roofline_hbm": {"stage_model_gbs": round(model64, 1), "peak": peak, "frac": round(model64 / peak, 4)},
                    "roofline_fp64": {"model_fft_tflops": round(flops64, 3), "peak_tflops": round(fpeak, 3),
                                      "peak_kind": "measured FP64 DGEMM (torch.matmul 8192^3)",
                                      "frac": round(flops64 / fpeak, 4)},
                    "kernels_ms_per_step": {k: round(v[1] / 2, 2)
                                            for k, v in sorted(rep64.items(), key=lambda kv: -kv[1][1])[:6]}}
    s64.close()
    p64.close()
    # FP32-bulk: autotuned, 10 timed steps
    if form != "fp32":
        p32, s32 = build_solver(api, initial, cfg, api.FP32, fused=True)
        s32.autotune()
        for _ in range(3):
            s32.step(1)
        p32.profile(True)
        ms32 = time_steps(p32, s32, 10, local)
        rep32 = p32.profile_report()
        p32.profile(False)
        roof32 = dominant_roofline(rep32, peak, load_traffic("fp32"))
        line["fp32_bulk"] = {"value": round(pts * cfg["ord"] * 10 / (ms32 * 1e-3) / 1e6, 2), "unit": UNIT,
                             "ms_per_step": round(ms32 / 10, 3), "roofline": roof32,
                             "stage_model": {"bytes_per_stage": 128 * N * 4,
                                             "frac": round(128 * N * 4 * cfg["ord"] * 10 / (ms32 * 1e-3) / 1e9 / peak, 4)}}
        s32.close()
        p32.close()
    # precision: every form against plain FP64 after 10 steps from the same initial field
    q64, r64 = build_solver(api, initial, cfg, api.FP64, fused=True)
    r64.step(10)
    prec = {"steps": 10, "reference": "plain FP64 GPU form (matches the FP64 oracle to 1e-11)",
            "metric": "relative L2 on the physical grid"}
    for f_ in ("nl32", "fp32"):
        pf, sf = build_solver(api, initial, cfg, api.FP32 if f_ == "fp32" else api.FP64, fused=True,
                              nl_fp32=f_ == "nl32")
        if f_ == form and caps:
            api.set_tile_caps(pf, caps[:4])
            api.set_option(pf, "velocity_split", caps[4])
        sf.step(10)
        prec[f_] = physical_errors(api, q64, sf, r64, names)
        sf.close()
        pf.close()
    r64.close()
    q64.close()
    rec = committed_precision()
    line["precision"] = {"gate": "<= 1e-5 relative L2 against FP64 after 1000 steps", "in_run_10_steps": prec,
                         "committed_1000_steps": rec,
                         "meets_gate": {"nl32": bool(rec and rec.get("max_1000", 1.0) <= 1e-5),
                                        "fp32": False}}


if __name__ == "__main__":
    main()
