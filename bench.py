"""Benchmark: grid-point RK3 steps per second of the Littleharsh time step.

Workload (configuration 2 of the benchmark set, the production FP64 drop-in on
one GPU): Re_b = 10000 (Re_tau ~ 550), Lx = 2pi, Lz = pi, 576 x 576 dealiased
physical points (384 x 384 Fourier modes), ny = 385 stretched points plus 32
canopy points per wall (450 u levels), 48 x 24 square posts per wall,
h = 0.1, 8 x 8 points per post; seeded laminar + 10% perturbation field,
projected divergence free; fixed dt from CFL 0.5.  FP64 throughout.

Metric: Ngal_x * Ngal_z * Ny_u * steps / second (whole job: summed over the
replicas of all ranks).  A "step" is one full RK3 step (three substages).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

With --precision fp64 (the default) the same run also measures the mixed form
(FP32 transforms, products, nonlinear term and canopy forcing; FP64 solves,
flow rate and statistics) on the same workload and reports it under "mixed",
and configuration 4's ensemble of 16 uneven replicas (FP64) under "ensemble".

--impl reference times the CPU FP64 restatement of the reference's step (the
Fortran reference cannot be built here) on all host cores, on a bounded
sample of the same workload: one untimed step, then the median of up to three
timed steps.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from littleharsh_gb300.workloads import CONFIG1, CONFIG2, CONFIG2_BANDS, MID288, XZ576_NY49, ensemble_configs  # noqa: E402

WORKLOADS = {
    "config2_576x576x450_fp64": CONFIG2,
    "config2_bands_576_384x450_fp64": CONFIG2_BANDS,
    "config1_96x96x130_fp64": CONFIG1,
    "mid_288x288x226_fp64": MID288,
    "xz576_ny49_fp64": XZ576_NY49,
}
DEFAULT_WORKLOAD = "config2_576x576x450_fp64"
METRIC = "grid-pt RK3 steps/s"
UNIT = "grid-pt steps/s"
BYTES_PER_POINT_FP64 = 576  # compulsory state traffic per spectral point per RK3 step


def _peaks() -> dict:
    """HBM and bf16 denominators from MEASURED_PEAKS.json (the profiling recipe's fallback if it is absent).
    The FP64 denominator is measured in the run itself (lh_fp64_peak)."""
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    out = {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "src": "fallback"}
    if os.path.exists(p):
        try:
            d = json.load(open(p))
            out = {"hbm_gbs": float(d["hbm_gbs"]), "bf16_tflops": float(d.get("bf16_tflops", 1900.0)),
                   "src": "measured"}
        except Exception:
            pass
    return out


# ----------------------------------------------------------------------------
# clocks during the timed region
# ----------------------------------------------------------------------------
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.index)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self) -> dict | None:
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out = ""
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


# ----------------------------------------------------------------------------
# model counts for the roofline
# ----------------------------------------------------------------------------
def _stages(n: int):
    """Radices of the DIT passes, in the order the kernels run them: 4s, 2s, 3s."""
    m, n4, n2, n3 = n, 0, 0, 0
    while m % 4 == 0:
        m //= 4
        n4 += 1
    while m % 2 == 0:
        m //= 2
        n2 += 1
    while m % 3 == 0:
        m //= 3
        n3 += 1
    return [4] * n4 + [2] * n2 + [3] * n3


def fft_flops(n: int, prune_last: bool = False) -> float:
    """FP64 operations (FMA = 2) of one complex DIT of length n as the kernels
    execute it.  Per butterfly with twiddles fused into the additions:
    radix 4: 38 (16 without twiddles), radix 2: 12 (4), radix 3: 32 (18), and
    28 for a last radix-3 stage whose middle output is skipped.  The first
    stage has no twiddles."""
    rad = _stages(n)
    tot = 0.0
    for s, r in enumerate(rad):
        first, last = s == 0, s == len(rad) - 1
        if first:
            per = {4: 16, 2: 4, 3: 18}[r]
        else:
            per = {4: 38, 2: 12, 3: 32}[r]
            if last and prune_last and r == 3:
                per = 28
        tot += (n / r) * per
    return tot


def xprod_flops(ngx, ngz, nkx, nlev) -> float:
    """x-pass with products for one substage, per level and z row: u and w
    inverted together by one complex transform of length ngx, v by a half-length
    real transform (pre-processing 12 per mode), six products forwarded as three
    pairs (split 8 per kept mode), interpolation and products 15 per point."""
    h = ngx // 2
    inv = fft_flops(ngx) + 8.0 * nkx + fft_flops(h) + 12.0 * h
    fwd = 3 * (fft_flops(ngx) + 16.0 * nkx)
    prod = 15.0 * ngx
    return nlev * ngz * (inv + fwd + prod)


def z_flops(ngz, nkx, nplanes, prune_last=False) -> float:
    return nplanes * nkx * fft_flops(ngz, prune_last)


# ----------------------------------------------------------------------------
def grid_points(cfg: dict, nyu: int, N) -> int:
    """Physical collocation points of one field: Ngalx * Ngalz per u level, the
    middle band's own Ngalx2 * Ngalz2 on its levels N(4,1)+1..N(4,2) when the
    workload has variable-resolution bands.  N is the lh_params N array
    (N(r, b) at [4 b + r - 1])."""
    fine = cfg["ngalx"] * cfg["ngalz"]
    if not cfg.get("ngalx2") and not cfg.get("ngalz2"):
        return fine * nyu
    coarse = (cfg.get("ngalx2") or cfg["ngalx"]) * (cfg.get("ngalz2") or cfg["ngalz"])
    nmid = N[2 * 4 + 3] - N[1 * 4 + 3]
    return fine * (nyu - nmid) + coarse * nmid


def band_geometry(cfg: dict, s):
    """(ngx, ngz, nkx, nz, centres, faces) of the plane work of each band: one
    entry without variable resolution; the wall bands' and the middle band's
    with it (middle band: u centres N(4,1)+1..N(4,2), v faces N(3,1)+1..N(3,2))."""
    nl_u, nl_v = s.nyu - 2, s.nyv - 2
    if not cfg.get("ngalx2") and not cfg.get("ngalz2"):
        return [(s.ngx, s.ngz, s.nkx, s.nz, nl_u, nl_v)]
    N = list(s.params.N)
    mid_u, mid_v = N[2 * 4 + 3] - N[1 * 4 + 3], N[2 * 4 + 2] - N[1 * 4 + 2]
    gx2, gz2 = cfg.get("ngalx2") or cfg["ngalx"], cfg.get("ngalz2") or cfg["ngalz"]
    return [(s.ngx, s.ngz, s.nkx, s.nz, nl_u - mid_u, nl_v - mid_v),
            (gx2, gz2, (2 * (gx2 // 3)) // 2 + 1, 2 * (gz2 // 3), mid_u, mid_v)]


def max_over_ranks(value: float, dist, device: str) -> float:
    """The slowest rank's timing (replicas only: no data moves between ranks)."""
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_value(world: int, points_per_rank: int, steps: int, ms_max: float) -> float:
    """Grid-point RK3 steps per second of all replicas together."""
    return world * points_per_rank * steps / (ms_max / 1e3)


def build_solver(cfg: dict, precision: int, seed: int):
    import littleharsh_gb300 as lh
    from littleharsh_gb300.initial import initial_field
    s = lh.Solver(lh.Config(**cfg), precision=precision)
    g = s.grid
    u1, u2, u3, p = initial_field(g["yu"], g["yv"], s.nz, s.nkx, s.nyp, seed=seed)
    s.set_fields(u1, u2, u3, p)
    s.project()
    dt = s.cfl_dt(0.5)
    s.set_time(0.0, dt, 0.0)
    s.tuned = s.autotune()  # launch shapes picked by timing on this grid (lh_autotune)
    return s, (u1, u2, u3, p)


def cpu_baseline(cfg: dict, threads: int, warmup: int = 1, timed: int = 2) -> dict:
    """The CPU FP64 restatement on the host cores: `warmup` untimed RK3 steps (first touch of its arrays), then
    the median of `timed` single-step timings of the same workload."""
    from oracle import pyoracle
    from littleharsh_gb300.initial import initial_field
    pyoracle.build()
    o = pyoracle.Oracle(**cfg, nthreads=threads)
    g = o.grid()
    o.set_fields(*initial_field(g["yu"], g["yv"], o.nz, o.nkx, o.nyp, seed=1))
    o.set_scalars(0.0, 1.0, 0.0)
    o.project()
    o.set_scalars(0.0, o.cfl_dt(0.5), 0.0, o.flowrate())
    for _ in range(max(warmup, 0)):
        o.step(1)
    secs = []
    for _ in range(max(timed, 1)):
        t0 = time.perf_counter()
        o.step(1)
        secs.append(time.perf_counter() - t0)
    sec = statistics.median(secs)
    pts = grid_points(cfg, o.nyu, [x for b in range(5) for x in (o.sz.N[0][b], o.sz.N[1][b], o.sz.N[2][b], o.sz.N[3][b])])
    return {"value": pts / sec, "unit": UNIT, "cores": threads, "kind": "port", "points": pts, "steps_timed": len(secs),
            "warmup": max(warmup, 0), "seconds_per_step": secs,
            "sample": f"median of {len(secs)} single RK3 steps after {max(warmup, 0)} untimed, "
                      f"{cfg['ngalx']}x{cfg['ngalz']}x{o.nyu} FP64 ({sec:.2f} s per step)"}


def run_reference(args, rank: int, world: int):
    """The reference's CPU path (the C restatement of its step, all host threads) on this arm's workload:
    a bounded sample, at most 1 warm-up and 3 timed steps."""
    if rank != 0:
        return
    cfg = WORKLOADS[args.workload]
    threads = os.cpu_count() or 1
    base = cpu_baseline(cfg, threads, warmup=min(max(args.warmup, 0), 1), timed=max(1, min(args.steps, 3)))
    v = base["value"]
    pts = base["points"]
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world,
            "steps": base["steps_timed"], "warmup": base["warmup"], "ms_per_step": 1e3 * pts / v,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded laminar + 10% perturbation, projected divergence-free)",
            "config": _config(args, cfg, world),
            "note": "CPU FP64 restatement of the reference step (the Fortran/MPI reference does not build here: no "
                    "Fortran compiler and FOU3D.f90 is missing)",
            "cpu_baseline": base,
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _config(args, cfg: dict, world: int) -> dict:
    """The workload description both arms print (identical keys and values)."""
    nyu = cfg["ny"] + 2 * cfg["dsty"] + 1
    nkx, nz = cfg["ngalx"] // 3 + 1, 2 * (cfg["ngalz"] // 3)
    return {"workload": args.workload, "grid_phys": [cfg["ngalx"], cfg["ngalz"], nyu],
            "modes": [2 * (cfg["ngalx"] // 3), nz], "posts": [cfg["ntilex"], cfg["ntilez"]],
            "post_height": cfg["posth"], "Re_b": cfg["Re"], "precision": args.precision,
            "parallelism": f"replicas x{world}",
            "l2": (f"inputs larger than L2 ({16 * nkx * nz * nyu / 1e6:.0f} MB per field)"
                   if 16 * nkx * nz * nyu > 129e6 else
                   f"fields of {16 * nkx * nz * nyu / 1e6:.0f} MB fit in L2 (a small case: no L2 flush between steps)"),
            "bands": [cfg.get("ngalx2") or cfg["ngalx"], cfg.get("ngalz2") or cfg["ngalz"]]
            if cfg.get("ngalx2") else None}


# The metric's third part, spin-up steps saved by the warm start, takes a long experiment (40 minutes on one
# GPU) that no bench run repeats; the line carries its committed result, labelled as such.
SPINUP = {
    "measured_in_this_run": False,
    "source": "profiles/warmstart_coarse96_fine192.md (python -m littleharsh_gb300.study warmstart --grid config1x2 "
              "--precision mixed ...)",
    "grids": "coarse 96x96x97 points (configuration 1) lifted onto 192x192x193, mixed form, 3 realisations per start",
    "steps_to_converged_statistics": {"laminar_noise": "> 46,300 (two of three never within 51,500 steps)",
                                      "lifted": 15167, "lifted_network": 15000},
    "first_block_deviation": {"laminar_noise": 0.996, "lifted": 0.110, "lifted_network": 0.112},
    "steps_saved_by_lifting": ">= 70 %", "network_gain_over_lifting": "none measurable",
}


def measure_ensemble(args, prec: int) -> dict:
    """Configuration 4: 16 replicas of uneven sizes advanced together from one graph per step with one stream per
    replica (the ensemble's default mode), beside batched launches (one per kernel kind, substage slot and grid
    class) and the replicas one by one, each with its own graph; the same start and steps in every mode."""
    import littleharsh_gb300 as lh
    cfgs = ensemble_configs()
    members = [build_solver(c, prec, seed=100 + i)[0] for i, c in enumerate(cfgs)]
    pts = sum(m.ngx * m.ngz * m.nyu for m in members)
    start = [m.get_fields() for m in members]
    times = [m.time() for m in members]

    def reset():
        for m, f, t in zip(members, start, times):
            m.set_fields(*f)
            m.set_time(t["t"], t["dt"], t["mpgx"], t["QxT"])
    res = {}
    for mode, name in ((lh.ENS_BATCHED, "batched"), (lh.ENS_STREAMS, "streams")):
        reset()
        e = lh.Ensemble(members, mode=mode)
        e.step(max(args.warmup, 1))
        sampler = ClockSampler(0)
        sampler.start()
        ms = e.step(args.steps)
        clocks = sampler.stop()
        res[name] = {"ms_per_step": ms / args.steps, "value": pts * args.steps / (ms / 1e3), "clocks": clocks,
                     **e.info()}
        e.close()
    reset()
    for m in members:
        m.step(max(args.warmup, 1))
    seq = 0.0
    for m in members:
        m.step(args.steps)
        seq += m.last_step_ms()[0]
    b = res["streams"]
    out = {"value": b["value"], "unit": UNIT, "ms_per_step": b["ms_per_step"], "mode": "streams",
           "replicas": len(members), "grids": sorted({(m.ngx, m.ngz, m.nyu) for m in members}),
           "streams": res["streams"], "batched": res["batched"],
           "sequential": {"value": pts * args.steps / (seq / 1e3), "ms_per_step": seq / args.steps,
                          "launches_per_step": sum(m.last_step_ms()[1] for m in members)},
           "speedup_vs_sequential": (seq / args.steps) / b["ms_per_step"],
           "batched_vs_streams": res["streams"]["ms_per_step"] / res["batched"]["ms_per_step"],
           "gpu_launches": b["launches_per_step"] * args.steps, "clocks": b["clocks"]}
    for m in members:
        m.close()
    return out


def run_ensemble(args, rank: int, world: int):
    import littleharsh_gb300 as lh
    prec = lh.PREC_MIXED if args.precision == "mixed" else lh.PREC_FP64
    e = measure_ensemble(args, prec)
    line = {"metric": METRIC, "value": e["value"], "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": e["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if prec == lh.PREC_FP64 else "mixed f32/f64",
            "data": "synthetic (seeded laminar + 10% perturbation, projected divergence-free)",
            "config": {"workload": "ensemble16_config4", "replicas": e["replicas"], "grids": e["grids"],
                       "precision": args.precision},
            **{k: e[k] for k in ("streams", "batched", "sequential", "speedup_vs_sequential", "batched_vs_streams",
                                 "gpu_launches", "clocks")}}
    print(json.dumps(line), flush=True)


def _model_per_launch(cfg: dict, s, prof: dict, csz: int) -> dict:
    """Compulsory bytes and model FLOPs per launch of each pipeline kernel, summed over the bands' planes (one
    band without variable resolution) and divided by the kernel's launches per step.  csz = bytes of one complex
    value of the mixed planes (16 FP64, 8 mixed)."""
    npl = s.nkx * s.nz
    model_step = {"zinv": [0, 0.0], "xprod": [0, 0.0], "zfwd": [0, 0.0]}
    for (gx, gz, kx, kz, nc, nf) in band_geometry(cfg, s):
        mpb = kx * gz
        prune = gz % 3 == 0 and kz * 3 == 2 * gz
        model_step["zinv"][0] += 3 * (2 * nc + nf) * (kx * kz * 16 + mpb * csz)
        model_step["zinv"][1] += 3 * z_flops(gz, kx, 2 * nc + nf)
        model_step["xprod"][0] += 3 * (2 * nc + nf + 4 * nc + 2 * nf) * mpb * csz
        model_step["xprod"][1] += 3 * xprod_flops(gx, gz, kx, nc)
        model_step["zfwd"][0] += 3 * (4 * nc + 2 * nf) * (mpb * csz + kx * kz * 16)
        model_step["zfwd"][1] += 3 * z_flops(gz, kx, 4 * nc + 2 * nf, prune_last=prune)
    model_step["assemble"] = [3 * 19 * s.nyu * npl * 16, 0.0]
    model_step["vsolve"] = [3 * 4 * (2 * s.nyu + s.nyv) * npl * 16, 0.0]
    model_step["psolve"] = [3 * ((16 + 16 + 16 + 8 + 8) * s.nyp * npl + 14 * 16 * s.nyp * npl), 0.0]
    return {k: (v[0] / max(prof.get(k, (0.0, 1))[1], 1), v[1] / max(prof.get(k, (0.0, 1))[1], 1))
            for k, v in model_step.items()}


def _traffic(workload: str, precision: str, kernel: str):
    """DRAM bytes per launch of `kernel` from one ncu capture (profiles/traffic.json), or None."""
    tp = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(tp):
        return None, None
    try:
        d = json.load(open(tp))
    except Exception:
        return None, None
    key = f"{workload}:{precision}:{kernel}"
    v = d.get(key)
    src = d.get("source", {})
    return v, (src.get(key) if v is not None and isinstance(src, dict) else None)


def _timed_steps(s, steps: int, warmup: int, dist, rt, clock_index: int):
    """W untimed steps, then K steps in one call bracketed by a barrier and device synchronisation on both sides;
    the solver's own CUDA events (on its stream) time the K graph launches.  Returns (ms, launches per step,
    clocks sampled during the timed region)."""
    if warmup > 0:
        s.step(warmup)

    def barrier():
        if dist is not None:
            dist.barrier()
    rt.cudaDeviceSynchronize()
    sampler = ClockSampler(clock_index)
    barrier()
    rt.cudaDeviceSynchronize()
    sampler.start()
    s.step(steps)
    rt.cudaDeviceSynchronize()
    barrier()
    clocks = sampler.stop()
    ms, launches = s.last_step_ms()
    return ms, launches, clocks


def _e2e(s, ic, steps: int, world: int, pts: int) -> dict:
    """The metric end to end through the C ABI with host buffers: every step uploads u, v, w, p from pinned host
    memory (lh_set_fields), advances one RK3 step and downloads the four fields (lh_get_fields); one untimed
    pass, then up to 5 timed steps."""
    import torch
    pin = [torch.empty(a.shape, dtype=torch.complex128, pin_memory=True).numpy() for a in ic]
    s.get_fields(out=pin)
    tinfo = s.time()
    nbytes = sum(a.nbytes for a in pin)
    n = max(1, min(steps, 5))

    def one():
        s.set_fields(*pin)
        s.set_time(tinfo["t"], tinfo["dt"], tinfo["mpgx"], tinfo["QxT"])
        s.step(1)
        s.get_fields(out=pin)
    one()
    t0 = time.perf_counter()
    for _ in range(n):
        one()
    sec = (time.perf_counter() - t0) / n
    return {"value": world * pts / sec, "unit": UNIT, "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
            "ms_per_step": sec * 1e3, "steps_timed": n}


def _roofline(args, cfg, s, prec_name: str, prof: dict, peaks: dict, fp64_peak: float | None) -> dict:
    """The dominant kernel's rooflines: algorithmic HBM bytes and model FLOPs per launch over its average launch
    time (per-kernel CUDA events of one step launched kernel by kernel).  The FP64 kernels are bound by the FP64
    pipe on this part (about one FP64 instruction per 8 bytes of HBM traffic), so the line reports that roofline
    when its fraction is the larger, with the HBM one beside it."""
    dom = max(prof, key=lambda k: prof[k][0])
    dms, dn = prof[dom]
    per_launch_ms = dms / max(dn, 1)
    model = _model_per_launch(cfg, s, prof, 16 if prec_name == "fp64" else 8)
    bytes_l, flops_l = model.get(dom, (0, 0.0))
    ach_gbs = bytes_l / (per_launch_ms * 1e-3) / 1e9 if bytes_l else None
    traffic, tsrc = _traffic(args.workload, prec_name, dom)
    hbm = {"achieved": ach_gbs, "peak": peaks["hbm_gbs"], "unit": "GB/s",
           "frac": (ach_gbs / peaks["hbm_gbs"]) if ach_gbs else None,
           "peak_src": "MEASURED_PEAKS.json hbm_gbs (measured)" if peaks["src"] == "measured" else "fallback 6.8 TB/s"}
    roof = {"kernel": dom, "per_launch_ms": per_launch_ms, "algorithmic_bytes_per_launch": bytes_l,
            "traffic": traffic, "traffic_src": tsrc}
    fp64 = None
    if flops_l and prec_name == "fp64" and fp64_peak:
        tf = flops_l / (per_launch_ms * 1e-3) / 1e12
        fp64 = {"achieved": tf, "peak": fp64_peak, "unit": "TFLOP/s", "frac": tf / fp64_peak,
                "model_flops_per_launch": flops_l,
                "peak_src": "measured in this run by the library's FP64 FMA probe (lh_fp64_peak)",
                "note": "model flops count an FMA as 2; every FP64 addition of the butterflies also takes a full "
                        "pipe slot, so the pipe is busier than this fraction"}
        c576 = dom == "xprod" and cfg.get("ngalx") == 576 and cfg.get("ngalz") == 576 and not cfg.get("ngalx2")
        if c576:
            fp64["pipe_active_ncu"] = 0.853
            fp64["pipe_active_src"] = ("profiles/k_xprod_xz576_fp64.txt: ncu sm__pipe_fp64_cycles_active of this "
                                       "kernel at configuration 2's transform lengths (a committed capture, not "
                                       "measured in this run)")
    if fp64 is not None and hbm["frac"] is not None and fp64["frac"] > hbm["frac"]:
        roof.update({"bound": "fp64", "achieved": fp64["achieved"], "peak": fp64["peak"], "unit": "TFLOP/s",
                     "frac": fp64["frac"], "fp64": fp64, "hbm": hbm})
    else:
        roof.update({"bound": "hbm", "achieved": hbm["achieved"], "peak": hbm["peak"], "unit": "GB/s",
                     "frac": hbm["frac"], "hbm": hbm})
        if fp64 is not None:
            roof["fp64"] = fp64
        elif flops_l:
            roof["fp32_model_tflops"] = flops_l / (per_launch_ms * 1e-3) / 1e12
    return roof


def _measure(args, cfg, prec: int, prec_name: str, rank: int, world: int, local_rank: int, dist, rt, peaks,
             fp64_peak):
    """One precision on the workload: device-timed K steps (max over ranks), then on rank 0 the per-kernel
    profile, the roofline and the end-to-end metric."""
    s, ic = build_solver(cfg, prec, seed=1 + rank)
    pts = grid_points(cfg, s.nyu, list(s.params.N))
    clock_index = (int(os.environ.get("CUDA_VISIBLE_DEVICES", str(local_rank)).split(",")[0])
                   if world == 1 else local_rank)
    ms, launches, clocks = _timed_steps(s, args.steps, args.warmup, dist, rt, clock_index)
    ms_max = max_over_ranks(ms, dist, f"cuda:{local_rank}")
    res = {"value": whole_job_value(world, pts, args.steps, ms_max), "ms_per_step": ms_max / args.steps,
           "gpu_launches": launches * args.steps, "clocks": clocks, "launch_shapes": getattr(s, "tuned", None),
           "grid": [s.ngx, s.ngz, s.nyu], "modes": [2 * (s.nkx - 1), s.nz], "spectral_points": s.nkx * s.nz * s.nyu}
    if rank == 0:
        prof = s.profile_step()
        res["roofline"] = _roofline(args, cfg, s, prec_name, prof, peaks, fp64_peak)
        res["kernels_ms_per_step"] = {k: {"ms_per_step": v[0], "launches_per_step": v[1]} for k, v in prof.items()}
        res["e2e"] = _e2e(s, ic, args.steps, world, pts)
    s.close()
    return res


def run_ours(args, rank: int, world: int, local_rank: int, dist):
    import ctypes

    import littleharsh_gb300 as lh
    cfg = WORKLOADS[args.workload]
    rt = ctypes.CDLL("libcudart.so")
    peaks = _peaks()
    fp64_peak = lh.fp64_peak() if rank == 0 else None
    main_prec = args.precision
    prec = lh.PREC_MIXED if main_prec == "mixed" else lh.PREC_FP64
    r = _measure(args, cfg, prec, main_prec, rank, world, local_rank, dist, rt, peaks, fp64_peak)
    mixed = None
    if main_prec == "fp64" and not args.no_mixed:
        # the mixed form (FP32 transforms, products, nonlinear term and canopy forcing; FP64 solves, flow rate,
        # statistics) on the same workload, same protocol
        mixed = _measure(args, cfg, lh.PREC_MIXED, "mixed", rank, world, local_rank, dist, rt, peaks, fp64_peak)
    if rank != 0:
        return
    out = {"metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64" if main_prec == "fp64" else "mixed f32/f64",
           "data": "synthetic (seeded laminar + 10% perturbation, projected divergence-free)",
           "config": _config(args, cfg, world), "launch_shapes": r["launch_shapes"],
           "gpu_launches": r["gpu_launches"], "e2e": r["e2e"], "roofline": r["roofline"],
           "kernels_ms_per_step": r["kernels_ms_per_step"], "clocks": r["clocks"],
           "fp64_peak_tflops": fp64_peak}
    if mixed is not None:
        out["mixed"] = {"value": mixed["value"], "unit": UNIT, "ms_per_step": mixed["ms_per_step"],
                        "speedup_vs_fp64": r["ms_per_step"] / mixed["ms_per_step"], "dtype": "mixed f32/f64",
                        "e2e": mixed["e2e"], "gpu_launches": mixed["gpu_launches"], "clocks": mixed["clocks"],
                        "roofline": mixed["roofline"], "kernels_ms_per_step": mixed["kernels_ms_per_step"],
                        "launch_shapes": mixed["launch_shapes"],
                        "precision": "FP32 transforms, products, nonlinear term and canopy forcing; FP64 viscous "
                                     "and pressure terms, Helmholtz and pressure solves, flow rate, statistics"}
    if main_prec == "fp64" and not args.no_ensemble and world == 1 and args.workload == DEFAULT_WORKLOAD:
        # configuration 4 (16 uneven replicas, FP64) on the same device, the same steps; reported beside the
        # headline, so a failure there is recorded in the line rather than ending the run
        try:
            out["ensemble"] = measure_ensemble(args, lh.PREC_FP64)
        except Exception as e:  # noqa: BLE001
            out["ensemble"] = {"error": f"{type(e).__name__}: {e}"}
    if main_prec == "fp64" and world == 1:
        out["spinup"] = SPINUP
    if not args.no_cpu_baseline and world == 1:
        try:
            out["cpu_baseline"] = cpu_baseline(cfg, os.cpu_count() or 1)
        except Exception as e:  # reported, never fatal to the GPU number
            out["cpu_baseline"] = {"value": None, "error": str(e)[:200]}
    print(json.dumps(out), flush=True)


def srnet_flops(Y: int, Z: int, X: int, train: bool) -> float:
    """Tensor FLOPs of one forward (or forward + backward) of the network on a volume:
    2 * 27 * cin * cout per voxel and convolution; the backward adds the data
    gradient of every convolution but the first and the weight gradient of all."""
    from littleharsh_gb300.srnet import layer_shapes
    v = Y * Z * X
    f = sum(2 * 27 * ci * co for ci, co in layer_shapes()) * v
    if not train:
        return float(f)
    dgrad = sum(2 * 27 * ci * co for ci, co in layer_shapes()[1:]) * v
    return float(f + dgrad + f)


def _conv_compare(peaks: dict, args) -> dict:
    """One 32 -> 32 convolution (bias + ReLU) and one 32 -> 32 weight gradient on configuration 1's volume:
    mma.sync against tcgen05, CUDA events over 20 launches after warm-up."""
    import torch
    import littleharsh_gb300 as lh
    from littleharsh_gb300 import warmstart as ws
    from littleharsh_gb300.srnet import _ptr, _stream
    from littleharsh_gb300.workloads import CONFIG1
    L = lh.load_library()
    gi = ws.GridInfo.from_config(CONFIG1)
    Y, Z, X = gi.nyu, gi.ngz, gi.ngx
    g = torch.Generator(device="cuda").manual_seed(1)
    x = torch.randn((Y, Z, X, 32), device="cuda", generator=g).to(torch.bfloat16)
    d = torch.randn((Y, Z, X, 32), device="cuda", generator=g).to(torch.bfloat16)
    dw = torch.zeros((27, 32, 32), dtype=torch.float32, device="cuda")
    db = torch.zeros(32, dtype=torch.float32, device="cuda")
    w = (torch.randn((27, 32, 32), device="cuda", generator=g) * 0.05).to(torch.bfloat16)
    bias = torch.zeros(32, dtype=torch.float32, device="cuda")
    y = torch.empty_like(x)
    flops = 2.0 * 27 * 32 * 32 * Y * Z * X
    out = {"volume": [Y, Z, X], "flops": flops}
    calls = [("wgrad_mma_sync", lambda: L.lh_sr_conv_wgrad(32, 32, _ptr(x), _ptr(d), _ptr(dw), _ptr(db), X, Y, Z,
                                                          _stream())),
             ("wgrad_tcgen05", lambda: L.lh_sr_conv_wgrad_tc(32, 32, _ptr(x), _ptr(d), _ptr(dw), _ptr(db), X, Y, Z,
                                                            _stream())),
             ("fwd_mma_sync", lambda: L.lh_sr_conv_fwd(32, 32, _ptr(x), _ptr(w), _ptr(bias), _ptr(y), 0, None, None,
                                                       9, X, Y, Z, _stream())),
             ("fwd_tcgen05", lambda: L.lh_sr_conv_fwd_tc(32, 32, _ptr(x), _ptr(w), _ptr(bias), _ptr(y), 0, None,
                                                         None, 9, X, Y, Z, _stream()))]
    for name, call in calls:
        if name == "wgrad_tcgen05" and Z % 16:
            continue
        for _ in range(max(args.warmup, 3)):
            if call():
                raise RuntimeError(f"{name} failed: {L.lh_last_error(None).decode()}")
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        n = 20
        a.record()
        for _ in range(n):
            call()
        b.record()
        torch.cuda.synchronize()
        ms = a.elapsed_time(b) / n
        out[f"us_{name}"] = ms * 1e3
        out[f"tflops_{name}"] = flops / (ms * 1e-3) / 1e12
        if peaks.get("bf16_tflops"):
            out[f"frac_of_bf16_peak_{name}"] = out[f"tflops_{name}"] / peaks["bf16_tflops"]
    return out


def run_srnet(args):
    """The super-resolution network's kernels: a training step on configuration 1's
    volume and inference on configuration 5's fine volume, CUDA events around
    each, bf16 tensor-core FLOP rates against the measured bf16 peak."""
    import torch
    from littleharsh_gb300 import warmstart as ws
    from littleharsh_gb300.srnet import SRNet
    from littleharsh_gb300.workloads import CONFIG1, CONFIG5_FINE
    peaks = _peaks()
    net = SRNet(seed=0)
    out = {"metric": "SR network bf16 TFLOP/s", "unit": "TFLOP/s", "higher_is_better": True, "n_gpus": 1,
           "dtype": "bf16 (fp32 accumulate)",
           "kernel": "3x3x3 implicit-GEMM conv on bf16 tensor cores: forward, data and weight gradients on mma.sync "
                     "m16n8k16 or on tcgen05 (TMEM accumulators), both timed"}
    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731
    cases = [("train_step_config1", CONFIG1, True), ("inference_config5_fine", CONFIG5_FINE, False)]
    if args.sr_small:  # profiler captures: the configuration-1 training step only
        cases = cases[:1]
    for name, cfg, train in cases:
        gi = ws.GridInfo.from_config(cfg)
        Y, Z, X = gi.nyu, gi.ngz, gi.ngx
        g = torch.Generator(device="cuda").manual_seed(0)
        x = torch.randn((Y, Z, X, 16), device="cuda", generator=g).to(torch.bfloat16)
        base = torch.randn((Y * Z * X, 3), device="cuda", generator=g)
        tgt = torch.randn((Y * Z * X, 3), device="cuda", generator=g)
        loss = torch.zeros(1, dtype=torch.float64, device="cuda")

        def step():
            if train:
                net.zero_grad()
                corr = net.forward(x, keep=True)
                net.backward(net.loss_grad(corr, base, tgt, loss))
                net.adam_step()
            else:
                net.forward(x)
        res = {}
        for tc in (False, True):
            net.tcgen05 = tc
            for _ in range(max(args.warmup, 1)):
                step()
            torch.cuda.synchronize()
            a, b = ev(), ev()
            n = max(args.steps, 1)
            a.record()
            for _ in range(n):
                step()
            b.record()
            torch.cuda.synchronize()
            res[tc] = a.elapsed_time(b) / n
        fl = srnet_flops(Y, Z, X, train)
        best = min(res, key=res.get)  # the faster forward form is the network's default
        tf = fl / (res[best] * 1e-3) / 1e12
        out[name] = {"volume": [Y, Z, X], "ms": res[best], "tflops": tf, "flops": fl,
                     "convolutions": "tcgen05" if best else "mma.sync",
                     "frac_of_bf16_peak": tf / peaks["bf16_tflops"] if peaks.get("bf16_tflops") else None,
                     "ms_mma_sync": res[False], "ms_tcgen05": res[True],
                     "tflops_tcgen05": fl / (res[True] * 1e-3) / 1e12}
        net.tcgen05 = True
        del x, base, tgt
        torch.cuda.empty_cache()
    out["conv_32x32_config1"] = _conv_compare(peaks, args)
    out["value"] = out["train_step_config1"]["tflops"]
    if "inference_config5_fine" not in out:
        out["note"] = "configuration-1 training step only (--sr-small)"
    out["peak_bf16_tflops"] = peaks.get("bf16_tflops")
    print(json.dumps(out), flush=True)


def run_cufft_compare(args):
    """The step's transforms against cuFFT (through torch.fft, called only) at the workload's shapes, beside
    the solver's own per-kernel times of one step: the z-inverse of one substage (u, w on the interior centres,
    v on the interior faces: nkx columns of ngz-point complex transforms per level and field) and the x
    transforms of the product pass (3 real inverse and 6 real forward transforms of ngx points per level and
    z row).  One-resolution workloads only."""
    import torch
    import littleharsh_gb300 as lh
    cfg = WORKLOADS[args.workload]
    if cfg.get("ngalx2") or cfg.get("ngalz2"):
        raise SystemExit("--cufft compares one-resolution workloads")
    out = {"metric": "transform time against cuFFT", "unit": "ms", "workload": args.workload, "cufft": {},
           "ours_per_launch": {}}
    for prec, name in ((lh.PREC_FP64, "fp64"), (lh.PREC_MIXED, "fp32")):
        s, _ = build_solver(cfg, prec, seed=1)
        prof = s.profile_step()
        out["ours_per_launch"][name] = {k: prof[k][0] / max(prof[k][1], 1) for k in ("zinv", "xprod")}
        ngx, ngz, nkx, nlev = s.ngx, s.ngz, s.nkx, s.nyu - 2
        s.close()
        cdt, rdt = (torch.complex128, torch.float64) if name == "fp64" else (torch.complex64, torch.float32)

        def timed(fn, reps=5):
            for _ in range(2):
                fn()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(reps):
                fn()
            e1.record()
            torch.cuda.synchronize()
            return e0.elapsed_time(e1) / reps
        res = {}
        A = torch.randn(3 * nlev, ngz, nkx, dtype=cdt, device="cuda")  # z strided by nkx, the solver's layout
        res["z_inverse_strided"] = timed(lambda: torch.fft.ifft(A, dim=1))
        Ac = A.permute(0, 2, 1).contiguous()
        del A
        res["z_inverse_contiguous"] = timed(lambda: torch.fft.ifft(Ac, dim=2))
        del Ac
        torch.cuda.empty_cache()
        rows = nlev * ngz
        S = torch.randn(3 * rows, ngx // 2 + 1, dtype=cdt, device="cuda")
        res["x_c2r_3"] = timed(lambda: torch.fft.irfft(S, n=ngx, dim=1))
        del S
        torch.cuda.empty_cache()
        R = torch.randn(6 * rows, ngx, dtype=rdt, device="cuda")
        res["x_r2c_6"] = timed(lambda: torch.fft.rfft(R, dim=1))
        del R
        torch.cuda.empty_cache()
        out["cufft"][name] = res
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default=DEFAULT_WORKLOAD)
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="fp64")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-mixed", action="store_true", help="with --precision fp64: skip the mixed form's line")
    ap.add_argument("--no-ensemble", action="store_true", help="skip the configuration-4 ensemble in the line")
    ap.add_argument("--ensemble", action="store_true", help="configuration 4: 16 replicas in one graph per step")
    ap.add_argument("--srnet", action="store_true", help="the warm start's network kernels (training and inference)")
    ap.add_argument("--sr-small", action="store_true", help="with --srnet: the configuration-1 training step only")
    ap.add_argument("--cufft", action="store_true", help="the step's transforms against cuFFT at the workload's shapes")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    else:
        try:
            import torch
            torch.cuda.set_device(0)
        except Exception:
            pass
    if args.cufft:
        run_cufft_compare(args)
    elif args.srnet:
        run_srnet(args)
    elif args.ensemble:
        run_ensemble(args, rank, world)
    else:
        run_ours(args, rank, world, local_rank, dist)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
