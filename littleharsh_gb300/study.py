"""Long runs of the time step: turbulence statistics and spin-up.

Two measurements are built on these helpers:

* FP64 against the mixed form on one grid: both start from the same seeded,
  projected field, advance together in one ensemble graph with the same dt,
  and their mean, rms and Reynolds-stress profiles are averaged over the same
  time window; the profile errors are reported against the FP64 run.
* Steps to stationarity of a run: windowed profiles and the mean pressure
  gradient (the drag that holds the flow rate constant) are recorded as the
  run goes; the run is stationary from the first window after which every
  windowed quantity stays within a tolerance of its converged value.

Profiles come from the device plane statistics (the sums that stats.f90:1-108
accumulates): with `n` accumulations over `ngx * ngz` points per plane, the
mean of u on plane j is Um[j] / (n ngx ngz) and its rms is
sqrt(U2m[j] / (n ngx ngz) - mean^2).  The (0,0) mode of v is zero at every
level, so <u'v'> is UVm / (n ngx ngz).
"""
from __future__ import annotations

import math
import time

import numpy as np

PROFILE_KEYS = ("U", "urms", "vrms", "wrms", "uv", "prms")


def profiles(count: int, st: dict, ngx: int, ngz: int) -> dict:
    """Mean, rms and Reynolds-stress profiles from flushed plane sums."""
    n = float(max(count, 1) * ngx * ngz)

    def rms(s2, s1):
        return np.sqrt(np.maximum(s2 / n - (s1 / n) ** 2, 0.0))

    return {"U": st["Um"] / n, "urms": rms(st["U2m"], st["Um"]), "vrms": rms(st["V2m"], st["Vm"]),
            "wrms": rms(st["W2m"], st["Wm"]), "uv": st["UVm"] / n, "prms": rms(st["P2m"], st["Pm"])}


# grid each profile lives on, and its parity under the mirror y -> -y
_GRID = {"U": ("u", 1), "urms": ("u", 1), "wrms": ("u", 1), "uv": ("u", -1), "vrms": ("v", 1), "prms": ("p", 1)}


def fold(prof: dict, grids: dict) -> dict:
    """Average each profile with its mirror image about the channel centre.

    The geometry is symmetric (canopies on both walls), so the two halves
    sample the same statistics; folding halves the sampling noise.  `grids`
    maps 'u', 'v', 'p' to the y coordinates of that grid; a grid that is not
    symmetric to 1e-12 is left unfolded.
    """
    out = {}
    for k, q in prof.items():
        g, sgn = _GRID[k]
        y = grids[g]
        if np.allclose(y, -y[::-1], rtol=0.0, atol=1e-12):
            out[k] = 0.5 * (q + sgn * q[::-1])
        else:
            out[k] = q.copy()
    return out


def interior(grids: dict) -> dict:
    """Masks of the levels strictly inside the box: every level but the first
    and last of each grid (the u/w ghost points and the v wall values; the p
    grid has no boundary levels)."""
    out = {}
    for g, y in grids.items():
        m = np.ones(y.size, bool)
        if g != "p":
            m[0] = m[-1] = False
        out[g] = m
    return out


def profile_errors(a: dict, b: dict, masks: dict) -> dict:
    """max |a - b| / max |b| over the interior levels, per profile (b is the reference)."""
    out = {}
    for k in PROFILE_KEYS:
        if k not in a or k not in b:
            continue
        m = masks[_GRID[k][0]]
        den = float(np.max(np.abs(b[k][m]))) if m.any() else 0.0
        out[k] = float(np.max(np.abs(a[k][m] - b[k][m])) / den) if den > 0 else 0.0
    return out


def tke(prof: dict, grids: dict) -> float:
    """Box-averaged turbulent kinetic energy 0.5 <u'u' + v'v' + w'w'>."""
    masks = interior(grids)

    def avg(q, y):
        m = masks["u"] if y is grids["u"] else masks["v"]
        if m.sum() < 2:
            return 0.0
        qq, yy = q[m], y[m]
        return float(np.sum(0.5 * (qq[1:] + qq[:-1]) * np.diff(yy)) / (yy[-1] - yy[0]))
    return 0.5 * (avg(prof["urms"] ** 2 + prof["wrms"] ** 2, grids["u"]) + avg(prof["vrms"] ** 2, grids["v"]))


def solver_grids(s) -> dict:
    g = s.grid
    yu = np.asarray(g["yu"])
    return {"u": yu, "v": np.asarray(g["yv"]), "p": yu[1:-1]}


def _add(acc, count, st):
    if acc is None:
        return [count, {k: v.copy() for k, v in st.items()}]
    acc[0] += count
    for k, v in st.items():
        acc[1][k] += v
    return acc


def seeded_start(solvers, seed: int, cfl: float, amp: float = 0.1):
    """The seeded laminar + perturbation field, projected once by the first
    solver and handed unchanged to the others; all get the first solver's
    CFL time step.  Returns dt."""
    from .initial import initial_field
    s0 = solvers[0]
    g = s0.grid
    s0.set_fields(*initial_field(g["yu"], g["yv"], s0.nz, s0.nkx, s0.nyp, seed=seed, amp=amp))
    s0.project()
    f = s0.get_fields()
    dt = s0.cfl_dt(cfl)
    for s in solvers:
        if s is not s0:
            s.set_fields(*f)
        s.set_time(0.0, dt, 0.0)
    return dt


class LongRun:
    """Several solvers advanced together in one ensemble graph, with windowed
    statistics.  Every `every` steps each solver accumulates its plane
    statistics and its mean pressure gradient is sampled; every `window` steps
    the sums are flushed into one window record per solver.  The common dt is
    re-evaluated at the end of each window as the smallest CFL step of the
    solvers, and changed when it moved by more than `dt_slack`."""

    def __init__(self, solvers, cfl: float = 0.5, window: int = 400, every: int = 10, dt_slack: float = 0.1):
        import littleharsh_gb300 as lh
        if window % every:
            raise ValueError("window must be a multiple of every")
        self.solvers = list(solvers)
        self.ens = lh.Ensemble(self.solvers) if len(self.solvers) > 1 else None
        self.cfl, self.window, self.every, self.dt_slack = cfl, window, every, dt_slack
        self.grids = solver_grids(self.solvers[0])
        self.records = [[] for _ in self.solvers]  # per solver: dicts per window
        self.steps = 0
        self.gpu_ms = 0.0

    def _step(self, n):
        if self.ens is not None:
            self.gpu_ms += self.ens.step(n)
        else:
            s = self.solvers[0]
            s.step(n)
            self.gpu_ms += s.last_step_ms()[0]
        self.steps += n

    def advance_window(self):
        mp = [[] for _ in self.solvers]
        for _ in range(self.window // self.every):
            self._step(self.every)
            for i, s in enumerate(self.solvers):
                s.stats_accumulate()
                mp[i].append(s.time()["mpgx"])
        dts = []
        for i, s in enumerate(self.solvers):
            n, st = s.stats_flush()
            tm = s.time()
            prof = fold(profiles(n, st, s.ngx, s.ngz), self.grids)
            if not all(np.all(np.isfinite(v)) for v in prof.values()):
                raise FloatingPointError(f"solver {i} diverged at step {self.steps}")
            self.records[i].append({"step": self.steps, "t": tm["t"], "dt": tm["dt"], "mpgx": float(np.mean(mp[i])),
                                    "tke": tke(prof, self.grids), "count": n, "sums": st, "prof": prof})
            dts.append(s.cfl_dt(self.cfl))
        dt_new, dt = min(dts), self.solvers[0].time()["dt"]
        if abs(dt_new - dt) > self.dt_slack * dt:
            for s in self.solvers:
                tm = s.time()
                s.set_time(tm["t"], dt_new, tm["mpgx"])

    def average(self, i: int, t_from: float) -> dict:
        """Folded profiles of solver i over the windows that start at or after t_from."""
        acc = None
        prev_t = 0.0
        for r in self.records[i]:
            if prev_t >= t_from:
                acc = _add(acc, r["count"], r["sums"])
            prev_t = r["t"]
        if acc is None:
            raise ValueError("no window after t_from")
        s = self.solvers[i]
        return fold(profiles(acc[0], acc[1], s.ngx, s.ngz), self.grids)

    def close(self):
        if self.ens is not None:
            self.ens.close()


def rel_l2(a, b) -> float:
    d = float(np.linalg.norm((np.asarray(a) - np.asarray(b)).ravel()))
    n = float(np.linalg.norm(np.asarray(b).ravel()))
    return d / n if n > 0 else d


def _series(run: LongRun):
    return [{"step": r["step"], "t": round(r["t"], 6), "dt": r["dt"],
             "mpgx": [run.records[i][w]["mpgx"] for i in range(len(run.solvers))],
             "tke": [run.records[i][w]["tke"] for i in range(len(run.solvers))]}
            for w, r in enumerate(run.records[0])]


def precision_study(cfg: dict, re_tau: float = 180.0, spinup_turnovers: float = 10.0, avg_turnovers: float = 20.0,
                    window: int = 400, every: int = 10, seed: int = 1, cfl: float = 0.5, max_steps: int = 400000,
                    max_seconds: float = 1e30, twin_eps: float = 1e-12, log=None) -> dict:
    """FP64 and the mixed form from one seeded field on one grid, beside an FP64
    twin started twin_eps away.

    Reports the relative L2 error of u, v, w, p after 10 steps, and the error
    of the mean, rms and Reynolds-stress profiles averaged over
    `avg_turnovers` eddy turnovers (delta / u_tau, u_tau = re_tau / Re with
    the bulk velocity and half height 1) after `spinup_turnovers` of spin-up,
    both against the FP64 run.
    """
    import littleharsh_gb300 as lh
    fp = lh.Solver(lh.Config(**cfg), precision=lh.PREC_FP64)
    mx = lh.Solver(lh.Config(**cfg), precision=lh.PREC_MIXED)
    dt0 = seeded_start([fp, mx], seed, cfl)
    # an FP64 twin started 1e-12 away: the difference between the two FP64 runs is
    # the sampling noise of the chaotic flow over the averaging window
    tw = lh.Solver(lh.Config(**cfg), precision=lh.PREC_FP64)
    f = fp.get_fields()
    rng = np.random.default_rng(seed + 1000)
    u1 = f[0].copy()
    u1[1:-1, :, 1:] += twin_eps * np.abs(u1).max() * (rng.standard_normal(u1[1:-1, :, 1:].shape)
                                                       + 1j * rng.standard_normal(u1[1:-1, :, 1:].shape))
    tw.set_fields(u1, f[1], f[2], f[3])
    tw.project()
    tw.set_time(0.0, dt0, 0.0)
    fp.step(10)
    mx.step(10)
    a, b = fp.get_fields(), mx.get_fields()
    l2 = {k: rel_l2(b[i], a[i]) for i, k in enumerate(("u", "v", "w", "p"))}
    tw.step(10)
    run = LongRun([fp, mx, tw], cfl=cfl, window=window, every=every)
    T = cfg["Re"] / re_tau
    t_spin, t_end = spinup_turnovers * T, (spinup_turnovers + avg_turnovers) * T
    w0 = time.perf_counter()
    while fp.time()["t"] < t_end and run.steps < max_steps and time.perf_counter() - w0 < max_seconds:
        run.advance_window()
        if log and len(run.records[0]) % 10 == 0:
            r = run.records[0][-1]
            log(f"step {run.steps} t {r['t']:.2f} dt {r['dt']:.4g} mpgx {r['mpgx']:.5g}/{run.records[1][-1]['mpgx']:.5g}"
                f"/{run.records[2][-1]['mpgx']:.5g} tke {r['tke']:.4g}/{run.records[1][-1]['tke']:.4g}"
                f"/{run.records[2][-1]['tke']:.4g}  ({time.perf_counter() - w0:.0f} s)")
    t_reached = fp.time()["t"]
    pf, pm, pt = run.average(0, t_spin), run.average(1, t_spin), run.average(2, t_spin)
    masks = interior(run.grids)
    errs = profile_errors(pm, pf, masks)
    noise = profile_errors(pt, pf, masks)
    # the same over the first half of the averaging window: errors that shrink with
    # the averaging time are sampling noise, not precision
    t_half = t_spin + 0.5 * (t_reached - t_spin)
    half = {}
    try:
        def upto(i):
            acc, prev = None, 0.0
            for r in run.records[i]:
                if prev >= t_spin and r["t"] <= t_half:
                    acc = _add(acc, r["count"], r["sums"])
                prev = r["t"]
            s = run.solvers[i]
            return fold(profiles(acc[0], acc[1], s.ngx, s.ngz), run.grids)
        h0 = upto(0)
        half = {"mixed_vs_fp64": profile_errors(upto(1), h0, masks), "fp64_twin_vs_fp64": profile_errors(upto(2), h0, masks)}
    except Exception:  # too short a run for two halves
        half = {}
    res = {"grid": [fp.ngx, fp.ngz, fp.nyu], "seed": seed, "cfl": cfl, "dt0": dt0, "l2_after_10_steps": l2,
           "turnover_time": T, "t_spinup": t_spin, "t_end": t_reached, "steps": run.steps + 10,
           "avg_turnovers": (t_reached - t_spin) / T, "profile_err_vs_fp64": errs,
           "max_profile_err": max(errs.values()) if errs else None,
           "fp64_twin_err_vs_fp64": noise, "max_twin_err": max(noise.values()) if noise else None,
           "twin_eps": twin_eps, "first_half": half,
           "gpu_ms_per_triple_step": run.gpu_ms / max(run.steps, 1),
           "profiles": {"y_u": run.grids["u"].tolist(), "y_v": run.grids["v"].tolist(),
                        "fp64": {k: v.tolist() for k, v in pf.items()},
                        "mixed": {k: v.tolist() for k, v in pm.items()},
                        "fp64_twin": {k: v.tolist() for k, v in pt.items()}},
           "series": _series(run)}
    tw.close()
    run.close()
    fp.close()
    mx.close()
    return res


def main(argv=None):
    import argparse
    import json
    from .workloads import CONFIG1, RE_TAU
    ap = argparse.ArgumentParser(prog="python -m littleharsh_gb300.study")
    sub = ap.add_subparsers(dest="cmd", required=True)
    p = sub.add_parser("precision", help="FP64 vs mixed on configuration 1's grid")
    p.add_argument("--spinup-turnovers", type=float, default=3.0)
    p.add_argument("--avg-turnovers", type=float, default=20.0)
    p.add_argument("--window", type=int, default=400)
    p.add_argument("--every", type=int, default=10)
    p.add_argument("--seed", type=int, default=1)
    p.add_argument("--max-steps", type=int, default=400000)
    p.add_argument("--max-seconds", type=float, default=1e30, help="end the run early (wall clock)")
    p.add_argument("--out", required=True)
    q = sub.add_parser("warmstart", help="learned warm start on configuration 1's geometry")
    q.add_argument("--grid", choices=("config1", "config1x2"), default="config1",
                   help="config1: fine configuration 1, coarse at half its resolution; config1x2: fine at twice "
                        "configuration 1's resolution, coarse configuration 1")
    q.add_argument("--precision", choices=("fp64", "mixed"), default="fp64")
    q.add_argument("--spinup-turnovers", type=float, default=15.0)
    q.add_argument("--eval-turnovers", type=float, default=15.0)
    q.add_argument("--snapshots", type=int, default=200)
    q.add_argument("--snap-every", type=int, default=100)
    q.add_argument("--epochs", type=int, default=20)
    q.add_argument("--window", type=int, default=200)
    q.add_argument("--avg-windows", type=int, default=10)
    q.add_argument("--seed", type=int, default=1)
    q.add_argument("--realisations", type=int, default=1)
    q.add_argument("--max-steps", type=int, default=2_000_000)
    q.add_argument("--out", required=True)
    e = sub.add_parser("precision-ensemble", help="several FP64 and mixed realisations on configuration 1's grid")
    e.add_argument("--realisations", type=int, default=3)
    e.add_argument("--spinup-turnovers", type=float, default=3.0)
    e.add_argument("--avg-turnovers", type=float, default=15.0)
    e.add_argument("--max-seconds", type=float, default=1e30)
    e.add_argument("--out", required=True)
    r = sub.add_parser("warmstart-scale", help="the warm start's path on configuration 5's grids, timed")
    r.add_argument("--out", required=True)
    a = ap.parse_args(argv)
    if a.cmd == "precision":
        res = precision_study(CONFIG1, re_tau=RE_TAU["config1"], spinup_turnovers=a.spinup_turnovers,
                              avg_turnovers=a.avg_turnovers, window=a.window, every=a.every, seed=a.seed,
                              max_steps=a.max_steps, max_seconds=a.max_seconds, log=lambda m: print(m, flush=True))
        with open(a.out, "w") as f:
            json.dump(res, f)
        print(json.dumps({k: res[k] for k in ("grid", "steps", "t_end", "avg_turnovers", "l2_after_10_steps",
                                              "profile_err_vs_fp64", "max_profile_err", "fp64_twin_err_vs_fp64",
                                              "max_twin_err", "first_half", "gpu_ms_per_triple_step")}))
    elif a.cmd == "precision-ensemble":
        res = precision_ensemble(CONFIG1, realisations=a.realisations, re_tau=RE_TAU["config1"],
                                 spinup_turnovers=a.spinup_turnovers, avg_turnovers=a.avg_turnovers,
                                 max_seconds=a.max_seconds, log=lambda m: print(m, flush=True))
        with open(a.out, "w") as f:
            json.dump(res, f)
        print(json.dumps({k: res[k] for k in ("realisations", "steps", "avg_turnovers", "mean_profile_err_mixed_vs_fp64",
                                              "fp64_mean_standard_error", "tke_fp64", "tke_mixed")}))
    elif a.cmd == "warmstart-scale":
        from . import warmstart
        from .workloads import CONFIG5_COARSE, CONFIG5_FINE
        res = warmstart.scale_check(CONFIG5_FINE, CONFIG5_COARSE, log=lambda m: print(m, flush=True))
        with open(a.out, "w") as f:
            json.dump(res, f)
    elif a.cmd == "warmstart":
        from . import warmstart
        from .workloads import CONFIG1_COARSE, CONFIG1_X2
        fine, coarse = (CONFIG1, CONFIG1_COARSE) if a.grid == "config1" else (CONFIG1_X2, CONFIG1)
        res = warmstart.experiment(fine, coarse, RE_TAU["config1"], spinup_turnovers=a.spinup_turnovers,
                                   snapshots=a.snapshots, snap_every=a.snap_every, train_epochs=a.epochs,
                                   eval_turnovers=a.eval_turnovers, window=a.window, avg_windows=a.avg_windows,
                                   seed=a.seed, max_steps=a.max_steps, realisations=a.realisations,
                                   precision=1 if a.precision == "mixed" else 0, log=lambda m: print(m, flush=True))
        with open(a.out, "w") as f:
            json.dump(res, f, default=float)
        print(json.dumps({"starts": {k: v["stationary_steps"] for k, v in res["starts"].items()},
                          "first_within": {k: v["first_within_steps"] for k, v in res["starts"].items()},
                          "tol_effective": res["reference_run"]["tol_effective"],
                          "val": res["training"]["history"][-1]}))




STAT_KEYS = ("U", "urms", "vrms", "wrms", "uv")


def block_profiles(records, lo: int, hi: int, ngx: int, ngz: int, grids: dict) -> dict:
    """Folded profiles of the windows lo..hi-1 of one solver's records."""
    acc = None
    for r in records[lo:hi]:
        acc = _add(acc, r["count"], r["sums"])
    return fold(profiles(acc[0], acc[1], ngx, ngz), grids)


def deviation(prof: dict, mpgx: float, ref_prof: dict, ref_mpgx: float, masks: dict) -> float:
    """Largest relative deviation of the mean, rms and Reynolds-stress profiles
    (each against the maximum of its reference) and of the mean pressure
    gradient from the reference statistics."""
    e = profile_errors(prof, ref_prof, masks)
    vals = [e[k] for k in STAT_KEYS if k in e]
    if ref_mpgx != 0:
        vals.append(abs(mpgx - ref_mpgx) / abs(ref_mpgx))
    return max(vals)


def deviation_series(records, ref_prof, ref_mpgx, ngx, ngz, grids, avg: int) -> list:
    """Deviation of every block of `avg` consecutive windows ending at each window."""
    masks = interior(grids)
    out = []
    for w in range(len(records)):
        lo = max(0, w - avg + 1)
        prof = block_profiles(records, lo, w + 1, ngx, ngz, grids)
        mp = float(np.mean([r["mpgx"] for r in records[lo:w + 1]]))
        out.append(deviation(prof, mp, ref_prof, ref_mpgx, masks))
    return out


def first_within(records, devs, tol: float, avg: int):
    """First step at which a block of `avg` windows comes within tol of the
    reference statistics (the step at which that block begins), or None."""
    for w in range(avg - 1, len(devs)):
        if devs[w] <= tol:
            first = w - avg + 1
            return records[first - 1]["step"] if first > 0 else 0
    return None


def stationary_from(records, devs, tol: float, avg: int, hold: int | None = None):
    """First step from which every later block of `avg` windows stays within
    tol of the reference statistics (the step at which the first such block
    begins), or None if the run never settles or has not stayed settled for
    `hold` windows (default avg) by its end."""
    ok_from = None
    for w in range(len(devs) - 1, -1, -1):
        if w < avg - 1:
            break
        if devs[w] <= tol:
            ok_from = w
        else:
            break
    if ok_from is None or len(devs) - ok_from < (avg if hold is None else hold):
        return None
    first = ok_from - avg + 1
    return records[first - 1]["step"] if first > 0 else 0


def precision_ensemble(cfg: dict, realisations: int = 3, re_tau: float = 180.0, spinup_turnovers: float = 3.0,
                       avg_turnovers: float = 15.0, window: int = 400, every: int = 10, seed: int = 11,
                       cfl: float = 0.5, max_steps: int = 400000, max_seconds: float = 1e30, log=None) -> dict:
    """FP64 and mixed runs from `realisations` seeded fields (one FP64 and one
    mixed run per field), all in one ensemble graph with a common dt.  The
    mean profiles of the FP64 runs are compared with those of the mixed runs;
    the spread of the FP64 runs' own profiles (standard error of their mean)
    is the sampling noise of that comparison."""
    import littleharsh_gb300 as lh
    sols = []
    for q in range(realisations):
        fp = lh.Solver(lh.Config(**cfg), precision=lh.PREC_FP64)
        mx = lh.Solver(lh.Config(**cfg), precision=lh.PREC_MIXED)
        seeded_start([fp, mx], seed + q, cfl)
        sols += [fp, mx]
    dt = min(s.cfl_dt(cfl) for s in sols)
    for s in sols:
        s.set_time(0.0, dt, 0.0)
    run = LongRun(sols, cfl=cfl, window=window, every=every)
    T = cfg["Re"] / re_tau
    t_spin, t_end = spinup_turnovers * T, (spinup_turnovers + avg_turnovers) * T
    w0 = time.perf_counter()
    while sols[0].time()["t"] < t_end and run.steps < max_steps and time.perf_counter() - w0 < max_seconds:
        run.advance_window()
        if log and len(run.records[0]) % 25 == 0:
            log(f"step {run.steps} t {sols[0].time()['t']:.1f} tke " +
                " ".join(f"{run.records[i][-1]['tke']:.4f}" for i in range(len(sols))) +
                f" ({time.perf_counter() - w0:.0f} s)")
    masks = interior(run.grids)
    profs = [run.average(i, t_spin) for i in range(len(sols))]
    fp_p, mx_p = profs[0::2], profs[1::2]
    mean = lambda ps: {k: np.mean([p[k] for p in ps], axis=0) for k in PROFILE_KEYS}  # noqa: E731
    fpm, mxm = mean(fp_p), mean(mx_p)
    err = profile_errors(mxm, fpm, masks)
    # standard error of the FP64 mean, per profile, relative to the profile's maximum
    sem = {}
    for k in PROFILE_KEYS:
        m = masks[_GRID[k][0]]
        arr = np.array([p[k][m] for p in fp_p])
        sd = arr.std(axis=0, ddof=1) if len(fp_p) > 1 else np.zeros(arr.shape[1])
        sem[k] = float(np.max(sd) / np.sqrt(len(fp_p)) / np.max(np.abs(fpm[k][m])))
    # the noise of a difference of two means: both groups' spreads, pointwise in y, at the point where the
    # difference is largest; and the difference seed by seed (a mixed run against the FP64 run from its field)
    diff_z, per_seed = {}, {}
    n = len(fp_p)
    for k in PROFILE_KEYS:
        m = masks[_GRID[k][0]]
        a = np.array([p[k][m] for p in fp_p])
        b = np.array([p[k][m] for p in mx_p])
        scale = np.max(np.abs(fpm[k][m]))
        d = b.mean(axis=0) - a.mean(axis=0)
        i = int(np.argmax(np.abs(d)))
        if n > 1:
            se = np.sqrt((a.std(axis=0, ddof=1) ** 2 + b.std(axis=0, ddof=1) ** 2) / n)
            diff_z[k] = {"diff": float(d[i] / scale), "se_diff": float(se[i] / scale),
                         "z": float(d[i] / se[i]) if se[i] > 0 else None}
        per_seed[k] = [float((b[q][i] - a[q][i]) / scale) for q in range(n)]
    tke_avg = []
    for i in range(len(sols)):
        rr = [r for r in run.records[i] if r["t"] >= t_spin]
        tke_avg.append(float(np.mean([r["tke"] for r in rr])) if rr else None)
    res = {"grid": [sols[0].ngx, sols[0].ngz, sols[0].nyu], "realisations": realisations, "seeds": [seed + q for q in range(realisations)],
           "steps": run.steps, "t_end": sols[0].time()["t"], "avg_turnovers": (sols[0].time()["t"] - t_spin) / T,
           "mean_profile_err_mixed_vs_fp64": err, "max_mean_profile_err": max(err.values()),
           "fp64_mean_standard_error": sem, "difference_at_its_largest": diff_z,
           "per_seed_difference_at_that_point": per_seed, "tke_fp64": tke_avg[0::2], "tke_mixed": tke_avg[1::2],
           "gpu_ms_per_ensemble_step": run.gpu_ms / max(run.steps, 1),
           "profiles": {"y_u": run.grids["u"].tolist(), "fp64_mean": {k: v.tolist() for k, v in fpm.items()},
                        "mixed_mean": {k: v.tolist() for k, v in mxm.items()}}}
    run.close()
    for s in sols:
        s.close()
    return res


if __name__ == "__main__":
    main()
