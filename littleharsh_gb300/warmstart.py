"""Learned warm start: coarse/fine pairs, lifting, training and the start itself.

The fine-grid solver's own snapshots give the training pairs: a snapshot is
spectrally filtered onto the coarse grid (Fourier modes truncated to the
coarse set, then linear interpolation in y onto the coarse levels) and lifted
back (modes zero-padded, linear interpolation onto the fine levels).  The
lifted field is the network input, the snapshot the target; the network learns
the correction that restores what the filter removed.  At start-up a
stationary field of the coarse solver is lifted the same way, corrected by the
network, returned to spectral space and made divergence free by the fine
solver's own Poisson step (Solver.project).

Conventions (those of the solver): spectral fields are plane-major
[level][kz index][kx index] with kx index 0..N1/2 and kz in FFT order;
physical values are the unnormalised inverse transform (sum of modes), so a
forward transform carries the 1/(ngx ngz) factor; the imaginary part of a
kx = 0 value is ignored by the real inverse.  Network volumes are
channels-last [level][z][x][c] on the u levels; v is carried at the u levels
(interpolated from its faces) and returned to the faces afterwards.

The transforms of this module only prepare data for the network (they run a
few times per snapshot, off the time step) and use torch.fft on the device.
"""
from __future__ import annotations

import math
import time

import numpy as np

from . import LhError


def _torch():
    import torch
    return torch


class GridInfo:
    """What the lifting needs to know about one solver's grid."""

    def __init__(self, s):
        self._init(s.grid, s.ngx, s.ngz, s.nkx, s.nz, s.ju0, s.list_u)

    @classmethod
    def from_config(cls, cfg: dict) -> "GridInfo":
        """The same information from the host set-up alone (no device needed)."""
        from . import Config, setup
        _, g, lu, _ = setup(Config(**cfg).to_input())
        n1, n2 = 2 * (cfg["ngalx"] // 3), 2 * (cfg["ngalz"] // 3)
        gi = cls.__new__(cls)
        gi._init(g, cfg["ngalx"], cfg["ngalz"], n1 // 2 + 1, n2, -max(cfg["dsty"], 0), lu)
        return gi

    def _init(self, g, ngx, ngz, nkx, nz, ju0, list_u):
        self.yu = np.asarray(g["yu"], np.float64)
        self.yv = np.asarray(g["yv"], np.float64)
        self.ngx, self.ngz, self.nkx, self.nz = ngx, ngz, nkx, nz
        self.nyu, self.nyv, self.nyp, self.ju0 = self.yu.size, self.yv.size, self.yu.size - 2, ju0
        # solid points of the canopy on the u levels (list rows: x index, z index (1-based), global j)
        m = np.zeros((self.nyu, self.ngz, self.ngx), np.float32)
        lu = np.asarray(list_u)
        if lu.size:
            m[lu[:, 2] - self.ju0, lu[:, 1] - 1, lu[:, 0] - 1] = 1.0
        self.mask = m

    @property
    def wc(self):
        """v -> centres: vc[jj] = v[jj-1] + wc[jj] (v[jj] - v[jj-1]), jj = 1..nyu-2."""
        jj = np.arange(1, self.nyu - 1)
        return (self.yu[jj] - self.yv[jj - 1]) / (self.yv[jj] - self.yv[jj - 1])

    @property
    def wf(self):
        """centres -> v: v[jv] = vc[jv] + wf[jv] (vc[jv+1] - vc[jv]), jv = 1..nyv-2."""
        jv = np.arange(1, self.nyv - 1)
        return (self.yv[jv] - self.yu[jv]) / (self.yu[jv + 1] - self.yu[jv])


# -- spectral <-> physical (3/2-padded grid) ------------------------------------------

def _kz_dst(nz_src: int, nz_dst: int):
    """Destination kz index of every source kz index (FFT order, negative kz at the end)."""
    kk = np.arange(nz_src)
    return np.where(kk < nz_src // 2, kk, kk - nz_src + nz_dst)


def spec_to_phys(f, ngx: int, ngz: int):
    """f: complex [L, nz, nkx] (torch, device) -> real [L, ngz, ngx]."""
    torch = _torch()
    L, nz, nkx = f.shape
    full = torch.zeros((L, ngz, ngx // 2 + 1), dtype=torch.complex128, device=f.device)
    full[:, torch.as_tensor(_kz_dst(nz, ngz), device=f.device), :nkx] = f
    return torch.fft.irfft2(full, s=(ngz, ngx), norm="forward")


def phys_to_spec(p, nz: int, nkx: int):
    """p: real [L, ngz, ngx] -> complex [L, nz, nkx] (the solver's forward transform, 1/(ngx ngz))."""
    torch = _torch()
    full = torch.fft.rfft2(p.to(torch.float64), norm="forward")
    ngz = p.shape[1]
    return full[:, torch.as_tensor(_kz_dst(nz, ngz), device=p.device), :nkx].contiguous()


def resample_modes(f, nz_dst: int, nkx_dst: int):
    """Truncate or zero-pad the Fourier modes of f [L, nz, nkx] to [L, nz_dst, nkx_dst]."""
    torch = _torch()
    L, nz, nkx = f.shape
    out = torch.zeros((L, nz_dst, nkx_dst), dtype=f.dtype, device=f.device)
    nk = min(nkx, nkx_dst)
    if nz_dst <= nz:  # truncate
        src = torch.as_tensor(_kz_dst(nz_dst, nz), device=f.device)
        out[:, :, :nk] = f[:, src, :nk]
    else:  # pad
        dst = torch.as_tensor(_kz_dst(nz, nz_dst), device=f.device)
        out[:, dst, :nk] = f[:, :, :nk]
    return out


def interp_levels(f, y_src: np.ndarray, y_dst: np.ndarray):
    """Linear interpolation along the first axis from levels y_src to y_dst
    (constant beyond the end levels)."""
    torch = _torch()
    ys = np.asarray(y_src, np.float64)
    yd = np.clip(np.asarray(y_dst, np.float64), ys[0], ys[-1])
    i1 = np.clip(np.searchsorted(ys, yd, side="right"), 1, ys.size - 1)
    i0 = i1 - 1
    t = (yd - ys[i0]) / (ys[i1] - ys[i0])
    shape = (-1,) + (1,) * (f.dim() - 1)
    tt = torch.as_tensor(t, dtype=torch.float64, device=f.device).reshape(shape)
    a = f[torch.as_tensor(i0, device=f.device)]
    b = f[torch.as_tensor(i1, device=f.device)]
    return a + (b - a) * tt


def v_to_centres(v, gi: GridInfo):
    """v on the faces [nyv, ...] -> the u levels [nyu, ...] (zero at the two ghost levels)."""
    torch = _torch()
    out = torch.zeros((gi.nyu,) + tuple(v.shape[1:]), dtype=v.dtype, device=v.device)
    wc = torch.as_tensor(gi.wc, dtype=torch.float64, device=v.device).reshape((-1,) + (1,) * (v.dim() - 1))
    out[1:gi.nyu - 1] = v[:-1] + (v[1:] - v[:-1]) * wc
    return out


def centres_to_v(vc, gi: GridInfo):
    """v at the u levels [nyu, ...] -> the faces [nyv, ...] (zero on the walls)."""
    torch = _torch()
    out = torch.zeros((gi.nyv,) + tuple(vc.shape[1:]), dtype=vc.dtype, device=vc.device)
    wf = torch.as_tensor(gi.wf, dtype=torch.float64, device=vc.device).reshape((-1,) + (1,) * (vc.dim() - 1))
    out[1:gi.nyv - 1] = vc[1:gi.nyv - 1] + (vc[2:gi.nyv] - vc[1:gi.nyv - 1]) * wf
    return out


# -- filter and lift ---------------------------------------------------------------

def coarsen(u1, u2, u3, fine: GridInfo, coarse: GridInfo):
    """Spectral filter of a fine field onto the coarse grid (modes, then levels)."""
    r = lambda f: resample_modes(f, coarse.nz, coarse.nkx)  # noqa: E731
    return (interp_levels(r(u1), fine.yu, coarse.yu), interp_levels(r(u2), fine.yv, coarse.yv),
            interp_levels(r(u3), fine.yu, coarse.yu))


def lift(u1, u2, u3, coarse: GridInfo, fine: GridInfo):
    """Coarse field onto the fine grid: zero-padded modes, linear in y."""
    r = lambda f: resample_modes(f, fine.nz, fine.nkx)  # noqa: E731
    return (r(interp_levels(u1, coarse.yu, fine.yu)), r(interp_levels(u2, coarse.yv, fine.yv)),
            r(interp_levels(u3, coarse.yu, fine.yu)))


def to_volume(u1, u2, u3, gi: GridInfo):
    """Spectral u, v, w -> physical fp32 [nyu, ngz, ngx, 3] with v at the u levels."""
    torch = _torch()
    pu = spec_to_phys(u1, gi.ngx, gi.ngz)
    pw = spec_to_phys(u3, gi.ngx, gi.ngz)
    pv = v_to_centres(spec_to_phys(u2, gi.ngx, gi.ngz), gi)
    return torch.stack([pu, pv, pw], dim=-1).to(torch.float32).contiguous()


def from_volume(vol, gi: GridInfo):
    """Physical [nyu, ngz, ngx, 3] -> spectral u1, u2 (faces), u3 (complex128, device)."""
    vol = vol.to(_torch().float64)
    u1 = phys_to_spec(vol[..., 0], gi.nz, gi.nkx)
    u3 = phys_to_spec(vol[..., 2], gi.nz, gi.nkx)
    u2 = phys_to_spec(centres_to_v(vol[..., 1], gi), gi.nz, gi.nkx)
    return u1, u2, u3


def net_input(base, gi: GridInfo):
    """bf16 [nyu, ngz, ngx, 16]: u, v, w of the lifted field, the solid mask, y, zeros."""
    torch = _torch()
    Y, Z, X, _ = base.shape
    x = torch.zeros((Y, Z, X, 16), dtype=torch.float32, device=base.device)
    x[..., :3] = base
    x[..., 3] = torch.as_tensor(gi.mask, device=base.device)
    x[..., 4] = torch.as_tensor(gi.yu, dtype=torch.float32, device=base.device).reshape(-1, 1, 1)
    return x.to(torch.bfloat16).contiguous()


def fields_to_device(fields):
    torch = _torch()
    return [torch.from_numpy(np.ascontiguousarray(f)).to("cuda") for f in fields]


class PairSet:
    """Training pairs on the device: network inputs (bf16), lifted bases and targets (fp32)."""

    def __init__(self, fine: GridInfo, coarse: GridInfo):
        self.fine, self.coarse = fine, coarse
        self.x, self.base, self.target = [], [], []

    def add_snapshot(self, u1, u2, u3):
        """A fine-grid snapshot (spectral, device tensors) -> one pair."""
        c = coarsen(u1, u2, u3, self.fine, self.coarse)
        lifted = lift(*c, self.coarse, self.fine)
        base = to_volume(*lifted, self.fine)
        tgt = to_volume(u1, u2, u3, self.fine)
        self.x.append(net_input(base, self.fine))
        self.base.append(base.reshape(-1, 3).contiguous())
        self.target.append(tgt.reshape(-1, 3).contiguous())

    def __len__(self):
        return len(self.x)


def mse_of(a, b) -> float:
    return float(((a.double() - b.double()) ** 2).mean())


def residual_scale(pairs: PairSet, idx) -> float:
    """rms of target - base over the pairs idx: the network predicts the
    residual in these units, so its output and the loss are O(1)."""
    acc, n = 0.0, 0
    for i in idx:
        d = (pairs.target[i] - pairs.base[i]).double()
        acc += float((d * d).sum())
        n += d.numel()
    return math.sqrt(acc / max(n, 1)) if acc > 0 else 1.0


def train(net, pairs: PairSet, train_idx, val_idx, epochs: int = 10, lr: float = 1e-3, seed: int = 0, log=None):
    """AdamW over the training pairs (one pair per step), cosine learning rate,
    on the residual target - base scaled by its rms (kept in net.sigma).
    Returns the history: per epoch the mean training loss (scaled units) and
    the validation MSE of the corrected field against that of the lifted field
    alone (physical units)."""
    torch = _torch()
    rng = np.random.default_rng(seed)
    net.sigma = residual_scale(pairs, train_idx)
    hist = []
    nsteps = epochs * len(train_idx)
    step = 0
    loss_acc = torch.zeros(1, dtype=torch.float64, device="cuda")
    zero = torch.zeros_like(pairs.base[train_idx[0]])
    t0 = time.perf_counter()
    for ep in range(epochs):
        order = rng.permutation(train_idx)
        loss_acc.zero_()
        for i in order:
            cur = lr * 0.5 * (1.0 + math.cos(math.pi * step / max(nsteps, 1)))
            tgt = ((pairs.target[i] - pairs.base[i]) * (1.0 / net.sigma)).contiguous()
            net.zero_grad()
            corr = net.forward(pairs.x[i], keep=True)
            dcorr = net.loss_grad(corr, zero, tgt, loss_acc)
            net.backward(dcorr)
            net.adam_step(cur)
            step += 1
        torch.cuda.synchronize()
        tr = loss_acc.item() / max(len(order), 1)
        v_net, v_lift = evaluate(net, pairs, val_idx)
        hist.append({"epoch": ep + 1, "train_loss_scaled": tr, "val_mse_net": v_net, "val_mse_lifted": v_lift,
                     "seconds": time.perf_counter() - t0})
        if log:
            log(f"epoch {ep + 1}: train {tr:.4e} (scaled)  val net {v_net:.4e}  val lifted {v_lift:.4e}  "
                f"({time.perf_counter() - t0:.1f} s)")
    return hist


def evaluate(net, pairs: PairSet, idx):
    """Mean validation MSE of (lifted + network correction) and of the lifted field alone."""
    torch = _torch()
    if len(idx) == 0:
        return float("nan"), float("nan")
    a, b = 0.0, 0.0
    sig = getattr(net, "sigma", 1.0)
    for i in idx:
        corr = net.forward(pairs.x[i])
        pred = pairs.base[i] + sig * corr.reshape(-1, 16)[:, :3]
        a += mse_of(pred, pairs.target[i])
        b += mse_of(pairs.base[i], pairs.target[i])
    torch.cuda.synchronize()
    return a / len(idx), b / len(idx)


def warm_field(net, cu1, cu2, cu3, coarse: GridInfo, fine: GridInfo, use_net: bool = True):
    """A coarse field (spectral, device) -> spectral u1, u2, u3 of the fine grid
    (numpy complex128), lifted and (with use_net) corrected by the network."""
    lifted = lift(cu1, cu2, cu3, coarse, fine)
    if not use_net:
        return [f.cpu().numpy() for f in lifted]
    base = to_volume(*lifted, fine)
    corr = net.forward(net_input(base, fine))
    vol = base + getattr(net, "sigma", 1.0) * corr[..., :3]
    return [f.cpu().numpy() for f in from_volume(vol, fine)]


def _log(log, msg):
    if log:
        log(msg)


def run_until(run, t_end: float, max_steps: int, on_window=None, log=None, tag=""):
    """Advance a study.LongRun until its first solver reaches t_end."""
    t0 = time.perf_counter()
    while run.solvers[0].time()["t"] < t_end and run.steps < max_steps:
        run.advance_window()
        if on_window:
            on_window(run)
        if log and len(run.records[0]) % 10 == 0:
            r = run.records[0][-1]
            _log(log, f"{tag} step {run.steps} t {r['t']:.1f} mpgx {r['mpgx']:.5g} tke {r['tke']:.4g} "
                      f"({time.perf_counter() - t0:.0f} s)")


def experiment(fine_cfg: dict, coarse_cfg: dict, re_tau: float, spinup_turnovers: float = 15.0,
               snapshots: int = 200, snap_every: int = 100, train_epochs: int = 20, eval_turnovers: float = 15.0,
               window: int = 200, every: int = 10, avg_windows: int = 10, tol: float = 0.005, cfl: float = 0.5,
               lr: float = 1e-3, seed: int = 1, max_steps: int = 2_000_000, realisations: int = 1,
               precision: int = 0, log=None) -> dict:
    """The learned warm start end to end on one fine/coarse grid pair.

    1. fine run from the seeded laminar + noise start: spin-up, then the
       converged statistics and `snapshots` snapshots `snap_every` steps apart;
    2. coarse run from its own seeded start to a stationary field;
    3. pairs from the snapshots (last 10% held out), network training;
    4. fine runs advanced together from: a fresh laminar + noise field, the
       lifted coarse field, and the lifted field corrected by the network (the
       last two projected divergence free), `realisations` of each (their own
       seeds and coarse runs); steps until each run's statistics stay within
       `tol` (or the noise floor of the converged statistics, if larger) of
       the converged ones.
    Every solver runs in `precision` (LH_PREC_FP64 or LH_PREC_MIXED).
    """
    import littleharsh_gb300 as lh
    from . import study
    from .srnet import SRNet
    T = fine_cfg["Re"] / re_tau
    res = {"fine": fine_cfg, "coarse": coarse_cfg, "turnover_time": T}

    # 1. fine spin-up, converged statistics, snapshots
    fine = lh.Solver(lh.Config(**fine_cfg), precision=precision)
    fgi = GridInfo(fine)
    t_phase = time.perf_counter()
    dt0 = study.seeded_start([fine], seed, cfl)
    qxt = fine.time()["QxT"]
    run = study.LongRun([fine], cfl=cfl, window=window, every=every)
    t_spin = spinup_turnovers * T
    run_until(run, t_spin, max_steps, log=log, tag="fine spin-up")
    spin_windows = len(run.records[0])
    coarse_gi = GridInfo.from_config(coarse_cfg)
    pairs = PairSet(fgi, coarse_gi)
    snaps_per_window = max(1, window // snap_every)
    if window % snap_every:
        raise ValueError("window must be a multiple of snap_every")
    t_snap0 = time.perf_counter()
    while len(pairs) < snapshots and run.steps < max_steps:
        # windows of the LongRun keep the statistics; snapshots inside them
        mp = []
        for _ in range(snaps_per_window):
            for _ in range(snap_every // every):
                run._step(every)
                fine.stats_accumulate()
                mp.append(fine.time()["mpgx"])
            if len(pairs) < snapshots:
                f = fields_to_device(fine.get_fields()[:3])
                pairs.add_snapshot(*f)
        n, st = fine.stats_flush()
        tm = fine.time()
        prof = study.fold(study.profiles(n, st, fine.ngx, fine.ngz), run.grids)
        run.records[0].append({"step": run.steps, "t": tm["t"], "dt": tm["dt"], "mpgx": float(np.mean(mp)),
                               "tke": study.tke(prof, run.grids), "count": n, "sums": st, "prof": prof})
        dtn = fine.cfl_dt(cfl)
        if abs(dtn - tm["dt"]) > run.dt_slack * tm["dt"]:
            fine.set_time(tm["t"], dtn, tm["mpgx"])
    recs = run.records[0]
    ref_prof = study.block_profiles(recs, spin_windows, len(recs), fine.ngx, fine.ngz, run.grids)
    ref_mpgx = float(np.mean([r["mpgx"] for r in recs[spin_windows:]]))
    # noise floor: deviation of blocks of the converged part from the converged statistics
    conv_devs = study.deviation_series(recs[spin_windows:], ref_prof, ref_mpgx, fine.ngx, fine.ngz, run.grids,
                                       avg_windows)[avg_windows - 1:]
    floor = float(np.percentile(conv_devs, 95)) if conv_devs else float("nan")
    tol_eff = max(tol, floor)
    fine_devs = study.deviation_series(recs, ref_prof, ref_mpgx, fine.ngx, fine.ngz, run.grids, avg_windows)
    res["reference_run"] = {"dt0": dt0, "steps": run.steps, "t": fine.time()["t"], "spinup_windows": spin_windows,
                            "seconds": time.perf_counter() - t_phase,
                            "snapshot_seconds": time.perf_counter() - t_snap0, "ref_mpgx": ref_mpgx,
                            "noise_floor": floor, "tol": tol, "tol_effective": tol_eff,
                            "plain_start_stationary_step": study.stationary_from(recs, fine_devs, tol_eff,
                                                                                 avg_windows),
                            "series": [{"step": r["step"], "t": r["t"], "mpgx": r["mpgx"], "tke": r["tke"],
                                        "dev": d} for r, d in zip(recs, fine_devs)]}
    _log(log, f"reference run: {run.steps} steps, noise floor {floor:.4f}, tol {tol_eff:.4f}")
    run.close()
    fine.close()

    # 2. coarse runs (one per realisation) to stationary fields, advanced together
    coarses = [lh.Solver(lh.Config(**coarse_cfg), precision=precision) for _ in range(realisations)]
    for q, c in enumerate(coarses):
        study.seeded_start([c], seed + 1 + 10 * q, cfl)
    crun = study.LongRun(coarses, cfl=cfl, window=window, every=every)
    run_until(crun, t_spin, max_steps, log=log, tag="coarse")
    cfs = [fields_to_device(c.get_fields()[:3]) for c in coarses]
    res["coarse_run"] = {"steps": crun.steps, "t": coarses[0].time()["t"],
                         "series": [{"step": r["step"], "t": r["t"], "mpgx": r["mpgx"], "tke": r["tke"]}
                                    for r in crun.records[0]]}
    crun.close()
    for c in coarses:
        c.close()

    # 3. training
    nval = max(1, len(pairs) // 10)
    idx = np.arange(len(pairs))
    net = SRNet(seed=seed, lr=lr)
    t_tr = time.perf_counter()
    hist = train(net, pairs, idx[:-nval], idx[-nval:], epochs=train_epochs, lr=lr, seed=seed, log=log)
    res["training"] = {"pairs": len(pairs), "val_pairs": nval, "epochs": train_epochs,
                       "seconds": time.perf_counter() - t_tr, "history": hist,
                       "params": int(sum(27 * ci * co + co for ci, co in net.shapes))}

    # 4. the three starts, `realisations` of each, advanced together in one ensemble
    names = ("laminar_noise", "lifted", "lifted_net")
    sols, kinds = [], []
    for q in range(realisations):
        for kind in names:
            s_ = lh.Solver(lh.Config(**fine_cfg), precision=precision)
            if kind == "laminar_noise":
                study.seeded_start([s_], seed + 2 + 10 * q, cfl)
            else:
                u1, u2, u3 = warm_field(net, *cfs[q], coarse_gi, fgi, use_net=(kind == "lifted_net"))
                s_.set_fields(u1, u2, u3, np.zeros((s_.nyp, s_.nz, s_.nkx), np.complex128))
                s_.project()
                s_.set_time(0.0, s_.cfl_dt(cfl), ref_mpgx, qxt)
            sols.append(s_)
            kinds.append(kind)
    dt_common = min(x.cfl_dt(cfl) for x in sols)
    for s_ in sols:
        tm = s_.time()
        s_.set_time(0.0, dt_common, tm["mpgx"], qxt)
    erun = study.LongRun(sols, cfl=cfl, window=window, every=every)
    t_eval = time.perf_counter()
    run_until(erun, eval_turnovers * T, max_steps, log=log, tag="starts")
    res["eval_seconds"] = time.perf_counter() - t_eval
    starts = {k: {"runs": []} for k in names}
    for i, kind in enumerate(kinds):
        rr = erun.records[i]
        devs = study.deviation_series(rr, ref_prof, ref_mpgx, sols[i].ngx, sols[i].ngz, erun.grids, avg_windows)
        starts[kind]["runs"].append({"stationary_step": study.stationary_from(rr, devs, tol_eff, avg_windows),
                                     "first_within_step": study.first_within(rr, devs, tol_eff, avg_windows),
                                     "first_dev": devs[avg_windows - 1] if len(devs) >= avg_windows else None,
                                     "series": [{"step": r["step"], "t": r["t"], "mpgx": r["mpgx"], "tke": r["tke"],
                                                 "dev": d} for r, d in zip(rr, devs)]})
    for kind in names:
        st = [r["stationary_step"] for r in starts[kind]["runs"]]
        ok = [x for x in st if x is not None]
        starts[kind]["stationary_steps"] = st
        starts[kind]["first_within_steps"] = [r["first_within_step"] for r in starts[kind]["runs"]]
        starts[kind]["mean_stationary_step"] = float(np.mean(ok)) if len(ok) == len(st) and ok else None
    res["starts"] = starts
    res["eval_steps"] = erun.steps
    res["dt_common_start"] = dt_common
    erun.close()
    for s_ in sols:
        s_.close()
    return res


def scale_check(fine_cfg: dict, coarse_cfg: dict, coarse_steps: int = 20, fine_steps: int = 3, seed: int = 1,
                cfl: float = 0.5, net=None, log=None) -> dict:
    """The warm start's path at full size, timed: a coarse field (a few steps
    from its seeded start), lifted onto the fine grid, corrected by the
    network (an untrained one, whose correction is zero, unless `net` is
    given), returned to spectral space, projected by the fine solver and
    stepped.  Reports the time of each part and the divergence after the
    projection."""
    import torch
    import littleharsh_gb300 as lh
    from . import study
    from .srnet import SRNet
    out = {"fine": [fine_cfg["ngalx"], fine_cfg["ngalz"]], "coarse": [coarse_cfg["ngalx"], coarse_cfg["ngalz"]]}
    c = lh.Solver(lh.Config(**coarse_cfg))
    study.seeded_start([c], seed, cfl)
    c.step(coarse_steps)
    cgi = GridInfo(c)
    cf = fields_to_device(c.get_fields()[:3])
    c.close()
    f = lh.Solver(lh.Config(**fine_cfg))
    fgi = GridInfo(f)
    out["fine_volume"] = [fgi.nyu, fgi.ngz, fgi.ngx]
    net = net or SRNet(seed=seed)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    lifted = lift(*cf, cgi, fgi)
    base = to_volume(*lifted, fgi)
    x = net_input(base, fgi)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    corr = net.forward(x)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    vol = base + getattr(net, "sigma", 1.0) * corr[..., :3]
    u1, u2, u3 = [g.cpu().numpy() for g in from_volume(vol, fgi)]
    del x, corr, base, vol, lifted
    torch.cuda.empty_cache()
    t3 = time.perf_counter()
    f.set_fields(u1, u2, u3, np.zeros((f.nyp, f.nz, f.nkx), np.complex128))
    f.project()
    div = f.divmax()
    t4 = time.perf_counter()
    f.set_time(0.0, f.cfl_dt(cfl), 0.0)
    f.step(fine_steps)
    ms = f.last_step_ms()[0] / max(fine_steps, 1)
    fields = f.get_fields()
    out.update({"lift_s": t1 - t0, "network_s": t2 - t1, "to_spectral_s": t3 - t2, "project_s": t4 - t3,
                "divmax_after_projection": div, "fine_ms_per_step": ms,
                "finite_after_steps": bool(all(np.all(np.isfinite(a)) for a in fields))})
    f.close()
    if log:
        log(str(out))
    return out
