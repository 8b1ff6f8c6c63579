"""littleharsh_gb300 -- GB300 (sm_103a) RK3 time step for Littleharsh.

Python host side of the C ABI in include/littleharsh.h.  It plays the part of
the reference's Fortran driver for users without a Fortran compiler: read
input.in, build the y grid and the canopy lists (start.f90 / y_grid_canopy.f90
/ geom_sym_canopy.f90, restated in C++ inside the library), create a solver
and advance it with `Solver.step` (the body of littleharsh.f90:161-201).

The compute path is the CUDA library built from littleharsh_gb300/csrc; there
is no CPU fallback.  Importing works without a GPU; creating a Solver needs
one and raises if the library or the device is missing.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

__all__ = ["Solver", "Config", "Input", "read_input", "load_library", "LhError", "PREC_FP64", "PREC_MIXED",
           "LAYOUT_PLANES", "LAYOUT_COLUMNS", "EXPORTED_SYMBOLS"]

PREC_FP64, PREC_MIXED = 0, 1
LAYOUT_PLANES, LAYOUT_COLUMNS = 0, 1
ABI_VERSION = 2

EXPORTED_SYMBOLS = [
    "lh_init", "lh_free", "lh_last_error", "lh_get_sizes", "lh_set_fields", "lh_get_fields", "lh_set_nonlinear",
    "lh_get_nonlinear", "lh_set_time", "lh_get_time", "lh_rk3_step", "lh_substage", "lh_get_rhs", "lh_divmax",
    "lh_cfl_dt", "lh_project", "lh_spectra_accumulate", "lh_spectra_flush", "lh_stats_accumulate",
    "lh_stats_flush", "lh_cond_accumulate", "lh_cond_flush", "lh_last_step_ms", "lh_profile_step",
    "lh_project_noalloc", "lh_set_monitor", "lh_get_monitor", "lh_fp64_peak", "lh_ensemble_create", "lh_ensemble_step", "lh_ensemble_last_error",
    "lh_ensemble_free", "lh_ensemble_set_mode", "lh_ensemble_info", "lh_autotune", "lh_get_launch_shapes", "lh_get_x_threads", "lh_get_z_threads", "lh_get_x_rows", "lh_write_restart", "lh_read_restart", "lh_write_stats", "lh_write_spectra", "lh_read_input", "lh_setup_grid", "lh_setup_canopy",
    # include/lh_srnet.h: kernels of the learned warm start
    "lh_sr_conv_fwd", "lh_sr_conv_fwd_tc", "lh_sr_tc_status", "lh_sr_conv_wgrad", "lh_sr_conv_wgrad_tc", "lh_sr_flip_weights", "lh_sr_mse", "lh_sr_adam",
]


class LhError(RuntimeError):
    """A failed call; `code` is the LH_E* return code (None when not from a call)."""

    def __init__(self, msg: str, code: int | None = None):
        super().__init__(msg)
        self.code = code


LH_EINVAL, LH_EUNSUPPORTED, LH_EFFT, LH_ECUDA, LH_ENOMEM, LH_ESTATE, LH_ENUMERIC = -1, -2, -3, -4, -5, -6, -7


class Params(C.Structure):
    _fields_ = [
        ("abi_version", C.c_int32), ("N", C.c_int32 * 20), ("Ngal", C.c_int32 * 20), ("nn", C.c_int32),
        ("flag_ctpress", C.c_int32), ("geometry_type", C.c_int32), ("dsty", C.c_int32),
        ("Re", C.c_double), ("alp", C.c_double), ("bet", C.c_double), ("ddthetavi", C.c_double),
        ("gridweighting", C.c_double * 6), ("precision", C.c_int32), ("ntilex", C.c_int32),
        ("ntilez", C.c_int32), ("reserved", C.c_int32), ("stream", C.c_void_p),
    ]


class Input(C.Structure):
    _fields_ = [
        ("Re", C.c_double), ("alp", C.c_double), ("bet", C.c_double),
        ("ngalx1", C.c_int32), ("ngalx2", C.c_int32), ("ngalz1", C.c_int32), ("ngalz2", C.c_int32),
        ("ny", C.c_int32), ("dyq", C.c_double), ("ppp", C.c_int32), ("flag_init", C.c_int32),
        ("fnameimb", C.c_char * 96), ("dirin", C.c_char * 96), ("dirout", C.c_char * 96),
        ("CFL", C.c_double), ("nwrite", C.c_int32), ("flag_ctpress", C.c_int32),
        ("mpgx", C.c_double), ("Kib", C.c_double), ("maxerr", C.c_double), ("maxt", C.c_double),
        ("maxA", C.c_double), ("physlim_bot", C.c_int32), ("physlim_top", C.c_int32),
        ("geometry_type", C.c_int32), ("ntilex", C.c_int32), ("ntilez", C.c_int32),
        ("posth", C.c_double), ("npeakx", C.c_int32), ("npeakz", C.c_int32),
        ("Lfracx", C.c_double), ("Lfracz", C.c_double),
        ("dsty", C.c_int32), ("dstx", C.c_int32), ("dstz", C.c_int32),
    ]

    def as_dict(self) -> dict:
        out = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            out[name] = v.decode() if isinstance(v, bytes) else v
        return out


_dp = C.POINTER(C.c_double)
_lib = None


def load_library(build: bool = True) -> C.CDLL:
    """Load (building first if needed) the in-tree CUDA library."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if build:
        path = _build.build()
    if not os.path.exists(path):
        raise LhError(f"CUDA library {path} is missing; run littleharsh_gb300/build.py")
    L = C.CDLL(path)
    vp, i32, cp = C.c_void_p, C.c_int32, C.c_char_p
    L.lh_init.argtypes = [C.POINTER(Params)] + [_dp] * 6 + [C.c_void_p, i32, C.c_void_p, i32, C.POINTER(vp)]
    L.lh_free.argtypes = [vp]
    L.lh_free.restype = None
    L.lh_last_error.argtypes = [vp]
    L.lh_last_error.restype = cp
    L.lh_get_sizes.argtypes = [vp, C.c_void_p]
    for nm in ("lh_set_fields", "lh_get_fields"):
        getattr(L, nm).argtypes = [vp] + [_dp] * 4 + [i32]
    for nm in ("lh_set_nonlinear", "lh_get_nonlinear", "lh_get_rhs"):
        getattr(L, nm).argtypes = [vp] + [_dp] * 3 + [i32]
    L.lh_set_time.argtypes = [vp] + [C.c_double] * 4
    L.lh_get_time.argtypes = [vp, _dp]
    L.lh_rk3_step.argtypes = [vp, i32]
    L.lh_set_monitor.argtypes = [vp, C.c_double, i32]
    L.lh_get_monitor.argtypes = [vp, _dp, C.POINTER(i32)]
    L.lh_fp64_peak.argtypes = [_dp]
    L.lh_substage.argtypes = [vp, i32, i32]
    L.lh_divmax.argtypes = [vp, _dp]
    L.lh_cfl_dt.argtypes = [vp, C.c_double, _dp]
    L.lh_project.argtypes = [vp]
    L.lh_spectra_accumulate.argtypes = [vp]
    L.lh_spectra_flush.argtypes = [vp] + [_dp] * 5 + [C.POINTER(i32), i32]
    L.lh_stats_accumulate.argtypes = [vp]
    L.lh_stats_flush.argtypes = [vp, _dp, C.POINTER(i32), i32]
    L.lh_cond_accumulate.argtypes = [vp]
    L.lh_cond_flush.argtypes = [vp, _dp, C.c_void_p, C.POINTER(i32), i32]
    L.lh_last_step_ms.argtypes = [vp, _dp, C.POINTER(i32)]
    L.lh_profile_step.argtypes = [vp, _dp, C.c_void_p, i32]
    L.lh_autotune.argtypes = [vp, C.POINTER(i32), C.POINTER(i32)]
    L.lh_get_launch_shapes.argtypes = [vp, C.POINTER(i32), C.POINTER(i32), C.POINTER(i32)]
    L.lh_get_x_threads.argtypes = [vp, C.POINTER(i32)]
    L.lh_get_z_threads.argtypes = [vp, C.POINTER(i32)]
    L.lh_get_x_rows.argtypes = [vp, C.POINTER(i32)]
    L.lh_project_noalloc.argtypes = [C.POINTER(Params)] + [_dp] * 3 + [C.c_void_p] * 3 + [C.c_double, C.c_void_p]
    L.lh_write_restart.argtypes = [vp, C.POINTER(Params), _dp, _dp, cp, cp, i32]
    L.lh_read_restart.argtypes = [vp, cp, cp, _dp, C.POINTER(i32)]
    L.lh_write_stats.argtypes = [vp, C.POINTER(Params)] + [_dp] * 4 + [cp, i32]
    L.lh_write_spectra.argtypes = [vp, C.POINTER(Params)] + [_dp] * 4 + [cp, cp, i32]
    L.lh_ensemble_create.argtypes = [C.c_void_p, i32, C.POINTER(vp)]
    L.lh_ensemble_step.argtypes = [vp, i32, _dp]
    L.lh_ensemble_last_error.argtypes = [vp]
    L.lh_ensemble_last_error.restype = cp
    L.lh_ensemble_free.argtypes = [vp]
    L.lh_ensemble_free.restype = None
    L.lh_ensemble_set_mode.argtypes = [vp, i32]
    L.lh_ensemble_info.argtypes = [vp, C.POINTER(i32), C.POINTER(i32)]
    L.lh_read_input.argtypes = [cp, C.POINTER(Input)]
    L.lh_setup_grid.argtypes = [C.POINTER(Input), C.POINTER(Params)] + [_dp] * 6
    L.lh_setup_canopy.argtypes = [C.POINTER(Input), C.POINTER(Params), C.c_void_p, C.POINTER(i32), C.c_void_p,
                                  C.POINTER(i32)]
    L.lh_sr_conv_fwd.argtypes = [i32, i32, vp, vp, vp, vp, i32, vp, vp, i32, i32, i32, i32, vp]
    L.lh_sr_conv_fwd_tc.argtypes = [i32, i32, vp, vp, vp, vp, i32, vp, vp, i32, i32, i32, i32, vp]
    L.lh_sr_tc_status.argtypes = [C.POINTER(i32)]
    L.lh_sr_conv_wgrad.argtypes = [i32, i32, vp, vp, vp, vp, i32, i32, i32, vp]
    L.lh_sr_conv_wgrad_tc.argtypes = [i32, i32, vp, vp, vp, vp, i32, i32, i32, vp]
    L.lh_sr_flip_weights.argtypes = [i32, i32, vp, vp, vp]
    L.lh_sr_mse.argtypes = [vp, vp, vp, vp, vp, C.c_int64, vp]
    L.lh_sr_adam.argtypes = [vp, vp, vp, vp, vp, i32] + [C.c_float] * 5 + [i32, vp]
    _lib = L
    return L


def _p(a: np.ndarray):
    if a is None:
        return None
    assert a.flags.c_contiguous and a.dtype in (np.float64, np.complex128)
    return a.ctypes.data_as(_dp)


def read_input(path: str) -> Input:
    """Parse input.in with the reference's fixed-column reader."""
    inp = Input()
    rc = load_library().lh_read_input(path.encode(), C.byref(inp))
    if rc:
        raise LhError(f"cannot parse {path} (code {rc})")
    return inp


class Config:
    """The input.in quantities the time step depends on.  ngalx/ngalz are the
    wall bands' physical points (Ngalx1, Ngalz1); ngalx2/ngalz2 the middle
    band's (Ngalx2, Ngalz2; 0 = the same, one resolution everywhere)."""

    def __init__(self, Re=2800.0, alp=1.0, bet=2.0, ngalx=96, ngalz=96, ny=97, dyq=13.6, ppp=5,
                 geometry_type=3, posth=0.2, dsty=16, dstx=2, dstz=4, ntilex=12, ntilez=6, flag_ctpress=0,
                 mpgx=0.0, CFL=0.5, ngalx2=0, ngalz2=0):
        self.__dict__.update(dict(Re=Re, alp=alp, bet=bet, ngalx=ngalx, ngalz=ngalz, ny=ny, dyq=dyq, ppp=ppp,
                                  geometry_type=geometry_type, posth=posth, dsty=dsty, dstx=dstx, dstz=dstz,
                                  ntilex=ntilex, ntilez=ntilez, flag_ctpress=flag_ctpress, mpgx=mpgx, CFL=CFL,
                                  ngalx2=ngalx2, ngalz2=ngalz2))

    def to_input(self) -> Input:
        i = Input()
        i.Re, i.alp, i.bet = self.Re, self.alp, self.bet
        i.ngalx1 = self.ngalx
        i.ngalx2 = self.ngalx2 or self.ngalx
        i.ngalz1 = self.ngalz
        i.ngalz2 = self.ngalz2 or self.ngalz
        i.ny, i.dyq, i.ppp = self.ny, self.dyq, self.ppp
        i.geometry_type, i.posth = self.geometry_type, self.posth
        i.dsty, i.dstx, i.dstz, i.ntilex, i.ntilez = self.dsty, self.dstx, self.dstz, self.ntilex, self.ntilez
        i.flag_ctpress, i.mpgx, i.CFL = self.flag_ctpress, self.mpgx, self.CFL
        i.flag_init = 3
        return i

    @staticmethod
    def from_input(i: Input) -> "Config":
        return Config(Re=i.Re, alp=i.alp, bet=i.bet, ngalx=i.ngalx1, ngalz=i.ngalz1, ny=i.ny, dyq=i.dyq,
                      ppp=i.ppp, geometry_type=i.geometry_type, posth=i.posth, dsty=i.dsty, dstx=i.dstx,
                      dstz=i.dstz, ntilex=i.ntilex, ntilez=i.ntilez, flag_ctpress=i.flag_ctpress, mpgx=i.mpgx,
                      CFL=i.CFL, ngalx2=i.ngalx2 if i.ngalx2 != i.ngalx1 else 0,
                      ngalz2=i.ngalz2 if i.ngalz2 != i.ngalz1 else 0)


def setup(inp: Input):
    """Grid and canopy lists for an Input, as the reference's start-up builds them."""
    L = load_library()
    prm = Params()
    dsty = max(inp.dsty, 0)
    nyu, nyv = inp.ny + 2 * dsty + 1, inp.ny + 2 * dsty
    g = {"yu": np.zeros(nyu), "yv": np.zeros(nyv), "dthdyu": np.zeros(nyu), "dthdyv": np.zeros(nyv),
         "dyu2i": np.zeros((nyu, 3)), "dyv2i": np.zeros((nyv, 3))}
    rc = L.lh_setup_grid(C.byref(inp), C.byref(prm), *[_p(g[k]) for k in ("yu", "yv", "dthdyu", "dthdyv", "dyu2i",
                                                                           "dyv2i")])
    if rc:
        raise LhError(f"lh_setup_grid failed ({rc})")
    nu, nv = C.c_int32(0), C.c_int32(0)
    rc = L.lh_setup_canopy(C.byref(inp), C.byref(prm), None, C.byref(nu), None, C.byref(nv))
    if rc:
        raise LhError(f"lh_setup_canopy failed ({rc})")
    lu = np.zeros((max(nu.value, 1), 3), np.int32)
    lv = np.zeros((max(nv.value, 1), 3), np.int32)
    if nu.value or nv.value:
        rc = L.lh_setup_canopy(C.byref(inp), C.byref(prm), lu.ctypes.data, C.byref(nu), lv.ctypes.data,
                               C.byref(nv))
        if rc:
            raise LhError(f"lh_setup_canopy failed ({rc})")
    return prm, g, lu[: nu.value], lv[: nv.value]


class Solver:
    """One GPU solver (one handle of the C ABI)."""

    def __init__(self, cfg: Config | Input, precision: int = PREC_FP64, grid: dict | None = None):
        L = load_library()
        inp = cfg.to_input() if isinstance(cfg, Config) else cfg
        self.config = cfg if isinstance(cfg, Config) else Config.from_input(cfg)
        prm, g, lu, lv = setup(inp)
        if grid is not None:  # caller-supplied grid arrays (e.g. from another implementation)
            g = {k: np.ascontiguousarray(v, dtype=np.float64) for k, v in grid.items() if k in g}
        prm.precision = precision
        self.params, self.grid, self.list_u, self.list_v = prm, g, lu, lv
        h = C.c_void_p()
        rc = L.lh_init(C.byref(prm), *[_p(g[k]) for k in ("yu", "yv", "dthdyu", "dthdyv", "dyu2i", "dyv2i")],
                       lu.ctypes.data if lu.size else None, lu.shape[0], lv.ctypes.data if lv.size else None,
                       lv.shape[0], C.byref(h))
        if rc:
            raise LhError(f"lh_init failed ({rc}): {L.lh_last_error(None).decode()}")
        self.h = h
        s = np.zeros(12, np.int32)
        self._check(L.lh_get_sizes(self.h, s.ctypes.data))
        (self.nkx, self.nz, self.ngx, self.ngz, self.nyu, self.nyv, self.nyp, self.ju0, self.jv0, self.jp0,
         self.nib_u, self.nib_v) = [int(x) for x in s]

    def _check(self, rc):
        if rc:
            raise LhError(f"littleharsh call failed ({rc}): {load_library().lh_last_error(self.h).decode()}", rc)

    def close(self):
        if getattr(self, "h", None):
            load_library().lh_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # shapes ---------------------------------------------------------------
    def shape(self, grid: str, layout: int = LAYOUT_PLANES):
        ny = {"u": self.nyu, "v": self.nyv, "p": self.nyp}[grid]
        return (ny, self.nz, self.nkx) if layout == LAYOUT_PLANES else (self.nz * self.nkx, ny)

    def zeros(self, grid: str, layout: int = LAYOUT_PLANES):
        return np.zeros(self.shape(grid, layout), dtype=np.complex128)

    # fields -----------------------------------------------------------------
    def set_fields(self, u1=None, u2=None, u3=None, p=None, layout: int = LAYOUT_PLANES):
        a = [None if x is None else np.ascontiguousarray(x, dtype=np.complex128) for x in (u1, u2, u3, p)]
        for x, gname in zip(a, "uvup"):
            if x is not None and x.shape != self.shape(gname, layout):
                raise LhError(f"field shape {x.shape} != {self.shape(gname, layout)}")
        self._check(load_library().lh_set_fields(self.h, *[_p(x) for x in a], layout))

    def get_fields(self, layout: int = LAYOUT_PLANES, out=None):
        """Download u1, u2, u3, p (into `out`, four arrays of the right shapes, if given)."""
        if out is None:
            out = [self.zeros("u", layout), self.zeros("v", layout), self.zeros("u", layout), self.zeros("p", layout)]
        for x, gname in zip(out, "uvup"):
            if x.shape != self.shape(gname, layout) or x.dtype != np.complex128 or not x.flags.c_contiguous:
                raise LhError("output array of the wrong shape or type")
        self._check(load_library().lh_get_fields(self.h, *[_p(x) for x in out], layout))
        return out

    def set_nonlinear(self, n1, n2, n3, layout: int = LAYOUT_PLANES):
        a = [np.ascontiguousarray(x, dtype=np.complex128) for x in (n1, n2, n3)]
        self._check(load_library().lh_set_nonlinear(self.h, *[_p(x) for x in a], layout))

    def get_nonlinear(self, layout: int = LAYOUT_PLANES):
        out = [self.zeros("u", layout), self.zeros("v", layout), self.zeros("u", layout)]
        self._check(load_library().lh_get_nonlinear(self.h, *[_p(x) for x in out], layout))
        return out

    def get_rhs(self, layout: int = LAYOUT_PLANES):
        out = [self.zeros("u", layout), self.zeros("v", layout), self.zeros("u", layout)]
        self._check(load_library().lh_get_rhs(self.h, *[_p(x) for x in out], layout))
        return out

    # time -------------------------------------------------------------------
    def set_time(self, t: float, dt: float, mpgx: float, QxT: float = -1.0):
        self._check(load_library().lh_set_time(self.h, t, dt, mpgx, QxT))

    def time(self) -> dict:
        o = np.zeros(5)
        self._check(load_library().lh_get_time(self.h, _p(o)))
        return dict(t=o[0], dt=o[1], mpgx=o[2], QxT=o[3], Qx=o[4])

    def step(self, n: int = 1):
        self._check(load_library().lh_rk3_step(self.h, n))

    def set_monitor(self, maxerr: float, every: int = 1):
        """Check max |div| against maxerr every `every` steps (0 = off); a step that exceeds it, or that
        leaves a NaN or infinity in the fields, raises LhError with code LH_ENUMERIC."""
        self._check(load_library().lh_set_monitor(self.h, maxerr, every))

    def monitor(self) -> dict:
        """The monitor's last max |div| (-1 before its first check) and the device's error bits."""
        d, e = C.c_double(0), C.c_int32(0)
        self._check(load_library().lh_get_monitor(self.h, C.byref(d), C.byref(e)))
        return {"divmax": d.value, "err_bits": e.value}

    def substage(self, krk: int, upto: int = 5):
        self._check(load_library().lh_substage(self.h, krk, upto))

    def last_step_ms(self):
        ms, n = C.c_double(0), C.c_int32(0)
        self._check(load_library().lh_last_step_ms(self.h, C.byref(ms), C.byref(n)))
        return ms.value, n.value

    KERNEL_KINDS = ("zinv", "xprod", "zfwd", "assemble", "ib_zinv", "ib_xmask", "ib_zfwd", "vsolve", "flowrate",
                    "psolve")

    def profile_step(self) -> dict:
        """One step launch by launch; {kind: (total ms, launches)}."""
        ms = np.zeros(len(self.KERNEL_KINDS))
        cnt = np.zeros(len(self.KERNEL_KINDS), np.int32)
        self._check(load_library().lh_profile_step(self.h, _p(ms), cnt.ctypes.data, len(ms)))
        return {k: (float(ms[i]), int(cnt[i])) for i, k in enumerate(self.KERNEL_KINDS)}

    def autotune(self) -> dict:
        """Pick the z tile width, the product pass's levels per CTA and its buffer split by timing
        (lh_autotune); returns the shapes the next step uses."""
        self._check(load_library().lh_autotune(self.h, None, None))
        return self.launch_shapes()

    def launch_shapes(self) -> dict:
        """The z tile width, levels per product-pass CTA, product-pass buffer split and threads per
        product-pass and z-pass CTA in use."""
        tx, ch, xs, xt, zt, xr = (C.c_int32(0) for _ in range(6))
        L = load_library()
        self._check(L.lh_get_launch_shapes(self.h, C.byref(tx), C.byref(ch), C.byref(xs)))
        self._check(L.lh_get_x_threads(self.h, C.byref(xt)))
        self._check(L.lh_get_z_threads(self.h, C.byref(zt)))
        self._check(L.lh_get_x_rows(self.h, C.byref(xr)))
        return {"tx": tx.value, "chunk": ch.value, "xsplit": xs.value, "xthreads": xt.value, "zthreads": zt.value,
                "xrows": xr.value}

    # diagnostics ------------------------------------------------------------
    def divmax(self) -> float:
        o = C.c_double(0)
        self._check(load_library().lh_divmax(self.h, C.byref(o)))
        return o.value

    def cfl_dt(self, cfl: float) -> float:
        o = C.c_double(0)
        self._check(load_library().lh_cfl_dt(self.h, cfl, C.byref(o)))
        return o.value

    def project(self):
        self._check(load_library().lh_project(self.h))

    STAT_ROWS = ("Um", "U2m", "Vm", "V2m", "Wm", "W2m", "Pm", "P2m", "UVm", "UWm", "VWm", "wxm", "wx2m")

    def stats_accumulate(self):
        self._check(load_library().lh_stats_accumulate(self.h))

    def stats_flush(self, reset: bool = True):
        """(count, dict row -> profile over the row's own grid levels)."""
        L = max(self.nyu, self.nyv)
        o = np.zeros((13, L))
        n = C.c_int32(0)
        self._check(load_library().lh_stats_flush(self.h, _p(o), C.byref(n), int(reset)))
        ny = dict(Um=self.nyu, U2m=self.nyu, Vm=self.nyv, V2m=self.nyv, Wm=self.nyu, W2m=self.nyu, Pm=self.nyp,
                  P2m=self.nyp, UVm=self.nyu, UWm=self.nyu, VWm=self.nyv, wxm=self.nyv, wx2m=self.nyv)
        return n.value, {k: o[r, :ny[k]].copy() for r, k in enumerate(self.STAT_ROWS)}

    COND_ROWS = ("UmC", "U2mC", "WmC", "W2mC", "UVmC", "UWmC", "VmC", "V2mC", "VWmC", "PmC", "P2mC", "wxmC",
                 "wx2mC")

    def cond_accumulate(self):
        self._check(load_library().lh_cond_accumulate(self.h))

    def cond_flush(self, reset: bool = True):
        """(count, dict name -> array [j1][kin][i]) of the conditional statistics."""
        L = load_library()
        dims = np.zeros(5, np.int32)
        n = C.c_int32(0)
        self._check(L.lh_cond_flush(self.h, None, dims.ctypes.data, C.byref(n), 0))
        nju, njv, njp, dnx, dnz = [int(x) for x in dims]
        sizes = [nju] * 6 + [njv] * 3 + [njp] * 2 + [njv] * 2
        out = np.zeros(max(sum(sizes) * dnx * dnz, 1))
        self._check(L.lh_cond_flush(self.h, _p(out), dims.ctypes.data, C.byref(n), int(reset)))
        res, off = {}, 0
        for name, nj in zip(self.COND_ROWS, sizes):
            res[name] = out[off:off + nj * dnx * dnz].reshape(nj, dnz, dnx)
            off += nj * dnx * dnz
        return n.value, res

    # the reference's files -------------------------------------------------
    def write_restart(self, directory: str, name: str, iteration: int = 0):
        g = self.grid
        self._check(load_library().lh_write_restart(self.h, C.byref(self.params), _p(g["yu"]), _p(g["yv"]),
                                                    directory.encode(), name.encode(), iteration))

    def read_restart(self, directory: str, name: str):
        t, it = C.c_double(0), C.c_int32(0)
        self._check(load_library().lh_read_restart(self.h, directory.encode(), name.encode(), C.byref(t),
                                                   C.byref(it)))
        return t.value, it.value

    def write_stats(self, path: str, iteration: int = 0):
        g = self.grid
        self._check(load_library().lh_write_stats(self.h, C.byref(self.params), _p(g["yu"]), _p(g["yv"]),
                                                  _p(g["dthdyu"]), _p(g["dthdyv"]), path.encode(), iteration))

    def write_spectra(self, directory: str, name: str, iteration: int = 0):
        g = self.grid
        self._check(load_library().lh_write_spectra(self.h, C.byref(self.params), _p(g["yu"]), _p(g["yv"]),
                                                    _p(g["dthdyu"]), _p(g["dthdyv"]), directory.encode(),
                                                    name.encode(), iteration))

    def spectra_accumulate(self):
        self._check(load_library().lh_spectra_accumulate(self.h))

    def spectra_flush(self, reset: bool = True):
        nc = self.nz * self.nkx
        o = [np.zeros((self.nyu, nc)), np.zeros((self.nyv, nc)), np.zeros((self.nyu, nc)), np.zeros((self.nyu, nc)),
             np.zeros((self.nyp, nc))]
        n = C.c_int32(0)
        self._check(load_library().lh_spectra_flush(self.h, *[_p(x) for x in o], C.byref(n), int(reset)))
        return n.value, o


ENS_STREAMS, ENS_BATCHED = 0, 1


class Ensemble:
    """Independent solvers advanced together, one CUDA graph launch per RK3 step: one stream per member (the
    default) or batched launches (one per kernel kind, substage slot and grid class, covering its members)."""

    def __init__(self, members, mode: int = ENS_STREAMS):
        self.members = list(members)
        L = load_library()
        arr = (C.c_void_p * len(self.members))(*[m.h.value for m in self.members])
        e = C.c_void_p()
        rc = L.lh_ensemble_create(arr, len(self.members), C.byref(e))
        if rc:
            raise LhError(f"lh_ensemble_create failed ({rc}): {L.lh_last_error(None).decode()}", rc)
        self.e = e
        self.set_mode(mode)

    def set_mode(self, mode: int):
        L = load_library()
        rc = L.lh_ensemble_set_mode(self.e, mode)
        if rc:
            raise LhError(f"lh_ensemble_set_mode failed ({rc}): {L.lh_ensemble_last_error(self.e).decode()}", rc)

    def info(self) -> dict:
        """Mode of the captured graph and its kernel launches per step."""
        m, n = C.c_int32(0), C.c_int32(0)
        load_library().lh_ensemble_info(self.e, C.byref(m), C.byref(n))
        return {"mode": "batched" if m.value == ENS_BATCHED else "streams", "launches_per_step": n.value}

    def step(self, n: int = 1) -> float:
        ms = C.c_double(0)
        L = load_library()
        rc = L.lh_ensemble_step(self.e, n, C.byref(ms))
        if rc:
            raise LhError(f"lh_ensemble_step failed ({rc}): {L.lh_ensemble_last_error(self.e).decode()}", rc)
        return ms.value

    def close(self):
        if getattr(self, "e", None):
            load_library().lh_ensemble_free(self.e)
            self.e = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def fp64_peak() -> float:
    """FP64 FMA throughput of the current device in TFLOP/s, measured by the library's probe kernel."""
    L = load_library()
    o = C.c_double(0)
    rc = L.lh_fp64_peak(C.byref(o))
    if rc:
        raise LhError(f"lh_fp64_peak failed ({rc}): {L.lh_last_error(None).decode()}", rc)
    return o.value


from .initial import initial_field  # noqa: E402

__all__.append("initial_field")
