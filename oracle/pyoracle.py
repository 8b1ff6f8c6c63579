"""ctypes wrapper of the CPU FP64 oracle (liblh_oracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, never by the product package.  The oracle is a
C restatement of the reference's RK3 step; see lh_oracle.h for what it
follows.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liblh_oracle.so")


def build(force: bool = False) -> str:
    """Compile liblh_oracle.so next to its source (gcc, OpenMP)."""
    src = os.path.join(HERE, "lh_oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.check_call(["make", "-s", "-C", HERE])
    return LIB_PATH


class Input(C.Structure):
    _fields_ = [
        ("Re", C.c_double), ("alp", C.c_double), ("bet", C.c_double),
        ("ngalx1", C.c_int32), ("ngalx2", C.c_int32), ("ngalz1", C.c_int32), ("ngalz2", C.c_int32),
        ("ny", C.c_int32), ("dyq", C.c_double), ("ppp", C.c_int32), ("flag_init", C.c_int32),
        ("fnameimb", C.c_char * 96), ("dirin", C.c_char * 96), ("dirout", C.c_char * 96),
        ("CFL", C.c_double), ("nwrite", C.c_int32), ("flag_ctpress", C.c_int32), ("mpgx", C.c_double),
        ("Kib", C.c_double), ("maxerr", C.c_double), ("maxt", C.c_double), ("maxA", C.c_double),
        ("physlim_bot", C.c_int32), ("physlim_top", C.c_int32),
        ("geometry_type", C.c_int32), ("ntilex", C.c_int32), ("ntilez", C.c_int32),
        ("posth", C.c_double), ("npeakx", C.c_int32), ("npeakz", C.c_int32),
        ("Lfracx", C.c_double), ("Lfracz", C.c_double),
        ("dsty", C.c_int32), ("dstx", C.c_int32), ("dstz", C.c_int32),
    ]


class Config(C.Structure):
    _fields_ = [
        ("Re", C.c_double), ("alp", C.c_double), ("bet", C.c_double),
        ("ngalx", C.c_int32), ("ngalz", C.c_int32), ("ny", C.c_int32),
        ("dyq", C.c_double), ("ppp", C.c_int32), ("geometry_type", C.c_int32),
        ("posth", C.c_double), ("dsty", C.c_int32), ("dstx", C.c_int32), ("dstz", C.c_int32),
        ("ntilex", C.c_int32), ("ntilez", C.c_int32), ("flag_ctpress", C.c_int32),
        ("nthreads", C.c_int32), ("ngalx2", C.c_int32), ("ngalz2", C.c_int32),
    ]


class Sizes(C.Structure):
    _fields_ = [
        ("ngx", C.c_int32), ("ngz", C.c_int32), ("nx", C.c_int32), ("nz", C.c_int32), ("nkx", C.c_int32),
        ("ju0", C.c_int32), ("ju1", C.c_int32), ("jv0", C.c_int32), ("jv1", C.c_int32),
        ("jp0", C.c_int32), ("jp1", C.c_int32), ("nyu", C.c_int32), ("nyv", C.c_int32), ("nyp", C.c_int32),
        ("nn", C.c_int32), ("dny", C.c_int32), ("N", (C.c_int32 * 5) * 4), ("Ngal", (C.c_int32 * 5) * 4),
        ("nibu_planes", C.c_int32), ("nibv_planes", C.c_int32),
    ]


_lib = None
_dp = C.POINTER(C.c_double)


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        L.lho_read_input.argtypes = [C.c_char_p, C.POINTER(Input)]
        L.lho_create.argtypes = [C.POINTER(Config), C.c_char_p, C.c_int]
        L.lho_create.restype = C.c_void_p
        L.lho_destroy.argtypes = [C.c_void_p]
        L.lho_get_sizes.argtypes = [C.c_void_p, C.POINTER(Sizes)]
        L.lho_get_grid.argtypes = [C.c_void_p] + [_dp] * 7
        L.lho_get_ib.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        for nm in ("lho_set_fields", "lho_get_fields"):
            getattr(L, nm).argtypes = [C.c_void_p] + [_dp] * 4
        for nm in ("lho_set_nonlinear", "lho_get_nonlinear", "lho_get_rhs"):
            getattr(L, nm).argtypes = [C.c_void_p] + [_dp] * 3
        L.lho_set_scalars.argtypes = [C.c_void_p] + [C.c_double] * 4
        L.lho_get_scalars.argtypes = [C.c_void_p, _dp]
        L.lho_flowrate.argtypes = [C.c_void_p]
        L.lho_flowrate.restype = C.c_double
        L.lho_substage.argtypes = [C.c_void_p, C.c_int, C.c_int]
        L.lho_step.argtypes = [C.c_void_p, C.c_int]
        L.lho_divmax.argtypes = [C.c_void_p]
        L.lho_divmax.restype = C.c_double
        L.lho_cfl_dt.argtypes = [C.c_void_p, C.c_double]
        L.lho_cfl_dt.restype = C.c_double
        L.lho_project.argtypes = [C.c_void_p]
        L.lho_stats_accumulate.argtypes = [C.c_void_p]
        L.lho_stats_get.argtypes = [C.c_void_p, _dp]
        L.lho_spectra_accumulate.argtypes = [C.c_void_p]
        L.lho_cond_accumulate.argtypes = [C.c_void_p]
        L.lho_cond_get.argtypes = [C.c_void_p, _dp, C.c_void_p]
        L.lho_spectra_get.argtypes = [C.c_void_p] + [_dp] * 5
        L.lho_fft_c2c.argtypes = [C.c_int, C.c_int, _dp]
        L.lho_rft.argtypes = [C.c_int, C.c_int, _dp]
        L.lho_plane_to_phys.argtypes = [C.c_void_p, _dp, _dp]
        L.lho_plane_to_spec.argtypes = [C.c_void_p, _dp, _dp]
        L.lho_tridiag_solve.argtypes = [C.c_int, _dp, _dp, _dp, _dp]
        _lib = L
    return _lib


def _p(a: np.ndarray):
    assert a.dtype in (np.float64, np.complex128) and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def read_input(path: str) -> dict:
    inp = Input()
    rc = lib().lho_read_input(path.encode(), C.byref(inp))
    if rc:
        raise ValueError(f"input.in parse failed ({rc})")
    out = {}
    for name, _ in Input._fields_:
        v = getattr(inp, name)
        out[name] = v.decode() if isinstance(v, bytes) else v
    return out


def fft_c2c(x: np.ndarray, sign: int) -> np.ndarray:
    a = np.ascontiguousarray(x, dtype=np.complex128).copy()
    if lib().lho_fft_c2c(a.size, sign, _p(a)):
        raise ValueError("length must factor into 2, 3, 4")
    return a


def rft(c: np.ndarray, n: int, iopt: int) -> np.ndarray:
    a = np.zeros(n + 2)
    a[: c.size] = c
    lib().lho_rft(n, iopt, _p(a))
    return a


def tridiag_solve(a1, a2, a3, rhs) -> np.ndarray:
    x = np.ascontiguousarray(rhs, dtype=np.float64).copy()
    f = [np.ascontiguousarray(v, dtype=np.float64) for v in (a1, a2, a3)]
    lib().lho_tridiag_solve(x.size, _p(f[0]), _p(f[1]), _p(f[2]), _p(x))
    return x


class Oracle:
    """One oracle solver instance (FP64, CPU)."""

    def __init__(self, Re, alp, bet, ngalx, ngalz, ny, dyq=13.6, ppp=5, geometry_type=3, posth=0.2,
                 dsty=16, dstx=2, dstz=4, ntilex=12, ntilez=6, flag_ctpress=0, nthreads=0, ngalx2=0, ngalz2=0):
        """ngalx2/ngalz2: the middle band's physical points (0: one resolution everywhere)."""
        cfg = Config(Re, alp, bet, ngalx, ngalz, ny, dyq, ppp, geometry_type, posth, dsty, dstx, dstz,
                     ntilex, ntilez, flag_ctpress, nthreads, ngalx2, ngalz2)
        err = C.create_string_buffer(256)
        h = lib().lho_create(C.byref(cfg), err, 256)
        if not h:
            raise ValueError(err.value.decode())
        self.h = C.c_void_p(h)
        sz = Sizes()
        lib().lho_get_sizes(self.h, C.byref(sz))
        self.sz = sz
        self.nkx, self.nz, self.ngx, self.ngz = sz.nkx, sz.nz, sz.ngx, sz.ngz
        self.nyu, self.nyv, self.nyp = sz.nyu, sz.nyv, sz.nyp

    def __del__(self):
        if getattr(self, "h", None):
            lib().lho_destroy(self.h)
            self.h = None

    # shapes ---------------------------------------------------------------
    def shape(self, grid: str):
        ny = {"u": self.nyu, "v": self.nyv, "p": self.nyp}[grid]
        return (ny, self.nz, self.nkx)

    def zeros(self, grid: str):
        return np.zeros(self.shape(grid), dtype=np.complex128)

    # data -------------------------------------------------------------------
    def grid(self) -> dict:
        s = self.sz
        g = {"yu": np.zeros(s.nyu), "yv": np.zeros(s.nyv), "dthdyu": np.zeros(s.nyu), "dthdyv": np.zeros(s.nyv),
             "dyu2i": np.zeros((s.nyu, 3)), "dyv2i": np.zeros((s.nyv, 3)), "gw": np.zeros(6)}
        lib().lho_get_grid(self.h, *[_p(g[k]) for k in ("yu", "yv", "dthdyu", "dthdyv", "dyu2i", "dyv2i", "gw")])
        g["gw"] = g["gw"].reshape(2, 3)  # gridweighting(band, c) -> gw[c-1, band-1]
        return g

    def ib(self):
        s = self.sz
        pu = np.zeros(s.nibu_planes, np.int32)
        pv = np.zeros(s.nibv_planes, np.int32)
        mu = np.zeros((s.nibu_planes, s.ngz, s.ngx), np.uint8)
        mv = np.zeros((s.nibv_planes, s.ngz, s.ngx), np.uint8)
        lib().lho_get_ib(self.h, pu.ctypes.data, mu.ctypes.data, pv.ctypes.data, mv.ctypes.data)
        return pu, mu, pv, mv

    def set_fields(self, u1, u2, u3, p):
        a = [np.ascontiguousarray(x, dtype=np.complex128) for x in (u1, u2, u3, p)]
        assert a[0].shape == self.shape("u") and a[1].shape == self.shape("v") and a[3].shape == self.shape("p")
        lib().lho_set_fields(self.h, *[_p(x) for x in a])

    def get_fields(self):
        out = [self.zeros("u"), self.zeros("v"), self.zeros("u"), self.zeros("p")]
        lib().lho_get_fields(self.h, *[_p(x) for x in out])
        return out

    def set_nonlinear(self, n1, n2, n3):
        a = [np.ascontiguousarray(x, dtype=np.complex128) for x in (n1, n2, n3)]
        lib().lho_set_nonlinear(self.h, *[_p(x) for x in a])

    def get_nonlinear(self):
        out = [self.zeros("u"), self.zeros("v"), self.zeros("u")]
        lib().lho_get_nonlinear(self.h, *[_p(x) for x in out])
        return out

    def get_rhs(self):
        out = [self.zeros("u"), self.zeros("v"), self.zeros("u")]
        lib().lho_get_rhs(self.h, *[_p(x) for x in out])
        return out

    def set_scalars(self, t, dt, mpgx, QxT=-1.0):
        lib().lho_set_scalars(self.h, t, dt, mpgx, QxT)

    def scalars(self):
        o = np.zeros(4)
        lib().lho_get_scalars(self.h, _p(o))
        return dict(t=o[0], dt=o[1], mpgx=o[2], QxT=o[3])

    def flowrate(self) -> float:
        return lib().lho_flowrate(self.h)

    def substage(self, krk: int, upto: int = 5):
        rc = lib().lho_substage(self.h, krk, upto)
        if rc:
            raise RuntimeError(f"substage failed ({rc})")

    def step(self, n: int = 1):
        rc = lib().lho_step(self.h, n)
        if rc:
            raise RuntimeError(f"step failed ({rc})")

    def divmax(self) -> float:
        return lib().lho_divmax(self.h)

    def cfl_dt(self, cfl: float) -> float:
        return lib().lho_cfl_dt(self.h, cfl)

    def project(self):
        lib().lho_project(self.h)

    def to_phys(self, plane: np.ndarray) -> np.ndarray:
        a = np.ascontiguousarray(plane, dtype=np.complex128)
        out = np.zeros((self.ngz, self.ngx))
        lib().lho_plane_to_phys(self.h, _p(a), _p(out))
        return out

    def to_spec(self, phys: np.ndarray) -> np.ndarray:
        a = np.ascontiguousarray(phys, dtype=np.float64)
        out = np.zeros((self.nz, self.nkx), dtype=np.complex128)
        lib().lho_plane_to_spec(self.h, _p(a), _p(out))
        return out

    def stats_accumulate(self):
        lib().lho_stats_accumulate(self.h)

    def stats(self):
        L = max(self.nyu, self.nyv)
        o = np.zeros((13, L))
        n = lib().lho_stats_get(self.h, _p(o))
        return n, o

    def spectra_accumulate(self):
        lib().lho_spectra_accumulate(self.h)

    COND_ROWS = ("UmC", "U2mC", "WmC", "W2mC", "UVmC", "UWmC", "VmC", "V2mC", "VWmC", "PmC", "P2mC", "wxmC",
                 "wx2mC")

    def cond_accumulate(self):
        lib().lho_cond_accumulate(self.h)

    def cond(self):
        """(count, dict name -> array [j1][kin][i]) of the conditional statistics."""
        dims = np.zeros(5, np.int32)
        lib().lho_cond_get(self.h, None, dims.ctypes.data)
        nju, njv, njp, dnx, dnz = [int(x) for x in dims]
        sizes = [nju] * 6 + [njv] * 3 + [njp] * 2 + [njv] * 2
        out = np.zeros(sum(sizes) * dnx * dnz)
        n = lib().lho_cond_get(self.h, _p(out) if out.size else None, dims.ctypes.data)
        res, off = {}, 0
        for name, nj in zip(self.COND_ROWS, sizes):
            res[name] = out[off:off + nj * dnx * dnz].reshape(nj, dnz, dnx)
            off += nj * dnx * dnz
        return n, res

    def spectra(self):
        nc = self.nz * self.nkx
        o = [np.zeros((self.nyu, nc)), np.zeros((self.nyv, nc)), np.zeros((self.nyu, nc)),
             np.zeros((self.nyu, nc)), np.zeros((self.nyp, nc))]
        lib().lho_spectra_get(self.h, *[_p(x) for x in o])
        return o
