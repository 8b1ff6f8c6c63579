"""The C host driver (littleharsh_gb300/driver/lh_driver.c): the reference's main program order
(littleharsh.f90:63-208) through the C ABI alone, compiled here with the system C compiler against
include/littleharsh.h.

Without a GPU: it compiles and links against the library, and refuses bad command lines.  On a GPU: from a
restart file written by the Python path (flag_init = 1 of an input.in derived from the reference's own), it
runs lh_read_input -> lh_setup_grid -> lh_setup_canopy -> lh_init -> lh_read_restart -> lh_cfl_dt ->
lh_set_time -> lh_set_monitor -> lh_rk3_step -> statistics -> lh_write_restart / lh_write_stats /
lh_write_spectra; the Python path makes the same calls through ctypes, and every file the two write is equal
byte for byte.  The parabolic start (flag_init = 3, mblock_ini_parabolic_profile) runs too.
"""
import os
import subprocess

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")

# input.in lines (1-based) of the reference's file and the values of a 24 x 24 x 42 canopy case
SMALL_INPUT = {10: "Re=       2800.d0", 15: "Ngalx1=        24", 16: "Ngalx2=        24", 17: "Ngalz1=        24",
               18: "Ngalz2=        24", 19: "ny    =        33", 20: "dyq   =     13.6d0", 21: "pp    =         5",
               34: "CFL   =     0.5d0", 35: "nwrite=        10", 36: "flpress    =    0", 38: "mpgx  =     0.d0",
               43: "maxerr=     1.d-8", 44: "maxt  =  2000.0d0", 50: "type  =         3", 55: "ntilex=         4",
               56: "ntilez=         4", 57: "posth =     0.2d0", 62: "dsty  =         4", 63: "dstx  =         2",
               64: "dstz  =         2"}


def _input(tmp_path, flag_init, dirin, extra=None):
    lines = open(os.path.join(GOLDEN, "input.in")).read().split("\n")
    rep = dict(SMALL_INPUT)
    rep[24] = f"flgin =         {flag_init}"
    rep[28] = "fnmeb =u1_start.dat"
    rep[30] = f"dirin ={dirin}/"
    rep[31] = f"dirout={tmp_path}/"
    rep.update(extra or {})
    for k, v in rep.items():
        lines[k - 1] = v
    p = tmp_path / "input.in"
    p.write_text("\n".join(lines))
    return str(p)


@pytest.fixture(scope="module")
def driver():
    from littleharsh_gb300 import build
    return build.build_driver()


def test_driver_builds_and_refuses_bad_arguments(driver):
    r = subprocess.run([driver], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr
    r = subprocess.run([driver, "input.in", "--bogus"], capture_output=True, text=True)
    assert r.returncode == 2 and "unknown argument" in r.stderr
    r = subprocess.run([driver, "/nonexistent/input.in"], capture_output=True, text=True)
    assert r.returncode == 1 and "lh_read_input" in r.stderr


@pytest.mark.gpu
def test_driver_equals_the_python_path(driver, tmp_path):
    import littleharsh_gb300 as lh
    from littleharsh_gb300.initial import initial_field
    din = tmp_path / "in"
    din.mkdir()
    inp_path = _input(tmp_path, 1, din)
    inp = lh.read_input(inp_path)
    # the start field, written by the Python path in the restart format
    s = lh.Solver(inp)
    g = s.grid
    s.set_fields(*initial_field(g["yu"], g["yv"], s.nz, s.nkx, s.nyp, seed=13))
    s.project()
    s.write_restart(str(din), "_start.dat")
    s.close()
    # the C driver
    cdir = tmp_path / "c"
    cdir.mkdir()
    r = subprocess.run([driver, inp_path, "--steps", "5", "--out", str(cdir), "--name", "_end.dat"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr + r.stdout
    assert "done: 5 steps" in r.stdout
    # the Python path, the same calls in the same order
    pdir = tmp_path / "py"
    pdir.mkdir()
    p = lh.Solver(inp)
    p.read_restart(str(din), "_start.dat")
    dt = p.cfl_dt(inp.CFL)
    p.set_time(0.0, dt, inp.mpgx, -1.0)
    p.set_monitor(inp.maxerr, inp.nwrite)
    p.step(5)
    p.stats_accumulate()
    p.cond_accumulate()
    p.spectra_accumulate()
    tm = p.time()
    p.set_time(tm["t"], p.cfl_dt(inp.CFL), tm["mpgx"], -1.0)
    p.write_restart(str(pdir), "_end.dat", iteration=5)
    p.write_stats(str(pdir / "stats_end.dat"), iteration=5)
    p.write_spectra(str(pdir), "_end.dat", iteration=5)
    names = sorted(os.listdir(pdir))
    assert names == sorted(os.listdir(cdir)) and len(names) == 10
    for n in names:
        a, b = (cdir / n).read_bytes(), (pdir / n).read_bytes()
        assert a == b, f"{n} differs"
    p.close()


@pytest.mark.gpu
def test_driver_parabolic_start(driver, tmp_path):
    """flag_init = 3: the parabolic profile of mblock_ini_parabolic_profile (u1(0,0) = Re mpgx (y^2 - 1) / 2,
    u2, u3, p constant (0,0) modes) at a constant pressure gradient, stepped to maxt."""
    import littleharsh_gb300 as lh
    inp_path = _input(tmp_path, 3, tmp_path, {36: "flpress    =    1", 38: "mpgx  =  -1.0d-3", 44: "maxt  =     0.02"})
    r = subprocess.run([driver, inp_path, "--name", "_par.dat"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr + r.stdout
    s = lh.Solver(lh.read_input(inp_path))
    t, it = s.read_restart(str(tmp_path), "_par.dat")
    assert t >= 0.02 and it > 0
    u1 = s.get_fields()[0]
    assert np.all(np.isfinite(u1)) and abs(u1[s.nyu // 2, 0, 0].real) > 0.5
    s.close()
