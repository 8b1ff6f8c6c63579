"""GPU parity with variable-resolution bands (Ngalx1 != Ngalx2): the CUDA step
against the oracle on the same inputs, as for one resolution.

The perturbation reaches kx, kz index 12, past the middle band's 8, so the
short columns carry energy from the start.
"""
import numpy as np
import pytest

from tests.helpers import projected_ic, rel_l2

pytestmark = pytest.mark.gpu

BAND48 = dict(Re=2800.0, alp=1.0, bet=2.0, ngalx=48, ngalz=48, ny=49, dyq=13.6, ppp=5, geometry_type=3, posth=0.2,
              dsty=8, dstx=1, dstz=2, ntilex=12, ntilez=6, flag_ctpress=0, ngalx2=24, ngalz2=24)
BAND_SMOOTH = dict(BAND48, geometry_type=0, posth=0.0, dsty=0, dstx=1, dstz=1, ntilex=1, ntilez=1)
SUBSTAGE_TOL = 1e-11
STEP10_TOL = 1e-10


def _pair(po, cfg, precision=0, seed=3):
    import littleharsh_gb300 as lh
    o = po.Oracle(**cfg)
    u1, u2, u3, p = projected_ic(o, seed=seed, kmax=12)
    dt = o.cfl_dt(0.5)
    Q = o.flowrate()
    o.set_fields(u1, u2, u3, p)
    o.set_scalars(0.0, dt, 0.0, Q)
    s = lh.Solver(lh.Config(**cfg), precision=precision)
    s.set_fields(u1, u2, u3, p)
    s.set_time(0.0, dt, 0.0, Q)
    return o, s


def _cmp(o, s, tol, what):
    for name, a, b in zip(("u1", "u2", "u3", "p"), s.get_fields(), o.get_fields()):
        e = rel_l2(a, b)
        assert e < tol, f"{what} {name}: rel L2 {e:.3e}"


@pytest.mark.parametrize("cfg", [BAND48, BAND_SMOOTH], ids=["canopy48_24", "smooth48_24"])
@pytest.mark.parametrize("upto", [1, 2, 3, 4, 5])
def test_band_substage_stages(oracle_mod, cfg, upto):
    o, s = _pair(oracle_mod, cfg)
    o.substage(1, upto)
    s.substage(1, upto)
    if upto <= 2:
        for name, a, b in zip(("r1", "r2", "r3"), s.get_rhs(), o.get_rhs()):
            assert rel_l2(a, b) < SUBSTAGE_TOL, f"stage {upto} {name}: {rel_l2(a, b):.3e}"
        for name, a, b in zip(("n1", "n2", "n3"), s.get_nonlinear(), o.get_nonlinear()):
            assert rel_l2(a, b) < SUBSTAGE_TOL, f"stage {upto} {name}: {rel_l2(a, b):.3e}"
    else:
        _cmp(o, s, SUBSTAGE_TOL, f"stage {upto}")


def test_band_ten_steps_fp64(oracle_mod):
    o, s = _pair(oracle_mod, BAND48)
    assert abs(s.cfl_dt(0.5) - o.cfl_dt(0.5)) < 1e-12 * o.cfl_dt(0.5)
    o.step(10)
    s.step(10)
    _cmp(o, s, STEP10_TOL, "10 steps")
    assert s.divmax() < 1e-9
    assert abs(s.time()["mpgx"] - o.scalars()["mpgx"]) < 1e-9 * abs(o.scalars()["mpgx"])


def test_band_statistics(oracle_mod):
    """Plane sums of the middle band's planes run over its own (coarser) points."""
    o, s = _pair(oracle_mod, BAND48)
    o.step(2)
    s.step(2)
    o.stats_accumulate()
    s.stats_accumulate()
    n, st = s.stats_flush()
    no, so = o.stats()
    assert n == no == 1
    ny = {"u": s.nyu, "v": s.nyv, "p": s.nyp}
    for r, (name, grid) in enumerate(zip(s.STAT_ROWS, "uuvvuuppuuvvv")):
        a, b = st[name], so[r, :ny[grid]]
        tol = 1e-11 * np.abs(b).max() + 1e-13 * s.ngx * s.ngz
        assert np.abs(a - b).max() < tol, f"{name}: {np.abs(a - b).max():.3e} >= {tol:.3e}"
    o.cond_accumulate()
    s.cond_accumulate()
    n, cg = s.cond_flush()
    no, co = o.cond()
    for name in s.COND_ROWS:
        a, b = cg[name], co[name]
        tol = 1e-11 * np.abs(b).max() + 1e-13 * s.ngx * s.ngz
        assert np.abs(a - b).max() < tol, name


def test_band_mixed_precision_close(oracle_mod):
    import littleharsh_gb300 as lh
    o, s = _pair(oracle_mod, BAND48, precision=lh.PREC_MIXED)
    o.step(10)
    s.step(10)
    for a, b in zip(s.get_fields(), o.get_fields()):
        assert rel_l2(a, b) < 1e-4


def test_two_row_product_pass_with_bands(oracle_mod, monkeypatch):
    """The mixed form's two-row product pass on every band (the fine bands' 48-point rows and the middle
    band's 24-point rows): bit for bit the one-row steps."""
    import littleharsh_gb300 as lh
    o, s0 = _pair(oracle_mod, BAND48, precision=lh.PREC_MIXED)
    sols = []
    for rows in ("1", "2"):
        monkeypatch.setenv("LH_XROWS", rows)
        s = lh.Solver(lh.Config(**BAND48), precision=lh.PREC_MIXED)
        assert s.launch_shapes()["xrows"] == int(rows)
        s.set_fields(*s0.get_fields())
        tm = s0.time()
        s.set_time(0.0, tm["dt"], 0.0, tm["QxT"])
        s.step(3)
        sols.append(s)
    for a, b in zip(sols[0].get_fields(), sols[1].get_fields()):
        np.testing.assert_array_equal(a, b)
