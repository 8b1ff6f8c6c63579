"""Error paths of the C ABI on a device: calls out of order, a bad substage index and a transform length that
does not factor into 2, 3 and 4 return their codes (LH_ESTATE -6, LH_EINVAL -1, LH_EFFT -3) with a reason, and
a handle stays usable after a refused call.  A non-finite field and a divergence above maxerr return
LH_ENUMERIC (-7); the failures are made on the host (a NaN uploaded into the field, a bound below round-off)."""
import numpy as np
import pytest

from tests.helpers import SMOOTH

pytestmark = pytest.mark.gpu


def _laminar(s):
    g = s.grid
    u1 = s.zeros("u")
    inside = np.abs(g["yu"]) < 1.0
    u1[:, 0, 0] = np.where(inside, 1.5 * (1.0 - g["yu"] ** 2), 0.0)
    return u1, s.zeros("v"), s.zeros("u"), s.zeros("p")


def test_calls_out_of_order_are_refused():
    import littleharsh_gb300 as lh
    s = lh.Solver(lh.Config(**SMOOTH))
    with pytest.raises(lh.LhError, match=r"\(-6\)"):
        s.step(1)  # no fields
    s.set_fields(*_laminar(s))
    with pytest.raises(lh.LhError, match=r"\(-6\)"):
        s.step(1)  # no dt
    s.set_time(0.0, 1e-3, 0.0)
    s.step(2)  # the refused calls left the handle usable
    assert np.all(np.isfinite(s.get_fields()[0])) and s.divmax() < 1e-12
    s.close()


def test_bad_substage_index_is_refused():
    import littleharsh_gb300 as lh
    s = lh.Solver(lh.Config(**SMOOTH))
    s.set_fields(*_laminar(s))
    s.set_time(0.0, 1e-3, 0.0)
    for k in (0, 4):
        with pytest.raises(lh.LhError, match=r"\(-1\)"):
            s.substage(k)
    s.substage(1)
    s.step(1)
    assert np.all(np.isfinite(s.get_fields()[0]))
    s.close()


def test_transform_length_without_radix_2_3_4_is_refused():
    import littleharsh_gb300 as lh
    with pytest.raises(lh.LhError, match=r"\(-3\)"):
        lh.Solver(lh.Config(**dict(SMOOTH, ngalx=30)))  # 30 = 2 x 3 x 5


def _seeded(s, seed=5):
    from littleharsh_gb300.initial import initial_field
    g = s.grid
    s.set_fields(*initial_field(g["yu"], g["yv"], s.nz, s.nkx, s.nyp, seed=seed))
    s.project()
    s.set_time(0.0, s.cfl_dt(0.5), 0.0)


def test_non_finite_field_is_reported():
    """A NaN uploaded into one point of u (host-side injection) reaches the pressure solve within the step, which
    flags it on the device; lh_rk3_step returns LH_ENUMERIC (-7).  Fresh fields clear the flag; the mean
    pressure gradient, which the failed steps' flow-rate correction also spoilt, is set again with the time."""
    import littleharsh_gb300 as lh
    from tests.helpers import SMALL
    s = lh.Solver(lh.Config(**SMALL))
    _seeded(s)
    good = s.get_fields()
    t = s.time()
    s.step(2)
    assert s.monitor()["err_bits"] == 0
    bad = [f.copy() for f in good]
    bad[0][5, 3, 2] = np.nan
    s.set_fields(*bad)
    with pytest.raises(lh.LhError, match=r"\(-7\)") as ei:
        s.step(3)
    assert ei.value.code == lh.LH_ENUMERIC and "non-finite" in str(ei.value)
    assert s.monitor()["err_bits"] == 1
    bad = [f.copy() for f in good]
    bad[3][4, 1, 1] = np.inf  # pressure too
    s.set_fields(*bad)
    with pytest.raises(lh.LhError, match=r"\(-7\)"):
        s.step(1)
    assert not np.isfinite(s.time()["mpgx"])
    s.set_fields(*good)
    s.set_time(t["t"], t["dt"], t["mpgx"], t["QxT"])
    s.step(2)
    assert s.monitor()["err_bits"] == 0 and np.all(np.isfinite(s.get_fields()[0]))
    s.close()


def test_divergence_monitor_against_maxerr():
    """The monitor checks max |div| (the reference's `error`) against maxerr after every block of steps: a
    bound below round-off is exceeded after the first block, input.in's maxerr = 1e-8 is not."""
    import littleharsh_gb300 as lh
    from tests.helpers import SMALL
    s = lh.Solver(lh.Config(**SMALL))
    _seeded(s)
    assert s.monitor()["divmax"] == -1.0
    s.set_monitor(1e-8, 2)
    s.step(5)  # blocks of 2, 2, 1
    d = s.monitor()["divmax"]
    assert 0.0 <= d < 1e-10
    assert abs(d - s.divmax()) <= 1e-16
    t0 = s.time()["t"]
    s.set_monitor(1e-30, 3)
    with pytest.raises(lh.LhError, match=r"\(-7\)") as ei:
        s.step(7)
    assert "maxerr" in str(ei.value)
    assert abs(s.time()["t"] - (t0 + 3 * s.time()["dt"])) < 1e-12  # stopped after the first block
    s.set_monitor(0.0, 0)  # off
    s.step(2)
    s.close()


def test_ensemble_reports_a_non_finite_member():
    import littleharsh_gb300 as lh
    from tests.helpers import SMALL
    a, b = lh.Solver(lh.Config(**SMALL)), lh.Solver(lh.Config(**SMOOTH))
    _seeded(a, 1)
    _seeded(b, 2)
    f = b.get_fields()
    f[2][3, 2, 1] = np.nan
    b.set_fields(*f)
    e = lh.Ensemble([a, b])
    with pytest.raises(lh.LhError, match="member 1"):
        e.step(1)
    e.close()
    a.close()
    b.close()
