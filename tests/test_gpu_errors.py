"""Error paths of the C ABI on a device: calls out of order, a bad substage index and a transform length that
does not factor into 2, 3 and 4 return their codes (LH_ESTATE -6, LH_EINVAL -1, LH_EFFT -3) with a reason, and
a handle stays usable after a refused call."""
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
