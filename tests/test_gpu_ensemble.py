"""Ensembles: several independent solvers of different sizes advanced by one
graph launch per RK3 step give exactly the results of stepping them alone."""
import numpy as np
import pytest

from tests.helpers import SMALL, projected_ic

pytestmark = pytest.mark.gpu

MEMBERS = [
    dict(SMALL),
    dict(SMALL, ngalx=36, ngalz=36, ny=41, dsty=6, ntilex=6, ntilez=6, dstx=2, dstz=2, posth=0.1, Re=3500.0),
    dict(SMALL, ngalx=48, ngalz=24, ny=33, dsty=4, ntilex=8, ntilez=4, dstx=2, dstz=3, Re=2000.0),
]


def _member(oracle_mod, cfg, seed):
    import littleharsh_gb300 as lh
    o = oracle_mod.Oracle(**cfg)
    f = projected_ic(o, seed=seed)
    dt = o.cfl_dt(0.5)
    s = lh.Solver(lh.Config(**cfg))
    s.set_fields(*f)
    s.set_time(0.0, dt, 0.0)
    return s, f, dt


def test_ensemble_matches_members_stepped_alone(oracle_mod):
    import littleharsh_gb300 as lh
    alone, ens = [], []
    for i, cfg in enumerate(MEMBERS):
        a, f, dt = _member(oracle_mod, cfg, seed=10 + i)
        a.step(3)
        alone.append(a)
        b = lh.Solver(lh.Config(**cfg))
        b.set_fields(*f)
        b.set_time(0.0, dt, 0.0)
        ens.append(b)
    e = lh.Ensemble(ens)
    ms = e.step(1)
    ms += e.step(2)
    assert ms > 0
    for a, b in zip(alone, ens):
        for x, y in zip(a.get_fields(), b.get_fields()):
            np.testing.assert_array_equal(x, y)
        assert abs(a.time()["t"] - b.time()["t"]) < 1e-15
    e.close()
