"""Ensembles: several independent solvers of different sizes advanced by one
graph launch per RK3 step give exactly the results of stepping them alone, in
both modes: batched launches (one per kernel kind and slot of the substage,
covering every member) and one stream per member.  The batched mode is also
checked at the sizes of configuration 4's three replica classes, with canopy
pitches and heights of its set, in FP64 and in the mixed form, and its
launches per step do not depend on the member count."""
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


@pytest.mark.parametrize("mode", [0, 1], ids=["streams", "batched"])
def test_ensemble_matches_members_stepped_alone(oracle_mod, mode):
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
    e = lh.Ensemble(ens, mode=mode)
    ms = e.step(1)
    ms += e.step(2)
    assert ms > 0
    assert e.info()["mode"] == ("batched" if mode else "streams")
    for a, b in zip(alone, ens):
        for x, y in zip(a.get_fields(), b.get_fields()):
            np.testing.assert_array_equal(x, y)
        assert abs(a.time()["t"] - b.time()["t"]) < 1e-15
    e.close()


def _config4_members(n_per_class):
    """Configuration 4's replica classes (144^2 x 154, 192^2 x 226, 288^2 x 306 points), n_per_class of each."""
    from littleharsh_gb300.workloads import ensemble_configs
    cfgs = ensemble_configs()
    out = []
    for lo in (0, 6, 12):
        out += cfgs[lo:lo + n_per_class]
    return out


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_batched_ensemble_at_configuration4_sizes(precision):
    """Bit for bit against the members stepped alone, also after the dt of one member changed between steps."""
    import littleharsh_gb300 as lh
    from littleharsh_gb300.initial import initial_field
    cfgs = _config4_members(1) + [_config4_members(2)[1]]
    alone, ens = [], []
    for i, cfg in enumerate(cfgs):
        pair = []
        for _ in range(2):
            s = lh.Solver(lh.Config(**cfg), precision=precision)
            g = s.grid
            s.set_fields(*initial_field(g["yu"], g["yv"], s.nz, s.nkx, s.nyp, seed=40 + i))
            s.project()
            s.set_time(0.0, s.cfl_dt(0.5), 0.0)
            pair.append(s)
        alone.append(pair[0])
        ens.append(pair[1])
    e = lh.Ensemble(ens, mode=lh.ENS_BATCHED)
    e.step(2)
    for a in alone:
        a.step(2)
    # a new dt for one member: its launches are captured again
    for s in (alone[0], ens[0]):
        t = s.time()
        s.set_time(t["t"], 0.9 * t["dt"], t["mpgx"])
    e.step(1)
    for a in alone:
        a.step(1)
    info = e.info()
    assert info["mode"] == "batched"
    for a, b in zip(alone, ens):
        for x, y in zip(a.get_fields(), b.get_fields()):
            np.testing.assert_array_equal(x, y)
    # the launches per step do not grow with the members: an ensemble of one member per grid class has as many
    e2 = lh.Ensemble(ens[:3], mode=lh.ENS_BATCHED)
    e2.step(1)
    assert e2.info()["launches_per_step"] == info["launches_per_step"]
    e2.close()
    e.close()
    for s in alone + ens:
        s.close()
