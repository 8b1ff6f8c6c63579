"""Analytic self-pinning of the oracle's RK3 step (the reference has no tests;
these pin the restatement to the equations it solves)."""
import numpy as np
import pytest

from tests.helpers import SMALL, SMOOTH, projected_ic, rel_l2


def _smooth(po, **kw):
    cfg = dict(SMOOTH)
    cfg.update(kw)
    return po.Oracle(**cfg)


def test_discrete_laminar_state_is_steady(oracle_mod):
    """Constant pressure gradient: the discrete Poiseuille profile (solution of
    L_y u = Re*mpgx with the ghost-point rows) is a fixed point of the step."""
    o = _smooth(oracle_mod, flag_ctpress=1, ny=49)
    g = o.grid()
    nyu = o.nyu
    Re, mpgx = 2800.0, -2.0 / 2800.0
    A = np.zeros((nyu, nyu))
    rhs = np.zeros(nyu)
    gw = g["gw"]  # gw[c, band]
    A[0, 0], A[0, 1] = 1.0, gw[0, 1]
    for j in range(1, nyu - 1):
        A[j, j - 1:j + 2] = g["dyu2i"][j]
        rhs[j] = Re * mpgx
    A[-1, -2], A[-1, -1] = gw[1, 1], 1.0
    us = np.linalg.solve(A, rhs)
    u1 = o.zeros("u")
    u1[:, 0, 0] = us
    o.set_fields(u1, o.zeros("v"), o.zeros("u"), o.zeros("p"))
    o.set_scalars(0.0, 0.01, mpgx)
    o.step(5)
    f = o.get_fields()
    assert rel_l2(f[0], u1) < 1e-12
    assert np.abs(f[1]).max() < 1e-14 and np.abs(f[2]).max() < 1e-14


@pytest.mark.parametrize("mode", ["mean_u", "w_kx1"])
def test_viscous_decay_rate(oracle_mod, mode):
    """A (0,0) u profile and a (kx=1, kz=0) w profile are linear: they decay by
    diffusion at (k^2 + (pi/2)^2)/Re for the lowest wall mode."""
    o = _smooth(oracle_mod, flag_ctpress=1, ny=129, dyq=1.5, Re=100.0)
    g = o.grid()
    yu = g["yu"]
    prof = np.cos(np.pi * yu / 2.0)
    u1, u3 = o.zeros("u"), o.zeros("u")
    if mode == "mean_u":
        u1[:, 0, 0] = prof
        k2 = 0.0
    else:
        u3[:, 0, 1] = prof
        k2 = 1.0
    o.set_fields(u1, o.zeros("v"), u3, o.zeros("p"))
    dt, n = 0.01, 50
    o.set_scalars(0.0, dt, 0.0)
    o.step(n)
    f = o.get_fields()
    c = f[0][:, 0, 0] if mode == "mean_u" else f[2][:, 0, 1]
    mid = slice(o.nyu // 4, 3 * o.nyu // 4)
    rate = -np.log(np.abs(c[mid]).sum() / np.abs(prof[mid]).sum()) / (n * dt)
    expect = (k2 + (np.pi / 2) ** 2) / 100.0
    assert abs(rate - expect) / expect < 5e-3


def test_projection_and_steps_keep_divergence_at_roundoff(oracle_mod):
    o = oracle_mod.Oracle(**SMALL)
    u1, u2, u3, p = projected_ic(o)
    assert o.divmax() < 1e-11
    o.set_scalars(0.0, o.cfl_dt(0.5), 0.0, o.flowrate())
    o.step(5)
    assert o.divmax() < 1e-11


def test_flow_rate_is_held(oracle_mod):
    """Constant flow rate (meanflow_ctU): Q stays at its initial value to the
    accuracy the reference's correction reaches."""
    o = oracle_mod.Oracle(**SMALL)
    projected_ic(o)
    Q0 = o.flowrate()
    o.set_scalars(0.0, o.cfl_dt(0.5), 0.0, Q0)
    for _ in range(10):
        o.step(1)
        assert abs(o.flowrate() - Q0) < 1e-6 * Q0
    assert o.scalars()["mpgx"] < 0.0


def test_canopy_forcing_damps_solid_points(oracle_mod):
    """Velocity at the solid points of the processed planes is driven towards 0."""
    o = oracle_mod.Oracle(**SMALL)
    projected_ic(o)
    o.set_scalars(0.0, o.cfl_dt(0.5), 0.0, o.flowrate())
    o.step(20)
    pu, mu, pv, mv = o.ib()
    f = o.get_fields()
    solid, fluid = [], []
    for q, j in enumerate(pu):
        phys = o.to_phys(f[0][j - o.sz.ju0])
        solid.append(np.abs(phys[mu[q] == 1]).max())
    mid = o.nyu // 2
    fluid = np.abs(o.to_phys(f[0][mid])).mean()
    assert max(solid) < 0.05 * fluid


def test_canopy_mask_is_tile_periodic(oracle_mod):
    o = oracle_mod.Oracle(**SMALL)
    pu, mu, pv, mv = o.ib()
    dnx, dnz = o.ngx // 4, o.ngz // 4
    m = mu[0]
    for ix in range(4):
        for iz in range(4):
            np.testing.assert_array_equal(m[iz * dnz:(iz + 1) * dnz, ix * dnx:(ix + 1) * dnx], m[:dnz, :dnx])
    assert m[:dnz, :dnx].sum() == 2 * 2
    # processed planes: u stems between wall and tips on both sides, v without the walls
    assert list(pu) == [-3, -2, -1, 0, 33, 34, 35, 36]
    assert list(pv) == [-3, -2, -1, 33, 34, 35]
