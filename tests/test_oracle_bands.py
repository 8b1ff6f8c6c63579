"""The oracle with variable-resolution bands (Ngalx1 != Ngalx2, start.f90:95-118,1037-1145).

Long columns (the middle band's modes) span every level; short columns (the
other modes of the wall bands) live only between their band's end rows, which
carry the reference's band-edge gridweighting (start.f90:497-503); the middle
band's planes are transformed at its own resolution.  These tests pin the
properties that follow from that structure.
"""
import numpy as np
import pytest

SMALL = dict(Re=2800.0, alp=1.0, bet=2.0, ngalx=48, ngalz=48, ny=49, dyq=13.6, ppp=5, geometry_type=3, posth=0.2,
             dsty=8, dstx=1, dstz=2, ntilex=12, ntilez=6, flag_ctpress=0)
BANDS = dict(ngalx2=24, ngalz2=24)


def make(oracle_mod, cfg, **kw):
    return oracle_mod.Oracle(**cfg, nthreads=4, **kw)


def long_mask(o, nkx2, nz2):
    kk = np.arange(o.nz)
    kz = np.where(kk < o.nz // 2, kk, kk - o.nz)
    return (np.arange(o.nkx)[None, :] < nkx2) & (kz[:, None] >= -(nz2 // 2)) & (kz[:, None] < nz2 // 2)


def seeded(o, seed=1, amp=0.1, kmax=8):
    from littleharsh_gb300.initial import initial_field
    g = o.grid()
    o.set_fields(*initial_field(g["yu"], g["yv"], o.nz, o.nkx, o.nyp, seed=seed, amp=amp, kmax=kmax))
    o.set_scalars(0.0, 1.0, 0.0)
    o.project()
    o.set_scalars(0.0, o.cfl_dt(0.5), 0.0, o.flowrate())


def test_equal_resolutions_are_one_band(oracle_mod):
    a = make(oracle_mod, SMALL)
    b = make(oracle_mod, SMALL, ngalx2=SMALL["ngalx"], ngalz2=SMALL["ngalz"])
    for o in (a, b):
        seeded(o)
        o.step(3)
    for x, y in zip(a.get_fields(), b.get_fields()):
        np.testing.assert_array_equal(x, y)


def test_band_limits(oracle_mod):
    o = make(oracle_mod, SMALL, **BANDS)
    N = np.array(o.sz.N)  # N[r][b] = N(r+1, b)
    assert N[0][1] == 32 and N[0][2] == 16 and N[0][3] == 32  # modes per band in x
    assert N[1][1] == 32 and N[1][2] == 16
    assert N[3][0] < N[3][1] < N[3][2] < N[3][3]  # u-grid band limits
    assert N[2][1] == N[3][1] - 1  # v's first band ends one plane below u's


def test_short_columns_stay_in_their_bands_and_the_step_is_divergence_free(oracle_mod):
    o = make(oracle_mod, SMALL, **BANDS)
    seeded(o, kmax=12)  # the perturbation reaches past the middle band's modes
    Q0 = o.flowrate()
    N = np.array(o.sz.N)
    lng = long_mask(o, 9, 16)
    yuj = np.arange(o.nyu) + o.sz.ju0
    yvj = np.arange(o.nyv) + o.sz.jv0
    ypj = np.arange(o.nyp) + o.sz.jp0
    for _ in range(3):
        o.step(4)
        u1, u2, u3, p = o.get_fields()
        assert o.divmax() < 1e-12
        assert abs(o.flowrate() - Q0) < 1e-7 * abs(Q0)
        # short modes are zero strictly inside the middle band (and on its planes)
        mid_u = (yuj > N[3][1] + 1) & (yuj < N[3][2])
        mid_v = (yvj > N[2][1] + 1) & (yvj < N[2][2])
        mid_p = (ypj > N[3][1]) & (ypj <= N[3][2])
        for f, m in ((u1, mid_u), (u3, mid_u), (u2, mid_v), (p, mid_p)):
            assert np.abs(f[m][:, ~lng]).max() == 0.0
        # v of the short columns vanishes on their band-edge rows
        for j in (N[2][1] + 1, N[2][2]):
            assert np.abs(u2[j - o.sz.jv0][~lng]).max() == 0.0
        # and they carry energy in the wall bands
        assert np.abs(u1[~mid_u][:, ~lng]).max() > 1e-6


def test_laminar_profile_is_a_fixed_point_with_bands(oracle_mod):
    cfg = dict(SMALL, geometry_type=0, dsty=0)
    o = make(oracle_mod, cfg, **BANDS)
    g = o.grid()
    u1 = o.zeros("u")
    inside = np.abs(g["yu"]) < 1.0
    u1[:, 0, 0] = np.where(inside, 1.5 * (1.0 - g["yu"] ** 2), 0.0)
    o.set_fields(u1, o.zeros("v"), o.zeros("u"), o.zeros("p"))
    o.set_scalars(0.0, 1.0, 0.0)
    o.project()
    ref = o.get_fields()[0].copy()
    o.set_scalars(0.0, 0.01, 0.0, o.flowrate())
    o.step(5)
    # the discrete Poiseuille profile under the constant flow rate drifts only by round-off and the
    # reference's one-index flow-rate sum; no other mode is excited
    u1b = o.get_fields()[0]
    assert np.abs(np.delete(u1b.reshape(o.nyu, -1), 0, axis=1)).max() < 1e-13
    assert np.abs(u1b[:, 0, 0] - ref[:, 0, 0]).max() < 1e-3


def test_middle_band_planes_use_their_own_resolution(oracle_mod):
    """x-Nyquist of the middle band squared: on its 3/2 plane (24 points) kx = 16 aliases onto -8, a kept
    mode of the middle band; on the wall bands' plane (48 points) it is a separate mode.  The product of a
    middle-level field therefore carries the aliased part, which a wall-band plane would not produce."""
    cfg = dict(SMALL, geometry_type=0, dsty=0)
    o = make(oracle_mod, cfg, **BANDS)
    N = np.array(o.sz.N)
    u1 = o.zeros("u")
    jm = (N[3][1] + N[3][2]) // 2 - o.sz.ju0  # a level of the middle band
    jw = (N[3][0] + N[3][1]) // 2 - o.sz.ju0  # a level of the bottom band
    for jj in (jm, jw):
        u1[jj, 0, 8] = 0.5  # kx index 8 = the middle band's x-Nyquist (N(1,2)/2)
    phys_m = o.to_phys(u1[jm])
    assert np.isfinite(phys_m).all()
    o.set_fields(u1, o.zeros("v"), o.zeros("u"), o.zeros("p"))
    o.set_scalars(0.0, 1e-3, 0.0, 0.0)
    o.substage(1, 1)
    n1 = o.get_nonlinear()[0]
    # d(uu)/dx at the middle level: the aliased kx = 16 -> -8 product lands on kx index 8
    assert abs(n1[jm, 0, 8]) > 1e-3
    # at the bottom-band level the same field's square has no kx = 8 part
    assert abs(n1[jw, 0, 8]) < 1e-14


def test_real_field_except_the_middle_bands_lone_mode(oracle_mod):
    """The physical field stays real: on the kx = 0 line every kz mode is the conjugate of its -kz partner,
    except the middle band's own -N2/2 mode, whose +N2/2 partner is a short column (zero on the middle band's
    levels) -- the same as the lone -N2/2 mode of one resolution."""
    from littleharsh_gb300.initial import initial_field
    o = make(oracle_mod, SMALL, **BANDS)
    g = o.grid()
    o.set_fields(*initial_field(g["yu"], g["yv"], o.nz, o.nkx, o.nyp, seed=3, kmax=max(o.nkx, o.nz // 2)))
    o.set_scalars(0.0, 1.0, 0.0)
    o.project()
    o.set_scalars(0.0, o.cfl_dt(0.5), 0.0, o.flowrate())
    o.step(3)
    nz, lone = o.nz, (2 * BANDS["ngalz2"] // 3) // 2
    for f in o.get_fields():
        line = f[:, :, 0]
        kk = np.array([k for k in range(1, nz // 2) if k != lone])
        assert np.abs(line[:, nz - kk] - np.conj(line[:, kk])).max() == 0.0
        # the lone mode's pair is not symmetric on the middle band's levels
        assert np.abs(line[:, nz - lone] - np.conj(line[:, lone])).max() > 0.0
