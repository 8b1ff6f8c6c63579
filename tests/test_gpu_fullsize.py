"""Configuration 2 at full size (576 x 576 points, 450 u levels, 48 x 24 posts; ~19 GB per solver).

Against the oracle on the same projected seeded field: two FP64 RK3 steps within 1e-10 relative L2 on u, v, w
and p, the mixed form within 1e-4 (the oracle takes a few seconds per step on the host's cores at this size);
the same for one step on the warm start's fine grid (configuration 5: 576 x 576 points, 385 levels).
Besides, properties that do not depend on the size hold after a few RK3 steps:

* the projection leaves the field divergence free (max |div| at round-off);
* the flow-rate correction holds the flow rate at its target;
* the field stays real: on the kx = 0 line every kz mode is the conjugate of its -kz partner (to round-off in
  FP64, to FP32 rounding in the mixed form);
* the mixed form stays within FP32-level distance of FP64 from the same start;
* the graph-replayed step equals the same substages launched one by one, bit for bit;
* the plane statistics' mean and mean square equal the (0,0) mode and Parseval's sum of the downloaded spectra;
* the same with the reference's variable-resolution bands (middle band 384 x 384 points).
"""
import numpy as np
import pytest

from tests.helpers import rel_l2

pytestmark = pytest.mark.gpu


def _start(cfg, precision, seed=1):
    import littleharsh_gb300 as lh
    from littleharsh_gb300.initial import initial_field
    s = lh.Solver(lh.Config(**cfg), precision=precision)
    g = s.grid
    s.set_fields(*initial_field(g["yu"], g["yv"], s.nz, s.nkx, s.nyp, seed=seed, kmax=max(s.nkx, s.nz // 2)))
    s.project()
    s.set_time(0.0, s.cfl_dt(0.5), 0.0)
    return s


def _hermitian_error(f, lone=()):
    """max |f(kx=0, -kz) - conj f(kx=0, kz)| over the modes with a partner, relative to max |f|.  The fine
    set's -N2/2 mode has no partner; with bands neither has the middle band's own -N2/2 mode (its +N2/2 partner
    is a short column, zero on the middle band's levels), so `lone` leaves that pair out, as the oracle's
    banded step does."""
    nz = f.shape[1]
    kk = np.array([k for k in range(1, nz // 2) if k not in lone])
    line = f[:, :, 0]
    return float(np.abs(line[:, nz - kk] - np.conj(line[:, kk])).max() / max(np.abs(f).max(), 1e-300))


def _check_properties(s, what, herm_tol=1e-12, lone=()):
    """herm_tol: FP64 keeps the symmetry to round-off; the mixed form's FP32 transforms compute kz and -kz by
    different paths, so its symmetry holds to FP32 rounding."""
    q = s.time()
    assert s.divmax() < 1e-9, f"{what}: max |div| {s.divmax():.3e}"
    assert abs(q["Qx"] - q["QxT"]) < 1e-7 * abs(q["QxT"]), f"{what}: flow rate {q['Qx']} vs {q['QxT']}"
    for name, f in zip(("u1", "u2", "u3", "p"), s.get_fields()):
        assert np.all(np.isfinite(f)), f"{what} {name}: not finite"
        e = _hermitian_error(f, lone)
        assert e < herm_tol, f"{what} {name}: kx = 0 line not Hermitian ({e:.2e})"


def test_configuration2_fp64_and_mixed():
    import littleharsh_gb300 as lh
    from littleharsh_gb300.workloads import CONFIG2
    fp = _start(CONFIG2, lh.PREC_FP64)
    _check_properties(fp, "projected start")
    mx = lh.Solver(lh.Config(**CONFIG2), precision=lh.PREC_MIXED)
    mx.set_fields(*fp.get_fields())
    t = fp.time()
    mx.set_time(0.0, t["dt"], 0.0, t["QxT"])
    fp.step(3)
    mx.step(3)
    _check_properties(fp, "FP64, 3 steps")
    _check_properties(mx, "mixed, 3 steps", herm_tol=1e-5)
    for name, a, b in zip(("u1", "u2", "u3"), mx.get_fields(), fp.get_fields()):
        assert rel_l2(a, b) < 1e-4, f"mixed vs FP64 {name}: {rel_l2(a, b):.2e}"
    mx.close()
    # plane statistics at full size against the downloaded spectra: the mean is the (0,0) mode, the mean square
    # Parseval's sum as the physical field sees it (kx > 0 twice, the kx = 0 line paired with -kz, the lone
    # -N2/2 mode half), both times the plane's points
    fp.stats_accumulate()
    n, st = fp.stats_flush()
    u1 = fp.get_fields()[0]
    pts = float(fp.ngx) * float(fp.ngz)
    nz = u1.shape[1]
    e = 2.0 * (np.abs(u1[:, :, 1:]) ** 2).sum(axis=(1, 2))
    line = u1[:, :, 0]
    kk = np.arange(nz)
    partner = line[:, (nz - kk) % nz]
    half = 0.5 * (np.abs(line) ** 2 + (line * partner).real)
    half[:, nz // 2] = 0.5 * np.abs(line[:, nz // 2]) ** 2
    e += half.sum(axis=1)
    assert n == 1
    np.testing.assert_allclose(st["Um"], pts * u1[:, 0, 0].real, rtol=1e-12, atol=1e-9 * pts)
    np.testing.assert_allclose(st["U2m"], pts * e, rtol=1e-10, atol=1e-12 * pts)
    fp.close()


def test_configuration2_graph_replay_equals_launch_by_launch():
    import littleharsh_gb300 as lh
    from littleharsh_gb300.workloads import CONFIG2
    a = _start(CONFIG2, lh.PREC_FP64, seed=2)
    b = lh.Solver(lh.Config(**CONFIG2))
    b.set_fields(*a.get_fields())
    t = a.time()
    b.set_time(0.0, t["dt"], 0.0, t["QxT"])
    a.step(1)  # captured CUDA graph
    for k in (1, 2, 3):
        b.substage(k)  # the same substages, launched one by one
    for x, y in zip(a.get_fields(), b.get_fields()):
        np.testing.assert_array_equal(x, y)
    b.close()
    a.close()


def test_configuration2_with_bands():
    import littleharsh_gb300 as lh
    from littleharsh_gb300.workloads import CONFIG2_BANDS
    s = _start(CONFIG2_BANDS, lh.PREC_FP64, seed=3)
    s.step(3)
    n2mid = 2 * CONFIG2_BANDS["ngalz2"] // 3  # the middle band's z modes
    _check_properties(s, "bands, 3 steps", lone=(n2mid // 2,))
    s.close()


def test_configuration2_against_the_oracle(oracle_mod):
    """The benchmarked grid stepped by the GPU (FP64 and mixed) and by the oracle from one projected field."""
    import littleharsh_gb300 as lh
    from littleharsh_gb300.workloads import CONFIG2
    from tests.helpers import projected_ic
    o = oracle_mod.Oracle(**CONFIG2)
    u1, u2, u3, p = projected_ic(o, seed=7)
    dt, Q = o.cfl_dt(0.5), o.flowrate()
    o.set_fields(u1, u2, u3, p)
    o.set_scalars(0.0, dt, 0.0, Q)
    o.step(2)
    ref = o.get_fields()
    mpgx = o.scalars()["mpgx"]
    del o
    for prec, tol in ((lh.PREC_FP64, 1e-10), (lh.PREC_MIXED, 1e-4)):
        s = lh.Solver(lh.Config(**CONFIG2), precision=prec)
        s.set_fields(u1, u2, u3, p)
        s.set_time(0.0, dt, 0.0, Q)
        s.step(2)
        for name, a, b in zip(("u1", "u2", "u3", "p"), s.get_fields(), ref):
            e = rel_l2(a, b)
            assert e < tol, f"precision {prec} {name}: rel L2 {e:.3e} >= {tol:.0e}"
        assert abs(s.time()["mpgx"] - mpgx) < (1e-9 if prec == lh.PREC_FP64 else 1e-4) * abs(mpgx)
        s.close()


def test_configuration5_fine_grid_against_the_oracle(oracle_mod):
    """The warm start's fine grid (576 x 576 points, 385 levels, Re_b 2800, 12 x 6 posts 12 x 24 points wide,
    64-level canopies) stepped once by the GPU (FP64 and mixed) and by the oracle from one projected field."""
    import littleharsh_gb300 as lh
    from littleharsh_gb300.workloads import CONFIG5_FINE
    from tests.helpers import projected_ic
    o = oracle_mod.Oracle(**CONFIG5_FINE)
    u1, u2, u3, p = projected_ic(o, seed=9)
    dt, Q = o.cfl_dt(0.5), o.flowrate()
    o.set_fields(u1, u2, u3, p)
    o.set_scalars(0.0, dt, 0.0, Q)
    o.step(1)
    ref = o.get_fields()
    mpgx = o.scalars()["mpgx"]
    del o
    for prec, tol in ((lh.PREC_FP64, 1e-10), (lh.PREC_MIXED, 1e-4)):
        s = lh.Solver(lh.Config(**CONFIG5_FINE), precision=prec)
        s.set_fields(u1, u2, u3, p)
        s.set_time(0.0, dt, 0.0, Q)
        s.step(1)
        for name, a, b in zip(("u1", "u2", "u3", "p"), s.get_fields(), ref):
            e = rel_l2(a, b)
            assert e < tol, f"precision {prec} {name}: rel L2 {e:.3e} >= {tol:.0e}"
        assert abs(s.time()["mpgx"] - mpgx) < (1e-9 if prec == lh.PREC_FP64 else 1e-4) * abs(mpgx)
        s.close()
