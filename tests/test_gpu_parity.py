"""GPU parity: the CUDA RK3 step against the CPU FP64 oracle on the same inputs.

Every test builds both from one configuration, feeds them the same projected
seeded field and compares with relative L2 norms.  The FP64 bar is 1e-10 after
10 RK3 steps (the tolerance of the target), tighter for single substages.
"""
import numpy as np
import pytest

from tests.helpers import C1, SMALL, SMOOTH, projected_ic, rel_l2

pytestmark = pytest.mark.gpu

SUBSTAGE_TOL = 1e-11
STEP10_TOL = 1e-10


def _pair(po, cfg, precision=0, seed=1):
    import littleharsh_gb300 as lh
    o = po.Oracle(**cfg)
    u1, u2, u3, p = projected_ic(o, seed=seed)
    dt = o.cfl_dt(0.5)
    Q = o.flowrate()
    o.set_fields(u1, u2, u3, p)
    o.set_scalars(0.0, dt, 0.0, Q)
    s = lh.Solver(lh.Config(**cfg), precision=precision)
    s.set_fields(u1, u2, u3, p)
    s.set_time(0.0, dt, 0.0, Q)
    return o, s


def _cmp_fields(o, s, tol, what=""):
    fo = o.get_fields()
    fs = s.get_fields()
    for name, a, b in zip(("u1", "u2", "u3", "p"), fs, fo):
        e = rel_l2(a, b)
        assert e < tol, f"{what} {name}: rel L2 {e:.3e} >= {tol:.1e}"


@pytest.mark.parametrize("cfg", [SMALL, SMOOTH], ids=["canopy24", "smooth24"])
@pytest.mark.parametrize("upto", [1, 2, 3, 4, 5])
def test_substage_stages(oracle_mod, cfg, upto):
    o, s = _pair(oracle_mod, cfg)
    o.substage(1, upto)
    s.substage(1, upto)
    if upto <= 2:
        for name, a, b in zip(("r1", "r2", "r3"), s.get_rhs(), o.get_rhs()):
            assert rel_l2(a, b) < SUBSTAGE_TOL, f"stage {upto} {name}: {rel_l2(a, b):.3e}"
        for name, a, b in zip(("n1", "n2", "n3"), s.get_nonlinear(), o.get_nonlinear()):
            assert rel_l2(a, b) < SUBSTAGE_TOL, f"stage {upto} {name}: {rel_l2(a, b):.3e}"
    else:
        _cmp_fields(o, s, SUBSTAGE_TOL, f"stage {upto}")
    if upto >= 4:
        assert abs(s.time()["mpgx"] - o.scalars()["mpgx"]) < 1e-10 * max(1.0, abs(o.scalars()["mpgx"]))


def test_three_substages_sequence(oracle_mod):
    o, s = _pair(oracle_mod, SMALL)
    for k in (1, 2, 3):
        o.substage(k, 5)
        s.substage(k, 5)
        _cmp_fields(o, s, SUBSTAGE_TOL, f"after kRK={k}")


@pytest.mark.parametrize("cfg,nsteps", [(SMALL, 10), (C1, 10), (C1, 100)],
                         ids=["canopy24", "config1_96x97", "config1_96x97_100steps"])
def test_ten_steps_fp64(oracle_mod, cfg, nsteps):
    """10 RK3 steps within 1e-10 (the target's bound); configuration 1 also over its stated 100-step run."""
    o, s = _pair(oracle_mod, cfg)
    o.step(nsteps)
    s.step(nsteps)
    _cmp_fields(o, s, STEP10_TOL, f"{nsteps} steps")
    assert abs(s.time()["mpgx"] - o.scalars()["mpgx"]) < 1e-9 * abs(o.scalars()["mpgx"])
    assert s.divmax() < 1e-9


def test_mixed_precision_close(oracle_mod):
    import littleharsh_gb300 as lh
    o, s = _pair(oracle_mod, SMALL, precision=lh.PREC_MIXED)
    o.step(10)
    s.step(10)
    fo, fs = o.get_fields(), s.get_fields()
    for name, a, b in zip(("u1", "u2", "u3"), fs, fo):
        e = rel_l2(a, b)
        assert e < 1e-4, f"mixed {name}: {e:.3e}"
    assert s.divmax() < 1e-9  # the projection stays FP64


def test_column_layout_roundtrip(oracle_mod):
    import littleharsh_gb300 as lh
    o, s = _pair(oracle_mod, SMALL)
    u1, u2, u3, p = s.get_fields(lh.LAYOUT_PLANES)
    c = s.get_fields(lh.LAYOUT_COLUMNS)
    # reference cfield f(j, column): column = kk*nkx + i, j fastest
    np.testing.assert_array_equal(c[0], u1.reshape(u1.shape[0], -1).T)
    np.testing.assert_array_equal(c[3], p.reshape(p.shape[0], -1).T)
    s.set_fields(*c, layout=lh.LAYOUT_COLUMNS)
    back = s.get_fields(lh.LAYOUT_PLANES)
    for a, b in zip(back, (u1, u2, u3, p)):
        np.testing.assert_array_equal(a, b)


def test_divergence_and_cfl(oracle_mod):
    o, s = _pair(oracle_mod, SMALL)
    assert abs(s.divmax() - o.divmax()) < 1e-12
    assert abs(s.cfl_dt(0.5) - o.cfl_dt(0.5)) < 1e-12 * o.cfl_dt(0.5)


def test_spectra(oracle_mod):
    o, s = _pair(oracle_mod, SMALL)
    o.step(2)
    s.step(2)
    o.spectra_accumulate()
    s.spectra_accumulate()
    n, sg = s.spectra_flush()
    so = o.spectra()
    assert n == 1
    for a, b in zip(sg, so):
        assert rel_l2(a, b) < 1e-10


def test_step_is_graph_replay(oracle_mod):
    o, s = _pair(oracle_mod, SMALL)
    s.step(3)
    ms, launches = s.last_step_ms()
    assert ms > 0 and launches > 0


def test_plane_statistics(oracle_mod):
    o, s = _pair(oracle_mod, SMALL)
    o.step(2)
    s.step(2)
    for _ in range(2):
        o.stats_accumulate()
        s.stats_accumulate()
    n, st = s.stats_flush()
    no, so = o.stats()
    assert n == no == 2
    ny = {"u": s.nyu, "v": s.nyv, "p": s.nyp}
    for r, (name, grid) in enumerate(zip(s.STAT_ROWS, "uuvvuuppuuvvv")):
        a, b = st[name], so[r, :ny[grid]]
        # means of v vanish by continuity: an absolute floor of 1e-13 per summed point covers round-off
        tol = 1e-11 * np.abs(b).max() + 1e-13 * s.ngx * s.ngz
        assert np.abs(a - b).max() < tol, f"{name}: {np.abs(a - b).max():.3e} >= {tol:.3e}"


def test_conditional_statistics(oracle_mod):
    o, s = _pair(oracle_mod, SMALL)
    o.step(1)
    s.step(1)
    for _ in range(2):
        o.cond_accumulate()
        s.cond_accumulate()
    n, cg = s.cond_flush()
    no, co = o.cond()
    assert n == no == 2
    for name in s.COND_ROWS:
        a, b = cg[name], co[name]
        assert a.shape == b.shape, name
        tol = 1e-11 * np.abs(b).max() + 1e-13 * s.ngx * s.ngz
        assert np.abs(a - b).max() < tol, f"{name}: {np.abs(a - b).max():.3e} >= {tol:.3e}"


def test_autotune_keeps_results(oracle_mod):
    """Launch shapes change which CTA computes what, not the arithmetic: a tuned solver steps bit for bit
    like an untuned one."""
    o, s = _pair(oracle_mod, SMALL)
    import littleharsh_gb300 as lh
    t = lh.Solver(lh.Config(**SMALL))
    t.set_fields(*s.get_fields())
    tm = s.time()
    t.set_time(0.0, tm["dt"], 0.0, tm["QxT"])
    shapes = t.autotune()
    assert shapes["tx"] in (1, 2, 4, 8, 16, 32) and shapes["chunk"] in (4, 8, 16, 32, 64)
    assert shapes["xthreads"] in (128, 256) and shapes["zthreads"] in (128, 256) and shapes["xrows"] == 1
    s.step(3)
    t.step(3)
    for a, b in zip(t.get_fields(), s.get_fields()):
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
def test_split_face_pair_keeps_results(oracle_mod, monkeypatch, mixed):
    """The x pass that transforms the face pair after the centre pairs (two buffer vectors instead of
    three) runs the same transforms one vector at a time: bit for bit the same step."""
    import littleharsh_gb300 as lh
    o, s0 = _pair(oracle_mod, C1)
    prec = lh.PREC_MIXED if mixed else lh.PREC_FP64
    sols = []
    for split in ("0", "1"):
        monkeypatch.setenv("LH_XSPLIT", split)
        s = lh.Solver(lh.Config(**C1), precision=prec)
        s.set_fields(*s0.get_fields())
        tm = s0.time()
        s.set_time(0.0, tm["dt"], 0.0, tm["QxT"])
        s.step(3)
        sols.append(s)
    for a, b in zip(sols[0].get_fields(), sols[1].get_fields()):
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
@pytest.mark.parametrize("which", ["x", "z"])
def test_pass_threads_keep_results(oracle_mod, monkeypatch, mixed, which):
    """128 or 256 threads per product-pass (x) or z-pass CTA share the same butterflies out differently,
    not the arithmetic: bit for bit the same step."""
    import littleharsh_gb300 as lh
    o, s0 = _pair(oracle_mod, C1)
    prec = lh.PREC_MIXED if mixed else lh.PREC_FP64
    sols = []
    for threads in ("256", "128"):
        monkeypatch.setenv(f"LH_{which.upper()}THREADS", threads)
        s = lh.Solver(lh.Config(**C1), precision=prec)
        assert s.launch_shapes()[f"{which}threads"] == int(threads)
        s.set_fields(*s0.get_fields())
        tm = s0.time()
        s.set_time(0.0, tm["dt"], 0.0, tm["QxT"])
        s.step(3)
        sols.append(s)
    for a, b in zip(sols[0].get_fields(), sols[1].get_fields()):
        np.testing.assert_array_equal(a, b)


def test_two_row_product_pass_keeps_results(oracle_mod, monkeypatch):
    """The mixed form's product pass with two z rows per CTA runs each row's transforms, products and
    truncation with the arithmetic of the one-row pass: bit for bit the same steps."""
    import littleharsh_gb300 as lh
    o, s0 = _pair(oracle_mod, C1)
    sols = []
    for rows in ("1", "2"):
        monkeypatch.setenv("LH_XROWS", rows)
        s = lh.Solver(lh.Config(**C1), precision=lh.PREC_MIXED)
        assert s.launch_shapes()["xrows"] == int(rows)
        s.set_fields(*s0.get_fields())
        tm = s0.time()
        s.set_time(0.0, tm["dt"], 0.0, tm["QxT"])
        s.step(3)
        sols.append(s)
    for a, b in zip(sols[0].get_fields(), sols[1].get_fields()):
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("cfg", [SMALL, C1], ids=["canopy24", "config1_96x97"])
def test_broadband_field(oracle_mod, cfg):
    """Every mode populated (not only |k| <= 8): the high modes, the 3/2 truncation and the Nyquist
    neighbours are exercised as in developed turbulence.  FP64 to the usual bar; the mixed form to
    FP32 accuracy."""
    import littleharsh_gb300 as lh
    from littleharsh_gb300.initial import initial_field
    o = oracle_mod.Oracle(**cfg)
    g = o.grid()
    kmax = max(o.nkx, o.nz)
    o.set_fields(*initial_field(g["yu"], g["yv"], o.nz, o.nkx, o.nyp, seed=7, amp=0.2, kmax=kmax))
    o.set_scalars(0.0, 1.0, 0.0)
    o.project()
    u1, u2, u3, p = o.get_fields()
    dt, Q = o.cfl_dt(0.5), o.flowrate()
    o.set_scalars(0.0, dt, 0.0, Q)
    sols = []
    for prec in (lh.PREC_FP64, lh.PREC_MIXED):
        s = lh.Solver(lh.Config(**cfg), precision=prec)
        s.set_fields(u1, u2, u3, p)
        s.set_time(0.0, dt, 0.0, Q)
        sols.append(s)
    o.step(3)
    for s in sols:
        s.step(3)
    ref = o.get_fields()
    for name, a, b in zip(("u1", "u2", "u3", "p"), sols[0].get_fields(), ref):
        assert rel_l2(a, b) < 1e-11, f"fp64 {name}: {rel_l2(a, b):.3e}"
    errs = [rel_l2(a, b) for a, b in zip(sols[1].get_fields(), ref)]
    assert max(errs[:3]) < 2e-6 and errs[3] < 1e-4, f"mixed: {errs}"


def test_constant_pressure_gradient(oracle_mod):
    """flag_ctpress = 1 (input.in's constant-pressure mode): the mean pressure gradient stays at its input
    value and no flow-rate correction runs; 10 FP64 steps against the oracle."""
    import littleharsh_gb300 as lh
    cfg = dict(SMALL, flag_ctpress=1)
    o = oracle_mod.Oracle(**cfg)
    u1, u2, u3, p = projected_ic(o, seed=4)
    dt, mp = o.cfl_dt(0.5), -0.01
    o.set_fields(u1, u2, u3, p)
    o.set_scalars(0.0, dt, mp, 0.0)
    s = lh.Solver(lh.Config(**cfg))
    s.set_fields(u1, u2, u3, p)
    s.set_time(0.0, dt, mp, 0.0)
    o.step(10)
    s.step(10)
    _cmp_fields(o, s, 1e-10, "constant pressure gradient, 10 steps")
    assert s.time()["mpgx"] == mp and o.scalars()["mpgx"] == mp
