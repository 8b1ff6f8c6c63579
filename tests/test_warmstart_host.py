"""Data preparation of the learned warm start, on the CPU (torch CPU tensors).

The lifting transforms must follow the solver's conventions: the oracle's
plane transforms (lho_plane_to_phys / lho_plane_to_spec) define them.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from littleharsh_gb300 import warmstart as ws  # noqa: E402
from littleharsh_gb300.workloads import CONFIG1  # noqa: E402

from littleharsh_gb300.workloads import CONFIG1_COARSE as COARSE1  # noqa: E402


@pytest.fixture(scope="module")
def grids():
    return ws.GridInfo.from_config(CONFIG1), ws.GridInfo.from_config(COARSE1)


def test_plane_transforms_follow_the_solver(oracle_mod, grids):
    fine, _ = grids
    o = oracle_mod.Oracle(**CONFIG1, nthreads=1)
    rng = np.random.default_rng(0)
    plane = rng.standard_normal((o.nz, o.nkx)) + 1j * rng.standard_normal((o.nz, o.nkx))  # kx=0 line not Hermitian
    ref = o.to_phys(plane)
    got = ws.spec_to_phys(torch.from_numpy(plane[None]), fine.ngx, fine.ngz)[0].numpy()
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-11 * np.abs(ref).max())
    phys = rng.standard_normal((fine.ngz, fine.ngx))
    np.testing.assert_allclose(ws.phys_to_spec(torch.from_numpy(phys[None]), fine.nz, fine.nkx)[0].numpy(),
                               o.to_spec(phys), rtol=0, atol=1e-13)


def test_mode_resampling_round_trip(grids):
    fine, coarse = grids
    rng = np.random.default_rng(1)
    c = torch.from_numpy(rng.standard_normal((3, coarse.nz, coarse.nkx)) + 1j * rng.standard_normal((3, coarse.nz, coarse.nkx)))
    up = ws.resample_modes(c, fine.nz, fine.nkx)
    assert up.shape == (3, fine.nz, fine.nkx)
    np.testing.assert_array_equal(ws.resample_modes(up, coarse.nz, coarse.nkx).numpy(), c.numpy())
    # the padded field is the same function: its values at the coarse physical points agree
    pc = ws.spec_to_phys(c, coarse.ngx, coarse.ngz).numpy()
    pf = ws.spec_to_phys(up, 2 * coarse.ngx, 2 * coarse.ngz).numpy()
    np.testing.assert_allclose(pf[:, ::2, ::2], pc, atol=1e-12)


def test_level_interpolation_and_staggering_are_exact_for_linear_profiles(grids):
    fine, coarse = grids
    a, b = 0.3, -1.7
    f = torch.from_numpy((a + b * coarse.yu)[:, None, None] * np.ones((1, 2, 3)))
    g = ws.interp_levels(f, coarse.yu, fine.yu).numpy()
    inside = (fine.yu >= coarse.yu[0]) & (fine.yu <= coarse.yu[-1])
    np.testing.assert_allclose(g[inside, 0, 0], (a + b * fine.yu)[inside], atol=1e-13)
    v = torch.from_numpy((a + b * fine.yv)[:, None])
    vc = ws.v_to_centres(v, fine).numpy()[:, 0]
    np.testing.assert_allclose(vc[1:-1], (a + b * fine.yu)[1:-1], atol=1e-13)
    back = ws.centres_to_v(torch.from_numpy((a + b * fine.yu)[:, None]), fine).numpy()[:, 0]
    np.testing.assert_allclose(back[1:-1], (a + b * fine.yv)[1:-1], atol=1e-13)


def test_canopy_mask_matches_the_geometry(grids):
    fine, coarse = grids
    for gi, cfg in ((fine, CONFIG1), (coarse, COARSE1)):
        solid = gi.mask.sum(axis=(1, 2))
        per_plane = cfg["ntilex"] * cfg["ntilez"] * cfg["dstx"] * cfg["dstz"]
        assert set(np.unique(solid)) <= {0.0, float(per_plane)}
        assert (solid > 0).sum() >= 2 * cfg["dsty"]
