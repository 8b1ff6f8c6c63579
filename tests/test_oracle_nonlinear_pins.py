"""Pins of the reconstructed nonlinear term that share no code with the oracle.

The reference's `nonlinear` (called at littleharsh.f90:171) lives in FOU3D.f90,
which the tree does not contain; the oracle and the GPU path implement one
reconstruction of it.  These tests check the oracle's N against facts that do
not depend on how it is coded:

* flux form: N is the divergence of the momentum flux, and the y-derivative is
  a difference of face (or centre) values scaled by the metric c_j =
  ddthetavi*dthdy(j).  So sum_j N(0,0,j)/c_j telescopes to the fluxes at the
  ends of the sum: zero for u and w (uv = vw = 0 on the wall faces), and for v
  the plane means of v^2 at the first and last interior centres.
* a manufactured few-mode field, whose N a short numpy evaluation below forms
  on its own: products by numpy FFTs on a grid fine enough that nothing
  aliases, linear y-interpolation between the staggered grids from the grid
  arrays, the divergence from the wavenumbers and the metric.
"""
import numpy as np
import pytest

from tests.helpers import C1, SMALL, SMOOTH, projected_ic


def _kz_index(nz):
    kk = np.arange(nz)
    return np.where(kk < nz // 2, kk, kk - nz)


# ---------------------------------------------------------------------------
# an independent evaluation of N in numpy
# ---------------------------------------------------------------------------
def _to_full(plane, M):
    """A plane [kk][i] of a real field -> its full M x M spectrum S[kz mod M, kx mod M] (kx < 0 by conjugation)."""
    nz, nkx = plane.shape
    kz = _kz_index(nz)
    S = np.zeros((M, M), np.complex128)
    for kk in range(nz):
        for i in range(nkx):
            a = plane[kk, i]
            if a == 0:
                continue
            S[kz[kk] % M, i % M] += a
            if i > 0:
                S[(-kz[kk]) % M, (-i) % M] += np.conj(a)
    return S


def _phys(S):
    M = S.shape[0]
    return np.real(np.fft.ifft2(S)) * M * M


def _coef(P, nz, nkx):
    """Kept modes [kk][i] of a physical product."""
    M = P.shape[0]
    F = np.fft.fft2(P) / (M * M)
    kz = _kz_index(nz)
    out = np.zeros((nz, nkx), np.complex128)
    for kk in range(nz):
        out[kk, :] = F[kz[kk] % M, :nkx]
    return out


def numpy_nonlinear(u1, u2, u3, g, alp, bet, M=64):
    """N1, N2, N3 of the staggered divergence form on the interior levels (zero elsewhere).

    Centres jj = 1..nyu-2 carry uu, uw, ww and vv (v interpolated to the centre linearly in y from the faces
    jj-1, jj, with v = 0 on the wall faces); faces jj = 1..nyv-2 carry uv and vw (u and w interpolated linearly
    in y from the centres jj and jj+1); uv = vw = 0 on the wall faces.
      N1(c) = i kx uu + i kz uw + c_u(c) [uv(face c) - uv(face c-1)]
      N3(c) = i kx uw + i kz ww + c_u(c) [vw(face c) - vw(face c-1)]
      N2(f) = i kx uv + i kz vw + c_v(f) [vv(centre f+1) - vv(centre f)]
    """
    nyu, nz, nkx = u1.shape
    nyv = u2.shape[0]
    yu, yv = g["yu"], g["yv"]
    cu, cv = g["dthdyu"], g["dthdyv"]  # ddthetavi = 1 (y_grid_canopy.f90:41-43)
    U = [None] * nyu
    W = [None] * nyu
    V = [np.zeros((M, M))] + [None] * (nyv - 2) + [np.zeros((M, M))]
    for j in range(1, nyu - 1):
        U[j] = _phys(_to_full(u1[j], M))
        W[j] = _phys(_to_full(u3[j], M))
    for j in range(1, nyv - 1):
        V[j] = _phys(_to_full(u2[j], M))
    kx = alp * np.arange(nkx)[None, :]
    kz = bet * _kz_index(nz)[:, None]
    uu, uw, ww, vv = ({} for _ in range(4))
    uv = {0: np.zeros((nz, nkx), complex), nyv - 1: np.zeros((nz, nkx), complex)}
    vw = {0: np.zeros((nz, nkx), complex), nyv - 1: np.zeros((nz, nkx), complex)}
    for c in range(1, nyu - 1):
        t = (yu[c] - yv[c - 1]) / (yv[c] - yv[c - 1])
        vc = V[c - 1] + t * (V[c] - V[c - 1])
        uu[c], uw[c], ww[c] = _coef(U[c] * U[c], nz, nkx), _coef(U[c] * W[c], nz, nkx), _coef(W[c] * W[c], nz, nkx)
        vv[c] = _coef(vc * vc, nz, nkx)
    for f in range(1, nyv - 1):
        t = (yv[f] - yu[f]) / (yu[f + 1] - yu[f])
        uf = U[f] + t * (U[f + 1] - U[f])
        wf = W[f] + t * (W[f + 1] - W[f])
        uv[f], vw[f] = _coef(uf * V[f], nz, nkx), _coef(wf * V[f], nz, nkx)
    N1, N2, N3 = np.zeros_like(u1), np.zeros_like(u2), np.zeros_like(u3)
    for c in range(1, nyu - 1):
        N1[c] = 1j * kx * uu[c] + 1j * kz * uw[c] + cu[c] * (uv[c] - uv[c - 1])
        N3[c] = 1j * kx * uw[c] + 1j * kz * ww[c] + cu[c] * (vw[c] - vw[c - 1])
    for f in range(1, nyv - 1):
        N2[f] = 1j * kx * uv[f] + 1j * kz * vw[f] + cv[f] * (vv[f + 1] - vv[f])
    return N1, N2, N3


def _few_modes(o, seed):
    """u, v, w with modes kx in 0..2, |kz| <= 2 (Hermitian on the kx = 0 line), random y profiles, v = 0 on the
    wall faces."""
    rng = np.random.default_rng(seed)
    nz, nkx = o.nz, o.nkx
    out = []
    for ny in (o.nyu, o.nyv, o.nyu):
        f = np.zeros((ny, nz, nkx), np.complex128)
        for i in range(3):
            for kz in range(-2, 3):
                if i == 0 and kz < 0:
                    continue
                a = rng.standard_normal(ny) + 1j * rng.standard_normal(ny)
                if i == 0 and kz == 0:
                    a = a.real + 1.0
                f[:, kz % nz, i] = a
                if i == 0 and kz > 0:
                    f[:, (-kz) % nz, 0] = np.conj(a)
        out.append(f)
    out[1][0] = 0.0
    out[1][-1] = 0.0
    return out


@pytest.mark.parametrize("cfg", [SMALL, SMOOTH], ids=["canopy24", "smooth24"])
def test_manufactured_field_nonlinear_term(oracle_mod, cfg):
    o = oracle_mod.Oracle(**cfg)
    g = o.grid()
    u1, u2, u3 = _few_modes(o, seed=11)
    o.set_fields(u1, u2, u3, o.zeros("p"))
    o.set_nonlinear(o.zeros("u"), o.zeros("v"), o.zeros("u"))
    o.set_scalars(0.0, 1e-3, 0.0)
    o.substage(1, 1)  # right-hand sides, with N formed from the current field and stored
    got = o.get_nonlinear()
    ref = numpy_nonlinear(u1, u2, u3, g, cfg["alp"], cfg["bet"])
    for name, a, b in zip(("N1", "N2", "N3"), got, ref):
        scale = np.abs(b).max()
        assert scale > 1.0
        assert np.abs(a - b).max() < 1e-12 * scale, f"{name}: {np.abs(a - b).max() / scale:.2e}"


@pytest.mark.parametrize("cfg", [SMALL, C1], ids=["canopy24", "config1_96x97"])
def test_flux_form_telescopes(oracle_mod, cfg):
    """sum_j N(0,0,j)/c_j over the interior levels: 0 for u and w, vv(0,0) at the last interior centre minus
    vv(0,0) at the first for v, where vv(0,0) of an interpolated v is the plane mean of its square (Parseval,
    evaluated from the spectral coefficients, independently of the transforms)."""
    o = oracle_mod.Oracle(**cfg)
    u1, u2, u3, p = projected_ic(o, seed=4, kmax=max(o.nkx, o.nz // 2))
    g = o.grid()
    o.set_fields(u1, u2, u3, p)
    o.set_scalars(0.0, 1e-3, 0.0)
    o.substage(1, 1)
    n1, n2, n3 = o.get_nonlinear()
    cu, cv = g["dthdyu"], g["dthdyv"]
    for name, n in (("N1", n1), ("N3", n3)):
        terms = n[1:-1, 0, 0].real / cu[1:-1]
        assert np.abs(n[1:-1, 0, 0].imag).max() < 1e-13 * np.abs(terms).max()
        s = terms.sum()
        assert abs(s) < 1e-13 * np.abs(terms).sum(), f"{name}: sum {s:.3e} of {np.abs(terms).sum():.3e}"

    def mean_sq(c):
        """Plane mean of v_c^2 for v_c interpolated to centre c: Parseval on the kept modes, kx > 0 counted
        twice; the kx = 0 line is Hermitian except its lone -N2/2 mode, whose real part alone reaches the
        physical plane."""
        yu, yv = g["yu"], g["yv"]
        t = (yu[c] - yv[c - 1]) / (yv[c] - yv[c - 1])
        v0 = u2[c - 1] if c - 1 > 0 else 0.0 * u2[0]
        v1 = u2[c] if c < o.nyv - 1 else 0.0 * u2[0]
        vc = v0 + t * (v1 - v0)
        e = 2.0 * np.sum(np.abs(vc[:, 1:]) ** 2) + np.sum(np.abs(vc[:, 0]) ** 2)
        lone = vc[o.nz // 2, 0]
        return e - abs(lone) ** 2 + lone.real ** 2

    terms2 = n2[1:-1, 0, 0].real / cv[1:-1]
    expect = mean_sq(o.nyu - 2) - mean_sq(1)
    assert abs(terms2.sum() - expect) < 1e-12 * np.abs(terms2).sum()
