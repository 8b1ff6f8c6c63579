"""Seeded initial field: laminar profile plus a random solenoidal perturbation.

The reference's initial-condition menu (getini, start.f90:1488-1594) offers a
restart file or a fixed parabolic profile (mblock_ini_parabolic_profile,
start.f90:1644-1784).  The benchmark configurations start instead from a
laminar profile between the canopy tips plus a seeded random perturbation with
|kx|, |kz| index <= kmax and Gaussian amplitudes, scaled to a given fraction of
the bulk velocity; the solver's own Poisson step (Solver.project) then makes
it divergence free.  The same arrays are fed to every implementation that is
compared, so the field only has to be reproducible, not identical to a
reference recipe.
"""
from __future__ import annotations

import numpy as np


def initial_field(yu: np.ndarray, yv: np.ndarray, nz: int, nkx: int, nyp: int, seed: int = 1, amp: float = 0.1,
                  kmax: int = 8):
    """Spectral u1, u2, u3, p in the plane layout [j][kk][i].

    u1 (0,0) holds 1.5*(1-y^2) between the tips (bulk velocity 1 there) and 0
    inside the canopies; every velocity component gets the perturbation,
    shaped in y by (1-y^2)^2 between the tips.  Modes with kx index 0 are
    given Hermitian partners so the physical field is real.  The rms of the
    perturbation over the channel between the tips is `amp`.
    """
    rng = np.random.default_rng(seed)
    nyu, nyv = yu.size, yv.size
    u1 = np.zeros((nyu, nz, nkx), np.complex128)
    u2 = np.zeros((nyv, nz, nkx), np.complex128)
    u3 = np.zeros((nyu, nz, nkx), np.complex128)
    p = np.zeros((nyp, nz, nkx), np.complex128)
    inside_u = np.abs(yu) < 1.0
    inside_v = np.abs(yv) < 1.0
    u1[:, 0, 0] = np.where(inside_u, 1.5 * (1.0 - yu**2), 0.0)
    env = {"u": np.where(inside_u, (1.0 - yu**2) ** 2, 0.0), "v": np.where(inside_v, (1.0 - yv**2) ** 2, 0.0)}
    kxm = min(kmax, nkx - 2)
    kzm = min(kmax, nz // 2 - 1)
    pert = []
    for f, g in ((u1, "u"), (u2, "v"), (u3, "u")):
        c = np.zeros((nz, nkx), np.complex128)
        for i in range(0, kxm + 1):
            for kz in range(-kzm, kzm + 1):
                if i == 0 and kz <= 0:
                    continue
                a = rng.standard_normal() + 1j * rng.standard_normal()
                c[kz % nz, i] = a
                if i == 0:
                    c[(-kz) % nz, 0] = np.conj(a)
        pert.append((f, g, c))
    # energy of the perturbation per unit volume between the tips (Parseval:
    # modes with kx > 0 stand for a conjugate pair)
    w = np.ones(nkx)
    w[1:] = 2.0
    e = 0.0
    for f, g, c in pert:
        y = yu if g == "u" else yv
        prof = env[g] ** 2
        dy = np.gradient(y)
        prof_int = float(np.sum(prof * dy * (np.abs(y) < 1.0))) / 2.0
        e += float(np.sum(np.abs(c) ** 2 * w[None, :])) * prof_int
    scale = amp / np.sqrt(max(e, 1e-300))
    for f, g, c in pert:
        f += scale * env[g][:, None, None] * c[None, :, :]
    return u1, u2, u3, p
