"""Shared set-up for the parity tests: one configuration, fed identically to
the CUDA solver and to the CPU oracle."""
from __future__ import annotations

import numpy as np

SMALL = dict(Re=2800.0, alp=1.0, bet=2.0, ngalx=24, ngalz=24, ny=33, dyq=13.6, ppp=5, geometry_type=3,
             posth=0.2, dsty=4, dstx=2, dstz=2, ntilex=4, ntilez=4, flag_ctpress=0)
# configuration 1: 96x96 dealiased, ny=97, 12x6 posts, h=0.2, 2x4 points per post
C1 = dict(Re=2800.0, alp=1.0, bet=2.0, ngalx=96, ngalz=96, ny=97, dyq=13.6, ppp=5, geometry_type=3,
          posth=0.2, dsty=16, dstx=2, dstz=4, ntilex=12, ntilez=6, flag_ctpress=0)
SMOOTH = dict(Re=2800.0, alp=1.0, bet=2.0, ngalx=24, ngalz=24, ny=33, dyq=13.6, ppp=5, geometry_type=0,
              posth=0.0, dsty=0, dstx=1, dstz=1, ntilex=1, ntilez=1, flag_ctpress=0)


def make_oracle(po, cfg: dict):
    return po.Oracle(**cfg)


def projected_ic(o, seed=1, amp=0.1, kmax=8):
    """Seeded IC projected divergence-free by the oracle's Poisson step."""
    from littleharsh_gb300.initial import initial_field
    g = o.grid()
    u1, u2, u3, p = initial_field(g["yu"], g["yv"], o.nz, o.nkx, o.nyp, seed=seed, amp=amp, kmax=kmax)
    o.set_fields(u1, u2, u3, p)
    o.set_scalars(0.0, 1.0, 0.0)
    o.project()
    return o.get_fields()


def rel_l2(a, b) -> float:
    d = np.linalg.norm((a - b).ravel())
    n = np.linalg.norm(b.ravel())
    return float(d / n) if n > 0 else float(d)
