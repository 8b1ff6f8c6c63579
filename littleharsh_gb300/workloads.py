"""The benchmark workloads as input.in quantities (single x/z resolution).

Re is the bulk Reynolds number on the half height (U_b = delta = 1), alp and
bet the fundamental wavenumbers (Lx = 2 pi, Lz = pi), ngalx/ngalz the
dealiased physical points (modes = 2/3 of them), ny the input.in y points
(the u grid adds 2 dsty + 1 canopy and ghost levels), dyq the stretching
ratio of the polynomial grid, posth the canopy height, dstx/dstz the post
width in points and ntilex/ntilez the posts per wall.
"""
from __future__ import annotations

# Re_tau ~ 180, 64 x 64 modes, 12 x 6 posts of height 0.2 a quarter of the pitch wide
CONFIG1 = dict(Re=2800.0, alp=1.0, bet=2.0, ngalx=96, ngalz=96, ny=97, dyq=13.6, ppp=5, geometry_type=3, posth=0.2,
               dsty=16, dstx=2, dstz=4, ntilex=12, ntilez=6, flag_ctpress=0)

# Re_tau ~ 550, 384 x 384 modes, 48 x 24 posts of height 0.1 resolved by 8 x 8 points
CONFIG2 = dict(Re=10000.0, alp=1.0, bet=2.0, ngalx=576, ngalz=576, ny=385, dyq=13.6, ppp=5, geometry_type=3,
               posth=0.1, dsty=32, dstx=8, dstz=8, ntilex=48, ntilez=24, flag_ctpress=0)

# configuration 2 with the reference's variable-resolution bands: the middle band
# (between the canopy layers) at 384 x 384 points (256 x 256 modes)
CONFIG2_BANDS = dict(CONFIG2, ngalx2=384, ngalz2=384)

# mid-size case for profiler captures: x-pass inputs larger than L2, ~2 GB on the device
MID288 = dict(Re=5000.0, alp=1.0, bet=2.0, ngalx=288, ngalz=288, ny=193, dyq=13.6, ppp=5, geometry_type=3, posth=0.1,
              dsty=16, dstx=4, dstz=4, ntilex=24, ntilez=12, flag_ctpress=0)

# capture case for the profiler: configuration 2's x and z lengths (the same transform lengths and shared-memory
# footprints per CTA) on 49 y points (58 u levels), ~2.5 GB on the device, x-pass inputs ~5x the L2
XZ576_NY49 = dict(CONFIG2, ny=49, dsty=4)

# configuration 1 at half the resolution in x, z and y: the coarse grid of the
# learned warm start on configuration 1's geometry (posts 1 x 2 points)
CONFIG1_COARSE = dict(CONFIG1, ngalx=48, ngalz=48, ny=49, dsty=8, dstx=1, dstz=2)

# configuration 1 at twice its resolution in x, z and y (128 x 128 modes, ny 193, posts 4 x 8 points): the fine
# grid of the warm start whose coarse grid is configuration 1 itself, a resolved DNS grid at Re_tau 180
CONFIG1_X2 = dict(CONFIG1, ngalx=192, ngalz=192, ny=193, dsty=32, dstx=4, dstz=8)

# configuration 5: configuration 1's flow and canopy (12 x 6 posts, h = 0.2, a
# quarter of the pitch wide) on the 384 x 385 x 384 fine grid and the
# 128 x 193 x 128 coarse grid (modes x ny x modes)
CONFIG5_FINE = dict(CONFIG1, ngalx=576, ngalz=576, ny=385, dsty=64, dstx=12, dstz=24)
CONFIG5_COARSE = dict(CONFIG1, ngalx=192, ngalz=192, ny=193, dsty=32, dstx=4, dstz=8)

RE_TAU = {"config1": 180.0, "config2": 550.0}


def ensemble_configs():
    """Configuration 4: 16 replicas of uneven sizes, canopy pitches pi/6, pi/8,
    pi/12 (12x6, 16x8, 24x12 tiles), heights 0.1/0.2, Re_b 2800-6900
    (Re_tau ~180-395), posts a quarter of the pitch wide."""
    sizes = [(144, 129, 12)] * 6 + [(192, 193, 16)] * 6 + [(288, 257, 24)] * 4
    tiles = [(12, 6), (16, 8), (24, 12)]
    res = [2800.0, 4500.0, 6900.0]
    out = []
    for i, (ng, ny, dsty) in enumerate(sizes):
        tx, tz = tiles[i % 3]
        out.append(dict(Re=res[i % 3], alp=1.0, bet=2.0, ngalx=ng, ngalz=ng, ny=ny, dyq=13.6, ppp=5, geometry_type=3,
                        posth=(0.1, 0.2)[i % 2], dsty=dsty, dstx=max(1, ng // tx // 4), dstz=max(1, ng // tz // 4),
                        ntilex=tx, ntilez=tz, flag_ctpress=0))
    return out
