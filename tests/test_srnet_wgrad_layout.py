"""The shared-memory layout of the tcgen05 weight gradient (lh_srnet.cu, k_conv_wgrad_tc), checked on the CPU.

The kernel's constants are restated here: tiles of WT_TY = 2 levels x WT_TZ = 16 z voxels x WT_TXW = 8 x
columns; the 32-channel operand S (halo lines x0 - 1 .. x0 + 9, z rows z0 - 1 .. z0 + 16, z pitch 19 rows of
16 bytes) and the other operand U (levels y0 - 1 .. y0 + 2, z pitch 17, column pitch 4 levels x chunks x 17 + 1)
in one stage buffer.  The test fills a stage buffer row by row as the producer warps do, reads every MMA's A
and B operands through the MN-major no-swizzle descriptor rule (element (mn, k) at start + (mn / 8) SBO +
(mn % 8) 2 + (k / 8) LBO + (k % 8) 16 bytes), accumulates D as the MMAs do and maps D to dW as the epilogue
does, then compares with the oracle's weight gradient exactly.  It also checks that every operand read stays
inside the stage buffer with the leading and stride byte offsets read either way, and how a warp's 16-byte
shared stores of the S and U rows spread over the bank groups.
"""
import numpy as np
import pytest

from oracle import sr_oracle as so

TXW, TY, TZ = 8, 2, 16
L = TXW + 3
ZR = TZ + 2
ZP, ZPU = 19, 17


def geom(cu):
    kcs, kcu, ul = 4, cu // 8, TY + 2
    srows = TY * L * kcs * ZP
    xip = ul * kcu * ZPU + 1
    return dict(KCS=kcs, KCU=kcu, UL=ul, SROWS=srows, XIP=xip, BUF=srows + TXW * xip, NCOL=3 * cu)


def s_row(c, kcs):
    kc, line = c % kcs, (c // kcs) % L
    r2 = c // (kcs * L)
    zr, t = r2 % ZR, r2 // ZR
    return kc, line, zr, t, ((t * L + line) * kcs + kc) * ZP + zr


def u_row(c, g):
    kcu, xi = c % g["KCU"], (c // g["KCU"]) % TXW
    r2 = c // (g["KCU"] * TXW)
    z, lev = r2 % TZ, r2 // TZ
    return kcu, xi, z, lev, g["SROWS"] + xi * g["XIP"] + (lev * g["KCU"] + kcu) * ZPU + z


def emulate(x, d):
    """dW, db of the kernel's layout and tap mapping for in (x) and dout (d), float64."""
    Y, Z, X, cin = x.shape
    cout = d.shape[-1]
    swap = cin == 16  # the 16 -> 32 layer: S is the output gradient, taps mirrored
    S, U = (d, x) if swap else (x, d)
    cu = U.shape[-1]
    g = geom(cu)
    kcs, kcu, srows, xip, buf_rows, ncol = g["KCS"], g["KCU"], g["SROWS"], g["XIP"], g["BUF"], g["NCOL"]
    Sf, Uf = S.reshape(-1, 32), U.reshape(-1, cu)
    D = np.zeros((128, 3 * ncol))
    db = np.zeros(cout)
    first = True
    nty, ntz, ntx = (Y + TY - 1) // TY, Z // TZ, X // TXW
    for tile in range(nty * ntz * ntx):
        xt, rest = tile % ntx, tile // ntx
        x0, z0, y0 = xt * TXW, (rest % ntz) * TZ, (rest // ntz) * TY
        buf = np.full((buf_rows, 8), np.nan)  # 16-byte rows of 8 channels; NaN = never written
        for c in range(TY * ZR * L * kcs):
            kc, line, zr, t, row = s_row(c, kcs)
            gy, gz, gx = y0 + t, (z0 + zr - 1) % Z, (x0 + line - 1) % X
            buf[row] = Sf[(gy * Z + gz) * X + gx, 8 * kc:8 * kc + 8] if gy < Y else 0.0
        for c in range(g["UL"] * TZ * TXW * kcu):
            kc, xi, z, lev, row = u_row(c, g)
            gy = y0 + lev - 1
            buf[row] = Uf[(gy * Z + z0 + z) * X + x0 + xi, 8 * kc:8 * kc + 8] if 0 <= gy < Y else 0.0
        flat = buf.reshape(-1)

        def read(start_row, lbo, sbo, mn):
            out = np.empty((mn, 16))
            for m in range(mn):
                for k in range(16):
                    off = start_row * 16 + (m // 8) * sbo + (m % 8) * 2 + (k // 8) * lbo + (k % 8) * 16
                    assert 0 <= off < buf_rows * 16
                    out[m, k] = flat[off // 2]
            return out

        # bias: the tile's own output-gradient voxels
        for t in range(TY):
            for xi in range(TXW):
                for z in range(TZ):
                    if swap:
                        for kc in range(kcs):
                            db[8 * kc:8 * kc + 8] += buf[((t * L + xi + 1) * kcs + kc) * ZP + z + 1]
                    else:
                        for kc in range(kcu):
                            db[8 * kc:8 * kc + 8] += buf[srows + xi * xip + ((t + 1) * kcu + kc) * ZPU + z]
        for t in range(TY):
            for xi in range(TXW):
                b_start = srows + xi * xip + t * kcu * ZPU
                B = read(b_start, 128, ZPU * 16, ncol)
                read(b_start, ZPU * 16, 128, ncol)  # the other reading of the byte offsets stays inside too
                assert not np.isnan(B).any()
                for dz in range(3):
                    a_start = (t * L + xi) * kcs * ZP + dz
                    A = read(a_start, 128, ZP * 16, 128)
                    read(a_start, ZP * 16, 128, 128)
                    assert not np.isnan(A[:96]).any()  # rows of the spare 4th line are discarded
                    blk = np.nan_to_num(A) @ B.T
                    cols = slice(dz * ncol, (dz + 1) * ncol)
                    D[:, cols] = blk if first else D[:, cols] + blk
                first = False
    dw = np.zeros((27, cout, cin))
    for l in range(3):
        for sch in range(32):
            for dz in range(3):
                for n in range(ncol):
                    lev, uch = n // cu, n % cu
                    val = D[32 * l + sch, dz * ncol + n]
                    if swap:
                        dw[lev * 9 + (2 - dz) * 3 + (2 - l), sch, uch] += val
                    else:
                        dw[(2 - lev) * 9 + dz * 3 + l, uch, sch] += val
    return dw, db


@pytest.mark.parametrize("cin,cout", [(32, 32), (32, 16), (16, 32)])
def test_weight_gradient_layout_reproduces_the_oracle(cin, cout):
    rng = np.random.default_rng(40 + cin + cout)
    Y, Z, X = 3, 16, 16  # an odd Y: the top tile's second level lies past the volume
    x = so.bf16_round(rng.standard_normal((Y, Z, X, cin)))
    d = so.bf16_round(rng.standard_normal((Y, Z, X, cout)))
    dw, db = emulate(x, d)
    ref, dbr = so.conv_wgrad(x, d)
    np.testing.assert_allclose(dw, ref, rtol=0, atol=1e-12 * np.abs(ref).max())
    np.testing.assert_allclose(db, dbr, rtol=0, atol=1e-12 * np.abs(dbr).max())


@pytest.mark.parametrize("cu", [32, 16])
def test_producer_stores_spread_over_the_banks(cu):
    """16-byte rows: bank group = row mod 8, and 32 stores of 16 bytes need 4 wavefronts at best.  The U
    stores always take 4; the S stores too, except in a warp that crosses from one z row of the halo to the
    next (44 chunks per z row), which takes 5."""
    g = geom(cu)
    worst_s, worst_u, waves_s = 0, 0, []
    for base in range(0, TY * ZR * L * 4 - 32, 32):
        ws = np.bincount(np.array([s_row(c, 4)[-1] for c in range(base, base + 32)]) % 8, minlength=8).max()
        worst_s = max(worst_s, ws)
        waves_s.append(ws)
    for base in range(0, g["UL"] * TZ * TXW * g["KCU"] - 32, 32):
        wu = np.bincount(np.array([u_row(c, g)[-1] for c in range(base, base + 32)]) % 8, minlength=8).max()
        worst_u = max(worst_u, wu)
    assert worst_u == 4 and worst_s <= 5 and np.mean(waves_s) < 4.5
