"""Self-pinning of the CPU oracle's building blocks against numpy and dense
linear algebra (the reference has no tests or golden vectors of its own)."""
import numpy as np
import pytest

from tests.helpers import SMALL


@pytest.mark.parametrize("n", [2, 3, 4, 6, 8, 12, 16, 18, 24, 36, 48, 96, 144, 288, 576])
def test_c2c_matches_numpy(oracle_mod, n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    f = oracle_mod.fft_c2c(x, -1)
    b = oracle_mod.fft_c2c(x, +1)
    assert np.abs(f - np.fft.fft(x)).max() < 1e-13 * n
    assert np.abs(b - np.fft.ifft(x) * n).max() < 1e-13 * n


def test_c2c_rejects_other_factors(oracle_mod):
    with pytest.raises(ValueError):
        oracle_mod.fft_c2c(np.ones(10), -1)


@pytest.mark.parametrize("n", [6, 12, 24, 96, 576])
def test_rft_packing_and_normalisation(oracle_mod, n):
    """rft_buff.f:24-86: forward packs cc(k)=c(2k+1)+i c(2k+2), k=0..n/2, scaled by
    1/n, with Im cc(0) = Im cc(n/2) = 0; the inverse is unnormalised."""
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n)
    c = oracle_mod.rft(x, n, -1)
    ref = np.fft.rfft(x) / n
    assert np.abs(c[0::2] - ref.real).max() < 1e-15 * n
    assert np.abs(c[1::2] - ref.imag).max() < 1e-15 * n
    assert c[1] == 0.0 and c[n + 1] == 0.0
    back = oracle_mod.rft(c, n, +1)[:n]
    assert np.abs(back - x).max() < 1e-14 * n


def test_rft_inverse_ignores_imaginary_of_mean_and_nyquist(oracle_mod):
    n = 12
    c = np.zeros(n + 2)
    c[0], c[1], c[n], c[n + 1] = 1.0, 5.0, 0.5, -7.0
    x = oracle_mod.rft(c, n, +1)[:n]
    expect = 1.0 + 0.5 * (-1.0) ** np.arange(n)
    assert np.abs(x - expect).max() < 1e-14


def _pad_spectrum(spec, ngz, ngx):
    nz, nkx = spec.shape
    full = np.zeros((ngz, ngx // 2 + 1), np.complex128)
    h = nz // 2
    full[:h, :nkx] = spec[:h]
    full[h + ngz - nz:, :nkx] = spec[h:]
    return full


def test_plane_transforms_match_numpy(oracle_mod):
    o = oracle_mod.Oracle(**SMALL)
    rng = np.random.default_rng(3)
    spec = rng.standard_normal((o.nz, o.nkx)) + 1j * rng.standard_normal((o.nz, o.nkx))
    phys = o.to_phys(spec)
    full = _pad_spectrum(spec, o.ngz, o.ngx)
    # z inverse (complex) then x inverse (real, Im of kx=0 dropped): numpy irfft semantics
    ref = np.fft.irfft(np.fft.ifft(full, axis=0) * o.ngz, n=o.ngx, axis=1) * o.ngx
    assert np.abs(phys - ref).max() < 1e-12
    x = rng.standard_normal((o.ngz, o.ngx))
    sp = o.to_spec(x)
    fr = np.fft.fft(np.fft.rfft(x, axis=1) / o.ngx, axis=0) / o.ngz
    h = o.nz // 2
    ref2 = np.concatenate([fr[:h, :o.nkx], fr[h + o.ngz - o.nz:, :o.nkx]], axis=0)
    assert np.abs(sp - ref2).max() < 1e-14


def test_three_halves_rule_has_no_aliasing(oracle_mod):
    """The product of two resolved modes, formed on the 3/2 grid and truncated,
    equals the analytic product restricted to the resolved modes."""
    o = oracle_mod.Oracle(**SMALL)
    nz, nkx = o.nz, o.nkx
    a = np.zeros((nz, nkx), np.complex128)
    b = np.zeros((nz, nkx), np.complex128)
    kxa, kza, kxb, kzb = nkx - 2, nz // 2 - 2, nkx - 3, -(nz // 2 - 3)
    a[kza % nz, kxa] = 0.5
    b[kzb % nz, kxb] = 0.25 - 0.5j
    prod = o.to_spec(o.to_phys(a) * o.to_phys(b))
    # cos-type products: a*b contains (kxa+kxb, kza+kzb) and (kxa-kxb, kza-kzb) pairs
    expect = np.zeros_like(prod)
    ca, cb = 0.5, 0.25 - 0.5j
    for (kx, kz, c) in ((kxa + kxb, kza + kzb, ca * cb), (kxa - kxb, kza - kzb, ca * np.conj(cb))):
        if kx < 0:
            kx, kz, c = -kx, -kz, np.conj(c)
        if kx < nkx and -(nz // 2) <= kz < nz // 2:
            expect[kz % nz, kx] += c
    # kx = 0 modes also carry the conjugate partner
    assert np.abs(prod - expect).max() < 1e-14


def test_tridiagonal_matches_dense(oracle_mod):
    rng = np.random.default_rng(7)
    n = 40
    a1 = rng.standard_normal(n) * 0.3
    a3 = rng.standard_normal(n) * 0.3
    a2 = 2.0 + rng.random(n)
    a1[0] = 0.0
    a3[-1] = 0.0
    A = np.diag(a2) + np.diag(a1[1:], -1) + np.diag(a3[:-1], 1)
    rhs = rng.standard_normal(n)
    x = oracle_mod.tridiag_solve(a1, a2, a3, rhs)
    assert np.abs(x - np.linalg.solve(A, rhs)).max() < 1e-13


def _parseval_sum(f, g, ngx, ngz):
    """sum over the padded physical plane of f*g from the spectral planes f, g
    (nz x nkx), with the real x-inverse's treatment of the kx = 0 line."""
    nz, nkx = f.shape
    tot = 2.0 * np.sum((f[:, 1:] * np.conj(g[:, 1:])).real)
    kk = np.arange(nz)
    pk = (nz - kk) % nz
    re = (f[:, 0] * np.conj(g[:, 0])).real
    cross = (f[:, 0] * g[pk, 0]).real
    line = 0.5 * (re + cross)
    line[nz // 2] = 0.5 * re[nz // 2]
    return ngx * ngz * (tot + line.sum())


def test_plane_sums_by_parseval(oracle_mod):
    """The identity the GPU statistics rely on: physical-plane sums of products
    equal weighted sums over the spectral coefficients, also for a kx = 0 line
    that is not Hermitian (its imaginary part is dropped by the inverse)."""
    o = oracle_mod.Oracle(**SMALL)
    rng = np.random.default_rng(5)
    f = rng.standard_normal((o.nz, o.nkx)) + 1j * rng.standard_normal((o.nz, o.nkx))
    g = rng.standard_normal((o.nz, o.nkx)) + 1j * rng.standard_normal((o.nz, o.nkx))
    pf, pg = o.to_phys(f), o.to_phys(g)
    assert abs((pf * pg).sum() - _parseval_sum(f, g, o.ngx, o.ngz)) < 1e-12 * abs((pf * pg).sum()) + 1e-10
    assert abs((pf * pf).sum() - _parseval_sum(f, f, o.ngx, o.ngz)) < 1e-12 * (pf * pf).sum()
    assert abs(pf.sum() - o.ngx * o.ngz * f[0, 0].real) < 1e-10


def test_omega_x_statistics_from_the_spectra(oracle_mod):
    """The oracle's omega_x rows (wxm, wx2m) against an evaluation from the spectral coefficients alone:
    omega_x(face j) = dthdyv(j) (w(centre j+1) - w(centre j)) - i kz v(face j) per mode; its plane sum is
    Ngx Ngz Re omega(0,0) and its sum of squares Ngx Ngz times Parseval's sum (kx > 0 twice, the Hermitian kx = 0
    line once; the field has no lone -N2/2 mode)."""
    from tests.helpers import projected_ic
    o = oracle_mod.Oracle(**SMALL)
    u1, u2, u3, p = projected_ic(o, seed=9)
    o.set_fields(u1, u2, u3, p)
    o.stats_accumulate()
    n, st = o.stats()
    assert n == 1
    g = o.grid()
    kz = 2.0 * np.where(np.arange(o.nz) < o.nz // 2, np.arange(o.nz), np.arange(o.nz) - o.nz)
    om = g["dthdyv"][:, None, None] * (u3[1:] - u3[:-1]) - 1j * kz[None, :, None] * u2
    pts = o.ngx * o.ngz
    mean = pts * om[:, 0, 0].real
    sq = pts * (2.0 * np.sum(np.abs(om[:, :, 1:]) ** 2, axis=(1, 2)) + np.sum(np.abs(om[:, :, 0]) ** 2, axis=1))
    nyv = o.nyv
    assert np.abs(st[11, :nyv] - mean).max() < 1e-11 * np.abs(mean).max() + 1e-12 * pts
    assert np.abs(st[12, :nyv] - sq).max() < 1e-11 * sq.max()
    assert sq.max() > 0
