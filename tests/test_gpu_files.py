"""The reference's file formats written and read by the library, checked with
an independent numpy reader of Fortran sequential unformatted records."""
import os

import numpy as np
import pytest

from tests.helpers import SMALL, projected_ic, rel_l2

pytestmark = pytest.mark.gpu


def fortran_records(path):
    data = open(path, "rb").read()
    out, pos = [], 0
    while pos < len(data):
        n = int(np.frombuffer(data, np.int32, 1, pos)[0])
        out.append(data[pos + 4:pos + 4 + n])
        assert int(np.frombuffer(data, np.int32, 1, pos + 4 + n)[0]) == n
        pos += 8 + n
    return out


def _solver(oracle_mod):
    import littleharsh_gb300 as lh
    o = oracle_mod.Oracle(**SMALL)
    u1, u2, u3, p = projected_ic(o, seed=4)
    s = lh.Solver(lh.Config(**SMALL))
    s.set_fields(u1, u2, u3, p)
    s.set_time(0.0, o.cfl_dt(0.5), 0.0)
    s.step(2)
    return s


def test_restart_roundtrip_in_read_in_format(oracle_mod, tmp_path):
    import littleharsh_gb300 as lh
    s = _solver(oracle_mod)
    name = "_0016x0016x0033_t00000.dat"
    s.write_restart(str(tmp_path), name, iteration=7)
    f = s.get_fields()
    N = np.array(s.params.N, np.int32)
    for tag, arr, ny, y in (("u1", f[0], s.nyu, s.grid["yu"]), ("u2", f[1], s.nyv, s.grid["yv"]),
                            ("u3", f[2], s.nyu, s.grid["yu"]), ("p", f[3], s.nyp, s.grid["yu"][1:])):
        recs = fortran_records(os.path.join(tmp_path, tag + name))
        assert len(recs) == 3 + ny
        hdr = recs[0]
        t, Re, alp, bet, mpgx = np.frombuffer(hdr, np.float64, 5)
        nband, it = np.frombuffer(hdr, np.int32, 2, 40)
        assert (nband, it) == (3, 7) and abs(t - s.time()["t"]) < 1e-15 and Re == SMALL["Re"]
        np.testing.assert_array_equal(np.frombuffer(recs[1], np.int32), N)
        for jj in range(ny):
            r = recs[3 + jj]
            jin, band, nx, nz = np.frombuffer(r, np.int32, 4)
            assert (nx, nz) == (2 * s.nkx, s.nz)
            assert jin == jj + (s.jp0 if tag == "p" else s.ju0)
            buff = np.frombuffer(r, np.float64, nx * nz, 24).reshape(nz, nx)  # buffSR(nx, nz), column-major
            np.testing.assert_array_equal(buff[:, 0::2] + 1j * buff[:, 1::2], arr[jj])
    s2 = lh.Solver(lh.Config(**SMALL))
    t, it = s2.read_restart(str(tmp_path), name)
    assert it == 7
    for a, b in zip(s2.get_fields(), f):
        np.testing.assert_array_equal(a, b)
    tm = s.time()
    s2.set_time(t, tm["dt"], tm["mpgx"], tm["QxT"])
    s.step(1)
    s2.step(1)
    for a, b in zip(s2.get_fields(), s.get_fields()):
        assert rel_l2(a, b) < 1e-14


def test_stats_file(oracle_mod, tmp_path):
    s = _solver(oracle_mod)
    s.stats_accumulate()
    s.cond_accumulate()
    n, st = s.stats_flush(reset=False)
    nc, cd = s.cond_flush(reset=False)
    path = os.path.join(tmp_path, "stats.dat")
    s.write_stats(path, iteration=3)
    recs = fortran_records(path)
    assert len(recs) == 5 + 13 + 13
    np.testing.assert_array_equal(np.frombuffer(recs[1], np.int32), np.array(s.params.Ngal, np.int32))
    assert np.frombuffer(recs[4], np.int32)[0] == 1
    names = ["Um", "U2m", "Vm", "V2m", "Wm", "W2m", "Pm", "P2m", "UVm", "UWm", "VWm", "wxm", "wx2m"]
    for k, name in enumerate(names):
        np.testing.assert_array_equal(np.frombuffer(recs[5 + k], np.float64), st[name])
    cnames = ["UmC", "U2mC", "VmC", "V2mC", "WmC", "W2mC", "PmC", "P2mC", "UVmC", "UWmC", "VWmC", "wxmC", "wx2mC"]
    for k, name in enumerate(cnames):
        np.testing.assert_array_equal(np.frombuffer(recs[18 + k], np.float64), cd[name].ravel())
    # the omega_x records hold the accumulated vorticity (not zeros)
    assert np.abs(st["wx2m"]).max() > 0 and np.abs(cd["wx2mC"]).max() > 0
    # write_stats resets the accumulators
    assert s.stats_flush()[0] == 0 and s.cond_flush()[0] == 0


def test_spectra_file_folds_kz(oracle_mod, tmp_path):
    s = _solver(oracle_mod)
    s.spectra_accumulate()
    n, sp = s.spectra_flush(reset=False)
    s.write_spectra(str(tmp_path), "_t.dat", iteration=1)
    recs = fortran_records(os.path.join(tmp_path, "spU__t.dat"))
    nz, nkx, nh = s.nz, s.nkx, s.nz // 2 + 1
    buf = np.frombuffer(recs[5], np.float64).reshape(s.nyu, nh, nkx)
    raw = sp[0].reshape(s.nyu, nz, nkx)
    expect = np.zeros((s.nyu, nh, nkx))
    for kk in range(nz):
        k = kk + 1
        kf = nz + 2 - k if k > nz // 2 else k
        expect[:, kf - 1] += raw[:, kk]
    expect[:, :, 1:] *= 2.0
    np.testing.assert_allclose(buf, expect, rtol=1e-15, atol=0)
