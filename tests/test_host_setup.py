"""Host-side set-up of the product (C++ restatement of start.f90's input reader,
y_grid_canopy and boundary_canopies) against the reference's own input.in and
the oracle's independent restatement.  No GPU is needed: these entry points
are host code inside the CUDA library."""
import os
import re

import numpy as np
import pytest

from tests.helpers import C1, SMALL, SMOOTH

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")

# Values of the reference's input.in, read off the file (start.f90:63-196 reads
# them with FORMATs (7X,D10.1), (7X,I10), (12X,I5) and (7X,A90)).
EXPECTED_INPUT = dict(Re=1452.0, alp=1.0, bet=2.0, ngalx1=576, ngalx2=144, ngalz1=288, ngalz2=144, ny=177,
                      dyq=15.0, ppp=5, flag_init=1, fnameimb="u1_0256x0256x0453_t06071.dat", dirin="./input/",
                      dirout="./output/", CFL=0.7, nwrite=10, flag_ctpress=0, mpgx=0.0, Kib=1.0, maxerr=1e-8,
                      maxt=2000.0, maxA=-4.0, physlim_bot=8, physlim_top=146, geometry_type=3, ntilex=8, ntilez=4,
                      posth=0.5, npeakx=13, npeakz=13, Lfracx=3.0, Lfracz=3.0, dsty=100, dstx=13, dstz=13)


@pytest.fixture(scope="module")
def lh():
    import littleharsh_gb300
    littleharsh_gb300.load_library()
    return littleharsh_gb300


def test_reads_reference_input(lh, oracle_mod):
    path = os.path.join(GOLDEN, "input.in")
    got = lh.read_input(path).as_dict()
    for k, v in EXPECTED_INPUT.items():
        assert got[k] == v, k
    assert oracle_mod.read_input(path) == got


def _write_input(tmp_path, replace: dict) -> str:
    lines = open(os.path.join(GOLDEN, "input.in")).read().split("\n")
    for lineno, text in replace.items():
        lines[lineno - 1] = text
    p = tmp_path / "input.in"
    p.write_text("\n".join(lines))
    return str(p)


def test_fortran_edit_descriptor_rules(lh, oracle_mod, tmp_path):
    # D10.1 without a decimal point carries one implied decimal; blanks are ignored
    p = _write_input(tmp_path, {10: "Re=       14520    ! no decimal point", 13: "alp   =    1 .5d0",
                                34: "CFL   =    5.0-1 !", 36: "flpress    =    1 !", 38: "mpgx  = -3.0e-3"})
    a = lh.read_input(p).as_dict()
    assert a["Re"] == 1452.0 and a["alp"] == 1.5 and a["CFL"] == 0.5
    assert a["flag_ctpress"] == 1 and a["mpgx"] == -3.0e-3
    assert oracle_mod.read_input(p) == a


def test_rejects_bad_pressure_flag(lh, tmp_path):
    p = _write_input(tmp_path, {36: "flpress    =    2 !"})
    with pytest.raises(lh.LhError):
        lh.read_input(p)


def test_rejects_nonpositive_tiles(lh, tmp_path):
    p = _write_input(tmp_path, {55: "ntilex=         0"})
    with pytest.raises(lh.LhError):
        lh.read_input(p)


@pytest.mark.parametrize("cfg", [SMALL, C1, SMOOTH], ids=["canopy24", "config1", "smooth"])
def test_grid_matches_oracle(lh, oracle_mod, cfg):
    prm, g, lu, lv = lh.setup(lh.Config(**cfg).to_input())
    o = oracle_mod.Oracle(**cfg)
    og = o.grid()
    for k in ("yu", "yv", "dthdyu", "dthdyv", "dyu2i", "dyv2i"):
        np.testing.assert_array_equal(g[k], og[k])
    np.testing.assert_array_equal(np.array(prm.gridweighting), og["gw"].ravel())
    N = np.array(prm.N).reshape(5, 4)
    assert [[N[b][r] for b in range(5)] for r in range(4)] == [list(row) for row in o.sz.N]
    assert prm.nn == cfg["ny"] - 2


def test_grid_geometry(lh):
    prm, g, _, _ = lh.setup(lh.Config(**C1).to_input())
    yv, yu, dsty = g["yv"], g["yu"], C1["dsty"]
    assert abs(yv[0] + 1.0 + C1["posth"]) < 1e-14          # bottom wall at -1-h
    assert abs(yv[dsty] + 1.0) < 1e-14                      # bottom canopy tip at -1
    assert abs(yv[-1] - 1.0 - C1["posth"]) < 1e-14          # top wall
    np.testing.assert_allclose(yv, -yv[::-1], atol=1e-14)   # symmetric channel
    np.testing.assert_allclose(yu, -yu[::-1], atol=1e-14)
    assert np.all(np.diff(yv) > 0) and np.all(np.diff(yu) > 0)
    # tanh-like stretching of configuration 1: dy_max/dy_min between the tips ~ dyq
    dy = np.diff(yv[dsty:len(yv) - dsty])
    assert abs(dy.max() / dy.min() - C1["dyq"]) < 0.2


@pytest.mark.parametrize("cfg", [SMALL, C1], ids=["canopy24", "config1"])
def test_canopy_lists_match_oracle_masks(lh, oracle_mod, cfg):
    prm, g, lu, lv = lh.setup(lh.Config(**cfg).to_input())
    o = oracle_mod.Oracle(**cfg)
    pu, mu, pv, mv = o.ib()
    # lists as boundary_canopies builds them: both canopies, each stem replicated on every tile
    stem = cfg["dsty"] * cfg["dstx"] * cfg["dstz"]
    assert lu.shape == (2 * cfg["ntilex"] * cfg["ntilez"] * stem, 3)
    for planes, masks, lst in ((pu, mu, lu), (pv, mv, lv)):
        for q, j in enumerate(planes):
            m = np.zeros_like(masks[q])
            sel = lst[lst[:, 2] == j]
            m[sel[:, 1] - 1, sel[:, 0] - 1] = 1
            np.testing.assert_array_equal(m, masks[q])


def test_header_declares_exported_symbols(lh):
    """Every lh_* function declared in include/*.h is exported by the library."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    inc = os.path.join(root, "include")
    declared = set()
    for f in sorted(os.listdir(inc)):
        if f.endswith(".h"):
            hdr = open(os.path.join(inc, f)).read()
            declared |= set(re.findall(r"^\s*(?:int|void|const char\s*\*)\s+(lh_[a-z0-9_]+)\s*\(", hdr, re.M))
    assert declared == set(lh.EXPORTED_SYMBOLS)
    L = lh.load_library()
    for name in declared:
        assert hasattr(L, name), name


def test_tcgen05_convolution_rejects_misaligned_tensors(lh):
    """The tcgen05 convolution moves its input, output, residual and gate 16 bytes at a time: a tensor that
    does not start on a 16-byte boundary is refused before anything is launched (addresses only, no GPU)."""
    L = lh.load_library()
    ok_in, ok_w, ok_out = 0x10000, 0x20000, 0x30000
    bias, res, gate = 0x40000, 0x50000, 0x60000
    BIAS, RES, GATE = 8, 2, 4
    args = dict(cin=32, cout=32, X=64, Y=4, Z=16)

    def call(inp, w, out, res_p, gate_p, flags):
        return L.lh_sr_conv_fwd_tc(args["cin"], args["cout"], inp, w, bias, out, 0, res_p, gate_p, flags,
                                   args["X"], args["Y"], args["Z"], None)
    assert call(ok_in, ok_w, ok_out + 8, None, None, BIAS) == -1
    assert call(ok_in + 4, ok_w, ok_out, None, None, BIAS) == -1
    assert call(ok_in, ok_w, ok_out, res + 2, None, BIAS | RES) == -1
    assert call(ok_in, ok_w, ok_out, None, gate + 8, BIAS | GATE) == -1
    assert b"misaligned" in L.lh_last_error(None)


def test_geometry_without_forcing_builder_is_refused(lh):
    """geometry_type 1 and 2 have no forcing builder in the reference's shipped solver: the grid set-up refuses
    them with LH_EUNSUPPORTED (-2) before any device work."""
    from tests.helpers import SMALL
    for gt in (1, 2):
        with pytest.raises(lh.LhError, match=r"\(-2\)"):
            lh.Solver(lh.Config(**dict(SMALL, geometry_type=gt)))
