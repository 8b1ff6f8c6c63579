"""lh_project_noalloc: the projection for callers that cannot allocate device
memory (their fields live in device arrays someone else owns, e.g. OpenACC or
CUDA Fortran arrays of a Fortran driver, or one pre-carved memory arena).

The caller owns the velocity arrays; the entry point keeps all its scratch in a
static device array.  Its output must equal lh_project's on the same input,
on two calls in a row (the second call sees the first call's leftovers in the
shared scratch), and a call after the first must leave the device's free memory
unchanged.  Its parameter checks are those of lh_init and run before any CUDA
call, so they are tested without a GPU.
"""
import ctypes as C

import numpy as np
import pytest

from tests.helpers import SMALL, rel_l2


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _call(L, prm, g, ptrs, dt=0.01, stream=None):
    return L.lh_project_noalloc(C.byref(prm), _dp(g["yu"]), _dp(g["dthdyu"]), _dp(g["dthdyv"]), *ptrs, dt, stream)


def _corruptions(prm):
    """Parameter blocks lh_init rejects: (description, edit)."""
    def n33(p):
        p.N[3 * 4 + 2] += 1  # N(3,3): v grid no longer one level shorter than the u grid
    def re0(p):
        p.Re = 0.0
    def odd(p):
        p.Ngal[1 * 4 + 0] += 1  # Ngal(1,1) odd and N(1,1) inconsistent
    def third(p):
        p.Ngal[3 * 4 + 0] //= 2  # the third band's x resolution differs from the first's
        p.N[3 * 4 + 0] //= 2
    def n30(p):
        p.N[0 * 4 + 2] += 1  # N(3,0) != N(4,0)
    return [("N(3,3)", n33), ("Re", re0), ("odd Ngal", odd), ("third band", third), ("N(3,0)", n30)]


def test_project_noalloc_rejects_what_lh_init_rejects():
    """The shared parameter checks: every block lh_init refuses is refused here with the same code, before any
    device work (dummy host pointers stand in for the fields and are never touched)."""
    import littleharsh_gb300 as lh
    L = lh.load_library()
    prm0, g, lu, lv = lh.setup(lh.Config(**SMALL).to_input())
    dummy = np.zeros(4)
    ptrs = [C.c_void_p(dummy.ctypes.data)] * 3
    for what, edit in _corruptions(prm0):
        prm = lh.Params.from_buffer_copy(prm0)
        edit(prm)
        h = C.c_void_p()
        rc_init = L.lh_init(C.byref(prm), *[_dp(g[k]) for k in ("yu", "yv", "dthdyu", "dthdyv", "dyu2i", "dyv2i")],
                            lu.ctypes.data, lu.shape[0], lv.ctypes.data, lv.shape[0], C.byref(h))
        assert rc_init == -1 and not h.value, what
        why_init = L.lh_last_error(None).decode()
        rc = _call(L, prm, g, ptrs)
        assert rc == rc_init, f"{what}: lh_project_noalloc returned {rc}, lh_init {rc_init}"
        assert L.lh_last_error(None).decode() == why_init, what
    assert all(v == 0 for v in dummy)


def test_project_noalloc_refuses_bands():
    """Two x/z resolutions are valid for lh_init but not built here: LH_EUNSUPPORTED."""
    import littleharsh_gb300 as lh
    L = lh.load_library()
    prm, g, _, _ = lh.setup(lh.Config(**dict(SMALL, ngalx=48, ngalz=48, ngalx2=24, ngalz2=24, ntilex=8,
                                              ntilez=8, dsty=4)).to_input())
    dummy = np.zeros(4)
    rc = _call(L, prm, g, [C.c_void_p(dummy.ctypes.data)] * 3)
    assert rc == -2, L.lh_last_error(None).decode()
    assert "resolutions" in L.lh_last_error(None).decode()


@pytest.mark.gpu
def test_project_noalloc_matches_project():
    torch = pytest.importorskip("torch")
    import littleharsh_gb300 as lh
    from littleharsh_gb300.initial import initial_field

    L = lh.load_library()
    s = lh.Solver(lh.Config(**SMALL))
    g = s.grid
    dt = 0.01
    for seed in (21, 22):
        u1, u2, u3, p = initial_field(g["yu"], g["yv"], s.nz, s.nkx, s.nyp, seed=seed)
        # the reference result: lh_project on a handle
        s.set_fields(u1, u2, u3, p)
        s.set_time(0.0, dt, 0.0)
        s.project()
        ref = s.get_fields()
        assert s.divmax() < 1e-10
        # the caller's own device arrays
        dev = [torch.from_numpy(np.ascontiguousarray(a).view(np.float64).copy()).to("cuda:0") for a in (u1, u2, u3)]
        torch.cuda.synchronize()
        stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        rc = L.lh_project_noalloc(C.byref(s.params), g["yu"].ctypes.data_as(C.POINTER(C.c_double)),
                                  g["dthdyu"].ctypes.data_as(C.POINTER(C.c_double)),
                                  g["dthdyv"].ctypes.data_as(C.POINTER(C.c_double)),
                                  C.c_void_p(dev[0].data_ptr()), C.c_void_p(dev[1].data_ptr()),
                                  C.c_void_p(dev[2].data_ptr()), dt, stream)
        assert rc == 0, L.lh_last_error(None).decode()
        got = [t.cpu().numpy().view(np.complex128).reshape(a.shape) for t, a in zip(dev, (u1, u2, u3))]
        for name, a, b in zip(("u1", "u2", "u3"), got, ref[:3]):
            e = rel_l2(a, b)
            assert e < 1e-11, f"seed {seed} {name}: rel L2 {e:.3e}"


@pytest.mark.gpu
def test_project_noalloc_allocates_nothing():
    """After a first call (which may place the 64 MiB array on the device under lazy module loading), further
    calls leave the device's free memory exactly as it was."""
    torch = pytest.importorskip("torch")
    import littleharsh_gb300 as lh
    from littleharsh_gb300.initial import initial_field

    L = lh.load_library()
    prm, g, _, _ = lh.setup(lh.Config(**SMALL).to_input())
    nkx, nz, nyp = prm.N[1 * 4 + 0] // 2 + 1, prm.N[1 * 4 + 1], len(g["yu"]) - 2
    u1, u2, u3, _ = initial_field(g["yu"], g["yv"], nz, nkx, nyp, seed=31)
    dev = [torch.from_numpy(np.ascontiguousarray(a).view(np.float64).copy()).to("cuda:0") for a in (u1, u2, u3)]
    ptrs = [C.c_void_p(t.data_ptr()) for t in dev]
    torch.cuda.synchronize()
    assert _call(L, prm, g, ptrs) == 0, L.lh_last_error(None).decode()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        assert _call(L, prm, g, ptrs) == 0, L.lh_last_error(None).decode()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, f"free device memory changed by {free1 - free0} bytes"


@pytest.mark.gpu
def test_project_noalloc_rejects_grids_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    import littleharsh_gb300 as lh

    L = lh.load_library()
    big = dict(SMALL, ngalx=576, ngalz=576, ny=385, dsty=32, ntilex=48, ntilez=24, dstx=8, dstz=8, posth=0.1)
    prm, g, _, _ = lh.setup(lh.Config(**big).to_input())
    x = torch.zeros(8, dtype=torch.float64, device="cuda:0")  # never touched: the size check comes first
    ptr = C.c_void_p(x.data_ptr())
    rc = L.lh_project_noalloc(C.byref(prm), g["yu"].ctypes.data_as(C.POINTER(C.c_double)),
                              g["dthdyu"].ctypes.data_as(C.POINTER(C.c_double)),
                              g["dthdyv"].ctypes.data_as(C.POINTER(C.c_double)), ptr, ptr, ptr, 0.01, None)
    assert rc == -1  # LH_EINVAL
    assert "limited to" in L.lh_last_error(None).decode()
