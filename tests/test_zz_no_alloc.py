"""lh_project_noalloc: the projection for callers that cannot allocate device
memory (their fields live in device arrays someone else owns, e.g. OpenACC or
CUDA Fortran arrays of a Fortran driver, or one pre-carved memory arena).

The caller owns the velocity arrays; the entry point keeps all its scratch in a
static device array.  Its output must equal lh_project's on the same input,
on two calls in a row (the second call sees the first call's leftovers in the
shared scratch).
"""
import ctypes as C

import numpy as np
import pytest

from tests.helpers import SMALL, rel_l2

pytestmark = pytest.mark.gpu


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
