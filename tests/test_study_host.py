"""Host logic of the long-run studies: profiles from plane sums, folding,
profile errors and the stationarity measures (CPU only, synthetic inputs)."""
import numpy as np

from littleharsh_gb300 import study


def _sums(n, ngx, ngz, U, urms, nyu=9):
    P = n * ngx * ngz
    st = {k: np.zeros(nyu) for k in ("Um", "U2m", "Vm", "V2m", "Wm", "W2m", "Pm", "P2m", "UVm", "UWm", "VWm")}
    st["Um"][:] = U * P
    st["U2m"][:] = (urms ** 2 + U ** 2) * P
    st["V2m"][:] = 0.25 * P
    st["P2m"][:] = 4.0 * P
    st["UVm"][:] = -0.1 * P
    return st


def test_profiles_recover_mean_and_rms():
    st = _sums(3, 8, 4, U=1.5, urms=0.2)
    pr = study.profiles(3, st, 8, 4)
    np.testing.assert_allclose(pr["U"], 1.5)
    np.testing.assert_allclose(pr["urms"], 0.2, rtol=1e-12)
    np.testing.assert_allclose(pr["vrms"], 0.5)
    np.testing.assert_allclose(pr["prms"], 2.0)
    np.testing.assert_allclose(pr["uv"], -0.1)


def test_fold_symmetric_and_antisymmetric():
    y = np.linspace(-1.1, 1.1, 9)
    grids = {"u": y, "v": y[:-1] + 0.5 * np.diff(y), "p": y[1:-1]}
    prof = {"U": 1 - y ** 2 + 0.1 * y, "uv": y.copy(), "vrms": np.ones(8), "urms": np.ones(9), "wrms": np.ones(9),
            "prms": np.ones(7)}
    f = study.fold(prof, grids)
    np.testing.assert_allclose(f["U"], 1 - y ** 2, atol=1e-15)   # the odd part averages out
    np.testing.assert_allclose(f["uv"], y, atol=1e-15)           # odd profile kept
    assert study.interior(grids)["u"].sum() == 7 and study.interior(grids)["p"].sum() == 7


def test_stationarity_measures():
    recs = [{"step": 100 * (i + 1)} for i in range(20)]
    devs = [1.0, 0.8, 0.5, 0.2, 0.05, 0.2, 0.04, 0.03, 0.05, 0.02] + [0.03] * 10
    # blocks of 2 windows: first block within 0.06 ends at window 4 -> begins at window 3 (step 300)
    assert study.first_within(recs, devs, 0.06, 2) == 300
    # stays within from window 6 on -> the block ending there begins at window 5 (step 500)
    assert study.stationary_from(recs, devs, 0.06, 2) == 500
    assert study.stationary_from(recs, devs, 0.001, 2) is None
    # a run that only settles in its last window has not stayed settled
    assert study.stationary_from(recs, [1.0] * 19 + [0.0], 0.5, 2) is None


def test_command_line_runs_after_every_definition():
    """`python -m littleharsh_gb300.study` calls main() from the module's last statement, so every
    function main() dispatches to exists by then."""
    import ast
    import inspect
    tree = ast.parse(inspect.getsource(study))
    last = tree.body[-1]
    assert isinstance(last, ast.If) and "__main__" in ast.unparse(last.test)
    assert not any(isinstance(n, (ast.FunctionDef, ast.ClassDef)) for n in tree.body[tree.body.index(last):])
