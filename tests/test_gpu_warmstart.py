"""The learned warm start on the device: pairs, a few training steps, the start.

Small versions of the experiment's steps on configuration 1's grid and its
half-resolution coarse grid: the network's training lowers the loss on the
pairs it sees, and the corrected field becomes divergence free under the
solver's projection and steps stably.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_pairs_training_and_start():
    import torch
    import littleharsh_gb300 as lh
    from littleharsh_gb300 import study, warmstart as ws
    from littleharsh_gb300.srnet import SRNet
    from littleharsh_gb300.workloads import CONFIG1, CONFIG1_COARSE
    fine = lh.Solver(lh.Config(**CONFIG1))
    study.seeded_start([fine], 3, 0.5)
    fgi = ws.GridInfo(fine)
    cgi = ws.GridInfo.from_config(CONFIG1_COARSE)
    pairs = ws.PairSet(fgi, cgi)
    for _ in range(3):
        fine.step(20)
        pairs.add_snapshot(*ws.fields_to_device(fine.get_fields()[:3]))
    assert len(pairs) == 3
    # the filter removes something, the lifted field keeps most of the snapshot
    b, t = pairs.base[0], pairs.target[0]
    err = ws.mse_of(b, t)
    assert 0.0 < err < 0.05 * float((t.double() ** 2).mean())
    net = SRNet(seed=0)
    v0 = ws.evaluate(net, pairs, [0, 1])
    assert v0[0] == pytest.approx(v0[1], rel=1e-6)  # the untrained correction is zero
    ws.train(net, pairs, [0, 1], [2], epochs=20, lr=1e-3)
    v1 = ws.evaluate(net, pairs, [0, 1])
    assert v1[0] < 0.9 * v0[0], (v0, v1)  # training lowers the error on the pairs it was trained on
    assert abs(v1[1] - v0[1]) < 1e-12  # the lifted fields are untouched
    # the start: coarse field -> lifted + corrected -> projected -> steps
    coarse = lh.Solver(lh.Config(**CONFIG1_COARSE))
    study.seeded_start([coarse], 4, 0.5)
    coarse.step(5)
    cf = ws.fields_to_device(coarse.get_fields()[:3])
    s = lh.Solver(lh.Config(**CONFIG1))
    u1, u2, u3 = ws.warm_field(net, *cf, cgi, fgi, use_net=True)
    s.set_fields(u1, u2, u3, np.zeros((s.nyp, s.nz, s.nkx), np.complex128))
    s.project()
    assert s.divmax() < 1e-10
    s.set_time(0.0, s.cfl_dt(0.5), 0.0)
    s.step(10)
    f = s.get_fields()
    assert all(np.all(np.isfinite(x)) for x in f)
    torch.cuda.synchronize()


def test_network_lowers_held_out_error():
    """Trained on pairs from one seeded flow, the network lowers the error of the lifted field on pairs from an
    independent flow it never saw (another seed), against plain lifting of the same coarse fields."""
    import littleharsh_gb300 as lh
    from littleharsh_gb300 import study, warmstart as ws
    from littleharsh_gb300.srnet import SRNet
    from littleharsh_gb300.workloads import CONFIG1, CONFIG1_COARSE
    fgi = ws.GridInfo.from_config(CONFIG1)
    cgi = ws.GridInfo.from_config(CONFIG1_COARSE)
    pairs = ws.PairSet(fgi, cgi)
    for seed in (3, 7):  # training flow, held-out flow
        fine = lh.Solver(lh.Config(**CONFIG1))
        study.seeded_start([fine], seed, 0.5)
        fine.step(200)
        for _ in range(6 if seed == 3 else 3):
            fine.step(40)
            pairs.add_snapshot(*ws.fields_to_device(fine.get_fields()[:3]))
        fine.close()
    train_idx, held_out = list(range(6)), [6, 7, 8]
    net = SRNet(seed=0)
    ws.train(net, pairs, train_idx, held_out, epochs=40, lr=1e-3)
    v_net, v_lift = ws.evaluate(net, pairs, held_out)
    assert v_net < 0.95 * v_lift, (v_net, v_lift)
