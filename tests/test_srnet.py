"""The super-resolution network's kernels against the numpy oracle.

CPU: the oracle's network gradient against central finite differences (no
bf16 rounding), and its flipped-weight identity for the data gradient.
GPU: every kernel of include/lh_srnet.h against the oracle on the same
bf16 operands, then the gradient of the whole network.
"""
import numpy as np
import pytest

from oracle import sr_oracle as so


def rand_params(rng, shapes, scale=0.15):
    out = []
    for ci, co in shapes:
        w = so.bf16_round(rng.standard_normal((27, co, ci)) * scale / np.sqrt(27 * ci) * 3)
        b = (rng.standard_normal(co) * 0.05).astype(np.float32)
        out.append((w, b))
    return out


def small_shapes(nb, cin=3, ch=4, cout=3):
    return [(cin, ch)] + [(ch, ch)] * (2 * nb) + [(ch, cout)]


def test_oracle_dgrad_is_flipped_forward():
    rng = np.random.default_rng(0)
    d = rng.standard_normal((3, 4, 5, 6))
    w = rng.standard_normal((27, 6, 2))
    np.testing.assert_allclose(so.conv_dgrad(d, w), so.conv_fwd(d, so.flip_weights(w)), rtol=1e-12, atol=1e-12)


def test_oracle_conv_adjoint():
    """<conv(x), d> = <x, dgrad(d)> and = <w, wgrad(x, d)>."""
    rng = np.random.default_rng(1)
    x = rng.standard_normal((3, 4, 5, 2))
    d = rng.standard_normal((3, 4, 5, 3))
    w = rng.standard_normal((27, 3, 2))
    lhs = np.sum(so.conv_fwd(x, w) * d)
    assert abs(lhs - np.sum(x * so.conv_dgrad(d, w))) < 1e-10 * abs(lhs) + 1e-10
    dw, _ = so.conv_wgrad(x, d)
    assert abs(lhs - np.sum(w * dw)) < 1e-10 * abs(lhs) + 1e-10


def test_oracle_network_gradient_finite_differences():
    rng = np.random.default_rng(2)
    nb = 1
    Y, Z, X = 3, 4, 4
    params = [(w.astype(np.float64), b.astype(np.float64)) for w, b in rand_params(rng, small_shapes(nb), 1.0)]
    # the tail has 16 output channels in the kernels; the oracle only needs >= 3
    x = rng.standard_normal((Y, Z, X, 3))
    base = rng.standard_normal((Y * Z * X, 3))
    target = rng.standard_normal((Y * Z * X, 3))
    loss, grads = so.network_loss_and_grads(params, x, base, target, nblocks=nb, round_bf16=False)
    h = 1e-6
    for li in range(len(params)):
        for which in (0, 1):
            arr = params[li][which]
            for _ in range(3):
                idx = tuple(int(rng.integers(0, n)) for n in arr.shape)
                old = arr[idx]
                arr[idx] = old + h
                lp, _ = so.network_loss_and_grads(params, x, base, target, nblocks=nb, round_bf16=False)
                arr[idx] = old - h
                lm, _ = so.network_loss_and_grads(params, x, base, target, nblocks=nb, round_bf16=False)
                arr[idx] = old
                fd = (lp - lm) / (2 * h)
                an = grads[li][which][idx]
                assert abs(fd - an) <= 1e-6 * max(1.0, abs(fd)), (li, which, idx, fd, an)


def test_oracle_bf16_round():
    a = np.array([1.0, 1.00390625, 1.005859375, -3.14159, 0.0, 1e-30], np.float32)
    r = so.bf16_round(a)
    assert r[0] == 1.0 and r[1] == 1.0  # halfway between 1 and 1+2^-7 rounds to even
    assert r[2] == np.float32(1.0078125)
    assert abs(r[3] + 3.140625) < 1e-7
    np.testing.assert_array_equal(so.from_bf16_bits(so.bf16_bits(a)), r)


# ---------------------------------------------------------------------------- GPU

def _t(a, dtype):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda").to(dtype).contiguous()


@pytest.fixture(scope="module")
def lib():
    import littleharsh_gb300 as lh
    return lh.load_library()


VOL = (5, 8, 32)  # Y, Z, X: one tile row in x, one in z, edges in y


@pytest.mark.gpu
@pytest.mark.parametrize("cin,cout,f32", [(16, 32, False), (32, 32, False), (32, 16, False), (32, 16, True)])
@pytest.mark.parametrize("flags", [0, so.BIAS | so.RELU, so.BIAS | so.RES, so.GATE | so.RES])
def test_conv_fwd(lib, cin, cout, f32, flags):
    import torch
    from littleharsh_gb300 import srnet
    rng = np.random.default_rng(cin * 100 + cout + flags)
    Y, Z, X = VOL
    x = so.bf16_round(rng.standard_normal((Y, Z, X, cin)))
    w = so.bf16_round(rng.standard_normal((27, cout, cin)) / np.sqrt(27 * cin))
    b = rng.standard_normal(cout).astype(np.float32)
    res = so.bf16_round(rng.standard_normal((Y, Z, X, cout)))
    gate = so.bf16_round(rng.standard_normal((Y, Z, X, cout)))
    ref = so.conv_fwd(x, w, b, res, gate, flags)
    out = torch.empty((Y, Z, X, cout), dtype=torch.float32 if f32 else torch.bfloat16, device="cuda")
    xt, wt, bt, rt, gt = _t(x, torch.bfloat16), _t(w, torch.bfloat16), _t(b, torch.float32), \
        _t(res, torch.bfloat16), _t(gate, torch.bfloat16)
    rc = lib.lh_sr_conv_fwd(cin, cout, srnet._ptr(xt), srnet._ptr(wt), srnet._ptr(bt), srnet._ptr(out), int(f32),
                            srnet._ptr(rt), srnet._ptr(gt), flags, X, Y, Z, None)
    assert rc == 0
    torch.cuda.synchronize()
    got = out.float().cpu().numpy()
    if f32:
        np.testing.assert_allclose(got, ref, rtol=1e-5, atol=1e-5)
    else:  # one bf16 rounding of the fp32 result
        np.testing.assert_allclose(got, ref, rtol=2 ** -8, atol=1e-3)


@pytest.mark.gpu
@pytest.mark.parametrize("cin,cout", [(16, 32), (32, 32), (32, 16)])
def test_conv_wgrad_and_dgrad(lib, cin, cout):
    import torch
    from littleharsh_gb300 import srnet
    rng = np.random.default_rng(7 + cin + cout)
    Y, Z, X = VOL
    x = so.bf16_round(rng.standard_normal((Y, Z, X, cin)))
    d = so.bf16_round(rng.standard_normal((Y, Z, X, cout)))
    w = so.bf16_round(rng.standard_normal((27, cout, cin)) / np.sqrt(27 * cin))
    dw_ref, db_ref = so.conv_wgrad(x, d)
    dw = torch.zeros((27, cout, cin), dtype=torch.float32, device="cuda")
    db = torch.zeros(cout, dtype=torch.float32, device="cuda")
    xt, dt = _t(x, torch.bfloat16), _t(d, torch.bfloat16)
    assert lib.lh_sr_conv_wgrad(cin, cout, srnet._ptr(xt), srnet._ptr(dt), srnet._ptr(dw), srnet._ptr(db), X, Y, Z,
                                None) == 0
    # data gradient: flipped weights through the forward kernel
    wt = _t(w, torch.bfloat16)
    wf = torch.empty(27 * cin * cout, dtype=torch.bfloat16, device="cuda")
    assert lib.lh_sr_flip_weights(cin, cout, srnet._ptr(wt), srnet._ptr(wf), None) == 0
    torch.cuda.synchronize()
    np.testing.assert_array_equal(wf.float().cpu().numpy().reshape(27, cin, cout), so.flip_weights(w))
    scale = np.abs(dw_ref).max()
    np.testing.assert_allclose(dw.cpu().numpy(), dw_ref, rtol=1e-4, atol=1e-5 * scale)
    np.testing.assert_allclose(db.cpu().numpy(), db_ref, rtol=1e-4, atol=1e-4)
    if (cout, cin) in ((32, 16), (32, 32), (16, 32)):
        dx = torch.empty((Y, Z, X, cin), dtype=torch.bfloat16, device="cuda")
        assert lib.lh_sr_conv_fwd(cout, cin, srnet._ptr(dt), srnet._ptr(wf), None, srnet._ptr(dx), 0, None, None, 0,
                                  X, Y, Z, None) == 0
        torch.cuda.synchronize()
        np.testing.assert_allclose(dx.float().cpu().numpy(), so.conv_dgrad(d, w), rtol=2 ** -8, atol=1e-3)


def test_conv_wgrad_tcgen05_rejects_z_not_multiple_of_16(lib):
    """Checked before any device work: the tcgen05 weight gradient reduces over 16 z voxels per MMA."""
    import littleharsh_gb300 as lh
    assert lib.lh_sr_conv_wgrad_tc(32, 32, None, None, None, None, 32, 5, 8, None) == lh.LH_EINVAL
    assert b"multiple of 16" in lib.lh_last_error(None)


@pytest.mark.gpu
@pytest.mark.parametrize("cin,cout", [(16, 32), (32, 32), (32, 16)])
@pytest.mark.parametrize("Y,Z,X", [(5, 16, 32), (9, 48, 512)], ids=["12_tiles", "960_tiles"])
def test_conv_wgrad_tcgen05(lib, cin, cout, Y, Z, X):
    """The tcgen05 weight and bias gradients against the oracle.  Tiles are 2 levels x 16 z x 8 x columns:
    an odd Y leaves the second level of the top tiles past the volume (zeros), and 960 tiles give every
    persistent CTA six or seven, so its ring of stage buffers wraps around.  (16, 32) takes the path with the
    output gradient as the shifted operand and mirrored taps."""
    import ctypes
    import torch
    from littleharsh_gb300 import srnet
    rng = np.random.default_rng(900 + cin + cout + Y)
    x = so.bf16_round(rng.standard_normal((Y, Z, X, cin)))
    d = so.bf16_round(rng.standard_normal((Y, Z, X, cout)))
    dw_ref, db_ref = so.conv_wgrad(x, d)
    dw = torch.zeros((27, cout, cin), dtype=torch.float32, device="cuda")
    db = torch.zeros(cout, dtype=torch.float32, device="cuda")
    xt, dt = _t(x, torch.bfloat16), _t(d, torch.bfloat16)
    assert lib.lh_sr_conv_wgrad_tc(cin, cout, srnet._ptr(xt), srnet._ptr(dt), srnet._ptr(dw), srnet._ptr(db), X, Y,
                                   Z, None) == 0
    torch.cuda.synchronize()
    timed_out = ctypes.c_int32(-1)
    assert lib.lh_sr_tc_status(ctypes.byref(timed_out)) == 0 and timed_out.value == 0
    scale = np.abs(dw_ref).max()
    np.testing.assert_allclose(dw.cpu().numpy(), dw_ref, rtol=1e-4, atol=1e-5 * scale)
    np.testing.assert_allclose(db.cpu().numpy(), db_ref, rtol=1e-4, atol=1e-4)


@pytest.mark.gpu
def test_mse_and_adam(lib):
    import torch
    from littleharsh_gb300 import srnet
    rng = np.random.default_rng(3)
    n = 4096
    corr = rng.standard_normal((n, 16)).astype(np.float32)
    base = rng.standard_normal((n, 3)).astype(np.float32)
    tgt = rng.standard_normal((n, 3)).astype(np.float32)
    L_ref, g_ref = so.mse(corr, base, tgt)
    ct, bt, tt = _t(corr, torch.float32), _t(base, torch.float32), _t(tgt, torch.float32)
    dc = torch.empty((n, 16), dtype=torch.bfloat16, device="cuda")
    loss = torch.zeros(1, dtype=torch.float64, device="cuda")
    assert lib.lh_sr_mse(srnet._ptr(ct), srnet._ptr(bt), srnet._ptr(tt), srnet._ptr(dc), srnet._ptr(loss), n,
                         None) == 0
    torch.cuda.synchronize()
    assert abs(loss.item() - L_ref) < 1e-5 * L_ref
    np.testing.assert_allclose(dc.float().cpu().numpy(), g_ref, rtol=2 ** -8, atol=1e-9)
    p = rng.standard_normal(1000).astype(np.float32)
    g = rng.standard_normal(1000).astype(np.float32)
    m = np.zeros(1000, np.float32)
    v = np.zeros(1000, np.float32)
    pt, gt, mt, vt = (_t(a, torch.float32) for a in (p, g, m, v))
    pb = torch.empty(1000, dtype=torch.bfloat16, device="cuda")
    for step in (1, 2, 3):
        assert lib.lh_sr_adam(srnet._ptr(pt), srnet._ptr(gt), srnet._ptr(mt), srnet._ptr(vt), srnet._ptr(pb), 1000,
                              1e-2, 0.9, 0.999, 1e-8, 1e-4, step, None) == 0
        p, m, v = so.adam(p.astype(np.float64), g, m, v, 1e-2, 0.9, 0.999, 1e-8, 1e-4, step)
    torch.cuda.synchronize()
    np.testing.assert_allclose(pt.cpu().numpy(), p, rtol=1e-5, atol=1e-6)
    np.testing.assert_array_equal(pb.float().cpu().numpy(), so.bf16_round(pt.cpu().numpy()))


@pytest.mark.gpu
@pytest.mark.parametrize("tcgen05", [True, False], ids=["tcgen05", "mma_sync"])
def test_network_gradient_matches_oracle(tcgen05):
    import torch
    from littleharsh_gb300 import srnet
    rng = np.random.default_rng(11)
    Y, Z, X = 4, 16, 32  # Z a multiple of 16: the weight gradients run on tcgen05 too
    params = srnet.init_params(seed=5)
    # larger second convolutions than the identity-like start and a random tail (it
    # starts at zero) so every path carries gradient
    params[-1][0][:, :3, :] = rng.standard_normal(params[-1][0][:, :3, :].shape) * 0.02
    params = [(so.bf16_round(w * (3.0 if i > 0 else 1.0)), (rng.standard_normal(b.shape) * 0.05).astype(np.float32))
              for i, (w, b) in enumerate(params)]
    net = srnet.SRNet(params=params, tcgen05=tcgen05)
    x = np.zeros((Y, Z, X, 16), np.float32)
    x[..., :5] = rng.standard_normal((Y, Z, X, 5))
    x = so.bf16_round(x)
    base = rng.standard_normal((Y * Z * X, 3)).astype(np.float32)
    tgt = rng.standard_normal((Y * Z * X, 3)).astype(np.float32)
    net.zero_grad()
    xt = _t(x, torch.bfloat16)
    corr = net.forward(xt, keep=True)
    loss = torch.zeros(1, dtype=torch.float64, device="cuda")
    dc = net.loss_grad(corr, _t(base, torch.float32), _t(tgt, torch.float32), loss)
    net.backward(dc)
    torch.cuda.synchronize()
    L_ref, g_ref = so.network_loss_and_grads(net.params_numpy(), x, base, tgt)
    assert abs(loss.item() - L_ref) < 1e-3 * L_ref
    # The oracle rounds to bf16 where the kernels store, but the kernels' fp32
    # sums run in another order, so an element can round to the neighbouring
    # bf16 value; such 2^-8 differences pass through the nine backward layers.
    # Every kernel is checked on its own above; here the whole chain is held
    # to a few bf16 ulps in norm and to the gradient's direction.
    off = 0
    g = net.grad.cpu().numpy()
    for (ci, co), (gw, gb) in zip(srnet.layer_shapes(), g_ref):
        nw = 27 * ci * co
        got_w, got_b = g[off:off + nw].reshape(27, co, ci), g[off + nw:off + nw + co]
        off += nw + co
        err = np.linalg.norm(got_w - gw) / max(np.linalg.norm(gw), 1e-30)
        cos = float(np.sum(got_w * gw) / (np.linalg.norm(got_w) * np.linalg.norm(gw)))
        assert err < 5e-2 and cos > 0.998, (ci, co, err, cos)
        errb = np.linalg.norm(got_b - gb) / max(np.linalg.norm(gb), 1e-30)
        assert errb < 5e-2, (ci, co, errb)


@pytest.mark.gpu
@pytest.mark.parametrize("cin,cout,f32", [(16, 32, False), (32, 32, False), (32, 16, False), (32, 16, True)])
@pytest.mark.parametrize("flags", [so.BIAS | so.RELU, so.GATE | so.RES])
def test_conv_fwd_tcgen05(lib, cin, cout, f32, flags):
    """The tcgen05 (TMEM accumulator) form of the forward convolution against the oracle."""
    import ctypes
    import torch
    from littleharsh_gb300 import srnet
    rng = np.random.default_rng(500 + cin * 10 + cout + flags)
    Y, Z, X = VOL
    x = so.bf16_round(rng.standard_normal((Y, Z, X, cin)))
    w = so.bf16_round(rng.standard_normal((27, cout, cin)) / np.sqrt(27 * cin))
    b = rng.standard_normal(cout).astype(np.float32)
    res = so.bf16_round(rng.standard_normal((Y, Z, X, cout)))
    gate = so.bf16_round(rng.standard_normal((Y, Z, X, cout)))
    ref = so.conv_fwd(x, w, b, res, gate, flags)
    out = torch.empty((Y, Z, X, cout), dtype=torch.float32 if f32 else torch.bfloat16, device="cuda")
    xt, wt, bt, rt, gt = _t(x, torch.bfloat16), _t(w, torch.bfloat16), _t(b, torch.float32), \
        _t(res, torch.bfloat16), _t(gate, torch.bfloat16)
    rc = lib.lh_sr_conv_fwd_tc(cin, cout, srnet._ptr(xt), srnet._ptr(wt), srnet._ptr(bt), srnet._ptr(out), int(f32),
                               srnet._ptr(rt), srnet._ptr(gt), flags, X, Y, Z, None)
    assert rc == 0
    torch.cuda.synchronize()
    timed_out = ctypes.c_int32(-1)
    assert lib.lh_sr_tc_status(ctypes.byref(timed_out)) == 0 and timed_out.value == 0
    got = out.float().cpu().numpy()
    if f32:
        np.testing.assert_allclose(got, ref, rtol=1e-5, atol=1e-5)
    else:
        np.testing.assert_allclose(got, ref, rtol=2 ** -8, atol=1e-3)


@pytest.mark.gpu
@pytest.mark.parametrize("Y,Z,X", [(80, 16, 64), (96, 32, 128)], ids=["320_tiles", "1536_tiles"])
def test_conv_fwd_tcgen05_many_tiles_per_cta(lib, Y, Z, X):
    """More tiles than SMs (tiles of 8 z-rows x 32 x-voxels): each persistent CTA pipelines several tiles
    through its ring of six halo buffers and its two accumulator sets, which wrap around many times."""
    import ctypes
    import torch
    from littleharsh_gb300 import srnet
    rng = np.random.default_rng(77)
    x = so.bf16_round(rng.standard_normal((Y, Z, X, 32)))
    w = so.bf16_round(rng.standard_normal((27, 32, 32)) / np.sqrt(27 * 32))
    b = rng.standard_normal(32).astype(np.float32)
    ref = so.conv_fwd(x, w, b, flags=so.BIAS | so.RELU)
    out = torch.empty((Y, Z, X, 32), dtype=torch.bfloat16, device="cuda")
    xt, wt, bt = _t(x, torch.bfloat16), _t(w, torch.bfloat16), _t(b, torch.float32)
    assert lib.lh_sr_conv_fwd_tc(32, 32, srnet._ptr(xt), srnet._ptr(wt), srnet._ptr(bt), srnet._ptr(out), 0, None,
                                 None, so.BIAS | so.RELU, X, Y, Z, None) == 0
    torch.cuda.synchronize()
    timed_out = ctypes.c_int32(-1)
    assert lib.lh_sr_tc_status(ctypes.byref(timed_out)) == 0 and timed_out.value == 0
    np.testing.assert_allclose(out.float().cpu().numpy(), ref, rtol=2 ** -8, atol=1e-3)
