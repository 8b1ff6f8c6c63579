"""The super-resolution network of the learned warm start.

A residual 3D convolutional network on channels-last volumes [Y][Z][X][C]:

    h0  = conv_head(x)                    16 -> 32 channels
    h_b = h_{b-1} + conv_b2(relu(conv_b1(h_{b-1})))   4 residual blocks, 32 channels
    c   = conv_tail(h_4)                  32 -> 16 channels (0..2 used), fp32

Input channels: u, v, w of the coarse field lifted onto the fine grid, the
solid mask of the canopy, the y coordinate, zeros.  The network predicts the
correction c that is added to the lifted u, v, w.  Every convolution, its data
and weight gradients, the loss and the AdamW update run in the kernels of
include/lh_srnet.h (BF16 tensor cores, fp32 accumulation); torch only holds
the device memory and orders the calls on its current stream.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import LhError, load_library

CIN0 = 16  # input channels (5 used)
CH = 32    # hidden channels
COUT = 16  # output channels (3 used)
NBLOCKS = 4
RELU, RES, GATE, BIAS = 1, 2, 4, 8


def _torch():
    import torch
    return torch


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def _stream():
    return C.c_void_p(_torch().cuda.current_stream().cuda_stream)


def _check(rc, what):
    if rc:
        raise LhError(f"{what} failed ({rc}): {load_library().lh_last_error(None).decode()}")


def layer_shapes(nblocks: int = NBLOCKS):
    """(cin, cout) of every convolution, in order."""
    return [(CIN0, CH)] + [(CH, CH)] * (2 * nblocks) + [(CH, COUT)]


def init_params(seed: int = 0, nblocks: int = NBLOCKS):
    """He-initialised fp32 weights [27][cout][cin] and zero biases (numpy).
    The second convolution of each block starts small and the tail at zero,
    so the untrained network's correction is exactly zero and each block
    starts close to the identity."""
    rng = np.random.default_rng(seed)
    out = []
    shapes = layer_shapes(nblocks)
    for i, (ci, co) in enumerate(shapes):
        std = math.sqrt(2.0 / (27 * ci))
        if i == len(shapes) - 1 or (i >= 1 and i % 2 == 0):
            std *= 0.1
        w = (rng.standard_normal((27, co, ci)) * std).astype(np.float32)
        if i == len(shapes) - 1:
            w[:] = 0.0  # zero correction at the start; unused output channels stay zero for good
        out.append((w, np.zeros(co, np.float32)))
    return out


class SRNet:
    """Parameters, activations and the training step on the current CUDA device."""

    def __init__(self, params=None, seed: int = 0, nblocks: int = NBLOCKS, lr: float = 1e-3,
                 betas=(0.9, 0.999), eps: float = 1e-8, weight_decay: float = 0.0, tcgen05: bool = True):
        torch = _torch()
        self.nblocks = nblocks
        self.shapes = layer_shapes(nblocks)
        params = params if params is not None else init_params(seed, nblocks)
        dev = torch.device("cuda")
        # one flat fp32 master vector (weights then bias per layer) for AdamW
        sizes = [27 * ci * co + co for ci, co in self.shapes]
        self.n = int(sum(sizes))
        self.master = torch.zeros(self.n, dtype=torch.float32, device=dev)
        self.grad = torch.zeros_like(self.master)
        self.m = torch.zeros_like(self.master)
        self.v = torch.zeros_like(self.master)
        self.wb16 = torch.zeros(self.n, dtype=torch.bfloat16, device=dev)
        self.views = []
        off = 0
        for (ci, co), (w, b) in zip(self.shapes, params):
            nw = 27 * ci * co
            self.master[off:off + nw] = torch.from_numpy(np.ascontiguousarray(w, np.float32).ravel()).to(dev)
            self.master[off + nw:off + nw + co] = torch.from_numpy(np.ascontiguousarray(b, np.float32)).to(dev)
            self.views.append(dict(ci=ci, co=co, w=self.wb16[off:off + nw], b=self.master[off + nw:off + nw + co],
                                   gw=self.grad[off:off + nw], gb=self.grad[off + nw:off + nw + co]))
            off += nw + co
        self.wb16.copy_(self.master.to(torch.bfloat16))
        # bf16 copies of the weights must start 16-byte aligned for the kernels' copies
        for vw in self.views:
            if vw["w"].data_ptr() % 16:
                raise LhError("weight slice is not 16-byte aligned")
        self.flip = [torch.zeros(27 * vw["ci"] * vw["co"], dtype=torch.bfloat16, device=dev) for vw in self.views]
        self.lr, self.betas, self.eps, self.wd = lr, betas, eps, weight_decay
        self.t = 0
        # forward, data-gradient and weight-gradient convolutions on tcgen05 (the default: the warp-specialised
        # TMEM kernels measure faster than mma.sync) or, when unset or Z is not a multiple of 8 (16 for the
        # weight gradient), on mma.sync
        self.tcgen05 = tcgen05
        self.sigma = 1.0  # scale of the correction (set by training: rms of the residual it learns)
        self._acts = None
        self._shape = None

    # -- parameters -------------------------------------------------------------
    def params_numpy(self):
        out = []
        for vw in self.views:
            out.append((vw["w"].float().cpu().numpy().reshape(27, vw["co"], vw["ci"]),
                        vw["b"].cpu().numpy().copy()))
        return out

    def state_dict(self):
        return {"master": self.master.cpu().numpy(), "nblocks": self.nblocks, "sigma": self.sigma}

    def load_state(self, state: dict):
        torch = _torch()
        self.master.copy_(torch.from_numpy(np.asarray(state["master"], np.float32)).cuda())
        self.wb16.copy_(self.master.to(torch.bfloat16))
        self.sigma = float(state.get("sigma", 1.0))

    # -- kernels ------------------------------------------------------------------
    def _conv(self, li, x, out, res=None, gate=None, flags=BIAS, out_f32=False, weights=None, cin=None, cout=None):
        L = load_library()
        vw = self.views[li]
        ci = cin if cin is not None else vw["ci"]
        co = cout if cout is not None else vw["co"]
        w = weights if weights is not None else vw["w"]
        Y, Z, X = self._shape
        fn = L.lh_sr_conv_fwd_tc if (self.tcgen05 and Z % 8 == 0) else L.lh_sr_conv_fwd
        _check(fn(ci, co, _ptr(x), _ptr(w), _ptr(vw["b"]) if flags & BIAS else None, _ptr(out),
                  int(out_f32), _ptr(res), _ptr(gate), flags, X, Y, Z, _stream()), "lh_sr_conv_fwd")

    def _wgrad(self, li, x, dout):
        L = load_library()
        vw = self.views[li]
        Y, Z, X = self._shape
        fn = L.lh_sr_conv_wgrad_tc if (self.tcgen05 and Z % 16 == 0) else L.lh_sr_conv_wgrad
        _check(fn(vw["ci"], vw["co"], _ptr(x), _ptr(dout), _ptr(vw["gw"]), _ptr(vw["gb"]), X, Y, Z, _stream()),
               "lh_sr_conv_wgrad")

    def _flip_all(self):
        L = load_library()
        for vw, ft in zip(self.views, self.flip):
            _check(L.lh_sr_flip_weights(vw["ci"], vw["co"], _ptr(vw["w"]), _ptr(ft), _stream()), "lh_sr_flip_weights")

    # -- forward / backward -----------------------------------------------------------
    def forward(self, x, keep: bool = False):
        """x: bf16 [Y, Z, X, 16] on the device.  Returns the fp32 correction [Y, Z, X, 16]."""
        torch = _torch()
        Y, Z, X, c = x.shape
        if c != CIN0 or x.dtype != torch.bfloat16 or not x.is_contiguous():
            raise LhError("input must be contiguous bf16 [Y, Z, X, 16]")
        self._shape = (Y, Z, X)
        new = lambda ch: torch.empty((Y, Z, X, ch), dtype=torch.bfloat16, device=x.device)  # noqa: E731
        h = new(CH)
        self._conv(0, x, h)
        acts = [x, h] if keep else None  # inference holds two activations at a time
        for b in range(self.nblocks):
            t = new(CH)
            self._conv(1 + 2 * b, h, t, flags=BIAS | RELU)
            h2 = new(CH)
            self._conv(2 + 2 * b, t, h2, res=h, flags=BIAS | RES)
            if keep:
                acts += [t, h2]
            del t
            h = h2
        corr = torch.empty((Y, Z, X, COUT), dtype=torch.float32, device=x.device)
        self._conv(len(self.views) - 1, h, corr, out_f32=True)
        self._acts = acts if keep else None
        return corr

    def backward(self, dcorr):
        """dcorr: bf16 [Y, Z, X, 16], the loss gradient of the last forward(keep=True).
        Accumulates the parameter gradients into self.grad."""
        torch = _torch()
        if self._acts is None:
            raise LhError("backward needs forward(keep=True)")
        acts = self._acts
        Y, Z, X = self._shape
        new = lambda ch: torch.empty((Y, Z, X, ch), dtype=torch.bfloat16, device=dcorr.device)  # noqa: E731
        self._flip_all()
        nl = len(self.views)
        h = acts[-1]
        self._wgrad(nl - 1, h, dcorr)
        dh = new(CH)
        self._conv(nl - 1, dcorr, dh, flags=0, weights=self.flip[nl - 1], cin=COUT, cout=CH)
        for b in reversed(range(self.nblocks)):
            t, h_in = acts[2 + 2 * b], acts[1 + 2 * b]
            l1, l2 = 1 + 2 * b, 2 + 2 * b
            self._wgrad(l2, t, dh)
            dpre = new(CH)
            self._conv(l2, dh, dpre, gate=t, flags=GATE, weights=self.flip[l2], cin=CH, cout=CH)
            self._wgrad(l1, h_in, dpre)
            dh2 = new(CH)
            self._conv(l1, dpre, dh2, res=dh, flags=RES, weights=self.flip[l1], cin=CH, cout=CH)
            dh = dh2
        self._wgrad(0, acts[0], dh)
        self._acts = None

    def loss_grad(self, corr, base, target, loss_acc):
        """MSE of base + corr against target (fp32 [V, 3]); returns bf16 dcorr and adds the loss to loss_acc."""
        torch = _torch()
        dcorr = torch.empty(corr.shape, dtype=torch.bfloat16, device=corr.device)
        nvox = corr.numel() // COUT
        _check(load_library().lh_sr_mse(_ptr(corr), _ptr(base), _ptr(target), _ptr(dcorr), _ptr(loss_acc), nvox,
                                        _stream()), "lh_sr_mse")
        return dcorr

    def zero_grad(self):
        self.grad.zero_()

    def adam_step(self, lr: float | None = None):
        self.t += 1
        _check(load_library().lh_sr_adam(_ptr(self.master), _ptr(self.grad), _ptr(self.m), _ptr(self.v),
                                         _ptr(self.wb16), self.n, self.lr if lr is None else lr, self.betas[0],
                                         self.betas[1], self.eps, self.wd, self.t, _stream()), "lh_sr_adam")
