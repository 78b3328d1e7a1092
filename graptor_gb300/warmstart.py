"""Learned warm start for the 3-D primal-dual solver.

The reference always starts the iteration from zero (u = p = v = w = lambda = 0,
radon_tgv_primal_dual_3d.py:1147-1176) and runs a fixed number of iterations.
Here a small 3-D U-Net looks at the iterate after a few cold iterations and
predicts the converged primal image u and the first dual field v; the solver then
continues from that state to the same gap tolerance, so the answer is still the
TGV minimiser and a cold start remains the fallback.

Network (``UNet3D``): three levels with 16-32-64 channels, two 3x3x3
convolutions + ReLU per level, 2x2x2 average pooling down, nearest upsampling
and skip concatenation up, a 1x1x1 head; the u channels are predicted as a
residual on the input.  Weights and activations are bfloat16, every sum is
float32, the optimizer (Adam) keeps float32 master weights.  Every forward and
backward operation is a kernel of libgraptor_gb300 (gt_nn_*); PyTorch only holds
the tensors and streams.

Normalisation: the input u is divided per channel by the mean intensity the
sinogram implies, s_c = sum(f_c) / (nang * Nz * N^2) (every projection of an
image sums to its mass); predicted u is multiplied back by s_c, predicted v by
alpha1 / ne^2 (the radius of v's ball).
"""
from __future__ import annotations

import ctypes
import math
import os
import time

import numpy as np

from . import _lib as L

F32, BF16 = 0, 1


def _p(t) -> ctypes.c_void_p:
    return ctypes.c_void_p(t.data_ptr())


def _ck(rc):
    L.check(rc)


def unet_layers(cin: int, cout: int, widths=(16, 32, 64)):
    """(name, Ci, Co, k) of the 11 convolutions, in forward order."""
    c1, c2, c3 = widths
    return [("enc1a", cin, c1, 3), ("enc1b", c1, c1, 3), ("enc2a", c1, c2, 3), ("enc2b", c2, c2, 3),
            ("bota", c2, c3, 3), ("botb", c3, c3, 3), ("dec2a", c2 + c3, c2, 3), ("dec2b", c2, c2, 3),
            ("dec1a", c1 + c2, c1, 3), ("dec1b", c1, c1, 3), ("head", c1, cout, 1)]


class UNet3D:
    """3-level 3-D U-Net on libgraptor_gb300 kernels.

    ``cin`` input channels; ``cout`` output channels, of which the first
    ``residual`` are added to the corresponding input channels."""

    def __init__(self, cin: int, cout: int, residual: int = 0, widths=(16, 32, 64), device: int = 0, seed: int = 0):
        import torch
        self.torch = torch
        self.cin, self.cout, self.residual, self.widths = cin, cout, residual, tuple(widths)
        self.dev = torch.device("cuda", device)
        self.layers = unet_layers(cin, cout, widths)
        self.offsets = {}
        off = 0
        for name, ci, co, k in self.layers:
            nw = co * ci * k ** 3
            self.offsets[name] = (off, off + nw, ci, co, k)  # weights at [off, off+nw), bias at [off+nw, +co)
            off += nw + co
        self.nparams = off
        g = torch.Generator().manual_seed(seed)
        master = torch.zeros(off, dtype=torch.float32)
        for name, ci, co, k in self.layers:
            o, ob, *_ = self.offsets[name]
            std = math.sqrt(2.0 / (ci * k ** 3)) if name != "head" else 1e-3
            master[o:ob] = torch.randn(ob - o, generator=g) * std
        self.master = master.to(self.dev)
        self.wb = torch.empty(off, dtype=torch.bfloat16, device=self.dev)
        self.wflip = torch.empty(off, dtype=torch.bfloat16, device=self.dev)
        self.grad = torch.zeros(off, dtype=torch.float32, device=self.dev)
        self.m = torch.zeros_like(self.grad)
        self.v = torch.zeros_like(self.grad)
        self.step_count = 0
        self._bufs = {}
        self._part = None
        self.refresh()

    # ------------------------------------------------------------------ parameters
    def refresh(self, stream=None):
        """bfloat16 working copy of the float32 master weights."""
        _ck(L.lib().gt_nn_cast(_p(self.master), F32, _p(self.wb), self.nparams, stream))

    def state_dict(self) -> dict:
        return {"cin": self.cin, "cout": self.cout, "residual": self.residual, "widths": self.widths,
                "master": self.master.cpu().numpy(), "step": self.step_count}

    @classmethod
    def from_state(cls, sd: dict, device: int = 0) -> "UNet3D":
        net = cls(int(sd["cin"]), int(sd["cout"]), int(sd["residual"]), tuple(int(w) for w in sd["widths"]),
                  device=device)
        net.master.copy_(net.torch.from_numpy(np.asarray(sd["master"], np.float32)))
        net.step_count = int(sd.get("step", 0))
        net.refresh()
        net.torch.cuda.synchronize(net.dev)
        return net

    def save(self, path: str):
        np.savez(path, **{k: np.asarray(v) for k, v in self.state_dict().items()})

    @classmethod
    def load(cls, path: str, device: int = 0) -> "UNet3D":
        return cls.from_state(dict(np.load(path)), device)

    def wptr(self, name, flipped=False):
        o = self.offsets[name][0]
        base = self.wflip if flipped else self.wb
        return ctypes.c_void_p(base.data_ptr() + 2 * o)

    def bptr(self, name, which="master"):
        _, ob, *_ = self.offsets[name]
        base = self.master if which == "master" else self.grad
        return ctypes.c_void_p(base.data_ptr() + 4 * ob)

    def gptr(self, name):
        return ctypes.c_void_p(self.grad.data_ptr() + 4 * self.offsets[name][0])

    # ------------------------------------------------------------------ buffers
    def buffers(self, B, D, H, W):
        key = (B, D, H, W)
        if key in self._bufs:
            return self._bufs[key]
        if D % 4 or H % 4 or W % 16:
            raise ValueError(f"U-Net input {D}x{H}x{W}: D and H must be multiples of 4, W of 16")
        t = self.torch
        c1, c2, c3 = self.widths
        f, h, q = (D, H, W), (D // 2, H // 2, W // 2), (D // 4, H // 4, W // 4)

        def bf(c, s):
            return t.empty((B, c) + s, dtype=t.bfloat16, device=self.dev)

        def fl(c, s):
            return t.empty((B, c) + s, dtype=t.float32, device=self.dev)

        b = {"a1": bf(c1, f), "cat1": bf(c1 + c2, f), "p1": bf(c1, h), "a2": bf(c2, h), "cat2": bf(c2 + c3, h),
             "p2": bf(c2, q), "a3": bf(c3, q), "b": bf(c3, q), "a4": bf(c2, h), "d2": bf(c2, h), "a5": bf(c1, f),
             "d1": bf(c1, f),
             "g_d1": fl(c1, f), "g_a5": fl(c1, f), "g_cat1": fl(c1 + c2, f), "g_d2": fl(c2, h), "g_a4": fl(c2, h),
             "g_cat2": fl(c2 + c3, h), "g_b": fl(c3, q), "g_a3": fl(c3, q), "g_p2": fl(c2, q), "g_a2": fl(c2, h),
             "g_p1": fl(c1, h), "g_a1": fl(c1, f), "g_x": fl(self.cin, f)}
        self._bufs = {key: b}  # one shape at a time
        return b

    def _kchunk(self, nvox, n_cols, co):
        tiles = ((n_cols + 63) // 64) * ((co + 15) // 16)
        chunks = max(1, min(512, math.ceil(2 * 152 * 4 / tiles)))
        return max(1024, math.ceil(nvox / chunks))

    def _ensure_part(self, B, D, H, W):
        need = 1
        for name, ci, co, k in self.layers:
            lvl = {"enc1a": 0, "enc1b": 0, "enc2a": 1, "enc2b": 1, "bota": 2, "botb": 2, "dec2a": 1, "dec2b": 1,
                   "dec1a": 0, "dec1b": 0, "head": 0}[name]
            nvox = B * (D >> lvl) * (H >> lvl) * (W >> lvl)
            kc = self._kchunk(nvox, ci * k ** 3, co)
            need = max(need, math.ceil(nvox / kc) * co * ci * k ** 3)
        if self._part is None or self._part.numel() < need:
            self._part = self.torch.empty(need, dtype=self.torch.float32, device=self.dev)

    # ------------------------------------------------------------------ forward / backward
    def _conv(self, name, x, Cx, xoff, xdt, y, Cy, yoff, ydt, shape, relu, acc=0, stream=None):
        _, _, ci, co, k = self.offsets[name]
        B, D, H, W = shape
        _ck(L.lib().gt_nn_conv3d(_p(x), xdt, ci, Cx, xoff, self.wptr(name), self.bptr(name), _p(y), ydt, co, Cy, yoff,
                                 B, D, H, W, k, relu, acc, stream))

    def forward(self, x, out, stream=None):
        """x: bfloat16 [B][cin][D][H][W]; out: float32 [B][cout][D][H][W], which must
        hold the residual base (input u in its first `residual` channels, zeros
        elsewhere): the head adds onto it."""
        B, _, D, H, W = x.shape
        b = self.buffers(B, D, H, W)
        c1, c2, c3 = self.widths
        f, h, q = (B, D, H, W), (B, D // 2, H // 2, W // 2), (B, D // 4, H // 4, W // 4)
        lib = L.lib()
        self._conv("enc1a", x, self.cin, 0, BF16, b["a1"], c1, 0, BF16, f, 1, stream=stream)
        self._conv("enc1b", b["a1"], c1, 0, BF16, b["cat1"], c1 + c2, 0, BF16, f, 1, stream=stream)
        _ck(lib.gt_nn_pool2(_p(b["cat1"]), c1 + c2, 0, _p(b["p1"]), c1, *h, stream))
        self._conv("enc2a", b["p1"], c1, 0, BF16, b["a2"], c2, 0, BF16, h, 1, stream=stream)
        self._conv("enc2b", b["a2"], c2, 0, BF16, b["cat2"], c2 + c3, 0, BF16, h, 1, stream=stream)
        _ck(lib.gt_nn_pool2(_p(b["cat2"]), c2 + c3, 0, _p(b["p2"]), c2, *q, stream))
        self._conv("bota", b["p2"], c2, 0, BF16, b["a3"], c3, 0, BF16, q, 1, stream=stream)
        self._conv("botb", b["a3"], c3, 0, BF16, b["b"], c3, 0, BF16, q, 1, stream=stream)
        _ck(lib.gt_nn_up2(_p(b["b"]), _p(b["cat2"]), c3, c2 + c3, c2, *h, stream))
        self._conv("dec2a", b["cat2"], c2 + c3, 0, BF16, b["a4"], c2, 0, BF16, h, 1, stream=stream)
        self._conv("dec2b", b["a4"], c2, 0, BF16, b["d2"], c2, 0, BF16, h, 1, stream=stream)
        _ck(lib.gt_nn_up2(_p(b["d2"]), _p(b["cat1"]), c2, c1 + c2, c1, *f, stream))
        self._conv("dec1a", b["cat1"], c1 + c2, 0, BF16, b["a5"], c1, 0, BF16, f, 1, stream=stream)
        self._conv("dec1b", b["a5"], c1, 0, BF16, b["d1"], c1, 0, BF16, f, 1, stream=stream)
        self._conv("head", b["d1"], c1, 0, BF16, out, self.cout, 0, F32, f, 0, acc=1, stream=stream)
        return out

    def _layer_bwd(self, name, gy, Cg, goff, y, relu, x, Cx, xoff, xdt, gx, Cgx, gxoff, shape, gx_acc=0, stream=None,
                   need_gx=True):
        """Gradients of one convolution: ReLU mask on gy (view of y), weight and bias
        gradients, and (if need_gx) the data gradient into gx."""
        _, _, ci, co, k = self.offsets[name]
        B, D, H, W = shape
        vol = D * H * W
        lib = L.lib()
        if relu:
            _ck(lib.gt_nn_relu_bwd(_p(gy), _p(y), BF16, co, Cg, goff, B, vol, stream))
        nvox = B * vol
        kc = self._kchunk(nvox, ci * k ** 3, co)
        _ck(lib.gt_nn_conv3d_wgrad(_p(gy), co, Cg, goff, _p(x), xdt, ci, Cx, xoff, B, D, H, W, k, kc, _p(self._part),
                                   self.gptr(name), 0, stream))
        _ck(lib.gt_nn_bias_grad(_p(gy), co, Cg, goff, B, vol, self.bptr(name, "grad"), 0, stream))
        if need_gx:
            _ck(lib.gt_nn_conv3d(_p(gy), F32, co, Cg, goff, self.wptr(name, True), None, _p(gx), F32, ci, Cgx, gxoff,
                                 B, D, H, W, k, 0, gx_acc, stream))

    def backward(self, x, dout, stream=None, need_input_grad=False):
        """Gradients of all parameters (written, not accumulated) for the loss
        gradient dout (float32, shape of the output), after forward(x)."""
        B, _, D, H, W = x.shape
        b = self.buffers(B, D, H, W)
        self._ensure_part(B, D, H, W)
        c1, c2, c3 = self.widths
        f, h, q = (B, D, H, W), (B, D // 2, H // 2, W // 2), (B, D // 4, H // 4, W // 4)
        lib = L.lib()
        for name, ci, co, k in self.layers:
            _ck(lib.gt_nn_flip_weights(self.wptr(name), self.wptr(name, True), co, ci, k, stream))
        lb = self._layer_bwd
        lb("head", dout, self.cout, 0, None, 0, b["d1"], c1, 0, BF16, b["g_d1"], c1, 0, f, stream=stream)
        lb("dec1b", b["g_d1"], c1, 0, b["d1"], 1, b["a5"], c1, 0, BF16, b["g_a5"], c1, 0, f, stream=stream)
        lb("dec1a", b["g_a5"], c1, 0, b["a5"], 1, b["cat1"], c1 + c2, 0, BF16, b["g_cat1"], c1 + c2, 0, f,
           stream=stream)
        _ck(lib.gt_nn_up2_bwd(_p(b["g_cat1"]), c1 + c2, c1, _p(b["g_d2"]), c2, *h, stream))
        lb("dec2b", b["g_d2"], c2, 0, b["d2"], 1, b["a4"], c2, 0, BF16, b["g_a4"], c2, 0, h, stream=stream)
        lb("dec2a", b["g_a4"], c2, 0, b["a4"], 1, b["cat2"], c2 + c3, 0, BF16, b["g_cat2"], c2 + c3, 0, h,
           stream=stream)
        _ck(lib.gt_nn_up2_bwd(_p(b["g_cat2"]), c2 + c3, c2, _p(b["g_b"]), c3, *q, stream))
        lb("botb", b["g_b"], c3, 0, b["b"], 1, b["a3"], c3, 0, BF16, b["g_a3"], c3, 0, q, stream=stream)
        lb("bota", b["g_a3"], c3, 0, b["a3"], 1, b["p2"], c2, 0, BF16, b["g_p2"], c2, 0, q, stream=stream)
        _ck(lib.gt_nn_pool2_bwd(_p(b["g_p2"]), _p(b["g_cat2"]), c2, c2 + c3, 0, *h, stream))
        lb("enc2b", b["g_cat2"], c2 + c3, 0, b["cat2"], 1, b["a2"], c2, 0, BF16, b["g_a2"], c2, 0, h, stream=stream)
        lb("enc2a", b["g_a2"], c2, 0, b["a2"], 1, b["p1"], c1, 0, BF16, b["g_p1"], c1, 0, h, stream=stream)
        _ck(lib.gt_nn_pool2_bwd(_p(b["g_p1"]), _p(b["g_cat1"]), c1, c1 + c2, 0, *f, stream))
        lb("enc1b", b["g_cat1"], c1 + c2, 0, b["cat1"], 1, b["a1"], c1, 0, BF16, b["g_a1"], c1, 0, f, stream=stream)
        lb("enc1a", b["g_a1"], c1, 0, b["a1"], 1, x, self.cin, 0, BF16, b["g_x"], self.cin, 0, f, stream=stream,
           need_gx=need_input_grad)
        if need_input_grad:
            return b["g_x"]
        return None

    def adam(self, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8, stream=None):
        self.step_count += 1
        _ck(L.lib().gt_nn_adam(_p(self.master), _p(self.wb), _p(self.grad), _p(self.m), _p(self.v), self.nparams,
                               lr, b1, b2, eps, self.step_count, stream))

    def mse(self, pred, target, dpred, part, stream=None):
        """Loss gradient into dpred; returns the device tensor of partial sums (sum them for n * loss)."""
        n = pred.numel()
        _ck(L.lib().gt_nn_mse(_p(pred), _p(target), n, _p(dpred), _p(part), stream))
        return part

    def residual_base(self, x, out, stream=None):
        """out = 0 except its first `residual` channels = x's (float32)."""
        B, _, D, H, W = x.shape
        vol = D * H * W
        out.zero_()
        for k in range(B):
            _ck(L.lib().gt_nn_cast(ctypes.c_void_p(x.data_ptr() + 2 * k * self.cin * vol), BF16,
                                   ctypes.c_void_p(out.data_ptr() + 4 * k * self.cout * vol), self.residual * vol,
                                   stream))

    def train_step(self, x, target, lr=1e-3, stream=None):
        """One Adam step on a batch x (bfloat16 [B][cin][D][H][W]) against target
        (float32 [B][cout][D][H][W]); returns the mean squared error as a device
        scalar tensor."""
        t = self.torch
        key = tuple(target.shape)
        if getattr(self, "_tkey", None) != key:
            self._tkey = key
            self._tout = t.empty(key, dtype=t.float32, device=self.dev)
            self._tdout = t.empty_like(self._tout)
            self._tpart = t.empty((self._tout.numel() + 255) // 256, dtype=t.float32, device=self.dev)
        out, dout, part = self._tout, self._tdout, self._tpart
        self.residual_base(x, out, stream)
        self.forward(x, out, stream)
        self.mse(out, target, dout, part, stream)
        self.backward(x, dout, stream)
        self.adam(lr, stream=stream)
        return part.sum() / out.numel()


# ---------------------------------------------------------------------- solver coupling
def channel_scales(f: np.ndarray, C: int, Nz: int, N: int, nang: int) -> np.ndarray:
    """Mean intensity per channel implied by the sinogram f[S][nang][nd] (s = c*Nz + z)."""
    f = np.asarray(f, np.float64).reshape(C, -1)
    s = f.sum(axis=1) / (nang * Nz * N * N)
    return np.maximum(s, 1e-12).astype(np.float32)


FIELD_COMPS = {"u": 1, "p": 3, "v": 3, "w": 6}
PAIRED = {"u": "ubar", "p": "pbar"}


def output_channels(C: int, fields) -> int:
    return sum(FIELD_COMPS[f] for f in fields) * C


def field_scales(fields, sc: np.ndarray, alpha, ne: float) -> np.ndarray:
    """Per-output-channel scale: u and p by the channel scale s_c, v by alpha1/ne^2,
    w by alpha0/ne^2 (the radii of the dual balls)."""
    C = sc.size
    out = []
    for fl in fields:
        k = FIELD_COMPS[fl]
        if fl in ("u", "p"):
            out.append(np.tile(sc, k))
        else:
            r = (alpha[1] if fl == "v" else alpha[0]) / (ne * ne)
            out.append(np.full(k * C, r, np.float32))
    return np.concatenate(out).astype(np.float32)


class WarmStarter:
    """Applies a trained UNet3D to a solver Problem (dim 3) on the problem's stream.

    The network's input is u after ``pre_iters`` cold iterations (C channels, divided
    by the channel scales).  Its output holds, for each field of ``fields`` in
    order, comps*C channels in the state's [k][c] order, normalised by
    :func:`field_scales`; the u channels are a residual on the input.  u and p
    also set their extrapolations (ubar = u, pbar = p), and lambda is set to the
    fixed point of its update for the predicted u (gt_dual_from_primal): without
    that the first iterations pull u back towards the cold-start state."""

    def __init__(self, net: UNet3D, fields=("u", "v"), pre_iters: int = 20, use=None, reset_dual: bool = True,
                 empty_weight: float = 1.0, cap: int = 0, repair: bool = True, use_network: bool = True):
        self.net, self.fields, self.pre_iters = net, tuple(fields), int(pre_iters)
        self.use = tuple(use) if use is not None else self.fields  # predicted fields written to the solver
        self.reset_dual = bool(reset_dual)
        self.empty_weight = float(empty_weight)  # fraction of the reset applied on bins without data
        self.repair = bool(repair)  # lift u along rays with data that the prediction misses
        self.use_network = bool(use_network)  # False: the lambda reset alone (for comparisons)
        self.cap = int(cap)  # 0: keep lambda where f > 10 K u; 10 / 100: lambda = mu (1 - cap) there
        if self.fields[0] != "u":
            raise ValueError("the first predicted field must be u (the residual channels)")

    def predict(self, x_norm: np.ndarray) -> np.ndarray:
        """Network output (normalised fields) for a normalised input u [C][Nz][N][N]."""
        import torch
        net = self.net
        C, Nz, N = x_norm.shape[0], x_norm.shape[1], x_norm.shape[2]
        x = torch.from_numpy(np.ascontiguousarray(x_norm, np.float32)).to(net.dev).to(torch.bfloat16)[None]
        out = torch.empty((1, net.cout, Nz, N, N), dtype=torch.float32, device=net.dev)
        net.residual_base(x, out)
        net.forward(x, out)
        torch.cuda.synchronize(net.dev)
        return out[0].cpu().numpy()

    STATE = ("u", "ubar", "p", "pbar", "v", "w", "lambda")

    def snapshot(self, prob) -> dict:
        """Device copies of the iterate (for the cold-start fallback)."""
        import torch
        lib = L.lib()
        snap = {}
        for fl in self.STATE:
            n = int(np.prod(prob._shape(fl)))
            t = torch.empty(n, dtype=torch.float32, device=self.net.dev)
            _ck(lib.gt_get_state_device(prob._h, L.FIELDS[fl], _p(t)))
            snap[fl] = t
        prob.synchronize()
        return snap

    def restore(self, prob, snap: dict):
        lib = L.lib()
        for fl, t in snap.items():
            _ck(lib.gt_set_state_device(prob._h, L.FIELDS[fl], _p(t)))
        prob.synchronize()

    def apply(self, prob, f: np.ndarray, keep_snapshot: bool = False):
        """Run pre_iters cold iterations, then write the network's prediction
        into the solver.  With keep_snapshot, returns device copies of the
        iterate before the prediction (see :func:`solve_warm`)."""
        import torch
        net = self.net
        if prob.dim != 3:
            raise ValueError("the warm start is for 3-D problems")
        C, Nz, N = prob.C, prob.Nz, prob.N
        cout = output_channels(C, self.fields)
        if net.cin != C or net.cout != cout or net.residual != C:
            raise ValueError(f"network has cin={net.cin}, cout={net.cout}; problem needs {C}, {cout}")
        lib = L.lib()
        st = lib.gt_problem_stream(prob._h)
        if self.pre_iters:
            prob.run(self.pre_iters)
        snap = self.snapshot(prob) if keep_snapshot else None
        vol = Nz * N * N
        sc = channel_scales(f, C, Nz, N, prob.nang)
        back_np = field_scales(self.fields, sc, prob.alpha, prob.scalars["normest"])
        dev = net.dev
        u = torch.empty(C * vol, dtype=torch.float32, device=dev)
        x = torch.empty((1, C, Nz, N, N), dtype=torch.bfloat16, device=dev)
        out = torch.zeros((1, cout, Nz, N, N), dtype=torch.float32, device=dev)
        res = torch.empty_like(out)
        inv = torch.from_numpy(1.0 / sc).to(dev)
        back = torch.from_numpy(back_np).to(dev)
        torch.cuda.synchronize(dev)  # buffers and scales ready before the problem stream uses them
        _ck(lib.gt_get_state_device(prob._h, L.FIELDS["u"], _p(u)))
        _ck(lib.gt_nn_scale(_p(u), F32, _p(x), BF16, C, 1, vol, _p(inv), 0, st))
        _ck(lib.gt_nn_scale(_p(u), F32, _p(out), F32, C, 1, vol, _p(inv), 0, st))
        if self.use_network:
            net.forward(x, out, st)
        ch = 0
        for fl in (self.fields if self.use_network else ()):
            n = FIELD_COMPS[fl] * C
            src = ctypes.c_void_p(out.data_ptr() + 4 * ch * vol)
            dst = ctypes.c_void_p(res.data_ptr() + 4 * ch * vol)
            _ck(lib.gt_nn_scale(src, F32, dst, F32, n, 1, vol, ctypes.c_void_p(back.data_ptr() + 4 * ch),
                                int(fl == "u"), st))
            if fl in self.use:
                _ck(lib.gt_set_state_device(prob._h, L.FIELDS[fl], dst))
                if fl in PAIRED:
                    _ck(lib.gt_set_state_device(prob._h, L.FIELDS[PAIRED[fl]], dst))
            ch += n
        # the data dual consistent with the predicted image (fixed point of its update)
        if self.reset_dual:
            _ck(lib.gt_dual_from_primal_ex(prob._h, {0: 0, 10: 2, 100: 4}[self.cap] | (8 if self.repair else 0),
                                           self.empty_weight))
        prob.synchronize()
        return snap if keep_snapshot else prob


# ---------------------------------------------------------------------- data, training, evaluation
def phantom_case(seed: int, N: int, Nz: int, C: int = 2, nang: int = 71, peaks=(1e4, 20.0), device: int = 0):
    """Sinogram f[S][nang][nd] (s = c*Nz + z) and angles of a seeded ellipsoid
    phantom (channel 0 dense, the others sparse), projected on the GPU, with
    Poisson noise at the given peak counts."""
    import torch

    from . import phantom, solver
    vol = phantom.ellipsoids_3d(N, Nz, C, 12, seed)  # [c, z, y, x]
    ang = phantom.angles_deg(nang)
    S = C * Nz
    dev = torch.device("cuda", device)
    img = torch.from_numpy(vol.reshape(S, N * N).T.copy()).to(dev)
    sino = torch.zeros(nang * N, S, device=dev)
    solver.radon(img.data_ptr(), sino.data_ptr(), ang, N, N, S)
    g = sino.cpu().numpy().T.reshape(C, Nz, nang, N)
    f = np.stack([phantom.poisson(g[c], peaks[c % len(peaks)], seed + c) for c in range(C)])
    return np.ascontiguousarray(f.reshape(S, nang, N)), ang


def problem_spec(N, Nz, C, ang, mu=(0.2, 5e-4), alpha=(4.0, 1.0)):
    """Keyword arguments of Problem for the warm-start workload (3-D TGV-KL, FROB coupling)."""
    return dict(dim=3, N=N, Nz=Nz, C=C, nd=N, angles=ang, alpha=alpha, mu=mu, discrepancy="KL",
                regularisation="TGV", coupling="FROB")


def generate_pairs(seeds, N, Nz, C=2, nang=71, mu=(0.2, 5e-4), alpha=(4.0, 1.0), fields=("u", "v"),
                   pre_iters=20, target_iters=5000, device=0, log=None, target_pweight=1.0, target_precise=False):
    """Training pairs from the plain solver: input = u after pre_iters cold
    iterations / s_c, target = the fields after target_iters iterations,
    normalised (:func:`field_scales`).  The problems run together as one Batch.
    After the input is taken the iterations towards the target may use another
    primal weight and the precise primal mode (targets closer to the minimiser).
    Returns host arrays x [n][C][Nz][N][N] and y [n][cout][Nz][N][N]."""
    from .solver import Batch
    cases = [phantom_case(s, N, Nz, C, nang, device=device) for s in seeds]
    specs = [problem_spec(N, Nz, C, ang, mu, alpha) for _, ang in cases]
    cout = output_channels(C, fields)
    xs = np.empty((len(seeds), C, Nz, N, N), np.float32)
    ys = np.empty((len(seeds), cout, Nz, N, N), np.float32)
    t0 = time.time()
    with Batch(specs, device=device) as b:
        for k, (f, _) in enumerate(cases):
            b[k].set_data(f)
        b.invalidate()
        b.run(pre_iters).synchronize()
        scs = []
        for k, (f, ang) in enumerate(cases):
            sc = channel_scales(f, C, Nz, N, len(ang))
            scs.append(sc)
            xs[k] = b[k].get("u").reshape(C, Nz, N, N) / sc[:, None, None, None]
        if target_pweight != 1.0 or target_precise:
            for k in range(len(cases)):
                if target_pweight != 1.0:
                    b[k].set_primal_weight(target_pweight)
                if target_precise:
                    b[k].set_precise_primal()
            b.invalidate()
        b.run(target_iters - pre_iters).synchronize()
        for k in range(len(cases)):
            fs = field_scales(fields, scs[k], alpha, b[k].scalars["normest"])
            parts = [b[k].get(fl).reshape(FIELD_COMPS[fl] * C, Nz, N, N) for fl in fields]
            ys[k] = np.concatenate(parts, 0) / fs[:, None, None, None]
    if log:
        log(f"generated {len(seeds)} pairs {N}x{N}x{Nz}x{C} in {time.time() - t0:.1f} s")
    return xs, ys


def train(net: UNet3D, xs: np.ndarray, ys: np.ndarray, steps: int = 2000, batch: int = 4, crop=(16, 64, 64),
          lr: float = 1e-3, lr_final: float = 1e-4, seed: int = 0, log=None, log_every: int = 100):
    """Adam on random crops of the pairs (kept on the device); cosine learning-rate
    decay.  Returns [(step, mean loss over the last log_every steps)]."""
    import torch
    dev = net.dev
    X = torch.from_numpy(xs).to(dev).to(torch.bfloat16)
    Y = torch.from_numpy(ys).to(dev)
    n, _, D, H, W = X.shape
    cd, ch, cw = min(crop[0], D), min(crop[1], H), min(crop[2], W)
    rng = np.random.default_rng(seed)
    xb = torch.empty((batch, net.cin, cd, ch, cw), dtype=torch.bfloat16, device=dev)
    yb = torch.empty((batch, net.cout, cd, ch, cw), dtype=torch.float32, device=dev)
    hist = []
    t0 = time.time()
    acc = torch.zeros((), device=dev)
    for it in range(steps):
        for b in range(batch):
            k = int(rng.integers(n))
            z0, y0, x0 = (int(rng.integers(0, s - c + 1)) for s, c in ((D, cd), (H, ch), (W, cw)))
            xb[b].copy_(X[k, :, z0:z0 + cd, y0:y0 + ch, x0:x0 + cw])
            yb[b].copy_(Y[k, :, z0:z0 + cd, y0:y0 + ch, x0:x0 + cw])
        rate = lr_final + 0.5 * (lr - lr_final) * (1 + math.cos(math.pi * it / max(steps - 1, 1)))
        acc += net.train_step(xb, yb, lr=rate)
        if (it + 1) % log_every == 0:
            v = float(acc) / log_every
            acc.zero_()
            hist.append((it + 1, v))
            if log:
                log(f"step {it + 1} loss {v:.4e} lr {rate:.2e} {time.time() - t0:.1f} s")
    torch.cuda.synchronize(dev)
    return hist


def solve_warm(prob, f, ws: "WarmStarter", tol: float, check_every: int = 100, max_iters: int = 40000,
               fallback_after: int = 10000):
    """Warm start, then iterate to relative gap <= tol.  When a check finds the
    gap not finite (K u = 0 on a bin with data: the image misses a ray the data
    sees), u is lifted along those rays (:meth:`Problem.repair_missed_rays`); if
    it is still not finite fallback_after iterations after the prediction, the
    iterate from before the prediction is restored and the cold iteration
    continues from it -- the plain solver is the fallback.  Returns (iterations including the cold
    ones before the prediction, gap, fell_back)."""
    snap = ws.apply(prob, f, keep_snapshot=True)
    done, fell_back = ws.pre_iters, False
    g = prob.gap()["relative"]
    while not (math.isfinite(g) and g <= tol) and done < max_iters:
        prob.run(check_every)
        done += check_every
        g = prob.gap()["relative"]
        if not math.isfinite(g) and prob.discrepancy == "KL":
            # the iterate misses a ray with data (infinite KL value): lift u along it
            prob.repair_missed_rays()
            g = prob.gap()["relative"]
        if not fell_back and not math.isfinite(g) and done - ws.pre_iters >= fallback_after:
            ws.restore(prob, snap)
            fell_back = True
            g = prob.gap()["relative"]
    return done, g, fell_back


def iterations_to_gap(prob, tol: float, check_every: int = 100, max_iters: int = 100000):
    """Iterate until the relative gap is finite and <= tol; returns (iterations, gap).
    (An infinite primal energy -- K u = 0 on a bin with data -- counts as not converged.)"""
    done = 0
    g = prob.gap()["relative"]
    while not (math.isfinite(g) and g <= tol) and done < max_iters:
        prob.run(check_every)
        done += check_every
        g = prob.gap()["relative"]
    return done, g


def evaluate(net: UNet3D, seeds, N, Nz, C=2, nang=71, mu=(0.2, 5e-4), alpha=(4.0, 1.0), fields=("u",),
             pre_iters=500, tol=1e-2, check_every=100, max_iters=40000, device=0, log=None):
    """Iterations and wall time to relative gap <= tol per held-out seed, for the
    cold start, the same procedure without the network (pre_iters cold
    iterations, lambda from K u of that iterate, missed-ray lift at checks) and
    the warm start (the same with the network's u).  Also the relative distance
    of each final u to the cold run's (the same minimiser)."""
    import torch

    from .solver import Problem
    ws = WarmStarter(net, fields, pre_iters)
    ws_reset = WarmStarter(net, fields, pre_iters, use_network=False)  # everything but the network
    rows = []
    for s in seeds:
        f, ang = phantom_case(s, N, Nz, C, nang, device=device)
        row = {"seed": int(s)}
        finals = {}
        for mode in ("cold", "reset", "warm"):
            with Problem(**problem_spec(N, Nz, C, ang, mu, alpha), device=device) as p:
                p.set_data(f)
                torch.cuda.synchronize(device)
                t0 = time.perf_counter()
                extra = 0
                fell_back = False
                if mode == "warm":
                    it, g, fell_back = solve_warm(p, f, ws, tol, check_every, max_iters)
                elif mode == "reset":
                    it, g, fell_back = solve_warm(p, f, ws_reset, tol, check_every, max_iters)
                else:
                    it, g = iterations_to_gap(p, tol, check_every, max_iters)
                p.synchronize()
                row[mode] = {"iterations": it + extra, "gap": g, "seconds": time.perf_counter() - t0}
                if mode == "warm":
                    row[mode]["fell_back"] = fell_back
                finals[mode] = p.get("u")
        for mode in ("reset", "warm"):
            row[mode]["distance_to_cold"] = float(np.linalg.norm(finals[mode] - finals["cold"]) /
                                                  np.linalg.norm(finals["cold"]))
        rows.append(row)
        if log:
            log(f"seed {s}: cold {row['cold']['iterations']} its {row['cold']['seconds']:.2f} s, "
                f"reset {row['reset']['iterations']} its, warm {row['warm']['iterations']} its "
                f"{row['warm']['seconds']:.2f} s")
    return rows


def _main(argv=None):
    import argparse
    import json
    ap = argparse.ArgumentParser(prog="python -m graptor_gb300.warmstart",
                                 description="Train / evaluate the warm-start U-Net on solver-generated pairs.")
    ap.add_argument("command", choices=("train", "evaluate"))
    ap.add_argument("--weights", required=True, help="npz file to write (train) or read (evaluate)")
    ap.add_argument("--N", type=int, default=128)
    ap.add_argument("--Nz", type=int, default=32)
    ap.add_argument("--C", type=int, default=2)
    ap.add_argument("--nang", type=int, default=71)
    ap.add_argument("--fields", default="u")
    ap.add_argument("--pairs", type=int, default=64, help="training problems (seeds 1000..)")
    ap.add_argument("--target-iters", type=int, default=8000)
    ap.add_argument("--pre-iters", type=int, default=500)
    ap.add_argument("--target-pweight", type=float, default=1.0,
                    help="primal weight of the iterations towards the target (after the input is taken)")
    ap.add_argument("--target-precise", action="store_true",
                    help="the iterations towards the target hold u as two floats (gt_set_precise_primal)")
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--batch", type=int, default=4)
    ap.add_argument("--crop", default="16,64,64")
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--eval-seeds", type=int, default=8, help="held-out seeds (seeds 9000..)")
    ap.add_argument("--tol", type=float, default=1e-2)
    ap.add_argument("--json", default=None)
    ap.add_argument("--pairs-file", default=None, help="npz cache of the training pairs (read if present, else written)")
    a = ap.parse_args(argv)
    fields = tuple(a.fields.split(","))
    log = lambda m: print(m, flush=True)
    out = {}
    if a.command == "train":
        seeds = list(range(1000, 1000 + a.pairs))
        # pairs are generated with u and v (the union of the fields a network may
        # predict) and can be cached in --pairs-file for several trainings
        gen_fields = ("u", "v")
        if a.pairs_file and os.path.exists(a.pairs_file):
            z = np.load(a.pairs_file)
            xs, ys = z["x"], z["y"]
            log(f"loaded {len(xs)} pairs from {a.pairs_file}")
        else:
            xs, ys = [], []
            for k in range(0, len(seeds), 16):
                x, y = generate_pairs(seeds[k:k + 16], a.N, a.Nz, a.C, a.nang, fields=gen_fields,
                                      pre_iters=a.pre_iters, target_iters=a.target_iters, log=log,
                                      target_pweight=a.target_pweight, target_precise=a.target_precise)
                xs.append(x)
                ys.append(y)
            xs, ys = np.concatenate(xs), np.concatenate(ys)
            if a.pairs_file:
                np.savez(a.pairs_file, x=xs, y=ys)
        # the channels of the requested fields, in generate_pairs' order (field-major)
        offs, o = {}, 0
        for fl in gen_fields:
            offs[fl] = o
            o += FIELD_COMPS[fl] * a.C
        ys = np.concatenate([ys[:, offs[fl]:offs[fl] + FIELD_COMPS[fl] * a.C] for fl in fields], 1)
        net = UNet3D(a.C, output_channels(a.C, fields), residual=a.C)
        log(f"U-Net parameters: {net.nparams}")
        hist = train(net, xs, ys, steps=a.steps, batch=a.batch, crop=tuple(int(c) for c in a.crop.split(",")),
                     lr=a.lr, log=log)
        net.save(a.weights)
        out["train"] = {"pairs": len(seeds), "loss": hist, "params": net.nparams}
    else:
        net = UNet3D.load(a.weights)
        rows = evaluate(net, range(9000, 9000 + a.eval_seeds), a.N, a.Nz, a.C, a.nang, fields=fields,
                        pre_iters=a.pre_iters, tol=a.tol, log=log)
        ci = np.array([r["cold"]["iterations"] for r in rows], float)
        wi = np.array([r["warm"]["iterations"] for r in rows], float)
        ct = np.array([r["cold"]["seconds"] for r in rows])
        wt = np.array([r["warm"]["seconds"] for r in rows])
        ri = np.array([r["reset"]["iterations"] for r in rows], float)
        out["evaluate"] = {"rows": rows, "tol": a.tol, "iter_ratio": float(ci.sum() / wi.sum()),
                           "time_ratio": float(ct.sum() / wt.sum()), "reset_iter_ratio": float(ci.sum() / ri.sum())}
        log(f"cold/warm iterations {ci.sum() / wi.sum():.2f}x, wall time {ct.sum() / wt.sum():.2f}x; "
            f"cold/reset-only iterations {ci.sum() / ri.sum():.2f}x")
    if a.json:
        with open(a.json, "w") as fh:
            json.dump(out, fh, indent=1)


if __name__ == "__main__":
    _main()
