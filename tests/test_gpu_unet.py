"""Warm-start network kernels (gt_nn_*) against PyTorch CPU float64.

Kernel tests run the float32 paths against float64 references of the same
operation (weights are bfloat16 on both sides).  The network test runs the
whole U-Net forward and backward (bfloat16 activations, float32 sums) against
a float64 autograd network that rounds the same activations to bfloat16
(straight-through), and reports the distance to the unrounded float64 network.
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
F = torch.nn.functional

pytestmark = pytest.mark.gpu


def _lib():
    from graptor_gb300 import _lib as L
    return L


_KEEP = []


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def _d(t):
    """Device copy kept alive until the test's next synchronisation (a temporary
    freed right after its pointer is taken could be reused by the caching
    allocator before the kernel reads it)."""
    d = t.cuda()
    _KEEP.append(d)
    return d


def rel(a, b):
    a = torch.as_tensor(a).double().cpu()
    b = torch.as_tensor(b).double().cpu()
    return float((a - b).norm() / max(b.norm(), 1e-300))


def _bf16(shape, g, scale=1.0):
    return (torch.randn(shape, generator=g) * scale).to(torch.bfloat16)


@pytest.mark.parametrize("k", [3, 1])
def test_conv_forward_views_accumulate(k):
    L = _lib()
    g = torch.Generator().manual_seed(11 + k)
    B, Ci, Co, D, H, W = 2, 5, 11, 4, 6, 8
    Cx, xoff, Cy, yoff = Ci + 3, 2, Co + 2, 1
    x = torch.randn((B, Cx, D, H, W), generator=g)
    w = _bf16((Co, Ci, k, k, k), g, 0.2)
    bias = torch.randn(Co, generator=g)
    y0 = torch.randn((B, Cy, D, H, W), generator=g)
    xd, wd, bd, yd = x.cuda(), w.cuda(), bias.cuda(), y0.clone().cuda()
    L.check(L.lib().gt_nn_conv3d(_p(xd), 0, Ci, Cx, xoff, _p(wd), _p(bd), _p(yd), 0, Co, Cy, yoff, B, D, H, W, k, 1, 1,
                                 None))
    torch.cuda.synchronize()
    ref = F.conv3d(x[:, xoff:xoff + Ci].double(), w.double(), bias.double(), padding=k // 2)
    expect = y0.double().clone()
    expect[:, yoff:yoff + Co] = torch.relu(expect[:, yoff:yoff + Co] + ref)
    out = yd.cpu()
    assert rel(out[:, yoff:yoff + Co], expect[:, yoff:yoff + Co]) < 1e-6
    # channels outside the view are untouched
    assert torch.equal(out[:, :yoff], y0[:, :yoff]) and torch.equal(out[:, yoff + Co:], y0[:, yoff + Co:])


@pytest.mark.parametrize("k", [3, 1])
def test_conv_backward_matches_autograd(k):
    L = _lib()
    lib = L.lib()
    g = torch.Generator().manual_seed(29 + k)
    B, Ci, Co, D, H, W = 2, 6, 9, 4, 8, 12
    Cx, xoff, Cg, goff = Ci + 2, 1, Co + 3, 3
    x = torch.randn((B, Cx, D, H, W), generator=g)
    w = _bf16((Co, Ci, k, k, k), g, 0.2)
    dy = torch.randn((B, Cg, D, H, W), generator=g)
    # float64 autograd reference
    x64 = x[:, xoff:xoff + Ci].double().requires_grad_()
    w64 = w.double().requires_grad_()
    b64 = torch.zeros(Co, dtype=torch.float64, requires_grad=True)
    yref = F.conv3d(x64, w64, b64, padding=k // 2)
    gx, gw, gb = torch.autograd.grad(yref, (x64, w64, b64), dy[:, goff:goff + Co].double())
    xd, wd, dyd = x.cuda(), w.cuda(), dy.cuda()
    wf = torch.empty_like(wd)
    L.check(lib.gt_nn_flip_weights(_p(wd), _p(wf), Co, Ci, k, None))
    dx = torch.zeros((B, Ci, D, H, W), device="cuda")
    L.check(lib.gt_nn_conv3d(_p(dyd), 0, Co, Cg, goff, _p(wf), None, _p(dx), 0, Ci, Ci, 0, B, D, H, W, k, 0, 0, None))
    nvox = B * D * H * W
    for kchunk in (nvox, 100, 37):
        nchunk = -(-nvox // kchunk)
        part = torch.empty(nchunk * Co * Ci * k ** 3, device="cuda")
        gwd = torch.empty((Co, Ci, k, k, k), device="cuda")
        L.check(lib.gt_nn_conv3d_wgrad(_p(dyd), Co, Cg, goff, _p(xd), 0, Ci, Cx, xoff, B, D, H, W, k, kchunk, _p(part),
                                       _p(gwd), 0, None))
        torch.cuda.synchronize()
        assert rel(gwd.cpu(), gw) < 1e-5, kchunk
    gbd = torch.empty(Co, device="cuda")
    L.check(lib.gt_nn_bias_grad(_p(dyd), Co, Cg, goff, B, D * H * W, _p(gbd), 0, None))
    torch.cuda.synchronize()
    assert rel(dx.cpu(), gx) < 1e-5
    assert rel(gbd.cpu(), gb) < 1e-5


def test_wgrad_bf16_input_and_accumulate():
    L = _lib()
    lib = L.lib()
    g = torch.Generator().manual_seed(5)
    B, Ci, Co, D, H, W, k = 1, 4, 16, 8, 8, 16, 3
    x = _bf16((B, Ci, D, H, W), g)
    dy = torch.randn((B, Co, D, H, W), generator=g)
    x64 = x.double().requires_grad_()
    w64 = torch.zeros((Co, Ci, k, k, k), dtype=torch.float64, requires_grad=True)
    (gw,) = torch.autograd.grad(F.conv3d(x64, w64, padding=1), (w64,), dy.double())
    xd, dyd = x.cuda(), dy.cuda()
    g0 = torch.randn((Co, Ci, k, k, k), generator=g)
    gwd = g0.clone().cuda()
    kchunk = 256
    part = torch.empty(-(-B * D * H * W // kchunk) * Co * Ci * 27, device="cuda")
    L.check(lib.gt_nn_conv3d_wgrad(_p(dyd), Co, Co, 0, _p(xd), 1, Ci, Ci, 0, B, D, H, W, k, kchunk, _p(part), _p(gwd),
                                   1, None))
    torch.cuda.synchronize()
    assert rel(gwd.cpu(), gw + g0.double()) < 1e-5


def test_pool_up_and_their_gradients():
    L = _lib()
    lib = L.lib()
    g = torch.Generator().manual_seed(7)
    B, C, Cs, off, D, H, W = 2, 3, 7, 2, 4, 8, 8
    x = _bf16((B, Cs, D, H, W), g)
    y = torch.empty((B, C, D // 2, H // 2, W // 2), dtype=torch.bfloat16, device="cuda")
    L.check(lib.gt_nn_pool2(_p(_d(x)), Cs, off, _p(y), C, B, D // 2, H // 2, W // 2, None))
    torch.cuda.synchronize()
    ref = F.avg_pool3d(x[:, off:off + C].double(), 2)
    assert rel(y.cpu().double(), ref) < 4e-3  # one bfloat16 rounding
    assert rel(y.cpu().double(), ref.to(torch.bfloat16).double()) < 1e-6
    # pool gradient (added into a view of a wider tensor)
    dy = torch.randn((B, C, D // 2, H // 2, W // 2), generator=g)
    dx0 = torch.randn((B, Cs, D, H, W), generator=g)
    dx = dx0.clone().cuda()
    L.check(lib.gt_nn_pool2_bwd(_p(_d(dy)), _p(dx), C, Cs, off, B, D, H, W, None))
    torch.cuda.synchronize()
    x64 = torch.zeros((B, C, D, H, W), dtype=torch.float64, requires_grad=True)
    (gx,) = torch.autograd.grad(F.avg_pool3d(x64, 2), (x64,), dy.double())
    expect = dx0.double().clone()
    expect[:, off:off + C] += gx
    assert rel(dx.cpu(), expect) < 1e-6
    # nearest upsampling into a view and its gradient
    xs = _bf16((B, C, D // 2, H // 2, W // 2), g)
    up = torch.zeros((B, Cs, D, H, W), dtype=torch.bfloat16, device="cuda")
    L.check(lib.gt_nn_up2(_p(_d(xs)), _p(up), C, Cs, off, B, D, H, W, None))
    torch.cuda.synchronize()
    assert torch.equal(up.cpu()[:, off:off + C], F.interpolate(xs.float(), scale_factor=2, mode="nearest").bfloat16())
    gup = torch.randn((B, Cs, D, H, W), generator=g)
    gxs = torch.empty((B, C, D // 2, H // 2, W // 2), device="cuda")
    L.check(lib.gt_nn_up2_bwd(_p(_d(gup)), Cs, off, _p(gxs), C, B, D // 2, H // 2, W // 2, None))
    torch.cuda.synchronize()
    xs64 = xs.double().requires_grad_()
    (gref,) = torch.autograd.grad(F.interpolate(xs64, scale_factor=2, mode="nearest"), (xs64,),
                                  gup[:, off:off + C].double())
    assert rel(gxs.cpu(), gref) < 1e-6


def test_relu_mask_scale_mse_adam():
    L = _lib()
    lib = L.lib()
    g = torch.Generator().manual_seed(3)
    B, C, Cy, off, vol = 2, 3, 5, 1, 40
    y = _bf16((B, Cy, vol), g)
    dy0 = torch.randn((B, Cy, vol), generator=g)
    dy = dy0.clone().cuda()
    L.check(lib.gt_nn_relu_bwd(_p(dy), _p(_d(y)), 1, C, Cy, off, B, vol, None))
    torch.cuda.synchronize()
    expect = dy0.clone()
    view = expect[:, off:off + C]
    view[y[:, off:off + C].float() <= 0] = 0
    assert torch.equal(dy.cpu(), expect)
    # per-(sample, channel) scale with floor, f32 -> bf16
    x = torch.randn((B, C, vol), generator=g)
    sc = torch.rand(B * C, generator=g) + 0.5
    out = torch.empty((B, C, vol), dtype=torch.bfloat16, device="cuda")
    L.check(lib.gt_nn_scale(_p(_d(x)), 0, _p(out), 1, C, B, vol, _p(_d(sc)), 1, None))
    torch.cuda.synchronize()
    ref = torch.clamp(x * sc.view(B, C, 1), min=0).bfloat16()
    assert torch.equal(out.cpu(), ref)
    # mse
    n = 1000
    pr, q = torch.randn(n, generator=g), torch.randn(n, generator=g)
    dp = torch.empty(n, device="cuda")
    part = torch.empty(-(-n // 256), device="cuda")
    L.check(lib.gt_nn_mse(_p(_d(pr)), _p(_d(q)), n, _p(dp), _p(part), None))
    torch.cuda.synchronize()
    assert rel(part.cpu().sum(), ((pr - q) ** 2).double().sum()) < 1e-6
    assert rel(dp.cpu(), 2 * (pr - q).double() / n) < 1e-6
    # adam, two steps against the textbook update in float64
    wm = torch.randn(n, generator=g)
    grads = [torch.randn(n, generator=g) for _ in range(2)]
    wmd, m, v = wm.clone().cuda(), torch.zeros(n, device="cuda"), torch.zeros(n, device="cuda")
    wb = torch.empty(n, dtype=torch.bfloat16, device="cuda")
    lr, b1, b2, eps = 1e-2, 0.9, 0.999, 1e-8
    w64, m64, v64 = wm.double(), torch.zeros(n, dtype=torch.float64), torch.zeros(n, dtype=torch.float64)
    for step, gr in enumerate(grads, 1):
        L.check(lib.gt_nn_adam(_p(wmd), _p(wb), _p(_d(gr)), _p(m), _p(v), n, lr, b1, b2, eps, step, None))
        m64 = b1 * m64 + (1 - b1) * gr.double()
        v64 = b2 * v64 + (1 - b2) * gr.double() ** 2
        w64 = w64 - lr * (m64 / (1 - b1 ** step)) / ((v64 / (1 - b2 ** step)).sqrt() + eps)
    torch.cuda.synchronize()
    assert rel(wmd.cpu(), w64) < 1e-6
    assert torch.equal(wb.cpu(), wmd.cpu().bfloat16())


# ------------------------------------------------------------------ whole network
def _ref_net(net, x, emulate):
    """float64 autograd U-Net with the weights of `net` (bfloat16 values, float32 biases)."""
    wb = net.wb.cpu().double()
    master = net.master.cpu().double()
    params = {}
    for name, ci, co, k in net.layers:
        o, ob, *_ = net.offsets[name]
        params[name] = (wb[o:ob].view(co, ci, k, k, k).clone().requires_grad_(),
                        master[ob:ob + co].clone().requires_grad_())

    def q(t):
        return t + (t.to(torch.bfloat16).double() - t).detach() if emulate else t

    def conv(t, name, relu=True):
        w, b = params[name]
        y = F.conv3d(t, w, b, padding=w.shape[-1] // 2)
        return torch.relu(y) if relu else y

    up = lambda t: F.interpolate(t, scale_factor=2, mode="nearest")
    a1 = q(conv(x, "enc1a"))
    e1 = q(conv(a1, "enc1b"))
    p1 = q(F.avg_pool3d(e1, 2))
    a2 = q(conv(p1, "enc2a"))
    e2 = q(conv(a2, "enc2b"))
    p2 = q(F.avg_pool3d(e2, 2))
    a3 = q(conv(p2, "bota"))
    bb = q(conv(a3, "botb"))
    a4 = q(conv(torch.cat([e2, up(bb)], 1), "dec2a"))
    d2 = q(conv(a4, "dec2b"))
    a5 = q(conv(torch.cat([e1, up(d2)], 1), "dec1a"))
    d1 = q(conv(a5, "dec1b"))
    out = conv(d1, "head", relu=False)
    base = torch.zeros_like(out)
    base[:, :net.residual] = x[:, :net.residual]
    return out + base, params


@pytest.mark.parametrize("tc", [0, 1])
def test_unet_forward_backward_vs_float64(tc):
    """tc = 0: every convolution on the CUDA cores, checked against a float64 network
    that rounds the same activations to bfloat16 (tight) and against the unrounded
    float64 network (loose).  tc = 1: the convolutions with 16k channels on the
    tensor cores; their FP32 sums run in another order, so some bfloat16 roundings
    of activations (and ReLU masks at zero) land on the other side of the
    emulation's -- checked against the unrounded network only, with the same bound."""
    L = _lib()
    L.check(L.lib().gt_nn_set_tensor_cores(tc))
    try:
        _unet_forward_backward_vs_float64(tc)
    finally:
        L.check(L.lib().gt_nn_set_tensor_cores(1))


def _unet_run(tc):
    """Output and gradient of the test network on its fixed batch."""
    from graptor_gb300.warmstart import UNet3D
    L = _lib()
    L.check(L.lib().gt_nn_set_tensor_cores(tc))
    g = torch.Generator().manual_seed(2024)
    cin, cout, B, D, H, W = 2, 8, 2, 8, 16, 16
    net = UNet3D(cin, cout, residual=cin, seed=1)
    o, ob, *_ = net.offsets["head"]
    net.master[o:ob] = (torch.randn(ob - o, generator=g) * 0.25).cuda()
    net.refresh()
    x = (torch.rand((B, cin, D, H, W), generator=g) * 2).to(torch.bfloat16)
    out = torch.empty((B, cout, D, H, W), device="cuda")
    net.residual_base(x.cuda(), out)
    net.forward(x.cuda(), out)
    G = torch.randn((B, cout, D, H, W), generator=g)
    net.backward(x.cuda(), G.cuda())
    torch.cuda.synchronize()
    L.check(L.lib().gt_nn_check())
    return net, out.cpu(), net.grad.cpu()


def test_unet_tensor_cores_agree_with_cuda_cores():
    """The whole network with its 16k-channel convolutions on the tensor cores
    against the same network on the CUDA cores: outputs within bfloat16 rounding;
    weight and bias gradients within 15 %, the scale at which either bfloat16
    network's gradients differ from the unrounded float64 network's (5-11 %:
    activations rounded to bfloat16, ReLU masks at zero)."""
    try:
        net, out1, g1 = _unet_run(1)
        _, out0, g0 = _unet_run(0)
    finally:
        _lib().check(_lib().lib().gt_nn_set_tensor_cores(1))
    assert rel(out1, out0) < 5e-3
    for name, ci, co, k in net.layers:
        o, ob, *_ = net.offsets[name]
        assert rel(g1[o:ob], g0[o:ob]) < 1.5e-1, name
        assert rel(g1[ob:ob + co], g0[ob:ob + co]) < 1.5e-1, name


def _unet_forward_backward_vs_float64(tc):
    from graptor_gb300.warmstart import UNet3D
    g = torch.Generator().manual_seed(2024)
    cin, cout, B, D, H, W = 2, 8, 2, 8, 16, 16
    net = UNet3D(cin, cout, residual=cin, seed=1)
    # a head with real weights, so every layer gets gradient
    o, ob, *_ = net.offsets["head"]
    net.master[o:ob] = (torch.randn(ob - o, generator=g) * 0.25).cuda()
    net.refresh()
    x = (torch.rand((B, cin, D, H, W), generator=g) * 2).to(torch.bfloat16)
    xd = x.cuda()
    out = torch.empty((B, cout, D, H, W), device="cuda")
    net.residual_base(xd, out)
    net.forward(xd, out)
    G = torch.randn((B, cout, D, H, W), generator=g)
    net.backward(xd, G.cuda())
    torch.cuda.synchronize()
    got_out, got_grad = out.cpu(), net.grad.cpu()
    report = {}
    cases = ((False, 5e-2, 3e-1),) if tc else ((True, 1e-3, 5e-3), (False, 5e-2, 3e-1))
    for emulate, tol_out, tol_grad in cases:
        ref, params = _ref_net(net, x.double(), emulate)
        names = [n for n, *_ in net.layers]
        leaves = [t for n in names for t in params[n]]
        grads = torch.autograd.grad(ref, leaves, G.double())
        e_out = rel(got_out, ref.detach())
        assert e_out < tol_out, (emulate, e_out)
        for i, (name, ci, co, k) in enumerate(net.layers):
            o, ob, *_ = net.offsets[name]
            ew = rel(got_grad[o:ob], grads[2 * i].flatten())
            eb = rel(got_grad[ob:ob + co], grads[2 * i + 1])
            report[(emulate, name)] = (ew, eb)
            assert ew < tol_grad and eb < tol_grad, (emulate, name, ew, eb)
    print({k: tuple(round(x, 6) for x in v) for k, v in report.items()})


def test_unet_overfits_one_batch():
    """A few hundred Adam steps of the project's kernels drive the loss on one
    fixed batch down by a large factor (the training loop works end to end)."""
    from graptor_gb300.warmstart import UNet3D
    g = torch.Generator().manual_seed(9)
    cin, cout, B, D, H, W = 1, 4, 2, 8, 16, 16
    net = UNet3D(cin, cout, residual=cin, seed=2)
    x = torch.rand((B, cin, D, H, W), generator=g).to(torch.bfloat16).cuda()
    # a smooth target: a blurred copy of x plus fields derived from it
    xf = x.float()
    blur = F.avg_pool3d(F.pad(xf, (1, 1, 1, 1, 1, 1), mode="replicate"), 3, stride=1)
    tgt = torch.cat([blur, 0.5 * torch.tanh(xf - blur).repeat(1, 3, 1, 1, 1)], 1).contiguous()
    losses = [float(net.train_step(x, tgt, lr=3e-3)) for _ in range(300)]
    assert np.isfinite(losses).all()
    assert losses[-1] < 0.1 * losses[0], (losses[0], losses[-1])


@pytest.mark.parametrize("k,Ci,Co,ydt", [(3, 16, 16, 0), (3, 32, 64, 1), (1, 48, 32, 0), (3, 16, 48, 0)])
def test_conv_tensor_cores_match_cuda_cores(k, Ci, Co, ydt):
    """The tcgen05 implicit-GEMM convolution (bfloat16 operands, FP32 accumulator in
    tensor memory) against the CUDA-core kernel on the same bfloat16 inputs, with
    channel views, bias, accumulation and ReLU; and against float64."""
    L = _lib()
    lib = L.lib()
    g = torch.Generator().manual_seed(100 + k + Ci + Co)
    B, D, H, W = 2, 5, 6, 12  # 720 voxels: five full 128-voxel tiles and a partial one
    Cx, xoff, Cy, yoff = Ci + 16, 16, Co + 3, 2
    x = _bf16((B, Cx, D, H, W), g)
    w = _bf16((Co, Ci, k, k, k), g, 0.1)
    bias = torch.randn(Co, generator=g)
    ytype = torch.bfloat16 if ydt else torch.float32
    y0 = torch.randn((B, Cy, D, H, W), generator=g).to(ytype)
    outs = []
    try:
        for tc in (0, 1):
            L.check(lib.gt_nn_set_tensor_cores(tc))
            y = _d(y0)
            xd, wd, bd = _d(x), _d(w), _d(bias)
            L.check(lib.gt_nn_conv3d(_p(xd), 1, Ci, Cx, xoff, _p(wd), _p(bd), _p(y), ydt, Co, Cy, yoff, B, D, H, W, k,
                                     1, 1, None))
            torch.cuda.synchronize()
            L.check(lib.gt_nn_check())
            outs.append(y.cpu().double())
    finally:
        L.check(lib.gt_nn_set_tensor_cores(1))
    ref = F.conv3d(x[:, xoff:xoff + Ci].double(), w.double(), bias.double(), padding=k // 2)
    ref = torch.relu(ref + y0[:, yoff:yoff + Co].double())
    sl = slice(yoff, yoff + Co)
    tol = 1e-2 if ydt else 1e-5
    assert rel(outs[1][:, sl], outs[0][:, sl]) < tol
    assert rel(outs[1][:, sl], ref) < (1e-2 if ydt else 1e-5)
    # channels outside the view are untouched
    assert torch.equal(outs[1][:, :yoff], y0[:, :yoff].double())
    assert torch.equal(outs[1][:, yoff + Co:], y0[:, yoff + Co:].double())


@pytest.mark.parametrize("W,H,Ci,Co,ydt", [(128, 2, 16, 16, 0), (256, 1, 32, 64, 1), (64, 4, 32, 32, 0),
                                           (32, 4, 16, 64, 0), (16, 8, 48, 16, 1), (8, 16, 16, 32, 0),
                                           (4, 32, 16, 16, 0)])
def test_staged_tensor_core_convolution(W, H, Ci, Co, ydt):
    """The 3x3x3 tensor-core kernel that stages each 16-channel chunk's input halo
    and weights in shared memory (rows of 128 voxels read straight from the halo for
    W >= 128, copied into an A tile for W < 128) against the kernel that gathers
    every tap from global memory, the CUDA cores and float64: channel views, bias,
    accumulation, ReLU, borders on every side."""
    L = _lib()
    lib = L.lib()
    g = torch.Generator().manual_seed(7 * W + H + Ci + Co)
    B, D = 2, 3
    Cx, xoff, Cy, yoff = Ci + 16, 16, Co + 3, 2
    x = _bf16((B, Cx, D, H, W), g)
    w = _bf16((Co, Ci, 3, 3, 3), g, 0.1)
    bias = torch.randn(Co, generator=g)
    ytype = torch.bfloat16 if ydt else torch.float32
    y0 = torch.randn((B, Cy, D, H, W), generator=g).to(ytype)
    outs = {}
    try:
        for mode in (0, 2, 1):
            L.check(lib.gt_nn_set_tensor_cores(mode))
            y = _d(y0)
            xd, wd, bd = _d(x), _d(w), _d(bias)
            L.check(lib.gt_nn_conv3d(_p(xd), 1, Ci, Cx, xoff, _p(wd), _p(bd), _p(y), ydt, Co, Cy, yoff, B, D, H, W, 3,
                                     1, 1, None))
            torch.cuda.synchronize()
            L.check(lib.gt_nn_check())
            outs[mode] = y.cpu().double()
    finally:
        L.check(lib.gt_nn_set_tensor_cores(1))
    ref = F.conv3d(x[:, xoff:xoff + Ci].double(), w.double(), bias.double(), padding=1)
    ref = torch.relu(ref + y0[:, yoff:yoff + Co].double())
    sl = slice(yoff, yoff + Co)
    tol = 1e-2 if ydt else 1e-5
    assert rel(outs[1][:, sl], outs[2][:, sl]) < tol
    assert rel(outs[1][:, sl], outs[0][:, sl]) < tol
    assert rel(outs[1][:, sl], ref) < tol
    assert torch.equal(outs[1][:, :yoff], y0[:, :yoff].double())
    assert torch.equal(outs[1][:, yoff + Co:], y0[:, yoff + Co:].double())
