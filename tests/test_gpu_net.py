"""The warm-start network's kernels against torch CPU float64 references.

Inputs and weights are BF16 (exactly representable, so the reference sees the
same numbers); the kernels accumulate in FP32.  Tolerances: BF16 outputs
carry one rounding (2^-8 relative) -> 1e-2 of the reference's magnitude plus
1e-3 of its maximum; FP32 weight gradients -> 1e-4 of their maximum.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env(built_lib):
    import torch
    import _flf
    _flf.load_library()
    return torch, _flf


def _ref_conv(torch, x, w, bias=None):
    """x [B,Z,Y,X,Ci], w [27,Ci,Co] (float64 CPU) -> [B,Z,Y,X,Co]."""
    Ci, Co = w.shape[1], w.shape[2]
    wt = w.reshape(3, 3, 3, Ci, Co).permute(4, 3, 0, 1, 2)
    y = torch.nn.functional.conv3d(x.permute(0, 4, 1, 2, 3), wt, bias=bias, padding=1)
    return y.permute(0, 2, 3, 4, 1)


def _close(torch, got, ref, rel=1e-2, absf=1e-3):
    got = got.double().cpu()
    err = (got - ref).abs()
    lim = rel * ref.abs() + absf * ref.abs().max()
    assert bool((err <= lim).all()), float((err - lim).max())


@pytest.mark.parametrize("shape,Ci,Co,relu", [
    ((2, 4, 6, 10), 16, 16, False), ((1, 3, 7, 9), 32, 64, True), ((1, 5, 5, 13), 64, 128, True),
    ((3, 2, 4, 4), 128, 32, False), ((1, 8, 16, 16), 16, 64, True),
    # the persistent patch-tiled kernel (16 / 32 channels in and out), ragged tiles
    ((2, 3, 9, 20), 16, 32, True), ((1, 5, 17, 33), 32, 16, False), ((1, 4, 8, 16), 32, 32, True),
    ((1, 2, 3, 5), 16, 16, True), ((2, 6, 24, 40), 16, 16, False),
    # few output tiles and a long K loop: split across CTAs through the workspace
    ((1, 3, 6, 6), 128, 64, True), ((1, 2, 5, 7), 64, 128, False), ((2, 3, 9, 9), 64, 32, True),
    # more than one 128-voxel tile with a ragged last one (the tcgen05 kernel of the wide layers)
    ((2, 6, 12, 23), 64, 64, True), ((1, 5, 11, 17), 128, 128, False), ((1, 4, 9, 30), 32, 128, True),
    ((1, 4, 9, 30), 128, 32, False),
])
def test_conv3d_forward(env, shape, Ci, Co, relu):
    torch, _flf = env
    g = torch.Generator().manual_seed(Ci * Co + shape[1])
    x = torch.randn(shape + (Ci,), generator=g).bfloat16()
    w = (torch.randn((27, Ci, Co), generator=g) / np.sqrt(27 * Ci)).bfloat16()
    b = torch.randn(Co, generator=g).float()
    y = torch.empty(shape + (Co,), dtype=torch.bfloat16, device="cuda")
    ws = torch.empty(4 * int(np.prod(shape)) * Co, device="cuda")    # room for 4 K slices
    ref = _ref_conv(torch, x.double(), w.double(), b.double())
    if relu:
        ref = ref.clamp_min(0)
    # without and with the packed weights (with them the wide layers run on tcgen05)
    wp = torch.empty((27, Ci, Co), dtype=torch.bfloat16, device="cuda")
    _flf.conv3d_pack(w.cuda(), wp)
    for packed in (None, wp):
        _flf.conv3d(x.cuda(), w.cuda(), b.cuda(), y, relu=relu, ws=ws, wp=packed)
        _close(torch, y, ref)
        # split layers add their K slices in a fixed order: the same bits again
        y2 = torch.empty_like(y)
        _flf.conv3d(x.cuda(), w.cuda(), b.cuda(), y2, relu=relu, ws=ws, wp=packed)
        assert torch.equal(y, y2)
    if max(Ci, Co) >= 64:
        # every work-item shape of the tcgen05 kernel (1..4 M tiles of 128 padded-row positions)
        try:
            for mode in (2, 3, 4, 5):
                _flf.conv_wide_tcgen05(mode)
                y.zero_()
                _flf.conv3d(x.cuda(), w.cuda(), b.cuda(), y, relu=relu, ws=ws, wp=wp)
                _close(torch, y, ref)
        finally:
            _flf.conv_wide_tcgen05(1)
    torch.cuda.synchronize()
    _flf.net_status()


@pytest.mark.parametrize("shape,Ci,Co", [((2, 4, 6, 10), 32, 16), ((1, 3, 6, 6), 64, 128), ((2, 5, 9, 13), 128, 64),
                                         ((1, 4, 7, 11), 32, 64)])
def test_conv3d_mask_and_data_gradient(env, shape, Ci, Co):
    torch, _flf = env
    g = torch.Generator().manual_seed(3)
    x = torch.randn(shape + (Ci,), generator=g).bfloat16().double().requires_grad_()
    w = (torch.randn((27, Ci, Co), generator=g) / 15).bfloat16()
    dy = torch.randn(shape + (Co,), generator=g).bfloat16()
    act = torch.randn(shape + (Ci,), generator=g).bfloat16()     # ReLU output of the layer before
    y = _ref_conv(torch, x, w.double())
    y.backward(dy.double())
    ref = x.grad * (act.double() > 0)
    w2 = torch.empty((27, Co, Ci), dtype=torch.bfloat16, device="cuda")
    _flf.conv3d_flip(w.cuda(), w2)
    dx = torch.empty(shape + (Ci,), dtype=torch.bfloat16, device="cuda")
    ws = torch.empty(4 * int(np.prod(shape)) * Ci, device="cuda")
    _flf.conv3d(dy.cuda(), w2, None, dx, mask=act.cuda(), ws=ws)
    _close(torch, dx, ref)
    # the data gradient on tcgen05 (packed flipped weights)
    w2p = torch.empty_like(w2)
    _flf.conv3d_pack(w2, w2p)
    dx.zero_()
    _flf.conv3d(dy.cuda(), w2, None, dx, mask=act.cuda(), ws=ws, wp=w2p)
    _close(torch, dx, ref)


@pytest.mark.parametrize("shape,Ci,Co,relu,masked", [
    # the network's wide layers at inference (24 x 456 x 456 volume: levels 2 and 3)
    ((1, 6, 114, 114), 32, 64, True, False), ((1, 6, 114, 114), 64, 64, True, False),
    ((1, 6, 114, 114), 64, 32, True, False), ((1, 3, 57, 57), 64, 128, True, False),
    ((1, 3, 57, 57), 128, 128, True, False), ((1, 3, 57, 57), 128, 64, True, False),
    # training crops (4 x 24 x 128 x 128) with the ReLU mask of a data gradient
    ((4, 6, 32, 32), 64, 64, False, True), ((4, 3, 16, 16), 128, 128, False, True),
    ((4, 6, 32, 32), 64, 32, False, True), ((4, 3, 16, 16), 64, 128, False, True),
    # the widest padded row a TMA box takes (254 + 2), and a wider one (mma.sync)
    ((1, 2, 9, 254), 64, 64, True, False), ((1, 2, 5, 300), 64, 64, True, False),
])
def test_wide_layers_against_fp32_conv(env, shape, Ci, Co, relu, masked):
    """The wide layers at the network's own shapes, against torch's FP32 conv3d on the
    same BF16 inputs (TF32 off), both kernels and every tcgen05 work-item shape."""
    torch, _flf = env
    g = torch.Generator().manual_seed(Ci + 7 * Co + shape[-1])
    x = torch.randn(shape + (Ci,), generator=g).bfloat16().cuda()
    w = (torch.randn((27, Ci, Co), generator=g) / np.sqrt(27 * Ci)).bfloat16().cuda()
    b = None if masked else torch.randn(Co, generator=g).float().cuda()
    mask = torch.randn(shape + (Co,), generator=g).bfloat16().cuda() if masked else None
    old = torch.backends.cudnn.allow_tf32
    torch.backends.cudnn.allow_tf32 = False
    try:
        wr = w.float().reshape(3, 3, 3, Ci, Co).permute(4, 3, 0, 1, 2).contiguous()
        ref = torch.nn.functional.conv3d(x.float().permute(0, 4, 1, 2, 3), wr, bias=b, padding=1)
        ref = ref.permute(0, 2, 3, 4, 1).double().cpu()
    finally:
        torch.backends.cudnn.allow_tf32 = old
    if relu:
        ref = ref.clamp_min(0)
    if masked:
        ref = ref * (mask.double().cpu() > 0)
    wp = torch.empty_like(w)
    _flf.conv3d_pack(w, wp)
    y = torch.empty(shape + (Co,), dtype=torch.bfloat16, device="cuda")
    ws = torch.empty(4 * int(np.prod(shape)) * Co, device="cuda")
    first = None
    try:
        for mode in (0, 1, 2, 3, 4, 5):
            _flf.conv_wide_tcgen05(mode)
            y.zero_()
            _flf.conv3d(x, w, b, y, relu=relu, mask=mask, ws=ws, wp=wp)
            _close(torch, y, ref)
            if mode == 1:
                first = y.clone()
        _flf.conv_wide_tcgen05(1)
        _flf.conv3d(x, w, b, y, relu=relu, mask=mask, ws=ws, wp=wp)
        assert torch.equal(y, first)      # the same bits on a second run
    finally:
        _flf.conv_wide_tcgen05(1)
    torch.cuda.synchronize()
    _flf.net_status()


@pytest.mark.parametrize("shape,Ci,Co", [((2, 4, 6, 10), 16, 16), ((1, 6, 9, 11), 32, 64), ((2, 3, 8, 8), 128, 128),
                                         ((1, 4, 4, 4), 64, 32)])
def test_conv3d_weight_and_bias_gradient(env, shape, Ci, Co):
    torch, _flf = env
    g = torch.Generator().manual_seed(Ci + Co)
    x = torch.randn(shape + (Ci,), generator=g).bfloat16()
    w = torch.zeros((27, Ci, Co), dtype=torch.float64, requires_grad=True)
    b = torch.zeros(Co, dtype=torch.float64, requires_grad=True)
    dy = torch.randn(shape + (Co,), generator=g).bfloat16()
    _ref_conv(torch, x.double(), w, b).backward(dy.double())
    ws = torch.empty(64 * 27 * Ci * Co, dtype=torch.float32, device="cuda")
    runs = []
    for use_ws in (False, True, True):
        dw = torch.zeros((27, Ci, Co), dtype=torch.float32, device="cuda")
        db = torch.zeros(Co, dtype=torch.float32, device="cuda")
        _flf.conv3d_wgrad(x.cuda(), dy.cuda(), dw, ws=ws if use_ws else None)
        _flf.bias_grad(dy.cuda(), db, ws=ws if use_ws else None)
        assert float((dw.double().cpu() - w.grad).abs().max()) <= 1e-4 * float(w.grad.abs().max())
        assert float((db.double().cpu() - b.grad).abs().max()) <= 1e-4 * float(b.grad.abs().max())
        runs.append((dw.cpu(), db.cpu()))
    # the partial sums are added in a fixed order: the same bits on every run
    assert torch.equal(runs[1][0], runs[2][0]) and torch.equal(runs[1][1], runs[2][1])


@pytest.mark.parametrize("B,Z,Y,X,C", [(2, 4, 6, 8, 16), (1, 2, 4, 130, 64), (1, 2, 2, 6, 128), (3, 2, 4, 2, 32)])
def test_pool_upsample_and_their_adjoints(env, B, Z, Y, X, C):
    torch, _flf = env
    g = torch.Generator().manual_seed(5 + C)
    x = torch.randn((B, Z, Y, X, C), generator=g).bfloat16()
    p = torch.empty((B, Z // 2, Y // 2, X // 2, C), dtype=torch.bfloat16, device="cuda")
    _flf.pool2(x.cuda(), p)
    ref = x.double().reshape(B, Z // 2, 2, Y // 2, 2, X // 2, 2, C).mean(dim=(2, 4, 6))
    _close(torch, p, ref)
    low = torch.randn((B, Z // 2, Y // 2, X // 2, C), generator=g).bfloat16()
    skip = torch.randn((B, Z, Y, X, C), generator=g).bfloat16()
    up = torch.empty((B, Z, Y, X, C), dtype=torch.bfloat16, device="cuda")
    _flf.up2_add(low.cuda(), skip.cuda(), up)
    upr = low.double().repeat_interleave(2, 1).repeat_interleave(2, 2).repeat_interleave(2, 3) + skip.double()
    _close(torch, up, upr)
    _flf.up2_add(low.cuda(), None, up)   # without the skip term
    _close(torch, up, upr - skip.double())
    # adjoints: <pool(x), q> = <x, pool^T(q)>, <up(l), u> = <l, up^T(u)>, with masks
    gp = torch.empty((B, Z, Y, X, C), dtype=torch.bfloat16, device="cuda")
    act = torch.randn((B, Z, Y, X, C), generator=g).bfloat16()
    _flf.pool2_bwd(low.cuda(), skip.cuda(), act.cuda(), gp)
    refp = (low.double().repeat_interleave(2, 1).repeat_interleave(2, 2).repeat_interleave(2, 3) / 8 +
            skip.double()) * (act.double() > 0)
    _close(torch, gp, refp)
    gl = torch.empty((B, Z // 2, Y // 2, X // 2, C), dtype=torch.bfloat16, device="cuda")
    actl = torch.randn((B, Z // 2, Y // 2, X // 2, C), generator=g).bfloat16()
    _flf.up2_bwd(skip.cuda(), actl.cuda(), gl)
    refl = skip.double().reshape(B, Z // 2, 2, Y // 2, 2, X // 2, 2, C).sum(dim=(2, 4, 6)) * (actl.double() > 0)
    _close(torch, gl, refl)


def test_mse_adam_and_blobs(env):
    torch, _flf = env
    g = torch.Generator().manual_seed(7)
    M, C = 1000, 16
    y = torch.randn((M, C), generator=g).bfloat16()
    t = torch.randn(M, generator=g)
    gr = torch.empty((M, C), dtype=torch.bfloat16, device="cuda")
    loss = torch.zeros(1, device="cuda")
    _flf.mse_grad(y.cuda(), t.cuda(), gr, loss)
    d = y[:, 0].double() - t.double()
    assert abs(float(loss) - float((d ** 2).mean())) <= 1e-5 * float((d ** 2).mean())
    _close(torch, gr[:, 0], 2 * d / M)
    assert float(gr[:, 1:].abs().max()) == 0
    w = torch.randn(500, generator=g)
    gw = torch.randn(500, generator=g)
    wd, m, v = w.clone().cuda(), torch.zeros(500, device="cuda"), torch.zeros(500, device="cuda")
    wb = torch.empty(500, dtype=torch.bfloat16, device="cuda")
    _flf.adam(wd, gw.cuda(), m, v, wb, 1e-2, 0.9, 0.999, 1e-8, 0.1, 0.001, 0.0)
    mr, vr = 0.1 * gw, 0.001 * gw * gw
    wr = w - 1e-2 * (mr / 0.1) / ((vr / 0.001).sqrt() + 1e-8)
    assert float((wd.cpu() - wr).abs().max()) < 1e-6
    assert float((wb.float().cpu() - wr).abs().max()) < 1e-2
    vol = torch.zeros((6, 20, 30), device="cuda")
    pts = torch.tensor([[2.0, 10.0, 12.5, 3.0], [0.2, 0.0, 29.0, 1.0]], device="cuda")
    _flf.render_blobs(vol, pts, 1.0)
    zz, yy, xx = np.meshgrid(np.arange(6), np.arange(20), np.arange(30), indexing="ij")
    ref = np.zeros((6, 20, 30))
    for z0, y0, x0, a in pts.cpu().numpy():
        cz, cy, cx = np.floor(np.array([z0, y0, x0]) + 0.5)
        near = (np.abs(zz - cz) <= 3) & (np.abs(yy - cy) <= 3) & (np.abs(xx - cx) <= 3)
        ref += near * a * np.exp(-((zz - z0) ** 2 + (yy - y0) ** 2 + (xx - x0) ** 2) / 2)
    assert np.max(np.abs(vol.cpu().numpy() - ref)) < 1e-5
    # fixed-point accumulation: the same volume, bit for bit on every run
    acc = torch.empty(6 * 20 * 30, dtype=torch.int64, device="cuda")
    outs = []
    for _ in range(2):
        v2 = torch.zeros((6, 20, 30), device="cuda")
        _flf.render_blobs(v2, pts, 1.0, acc=acc)
        assert np.max(np.abs(v2.cpu().numpy() - ref)) < 1e-5
        outs.append(v2.cpu())
    assert torch.equal(outs[0], outs[1])


@pytest.mark.parametrize("rows", [0, -1, 1, 4, 5])
@pytest.mark.parametrize("shape,relu,masked", [((1, 2, 3, 5), True, False), ((2, 3, 4, 130), False, False),
                                               ((1, 4, 9, 300), True, True), ((2, 5, 6, 128), True, False)])
def test_conv3d_tcgen05(env, shape, relu, masked, rows):
    """The 16 -> 16 convolution on the tcgen05 tensor cores (TMEM accumulator);
    rows = 0 is the warp-specialised kernel with TMA-staged slabs, -1 the same
    with 32-byte swizzled slabs."""
    torch, _flf = env
    g = torch.Generator().manual_seed(sum(shape))
    x = torch.randn(shape + (16,), generator=g).bfloat16()
    w = (torch.randn((27, 16, 16), generator=g) / np.sqrt(27 * 16)).bfloat16()
    b = torch.randn(16, generator=g).float()
    m = torch.randn(shape + (16,), generator=g).bfloat16() if masked else None
    y = torch.empty(shape + (16,), dtype=torch.bfloat16, device="cuda")
    _flf.conv3d_tc(x.cuda(), w.cuda(), b.cuda(), y, relu=relu, mask=m.cuda() if masked else None, rows=rows)
    torch.cuda.synchronize()
    _flf.net_status()
    ref = _ref_conv(torch, x.double(), w.double(), b.double())
    if relu:
        ref = ref.clamp_min(0)
    if masked:
        ref = ref * (m.double() > 0)
    _close(torch, y, ref)


@pytest.mark.parametrize("rows", [0, -1])
@pytest.mark.parametrize("shape,relu,masked", [((1, 6, 200, 700), True, True), ((3, 9, 10, 130), False, False),
                                               ((1, 1, 1, 1), True, False)])
def test_conv3d_tcgen05_warp_specialised_many_items(env, shape, relu, masked, rows):
    """More work items than SMs (each CTA walks several columns through its slab
    ring), z split into chunks, and a single voxel."""
    torch, _flf = env
    g = torch.Generator().manual_seed(shape[2])
    x = torch.randn(shape + (16,), generator=g).bfloat16()
    w = (torch.randn((27, 16, 16), generator=g) / np.sqrt(27 * 16)).bfloat16()
    b = torch.randn(16, generator=g).float()
    m = torch.randn(shape + (16,), generator=g).bfloat16() if masked else None
    y = torch.empty(shape + (16,), dtype=torch.bfloat16, device="cuda")
    _flf.conv3d_tc(x.cuda(), w.cuda(), b.cuda(), y, relu=relu, mask=m.cuda() if masked else None, rows=rows)
    torch.cuda.synchronize()
    _flf.net_status()
    ref = _ref_conv(torch, x.double(), w.double(), b.double())
    if relu:
        ref = ref.clamp_min(0)
    if masked:
        ref = ref * (m.double() > 0)
    _close(torch, y, ref)


@pytest.mark.parametrize("ci,co", [(16, 16), (16, 32), (32, 16), (32, 32)])
@pytest.mark.parametrize("shape", [(2, 4, 6, 10), (1, 5, 17, 260), (1, 6, 40, 300)])
def test_conv3d_dispatch_to_tcgen05(env, shape, ci, co):
    """flf_conv3d routes 16 / 32 -> 16 / 32 channels to the tcgen05 kernel when
    selected; the result agrees with float64 and with the mma.sync kernels to the
    BF16 rounding of the output (the largest shape has more work items than SMs)."""
    torch, _flf = env
    g = torch.Generator().manual_seed(17 + ci + co)
    x = torch.randn(shape + (ci,), generator=g).bfloat16().cuda()
    w = (torch.randn((27, ci, co), generator=g) / np.sqrt(27 * ci)).bfloat16().cuda()
    b = torch.randn(co, generator=g).float().cuda()
    out = {}
    for on in (False, True):
        old = _flf.conv16_tcgen05(on)
        try:
            y = torch.empty(shape + (co,), dtype=torch.bfloat16, device="cuda")
            _flf.conv3d(x, w, b, y, relu=True)
            torch.cuda.synchronize()
            _flf.net_status()
            out[on] = y
        finally:
            _flf.conv16_tcgen05(old)
    ref = _ref_conv(torch, x.double().cpu(), w.double().cpu(), b.double().cpu()).clamp_min(0)
    _close(torch, out[True], ref)
    assert float((out[True].float() - out[False].float()).abs().max()) <= 1e-2 * float(ref.abs().max())


@pytest.mark.parametrize("ci,co", [(16, 16), (16, 32), (32, 16), (32, 32)])
@pytest.mark.parametrize("shape", [(4, 24, 128, 128), (4, 12, 64, 64)])
def test_conv3d_tcgen05_training_shapes(env, shape, ci, co):
    """The network's training batches (4 crops of 24 x 128 x 128 and their level-1
    halves) with a gradient mask: every work item of every CTA agrees with the
    mma.sync kernels to the BF16 rounding of the output."""
    torch, _flf = env
    g = torch.Generator(device="cuda").manual_seed(ci * 3 + co + shape[1])
    x = torch.randn(shape + (ci,), generator=g, device="cuda").bfloat16()
    w = (torch.randn((27, ci, co), generator=g, device="cuda") / np.sqrt(27 * ci)).bfloat16()
    m = torch.randn(shape + (co,), generator=g, device="cuda").bfloat16()
    out = {}
    for on in (False, True):
        old = _flf.conv16_tcgen05(on)
        try:
            y = torch.full(shape + (co,), float("nan"), dtype=torch.bfloat16, device="cuda")
            _flf.conv3d(x, w, None, y, mask=m)
            torch.cuda.synchronize()
            _flf.net_status()
            out[on] = y.float()
        finally:
            _flf.conv16_tcgen05(old)
    assert bool(torch.isfinite(out[True]).all())
    err = (out[True] - out[False]).abs()
    lim = 1e-2 * out[False].abs() + 1e-3 * float(out[False].abs().max())
    assert bool((err <= lim).all()), (float(err.max()), int((err > lim).sum()))


@pytest.mark.parametrize("ci,co", [(16, 32), (32, 16), (32, 32)])
def test_conv3d_tcgen05_inference_level1_shape(env, ci, co):
    """The network's level-1 layers at inference size (12 x 228 x 228: a partial
    second x segment, three or more items per CTA) with bias and ReLU: the tcgen05
    kernels agree with the mma.sync kernels to the BF16 rounding of the output."""
    torch, _flf = env
    shape = (1, 12, 228, 228)
    g = torch.Generator(device="cuda").manual_seed(ci + 2 * co)
    x = torch.randn(shape + (ci,), generator=g, device="cuda").bfloat16()
    w = (torch.randn((27, ci, co), generator=g, device="cuda") / np.sqrt(27 * ci)).bfloat16()
    b = torch.randn(co, generator=g, device="cuda")
    out = {}
    for mode in (0, 2):
        old = _flf.conv16_tcgen05(mode)
        try:
            y = torch.full(shape + (co,), float("nan"), dtype=torch.bfloat16, device="cuda")
            _flf.conv3d(x, w, b, y, relu=True)
            torch.cuda.synchronize()
            _flf.net_status()
            out[mode] = y.float()
        finally:
            _flf.conv16_tcgen05(old)
    assert bool(torch.isfinite(out[2]).all())
    err = (out[2] - out[0]).abs()
    lim = 1e-2 * out[0].abs() + 1e-3 * float(out[0].abs().max())
    assert bool((err <= lim).all()), (float(err.max()), int((err > lim).sum()))


@pytest.mark.parametrize("shape", [(2, 4, 6, 10), (1, 2, 2, 2), (1, 6, 8, 140), (1, 10, 12, 258), (4, 24, 128, 128),
                                   (1, 14, 40, 456)])
@pytest.mark.parametrize("mode", [0, 2])
@pytest.mark.parametrize("relu", [False, True])
def test_conv3d_pool(env, shape, mode, relu):
    """flf_conv3d_pool (the convolution with the 2x2x2 average pooling of its output
    summed in the epilogue) gives the same bits as flf_conv3d followed by flf_pool2, for
    one to several plane pairs per item, ragged x segments and the training crops."""
    torch, _flf = env
    B, Z, Y, X = shape
    g = torch.Generator(device="cuda").manual_seed(B + 3 * Z + Y + X)
    x = torch.randn(shape + (16,), generator=g, device="cuda").bfloat16()
    w = (torch.randn((27, 16, 16), generator=g, device="cuda") / 12).bfloat16()
    b = torch.randn(16, generator=g, device="cuda")
    old = _flf.conv16_tcgen05(mode)
    try:
        ref = torch.full_like(x, float("nan"))
        _flf.conv3d(x, w, b, ref, relu=relu)
        pref = torch.full((B, Z // 2, Y // 2, X // 2, 16), float("nan"), dtype=torch.bfloat16, device="cuda")
        _flf.pool2(ref, pref)
        y = torch.full_like(x, float("nan"))
        pooled = torch.full_like(pref, float("nan"))
        _flf.conv3d_pool(x, w, b, y, pooled, relu=relu)
        torch.cuda.synchronize()
        _flf.net_status()
    finally:
        _flf.conv16_tcgen05(old)
    assert bool(torch.isfinite(pref).all())
    assert torch.equal(y, ref)
    assert torch.equal(pooled, pref)


@pytest.mark.parametrize("shape", [(1, 4, 6, 130), (2, 3, 9, 20), (1, 24, 40, 456)])
@pytest.mark.parametrize("mode", [0, 2])
def test_conv3d_x1(env, shape, mode):
    """flf_conv3d_x1 (the first layer: a 3x3x1 convolution over the taps dx = 1) against
    float64 conv3d with the other taps zero; the tcgen05 kernel ignores them, the
    mma.sync kernel computes the full sum."""
    torch, _flf = env
    g = torch.Generator().manual_seed(sum(shape))
    x = torch.randn(shape + (16,), generator=g).bfloat16()
    w = (torch.randn((27, 16, 16), generator=g) / 12).bfloat16()
    off = [t for t in range(27) if t % 3 != 1]
    w0 = w.clone()
    w0[off] = 0
    b = torch.randn(16, generator=g).float()
    ref = _ref_conv(torch, x.double(), w0.double(), b.double()).clamp_min(0)
    y = torch.empty(shape + (16,), dtype=torch.bfloat16, device="cuda")
    old = _flf.conv16_tcgen05(mode)
    try:
        _flf.conv3d_x1(x.cuda(), (w if mode else w0).cuda(), b.cuda(), y, relu=True)
    finally:
        _flf.conv16_tcgen05(old)
    _close(torch, y, ref)
    torch.cuda.synchronize()
    _flf.net_status()
