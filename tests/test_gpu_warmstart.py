"""The learned warm start: the whole network's gradients against a torch CPU
float64 restatement, training, and RL from the warm start.

Gradient check: the device network keeps activations and activation
gradients in BF16.  The float64 restatement does the same: every activation
is rounded to BF16 in the forward pass and its gradient is rounded to BF16 in
the backward pass (the tensors the device kernels write), with everything else
in float64.  What is left is the device's FP32 accumulation order, so each
parameter gradient must agree in direction (cosine >= 0.998) and to 2 % in
norm (the coarsest levels sum over few voxels, where one BF16 rounding that
falls the other way moves a gradient most).
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env(built_lib):
    import torch
    import warmstart
    return torch, warmstart


def _bf16_round(torch):
    """Identity that rounds its value to BF16 going forward and its gradient to
    BF16 going back: the activations and activation gradients the device keeps."""

    class R(torch.autograd.Function):
        @staticmethod
        def forward(ctx, t):
            return t.to(torch.bfloat16).double()

        @staticmethod
        def backward(ctx, g):
            return g.to(torch.bfloat16).double()

    return R.apply


def _reference_forward(torch, ws_mod, net, x):
    """The network in float64 on the CPU with the device network's BF16 weights,
    with BF16 rounding of every activation and activation gradient."""
    F = torch.nn.functional
    R = _bf16_round(torch)
    P = {n: (q["wb"].double().cpu().requires_grad_(), q["b"].double().cpu().requires_grad_())
         for n, q in net.p.items()}

    def conv(name, t, relu):
        w, b = P[name]
        ci, co = w.shape[1], w.shape[2]
        y = F.conv3d(t, w.reshape(3, 3, 3, ci, co).permute(4, 3, 0, 1, 2), b, padding=1)
        return R(F.relu(y) if relu else y)

    def up(t):
        return t.repeat_interleave(2, 2).repeat_interleave(2, 3).repeat_interleave(2, 4)

    def pool(t):
        return R(F.avg_pool3d(t, 2))

    t = R(x.double().cpu().permute(0, 4, 1, 2, 3))
    e0 = conv("e0b", conv("e0a", t, True), True)
    e1 = conv("e1b", conv("e1a", pool(e0), True), True)
    e2 = conv("e2b", conv("e2a", pool(e1), True), True)
    e3 = conv("e3b", conv("e3a", pool(e2), True), True)
    d2 = conv("d2", R(up(conv("u2", e3, True)) + e2), True)
    d1 = conv("d1", R(up(conv("u1", d2, True)) + e1), True)
    d0 = conv("d0", R(up(conv("u0", d1, True)) + e0), True)
    out = conv("head", d0, False)
    return out.permute(0, 2, 3, 4, 1), P


@pytest.mark.parametrize("tcgen05", [False, True])
def test_network_gradients_match_float64(env, tcgen05):
    torch, ws_mod = env
    import _flf
    old = _flf.conv16_tcgen05(tcgen05)
    try:
        _gradients_match(torch, ws_mod)
    finally:
        _flf.conv16_tcgen05(old)


def _gradients_match(torch, ws_mod):
    net = ws_mod.UNet3D(seed=3)
    g = torch.Generator().manual_seed(0)
    x = torch.zeros((2, 8, 16, 24, ws_mod.CIN))
    x[..., :3] = torch.rand((2, 8, 16, 24, 3), generator=g)
    x = x.bfloat16()
    target = torch.rand((2, 8, 16, 24), generator=g)
    out, cache = net.forward(x.cuda())
    ref, P = _reference_forward(torch, ws_mod, net, x)
    # outputs differ only where FP32 and FP64 sums round to neighbouring BF16 values
    assert float((out.double().cpu() - ref.detach()).abs().max()) <= 0.02 * float(ref.detach().abs().max())
    dout = torch.empty_like(out)
    loss = torch.zeros(1, device="cuda")
    import _flf
    _flf.mse_grad(out, target.cuda(), dout, loss)
    R = _bf16_round(torch)
    ((R(ref[..., 0]) - target.double()) ** 2).mean().backward()
    net.backward(cache, dout)
    worst = []
    for name, q in net.p.items():
        for key, gref in (("gw", P[name][0].grad), ("gb", P[name][1].grad)):
            gd = q[key].double().cpu()
            if name == "head" and key == "gw":
                gd, gref = gd[:, :, 0], gref[:, :, 0]
            if name == "head" and key == "gb":
                gd, gref = gd[:1], gref[:1]
            nr = float(gref.norm())
            if nr == 0:
                continue
            cos = float((gd * gref).sum() / (gd.norm() * gref.norm() + 1e-300))
            worst.append((1 - cos, abs(float(gd.norm()) - nr) / nr, name, key))
    wc = max(worst)
    wn = max(worst, key=lambda w: w[1])
    print("largest 1 - cosine %.2e (%s %s), largest norm difference %.2e (%s %s)"
          % (wc[0], wc[2], wc[3], wn[1], wn[2], wn[3]))
    assert wc[0] <= 2e-3, wc
    assert wn[1] <= 0.02, wn


def test_training_and_warm_started_rl(env):
    torch, ws_mod = env
    import projector
    import psfmatrix
    import synthetic
    N = 5
    H, Ht = synthetic.synthetic_psf(N, np.arange(-4, 5, 2), 3)
    hm = psfmatrix.HMatrixArrays(H, Ht)
    p = projector.Projector_gb300()
    Y = X = 60
    ws = ws_mod.WarmStart(p, hm, Y, X, beads=30)
    ws.train(steps=150, batch=2, crop=32, volumes_per_refresh=4, refresh_every=10, target_iters=16, log_every=10)
    first = np.mean([l for _, l in ws.losses[:2]])
    last = np.mean([l for _, l in ws.losses[-3:]])
    assert last < first
    rng = np.random.default_rng(99)
    truth, img, htf = ws.make_batch(2, rng)
    x0 = ws.initial_volume(htf)
    assert x0.shape == htf.shape and bool(torch.isfinite(x0).all()) and float(x0.min()) > 0
    s = torch.cuda.current_stream().cuda_stream

    def resid(x):
        hx = torch.empty_like(img)
        ws.ctx.forward(x, hx, 2, Y, X, None, stream=s)
        return float(torch.linalg.vector_norm(img.double() - hx.double()) / torch.linalg.vector_norm(img.double()))

    # what the network gains: RL from its start volume reaches the data-fit
    # residual of 8 plain-RL iterations from a uniform volume in fewer iterations
    xu = torch.ones_like(htf)
    p.RichardsonLucy(hm, xu, htf, 8)
    r_plain = resid(xu)
    xw = ws.initial_volume(htf)
    need = None
    for k in range(9):
        if k:
            p.RichardsonLucy(hm, xw, htf, 1)
        if resid(xw) <= r_plain:
            need = k
            break
    print("plain RL-8 residual %.5f; warm start reaches it after %s RL iterations" % (r_plain, need))
    assert need is not None and need < 8, need


def test_training_repeats_bit_for_bit(env):
    """No reduction of training uses floating-point atomics (weight and bias
    gradients add their partial sums in a fixed order, the training volumes are
    rendered with fixed-point sums), so two runs with the same seeds give the
    same weights, bit for bit."""
    torch, ws_mod = env
    import projector
    import psfmatrix
    import synthetic
    N = 5
    H, Ht = synthetic.synthetic_psf(N, np.arange(-4, 5, 2), 3)
    hm = psfmatrix.HMatrixArrays(H, Ht)
    runs = []
    for _ in range(2):
        p = projector.Projector_gb300()
        ws = ws_mod.WarmStart(p, hm, 60, 60, beads=30, filaments=2)
        ws.train(steps=30, batch=2, crop=32, volumes_per_refresh=4, refresh_every=10, target_iters=4)
        runs.append({k: v.copy() for k, v in ws.net.state_dict().items()})
    assert runs[0].keys() == runs[1].keys()
    for k in runs[0]:
        assert np.array_equal(runs[0][k], runs[1][k]), k


def test_warm_start_graph_matches_direct(env):
    """WarmStartGraph (back projection, network, head and RL iterations as one CUDA
    graph) gives the direct launches' volume bit for bit; a graph whose context
    buffers were freed refuses to replay, and DeconvRLWarm(graph=True) captures
    again."""
    torch, ws_mod = env
    import _flf
    import projector
    import psfmatrix
    import synthetic
    N = 5
    H, Ht = synthetic.synthetic_psf(N, np.arange(-4, 5, 2), 3)
    hm = psfmatrix.HMatrixArrays(H, Ht)
    p = projector.Projector_gb300()
    ws = ws_mod.WarmStart(p, hm, 60, 60, beads=30)
    _, img, _ = ws.make_batch(2, np.random.default_rng(3))
    direct = ws_mod.DeconvRLWarm(ws, img, 2).clone()
    g = ws_mod.WarmStartGraph(ws, 2, 2)
    assert torch.equal(g.replay(img), direct)
    out = torch.empty(tuple(direct.shape), dtype=torch.float32, pin_memory=True).numpy()
    r = ws_mod.DeconvRLWarm(ws, img.cpu().numpy(), 2, out=out, graph=True)
    assert r is out and np.array_equal(out, direct.cpu().numpy())
    ws.ctx.clear_cache()
    with pytest.raises(_flf.FlfError, match="FLF_E_STATE"):
        g.replay(img)
    again = ws_mod.DeconvRLWarm(ws, img, 2, graph=True)
    assert torch.equal(again, direct)


@pytest.mark.parametrize("tcgen05", [False, True])
def test_fused_input_and_head_kernels(env, tcgen05):
    """flf_ws_input / flf_ws_head against their torch formulas (head on the
    mma.sync and on the warp-specialised tcgen05 kernel)."""
    torch, ws_mod = env
    import _flf
    old = _flf.conv16_tcgen05(tcgen05)
    try:
        _input_and_head(torch, _flf)
        torch.cuda.synchronize()
        _flf.net_status()
    finally:
        _flf.conv16_tcgen05(old)


def _input_and_head(torch, _flf):
    g = torch.Generator().manual_seed(11)
    Z, T, Y, X = 5, 2, 13, 21
    Zp, Yp, Xp = 8, 16, 24
    htf = (torch.rand((Z, T, Y, X), generator=g) + 0.5).cuda()
    hth1 = (torch.rand((Z, 1, Y, X), generator=g) + 0.2).cuda()
    ht1 = (torch.rand((Z, 1, Y, X), generator=g) + 0.2).cuda()
    c2, c3 = 1.0 / float(hth1.mean()), 1.0 / float(ht1.mean())
    out = torch.empty((T, Zp, Yp, Xp, 16), dtype=torch.bfloat16, device="cuda")
    sums = torch.empty(T, device="cuda")
    _flf.ws_input(htf, hth1, ht1, sums, out, c2, c3)
    x1 = htf / hth1
    m = x1.reshape(Z, T, -1).mean(dim=(0, 2))
    assert float((sums / (Z * Y * X) - m).abs().max()) <= 1e-5 * float(m.abs().max())
    feat = torch.zeros((T, Zp, Yp, Xp + 2, 4), device="cuda")   # the features, one zero column each side
    feat[:, :Z, :Y, 1:X + 1, 0] = (x1 / m[None, :, None, None]).permute(1, 0, 2, 3)
    feat[:, :Z, :Y, 1:X + 1, 1] = (htf / ht1 / m[None, :, None, None]).permute(1, 0, 2, 3)
    feat[:, :Z, :Y, 1:X + 1, 2] = (hth1 * c2).expand(Z, T, Y, X).permute(1, 0, 2, 3)
    feat[:, :Z, :Y, 1:X + 1, 3] = (ht1 * c3).expand(Z, T, Y, X).permute(1, 0, 2, 3)
    ref = torch.zeros((T, Zp, Yp, Xp, 16), device="cuda")
    for k in range(3):   # channel 4k + j holds feature j at x + k - 1
        ref[..., 4 * k:4 * k + 4] = feat[:, :, :, k:k + Xp]
    assert float((out.float() - ref).abs().max()) <= 1e-2 * float(ref.abs().max())
    d = torch.rand((T, Zp, Yp, Xp, 16), generator=g).bfloat16().cuda()
    wfull = torch.zeros((27, 16, 16))
    wfull[:, :, 0] = torch.randn((27, 16), generator=g) / 20
    wfull = wfull.bfloat16()
    x0 = torch.empty((Z, T, Y, X), device="cuda")
    _flf.ws_head(d, wfull.cuda(), 0.1, 1e-3, sums, x0)
    W = wfull[:, :, 0].double().reshape(3, 3, 3, 16).permute(3, 0, 1, 2)[None]
    conv = torch.nn.functional.conv3d(d.double().cpu().permute(0, 4, 1, 2, 3), W, padding=1)[:, 0] + 0.1
    want = conv.clamp_min(1e-3)[:, :Z, :Y, :X].permute(1, 0, 2, 3) * (sums.double().cpu() / (Z * Y * X))[None, :,
                                                                                                         None, None]
    assert float((x0.double().cpu() - want).abs().max()) <= 1e-4 * float(want.abs().max())
