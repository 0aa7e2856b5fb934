"""Learned warm start for Richardson-Lucy: a 3-D U-Net on the normalised back projection.

The network maps the first RL iterate ``Htf / HtH1`` (with ``Htf / Ht1`` and
the two sensitivity maps as further input channels) to an estimate of the
volume; RL then runs from
that estimate instead of from a uniform volume.  Everything runs on the
GPU with this package's own kernels (include/flf.h, csrc/flf_net.cu):
BF16 activations and weights, FP32 accumulation, FP32 master weights and Adam;
torch provides the tensors only.

Architecture (channels-last [B][Z][Y][X][C], 3x3x3 convolutions, ReLU):
four levels of 16-32-64-128 channels with two convolutions each on the way
down (2x2x2 average pooling between levels; the input carries each voxel's x
neighbours as channels, so the first convolution's x taps are channels and it
runs as a 3x3x1 convolution), and on the way up a
convolution that halves the channels at the coarse level, nearest 2x
upsampling plus the encoder feature of that level (additive skip), and one
convolution; a 16-channel head whose channel 0 is the prediction.  Volumes
are zero-padded to multiples of 8 in Z, Y and X.

Training data come from the method itself: random bead and filament volumes
(``k_render_blobs``) are forward projected with the GPU projector, a
background is added and Poisson noise drawn, and the noisy image is back
projected.  The target is the volume that plain RL reaches from a uniform
start after ``target_iters`` iterations (32 by default).  The Prevedel update
x <- x Htf / (Ht H x) sees the image only through Htf, so that volume is a
function of the network's input; RL's data-fit residual falls slowly with the
iterations (microscope images carry background the volume cannot explain
where the lenslets are dark), so a good prediction of the 32-iteration volume
sits below the 8-iteration residual without further iterations.  Input and
target are divided by the mean of the input (the Prevedel update is invariant
to the start volume's scale after its first iteration); the loss is their mean
squared error.
"""

import time

import numpy as np

import _flf

try:
    import torch
except ImportError:  # torch is needed for device arrays
    torch = None

__all__ = ["UNet3D", "WarmStart", "WarmStartGraph", "synthetic_volume_points", "DeconvRLWarm"]

CIN = 16
# (name, input channels, output channels, ReLU)
LAYERS = [("e0a", CIN, 16, True), ("e0b", 16, 16, True), ("e1a", 16, 32, True), ("e1b", 32, 32, True),
          ("e2a", 32, 64, True), ("e2b", 64, 64, True), ("e3a", 64, 128, True), ("e3b", 128, 128, True),
          ("u2", 128, 64, True), ("d2", 64, 64, True), ("u1", 64, 32, True), ("d1", 32, 32, True),
          ("u0", 32, 16, True), ("d0", 16, 16, True), ("head", 16, 16, False)]


# The first layer is a 3x3x1 convolution (flf_conv3d_x1): the network input holds
# the four features of x - 1, x and x + 1 as channels 0..11, so the layer's x taps
# are channels and only the taps with dx = 1 (the centre) are kept.  Taps are
# ordered dz*9 + dy*3 + dx.
X1_LAYER = "e0a"
_OFF_CENTRE_X = [t for t in range(27) if t % 3 != 1]


def learning_rate(step, steps, lr, warmup):
    """Training schedule: a linear ramp over the first ``warmup`` steps times a cosine
    from ``lr`` at step 0 to zero at the last of ``steps`` steps."""
    frac = step / max(steps - 1, 1)
    ramp = min(1.0, (step + 1) / warmup) if warmup > 0 else 1.0
    return lr * ramp * 0.5 * (1 + np.cos(np.pi * frac))


def _bf(shape, dev):
    return torch.empty(shape, dtype=torch.bfloat16, device=dev)


class UNet3D:
    """The warm-start network: parameters, forward, backward and Adam on the device."""

    def __init__(self, device=0, seed=0):
        if torch is None:
            raise _flf.FlfError(-4, "PyTorch is required for device arrays")
        _flf.load_library()
        self.dev = torch.device("cuda", device)
        g = torch.Generator().manual_seed(seed)
        self.p = {}
        for name, ci, co, relu in LAYERS:
            std = np.sqrt((2.0 if relu else 1.0) / (27 * ci))
            w = torch.randn((27, ci, co), generator=g) * std
            if name == "head":
                w[:, :, 1:] = 0
            if name == X1_LAYER:   # a 3x3x1 convolution: only the taps at the centre x offset
                w[_OFF_CENTRE_X] = 0
            b = torch.zeros(co)
            self.p[name] = {"w": w.to(self.dev), "b": b.to(self.dev), "ci": ci, "co": co, "relu": relu}
        self.adam_t = 0
        self.loads = 0
        self._ws = None             # split-K workspace of the convolutions
        for q in self.p.values():
            q["wb"] = _bf(q["w"].shape, self.dev)
            q["wf"] = _bf((27, q["co"], q["ci"]), self.dev)
            if max(q["ci"], q["co"]) >= 64:   # the wide layers' tcgen05 kernel reads packed weights
                q["wp"] = _bf(q["w"].shape, self.dev)
                q["wfp"] = _bf((27, q["co"], q["ci"]), self.dev)
            for k in ("gw", "mw", "vw"):
                q[k] = torch.zeros_like(q["w"])
            for k in ("gb", "mb", "vb"):
                q[k] = torch.zeros_like(q["b"])
        self._sync_weights()

    def _sync_weights(self):
        s = torch.cuda.current_stream(self.dev).cuda_stream
        for q in self.p.values():
            q["wb"].copy_(q["w"])
            self._derive(q, s)

    @staticmethod
    def _derive(q, s):
        """The flipped weights of the data gradient and, for the wide layers, both
        weight sets packed for the tcgen05 kernel, from the BF16 weights."""
        _flf.conv3d_flip(q["wb"], q["wf"], s)
        if "wp" in q:
            _flf.conv3d_pack(q["wb"], q["wp"], s)
            _flf.conv3d_pack(q["wf"], q["wfp"], s)

    def num_parameters(self):
        return int(sum(q["w"].numel() + q["b"].numel() for q in self.p.values()))

    def _conv(self, name, x, relu=None, mask=None, flip=False, out=None):
        q = self.p[name]
        co = q["ci"] if flip else q["co"]
        y = out if out is not None else _bf(tuple(x.shape[:4]) + (co,), self.dev)
        if relu is None:
            relu = q["relu"] and not flip       # a data gradient is linear
        if name == X1_LAYER and not flip and mask is None:
            _flf.conv3d_x1(x, q["wb"], q["b"], y, relu=relu, stream=torch.cuda.current_stream(self.dev).cuda_stream)
            return y
        # split-K layers (few output tiles: the coarse levels) write one slice per split
        need = y.numel() * (4 if y.numel() < (1 << 23) else 1)
        if self._ws is None or self._ws.numel() < need:
            self._ws = torch.empty(need, dtype=torch.float32, device=self.dev)
        _flf.conv3d(x, q["wf"] if flip else q["wb"], None if flip else q["b"], y, relu=relu, mask=mask,
                    stream=torch.cuda.current_stream(self.dev).cuda_stream, ws=self._ws,
                    wp=q.get("wfp") if flip else q.get("wp"))
        return y

    def _pool(self, x):
        B, Z, Y, X, C = x.shape
        y = _bf((B, Z // 2, Y // 2, X // 2, C), self.dev)
        _flf.pool2(x, y, torch.cuda.current_stream(self.dev).cuda_stream)
        return y

    def _conv_pool(self, name, x):
        """A 16 -> 16 layer and the 2x2x2 average pooling of its output, one launch."""
        q = self.p[name]
        B, Z, Y, X, _ = x.shape
        y = _bf((B, Z, Y, X, q["co"]), self.dev)
        pooled = _bf((B, Z // 2, Y // 2, X // 2, q["co"]), self.dev)
        _flf.conv3d_pool(x, q["wb"], q["b"], y, pooled, relu=q["relu"],
                         stream=torch.cuda.current_stream(self.dev).cuda_stream)
        return y, pooled

    def _up_add(self, low, skip):
        y = _bf(tuple(skip.shape[:4]) + (low.shape[4],), self.dev)
        _flf.up2_add(low, skip, y, torch.cuda.current_stream(self.dev).cuda_stream)
        return y

    def forward(self, x, head=True):
        """x [B, Z, Y, X, 16] bf16 (Z, Y, X multiples of 8) -> (out [B, Z, Y, X, 16], cache);
        with head=False the last features d0 come back in place of out."""
        a = {"x": x}
        a["e0a"] = self._conv("e0a", x)
        a["e0b"], a["p1"] = self._conv_pool("e0b", a["e0a"])
        a["e1a"] = self._conv("e1a", a["p1"])
        a["e1b"] = self._conv("e1b", a["e1a"])
        a["p2"] = self._pool(a["e1b"])
        a["e2a"] = self._conv("e2a", a["p2"])
        a["e2b"] = self._conv("e2b", a["e2a"])
        a["p3"] = self._pool(a["e2b"])
        a["e3a"] = self._conv("e3a", a["p3"])
        a["e3b"] = self._conv("e3b", a["e3a"])
        a["u2"] = self._conv("u2", a["e3b"])
        a["s2"] = self._up_add(a["u2"], a["e2b"])
        a["d2"] = self._conv("d2", a["s2"])
        a["u1"] = self._conv("u1", a["d2"])
        a["s1"] = self._up_add(a["u1"], a["e1b"])
        a["d1"] = self._conv("d1", a["s1"])
        a["u0"] = self._conv("u0", a["d1"])
        a["s0"] = self._up_add(a["u0"], a["e0b"])
        a["d0"] = self._conv("d0", a["s0"])
        if not head:
            return a["d0"], a
        a["out"] = self._conv("head", a["d0"])
        return a["out"], a

    def _wgrad(self, name, x, g):
        q = self.p[name]
        s = torch.cuda.current_stream(self.dev).cuda_stream
        need = max(64 * q["w"].numel(), g.numel() // 2048 + q["co"])   # wgrad chunks / bias row blocks
        if self._ws is None or self._ws.numel() < need:
            self._ws = torch.empty(need, dtype=torch.float32, device=self.dev)
        _flf.conv3d_wgrad(x, g, q["gw"], s, ws=self._ws)
        _flf.bias_grad(g, q["gb"], s, ws=self._ws)

    def backward(self, a, dout):
        """Gradients of all parameters (accumulated into gw / gb) for dL/d(out) = dout."""
        s = torch.cuda.current_stream(self.dev).cuda_stream
        for q in self.p.values():
            q["gw"].zero_()
            q["gb"].zero_()
        # head (linear) and d0
        self._wgrad("head", a["d0"], dout)
        g = self._conv("head", dout, flip=True, mask=a["d0"])            # d(pre d0)
        self._wgrad("d0", a["s0"], g)
        gs0 = self._conv("d0", g, flip=True)                             # d s0
        gu0 = _bf(a["u0"].shape, self.dev)
        _flf.up2_bwd(gs0, a["u0"], gu0, s)                               # d(pre u0)
        self._wgrad("u0", a["d1"], gu0)
        g = self._conv("u0", gu0, flip=True, mask=a["d1"])               # d(pre d1)
        self._wgrad("d1", a["s1"], g)
        gs1 = self._conv("d1", g, flip=True)
        gu1 = _bf(a["u1"].shape, self.dev)
        _flf.up2_bwd(gs1, a["u1"], gu1, s)
        self._wgrad("u1", a["d2"], gu1)
        g = self._conv("u1", gu1, flip=True, mask=a["d2"])
        self._wgrad("d2", a["s2"], g)
        gs2 = self._conv("d2", g, flip=True)
        gu2 = _bf(a["u2"].shape, self.dev)
        _flf.up2_bwd(gs2, a["u2"], gu2, s)
        self._wgrad("u2", a["e3b"], gu2)
        g = self._conv("u2", gu2, flip=True, mask=a["e3b"])              # d(pre e3b)
        self._wgrad("e3b", a["e3a"], g)
        g = self._conv("e3b", g, flip=True, mask=a["e3a"])
        self._wgrad("e3a", a["p3"], g)
        gp3 = self._conv("e3a", g, flip=True)                            # d p3
        g = _bf(a["e2b"].shape, self.dev)
        _flf.pool2_bwd(gp3, gs2, a["e2b"], g, s)                         # d(pre e2b): pool path + skip
        self._wgrad("e2b", a["e2a"], g)
        g = self._conv("e2b", g, flip=True, mask=a["e2a"])
        self._wgrad("e2a", a["p2"], g)
        gp2 = self._conv("e2a", g, flip=True)
        g = _bf(a["e1b"].shape, self.dev)
        _flf.pool2_bwd(gp2, gs1, a["e1b"], g, s)
        self._wgrad("e1b", a["e1a"], g)
        g = self._conv("e1b", g, flip=True, mask=a["e1a"])
        self._wgrad("e1a", a["p1"], g)
        gp1 = self._conv("e1a", g, flip=True)
        g = _bf(a["e0b"].shape, self.dev)
        _flf.pool2_bwd(gp1, gs0, a["e0b"], g, s)
        self._wgrad("e0b", a["e0a"], g)
        g = self._conv("e0b", g, flip=True, mask=a["e0a"])
        self._wgrad("e0a", a["x"], g)

    def adam_step(self, lr, b1=0.9, b2=0.999, eps=1e-8, wd=0.0):
        self.adam_t += 1
        c1, c2 = 1 - b1 ** self.adam_t, 1 - b2 ** self.adam_t
        s = torch.cuda.current_stream(self.dev).cuda_stream
        for name, q in self.p.items():
            if name == "head":
                q["gw"][:, :, 1:] = 0
            if name == X1_LAYER:
                q["gw"][_OFF_CENTRE_X] = 0
            _flf.adam(q["w"], q["gw"], q["mw"], q["vw"], q["wb"], lr, b1, b2, eps, c1, c2, wd, s)
            _flf.adam(q["b"], q["gb"], q["mb"], q["vb"], None, lr, b1, b2, eps, c1, c2, 0.0, s)
            self._derive(q, s)

    def state_dict(self):
        return {"%s.%s" % (n, k): q[k].cpu().numpy() for n, q in self.p.items() for k in ("w", "b")}

    def load_state_dict(self, d):
        for n, q in self.p.items():
            q["w"].copy_(torch.as_tensor(d["%s.w" % n]))
            q["b"].copy_(torch.as_tensor(d["%s.b" % n]))
        self.loads += 1
        self._sync_weights()

    def save(self, path):
        np.savez(path, **self.state_dict())

    def load(self, path):
        with np.load(path) as d:
            self.load_state_dict(dict(d))


def synthetic_volume_points(shape, beads, filaments, rng, bead_amp=(500.0, 1000.0), fil_intensity=500.0,
                            fil_steps=60):
    """Blob list (z, y, x, amplitude) of a bead + filament volume: uniform bead positions
    and amplitudes, random-walk filaments drawn as a chain of unit-spaced blobs."""
    Z, Y, X = shape
    pts = [np.stack([rng.uniform(0, Z - 1, beads), rng.uniform(0, Y - 1, beads), rng.uniform(0, X - 1, beads),
                     rng.uniform(*bead_amp, beads)], axis=1)]
    for _ in range(filaments):
        p = np.array([rng.uniform(0, Z - 1), rng.uniform(0, Y - 1), rng.uniform(0, X - 1)])
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        path = []
        for _ in range(fil_steps):
            d = d + 0.3 * rng.normal(size=3)
            d /= np.linalg.norm(d)
            p = p + d
            if not (0 <= p[0] <= Z - 1 and 0 <= p[1] <= Y - 1 and 0 <= p[2] <= X - 1):
                break
            path.append(p.copy())
        if path:
            q = np.array(path)
            pts.append(np.concatenate([q, np.full((len(q), 1), fil_intensity * 0.4)], axis=1))
    return np.ascontiguousarray(np.concatenate(pts).astype(np.float32))


class WarmStart:
    """A trained (or training) warm-start network for one PSF matrix and image size.

    ``projector`` is a ``Projector_gb300``; ``hMatrix`` its PSF matrix.  Call
    ``train`` once (or ``load`` saved weights), then ``initial_volume`` gives
    the RL start for camera images of the same size.
    """

    def __init__(self, projector, hMatrix, Y, X, device=0, seed=0, background=100.0, beads=200, filaments=0,
                 sigma=1.0):
        self.proj, self.hm = projector, hMatrix
        self.Y, self.X, self.Z = int(Y), int(X), int(hMatrix.numZ)
        self.dev = torch.device("cuda", device)
        self.net = UNet3D(device, seed)
        self.background, self.beads, self.filaments, self.sigma = background, beads, filaments, sigma
        projector._prepare(self.ctx, self.Y, self.X, hMatrix)
        self.pad = tuple(-(-v // 8) * 8 for v in (self.Z, self.Y, self.X))
        ones = torch.ones((1, self.Y, self.X), device=self.dev)
        self.ht1 = torch.empty((self.Z, 1, self.Y, self.X), device=self.dev)
        self.ctx.backward(ones, self.ht1, 1, self.Y, self.X, None, stream=self._s())
        self.ht1.clamp_(min=1e-12)
        # HtH1 = Ht H 1: the first Prevedel iteration from a uniform volume is Htf / HtH1
        h1 = torch.empty((1, self.Y, self.X), device=self.dev)
        self.ctx.forward(torch.ones((self.Z, 1, self.Y, self.X), device=self.dev), h1, 1, self.Y, self.X, None,
                         stream=self._s())
        self.hth1 = torch.empty((self.Z, 1, self.Y, self.X), device=self.dev)
        self.ctx.backward(h1, self.hth1, 1, self.Y, self.X, None, stream=self._s())
        self.hth1.clamp_(min=1e-12)
        self.c2 = float(1.0 / self.hth1.mean())
        self.c3 = float(1.0 / self.ht1.mean())
        self.losses = []         # (step, loss) of train()
        self.tune_losses = []    # (step, residual loss) of finetune_residual()

    @property
    def ctx(self):
        """The projector's context for this PSF matrix (prepared for Y x X)."""
        c = self.proj.context(self.hm)
        self.proj._prepare(c, self.Y, self.X, self.hm)
        return c

    def _s(self):
        return torch.cuda.current_stream(self.dev).cuda_stream

    def _inputs(self, htf):
        """Network input (channels-last bf16, padded) and the frame sums of the first RL
        iterate, from Htf [Z, T, Y, X] (flf_ws_input).  Channels: the first RL iterate
        Htf / HtH1 and Htf / Ht1, both over the frame's mean of the first, and the
        sensitivity maps HtH1 and Ht1 over their means."""
        T = int(htf.shape[1])
        Zp, Yp, Xp = self.pad
        x = torch.empty((T, Zp, Yp, Xp, CIN), dtype=torch.bfloat16, device=self.dev)
        sums = torch.empty(T, dtype=torch.float32, device=self.dev)
        _flf.ws_input(htf.contiguous(), self.hth1, self.ht1, sums, x, self.c2, self.c3, self._s())
        return x, sums / float(self.Z * self.Y * self.X)

    def make_batch(self, T, rng):
        """T synthetic (truth [Z, T, Y, X], noisy image [T, Y, X], Htf [Z, T, Y, X])."""
        truth = torch.zeros((T, self.Z, self.Y, self.X), device=self.dev)
        acc = torch.empty(self.Z * self.Y * self.X, dtype=torch.int64, device=self.dev)
        for t in range(T):
            pts = torch.as_tensor(synthetic_volume_points((self.Z, self.Y, self.X), self.beads, self.filaments, rng),
                                  device=self.dev)
            _flf.render_blobs(truth[t], pts, self.sigma, self._s(), acc=acc)
        truth = truth.permute(1, 0, 2, 3).contiguous()
        clean = torch.empty((T, self.Y, self.X), device=self.dev)
        self.ctx.forward(truth, clean, T, self.Y, self.X, None, stream=self._s())
        gen = torch.Generator(device=self.dev).manual_seed(int(rng.integers(1 << 62)))
        img = torch.poisson((clean + self.background).clamp_min(0), generator=gen)
        htf = torch.empty((self.Z, T, self.Y, self.X), device=self.dev)
        self.ctx.backward(img, htf, T, self.Y, self.X, None, stream=self._s())
        return truth, img, htf

    def rl_target(self, htf, iters):
        """Plain RL from a uniform volume (the method the network stands in for)."""
        x = torch.ones_like(htf)
        self.proj.RichardsonLucy(self.hm, x, htf, iters)
        return x

    def train(self, steps=1500, batch=4, crop=128, volumes_per_refresh=8, refresh_every=8, lr=1e-3, seed=1,
              target_iters=32, log_every=0, kernels=None, warmup=None):
        """Train on crops of freshly generated synthetic volumes; returns seconds taken.

        The learning rate rises linearly over the first ``warmup`` steps (default
        steps / 16) and then follows a cosine from ``lr`` to zero over all
        ``steps``.  Without the ramp, Adam's first full-size steps drive the loss
        up by two orders of magnitude and leave most ReLUs dead, on a plateau of
        about the target's variance.

        kernels selects the 16 / 32-channel convolution kernels used while training
        (forward and data gradients; a mode of _flf.conv16_tcgen05), None keeps the
        library's current choice."""
        if warmup is None:
            warmup = steps // 16
        old = _flf.conv16_tcgen05(kernels) if kernels is not None else None
        try:
            return self._train(steps, batch, crop, volumes_per_refresh, refresh_every, lr, seed, target_iters,
                               log_every, warmup)
        finally:
            if old is not None:
                _flf.conv16_tcgen05(old)

    def _train(self, steps, batch, crop, volumes_per_refresh, refresh_every, lr, seed, target_iters, log_every,
               warmup):
        rng = np.random.default_rng(seed)
        t0 = time.time()
        cy, cx = min(crop, self.pad[1]), min(crop, self.pad[2])
        pool = None
        for step in range(steps):
            if step % refresh_every == 0:
                _, _, htf = self.make_batch(volumes_per_refresh, rng)
                xin, scale = self._inputs(htf)
                ref = self.rl_target(htf, target_iters)
                Zp, Yp, Xp = self.pad
                tgt = torch.zeros((volumes_per_refresh, Zp, Yp, Xp), device=self.dev)
                tgt[:, :self.Z, :self.Y, :self.X] = (ref / scale[None, :, None, None]).permute(1, 0, 2, 3)
                pool = (xin, tgt)
            idx = rng.integers(0, pool[0].shape[0], batch)
            ys = rng.integers(0, self.pad[1] - cy + 1, batch) // 8 * 8
            xs = rng.integers(0, self.pad[2] - cx + 1, batch) // 8 * 8
            xb = torch.stack([pool[0][i, :, y:y + cy, x:x + cx] for i, y, x in zip(idx, ys, xs)]).contiguous()
            tb = torch.stack([pool[1][i, :, y:y + cy, x:x + cx] for i, y, x in zip(idx, ys, xs)]).contiguous()
            out, cache = self.net.forward(xb)
            dout = torch.empty_like(out)
            loss = torch.zeros(1, device=self.dev)
            _flf.mse_grad(out, tb, dout, loss, self._s())
            self.net.backward(cache, dout)
            self.net.adam_step(learning_rate(step, steps, lr, warmup))
            if log_every and (step % log_every == 0 or step == steps - 1):
                self.losses.append((step, float(loss)))
        torch.cuda.synchronize(self.dev)
        _flf.net_status()   # raise if a bounded wait in a tensor-core convolution gave up
        return time.time() - t0

    def finetune_residual(self, steps=200, lr=1e-4, frames=1, seed=7, floor=1e-3, log_every=0):
        """Fine-tune on the data-fit residual itself, on whole volumes: loss =
        ||y - H x0||^2 / ||y||^2 for the start volume x0 the network gives, with the
        gradient 2 Ht(H x0 - y) / ||y||^2 from the GPU projector."""
        rng = np.random.default_rng(seed)
        t0 = time.time()
        Z, Y, X = self.Z, self.Y, self.X
        s = self._s()
        for step in range(steps):
            _, img, htf = self.make_batch(frames, rng)
            xin, scale = self._inputs(htf)
            out, cache = self.net.forward(xin)
            pred = out[:, :Z, :Y, :X, 0].float()                            # [T, Z, Y, X]
            sc = scale[:, None, None, None]
            x0 = (pred.clamp_min(floor) * sc).permute(1, 0, 2, 3).contiguous()
            hx = torch.empty_like(img)
            self.ctx.forward(x0, hx, frames, Y, X, None, stream=s)
            r = hx - img
            ny = (img.double() ** 2).sum()
            loss = float((r.double() ** 2).sum() / ny)
            gx = torch.empty_like(htf)
            self.ctx.backward((r * float(2.0 / ny)).contiguous(), gx, frames, Y, X, None, stream=s)
            gp = gx.permute(1, 0, 2, 3) * sc * (pred > floor)
            dout = torch.zeros_like(out)
            dout[:, :Z, :Y, :X, 0] = gp.to(torch.bfloat16)
            self.net.backward(cache, dout)
            self.net.adam_step(lr)
            if log_every and (step % log_every == 0 or step == steps - 1):
                self.tune_losses.append((step, loss))
            del cache, out
        torch.cuda.synchronize(self.dev)
        _flf.net_status()   # raise if a bounded wait in a tensor-core convolution gave up
        return time.time() - t0

    def initial_volume(self, htf, floor=1e-3):
        """RL start volume [Z, T, Y, X] from Htf [Z, T, Y, X] (device): the network's
        prediction, clamped below at floor x the frame mean of the first RL iterate (RL
        keeps zeros at zero), written by the head kernel (flf_ws_head)."""
        htf = htf.contiguous()
        T = int(htf.shape[1])
        Zp, Yp, Xp = self.pad
        xin = torch.empty((T, Zp, Yp, Xp, CIN), dtype=torch.bfloat16, device=self.dev)
        sums = torch.empty(T, dtype=torch.float32, device=self.dev)
        _flf.ws_input(htf, self.hth1, self.ht1, sums, xin, self.c2, self.c3, self._s())
        feats, _ = self.net.forward(xin, head=False)
        key = (self.net.adam_t, self.net.loads)
        if getattr(self, "_head_key", None) != key:
            q = self.net.p["head"]
            self._head = (q["wb"], float(q["b"][0]))
            self._head_key = key
        x0 = torch.empty_like(htf)
        _flf.ws_head(feats, self._head[0], self._head[1], floor, sums, x0, self._s())
        return x0


    def save(self, path):
        """Network weights plus the image size and plane count they were trained for."""
        d = self.net.state_dict()
        d["meta.shape"] = np.array([self.Z, self.Y, self.X], np.int64)
        d["meta.nnum"] = np.array([self.hm.Nnum], np.int64)
        np.savez(path, **d)

    def load(self, path):
        """Weights saved by save(); the image size and plane count must match."""
        with np.load(path) as f:
            d = dict(f)
        shape = tuple(int(v) for v in d.pop("meta.shape", np.array([self.Z, self.Y, self.X])))
        nnum = int(d.pop("meta.nnum", np.array([self.hm.Nnum]))[0])
        if shape != (self.Z, self.Y, self.X) or nnum != self.hm.Nnum:
            raise ValueError("%s was trained for %d planes of %d x %d px at Nnum %d, not %d planes of %d x %d at %d"
                             % (path, shape[0], shape[1], shape[2], nnum, self.Z, self.Y, self.X, self.hm.Nnum))
        self.net.load_state_dict(d)
        return self

    @staticmethod
    def trained_shape(path):
        """(Z, Y, X) a saved network was trained for."""
        with np.load(path) as f:
            return tuple(int(v) for v in f["meta.shape"])


class WarmStartGraph:
    """The whole warm-started deconvolution of T frames of the trained size as one
    CUDA graph: back projection, network input, network, head and ``maxIter`` RL
    iterations, on static device buffers (``img`` [T, Y, X] in, ``x`` [Z, T, Y, X]
    out).  One direct run first sizes every workspace and builds the transfer
    matrices; the capture then records the same launches (the RL iterations as
    direct launches, not as a nested graph).  ``replay`` copies a new image in
    (host or device), replays, and copies the volume to ``out`` when given."""

    def __init__(self, warm, T, maxIter=0, prevedel=True):
        self.warm, self.T, self.maxIter, self.prevedel = warm, int(T), int(maxIter), bool(prevedel)
        p = warm.proj
        self.img = torch.zeros((self.T, warm.Y, warm.X), dtype=torch.float32, device=warm.dev)
        self.htf = torch.empty((warm.Z, self.T, warm.Y, warm.X), dtype=torch.float32, device=warm.dev)
        saved = p.useGraphs
        p.useGraphs = False
        try:
            self._run()                          # sizes workspaces, builds matrices, sets kernel attributes
            torch.cuda.synchronize(warm.dev)
            self.graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(self.graph, capture_error_mode="relaxed"):
                self.x = self._run()
        finally:
            p.useGraphs = saved
        torch.cuda.synchronize(warm.dev)
        # the graph holds the context's buffers (valid while the epoch stands) and the
        # head bias as a value (valid while the weights are those of the capture)
        self.key = (warm.ctx.memory_epoch(), warm.net.adam_t, warm.net.loads)

    def valid(self):
        w = self.warm
        return self.key == (w.ctx.memory_epoch(), w.net.adam_t, w.net.loads)

    def _run(self):
        w = self.warm
        w.ctx.backward(self.img, self.htf, self.T, w.Y, w.X, None, stream=w._s())
        x = w.initial_volume(self.htf)
        if self.maxIter > 0:
            w.proj.RichardsonLucy(w.hm, x, self.htf if self.prevedel else self.img, self.maxIter,
                                  prevedel=self.prevedel)
        return x

    def replay(self, im=None, out=None):
        """Deconvolve ``im`` ([T, Y, X], host or device; None: the image already in
        ``self.img``); returns ``self.x``, or ``out`` (a float32 host array) filled."""
        if not self.valid():
            raise _flf.FlfError(-4, "the warm-start graph refers to freed buffers or earlier weights: capture it again")
        if im is not None:
            src = im if isinstance(im, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(im, np.float32))
            self.img.copy_(src.reshape(self.img.shape))
        self.graph.replay()
        if out is not None:
            return self.warm.proj.asnumpy(self.x, out=out)
        return self.x


def DeconvRLWarm(warm, im, maxIter, prevedel=True, projector=None, out=None, graph=False):
    """RL from the network's start volume: back projection, warm start, ``maxIter``
    Prevedel iterations (the reference's default update), on the device; returns the
    volume [Z, T, Y, X] as a device tensor, or, with ``out`` (a float32 numpy array of
    that shape, e.g. a view of pinned host memory), copied into ``out``.  With
    ``graph`` the whole deconvolution replays one CUDA graph (WarmStartGraph, kept
    per frame count, iteration count and update; the returned tensor is the graph's
    own output buffer, overwritten by the next call)."""
    if graph and projector is None:
        T = int(np.shape(im)[0])
        key = (T, int(maxIter), bool(prevedel))
        cache = warm.__dict__.setdefault("_step_graphs", {})
        if key not in cache or not cache[key].valid():
            cache.pop(key, None)
            cache[key] = WarmStartGraph(warm, T, maxIter, prevedel)
        return cache[key].replay(im, out=out)
    p = projector or warm.proj
    img = p.asnative(im)
    T, Y, X = img.shape
    htf = torch.empty((warm.Z, T, Y, X), device=warm.dev)
    warm.ctx.backward(img, htf, T, Y, X, None, stream=warm._s())
    x = warm.initial_volume(htf)
    if maxIter > 0:
        p.RichardsonLucy(warm.hm, x, htf if prevedel else img, maxIter, prevedel=prevedel)
    if out is not None:
        return p.asnumpy(x, out=out)
    return x


def main(argv=None):
    """Command line: train a warm-start network for a PSF matrix and image size.

    python warmstart.py -p PSF.mat -s Y X -o net.npz [--steps N] [--beads B] [--filaments F]
    """
    import argparse
    import sys

    import projector as proj
    import psfmatrix

    ap = argparse.ArgumentParser(description="Train the learned RL warm start for one PSF matrix and image size.")
    ap.add_argument("-p", "--psf", required=True, help="PSF .mat path (its memmap folder is used when present)")
    ap.add_argument("-s", "--size", required=True, nargs=2, type=int, metavar=("Y", "X"), help="image size in pixels")
    ap.add_argument("-o", "--out", required=True, help="output .npz for the network weights")
    ap.add_argument("--steps", type=int, default=1600, help="training steps")
    ap.add_argument("--beads", type=int, default=200, help="beads per synthetic training volume")
    ap.add_argument("--filaments", type=int, default=0, help="filaments per synthetic training volume")
    ap.add_argument("--target-iters", type=int, default=32, help="plain-RL iterations the network learns to reach")
    args = ap.parse_args(sys.argv[1:] if argv is None else argv)
    hm = psfmatrix.LoadMatrix(args.psf, createPSF=True)
    p = proj.Projector_gb300()
    ws = WarmStart(p, hm, args.size[0], args.size[1], beads=args.beads, filaments=args.filaments)
    sec = ws.train(steps=args.steps, target_iters=args.target_iters)
    ws.save(args.out)
    print("trained %d steps in %.1f s -> %s" % (args.steps, sec, args.out), flush=True)
    return args.out


if __name__ == "__main__":
    main()
