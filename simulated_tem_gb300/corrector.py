"""The learned corrector: an M = 2 voxel-grid image lifted to M = 8 quality.

A four-level convolutional encoder-decoder (U-Net; 32, 64, 128, 256 channels, 3 x 3
convolutions with ReLU, 2 x 2 average pooling, nearest upsampling with skip
concatenation, a 1 x 1 head) maps four planes on the fine pixel grid -- the contrast of
the coarse dark- and bright-field images interpolated onto it (their deviation from the
image mean, scaled: the contrast is a few 1e-3 on a level of 0.1-0.7 and would not survive
BF16 otherwise), a constant s_g plane and the mean level -- to a correction, scaled by
RES_SCALE, that is added to the interpolated dark field.  Weights and activations are BF16 with
FP32 accumulation; every layer, forward and backward, and the Adam update run in
libstem_nn's kernels (tensor-core convolutions on sm_103a).  torch holds device memory.

Training pairs are made by the imaging path itself (the same cell and condition solved at
M = 2 and M = 8).  At inference the plain fine-grid solve is the fallback: a second head channel, trained to
predict the largest needed correction within ERR_WINDOW pixels, flags tiles that are
recomputed at M = 8 (the columns of those tiles only), and the fine solve is the judge of
the corrector's error in the tests and the bench.
"""
import numpy as np

from . import nn as N

CH = (32, 64, 128, 256)
IN_C = 16    # packed input channels (N_IN used)
N_IN = 4     # input planes: DF contrast, BF contrast, s_g, mean level
OUT_C = 16   # head channels: 0 the correction, 1 the expected local error (the fallback's guide)
ERR_WEIGHT = 0.1  # weight of channel 1's loss
ERR_WINDOW = 33   # channel 1 learns the largest |correction| within this window (pixels)
SG_SCALE = 50.0    # s_g (1/A) -> input plane value
CONTRAST = 20.0    # (DF - mean) -> input plane value
RES_SCALE = 100.0  # the network predicts (fine - interpolated coarse) * RES_SCALE


def _layer_specs():
    c0, c1, c2, c3 = CH
    return [
        ("enc0a", IN_C, c0, 9, True), ("enc0b", c0, c0, 9, True),
        ("enc1a", c0, c1, 9, True), ("enc1b", c1, c1, 9, True),
        ("enc2a", c1, c2, 9, True), ("enc2b", c2, c2, 9, True),
        ("bota", c2, c3, 9, True), ("botb", c3, c3, 9, True),
        ("dec2a", c3 + c2, c2, 9, True), ("dec2b", c2, c2, 9, True),
        ("dec1a", c2 + c1, c1, 9, True), ("dec1b", c1, c1, 9, True),
        ("dec0a", c1 + c0, c0, 9, True), ("dec0b", c0, c0, 9, True),
        ("head", c0, OUT_C, 1, False),
    ]


class UNet:
    """Parameters in one flat FP32 master buffer (weights, then biases) with a BF16 mirror;
    Adam moments and the gradient are flat buffers of the same layout."""

    def __init__(self, device="cuda", seed=0, head_std=1e-3):
        import torch
        self.device = device
        self.specs = _layer_specs()
        self.off_w, self.off_b = {}, {}
        n = 0
        for name, cin, cout, taps, _ in self.specs:
            self.off_w[name] = (n, cout * taps * cin)
            n += cout * taps * cin
        for name, cin, cout, taps, _ in self.specs:
            self.off_b[name] = (n, cout)
            n += cout
        self.n_params = n
        rng = np.random.default_rng(seed)
        host = np.zeros(n, dtype=np.float32)
        for name, cin, cout, taps, _ in self.specs:
            o, k = self.off_w[name]
            std = head_std if name == "head" else np.sqrt(2.0 / (taps * cin))
            host[o:o + k] = rng.standard_normal(k).astype(np.float32) * std
        self.master = torch.from_numpy(host).to(device)
        self.w16 = torch.empty(n, dtype=torch.bfloat16, device=device)
        N.to_bf16(self.master, self.w16)
        self.m = torch.zeros(n, dtype=torch.float32, device=device)
        self.v = torch.zeros(n, dtype=torch.float32, device=device)
        self.grad = torch.zeros(n, dtype=torch.float32, device=device)
        self.step_count = 0
        self.wt = {}
        self.refresh_flipped()

    # -- parameter views
    def weight(self, name):
        o, k = self.off_w[name]
        spec = self._spec(name)
        return self.w16[o:o + k].view(spec[2], spec[3], spec[1])

    def bias(self, name):
        o, k = self.off_b[name]
        return self.master[o:o + k]

    def gweight(self, name):
        o, k = self.off_w[name]
        spec = self._spec(name)
        return self.grad[o:o + k].view(spec[2], spec[3], spec[1])

    def gbias(self, name):
        o, k = self.off_b[name]
        return self.grad[o:o + k]

    def _spec(self, name):
        for s in self.specs:
            if s[0] == name:
                return s
        raise KeyError(name)

    def refresh_flipped(self):
        """Input-gradient weights (flipped, transposed) of every layer but the first."""
        for name, cin, cout, taps, _ in self.specs[1:]:
            self.wt[name] = N.weight_flip(self.weight(name), out=self.wt.get(name))

    # -- forward
    def _conv(self, name, x, out_fp32=False):
        _, cin, cout, taps, relu = self._spec(name)
        return N.conv2d(x, self.weight(name), self.bias(name), relu=relu, out_fp32=out_fp32)

    def forward(self, x, keep=False):
        """x: BF16 NHWC (B, H, W, 16), H and W multiples of 8; returns FP32 (B, H, W, 16)."""
        a = {"x0": x}
        a["e0a"] = self._conv("enc0a", x)
        a["e0"] = self._conv("enc0b", a["e0a"])
        a["p1"] = N.avgpool2(a["e0"])
        a["e1a"] = self._conv("enc1a", a["p1"])
        a["e1"] = self._conv("enc1b", a["e1a"])
        a["p2"] = N.avgpool2(a["e1"])
        a["e2a"] = self._conv("enc2a", a["p2"])
        a["e2"] = self._conv("enc2b", a["e2a"])
        a["p3"] = N.avgpool2(a["e2"])
        a["e3a"] = self._conv("bota", a["p3"])
        a["e3"] = self._conv("botb", a["e3a"])
        a["c2"] = N.upsample2_concat(a["e3"], a["e2"])
        a["d2a"] = self._conv("dec2a", a["c2"])
        a["d2"] = self._conv("dec2b", a["d2a"])
        a["c1"] = N.upsample2_concat(a["d2"], a["e1"])
        a["d1a"] = self._conv("dec1a", a["c1"])
        a["d1"] = self._conv("dec1b", a["d1a"])
        a["c0"] = N.upsample2_concat(a["d1"], a["e0"])
        a["d0a"] = self._conv("dec0a", a["c0"])
        a["d0"] = self._conv("dec0b", a["d0a"])
        out = self._conv("head", a["d0"], out_fp32=True)
        self.acts = a if keep else None
        return out

    # -- backward
    def _layer_bwd(self, name, x_in, g_pre, mask_in, need_dx=True):
        """Gradients of conv `name` given dL/d(pre-activation) g_pre and its input x_in;
        returns dL/dx_in, masked by mask_in > 0 (the ReLU that produced x_in) when given."""
        _, cin, cout, taps, _ = self._spec(name)
        N.conv2d_wgrad(x_in, g_pre, taps, self.gweight(name))
        N.bias_grad(g_pre, self.gbias(name))
        if not need_dx:
            return None
        return N.conv2d(g_pre, self.wt[name], mask=mask_in)

    def backward(self, g_out):
        """g_out: BF16 (B, H, W, 16), dL/d(head output).  Fills self.grad (zeroed first)."""
        import torch
        a = self.acts
        N.zero_(self.grad)
        c0, c1, c2, c3 = CH
        g = self._layer_bwd("head", a["d0"], g_out, a["d0"])
        g = self._layer_bwd("dec0b", a["d0a"], g, a["d0a"])
        g = self._layer_bwd("dec0a", a["c0"], g, a["c0"])
        B, H, W, _ = g.shape
        g_u = torch.empty((B, H, W, c1), dtype=torch.bfloat16, device=g.device)
        g_e0 = torch.empty((B, H, W, c0), dtype=torch.bfloat16, device=g.device)
        N.split(g, c1, g_u, g_e0)
        g = N.upsample2_bwd(g_u)                      # dL/d d1 (masked by the concat)
        g = self._layer_bwd("dec1b", a["d1a"], g, a["d1a"])
        g = self._layer_bwd("dec1a", a["c1"], g, a["c1"])
        B, H, W, _ = g.shape
        g_u = torch.empty((B, H, W, c2), dtype=torch.bfloat16, device=g.device)
        g_e1 = torch.empty((B, H, W, c1), dtype=torch.bfloat16, device=g.device)
        N.split(g, c2, g_u, g_e1)
        g = N.upsample2_bwd(g_u)                      # dL/d d2
        g = self._layer_bwd("dec2b", a["d2a"], g, a["d2a"])
        g = self._layer_bwd("dec2a", a["c2"], g, a["c2"])
        B, H, W, _ = g.shape
        g_u = torch.empty((B, H, W, c3), dtype=torch.bfloat16, device=g.device)
        g_e2 = torch.empty((B, H, W, c2), dtype=torch.bfloat16, device=g.device)
        N.split(g, c3, g_u, g_e2)
        g = N.upsample2_bwd(g_u)                      # dL/d e3
        g = self._layer_bwd("botb", a["e3a"], g, a["e3a"])
        g = self._layer_bwd("bota", a["p3"], g, None)  # dL/d p3 (pooled, no ReLU)
        g_e2 = N.add_(N.avgpool2_bwd(g), g_e2)
        N.relu_mask(g_e2, a["e2"])
        g = self._layer_bwd("enc2b", a["e2a"], g_e2, a["e2a"])
        g = self._layer_bwd("enc2a", a["p2"], g, None)
        g_e1 = N.add_(N.avgpool2_bwd(g), g_e1)
        N.relu_mask(g_e1, a["e1"])
        g = self._layer_bwd("enc1b", a["e1a"], g_e1, a["e1a"])
        g = self._layer_bwd("enc1a", a["p1"], g, None)
        g_e0 = N.add_(N.avgpool2_bwd(g), g_e0)
        N.relu_mask(g_e0, a["e0"])
        g = self._layer_bwd("enc0b", a["e0a"], g_e0, a["e0a"])
        self._layer_bwd("enc0a", a["x0"], g, None, need_dx=False)

    def adam_step(self, lr, wd=0.0):
        self.step_count += 1
        N.adam(self.master, self.m, self.v, self.grad, self.step_count, lr, w16=self.w16, wd=wd)
        self.refresh_flipped()

    # -- persistence
    def save(self, path, **meta):
        np.savez_compressed(path, master=self.master.cpu().numpy(), ch=np.array(CH), in_c=IN_C, out_c=OUT_C,
                            sg_scale=SG_SCALE, contrast=CONTRAST, res_scale=RES_SCALE, **meta)

    def load(self, path):
        import torch
        d = np.load(path)
        if (tuple(d["ch"]) != CH or int(d["in_c"]) != IN_C or int(d["out_c"]) != OUT_C
                or float(d["contrast"]) != CONTRAST or float(d["res_scale"]) != RES_SCALE):
            raise ValueError("corrector weights do not match this network")
        self.meta = {k: d[k] for k in d.files if k not in ("master",)}
        self.master.copy_(torch.from_numpy(d["master"].astype(np.float32)))
        N.to_bf16(self.master, self.w16)
        self.refresh_flipped()
        return self



# ---------------------------------------------------------------------------
# Training pairs made by the imaging path
# ---------------------------------------------------------------------------

XI0, XIG, KV = 103.9, 207.5, 200.0


def condition(cell, M, sg, g=(1, 1, 0)):
    """(DynamicalTwoBeamImaging, wrapped positions) of a cell imaged at voxel grid M, M."""
    from . import imaging, synth
    t, x, _ = imaging.d2bi_condition(cell.a_super, synth.A0_FE, (0, 0, 1), g, cell.pos, sg=sg, xi0=XI0, xig=XIG,
                                     V=KV, M=(M, M))
    return t, x


def pad8(n):
    return (n + 7) // 8 * 8


def coarse_planes(img2_dev, G2, G8, sg, Hp=None, Wp=None):
    """FP32 (5, Hp, Wp) planes on the fine grid from a coarse FP64 device image: the N_IN
    network inputs and the interpolated dark field (the base of the correction)."""
    import torch
    Hp = Hp or pad8(G8.My)
    Wp = Wp or pad8(G8.Mx)
    mean = torch.empty(1, dtype=torch.float64, device=img2_dev.device)
    N.image_mean(img2_dev, mean)
    planes = torch.empty((5, Hp, Wp), dtype=torch.float32, device=img2_dev.device)
    N.resample_planes(img2_dev, G2.Mx, G2.My, G8.Mx, G8.My, Wp, Hp, sg * SG_SCALE, mean, CONTRAST, planes)
    return planes


def make_pairs(ctx, cell, sgs, crop, per_image, rng, fp32=True):
    """For each s_g: the cell solved at M = 2 and M = 8, the coarse planes on the fine grid,
    and `per_image` random crop x crop windows.  Returns host arrays (inputs FP32 (n, N_IN,
    crop, crop), targets FP32 (n, crop, crop) = (fine - interpolated coarse dark field) *
    RES_SCALE)."""
    import torch

    from . import _lib
    flags = _lib.ST_FLAG_FP32 if fp32 else 0
    ins, tgs = [], []
    for sg in sgs:
        t2, x2 = condition(cell, 2, sg)
        t8, x8 = condition(cell, 8, sg)
        G2, aa2 = t2.image_geometry(len(x2))
        G8, aa8 = t8.image_geometry(len(x8))
        img2 = ctx.image(G2, x2, aa2, flags=flags)
        img8 = ctx.image(G8, x8, aa8, flags=flags)
        d2 = torch.from_numpy(np.ascontiguousarray(img2.T)).cuda()
        planes = coarse_planes(d2, G2, G8, sg).cpu().numpy()[:, :G8.My, :G8.Mx]
        fine = np.ascontiguousarray(img8.T).astype(np.float32)  # (My8, Mx8)
        if G8.My < crop or G8.Mx < crop:
            continue
        for _ in range(per_image):
            # half the crops touch an image edge in x, half in y (the network sees the edges,
            # where the coarse image extrapolates, as often as the interior)
            def corner(n):
                r = rng.random()
                return 0 if r < 0.25 else n - crop if r < 0.5 else int(rng.integers(0, n - crop + 1))
            y0, x0 = corner(G8.My), corner(G8.Mx)
            pin = planes[:, y0:y0 + crop, x0:x0 + crop]
            ins.append(pin[:N_IN])
            tgs.append((fine[y0:y0 + crop, x0:x0 + crop] - pin[4]) * RES_SCALE)
    if not ins:
        return np.zeros((0, N_IN, crop, crop), np.float32), np.zeros((0, crop, crop), np.float32)
    return np.stack(ins).astype(np.float32), np.stack(tgs).astype(np.float32)


def local_error(targets, window=ERR_WINDOW):
    """Channel 1's target: the largest |target| within window x window pixels around each
    pixel (a bound for the error anywhere in a tile of that size containing it)."""
    from scipy.ndimage import maximum_filter
    return np.stack([maximum_filter(np.abs(t), size=window, mode="nearest") for t in targets]).astype(np.float32)


class Trainer:
    """Adam on the MSE between the predicted correction and fine - interpolated coarse."""

    def __init__(self, model, inputs, targets, batch=8):
        """inputs FP32 (n, N_IN, S, S), targets FP32 (n, S, S), host arrays; kept on the device
        as packed BF16 NHWC inputs and FP32 targets."""
        import torch
        self.model = model
        self.batch = batch
        n, _, S, _ = inputs.shape
        self.n, self.S = n, S
        planes = torch.from_numpy(np.ascontiguousarray(inputs.transpose(1, 0, 2, 3))).cuda()  # (N_IN, n, S, S)
        self.x = N.pack(planes, IN_C)  # (n, S, S, 16)
        del planes
        self.y = torch.from_numpy(np.ascontiguousarray(targets)).cuda()
        self.y1 = torch.from_numpy(local_error(targets)).cuda()
        self.loss = torch.zeros(1, dtype=torch.float32, device="cuda")
        self.g = torch.empty((batch, S, S, OUT_C), dtype=torch.bfloat16, device="cuda")
        self.pos = 0

    def step(self, lr):
        b = self.batch
        if self.pos + b > self.n:
            self.pos = 0
        x = self.x[self.pos:self.pos + b]
        y = self.y[self.pos:self.pos + b]
        y1 = self.y1[self.pos:self.pos + b]
        self.pos += b
        out = self.model.forward(x, keep=True)
        N.mse(out, y, self.g, self.loss, ERR_WEIGHT, target1=y1)
        self.model.backward(self.g)
        self.model.adam_step(lr)

    def run(self, steps, lr=2e-3, lr_end=1e-4, log_every=0):
        import torch
        hist = []
        for i in range(steps):
            frac = i / max(1, steps - 1)
            lr_i = lr * (lr_end / lr) ** frac  # exponential decay
            if log_every and i % log_every == 0:
                N.zero_(self.loss)
            self.step(lr_i)
            if log_every and i % log_every == 0:
                torch.cuda.synchronize()
                hist.append((i, float(self.loss.item())))
        return hist


def evaluate(model, inputs, targets, batch=8):
    """Max and RMS |error| of the corrected and of the uncorrected (interpolated) dark field
    against the fine image (intensity units), over host arrays inputs (n, N_IN, S, S) and
    scaled targets (n, S, S)."""
    import torch
    n = inputs.shape[0]
    mx_c = mx_u = 0.0
    ss_c = ss_u = 0.0
    cnt = 0
    for i in range(0, n, batch):
        pin = torch.from_numpy(np.ascontiguousarray(inputs[i:i + batch].transpose(1, 0, 2, 3))).cuda()
        out = model.forward(N.pack(pin, IN_C))
        pred = out[..., 0].cpu().numpy()
        t = targets[i:i + batch]
        e_c, e_u = (pred - t) / RES_SCALE, -t / RES_SCALE
        mx_c, mx_u = max(mx_c, float(np.abs(e_c).max())), max(mx_u, float(np.abs(e_u).max()))
        ss_c += float((e_c.astype(np.float64) ** 2).sum())
        ss_u += float((e_u.astype(np.float64) ** 2).sum())
        cnt += t.size
    return {"max_corrected": mx_c, "max_uncorrected": mx_u, "rms_corrected": (ss_c / cnt) ** 0.5,
            "rms_uncorrected": (ss_u / cnt) ** 0.5}


# ---------------------------------------------------------------------------
# Inference: coarse solve + corrector, fine solve on the tiles it cannot be trusted on
# ---------------------------------------------------------------------------

class CorrectedImager:
    """M = 8 images from the M = 2 solve and the corrector, with the plain fine-grid solve
    as the fallback on T x T tiles whose predicted correction exceeds `tau`."""

    def __init__(self, model, ctx, tile=16, tau=0.05, border=None):
        """border: recompute the image's outer ring of tiles whatever their predicted error
        (default: as the model was calibrated, model.meta["border"], else True)."""
        self.model, self.ctx, self.T, self.tau = model, ctx, tile, tau
        if border is None:
            border = bool(int(getattr(model, "meta", {}).get("border", 1)))
        self.border = border

    def image(self, t2, t8, x_dev, n_atoms, sg, fallback=True, stream=0, diag=None, times=None):
        """Returns (FP64 device image (My8, Mx8), number of fallback tiles, tile count).  A
        dict `diag` receives the tile maxima of the predicted error magnitude (intensity
        units, host); tiles above tau are recomputed by the plain M = 8 solve.  The tile
        mask is made on the device, so nothing waits on the host between the network and
        the fine solve; the count is read once all of it is queued.  A dict `times`
        receives the GPU milliseconds of each stage (CUDA events on the current stream)."""
        import torch

        from . import _lib
        ev = []

        def mark():
            if times is not None:
                e = torch.cuda.Event(enable_timing=True)
                e.record()
                ev.append(e)

        G2, aa2 = t2.image_geometry(n_atoms)
        G8, aa8 = t8.image_geometry(n_atoms)
        dev = x_dev.device
        mark()
        img2 = torch.empty((G2.My, G2.Mx), dtype=torch.float64, device=dev)
        self.ctx.image_device(G2, x_dev.data_ptr(), n_atoms, aa2, _lib.ST_FLAG_FP32, img2.data_ptr(), stream=stream)
        mark()
        planes = coarse_planes(img2, G2, G8, sg)
        Hp, Wp = planes.shape[1:]
        out = self.model.forward(N.pack(planes[:N_IN].view(N_IN, 1, Hp, Wp), IN_C))
        img = torch.empty((G8.My, G8.Mx), dtype=torch.float64, device=dev)
        N.apply_correction(planes[4], out[0], G8.Mx, G8.My, 1.0 / RES_SCALE, img)
        mark()
        T = self.T
        ntx, nty = (G8.Mx + T - 1) // T, (G8.My + T - 1) // T
        if not fallback and diag is None:
            self._times(times, ev, ["m2_solve", "network"])
            return img, 0, ntx * nty
        tmax = torch.empty((nty, ntx), dtype=torch.float32, device=dev)
        N.tile_maxabs(out[0], G8.Mx, G8.My, T, tmax, ch=1)  # the predicted error magnitude
        if diag is not None:
            diag["tile_max"] = tmax.cpu().numpy() / RES_SCALE
        if not fallback:
            self._times(times, ev, ["m2_solve", "network"])
            return img, 0, ntx * nty
        # every tile above tau, and the image's outer ring if the model was calibrated so
        mask = torch.empty((nty, ntx), dtype=torch.uint8, device=dev)
        count = torch.empty((), dtype=torch.int32, device=dev)
        N.tile_flags(tmax, self.tau * RES_SCALE, mask, count, border=self.border)
        fine = torch.empty((G8.My, G8.Mx), dtype=torch.float64, device=dev)
        self.ctx.image_device_masked(G8, x_dev.data_ptr(), n_atoms, aa8, _lib.ST_FLAG_FP32, fine.data_ptr(),
                                     mask.data_ptr(), T, stream=stream)
        N.merge_tiles(fine, mask, T, G8.Mx, G8.My, img)
        mark()
        nflag = int(count.item())
        self._times(times, ev, ["m2_solve", "network", "fallback"])
        return img, nflag, ntx * nty

    @staticmethod
    def _times(times, ev, names):
        if times is None:
            return
        ev[-1].synchronize()
        for name, a, b in zip(names, ev[:-1], ev[1:]):
            times[name] = times.get(name, 0.0) + a.elapsed_time(b)



# ---------------------------------------------------------------------------
# Training data at scale, calibration of the fallback, the training command
# ---------------------------------------------------------------------------

def random_cell(rng, lo=100_000, hi=1_200_000, nxy=(64, 100)):
    """A seeded bcc Fe cell with about log-uniform [lo, hi] atoms, at least 64 lattice cells
    wide (an M = 8 image then holds a 512 x 512 crop), Poisson(10) voids of radius U(4, 15) A
    and, in 70 % of the cells, a screw dislocation."""
    from . import synth
    n = float(np.exp(rng.uniform(np.log(lo), np.log(hi))))
    nx = int(rng.integers(nxy[0], nxy[1] + 1))
    ny = int(rng.integers(nxy[0], nxy[1] + 1))
    nz = max(8, int(round(n / (2 * nx * ny))))
    return synth.make_cell(nx, ny, nz, int(rng.integers(1 << 31)), n_voids=int(rng.poisson(10)),
                           void_radius=(4.0, 15.0), with_screw=bool(rng.random() < 0.7))


def build_dataset(ctx, n_pairs, crop, seed, conds_per_cell=10, crops_per_image=5, **cell_kw):
    """n_pairs training pairs: cells from random_cell, each imaged at conds_per_cell s_g values
    U(-0.02, 0.02) at M = 2 and M = 8, crops_per_image random crop x crop windows each."""
    rng = np.random.default_rng(seed)
    xs, ys, n = [], [], 0
    while n < n_pairs:
        cell = random_cell(rng, **cell_kw)
        a, b = make_pairs(ctx, cell, list(rng.uniform(-0.02, 0.02, conds_per_cell)), crop, crops_per_image, rng)
        if len(a) == 0:
            continue
        xs.append(a)
        ys.append(b)
        n += len(a)
    return np.concatenate(xs)[:n_pairs], np.concatenate(ys)[:n_pairs]


def calibrate(model, ctx, conditions, tile=16, target=1e-2):
    """The fallback threshold over whole validation images (cell, s_g): the largest tau for
    which every tile whose corrected error exceeds `target` has a predicted local error
    above tau (so it falls back).  Two rules are calibrated: every tile judged by its
    prediction, and the image's outer ring of tiles always recomputed with the interior
    judged; the one that recomputes fewer tiles is kept.  Returns (tau, border, report)."""
    import torch

    from . import _lib
    imager = CorrectedImager(model, ctx, tile=tile, tau=np.inf, border=False)
    ring_pred, ring_bad, in_pred, in_bad, worst = [], [], [], [], 0.0
    for cell, sg in conditions:
        t2, x = condition(cell, 2, sg)
        t8, _ = condition(cell, 8, sg)
        G8, aa8 = t8.image_geometry(len(x))
        fine = ctx.image(G8, x, aa8, flags=_lib.ST_FLAG_FP32).T  # (My8, Mx8)
        diag = {}
        img, _, _ = imager.image(t2, t8, torch.from_numpy(x).cuda(), len(x), sg, fallback=False, diag=diag)
        err = np.abs(img.cpu().numpy() - fine)
        worst = max(worst, float(err.max()))
        tm = diag["tile_max"]
        ny, nx = tm.shape
        for ty in range(ny):
            for tx in range(nx):
                e = err[ty * tile:(ty + 1) * tile, tx * tile:(tx + 1) * tile].max()
                ring = ty == 0 or tx == 0 or ty == ny - 1 or tx == nx - 1
                (ring_pred if ring else in_pred).append(tm[ty, tx])
                if e > target:
                    (ring_bad if ring else in_bad).append(tm[ty, tx])
    ring_pred, in_pred = np.array(ring_pred), np.array(in_pred)
    n_tiles = ring_pred.size + in_pred.size

    def tau_of(bad, pred):
        return 0.9 * float(min(bad)) if bad else float(pred.max()) * 1.1 + 1e-6

    tau_all = tau_of(ring_bad + in_bad, np.concatenate([ring_pred, in_pred]))
    frac_all = float(((ring_pred > tau_all).sum() + (in_pred > tau_all).sum()) / n_tiles)
    tau_in = tau_of(in_bad, in_pred)
    frac_ring = float((ring_pred.size + (in_pred > tau_in).sum()) / n_tiles)
    border = frac_ring < frac_all
    tau = tau_in if border else tau_all
    return tau, border, {"tiles": int(n_tiles), "ring_tiles": int(ring_pred.size),
                         "tiles_above_target": len(ring_bad) + len(in_bad), "ring_tiles_above_target": len(ring_bad),
                         "fallback_fraction": frac_ring if border else frac_all,
                         "fallback_fraction_every_tile_judged": frac_all,
                         "fallback_fraction_ring_always": frac_ring, "border": bool(border),
                         "max_error_without_fallback": worst}


def train_main(argv=None):
    """python -m simulated_tem_gb300.corrector --out weights.npz [--pairs N --crop S --steps K]"""
    import argparse
    import json
    import time

    import torch

    from . import imaging
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", required=True)
    ap.add_argument("--pairs", type=int, default=2000)
    ap.add_argument("--crop", type=int, default=512)
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--batch", type=int, default=8)
    ap.add_argument("--lr", type=float, default=3e-3)
    ap.add_argument("--seed", type=int, default=20261208)
    ap.add_argument("--val-cells", type=int, default=4)
    args = ap.parse_args(argv)
    ctx = imaging.Context(0)
    t0 = time.time()
    xtr, ytr = build_dataset(ctx, args.pairs, args.crop, args.seed)
    xva, yva = build_dataset(ctx, max(16, args.pairs // 20), args.crop, args.seed + 1)
    t_data = time.time() - t0
    print("data: %d training pairs, %d validation pairs of %d px, %.1f s" % (len(xtr), len(xva), args.crop, t_data),
          flush=True)
    model = UNet(seed=args.seed)
    trainer = Trainer(model, xtr, ytr, batch=args.batch)
    del xtr, ytr
    t0 = time.time()
    seg = 4
    for k in range(seg):
        lr0, lr1 = args.lr * 0.3 ** k, args.lr * 0.3 ** (k + 1)
        trainer.run(args.steps // seg, lr=lr0, lr_end=lr1)
        torch.cuda.synchronize()
        ev = evaluate(model, xva, yva)
        print("  %d/%d steps, %.1f s: validation rms %.3e (interpolated %.3e), max %.3e (%.3e)"
              % ((k + 1) * (args.steps // seg), args.steps, time.time() - t0, ev["rms_corrected"],
                 ev["rms_uncorrected"], ev["max_corrected"], ev["max_uncorrected"]), flush=True)
    t_train = time.time() - t0
    rng = np.random.default_rng(args.seed + 2)
    conds = [(random_cell(rng), float(rng.uniform(-0.02, 0.02))) for _ in range(args.val_cells)]
    tau, border, report = calibrate(model, ctx, conds)
    report.update({"tau": tau, "validation": ev, "train_seconds": t_train, "data_seconds": t_data,
                   "pairs": args.pairs, "crop": args.crop, "steps": args.steps, "batch": args.batch})
    print(json.dumps(report), flush=True)
    model.save(args.out, tau=tau, border=int(border), report=json.dumps(report))
    return report


if __name__ == "__main__":
    train_main()
