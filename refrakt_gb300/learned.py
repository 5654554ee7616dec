"""Learned density estimation: data generation, training and evaluation around the C-ABI
denoiser (rf_denoiser_*), with the plain adaptive-DE path as its fallback and as the standard
its error is measured against.

The renderer generates its own training pairs: for each random genome, the features of a
short-run render (16 samples per pixel: the histogram's log density and colour, and the plain
path's adaptive-DE image of it, on which the network predicts a residual) and the converged
target (the 1000-spp adaptive-DE tonemapped image) — both through the batched persistent launch.  Training
and inference run the library's own tensor-core kernels; PyTorch only holds device buffers.

A frame rendered on the learned path carries an error estimate: two independent short runs are
denoised, and half the mean absolute difference of the two outputs estimates the error of their
average.  Frames whose estimate exceeds the bound are rendered on the plain path instead.
"""
import math

import numpy as np

from . import Batch, SYNTH_RANDOM, Flame

DE = (9, 0, 0.4)  # adaptive DE of the plain path: max radius, min radius, curve


def level(spp):
    """Feature channel 7: the short run's sample count, log2(spp) / 10."""
    return math.log2(spp) / 10.0


def genome(R, comp, seed, w, h):
    """A training / held-out genome: 2-12 xforms by seed, with a final xform, 3 random
    variations per xform from the implemented set, affine coefficients in [-1.2, 1.2]."""
    f = Flame.synthesize(comp, SYNTH_RANDOM, seed, w, h, n_xforms=2 + seed % 11, final_xform=True)
    f.set_estimator(*DE)
    return f


def render_features(flames, w, h, spp, seeds, out, device=0, chunk=256):
    """Features [len(flames), h, w, 8] bf16 of spp-sample renders into `out`: the raw histogram's
    log density and colour, and the plain path's image (adaptive DE + tonemap) of it."""
    for c0 in range(0, len(flames), chunk):
        part = flames[c0:c0 + chunk]
        b = Batch([(f, w, h, spp * w * h, s) for f, s in zip(part, seeds[c0:c0 + chunk])],
                  density_estimation=True, image_f32=True, device=device)
        b.run()
        b.sync()
        for i in range(len(part)):
            b.features(i, out[c0 + i], level=level(spp))
        b.close()


def render_images(flames, w, h, spp, seeds, out, device=0, chunk=256, de=True):
    """Tonemapped RGB [len(flames), h, w, 3] float32 of spp-sample renders (adaptive DE) into `out`."""
    import torch
    tmp = torch.empty(h, w, 4, device=out.device)
    for c0 in range(0, len(flames), chunk):
        part = flames[c0:c0 + chunk]
        b = Batch([(f, w, h, spp * w * h, s) for f, s in zip(part, seeds[c0:c0 + chunk])],
                  density_estimation=de, image_f32=True, device=device)
        b.run()
        b.sync()
        for i in range(len(part)):
            b.image_f32(i, tmp)
            out[c0 + i].copy_(tmp[..., :3])
        b.close()


def l1(a, b):
    """Mean absolute error per image (RGB in [0, 1])."""
    return (a - b).abs().flatten(1).mean(1)


def validation_l1(net, feats, targets, batch=4):
    """Mean L1 of the network's images of `feats` against `targets` (held-out genomes)."""
    import torch
    out = torch.empty(feats.shape[0], feats.shape[1], feats.shape[2], 3, device=feats.device)
    infer_all(net, feats, out, batch)
    return float(l1(out, targets).mean())


def train(net, feats, targets, steps, batch=4, lr=1e-3, seed=0, log=None, crop=0, val=None, val_every=500):
    """Adam on random minibatches; cosine learning-rate decay to lr / 20.  `feats` is one
    [n, h, w, 8] tensor or a list of them (one per input sample count, each against the same
    targets): every minibatch image draws its sample count at random.  With `crop` (a multiple
    of 8) each minibatch entry is a random crop of that size, so one step sees more genomes.
    With `val` = (features, targets) of genomes kept out of training, the validation L1 is
    measured every `val_every` steps and the parameters of the best measurement are restored at
    the end (early stopping: the network is kept from fitting its targets' own noise).  Returns
    the training losses; with `val`, also the validation history as (step, L1) pairs."""
    import torch
    g = torch.Generator().manual_seed(seed)
    levels = feats if isinstance(feats, (list, tuple)) else [feats]
    n, H, W = levels[0].shape[:3]
    losses = []
    history, best = [], None
    for s in range(steps):
        idx = torch.randint(0, n, (batch,), generator=g).tolist()
        lv = torch.randint(0, len(levels), (batch,), generator=g).tolist()
        if crop:
            ys = (torch.randint(0, (H - crop) // 8 + 1, (batch,), generator=g) * 8).tolist()
            xs = (torch.randint(0, (W - crop) // 8 + 1, (batch,), generator=g) * 8).tolist()
            f = torch.stack([levels[l][i, y:y + crop, x:x + crop] for l, i, y, x in zip(lv, idx, ys, xs)])
            t = torch.stack([targets[i, y:y + crop, x:x + crop] for i, y, x in zip(idx, ys, xs)])
        else:
            f = torch.stack([levels[l][i] for l, i in zip(lv, idx)])
            t = torch.stack([targets[i] for i in idx])
        # random flips keep the attractors' orientation statistics symmetric
        if s % 2:
            f, t = f.flip(2).contiguous(), t.flip(2).contiguous()
        a = lr * (0.05 + 0.95 * 0.5 * (1 + math.cos(math.pi * s / max(1, steps))))
        losses.append(net.train_step(f, t, a))
        if log and (s % 100 == 0 or s == steps - 1):
            log("step %d loss %.5f lr %.2e" % (s, losses[-1], a))
        if val is not None and ((s + 1) % val_every == 0 or s == steps - 1):
            v = validation_l1(net, val[0], val[1])
            history.append((s + 1, v))
            if best is None or v < best[0]:
                best = (v, net.params())
            if log:
                log("step %d validation L1 %.5f (best %.5f)" % (s + 1, v, best[0]))
    if val is None:
        return losses
    net.set_params(best[1])
    return losses, history


def infer_all(net, feats, out, batch=4):
    for i in range(0, feats.shape[0], batch):
        net.infer(feats[i:i + batch].contiguous(), out[i:i + batch])


def plain_equivalent_spp(spps, errs, e):
    """The plain path's samples per pixel at error e, by log-log interpolation of its curve."""
    ls, le = np.log(np.asarray(spps, float)), np.log(np.asarray(errs, float))
    order = np.argsort(le)
    return float(np.exp(np.interp(math.log(e), le[order], ls[order])))


class LearnedRenderer:
    """The learned path for one frame with its fallback: two short runs of `spp` samples per
    pixel are denoised; the error estimate is half the mean absolute difference of the two
    denoised outputs plus `plain_weight` times that of the two plain images (the sampling noise
    the network has to remove); above `bound` the frame is rendered on the plain path
    (`plain_spp`, adaptive DE) instead.  `scale` calibrates the estimate against held-out
    frames' true errors (the split estimate sees only the variance of the two runs)."""

    def __init__(self, net, spp=16, bound=0.02, plain_spp=1000, plain_weight=0.0, scale=1.0, device=0):
        self.net, self.spp, self.bound, self.plain_spp, self.device = net, spp, bound, plain_spp, device
        self.plain_weight, self.scale = plain_weight, scale

    def estimate(self, flame, w, h, seed=0):
        """(denoised average, learned split estimate, plain split estimate) of two short runs."""
        import torch
        feats = torch.empty(2, h, w, 8, dtype=torch.bfloat16, device="cuda")
        render_features([flame, flame], w, h, self.spp, [seed, seed + 1], feats, self.device)
        out = torch.empty(2, h, w, 3, device="cuda")
        self.net.infer(feats, out)
        est = 0.5 * float((out[0] - out[1]).abs().mean())
        plain = 0.5 * float((feats[0, ..., 4:7].float() - feats[1, ..., 4:7].float()).abs().mean())
        return 0.5 * (out[0] + out[1]), est, plain

    def render(self, flame, w, h, seed=0):
        """(image, error estimate, fell back)."""
        import torch
        img, est, plain = self.estimate(flame, w, h, seed)
        e = self.scale * (est + self.plain_weight * plain)
        if e <= self.bound:
            return img, e, False
        full = torch.empty(1, h, w, 3, device="cuda")
        render_images([flame], w, h, self.plain_spp, [seed], full, self.device)
        return full[0], e, True
