"""The learned path end to end at a small size: the renderer generates training pairs, the
U-Net trains on them (loss falls), inference beats the raw short run against the long-run
target, and the fallback policy switches to the plain path exactly when its estimate exceeds
the bound."""
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_small_pipeline(rk, compiler):
    from refrakt_gb300 import learned as LD
    S, n = 128, 32
    seeds = list(range(1000, 1000 + n))
    fl = [LD.genome(rk, compiler, s, S, S) for s in seeds]
    feats = torch.empty(n, S, S, 8, dtype=torch.bfloat16, device="cuda")
    targets = torch.empty(n, S, S, 3, device="cuda")
    LD.render_features(fl, S, S, 16, [s + 1 for s in seeds], feats)
    LD.render_images(fl, S, S, 1000, [s + 2 for s in seeds], targets)
    assert torch.isfinite(targets).all() and float(targets.max()) > 0
    assert torch.isfinite(feats.float()).all() and float(feats.float()[..., 0].max()) > 0
    net = rk.Denoiser(4 * S * S, seed=3)
    losses = LD.train(net, feats, targets, 300, batch=4, lr=2e-3)
    # the residual starts at the plain image's error, so the fall is moderate
    assert sum(losses[-20:]) / 20 < 0.85 * sum(losses[:20]) / 20
    # on the training genomes the denoised short run is closer to the target than the plain
    # path's image of the same short run (feature channels 4..6)
    den = torch.empty(n, S, S, 3, device="cuda")
    LD.infer_all(net, feats, den)
    plain = feats.float()[..., 4:7]
    assert float(LD.l1(den, targets).mean()) < float(LD.l1(plain, targets).mean())


@pytest.mark.parametrize("bound,expect_fallback", [(0.0, True), (1.0, False)])
def test_fallback_policy(rk, compiler, bound, expect_fallback):
    from refrakt_gb300 import learned as LD
    S = 64
    f = LD.genome(rk, compiler, 1234, S, S)
    net = rk.Denoiser(2 * S * S, seed=1)
    out, est, fb = LD.LearnedRenderer(net, spp=16, bound=bound).render(f, S, S, seed=9)
    assert fb == expect_fallback
    assert est >= 0.0 and out.shape == (S, S, 3) and torch.isfinite(out).all()
