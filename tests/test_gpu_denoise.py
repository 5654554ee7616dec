"""The learned density estimator's U-Net against a PyTorch FP32 restatement of the same network
built from the library's own layer table and parameters: forward outputs (BF16 weights and
activations, FP32 accumulation), backward gradients (cosine similarity per layer), and a
training smoke run whose loss falls."""
import numpy as np
import pytest
import torch
import torch.nn.functional as F

pytestmark = pytest.mark.gpu


def _bf(x):
    return x.to(torch.bfloat16).float()


def torch_unet(layers, params, feats, round_acts=True):
    """feats: [n, h, w, 8] float; returns the pre-clamp output [n, h, w, 3] and per-layer weights."""
    x0 = feats.permute(0, 3, 1, 2)
    acts, ws, o = [], [], 0
    for L in layers:
        cin = L["in_a"] + L["in_b"]
        k = 3 if L["taps"] == 9 else 1
        nw = L["out"] * L["taps"] * cin
        w = torch.tensor(params[o:o + nw], device=feats.device).view(L["out"], k, k, cin).permute(0, 3, 1, 2)
        b = torch.tensor(params[o + nw:o + nw + L["out"]], device=feats.device)
        o += nw + L["out"]
        w = _bf(w).requires_grad_(True)
        b = b.clone().requires_grad_(True)
        ws.append((w, b))

        def src(s):
            if s == -1:
                return x0
            if s <= -100:  # pooled output of the level above's last encoder conv
                lvl = -100 - s
                return F.avg_pool2d(acts[2 * (lvl - 1) + 1], 2)
            return acts[s]
        xa = src(L["src_a"])
        if L["upsample"]:
            xa = F.interpolate(xa, scale_factor=2, mode="nearest")
        x = torch.cat([xa, acts[L["src_b"]]], 1) if L["in_b"] else xa
        if round_acts:
            x = _bf(x.detach()) + (x - x.detach())  # BF16 storage, identity gradient
        y = F.conv2d(x, w, b, padding=k // 2)
        if L["relu"]:
            y = F.relu(y)
        acts.append(y)
    return acts[-1].permute(0, 2, 3, 1), ws


@pytest.fixture(scope="module")
def net(rk):
    d = rk.Denoiser(4 * 64 * 64, seed=5)
    # random parameters everywhere (the output layer starts at zero after creation)
    rng = np.random.default_rng(0)
    p, o = np.zeros(d.num_params(), np.float32), 0
    for L in d.layers():
        k = L["taps"] * (L["in_a"] + L["in_b"])
        p[o:o + L["out"] * k] = rng.normal(0, np.sqrt(2.0 / k), L["out"] * k)
        o += L["out"] * k
        p[o:o + L["out"]] = rng.normal(0, 0.05, L["out"])
        o += L["out"]
    d.set_params(p)
    return d


def _feats(n, h, w, seed):
    g = torch.Generator(device="cuda").manual_seed(seed)
    f = torch.zeros(n, h, w, 8, device="cuda")
    f[..., :7] = torch.rand(n, h, w, 7, device="cuda", generator=g)
    return f.to(torch.bfloat16)


def test_layer_table(net):
    L = net.layers()
    assert len(L) == 15
    assert [l["out"] for l in L[:8]] == [32, 32, 48, 48, 64, 64, 96, 96]
    assert L[-1]["taps"] == 1 and L[-1]["out"] == 3 and not L[-1]["relu"]
    assert net.num_params() == sum(l["out"] * l["taps"] * (l["in_a"] + l["in_b"]) + l["out"] for l in L)


@pytest.mark.parametrize("n,h,w", [(1, 32, 32), (2, 48, 64)])
def test_forward_matches_torch(rk, net, n, h, w):
    f = _feats(n, h, w, n + h)
    out = torch.zeros(n, h, w, 3, device="cuda")
    net.infer(f, out)
    torch.cuda.synchronize()
    ref, _ = torch_unet(net.layers(), net.params(), f.float())
    ref = (f.float()[..., 4:7] + ref).clamp(0, 1).detach()
    err = (out - ref).abs()
    assert float(err.mean()) < 2e-3, float(err.mean())
    assert float(err.max()) < 3e-2, float(err.max())


def test_gradients_match_autograd(rk, net):
    n, h, w = 2, 32, 32
    f = _feats(n, h, w, 9)
    g = torch.Generator(device="cuda").manual_seed(10)
    target = torch.rand(n, h, w, 3, device="cuda", generator=g)
    net.train_step(f, target, 0.0)  # lr 0: gradients only
    got = net.gradients()
    ref, ws = torch_unet(net.layers(), net.params(), f.float())
    loss = (f.float()[..., 4:7] + ref - target).abs().mean()
    loss.backward()
    o = 0
    for (w_, b_), L in zip(ws, net.layers()):
        gw = w_.grad.permute(0, 2, 3, 1).reshape(-1).cpu().numpy()
        nw = gw.size
        mine = got[o:o + nw]
        o += nw
        gb = b_.grad.cpu().numpy()
        mb = got[o:o + gb.size]
        o += gb.size
        cos = float(np.dot(gw, mine) / (np.linalg.norm(gw) * np.linalg.norm(mine) + 1e-30))
        assert cos > 0.98, (L, cos)
        assert np.linalg.norm(mine - gw) <= 0.2 * np.linalg.norm(gw) + 1e-6, L
        assert np.allclose(mb, gb, rtol=0.1, atol=0.05 * np.abs(gb).max() + 1e-6), L


def test_output_starts_at_the_plain_image(rk):
    d = rk.Denoiser(64 * 64, seed=2)
    f = _feats(1, 32, 32, 4)
    out = torch.zeros(1, 32, 32, 3, device="cuda")
    d.infer(f, out)
    torch.cuda.synchronize()
    assert torch.equal(out, f.float()[..., 4:7].clamp(0, 1))


def test_training_reduces_loss(rk):
    net = rk.Denoiser(4 * 64 * 64, seed=1)
    f = _feats(4, 64, 64, 3)
    # a smooth target that depends on the input: a blurred copy of its first three channels
    x = f.float()[..., :3].permute(0, 3, 1, 2)
    target = F.avg_pool2d(x, 5, stride=1, padding=2).permute(0, 2, 3, 1).contiguous()
    losses = [net.train_step(f, target, 2e-3) for _ in range(150)]
    assert losses[-1] < 0.35 * losses[0], (losses[0], losses[-1])


def test_features_of_histogram(rk):
    W, H = 64, 48
    g = torch.Generator(device="cuda").manual_seed(2)
    bins = torch.rand(H, W, 4, device="cuda", generator=g) * 5
    bins[::3, ::5] = 0
    out = torch.zeros(H, W, 8, dtype=torch.bfloat16, device="cuda")
    rk.denoiser_features(bins, W, H, out, k2=0.0)
    torch.cuda.synchronize()
    b = bins.double()
    k2 = W * H / float(b[..., 3].sum())
    a = b[..., 3]
    l = torch.where(a > 0, torch.log10(1 + a * k2), torch.zeros_like(a))
    s = torch.where(a > 0, l / a, torch.zeros_like(a))
    base = torch.rand(H, W, 4, device="cuda", generator=g)
    out2 = torch.zeros_like(out)
    rk.denoiser_features(bins, W, H, out2, k2=0.0, base=base)
    torch.cuda.synchronize()
    ref = torch.cat([l[..., None], b[..., :3] * s[..., None], torch.zeros(H, W, 4, device="cuda", dtype=torch.float64)], -1)
    assert torch.allclose(out.double(), ref, rtol=2 ** -7, atol=1e-6)
    ref[..., 4:7] = base[..., :3].double()
    assert torch.allclose(out2.double(), ref, rtol=2 ** -7, atol=1e-6)
