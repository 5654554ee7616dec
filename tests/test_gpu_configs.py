"""Parity of the CUDA path with the FP64 oracle on the benchmark workloads' own genomes.

Each workload genome (tests/golden/genomes/, the same files bench.py renders) is drawn on a bin
grid reduced in resolution only — the genome's camera scales with the grid — and compared with
the oracle's chaos game (shaders/flame.glsl:41-90) on the same grid:

  * the hit histogram: relative L1 against the oracle within 1.5x the oracle's own two-seed
    noise floor at that sample count;
  * the image: the same points through adaptive DE (density_vert.glsl restated) and the
    log-density tonemap (tonemap.glsl:18-38), mean absolute RGB difference within 1.5x the
    floor of the oracle's own images;
  * the reference's real genome (flames/electricsheep.247.11256.flam3: post affine, 10 xforms,
    final xform, rotated camera): the xform-id stream bit-exact and both statistics within noise;
  * walker loss: the fraction of points that reach the frame over hundreds of passes against the
    FP32 oracle, without the walker reset (the reference's behaviour: lost walkers stay lost)
    and with it (flame.glsl:68);
  * rf_render (the end-to-end call) against the step-wise calls with the same seed, and its
    quality stop (main.cpp:411-412).

The measured ratios (L1 / floor) are printed per config.
"""
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest
import torch

from conftest import ROOT

pytestmark = pytest.mark.gpu

GENOMES = os.path.join(ROOT, "tests", "golden", "genomes")
SHEEP = "electricsheep.247.11256.flam3"

# genome file -> (reduced bin grid, supersample of the image, DE (R, min, curve) or None, reset)
CONFIGS = {
    "frame1080": ("frame1080.flam3", (480, 270), 2, (9, 0, 0.4), True),
    "frame1080-noreset": ("frame1080.flam3", (480, 270), 2, (9, 0, 0.4), False),
    "small": ("small.flam3", (128, 128), 1, None, True),
    "contract": ("contract.flam3", (480, 270), 1, None, True),
    "spacefill": ("spacefill.flam3", (256, 256), 2, None, True),
    "electricsheep": (SHEEP, (200, 148), 1, (11, 0, 0.6), False),
}
N, F, D = 8192, 20, 96
ORACLE_SEEDS = (101, 102, 103, 104)
GPU_SEEDS = (201, 202)


def _xml(name):
    with open(os.path.join(GENOMES, name)) as f:
        return f.read()


def _l1(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.abs(a / a.sum() - b / b.sum()).sum())


def _img_l1(a, b):
    return float(np.abs(np.asarray(a, np.float64)[..., :3] - np.asarray(b, np.float64)[..., :3]).mean())


def _oracle_runs(orc, xml, W, H, reset, draw=D, fp64=True):
    g = orc.Genome(xml)
    with ThreadPoolExecutor(len(ORACLE_SEEDS)) as ex:
        return list(ex.map(lambda s: g.chaos(N, W, H, fuse=F, draw=draw, seed=s, fp64=fp64, badval_reset=reset),
                           ORACLE_SEEDS))


def _gpu_run(rk, compiler, xml, W, H, seed, reset, draw=D, cta_slots=4096):
    f = rk.Flame.from_xml(xml, compiler)
    sim = rk.Sim(N, seed=seed, cta_slots=cta_slots, steps_per_launch=32)
    sim.set_bad_value_reset(reset)
    sim.warmup(f, F - 1)
    bins = torch.zeros(H, W, 4, device="cuda")
    hits = torch.zeros(H, W, dtype=torch.int32, device="cuda")
    sim.draw_to_bins(f, bins, hits, W, H, draw)
    c = sim.counters()
    sim.close()
    return bins, hits, c


def _oracle_image(orc, rgba, de, ss, info):
    src = rgba
    if de:
        src = orc.density_estimate(rgba, de[0], de[1], float(np.float32(de[2])))
    k2 = src.shape[0] * src.shape[1] / src[..., 3].sum()
    return orc.tonemap(src, info["gamma"], info["brightness"], info["vibrancy"], k2, ss=ss)


def _gpu_image(rk, bins, W, H, de, ss, info):
    src = bins
    if de:
        src = torch.zeros_like(bins)
        rk.density_estimate(bins, W, H, de[0], de[1], de[2], src)
    img = torch.zeros(H // ss, W // ss, 4, device="cuda")
    rk.tonemap(src, W, H, ss, info["gamma"], info["brightness"], info["vibrancy"], 0.0, img, None)
    torch.cuda.synchronize()
    return img.cpu().numpy()


@pytest.mark.parametrize("cfg", sorted(CONFIGS))
def test_config_histogram_and_image_within_noise(rk, orc, compiler, cfg):
    name, (W, H), ss, de, reset = CONFIGS[cfg]
    xml = _xml(name)
    info = rk.Flame.from_xml(xml, compiler).info()
    refs = _oracle_runs(orc, xml, W, H, reset)
    ref_hits = [r["hits"].astype(np.float64) for r in refs]
    ref_imgs = [_oracle_image(orc, r["rgba"], de, ss, info) for r in refs]
    pairs = [(i, j) for i in range(len(refs)) for j in range(i + 1, len(refs))]
    floor_h = np.mean([_l1(ref_hits[i], ref_hits[j]) for i, j in pairs])
    floor_i = np.mean([_img_l1(ref_imgs[i], ref_imgs[j]) for i, j in pairs])
    cross_h, cross_i = [], []
    for s in GPU_SEEDS:
        bins, hits, _ = _gpu_run(rk, compiler, xml, W, H, s, reset)
        g = hits.cpu().numpy().astype(np.float64)
        img = _gpu_image(rk, bins, W, H, de, ss, info)
        cross_h += [_l1(g, r) for r in ref_hits]
        cross_i += [_img_l1(img, r) for r in ref_imgs]
    ch, ci = float(np.mean(cross_h)), float(np.mean(cross_i))
    print("%s: histogram L1 %.4f / floor %.4f = %.2f; image L1 %.5f / floor %.5f = %.2f"
          % (cfg, ch, floor_h, ch / floor_h, ci, floor_i, ci / floor_i))
    assert sum(r["drawn"] for r in refs) > 0.2 * len(refs) * N * D
    assert ch <= 1.5 * floor_h
    assert ci <= 1.5 * floor_i


def test_reference_genome_xid_stream_bit_exact(rk, orc, compiler):
    """The reference's own genome: post affine, 10 xforms, final xform (variation_table.cpp:154-158)."""
    xml = _xml(SHEEP)
    f = rk.Flame.from_xml(xml, compiler)
    assert f.info()["num_xforms"] == 10 and f.info()["has_final"]
    assert any(b.get("post") for b in f.param_layout()["xforms"])  # xform 6 carries a post affine
    n, fuse, draw = 8192, 12, 29
    sim = rk.Sim(n, cta_slots=1024, steps_per_launch=8, seed=5)
    sim.enable_xid_trace(fuse + draw)
    sim.warmup(f, fuse - 1)
    bins = torch.zeros(148, 200, 4, device="cuda")
    hits = torch.zeros(148, 200, dtype=torch.int32, device="cuda")
    sim.draw_to_bins(f, bins, hits, 200, 148, draw)
    got = sim.read_xid_trace(fuse + draw)
    want = orc.Genome(xml).xid_sequence(n, fuse, draw, seed=5)
    assert np.array_equal(got, want)
    assert len(np.unique(want)) == 10
    c = sim.counters()
    # emitted points: every drawing step whose xform and final xform have opacity > 0
    assert c["emitted"] == draw * n and c["drawn"] == int(hits.sum().item())


@pytest.mark.parametrize("reset", [False, True])
def test_walker_loss_matches_oracle(rk, orc, compiler, reset):
    """Over 512 passes the headline genome loses walkers to NaN / infinity (variations with poles).
    Without the reset (the reference) the fraction of points reaching the frame falls as they are
    lost; with it, lost walkers restart.  The GPU's binned fraction matches the FP32 oracle's."""
    xml = _xml("frame1080.flam3")
    W, H, draw = 480, 270, 512
    r = orc.Genome(xml).chaos(N, W, H, fuse=F, draw=draw, seed=7, fp64=False, badval_reset=reset)
    want = r["drawn"] / (N * draw)
    got = []
    for s in GPU_SEEDS:
        _, hits, c = _gpu_run(rk, compiler, xml, W, H, s, reset, draw=draw)
        got.append(c["drawn"] / (N * draw))
        assert c["drawn"] == int(hits.sum().item())
    print("binned fraction over %d passes (reset %s): gpu %s, oracle %.4f" % (draw, reset, got, want))
    for v in got:
        assert abs(v - want) <= 0.05 * want
    if reset:
        assert want > 0.9
    else:
        assert want < 0.8  # walkers are lost: the reference's behaviour


LINEAR = ('<flame size="256 256" scale="64" center="0 0" estimator_radius="5" estimator_minimum="0" '
          'estimator_curve="0.5"><xform weight="0.5" color="0" color_speed="0.5" '
          'opacity="1" coefs="0.5 0 0 0.5 -0.5 0.3" linear="1"/><xform weight="0.3" color="1" color_speed="0.5" '
          'opacity="1" coefs="0.4 0.3 -0.3 0.4 0.5 0.2" linear="0.9"/><xform weight="0.2" color="0.5" '
          'color_speed="0.5" opacity="1" coefs="-0.5 0.1 0.2 0.6 0 -0.5" linear="1.1"/>'
          + "".join('<color index="%d" rgb="%d %d %d"/>' % (i, i, 255 - i, (i * 7) % 256) for i in range(256))
          + "</flame>")


def _stepwise(rk, f, sim, W, H, ss, points, fuse, de, info):
    bins = torch.zeros(H * ss, W * ss, 4, device="cuda")
    hits = torch.zeros(H * ss, W * ss, dtype=torch.int32, device="cuda")
    sim.warmup(f, fuse - 1, tss_width=0.0)
    sim.draw_to_bins(f, bins, hits, W * ss, H * ss, (points + sim.walkers - 1) // sim.walkers)
    src = bins
    if de:
        src = torch.zeros_like(bins)
        rk.density_estimate(bins, W * ss, H * ss, info["estimator_radius"], info["estimator_min"],
                            info["estimator_curve"], src)
    img8 = torch.zeros(H, W, 4, dtype=torch.uint8, device="cuda")
    rk.tonemap(src, W * ss, H * ss, ss, info["gamma"], info["brightness"], info["vibrancy"], 0.0, None, img8)
    torch.cuda.synchronize()
    return img8.cpu().numpy(), int(hits.sum().item())


@pytest.mark.parametrize("genome,size,ss,reset", [("linear", (256, 256), 1, False), ("frame1080", (240, 135), 2, True),
                                                  (SHEEP, (200, 148), 1, False)])
def test_render_matches_stepwise(rk, compiler, genome, size, ss, reset):
    """rf_render (the end-to-end call the benchmark's e2e figure times) against rf_warmup +
    rf_draw_to_bins + rf_density_estimate + rf_tonemap on a fresh simulation with the same seed:
    the same walkers, so the same counts; the colour sums differ only in the order of their FP32
    reductions, so the RGBA8 images agree to one step at the rare pixels where that order moves
    a value across a rounding boundary."""
    xml = LINEAR if genome == "linear" else _xml(genome if genome.endswith(".flam3") else genome + ".flam3")
    f = rk.Flame.from_xml(xml, compiler)
    info = f.info()
    W, H = size
    points = 64 * W * ss * H * ss
    n = 16384
    a = rk.Sim(n, seed=9, cta_slots=4096)
    a.set_bad_value_reset(reset)
    img, st = a.render(f, W, H, points, supersample=ss, fuse_passes=20, density_estimation=True)
    b = rk.Sim(n, seed=9, cta_slots=4096)
    b.set_bad_value_reset(reset)
    want, drawn = _stepwise(rk, f, b, W, H, ss, points, 20, True, info)
    assert st["binned"] == drawn and st["points"] == ((points + n - 1) // n) * n
    d = np.abs(img.astype(np.int32) - want.astype(np.int32))
    print("%s: %d of %d bytes differ (max %d)" % (genome, int((d > 0).sum()), d.size, int(d.max())))
    assert d.max() <= 1
    assert (d > 0).mean() <= 1e-3
    assert np.all(img[..., 3] == 255)
    a.close()
    b.close()


def test_render_applies_the_genome_spatial_filter(rk, compiler):
    """The reference genome carries filter="1" filter_shape="gaussian": rf_render at supersample 4
    draws the Gaussian window over the density-estimated bins, as rf_density_estimate followed by
    rf_tonemap_filter on a simulation with the same seed."""
    xml = _xml(SHEEP)
    f = rk.Flame.from_xml(xml, compiler)
    info = f.info()
    assert info["filter"] == 1.0 and info["filter_shape"] == rk.FILTER_GAUSSIAN
    W, H, ss, n = 100, 74, 4, 16384
    points = 32 * W * ss * H * ss
    a = rk.Sim(n, seed=4)
    img, st = a.render(f, W, H, points, supersample=ss, fuse_passes=20, density_estimation=True)
    b = rk.Sim(n, seed=4)
    bins = torch.zeros(H * ss, W * ss, 4, device="cuda")
    hits = torch.zeros(H * ss, W * ss, dtype=torch.int32, device="cuda")
    b.warmup(f, 19, tss_width=0.0)
    b.draw_to_bins(f, bins, hits, W * ss, H * ss, (points + n - 1) // n)
    de = torch.zeros_like(bins)
    rk.density_estimate(bins, W * ss, H * ss, info["estimator_radius"], info["estimator_min"],
                        info["estimator_curve"], de)
    want = torch.zeros(H, W, 4, dtype=torch.uint8, device="cuda")
    rk.tonemap_filter(de, W * ss, H * ss, ss, info["filter"], info["filter_shape"], info["gamma"],
                      info["brightness"], info["vibrancy"], 0.0, None, want)
    torch.cuda.synchronize()
    d = np.abs(img.astype(np.int32) - want.cpu().numpy().astype(np.int32))
    assert d.max() <= 1 and (d > 0).mean() <= 1e-3
    a.close()
    b.close()


def test_render_quality_stop(rk, compiler):
    """stop_on_binned: passes are drawn until the binned count reaches the target (the reference's
    accumulated < quality * W * H loop, main.cpp:411-412); walker-steps exceed it by the points
    that miss the frame."""
    xml = _xml("frame1080.flam3")
    f = rk.Flame.from_xml(xml, compiler)
    W, H, n = 240, 135, 16384
    target = 200 * W * H
    for reset in (True, False):
        s = rk.Sim(n, seed=3, cta_slots=4096)
        s.set_bad_value_reset(reset)
        _, st = s.render(f, W, H, target, fuse_passes=20, density_estimation=False, stop_on_binned=True)
        print("reset %s: binned %d for target %d in %d walker-steps" % (reset, st["binned"], target, st["points"]))
        assert st["binned"] >= target
        assert st["points"] > st["binned"]
        # the rounds stop within one round of passes past the target
        assert st["binned"] <= target + 2 * 32 * n
        s.close()
