"""Batched rendering (rf_batch_*): many genomes in one persistent launch, captured in a CUDA graph.

  * every work unit is the reference's chaos game of cta_slots walkers on a documented seed and
    shuffle schedule, so an affine genome's per-item histogram equals the sum of the FP32 oracle's
    per-unit histograms, count for count, on every replay of the graph;
  * a nonlinear genome's batched histogram is within the oracle's own seed-to-seed noise;
  * the captured density-estimation and tonemap tail equals the standalone entry points run on
    the batch's bins;
  * the autotuner picks a supported shape and covers every requested point.
"""
import numpy as np
import pytest
import torch

from test_gpu_parity import LINEAR, _l1

pytestmark = pytest.mark.gpu

STRIDE = 0x9E3779B97F4A7C15
MASK = (1 << 64) - 1

LINEAR2 = ('<flame size="128 96" scale="40" center="0.1 -0.1" rotate="20"><xform weight="0.6" color="0.2" '
           'color_speed="0.3" opacity="1" coefs="0.6 -0.1 0.1 0.5 0.3 -0.2" linear="1"/><xform weight="0.4" '
           'color="0.9" color_speed="0.7" opacity="0.8" coefs="-0.4 0.2 0.3 0.5 -0.4 0.4" linear="1"/>'
           + "".join('<color index="%d" rgb="%d %d %d"/>' % (i, (i * 3) % 256, i, 255 - i) for i in range(256))
           + "</flame>")


def _oracle_item(orc, xml, W, H, seed, units, slots, F, D):
    og = orc.Genome(xml)
    hits = np.zeros((H, W), np.uint64)
    rgba = np.zeros((H, W, 4), np.float64)
    for u in range(units):
        r = og.chaos(slots, W, H, fuse=F, draw=D, seed=(seed + u * STRIDE) & MASK, fp64=False, shuffle_mode=1,
                     cta_slots=slots, steps_per_launch=1 << 30, table_size=1024, table_seed=0x5EED + slots)
        hits += r["hits"]
        rgba += r["rgba"]
    return hits, rgba


@pytest.mark.parametrize("slots", [1024, 4096])
def test_affine_items_equal_oracle_units(rk, orc, compiler, slots):
    F, D = 20, 24
    specs = [(LINEAR, 256, 256, 3, 11), (LINEAR2, 128, 96, 2, 5)]  # xml, W, H, units, seed
    flames = [rk.Flame.from_xml(x, compiler) for x, *_ in specs]
    items = [(f, W, H, u * slots * D, s) for f, (_, W, H, u, s) in zip(flames, specs)]
    b = rk.Batch(items, fuse_passes=F, cta_slots=slots, unit_passes=D, density_estimation=False, k2=1e-3)
    info = b.info()
    assert (info["cta_slots"], info["units"], info["unit_passes"]) == (slots, 5, D)
    for rep in range(2):  # graph replays are deterministic in counts
        b.run()
        st = b.sync()
        assert st["points"] == 5 * slots * D
        assert st["steps"] == 5 * slots * (F + D)
        binned = 0
        for i, (xml, W, H, u, s) in enumerate(specs):
            rgba, hits = b.bins(i)
            oh, orgba = _oracle_item(orc, xml, W, H, s, u, slots, F, D)
            assert int(oh.sum()) > u * slots * D // 2
            assert np.array_equal(hits.astype(np.uint64), oh), "item %d replay %d" % (i, rep)
            assert np.allclose(rgba, orgba, rtol=1e-4, atol=1e-3)
            binned += int(oh.sum())
        assert st["binned"] == binned


def test_items_with_equal_seeds_share_streams(rk, compiler):
    """Two items of one genome and one seed draw the same points; another seed does not."""
    f = rk.Flame.from_xml(LINEAR, compiler)
    pts = 2 * 1024 * 16
    b = rk.Batch([(f, 64, 64, pts, 4), (f, 64, 64, pts, 4), (f, 64, 64, pts, 5)], cta_slots=1024, unit_passes=16,
                 density_estimation=False)
    b.run()
    b.sync()
    h = [b.bins(i)[1] for i in range(3)]
    assert np.array_equal(h[0], h[1])
    assert not np.array_equal(h[0], h[2])


@pytest.mark.parametrize("kind,seed", [(0, 0), (1, 1)])
def test_batched_histogram_within_oracle_noise(rk, orc, compiler, kind, seed):
    W = H = 96
    f = rk.Flame.synthesize(compiler, kind, seed, W, H, n_xforms=6, final_xform=(kind == 1))
    og = orc.Genome(f.to_xml())
    N, F, D = 8192, 20, 48
    refs = [og.chaos(N, W, H, fuse=F, draw=D, seed=s, want_rgba=False)["hits"].astype(np.float64)
            for s in (101, 102, 103, 104)]
    floor = np.mean([_l1(refs[i], refs[j]) for i in range(4) for j in range(i + 1, 4)])
    b = rk.Batch([(f, W, H, N * D, 201), (f, W, H, N * D, 202)], fuse_passes=F, cta_slots=1024, unit_passes=D,
                 density_estimation=False)
    b.run()
    b.sync()
    gpus = [b.bins(i)[1].astype(np.float64) for i in range(2)]
    cross = np.mean([_l1(g, r) for g in gpus for r in refs])
    print("L1 batch-vs-oracle %.4f, oracle floor %.4f (ratio %.2f)" % (cross, floor, cross / floor))
    assert cross <= 1.5 * floor


@pytest.mark.parametrize("use_graph", [True, False])
def test_captured_tail_equals_entry_points(rk, compiler, use_graph):
    fa = rk.Flame.synthesize(compiler, rk.SYNTH_SMALL, 3, 160, 120)
    fb = rk.Flame.synthesize(compiler, rk.SYNTH_RANDOM, 4, 96, 64, n_xforms=5)
    fa.set_estimator(6, 0, 0.4)
    fb.set_estimator(3, 1, 0.6)
    items = [(fa, 160, 120, 1 << 22, 1, 2), (fb, 96, 64, 1 << 21, 2, 1)]
    b = rk.Batch(items, cta_slots=2048, density_estimation=True, k2=0.0, use_graph=use_graph)
    b.run()
    b.sync()
    for i, (f, w, h, _, _, ss) in enumerate(items):
        info = f.info()
        rgba, _ = b.bins(i)
        d_in = torch.from_numpy(rgba).cuda()
        d_de = torch.zeros_like(d_in)
        rk.density_estimate(d_in, w * ss, h * ss, info["estimator_radius"], info["estimator_min"],
                            info["estimator_curve"], d_de)
        img8 = torch.zeros(h, w, 4, dtype=torch.uint8, device="cuda")
        rk.tonemap(d_de, w * ss, h * ss, ss, info["gamma"], info["brightness"], info["vibrancy"], 0.0, None, img8)
        torch.cuda.synchronize()
        got, want = b.image(i).astype(np.int32), img8.cpu().numpy().astype(np.int32)
        # the automatic k2 comes from an FP64 atomic sum, whose order may move its last bit
        assert np.abs(got - want).max() <= 1
        assert np.mean(got == want) > 0.999


def test_splat_strategies_agree_and_autotune_picks_warp_for_compact(rk, compiler):
    """Warp-aggregated and per-point reductions give the same counts; AUTO picks the warp path for
    a contracting genome and the per-point path for a spread one."""
    fc = rk.Flame.synthesize(compiler, rk.SYNTH_CONTRACT, 4, 256, 256)
    fs = rk.Flame.synthesize(compiler, rk.SYNTH_RANDOM, 1, 256, 256, n_xforms=8)
    items = [(fc, 256, 256, 1024 * 64, 3), (fs, 256, 256, 1024 * 64, 4)]
    res = {}
    for mode in (rk.SPLAT_GLOBAL, rk.SPLAT_WARP, rk.SPLAT_AUTO):
        b = rk.Batch(items, cta_slots=1024, unit_passes=64, density_estimation=False, splat=mode)
        b.run()
        b.sync()
        res[mode] = [b.bins(i) for i in range(2)]
        if mode == rk.SPLAT_AUTO:
            assert b.info()["splat"] == [rk.SPLAT_WARP, rk.SPLAT_GLOBAL]
        b.close()
    for i in range(2):
        g, w = res[rk.SPLAT_GLOBAL][i], res[rk.SPLAT_WARP][i]
        assert np.array_equal(g[1], w[1])
        assert np.allclose(g[0], w[0], rtol=1e-4, atol=1e-3)


def test_autotuned_units_fill_the_gpu(rk, compiler):
    # a single short render is cut into about one unit per SM, not a few long ones
    import torch
    f = rk.Flame.synthesize(compiler, rk.SYNTH_RANDOM, 7, 1024, 1024, n_xforms=4)
    b = rk.Batch([(f, 1024, 1024, 16 * 1024 * 1024, 1)], density_estimation=False)
    info = b.info()
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    assert info["units"] >= sms // 2, info
    b.run()
    assert b.sync()["points"] >= 16 * 1024 * 1024
    b.close()


def test_autotuned_shape_covers_points(rk, compiler):
    fl = [rk.Flame.synthesize(compiler, rk.SYNTH_RANDOM, s, 128, 128, n_xforms=2 + s % 8) for s in range(12)]
    pts = [(1 + s % 3) * 3_000_000 for s in range(12)]
    b = rk.Batch([(f, 128, 128, p, s) for s, (f, p) in enumerate(zip(fl, pts))], density_estimation=True)
    info = b.info()
    assert info["cta_slots"] in (1024, 2048, 4096)
    assert info["unit_passes"] >= 1 and info["units"] >= 12
    b.run()
    st = b.sync()
    assert st["points"] >= sum(pts)
    assert st["points"] <= sum(pts) + 12 * info["cta_slots"] * info["unit_passes"]
    assert st["binned"] > 0.3 * sum(pts)
    for i in range(12):
        assert b.image(i)[..., :3].max() > 0


@pytest.mark.parametrize("kind", ["affine", "random"])
def test_specialised_group_equals_interpreted(rk, compiler, kind):
    """A genome structure with >= 2 units per SM gets its own specialised persistent launch (the
    rest share the interpreted one); the histograms equal the interpreted kernel's count for
    count."""
    if kind == "affine":
        fl = [rk.Flame.from_xml(LINEAR, compiler)]
    else:
        fl = [rk.Flame.synthesize(compiler, rk.SYNTH_RANDOM, 2, 128, 128, n_xforms=5, final_xform=True)]
    other = rk.Flame.synthesize(compiler, rk.SYNTH_SMALL, 3, 96, 96)
    units = 2 * torch.cuda.get_device_properties(0).multi_processor_count + 8
    items = [(fl[0], 128, 128, units * 1024 * 16, 21), (fl[0], 128, 128, 4 * 1024 * 16, 22), (other, 96, 96, 1024 * 16, 23)]
    res = []
    for spec in (0, -1):
        b = rk.Batch(items, cta_slots=1024, unit_passes=16, density_estimation=False, specialize=spec)
        info = b.info()
        assert info["specialized"] == ([1, 1, 0] if spec == 0 else [0, 0, 0])
        b.run()
        st = b.sync()
        res.append(([b.bins(i) for i in range(3)], st))
        b.close()
    (a, sa), (c, sc) = res
    assert sa["points"] == sc["points"] and sa["binned"] == sc["binned"]
    for i in range(3):
        assert np.array_equal(a[i][1], c[i][1]), i
        assert np.allclose(a[i][0], c[i][0], rtol=1e-4, atol=1e-3)


def test_every_structure_specialised_equals_interpreted(rk, compiler):
    """specialize = 2: every genome structure gets its own specialised persistent launch (the
    launches overlap on forked streams); every item's counts equal the interpreted kernel's."""
    fl = [rk.Flame.synthesize(compiler, rk.SYNTH_RANDOM, 40 + k, 96, 96, n_xforms=2 + k % 6, final_xform=k % 2 == 1)
          for k in range(6)]
    items = [(f, 96, 96, 3 * 1024 * 16, 60 + k) for k, f in enumerate(fl)]
    res = []
    for spec in (2, -1):
        b = rk.Batch(items, cta_slots=1024, unit_passes=16, density_estimation=False, specialize=spec)
        info = b.info()
        assert info["specialized"] == ([1] * 6 if spec == 2 else [0] * 6)
        b.run()
        st = b.sync()
        res.append(([b.bins(i) for i in range(6)], st))
        b.close()
    (a, sa), (c, sc) = res
    assert sa["points"] == sc["points"] and sa["binned"] == sc["binned"]
    for i in range(6):
        assert np.array_equal(a[i][1], c[i][1]), i
        assert np.allclose(a[i][0], c[i][0], rtol=1e-4, atol=1e-3)
