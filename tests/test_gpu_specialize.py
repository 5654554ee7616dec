"""Genome-specialised chaos kernels (compiled at run time) against the interpreted kernel:
identical xform-id streams and emitted counts, bit-exact histogram counts on an affine genome
(and against the FP32 oracle), histograms within the seed-to-seed noise on nonlinear genomes."""
import numpy as np
import pytest
import torch

from test_gpu_parity import LINEAR, _bins, _l1

pytestmark = pytest.mark.gpu


def _run(rk, f, N, W, H, F, D, seed, specialize, trace=0, pipe=True, **kw):
    sim = rk.Sim(N, seed=seed, specialize=specialize, **kw)
    sim.set_exchange(rk.EXCHANGE_PIPELINED if pipe is True else rk.EXCHANGE_BARRIER if pipe is False else pipe)
    if trace:
        sim.enable_xid_trace(trace)
    sim.warmup(f, F - 1)
    assert sim.specialized() == (specialize >= 0)
    bins, hits = _bins(W, H)
    sim.draw_to_bins(f, bins, hits, W, H, D)
    out = {"hits": hits.cpu().numpy().astype(np.uint64), "rgba": bins.cpu().numpy(), "counters": sim.counters()}
    if trace:
        out["trace"] = sim.read_xid_trace(trace)
    sim.close()
    return out


@pytest.mark.parametrize("cta,threads", [(4096, 1024), (2048, 512), (2048, 1024), (1024, 1024)])
def test_affine_genome_bit_exact(rk, orc, compiler, cta, threads):
    """Specialised kernel with the pipelined walker exchange, specialised kernel with a barrier per
    pass, interpreted kernel: the same counts as the FP32 oracle on the Sim's shuffle table (built
    for threads / slots phases per pass), for every CTA shape."""
    f = rk.Flame.from_xml(LINEAR, compiler)
    N, F, D = 8192, 20, 40
    kw = dict(cta_slots=cta, cta_threads=threads, steps_per_launch=32)
    a = _run(rk, f, N, 256, 256, F, D, 3, 1, **kw)
    p = _run(rk, f, N, 256, 256, F, D, 3, 1, pipe=False, **kw)
    b = _run(rk, f, N, 256, 256, F, D, 3, -1, **kw)
    r = orc.Genome(LINEAR).chaos(N, 256, 256, fuse=F, draw=D, seed=3, fp64=False, shuffle_mode=1, cta_slots=cta,
                                 cta_threads=threads, steps_per_launch=32, table_size=1024)
    for o in (a, p, b):
        assert np.array_equal(o["hits"], r["hits"])
        assert np.allclose(o["rgba"], a["rgba"], rtol=1e-4, atol=1e-3)


@pytest.mark.parametrize("L", [1, 2, 7, 256])
def test_pipelined_exchange_equals_barrier_exchange(rk, compiler, L):
    """On a nonlinear genome with the walker reset and a final xform, the pipelined exchange and
    the automatic choice (which times both forms on its first two drawing launches of >= 32 passes) draw the
    same xform-id streams and the same counts as the barrier form, for launches of any length (the
    first pass of each launch is the gather, the last one draws no next xform)."""
    W = H = 128
    f = rk.Flame.synthesize(compiler, 1, 9, W, H, n_xforms=8, final_xform=True, force_parametric=True)
    out = []
    for pipe in (True, False, rk.EXCHANGE_AUTO):
        o = _run(rk, f, 8192, W, H, 20, 24, 7, 1, trace=44, pipe=pipe, steps_per_launch=L)
        out.append(o)
    for o in out[1:]:
        assert np.array_equal(out[0]["trace"], o["trace"])
        assert out[0]["counters"] == o["counters"]
        assert np.array_equal(out[0]["hits"], o["hits"])
        assert np.allclose(out[0]["rgba"], o["rgba"], rtol=1e-4, atol=1e-3)


@pytest.mark.parametrize("kind,seed,nx", [(1, 1, 8), (1, 9, 12), (0, 0, 0), (2, 4, 0), (3, 5, 0)])
def test_nonlinear_genomes_match_interpreter(rk, compiler, kind, seed, nx):
    W = H = 128
    f = rk.Flame.synthesize(compiler, kind, seed, W, H, n_xforms=nx, final_xform=(kind == 1),
                            force_parametric=(kind == 1 and nx >= 3))
    N, F, D = 8192, 20, 48
    a = _run(rk, f, N, W, H, F, D, 11, 1, trace=F + D)
    b = _run(rk, f, N, W, H, F, D, 11, -1, trace=F + D)
    c = _run(rk, f, N, W, H, F, D, 12, -1)
    assert np.array_equal(a["trace"], b["trace"])                       # xform-id streams
    assert a["counters"]["emitted"] == b["counters"]["emitted"]          # emitted draws
    same = np.array_equal(a["hits"], b["hits"])
    la, floor = _l1(a["hits"], b["hits"]), _l1(b["hits"], c["hits"])
    print("identical=%s L1 spec-vs-interp %.4g, interp two-seed %.4g" % (same, la, floor))
    assert same or la <= 1.5 * floor


@pytest.mark.parametrize("kind", [0, 3])
def test_interleaved_bin_records_equal_direct_planes(rk, compiler, kind):
    """Drawing through interleaved 32-byte records (merged into the caller's planes after each
    call) gives the direct planes' counts exactly, over two consecutive draw calls."""
    W = H = 256
    f = rk.Flame.synthesize(compiler, kind, 5, W, H)
    out = []
    for layout in (rk.BINS_DIRECT, rk.BINS_INTERLEAVED):
        sim = rk.Sim(8192, seed=4)
        sim.set_bin_layout(layout)
        sim.warmup(f, 19)
        bins, hits = _bins(W, H)
        sim.draw_to_bins(f, bins, hits, W, H, 20)
        sim.draw_to_bins(f, bins, hits, W, H, 20)
        out.append((bins.cpu().numpy(), hits.cpu().numpy()))
        sim.close()
    (b0, h0), (b1, h1) = out
    assert int(h0.sum()) > 0
    assert np.array_equal(h0, h1)
    assert np.allclose(b0, b1, rtol=1e-4, atol=1e-3)


@pytest.mark.parametrize("specialize", [0, -1])
def test_temporal_samples_with_rotation(rk, orc, compiler, specialize):
    """Motion blur (animate.tpl.glsl): 4 temporal samples whose xforms rotate by
    0.31415926535 * dt * rotation_frequency; the histogram against the FP32 oracle on the
    kernel's schedule is within the oracle's own seed-to-seed noise (the rotation's sin/cos are
    FP32 library calls on both sides, so trajectories are not bit-identical)."""
    xml = LINEAR.replace('linear="1"/>', 'linear="1" animate="1"/>', 1)
    f = rk.Flame.from_xml(xml, compiler)
    N, F, D, T, tss = 16384, 20, 32, 4, 0.5
    sim = rk.Sim(N, temporal_samples=T, seed=6, specialize=specialize, steps_per_launch=32)
    sim.warmup(f, F - 1, tss_width=tss)
    bins, hits = _bins(256, 256)
    sim.draw_to_bins(f, bins, hits, 256, 256, D)
    g = hits.cpu().numpy().astype(np.float64)
    og = orc.Genome(xml)
    refs = [og.chaos(N, 256, 256, fuse=F, draw=D, seed=s, temporal_samples=T, fp64=False, shuffle_mode=1,
                     cta_slots=4096, steps_per_launch=32, table_size=1024, tss_width=tss,
                     want_rgba=False)["hits"].astype(np.float64) for s in (6, 7, 8)]
    floor = np.mean([_l1(refs[1], refs[2])])
    l1 = _l1(g, refs[0])
    print("T=4 rotation: L1 gpu-vs-oracle(same seed) %.4g, oracle two-seed %.4g" % (l1, floor))
    assert l1 <= 1.5 * floor
    # static genome (no animate): the temporal samples do not rotate and stay bit-exact
    f2 = rk.Flame.from_xml(LINEAR, compiler)
    sim2 = rk.Sim(N, temporal_samples=T, seed=6, specialize=specialize, steps_per_launch=32)
    sim2.warmup(f2, F - 1, tss_width=tss)
    bins2, hits2 = _bins(256, 256)
    sim2.draw_to_bins(f2, bins2, hits2, 256, 256, D)
    r2 = orc.Genome(LINEAR).chaos(N, 256, 256, fuse=F, draw=D, seed=6, temporal_samples=T, fp64=False, shuffle_mode=1,
                                  cta_slots=4096, steps_per_launch=32, table_size=1024, tss_width=tss, want_rgba=False)
    assert np.array_equal(hits2.cpu().numpy().astype(np.uint64), r2["hits"])


def test_splat_strategies_after_warmup(rk, compiler):
    """The specialised kernel is compiled with the splat strategy set at warmup; setting another
    one afterwards switches to the kernel for it.  On an affine genome every strategy gives the
    same counts (the same trajectories) and colour sums equal up to FP32 summation order."""
    W = H = 128
    f = rk.Flame.from_xml(LINEAR, compiler)
    out = {}
    for mode in (rk.SPLAT_AUTO, rk.SPLAT_GLOBAL, rk.SPLAT_WARP):
        sim = rk.Sim(8192, seed=6)
        sim.set_splat(rk.SPLAT_AUTO)
        sim.warmup(f, 19)
        assert sim.specialized()
        sim.set_splat(mode)  # after warmup: the next draw fetches (or compiles) this strategy's kernel
        bins, hits = _bins(W, H)
        sim.draw_to_bins(f, bins, hits, W, H, 24)
        sim.draw_to_bins(f, bins, hits, W, H, 8)
        out[mode] = (bins.cpu().numpy(), hits.cpu().numpy())
        sim.close()
    b0, h0 = out[rk.SPLAT_AUTO]
    assert int(h0.sum()) > 0
    for mode, (b, h) in out.items():
        assert np.array_equal(h, h0), mode
        assert np.allclose(b, b0, rtol=1e-4, atol=1e-3), mode


@pytest.mark.parametrize("specialize,slots,tile,exchange", [(0, 2048, (20, 30, 70, 50), 2), (-1, 2048, (0, 50, 128, 30), 2),
                                                            (0, 4096, (40, 40, 32, 32), 2), (0, 2048, (0, 0, 0, 0), 2),
                                                            (0, 4096, (40, 40, 32, 32), 1), (0, 4096, (32, 50, 64, 20), 0)])
def test_tile_splat_bit_exact(rk, orc, compiler, specialize, slots, tile, exchange):
    """RF_SPLAT_TILE: the points inside the tile accumulate in each CTA's shared memory and reach
    the bins once per launch, the rest go straight to the L2.  On the affine genome the counts are
    bit-exact against the FP32 oracle on the kernel's shuffle schedule and the colour sums agree up
    to FP32 summation order, whatever the tile (part of the grid, a band, an empty tile) and the
    walker exchange (0 barrier, 1 pipelined, 2 chosen by timing)."""
    W = H = 128
    f = rk.Flame.from_xml(LINEAR, compiler)
    N, F, D = 8192, 20, 40
    sim = rk.Sim(N, seed=5, cta_slots=slots, specialize=specialize, steps_per_launch=32)
    sim.set_exchange(exchange)
    sim.set_splat(rk.SPLAT_TILE)
    sim.set_splat_tile(*tile)
    sim.warmup(f, F - 1)
    bins, hits = _bins(W, H)
    sim.draw_to_bins(f, bins, hits, W, H, D)
    r = orc.Genome(LINEAR).chaos(N, W, H, fuse=F, draw=D, seed=5, fp64=False, shuffle_mode=1, cta_slots=slots,
                                 steps_per_launch=32, table_size=1024)
    g = hits.cpu().numpy().astype(np.uint64)
    x0, y0, w, h = tile
    inside = int(g[y0:y0 + h, x0:x0 + w].sum())
    print("tile %s: %d of %d points inside" % (tile, inside, int(g.sum())))
    assert np.array_equal(g, r["hits"])
    assert np.allclose(bins.cpu().numpy(), r["rgba"], rtol=1e-4, atol=1e-3)
    if w * h:
        assert inside > 0
    sim.close()


@pytest.mark.parametrize("genome,W,H,want_tile", [("contract", 480, 270, True), ("frame1080", 1920, 1080, False)])
def test_auto_splat_fits_a_tile_to_compact_attractors(rk, compiler, genome, W, H, want_tile):
    """RF_SPLAT_AUTO fits a shared-memory tile after its first drawing launch of >= 32 passes
    when the hits concentrate (the contracting genome), times one launch through it against that
    first one and keeps it when faster — on the full GPU, by a wide margin for this genome — and
    fits none when the attractor is spread (the 1080p genome).  Counts never change: they equal
    a warp-aggregated run's on the same seed."""
    import os
    xml = open(os.path.join(os.path.dirname(__file__), "golden", "genomes", genome + ".flam3")).read()
    f = rk.Flame.from_xml(xml, compiler)
    N, F, D = 622592, 20, 3 * 256  # one 4096-slot CTA per SM
    out = {}
    for splat in (rk.SPLAT_AUTO, rk.SPLAT_WARP):
        sim = rk.Sim(N, seed=8)
        sim.set_splat(splat)
        sim.warmup(f, F - 1)
        bins, hits = _bins(W, H)
        sim.draw_to_bins(f, bins, hits, W, H, D)
        out[splat] = (hits.cpu().numpy(), sim.splat_tile())
        sim.close()
    tile = out[rk.SPLAT_AUTO][1]
    print(genome, "tile", tile)
    assert (tile is not None) == want_tile
    assert out[rk.SPLAT_WARP][1] is None
    if want_tile:
        assert tile[2] * tile[3] > 0 and tile[0] + tile[2] <= W and tile[1] + tile[3] <= H
    assert np.array_equal(out[rk.SPLAT_AUTO][0], out[rk.SPLAT_WARP][0])


def test_tile_splat_rejects_bad_tiles(rk, compiler):
    f = rk.Flame.from_xml(LINEAR, compiler)
    sim = rk.Sim(8192, seed=5, cta_slots=4096)
    sim.set_splat(rk.SPLAT_TILE)
    sim.warmup(f, 19)
    bins, hits = _bins(128, 128)
    sim.set_splat_tile(100, 0, 40, 10)  # beyond the grid's right edge
    with pytest.raises(rk.RefraktError) as e:
        sim.draw_to_bins(f, bins, hits, 128, 128, 4)
    assert e.value.status == 1
    sim.set_splat_tile(0, 0, 128, 100)  # 12,800 bins do not fit beside 4096 walker slots
    with pytest.raises(rk.RefraktError) as e:
        sim.draw_to_bins(f, bins, hits, 128, 128, 4)
    assert e.value.status == 5
    sim.close()
