"""Parity of the CUDA path with the oracle and the reference's own code, through the C ABI.

  * xform-id streams: bit-exact with the reference RNG scheme (lane 0 of each 256-walker group
    draws, random-drawing variations and final xform included, T > 1 included);
  * emitted-point counts: exact;
  * a linear genome: bit-exact histogram counts against the FP32 oracle run on the kernel's
    documented shuffle schedule;
  * single-step xform outputs: within 4 FP32 ULP of the FP64 evaluation (norm-wise, see
    ulp_error) and with the RNG stream advanced exactly as the reference's;
  * histograms: relative L1 against the FP64 oracle within 1.5x the oracle's two-seed noise;
  * density estimation, tonemap, FP64 statistics, shuffle tables against the oracle.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _dev(a, dtype=None):
    t = torch.from_numpy(np.ascontiguousarray(a))
    if dtype is not None:
        t = t.view(dtype)
    return t.cuda()


def _l1(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.abs(a / a.sum() - b / b.sum()).sum())


def _bins(W, H):
    return torch.zeros(H, W, 4, device="cuda"), torch.zeros(H, W, dtype=torch.int32, device="cuda")


# --------------------------------------------------------------------------------------------
# exact pins
# --------------------------------------------------------------------------------------------
@pytest.mark.parametrize("seed,T", [(7, 1), (8, 2), (9, 1)])
def test_xid_stream_bit_exact(rk, orc, compiler, seed, T):
    f = rk.Flame.synthesize(compiler, rk.SYNTH_RANDOM, seed, 128, 128, n_xforms=7, final_xform=True,
                            force_parametric=True)
    N, F, D = 8192, 12, 29
    sim = rk.Sim(N, temporal_samples=T, cta_slots=1024, steps_per_launch=8, seed=seed)
    sim.enable_xid_trace(F + D)
    sim.warmup(f, F - 1)
    bins, hits = _bins(128, 128)
    sim.draw_to_bins(f, bins, hits, 128, 128, D)
    got = sim.read_xid_trace(F + D)
    want = orc.Genome(f.to_xml()).xid_sequence(N, F, D, seed=seed, temporal_samples=T)
    assert np.array_equal(got, want)
    assert len(np.unique(want)) == 7


def test_emitted_count_exact(rk, orc, compiler):
    xml = ('<flame size="64 64" scale="16"><xform weight="0.5" color="0" color_speed="0.5" opacity="1" '
           'coefs="0.5 0 0 0.5 0.2 0" linear="1"/><xform weight="0.3" color="1" color_speed="0.5" opacity="0" '
           'coefs="0.5 0 0 0.5 -0.2 0" linear="1"/><xform weight="0.2" color="1" color_speed="0.5" opacity="0.5" '
           'coefs="0.5 0.1 0 0.5 0 0.2" julia="1"/></flame>')
    f = rk.Flame.from_xml(xml, compiler)
    N, F, D = 4096, 5, 23
    sim = rk.Sim(N, seed=3, steps_per_launch=4)
    sim.warmup(f, F - 1)
    bins, hits = _bins(64, 64)
    drawn = sim.draw_to_bins(f, bins, hits, 64, 64, D)
    seq = orc.Genome(xml).xid_sequence(N, F, D, seed=3)
    c = sim.counters()
    assert c["emitted"] == int((seq[F:] != 1).sum()) * 256
    assert drawn == c["drawn"] == int(hits.sum().item())
    assert c["steps"] == N * (F + D)


LINEAR = ('<flame size="256 256" scale="64" center="0 0"><xform weight="0.5" color="0" color_speed="0.5" '
          'opacity="1" coefs="0.5 0 0 0.5 -0.5 0.3" linear="1"/><xform weight="0.3" color="1" color_speed="0.5" '
          'opacity="1" coefs="0.4 0.3 -0.3 0.4 0.5 0.2" linear="0.9"/><xform weight="0.2" color="0.5" '
          'color_speed="0.5" opacity="1" coefs="-0.5 0.1 0.2 0.6 0 -0.5" linear="1.1"/>'
          + "".join('<color index="%d" rgb="%d %d %d"/>' % (i, i, 255 - i, (i * 7) % 256) for i in range(256))
          + "</flame>")


@pytest.mark.parametrize("cta,L", [(4096, 32), (2048, 7), (1024, 16), (512, 5), (1024, 1)])
def test_linear_genome_histogram_bit_exact(rk, orc, compiler, cta, L):
    """Affine-only genome: every operation is an explicit FP32 fma/mul/add, so the CUDA kernel and
    the FP32 oracle on the same shuffle schedule produce the same walkers and the same counts."""
    f = rk.Flame.from_xml(LINEAR, compiler)
    N, F, D = 4096, 20, 40
    sim = rk.Sim(N, cta_slots=cta, steps_per_launch=L, seed=3)
    sim.warmup(f, F - 1)
    bins, hits = _bins(256, 256)
    sim.draw_to_bins(f, bins, hits, 256, 256, D)
    r = orc.Genome(LINEAR).chaos(N, 256, 256, fuse=F, draw=D, seed=3, fp64=False, shuffle_mode=1,
                                 cta_slots=cta, steps_per_launch=L, table_size=1024)
    g = hits.cpu().numpy().astype(np.uint64)
    assert int(r["hits"].sum()) > N * D // 2
    assert np.array_equal(g, r["hits"])
    # colour sums differ only by the order of the FP32 atomic additions
    assert np.allclose(bins.cpu().numpy(), r["rgba"], rtol=1e-4, atol=1e-3)


# --------------------------------------------------------------------------------------------
# single step against FP64
# --------------------------------------------------------------------------------------------
def ulp_error(gpu, ref):
    """Norm-wise error in FP32 ULPs of the result: |gpu - ref| / ulp(max(|ref|, 2^-16))."""
    err = np.hypot(gpu[:, 0] - ref[:, 0], gpu[:, 1] - ref[:, 1])
    mag = np.maximum(np.hypot(ref[:, 0], ref[:, 1]), 2.0 ** -16).astype(np.float32)
    return err / np.spacing(mag).astype(np.float64)


def _probe(rk, f, xi, xyc, st, first_run=False):
    d_in = _dev(xyc.astype(np.float32))
    d_rng = _dev(st.astype(np.uint32), torch.int32)
    d_out = torch.zeros(xyc.shape[0], 4, device="cuda")
    rk.probe_xform(f, xi, d_in, d_rng, d_out, first_run=first_run)
    return d_out.cpu().numpy().astype(np.float64), d_rng.cpu().numpy().view(np.uint32)


def _case_xml(case):
    attrs = " ".join('%s="%.9g"' % (p, v) for p, v in case["params"].items())
    coefs = " ".join("%.9g" % v for v in case["affine"])
    extra = ' linear="1"' if case["pre_xform"] else ""
    return ('<flame size="16 16" scale="1"><xform weight="1" color="0.5" color_speed="0.5" opacity="1" '
            'coefs="%s" %s="%.9g"%s %s/></flame>' % (coefs, case["variation"], case["weight"], extra, attrs))


def _within_tolerance(u_gpu, u_cpu32, calls):
    """Error budget of one step against FP64: 4 FP32 ULP per FP32 library call on the path
    (sin, cos, pow, exp, log, atan2, sqrt ...; each is itself accurate to 1-2 ULP), at least
    4 ULP; or, where an independent FP32 evaluation of the same formula (the oracle with the
    host's libm) is itself further from FP64 — the formula is ill-conditioned in FP32 at that
    point — within twice that distance."""
    return (u_gpu <= 4.0 * max(1, calls)) | (u_gpu <= 2.0 * u_cpu32)


def test_single_step_against_reference_snippets(rk, orc, compiler, golden):
    """Each of the 68 variations against the reference snippets' FP64 values (tests/golden)."""
    worst = {}
    n_flat = n_all = 0
    bad = []
    for case in golden["variations"]:
        xml = _case_xml(case)
        f = rk.Flame.from_xml(xml, compiler)
        st = orc.jsf_warmup(case["seed"])[None, :]
        xyc = np.array([[case["xy"][0], case["xy"][1], 0.5]])
        out, st2 = _probe(rk, f, 0, xyc, st)
        assert st2[0].tolist() == case["state_after"], case["variation"]
        ref = np.array([case["value"]])
        if not np.all(np.isfinite(ref)):
            continue
        c32, _ = orc.Genome(xml).eval_xform(0, xyc.astype(np.float32), st, fp64=False)
        u = float(ulp_error(out[:, :2], ref)[0])
        u32 = float(ulp_error(c32[:, :2], ref)[0])
        n_all += 1
        n_flat += u <= 4.0
        worst[case["variation"]] = max(worst.get(case["variation"], 0.0), u)
        if not _within_tolerance(u, u32, golden["libm_calls"][case["variation"]]):
            bad.append((case["variation"], u, u32))
    print("single-step within 4 ulp of FP64: %d / %d; worst: %s" % (n_flat, n_all, sorted(worst.items(), key=lambda kv: -kv[1])[:6]))
    assert not bad, bad
    assert n_flat / n_all >= 0.9


@pytest.mark.parametrize("seed", [11, 12])
def test_single_step_random_genomes(rk, orc, compiler, golden, seed):
    f = rk.Flame.synthesize(compiler, rk.SYNTH_RANDOM, seed, 256, 256, n_xforms=8, final_xform=True,
                            force_parametric=True)
    og = orc.Genome(f.to_xml())
    lay = f.param_layout()
    n = 2048
    rng = np.random.default_rng(seed)
    xyc = np.stack([rng.uniform(-1.5, 1.5, n), rng.uniform(-1.5, 1.5, n), rng.uniform(0, 1, n)], 1).astype(np.float32)
    st = np.stack([orc.jsf_warmup(i * 7 + seed) for i in range(n)]).astype(np.uint32)
    flat = []
    for xi in list(range(8)) + [-1]:
        block = lay["final_xform"] if xi < 0 else lay["xforms"][xi]
        calls = sum(golden["libm_calls"][v] for v in block["variations"])
        for first in (False, True):
            out, st2 = _probe(rk, f, xi, xyc, st, first_run=first)
            ref, rst = og.eval_xform(xi, xyc, st, first_run=first)
            c32, _ = og.eval_xform(xi, xyc, st, first_run=first, fp64=False)
            assert np.array_equal(st2, rst), (xi, first)
            fin = np.all(np.isfinite(ref[:, :2]), 1) & (np.hypot(ref[:, 0], ref[:, 1]) < 1e30)
            u = ulp_error(out[fin, :2], ref[fin, :2])
            u32 = ulp_error(c32[fin, :2], ref[fin, :2])
            ok = _within_tolerance(u, u32, calls)
            # a composed xform passes several arguments through floor/trunc/round/compare
            # (fan, rings2, ngon, julian, rectangles, boarders ...); when two FP32 evaluations
            # put such an argument on different sides of a step the outputs differ by the step.
            # These flips are allowed for 0.5 % of points.
            if ok.mean() < 1.0:
                i = np.argwhere(~ok)[:3, 0]
                print("xform %d beyond budget: gpu %s fp64 %s fp32 %s" % (xi, out[fin][i, :2], ref[fin][i, :2], c32[fin][i, :2]))
            assert ok.mean() >= 0.995, (xi, first, calls, np.percentile(u, [50, 99, 100]))
            flat.append(np.mean(u <= 4.0))
            # colour: one FP32 mul-mul-add; opacity copied
            assert np.allclose(out[:, 2], ref[:, 2], rtol=1e-6, atol=1e-7)
            assert np.array_equal(out[:, 3], ref[:, 3])
    print("fraction within a flat 4 ulp: %.4f" % np.mean(flat))


# --------------------------------------------------------------------------------------------
# statistics
# --------------------------------------------------------------------------------------------
@pytest.mark.parametrize("kind,seed,L", [(0, 0, 4), (0, 0, 32), (1, 1, 4)])
def test_histogram_l1_within_noise(rk, orc, compiler, kind, seed, L):
    W = H = 96
    f = rk.Flame.synthesize(compiler, kind, seed, W, H, n_xforms=6, final_xform=(kind == 1))
    og = orc.Genome(f.to_xml())
    N, F, D = 8192, 20, 48
    refs = [og.chaos(N, W, H, fuse=F, draw=D, seed=s, want_rgba=False)["hits"].astype(np.float64) for s in (101, 102, 103, 104)]
    floor = np.mean([_l1(refs[i], refs[j]) for i in range(4) for j in range(i + 1, 4)])
    gpus = []
    for s in (201, 202):
        sim = rk.Sim(N, seed=s, steps_per_launch=L)
        sim.warmup(f, F - 1)
        bins, hits = _bins(W, H)
        sim.draw_to_bins(f, bins, hits, W, H, D)
        gpus.append(hits.cpu().numpy().astype(np.float64))
    cross = np.mean([_l1(g, r) for g in gpus for r in refs])
    print("L1 gpu-vs-oracle %.4f, oracle two-seed floor %.4f (ratio %.2f)" % (cross, floor, cross / floor))
    assert cross <= 1.5 * floor


# --------------------------------------------------------------------------------------------
# image passes and helpers
# --------------------------------------------------------------------------------------------
@pytest.fixture(scope="module")
def small_hist(rk, compiler):
    W, H = 256, 192
    f = rk.Flame.synthesize(compiler, rk.SYNTH_SMALL, 0, W, H)
    sim = rk.Sim(65536, seed=1)
    sim.warmup(f, 19)
    bins, hits = _bins(W, H)
    sim.draw_to_bins(f, bins, hits, W, H, 16)
    return W, H, bins


@pytest.mark.parametrize("R,mn,curve", [(9, 0, 0.4), (3, 1, 0.6), (0, 0, 0.4), (20, 0, 0.3), (5, 2, -0.5), (4, 0, 0.0)])
def test_density_estimation_matches_oracle(rk, orc, small_hist, R, mn, curve):
    W, H, bins = small_hist
    out = torch.zeros_like(bins)
    rk.density_estimate(bins, W, H, R, mn, curve, out)
    torch.cuda.synchronize()
    # the curve is an FP32 uniform (density_vert.glsl:5); radii are exact functions of that value
    ref = orc.density_estimate(bins.cpu().numpy().astype(np.float64), R, mn, float(np.float32(curve)))
    got = out.cpu().numpy()
    assert np.allclose(got, ref, rtol=2e-5, atol=1e-4 * max(1.0, float(np.abs(ref).max()) * 1e-3))


@pytest.mark.parametrize("ss,k2", [(1, 1e-4), (2, 1e-2), (4, 0.0)])
def test_tonemap_matches_oracle(rk, orc, small_hist, ss, k2):
    W, H, bins = small_hist
    img = torch.zeros(H // ss, W // ss, 4, device="cuda")
    img8 = torch.zeros(H // ss, W // ss, 4, dtype=torch.uint8, device="cuda")
    rk.tonemap(bins, W, H, ss, 2.2, 4.0, 0.8, k2, img, img8)
    torch.cuda.synchronize()
    b = bins.cpu().numpy().astype(np.float64)
    kk = k2 if k2 > 0 else W * H / b[..., 3].sum()
    ref = orc.tonemap(b, 2.2, 4.0, 0.8, kk, ss=ss)
    assert np.allclose(img.cpu().numpy(), ref, atol=2e-5)
    assert np.max(np.abs(img8.cpu().numpy().astype(np.int32) - np.rint(ref * 255))) <= 1


@pytest.mark.parametrize("R,mn,curve,ss,k2", [(9, 0, 0.4, 1, 0.0), (9, 0, 0.4, 2, 0.0), (5, 1, 0.6, 4, 1e-3),
                                              (12, 0, 0.3, 8, 0.0), (3, 0, 0.5, 2, 1e-2), (20, 0, 0.3, 2, 0.0),
                                              (6, 0, 0.4, 3, 0.0), (0, 2, 0.4, 1, 0.0)])
def test_density_tonemap_matches_separate_passes(rk, small_hist, R, mn, curve, ss, k2):
    """rf_density_tonemap (the estimator's output tonemapped on chip, k2 from the radius pass's
    density sum) against rf_density_estimate followed by rf_tonemap; R = 20 and ss = 3 take the
    unfused sequence.  The density sums differ only in FP64 summation order."""
    W, H, bins = small_hist
    W, H = W - W % ss, H - H % ss
    b = bins[:H, :W].contiguous()
    de = torch.zeros_like(b)
    rk.density_estimate(b, W, H, R, mn, curve, de)
    want = torch.zeros(H // ss, W // ss, 4, device="cuda")
    want8 = torch.zeros(H // ss, W // ss, 4, dtype=torch.uint8, device="cuda")
    rk.tonemap(de, W, H, ss, 2.2, 4.0, 0.8, k2, want, want8)
    got = torch.zeros_like(want)
    got8 = torch.zeros_like(want8)
    rk.density_tonemap(b, W, H, R, mn, curve, ss, 2.2, 4.0, 0.8, k2, got, got8)
    torch.cuda.synchronize()
    assert np.allclose(got.cpu().numpy(), want.cpu().numpy(), atol=2e-6)
    d = np.abs(got8.cpu().numpy().astype(np.int32) - want8.cpu().numpy().astype(np.int32))
    assert d.max() <= 1 and (d > 0).mean() < 1e-3


@pytest.mark.parametrize("ss,radius,shape,k2", [(2, 1.0, 0, 0.0), (4, 1.0, 0, 1e-3), (1, 0.7, 0, 0.0), (3, 1.0, 3, 0.0),
                                               (2, 1.5, 2, 1e-2), (2, 1.0, 1, 0.0), (4, 2.5, 0, 0.0)])
def test_flam3_spatial_filter_matches_oracle(rk, orc, small_hist, ss, radius, shape, k2):
    """rf_tonemap_filter (flam3's filter / filter_shape, which the reference ignores) against the
    oracle's FP64 restatement: taps, window placement at the grid's edges, log scaling, finish."""
    W, H, bins = small_hist
    W, H = W - W % ss, H - H % ss
    b = bins[:H, :W].contiguous()
    img = torch.zeros(H // ss, W // ss, 4, device="cuda")
    img8 = torch.zeros(H // ss, W // ss, 4, dtype=torch.uint8, device="cuda")
    rk.tonemap_filter(b, W, H, ss, radius, shape, 2.2, 4.0, 0.8, k2, img, img8)
    torch.cuda.synchronize()
    bb = b.cpu().numpy().astype(np.float64)
    kk = k2 if k2 > 0 else W * H / bb[..., 3].sum()
    ref = orc.tonemap_filter(bb, ss, radius, shape, 2.2, 4.0, 0.8, kk)
    assert np.allclose(img.cpu().numpy(), ref, atol=2e-5)
    assert np.max(np.abs(img8.cpu().numpy().astype(np.int32) - np.rint(ref * 255))) <= 1
    # radius 0 is the ss x ss box of rf_tonemap
    box = torch.zeros_like(img)
    rk.tonemap_filter(b, W, H, ss, 0.0, shape, 2.2, 4.0, 0.8, k2, box, None)
    want = torch.zeros_like(img)
    rk.tonemap(b, W, H, ss, 2.2, 4.0, 0.8, k2, want, None)
    torch.cuda.synchronize()
    assert torch.equal(box, want)


def test_hist_stats_fp64(rk, small_hist):
    W, H, bins = small_hist
    st = rk.hist_stats(bins, W, H)
    a = bins.cpu().numpy()[..., 3].astype(np.float64)
    assert st["sum"] == pytest.approx(a.sum(), rel=1e-12)
    assert st["max"] == a.max() and st["nonzero"] == int((a > 0).sum())


@pytest.mark.parametrize("n", [1, 3, 256, 1000, 1024, 65536])
def test_shuffle_tables_are_permutations(rk, orc, n):
    count = 4
    out = torch.zeros(count * n, dtype=torch.int16, device="cuda")
    rk.shuffle_generate(n, count, 99, out)
    t = out.cpu().numpy().view(np.uint16).reshape(count, n).astype(np.int64)
    for k in range(count):
        assert sorted(t[k].tolist()) == list(range(n))
        key = orc.derive_key(99, k, 0, 3)
        assert [orc.feistel(j, n, key) for j in range(min(n, 64))] == t[k, :min(n, 64)].tolist()
