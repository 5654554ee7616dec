"""The oracle against the reference's own code (golden vectors from tests/golden/make_golden.py).

The reference has no tests; these pins come from compiling its own sources here: src/util.hpp
(jsf32 seeding), src/hammersley.cpp, the ranval/randf of shaders/include/random.glsl and every
variation snippet of variations.yaml.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import REFERENCE, ROOT


def test_jsf_warmup_matches_reference(orc, golden):
    for e in golden["jsf"]:
        assert orc.jsf_warmup(e["seed"]).tolist() == e["state"], e["seed"]


def test_glsl_randf_stream_matches_reference(orc, golden):
    for e in golden["jsf"]:
        vals, st = orc.randf_stream(np.array(e["state"], np.uint32), 8)
        assert vals.tolist() == [np.float32(v) for v in e["randf"]]
        assert st.tolist() == e["state_after_8"]
        # randf = float(u) / 2^32: never above 1, 1.0 reachable only when u rounds up to 2^32
        assert all(0.0 <= v <= 1.0 for v in vals)


def test_hammersley_matches_reference(orc, golden):
    for e in golden["hammersley"]:
        pts = orc.sample_points(e["count"])
        assert np.array_equal(pts[:, :2], np.array(e["xy"], np.float32)), e["count"]
        assert np.all(pts[:, 2:] == 0)


def _xform_xml(case):
    attrs = " ".join('%s="%.9g"' % (p, v) for p, v in case["params"].items())
    coefs = " ".join("%.9g" % v for v in case["affine"])
    extra = ' linear="1"' if case["pre_xform"] else ""
    return ('<flame size="16 16" scale="1"><xform weight="1" color="0.5" color_speed="0.5" opacity="1" '
            'coefs="%s" %s="%.9g"%s %s/></flame>' % (coefs, case["variation"], case["weight"], extra, attrs))


def test_variations_fp64_match_reference_snippets(orc, golden):
    """Every compiling variation, in FP64, against the reference snippet compiled as C++."""
    seen = set()
    for case in golden["variations"]:
        g = orc.Genome(_xform_xml(case))
        st = orc.jsf_warmup(case["seed"])[None, :]
        out, st2 = g.eval_xform(0, np.array([[case["xy"][0], case["xy"][1], 0.5]], np.float32), st)
        ref = np.array(case["value"])
        got = out[0, :2]
        both_bad = ~np.isfinite(ref) & ~np.isfinite(got)
        ok = both_bad | np.isclose(got, ref, rtol=1e-12, atol=1e-300)
        assert ok.all(), (case["variation"], got, ref)
        assert g.xform_draws(0) == case["draws"], case["variation"]
        assert st2[0].tolist() == case["state_after"], case["variation"]
        seen.add(case["variation"])
    assert len(seen) == 68


def test_broken_variations_do_not_load(orc, golden):
    assert len(golden["does_not_compile"]) == 8
    for name in golden["does_not_compile"]:
        xml = ('<flame size="16 16" scale="1"><xform weight="1" color="0" color_speed="0" opacity="1" '
               'coefs="1 0 0 1 0 0" linear="1" %s="0.5"/></flame>' % name)
        # parameters of the broken entries are accepted; the variation itself is refused
        with pytest.raises(ValueError):
            orc.Genome(xml)


@pytest.mark.skipif(not os.path.isfile(os.path.join(REFERENCE, "variations.yaml")), reason="reference checkout absent")
def test_golden_vectors_reproduce_from_reference(tmp_path, golden):
    """Regenerate the fixture from the reference checkout and compare with the committed copy."""
    env = dict(os.environ)
    r = subprocess.run([sys.executable, os.path.join(ROOT, "tests", "golden", "make_golden.py"), REFERENCE],
                       capture_output=True, text=True, env=env, cwd=ROOT)
    assert r.returncode == 0, r.stderr
    import json
    with open(os.path.join(ROOT, "tests", "golden", "reference_vectors.json")) as f:
        fresh = json.load(f)
    assert fresh == golden


# --------------------------------------------------------------------------------------------
# the reference's image shaders and shader templates, compiled here (make_golden.shader_vectors)
# --------------------------------------------------------------------------------------------
def test_tonemap_matches_reference_shader(orc, golden):
    """shaders/tonemap.glsl:18-38 per pixel.  The shader's literals (.5, log10 e) are FP32
    constants and the oracle's FP64, hence the 1e-7 relative tolerance."""
    for c in golden["tonemap"]:
        got = orc.tonemap(np.array(c["in"], np.float64).reshape(1, 1, 4), c["gamma"], c["brightness"],
                          c["vibrancy"], c["k2"])[0, 0]
        assert np.allclose(got, c["out"], rtol=1e-7, atol=1e-9), c


def test_density_radius_matches_reference_shader(orc, golden):
    """density_vert.glsl:35-44 max(min, min(R, int(R / pow(a, curve)))) with FP32 curves: the
    oracle's exact thresholds give the shader's radius for every density."""
    n = 0
    for c in golden["de_radius"]:
        for a, r in zip(c["a"], c["r"]):
            assert orc.de_radius(a, c["R"], c["min"], c["curve"]) == r, (c["R"], c["min"], c["curve"], a)
            n += 1
    assert n > 10000


def test_density_kernel_matches_reference_shaders(orc, golden):
    """density_vert.glsl:46-62 (norm_factor = 0.63661977236 / r^2; sprite size 2r + 1) and
    density_frag.glsl:9-18 (weight (1 - |2(pc + offset) - 1|^2) * norm_factor, discard beyond 1)
    at every sprite pixel's centre.  With the offset at zero the sprite is the oracle's symmetric
    disc exactly; the reference's own offset 1/(4r + 2) shifts it by half a pixel in the GL
    rasteriser (recorded here, not reproduced)."""
    for k in golden["de_kernel"]:
        r = k["r"]
        assert k["offset"] == pytest.approx([1.0 / (4 * r + 2), -1.0 / (4 * r + 2)])
        assert k["norm_factor"] == pytest.approx(0.63661977236 / (r * r), rel=1e-7)
        inside = 0
        for dx, dy, w in k["weights"]:
            ow = orc.de_weight(dx, dy, r)
            if w is None:
                assert ow < 0, (r, dx, dy)
            else:
                inside += 1
                assert ow == pytest.approx(w, rel=1e-7, abs=1e-12), (r, dx, dy)
        assert inside == sum(1 for dx in range(-r, r + 1) for dy in range(-r, r + 1)
                             if 4 * (dx * dx + dy * dy) <= (2 * r + 1) ** 2)


def test_xform_selection_matches_reference_template(orc, golden):
    """xform_select.tpl.glsl rendered for 2-12 xforms: the same xform for every draw, including
    draws on and one ulp either side of each cumulative-weight boundary (FP32 sums)."""
    for c in golden["xform_select"]:
        g = orc.Genome(c["xml"])
        lay = g.layout()
        fp = g.param_buffer()
        assert [float(fp[b["weight"]]) for b in lay["xforms"]] == c["weights"]
        got = [g.select(r) for r in c["r"]]
        assert got == c["id"], c["xml"][:80]


def test_animate_matches_reference_template(orc, golden):
    """animate.tpl.glsl: every temporal sample's parameters (affines rotated by
    0.31415926535 * dt * rotation_frequency).  The oracle rotates in FP32 as the shader does;
    the compiled template here in FP64.  The template does not copy rotation_frequency (the
    iterate shader never reads it), so those slots are left out of the comparison."""
    for c in golden["animate"]:
        with open(os.path.join(ROOT, "tests", "golden", "genomes", golden["animate_genomes"][c["genome"]])) as f:
            g = orc.Genome(f.read())
        lay = g.layout()
        blocks = lay["xforms"] + ([lay["final_xform"]] if "final_xform" in lay else [])
        keep = np.ones(lay["size"], bool)
        keep[[b["rotation_frequency"] for b in blocks]] = False
        got = g.animate_params(c["T"], c["tss_width"], c["t"])
        want = np.array(c["params"])
        assert np.allclose(got[keep], want[keep], rtol=2e-6, atol=2e-7), (c["genome"], c["T"], c["t"])
    # the reference genome's xforms carry animate="1": their affines do rotate
    c0 = [c for c in golden["animate"] if c["genome"] == 0 and c["t"] == 0][0]
    with open(os.path.join(ROOT, "tests", "golden", "genomes", golden["animate_genomes"][0])) as f:
        base = orc.Genome(f.read()).param_buffer()
    assert not np.allclose(base, c0["params"])
