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
