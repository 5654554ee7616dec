"""Host logic of the product library, through the C ABI, without a GPU: symbol exports, the
variation table, YAML and flam3 loading (including the reference's error behaviour), the
parameter buffer and layout, the screen affine, synthetic genomes, PNG output."""
import os
import re
import struct
import sys
import zlib

import numpy as np
import pytest

from conftest import REFERENCE, ROOT, reference_file


def _declared_symbols():
    with open(os.path.join(ROOT, "include", "refrakt.h")) as f:
        text = f.read()
    return sorted(set(re.findall(r"RF_API[^;(]*?\b(rf_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol(rk):
    names = _declared_symbols()
    assert len(names) >= 40
    lib = rk.library()
    for n in names:
        assert hasattr(lib, n), n
    assert lib.rf_abi_version() == 1


def test_registry_matches_reference_table(compiler, golden):
    c = compiler
    names = [e["name"] for e in golden["registry"]]
    assert sorted(c.variations()) == sorted(names)  # map order = sorted
    assert c.variations() == sorted(names)
    broken = set(golden["does_not_compile"])
    for e in golden["registry"]:
        assert c.is_variation(e["name"])
        assert c.get_parameters_for_variation(e["name"]) == e["params"]
        assert c.is_supported(e["name"]) == (e["name"] not in broken), e["name"]
        for p in e["params"]:
            assert c.is_param(p) and c.param_owner(p) == e["name"]
    for k in golden["common"]:
        assert c.is_common(k)
    assert not c.is_variation("x") and not c.is_param("linear") and not c.is_common("linear")


@pytest.mark.skipif(reference_file("variations.yaml") is None, reason="reference checkout absent")
def test_reference_yaml_loads_with_68_supported(rk):
    c = rk.FlameCompiler(os.path.join(REFERENCE, "variations.yaml"))
    vs = c.variations()
    assert len(vs) == 76
    assert sum(c.is_supported(v) for v in vs) == 68


def test_yaml_reconciliation(rk, tmp_path):
    y = tmp_path / "v.yaml"
    y.write_text(
        "common:\n  r: length($v)\n\n"
        "variations:\n"
        "  linear:\n    result: ($v)\n\n"
        "  # a parameter list that differs from the device implementation\n"
        "  julian:\n    param:\n      julian_power: {}\n    result: |-\n      $v\n\n"
        "  brand_new:\n    param:\n      brand_new_k: {}\n    flags: [no_weight_mul]\n    result: \"$v * 2.0\"\n"
        "  oscope:\n")
    c = rk.FlameCompiler(str(y))
    assert c.is_variation("linear") and c.is_supported("linear")
    assert c.is_variation("julian") and not c.is_supported("julian")
    assert c.is_variation("brand_new") and not c.is_supported("brand_new")
    assert c.is_param("brand_new_k") and c.param_owner("brand_new_k") == "brand_new"
    assert c.is_variation("oscope") and not c.is_supported("oscope")
    assert c.is_common("r") and not c.is_common("phi")
    xml = '<flame size="8 8" scale="1"><xform weight="1" color="0" color_speed="0" opacity="1" coefs="1 0 0 1 0 0" brand_new="1" brand_new_k="2"/></flame>'
    with pytest.raises(rk.RefraktError) as e:
        rk.Flame.from_xml(xml, c)
    assert e.value.status == 4  # UNSUPPORTED


def test_yaml_snippet_text_must_be_the_reference_formula(rk, tmp_path):
    """The kernels implement the reference's formulas, so a caller's entry is evaluated only when
    its snippet is the reference's text (whitespace aside); an edited body is unsupported
    (flame_compiler generates code from whatever the file says, variation_table.cpp:182-215)."""
    y = tmp_path / "v.yaml"
    y.write_text("variations:\n"
                 "  linear:\n    result: |-\n      (  $v\n      )\n"            # re-wrapped: the same formula
                 "  spherical:\n    result: $v * ($rsq + EPS)\n")                # edited
    c = rk.FlameCompiler(str(y))
    assert c.is_supported("linear")
    assert c.is_variation("spherical") and not c.is_supported("spherical")
    xml = '<flame size="8 8" scale="1"><xform weight="1" color="0" color_speed="0" opacity="1" coefs="1 0 0 1 0 0" spherical="1"/></flame>'
    with pytest.raises(rk.RefraktError) as e:
        rk.Flame.from_xml(xml, c)
    assert e.value.status == 4  # UNSUPPORTED


@pytest.mark.skipif(reference_file("variations.yaml") is None, reason="reference checkout absent")
def test_edited_reference_yaml_disables_only_the_edited_variation(rk, tmp_path):
    text = open(os.path.join(REFERENCE, "variations.yaml")).read()
    edited = text.replace("    result: $v / ($rsq + EPS)\n", "    result: $v / ($rsq + 2.0 * EPS)\n", 1)
    assert edited != text
    y = tmp_path / "variations.yaml"
    y.write_text(edited)
    c = rk.FlameCompiler(str(y))
    assert not c.is_supported("spherical")
    assert sum(c.is_supported(v) for v in c.variations()) == 67


@pytest.mark.skipif(reference_file("variations.yaml") is None, reason="reference checkout absent")
def test_snippet_hash_table_is_current():
    """refrakt_gb300/csrc/snippet_hashes.cpp holds the hashes gen_snippet_hashes.py computes from
    the reference's variations.yaml."""
    import re
    sys.path.insert(0, os.path.join(ROOT, "refrakt_gb300"))
    import gen_snippet_hashes
    h = gen_snippet_hashes.hashes(os.path.join(REFERENCE, "variations.yaml"))
    with open(os.path.join(ROOT, "refrakt_gb300", "csrc", "snippet_hashes.cpp")) as f:
        table = dict(re.findall(r'\{"(\w+)", 0x([0-9a-f]+)ull\}', f.read()))
    assert len(table) == 68
    for name, v in table.items():
        assert h[name] == v, name


def test_yaml_errors(rk, tmp_path):
    with pytest.raises(rk.RefraktError) as e:
        rk.FlameCompiler(str(tmp_path / "missing.yaml"))
    assert e.value.status == 8
    bad = tmp_path / "bad.yaml"
    bad.write_text("variations:\n  linear:\n      result: x\n   oops\n")
    with pytest.raises(rk.RefraktError) as e:
        rk.FlameCompiler(str(bad))
    assert e.value.status == 2


GENOME = ('<flame size="640 480" center="0.1 -0.2" scale="120" rotate="15" estimator_radius="7" '
          'estimator_minimum="1" estimator_curve="0.5" brightness="4" gamma="2.5" vibrancy="0.8">'
          '<xform weight="0.4" color="0.1" color_speed="0.7" opacity="1" animate="1" coefs="0.5 0.1 -0.2 0.6 0.3 -0.1" '
          'spherical="0.6" julian="0.4" julian_power="3" julian_dist="1" pre_blur="0.05"/>'
          '<xform weight="0.6" color="0.9" color_speed="0.3" opacity="0.5" coefs="-0.4 0.3 0.2 0.5 -0.6 0.2" '
          'post="1.1 0 0.1 0.9 0.05 0" pdj="0.7" pdj_a="1.1" pdj_b="-1.4" pdj_c="2" pdj_d="0.3" swirl="0.2"/>'
          '<finalxform color="0" color_speed="0" opacity="1" coefs="1 0 0 1 0 0" linear="1" radial_blur="0.1" radial_blur_angle="0.5"/>'
          '<color index="0" rgb="10.9 20 30"/><color index="255" rgb="255 128 1.99"/></flame>')


def test_flame_matches_oracle_layout(rk, orc, compiler):
    f = rk.Flame.from_xml(GENOME, compiler)
    o = orc.Genome(GENOME)
    assert np.array_equal(f.param_buffer(), o.param_buffer())
    info = f.info()
    assert info["num_xforms"] == 2 and info["has_final"]
    assert info["estimator_min"] == 1  # estimator_minimum accepted
    assert info["total_params"] == len(o.param_buffer())
    lay = f.param_layout()
    x0 = lay["xforms"][0]
    # map (alphabetical) order of variations and parameters, flame.cpp:47-50
    assert list(x0["variations"].keys()) == ["julian", "pre_blur", "spherical"]
    assert list(x0["param"].keys()) == ["julian_dist", "julian_power"]
    assert x0["meta"]["start"] == 0 and x0["weight"] == 0 and x0["affine"] == [1, 2, 3, 4, 5, 6]
    assert "post" in lay["xforms"][1] and "final_xform" in lay
    assert lay["size"] == info["total_params"]
    for w, h in [(640, 480), (1920, 1080), (17, 3)]:
        assert np.array_equal(np.array(f.screen_affine(w, h), np.float32), o.screen_affine(w, h))
    # palette: the integer part of each component / 256 (flame.cpp:217), as the XML writer
    # shows it (component x 256)
    xml = f.to_xml()
    for k, want in [(0, "10 20 30"), (255, "255 128 1")]:
        assert '<color index="%d" rgb="%s"' % (k, want) in xml
    assert f.xform_draws(0) == 1 + 5 and f.xform_draws(1) == 0 and f.xform_draws(-1) == 4
    assert [o.xform_draws(i) for i in (0, 1, -1)] == [6, 0, 4]


def test_flame_xml_round_trip(rk, orc, compiler):
    f = rk.Flame.from_xml(GENOME, compiler)
    x = f.to_xml()
    g = rk.Flame.from_xml(x, compiler)
    assert g.to_xml() == x
    assert np.array_equal(g.param_buffer(), f.param_buffer())
    assert np.array_equal(orc.Genome(x).param_buffer(), f.param_buffer())


@pytest.mark.parametrize("bad,status", [
    ('<flame size="8 8"><xform weight="1" coefs="1 0 0 1 0 0" linear="1" sparkle="1"/></flame>', 3),
    ('<flame size="8 8"><xform weight="1" coefs="1 0 0 1 0 0" linear="1" bent2="1" bent2_x="1" bent2_y="1"/></flame>', 4),
    ('<flame size="8 8"><xform weight="1" coefs="1 0 0 1 0 0" julian="1" julian_power="2"/></flame>', 1),
    ('<flame size="8 8"><xform weight="0" coefs="1 0 0 1 0 0" linear="1"/></flame>', 1),
    ('<flame size="8 8"><xform weight="1" coefs="1 0 0 1 0 0" pre_blur="1"/></flame>', 1),
    ('<flame size="8 8"><xform weight="1" coefs="1 0 0 1 0 0" linear="1"></flame>', 2),
    ('<flame size="8 8"><xform weight="1" coefs="1 0 0 1 0 0" linear="1"/><color index="300" rgb="1 2 3"/></flame>', 2),
    ('<notaflame/>', 2),
])
def test_flame_load_errors(rk, compiler, bad, status):
    with pytest.raises(rk.RefraktError) as e:
        rk.Flame.from_xml(bad, compiler)
    assert e.value.status == status


def test_parameter_buffer_capacity(rk, compiler):
    # 60 xforms x 20 floats > 1024 (fp[1024], flame.glsl:27)
    xf = '<xform weight="1" color="0" color_speed="0" opacity="1" coefs="1 0 0 1 0 0" post="1 0 0 1 0 0" linear="1"/>'
    with pytest.raises(rk.RefraktError) as e:
        rk.Flame.from_xml('<flame size="8 8">' + xf * 60 + "</flame>", compiler)
    assert e.value.status == 5


def test_flames_wrapper_and_hex_palette(rk, compiler):
    xml = ('<?xml version="1.0"?><!-- sheep --><flames><flame size="8 8" scale="2">'
           '<xform weight="1" color="0" color_speed="0" opacity="1" coefs="1 0 0 1 0 0" linear="1" symmetry="0.5"/>'
           '<palette count="2" format="RGB">FF0080\n102030</palette></flame></flames>')
    f = rk.Flame.from_xml(xml, compiler)
    lay = f.param_layout()
    buf = f.param_buffer()
    assert buf[lay["xforms"][0]["color_speed"]] == pytest.approx(0.25)


def test_edit_validation(rk, compiler):
    f = rk.Flame.from_xml(GENOME, compiler)
    before = f.param_buffer().copy()
    f.set_xform_value(0, "coefs4", 0.75)
    lay = f.param_layout()
    assert f.param_buffer()[lay["xforms"][0]["affine"][4]] == np.float32(0.75)
    with pytest.raises(rk.RefraktError):
        f.set_xform_value(0, "spherical_typo", 1.0)
    with pytest.raises(rk.RefraktError):
        f.set_xform_value(0, "bent2", 1.0)  # refused; the genome stays as it was
    after = f.param_buffer()
    assert len(after) == len(before)


SYNTH = [(0, 0, 512, 512, 0, False, False), (1, 1, 3840, 2160, 8, True, True), (2, 4, 1920, 1080, 0, False, False),
         (3, 5, 8192, 8192, 0, False, False), (1, 2, 512, 512, 4, False, False), (1, 3, 512, 512, 10, False, False)]


@pytest.mark.parametrize("kind,seed,w,h,nx,fin,force", SYNTH)
def test_synthetic_genomes(rk, orc, compiler, kind, seed, w, h, nx, fin, force):
    a = rk.Flame.synthesize(compiler, kind, seed, w, h, n_xforms=nx, final_xform=fin, force_parametric=force)
    b = rk.Flame.synthesize(compiler, kind, seed, w, h, n_xforms=nx, final_xform=fin, force_parametric=force)
    x = a.to_xml()
    assert x == b.to_xml()  # seeded, deterministic
    o = orc.Genome(x)  # the oracle reads the same genome through its own loader
    assert np.array_equal(a.param_buffer(), o.param_buffer())
    info = a.info()
    expect_nx = {0: 3, 2: 6, 3: 16}.get(kind, nx or 8)
    assert info["num_xforms"] == expect_nx and info["has_final"] == fin
    assert tuple(info["size"]) == (w, h)
    if force:
        lay = a.param_layout()
        assert "julian" in lay["xforms"][0]["variations"] and "ngon" in lay["xforms"][1]["variations"]
        assert "pdj" in lay["xforms"][2]["variations"]
        buf = a.param_buffer()
        jp = buf[lay["xforms"][0]["param"]["julian_power"]]
        assert jp == int(jp) and 2 <= jp <= 6


def test_png_writer(rk, tmp_path):
    img = (np.arange(7 * 5 * 4) % 251).astype(np.uint8).reshape(5, 7, 4)
    p = tmp_path / "t.png"
    rk.write_png(str(p), img)
    data = p.read_bytes()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat = 8, b""
    while pos < len(data):
        n = struct.unpack(">I", data[pos:pos + 4])[0]
        typ = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        assert struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])[0] == zlib.crc32(typ + body)
        if typ == b"IHDR":
            assert struct.unpack(">II", body[:8]) == (7, 5)
        if typ == b"IDAT":
            idat += body
        pos += 12 + n
    raw = zlib.decompress(idat)
    rows = [raw[i * (7 * 4 + 1) + 1:(i + 1) * (7 * 4 + 1)] for i in range(5)]
    assert np.array_equal(np.frombuffer(b"".join(rows), np.uint8).reshape(5, 7, 4), img)


def test_reference_fixture_genome(rk, orc, compiler):
    # the reference's flames/electricsheep.247.11256.flam3, copied by tests/golden/make_genomes.py
    path = os.path.join(ROOT, "tests", "golden", "genomes", "electricsheep.247.11256.flam3")
    f = rk.Flame.load_flame(path, compiler)
    with open(path) as fh:
        o = orc.Genome(fh.read())
    assert np.array_equal(f.param_buffer(), o.param_buffer())
    info = f.info()
    assert info["num_xforms"] == 10 and info["has_final"]
    assert tuple(info["size"]) == (800, 592) and info["estimator_radius"] == 11
    for w, h in [(1280, 720), (800, 592)]:
        assert np.array_equal(np.array(f.screen_affine(w, h), np.float32), o.screen_affine(w, h))


def test_no_device_is_reported(rk):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(rk.RefraktError) as e:
        rk.Sim(4096)
    assert e.value.status in (6, 9)


def test_interpolation_endpoints_and_midpoint(rk, compiler):
    a = rk.Flame.synthesize(compiler, rk.SYNTH_RANDOM, 2, 512, 512, n_xforms=4)
    b = rk.Flame.synthesize(compiler, rk.SYNTH_RANDOM, 3, 512, 512, n_xforms=10)
    f0, f1, fh = a.interpolate(b, 0.0), a.interpolate(b, 1.0), a.interpolate(b, 0.5)
    assert f0.info()["num_xforms"] == 10 and fh.info()["num_xforms"] == 10
    la, lb, l0, l1, lh = (x.param_layout() for x in (a, b, f0, f1, fh))
    pa, pb, p0, p1, ph = (x.param_buffer() for x in (a, b, f0, f1, fh))
    for i in range(10):
        for k in range(6):
            wa = pa[la["xforms"][i]["affine"][k]] if i < 4 else pb[lb["xforms"][i]["affine"][k]]
            wb = pb[lb["xforms"][i]["affine"][k]]
            assert p0[l0["xforms"][i]["affine"][k]] == pytest.approx(wa)
            assert p1[l1["xforms"][i]["affine"][k]] == pytest.approx(wb)
            assert ph[lh["xforms"][i]["affine"][k]] == pytest.approx(0.5 * (wa + wb), abs=1e-6)
        # xforms beyond a's four start at selection weight 0
        if i >= 4:
            assert p0[l0["xforms"][i]["weight"]] == 0.0
        for v, idx in l1["xforms"][i]["variations"].items():
            want = pb[lb["xforms"][i]["variations"][v]] if v in lb["xforms"][i]["variations"] else 0.0
            assert p1[idx] == pytest.approx(want, abs=1e-7)


def test_batch_rejects_bad_arguments_before_device_work(rk, compiler):
    import ctypes
    L = rk.library()
    h = ctypes.c_void_p()
    d = rk.BatchDesc(0, 0, 0, 1, 0.0, 1, 0)
    assert L.rf_batch_create(None, 0, ctypes.byref(d), ctypes.byref(h)) == 1
    f = rk.Flame.synthesize(compiler, rk.SYNTH_SMALL, 0, 64, 64)
    items = (rk.BatchItem * 1)(rk.BatchItem(f._h, 64, 64, 1, 0, 0))  # zero points
    assert L.rf_batch_create(items, 1, ctypes.byref(d), ctypes.byref(h)) == 1
    assert not h.value
    assert L.rf_batch_run(None) == 1 and L.rf_batch_sync(None, None) == 1
    assert L.rf_batch_destroy(None) == 0


def test_specialised_kernel_source_and_compile(rk, compiler):
    """The generated source names each xform's variations as constants and compiles for
    sm_103a with the run-time compiler (no device needed)."""
    f = rk.Flame.synthesize(compiler, rk.SYNTH_RANDOM, 1, 256, 256, n_xforms=8, final_xform=True, force_parametric=True)
    src = f.kernel_source(1024, 4096)
    lay = f.param_layout()
    nvar = sum(len(x["variations"]) for x in lay["xforms"]) + len(lay["final_xform"]["variations"])
    assert src.count("vary_impl(") == nvar  # one inlined call per (xform, variation)
    assert "case -1:" in src and "chaos_body<1024, 4, rfk::GenEval, -1, -1, 0>" in src
    assert f.kernel_source(1024, 4096) == src  # deterministic: the cache key
    g = rk.Flame.synthesize(compiler, rk.SYNTH_SMALL, 0, 256, 256)
    assert g.kernel_source(512, 2048).count("case ") == 2  # 3 xforms: cases 0, 1 and default
    assert f.kernel_compile(1024, 4096) > 10000
    assert g.kernel_compile(256, 256) > 10000


def test_genome_from_struct_equals_xml(rk, compiler):
    """rf_flame_from_struct builds the same genome (parameter buffer) as the flam3 loader."""
    xml = ('<flame size="256 192" center="0.1 -0.2" scale="50" rotate="10" gamma="2.2" brightness="4" '
           'vibrancy="1" estimator_radius="9" estimator_minimum="0" estimator_curve="0.4">'
           '<xform weight="0.5" color="0.2" color_speed="0.5" opacity="1" coefs="0.5 0.1 -0.1 0.5 0.2 0" '
           'linear="0.7" julian="0.3" julian_power="3" julian_dist="1"/>'
           '<xform weight="0.5" color="0.8" color_speed="0.4" opacity="0.9" coefs="-0.4 0 0.2 0.6 0 0.3" '
           'post="1 0 0 1 0.1 0" spherical="1"/>'
           '<finalxform color="0" color_speed="0" opacity="1" coefs="1 0 0 1 0 0" sinusoidal="1"/>'
           + "".join('<color index="%d" rgb="%d %d %d"/>' % (i, i, (3 * i) % 256, 255 - i) for i in range(256))
           + '</flame>')
    a = rk.Flame.from_xml(xml, compiler)
    pal = [(i / 256.0, ((3 * i) % 256) / 256.0, (255 - i) / 256.0) for i in range(256)]
    b = rk.Flame.from_struct(compiler, {
        "size": (256, 192), "center": (0.1, -0.2), "scale": 50, "rotate": 10, "estimator": (9, 0, 0.4),
        "gamma": 2.2, "vibrancy": 1, "brightness": 4, "palette": pal,
        "xforms": [
            {"weight": 0.5, "color": 0.2, "color_speed": 0.5, "opacity": 1, "coefs": (0.5, 0.1, -0.1, 0.5, 0.2, 0),
             "vars": {"linear": 0.7, "julian": 0.3}, "params": {"julian_power": 3, "julian_dist": 1}},
            {"weight": 0.5, "color": 0.8, "color_speed": 0.4, "opacity": 0.9, "coefs": (-0.4, 0, 0.2, 0.6, 0, 0.3),
             "post": (1, 0, 0, 1, 0.1, 0), "vars": {"spherical": 1}}],
        "final_xform": {"weight": 0, "color": 0, "color_speed": 0, "opacity": 1, "coefs": (1, 0, 0, 1, 0, 0),
                        "vars": {"sinusoidal": 1}}})
    assert np.array_equal(a.param_buffer(), b.param_buffer())
    assert a.param_layout() == b.param_layout()
    assert a.kernel_source() == b.kernel_source()
    with pytest.raises(rk.RefraktError):
        rk.Flame.from_struct(compiler, {"size": (8, 8), "scale": 1, "palette": pal,
                                        "xforms": [{"weight": 1, "coefs": (1, 0, 0, 1, 0, 0), "vars": {"nope": 1}}]})


def test_gemm_and_conv_validate_arguments_before_device_work(rk):
    # placeholder addresses (16-byte aligned, never dereferenced): every call below must be
    # refused by the argument checks, so no device is needed
    L = rk.library()
    P, Q = 1 << 20, 1 << 21
    INVALID = 1  # RF_ERR_INVALID_ARG
    f32, bf16, atomic = rk.GEMM_STORE_F32, rk.GEMM_STORE_BF16, rk.GEMM_ATOMIC_F32

    def gemm(A=P, B=Q, C=P, M=128, N=64, K=64, lda=64, ldb=64, ldc=64, mode=f32, splits=1):
        return L.rf_gemm_bf16(A, B, C, M, N, K, lda, ldb, ldc, mode, None, 0, splits, None)

    assert gemm(A=None) == INVALID
    assert gemm(M=0) == INVALID
    assert gemm(K=60, lda=64, ldb=64) == INVALID       # K not a multiple of 8
    assert gemm(lda=32) == INVALID                      # stride below K
    assert gemm(ldc=32) == INVALID                      # output rows narrower than N
    assert gemm(A=P + 8) == INVALID                     # operand not 16-byte aligned
    assert gemm(mode=7) == INVALID
    assert gemm(splits=4, mode=f32) == INVALID          # split K without atomic accumulation

    def conv(xa=P, ca=32, up=0, xb=None, cb=0, n=1, h=16, w=16, B=Q, N=32, ldb=288, C=P, ldc=32, mode=bf16):
        return L.rf_conv3x3_bf16(xa, ca, up, xb, cb, n, h, w, B, N, ldb, C, ldc, mode, None, 0, None)

    assert conv(xa=None) == INVALID
    assert conv(ca=12, ldb=108) == INVALID              # channels not a multiple of 8
    assert conv(cb=16) == INVALID                       # skip channels without a skip tensor
    assert conv(ldb=280) == INVALID                     # weights narrower than 9 (ca + cb)
    assert conv(ldc=16) == INVALID                      # output rows narrower than N
    assert conv(up=1, h=15) == INVALID                  # an upsampled input needs even h, w
    assert conv(h=70000) == INVALID                     # beyond the 16-bit row / column range
    assert conv(B=Q + 4) == INVALID                     # weights not 16-byte aligned
    assert conv(mode=9) == INVALID
    assert b"rf_conv3x3_bf16" in L.rf_last_error()


def test_sim_setters_and_queries_reject_null_handles(rk):
    """The Sim's tuning switches and queries check their arguments before touching a device."""
    import ctypes
    lib = rk.library()
    out = (ctypes.c_uint32 * 4)()
    assert lib.rf_set_exchange(None, rk.EXCHANGE_AUTO) == 1
    assert lib.rf_sim_exchange(None) == -1
    assert lib.rf_sim_splat_tile(None, out) == -1
    assert lib.rf_set_splat(None, rk.SPLAT_AUTO) == 1
    assert lib.rf_set_bad_value_reset(None, 1) == 1
