"""Generates tests/golden/reference_vectors.json from the reference's own code.

Runs only where the reference checkout exists: oracle/ref_build.py compiles the reference's
src/util.hpp (jsf32 seeding), src/hammersley.cpp (start points), the ranval/randf functions of
shaders/include/random.glsl and every variations.yaml snippet (through oracle/glsl_shim.h) into
oracle/_ref/libref.so, and this script records their outputs:

  jsf        warmup_ctx states and the GLSL stream (ranval words, randf values) per seed
  hammersley make_sample_points(count) for several counts
  registry   variation names, parameters, flags in variations.yaml order; the snippets that
             do not compile
  variations per compiling variation, cases of (point, affine, weight, parameters, RNG state)
             with the snippet's FP64 value, its RNG draw count and the state afterwards
  tonemap    shaders/tonemap.glsl on single pixels over gamma / brightness / vibrancy / k2
  de_radius  density_vert.glsl's estimator radius over densities, radii, minimums, FP32 curves
  de_kernel  density_vert.glsl's normalisation and density_frag.glsl's weight per sprite pixel,
             evaluated at each pixel's centre with the sprite offset set to zero
  xform_select  xform_select.tpl.glsl rendered for genomes of 2-12 xforms: the xform chosen
             for random draws and for draws on and next to every cumulative-weight boundary
  animate    animate.tpl.glsl rendered for two genomes: every temporal sample's parameters

Usage: python tests/golden/make_golden.py [reference_dir]
(default: $REFRAKT_REFERENCE, else <repo>/../reference)
"""
import ctypes
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle as O  # noqa: E402
import ref_build  # noqa: E402
import yaml_lite  # noqa: E402

CASES_PER_VARIATION = 8


def xform_xml(name, w, aff, params, pre):
    attrs = " ".join('%s="%.9g"' % (p, v) for p, v in params.items())
    coefs = " ".join("%.9g" % v for v in aff)
    extra = ' linear="1"' if pre else ""
    return ('<flame size="16 16" scale="1"><xform weight="1" color="0.5" color_speed="0.5" opacity="1" '
            'coefs="%s" %s="%.9g"%s %s/></flame>' % (coefs, name, w, extra, attrs))


def _f32(v):
    return float(np.float32(v))


def select_genome(n, rng):
    ws = rng.uniform(0.05, 1.0, n)
    body = "".join('<xform weight="%.9g" color="0" color_speed="0.5" opacity="1" coefs="1 0 0 1 0 0" linear="1"/>'
                   % w for w in ws)
    return '<flame size="16 16" scale="1">%s</flame>' % body


def shader_vectors(ref):
    """The reference's image shaders and shader templates compiled here (ref_build.build_shader_pins)."""
    rng = np.random.default_rng(20261204)
    sel_xml = [select_genome(n, rng) for n in range(2, 13)]
    with open(os.path.join(ROOT, "tests", "golden", "genomes", "electricsheep.247.11256.flam3")) as f:
        sheep = f.read()
    with open(os.path.join(ROOT, "tests", "golden", "genomes", "frame1080.flam3")) as f:
        frame = f.read()
    ani_xml = [sheep, frame]
    sel_g = [O.Genome(x) for x in sel_xml]
    ani_g = [O.Genome(x) for x in ani_xml]
    L = ctypes.CDLL(ref_build.build_shader_pins(ref, [g.layout() for g in sel_g], [g.layout() for g in ani_g]))
    dp = ctypes.POINTER(ctypes.c_double)
    L.ref_tonemap_pixel.argtypes = [ctypes.c_void_p] + [ctypes.c_double] * 4 + [ctypes.c_void_p]
    L.ref_de_vertex.argtypes = [ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                ctypes.POINTER(ctypes.c_int), dp, ctypes.c_void_p]
    L.ref_de_fragment.argtypes = [ctypes.c_int] + [ctypes.c_double] * 5 + [dp]
    out = {}
    # tonemap.glsl: bins with density (a = 0 divides 0 by 0 in the shader)
    tm = []
    for _ in range(256):
        a = _f32(10 ** rng.uniform(-2, 4))
        px = [_f32(a * rng.uniform(0, 1)) for _ in range(3)] + [a]
        g, b, v, k2 = _f32(rng.uniform(1, 4.5)), _f32(rng.uniform(0.5, 40)), _f32(rng.uniform(0, 1)), \
            _f32(10 ** rng.uniform(-5, 0))
        o = np.zeros(4)
        L.ref_tonemap_pixel(np.array(px).ctypes.data, g, b, v, k2, o.ctypes.data)
        tm.append({"in": px, "gamma": g, "brightness": b, "vibrancy": v, "k2": k2, "out": o.tolist()})
    out["tonemap"] = tm
    # density_vert.glsl: radius per density
    rad = []
    for R in (1, 2, 5, 9, 11, 20, 100):
        for mn in (0, 1, 3):
            for c in (0.4, 0.6, 1.0, 0.3, -0.5, 0.25, 2.0):
                c = _f32(c)
                dens = [float(k) for k in range(1, 400, 7)] + [_f32(x) for x in 10 ** rng.uniform(-3, 6, 24)]
                rs = []
                for a in dens:
                    r, nf, off = ctypes.c_int(), ctypes.c_double(), np.zeros(2)
                    L.ref_de_vertex(a, R, mn, c, ctypes.byref(r), ctypes.byref(nf), off.ctypes.data)
                    rs.append(r.value)
                rad.append({"R": R, "min": mn, "curve": c, "a": dens, "r": rs})
    out["de_radius"] = rad
    # density_vert.glsl normalisation and offset; density_frag.glsl weight at each sprite pixel's
    # centre (gl_PointCoord = (d + r + 0.5) / (2r + 1)) with the offset set to zero
    ker = []
    for r in range(1, 13):
        a = float(r)  # any density: the radius is forced through estimator_min = r, R = r
        rr, nf, off = ctypes.c_int(), ctypes.c_double(), np.zeros(2)
        L.ref_de_vertex(a, r, r, _f32(0.4), ctypes.byref(rr), ctypes.byref(nf), off.ctypes.data)
        ws = []
        for dy in range(-r - 1, r + 2):
            for dx in range(-r - 1, r + 2):
                w = ctypes.c_double()
                keep = L.ref_de_fragment(r, nf.value, 0.0, 0.0, (dx + r + 0.5) / (2 * r + 1),
                                         (dy + r + 0.5) / (2 * r + 1), ctypes.byref(w))
                ws.append([dx, dy, w.value if keep else None])
        ker.append({"r": rr.value, "norm_factor": nf.value, "offset": off.tolist(), "weights": ws})
    out["de_kernel"] = ker
    # xform_select.tpl.glsl
    sel = []
    for k, (x, g) in enumerate(zip(sel_xml, sel_g)):
        fp = g.param_buffer()
        fn = getattr(L, "ref_select_%d" % k)
        fn.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_float]
        lay = g.layout()
        cum = np.cumsum(np.array([fp[b["weight"]] for b in lay["xforms"]], np.float32), dtype=np.float32)
        draws = [_f32(v) for v in rng.uniform(0, 1, 48)] + [0.0, 1.0]
        for c in cum[:-1]:
            draws += [_f32(c), float(np.nextafter(np.float32(c), np.float32(0))),
                      float(np.nextafter(np.float32(c), np.float32(2)))]
        ids = [int(fn(fp.ctypes.data, len(fp), d)) for d in draws]
        sel.append({"xml": x, "weights": [float(fp[b["weight"]]) for b in lay["xforms"]], "r": draws, "id": ids})
    out["xform_select"] = sel
    # animate.tpl.glsl
    ani = []
    for k, (x, g) in enumerate(zip(ani_xml, ani_g)):
        fp = g.param_buffer()
        fn = getattr(L, "ref_animate_%d" % k)
        fn.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_void_p]
        for T, tss in ((32, 0.5), (64, 0.0416666667)):
            for t in (0, 1, T // 4, T // 2 - 1, T // 2, T - 1):
                o = np.zeros(len(fp), np.float32)
                fn(fp.ctypes.data, len(fp), T, t, tss, o.ctypes.data)
                ani.append({"genome": k, "T": T, "tss_width": tss, "t": t, "params": o.tolist()})
    out["animate"] = ani
    out["animate_genomes"] = ["electricsheep.247.11256.flam3", "frame1080.flam3"]
    return out


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else ref_build.reference_dir()
    if not ref_build.build(ref):
        sys.exit("reference checkout not found")
    O.build()
    R = O.ref_lib()
    out = {"source": "reference src/util.hpp, src/hammersley.cpp, shaders/include/random.glsl, variations.yaml"}

    # --- jsf32
    seeds = [0, 1, 2, 7, 255, 256, 65535, 65536, 123456789, 2**31 - 1, 2**31, 2**32 - 1]
    jsf = []
    for s in seeds:
        st = (ctypes.c_uint32 * 4)()
        R.ref_jsf_warmup(s, st)
        state = list(st)
        words, floats = [], []
        g = (ctypes.c_uint32 * 4)(*state)
        for _ in range(8):
            floats.append(float(R.ref_glsl_randf(g)))
        g2 = (ctypes.c_uint32 * 4)(*state)
        cpu = [int(R.ref_jsf_ranval_cpu(g2)) for _ in range(4)]
        jsf.append({"seed": s, "state": state, "randf": floats, "cpu_ranval": cpu, "state_after_8": list(g)})
    out["jsf"] = jsf

    # --- Hammersley start points
    ham = []
    for count in [2, 3, 8, 16, 100, 256, 1000, 4096]:
        buf = np.zeros((count, 4), np.float32)
        R.ref_sample_points(count, buf.ctypes.data_as(ctypes.c_void_p))
        ham.append({"count": count, "xy": buf[:, :2].tolist()})
    out["hammersley"] = ham

    # --- registry and the snippets that do not compile
    lib = yaml_lite.load(os.path.join(ref, "variations.yaml"))
    reg = []
    for name, d in lib["variations"].items():
        d = d or {}
        reg.append({"name": name, "params": list((d.get("param") or {}).keys()),
                    "flags": list(d.get("flags") or [])})
    out["registry"] = reg
    # FP32 library calls (sin, cos, pow, exp, log, atan, sqrt, ...) on each variation's path,
    # precalcs included: the error budget of a single step is counted in these
    common_calls = {"r": 1, "a": 1, "phi": 1, "sinr": 1, "cosr": 1}
    pat = re.compile(r"\b(sin|cos|tan|sincos|sinhcosh|sinh|cosh|pow|exp|log|log10|atan|sqrt|length)\s*\(")
    calls = {}
    for name, d in lib["variations"].items():
        d = d or {}
        text = (d.get("src") or "") + "\n" + (d.get("result") or "")
        used = set(re.findall(r"\$([a-z0-9_]+)", text))
        calls[name] = len(pat.findall(text)) + sum(common_calls.get(u, 0) for u in used)
    out["libm_calls"] = calls
    # FP32 arithmetic operators (+ - * /) in each variation's formula, precalcs included
    # (r = sqrt(x*x + y*y): 3, rsq: 3, sina / cosa = x / r: 1 each), numeric literals removed first
    common_ops = {"r": 3, "rsq": 3, "sina": 1, "cosa": 1}
    lit = re.compile(r"\b\d+\.?\d*(?:[eE][-+]?\d+)?[fF]?")
    arith = {}
    for name, d in lib["variations"].items():
        d = d or {}
        text = (d.get("src") or "") + "\n" + (d.get("result") or "")
        used = set(re.findall(r"\$([a-z0-9_]+)", text))
        arith[name] = len(re.findall(r"[-+*/]", lit.sub("0", text))) + sum(common_ops.get(u, 0) for u in used)
    out["arith_ops"] = arith
    out["common"] = list(lib["common"].keys())
    with open(os.path.join(O.HERE, "_ref", "broken.txt")) as f:
        out["does_not_compile"] = [ln.strip() for ln in f if ln.strip()]

    # --- variation snippets evaluated in FP64
    rng = np.random.default_rng(20261203)
    cases = []
    n = R.ref_var_count()
    for i in range(n):
        name = R.ref_var_name(i).decode()
        npar, pre, nowm, comp = (ctypes.c_int() for _ in range(4))
        R.ref_var_info(i, ctypes.byref(npar), ctypes.byref(pre), ctypes.byref(nowm), ctypes.byref(comp))
        if not comp.value:
            continue
        pnames = [r["params"] for r in reg if r["name"] == name][0]
        for k in range(CASES_PER_VARIATION):
            aff = rng.uniform(-1.5, 1.5, 6).astype(np.float32)
            w = np.float32(rng.uniform(0.2, 1.5))
            P = rng.uniform(-2.5, 2.5, len(pnames)).astype(np.float32)
            P = np.where(np.abs(P) < 0.3, np.float32(0.8), P).astype(np.float32)
            params = dict(zip(pnames, [float(v) for v in P]))
            xy = rng.uniform(-1.8, 1.8, 2).astype(np.float32)
            seed = int(rng.integers(0, 2**32 - 1))
            st0 = O.jsf_warmup(seed)
            # the post-affine point, in FP64 as the oracle and the reference prelude form it
            lin = O.Genome(xform_xml("linear", 1.0, aff, {}, False))
            p, _ = lin.eval_xform(0, np.array([[xy[0], xy[1], 0.5]], np.float32), st0[None, :])
            xp, yp = float(p[0, 0]), float(p[0, 1])
            st = (ctypes.c_uint32 * 4)(*[int(v) for v in st0])
            res = np.zeros(2)
            Pd = P.astype(np.float64)
            Cd = aff.astype(np.float64)
            draws = R.ref_vary(i, xp, yp, float(w), Pd.ctypes.data_as(ctypes.c_void_p),
                               Cd.ctypes.data_as(ctypes.c_void_p), st, res.ctypes.data_as(ctypes.c_void_p))
            value = [xp + res[0], yp + res[1]] if pre.value else [res[0], res[1]]
            cases.append({"variation": name, "xy": [float(xy[0]), float(xy[1])], "affine": [float(v) for v in aff],
                          "weight": float(w), "params": params, "seed": seed, "pre_xform": bool(pre.value),
                          "value": [float(v) for v in value], "draws": int(draws), "state_after": list(st)})
    out["variations"] = cases
    out.update(shader_vectors(ref))
    path = os.path.join(HERE, "reference_vectors.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=0, sort_keys=True)
    print(path, len(cases), "variation cases")


if __name__ == "__main__":
    main()
