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

Usage: python tests/golden/make_golden.py [reference_dir]
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


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("REFRAKT_REFERENCE", "/root/reference")
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
    path = os.path.join(HERE, "reference_vectors.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=0, sort_keys=True)
    print(path, len(cases), "variation cases")


if __name__ == "__main__":
    main()
