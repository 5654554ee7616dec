"""Build recipe for oracle/_ref — the reference's own code compiled here (TEST INFRASTRUCTURE).

Compiles, from the sources where they lie in the reference checkout, into oracle/_ref/libref.so:
  * src/util.hpp (jsf32 seeding) and src/hammersley.cpp (start points), driven by
    oracle/ref_kat.cpp;
  * the GLSL of shaders/include/math.glsl, the ranval/randf functions of
    shaders/include/random.glsl and every variation snippet of variations.yaml, rewritten
    textually into C++ over oracle/glsl_shim.h.  The snippet rewrite applies the reference's
    own macro rules (src/util.cpp:6-9 replace_macro, src/variation_table.cpp:174-180 and
    :107-161): $x -> v.x, $y -> v.y, $v -> v.xy, $weight, parameters, precalcs.

Nothing generated here is committed (oracle/_ref is git-ignored).  Usage:
    python oracle/ref_build.py [reference_dir]
Exits 0 without building when the reference checkout is absent.
"""
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
sys.path.insert(0, HERE)
import yaml_lite  # noqa: E402

PRECALC_ORDER = ["r", "rsq", "a", "phi", "sina", "cosa", "sinr", "cosr"]


def replace_macro(s, name, value):
    # src/util.cpp:8 — "\$name([^a-zA-Z0-9_])" -> value + "$1"
    return re.sub(r"\$" + re.escape(name) + r"([^a-zA-Z0-9_])", lambda m: value + m.group(1), s)


def find_macros(s):
    return set(re.findall(r"\$([a-z0-9_]+)", s))


def default_replace_macros(s):
    # src/variation_table.cpp:174-180
    s = replace_macro(s, "x", "v.x")
    s = replace_macro(s, "y", "v.y")
    s = replace_macro(s, "v", "v.xy")
    s = replace_macro(s, "result", "result")
    return s


FLOAT_LIT = re.compile(r"(?<![\w.])((?:\d+\.\d*|\.\d+)(?:[eE][-+]?\d+)?|\d+[eE][-+]?\d+)[fF]?(?![\w.])")


def glsl_to_cpp(s, keep_float=False):
    if not keep_float:
        s = re.sub(r"\bfloat\b", "real", s)
    s = re.sub(r"\bv\.xy\b(?!\()", "v.xy()", s)
    s = re.sub(r"\.yx\b(?!\()", ".yx()", s)
    s = FLOAT_LIT.sub(lambda m: "F32(%s)" % m.group(1), s)
    return s


def sequence_randf(code):
    """Hoist the randf() calls of each statement into temporaries declared just before it, in
    textual (left-to-right) order — the order GLSL evaluates them in.  C++ leaves the order of
    operand evaluation unspecified, so without this a multi-draw expression would consume the
    RNG stream in a compiler-chosen order."""
    out = []
    stmt_start = 0
    counter = [0]
    i = 0
    pieces = []
    # split into statements at ';', '{' and '}' (kept with the preceding text)
    for j, ch in enumerate(code):
        if ch in ";{}":
            pieces.append(code[stmt_start:j + 1])
            stmt_start = j + 1
    pieces.append(code[stmt_start:])
    for piece in pieces:
        n = piece.count("randf()")
        if n == 0:
            out.append(piece)
            continue
        lead = len(piece) - len(piece.lstrip())
        decls = []
        body = piece
        for _ in range(n):
            name = "rnd_%d" % counter[0]
            counter[0] += 1
            decls.append("real %s = randf(); " % name)
            body = body.replace("randf()", name, 1)
        out.append(piece[:lead] + "".join(decls) + body[lead:])
    return "".join(out)


def extract_function(src, signature_regex):
    m = re.search(signature_regex, src)
    if not m:
        raise RuntimeError("function not found: " + signature_regex)
    i = src.index("{", m.start())
    depth = 0
    for j in range(i, len(src)):
        if src[j] == "{":
            depth += 1
        elif src[j] == "}":
            depth -= 1
            if depth == 0:
                return src[m.start():j + 1]
    raise RuntimeError("unbalanced braces")


def generate(ref, probe_dir=None):
    lib = yaml_lite.load(os.path.join(ref, "variations.yaml"))
    common = {k: default_replace_macros(v) for k, v in lib["common"].items()}
    math_glsl = open(os.path.join(ref, "shaders/include/math.glsl")).read()
    random_glsl = open(os.path.join(ref, "shaders/include/random.glsl")).read()

    out = []
    out.append("// GENERATED by oracle/ref_build.py from the reference checkout. Do not commit.")
    out.append('#include "glsl_shim.h"')
    out.append("#include <cstring>")
    out.append("namespace glsl {")
    out.append("// ---- shaders/include/math.glsl")
    out.append(glsl_to_cpp(math_glsl))
    out.append("// ---- shaders/include/random.glsl: state, rot32, ranval, randf")
    out.append("uvec4 local_random_state;")
    out.append("static int g_draws = 0;")
    m = re.search(r"#define rot32.*", random_glsl)
    out.append(m.group(0))
    ranval = extract_function(random_glsl, r"uint\s+ranval\s*\(\s*\)")
    out.append(ranval.replace("ranval()", "ranval_ref()", 1))
    out.append("uint ranval() { g_draws++; return ranval_ref(); }")
    randf = extract_function(random_glsl, r"float\s+randf\s*\(\s*\)")
    out.append(glsl_to_cpp(randf, keep_float=True))

    entries = []
    funcs = []
    for name, d in lib["variations"].items():
        d = d or {}
        src = default_replace_macros(d.get("src") or "")
        res = default_replace_macros(d.get("result") or "")
        params = list((d.get("param") or {}).keys())
        flags = set(d.get("flags") or [])
        if not res.strip():
            entries.append((name, None, params, flags))
            continue
        weight_str = "" if "no_weight_mul" in flags else "$weight *"
        code = (src + "\n" if src else "") + "vec2 result = " + weight_str + res + ";\n"
        code = replace_macro(code, "weight", "weight")
        for p in params:
            code = replace_macro(code, p, p)
        used = {m for m in find_macros(code) if m in common}
        for m in list(used):
            used |= {dd for dd in find_macros(common[m]) if dd in common}
        decls = ["real %s = %s;" % (p, glsl_to_cpp(common[p]).replace("$", "")) for p in PRECALC_ORDER if p in used]
        code = sequence_randf(code.replace("$", ""))
        fn = "var_" + name
        body = ["static vec2 %s(vin v, real weight, const real* P, const real* C) {" % fn,
                "  const real c00 = C[0], c01 = C[1], c10 = C[2], c11 = C[3], c20 = C[4], c21 = C[5];",
                "  (void)c00; (void)c01; (void)c10; (void)c11; (void)c20; (void)c21; (void)weight; (void)P;"]
        for i, p in enumerate(params):
            body.append("  const real %s = P[%d]; (void)%s;" % (p, i, p))
        body += ["  " + x for x in decls]
        body.append("  // variations.yaml: %s" % name)
        body += ["  " + ln for ln in glsl_to_cpp(code).split("\n")]
        body.append("  return result;")
        body.append("}")
        entries.append((name, fn, params, flags))
        funcs.append((name, "\n".join(body)))
    # Probe-compile every snippet on its own: the ones that do not compile as C++ are left out
    # of the table (and listed in broken.txt), mirroring the shader-compile failure that makes
    # the reference reject a genome using them (src/flame.cpp:222-225).
    prelude = "\n".join(out) + "\n"
    ok = set()
    if probe_dir is not None:
        from concurrent.futures import ThreadPoolExecutor

        def probe(item):
            nm, text = item
            path = os.path.join(probe_dir, "probe_%s.cpp" % nm)
            with open(path, "w") as f:
                f.write(prelude + text + "\n}\n")
            r = subprocess.run(["g++", "-std=c++20", "-fsyntax-only", "-w", "-I", HERE, path],
                               capture_output=True)
            os.remove(path)
            return nm, r.returncode == 0

        with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
            for nm, good in ex.map(probe, funcs):
                if good:
                    ok.add(nm)
    else:
        ok = {nm for nm, _ in funcs}
    for nm, text in funcs:
        if nm in ok:
            out.append(text)
    entries = [(n, fn if n in ok else None, pr, fl) for (n, fn, pr, fl) in entries]
    broken = sorted(n for (n, fn, pr, fl) in entries if fn is None)
    out.append("struct Entry { const char* name; vec2 (*fn)(vin, real, const real*, const real*); int nparams; int pre; int nowm; };")
    out.append("static const Entry kTable[] = {")
    for name, fn, params, flags in entries:
        out.append('  {"%s", %s, %d, %d, %d},' % (name, fn or "nullptr", len(params),
                                                  int("pre_xform" in flags), int("no_weight_mul" in flags)))
    out.append("};")
    out.append("}  // namespace glsl")
    out.append(r'''
extern "C" {
int ref_var_count() { return (int)(sizeof(glsl::kTable) / sizeof(glsl::kTable[0])); }
const char* ref_var_name(int i) { return glsl::kTable[i].name; }
int ref_var_info(int i, int* nparams, int* pre, int* nowm, int* compiled) {
    const auto& e = glsl::kTable[i];
    *nparams = e.nparams; *pre = e.pre; *nowm = e.nowm; *compiled = e.fn != nullptr;
    return 0;
}
// Evaluates one weighted variation term on the post-affine point (x, y).  st is the slot's
// JSF state (advanced in place).  Returns the number of ranval() calls, or -1.
int ref_vary(int i, double x, double y, double w, const double* P, const double* C, uint32_t* st, double* out) {
    const auto& e = glsl::kTable[i];
    if (!e.fn) return -1;
    glsl::local_random_state = glsl::uvec4{st[0], st[1], st[2], st[3]};
    glsl::g_draws = 0;
    glsl::vin v{x, y};
    glsl::vec2 r = e.fn(v, w, P, C);
    st[0] = glsl::local_random_state.x; st[1] = glsl::local_random_state.y;
    st[2] = glsl::local_random_state.z; st[3] = glsl::local_random_state.w;
    out[0] = r.x; out[1] = r.y;
    return glsl::g_draws;
}
float ref_glsl_randf(uint32_t* st) {
    glsl::local_random_state = glsl::uvec4{st[0], st[1], st[2], st[3]};
    float v = glsl::randf();
    st[0] = glsl::local_random_state.x; st[1] = glsl::local_random_state.y;
    st[2] = glsl::local_random_state.z; st[3] = glsl::local_random_state.w;
    return v;
}
}
''')
    return "\n".join(out) + "\n", broken


def build(ref=None, quiet=False):
    ref = ref or os.environ.get("REFRAKT_REFERENCE", "/root/reference")
    if not os.path.isfile(os.path.join(ref, "variations.yaml")):
        if not quiet:
            print("ref_build: reference checkout not found at %s; skipping oracle/_ref" % ref)
        return None
    os.makedirs(OUT, exist_ok=True)
    gen = os.path.join(OUT, "ref_glsl.cpp")
    text, broken = generate(ref, probe_dir=OUT)
    with open(gen, "w") as f:
        f.write(text)
    with open(os.path.join(OUT, "broken.txt"), "w") as f:
        f.write("\n".join(broken) + "\n")
    lib = os.path.join(OUT, "libref.so")
    cmd = ["g++", "-std=c++20", "-O1", "-fPIC", "-shared", "-w", "-ffp-contract=off",
           "-include", "cstdint", "-include", "array",
           "-I", HERE, "-I", os.path.join(ref, "src"),
           os.path.join(HERE, "ref_kat.cpp"), os.path.join(ref, "src", "hammersley.cpp"), gen,
           "-o", lib]
    subprocess.run(cmd, check=True)
    return lib


if __name__ == "__main__":
    p = build(sys.argv[1] if len(sys.argv) > 1 else None)
    if p:
        print(p)
