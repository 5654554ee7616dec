"""Build recipe for oracle/_ref — the reference's own code compiled here (TEST INFRASTRUCTURE).

Compiles, from the sources where they lie in the reference checkout, into oracle/_ref/libref.so:
  * src/util.hpp (jsf32 seeding) and src/hammersley.cpp (start points), driven by
    oracle/ref_kat.cpp;
  * the GLSL of shaders/include/math.glsl, the ranval/randf functions of
    shaders/include/random.glsl and every variation snippet of variations.yaml, rewritten
    textually into C++ over oracle/glsl_shim.h.  The snippet rewrite applies the reference's
    own macro rules (src/util.cpp:6-9 replace_macro, src/variation_table.cpp:174-180 and
    :107-161): $x -> v.x, $y -> v.y, $v -> v.xy, $weight, parameters, precalcs.

A second library, oracle/_ref/libref_shaders.so (build_shader_pins), compiles the reference's
whole image shaders and its shader templates the same way:
  * shaders/tonemap.glsl (the compute shader's main, image load/store stubbed);
  * shaders/density_vert.glsl and shaders/density_frag.glsl (the point-sprite radius, offset,
    normalisation and per-fragment kernel weight; projection and rasteriser stubbed);
  * shaders/templates/xform_select.tpl.glsl and animate.tpl.glsl rendered for given parameter
    layouts (oracle/inja_lite.py, the inja subset they use), as src/variation_table.cpp:260 and
    src/flame.cpp:334 render them.

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
# The reference checkout: $REFRAKT_REFERENCE, else a directory named `reference` beside this
# repository's root (<repo>/../reference).
DEFAULT_REFERENCE = os.path.join(os.path.dirname(HERE), os.pardir, "reference")


def reference_dir():
    return os.path.normpath(os.environ.get("REFRAKT_REFERENCE") or DEFAULT_REFERENCE)
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


# ---------------------------------------------------------------------------------------------
# whole shaders and shader templates
# ---------------------------------------------------------------------------------------------
def shader_to_cpp(src, name, keep_float=False):
    """A GLSL shader (or rendered template) as C++ over glsl_shim.h: the version line, layout
    qualifiers, storage-buffer blocks, image and interface declarations removed (the harness
    declares those globals), `uniform` declarations turned into globals, `discard` into a flag
    and a return, `.rgb` into the shim's accessors, main() renamed."""
    s = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    s = re.sub(r"//[^\n]*", "", s)
    s = re.sub(r"^\s*#version[^\n]*", "", s, flags=re.M)
    s = re.sub(r"layout\s*\([^)]*\)\s*buffer\s+\w+\s*\{[^}]*\}\s*;", "", s)
    s = re.sub(r"layout\s*\([^)]*\)\s*in\s*;", "", s)
    s = re.sub(r"layout\s*\([^)]*\)\s*uniform\s+image2D\s+\w+\s*;", "", s)
    s = re.sub(r"^\s*(flat\s+)?(in|out)\s+\w+\s+\w+\s*;", "", s, flags=re.M)
    s = re.sub(r"\buniform\s+", "", s)
    s = re.sub(r"\bdiscard\s*;", "{ g_discard = true; return; }", s)
    s = re.sub(r"(\w+)\.rgb\s*=\s*([^;]+);", r"\1.set_rgb(\2);", s)
    s = re.sub(r"(\w+)\.rgb\b", r"\1.rgb()", s)
    s = re.sub(r"\bvoid\s+main\s*\(\s*\)", "void %s_main()" % name, s)
    return glsl_to_cpp(s, keep_float=keep_float)


def shader_pins_source(ref, selects, animates):
    """C++ of the shader pins; `selects` and `animates` are parameter layouts (the reference's
    buffer_map_ JSON) to render xform_select.tpl.glsl and animate.tpl.glsl with."""
    import inja_lite
    rd = lambda p: open(os.path.join(ref, p)).read()
    out = ["// GENERATED by oracle/ref_build.py from the reference checkout. Do not commit.",
           '#include "glsl_shim.h"', "#include <cstring>"]
    # tonemap.glsl
    out += ["namespace glsl { namespace sh_tonemap {",
            "static uvec3 gl_GlobalInvocationID{0, 0, 0, {0, 0}};",
            "static int image_in = 0, image_out = 1; static vec4 g_in, g_out;",
            "static vec4 imageLoad(int, ivec2) { return g_in; }",
            "static void imageStore(int, ivec2, vec4 c) { g_out = c; }",
            shader_to_cpp(rd("shaders/tonemap.glsl"), "tonemap"), "}}"]
    # density_vert.glsl + density_frag.glsl: the vertex stage's flat outputs are the fragment
    # stage's inputs (radius, color, offset, norm_factor)
    out += ["namespace glsl { namespace sh_density {",
            "static int radius; static vec4 color; static vec2 offset; static real norm_factor;",
            "static vec4 outColor; static bool g_discard; static vec4 gl_Position; static real gl_PointSize;",
            "static vec2 gl_PointCoord; static int gl_VertexID = 0; static vec4 bins[1];",
            shader_to_cpp(rd("shaders/density_vert.glsl"), "vert"),
            shader_to_cpp(rd("shaders/density_frag.glsl"), "frag"), "}}"]
    sel_t = rd("shaders/templates/xform_select.tpl.glsl")
    for k, lay in enumerate(selects):
        out += ["namespace glsl { namespace sh_select%d { static float fp[4096];" % k,
                shader_to_cpp(inja_lite.render(sel_t, lay), "select", keep_float=True), "}}"]
    ani_t = rd("shaders/templates/animate.tpl.glsl")
    for k, lay in enumerate(animates):
        out += ["namespace glsl { namespace sh_animate%d {" % k,
                "static real fp[4096]; static real fp_inflated[1 << 17];",
                "static uvec3 gl_GlobalInvocationID, gl_NumWorkGroups, gl_WorkGroupSize;",
                shader_to_cpp(inja_lite.render(ani_t, lay), "animate"), "}}"]
    out.append('extern "C" {')
    out.append("""// tonemap.glsl on one pixel (k2 is the shader's scale_constant)
int ref_tonemap_pixel(const double* in, double gamma, double brightness, double vibrancy, double k2, double* o) {
    using namespace glsl::sh_tonemap;
    glsl::sh_tonemap::gamma = gamma; glsl::sh_tonemap::brightness = brightness;
    glsl::sh_tonemap::vibrancy = vibrancy;
    scale_constant = k2;
    g_in = glsl::vec4(in[0], in[1], in[2], in[3]);
    tonemap_main();
    o[0] = g_out.r; o[1] = g_out.g; o[2] = g_out.b; o[3] = g_out.a;
    return 0;
}
// density_vert.glsl for one bin of density a: returns 0 when the bin is culled (a == 0)
int ref_de_vertex(double a, int R, int minr, double curve, int* radius_out, double* norm_out, double* off_out) {
    using namespace glsl::sh_density;
    estimator_radius = R; estimator_min = minr; estimator_curve = curve; row_width = 1; height = 1;
    bins[0] = glsl::vec4(1.0, 1.0, 1.0, a);
    radius = -1;
    vert_main();
    if (radius < 0) return 0;
    *radius_out = radius; *norm_out = norm_factor; off_out[0] = offset.x; off_out[1] = offset.y;
    return 1;
}
// density_frag.glsl for a sprite of `radius` (bin colour 1, 1, 1, 1) at gl_PointCoord (pcx, pcy)
// with the vertex stage's offset; returns 0 when the fragment is discarded
int ref_de_fragment(int r, double nf, double offx, double offy, double pcx, double pcy, double* w) {
    using namespace glsl::sh_density;
    radius = r; norm_factor = nf; offset = glsl::vec2(offx, offy); color = glsl::vec4(1.0, 1.0, 1.0, 1.0);
    gl_PointCoord = glsl::vec2(pcx, pcy); g_discard = false;
    frag_main();
    if (g_discard) return 0;
    *w = outColor.a;
    return 1;
}""")
    for k in range(len(selects)):
        out.append("""int ref_select_%d(const float* fp, int n, float r) {
    std::memcpy(glsl::sh_select%d::fp, fp, sizeof(float) * n);
    return glsl::sh_select%d::get_xform_id(r);
}""" % (k, k, k))
    for k in range(len(animates)):
        out.append("""int ref_animate_%d(const float* fp, int n, int T, int t, float tss_width, float* o) {
    using namespace glsl::sh_animate%d;
    for (int i = 0; i < n; i++) glsl::sh_animate%d::fp[i] = fp[i];
    temporal_sample_width = tss_width;
    gl_NumWorkGroups = glsl::uvec3{(glsl::uint)(T / 32), 1, 1, {0, 0}};
    gl_WorkGroupSize = glsl::uvec3{32, 1, 1, {0, 0}};
    gl_GlobalInvocationID = glsl::uvec3{(glsl::uint)t, 0, 0, {(glsl::uint)t, 0}};
    animate_main();
    for (int i = 0; i < n; i++) o[i] = (float)fp_inflated[t * n + i];
    return 0;
}""" % (k, k, k))
    out.append("}")
    return "\n".join(out) + "\n"


def build_shader_pins(ref, selects, animates):
    """Compiles oracle/_ref/libref_shaders.so for these layouts; returns its path."""
    os.makedirs(OUT, exist_ok=True)
    gen = os.path.join(OUT, "ref_shaders.cpp")
    with open(gen, "w") as f:
        f.write(shader_pins_source(ref, selects, animates))
    lib = os.path.join(OUT, "libref_shaders.so")
    subprocess.run(["g++", "-std=c++20", "-O1", "-fPIC", "-shared", "-w", "-ffp-contract=off", "-I", HERE, gen,
                    "-o", lib], check=True)
    return lib


def build(ref=None, quiet=False):
    ref = ref or reference_dir()
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
