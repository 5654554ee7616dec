// CPU oracle for the fractal-flame chaos game — TEST INFRASTRUCTURE ONLY.
//
// A scalar C++ restatement of the reference renderer's arithmetic (untrioctium/refrakt):
//   shaders/flame.glsl, shaders/include/{random,math}.glsl, shaders/templates/*.tpl.glsl,
//   variations.yaml (as emitted by src/variation_table.cpp), src/flame.cpp, src/hammersley.cpp,
//   shaders/density_{vert,frag}.glsl, shaders/tonemap.glsl.
// Loaded only by the test suite, the smoke check and the benchmark's CPU-baseline leg.
// Built with -ffp-contract=off so that FP32 mode rounds every operation as written.

#include "oracle.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <random>
#include <string>
#include <thread>
#include <vector>

namespace {

// ---------------------------------------------------------------------------------------------
// JSF32 — shaders/include/random.glsl:29-41 (device), src/util.hpp:75-95 (host seeding)
// ---------------------------------------------------------------------------------------------
struct Jsf { uint32_t a, b, c, d; };

inline uint32_t rot32(uint32_t x, int k) { return (x << k) | (x >> (32 - k)); }

// random.glsl:30-37: the GLSL ranval returns the new `a` (util.hpp:87 returns `d`, but the host
// copy is only used to warm states, so its return value never reaches a walker).
inline uint32_t jsf_next(Jsf& s) {
    uint32_t e = s.a - rot32(s.b, 27);
    s.a = s.b ^ rot32(s.c, 17);
    s.b = s.c + s.d;
    s.c = s.d + e;
    s.d = e + s.a;
    return s.a;
}

// util.hpp:90-95
inline void jsf_warmup(Jsf& s, uint32_t seed) {
    s.a = 0xf1ea5eedu;
    s.b = s.c = s.d = seed;
    for (int i = 0; i < 20; i++) (void)jsf_next(s);
}

// random.glsl:39-41: clamp(float(u) / 4294967295.0f, 0, 1).  The FP32 literal 4294967295.0f
// is 2^32, so this is float(u) * 2^-32 and 1.0 is reachable.
inline float randf(Jsf& s) {
    float v = (float)jsf_next(s) / 4294967295.0f;
    return std::min(std::max(v, 0.0f), 1.0f);
}

// ---------------------------------------------------------------------------------------------
// hashing for the kernel's shuffle schedule (splitmix64 finaliser, Vigna; lowbias32, Wellons)
// ---------------------------------------------------------------------------------------------
inline uint64_t mix64(uint64_t x) {
    x ^= x >> 30; x *= 0xbf58476d1ce4e5b9ull;
    x ^= x >> 27; x *= 0x94d049bb133111ebull;
    x ^= x >> 31;
    return x;
}
inline uint32_t lowbias32(uint32_t x) {
    x ^= x >> 16; x *= 0x7feb352du;
    x ^= x >> 15; x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}
uint64_t derive_key(uint64_t seed, uint64_t a, uint64_t b, uint64_t tag) {
    uint64_t k = mix64(seed + 0x9e3779b97f4a7c15ull);
    k = mix64(k ^ (tag * 0xd1b54a32d192ed03ull));
    k = mix64(k ^ (a + 0x632be59bd9b4e019ull));
    k = mix64(k ^ (b + 0x8cb92ba72f3d8dd7ull));
    return k;
}
// 4-round balanced Feistel network on 2*h bits, cycle-walked into [0, n).
uint32_t feistel(uint32_t x, uint32_t n, uint64_t key) {
    if (n <= 1) return 0;
    uint32_t bits = 0;
    while ((1u << bits) < n) bits++;
    if (bits < 2) bits = 2;
    if (bits & 1) bits++;
    const uint32_t h = bits / 2, mask = (1u << h) - 1u;
    const uint32_t k0 = (uint32_t)key, k1 = (uint32_t)(key >> 32);
    const uint32_t k2 = lowbias32(k0 ^ 0x68e31da4u), k3 = lowbias32(k1 ^ 0xb5297a4du);
    const uint32_t ks[4] = {k0, k1, k2, k3};
    do {
        uint32_t L = x >> h, R = x & mask;
        for (int r = 0; r < 4; r++) {
            uint32_t f = lowbias32(R ^ ks[r]) & mask;
            uint32_t nl = R;
            R = L ^ f;
            L = nl;
        }
        x = (L << h) | R;
    } while (x >= n);
    return x;
}
enum : uint64_t { TAG_GLOBAL = 1, TAG_LOCAL = 2, TAG_TABLE = 3 };

// ---------------------------------------------------------------------------------------------
// Variation registry — names, parameters (variations.yaml order), flags, RNG draws per call.
// IDs are positions in variations.yaml:12-551.  `broken` entries fail to compile in the
// reference (see the file:line notes), so a genome that uses them fails to load.
// ---------------------------------------------------------------------------------------------
enum { FL_NO_WEIGHT_MUL = 1, FL_PRE_XFORM = 2 };
struct VarDef {
    const char* name;
    std::vector<const char*> params;
    int flags;
    int draws;
    bool broken;
};
const std::vector<VarDef>& registry() {
    static const std::vector<VarDef> t = {
        {"linear", {}, 0, 0, false},
        {"sinusoidal", {}, 0, 0, false},
        {"spherical", {}, 0, 0, false},
        {"swirl", {}, 0, 0, false},
        {"horseshoe", {}, 0, 0, false},
        {"polar", {}, 0, 0, false},
        {"handkerchief", {}, 0, 0, false},
        {"heart", {}, 0, 0, false},
        {"disc", {}, 0, 0, false},
        {"spiral", {}, 0, 0, false},
        {"hyperbolic", {}, 0, 0, false},
        {"diamond", {}, 0, 0, false},
        {"ex", {}, 0, 0, false},
        {"julia", {}, 0, 1, false},
        {"bent", {}, 0, 0, false},
        {"waves", {}, 0, 0, false},
        {"fisheye", {}, 0, 0, false},
        {"popcorn", {}, 0, 0, false},
        {"exponential", {}, 0, 0, false},
        {"power", {}, 0, 0, false},
        {"cosine", {}, 0, 0, false},
        {"rings", {}, 0, 0, false},
        {"fan", {}, 0, 0, false},
        {"blob", {"blob_high", "blob_low", "blob_waves"}, 0, 0, false},
        {"pdj", {"pdj_a", "pdj_b", "pdj_c", "pdj_d"}, 0, 0, false},
        {"fan2", {"fan2_x", "fan2_y"}, 0, 0, false},
        {"rings2", {"rings2_val"}, 0, 0, false},
        {"eyefish", {}, 0, 0, false},
        {"bubble", {}, 0, 0, false},
        {"perspective", {"perspective_angle", "perspective_dist"}, 0, 0, false},
        {"noise", {}, 0, 2, false},
        {"julian", {"julian_power", "julian_dist"}, 0, 1, false},
        {"juliascope", {"juliascope_power", "juliascope_dist"}, 0, 1, false},
        {"blur", {}, 0, 2, false},
        {"gaussian_blur", {}, 0, 5, false},
        {"radial_blur", {"radial_blur_angle"}, FL_NO_WEIGHT_MUL, 4, false},
        {"pie", {"pie_slices", "pie_rotation", "pie_thickness"}, 0, 3, false},
        {"ngon", {"ngon_power", "ngon_sides", "ngon_corners", "ngon_circle"}, 0, 0, false},
        {"curl", {"curl_c1", "curl_c2"}, 0, 0, false},
        {"rectangles", {"rectangles_x", "rectangles_y"}, 0, 0, false},
        {"arch", {}, 0, 1, false},
        {"tangent", {}, 0, 0, false},
        {"square", {}, 0, 2, false},
        {"rays", {}, 0, 1, false},
        {"blade", {}, 0, 1, false},
        {"secant2", {}, 0, 0, false},
        {"twintrian", {}, 0, 1, true},  // variations.yaml:283 uses undeclared `diff`
        {"cross", {}, 0, 0, false},
        {"disc2", {"disc2_rot", "disc2_twist"}, 0, 0, false},
        {"super_shape", {"super_shape_n1", "super_shape_n2", "super_shape_n3", "super_shape_m",
                         "super_shape_holes", "super_shape_rnd"}, 0, 1, false},
        {"flower", {"flower_holes", "flower_petals"}, 0, 1, false},
        {"conic", {"conic_holes", "conic_eccentricity"}, 0, 1, false},
        {"parabola", {"parabola_height", "parabola_width"}, 0, 2, false},
        {"bent2", {"bent2_x", "bent2_y"}, 0, 0, true},        // :337 ternary without `?`
        {"bipolar", {"bipolar_shift"}, 0, 0, true},           // :348 bare `y`
        {"boarders", {}, 0, 1, false},
        {"butterfly", {}, 0, 0, false},
        {"cell", {"cell_size"}, 0, 0, true},                  // :405-410 `cell.xy`, braces
        {"cpow", {"cpow_power", "cpow_r", "cpow_i"}, 0, 1, true},  // :423 undeclared cpow_vd
        {"curve", {"curve_xlength", "curve_ylength", "curve_xamp", "curve_yamp"}, 0, 0, false},
        {"edisc", {}, 0, 0, true},                            // :443 undeclared edisc_xmx
        {"foci", {}, 0, 0, false},
        {"oscope", {}, 0, 0, true},                           // :457 empty entry
        {"loonie", {}, 0, 0, false},
        {"exp", {}, 0, 0, false},
        {"log", {}, 0, 0, false},
        {"sin", {}, 0, 0, false},
        {"cos", {}, 0, 0, false},
        {"sinh", {}, 0, 0, false},
        {"pre_blur", {}, FL_PRE_XFORM, 5, false},
        {"waves2", {"waves2_scalex", "waves2_scaley", "waves2_freqx", "waves2_freqy"}, 0, 0, false},
        {"cylinder", {}, 0, 0, false},
        {"coth", {}, 0, 0, true},                             // :506 trailing `f`
        {"auger", {"auger_freq", "auger_scale", "auger_sym", "auger_weight"}, 0, 0, false},
        {"flux", {"flux_spread"}, 0, 0, false},
        {"mobius", {"mobius_re_a", "mobius_re_b", "mobius_re_c", "mobius_re_d", "mobius_im_a",
                    "mobius_im_b", "mobius_im_c", "mobius_im_d"}, 0, 0, false},
    };
    return t;
}
int var_id(const std::string& n) {
    const auto& t = registry();
    for (size_t i = 0; i < t.size(); i++) if (n == t[i].name) return (int)i;
    return -1;
}
bool is_param(const std::string& n) {
    for (const auto& v : registry())
        for (auto p : v.params) if (n == p) return true;
    return false;
}

// ---------------------------------------------------------------------------------------------
// Genome (src/flame.hpp:21-61) and its loader (src/flame.cpp:160-226)
// ---------------------------------------------------------------------------------------------
struct Xform {
    float affine[6] = {0, 0, 0, 0, 0, 0};
    bool has_post = false;
    float post[6] = {0, 0, 0, 0, 0, 0};
    std::map<std::string, float> vars;    // std::map: alphabetical, as the reference
    std::map<std::string, float> params;
    float weight = 0, color = 0, color_speed = 0, rotation_frequency = 0, opacity = 0;
    // resolved: variations in codegen order with their parameter values
    struct Term { int id; float w; std::vector<float> p; };
    std::vector<Term> pre, terms;
};

}  // namespace

struct orc_genome {
    std::vector<Xform> xf;
    bool has_final = false;
    Xform fin;
    float palette[256][4];
    unsigned size[2] = {0, 0};
    float center[2] = {0, 0};
    float scale = 0, rotate = 0;
    int est_min = 0, est_radius = 0;
    float est_curve = 0, gamma = 0, vibrancy = 0, brightness = 0;
    std::vector<float> norm_w;  // xform weight / sum (flame.cpp:78-82), FP32
};

namespace {

// -------- minimal XML reader (elements, attributes, comments, declarations) --------
struct XNode {
    std::string name;
    std::vector<std::pair<std::string, std::string>> attrs;
    std::vector<XNode> kids;
};
std::string xml_unescape(const std::string& s) {
    std::string o;
    for (size_t i = 0; i < s.size(); i++) {
        if (s[i] == '&') {
            size_t e = s.find(';', i);
            if (e != std::string::npos) {
                std::string ent = s.substr(i + 1, e - i - 1);
                if (ent == "amp") o += '&';
                else if (ent == "lt") o += '<';
                else if (ent == "gt") o += '>';
                else if (ent == "quot") o += '"';
                else if (ent == "apos") o += '\'';
                else o += s.substr(i, e - i + 1);
                i = e;
                continue;
            }
        }
        o += s[i];
    }
    return o;
}
struct XParser {
    const char* s;
    size_t n, i = 0;
    std::string err;
    void ws() { while (i < n && (unsigned char)s[i] <= ' ') i++; }
    bool skip_misc() {
        for (;;) {
            while (i < n && s[i] != '<') i++;
            if (i >= n) return false;
            if (!strncmp(s + i, "<!--", 4)) { const char* e = strstr(s + i, "-->"); if (!e) return false; i = e - s + 3; continue; }
            if (!strncmp(s + i, "<?", 2)) { const char* e = strstr(s + i, "?>"); if (!e) return false; i = e - s + 2; continue; }
            if (!strncmp(s + i, "<!", 2)) { while (i < n && s[i] != '>') i++; i++; continue; }
            return true;
        }
    }
    bool element(XNode& out) {
        if (s[i] != '<') { err = "expected <"; return false; }
        i++;
        size_t b = i;
        while (i < n && !isspace((unsigned char)s[i]) && s[i] != '>' && s[i] != '/') i++;
        out.name.assign(s + b, i - b);
        for (;;) {
            ws();
            if (i >= n) { err = "eof in tag"; return false; }
            if (s[i] == '/') { if (i + 1 < n && s[i + 1] == '>') { i += 2; return true; } err = "bad /"; return false; }
            if (s[i] == '>') { i++; break; }
            size_t ab = i;
            while (i < n && s[i] != '=' && !isspace((unsigned char)s[i])) i++;
            std::string an(s + ab, i - ab);
            ws();
            if (i >= n || s[i] != '=') { err = "attr without ="; return false; }
            i++; ws();
            if (i >= n || (s[i] != '"' && s[i] != '\'')) { err = "unquoted attr"; return false; }
            char q = s[i++];
            size_t vb = i;
            while (i < n && s[i] != q) i++;
            if (i >= n) { err = "eof in attr"; return false; }
            out.attrs.push_back({an, xml_unescape(std::string(s + vb, i - vb))});
            i++;
        }
        for (;;) {
            // children / text until </name>
            while (i < n && s[i] != '<') i++;
            if (i >= n) { err = "eof in element"; return false; }
            if (!strncmp(s + i, "</", 2)) {
                const char* e = strchr(s + i, '>');
                if (!e) { err = "eof in end tag"; return false; }
                i = e - s + 1;
                return true;
            }
            if (!strncmp(s + i, "<!--", 4) || !strncmp(s + i, "<?", 2) || !strncmp(s + i, "<!", 2)) { if (!skip_misc()) { err = "eof"; return false; } if (!strncmp(s + i, "</", 2)) continue; }
            XNode k;
            if (!element(k)) return false;
            out.kids.push_back(std::move(k));
        }
    }
};

template <size_t N, class Conv>
void parse_list(const std::string& in, float* out, Conv cv) {  // util.hpp:13-26 parse_strings
    size_t i = 0, k = 0;
    while (k < N) {
        while (i < in.size() && isspace((unsigned char)in[i])) i++;
        if (i >= in.size()) break;
        size_t b = i;
        while (i < in.size() && !isspace((unsigned char)in[i])) i++;
        out[k++] = cv(in.substr(b, i - b));
    }
}
float as_float(const std::string& v) { return (float)strtod(v.c_str(), nullptr); }

bool resolve_xform(Xform& x, std::string& err) {
    // codegen order (src/variation_table.cpp:107-123): map (alphabetical) order; pre_xform
    // variations go to the affine prelude, the rest accumulate into `result`.
    x.pre.clear(); x.terms.clear();
    for (const auto& [name, w] : x.vars) {
        int id = var_id(name);
        const VarDef& d = registry()[id];
        if (d.broken) { err = "variation '" + name + "' does not compile in the reference"; return false; }
        Xform::Term t{id, w, {}};
        for (auto p : d.params) {
            auto it = x.params.find(p);
            if (it == x.params.end()) { err = std::string("missing parameter ") + p; return false; }
            t.p.push_back(it->second);
        }
        if (d.flags & FL_PRE_XFORM) x.pre.push_back(t); else x.terms.push_back(t);
    }
    if (x.terms.empty()) { err = "xform without variations"; return false; }
    return true;
}

int load_genome(const char* xml, orc_genome* g, std::string& err) {
    XParser p{xml, strlen(xml)};
    XNode root;
    bool found = false;
    while (p.skip_misc()) {
        XNode top;
        if (!p.element(top)) { err = p.err; return -1; }
        if (top.name == "flame") { root = std::move(top); found = true; break; }
    }
    if (!found) { err = "no <flame> element"; return -1; }
    auto attr = [&](const XNode& nd, const char* k) -> std::string {
        for (auto& a : nd.attrs) if (a.first == k) return a.second;
        return "";
    };
    parse_list<2>(attr(root, "center"), g->center, [](const std::string& v) { return std::stof(v); });
    g->scale = as_float(attr(root, "scale"));
    g->rotate = as_float(attr(root, "rotate"));
    g->est_curve = as_float(attr(root, "estimator_curve"));
    g->est_min = atoi(attr(root, "estimator_min").c_str());
    g->est_radius = atoi(attr(root, "estimator_radius").c_str());
    g->brightness = as_float(attr(root, "brightness"));
    g->gamma = as_float(attr(root, "gamma"));
    g->vibrancy = as_float(attr(root, "vibrancy"));
    {
        float sz[2] = {0, 0};
        parse_list<2>(attr(root, "size"), sz, [](const std::string& v) { return (float)std::stoi(v); });
        g->size[0] = (unsigned)sz[0]; g->size[1] = (unsigned)sz[1];
    }
    memset(g->palette, 0, sizeof(g->palette));
    for (const auto& k : root.kids) {
        if (k.name == "xform" || k.name == "finalxform") {
            Xform x;
            for (const auto& [name, val] : k.attrs) {
                if (name == "weight") x.weight = as_float(val);
                else if (name == "color") x.color = as_float(val);
                else if (name == "color_speed") x.color_speed = as_float(val);
                // flame.cpp:190 compares the node name against "final_xform", which never
                // matches "finalxform": any animate > 0 gives rotation frequency 1.
                else if (name == "animate") x.rotation_frequency = (as_float(val) > 0 && k.name != "final_xform") ? 1.0f : 0.0f;
                else if (name == "opacity") x.opacity = as_float(val);
                else if (is_param(name)) x.params[name] = as_float(val);
                else if (var_id(name) >= 0) x.vars[name] = as_float(val);
                else if (name == "coefs") parse_list<6>(val, x.affine, [](const std::string& v) { return (float)std::stod(v); });
                else if (name == "post") { x.has_post = true; parse_list<6>(val, x.post, [](const std::string& v) { return (float)std::stod(v); }); }
                else { err = "unknown attribute " + name; return -1; }
            }
            if (!resolve_xform(x, err)) return -1;
            if (k.name == "finalxform") { g->fin = x; g->has_final = true; }
            else g->xf.push_back(x);
        } else if (k.name == "color") {
            unsigned long long idx = strtoull(attr(k, "index").c_str(), nullptr, 10);
            if (idx > 255) { err = "palette index out of range"; return -1; }
            float rgb[4] = {0, 0, 0, 0};
            try {
                parse_list<4>(attr(k, "rgb"), rgb, [](const std::string& v) { return std::stoi(v) / 256.0f; });
            } catch (...) { err = "bad rgb"; return -1; }
            for (int c = 0; c < 3; c++) g->palette[idx][c] = rgb[c];
            g->palette[idx][3] = 1.0f;
        }
    }
    if (g->xf.empty()) { err = "no xforms"; return -1; }
    float total = 0.0f;
    for (const auto& x : g->xf) total += x.weight;
    if (!(total > 0.0f)) { err = "total xform weight is not positive"; return -1; }
    g->norm_w.clear();
    for (const auto& x : g->xf) g->norm_w.push_back(x.weight / total);
    return 0;
}

// ---------------------------------------------------------------------------------------------
// Variations — variations.yaml:13-551 as emitted by variation_table.cpp:97-165.
// Literals are FP32 values, as in GLSL.  Each case names its yaml line.
// ---------------------------------------------------------------------------------------------
template <class T> struct P2 { T x, y; };
#define F32(v) ((T)(float)(v))

template <class T>
struct Pre {  // common precalcs, variations.yaml:1-9
    T x, y, r, rsq, a, phi, sina, cosa, sinr, cosr;
    void init(T vx, T vy) {
        x = vx; y = vy;
        r = std::sqrt(x * x + y * y);
        rsq = x * x + y * (y);
        a = std::atan2(x, y);
        phi = std::atan2(y, x);
        sina = x / r;
        cosa = y / r;
        sinr = std::sin(r);
        cosr = std::cos(r);
    }
};

template <class T> inline T mod2(T x, T y) { return x - y * std::trunc(x / y); }  // math.glsl:13-15
template <class T> inline T mix(T x, T y, T a) { return x * ((T)1 - a) + y * a; }

template <class T>
P2<T> vary(int id, const Pre<T>& c, T w, const float* aff, const float* pp, Jsf& rng) {
    const T PI = F32(3.141592653589793);
    const T EPS = F32(1e-10);
    const T x = c.x, y = c.y, r = c.r, rsq = c.rsq, a = c.a, phi = c.phi;
    const T sina = c.sina, cosa = c.cosa, sinr = c.sinr, cosr = c.cosr;
    auto P = [&](int i) { return (T)pp[i]; };
    auto A = [&](int i) { return (T)aff[i]; };  // c00 c01 c10 c11 c20 c21
    auto rnd = [&]() { return (T)randf(rng); };
    using std::sin; using std::cos; using std::exp; using std::log; using std::pow; using std::sqrt;
    switch (id) {
    case 0: return {x, y};                                             // linear :13-14
    case 1: return {sin(x), sin(y)};                                   // sinusoidal :16-17
    case 2: { T d = rsq + EPS; return {x / d, y / d}; }                // spherical :19-20
    case 3: { T c1 = sin(rsq), c2 = cos(rsq);                          // swirl :22-26
              return {c1 * x - c2 * y, c2 * x + c1 * y}; }
    case 4: { T d = r + EPS;                                           // horseshoe :28-29
              return {(x + y) * (x - y) / d, F32(2.0) * x * y / d}; }
    case 5: return {a / PI, r - (T)1};                                 // polar :31-32
    case 6: return {r * sin(a + r), r * cos(a - r)};                   // handkerchief :34-35
    case 7: return {r * sin(r * a), -(r * cos(r * a))};                // heart :37-38
    case 8: return {a * sin(r * PI) / PI, a * cos(r * PI) / PI};       // disc :40-41
    case 9: { T d = r + EPS; return {(cosa + sinr) / d, (sina - cosr) / d}; }  // spiral :43-44
    case 10: return {sina / (r + EPS), cosa * r};                      // hyperbolic :46-47
    case 11: return {sina * cosr, cosa * sinr};                        // diamond :49-50
    case 12: { T n0 = sin(a + r), n1 = cos(a - r);                     // ex :52-58
               T m0 = n0 * n0 * n0 * r, m1 = n1 * n1 * n1 * r;
               return {m0 + m1, m0 - m1}; }
    case 13: { T u = rnd(); T th = F32(0.5) * a + std::round(u) * PI;  // julia :60-62
               T s = sqrt(r); return {s * cos(th), s * sin(th)}; }
    case 14: return {(x < 0) ? F32(2.0) * x : x, (y < 0) ? y / F32(2.0) : y};  // bent :64-69
    case 15: return {x + A(2) * sin(y / (A(4) * A(4) + EPS)),          // waves :71-76
                     y + A(3) * sin(x / (A(5) * A(5) + EPS))};
    case 16: { T k = F32(2.0) / (r + (T)1); return {k * y, k * x}; }  // fisheye :78-79
    case 17: return {x + A(4) * sin(std::tan((T)3 * y)),               // popcorn :81-86
                     y + A(5) * sin(std::tan((T)3 * x))};
    case 18: { T e = exp(x - (T)1);                                    // exponential :88-89
               return {e * cos(PI * y), e * sin(PI * y)}; }
    case 19: { T k = pow(r, sina); return {k * cosa, k * sina}; }      // power :91-92
    case 20: return {cos(PI * x) * std::cosh(y), -sin(PI * x) * std::sinh(y)};  // cosine :94-95
    case 21: { T dx = A(4) * A(4) + EPS;                               // rings :97-100
               T k = mod2(r + dx, F32(2.0) * dx) - dx + r * ((T)1 - dx);
               return {k * cosa, k * sina}; }
    case 22: { T dx = PI * (A(4) * A(4) + EPS), dx2 = dx * F32(0.5);   // fan :102-108
               T fa = a;
               fa += (mod2(fa + A(5), dx) > dx2) ? -dx2 : dx2;
               return {r * cos(fa), r * sin(fa)}; }
    case 23: { T k = r * (P(1) + (P(0) - P(1)) * (F32(0.5) + F32(0.5) * sin(P(2) * a)));  // blob :110-115
               return {k * sina, k * cosa}; }
    case 24: return {sin(P(0) * y) - cos(P(1) * x), sin(P(2) * x) - cos(P(3) * y)};  // pdj :117-127
    case 25: { T dx = PI * (P(0) * P(0) + EPS), dx2 = F32(0.5) * dx;  // fan2 :129-141
               T fa = a;
               T t = a + P(1) - dx * std::floor((a + P(1)) / dx);
               if (t > dx2) fa = fa - dx2; else fa = fa + dx2;
               return {r * sin(fa), r * cos(fa)}; }
    case 26: { T dx = P(0) * P(0) + EPS;                               // rings2 :143-150
               T rr = r;
               rr += F32(-2.0) * dx * std::trunc((rr + dx) / (F32(2.0) * dx)) + rr * ((T)1 - dx);
               return {rr * sina, rr * cosa}; }
    case 27: { T k = F32(2.0) / (r + (T)1); return {k * x, k * y}; }  // eyefish :152-153
    case 28: { T d = std::fma(rsq, F32(0.25), (T)1); return {x / d, y / d}; }  // bubble :155-156
    case 29: { T d = P(1) - y * sin(P(0));                             // perspective :158-164
               return {x * P(1) / d, P(1) * cos(P(0)) * y / d}; }
    case 30: { T u1 = rnd(); T u2 = rnd(); T th = u2 * F32(2.0) * PI;  // noise :166-167
               return {x * u1 * cos(th), y * u1 * sin(th)}; }
    case 31: { T t = std::trunc(std::fabs(P(0)) * rnd());              // julian :169-180
               T k = pow(r, P(1) / P(0));
               T th = (phi + F32(2.0) * PI * t) / P(0);
               return {k * cos(th), k * sin(th)}; }
    case 32: { long long ti = (long long)std::trunc(std::fabs(P(0)) * rnd());  // juliascope :182-193
               T k = pow(r, P(1) / P(0));
               T sg = ((ti & 1) == 0) ? (T)1 : (T)-1;
               T th = (F32(2.0) * PI * (T)ti + sg * phi) / P(0);
               return {k * cos(th), k * sin(th)}; }
    case 33: { T u1 = rnd(); T u2 = rnd(); T th = u2 * F32(2.0) * PI;  // blur :195-196
               return {u1 * cos(th), u1 * sin(th)}; }
    case 34: { T s = rnd(); s = s + rnd(); s = s + rnd(); s = s + rnd(); s = s - F32(2.0);  // gaussian_blur :198-199
               T th = rnd() * F32(2.0) * PI;
               return {s * cos(th), s * sin(th)}; }
    case 35: { T ang = P(0) * PI / F32(2.0);                            // radial_blur :201-210
               T szx = sin(ang), szy = cos(ang);
               T s = rnd(); s = s + rnd(); s = s + rnd(); s = s + rnd();
               T rndg = w * (s - F32(2.0));
               T tx = sin(phi + szx * rndg), ty = cos(phi + szx * rndg);
               T rz = szy * rndg - (T)1;
               return {r * ty + rz * x, r * tx + rz * y}; }
    case 36: { T u1 = rnd(); T u2 = rnd(); T u3 = rnd();               // pie :212-217
               T th = P(1) + F32(2.0) * PI * (std::trunc(u2 * P(0) + F32(0.5)) + u3 * P(2)) / P(0);
               return {u1 * sin(th), u1 * cos(th)}; }
    case 37: { T rf = pow(rsq, P(0) * F32(0.5));                       // ngon :219-230
               T b = F32(2.0) * PI / (P(1) + EPS);
               T nphi = phi - (b * std::floor(a / b));
               if (nphi > b * F32(0.5)) nphi -= b;
               T k = (P(2) * ((T)1 / (cos(nphi) + EPS) - (T)1) + P(3)) / (rf + EPS);
               return {k * x, k * y}; }
    case 38: { T re = (T)1 + P(0) * x + P(1) * (x * x - y * y);       // curl :232-239
               T im = P(0) * y + F32(2.0) * P(1) * x * y;
               T d = re * re + im * im;
               return {(x * re + y * im) / d, (y * re - x * im) / d}; }
    case 39: return {(P(0) == 0) ? x : ((T)2 * std::floor(x / P(0)) + (T)1) * P(0) - x,  // rectangles :241-249
                     (P(1) == 0) ? y : ((T)2 * std::floor(y / P(1)) + (T)1) * P(1) - y};
    case 40: { T ang = rnd() * w * PI; T sx = sin(ang), cy = cos(ang);  // arch :251-254
               return {sx, sx * sx / cy}; }
    case 41: return {sin(x) / cos(y), std::tan(y)};                    // tangent :256-257
    case 42: { T u1 = rnd(); T u2 = rnd(); return {u1 - F32(0.5), u2 - F32(0.5)}; }  // square :259-260
    case 43: { T ang = w * rnd() * PI; T rr = w / (rsq + EPS);        // rays :262-266
               T k = std::tan(ang) * rr; return {k * cos(x), k * sin(y)}; }
    case 44: { T ang = rnd() * w * r; T sx = sin(ang), cy = cos(ang); // blade :268-271
               return {x * (cy + sx), x * (cy - sx)}; }
    case 45: { T cr = cos(w * r); T icr = (T)1 / cr;                   // secant2 :273-277
               return {x, icr + ((cr < 0) ? (T)1 : (T)-1)}; }
    case 47: { T s = x * x - y * y; T k = sqrt((T)1 / (s * s + EPS));  // cross :286-289
               return {x * k, y * k}; }
    case 48: { T tp = P(0) * PI;                                       // disc2 :291-301
               T ax = sin(P(1)), ay = cos(P(1));
               ay -= (T)1;
               T k = (T)1 + P(1) + ((P(1) > F32(2.0) * PI) ? F32(-2.0) : F32(2.0)) * PI;
               ax *= k; ay *= k;
               T tx = sin(tp * (x + y)), ty = cos(tp * (x + y));
               return {(tx + ay) * a / PI, (ty + ax) * a / PI}; }
    case 49: { T ang = P(3) * F32(0.25) * phi + PI * F32(0.25);      // super_shape :303-313
               T sx = sin(ang), cy = cos(ang);
               T u = rnd();
               T k = (mix(r, u, P(5)) - P(4)) *
                     pow(pow(std::fabs(cy), P(1)) + pow(std::fabs(sx), P(2)), (T)-1 / P(0)) / r;
               return {x * k, y * k}; }
    case 50: { T u = rnd(); T k = (u - P(0)) * cos(P(1) * phi) / r;   // flower :315-319
               return {x * k, y * k}; }
    case 51: { T u = rnd(); T k = (u - P(0)) * P(1) / ((T)1 + P(1) * x / r) / r;  // conic :321-325
               return {x * k, y * k}; }
    case 52: { T u1 = rnd(); T u2 = rnd();                             // parabola :327-331
               return {P(0) * sinr * sinr * u1, P(1) * cosr * u2}; }
    case 55: {                                                         // boarders :351-390
        T rx = std::round(x), ry = std::round(y);
        T ox = x - rx, oy = y - ry;
        const T h = F32(0.5), q = F32(0.25);
        if (rnd() >= F32(0.75)) return {ox * h + rx, oy * h + ry};
        if (std::fabs(ox) >= std::fabs(oy)) {
            if (ox > 0) return {ox * h + rx + q, oy * h + ry + q * oy / ox};
            return {ox * h + rx - q, oy * h + ry - q * oy / ox};
        }
        if (oy > 0) return {ox * h + rx + q * ox / oy, oy * h + ry + q};
        return {ox * h + rx - q * ox / oy, oy * h + ry - q};
    }
    case 56: { T y2 = F32(2.0) * y;                                    // butterfly :392-395
               T k = F32(1.3029400317411197908970256609023) * sqrt(std::fabs(x * y) / (EPS + x * x + y2 * y2));
               return {k * x, k * y2}; }
    case 59: return {x + P(2) * exp(-y * y / std::max(P(0) * P(0), F32(1e-20))),  // curve :425-435
                     y + P(3) * exp(-x * x / std::max(P(1) * P(1), F32(1e-20)))};
    case 61: { T ex = exp(x) * F32(0.5); T enx = F32(0.25) / ex;       // foci :450-455
               T sx = sin(y), cy = cos(y); T d = ex + enx - cy;
               return {(ex - enx) / d, sx / d}; }
    case 63: { T w2 = w * w;                                           // loonie :459-462
               T k = (rsq < w2) ? sqrt(w2 / rsq - (T)1) : (T)1;
               return {x * k, y * k}; }
    case 64: { T e = exp(x); return {e * cos(y), e * sin(y)}; }        // exp :464-465
    case 65: return {F32(0.5) * log(rsq), phi};                        // log :467-468
    case 66: return {sin(x) * std::cosh(y), cos(x) * std::sinh(y)};    // sin :470-471
    case 67: return {cos(x) * std::cosh(y), sin(x) * std::sinh(y)};    // cos :473-474
    case 68: { T sx = sin(y), cy = cos(y);                             // sinh :476-479
               return {std::sinh(x) * cy, std::cosh(x) * sx}; }
    case 69: { T s = rnd(); s = s + rnd(); s = s + rnd(); s = s + rnd(); s = s - F32(2.0);  // pre_blur :481-483
               T th = rnd() * F32(2.0) * PI;
               return {s * cos(th), s * sin(th)}; }
    case 70: return {x + P(0) * sin(y * P(2)), y + P(1) * sin(x * P(3))};  // waves2 :485-495
    case 71: return {sin(x), y};                                       // cylinder :497-498
    case 73: { T s = sin(x * P(0)), t = sin(y * P(0));                 // auger :508-519
               T dy = y + P(3) * (P(1) * s / F32(2.0) + std::fabs(y) * s);
               T dx = x + P(3) * (P(1) * t / F32(2.0) + std::fabs(x) * t);
               return {x + P(2) * (dx - x), dy}; }
    case 74: { T xpw = x + w, xmw = x - w;                             // flux :521-530
               T k = ((T)2 + P(0)) * sqrt(sqrt(y * y + xpw * xpw) / sqrt(y * y + xmw * xmw));
               T th = (std::atan2(y, xmw) - std::atan2(y, xpw)) * F32(0.5);
               return {k * cos(th), k * sin(th)}; }
    case 75: { T reu = P(0) * x - P(4) * y + P(1);                     // mobius :532-551
               T imu = P(0) * y + P(4) * x + P(5);
               T rev = P(2) * x - P(6) * y + P(3);
               T imv = P(2) * y + P(6) * x + P(7);
               T d = rev * rev + imv * imv;
               return {(reu * rev + imu * imv) / d, (imu * rev - reu * imv) / d}; }
    default: break;
    }
    return {(T)NAN, (T)NAN};
}

// ---------------------------------------------------------------------------------------------
// dispatch(): variation_table.cpp:97-165 (xform body) and :241-243 (colour, opacity)
// ---------------------------------------------------------------------------------------------
template <class T>
void dispatch(const Xform& xf, T& x, T& y, T& c, T& w, bool first_run, Jsf& rng) {
    const float* A = xf.affine;
    // affine prelude, :105 — fma(c00, x, fma(c10, y, c20)), fma(c01, x, fma(c11, y, c21))
    T vx = std::fma((T)A[0], x, std::fma((T)A[2], y, (T)A[4]));
    T vy = std::fma((T)A[1], x, std::fma((T)A[3], y, (T)A[5]));
    Pre<T> pc;
    for (const auto& t : xf.pre) {  // :115-117, `v.xy += $weight * <result>`
        pc.x = vx; pc.y = vy;
        P2<T> d = vary<T>(t.id, pc, (T)t.w, A, t.p.data(), rng);
        vx = vx + (T)t.w * d.x;
        vy = vy + (T)t.w * d.y;
    }
    pc.init(vx, vy);
    P2<T> res{0, 0};
    bool first = true;
    for (const auto& t : xf.terms) {  // :107-123
        P2<T> d = vary<T>(t.id, pc, (T)t.w, A, t.p.data(), rng);
        if (!(registry()[t.id].flags & FL_NO_WEIGHT_MUL)) { d.x = (T)t.w * d.x; d.y = (T)t.w * d.y; }
        if (first) { res = d; first = false; }
        else { res.x = res.x + d.x; res.y = res.y + d.y; }
    }
    if (xf.has_post) {  // :155-157
        const float* Q = xf.post;
        T px = std::fma((T)Q[0], res.x, std::fma((T)Q[2], res.y, (T)Q[4]));
        T py = std::fma((T)Q[1], res.x, std::fma((T)Q[3], res.y, (T)Q[5]));
        res.x = px; res.y = py;
    }
    // :242 — vec4(result, mix(first_run ? randf() : v.z, color, color_speed), opacity)
    T cin = first_run ? (T)randf(rng) : c;
    T cs = (T)xf.color_speed;
    T omcs = (T)((float)1.0f - xf.color_speed);
    if (sizeof(T) == 8) omcs = (T)1 - cs;
    c = cin * omcs + (T)xf.color * cs;
    x = res.x; y = res.y;
    w = (T)xf.opacity;
}

int xform_draws(const Xform& xf, bool first_run) {
    int n = 0;
    for (const auto& t : xf.pre) n += registry()[t.id].draws;
    for (const auto& t : xf.terms) n += registry()[t.id].draws;
    return n + (first_run ? 1 : 0);
}

// xform_select.tpl.glsl: sequential FP32 sum of normalised weights, first i with sum >= r,
// the last xform unconditional.
// math.glsl:22 badval, and the walker reset flame.glsl:68 keeps commented out: result.xyw =
// vec3(vec2(randf(), randf()) * 2.0 - 1.0, 0.0) when x or y is NaN or beyond +-1e10.  The FP32
// walker is tested in FP32, the FP64 oracle's in double.
template <class T>
bool reset_bad(T& x, T& y, T& w, Jsf& s) {
    auto bad = [](T v) { return !(std::fabs(v) <= (T)1e10f); };
    if (!(bad(x) || bad(y))) return false;
    float u1 = randf(s);
    float u2 = randf(s);
    x = (T)(u1 * 2.0f - 1.0f);
    y = (T)(u2 * 2.0f - 1.0f);
    w = 0;
    return true;
}

int select_xform(const orc_genome* g, float r) {
    const int n = (int)g->xf.size();
    float sum = 0.0f;
    for (int i = 0; i < n - 1; i++) {
        sum = (i == 0) ? g->norm_w[0] : sum + g->norm_w[i];
        if (sum >= r) return i;
    }
    return n - 1;
}

// animate.tpl.glsl:18-96: per temporal sample, rotate the linear part of each affine.
void animate(const orc_genome* g, uint32_t T_, float tss_width, std::vector<std::vector<Xform>>& xf,
             std::vector<Xform>& fin) {
    xf.assign(T_, g->xf);
    fin.assign(T_, g->fin);
    if (T_ < 2) return;  // T = 1: the template's dt = 0/0; this restatement uses dt = 0
    const int half = (int)(T_ / 2);
    const float rps = 0.31415926535f;
    for (uint32_t t = 0; t < T_; t++) {
        float dt = (float)((int)t - half) / (float)half * tss_width;
        auto rotate = [&](Xform& x) {
            float ang = rps * dt * x.rotation_frequency;
            float s = std::sin(ang), c = std::cos(ang);
            float a0 = x.affine[0], a1 = x.affine[1], a2 = x.affine[2], a3 = x.affine[3];
            x.affine[0] = a0 * c + a2 * s;
            x.affine[1] = a1 * c + a3 * s;
            x.affine[2] = a2 * c - a0 * s;
            x.affine[3] = a3 * c - a1 * s;
        };
        for (auto& x : xf[t]) rotate(x);
        if (g->has_final) rotate(fin[t]);
    }
}

// src/flame.hpp:97-128 and flame.cpp:289-296
void screen_affine(const orc_genome* g, uint32_t W, uint32_t H, float out[6]) {
    float a[6] = {1, 0, 0, 1, 0, 0};
    auto translate = [](float* m, float t0, float t1) {
        m[4] = m[0] * t0 + m[2] * t1 + m[4];
        m[5] = m[1] * t0 + m[3] * t1 + m[5];
    };
    translate(a, (float)W / 2.0f, (float)H / 2.0f);
    float s = g->scale * (float)H / (float)g->size[1];
    for (int i = 0; i < 4; i++) a[i] *= s;
    {
        float rad = 0.01745329251f * g->rotate;
        float sn = std::sin(rad), cs = std::cos(rad);
        float a0 = a[0], a1 = a[1], a2 = a[2], a3 = a[3];
        a[0] = a0 * cs + a2 * sn;
        a[1] = a1 * cs + a3 * sn;
        a[2] = a2 * cs - a0 * sn;
        a[3] = a3 * cs - a1 * sn;
    }
    translate(a, -g->center[0], -g->center[1]);
    memcpy(out, a, sizeof(a));
}

// hammersley.cpp:29-48
uint32_t rev32(uint32_t n) {
    n = (n << 16) | (n >> 16);
    n = ((n & 0x00ff00ffu) << 8) | ((n & 0xff00ff00u) >> 8);
    n = ((n & 0x0f0f0f0fu) << 4) | ((n & 0xf0f0f0f0u) >> 4);
    n = ((n & 0x33333333u) << 2) | ((n & 0xccccccccu) >> 2);
    n = ((n & 0x55555555u) << 1) | ((n & 0xaaaaaaaau) >> 1);
    return n;
}
uint32_t next_pow2(uint32_t v) {
    v--; v |= v >> 1; v |= v >> 2; v |= v >> 4; v |= v >> 8; v |= v >> 16; v++;
    return v;
}
void sample_point(uint32_t i, uint32_t count, float& x, float& y) {
    uint32_t mx = (count % 2 == 0) ? count : next_pow2(count);
    float inv = 1.0f / (float)mx;
    uint32_t v = mx, r = 0;
    while (v >>= 1) r++;
    x = (float)((double)((float)i * inv) * 2.0 - 1.0);
    uint32_t fb = (r == 0) ? 0u : (rev32(i) >> (32 - r));
    y = (float)((double)((float)fb * inv) * 2.0 - 1.0);
}

// sin and cos of t in [0, 1] for the first-pass jitter (flame.glsl:64, where t = sqrt(randf())):
// Taylor series about 0 through t^13 / t^14, Horner form, FP32 fma — below 1 ulp on [0, 1]
// and evaluated identically by the CUDA kernel, so the jittered start points agree bit for bit.
inline void jitter_sincos(float t, float& s, float& c) {
    const float t2 = t * t;
    float p = 1.0f / 6227020800.0f;          // 1/13!
    p = std::fma(p, t2, -1.0f / 39916800.0f); // 1/11!
    p = std::fma(p, t2, 1.0f / 362880.0f);    // 1/9!
    p = std::fma(p, t2, -1.0f / 5040.0f);     // 1/7!
    p = std::fma(p, t2, 1.0f / 120.0f);
    p = std::fma(p, t2, -1.0f / 6.0f);
    p = std::fma(p, t2, 1.0f);
    s = t * p;
    float q = -1.0f / 87178291200.0f;         // -1/14!
    q = std::fma(q, t2, 1.0f / 479001600.0f);  // 1/12!
    q = std::fma(q, t2, -1.0f / 3628800.0f);   // -1/10!
    q = std::fma(q, t2, 1.0f / 40320.0f);      // 1/8!
    q = std::fma(q, t2, -1.0f / 720.0f);
    q = std::fma(q, t2, 1.0f / 24.0f);
    q = std::fma(q, t2, -0.5f);
    c = std::fma(q, t2, 1.0f);
}

inline uint32_t palette_index(double c) {  // flame.glsl:84: min(255, uint(ceil(c * 255)))
    float v = std::ceil((float)c * 255.0f);
    if (!(v > 0.0f)) return 0;
    if (v >= 255.0f) return 255;
    return (uint32_t)v;
}

// ---------------------------------------------------------------------------------------------
// Chaos game — flame.glsl:41-90, flame.cpp:228-330
// ---------------------------------------------------------------------------------------------
// Permutation k of the CUDA kernel's shuffle table over a CTA's n slots (kernels.cu
// shuffle_table_kernel).  phases = S >= 3: the pipelined table, P = n/S slots per phase — the
// last phase's destinations [n-P, n) take the first P of a keyed order of [P, n) (never the
// previous pass's first phase), the first phase's destinations [0, P) the first P not yet taken of
// a keyed order of [0, n-P) (never its last phase), the middle destinations the rest in a keyed
// order of [0, n).
void shuffle_table(uint64_t seed, uint32_t k, uint32_t n, uint32_t phases, uint32_t* out) {
    const uint32_t P = phases >= 3 ? n / phases : 0;
    if (!P) {
        const uint64_t key = derive_key(seed, k, 0, TAG_TABLE);
        for (uint32_t j = 0; j < n; j++) out[j] = feistel(j, n, key);
        return;
    }
    std::vector<char> taken(n, 0);
    const uint64_t k3 = derive_key(seed, k, 3, TAG_TABLE), k1 = derive_key(seed, k, 1, TAG_TABLE),
                   k2 = derive_key(seed, k, 2, TAG_TABLE);
    for (uint32_t d = 0; d < P; d++) {
        const uint32_t src = P + feistel(d, n - P, k3);
        out[n - P + d] = src;
        taken[src] = 1;
    }
    uint32_t d = 0;
    for (uint32_t i = 0; i < n - P && d < P; i++) {
        const uint32_t src = feistel(i, n - P, k1);
        if (!taken[src]) { out[d++] = src; taken[src] = 1; }
    }
    d = P;
    for (uint32_t i = 0; i < n && d < n - P; i++) {
        const uint32_t src = feistel(i, n, k2);
        if (!taken[src]) { out[d++] = src; taken[src] = 1; }
    }
}

template <class T>
int chaos(const orc_genome* g, const orc_chaos_cfg* cfg, double* rgba, uint64_t* hits, uint8_t* trace,
          uint64_t* counters) {
    const uint64_t N = cfg->walkers;
    const uint32_t TS = std::max(1u, cfg->temporal_samples);
    if (N == 0 || N % TS) return -1;
    const uint64_t ppts = N / TS;
    if (ppts % 256) return -1;
    if (cfg->fuse_passes < 1) return -1;
    const uint64_t groups_ts = ppts / 256, groups = N / 256;
    const uint32_t W = cfg->width, H = cfg->height;
    const uint32_t passes = cfg->fuse_passes + cfg->draw_passes;
    if (cfg->shuffle_mode == 1) {
        if (cfg->cta_slots == 0 || ppts % cfg->cta_slots || cfg->steps_per_launch == 0 || cfg->table_size == 0) return -1;
    }

    std::vector<std::vector<Xform>> xf;
    std::vector<Xform> fin;
    animate(g, TS, cfg->tss_width, xf, fin);
    float ss[6];
    screen_affine(g, W, H, ss);

    std::vector<Jsf> rng(N);
    for (uint64_t i = 0; i < N; i++) jsf_warmup(rng[i], (uint32_t)(i + cfg->seed * N));
    std::vector<T> px(N), py(N), pc(N), nx(N), ny(N), nc(N);
    std::vector<float> sx(ppts), sy(ppts);
    for (uint64_t i = 0; i < ppts; i++) sample_point((uint32_t)i, (uint32_t)ppts, sx[i], sy[i]);

    // permutation sources
    std::mt19937_64 perm_rng(cfg->seed * 0x2545F4914F6CDD1Dull + 7);
    std::vector<uint32_t> shuf_in(ppts), shuf_out(ppts);
    std::vector<std::vector<uint32_t>> table;
    const uint32_t cs_ = cfg->cta_slots;
    if (cfg->shuffle_mode == 1) {
        table.assign(cfg->table_size, std::vector<uint32_t>(cs_));
        const uint64_t tseed = cfg->table_seed_set ? cfg->table_seed : cfg->seed;
        for (uint32_t k = 0; k < cfg->table_size; k++) shuffle_table(tseed, k, cs_, cfg->table_phases, table[k].data());
    }
    auto is_launch_start = [&](uint32_t p) {
        const uint32_t F = cfg->fuse_passes, L = cfg->steps_per_launch;
        return (p < F) ? (p % L == 0) : ((p - F) % L == 0);
    };
    std::vector<uint8_t> xid(groups);
    uint64_t drawn = 0, emitted = 0;
    std::vector<uint32_t> srcidx(N), dstidx(N);

    for (uint32_t p = 0; p < passes; p++) {
        const bool first = (p == 0), draw = (p >= cfg->fuse_passes);
        // source / destination slot of every walker for this pass
        if (cfg->shuffle_mode == 0) {
            for (uint64_t i = 0; i < ppts; i++) shuf_in[i] = (uint32_t)i;
            std::shuffle(shuf_in.begin(), shuf_in.end(), perm_rng);
            for (uint64_t i = 0; i < ppts; i++) shuf_out[i] = (uint32_t)i;
            if (!draw) std::shuffle(shuf_out.begin(), shuf_out.end(), perm_rng);  // random_write in fuse passes
            for (uint64_t t = 0; t < TS; t++)
                for (uint64_t j = 0; j < ppts; j++) {
                    srcidx[t * ppts + j] = shuf_in[j];
                    dstidx[t * ppts + j] = (uint32_t)(t * ppts + shuf_out[j]);
                }
        } else {
            const bool gstart = is_launch_start(p);
            const uint64_t chunks_ts = ppts / cs_;
            for (uint64_t t = 0; t < TS; t++) {
                uint64_t gkey = derive_key(cfg->seed, p, t, TAG_GLOBAL);
                for (uint64_t ch = 0; ch < chunks_ts; ch++) {
                    uint32_t k = (uint32_t)(derive_key(cfg->seed, p, t * chunks_ts + ch, TAG_LOCAL) % cfg->table_size);
                    for (uint32_t j = 0; j < cs_; j++) {
                        uint64_t gid = ch * cs_ + j;
                        srcidx[t * ppts + gid] = gstart ? feistel((uint32_t)gid, (uint32_t)ppts, gkey)
                                                        : (uint32_t)(ch * cs_ + table[k][j]);
                        dstidx[t * ppts + gid] = (uint32_t)(t * ppts + gid);
                    }
                }
            }
        }
        for (uint64_t t = 0; t < TS; t++) {
            for (uint64_t gid = 0; gid < ppts; gid++) {
                const uint64_t slot = t * ppts + gid;
                Jsf& s = rng[slot];
                const uint64_t grp = t * groups_ts + gid / 256;
                if (gid % 256 == 0) {  // flame.glsl:51-53, lane 0 draws for its workgroup
                    xid[grp] = (uint8_t)select_xform(g, randf(s));
                    if (trace) trace[(uint64_t)p * groups + grp] = xid[grp];
                }
                const uint32_t src = srcidx[slot];
                T x, y, c;
                if (first) {  // :58-65 — sample points, jitter
                    x = (T)sx[src]; y = (T)sy[src]; c = 0;
                    float u1 = randf(s);
                    float u2 = randf(s);
                    float A = u1 * 0.1f * 3.14159265358979f * 2.0f;
                    float sn, cs;
                    jitter_sincos(std::sqrt(u2), sn, cs);
                    x = (T)((float)x + A * sn);
                    y = (T)((float)y + A * cs);
                } else {
                    x = px[t * ppts + src]; y = py[t * ppts + src]; c = pc[t * ppts + src];
                }
                T w;
                dispatch<T>(xf[t][xid[grp]], x, y, c, w, first, s);
                if (cfg->badval_reset) reset_bad<T>(x, y, w, s);
                nx[dstidx[slot]] = x; ny[dstidx[slot]] = y; nc[dstidx[slot]] = c;
                if (draw) {
                    T dx = x, dy = y, dc = c, dw = w;
                    if (g->has_final) {  // flame.cpp:23
                        T fw;
                        dispatch<T>(fin[t], dx, dy, dc, fw, false, s);
                        dw = fw * w;
                    }
                    if (dw > 0) emitted++;
                    // flame.glsl:78-86
                    float fx = (float)dx, fy = (float)dy;
                    T sx_ = std::fma((T)ss[0], (T)fx, std::fma((T)ss[2], (T)fy, (T)ss[4]));
                    T sy_ = std::fma((T)ss[1], (T)fx, std::fma((T)ss[3], (T)fy, (T)ss[5]));
                    if (sizeof(T) == 8) {  // FP64 oracle keeps the walker in double
                        sx_ = std::fma((T)ss[0], dx, std::fma((T)ss[2], dy, (T)ss[4]));
                        sy_ = std::fma((T)ss[1], dx, std::fma((T)ss[3], dy, (T)ss[5]));
                    }
                    if (sx_ >= 0 && sy_ >= 0 && sx_ < (T)W && sy_ < (T)H && dw > 0) {
                        uint32_t bx = (uint32_t)std::floor(sx_), by = (uint32_t)std::floor(sy_);
                        uint64_t idx = (uint64_t)(H - by - 1) * W + bx;
                        uint32_t ci = palette_index((double)dc);
                        if (rgba) {
                            for (int k = 0; k < 3; k++) rgba[idx * 4 + k] += (double)g->palette[ci][k];
                            rgba[idx * 4 + 3] += (double)dw;
                        }
                        if (hits) hits[idx] += 1;
                        drawn++;
                    }
                }
            }
        }
        std::swap(px, nx); std::swap(py, ny); std::swap(pc, nc);
    }
    if (counters) { counters[0] = drawn; counters[1] = emitted; }
    return 0;
}

}  // namespace

// =============================================================================================
// C API
// =============================================================================================
extern "C" {

void orc_jsf_warmup(uint32_t seed, uint32_t st[4]) {
    Jsf s; jsf_warmup(s, seed);
    st[0] = s.a; st[1] = s.b; st[2] = s.c; st[3] = s.d;
}
uint32_t orc_jsf_next(uint32_t st[4]) {
    Jsf s{st[0], st[1], st[2], st[3]};
    uint32_t v = jsf_next(s);
    st[0] = s.a; st[1] = s.b; st[2] = s.c; st[3] = s.d;
    return v;
}
float orc_randf(uint32_t st[4]) {
    Jsf s{st[0], st[1], st[2], st[3]};
    float v = randf(s);
    st[0] = s.a; st[1] = s.b; st[2] = s.c; st[3] = s.d;
    return v;
}
void orc_sample_points(uint32_t count, float* out4) {
    for (uint32_t i = 0; i < count; i++) {
        sample_point(i, count, out4[4 * i], out4[4 * i + 1]);
        out4[4 * i + 2] = 0; out4[4 * i + 3] = 0;
    }
}
uint32_t orc_feistel(uint32_t x, uint32_t n, uint64_t key) { return feistel(x, n, key); }
uint64_t orc_derive_key(uint64_t seed, uint64_t a, uint64_t b, uint64_t tag) { return derive_key(seed, a, b, tag); }
void orc_shuffle_table(uint32_t n, uint32_t count, uint64_t seed, uint32_t phases, uint32_t* out) {
    for (uint32_t k = 0; k < count; k++) shuffle_table(seed, k, n, phases, out + (size_t)k * n);
}

int orc_genome_from_xml(const char* xml, orc_genome** out, char* err, int errlen) {
    auto* g = new orc_genome();
    std::string e;
    int rc = -1;
    try { rc = load_genome(xml, g, e); } catch (const std::exception& ex) { e = ex.what(); rc = -1; }
    if (rc != 0) {
        if (err && errlen > 0) snprintf(err, errlen, "%s", e.c_str());
        delete g;
        *out = nullptr;
        return -1;
    }
    *out = g;
    return 0;
}
void orc_genome_free(orc_genome* g) { delete g; }
int orc_genome_num_xforms(const orc_genome* g) { return (int)g->xf.size(); }
int orc_genome_has_final(const orc_genome* g) { return g->has_final ? 1 : 0; }

// flame.cpp:33-103
int orc_genome_param_buffer(const orc_genome* g, float* out, int cap) {
    std::vector<float> buf;
    auto push = [&](const Xform& x, float w) {
        buf.push_back(w);
        for (int i = 0; i < 6; i++) buf.push_back(x.affine[i]);
        if (x.has_post) for (int i = 0; i < 6; i++) buf.push_back(x.post[i]);
        for (auto& [n, v] : x.vars) buf.push_back(v);
        for (auto& [n, v] : x.params) buf.push_back(v);
        buf.push_back(x.color);
        buf.push_back(x.color_speed);
        buf.push_back(x.opacity);
        buf.push_back(x.rotation_frequency);
    };
    float total = 0.0f;
    for (const auto& x : g->xf) total += x.weight;
    for (const auto& x : g->xf) push(x, x.weight / total);
    if (g->has_final) push(g->fin, g->fin.weight / total);
    if (out) for (int i = 0; i < (int)buf.size() && i < cap; i++) out[i] = buf[i];
    return (int)buf.size();
}
// flame.cpp:33-71 make_shader_buffer_map: the offsets of the buffer above, as JSON
int orc_genome_layout_json(const orc_genome* g, char* out, int cap) {
    std::string js = "{\"xforms\": [";
    int off = 0;
    auto block = [&](const Xform& x) {
        std::string b = "{\"weight\": " + std::to_string(off++) + ", \"affine\": [";
        for (int i = 0; i < 6; i++) b += (i ? ", " : "") + std::to_string(off++);
        b += "]";
        if (x.has_post) {
            b += ", \"post\": [";
            for (int i = 0; i < 6; i++) b += (i ? ", " : "") + std::to_string(off++);
            b += "]";
        }
        b += ", \"variations\": {";
        bool first = true;
        for (auto& kv : x.vars) { b += (first ? "\"" : ", \"") + kv.first + "\": " + std::to_string(off++); first = false; }
        b += "}, \"param\": {";
        first = true;
        for (auto& kv : x.params) { b += (first ? "\"" : ", \"") + kv.first + "\": " + std::to_string(off++); first = false; }
        b += "}, \"color\": " + std::to_string(off++);
        b += ", \"color_speed\": " + std::to_string(off++);
        b += ", \"opacity\": " + std::to_string(off++);
        b += ", \"rotation_frequency\": " + std::to_string(off++) + "}";
        return b;
    };
    for (size_t i = 0; i < g->xf.size(); i++) js += (i ? ", " : "") + block(g->xf[i]);
    js += "]";
    if (g->has_final) js += ", \"final_xform\": " + block(g->fin);
    js += ", \"size\": " + std::to_string(off) + "}";
    if (out && cap > 0) snprintf(out, (size_t)cap, "%s", js.c_str());
    return (int)js.size();
}

int orc_animate_params(const orc_genome* g, uint32_t T, float tss_width, uint32_t t, float* out, int cap) {
    if (T == 0 || t >= T) return -1;
    std::vector<std::vector<Xform>> xf;
    std::vector<Xform> fin;
    animate(g, T, tss_width, xf, fin);
    orc_genome tmp = *g;
    tmp.xf = xf[t];
    tmp.fin = fin[t];
    return orc_genome_param_buffer(&tmp, out, cap);
}

void orc_genome_info(const orc_genome* g, double* o) {
    o[0] = g->size[0]; o[1] = g->size[1]; o[2] = g->center[0]; o[3] = g->center[1];
    o[4] = g->scale; o[5] = g->rotate; o[6] = g->est_radius; o[7] = g->est_min; o[8] = g->est_curve;
    o[9] = g->gamma; o[10] = g->vibrancy; o[11] = g->brightness;
}
void orc_screen_affine(const orc_genome* g, uint32_t w, uint32_t h, float out6[6]) { screen_affine(g, w, h, out6); }
int orc_xform_draws(const orc_genome* g, int xi, int first_run) {
    if (xi < 0) return g->has_final ? xform_draws(g->fin, first_run != 0) : 0;
    if (xi >= (int)g->xf.size()) return -1;
    return xform_draws(g->xf[xi], first_run != 0);
}
int orc_select_xform(const orc_genome* g, float r) { return select_xform(g, r); }

int orc_eval_xform(const orc_genome* g, int xi, int fp64, int n, const float* in, uint32_t* st,
                   int first_run, double* out) {
    if (xi >= (int)g->xf.size() || (xi < 0 && !g->has_final)) return -1;
    const Xform& xf = (xi < 0) ? g->fin : g->xf[xi];
    for (int i = 0; i < n; i++) {
        Jsf s{st[4 * i], st[4 * i + 1], st[4 * i + 2], st[4 * i + 3]};
        if (fp64) {
            double x = in[3 * i], y = in[3 * i + 1], c = in[3 * i + 2], w;
            dispatch<double>(xf, x, y, c, w, first_run != 0, s);
            out[4 * i] = x; out[4 * i + 1] = y; out[4 * i + 2] = c; out[4 * i + 3] = w;
        } else {
            float x = in[3 * i], y = in[3 * i + 1], c = in[3 * i + 2], w;
            dispatch<float>(xf, x, y, c, w, first_run != 0, s);
            out[4 * i] = x; out[4 * i + 1] = y; out[4 * i + 2] = c; out[4 * i + 3] = w;
        }
        st[4 * i] = s.a; st[4 * i + 1] = s.b; st[4 * i + 2] = s.c; st[4 * i + 3] = s.d;
    }
    return 0;
}

int orc_chaos(const orc_genome* g, const orc_chaos_cfg* cfg, double* rgba, uint64_t* hits,
              uint8_t* trace, uint64_t* counters) {
    if (g->xf.size() > 255) return -1;
    return cfg->fp64 ? chaos<double>(g, cfg, rgba, hits, trace, counters)
                     : chaos<float>(g, cfg, rgba, hits, trace, counters);
}

int orc_xid_sequence(const orc_genome* g, uint64_t N, uint32_t TS, uint64_t seed, uint32_t fuse,
                     uint32_t draw, uint8_t* out) {
    TS = std::max(1u, TS);
    if (N % TS || (N / TS) % 256 || fuse < 1) return -1;
    const uint64_t ppts = N / TS, groups = N / 256;
    std::vector<Jsf> lane0(groups);
    for (uint64_t t = 0; t < TS; t++)
        for (uint64_t q = 0; q < ppts / 256; q++) {
            uint64_t slot = t * ppts + q * 256;
            jsf_warmup(lane0[t * (ppts / 256) + q], (uint32_t)(slot + seed * N));
        }
    const int fin_draws = g->has_final ? xform_draws(g->fin, false) : 0;
    for (uint32_t p = 0; p < fuse + draw; p++) {
        const bool first = (p == 0), drw = (p >= fuse);
        for (uint64_t q = 0; q < groups; q++) {
            Jsf& s = lane0[q];
            int x = select_xform(g, randf(s));
            out[(uint64_t)p * groups + q] = (uint8_t)x;
            int skip = (first ? 2 : 0) + xform_draws(g->xf[x], first) + (drw ? fin_draws : 0);
            for (int k = 0; k < skip; k++) (void)jsf_next(s);
        }
    }
    return 0;
}

uint64_t orc_cpu_baseline(const orc_genome* g, uint64_t N, uint32_t passes, uint32_t W, uint32_t H,
                          int threads, uint64_t seed, int badval_reset, float* rgba_out, uint32_t* hits_out,
                          uint64_t* binned_out) {
    // FP32 transcription of flame.glsl's draw pass over walker slices (one temporal sample per
    // slice, shuffled within the slice), private histograms merged at the end.
    threads = std::max(1, threads);
    const uint64_t groups = N / 256;
    if (groups == 0) return 0;
    float ss[6];
    screen_affine(g, W, H, ss);
    std::vector<std::vector<float>> prgba(threads);
    std::vector<std::vector<uint32_t>> phits(threads);
    std::vector<uint64_t> done(threads, 0), binned(threads, 0);
    auto work = [&](int ti) {
        uint64_t g0 = groups * ti / threads, g1 = groups * (ti + 1) / threads;
        uint64_t n = (g1 - g0) * 256, base = g0 * 256;
        if (n == 0) return;
        std::vector<float>& hr = prgba[ti];
        std::vector<uint32_t>& hh = phits[ti];
        hr.assign((size_t)W * H * 4, 0.0f);
        hh.assign((size_t)W * H, 0u);
        std::vector<Jsf> rng(n);
        for (uint64_t i = 0; i < n; i++) jsf_warmup(rng[i], (uint32_t)(base + i + seed * N));
        std::vector<float> px(n), py(n), pc(n), nx(n), ny(n), nc(n);
        std::vector<uint32_t> perm(n);
        for (uint64_t i = 0; i < n; i++) { float a, b; sample_point((uint32_t)i, (uint32_t)n, a, b); px[i] = a; py[i] = b; pc[i] = 0.5f; perm[i] = (uint32_t)i; }
        std::mt19937_64 pr(seed * 7919 + ti);
        uint64_t cnt = 0, nb = 0;
        for (uint32_t p = 0; p < passes; p++) {
            std::shuffle(perm.begin(), perm.end(), pr);
            int xid = 0;
            for (uint64_t i = 0; i < n; i++) {
                Jsf& s = rng[i];
                if (i % 256 == 0) xid = select_xform(g, randf(s));
                float x = px[perm[i]], y = py[perm[i]], c = pc[perm[i]], w;
                dispatch<float>(g->xf[xid], x, y, c, w, false, s);
                if (badval_reset) reset_bad<float>(x, y, w, s);
                nx[i] = x; ny[i] = y; nc[i] = c;
                if (g->has_final) { float fw; dispatch<float>(g->fin, x, y, c, fw, false, s); w *= fw; }
                float sx_ = std::fma(ss[0], x, std::fma(ss[2], y, ss[4]));
                float sy_ = std::fma(ss[1], x, std::fma(ss[3], y, ss[5]));
                if (sx_ >= 0 && sy_ >= 0 && sx_ < (float)W && sy_ < (float)H && w > 0) {
                    uint32_t bx = (uint32_t)sx_, by = (uint32_t)sy_;
                    size_t idx = (size_t)(H - by - 1) * W + bx;
                    uint32_t ci = palette_index(c);
                    hr[idx * 4] += g->palette[ci][0]; hr[idx * 4 + 1] += g->palette[ci][1];
                    hr[idx * 4 + 2] += g->palette[ci][2]; hr[idx * 4 + 3] += w;
                    hh[idx] += 1;
                    nb++;
                }
                cnt++;
            }
            std::swap(px, nx); std::swap(py, ny); std::swap(pc, nc);
        }
        done[ti] = cnt;
        binned[ti] = nb;
    };
    std::vector<std::thread> th;
    for (int t = 0; t < threads; t++) th.emplace_back(work, t);
    for (auto& t : th) t.join();
    uint64_t total = 0, total_binned = 0;
    for (int t = 0; t < threads; t++) {
        total += done[t];
        total_binned += binned[t];
        if (prgba[t].empty()) continue;
        if (rgba_out) for (size_t i = 0; i < prgba[t].size(); i++) rgba_out[i] += prgba[t][i];
        if (hits_out) for (size_t i = 0; i < phits[t].size(); i++) hits_out[i] += phits[t][i];
    }
    if (binned_out) *binned_out = total_binned;
    return total;
}

}  // extern "C"

namespace {
// density_vert.glsl:35-44: min(R, int(R / pow(a, curve))) in real arithmetic.  int(v) <= k
// thresholds: k * a^curve <= R  <=>  a <= (R/k)^(1/curve) for curve > 0 (>= for curve < 0).
int de_radius(double a, int R, double curve) {
    if (curve == 0.0) return R;
    int r = 0;
    for (int k = 1; k <= R; k++) {
        double t = std::pow((double)R / (double)k, 1.0 / curve);
        bool ok = (curve > 0.0) ? (a <= t) : (a >= t);
        if (ok) r = k;
    }
    return r;
}
}  // namespace

extern "C" {

int orc_de_radius(double a, int R, int minr, double curve) { return std::max(minr, de_radius(a, R, curve)); }

double orc_de_weight(int dx, int dy, int r) {
    if (r == 0) return (dx == 0 && dy == 0) ? 1.0 : -1.0;
    const int d2 = dx * dx + dy * dy;
    if (4 * d2 > (2 * r + 1) * (2 * r + 1)) return -1.0;
    return (1.0 - (double)d2 / ((r + 0.5) * (r + 0.5))) * (0.63661977236 / (double)(r * r));
}

// density_vert.glsl:26-63, density_frag.glsl:9-18, restated symmetrically: every bin with a > 0
// spreads over the pixels (dx, dy) with 4*(dx^2+dy^2) <= (2r+1)^2, weight
// (1 - (dx^2+dy^2)/(r+0.5)^2) * 0.63661977236 / r^2; r = 0 copies the bin.
// r = max(min, min(R, int(R / a^curve))) evaluated in real arithmetic.
int orc_density_estimate(const double* in, uint32_t w, uint32_t h, int R, int minr, double curve, double* out) {
    if (R < 0 || R > 100) return -1;
    std::fill(out, out + (size_t)w * h * 4, 0.0);
    for (uint32_t qy = 0; qy < h; qy++)
        for (uint32_t qx = 0; qx < w; qx++) {
            const double* c = in + ((size_t)qy * w + qx) * 4;
            double a = c[3];
            if (!(a > 0.0) && !(a < 0.0)) continue;  // a == 0 (or NaN) is culled
            int r = std::max(minr, de_radius(a, R, curve));
            if (r == 0) { for (int k = 0; k < 4; k++) out[((size_t)qy * w + qx) * 4 + k] += c[k]; continue; }
            double nf = 0.63661977236 / (double)(r * r);
            double den = (r + 0.5) * (r + 0.5);
            for (int dy = -r; dy <= r; dy++)
                for (int dx = -r; dx <= r; dx++) {
                    int d2 = dx * dx + dy * dy;
                    if (4 * d2 > (2 * r + 1) * (2 * r + 1)) continue;
                    int px = (int)qx + dx, py = (int)qy + dy;
                    if (px < 0 || py < 0 || px >= (int)w || py >= (int)h) continue;
                    double wt = (1.0 - (double)d2 / den) * nf;
                    for (int k = 0; k < 4; k++) out[((size_t)py * w + px) * 4 + k] += c[k] * wt;
                }
        }
    return 0;
}

// tonemap.glsl:18-38 with an ss x ss box filter: per bin c *= 0.5*brightness*log10(1+a*k2)/a,
// mean over each block, then gamma / vibrancy / clamp.  ss = 1 is the shader itself.  A block
// without density (where the shader divides 0 by 0) maps to opaque black.
int orc_tonemap(const double* in, uint32_t w, uint32_t h, uint32_t ss, double gamma, double brightness,
                double vibrancy, double k2, double* out) {
    if (ss == 0 || w % ss || h % ss) return -1;
    const uint32_t ow = w / ss, oh = h / ss;
    for (uint32_t oy = 0; oy < oh; oy++)
        for (uint32_t ox = 0; ox < ow; ox++) {
            double acc[4] = {0, 0, 0, 0};
            for (uint32_t j = 0; j < ss; j++)
                for (uint32_t i = 0; i < ss; i++) {
                    const double* c = in + (((size_t)(oy * ss + j)) * w + ox * ss + i) * 4;
                    double a = c[3];
                    if (!(a > 0.0)) continue;
                    double ls = 0.5 * brightness * std::log(1.0 + a * k2) * 0.434294481903251827651128918916 / a;
                    for (int k = 0; k < 4; k++) acc[k] += c[k] * ls;
                }
            double* o = out + ((size_t)oy * ow + ox) * 4;
            const double n = (double)ss * ss;
            double al = acc[3] / n;
            if (!(al > 0.0)) { o[0] = o[1] = o[2] = 0.0; o[3] = 1.0; continue; }
            double ig = 1.0 / gamma;
            double gf = std::pow(al, ig) / al;
            for (int k = 0; k < 3; k++) {
                double v = acc[k] / n;
                double t = std::pow(v, ig) * (1.0 - vibrancy) + gf * v * vibrancy;
                o[k] = std::min(std::max(t, 0.0), 1.0);
            }
            o[3] = 1.0;
        }
    return 0;
}

// flam3's spatial filter functions and their supports (the published definitions: Gaussian
// exp(-2x^2) sqrt(2/pi) on [-1.5, 1.5], box on [-0.5, 0.5], triangle 1 - |x| on [-1, 1], the cubic
// Hermite 2|x|^3 - 3x^2 + 1 on [-1, 1])
static double filter_support(int shape) { return shape == 1 ? 0.5 : (shape == 0 ? 1.5 : 1.0); }
static double filter_value(int shape, double x) {
    const double t = std::fabs(x);
    switch (shape) {
        case 0: return std::exp(-2.0 * x * x) * std::sqrt(2.0 / 3.14159265358979323846);
        case 1: return t <= 0.5 ? 1.0 : 0.0;
        case 2: return t < 1.0 ? 1.0 - t : 0.0;
        case 3: return t < 1.0 ? (2.0 * t - 3.0) * t * t + 1.0 : 0.0;
        default: return 0.0;
    }
}

// Taps of the separable filter over the supersampled bins: the window spans
// fw = 2 * support * ss * radius bins, rounded up to an integer width of the same parity as ss
// (so the window centres on the output pixel's ss x ss block), sampled at the centre of each
// cell with the coordinate stretched so the window covers exactly the support; normalised.
int orc_filter_kernel(uint32_t ss, double radius, int shape, double* taps, int cap) {
    if (ss == 0 || !(radius > 0.0) || shape < 0 || shape > 3) return -1;
    const double support = filter_support(shape);
    const double fw = 2.0 * support * (double)ss * radius;
    int fwidth = (int)fw + 1;
    if ((fwidth ^ (int)ss) & 1) fwidth++;
    if (fwidth > cap) return -1;
    const double adjust = fw > 0.0 ? support * (double)fwidth / fw : 1.0;
    double sum = 0.0;
    for (int i = 0; i < fwidth; i++) {
        taps[i] = filter_value(shape, ((2.0 * i + 1.0) / (double)fwidth - 1.0) * adjust);
        sum += taps[i];
    }
    for (int i = 0; i < fwidth; i++) taps[i] /= sum;
    return fwidth;
}

int orc_tonemap_filter(const double* in, uint32_t w, uint32_t h, uint32_t ss, double radius, int shape,
                       double gamma, double brightness, double vibrancy, double k2, double* out) {
    if (ss == 0 || w % ss || h % ss) return -1;
    double taps[256];
    const int fwidth = orc_filter_kernel(ss, radius, shape, taps, 256);
    if (fwidth < 0) return -1;
    const int pad = (fwidth - (int)ss) / 2;
    // per-bin log-density scaling (tonemap.glsl:26), zero where there is no density
    std::vector<double> L((size_t)w * h * 4, 0.0);
    for (size_t i = 0; i < (size_t)w * h; i++) {
        const double a = in[i * 4 + 3];
        if (!(a > 0.0)) continue;
        const double ls = 0.5 * brightness * std::log(1.0 + a * k2) * 0.434294481903251827651128918916 / a;
        for (int k = 0; k < 4; k++) L[i * 4 + k] = in[i * 4 + k] * ls;
    }
    const uint32_t ow = w / ss, oh = h / ss;
    for (uint32_t oy = 0; oy < oh; oy++)
        for (uint32_t ox = 0; ox < ow; ox++) {
            double acc[4] = {0, 0, 0, 0};
            for (int j = 0; j < fwidth; j++) {
                const int y = (int)(oy * ss) - pad + j;
                if (y < 0 || y >= (int)h) continue;
                for (int i = 0; i < fwidth; i++) {
                    const int x = (int)(ox * ss) - pad + i;
                    if (x < 0 || x >= (int)w) continue;
                    const double wt = taps[i] * taps[j];
                    for (int k = 0; k < 4; k++) acc[k] += wt * L[((size_t)y * w + x) * 4 + k];
                }
            }
            double* o = out + ((size_t)oy * ow + ox) * 4;
            if (!(acc[3] > 0.0)) { o[0] = o[1] = o[2] = 0.0; o[3] = 1.0; continue; }
            const double ig = 1.0 / gamma, gf = std::pow(acc[3], ig) / acc[3];
            for (int k = 0; k < 3; k++) {
                const double t = std::pow(acc[k], ig) * (1.0 - vibrancy) + gf * acc[k] * vibrancy;
                o[k] = std::min(std::max(t, 0.0), 1.0);
            }
            o[3] = 1.0;
        }
    return 0;
}

int orc_downsample(const double* in, uint32_t w, uint32_t h, uint32_t ss, double* out) {
    if (ss == 0 || w % ss || h % ss) return -1;
    uint32_t ow = w / ss, oh = h / ss;
    for (uint32_t y = 0; y < oh; y++)
        for (uint32_t x = 0; x < ow; x++)
            for (int k = 0; k < 4; k++) {
                double s = 0;
                for (uint32_t j = 0; j < ss; j++)
                    for (uint32_t i = 0; i < ss; i++) s += in[(((size_t)(y * ss + j)) * w + x * ss + i) * 4 + k];
                out[((size_t)y * ow + x) * 4 + k] = s / (double)(ss * ss);
            }
    return 0;
}

}  // extern "C"
