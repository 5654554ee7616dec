// Genome model: flam3 loading (src/flame.cpp:160-226), the flat parameter buffer and its
// layout (flame.cpp:33-103), the compiled program the kernels interpret (program.h), the
// screen affine (flame.cpp:289-296) and the seeded synthetic genomes of the benchmarks.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <sstream>

#include "internal.h"

namespace rfk {

namespace {

// util.hpp:13-26 parse_strings: whitespace-separated tokens, missing ones stay 0.  Each token is
// converted where it lies: the conversions (strtod, strtol) stop at the whitespace that ends it.
template <class Conv>
void parse_list(const std::string& in, float* out, int n, Conv cv) {
    const char* p = in.c_str();
    const char* end = p + in.size();
    int k = 0;
    while (k < n) {
        while (p < end && isspace((unsigned char)*p)) p++;
        if (p >= end) break;
        out[k++] = cv(p);
        while (p < end && !isspace((unsigned char)*p)) p++;
    }
}
// a token as a float, 0 when it does not start with a number (pugixml as_float)
float token_float(const char* v) {
    char* e = nullptr;
    const double d = strtod(v, &e);
    return e != v ? (float)d : 0.0f;
}
bool num(const std::string& s, double& v) {
    const char* p = s.c_str();
    char* e = nullptr;
    v = strtod(p, &e);
    return e != p;
}
float as_float(const std::string& s) {  // pugixml as_float: 0 when unparsable
    double v;
    return num(s, v) ? (float)v : 0.0f;
}
int as_int(const std::string& s) { return (int)strtol(s.c_str(), nullptr, 10); }

int apply_xform_attr(Xform& x, const std::string& name, const std::string& val, bool is_final,
                     const Registry& reg, std::string& err) {
    if (name == "weight") x.weight = as_float(val);
    else if (name == "color") x.color = as_float(val);
    else if (name == "color_speed") x.color_speed = as_float(val);
    // flame.cpp:190 tests the element name against "final_xform", which a <finalxform> never
    // equals, so a final xform with animate > 0 also rotates; kept as the reference does it.
    else if (name == "animate") x.rotation_frequency = (as_float(val) > 0) ? 1.0f : 0.0f;
    else if (name == "opacity") x.opacity = as_float(val);
    else if (reg.param_owner.count(name)) x.params[name] = as_float(val);
    else if (reg.vars.count(name)) x.vars[name] = as_float(val);
    else if (name == "coefs") parse_list(val, x.affine, 6, token_float);
    else if (name == "post") {
        x.has_post = true;
        for (int i = 0; i < 6; i++) x.post[i] = 0;
        parse_list(val, x.post, 6, token_float);
    }
    // flam3 files older than color_speed carry `symmetry`; flam3 maps it to (1 - symmetry) / 2
    else if (name == "symmetry") x.color_speed = (1.0f - as_float(val)) * 0.5f;
    else {
        err = "unknown attribute `" + name + "` in " + (is_final ? "finalxform" : "xform");
        return RF_ERR_UNKNOWN_NAME;
    }
    return RF_OK;
}

void fmt_float(std::ostringstream& o, float v) {
    char b[32];
    snprintf(b, sizeof b, "%.9g", (double)v);
    o << b;
}

}  // namespace

int genome_from_xml(const std::string& xml, const Registry& reg, Genome& g) {
    std::vector<XNode> roots;
    std::string err;
    if (!parse_xml(xml, roots, err)) return fail(RF_ERR_PARSE, "flam3: " + err);
    const XNode* fl = nullptr;
    for (const auto& r : roots) {
        if (r.name == "flame") { fl = &r; break; }
        if (r.name == "flames")  // electric-sheep files wrap genomes in <flames>
            for (const auto& k : r.kids) if (k.name == "flame") { fl = &k; break; }
        if (fl) break;
    }
    if (!fl) return fail(RF_ERR_PARSE, "flam3: no <flame> element");
    g = Genome();
    auto A = [&](const char* k) -> std::string { const std::string* v = fl->attr(k); return v ? *v : std::string(); };
    parse_list(A("center"), g.center, 2, token_float);
    g.scale = as_float(A("scale"));
    g.rotate = as_float(A("rotate"));
    g.est_curve = as_float(A("estimator_curve"));
    // flame.cpp:171 reads `estimator_min`; flam3 itself writes `estimator_minimum`
    g.est_min = fl->attr("estimator_min") ? as_int(A("estimator_min")) : as_int(A("estimator_minimum"));
    g.est_radius = as_int(A("estimator_radius"));
    g.brightness = as_float(A("brightness"));
    g.gamma = as_float(A("gamma"));
    g.vibrancy = as_float(A("vibrancy"));
    {
        float sz[2] = {0, 0};
        parse_list(A("size"), sz, 2, [](const char* v) { return (float)strtol(v, nullptr, 10); });
        g.size[0] = (unsigned)std::max(0.0f, sz[0]);
        g.size[1] = (unsigned)std::max(0.0f, sz[1]);
    }
    if (fl->attr("supersample")) g.supersample = (unsigned)std::max(1, as_int(A("supersample")));
    g.filter = as_float(A("filter"));
    {  // flam3 filter shapes; the ones without a kernel here are drawn with the Gaussian
        const std::string fs = A("filter_shape");
        g.filter_shape = fs == "box" ? RF_FILTER_BOX : fs == "triangle" ? RF_FILTER_TRIANGLE
                       : fs == "hermite" ? RF_FILTER_HERMITE : RF_FILTER_GAUSSIAN;
    }
    for (const auto& k : fl->kids) {
        if (k.name == "xform" || k.name == "finalxform") {
            Xform x;
            bool fin = (k.name == "finalxform");
            for (const auto& [name, val] : k.attrs) {
                int rc = apply_xform_attr(x, name, val, fin, reg, err);
                if (rc) return fail(rc, "flam3: " + err);
            }
            if (fin) { g.final_xf = x; g.has_final = true; }
            else g.xforms.push_back(x);
        } else if (k.name == "color") {
            const std::string* idx = k.attr("index");
            const std::string* rgb = k.attr("rgb");
            if (!idx || !rgb) return fail(RF_ERR_PARSE, "flam3: <color> needs index and rgb");
            long i = strtol(idx->c_str(), nullptr, 10);
            if (i < 0 || i > 255) return fail(RF_ERR_PARSE, "flam3: palette index out of range");
            // flame.cpp:217: std::stoi(v) / 256.0f — the integer part of each component
            float c[3] = {0, 0, 0};
            parse_list(*rgb, c, 3, [](const char* v) { return (float)strtol(v, nullptr, 10) / 256.0f; });
            for (int q = 0; q < 3; q++) g.palette[i][q] = c[q];
            g.palette[i][3] = 1.0f;
        } else if (k.name == "palette") {
            // flam3 hex palette block: `count` RRGGBB triplets, bytes divided by 256 as above
            std::string hex;
            for (char ch : k.text) if (isxdigit((unsigned char)ch)) hex += ch;
            size_t n = std::min<size_t>(256, hex.size() / 6);
            for (size_t i = 0; i < n; i++) {
                for (int q = 0; q < 3; q++)
                    g.palette[i][q] = (float)strtol(hex.substr(i * 6 + q * 2, 2).c_str(), nullptr, 16) / 256.0f;
                g.palette[i][3] = 1.0f;
            }
        }
    }
    return genome_validate(g, reg);
}

// The checks the reference's shader compile performs implicitly (flame.cpp:222-225), made
// explicit: every variation evaluable with all its parameters, at least one accumulated term
// per xform, a positive total weight, the parameter buffer within fp[1024].
int genome_validate(const Genome& g, const Registry& reg) {
    if (g.xforms.empty()) return fail(RF_ERR_INVALID_ARG, "genome has no xforms");
    if ((int)g.xforms.size() > kMaxXforms) return fail(RF_ERR_CAPACITY, "more than 255 xforms");
    float total = 0.0f;
    for (const auto& x : g.xforms) total += x.weight;
    if (!(total > 0.0f) || !std::isfinite(total)) return fail(RF_ERR_INVALID_ARG, "total xform weight must be positive and finite");
    auto check = [&](const Xform& x, const char* what) -> int {
        int terms = 0;
        for (const auto& [name, w] : x.vars) {
            auto it = reg.vars.find(name);
            if (it == reg.vars.end()) return fail(RF_ERR_UNKNOWN_NAME, std::string(what) + ": unknown variation " + name);
            const VariationDef& d = it->second;
            if (d.kernel_id < 0) return fail(RF_ERR_UNSUPPORTED, "variation `" + name + "`: " + d.note);
            for (const auto& p : d.params)
                if (!x.params.count(p))
                    return fail(RF_ERR_INVALID_ARG, "variation `" + name + "` needs parameter `" + p + "`");
            if (!(d.flags & VF_PRE_XFORM)) terms++;
        }
        if (terms == 0) return fail(RF_ERR_INVALID_ARG, std::string(what) + " has no variations");
        return 0;
    };
    for (size_t i = 0; i < g.xforms.size(); i++)
        if (int rc = check(g.xforms[i], "xform")) return rc;
    if (g.has_final)
        if (int rc = check(g.final_xf, "finalxform")) return rc;
    std::vector<float> buf;
    if (int rc = genome_param_buffer(g, buf, nullptr)) return rc;
    std::vector<uint32_t> prog;
    return genome_program(g, reg, prog);
}

// flame.cpp:33-103: per xform weight, affine[6], post[6] if present, variation weights and
// parameters in map order, color, color_speed, opacity, rotation_frequency; final xform last.
int genome_param_buffer(const Genome& g, std::vector<float>& buf, std::string* layout) {
    buf.clear();
    float total = 0.0f;
    for (const auto& x : g.xforms) total += x.weight;
    // one walk fills the buffer; the layout JSON (indices into it) is written only when asked for
    const bool want = layout != nullptr;
    const auto idx = [&]() { return std::to_string(buf.size()); };
    const auto push = [&](const Xform& x) {
        std::string aff, post, vars, prm;
        const size_t start = buf.size();
        buf.push_back(x.weight / total);
        for (int i = 0; i < 6; i++) {
            if (want) aff += (i ? "," : "") + idx();
            buf.push_back(x.affine[i]);
        }
        if (x.has_post)
            for (int i = 0; i < 6; i++) {
                if (want) post += (i ? "," : "") + idx();
                buf.push_back(x.post[i]);
            }
        bool first = true;
        for (const auto& [n, v] : x.vars) {
            if (want) vars += (first ? "\"" : ",\"") + n + "\":" + idx();
            buf.push_back(v);
            first = false;
        }
        first = true;
        for (const auto& [n, v] : x.params) {
            if (want) prm += (first ? "\"" : ",\"") + n + "\":" + idx();
            buf.push_back(v);
            first = false;
        }
        const size_t color = buf.size();
        buf.push_back(x.color);
        buf.push_back(x.color_speed);
        buf.push_back(x.opacity);
        buf.push_back(x.rotation_frequency);
        if (!want) return std::string();
        const size_t end = buf.size() - 1;
        std::string m = "{\"meta\":{\"start\":" + std::to_string(start) + ",\"end\":" + std::to_string(end) +
                        ",\"size\":" + std::to_string(end - start + 1) + "},\"weight\":" + std::to_string(start) +
                        ",\"affine\":[" + aff + "]";
        if (x.has_post) m += ",\"post\":[" + post + "]";
        m += ",\"variations\":{" + vars + "},\"param\":{" + prm + "},\"color\":" + std::to_string(color) +
             ",\"color_speed\":" + std::to_string(color + 1) + ",\"opacity\":" + std::to_string(color + 2) +
             ",\"rotation_frequency\":" + std::to_string(color + 3) + "}";
        return m;
    };
    std::string js = "{\"xforms\":[";
    for (size_t i = 0; i < g.xforms.size(); i++) {
        const std::string m = push(g.xforms[i]);
        if (want) js += (i ? "," : "") + m;
    }
    js += "]";
    if (g.has_final) {
        const std::string m = push(g.final_xf);
        if (want) js += ",\"final_xform\":" + m;
    }
    if (want) *layout = js + ",\"size\":" + std::to_string(buf.size()) + "}";
    if ((int)buf.size() > kMaxParams)
        return fail(RF_ERR_CAPACITY, "parameter buffer of " + std::to_string(buf.size()) + " floats exceeds 1024");
    return 0;
}

namespace {
inline uint32_t fbits(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }

void emit_block(const Xform& x, const Registry& reg, std::vector<uint32_t>& w) {
    const size_t base = w.size();
    std::vector<std::pair<const VariationDef*, float>> pre, terms;
    uint32_t mask = 0;
    int draws = 0;
    for (const auto& [n, wt] : x.vars) {
        const VariationDef& d = reg.vars.at(n);
        draws += d.draws;
        if (d.flags & VF_PRE_XFORM) pre.push_back({&d, wt});
        else { terms.push_back({&d, wt}); mask |= d.precalc; }
    }
    if (mask & (PC_SINA | PC_COSA | PC_SINR | PC_COSR)) mask |= PC_R;
    w.resize(base + X_TERMS, 0);
    w[base + X_NPRE] = (uint32_t)pre.size();
    w[base + X_NTERM] = (uint32_t)terms.size();
    w[base + X_MASK] = mask;
    w[base + X_HASPOST] = x.has_post ? 1u : 0u;
    for (int i = 0; i < 6; i++) w[base + X_AFF + i] = fbits(x.affine[i]);
    for (int i = 0; i < 6; i++) w[base + X_POST + i] = fbits(x.has_post ? x.post[i] : (i == 0 || i == 3 ? 1.0f : 0.0f));
    w[base + X_COLOR] = fbits(x.color);
    w[base + X_CS] = fbits(x.color_speed);
    w[base + X_OMCS] = fbits(1.0f - x.color_speed);
    w[base + X_OPACITY] = fbits(x.opacity);
    w[base + X_DRAWS] = (uint32_t)draws;
    w[base + X_ROTF] = fbits(x.rotation_frequency);
    const size_t ent = w.size();
    const size_t n_ent = pre.size() + terms.size();
    w.resize(ent + 3 * n_ent, 0);
    size_t k = 0;
    auto put = [&](const std::pair<const VariationDef*, float>& t) {
        const VariationDef& d = *t.first;
        uint32_t id = (uint32_t)d.kernel_id | ((d.flags & VF_NO_WEIGHT_MUL) ? kTermNoWeightMul : 0u);
        w[ent + 3 * k] = id;
        w[ent + 3 * k + 1] = fbits(t.second);
        w[ent + 3 * k + 2] = (uint32_t)(w.size() - base);
        for (const auto& p : d.params) w.push_back(fbits(x.params.at(p)));
        k++;
    };
    for (const auto& t : pre) put(t);
    for (const auto& t : terms) put(t);
}
}  // namespace

int genome_program(const Genome& g, const Registry& reg, std::vector<uint32_t>& w) {
    const uint32_t nx = (uint32_t)g.xforms.size();
    w.assign(H_XOFF + nx, 0);
    w[H_MAGIC] = kProgMagic;
    w[H_NX] = nx;
    w[H_HASFINAL] = g.has_final ? 1u : 0u;
    float total = 0.0f;
    for (const auto& x : g.xforms) total += x.weight;
    w[H_WOFF] = (uint32_t)w.size();
    for (const auto& x : g.xforms) w.push_back(fbits(x.weight / total));  // flame.cpp:82
    for (uint32_t i = 0; i < nx; i++) {
        w[H_XOFF + i] = (uint32_t)w.size();
        emit_block(g.xforms[i], reg, w);
    }
    if (g.has_final) {
        w[H_FINAL] = (uint32_t)w.size();
        emit_block(g.final_xf, reg, w);
    }
    w[H_WORDS] = (uint32_t)w.size();
    if ((int)w.size() > kProgMaxWords)
        return fail(RF_ERR_CAPACITY, "compiled genome of " + std::to_string(w.size()) + " words exceeds " +
                                         std::to_string(kProgMaxWords));
    return 0;
}

// flame.hpp:97-128 helpers composed as flame.cpp:289-296, in FP32 as the reference.
void genome_screen_affine(const Genome& g, uint32_t W, uint32_t H, float out[6]) {
    float a[6] = {1, 0, 0, 1, 0, 0};
    auto translate = [](float* m, float t0, float t1) {
        m[4] = m[0] * t0 + m[2] * t1 + m[4];
        m[5] = m[1] * t0 + m[3] * t1 + m[5];
    };
    translate(a, (float)W / 2.0f, (float)H / 2.0f);
    float s = g.scale * (float)H / (float)g.size[1];
    for (int i = 0; i < 4; i++) a[i] *= s;
    {
        float rad = 0.01745329251f * g.rotate;
        float sn = sinf(rad), cs = cosf(rad);
        float a0 = a[0], a1 = a[1], a2 = a[2], a3 = a[3];
        a[0] = a0 * cs + a2 * sn;
        a[1] = a1 * cs + a3 * sn;
        a[2] = a2 * cs - a0 * sn;
        a[3] = a3 * cs - a1 * sn;
    }
    translate(a, -g.center[0], -g.center[1]);
    memcpy(out, a, sizeof(a));
}

int genome_xform_draws(const Genome& g, const Registry& reg, int xi) {
    const Xform* x = nullptr;
    if (xi < 0) { if (!g.has_final) return 0; x = &g.final_xf; }
    else if (xi < (int)g.xforms.size()) x = &g.xforms[xi];
    else return -1;
    int n = 0;
    for (const auto& [name, w] : x->vars) n += reg.vars.at(name).draws;
    return n;
}

std::string genome_to_xml(const Genome& g) {
    std::ostringstream o;
    o << "<flame size=\"" << g.size[0] << " " << g.size[1] << "\" center=\"";
    fmt_float(o, g.center[0]); o << " "; fmt_float(o, g.center[1]);
    o << "\" scale=\""; fmt_float(o, g.scale);
    o << "\" rotate=\""; fmt_float(o, g.rotate);
    o << "\" supersample=\"" << g.supersample;
    if (g.filter > 0.0f) {
        static const char* shapes[] = {"gaussian", "box", "triangle", "hermite"};
        o << "\" filter=\"";
        fmt_float(o, g.filter);
        o << "\" filter_shape=\"" << shapes[g.filter_shape & 3];
    }
    o << "\" estimator_radius=\"" << g.est_radius << "\" estimator_min=\"" << g.est_min;
    o << "\" estimator_curve=\""; fmt_float(o, g.est_curve);
    o << "\" brightness=\""; fmt_float(o, g.brightness);
    o << "\" gamma=\""; fmt_float(o, g.gamma);
    o << "\" vibrancy=\""; fmt_float(o, g.vibrancy);
    o << "\">\n";
    auto xf = [&](const Xform& x, bool fin) {
        o << "   <" << (fin ? "finalxform" : "xform");
        if (!fin) { o << " weight=\""; fmt_float(o, x.weight); o << "\""; }
        o << " color=\""; fmt_float(o, x.color);
        o << "\" color_speed=\""; fmt_float(o, x.color_speed);
        o << "\" opacity=\""; fmt_float(o, x.opacity); o << "\"";
        if (x.rotation_frequency != 0.0f) o << " animate=\"1\"";
        o << " coefs=\"";
        for (int i = 0; i < 6; i++) { if (i) o << " "; fmt_float(o, x.affine[i]); }
        o << "\"";
        if (x.has_post) {
            o << " post=\"";
            for (int i = 0; i < 6; i++) { if (i) o << " "; fmt_float(o, x.post[i]); }
            o << "\"";
        }
        for (const auto& [n, v] : x.vars) { o << " " << n << "=\""; fmt_float(o, v); o << "\""; }
        for (const auto& [n, v] : x.params) { o << " " << n << "=\""; fmt_float(o, v); o << "\""; }
        o << "/>\n";
    };
    for (const auto& x : g.xforms) xf(x, false);
    if (g.has_final) xf(g.final_xf, true);
    for (int i = 0; i < 256; i++) {
        if (g.palette[i][3] == 0.0f && g.palette[i][0] == 0.0f && g.palette[i][1] == 0.0f && g.palette[i][2] == 0.0f) continue;
        o << "   <color index=\"" << i << "\" rgb=\"";
        for (int q = 0; q < 3; q++) o << (q ? " " : "") << (int)lrintf(g.palette[i][q] * 256.0f);
        o << "\"/>\n";
    }
    o << "</flame>\n";
    return o.str();
}

// ---------------------------------------------------------------------------------------------
// Seeded synthetic genomes.  Draws come from std::mt19937_64(seed) in the order written below;
// uniforms are (x >> 11) * 2^-53, so the genomes are identical on every platform.
// ---------------------------------------------------------------------------------------------
namespace {

struct Draw {
    std::mt19937_64 e;
    explicit Draw(uint64_t s) : e(s) {}
    double u01() { return (double)(e() >> 11) * (1.0 / 9007199254740992.0); }
    float U(double a, double b) { return (float)(a + (b - a) * u01()); }
    int I(int lo, int hi) { int v = lo + (int)(u01() * (double)(hi - lo + 1)); return std::min(v, hi); }
};

// random smooth palette: Catmull-Rom spline through 8 uniform control colours (ends clamped),
// sampled at 256 points and quantised to the flam3 integer form (k / 256)
void spline_palette(Draw& d, Genome& g) {
    float cp[8][3];
    for (auto& c : cp)
        for (float& v : c) v = d.U(0, 1);
    for (int k = 0; k < 256; k++) {
        double t = (double)k / 255.0 * 7.0;
        int s = std::min(6, (int)t);
        double u = t - s;
        for (int q = 0; q < 3; q++) {
            double p0 = cp[std::max(0, s - 1)][q], p1 = cp[s][q], p2 = cp[s + 1][q], p3 = cp[std::min(7, s + 2)][q];
            double v = 0.5 * ((2 * p1) + (-p0 + p2) * u + (2 * p0 - 5 * p1 + 4 * p2 - p3) * u * u +
                              (-p0 + 3 * p1 - 3 * p2 + p3) * u * u * u);
            int qv = (int)std::floor(std::min(std::max(v, 0.0), 1.0) * 256.0);
            g.palette[k][q] = (float)std::min(255, qv) / 256.0f;
        }
        g.palette[k][3] = 1.0f;
    }
}

struct PRange { const char* name; double lo, hi; bool integer; };
const PRange kParamRanges[] = {
    {"blob_high", 0.5, 1.5, false}, {"blob_low", 0.0, 0.5, false}, {"blob_waves", 2, 7, true},
    {"pdj_a", -3, 3, false}, {"pdj_b", -3, 3, false}, {"pdj_c", -3, 3, false}, {"pdj_d", -3, 3, false},
    {"fan2_x", -1, 1, false}, {"fan2_y", -1, 1, false}, {"rings2_val", 0.1, 1.0, false},
    {"perspective_angle", 0, 1, false}, {"perspective_dist", 1.5, 3, false},
    {"julian_power", 2, 6, true}, {"julian_dist", 1, 1, false},
    {"juliascope_power", 2, 6, true}, {"juliascope_dist", 1, 1, false},
    {"radial_blur_angle", -1, 1, false},
    {"pie_slices", 3, 8, true}, {"pie_rotation", 0, 6.2831853, false}, {"pie_thickness", 0.1, 0.9, false},
    {"ngon_power", 3, 3, false}, {"ngon_sides", 3, 8, true}, {"ngon_corners", 2, 2, false}, {"ngon_circle", 1, 1, false},
    {"curl_c1", -1, 1, false}, {"curl_c2", -0.5, 0.5, false},
    {"rectangles_x", 0.2, 1, false}, {"rectangles_y", 0.2, 1, false},
    {"disc2_rot", -1, 1, false}, {"disc2_twist", -1, 1, false},
    {"super_shape_n1", 1, 4, false}, {"super_shape_n2", 0.5, 2, false}, {"super_shape_n3", 0.5, 2, false},
    {"super_shape_m", 2, 8, true}, {"super_shape_holes", 0, 0.2, false}, {"super_shape_rnd", 0, 0.5, false},
    {"flower_holes", 0, 0.3, false}, {"flower_petals", 2, 8, true},
    {"conic_holes", 0, 0.3, false}, {"conic_eccentricity", 0.3, 1, false},
    {"parabola_height", 0.3, 1, false}, {"parabola_width", 0.3, 1, false},
    {"curve_xlength", 0.5, 2, false}, {"curve_ylength", 0.5, 2, false}, {"curve_xamp", -1, 1, false}, {"curve_yamp", -1, 1, false},
    {"waves2_scalex", -0.5, 0.5, false}, {"waves2_scaley", -0.5, 0.5, false}, {"waves2_freqx", 1, 4, false}, {"waves2_freqy", 1, 4, false},
    {"auger_freq", 1, 5, false}, {"auger_scale", -1, 1, false}, {"auger_sym", 0, 1, false}, {"auger_weight", 0, 1, false},
    {"flux_spread", 0, 1, false},
    {"mobius_re_a", -1, 1, false}, {"mobius_re_b", -1, 1, false}, {"mobius_re_c", -1, 1, false}, {"mobius_re_d", -1, 1, false},
    {"mobius_im_a", -1, 1, false}, {"mobius_im_b", -1, 1, false}, {"mobius_im_c", -1, 1, false}, {"mobius_im_d", -1, 1, false},
};

float draw_param(Draw& d, const std::string& p) {
    for (const auto& r : kParamRanges)
        if (p == r.name) return r.integer ? (float)d.I((int)r.lo, (int)r.hi) : d.U(r.lo, r.hi);
    return d.U(-1, 1);
}

void base_fields(Genome& g, uint32_t W, uint32_t H) {
    g.size[0] = W; g.size[1] = H;
    g.center[0] = g.center[1] = 0.0f;
    g.rotate = 0.0f;
    g.gamma = 2.2f; g.brightness = 4.0f; g.vibrancy = 1.0f;
    g.est_radius = 0; g.est_min = 0; g.est_curve = 0.4f;
}

}  // namespace

int genome_synthesize(int kind, uint64_t seed, uint32_t n_xforms, int final_xform, int force_param,
                      uint32_t W, uint32_t H, const Registry& reg, Genome& g) {
    if (W == 0 || H == 0) return fail(RF_ERR_INVALID_ARG, "synthesize: width and height must be positive");
    g = Genome();
    Draw d(seed);
    base_fields(g, W, H);
    auto xform_common = [&](Xform& x, double lo, double hi) {
        for (float& a : x.affine) a = d.U(lo, hi);
        x.weight = d.U(0.1, 1.0);
        x.color = d.U(0, 1);
        x.color_speed = 0.5f;
        x.opacity = 1.0f;
    };
    auto normalised = [&](Xform& x, const std::vector<std::string>& names) {
        std::vector<float> w;
        float s = 0;
        for (size_t i = 0; i < names.size(); i++) { w.push_back(d.U(0, 1)); s += w.back(); }
        if (!(s > 0)) s = 1;
        for (size_t i = 0; i < names.size(); i++) x.vars[names[i]] = w[i] / s;
    };
    if (kind == RF_SYNTH_SMALL) {
        // 3 xforms: affine U[-1,1], weight U[0.1,1], colour U[0,1], variation weights U[0,1]
        // normalised over {linear, sinusoidal, spherical}; [-2,2] spans the bin grid's height
        for (int i = 0; i < 3; i++) {
            Xform x;
            xform_common(x, -1, 1);
            normalised(x, {"linear", "sinusoidal", "spherical"});
            g.xforms.push_back(x);
        }
        g.scale = (float)H / 4.0f;
    } else if (kind == RF_SYNTH_RANDOM) {
        // n xforms (default 8): affine U[-1.2,1.2], weight U[0.1,1], colour U[0,1], then three
        // distinct supported variations (uniform over the table order; with force_parametric,
        // xforms 0, 1, 2 take julian, ngon, pdj first), weights U[0,1] normalised, then the
        // parameters of each chosen variation (kParamRanges; julian power an integer 2..6,
        // dist 1; ngon sides 3..8, power 3, corners 2, circle 1; pdj U[-3,3]).
        uint32_t n = n_xforms ? n_xforms : 8;
        std::vector<std::string> pool;
        for (const auto& v : builtin_variations())
            if (v.kernel_id >= 0 && reg.vars.count(v.name) && reg.vars.at(v.name).kernel_id >= 0) pool.push_back(v.name);
        static const char* forced[3] = {"julian", "ngon", "pdj"};
        for (uint32_t i = 0; i < n; i++) {
            Xform x;
            xform_common(x, -1.2, 1.2);
            std::vector<std::string> pick, avail = pool;
            if (force_param && i < 3) {
                pick.push_back(forced[i]);
                avail.erase(std::find(avail.begin(), avail.end(), std::string(forced[i])));
            }
            while (pick.size() < 3) {
                int k = d.I(0, (int)avail.size() - 1);
                pick.push_back(avail[k]);
                avail.erase(avail.begin() + k);
            }
            // an xform needs one accumulated term: pre_blur alone in `pick` never happens with 3 picks
            normalised(x, pick);
            for (const auto& v : pick)
                for (const auto& p : reg.vars.at(v).params)
                    if (!x.params.count(p)) x.params[p] = draw_param(d, p);
            g.xforms.push_back(x);
        }
        if (final_xform) {
            // final xform: a similarity, rotation U[0, 2pi), scale U[0.8, 1.2]; keeps the colour
            Xform f;
            float th = d.U(0, 6.283185307179586), s = d.U(0.8, 1.2);
            float c = s * cosf(th), sn = s * sinf(th);
            float a[6] = {c, sn, -sn, c, 0, 0};
            memcpy(f.affine, a, sizeof a);
            f.vars["linear"] = 1.0f;
            f.color = 0; f.color_speed = 0; f.opacity = 1.0f;
            g.final_xf = f;
            g.has_final = true;
        }
        g.scale = (float)H / 5.0f;
        g.est_radius = 9; g.est_min = 0; g.est_curve = 0.4f;
    } else if (kind == RF_SYNTH_CONTRACT) {
        // 6 xforms: linear parts U[-1,1]*0.05, translations U[-0.02,0.02], linear variation;
        // framed at 1500 bins per unit so the attractor covers a few thousand bins
        for (int i = 0; i < 6; i++) {
            Xform x;
            for (int k = 0; k < 4; k++) x.affine[k] = d.U(-1, 1) * 0.05f;
            for (int k = 4; k < 6; k++) x.affine[k] = d.U(-0.02, 0.02);
            x.weight = d.U(0.1, 1.0);
            x.color = d.U(0, 1);
            x.color_speed = 0.5f; x.opacity = 1.0f;
            x.vars["linear"] = 1.0f;
            g.xforms.push_back(x);
        }
        g.scale = 1500.0f * (float)H / 1080.0f;
    } else if (kind == RF_SYNTH_SPACEFILL) {
        // 16 xforms: affine U[-1,1], spherical + swirl weights U[0,1] normalised
        for (int i = 0; i < 16; i++) {
            Xform x;
            xform_common(x, -1, 1);
            normalised(x, {"spherical", "swirl"});
            g.xforms.push_back(x);
        }
        g.scale = (float)H / 4.0f;
    } else {
        return fail(RF_ERR_INVALID_ARG, "synthesize: unknown kind " + std::to_string(kind));
    }
    spline_palette(d, g);
    return genome_validate(g, reg);
}

// ---------------------------------------------------------------------------------------------
// Interpolation between two genomes (animation frames; the reference only rotates affines over
// time, main.cpp:383-395).  Xform i of the shorter genome is padded with a copy of the longer
// genome's xform i at selection weight 0; every numeric field is lerped, variation weights of
// variations present on one side only lerp from 0; parameters present on one side are taken
// as they are.
// ---------------------------------------------------------------------------------------------
namespace {
inline float lerpf(float a, float b, float t) { return a + (b - a) * t; }

Xform lerp_xform(const Xform& a, const Xform& b, float t) {
    Xform o;
    for (int i = 0; i < 6; i++) o.affine[i] = lerpf(a.affine[i], b.affine[i], t);
    o.has_post = a.has_post || b.has_post;
    if (o.has_post) {
        const float id[6] = {1, 0, 0, 1, 0, 0};
        for (int i = 0; i < 6; i++)
            o.post[i] = lerpf(a.has_post ? a.post[i] : id[i], b.has_post ? b.post[i] : id[i], t);
    }
    o.weight = lerpf(a.weight, b.weight, t);
    o.color = lerpf(a.color, b.color, t);
    o.color_speed = lerpf(a.color_speed, b.color_speed, t);
    o.opacity = lerpf(a.opacity, b.opacity, t);
    o.rotation_frequency = t < 0.5f ? a.rotation_frequency : b.rotation_frequency;
    for (const auto& [n, w] : a.vars) o.vars[n] = lerpf(w, b.vars.count(n) ? b.vars.at(n) : 0.0f, t);
    for (const auto& [n, w] : b.vars)
        if (!a.vars.count(n)) o.vars[n] = lerpf(0.0f, w, t);
    for (const auto& [n, v] : a.params) o.params[n] = b.params.count(n) ? lerpf(v, b.params.at(n), t) : v;
    for (const auto& [n, v] : b.params)
        if (!a.params.count(n)) o.params[n] = v;
    return o;
}
}  // namespace

int genome_interpolate(const Genome& a, const Genome& b, float t, const Registry& reg, Genome& out) {
    out = a;
    const size_t n = std::max(a.xforms.size(), b.xforms.size());
    out.xforms.clear();
    for (size_t i = 0; i < n; i++) {
        Xform xa, xb;
        if (i < a.xforms.size()) xa = a.xforms[i]; else { xa = b.xforms[i]; xa.weight = 0.0f; }
        if (i < b.xforms.size()) xb = b.xforms[i]; else { xb = a.xforms[i]; xb.weight = 0.0f; }
        out.xforms.push_back(lerp_xform(xa, xb, t));
    }
    if (a.has_final || b.has_final) {
        Xform ident;
        ident.affine[0] = ident.affine[3] = 1.0f;
        ident.vars["linear"] = 1.0f;
        ident.opacity = 1.0f;
        out.final_xf = lerp_xform(a.has_final ? a.final_xf : ident, b.has_final ? b.final_xf : ident, t);
        out.has_final = true;
    }
    for (int k = 0; k < 256; k++)
        for (int q = 0; q < 4; q++) out.palette[k][q] = lerpf(a.palette[k][q], b.palette[k][q], t);
    for (int q = 0; q < 2; q++) out.center[q] = lerpf(a.center[q], b.center[q], t);
    out.scale = lerpf(a.scale, b.scale, t);
    out.rotate = lerpf(a.rotate, b.rotate, t);
    out.gamma = lerpf(a.gamma, b.gamma, t);
    out.brightness = lerpf(a.brightness, b.brightness, t);
    out.vibrancy = lerpf(a.vibrancy, b.vibrancy, t);
    out.est_curve = lerpf(a.est_curve, b.est_curve, t);
    out.est_radius = (int)lrintf(lerpf((float)a.est_radius, (float)b.est_radius, t));
    out.est_min = (int)lrintf(lerpf((float)a.est_min, (float)b.est_min, t));
    return genome_validate(out, reg);
}

}  // namespace rfk
