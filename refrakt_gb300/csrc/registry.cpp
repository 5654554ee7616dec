// Variation registry: the built-in table of the reference's variation library and the
// reconciliation of a caller-supplied variations.yaml with it.
//
// The reference's flame_compiler (src/variation_table.cpp:182-215) loads variations.yaml and
// generates GLSL per genome.  This library evaluates variations with hand-written device code
// (kernels.cu), so a YAML file only names variations and parameters; an entry is supported
// when its snippet text hashes to the snippet the device code implements.
#include <cstdio>
#include <fstream>
#include <sstream>

#include "internal.h"

namespace rfk {

namespace {

struct Row {
    const char* name;
    std::vector<std::string> params;
    int flags;
    int draws;
    uint32_t pc;
    const char* broken;  // non-null: does not compile in the reference (variations.yaml line)
};

const std::vector<Row>& rows() {
    // Order and parameter lists follow variations.yaml:12-551; draws count the randf() calls of
    // each snippet; pc lists the precalcs it reads.
    static const std::vector<Row> r = {
        {"linear", {}, 0, 0, 0, nullptr},
        {"sinusoidal", {}, 0, 0, 0, nullptr},
        {"spherical", {}, 0, 0, PC_RSQ, nullptr},
        {"swirl", {}, 0, 0, PC_RSQ, nullptr},
        {"horseshoe", {}, 0, 0, PC_R, nullptr},
        {"polar", {}, 0, 0, PC_A | PC_R, nullptr},
        {"handkerchief", {}, 0, 0, PC_R | PC_A, nullptr},
        {"heart", {}, 0, 0, PC_R | PC_A, nullptr},
        {"disc", {}, 0, 0, PC_A | PC_R, nullptr},
        {"spiral", {}, 0, 0, PC_R | PC_SINA | PC_COSA | PC_SINR | PC_COSR, nullptr},
        {"hyperbolic", {}, 0, 0, PC_R | PC_SINA | PC_COSA, nullptr},
        {"diamond", {}, 0, 0, PC_SINA | PC_COSA | PC_SINR | PC_COSR, nullptr},
        {"ex", {}, 0, 0, PC_A | PC_R, nullptr},
        {"julia", {}, 0, 1, PC_R | PC_A, nullptr},
        {"bent", {}, 0, 0, 0, nullptr},
        {"waves", {}, 0, 0, 0, nullptr},
        {"fisheye", {}, 0, 0, PC_R, nullptr},
        {"popcorn", {}, 0, 0, 0, nullptr},
        {"exponential", {}, 0, 0, 0, nullptr},
        {"power", {}, 0, 0, PC_R | PC_SINA | PC_COSA, nullptr},
        {"cosine", {}, 0, 0, 0, nullptr},
        {"rings", {}, 0, 0, PC_R | PC_SINA | PC_COSA, nullptr},
        {"fan", {}, 0, 0, PC_A | PC_R, nullptr},
        {"blob", {"blob_high", "blob_low", "blob_waves"}, 0, 0, PC_R | PC_A | PC_SINA | PC_COSA, nullptr},
        {"pdj", {"pdj_a", "pdj_b", "pdj_c", "pdj_d"}, 0, 0, 0, nullptr},
        {"fan2", {"fan2_x", "fan2_y"}, 0, 0, PC_A | PC_R, nullptr},
        {"rings2", {"rings2_val"}, 0, 0, PC_R | PC_SINA | PC_COSA, nullptr},
        {"eyefish", {}, 0, 0, PC_R, nullptr},
        {"bubble", {}, 0, 0, PC_RSQ, nullptr},
        {"perspective", {"perspective_angle", "perspective_dist"}, 0, 0, 0, nullptr},
        {"noise", {}, 0, 2, 0, nullptr},
        {"julian", {"julian_power", "julian_dist"}, 0, 1, PC_R | PC_PHI, nullptr},
        {"juliascope", {"juliascope_power", "juliascope_dist"}, 0, 1, PC_R | PC_PHI, nullptr},
        {"blur", {}, 0, 2, 0, nullptr},
        {"gaussian_blur", {}, 0, 5, 0, nullptr},
        {"radial_blur", {"radial_blur_angle"}, VF_NO_WEIGHT_MUL, 4, PC_PHI | PC_R, nullptr},
        {"pie", {"pie_slices", "pie_rotation", "pie_thickness"}, 0, 3, 0, nullptr},
        {"ngon", {"ngon_power", "ngon_sides", "ngon_corners", "ngon_circle"}, 0, 0, PC_RSQ | PC_PHI | PC_A, nullptr},
        {"curl", {"curl_c1", "curl_c2"}, 0, 0, 0, nullptr},
        {"rectangles", {"rectangles_x", "rectangles_y"}, 0, 0, 0, nullptr},
        {"arch", {}, 0, 1, 0, nullptr},
        {"tangent", {}, 0, 0, 0, nullptr},
        {"square", {}, 0, 2, 0, nullptr},
        {"rays", {}, 0, 1, PC_RSQ, nullptr},
        {"blade", {}, 0, 1, PC_R, nullptr},
        {"secant2", {}, 0, 0, PC_R, nullptr},
        {"twintrian", {}, 0, 1, PC_R, "variations.yaml:283 reads an undeclared `diff`"},
        {"cross", {}, 0, 0, 0, nullptr},
        {"disc2", {"disc2_rot", "disc2_twist"}, 0, 0, PC_A, nullptr},
        {"super_shape", {"super_shape_n1", "super_shape_n2", "super_shape_n3", "super_shape_m",
                         "super_shape_holes", "super_shape_rnd"}, 0, 1, PC_PHI | PC_R, nullptr},
        {"flower", {"flower_holes", "flower_petals"}, 0, 1, PC_PHI | PC_R, nullptr},
        {"conic", {"conic_holes", "conic_eccentricity"}, 0, 1, PC_R, nullptr},
        {"parabola", {"parabola_height", "parabola_width"}, 0, 2, PC_R | PC_SINR | PC_COSR, nullptr},
        {"bent2", {"bent2_x", "bent2_y"}, 0, 0, 0, "variations.yaml:337 ternaries lack `?`"},
        {"bipolar", {"bipolar_shift"}, 0, 0, PC_RSQ, "variations.yaml:348 assigns an undeclared `y`"},
        {"boarders", {}, 0, 1, 0, nullptr},
        {"butterfly", {}, 0, 0, 0, nullptr},
        {"cell", {"cell_size"}, 0, 0, 0, "variations.yaml:405-410 `cell.xy` and unbalanced braces"},
        {"cpow", {"cpow_power", "cpow_r", "cpow_i"}, 0, 1, PC_RSQ | PC_PHI, "variations.yaml:423 reads an undeclared `cpow_vd`"},
        {"curve", {"curve_xlength", "curve_ylength", "curve_xamp", "curve_yamp"}, 0, 0, 0, nullptr},
        {"edisc", {}, 0, 0, PC_RSQ, "variations.yaml:443 reads an undeclared `edisc_xmx`"},
        {"foci", {}, 0, 0, 0, nullptr},
        {"oscope", {}, 0, 0, 0, "variations.yaml:457 is an empty entry"},
        {"loonie", {}, 0, 0, PC_RSQ, nullptr},
        {"exp", {}, 0, 0, 0, nullptr},
        {"log", {}, 0, 0, PC_RSQ | PC_PHI, nullptr},
        {"sin", {}, 0, 0, 0, nullptr},
        {"cos", {}, 0, 0, 0, nullptr},
        {"sinh", {}, 0, 0, 0, nullptr},
        {"pre_blur", {}, VF_PRE_XFORM, 5, 0, nullptr},
        {"waves2", {"waves2_scalex", "waves2_scaley", "waves2_freqx", "waves2_freqy"}, 0, 0, 0, nullptr},
        {"cylinder", {}, 0, 0, 0, nullptr},
        {"coth", {}, 0, 0, 0, "variations.yaml:506 a stray `f` follows the result"},
        {"auger", {"auger_freq", "auger_scale", "auger_sym", "auger_weight"}, 0, 0, 0, nullptr},
        {"flux", {"flux_spread"}, 0, 0, 0, nullptr},
        {"mobius", {"mobius_re_a", "mobius_re_b", "mobius_re_c", "mobius_re_d", "mobius_im_a",
                    "mobius_im_b", "mobius_im_c", "mobius_im_d"}, 0, 0, 0, nullptr},
    };
    return r;
}

}  // namespace

const std::vector<VariationDef>& builtin_variations() {
    static const std::vector<VariationDef> defs = [] {
        std::vector<VariationDef> v;
        int id = 0;
        for (const auto& r : rows()) {
            VariationDef d;
            d.name = r.name;
            d.params = r.params;
            d.flags = r.flags;
            d.draws = r.draws;
            d.precalc = r.pc;
            d.kernel_id = r.broken ? -1 : id;
            if (r.broken) d.note = std::string("does not compile in the reference: ") + r.broken;
            v.push_back(d);
            id++;
        }
        return v;
    }();
    return defs;
}

std::shared_ptr<const Registry> builtin_registry() {
    static const std::shared_ptr<const Registry> reg = [] {
        auto r = std::make_shared<Registry>();
        for (const auto& d : builtin_variations()) {
            r->vars[d.name] = d;
            for (const auto& p : d.params) r->param_owner[p] = d.name;
        }
        // variations.yaml:1-10
        r->common = {{"r", "length(v)"}, {"rsq", "x*x + y*y"}, {"a", "atan(x, y)"}, {"phi", "atan(y, x)"},
                     {"sina", "x / r"}, {"cosa", "y / r"}, {"sinr", "sin(r)"}, {"cosr", "cos(r)"},
                     {"lr", "local invocation index / (group size - 1)"}};
        return std::shared_ptr<const Registry>(r);
    }();
    return reg;
}

// FNV-1a over the snippet texts (src, a 0x1f separator, result) as a YAML reader returns them.
// Hashes of the reference's snippets (snippet_hashes.cpp, generated by gen_snippet_hashes.py).
const std::map<std::string, uint64_t>& builtin_snippet_hashes();

int load_registry_yaml(const std::string& path, std::shared_ptr<const Registry>& out) {
    std::ifstream f(path);
    if (!f) return fail(RF_ERR_IO, "cannot read variation library " + path);
    std::stringstream ss;
    ss << f.rdbuf();
    YNode root;
    std::string err;
    if (!parse_yaml(ss.str(), root, err)) return fail(RF_ERR_PARSE, "variation library " + path + ": " + err);
    const YNode* vars = root.get("variations");
    if (!vars || vars->kind != YNode::Map) return fail(RF_ERR_PARSE, "variation library has no `variations` mapping");
    auto reg = std::make_shared<Registry>();
    std::map<std::string, const VariationDef*> builtin;
    for (const auto& d : builtin_variations()) builtin[d.name] = &d;
    const auto& hashes = builtin_snippet_hashes();
    for (const auto& [name, node] : vars->map) {
        VariationDef d;
        d.name = name;
        std::string src, res;
        if (node.kind == YNode::Map) {
            if (const YNode* p = node.get("param"); p && p->kind == YNode::Map)
                for (const auto& kv : p->map) d.params.push_back(kv.first);
            if (const YNode* fl = node.get("flags"); fl && fl->kind == YNode::List)
                for (const auto& s : fl->list) {
                    if (s == "no_weight_mul") d.flags |= VF_NO_WEIGHT_MUL;
                    if (s == "pre_xform") d.flags |= VF_PRE_XFORM;
                }
            if (const YNode* s = node.get("src"); s && s->kind == YNode::Scalar) src = s->text;
            if (const YNode* s = node.get("result"); s && s->kind == YNode::Scalar) res = s->text;
        }
        auto it = builtin.find(name);
        if (it == builtin.end()) {
            d.note = "no device implementation of variation `" + name + "`";
        } else if (it->second->kernel_id < 0) {
            d.note = it->second->note;
        } else {
            auto hv = hashes.find(name);
            uint64_t h = snippet_hash(src, res);
            if (d.params != it->second->params || d.flags != it->second->flags) {
                d.note = "parameters or flags of `" + name + "` differ from the device implementation";
            } else if (hv == hashes.end() || hv->second != h) {
                d.note = "snippet of `" + name + "` differs from the one the device code implements";
            } else {
                d.kernel_id = it->second->kernel_id;
                d.draws = it->second->draws;
                d.precalc = it->second->precalc;
            }
        }
        for (const auto& p : d.params) reg->param_owner[p] = name;
        reg->vars[name] = d;
    }
    if (const YNode* c = root.get("common"); c && c->kind == YNode::Map)
        for (const auto& [k, v] : c->map) reg->common[k] = v.text;
    out = reg;
    return 0;
}

}  // namespace rfk
