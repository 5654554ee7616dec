// Host-side internals of the refrakt_gb300 library (not part of the ABI).
#pragma once

#include <stdint.h>

#include <map>
#include <memory>
#include <string>
#include <vector>

#include "program.h"
#include "refrakt.h"

namespace rfk {

// ---------------------------------------------------------------------------------------------
// errors: every ABI entry point returns a status and leaves a per-thread message
// ---------------------------------------------------------------------------------------------
int fail(int status, const std::string& msg);
void clear_error();

// ---------------------------------------------------------------------------------------------
// variation registry — the names, parameters and flags of the reference's variations.yaml
// (variations.yaml:12-551, read by src/variation_table.cpp:182-215)
// ---------------------------------------------------------------------------------------------
enum : int { VF_NO_WEIGHT_MUL = 1, VF_PRE_XFORM = 2 };

struct VariationDef {
    std::string name;
    std::vector<std::string> params;  // declaration order
    int flags = 0;
    int draws = 0;                    // RNG draws per evaluation
    uint32_t precalc = 0;             // PC_* bits the formula reads
    int kernel_id = -1;               // case of the device switch; -1: not evaluable
    std::string note;                 // why a variation is unsupported
};

struct Registry {
    std::map<std::string, VariationDef> vars;        // map order, as the reference's vars_
    std::map<std::string, std::string> param_owner;  // param -> variation
    std::map<std::string, std::string> common;       // precalc name -> expression text
};

// the built-in table (the kernels' variation set)
const std::vector<VariationDef>& builtin_variations();
std::shared_ptr<const Registry> builtin_registry();
// parse a variation YAML and reconcile it with the kernels' set
int load_registry_yaml(const std::string& path, std::shared_ptr<const Registry>& out);
uint64_t snippet_hash(const std::string& src, const std::string& result);

// ---------------------------------------------------------------------------------------------
// mini parsers
// ---------------------------------------------------------------------------------------------
struct YNode {
    enum Kind { Null, Scalar, Map, List } kind = Null;
    std::string text;
    std::vector<std::pair<std::string, YNode>> map;
    std::vector<std::string> list;
    const YNode* get(const std::string& k) const {
        for (const auto& kv : map) if (kv.first == k) return &kv.second;
        return nullptr;
    }
};
bool parse_yaml(const std::string& text, YNode& out, std::string& err);

struct XNode {
    std::string name;
    std::vector<std::pair<std::string, std::string>> attrs;
    std::vector<XNode> kids;
    std::string text;
    const std::string* attr(const char* k) const {
        for (const auto& a : attrs) if (a.first == k) return &a.second;
        return nullptr;
    }
};
bool parse_xml(const std::string& text, std::vector<XNode>& roots, std::string& err);

// ---------------------------------------------------------------------------------------------
// genome (src/flame.hpp:21-61)
// ---------------------------------------------------------------------------------------------
struct Xform {
    float affine[6] = {0, 0, 0, 0, 0, 0};
    bool has_post = false;
    float post[6] = {1, 0, 0, 1, 0, 0};
    std::map<std::string, float> vars;    // map order = codegen order (variation_table.cpp:107)
    std::map<std::string, float> params;  // map order = buffer order (flame.cpp:50)
    float weight = 0, color = 0, color_speed = 0, rotation_frequency = 0, opacity = 0;
};

struct Genome {
    std::vector<Xform> xforms;
    bool has_final = false;
    Xform final_xf;
    float palette[256][4] = {};
    unsigned size[2] = {0, 0};
    float center[2] = {0, 0};
    float scale = 0, rotate = 0;
    int est_min = 0, est_radius = 0;
    float est_curve = 0;
    float gamma = 0, vibrancy = 0, brightness = 0;
    // flam3 fields the reference ignores, kept for output framing
    unsigned supersample = 1;
    float filter = 0;      // spatial filter radius (output pixels); 0: the ss x ss box
    int filter_shape = 0;  // rf_filter_shape
};

int genome_from_xml(const std::string& xml, const Registry& reg, Genome& g);
std::string genome_to_xml(const Genome& g);
int genome_validate(const Genome& g, const Registry& reg);
int genome_param_buffer(const Genome& g, std::vector<float>& buf, std::string* layout_json);
int genome_program(const Genome& g, const Registry& reg, std::vector<uint32_t>& prog);
void genome_screen_affine(const Genome& g, uint32_t w, uint32_t h, float out[6]);
int genome_xform_draws(const Genome& g, const Registry& reg, int xi);
int genome_interpolate(const Genome& a, const Genome& b, float t, const Registry& reg, Genome& out);
int genome_synthesize(int kind, uint64_t seed, uint32_t n_xforms, int final_xform, int force_param,
                      uint32_t width, uint32_t height, const Registry& reg, Genome& g);

}  // namespace rfk
