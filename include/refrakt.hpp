// refrakt_gb300 — C++ mirror of the reference's flame_compiler and flame classes over the C ABI
// (include/refrakt.h).  Header-only; link librefrakt_gb300.so.
//
// The reference's interface (src/variation_table.hpp:20-59, src/flame.hpp:41-173) keeps its
// names and call pattern here:
//
//     refrakt::flame::set_sim_parameters(2048 * 1024, 512, 1024);    // flame.cpp:105
//     refrakt::flame_compiler variations{};                          // variation_table.cpp:182
//     auto f = refrakt::flame::load_flame("flames/x.flam3", variations);  // nullptr on failure
//     if (f->needs_warmup()) f->warmup(16, 1.2f / 60.0f);
//     std::size_t binned = f->draw_to_bins(bins, width, height, 128);
//
// The reference's bins are a GL storage buffer of vec4; here they are caller-owned device
// memory: `bins` is a float4 (RGB sums, opacity sum) device array of width * height, and an
// optional uint32 count array.  Errors that the reference reports by printing and returning
// nullptr do the same in load_flame; every other failure throws refrakt::error.
#ifndef REFRAKT_GB300_HPP
#define REFRAKT_GB300_HPP

#include <cstddef>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "refrakt.h"

namespace refrakt {

class error : public std::runtime_error {
public:
    error(int status, const std::string& what) : std::runtime_error(what), status_(status) {}
    int status() const { return status_; }
private:
    int status_;
};

inline void check(int rc) {
    if (rc != RF_OK) throw error(rc, rf_last_error());
}

// flame_compiler (src/variation_table.hpp:20-59)
class flame_compiler {
public:
    // The reference reads variations.yaml from the working directory; the default constructor
    // uses the built-in copy of that table, the path constructor reads a file.
    flame_compiler() { check(rf_compiler_create(nullptr, &h_)); }
    explicit flame_compiler(const std::string& yaml_path) { check(rf_compiler_create(yaml_path.c_str(), &h_)); }
    ~flame_compiler() { rf_compiler_destroy(h_); }
    flame_compiler(const flame_compiler&) = delete;
    flame_compiler& operator=(const flame_compiler&) = delete;

    bool is_param(const std::string& n) const { return rf_compiler_is_param(h_, n.c_str()) != 0; }
    bool is_variation(const std::string& n) const { return rf_compiler_is_variation(h_, n.c_str()) != 0; }
    bool is_common(const std::string& n) const { return rf_compiler_is_common(h_, n.c_str()) != 0; }
    bool is_supported(const std::string& n) const { return rf_compiler_is_supported(h_, n.c_str()) != 0; }
    std::string param_owner(const std::string& p) const {
        char buf[256];
        check(rf_compiler_param_owner(h_, p.c_str(), buf, sizeof buf));
        return buf;
    }
    std::vector<std::string> get_parameters_for_variation(const std::string& n) const {
        char buf[1024];
        check(rf_compiler_variation_params(h_, n.c_str(), buf, sizeof buf));
        std::vector<std::string> out;
        std::string s(buf);
        size_t p = 0;
        while (!s.empty() && p <= s.size()) {
            size_t c = s.find(',', p);
            if (c == std::string::npos) c = s.size();
            out.push_back(s.substr(p, c - p));
            p = c + 1;
        }
        return out;
    }
    std::vector<std::string> variations() const {
        std::vector<std::string> out;
        char buf[256];
        for (int i = 0, n = rf_compiler_num_variations(h_); i < n; i++) {
            check(rf_compiler_variation_name(h_, i, buf, sizeof buf));
            out.push_back(buf);
        }
        return out;
    }
    const rf_compiler* handle() const { return h_; }

private:
    rf_compiler* h_ = nullptr;
};

// flame (src/flame.hpp:41-173)
class flame {
public:
    // flame::load_flame (flame.cpp:160-226): nullptr when the genome cannot be used.
    static std::unique_ptr<flame> load_flame(const std::string& path, const flame_compiler& vt) {
        rf_flame* h = nullptr;
        if (rf_flame_load(path.c_str(), vt.handle(), &h) != RF_OK) return nullptr;
        return std::unique_ptr<flame>(new flame(h));
    }
    static std::unique_ptr<flame> from_xml(const std::string& xml, const flame_compiler& vt) {
        rf_flame* h = nullptr;
        if (rf_flame_load_xml(xml.c_str(), vt.handle(), &h) != RF_OK) return nullptr;
        return std::unique_ptr<flame>(new flame(h));
    }

    // flame::set_sim_parameters (flame.cpp:105-158): the walker pool every flame draws with.
    static void set_sim_parameters(std::size_t total_particles, std::size_t temporal_samples,
                                   std::size_t shuffle_count, int device = 0) {
        rf_sim_desc d{};
        d.walkers = total_particles;
        d.temporal_samples = (uint32_t)temporal_samples;
        d.shuffle_count = (uint32_t)shuffle_count;
        d.device = device;
        rf_sim* s = nullptr;
        check(rf_sim_create(&d, &s));
        sim().reset(s);
    }

    bool needs_warmup() const { return !sim() || rf_needs_warmup(sim().get(), h_) != 0; }
    void warmup(std::size_t num_passes, float tss_width) { check(rf_warmup(need_sim(), h_, (uint32_t)num_passes, tss_width)); }
    // draw_to_bins(bins, bins_width, num_iter) (flame.cpp:283-330); bins are device memory.
    std::size_t draw_to_bins(float* bins_rgba, std::size_t bins_width, std::size_t bins_height, int num_iter,
                             uint32_t* bins_hits = nullptr) {
        uint64_t drawn = 0;
        check(rf_draw_to_bins(need_sim(), h_, bins_rgba, bins_hits, (uint32_t)bins_width, (uint32_t)bins_height,
                              (uint32_t)num_iter, &drawn));
        return (std::size_t)drawn;
    }

    rf_flame_info info() const {
        rf_flame_info i{};
        check(rf_flame_get_info(h_, &i));
        return i;
    }
    std::vector<float> param_buffer() const {
        size_t n = 0;
        check(rf_flame_param_buffer(h_, nullptr, 0, &n));
        std::vector<float> v(n);
        check(rf_flame_param_buffer(h_, v.data(), n, &n));
        return v;
    }
    // print_debug_info (flame.hpp:130): the parameter layout as JSON
    std::string buffer_map_json() const {
        size_t n = 0;
        check(rf_flame_param_layout(h_, nullptr, 0, &n));
        std::string s(n, '\0');
        check(rf_flame_param_layout(h_, &s[0], n, &n));
        s.resize(n ? n - 1 : 0);
        return s;
    }
    std::string to_xml() const {
        size_t n = 0;
        check(rf_flame_to_xml(h_, nullptr, 0, &n));
        std::string s(n, '\0');
        check(rf_flame_to_xml(h_, &s[0], n, &n));
        s.resize(n ? n - 1 : 0);
        return s;
    }
    void set_xform_value(int xform, const std::string& name, float v) { check(rf_flame_set_xform_value(h_, xform, name.c_str(), v)); }
    rf_flame* handle() const { return h_; }
    static rf_sim* simulation() { return sim().get(); }

    ~flame() { rf_flame_free(h_); }
    flame(const flame&) = delete;
    flame& operator=(const flame&) = delete;

private:
    explicit flame(rf_flame* h) : h_(h) {}
    struct sim_deleter { void operator()(rf_sim* s) const { rf_sim_destroy(s); } };
    // the reference keeps the walker pool in static members (flame.hpp:150-156)
    static std::unique_ptr<rf_sim, sim_deleter>& sim() {
        static std::unique_ptr<rf_sim, sim_deleter> s;
        return s;
    }
    static rf_sim* need_sim() {
        if (!sim()) throw error(RF_ERR_INVALID_ARG, "flame::set_sim_parameters has not been called");
        return sim().get();
    }
    rf_flame* h_;
};

}  // namespace refrakt

#endif
