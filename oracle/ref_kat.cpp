// Known-answer entry points over the reference's own host sources — TEST INFRASTRUCTURE ONLY.
// Compiled by oracle/ref_build.py together with the reference's src/hammersley.cpp, with the
// reference's src/ directory on the include path; never part of the product library.
#include <array>
#include <cstdint>
#include <vector>

#include "util.hpp"  // reference src/util.hpp: jsf32::ctx, jsf32::ranval, jsf32::warmup_ctx

std::vector<std::array<float, 4>> make_sample_points(std::uint32_t count);  // src/hammersley.cpp:29

extern "C" {

void ref_jsf_warmup(uint32_t seed, uint32_t out[4]) {
    jsf32::ctx c;
    jsf32::warmup_ctx(c, seed);
    out[0] = c.a; out[1] = c.b; out[2] = c.c; out[3] = c.d;
}

// util.hpp's ranval (returns d; used by the reference only to warm states)
uint32_t ref_jsf_ranval_cpu(uint32_t st[4]) {
    jsf32::ctx c{st[0], st[1], st[2], st[3]};
    uint32_t v = jsf32::ranval(c);
    st[0] = c.a; st[1] = c.b; st[2] = c.c; st[3] = c.d;
    return v;
}

void ref_sample_points(uint32_t count, float* out4) {
    auto pts = make_sample_points(count);
    for (uint32_t i = 0; i < count; i++)
        for (int k = 0; k < 4; k++) out4[4 * i + k] = pts[i][k];
}

}
