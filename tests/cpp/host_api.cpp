// C++ client of include/refrakt.hpp: the reference's call pattern against the GB300 library.
// Host-only part (no GPU): the variation table and genome loading.  With --gpu it also warms a
// walker pool and draws into device bins.
#include <cstdio>
#include <cstring>
#include <string>

#include <cuda_runtime.h>

#include "refrakt.hpp"

int main(int argc, char** argv) {
    bool gpu = argc > 1 && !strcmp(argv[1], "--gpu");
    refrakt::flame_compiler variations{};
    if (!variations.is_variation("julian") || !variations.is_param("julian_power") ||
        variations.param_owner("julian_dist") != "julian" || variations.is_supported("bent2")) {
        std::printf("FAIL compiler\n");
        return 1;
    }
    const std::string xml =
        "<flame size=\"64 64\" scale=\"16\"><xform weight=\"1\" color=\"0\" color_speed=\"0.5\" opacity=\"1\" "
        "coefs=\"0.5 0 0 0.5 0.2 0\" linear=\"1\"/><xform weight=\"1\" color=\"1\" color_speed=\"0.5\" "
        "opacity=\"1\" coefs=\"0.5 0 0 0.5 -0.2 0\" julian=\"1\" julian_power=\"3\" julian_dist=\"1\"/></flame>";
    auto f = refrakt::flame::from_xml(xml, variations);
    if (!f || f->info().num_xforms != 2 || f->param_buffer().size() != f->info().total_params) {
        std::printf("FAIL load\n");
        return 1;
    }
    // the reference returns nullptr for a genome with an unknown attribute (flame.cpp:196)
    if (refrakt::flame::from_xml("<flame size=\"8 8\"><xform weight=\"1\" linear=\"1\" bogus=\"1\"/></flame>", variations)) {
        std::printf("FAIL unknown attribute accepted\n");
        return 1;
    }
    if (gpu) {
        refrakt::flame::set_sim_parameters(8192, 1, 1024);
        if (!f->needs_warmup()) { std::printf("FAIL needs_warmup\n"); return 1; }
        f->warmup(16, 1.2f / 60.0f);
        float* bins = nullptr;
        cudaMalloc(&bins, 64 * 64 * 16);
        cudaMemset(bins, 0, 64 * 64 * 16);
        std::size_t binned = f->draw_to_bins(bins, 64, 64, 8);
        cudaFree(bins);
        if (binned == 0 || binned > 8192u * 8u) { std::printf("FAIL draw %zu\n", binned); return 1; }
        std::printf("drawn %zu\n", binned);
    }
    std::printf("OK\n");
    return 0;
}
