// Definitions of the opaque ABI handles, shared by the host runtime's translation units.
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "internal.h"

struct rf_compiler {
    std::shared_ptr<const rfk::Registry> reg;
};

struct rf_flame {
    rfk::Genome g;
    std::shared_ptr<const rfk::Registry> reg;
    uint64_t uid = 0;
    uint64_t version = 0;
};

struct rf_sim {
    rf_sim_desc d{};
    int device = 0;
    cudaStream_t stream = nullptr;
    uint64_t N = 0;
    uint32_t T = 1, ppts = 0, slots = 4096, threads = 1024, L = 32, table_size = 1024;
    float4* walk[2] = {nullptr, nullptr};
    int cur = 0;
    uint4* rng = nullptr;
    uint16_t* table = nullptr;
    uint32_t* base_prog = nullptr;
    uint32_t* progs = nullptr;
    uint32_t prog_stride = 0, prog_words = 0;
    float4* palette = nullptr;
    unsigned long long* counters = nullptr;  // [0] drawn [1] emitted [2] walker-steps [3] exchange waits that ran out
    uint8_t* trace = nullptr;
    uint32_t trace_passes = 0;
    uint64_t warmed_uid = 0, warmed_version = 0;
    uint32_t pass = 0;
    int splat = RF_SPLAT_AUTO;
    const void* spec = nullptr;  // genome-specialised kernel of the warmed flame (specialize.cpp)
    int spec_splat = -1;              // the splat strategy compiled into it (ChaosArgs.splat code)
    int reset = 0;                    // walker reset of flame.glsl:68 (rf_set_bad_value_reset)
    uint32_t tile[4] = {0, 0, 0, 0};  // the tile splat's bins: x0, y0, w, h (rf_set_splat_tile)
    // RF_SPLAT_AUTO on a compact attractor, per bin grid auto_tile_wh: 0 undecided (the next
    // drawing launch of >= 32 passes warms the grid up); 2 the next one is timed untiled, then a
    // tile is fitted to the hits; 3 a tile fitted (the next launch of that length is timed with
    // it); 4 both timed, deciding when the second has finished; 1 the tile splat over auto_tile;
    // -1 no tile
    int auto_tile_state = 0;
    uint32_t auto_tile[4] = {0, 0, 0, 0};
    uint32_t auto_tile_wh[2] = {0, 0};
    uint32_t auto_tile_passes = 0;
    cudaEvent_t tile_ev[4] = {nullptr, nullptr, nullptr, nullptr};
    int spec_reset = -1;              // the reset setting compiled into the specialised kernel
    int spec_pipe = 0;                // 1: the specialised kernel has the pipelined walker exchange
    uint32_t table_phases = 0;        // phases per pass the shuffle table is pipelined for (0: uniform)
    int exchange = RF_EXCHANGE_AUTO;  // rf_set_exchange
    // RF_EXCHANGE_AUTO: 0/1 — the next full drawing launch is timed as the barrier / pipelined form;
    // 2 — both timed, deciding when the second has finished; 3 — decided (tune_pipe)
    int tune_step = 0;
    uint32_t tune_passes = 0;         // the length of the first timed launch (the second must match)
    int tune_pipe = 1;                // the form chosen (the pipelined one until decided)
    cudaEvent_t tune_ev[4] = {nullptr, nullptr, nullptr, nullptr};
    std::vector<uint32_t> spec_prog;  // the warmed program, to specialise again for another strategy
    int bin_layout = RF_BINS_AUTO;
    uint32_t rgba_shift = 0, count_shift = 0;  // BinTarget addressing of the next launches
    float4* rec = nullptr;       // interleaved bin records (32 B per bin), all zero between calls
    size_t rec_n = 0;
    // rf_render scratch
    float4* r_bins = nullptr;
    uint32_t* r_hits = nullptr;
    float4* r_de = nullptr;
    uchar4* r_img = nullptr;
    double* r_stats = nullptr;
    uint8_t* r_rad = nullptr;     // density estimation: a radius byte per bin
    float* r_dw = nullptr;        // density estimation: kernel weights of every radius up to 100
    size_t r_bins_n = 0, r_img_n = 0, r_rad_n = 0;
};

