// Arguments of one chaos launch (kernels.cu, and the genome-specialised kernels compiled at
// run time, specialize.cpp).  Self-contained so the run-time compiler can include it.
#pragma once

#include "rtc_types.h"

namespace rfk {

struct ChaosArgs {
    const uint32_t* progs;   // one compiled genome per temporal sample
    uint32_t prog_stride;    // words between copies
    uint32_t prog_words;     // words staged per CTA
    const float4* walk_in;   // N walkers (x, y, colour, unused)
    float4* walk_out;
    uint4* rng;              // N JSF32 states
    const uint16_t* table;   // table_size permutations of a CTA's slots (the mixing domain)
    uint32_t table_size;
    uint32_t ppts;           // walkers per temporal sample
    uint32_t chunks_per_ts;  // CTAs (mixing domains) per temporal sample
    uint32_t pass0;          // pass index of this launch's first pass
    uint32_t steps;          // passes in this launch
    uint64_t seed;
    int first_run;           // pass 0 reads the start points, jitters, draws colours
    int draw;
    int splat;               // 0: a reduction per point; 1: warp-aggregated; 2: adaptive; 3: tile (splat.cuh)
    int reset;               // 1: walkers that leave the plane restart (reset_bad_walker, device.cuh)
    uint32_t rgba_shift;     // bin addressing (splat.cuh BinTarget): 0 and 0 for the caller's
    uint32_t count_shift;    //   planes, 1 and 3 for interleaved 32-byte records
    float ss[6];             // screen affine
    // splat 3: the bins of columns [tile_x0, tile_x0 + tile_w) and rows [tile_y0, tile_y0 + tile_h)
    // (rows after flame.glsl:84's flip) accumulate in the CTA's shared memory for the whole launch
    // and are added to the bins once at its end
    uint32_t tile_x0, tile_y0, tile_w, tile_h;
    uint32_t W, H;
    float4* bins;            // RGBA sums
    uint32_t* hits;          // counts (may be null)
    const float4* palette;   // 256 entries
    unsigned long long* counters;  // [0] drawn [1] emitted [2] walker-steps
    uint8_t* trace;          // xform id per (pass, 256-group), may be null
    uint32_t trace_passes;
    uint32_t n_groups;
};

}  // namespace rfk
