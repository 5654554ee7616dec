// Instance table, work units and arguments of the batched persistent chaos launch (batch.cu and
// the genome-specialised batch kernels compiled at run time).  Self-contained so the run-time
// compiler can include it.
#pragma once

#include "rtc_types.h"

namespace rfk {

struct BatchInstance {
    const uint32_t* prog;   // compiled genome (program.h)
    uint32_t prog_words;
    uint32_t fuse;          // discarded passes at the start of every unit
    const float4* palette;  // 256 entries
    float4* bins;           // RGBA sums, W * H
    uint32_t* hits;         // counts, may be null
    uint32_t W, H;
    uint32_t splat;         // 0: a reduction per point; 1: warp-aggregated (splat.cuh)
    uint32_t reset;         // 1: walkers that leave the plane restart (reset_bad_walker, device.cuh)
    float ss[6];            // screen affine
};

// One unit is the chaos game of a single temporal sample of SLOTS walkers, seeded like the
// reference seeds a simulation of SLOTS walkers with `seed` (slot i: warmup_ctx(i + seed*SLOTS),
// flame.cpp:138-141), its start points and per-pass shuffles keyed by `seed`.
struct BatchUnit {
    uint32_t instance;      // index into the instance table
    uint32_t draw;          // drawing passes of this unit
    uint64_t seed;
};

struct BatchArgs {
    const BatchInstance* inst;
    const BatchUnit* units;
    uint32_t n_units;
    unsigned int* queue;            // next unit; zero before every launch
    const uint16_t* table;          // table_size permutations of SLOTS
    uint32_t table_size;
    uint32_t max_prog_words;
    unsigned long long* counters;   // [0] drawn [1] emitted [2] walker-steps
};

}  // namespace rfk
