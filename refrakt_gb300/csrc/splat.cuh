// Histogram splat of one point per lane (flame.glsl:81-86): RGBA sums (palette colour, opacity)
// and a hit count per bin, as L2 reductions.
//
//   splat_global — one red.global.add.v4.f32 and one red.global.add.u32 per point.
//   splat_warp   — warp-aggregated: lanes whose points fall into the same bin are found with
//                  match.any; the lowest lane of each set adds the set's colours and issues one
//                  v4 reduction and one count reduction of the set's size.  Where the attractor is
//                  compact (every lane of a warp applies the same xform, so a contracting map
//                  sends the warp's 32 walkers into a few bins) this divides the reductions on the
//                  hottest addresses by up to 32.  The colour sums are added in a tree over the
//                  set's lanes (the peer reduction of E. Westphal, "Voting and shuffling to
//                  optimize atomic operations", GTC 2015), so only their FP32 rounding order
//                  differs from splat_global; the counts are exact either way.
//   splat_adaptive — per warp and pass: lane pairs (2i, 2i+1) compare bins with one shuffle;
//                  the warp takes splat_warp when any pair shares a bin (a compact attractor),
//                  splat_global otherwise, so spread attractors pay one shuffle and one vote.
//   splat_tile   — a per-CTA histogram tile in shared memory for compact attractors: points in
//                  the tile's rectangle of bins go to shared-memory atomics (aggregated within
//                  the warp as splat_adaptive does), the others to splat_global; the chaos
//                  kernel adds the tile's non-empty bins to the histogram once per launch, so
//                  the L2 sees a few reductions per bin per CTA instead of one per point.
#pragma once

#include "rtc_types.h"

namespace rfk {

constexpr uint32_t kNoBin = 0xffffffffu;

// Where a bin's RGBA sums and count live: rgba + (bin << rs) (float4 units) and
// count + (bin << cs) (uint32 units).  The caller's planes: rs = cs = 0.  The interleaved
// 32-byte record {RGBA, count, pad} of histograms larger than L2: rs = 1, cs = 3, count = the
// record base + 4 -- one DRAM sector per point instead of two.
struct BinTarget {
    float4* rgba;
    uint32_t* count;  // may be null
    uint32_t rs, cs;
    __device__ __forceinline__ float4* at_rgba(uint32_t bin) const { return rgba + ((size_t)bin << rs); }
    __device__ __forceinline__ uint32_t* at_count(uint32_t bin) const { return count + ((size_t)bin << cs); }
};

__device__ __forceinline__ void red_add_f32x4(float4* p, float a, float b, float c, float d) {
    asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(p), "f"(a), "f"(b), "f"(c), "f"(d)
                 : "memory");
}
__device__ __forceinline__ void red_add_u32x1(uint32_t* p, uint32_t v) {
    asm volatile("red.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ void splat_global(const BinTarget& t, uint32_t bin, float4 v) {
    if (bin == kNoBin) return;
    red_add_f32x4(t.at_rgba(bin), v.x, v.y, v.z, v.w);
    if (t.count) red_add_u32x1(t.at_count(bin), 1u);
}

// Every lane of the warp must call this (bin = kNoBin for lanes without a point).
__device__ __forceinline__ void splat_warp(const BinTarget& t, uint32_t bin, float4 v) {
    const unsigned lane = threadIdx.x & 31u;
    const unsigned peers = __match_any_sync(0xffffffffu, bin);
    if (__all_sync(0xffffffffu, peers == (1u << lane))) {  // no two lanes share a bin
        splat_global(t, bin, v);
        return;
    }
    unsigned rank = __popc(peers & ((1u << lane) - 1u));
    unsigned above = peers & (0xfffffffeu << lane);
    while (__any_sync(0xffffffffu, above != 0u)) {
        const int next = __ffs(above);  // 1 + lane of the next peer above, 0 if none
        const int srcl = next ? next - 1 : (int)lane;
        const float tx = __shfl_sync(0xffffffffu, v.x, srcl);
        const float ty = __shfl_sync(0xffffffffu, v.y, srcl);
        const float tz = __shfl_sync(0xffffffffu, v.z, srcl);
        const float tw = __shfl_sync(0xffffffffu, v.w, srcl);
        if (next) {
            v.x += tx;
            v.y += ty;
            v.z += tz;
            v.w += tw;
        }
        above &= __ballot_sync(0xffffffffu, (rank & 1u) == 0u);  // lanes at odd rank are merged
        rank >>= 1;
    }
    if (bin != kNoBin && (peers & ((1u << lane) - 1u)) == 0u) {  // lowest lane of its set
        red_add_f32x4(t.at_rgba(bin), v.x, v.y, v.z, v.w);
        if (t.count) red_add_u32x1(t.at_count(bin), (uint32_t)__popc(peers));
    }
}

// The peer reduction of splat_warp: every lane of the warp calls it with its key (kNoBin for
// none); the lowest lane of each set of equal keys returns true with the set's colour sum in v
// and the set's size in n.
__device__ __forceinline__ bool warp_aggregate(uint32_t key, float4& v, uint32_t& n) {
    const unsigned lane = threadIdx.x & 31u;
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    unsigned rank = __popc(peers & ((1u << lane) - 1u));
    unsigned above = peers & (0xfffffffeu << lane);
    while (__any_sync(0xffffffffu, above != 0u)) {
        const int next = __ffs(above);
        const int srcl = next ? next - 1 : (int)lane;
        const float tx = __shfl_sync(0xffffffffu, v.x, srcl);
        const float ty = __shfl_sync(0xffffffffu, v.y, srcl);
        const float tz = __shfl_sync(0xffffffffu, v.z, srcl);
        const float tw = __shfl_sync(0xffffffffu, v.w, srcl);
        if (next) {
            v.x += tx;
            v.y += ty;
            v.z += tz;
            v.w += tw;
        }
        above &= __ballot_sync(0xffffffffu, (rank & 1u) == 0u);
        rank >>= 1;
    }
    n = (uint32_t)__popc(peers);
    return key != kNoBin && (peers & ((1u << lane) - 1u)) == 0u;
}

// The CTA's shared-memory histogram tile (splat_tile): RGBA sums and counts of tile_w x tile_h bins.
struct TileTarget {
    float4* rgba;
    uint32_t* count;
};

__device__ __forceinline__ void tile_or_global_add(const BinTarget& t, const TileTarget& tt, uint32_t key, float4 v,
                                                   uint32_t n) {
    if (key & 0x80000000u) {  // a tile bin
        const uint32_t local = key & 0x7fffffffu;
        atomicAdd(&tt.rgba[local].x, v.x);
        atomicAdd(&tt.rgba[local].y, v.y);
        atomicAdd(&tt.rgba[local].z, v.z);
        atomicAdd(&tt.rgba[local].w, v.w);
        atomicAdd(&tt.count[local], n);
    } else {
        red_add_f32x4(t.at_rgba(key), v.x, v.y, v.z, v.w);
        if (t.count) red_add_u32x1(t.at_count(key), n);
    }
}

// Every lane of the warp must call this; `local` is the point's index in the tile, or kNoBin when
// the point misses the tile (then `bin`, its histogram bin or kNoBin, takes the L2).  Tile bins
// and histogram bins are aggregated within the warp alike (as splat_adaptive), under keys that
// cannot collide (tile bins carry the top bit; the bin grid holds fewer than 2^31 bins).
__device__ __forceinline__ void splat_tile(const BinTarget& t, const TileTarget& tt, uint32_t bin, uint32_t local,
                                           float4 v) {
    const uint32_t key = local != kNoBin ? (local | 0x80000000u) : bin;
    const uint32_t other = __shfl_xor_sync(0xffffffffu, key, 1);
    if (__any_sync(0xffffffffu, key != kNoBin && key == other)) {
        uint32_t n;
        if (warp_aggregate(key, v, n)) tile_or_global_add(t, tt, key, v, n);
    } else if (key != kNoBin) {
        tile_or_global_add(t, tt, key, v, 1u);
    }
}

// Every lane of the warp must call this.
__device__ __forceinline__ void splat_adaptive(const BinTarget& t, uint32_t bin, float4 v) {
    const uint32_t other = __shfl_xor_sync(0xffffffffu, bin, 1);
    if (__any_sync(0xffffffffu, bin != kNoBin && bin == other)) splat_warp(t, bin, v);
    else splat_global(t, bin, v);
}

}  // namespace rfk
