// The batched persistent chaos launch's body (batch.cu, and the genome-specialised batch kernels
// compiled at run time, specialize.cpp), parameterised by the xform evaluator as chaos_body.cuh.
//
// The work is cut into units: one unit is a self-contained chaos game of SLOTS walkers of one
// genome — its own JSF32 seeds, start points, fuse passes and draw passes — which is the
// reference's own organisation of a temporal sample (flame.cpp:112, 4096 walkers per sample at
// its defaults) run to completion inside one CTA.  Walkers and RNG states never leave shared
// memory.  A persistent grid pulls units from a global counter (the work queue), so genomes of
// different cost share the GPU without a launch per genome.
#pragma once

#include "batch_args.h"
#include "chaos_body.cuh"

namespace rfk {

__host__ __device__ inline size_t batch_smem_bytes(int slots, uint32_t max_prog_words) {
    size_t b = ((size_t)max_prog_words * 4 + 15) & ~(size_t)15;
    b += 256 * 16;                              // palette
    b += (size_t)2 * slots * 16;                // walker exchange
    b += (size_t)slots * 16;                    // JSF32 states
    b += (size_t)2 * (slots / kGroup) * 4;      // group xform ids
    b += 16;                                    // unit id, permutation ids
    return b;
}

template <int THREADS, int SPT, class Eval>
__device__ __forceinline__ void batch_body(const BatchArgs& A) {
    constexpr uint32_t SLOTS = (uint32_t)THREADS * SPT;
    constexpr int G = SLOTS / kGroup;
    extern __shared__ __align__(16) unsigned char smem[];
    uint32_t* s_prog = reinterpret_cast<uint32_t*>(smem);
    float4* s_pal = reinterpret_cast<float4*>(smem + (((size_t)A.max_prog_words * 4 + 15) & ~(size_t)15));
    float4* s_w = s_pal + 256;
    uint4* s_rng = reinterpret_cast<uint4*>(s_w + 2 * SLOTS);
    int* s_xid = reinterpret_cast<int*>(s_rng + SLOTS);
    uint32_t* s_misc = reinterpret_cast<uint32_t*>(s_xid + 2 * G);  // [0] unit, [1..2] permutation ids

    const int tid = threadIdx.x;
    const int dphase = draw_phase<THREADS, SPT>(tid);
    uint32_t drawn = 0, emitted = 0;
    unsigned long long steps = 0;

    for (;;) {
        if (tid == 0) s_misc[0] = atomicAdd(A.queue, 1u);
        __syncthreads();
        const uint32_t u = s_misc[0];
        if (u >= A.n_units) break;
        const BatchUnit unit = A.units[u];
        const BatchInstance& I = A.inst[unit.instance];
        for (uint32_t i = tid; i < I.prog_words; i += THREADS) s_prog[i] = I.prog[i];
        for (int i = tid; i < 256; i += THREADS) s_pal[i] = I.palette[i];
        const uint32_t passes = I.fuse + unit.draw;
        // seeds and start points of this unit's slots (flame.cpp:138-141, hammersley.cpp:29-48)
        const uint64_t gkey0 = derive_key(unit.seed, 0, 0, TAG_GLOBAL);
        for (int k = 0; k < SPT; k++) {
            const uint32_t ls = phase_slot<THREADS>(k, tid);
            const Jsf r = jsf_seed((uint32_t)(ls + unit.seed * SLOTS));
            s_rng[ls] = make_uint4(r.a, r.b, r.c, r.d);
            float4 w;
            sample_point(feistel(ls, SLOTS, gkey0), SLOTS, w.x, w.y);
            w.z = 0.0f;
            w.w = 0.0f;
            s_w[ls] = w;
        }
        // the pass that starts drawing gathers through a keyed Feistel permutation of the whole
        // unit; every other pass after the first through a permutation of the shared table
        const uint64_t gkeyF = derive_key(unit.seed, I.fuse, 0, TAG_GLOBAL);
        __syncthreads();
        const uint32_t foff = s_prog[H_FINAL];
        const float Wf = (float)I.W, Hf = (float)I.H;
        for (uint32_t s = 0; s < passes; s++) {
            const int buf = s & 1;
            const bool draw = s >= I.fuse;
            // pass s + 1's permutation id; pass s's was written before the previous pass's barrier
            if (tid == 0) s_misc[1 + (buf ^ 1)] = (uint32_t)(derive_key(unit.seed, s + 1, 0, TAG_LOCAL) % A.table_size);
            // this pass's sources, loaded before the barrier
            const uint32_t perm = s_misc[1 + buf];
            uint32_t src[SPT];
#pragma unroll
            for (int k = 0; k < SPT; k++) {
                const uint32_t ls = phase_slot<THREADS>(k, tid);
                src[k] = (s == 0) ? ls : (s == I.fuse) ? feistel(ls, SLOTS, gkeyF) : (uint32_t)A.table[(size_t)perm * SLOTS + ls];
            }
            if (dphase >= 0) {  // flame.glsl:51-53
                const uint32_t ls = phase_slot<THREADS>(dphase, tid);
                const uint4 r4 = s_rng[ls];
                Jsf rng{r4.x, r4.y, r4.z, r4.w};
                const int xi = select_xform(s_prog, randf(rng));
                s_rng[ls] = make_uint4(rng.a, rng.b, rng.c, rng.d);
                s_xid[buf * G + ls / kGroup] = xi;
            }
            __syncthreads();
#pragma unroll 1
            for (int k = 0; k < SPT; k++) {
                const uint32_t ls = phase_slot<THREADS>(k, tid);
                uint32_t j = src[0];
#pragma unroll
                for (int q = 1; q < SPT; q++)
                    if (q == k) j = src[q];
                const float4 v = s_w[buf * SLOTS + j];
                float x = v.x, y = v.y, c = v.z;
                const uint4 r4 = s_rng[ls];
                Jsf rng{r4.x, r4.y, r4.z, r4.w};
                const int xi = s_xid[buf * G + ls / kGroup];
                const bool first = s == 0;
                if (first) {  // flame.glsl:64
                    const float u1 = randf(rng);
                    const float u2 = randf(rng);
                    const float amp = __fmul_rn(__fmul_rn(__fmul_rn(u1, 0.1f), kPI), 2.0f);
                    float sn, cs;
                    jitter_sincos(sqrtf(u2), sn, cs);
                    x = __fadd_rn(x, __fmul_rn(amp, sn));
                    y = __fadd_rn(y, __fmul_rn(amp, cs));
                }
                float ex = x, ey = y, ec = c, op = 0.0f;
                bool fr = first;
                const bool with_final = draw && foff != 0;
                for (int it = 0;; it++) {
                    float o;
                    Eval::apply(s_prog, it == 0 ? xi : -1, foff, ex, ey, ec, o, fr, rng);
                    if (it == 0) {
                        if (I.reset) reset_bad_walker(ex, ey, o, rng);  // flame.glsl:68
                        x = ex; y = ey; c = ec; op = o;
                    } else {
                        op = o * op;
                    }
                    if (it == 1 || !with_final) break;
                    fr = false;
                }
                s_w[(buf ^ 1) * SLOTS + ls] = make_float4(x, y, c, 0.0f);
                s_rng[ls] = make_uint4(rng.a, rng.b, rng.c, rng.d);
                if (draw) {
                    if (op > 0.0f) emitted++;
                    const float px = fmaf(I.ss[0], ex, fmaf(I.ss[2], ey, I.ss[4]));
                    const float py = fmaf(I.ss[1], ex, fmaf(I.ss[3], ey, I.ss[5]));
                    uint32_t bin = kNoBin;
                    float4 val = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                    if (px >= 0.0f && py >= 0.0f && px < Wf && py < Hf && op > 0.0f) {
                        const uint32_t bx = (uint32_t)px, by = (uint32_t)py;
                        bin = (I.H - 1 - by) * I.W + bx;
                        const float4 col = s_pal[palette_index(ec)];
                        val = make_float4(col.x, col.y, col.z, op);
                        drawn++;
                    }
                    const BinTarget t{I.bins, I.hits, 0u, 0u};
                    if (I.splat) splat_warp(t, bin, val);
                    else splat_global(t, bin, val);
                }
            }
        }
        steps += (unsigned long long)SLOTS * passes;
        __syncthreads();  // the next unit reuses the shared buffers
    }
    const uint32_t d = __reduce_add_sync(0xffffffffu, drawn);
    const uint32_t e = __reduce_add_sync(0xffffffffu, emitted);
    if ((tid & 31) == 0) {
        atomicAdd(A.counters + 0, (unsigned long long)d);
        atomicAdd(A.counters + 1, (unsigned long long)e);
    }
    if (tid == 0) atomicAdd(A.counters + 2, steps);
}

}  // namespace rfk
