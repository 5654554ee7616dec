// The chaos game of one CTA with WIDE slots evaluated together (genome-specialised kernels
// only, specialize.cpp): each thread's slots come in runs of WIDE consecutive slots of one
// 256-slot group, so they share the group's xform and the generated evaluator applies it to all
// WIDE walkers in one straight-line body — independent dependency chains the scheduler can
// interleave.  Slots, their RNG streams, the walker shuffle and the RNG draw order are those of
// chaos_body.cuh; only which thread serves which slot, and the order of the histogram
// reductions, differ.
#pragma once

#include "chaos_body.cuh"

namespace rfk {

template <int THREADS, int SPT, int WIDE, class Eval>
__device__ __forceinline__ void chaos_body_wide(const ChaosArgs& A) {
    constexpr uint32_t SLOTS = (uint32_t)THREADS * SPT;
    constexpr int NB = SPT / WIDE;                 // batches of WIDE slots per thread and pass
    constexpr uint32_t BATCH = THREADS * WIDE;     // slots per batch
    static_assert(SPT % WIDE == 0 && (THREADS * WIDE) % kGroup == 0 && kGroup % (32 * WIDE) == 0,
                  "a warp's WIDE-slot runs must stay inside one 256-slot group");
    constexpr int G = SLOTS / kGroup;
    extern __shared__ __align__(16) unsigned char smem[];
    uint32_t* s_prog = reinterpret_cast<uint32_t*>(smem);
    float4* s_pal = reinterpret_cast<float4*>(smem + (((size_t)A.prog_words * 4 + 15) & ~(size_t)15));
    float4* s_w = s_pal + 256;
    uint4* s_rng = reinterpret_cast<uint4*>(s_w + 2 * SLOTS);
    int* s_xid = reinterpret_cast<int*>(s_rng + SLOTS);
    uint32_t* s_perm = reinterpret_cast<uint32_t*>(s_xid + 2 * G);

    const int tid = threadIdx.x;
    const uint32_t chunk = blockIdx.x;  // mixing domain
    const uint32_t ts = chunk / A.chunks_per_ts;
    const uint32_t gid0 = (chunk - ts * A.chunks_per_ts) * SLOTS;  // first slot within the temporal sample
    const size_t ts_base = (size_t)ts * A.ppts;

    const uint32_t* prog = A.progs + (size_t)ts * A.prog_stride;
    for (uint32_t i = tid; i < A.prog_words; i += THREADS) s_prog[i] = prog[i];
    if (A.draw)
        for (int i = tid; i < 256; i += THREADS) s_pal[i] = A.palette[i];
    for (uint32_t s = tid; s < A.steps; s += THREADS)
        s_perm[s] = (uint32_t)(derive_key(A.seed, (uint64_t)A.pass0 + s, chunk, TAG_LOCAL) % A.table_size);

    // JSF32 states, and every walker gathered through a keyed permutation of its temporal
    // sample (pass 0 of a warmup reads the start points instead, flame.glsl:58-61)
    const uint64_t gkey = derive_key(A.seed, A.pass0, ts, TAG_GLOBAL);
    for (int k = 0; k < SPT; k++) {
        const uint32_t ls = (k / WIDE) * BATCH + tid * WIDE + (k % WIDE);
        s_rng[ls] = A.rng[ts_base + gid0 + ls];
        const uint32_t src = feistel(gid0 + ls, A.ppts, gkey);
        float4 w;
        if (A.first_run) {
            sample_point(src, A.ppts, w.x, w.y);
            w.z = 0.0f;
            w.w = 0.0f;
        } else {
            w = A.walk_in[ts_base + src];
        }
        s_w[ls] = w;
    }
    __syncthreads();

    const uint32_t foff = s_prog[H_FINAL];
    const bool has_final = A.draw && foff != 0;
    const bool lane0 = ((tid * WIDE) % kGroup) == 0;  // holds the first slot of a group in each batch
    const float W = (float)A.W, H = (float)A.H;
    uint32_t drawn = 0, emitted = 0;

    for (uint32_t s = 0; s < A.steps; s++) {
        const int buf = s & 1;
        if (lane0) {  // flame.glsl:51-53: the group's first slot draws the group's xform
#pragma unroll 1
            for (int b = 0; b < NB; b++) {
                const uint32_t ls = b * BATCH + tid * WIDE;
                const uint4 r4 = s_rng[ls];
                Jsf rng{r4.x, r4.y, r4.z, r4.w};
                const int xi = select_xform(s_prog, randf(rng));
                s_rng[ls] = make_uint4(rng.a, rng.b, rng.c, rng.d);
                s_xid[buf * G + ls / kGroup] = xi;
                if (A.trace && A.pass0 + s < A.trace_passes)
                    A.trace[(size_t)(A.pass0 + s) * A.n_groups + (ts_base + gid0 + ls) / kGroup] = (uint8_t)xi;
            }
        }
        __syncthreads();
        const bool first = A.first_run && s == 0;
#pragma unroll 1
        for (int b = 0; b < NB; b++) {
            const uint32_t ls0 = b * BATCH + tid * WIDE;
            const int xi = s_xid[buf * G + ls0 / kGroup];  // one group for the WIDE slots
            float x[WIDE], y[WIDE], c[WIDE], op[WIDE];
            Jsf rng[WIDE];
#pragma unroll
            for (int q = 0; q < WIDE; q++) {
                const uint32_t ls = ls0 + q;
                const uint32_t j = (s == 0) ? ls : (uint32_t)A.table[(size_t)s_perm[s] * SLOTS + ls];
                const float4 v = s_w[buf * SLOTS + j];
                x[q] = v.x; y[q] = v.y; c[q] = v.z;
                const uint4 r4 = s_rng[ls];
                rng[q] = Jsf{r4.x, r4.y, r4.z, r4.w};
                if (first) {  // flame.glsl:64: xy += randf() * .1 * PI * 2.0 * sincos(sqrt(randf()))
                    const float u1 = randf(rng[q]);
                    const float u2 = randf(rng[q]);
                    const float amp = __fmul_rn(__fmul_rn(__fmul_rn(u1, 0.1f), kPI), 2.0f);
                    float sn, cs;
                    jitter_sincos(sqrtf(u2), sn, cs);
                    x[q] = __fadd_rn(x[q], __fmul_rn(amp, sn));
                    y[q] = __fadd_rn(y[q], __fmul_rn(amp, cs));
                }
            }
            // the xform on all WIDE slots at once, then (when drawing) the final xform on copies
            Eval::apply_wide(s_prog, xi, x, y, c, op, first, rng);
            float ex[WIDE], ey[WIDE], ec[WIDE], fo[WIDE];
#pragma unroll
            for (int q = 0; q < WIDE; q++) {
                ex[q] = x[q]; ey[q] = y[q]; ec[q] = c[q]; fo[q] = 1.0f;
                s_w[(buf ^ 1) * SLOTS + ls0 + q] = make_float4(x[q], y[q], c[q], 0.0f);
            }
            if (has_final) Eval::apply_wide(s_prog, -1, ex, ey, ec, fo, false, rng);
#pragma unroll
            for (int q = 0; q < WIDE; q++) {
                s_rng[ls0 + q] = make_uint4(rng[q].a, rng[q].b, rng[q].c, rng[q].d);
                if (!A.draw) continue;
                const float o = has_final ? fo[q] * op[q] : op[q];
                if (o > 0.0f) emitted++;
                const float px = fmaf(A.ss[0], ex[q], fmaf(A.ss[2], ey[q], A.ss[4]));
                const float py = fmaf(A.ss[1], ex[q], fmaf(A.ss[3], ey[q], A.ss[5]));
                uint32_t bin = kNoBin;
                float4 val = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                if (px >= 0.0f && py >= 0.0f && px < W && py < H && o > 0.0f) {
                    const uint32_t bx = (uint32_t)px, by = (uint32_t)py;
                    bin = (A.H - 1 - by) * A.W + bx;  // flame.glsl:84 row flip; W*H < 2^32 - 1
                    const float4 col = s_pal[palette_index(ec[q])];
                    val = make_float4(col.x, col.y, col.z, o);
                    drawn++;
                }
                const BinTarget t{A.bins, A.hits, A.rgba_shift, A.count_shift};
                if (A.splat == 1) splat_warp(t, bin, val);
                else if (A.splat == 2) splat_adaptive(t, bin, val);
                else splat_global(t, bin, val);
            }
        }
    }
    // each slot's final walker and state were written by the thread that owns the slot
    const int out_buf = A.steps & 1;
    for (int k = 0; k < SPT; k++) {
        const uint32_t ls = (k / WIDE) * BATCH + tid * WIDE + (k % WIDE);
        A.walk_out[ts_base + gid0 + ls] = s_w[out_buf * SLOTS + ls];
        A.rng[ts_base + gid0 + ls] = s_rng[ls];
    }

    if (A.draw) {
        const uint32_t d = __reduce_add_sync(0xffffffffu, drawn);
        const uint32_t e = __reduce_add_sync(0xffffffffu, emitted);
        if ((tid & 31) == 0) {
            atomicAdd(A.counters + 0, (unsigned long long)d);
            atomicAdd(A.counters + 1, (unsigned long long)e);
        }
    }
    if (tid == 0) atomicAdd(A.counters + 2, (unsigned long long)SLOTS * A.steps);
}

}  // namespace rfk
