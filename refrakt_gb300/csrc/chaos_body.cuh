// The chaos game of one CTA (the body of chaos_kernel, kernels.cu, and of the genome-specialised
// kernels compiled at run time, specialize.cpp), parameterised by the xform evaluator:
// `Eval::apply(prog, xi, final_offset, x, y, c, op, first_run, rng)` applies regular xform xi,
// or the final xform for xi = -1.  InterpEval interprets the compiled genome program
// (variations.cuh); a specialised evaluator is generated per genome structure.  The kernel calls
// apply from one site for both (a two-iteration loop), so the evaluator is inlined once.
//
// The reference runs one GLSL invocation per walker per pass and ping-pongs every walker
// through memory between passes (shaders/flame.glsl:41-90, src/flame.cpp:228-330).  Here one
// CTA owns a block of walker slots (the mixing domain) for L consecutive passes: the genome is
// staged once in shared memory, the slots' walkers and JSF32 states stay in shared memory, and
// between passes the walkers are permuted among the CTA's slots through a double-buffered
// shared-memory exchange (the walker shuffle).  At each launch boundary every walker is gathered
// from HBM through a keyed permutation of its temporal sample, so walkers also mix across CTAs.
//
// Per slot and pass the order of RNG draws is the reference's: the first slot of each 256-slot
// group draws the group's xform id (flame.glsl:51-53), then the first-pass jitter (:64), the
// variations in codegen order, the first-pass colour (variation_table.cpp:242) and, when
// drawing, the final xform (flame.cpp:23).
#pragma once

#include "chaos_args.h"
#include "splat.cuh"
#include "variations.cuh"

namespace rfk {

struct InterpEval {
    static __device__ __forceinline__ void apply(const uint32_t* prog, int xi, uint32_t final_off, float& x, float& y,
                                                 float& c, float& op, bool first_run, Jsf& rng) {
        eval_xform(prog + (xi >= 0 ? prog[H_XOFF + xi] : final_off), x, y, c, op, first_run, rng);
    }
};

// The slot a thread serves in phase k of a pass: phase k covers slots [k * THREADS, (k + 1) *
// THREADS), and warps are permuted per phase (warp w serves warp w ^ k's 32 slots), so the 256-slot
// groups' first slots fall to SPT * THREADS / 256 different warps, one per warp: the group xform
// draws at the start of a pass run in parallel instead of SPT after another.
template <int THREADS>
__device__ __forceinline__ uint32_t phase_slot(int k, int tid) {
    return (uint32_t)(k * THREADS + (tid ^ (32 * k)));
}
// the phase in which thread tid serves a group's first slot, or -1
template <int THREADS, int SPT>
__device__ __forceinline__ int draw_phase(int tid) {
    const int k = (tid % kGroup) >> 5;
    return ((tid & 31) == 0 && k < SPT) ? k : -1;
}

// Shared memory of a chaos CTA (dynamic, in this order):
//   program words (prog_words), palette float4[256], walker exchange float4 [2][SLOTS],
//   JSF32 states uint4[SLOTS], group xform ids int[2][SLOTS/256], per-pass permutation ids
//   uint32[steps], (8-byte aligned) the pipelined exchange's two mbarriers; with the tile splat
//   (16-byte aligned) the tile's float4 RGBA sums and uint32 counts
__host__ __device__ inline size_t chaos_smem_bytes(int slots, uint32_t prog_words, uint32_t steps,
                                                   uint32_t tile_bins = 0, int pipe = 0) {
    size_t b = ((size_t)prog_words * 4 + 15) & ~(size_t)15;
    b += 256 * 16;
    b += (size_t)2 * slots * 16;
    b += (size_t)slots * 16;
    b += (size_t)2 * (slots / kGroup) * 4;
    b += (size_t)steps * 4;
    if (pipe) b = ((b + 7) & ~(size_t)7) + 16;
    if (tile_bins) b = ((b + 15) & ~(size_t)15) + (size_t)tile_bins * 20;
    return b;
}

// The pipelined walker exchange's two CTA-wide mbarriers: [0] completes when every thread has
// finished the first SPT-1 phases of a pass, [1] when every thread has finished the pass.
__device__ __forceinline__ uint32_t xbar_addr(const uint64_t* b) { return (uint32_t)__cvta_generic_to_shared(b); }
__device__ __forceinline__ void xbar_init(uint64_t* b, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(xbar_addr(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void xbar_arrive(uint64_t* b) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(xbar_addr(b)) : "memory");
}
// waits (bounded) for the completion of the barrier's phase of the given parity: 2^16 tries, each
// suspending the thread for at most 16 us (the suspend-time hint), so about a second at most;
// false when the wait ran out
__device__ __forceinline__ bool xbar_wait(uint64_t* b, uint32_t parity) {
    for (uint32_t i = 0; i < (1u << 16); i++) {
        uint32_t ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
            " selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(xbar_addr(b)), "r"(parity), "r"(16384u)
            : "memory");
        if (ok) return true;
    }
    return false;
}

// One CTA of THREADS threads owns SLOTS = THREADS * SPT walker slots — the walker shuffle's mixing
// domain — for the launch's passes.  Every slot's walker and JSF32 state live in shared memory;
// each thread serves SPT slots per pass (phase_slot(k, tid), in SPT different 256-slot groups, so
// a warp's work per pass averages over SPT xforms).  64 registers per thread:
// 1024 threads x 1, 512 x 2 or 256 x 4 CTAs per SM.
// SPLAT >= 0 fixes the splat strategy at compile time (0 global, 1 warp-aggregated, 2 adaptive),
// so the hot loop carries only that one; -1 dispatches on A.splat.  RESET >= 0 likewise fixes
// the walker reset of flame.glsl:68 (reset_bad_walker); -1 reads A.reset.
//
// PIPE = 1 (SPT >= 3) replaces the pass barrier by the pipelined exchange.  The shuffle table's
// permutations (shuffle_table_pipe_kernel) send the first phase's slots no walker of the previous
// pass's last phase and the last phase's slots no walker of its first phase.  So a warp starts the
// next pass as soon as every warp has finished the first SPT-1 phases of this one (mbarrier 0:
// the first phase's sources are written, and the first phase's slots — which it overwrites — are
// no longer read), and waits for the whole previous pass (mbarrier 1) only before its second
// phase: the slowest warps' last phase overlaps the others' next pass, with the walkers still
// double-buffered.  A group's xform for pass s + 1 is drawn right after its first slot's pass-s
// evaluation (the same point of that slot's RNG stream) into the other xform-id buffer.
template <int THREADS, int SPT, class Eval, int SPLAT = -1, int RESET = -1, int PIPE = 0>
__device__ __forceinline__ void chaos_body(const ChaosArgs& A) {
    static_assert(!PIPE || SPT >= 3, "the pipelined exchange needs three phases");
    constexpr uint32_t SLOTS = (uint32_t)THREADS * SPT;
    constexpr int G = SLOTS / kGroup;
    extern __shared__ __align__(16) unsigned char smem[];
    uint32_t* s_prog = reinterpret_cast<uint32_t*>(smem);
    float4* s_pal = reinterpret_cast<float4*>(smem + (((size_t)A.prog_words * 4 + 15) & ~(size_t)15));
    float4* s_w = s_pal + 256;
    uint4* s_rng = reinterpret_cast<uint4*>(s_w + 2 * SLOTS);
    int* s_xid = reinterpret_cast<int*>(s_rng + SLOTS);
    uint32_t* s_perm = reinterpret_cast<uint32_t*>(s_xid + 2 * G);
    uint64_t* s_bar = reinterpret_cast<uint64_t*>(((unsigned long long)(s_perm + A.steps) + 7) & ~7ull);
    // the tile splat's shared-memory histogram (splat 3)
    const bool tiled = SPLAT == 3 || (SPLAT < 0 && A.splat == 3);
    const uint32_t tile_bins = tiled && A.draw ? A.tile_w * A.tile_h : 0u;
    TileTarget tt{nullptr, nullptr};
    if (tile_bins) {
        tt.rgba = reinterpret_cast<float4*>(
            smem + ((chaos_smem_bytes(SLOTS, A.prog_words, A.steps, 0, PIPE) + 15) & ~(size_t)15));
        tt.count = reinterpret_cast<uint32_t*>(tt.rgba + tile_bins);
    }

    const int tid = threadIdx.x;
    for (uint32_t i = tid; i < tile_bins; i += THREADS) {
        tt.rgba[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        tt.count[i] = 0u;
    }
    const uint32_t chunk = blockIdx.x;  // mixing domain
    const uint32_t ts = chunk / A.chunks_per_ts;
    const uint32_t gid0 = (chunk - ts * A.chunks_per_ts) * SLOTS;  // first slot within the temporal sample
    const size_t ts_base = (size_t)ts * A.ppts;

    if (PIPE && tid == 0) {
        xbar_init(s_bar + 0, THREADS);
        xbar_init(s_bar + 1, THREADS);
    }
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
        const uint32_t ls = phase_slot<THREADS>(k, tid);
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

    const uint32_t foff = s_prog[H_FINAL];
    const bool has_final = A.draw && foff != 0;
    const int dphase = draw_phase<THREADS, SPT>(tid);
    const float W = (float)A.W, H = (float)A.H;
    const bool reset = RESET >= 0 ? RESET != 0 : A.reset != 0;
    uint32_t drawn = 0, emitted = 0;
    // flame.glsl:51-53: the first slot of each 256-slot group draws the group's xform for pass s
    // from its own RNG stream (the pipelined exchange draws inside the pass loop instead)
    auto draw_group_xform = [&](uint32_t s, uint32_t ls, Jsf& rng) {
        const int xi = select_xform(s_prog, randf(rng));
        s_xid[(s & 1) * G + ls / kGroup] = xi;
        if (A.trace && A.pass0 + s < A.trace_passes)
            A.trace[(size_t)(A.pass0 + s) * A.n_groups + (ts_base + gid0 + ls) / kGroup] = (uint8_t)xi;
    };
    if (PIPE && dphase >= 0) {
        const uint32_t ls = phase_slot<THREADS>(dphase, tid);
        const uint4 r4 = s_rng[ls];
        Jsf rng{r4.x, r4.y, r4.z, r4.w};
        draw_group_xform(0, ls, rng);
        s_rng[ls] = make_uint4(rng.a, rng.b, rng.c, rng.d);
    }
    __syncthreads();
    // PIPE: false after a wait ran out — the thread counts it (the host reports RF_ERR_TIMEOUT)
    // and waits no more, so the launch still ends
    bool synced = true;

    for (uint32_t s = 0; s < A.steps; s++) {
        const int buf = s & 1;
        // this pass's sources in the exchange buffer (identity on the gather pass)
        uint32_t src[SPT];
#pragma unroll
        for (int k = 0; k < SPT; k++)
            src[k] = (s == 0) ? phase_slot<THREADS>(k, tid) : (uint32_t)A.table[(size_t)s_perm[s] * SLOTS + phase_slot<THREADS>(k, tid)];
        if (!PIPE) {
            if (dphase >= 0) {
                const uint32_t ls = phase_slot<THREADS>(dphase, tid);
                const uint4 r4 = s_rng[ls];
                Jsf rng{r4.x, r4.y, r4.z, r4.w};
                draw_group_xform(s, ls, rng);
                s_rng[ls] = make_uint4(rng.a, rng.b, rng.c, rng.d);
            }
            __syncthreads();
        }
#pragma unroll 1
        for (int k = 0; k < SPT; k++) {
            const uint32_t ls = phase_slot<THREADS>(k, tid);
            uint32_t j = src[0];
#pragma unroll
            for (int q = 1; q < SPT; q++)
                if (q == k) j = src[q];
            // PIPE: the first phase reads walkers of the previous pass's first SPT-1 phases, the
            // others any of its walkers
            if (PIPE && synced && s > 0 && k < 2 && !xbar_wait(s_bar + k, (s - 1) & 1)) {
                synced = false;
                atomicAdd(A.counters + 3, 1ull);
            }
            const float4 v = s_w[buf * SLOTS + j];
            float x = v.x, y = v.y, c = v.z;
            const uint4 r4 = s_rng[ls];
            Jsf rng{r4.x, r4.y, r4.z, r4.w};
            const int xi = s_xid[buf * G + ls / kGroup];
            const bool first = A.first_run && s == 0;
            if (first) {  // flame.glsl:64: xy += randf() * .1 * PI * 2.0 * sincos(sqrt(randf()))
                const float u1 = randf(rng);
                const float u2 = randf(rng);
                const float amp = __fmul_rn(__fmul_rn(__fmul_rn(u1, 0.1f), kPI), 2.0f);
                float sn, cs;
                jitter_sincos(sqrtf(u2), sn, cs);
                x = __fadd_rn(x, __fmul_rn(amp, sn));
                y = __fadd_rn(y, __fmul_rn(amp, cs));
            }
            // the xform, then (when drawing) the final xform on a copy — one evaluator call site
            float ex = x, ey = y, ec = c, op = 0.0f;
            bool fr = first;
            for (int it = 0;; it++) {
                float o;
                Eval::apply(s_prog, it == 0 ? xi : -1, foff, ex, ey, ec, o, fr, rng);
                if (it == 0) {
                    if (reset) reset_bad_walker(ex, ey, o, rng);  // flame.glsl:68, before pos_out
                    x = ex; y = ey; c = ec; op = o;
                } else {
                    op = o * op;
                }
                if (it == 1 || !has_final) break;
                fr = false;
            }
            s_w[(buf ^ 1) * SLOTS + ls] = make_float4(x, y, c, 0.0f);
            // the group's xform for the next pass, at the point of the slot's stream where the
            // pass-barrier form draws it
            if (PIPE && k == dphase && s + 1 < A.steps) draw_group_xform(s + 1, ls, rng);
            s_rng[ls] = make_uint4(rng.a, rng.b, rng.c, rng.d);
            if (PIPE && k >= SPT - 2) xbar_arrive(s_bar + (k - (SPT - 2)));
            if (A.draw) {
                if (op > 0.0f) emitted++;
                const float px = fmaf(A.ss[0], ex, fmaf(A.ss[2], ey, A.ss[4]));
                const float py = fmaf(A.ss[1], ex, fmaf(A.ss[3], ey, A.ss[5]));
                uint32_t bin = kNoBin, local = kNoBin;
                float4 val = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                if (px >= 0.0f && py >= 0.0f && px < W && py < H && op > 0.0f) {
                    const uint32_t bx = (uint32_t)px, by = (uint32_t)py;
                    const uint32_t row = A.H - 1 - by;  // flame.glsl:84 row flip; W*H < 2^32 - 1
                    bin = row * A.W + bx;
                    if (tile_bins && bx - A.tile_x0 < A.tile_w && row - A.tile_y0 < A.tile_h)
                        local = (row - A.tile_y0) * A.tile_w + (bx - A.tile_x0);
                    const float4 col = s_pal[palette_index(ec)];
                    val = make_float4(col.x, col.y, col.z, op);
                    drawn++;
                }
                const BinTarget t{A.bins, A.hits, A.rgba_shift, A.count_shift};
                if constexpr (SPLAT == 0) {
                    splat_global(t, bin, val);
                } else if constexpr (SPLAT == 1) {
                    splat_warp(t, bin, val);
                } else if constexpr (SPLAT == 2) {
                    splat_adaptive(t, bin, val);
                } else if constexpr (SPLAT == 3) {
                    splat_tile(t, tt, bin, local, val);
                } else {
                    if (A.splat == 1) splat_warp(t, bin, val);
                    else if (A.splat == 2) splat_adaptive(t, bin, val);
                    else if (A.splat == 3) splat_tile(t, tt, bin, local, val);
                    else splat_global(t, bin, val);
                }
            }
        }
    }
    // the tile's non-empty bins into the histogram, once per launch
    if (tile_bins) {
        __syncthreads();
        const BinTarget t{A.bins, A.hits, A.rgba_shift, A.count_shift};
        for (uint32_t i = tid; i < tile_bins; i += THREADS) {
            const uint32_t n = tt.count[i];
            if (!n) continue;
            const uint32_t row = A.tile_y0 + i / A.tile_w, col = A.tile_x0 + i % A.tile_w;
            const float4 v = tt.rgba[i];
            red_add_f32x4(t.at_rgba(row * A.W + col), v.x, v.y, v.z, v.w);
            if (t.count) red_add_u32x1(t.at_count(row * A.W + col), n);
        }
    }
    // each slot's final walker and state were written by the thread that owns the slot
    const int out_buf = A.steps & 1;
    for (int k = 0; k < SPT; k++) {
        const uint32_t ls = phase_slot<THREADS>(k, tid);
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
