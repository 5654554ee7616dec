// Chaos-game kernels for sm_103a: the interpreted chaos kernel (its body, the walker shuffle
// and the reference's RNG draw order are in chaos_body.cuh), RNG seeding, the walker-shuffle
// table, temporal-sample animation and the single-step probe.
#include <cuda_runtime.h>

#include "chaos_body.cuh"
#include "kernels.h"

namespace rfk {

template <int THREADS, int SPT>
__global__ void __launch_bounds__(THREADS, 1024 / THREADS) chaos_kernel(const ChaosArgs A) {
    chaos_body<THREADS, SPT, InterpEval>(A);
}

// Interleaved bin records (32 bytes: float4 RGBA, uint32 count, pad) added into the caller's
// planes, then cleared for the next call.
__global__ void merge_records_kernel(float4* __restrict__ rec, size_t n, float4* __restrict__ bins,
                                     uint32_t* __restrict__ hits) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float4 v = rec[2 * i];
        const uint32_t c = reinterpret_cast<const uint32_t*>(rec + 2 * i + 1)[0];
        if (v.x != 0.0f || v.y != 0.0f || v.z != 0.0f || v.w != 0.0f) {
            float4 b = bins[i];
            b.x += v.x; b.y += v.y; b.z += v.z; b.w += v.w;
            bins[i] = b;
            rec[2 * i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
        if (c) {
            if (hits) hits[i] += c;
            rec[2 * i + 1] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
    }
}

cudaError_t launch_merge_records(float4* rec, size_t n, float4* bins, uint32_t* hits, cudaStream_t st) {
    merge_records_kernel<<<152 * 16, 256, 0, st>>>(rec, n, bins, hits);
    return cudaGetLastError();
}

// src/flame.cpp:138-141 — slot i seeded with warmup_ctx(i + seed * N)
__global__ void init_rng_kernel(uint4* rng, uint64_t n, uint64_t seed) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Jsf s = jsf_seed((uint32_t)(i + seed * n));
    rng[i] = make_uint4(s.a, s.b, s.c, s.d);
}

// the walker-shuffle table: `count` keyed permutations of [0, n), one entry per thread
__global__ void shuffle_table_kernel(uint16_t* out, uint32_t n, uint32_t count, uint64_t seed) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (uint64_t)n * count) return;
    const uint32_t k = (uint32_t)(i / n), j = (uint32_t)(i - (uint64_t)k * n);
    out[i] = (uint16_t)feistel(j, n, derive_key(seed, k, 0, TAG_TABLE));
}

// The pipelined exchange's table (chaos_body.cuh, PIPE): with P = n/S slots per phase, the last
// phase's destinations [n-P, n) take the first P of a keyed order of [P, n) — never a walker of
// the previous pass's first phase, whose slots a fast thread may already overwrite — and the first
// phase's destinations [0, P) the first P not yet taken of a keyed order of [0, n-P) — never a
// walker of the previous pass's last phase, which a slow thread may still be computing; the middle
// destinations take the rest in a keyed order of [0, n).  One warp per permutation: the lanes walk
// each keyed order 32 entries at a time and a ballot ranks the free ones, so the result is the
// sequential scan's.  The taken-slot bitmap is in shared memory (n / 32 words per warp).
// n <= kMaxPipeSlots, S >= 3 (then enough sources stay free for the first phase).
constexpr uint32_t kMaxPipeSlots = 4096;
constexpr int kPipeTableWarps = 8;  // permutations per CTA
__global__ void __launch_bounds__(32 * kPipeTableWarps)
    shuffle_table_pipe_kernel(uint16_t* out, uint32_t n, uint32_t count, uint64_t seed, uint32_t phases) {
    __shared__ uint32_t s_taken[kPipeTableWarps][kMaxPipeSlots / 32];
    const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const uint32_t k = blockIdx.x * kPipeTableWarps + w;
    if (k >= count) return;  // whole warps leave together
    uint32_t* taken = s_taken[w];
    for (uint32_t i = lane; i < n / 32; i += 32) taken[i] = 0;
    __syncwarp();
    const uint32_t P = n / phases;
    uint16_t* o = out + (size_t)k * n;
    const uint64_t k3 = derive_key(seed, k, 3, TAG_TABLE), k1 = derive_key(seed, k, 1, TAG_TABLE),
                   k2 = derive_key(seed, k, 2, TAG_TABLE);
    for (uint32_t d = lane; d < P; d += 32) {
        const uint32_t src = P + feistel(d, n - P, k3);
        o[n - P + d] = (uint16_t)src;
        atomicOr(&taken[src >> 5], 1u << (src & 31));
    }
    __syncwarp();
    // the untaken entries of a keyed order of [0, len), in order, to destinations [d0, d1)
    auto scan = [&](uint32_t len, uint64_t key, uint32_t d0, uint32_t d1) {
        uint32_t d = d0;
        for (uint32_t base = 0; base < len && d < d1; base += 32) {
            const uint32_t i = base + lane;
            const uint32_t src = i < len ? feistel(i, len, key) : 0u;
            const bool free = i < len && !((taken[src >> 5] >> (src & 31)) & 1u);
            const uint32_t ballot = __ballot_sync(0xffffffffu, free);
            const uint32_t rank = __popc(ballot & ((1u << lane) - 1u));
            if (free && d + rank < d1) {
                o[d + rank] = (uint16_t)src;
                atomicOr(&taken[src >> 5], 1u << (src & 31));
            }
            d = min(d + (uint32_t)__popc(ballot), d1);
            __syncwarp();
        }
    };
    scan(n - P, k1, 0, P);
    scan(n, k2, P, n - P);
}

// animate.tpl.glsl:18-96 — one program copy per temporal sample, each xform's linear part
// rotated by 0.31415926535 * dt * rotation_frequency, dt = (t - T/2) / (T/2) * tss_width.
__global__ void animate_kernel(const uint32_t* base, uint32_t words, uint32_t T, float tss_width,
                               uint32_t* out, uint32_t stride) {
    const uint32_t t = blockIdx.x;
    uint32_t* dst = out + (size_t)t * stride;
    for (uint32_t i = threadIdx.x; i < words; i += blockDim.x) dst[i] = base[i];
    __syncthreads();
    if (T < 2 || threadIdx.x != 0) return;  // T = 1: the template divides 0 by 0; no rotation
    const int half = (int)(T / 2);
    const float dt = (float)((int)t - half) / (float)half * tss_width;
    const uint32_t nx = base[H_NX];
    for (uint32_t k = 0; k <= nx; k++) {
        const uint32_t off = (k < nx) ? base[H_XOFF + k] : base[H_FINAL];
        if (off == 0) continue;
        float* a = reinterpret_cast<float*>(dst + off + X_AFF);
        const float ang = 0.31415926535f * dt * __uint_as_float(base[off + X_ROTF]);
        float sn, cs;
        sincosf(ang, &sn, &cs);
        const float a0 = a[0], a1 = a[1], a2 = a[2], a3 = a[3];
        a[0] = a0 * cs + a2 * sn;
        a[1] = a1 * cs + a3 * sn;
        a[2] = a2 * cs - a0 * sn;
        a[3] = a3 * cs - a1 * sn;
    }
}

// single dispatch() per point, for parity tests
__global__ void probe_kernel(const uint32_t* prog, int xform, uint32_t n, const float* in, uint32_t* rng,
                             int first_run, float* out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t off = (xform < 0) ? prog[H_FINAL] : prog[H_XOFF + xform];
    Jsf s{rng[4 * i], rng[4 * i + 1], rng[4 * i + 2], rng[4 * i + 3]};
    float x = in[3 * i], y = in[3 * i + 1], c = in[3 * i + 2], op;
    eval_xform(prog + off, x, y, c, op, first_run != 0, s);
    out[4 * i] = x; out[4 * i + 1] = y; out[4 * i + 2] = c; out[4 * i + 3] = op;
    rng[4 * i] = s.a; rng[4 * i + 1] = s.b; rng[4 * i + 2] = s.c; rng[4 * i + 3] = s.d;
}

// ---------------------------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------------------------
size_t chaos_smem(int slots, uint32_t prog_words, uint32_t steps, uint32_t tile_bins, int pipe) {
    return chaos_smem_bytes(slots, prog_words, steps, tile_bins, pipe);
}

template <int THREADS, int SPT>
static cudaError_t launch_chaos_t(const ChaosArgs& a, uint32_t grid, cudaStream_t st) {
    const size_t smem = chaos_smem_bytes(THREADS * SPT, a.prog_words, a.steps,
                                         a.splat == 3 && a.draw ? a.tile_w * a.tile_h : 0u);
    auto kern = chaos_kernel<THREADS, SPT>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<grid, THREADS, smem, st>>>(a);
    return cudaGetLastError();
}

bool chaos_shape_supported(int threads, int slots) {
    switch (threads * 8 + slots / threads) {
    case 256 * 8 + 1: case 512 * 8 + 1: case 512 * 8 + 2: case 512 * 8 + 4:
    case 1024 * 8 + 1: case 1024 * 8 + 2: case 1024 * 8 + 4: return slots % threads == 0;
    default: return false;
    }
}

cudaError_t launch_chaos(int threads, int slots, const ChaosArgs& a, uint32_t grid, cudaStream_t st) {
    if (!chaos_shape_supported(threads, slots)) return cudaErrorInvalidValue;
    switch (threads * 8 + slots / threads) {
    case 256 * 8 + 1: return launch_chaos_t<256, 1>(a, grid, st);
    case 512 * 8 + 1: return launch_chaos_t<512, 1>(a, grid, st);
    case 512 * 8 + 2: return launch_chaos_t<512, 2>(a, grid, st);
    case 512 * 8 + 4: return launch_chaos_t<512, 4>(a, grid, st);
    case 1024 * 8 + 1: return launch_chaos_t<1024, 1>(a, grid, st);
    case 1024 * 8 + 2: return launch_chaos_t<1024, 2>(a, grid, st);
    case 1024 * 8 + 4: return launch_chaos_t<1024, 4>(a, grid, st);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_init_rng(uint4* rng, uint64_t n, uint64_t seed, cudaStream_t st) {
    const uint32_t b = 256;
    init_rng_kernel<<<(unsigned)((n + b - 1) / b), b, 0, st>>>(rng, n, seed);
    return cudaGetLastError();
}

cudaError_t launch_shuffle_table(uint16_t* out, uint32_t n, uint32_t count, uint64_t seed, cudaStream_t st,
                                 uint32_t phases) {
    const uint64_t total = (uint64_t)n * count;
    const uint32_t b = 256;
    if (phases >= 3) {
        if (n > kMaxPipeSlots || n % phases) return cudaErrorInvalidValue;
        shuffle_table_pipe_kernel<<<(count + kPipeTableWarps - 1) / kPipeTableWarps, 32 * kPipeTableWarps, 0, st>>>(
            out, n, count, seed, phases);
        return cudaGetLastError();
    }
    shuffle_table_kernel<<<(unsigned)((total + b - 1) / b), b, 0, st>>>(out, n, count, seed);
    return cudaGetLastError();
}

cudaError_t launch_animate(const uint32_t* base, uint32_t words, uint32_t T, float tss, uint32_t* out,
                           uint32_t stride, cudaStream_t st) {
    animate_kernel<<<T, 128, 0, st>>>(base, words, T, tss, out, stride);
    return cudaGetLastError();
}

cudaError_t launch_probe(const uint32_t* prog, int xform, uint32_t n, const float* in, uint32_t* rng, int first_run,
                         float* out, cudaStream_t st) {
    const uint32_t b = 128;
    probe_kernel<<<(n + b - 1) / b, b, 0, st>>>(prog, xform, n, in, rng, first_run, out);
    return cudaGetLastError();
}

}  // namespace rfk
