// Chaos-game kernels for sm_103a.
//
// The reference runs one GLSL invocation per walker per pass and ping-pongs every walker
// through memory between passes (shaders/flame.glsl:41-90, src/flame.cpp:228-330).  Here one
// CTA owns `CTA` walker slots for L consecutive passes: the walkers and their JSF32 states stay
// in registers, the genome is staged once in shared memory, and between passes the walkers are
// permuted among the CTA's slots through shared memory (the walker shuffle).  At each launch
// boundary every walker is gathered from HBM through a keyed permutation of its temporal
// sample, so walkers also mix across CTAs.
//
// Per slot and pass the order of RNG draws is the reference's: lane 0 of each 256-slot group
// draws the group's xform id (flame.glsl:51-53), then the first-pass jitter (:64), the
// variations in codegen order, the first-pass colour (variation_table.cpp:242) and, when
// drawing, the final xform (flame.cpp:23).
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include "kernels.h"
#include "variations.cuh"

namespace cg = cooperative_groups;

namespace rfk {

__device__ __forceinline__ void red_add_v4(float4* p, float a, float b, float c, float d) {
    asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(p), "f"(a), "f"(b), "f"(c), "f"(d)
                 : "memory");
}
__device__ __forceinline__ void red_add_u32(uint32_t* p, uint32_t v) {
    asm volatile("red.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Shared memory of a chaos CTA (dynamic, in this order):
//   program words (prog_words), palette float4[256], walker exchange float4 [2][CTA],
//   group xform ids int[2][CTA/256], per-pass permutation ids uint32[steps]
__host__ __device__ inline size_t chaos_smem_bytes(int cta, uint32_t prog_words, uint32_t steps) {
    size_t b = ((size_t)prog_words * 4 + 15) & ~(size_t)15;
    b += 256 * 16;
    b += (size_t)2 * cta * 16;
    b += (size_t)2 * (cta / kGroup) * 4;
    b += (size_t)steps * 4;
    return b;
}

// The walker shuffle spans a mixing domain of CTA * CLUSTER slots.  With CLUSTER > 1 the CTAs
// of a thread-block cluster read each other's exchange buffers through distributed shared
// memory and synchronise with one cluster barrier per pass.  64 registers per thread at every
// CTA size: 1024 x 1, 512 x 2 or 256 x 4 CTAs per SM.
template <int CTA, int CLUSTER>
__global__ void __launch_bounds__(CTA, 1024 / CTA) chaos_kernel(const ChaosArgs A) {
    constexpr int G = CTA / kGroup;
    constexpr uint32_t DOMAIN = (uint32_t)CTA * CLUSTER;
    extern __shared__ __align__(16) unsigned char smem[];
    uint32_t* s_prog = reinterpret_cast<uint32_t*>(smem);
    float4* s_pal = reinterpret_cast<float4*>(smem + (((size_t)A.prog_words * 4 + 15) & ~(size_t)15));
    float4* s_w = s_pal + 256;
    int* s_xid = reinterpret_cast<int*>(s_w + 2 * CTA);
    uint32_t* s_perm = reinterpret_cast<uint32_t*>(s_xid + 2 * G);

    const int tid = threadIdx.x;
    const uint32_t crank = (CLUSTER > 1) ? cg::this_cluster().block_rank() : 0u;
    const uint32_t chunk = blockIdx.x / CLUSTER;  // mixing domain
    const uint32_t ts = chunk / A.chunks_per_ts;
    const uint32_t lslot = crank * CTA + tid;     // slot within the domain
    const uint32_t gid = (chunk - ts * A.chunks_per_ts) * DOMAIN + lslot;  // slot within its temporal sample
    const size_t slot = (size_t)ts * A.ppts + gid;

    const uint32_t* prog = A.progs + (size_t)ts * A.prog_stride;
    for (uint32_t i = tid; i < A.prog_words; i += CTA) s_prog[i] = prog[i];
    if (A.draw)
        for (int i = tid; i < 256; i += CTA) s_pal[i] = A.palette[i];
    for (uint32_t s = tid; s < A.steps; s += CTA)
        s_perm[s] = (uint32_t)(derive_key(A.seed, (uint64_t)A.pass0 + s, chunk, TAG_LOCAL) % A.table_size);

    const uint4 r4 = A.rng[slot];
    Jsf rng{r4.x, r4.y, r4.z, r4.w};

    // launch-boundary gather through a keyed permutation of the temporal sample
    const uint32_t src = feistel(gid, A.ppts, derive_key(A.seed, A.pass0, ts, TAG_GLOBAL));
    float x, y, c;
    if (A.first_run) {
        sample_point(src, A.ppts, x, y);  // flame.glsl:58-61 reads the start points
        c = 0.0f;
    } else {
        const float4 w = A.walk_in[(size_t)ts * A.ppts + src];
        x = w.x; y = w.y; c = w.z;
    }
    if (CLUSTER > 1) cg::this_cluster().sync(); else __syncthreads();

    const uint32_t foff = s_prog[H_FINAL];
    const bool has_final = A.draw && foff != 0;
    const int grp = tid / kGroup;
    const bool lane0 = (tid % kGroup) == 0;
    const size_t group_global = slot / kGroup;
    const float W = (float)A.W, H = (float)A.H;
    uint32_t drawn = 0, emitted = 0;
    uint32_t perm_next = 0;
    if (A.steps > 1) perm_next = A.table[(size_t)s_perm[1] * DOMAIN + lslot];

    for (uint32_t s = 0; s < A.steps; s++) {
        const int buf = s & 1;
        if (lane0) {
            const int xi = select_xform(s_prog, randf(rng));
            s_xid[buf * G + grp] = xi;
            if (A.trace && A.pass0 + s < A.trace_passes)
                A.trace[(size_t)(A.pass0 + s) * A.n_groups + group_global] = (uint8_t)xi;
        }
        if (s > 0) s_w[buf * CTA + tid] = make_float4(x, y, c, 0.0f);
        if (CLUSTER > 1) cg::this_cluster().sync(); else __syncthreads();
        if (s > 0) {
            const uint32_t j = perm_next;  // source slot in the domain
            float4 v;
            if (CLUSTER > 1) {
                const float4* src = cg::this_cluster().map_shared_rank(s_w + buf * CTA + (j % CTA), j / CTA);
                v = *src;
            } else {
                v = s_w[buf * CTA + j];
            }
            x = v.x; y = v.y; c = v.z;
            if (s + 1 < A.steps) perm_next = A.table[(size_t)s_perm[s + 1] * DOMAIN + lslot];
        }
        const int xi = s_xid[buf * G + grp];
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
        // the xform, then (when drawing) the final xform on a copy — one inlined evaluator
        const uint32_t* blk = s_prog + s_prog[H_XOFF + xi];
        float ex = x, ey = y, ec = c, op = 0.0f;
        bool fr = first;
        for (int it = 0;; it++) {
            float o;
            eval_xform(blk, ex, ey, ec, o, fr, rng);
            if (it == 0) { x = ex; y = ey; c = ec; op = o; }
            else op = o * op;
            if (it == 1 || !has_final) break;
            blk = s_prog + foff;
            fr = false;
        }
        if (A.draw) {
            if (op > 0.0f) emitted++;
            const float px = fmaf(A.ss[0], ex, fmaf(A.ss[2], ey, A.ss[4]));
            const float py = fmaf(A.ss[1], ex, fmaf(A.ss[3], ey, A.ss[5]));
            if (px >= 0.0f && py >= 0.0f && px < W && py < H && op > 0.0f) {
                const uint32_t bx = (uint32_t)px, by = (uint32_t)py;
                const size_t idx = (size_t)(A.H - 1 - by) * A.W + bx;  // flame.glsl:84 row flip
                const float4 col = s_pal[palette_index(ec)];
                red_add_v4(A.bins + idx, col.x, col.y, col.z, op);
                if (A.hits) red_add_u32(A.hits + idx, 1u);
                drawn++;
            }
        }
    }
    A.walk_out[slot] = make_float4(x, y, c, 0.0f);
    A.rng[slot] = make_uint4(rng.a, rng.b, rng.c, rng.d);
    // no CTA leaves while a peer may still read its exchange buffer
    if (CLUSTER > 1) cg::this_cluster().sync();

    if (A.draw) {
        const uint32_t d = __reduce_add_sync(0xffffffffu, drawn);
        const uint32_t e = __reduce_add_sync(0xffffffffu, emitted);
        if ((tid & 31) == 0) {
            atomicAdd(A.counters + 0, (unsigned long long)d);
            atomicAdd(A.counters + 1, (unsigned long long)e);
        }
    }
    if (tid == 0) atomicAdd(A.counters + 2, (unsigned long long)CTA * A.steps);
}

// src/flame.cpp:138-141 — slot i seeded with warmup_ctx(i + seed * N)
__global__ void init_rng_kernel(uint4* rng, uint64_t n, uint64_t seed) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Jsf s = jsf_seed((uint32_t)(i + seed * n));
    rng[i] = make_uint4(s.a, s.b, s.c, s.d);
}

// the walker-shuffle table: `count` keyed permutations of [0, n)
__global__ void shuffle_table_kernel(uint16_t* out, uint32_t n, uint32_t count, uint64_t seed) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (uint64_t)n * count) return;
    const uint32_t k = (uint32_t)(i / n), j = (uint32_t)(i - (uint64_t)k * n);
    out[i] = (uint16_t)feistel(j, n, derive_key(seed, k, 0, TAG_TABLE));
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
size_t chaos_smem(int cta, uint32_t prog_words, uint32_t steps) { return chaos_smem_bytes(cta, prog_words, steps); }

template <int CTA, int CLUSTER>
static cudaError_t launch_chaos_t(const ChaosArgs& a, uint32_t grid, cudaStream_t st) {
    const size_t smem = chaos_smem_bytes(CTA, a.prog_words, a.steps);
    auto kern = chaos_kernel<CTA, CLUSTER>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    if (CLUSTER == 1) {
        kern<<<grid, CTA, smem, st>>>(a);
        return cudaGetLastError();
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(CTA);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = CLUSTER;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, a);
}

cudaError_t launch_chaos(int cta, int cluster, const ChaosArgs& a, uint32_t grid, cudaStream_t st) {
    switch (cta * 16 + cluster) {
    case 256 * 16 + 1: return launch_chaos_t<256, 1>(a, grid, st);
    case 512 * 16 + 1: return launch_chaos_t<512, 1>(a, grid, st);
    case 1024 * 16 + 1: return launch_chaos_t<1024, 1>(a, grid, st);
    case 512 * 16 + 2: return launch_chaos_t<512, 2>(a, grid, st);
    case 512 * 16 + 4: return launch_chaos_t<512, 4>(a, grid, st);
    case 512 * 16 + 8: return launch_chaos_t<512, 8>(a, grid, st);
    case 1024 * 16 + 2: return launch_chaos_t<1024, 2>(a, grid, st);
    case 1024 * 16 + 4: return launch_chaos_t<1024, 4>(a, grid, st);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_init_rng(uint4* rng, uint64_t n, uint64_t seed, cudaStream_t st) {
    const uint32_t b = 256;
    init_rng_kernel<<<(unsigned)((n + b - 1) / b), b, 0, st>>>(rng, n, seed);
    return cudaGetLastError();
}

cudaError_t launch_shuffle_table(uint16_t* out, uint32_t n, uint32_t count, uint64_t seed, cudaStream_t st) {
    const uint64_t total = (uint64_t)n * count;
    const uint32_t b = 256;
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
