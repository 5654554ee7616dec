// Device helpers of the chaos game: the JSF32 generator, keyed permutations for the walker
// shuffle, start points, and the first-pass jitter.
#pragma once

#include "rtc_types.h"

#include "program.h"

namespace rfk {

// JSF32 — shaders/include/random.glsl:29-37.  The GLSL ranval returns the new `a`.
struct Jsf { uint32_t a, b, c, d; };

__device__ __forceinline__ uint32_t rotl32(uint32_t x, int k) { return __funnelshift_l(x, x, k); }

__device__ __forceinline__ uint32_t jsf_next(Jsf& s) {
    const uint32_t e = s.a - rotl32(s.b, 27);
    s.a = s.b ^ rotl32(s.c, 17);
    s.b = s.c + s.d;
    s.c = s.d + e;
    s.d = e + s.a;
    return s.a;
}

// random.glsl:39-41: clamp(float(u) / 4294967295.0f, 0, 1).  The FP32 literal is 2^32, so the
// quotient is exactly float(u) * 2^-32 (already within [0, 1]).
__device__ __forceinline__ float randf(Jsf& s) { return __uint2float_rn(jsf_next(s)) * 0x1p-32f; }

// src/util.hpp:90-95 warmup_ctx
__device__ __forceinline__ Jsf jsf_seed(uint32_t seed) {
    Jsf s{0xf1ea5eedu, seed, seed, seed};
    for (int i = 0; i < 20; i++) (void)jsf_next(s);
    return s;
}

// --- keyed permutations (splitmix64 finaliser by S. Vigna; lowbias32 by C. Wellons) ---
__host__ __device__ __forceinline__ uint64_t mix64(uint64_t x) {
    x ^= x >> 30; x *= 0xbf58476d1ce4e5b9ull;
    x ^= x >> 27; x *= 0x94d049bb133111ebull;
    x ^= x >> 31;
    return x;
}
__host__ __device__ __forceinline__ uint32_t lowbias32(uint32_t x) {
    x ^= x >> 16; x *= 0x7feb352du;
    x ^= x >> 15; x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}
__host__ __device__ __forceinline__ uint64_t derive_key(uint64_t seed, uint64_t a, uint64_t b, uint64_t tag) {
    uint64_t k = mix64(seed + 0x9e3779b97f4a7c15ull);
    k = mix64(k ^ (tag * 0xd1b54a32d192ed03ull));
    k = mix64(k ^ (a + 0x632be59bd9b4e019ull));
    k = mix64(k ^ (b + 0x8cb92ba72f3d8dd7ull));
    return k;
}
// 4-round balanced Feistel network over 2h bits, cycle-walked into [0, n).  A bijection of
// [0, n) for every key; the walk terminates because the cycle through x contains x < n.
__host__ __device__ __forceinline__ uint32_t feistel(uint32_t x, uint32_t n, uint64_t key) {
    if (n <= 1) return 0;
    uint32_t bits = 0;
    while ((1u << bits) < n) bits++;
    if (bits < 2) bits = 2;
    if (bits & 1) bits++;
    const uint32_t h = bits / 2, mask = (1u << h) - 1u;
    const uint32_t k0 = (uint32_t)key, k1 = (uint32_t)(key >> 32);
    const uint32_t k2 = lowbias32(k0 ^ 0x68e31da4u), k3 = lowbias32(k1 ^ 0xb5297a4du);
    do {
        uint32_t L = x >> h, R = x & mask;
#pragma unroll
        for (int r = 0; r < 4; r++) {
            const uint32_t kr = (r == 0) ? k0 : (r == 1) ? k1 : (r == 2) ? k2 : k3;
            const uint32_t f = lowbias32(R ^ kr) & mask;
            const uint32_t nl = R;
            R = L ^ f;
            L = nl;
        }
        x = (L << h) | R;
    } while (x >= n);
    return x;
}

// src/hammersley.cpp:29-48 make_sample_points, point i of `count`, evaluated on the fly.
// (double)(f) * 2.0 - 1.0 is exact in double for f >= 2^-32, so a single FP32 rounding of
// 2f - 1 reproduces the host's float result.
__device__ __forceinline__ void sample_point(uint32_t i, uint32_t count, float& x, float& y) {
    uint32_t mx = count;
    if (count & 1u) { mx = count - 1; mx |= mx >> 1; mx |= mx >> 2; mx |= mx >> 4; mx |= mx >> 8; mx |= mx >> 16; mx++; }
    const float inv = __fdiv_rn(1.0f, __uint2float_rn(mx));
    const uint32_t r = 31 - __clz(mx);
    const float fx = __fmul_rn(__uint2float_rn(i), inv);
    x = __fsub_rn(__fmul_rn(fx, 2.0f), 1.0f);
    const uint32_t fb = (r == 0) ? 0u : (__brev(i) >> (32 - r));
    const float fy = __fmul_rn(__uint2float_rn(fb), inv);
    y = __fsub_rn(__fmul_rn(fy, 2.0f), 1.0f);
}

// sin and cos of t in [0, 1] for the first-pass jitter (flame.glsl:64, t = sqrt(randf())):
// Taylor series about 0 through t^13 / t^14 in Horner form with FP32 fma (below 1 ulp on
// [0, 1]); the host oracle evaluates the identical sequence.
__device__ __forceinline__ void jitter_sincos(float t, float& s, float& c) {
    const float t2 = __fmul_rn(t, t);
    float p = 1.0f / 6227020800.0f;
    p = fmaf(p, t2, -1.0f / 39916800.0f);
    p = fmaf(p, t2, 1.0f / 362880.0f);
    p = fmaf(p, t2, -1.0f / 5040.0f);
    p = fmaf(p, t2, 1.0f / 120.0f);
    p = fmaf(p, t2, -1.0f / 6.0f);
    p = fmaf(p, t2, 1.0f);
    s = __fmul_rn(t, p);
    float q = -1.0f / 87178291200.0f;
    q = fmaf(q, t2, 1.0f / 479001600.0f);
    q = fmaf(q, t2, -1.0f / 3628800.0f);
    q = fmaf(q, t2, 1.0f / 40320.0f);
    q = fmaf(q, t2, -1.0f / 720.0f);
    q = fmaf(q, t2, 1.0f / 24.0f);
    q = fmaf(q, t2, -0.5f);
    c = fmaf(q, t2, 1.0f);
}

// xform_select.tpl.glsl: sequential FP32 sum of the normalised weights; first i with
// sum >= r; the last xform unconditionally.
__device__ __forceinline__ int select_xform(const uint32_t* prog, float r) {
    const uint32_t n = prog[H_NX];
    const float* w = reinterpret_cast<const float*>(prog + prog[H_WOFF]);
    float sum = 0.0f;
    for (uint32_t i = 0; i + 1 < n; i++) {
        sum = (i == 0) ? w[0] : __fadd_rn(sum, w[i]);
        if (sum >= r) return (int)i;
    }
    return (int)n - 1;
}

// math.glsl:22 `badval`: NaN, or beyond +-1e10.
__device__ __forceinline__ bool bad_value(float v) { return !(fabsf(v) <= 1e10f); }

// The walker reset the reference keeps commented out after dispatch (flame.glsl:68):
// `if (badval(result.x) || badval(result.y)) result.xyw = vec3(vec2(randf(), randf()) * 2.0 - 1.0, 0.0)`.
// A walker that left the plane (NaN, infinity, |v| > 1e10) restarts at a uniform point of
// [-1, 1]^2 with opacity 0, so the restart itself is not drawn.  u * 2 is exact, so the FP32 fma
// rounds 2u - 1 once, as the shader's mul-then-sub does.  Returns true when it reset.
__device__ __forceinline__ bool reset_bad_walker(float& x, float& y, float& op, Jsf& rng) {
    if (!(bad_value(x) || bad_value(y))) return false;
    const float u1 = randf(rng);
    const float u2 = randf(rng);
    x = fmaf(u1, 2.0f, -1.0f);
    y = fmaf(u2, 2.0f, -1.0f);
    op = 0.0f;
    return true;
}

// flame.glsl:84: min(255, uint(ceil(c * 255.0))); negative or NaN colours index 0.
__device__ __forceinline__ uint32_t palette_index(float c) {
    const float v = ceilf(__fmul_rn(c, 255.0f));
    if (!(v > 0.0f)) return 0u;
    return v >= 255.0f ? 255u : (uint32_t)v;
}

}  // namespace rfk
