// The variation library on the device: one switch case per supported entry of the
// reference's variations.yaml, each naming its yaml lines.  A genome's xforms reference these
// cases by id (program.h); a 256-walker group evaluates one xform per pass, so every warp takes
// the same case.  RNG draws happen in the snippets' textual order, which GLSL evaluates left to
// right, so a slot's stream advances exactly as in the reference.
#pragma once

#include "device.cuh"

#ifndef RFK_INLINE_MATH
// The FP32 library functions with long argument-reduction paths are called out of line: one
// shared copy each instead of one per call site keeps the chaos kernels' code within the
// instruction caches (genome-specialised kernels inline every xform's variations; the
// interpreted kernel's variation switch has 68 cases).  The same functions are called, so the
// results are unchanged.  Measured on the 1080p genome: 40.9 -> 45.8 Gpoints/s (specialised).
namespace rfk {
static __device__ __noinline__ float m_sinf(float x) { return sinf(x); }
static __device__ __noinline__ float m_cosf(float x) { return cosf(x); }
static __device__ __noinline__ float m_tanf(float x) { return tanf(x); }
static __device__ __noinline__ float m_expf(float x) { return expf(x); }
static __device__ __noinline__ float m_logf(float x) { return logf(x); }
static __device__ __noinline__ float m_sinhf(float x) { return sinhf(x); }
static __device__ __noinline__ float m_coshf(float x) { return coshf(x); }
static __device__ __noinline__ float m_powf(float x, float y) { return powf(x, y); }
static __device__ __noinline__ float m_atan2f(float y, float x) { return atan2f(y, x); }
static __device__ __noinline__ float2 m_sincosf(float x) {
    float s, c;
    sincosf(x, &s, &c);
    return make_float2(s, c);
}
}  // namespace rfk
#define sinf(a_) ::rfk::m_sinf(a_)
#define cosf(a_) ::rfk::m_cosf(a_)
#define tanf(a_) ::rfk::m_tanf(a_)
#define expf(a_) ::rfk::m_expf(a_)
#define logf(a_) ::rfk::m_logf(a_)
#define sinhf(a_) ::rfk::m_sinhf(a_)
#define coshf(a_) ::rfk::m_coshf(a_)
#define powf(a_, b_) ::rfk::m_powf(a_, b_)
#define atan2f(a_, b_) ::rfk::m_atan2f(a_, b_)
#define sincosf(a_, s_, c_)                             \
    do {                                                \
        const float2 rfk_sc_ = ::rfk::m_sincosf(a_);    \
        *(s_) = rfk_sc_.x;                              \
        *(c_) = rfk_sc_.y;                              \
    } while (0)
#endif

namespace rfk {

constexpr float kPI = 3.14159265358979f;  // math.glsl:1, FP32
constexpr float kEPS = 1e-10f;            // math.glsl:4

struct Pre {  // common precalcs, variations.yaml:1-9
    float x, y, r, rsq, a, phi, sina, cosa, sinr, cosr;
};

__device__ __forceinline__ void precalc(Pre& p, float x, float y, uint32_t m) {
    p.x = x; p.y = y;
    p.r = p.rsq = p.a = p.phi = p.sina = p.cosa = p.sinr = p.cosr = 0.0f;
    if (m & (PC_R | PC_RSQ)) {
        const float q = fmaf(x, x, y * y);
        p.rsq = q;
        p.r = sqrtf(q);
    }
    if (m & PC_A) p.a = atan2f(x, y);
    if (m & PC_PHI) p.phi = atan2f(y, x);
    if (m & PC_SINA) p.sina = x / p.r;
    if (m & PC_COSA) p.cosa = y / p.r;
    if (m & (PC_SINR | PC_COSR)) sincosf(p.r, &p.sinr, &p.cosr);
}

__device__ __forceinline__ float mod2f(float x, float y) { return x - y * truncf(x / y); }  // math.glsl:13

struct VaryOut {  // a variation's value and the slot's RNG state after it
    float x, y;
    Jsf rng;
};

#ifndef RFK_VARY_INLINE
#define RFK_VARY_ATTR static __device__ __noinline__
#else
#define RFK_VARY_ATTR static __device__ __forceinline__
#endif

// Unweighted value of variation `id` (radial_blur applies its weight internally).  Kept out of
// line: the 68 cases inlined into the chaos loop need ~120 registers and spill heavily at 64;
// as a call, the loop stays within 64 registers and only the case taken pays for its own.
// Everything passes by value so nothing is materialised on the stack.
__device__ __forceinline__ float2 vary_impl(uint32_t id, const Pre p, float w, const float* __restrict__ aff,
                                            const float* __restrict__ P, Jsf& rng) {
    const float x = p.x, y = p.y, r = p.r, rsq = p.rsq, a = p.a, phi = p.phi;
    float s, c;
    switch (id) {
    case 0: return make_float2(x, y);                                          // linear :13
    case 1: return make_float2(sinf(x), sinf(y));                              // sinusoidal :16
    case 2: { const float k = 1.0f / (rsq + kEPS); return make_float2(x * k, y * k); }  // spherical :19
    case 3: sincosf(rsq, &s, &c); return make_float2(s * x - c * y, c * x + s * y);     // swirl :22
    case 4: { const float k = 1.0f / (r + kEPS);                               // horseshoe :28
              return make_float2((x + y) * (x - y) * k, 2.0f * x * y * k); }
    case 5: return make_float2(a / kPI, r - 1.0f);                             // polar :31
    case 6: return make_float2(r * sinf(a + r), r * cosf(a - r));              // handkerchief :34
    case 7: sincosf(r * a, &s, &c); return make_float2(r * s, -(r * c));       // heart :37
    case 8: { sincosf(r * kPI, &s, &c); const float k = a / kPI;               // disc :40
              return make_float2(k * s, k * c); }
    case 9: { const float k = 1.0f / (r + kEPS);                               // spiral :43
              return make_float2((p.cosa + p.sinr) * k, (p.sina - p.cosr) * k); }
    case 10: return make_float2(p.sina / (r + kEPS), p.cosa * r);              // hyperbolic :46
    case 11: return make_float2(p.sina * p.cosr, p.cosa * p.sinr);             // diamond :49
    case 12: { const float n0 = sinf(a + r), n1 = cosf(a - r);                 // ex :52
               const float m0 = n0 * n0 * n0 * r, m1 = n1 * n1 * n1 * r;
               return make_float2(m0 + m1, m0 - m1); }
    case 13: { const float u = randf(rng);                                     // julia :60
               sincosf(0.5f * a + roundf(u) * kPI, &s, &c);
               const float q = sqrtf(r);
               return make_float2(q * c, q * s); }
    case 14: return make_float2(x < 0.0f ? 2.0f * x : x, y < 0.0f ? y * 0.5f : y);  // bent :64
    case 15: return make_float2(x + aff[2] * sinf(y / (aff[4] * aff[4] + kEPS)),    // waves :71
                                y + aff[3] * sinf(x / (aff[5] * aff[5] + kEPS)));
    case 16: { const float k = 2.0f / (r + 1.0f); return make_float2(k * y, k * x); }  // fisheye :78
    case 17: return make_float2(x + aff[4] * sinf(tanf(3.0f * y)),              // popcorn :81
                                y + aff[5] * sinf(tanf(3.0f * x)));
    case 18: { const float e = expf(x - 1.0f); sincosf(kPI * y, &s, &c);       // exponential :88
               return make_float2(e * c, e * s); }
    case 19: { const float k = powf(r, p.sina); return make_float2(k * p.cosa, k * p.sina); }  // power :91
    case 20: sincosf(kPI * x, &s, &c);                                          // cosine :94
             return make_float2(c * coshf(y), -s * sinhf(y));
    case 21: { const float dx = aff[4] * aff[4] + kEPS;                        // rings :97
               const float k = mod2f(r + dx, 2.0f * dx) - dx + r * (1.0f - dx);
               return make_float2(k * p.cosa, k * p.sina); }
    case 22: { const float dx = kPI * (aff[4] * aff[4] + kEPS), dx2 = dx * 0.5f;  // fan :102
               const float fa = a + ((mod2f(a + aff[5], dx) > dx2) ? -dx2 : dx2);
               sincosf(fa, &s, &c);
               return make_float2(r * c, r * s); }
    case 23: { const float k = r * (P[1] + (P[0] - P[1]) * (0.5f + 0.5f * sinf(P[2] * a)));  // blob :110
               return make_float2(k * p.sina, k * p.cosa); }
    case 24: return make_float2(sinf(P[0] * y) - cosf(P[1] * x),                 // pdj :117
                                sinf(P[2] * x) - cosf(P[3] * y));
    case 25: { const float dx = kPI * (P[0] * P[0] + kEPS), dx2 = 0.5f * dx;   // fan2 :129
               const float t = a + P[1] - dx * floorf((a + P[1]) / dx);
               sincosf(t > dx2 ? a - dx2 : a + dx2, &s, &c);
               return make_float2(r * s, r * c); }
    case 26: { const float dx = P[0] * P[0] + kEPS;                            // rings2 :143
               const float rr = r + (-2.0f * dx * truncf((r + dx) / (2.0f * dx)) + r * (1.0f - dx));
               return make_float2(rr * p.sina, rr * p.cosa); }
    case 27: { const float k = 2.0f / (r + 1.0f); return make_float2(k * x, k * y); }  // eyefish :152
    case 28: { const float k = 1.0f / fmaf(rsq, 0.25f, 1.0f); return make_float2(x * k, y * k); }  // bubble :155
    case 29: { sincosf(P[0], &s, &c); const float d = P[1] - y * s;           // perspective :158
               return make_float2(x * P[1] / d, P[1] * c * y / d); }
    case 30: { const float u1 = randf(rng); const float u2 = randf(rng);       // noise :166
               sincosf(u2 * 2.0f * kPI, &s, &c);
               return make_float2(x * u1 * c, y * u1 * s); }
    case 31: { const float t = truncf(fabsf(P[0]) * randf(rng));              // julian :169
               const float k = powf(r, P[1] / P[0]);
               sincosf((phi + 2.0f * kPI * t) / P[0], &s, &c);
               return make_float2(k * c, k * s); }
    case 32: { const float t = truncf(fabsf(P[0]) * randf(rng));              // juliascope :182
               const float k = powf(r, P[1] / P[0]);
               const float sg = (((int)t) & 1) ? -1.0f : 1.0f;
               sincosf((2.0f * kPI * t + sg * phi) / P[0], &s, &c);
               return make_float2(k * c, k * s); }
    case 33: { const float u1 = randf(rng); const float u2 = randf(rng);       // blur :195
               sincosf(u2 * 2.0f * kPI, &s, &c);
               return make_float2(u1 * c, u1 * s); }
    case 34: { float q = randf(rng); q += randf(rng); q += randf(rng); q += randf(rng);  // gaussian_blur :198
               q -= 2.0f;
               sincosf(randf(rng) * 2.0f * kPI, &s, &c);
               return make_float2(q * c, q * s); }
    case 35: { float zs, zc; sincosf(P[0] * kPI / 2.0f, &zs, &zc);            // radial_blur :201
               float q = randf(rng); q += randf(rng); q += randf(rng); q += randf(rng);
               const float g = w * (q - 2.0f);
               sincosf(phi + zs * g, &s, &c);
               const float rz = zc * g - 1.0f;
               return make_float2(r * c + rz * x, r * s + rz * y); }
    case 36: { const float u1 = randf(rng); const float u2 = randf(rng); const float u3 = randf(rng);  // pie :212
               sincosf(P[1] + 2.0f * kPI * (truncf(u2 * P[0] + 0.5f) + u3 * P[2]) / P[0], &s, &c);
               return make_float2(u1 * s, u1 * c); }
    case 37: { const float rf = powf(rsq, P[0] * 0.5f);                       // ngon :219
               const float b = 2.0f * kPI / (P[1] + kEPS);
               float t = phi - b * floorf(a / b);
               if (t > b * 0.5f) t -= b;
               const float k = (P[2] * (1.0f / (cosf(t) + kEPS) - 1.0f) + P[3]) / (rf + kEPS);
               return make_float2(k * x, k * y); }
    case 38: { const float re = 1.0f + P[0] * x + P[1] * (x * x - y * y);     // curl :232
               const float im = P[0] * y + 2.0f * P[1] * x * y;
               const float k = 1.0f / (re * re + im * im);
               return make_float2((x * re + y * im) * k, (y * re - x * im) * k); }
    case 39: return make_float2(P[0] == 0.0f ? x : (2.0f * floorf(x / P[0]) + 1.0f) * P[0] - x,  // rectangles :241
                                P[1] == 0.0f ? y : (2.0f * floorf(y / P[1]) + 1.0f) * P[1] - y);
    case 40: sincosf(randf(rng) * w * kPI, &s, &c);                             // arch :251
             return make_float2(s, s * s / c);
    case 41: return make_float2(sinf(x) / cosf(y), tanf(y));                   // tangent :256
    case 42: { const float u1 = randf(rng); const float u2 = randf(rng);       // square :259
               return make_float2(u1 - 0.5f, u2 - 0.5f); }
    case 43: { const float ang = w * randf(rng) * kPI;                         // rays :262
               const float k = tanf(ang) * (w / (rsq + kEPS));
               return make_float2(k * cosf(x), k * sinf(y)); }
    case 44: sincosf(randf(rng) * w * r, &s, &c);                               // blade :268
             return make_float2(x * (c + s), x * (c - s));
    case 45: { const float cr = cosf(w * r);                                   // secant2 :273
               return make_float2(x, 1.0f / cr + (cr < 0.0f ? 1.0f : -1.0f)); }
    case 47: { const float q = x * x - y * y;                                  // cross :286
               const float k = sqrtf(1.0f / (q * q + kEPS));
               return make_float2(x * k, y * k); }
    case 48: { float ax, ay; sincosf(P[1], &ax, &ay);                          // disc2 :291
               ay -= 1.0f;
               const float k = 1.0f + P[1] + ((P[1] > 2.0f * kPI) ? -2.0f : 2.0f) * kPI;
               ax *= k; ay *= k;
               sincosf(P[0] * kPI * (x + y), &s, &c);
               const float f = a / kPI;
               return make_float2((s + ay) * f, (c + ax) * f); }
    case 49: { sincosf(P[3] * 0.25f * phi + kPI * 0.25f, &s, &c);             // super_shape :303
               const float u = randf(rng);
               const float m = r * (1.0f - P[5]) + u * P[5];
               const float k = (m - P[4]) * powf(powf(fabsf(c), P[1]) + powf(fabsf(s), P[2]), -1.0f / P[0]) / r;
               return make_float2(x * k, y * k); }
    case 50: { const float k = (randf(rng) - P[0]) * cosf(P[1] * phi) / r;    // flower :315
               return make_float2(x * k, y * k); }
    case 51: { const float k = (randf(rng) - P[0]) * P[1] / (1.0f + P[1] * x / r) / r;  // conic :321
               return make_float2(x * k, y * k); }
    case 52: { const float u1 = randf(rng); const float u2 = randf(rng);       // parabola :327
               return make_float2(P[0] * p.sinr * p.sinr * u1, P[1] * p.cosr * u2); }
    case 55: { const float rx = roundf(x), ry = roundf(y);                     // boarders :351
               const float ox = x - rx, oy = y - ry;
               if (randf(rng) >= 0.75f) return make_float2(ox * 0.5f + rx, oy * 0.5f + ry);
               if (fabsf(ox) >= fabsf(oy)) {
                   if (ox > 0.0f) return make_float2(ox * 0.5f + rx + 0.25f, oy * 0.5f + ry + 0.25f * oy / ox);
                   return make_float2(ox * 0.5f + rx - 0.25f, oy * 0.5f + ry - 0.25f * oy / ox);
               }
               if (oy > 0.0f) return make_float2(ox * 0.5f + rx + 0.25f * ox / oy, oy * 0.5f + ry + 0.25f);
               return make_float2(ox * 0.5f + rx - 0.25f * ox / oy, oy * 0.5f + ry - 0.25f); }
    case 56: { const float y2 = 2.0f * y;                                      // butterfly :392
               const float k = 1.3029400317411197908970256609023f * sqrtf(fabsf(x * y) / (kEPS + x * x + y2 * y2));
               return make_float2(k * x, k * y2); }
    case 59: return make_float2(x + P[2] * expf(-y * y / fmaxf(P[0] * P[0], 1e-20f)),  // curve :425
                                y + P[3] * expf(-x * x / fmaxf(P[1] * P[1], 1e-20f)));
    case 61: { const float e = expf(x) * 0.5f, en = 0.25f / e;                 // foci :450
               sincosf(y, &s, &c);
               const float k = 1.0f / (e + en - c);
               return make_float2((e - en) * k, s * k); }
    case 63: { const float w2 = w * w;                                         // loonie :459
               const float k = (rsq < w2) ? sqrtf(w2 / rsq - 1.0f) : 1.0f;
               return make_float2(x * k, y * k); }
    case 64: { const float e = expf(x); sincosf(y, &s, &c); return make_float2(e * c, e * s); }  // exp :464
    case 65: return make_float2(0.5f * logf(rsq), phi);                        // log :467
    case 66: sincosf(x, &s, &c); return make_float2(s * coshf(y), c * sinhf(y));   // sin :470
    case 67: sincosf(x, &s, &c); return make_float2(c * coshf(y), s * sinhf(y));   // cos :473
    case 68: sincosf(y, &s, &c); return make_float2(sinhf(x) * c, coshf(x) * s);   // sinh :476
    case 69: { float q = randf(rng); q += randf(rng); q += randf(rng); q += randf(rng);  // pre_blur :481
               q -= 2.0f;
               sincosf(randf(rng) * 2.0f * kPI, &s, &c);
               return make_float2(q * c, q * s); }
    case 70: return make_float2(x + P[0] * sinf(y * P[2]), y + P[1] * sinf(x * P[3]));  // waves2 :485
    case 71: return make_float2(sinf(x), y);                                   // cylinder :497
    case 73: { const float su = sinf(x * P[0]), tu = sinf(y * P[0]);          // auger :508
               const float dy = y + P[3] * (P[1] * su * 0.5f + fabsf(y) * su);
               const float dx = x + P[3] * (P[1] * tu * 0.5f + fabsf(x) * tu);
               return make_float2(x + P[2] * (dx - x), dy); }
    case 74: { const float xp = x + w, xm = x - w;                             // flux :521
               const float k = (2.0f + P[0]) * sqrtf(sqrtf(y * y + xp * xp) / sqrtf(y * y + xm * xm));
               sincosf((atan2f(y, xm) - atan2f(y, xp)) * 0.5f, &s, &c);
               return make_float2(k * c, k * s); }
    case 75: { const float ru = P[0] * x - P[4] * y + P[1];                    // mobius :532
               const float iu = P[0] * y + P[4] * x + P[5];
               const float rv = P[2] * x - P[6] * y + P[3];
               const float iv = P[2] * y + P[6] * x + P[7];
               const float k = 1.0f / (rv * rv + iv * iv);
               return make_float2((ru * rv + iu * iv) * k, (iu * rv - ru * iv) * k); }
    default: break;
    }
    return make_float2(__int_as_float(0x7fffffff), __int_as_float(0x7fffffff));
}

RFK_VARY_ATTR VaryOut vary_call(uint32_t id, const Pre p, float w, const float* __restrict__ aff,
                                const float* __restrict__ P, Jsf rng) {
    const float2 v = vary_impl(id, p, w, aff, P, rng);
    return VaryOut{v.x, v.y, rng};
}

__device__ __forceinline__ float2 vary(uint32_t id, const Pre& p, float w, const float* __restrict__ aff,
                                       const float* __restrict__ P, Jsf& rng) {
    const VaryOut o = vary_call(id, p, w, aff, P, rng);
    rng = o.rng;
    return make_float2(o.x, o.y);
}

// dispatch() of one xform block: src/variation_table.cpp:97-165 (affine prelude, pre_xform
// terms, precalcs, weighted terms in map order, post) and :241-243 (colour, opacity).
__device__ __forceinline__ void eval_xform(const uint32_t* __restrict__ blk, float& x, float& y, float& c,
                                           float& op, bool first_run, Jsf& rng) {
    const float* fb = reinterpret_cast<const float*>(blk);
    float vx = fmaf(fb[X_AFF + 0], x, fmaf(fb[X_AFF + 2], y, fb[X_AFF + 4]));
    float vy = fmaf(fb[X_AFF + 1], x, fmaf(fb[X_AFF + 3], y, fb[X_AFF + 5]));
    const uint32_t npre = blk[X_NPRE], nterm = blk[X_NTERM];
    const uint32_t* e = blk + X_TERMS;
    Pre pc;
    for (uint32_t k = 0; k < npre; k++, e += 3) {
        pc.x = vx; pc.y = vy;
        const float wt = __uint_as_float(e[1]);
        const float2 d = vary(e[0] & 0xffu, pc, wt, fb + X_AFF, fb + e[2], rng);
        vx = __fadd_rn(vx, __fmul_rn(wt, d.x));
        vy = __fadd_rn(vy, __fmul_rn(wt, d.y));
    }
    precalc(pc, vx, vy, blk[X_MASK]);
    float rx = 0.0f, ry = 0.0f;
    for (uint32_t k = 0; k < nterm; k++, e += 3) {
        const float wt = __uint_as_float(e[1]);
        float2 d = vary(e[0] & 0xffu, pc, wt, fb + X_AFF, fb + e[2], rng);
        if (!(e[0] & kTermNoWeightMul)) { d.x = __fmul_rn(wt, d.x); d.y = __fmul_rn(wt, d.y); }
        if (k == 0) { rx = d.x; ry = d.y; }
        else { rx = __fadd_rn(rx, d.x); ry = __fadd_rn(ry, d.y); }
    }
    if (blk[X_HASPOST]) {
        const float px = fmaf(fb[X_POST + 0], rx, fmaf(fb[X_POST + 2], ry, fb[X_POST + 4]));
        const float py = fmaf(fb[X_POST + 1], rx, fmaf(fb[X_POST + 3], ry, fb[X_POST + 5]));
        rx = px; ry = py;
    }
    const float cin = first_run ? randf(rng) : c;
    c = __fadd_rn(__fmul_rn(cin, fb[X_OMCS]), __fmul_rn(fb[X_COLOR], fb[X_CS]));
    x = rx; y = ry;
    op = fb[X_OPACITY];
}

}  // namespace rfk
