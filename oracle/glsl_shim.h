// GLSL-to-C++ shim — TEST INFRASTRUCTURE ONLY.
//
// Just enough of GLSL 4.60's types and built-ins for the reference's own shader snippets
// (variations.yaml, shaders/include/math.glsl, the ranval/randf functions of
// shaders/include/random.glsl) to compile as C++ after the textual rewrites done by
// oracle/ref_build.py.  Snippet arithmetic runs in `real` (double); GLSL float literals are
// rounded to FP32 first (F32) so constants keep their shader values.
#ifndef REFRAKT_GLSL_SHIM_H
#define REFRAKT_GLSL_SHIM_H

#include <cmath>
#include <cstdint>

namespace glsl {

typedef double real;
typedef uint32_t uint;

#define F32(v) ((::glsl::real)(float)(v))

struct vec2 {
    real x, y;
    vec2() : x(0), y(0) {}
    vec2(real a, real b) : x(a), y(b) {}
    explicit vec2(real a) : x(a), y(a) {}
    vec2 yx() const { return vec2(y, x); }
    vec2& operator+=(const vec2& o) { x += o.x; y += o.y; return *this; }
    vec2& operator-=(const vec2& o) { x -= o.x; y -= o.y; return *this; }
    vec2& operator*=(real s) { x *= s; y *= s; return *this; }
    vec2& operator*=(const vec2& o) { x *= o.x; y *= o.y; return *this; }
    vec2& operator/=(real s) { x /= s; y /= s; return *this; }
};
inline vec2 operator+(vec2 a, vec2 b) { return vec2(a.x + b.x, a.y + b.y); }
inline vec2 operator-(vec2 a, vec2 b) { return vec2(a.x - b.x, a.y - b.y); }
inline vec2 operator*(vec2 a, vec2 b) { return vec2(a.x * b.x, a.y * b.y); }
inline vec2 operator/(vec2 a, vec2 b) { return vec2(a.x / b.x, a.y / b.y); }
inline vec2 operator*(vec2 a, real s) { return vec2(a.x * s, a.y * s); }
inline vec2 operator*(real s, vec2 a) { return vec2(s * a.x, s * a.y); }
inline vec2 operator/(vec2 a, real s) { return vec2(a.x / s, a.y / s); }
inline vec2 operator+(vec2 a, real s) { return vec2(a.x + s, a.y + s); }
inline vec2 operator-(vec2 a, real s) { return vec2(a.x - s, a.y - s); }
inline vec2 operator-(vec2 a) { return vec2(-a.x, -a.y); }

struct uvec4 { uint x, y, z, w; };

inline real sin(real v) { return std::sin(v); }
inline real cos(real v) { return std::cos(v); }
inline real tan(real v) { return std::tan(v); }
inline real sinh(real v) { return std::sinh(v); }
inline real cosh(real v) { return std::cosh(v); }
inline real exp(real v) { return std::exp(v); }
inline real log(real v) { return std::log(v); }
inline real pow(real a, real b) { return std::pow(a, b); }
inline real sqrt(real v) { return std::sqrt(v); }
inline real abs(real v) { return std::fabs(v); }
inline real floor(real v) { return std::floor(v); }
inline real trunc(real v) { return std::trunc(v); }
inline real round(real v) { return std::round(v); }  // GLSL leaves .5 open; half away from zero
inline real atan(real v) { return std::atan(v); }
inline real atan(real y, real x) { return std::atan2(y, x); }
inline real fma(real a, real b, real c) { return std::fma(a, b, c); }
inline real mix(real x, real y, real a) { return x * (1.0 - a) + y * a; }
inline real max(real a, real b) { return a > b ? a : b; }
inline real min(real a, real b) { return a < b ? a : b; }
inline real length(vec2 v) { return std::sqrt(v.x * v.x + v.y * v.y); }
inline vec2 sin(vec2 v) { return vec2(std::sin(v.x), std::sin(v.y)); }
template <class T, class U, class V>
inline T clamp(T x, U lo, V hi) { return x < (T)lo ? (T)lo : (x > (T)hi ? (T)hi : x); }

// the point a snippet sees: v.x, v.y and v.xy
struct vin {
    real x, y;
    vec2 xy() const { return vec2(x, y); }
};

// ---- what the whole shaders (tonemap.glsl, density_{vert,frag}.glsl, the templates) need
inline real dot(vec2 a, vec2 b) { return a.x * b.x + a.y * b.y; }
struct vec3 {
    real x, y, z;
    vec3() : x(0), y(0), z(0) {}
    vec3(real a, real b, real c) : x(a), y(b), z(c) {}
    explicit vec3(real a) : x(a), y(a), z(a) {}
};
inline vec3 operator*(real s, vec3 v) { return vec3(s * v.x, s * v.y, s * v.z); }
inline vec3 operator*(vec3 v, real s) { return vec3(s * v.x, s * v.y, s * v.z); }
inline vec3 pow(vec3 a, vec3 b) { return vec3(std::pow(a.x, b.x), std::pow(a.y, b.y), std::pow(a.z, b.z)); }
inline vec3 mix(vec3 x, vec3 y, real a) { return vec3(mix(x.x, y.x, a), mix(x.y, y.y, a), mix(x.z, y.z, a)); }
inline vec3 clamp(vec3 v, real lo, real hi) { return vec3(clamp(v.x, lo, hi), clamp(v.y, lo, hi), clamp(v.z, lo, hi)); }
// vec4 as the shaders use it: .r .g .b .a, .rgb read (rgb()) and written (set_rgb, textual rewrite)
struct vec4 {
    real r, g, b, a;
    vec4() : r(0), g(0), b(0), a(0) {}
    vec4(real x, real y, real z, real w) : r(x), g(y), b(z), a(w) {}
    vec4(vec2 v, real z, real w) : r(v.x), g(v.y), b(z), a(w) {}
    vec3 rgb() const { return vec3(r, g, b); }
    void set_rgb(vec3 v) { r = v.x; g = v.y; b = v.z; }
    vec4& operator*=(real s) { r *= s; g *= s; b *= s; a *= s; return *this; }
};
inline vec4 operator*(vec4 v, real s) { return vec4(v.r * s, v.g * s, v.b * s, v.a * s); }
struct uvec2 { uint x, y; };
struct uvec3 { uint x, y, z; uvec2 xy; };
struct ivec2 {
    int x, y;
    ivec2() : x(0), y(0) {}
    ivec2(int a, int b) : x(a), y(b) {}
    explicit ivec2(uvec2 u) : x((int)u.x), y((int)u.y) {}
};
// the vertex shader's projection: identity (its output position is not part of the pins)
struct mat4 {};
inline vec4 operator*(mat4, vec4 v) { return v; }

}  // namespace glsl

#endif
