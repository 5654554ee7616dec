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

}  // namespace glsl

#endif
