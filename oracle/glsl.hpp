// glsl.hpp — a small GLSL 4.60 compatibility layer for C++20 (test infrastructure).
//
// It gives the CPU oracle GLSL's value types (vec2..4, ivec, uvec, bvec, mat3,
// mat4), its built-in functions and a software model of the Vulkan texture units
// the reference's compute shaders sample through (linear filtering at texel
// centres with CLAMP_TO_EDGE, nearest texelFetch, UNORM/SNORM/FP16 decode and the
// float -> UNORM/SNORM/FP16 conversions of imageStore).
//
// Conventions that the GLSL and Vulkan specifications leave to the implementation
// are fixed here once, for the oracle and for the compiled reference shaders
// alike:
//   * float literals are single precision (compile with -fsingle-precision-constant);
//   * no FMA contraction (compile with -ffp-contract=off);
//   * linear filtering uses exact float weights (hardware uses 8-bit fractions);
//   * UNORM16 decode is u / 65535, SNORM8 is max(c / 127, -1);
//   * float -> UNORM/SNORM stores round to nearest even after clamping;
//   * round() rounds halves away from zero (C roundf).
//
// Multi-letter swizzles (.xyz, .rgb, .xy, .rg, .yz, .zw) are macros that expand to
// member calls returning a proxy; single-letter components are data members.
// Nothing here is used by the product library.
#pragma once
#include "prelude.hpp"

namespace glsl {

typedef unsigned int uint;

// ---------------------------------------------------------------- scalar math
inline float abs(float x) { return gl_fabs(x); }
inline int abs(int x) { return x < 0 ? -x : x; }
inline float sign(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }
inline float floor(float x) { return gl_floor(x); }
inline float ceil(float x) { return gl_ceil(x); }
inline float trunc(float x) { return gl_trunc(x); }
inline float fract(float x) { return x - gl_floor(x); }
inline float round(float x) { return gl_round(x); }
inline float roundEven(float x) { return gl_rint(x); }
inline float mod(float x, float y) { return x - y * gl_floor(x / y); }
// GLSL: min returns y if y < x, else x; max returns y if x < y, else x.
inline float min(float x, float y) { return y < x ? y : x; }
inline float max(float x, float y) { return x < y ? y : x; }
inline int min(int x, int y) { return y < x ? y : x; }
inline int max(int x, int y) { return x < y ? y : x; }
inline uint min(uint x, uint y) { return y < x ? y : x; }
inline uint max(uint x, uint y) { return x < y ? y : x; }
inline float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }
inline int clamp(int x, int lo, int hi) { return min(max(x, lo), hi); }
inline uint clamp(uint x, uint lo, uint hi) { return min(max(x, lo), hi); }
// mix as the GLSL specification defines it: x * (1 - a) + y * a.
inline float mix(float x, float y, float a) { return x * (1.0f - a) + y * a; }
inline float step(float edge, float x) { return x < edge ? 0.0f : 1.0f; }
inline float smoothstep(float e0, float e1, float x) {
    float t = clamp((x - e0) / (e1 - e0), 0.0f, 1.0f);
    return t * t * (3.0f - 2.0f * t);
}
inline float sqrt(float x) { return gl_sqrt(x); }
inline float inversesqrt(float x) { return 1.0f / gl_sqrt(x); }
inline float pow(float x, float y) { return gl_pow(x, y); }
inline float exp(float x) { return gl_exp(x); }
inline float exp2(float x) { return gl_exp2(x); }
inline float log(float x) { return gl_log(x); }
inline float log2(float x) { return gl_log2(x); }
inline float sin(float x) { return gl_sin(x); }
inline float cos(float x) { return gl_cos(x); }
inline float tan(float x) { return gl_tan(x); }
inline float asin(float x) { return gl_asin(x); }
inline float acos(float x) { return gl_acos(x); }
inline float atan(float y, float x) { return gl_atan2(y, x); }
inline float atan(float x) { return gl_atan(x); }
inline float radians(float d) { return d * (3.14159265358979f / 180.0f); }

template <class T> struct tvec2;
template <class T> struct tvec3;
template <class T> struct tvec4;

// Swizzle proxy: refers to components I... of vector V and behaves as an R.
template <class V, class R, int... I> struct swz {
    V* p;
    operator R() const { return R((*p)[I]...); }
    R get() const { return R((*p)[I]...); }
    swz& operator=(const R& v) {
        int k = 0;
        ((((*p)[I] = v[k]), ++k), ...);
        return *this;
    }
    swz& operator+=(const R& v) { return *this = get() + v; }
    swz& operator-=(const R& v) { return *this = get() - v; }
    swz& operator*=(const R& v) { return *this = get() * v; }
    swz& operator/=(const R& v) { return *this = get() / v; }
    swz& operator*=(typename R::value_type s) { return *this = get() * s; }
    swz& operator/=(typename R::value_type s) { return *this = get() / s; }
    typename R::value_type operator[](int i) const { return get()[i]; }
};

#define GLSL_VEC_COMMON(N)                                                                  \
    typedef T value_type;                                                                  \
    T& operator[](int i) { return d_[i]; }                                                 \
    const T& operator[](int i) const { return d_[i]; }                                     \
    friend tvec##N operator+(const tvec##N& a, const tvec##N& b) { tvec##N r; for (int i = 0; i < N; i++) r.d_[i] = a.d_[i] + b.d_[i]; return r; } \
    friend tvec##N operator-(const tvec##N& a, const tvec##N& b) { tvec##N r; for (int i = 0; i < N; i++) r.d_[i] = a.d_[i] - b.d_[i]; return r; } \
    friend tvec##N operator*(const tvec##N& a, const tvec##N& b) { tvec##N r; for (int i = 0; i < N; i++) r.d_[i] = a.d_[i] * b.d_[i]; return r; } \
    friend tvec##N operator/(const tvec##N& a, const tvec##N& b) { tvec##N r; for (int i = 0; i < N; i++) r.d_[i] = a.d_[i] / b.d_[i]; return r; } \
    friend tvec##N operator+(const tvec##N& a, T b) { tvec##N r; for (int i = 0; i < N; i++) r.d_[i] = a.d_[i] + b; return r; } \
    friend tvec##N operator-(const tvec##N& a, T b) { tvec##N r; for (int i = 0; i < N; i++) r.d_[i] = a.d_[i] - b; return r; } \
    friend tvec##N operator*(const tvec##N& a, T b) { tvec##N r; for (int i = 0; i < N; i++) r.d_[i] = a.d_[i] * b; return r; } \
    friend tvec##N operator/(const tvec##N& a, T b) { tvec##N r; for (int i = 0; i < N; i++) r.d_[i] = a.d_[i] / b; return r; } \
    friend tvec##N operator+(T a, const tvec##N& b) { tvec##N r; for (int i = 0; i < N; i++) r.d_[i] = a + b.d_[i]; return r; } \
    friend tvec##N operator-(T a, const tvec##N& b) { tvec##N r; for (int i = 0; i < N; i++) r.d_[i] = a - b.d_[i]; return r; } \
    friend tvec##N operator*(T a, const tvec##N& b) { tvec##N r; for (int i = 0; i < N; i++) r.d_[i] = a * b.d_[i]; return r; } \
    friend tvec##N operator/(T a, const tvec##N& b) { tvec##N r; for (int i = 0; i < N; i++) r.d_[i] = a / b.d_[i]; return r; } \
    friend tvec##N operator-(const tvec##N& a) { tvec##N r; for (int i = 0; i < N; i++) r.d_[i] = -a.d_[i]; return r; } \
    friend tvec##N operator>>(const tvec##N& a, T b) { tvec##N r; for (int i = 0; i < N; i++) r.d_[i] = a.d_[i] >> b; return r; } \
    friend tvec##N operator<<(const tvec##N& a, T b) { tvec##N r; for (int i = 0; i < N; i++) r.d_[i] = a.d_[i] << b; return r; } \
    friend tvec##N operator^(const tvec##N& a, const tvec##N& b) { tvec##N r; for (int i = 0; i < N; i++) r.d_[i] = a.d_[i] ^ b.d_[i]; return r; } \
    friend tvec##N operator&(const tvec##N& a, T b) { tvec##N r; for (int i = 0; i < N; i++) r.d_[i] = a.d_[i] & b; return r; } \
    tvec##N& operator+=(const tvec##N& b) { return *this = *this + b; }                  \
    tvec##N& operator-=(const tvec##N& b) { return *this = *this - b; }                  \
    tvec##N& operator*=(const tvec##N& b) { return *this = *this * b; }                  \
    tvec##N& operator/=(const tvec##N& b) { return *this = *this / b; }                  \
    tvec##N& operator+=(T b) { return *this = *this + b; }                               \
    tvec##N& operator-=(T b) { return *this = *this - b; }                               \
    tvec##N& operator*=(T b) { return *this = *this * b; }                               \
    tvec##N& operator/=(T b) { return *this = *this / b; }                               \
    tvec##N& operator^=(const tvec##N& b) { return *this = *this ^ b; }                  \
    tvec##N& operator>>=(T b) { return *this = *this >> b; }

template <class T> struct tvec2 {
    union {
        struct { T x, y; };
        struct { T r, g; };
        T d_[2];
    };
    tvec2() : x(0), y(0) {}
    explicit tvec2(T s) : x(s), y(s) {}
    tvec2(T a, T b) : x(a), y(b) {}
    template <class U> explicit tvec2(const tvec2<U>& o) : x(T(o.x)), y(T(o.y)) {}
    template <class U> explicit tvec2(const tvec3<U>& o) : x(T(o.x)), y(T(o.y)) {}
    template <class V, class R, int... I> explicit tvec2(const swz<V, R, I...>& s) : tvec2(s.get()) {}
    tvec2(const tvec2& o) { x = o.x; y = o.y; }
    tvec2& operator=(const tvec2& o) { x = o.x; y = o.y; return *this; }
    GLSL_VEC_COMMON(2)
};

template <class T> struct tvec3 {
    union {
        struct { T x, y, z; };
        struct { T r, g, b; };
        T d_[3];
    };
    tvec3() : x(0), y(0), z(0) {}
    explicit tvec3(T s) : x(s), y(s), z(s) {}
    tvec3(T a, T b, T c) : x(a), y(b), z(c) {}
    tvec3(const tvec2<T>& v, T c) : x(v.x), y(v.y), z(c) {}
    tvec3(T a, const tvec2<T>& v) : x(a), y(v.x), z(v.y) {}
    template <class U> explicit tvec3(const tvec3<U>& o) : x(T(o.x)), y(T(o.y)), z(T(o.z)) {}
    template <class U> explicit tvec3(const tvec4<U>& o) : x(T(o.x)), y(T(o.y)), z(T(o.z)) {}
    template <class V, class R, int... I> explicit tvec3(const swz<V, R, I...>& s) : tvec3(s.get()) {}
    tvec3(const tvec3& o) { x = o.x; y = o.y; z = o.z; }
    tvec3& operator=(const tvec3& o) { x = o.x; y = o.y; z = o.z; return *this; }
    swz<tvec3, tvec2<T>, 0, 1> xy_() { return {this}; }
    swz<tvec3, tvec2<T>, 1, 2> yz_() { return {this}; }
    swz<tvec3, tvec2<T>, 0, 1> rg_() { return {this}; }
    swz<tvec3, tvec3<T>, 0, 1, 2> xyz_() { return {this}; }
    swz<tvec3, tvec3<T>, 0, 1, 2> rgb_() { return {this}; }
    tvec2<T> xy_() const { return tvec2<T>(x, y); }
    tvec2<T> yz_() const { return tvec2<T>(y, z); }
    tvec2<T> rg_() const { return tvec2<T>(x, y); }
    tvec3<T> xyz_() const { return *this; }
    tvec3<T> rgb_() const { return *this; }
    GLSL_VEC_COMMON(3)
};

template <class T> struct tvec4 {
    union {
        struct { T x, y, z, w; };
        struct { T r, g, b, a; };
        T d_[4];
    };
    tvec4() : x(0), y(0), z(0), w(0) {}
    explicit tvec4(T s) : x(s), y(s), z(s), w(s) {}
    tvec4(T a0, T a1, T a2, T a3) : x(a0), y(a1), z(a2), w(a3) {}
    tvec4(const tvec3<T>& v, T c) : x(v.x), y(v.y), z(v.z), w(c) {}
    tvec4(const tvec2<T>& v, T c, T e) : x(v.x), y(v.y), z(c), w(e) {}
    tvec4(const tvec2<T>& v, const tvec2<T>& q) : x(v.x), y(v.y), z(q.x), w(q.y) {}
    template <class U> explicit tvec4(const tvec4<U>& o) : x(T(o.x)), y(T(o.y)), z(T(o.z)), w(T(o.w)) {}
    template <class V, class R, int... I> explicit tvec4(const swz<V, R, I...>& s) : tvec4(s.get()) {}
    tvec4(const tvec4& o) { x = o.x; y = o.y; z = o.z; w = o.w; }
    tvec4& operator=(const tvec4& o) { x = o.x; y = o.y; z = o.z; w = o.w; return *this; }
    swz<tvec4, tvec2<T>, 0, 1> xy_() { return {this}; }
    swz<tvec4, tvec2<T>, 1, 2> yz_() { return {this}; }
    swz<tvec4, tvec2<T>, 2, 3> zw_() { return {this}; }
    swz<tvec4, tvec2<T>, 0, 1> rg_() { return {this}; }
    swz<tvec4, tvec3<T>, 0, 1, 2> xyz_() { return {this}; }
    swz<tvec4, tvec3<T>, 0, 1, 2> rgb_() { return {this}; }
    tvec2<T> xy_() const { return tvec2<T>(x, y); }
    tvec2<T> yz_() const { return tvec2<T>(y, z); }
    tvec2<T> zw_() const { return tvec2<T>(z, w); }
    tvec2<T> rg_() const { return tvec2<T>(x, y); }
    tvec3<T> xyz_() const { return tvec3<T>(x, y, z); }
    tvec3<T> rgb_() const { return tvec3<T>(x, y, z); }
    GLSL_VEC_COMMON(4)
};
#undef GLSL_VEC_COMMON

typedef tvec2<float> vec2;
typedef tvec3<float> vec3;
typedef tvec4<float> vec4;
typedef tvec2<int> ivec2;
typedef tvec3<int> ivec3;
typedef tvec4<int> ivec4;
typedef tvec2<uint> uvec2;
typedef tvec3<uint> uvec3;
typedef tvec4<uint> uvec4;

struct bvec2 { bool x, y; };
struct bvec3 { bool x, y, z; };
inline bool any(bvec2 b) { return b.x || b.y; }
inline bool any(bvec3 b) { return b.x || b.y || b.z; }
inline bool all(bvec3 b) { return b.x && b.y && b.z; }

// ------------------------------------------------------ component-wise functions
#define GLSL_F1(name)                                                                      \
    inline vec2 name(const vec2& v) { return vec2(name(v.x), name(v.y)); }                \
    inline vec3 name(const vec3& v) { return vec3(name(v.x), name(v.y), name(v.z)); }     \
    inline vec4 name(const vec4& v) { return vec4(name(v.x), name(v.y), name(v.z), name(v.w)); }
GLSL_F1(abs) GLSL_F1(floor) GLSL_F1(ceil) GLSL_F1(fract) GLSL_F1(round) GLSL_F1(roundEven)
GLSL_F1(sqrt) GLSL_F1(exp) GLSL_F1(exp2) GLSL_F1(log) GLSL_F1(log2) GLSL_F1(sin) GLSL_F1(cos)
GLSL_F1(sign)
#undef GLSL_F1

#define GLSL_F2(name, V, S)                                                                \
    inline V name(const V& a, const V& b) { V r; for (int i = 0; i < (int)(sizeof(V) / sizeof(S)); i++) r[i] = name(a[i], b[i]); return r; } \
    inline V name(const V& a, S b) { V r; for (int i = 0; i < (int)(sizeof(V) / sizeof(S)); i++) r[i] = name(a[i], b); return r; }
GLSL_F2(min, vec2, float) GLSL_F2(min, vec3, float) GLSL_F2(min, vec4, float)
GLSL_F2(max, vec2, float) GLSL_F2(max, vec3, float) GLSL_F2(max, vec4, float)
GLSL_F2(min, ivec2, int) GLSL_F2(min, ivec3, int) GLSL_F2(max, ivec2, int) GLSL_F2(max, ivec3, int)
GLSL_F2(pow, vec2, float) GLSL_F2(pow, vec3, float) GLSL_F2(pow, vec4, float)
GLSL_F2(mod, vec3, float)
#undef GLSL_F2

#define GLSL_CLAMP(V, S)                                                                   \
    inline V clamp(const V& x, const V& lo, const V& hi) { return min(max(x, lo), hi); }  \
    inline V clamp(const V& x, S lo, S hi) { return min(max(x, lo), hi); }
GLSL_CLAMP(vec2, float) GLSL_CLAMP(vec3, float) GLSL_CLAMP(vec4, float)
GLSL_CLAMP(ivec2, int) GLSL_CLAMP(ivec3, int)
#undef GLSL_CLAMP

#define GLSL_MIX(V)                                                                        \
    inline V mix(const V& x, const V& y, float a) { return x * (1.0f - a) + y * a; }      \
    inline V mix(const V& x, const V& y, const V& a) { return x * (1.0f - a) + y * a; }
GLSL_MIX(vec2) GLSL_MIX(vec3) GLSL_MIX(vec4)
#undef GLSL_MIX
inline vec3 mix(const vec3& x, const vec3& y, bvec3 a) {
    return vec3(a.x ? y.x : x.x, a.y ? y.y : x.y, a.z ? y.z : x.z);
}
inline vec3 step(float edge, const vec3& x) { return vec3(step(edge, x.x), step(edge, x.y), step(edge, x.z)); }
inline vec3 step(const vec3& edge, const vec3& x) { return vec3(step(edge.x, x.x), step(edge.y, x.y), step(edge.z, x.z)); }
inline vec3 smoothstep(float e0, float e1, const vec3& x) {
    return vec3(smoothstep(e0, e1, x.x), smoothstep(e0, e1, x.y), smoothstep(e0, e1, x.z));
}

inline float dot(const vec2& a, const vec2& b) { return a.x * b.x + a.y * b.y; }
inline float dot(const vec3& a, const vec3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float dot(const vec4& a, const vec4& b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
inline vec3 cross(const vec3& a, const vec3& b) {
    return vec3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
inline float length(float x) { return abs(x); }
inline float length(const vec2& v) { return sqrt(dot(v, v)); }
inline float length(const vec3& v) { return sqrt(dot(v, v)); }
inline float length(const vec4& v) { return sqrt(dot(v, v)); }
inline float distance(const vec3& a, const vec3& b) { return length(a - b); }
inline vec2 normalize(const vec2& v) { return v / length(v); }
inline vec3 normalize(const vec3& v) { return v / length(v); }
inline vec3 reflect(const vec3& i, const vec3& n) { return i - 2.0f * dot(n, i) * n; }

inline bvec3 equal(const vec3& a, const vec3& b) { return {a.x == b.x, a.y == b.y, a.z == b.z}; }
inline bvec2 lessThan(const ivec2& a, const ivec2& b) { return {a.x < b.x, a.y < b.y}; }
inline bvec3 lessThan(const ivec3& a, const ivec3& b) { return {a.x < b.x, a.y < b.y, a.z < b.z}; }
inline bvec2 greaterThanEqual(const ivec2& a, const ivec2& b) { return {a.x >= b.x, a.y >= b.y}; }
inline bvec3 greaterThanEqual(const ivec3& a, const ivec3& b) { return {a.x >= b.x, a.y >= b.y, a.z >= b.z}; }
inline bvec2 greaterThanEqual(const uvec2& a, const uvec2& b) { return {a.x >= b.x, a.y >= b.y}; }
inline bvec3 greaterThanEqual(const uvec3& a, const uvec3& b) { return {a.x >= b.x, a.y >= b.y, a.z >= b.z}; }

// ------------------------------------------------------------------- matrices
// Column-major, as in GLSL: m[c] is column c.
struct mat3 {
    vec3 c[3];
    mat3() { c[0] = vec3(1, 0, 0); c[1] = vec3(0, 1, 0); c[2] = vec3(0, 0, 1); }
    explicit mat3(float s) { c[0] = vec3(s, 0, 0); c[1] = vec3(0, s, 0); c[2] = vec3(0, 0, s); }
    mat3(const vec3& a, const vec3& b, const vec3& d) { c[0] = a; c[1] = b; c[2] = d; }
    mat3(float a0, float a1, float a2, float b0, float b1, float b2, float d0, float d1, float d2) {
        c[0] = vec3(a0, a1, a2); c[1] = vec3(b0, b1, b2); c[2] = vec3(d0, d1, d2);
    }
    explicit mat3(const struct mat4& m);
    vec3& operator[](int i) { return c[i]; }
    const vec3& operator[](int i) const { return c[i]; }
};
struct mat4 {
    vec4 c[4];
    vec4& operator[](int i) { return c[i]; }
    const vec4& operator[](int i) const { return c[i]; }
};
inline mat3::mat3(const mat4& m) {
    for (int i = 0; i < 3; i++) c[i] = vec3(m.c[i].x, m.c[i].y, m.c[i].z);
}
inline vec3 operator*(const mat3& m, const vec3& v) {
    return m.c[0] * v.x + m.c[1] * v.y + m.c[2] * v.z;
}
inline vec4 operator*(const mat4& m, const vec4& v) {
    return m.c[0] * v.x + m.c[1] * v.y + m.c[2] * v.z + m.c[3] * v.w;
}
inline mat3 transpose(const mat3& m) {
    return mat3(m.c[0].x, m.c[1].x, m.c[2].x, m.c[0].y, m.c[1].y, m.c[2].y, m.c[0].z, m.c[1].z, m.c[2].z);
}
// Inverse by the adjugate over the determinant.
inline mat3 inverse(const mat3& m) {
    float a00 = m.c[0].x, a01 = m.c[0].y, a02 = m.c[0].z;
    float a10 = m.c[1].x, a11 = m.c[1].y, a12 = m.c[1].z;
    float a20 = m.c[2].x, a21 = m.c[2].y, a22 = m.c[2].z;
    float b01 = a22 * a11 - a12 * a21;
    float b11 = -a22 * a10 + a12 * a20;
    float b21 = a21 * a10 - a11 * a20;
    float det = a00 * b01 + a01 * b11 + a02 * b21;
    return mat3(b01 / det, (-a22 * a01 + a02 * a21) / det, (a12 * a01 - a02 * a11) / det,
                b11 / det, (a22 * a00 - a02 * a20) / det, (-a12 * a00 + a02 * a10) / det,
                b21 / det, (-a21 * a00 + a01 * a20) / det, (a11 * a00 - a01 * a10) / det);
}

// ------------------------------------------------------- texel formats and units
enum Format : int {
    R16_UNORM, RG16_UNORM, RGBA8_SNORM, RGBA8_UNORM, R32F, RG32F, RGBA32F, RGBA16F, R16F,
    R8_UINT, RGBA8_UINT,
    R16_BF16,  // appended: the values above are part of the reference harness's interface (oracle/ref.py)
    RG16F, RG16_BF16  // the precision variant's label mask (two binary16 / bfloat16 channels)
};
inline int format_bytes(Format f) {
    switch (f) {
        case R16_UNORM: case R16F: case R16_BF16: return 2;
        case RG16_UNORM: case RGBA8_SNORM: case RGBA8_UNORM: case R32F: case RGBA8_UINT: case RG16F:
        case RG16_BF16: return 4;
        case RG32F: case RGBA16F: return 8;
        case RGBA32F: return 16;
        case R8_UINT: return 1;
    }
    return 0;
}
inline float half_to_float(uint16_t h) { _Float16 v; std::memcpy(&v, &h, 2); return (float)v; }
inline uint16_t float_to_half(float f) { _Float16 v = (_Float16)f; uint16_t h; std::memcpy(&h, &v, 2); return h; }
// bfloat16: the upper half of a binary32; rounding to nearest even (finite values).
inline float bf16_to_float(uint16_t v) { uint32_t w = (uint32_t)v << 16; f32 x; std::memcpy(&x, &w, 4); return x; }
inline uint16_t float_to_bf16(float f) {
    f32 x = (f32)f; uint32_t w; std::memcpy(&w, &x, 4);
    return (uint16_t)((w + 0x7fffu + ((w >> 16) & 1u)) >> 16);
}

// Decodes texel `i` (linear index) of `data` in format `f` to floats.
inline vec4 decode(const void* data, Format f, long i) {
    const uint8_t* b = (const uint8_t*)data + i * format_bytes(f);
    switch (f) {
        case R16_UNORM: { uint16_t v; std::memcpy(&v, b, 2); return vec4(float(v) / 65535.0f, 0, 0, 1); }
        case RG16_UNORM: { uint16_t v[2]; std::memcpy(v, b, 4); return vec4(float(v[0]) / 65535.0f, float(v[1]) / 65535.0f, 0, 1); }
        case RGBA8_SNORM: { int8_t v[4]; std::memcpy(v, b, 4); vec4 r; for (int k = 0; k < 4; k++) r[k] = max(float(v[k]) / 127.0f, -1.0f); return r; }
        case RGBA8_UNORM: { vec4 r; for (int k = 0; k < 4; k++) r[k] = float(b[k]) / 255.0f; return r; }
        case R32F: { f32 v; std::memcpy(&v, b, 4); return vec4(v, 0, 0, 1); }
        case RG32F: { f32 v[2]; std::memcpy(v, b, 8); return vec4(v[0], v[1], 0, 1); }
        case RGBA32F: { f32 v[4]; std::memcpy(v, b, 16); return vec4(v[0], v[1], v[2], v[3]); }
        case RGBA16F: { uint16_t v[4]; std::memcpy(v, b, 8); return vec4(half_to_float(v[0]), half_to_float(v[1]), half_to_float(v[2]), half_to_float(v[3])); }
        case R16F: { uint16_t v; std::memcpy(&v, b, 2); return vec4(half_to_float(v), 0, 0, 1); }
        case R16_BF16: {  // the upper half of a binary32 (not a Vulkan format: the precision variant's density)
            uint16_t v; std::memcpy(&v, b, 2);
            uint32_t w = (uint32_t)v << 16; f32 x; std::memcpy(&x, &w, 4);
            return vec4(x, 0, 0, 1);
        }
        case R8_UINT: return vec4(float(b[0]), 0, 0, 1);
        case RGBA8_UINT: return vec4(float(b[0]), float(b[1]), float(b[2]), float(b[3]));
        case RG16F: { uint16_t v[2]; std::memcpy(v, b, 4); return vec4(half_to_float(v[0]), half_to_float(v[1]), 0, 1); }
        case RG16_BF16: { uint16_t v[2]; std::memcpy(v, b, 4); return vec4(bf16_to_float(v[0]), bf16_to_float(v[1]), 0, 1); }
    }
    return vec4(0.0f);
}
inline uint16_t to_unorm16(float f) { return (uint16_t)gl_rint(clamp(f, 0.0f, 1.0f) * 65535.0f); }
inline uint8_t to_unorm8(float f) { return (uint8_t)gl_rint(clamp(f, 0.0f, 1.0f) * 255.0f); }
inline int8_t to_snorm8(float f) { return (int8_t)gl_rint(clamp(f, -1.0f, 1.0f) * 127.0f); }

// Encodes `v` into texel `i` of `data` (the conversions of imageStore).
inline void encode(void* data, Format f, long i, const vec4& v) {
    uint8_t* b = (uint8_t*)data + i * format_bytes(f);
    switch (f) {
        case R16_UNORM: { uint16_t q = to_unorm16(v.x); std::memcpy(b, &q, 2); break; }
        case RG16_UNORM: { uint16_t q[2] = {to_unorm16(v.x), to_unorm16(v.y)}; std::memcpy(b, q, 4); break; }
        case RGBA8_SNORM: { int8_t q[4]; for (int k = 0; k < 4; k++) q[k] = to_snorm8(v[k]); std::memcpy(b, q, 4); break; }
        case RGBA8_UNORM: { for (int k = 0; k < 4; k++) b[k] = to_unorm8(v[k]); break; }
        case R32F: { f32 q = (f32)v.x; std::memcpy(b, &q, 4); break; }
        case RG32F: { f32 q[2] = {(f32)v.x, (f32)v.y}; std::memcpy(b, q, 8); break; }
        case RGBA32F: { f32 q[4] = {(f32)v.x, (f32)v.y, (f32)v.z, (f32)v.w}; std::memcpy(b, q, 16); break; }
        case RGBA16F: { uint16_t q[4]; for (int k = 0; k < 4; k++) q[k] = float_to_half(v[k]); std::memcpy(b, q, 8); break; }
        case R16F: { uint16_t q = float_to_half(v.x); std::memcpy(b, &q, 2); break; }
        case R16_BF16: {  // round to nearest even (finite values)
            f32 x = (f32)v.x; uint32_t w; std::memcpy(&w, &x, 4);
            uint16_t q = (uint16_t)((w + 0x7fffu + ((w >> 16) & 1u)) >> 16); std::memcpy(b, &q, 2); break;
        }
        case R8_UINT: b[0] = (uint8_t)v.x; break;
        case RGBA8_UINT: for (int k = 0; k < 4; k++) b[k] = (uint8_t)v[k]; break;
        case RG16F: { uint16_t q[2] = {float_to_half(v.x), float_to_half(v.y)}; std::memcpy(b, q, 4); break; }
        case RG16_BF16: { uint16_t q[2] = {float_to_bf16(v.x), float_to_bf16(v.y)}; std::memcpy(b, q, 4); break; }
    }
}

enum Filter : int { NEAREST = 0, LINEAR = 1 };
enum Address : int { CLAMP_TO_EDGE = 0, CLAMP_TO_BORDER_WHITE = 1 };

// A bound texture: data in x-fastest order, its size, format and sampler state.
struct Texture {
    const void* data = nullptr;
    Format format = R32F;
    int w = 1, h = 1, d = 1;
    Filter filter = LINEAR;
    Address address = CLAMP_TO_EDGE;
    vec4 texel(int x, int y, int z) const {
        if (address == CLAMP_TO_BORDER_WHITE && (x < 0 || y < 0 || z < 0 || x >= w || y >= h || z >= d))
            return vec4(1.0f);
        x = clamp(x, 0, w - 1);
        y = clamp(y, 0, h - 1);
        z = clamp(z, 0, d - 1);
        return decode(data, format, ((long)z * h + y) * w + x);
    }
};
struct sampler1D : Texture {};
struct sampler2D : Texture {};
struct sampler3D : Texture {};
struct usampler3D : Texture {};

// Linear filtering in one axis: texel coordinate u = tc * size - 0.5, taps at
// floor(u) and floor(u) + 1 with weights 1 - frac and frac.
inline vec4 sample_linear(const Texture& t, vec3 tc, int dims) {
    float u = tc.x * float(t.w) - 0.5f;
    float v = dims > 1 ? tc.y * float(t.h) - 0.5f : 0.0f;
    float q = dims > 2 ? tc.z * float(t.d) - 0.5f : 0.0f;
    int i0 = (int)floor(u), j0 = (int)floor(v), k0 = (int)floor(q);
    float a = u - float(i0), b = v - float(j0), c = q - float(k0);
    if (dims < 2) { b = 0.0f; j0 = 0; }
    if (dims < 3) { c = 0.0f; k0 = 0; }
    vec4 r(0.0f);
    for (int dk = 0; dk < (dims > 2 ? 2 : 1); dk++)
        for (int dj = 0; dj < (dims > 1 ? 2 : 1); dj++)
            for (int di = 0; di < 2; di++) {
                float wgt = (di ? a : 1.0f - a) * (dims > 1 ? (dj ? b : 1.0f - b) : 1.0f) *
                            (dims > 2 ? (dk ? c : 1.0f - c) : 1.0f);
                r += t.texel(i0 + di, j0 + dj, k0 + dk) * wgt;
            }
    return r;
}
inline vec4 sample_nearest(const Texture& t, vec3 tc) {
    int i = (int)floor(tc.x * float(t.w));
    int j = (int)floor(tc.y * float(t.h));
    int k = (int)floor(tc.z * float(t.d));
    return t.texel(i, j, k);
}
inline vec4 textureLod(const sampler3D& t, vec3 tc, float) {
    return t.filter == LINEAR ? sample_linear(t, tc, 3) : sample_nearest(t, tc);
}
inline vec4 textureLod(const sampler2D& t, vec2 tc, float) {
    return t.filter == LINEAR ? sample_linear(t, vec3(tc, 0.5f), 2) : sample_nearest(t, vec3(tc, 0.5f));
}
inline vec4 textureLod(const sampler1D& t, float tc, float) {
    return t.filter == LINEAR ? sample_linear(t, vec3(tc, 0.5f, 0.5f), 1) : sample_nearest(t, vec3(tc, 0.5f, 0.5f));
}
inline vec4 texelFetch(const sampler3D& t, ivec3 p, int) { return t.texel(p.x, p.y, p.z); }
inline vec4 texelFetch(const sampler2D& t, ivec2 p, int) { return t.texel(p.x, p.y, 0); }
inline vec4 texelFetch(const sampler1D& t, int p, int) { return t.texel(p, 0, 0); }
inline uvec4 texelFetch(const usampler3D& t, ivec3 p, int) { return uvec4(t.texel(p.x, p.y, p.z)); }
inline ivec3 textureSize(const sampler3D& t, int) { return ivec3(t.w, t.h, t.d); }
inline ivec3 textureSize(const usampler3D& t, int) { return ivec3(t.w, t.h, t.d); }
inline ivec2 textureSize(const sampler2D& t, int) { return ivec2(t.w, t.h); }
inline int textureSize(const sampler1D& t, int) { return t.w; }

// A storage image: loads decode, stores convert (see encode).
struct Image {
    void* data = nullptr;
    Format format = RGBA32F;
    int w = 1, h = 1, d = 1;
};
struct image2D : Image {};
struct image3D : Image {};
inline vec4 imageLoad(const image2D& im, ivec2 p) { return decode(im.data, im.format, (long)p.y * im.w + p.x); }
inline vec4 imageLoad(const image3D& im, ivec3 p) { return decode(im.data, im.format, ((long)p.z * im.h + p.y) * im.w + p.x); }
inline void imageStore(image2D& im, ivec2 p, vec4 v) { encode(im.data, im.format, (long)p.y * im.w + p.x, v); }
inline void imageStore(image3D& im, ivec3 p, vec4 v) { encode(im.data, im.format, ((long)p.z * im.h + p.y) * im.w + p.x, v); }
inline ivec2 imageSize(const image2D& im) { return ivec2(im.w, im.h); }
inline ivec3 imageSize(const image3D& im) { return ivec3(im.w, im.h, im.d); }

}  // namespace glsl

// Multi-letter swizzles.
#define xyz xyz_()
#define rgb rgb_()
#define xy xy_()
#define yz yz_()
#define zw zw_()
#define rg rg_()

// Using-declarations of every GLSL name, for code in its own namespace (so that
// unqualified calls resolve here and never to the C library's overloads).
#define GLSL_USING                                                                          \
    using glsl::uint; using glsl::vec2; using glsl::vec3; using glsl::vec4; using glsl::ivec2; \
    using glsl::ivec3; using glsl::ivec4; using glsl::uvec2; using glsl::uvec3; using glsl::uvec4; \
    using glsl::bvec2; using glsl::bvec3; using glsl::mat3; using glsl::mat4; using glsl::abs;   \
    using glsl::sign; using glsl::floor; using glsl::ceil; using glsl::trunc; using glsl::fract;  \
    using glsl::round; using glsl::roundEven; using glsl::mod; using glsl::min; using glsl::max; \
    using glsl::clamp; using glsl::mix; using glsl::step; using glsl::smoothstep; using glsl::sqrt; \
    using glsl::inversesqrt; using glsl::pow; using glsl::exp; using glsl::exp2; using glsl::log; \
    using glsl::log2; using glsl::sin; using glsl::cos; using glsl::tan; using glsl::asin;       \
    using glsl::acos; using glsl::atan; using glsl::radians; using glsl::dot; using glsl::cross; \
    using glsl::length; using glsl::distance; using glsl::normalize; using glsl::reflect;        \
    using glsl::equal; using glsl::lessThan; using glsl::greaterThanEqual; using glsl::any;      \
    using glsl::all; using glsl::transpose; using glsl::inverse; using glsl::sampler1D;          \
    using glsl::sampler2D; using glsl::sampler3D; using glsl::usampler3D; using glsl::image2D;   \
    using glsl::image3D; using glsl::textureLod; using glsl::texelFetch; using glsl::textureSize; \
    using glsl::imageLoad; using glsl::imageStore; using glsl::imageSize;
