/*
 * glsl_compat.hpp — the subset of GLSL 4.50 that igx_raytracing's
 * res/shaders/primitive.glsl and res/shaders/trace.glsl use, written as C++
 * so those shader sources compile on the host unchanged apart from one
 * mechanical rewrite of the `inout` parameter qualifier (done by the recipe
 * in oracle/Makefile).
 *
 * TEST INFRASTRUCTURE ONLY: it builds the reference's own traversal as a
 * host library that pins the oracle restatement.
 *
 * Semantics chosen for the builtins (GLSL leaves their precision open):
 * binary32, no FMA contraction (compile with -ffp-contract=off), dot summed
 * left to right, cross in the component order of the GLSL specification,
 * normalize(x) = x / sqrt(dot(x, x)), min/max as the specification's
 * `y < x ? y : x` / `x < y ? y : x`.
 */
#ifndef IGXRT_GLSL_COMPAT_HPP
#define IGXRT_GLSL_COMPAT_HPP

#include <stdint.h>
#include <string.h>

typedef unsigned int uint;

struct vec2;
struct vec3;
struct vec4;
struct uvec2;
struct uvec3;

/* Read-only swizzle views living in the same storage as the vector. */
template <int N, int A, int B>
struct swz2 {
    float v[N];
    inline operator vec2() const;
};
template <int N, int A, int B, int C>
struct swz3 {
    float v[N];
    inline operator vec3() const;
};
template <int N, int A, int B>
struct uswz2 {
    uint v[N];
    inline operator uvec2() const;
};

struct vec2 {
    union {
        struct { float x, y; };
        struct { float r, g; };
    };
    vec2() : x(0), y(0) {}
    vec2(float a, float b) : x(a), y(b) {}
    explicit vec2(float s) : x(s), y(s) {}
    explicit vec2(const uvec2& u);
};

struct vec3 {
    union {
        struct { float x, y, z; };
        struct { float r, g, b; };
        swz2<3, 0, 1> xy;
        swz2<3, 1, 2> yz;
        swz2<3, 0, 2> xz;
        swz2<3, 0, 1> rg;
    };
    vec3() : x(0), y(0), z(0) {}
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    explicit vec3(float s) : x(s), y(s), z(s) {}
    vec3(const vec2& a, float c) : x(a.x), y(a.y), z(c) {}
    vec3(float a, const vec2& bc) : x(a), y(bc.x), z(bc.y) {}
    explicit vec3(const uvec3& u);
};

struct vec4 {
    union {
        struct { float x, y, z, w; };
        struct { float r, g, b, a; };
        swz3<4, 0, 1, 2> xyz;
        swz2<4, 0, 1> rg;
        swz2<4, 2, 3> ba;
        swz2<4, 0, 1> xy;
    };
    vec4() : x(0), y(0), z(0), w(0) {}
    vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    explicit vec4(float s) : x(s), y(s), z(s), w(s) {}
    vec4(const vec3& a, float d) : x(a.x), y(a.y), z(a.z), w(d) {}
    vec4(const vec2& a, const vec2& b) : x(a.x), y(a.y), z(b.x), w(b.y) {}
};

struct uvec2 {
    union {
        struct { uint x, y; };
        struct { uint r, g; };
    };
    uvec2() : x(0), y(0) {}
    uvec2(uint a, uint b) : x(a), y(b) {}
    explicit uvec2(uint s) : x(s), y(s) {}
};

struct uvec3 {
    union {
        struct { uint x, y, z; };
        struct { uint r, g, b; };
    };
    uvec3() : x(0), y(0), z(0) {}
    uvec3(uint a, uint b, uint c) : x(a), y(b), z(c) {}
    explicit uvec3(const vec3& f) : x((uint)f.x), y((uint)f.y), z((uint)f.z) {}
};

inline vec2::vec2(const uvec2& u) : x((float)u.x), y((float)u.y) {}
inline vec3::vec3(const uvec3& u) : x((float)u.x), y((float)u.y), z((float)u.z) {}

template <int N, int A, int B>
inline swz2<N, A, B>::operator vec2() const { return vec2(v[A], v[B]); }
template <int N, int A, int B, int C>
inline swz3<N, A, B, C>::operator vec3() const { return vec3(v[A], v[B], v[C]); }
template <int N, int A, int B>
inline uswz2<N, A, B>::operator uvec2() const { return uvec2(v[A], v[B]); }

/* ---- float vector arithmetic (component-wise, binary32) ---------------- */

#define IGX_VEC_OPS(V, ...)                                                                   \
    inline V operator+(const V& a, const V& b) { V r; for (int i = 0; i < n_##V; ++i) (&r.x)[i] = (&a.x)[i] + (&b.x)[i]; return r; } \
    inline V operator-(const V& a, const V& b) { V r; for (int i = 0; i < n_##V; ++i) (&r.x)[i] = (&a.x)[i] - (&b.x)[i]; return r; } \
    inline V operator*(const V& a, const V& b) { V r; for (int i = 0; i < n_##V; ++i) (&r.x)[i] = (&a.x)[i] * (&b.x)[i]; return r; } \
    inline V operator/(const V& a, const V& b) { V r; for (int i = 0; i < n_##V; ++i) (&r.x)[i] = (&a.x)[i] / (&b.x)[i]; return r; } \
    inline V operator+(const V& a, float s) { V r; for (int i = 0; i < n_##V; ++i) (&r.x)[i] = (&a.x)[i] + s; return r; } \
    inline V operator-(const V& a, float s) { V r; for (int i = 0; i < n_##V; ++i) (&r.x)[i] = (&a.x)[i] - s; return r; } \
    inline V operator*(const V& a, float s) { V r; for (int i = 0; i < n_##V; ++i) (&r.x)[i] = (&a.x)[i] * s; return r; } \
    inline V operator/(const V& a, float s) { V r; for (int i = 0; i < n_##V; ++i) (&r.x)[i] = (&a.x)[i] / s; return r; } \
    inline V operator+(float s, const V& a) { V r; for (int i = 0; i < n_##V; ++i) (&r.x)[i] = s + (&a.x)[i]; return r; } \
    inline V operator-(float s, const V& a) { V r; for (int i = 0; i < n_##V; ++i) (&r.x)[i] = s - (&a.x)[i]; return r; } \
    inline V operator*(float s, const V& a) { V r; for (int i = 0; i < n_##V; ++i) (&r.x)[i] = s * (&a.x)[i]; return r; } \
    inline V operator/(float s, const V& a) { V r; for (int i = 0; i < n_##V; ++i) (&r.x)[i] = s / (&a.x)[i]; return r; } \
    inline V operator-(const V& a) { V r; for (int i = 0; i < n_##V; ++i) (&r.x)[i] = -(&a.x)[i]; return r; } \
    inline V& operator+=(V& a, const V& b) { a = a + b; return a; }                            \
    inline V& operator-=(V& a, const V& b) { a = a - b; return a; }                            \
    inline V& operator*=(V& a, const V& b) { a = a * b; return a; }                            \
    inline V& operator/=(V& a, const V& b) { a = a / b; return a; }                            \
    inline V& operator*=(V& a, float s) { a = a * s; return a; }                               \
    inline V& operator/=(V& a, float s) { a = a / s; return a; }                               \
    inline V min(const V& a, const V& b) { V r; for (int i = 0; i < n_##V; ++i) { float x = (&a.x)[i], y = (&b.x)[i]; (&r.x)[i] = y < x ? y : x; } return r; } \
    inline V max(const V& a, const V& b) { V r; for (int i = 0; i < n_##V; ++i) { float x = (&a.x)[i], y = (&b.x)[i]; (&r.x)[i] = x < y ? y : x; } return r; }

enum { n_vec2 = 2, n_vec3 = 3, n_vec4 = 4 };
IGX_VEC_OPS(vec2)
IGX_VEC_OPS(vec3)
IGX_VEC_OPS(vec4)
#undef IGX_VEC_OPS

/* ---- unsigned vectors ---------------------------------------------------- */

inline uvec3 operator&(const uvec3& a, uint m) { return uvec3(a.x & m, a.y & m, a.z & m); }
inline uvec3 operator>>(const uvec3& a, uint s) { return uvec3(a.x >> s, a.y >> s, a.z >> s); }
inline uvec2 operator&(const uvec2& a, uint m) { return uvec2(a.x & m, a.y & m); }
inline uvec2 operator>>(const uvec2& a, uint s) { return uvec2(a.x >> s, a.y >> s); }

/* ---- scalar builtins ------------------------------------------------------ */

inline float min(float x, float y) { return y < x ? y : x; }
inline float max(float x, float y) { return x < y ? y : x; }
inline float abs(float x) { return __builtin_fabsf(x); }
inline float sign(float x) { return x > 0 ? 1.0f : (x < 0 ? -1.0f : 0.0f); }
inline float sqrt(float x) { return __builtin_sqrtf(x); }
/* asin and atan: the GLSL specification leaves their precision to the
 * implementation.  They are fixed here as the correctly rounded binary32
 * values, evaluated in binary64 and rounded once (a host libm's binary32
 * asinf / atanf are not correctly rounded and differ between libraries), so
 * the sphere uv of primitive.glsl:198-204 has one exact answer. */
inline float asin(float x) { return (float)__builtin_asin((double)x); }
inline float atan(float y_over_x) { return (float)__builtin_atan((double)y_over_x); }
inline bool isnan(float x) { return x != x; }

/* ---- geometric builtins --------------------------------------------------- */

inline float dot(const vec2& a, const vec2& b) { return a.x * b.x + a.y * b.y; }
inline float dot(const vec3& a, const vec3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float dot(const vec4& a, const vec4& b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
inline vec3 cross(const vec3& a, const vec3& b) {
    return vec3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
inline float length(const vec3& a) { return sqrt(dot(a, a)); }
inline vec3 normalize(const vec3& a) { return a / length(a); }

/* ---- relational builtins -------------------------------------------------- */

struct bvec3 {
    bool x, y, z;
};
inline bvec3 equal(const vec3& a, const vec3& b) { return bvec3{a.x == b.x, a.y == b.y, a.z == b.z}; }
inline bool all(const bvec3& b) { return b.x && b.y && b.z; }

/* ---- packing builtins (exact) --------------------------------------------- */

inline float igx_half_to_float(uint h) {
    const uint sign = (h >> 15) & 1u, exp = (h >> 10) & 31u, man = h & 1023u;
    float mag;
    if (exp == 0)
        mag = (float)man * (1.0f / 16777216.0f); /* man * 2^-24 */
    else if (exp == 31)
        mag = man ? __builtin_nanf("") : __builtin_inff();
    else {
        uint bits = ((exp + 112u) << 23) | (man << 13);
        memcpy(&mag, &bits, 4);
    }
    return sign ? -mag : mag;
}

/* float -> half, round to nearest even (GLSL packHalf2x16). */
inline uint igx_float_to_half(float f) {
    uint x;
    memcpy(&x, &f, 4);
    const uint sign = (x >> 16) & 0x8000u;
    const uint absx = x & 0x7fffffffu;
    if (absx >= 0x7f800000u)
        return sign | 0x7c00u | (absx > 0x7f800000u ? 0x200u : 0u);
    if (absx >= 0x477ff000u) /* rounds to >= 65520: overflow to inf */
        return sign | 0x7c00u;
    if (absx < 0x38800000u) { /* below the smallest normal half */
        if (absx < 0x33000000u)
            return sign; /* < 2^-25: rounds to zero */
        const uint e = absx >> 23;
        const uint m = (absx & 0x7fffffu) | 0x800000u;
        const uint shift = 126u - e; /* 14 .. 24 */
        uint hm = m >> shift;
        const uint rem = m & ((1u << shift) - 1u), halfway = 1u << (shift - 1u);
        if (rem > halfway || (rem == halfway && (hm & 1u)))
            ++hm;
        return sign | hm;
    }
    uint h = ((absx >> 13) - (112u << 10));
    const uint rem = absx & 0x1fffu;
    if (rem > 0x1000u || (rem == 0x1000u && (h & 1u)))
        ++h;
    return sign | h;
}

inline vec2 unpackHalf2x16(uint v) { return vec2(igx_half_to_float(v & 0xffffu), igx_half_to_float(v >> 16)); }
inline uint packHalf2x16(const vec2& v) { return igx_float_to_half(v.x) | (igx_float_to_half(v.y) << 16); }

#endif
