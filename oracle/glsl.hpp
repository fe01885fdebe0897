// GLSL-semantics vector/matrix shim for the CPU oracle (test infrastructure only).
//
// The oracle restates the reference's GLSL 4.3 compute shaders in C++. This header gives
// those restatements the GLSL types and built-ins they use, with one fixed evaluation order so
// that an FP32 build (compiled with -ffp-contract=off, no fast-math) is bit-reproducible and can
// be compared word for word with the CUDA kernels:
//   * dot(a, b)      = ((a.x*b.x + a.y*b.y) + a.z*b.z) [+ a.w*b.w], left to right
//   * length(v)      = sqrt(dot(v, v))           (IEEE square root)
//   * normalize(v)   = v / length(v)             (GLSL spec definition, three IEEE divides)
//   * cross(a, b)    = (a.y*b.z - b.y*a.z, a.z*b.x - b.z*a.x, a.x*b.y - b.x*a.y)
//   * mat * vec      = col0*v.x + col1*v.y + col2*v.z [+ col3*v.w], summed left to right
//   * min(x, y)      = y < x ? y : x ; max(x, y) = x < y ? y : x   (GLSL spec wording)
// Scalar type T is float (reference precision) or double (the FP64 oracle).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

namespace glsl {

using uint = uint32_t;

template <class T> inline T gmin(T x, T y) { return y < x ? y : x; }
template <class T> inline T gmax(T x, T y) { return x < y ? y : x; }
template <class T> inline T gclamp(T x, T lo, T hi) { return gmin(gmax(x, lo), hi); }
template <class T> inline T gsign(T x) { return x > T(0) ? T(1) : (x < T(0) ? T(-1) : T(0)); }
template <class T> inline T smoothstep(T e0, T e1, T x) {
    T t = gclamp((x - e0) / (e1 - e0), T(0), T(1));
    return t * t * (T(3) - T(2) * t);
}

// float -> uint conversion with the GPU's saturating semantics (NaN -> 0). C++ leaves
// out-of-range conversions undefined; the CUDA kernels use cvt.rzi.u32 which saturates.
template <class T> inline uint to_uint(T x) {
    if (!(x > T(0))) return 0u;
    if (x >= T(4294967296.0)) return 0xFFFFFFFFu;
    return (uint)x;
}
// float -> int conversion, truncation toward zero, saturating (cvt.rzi.s32).
template <class T> inline int32_t to_int(T x) {
    if (x != x) return 0;
    if (x >= T(2147483648.0)) return INT32_MAX;
    if (x <= T(-2147483648.0)) return INT32_MIN;
    return (int32_t)x;
}

inline uint floatBitsToUint(float f) { uint u; std::memcpy(&u, &f, 4); return u; }
inline float uintBitsToFloat(uint u) { float f; std::memcpy(&f, &u, 4); return f; }

template <class T> struct tvec2 {
    T x, y;
    tvec2() : x(0), y(0) {}
    tvec2(T a, T b) : x(a), y(b) {}
    explicit tvec2(T s) : x(s), y(s) {}
    template <class U> explicit tvec2(const tvec2<U>& o) : x(T(o.x)), y(T(o.y)) {}
};
template <class T> struct tvec3 {
    T x, y, z;
    tvec3() : x(0), y(0), z(0) {}
    tvec3(T a, T b, T c) : x(a), y(b), z(c) {}
    explicit tvec3(T s) : x(s), y(s), z(s) {}
    template <class U> explicit tvec3(const tvec3<U>& o) : x(T(o.x)), y(T(o.y)), z(T(o.z)) {}
};
template <class T> struct tvec4 {
    T x, y, z, w;
    tvec4() : x(0), y(0), z(0), w(0) {}
    tvec4(T a, T b, T c, T d) : x(a), y(b), z(c), w(d) {}
    tvec4(const tvec3<T>& v, T d) : x(v.x), y(v.y), z(v.z), w(d) {}
    tvec3<T> xyz() const { return tvec3<T>(x, y, z); }
};

#define GLSL_VEC_BINOP(OP)                                                                          \
    template <class T> inline tvec2<T> operator OP(tvec2<T> a, tvec2<T> b) { return {a.x OP b.x, a.y OP b.y}; } \
    template <class T> inline tvec2<T> operator OP(tvec2<T> a, T s) { return {a.x OP s, a.y OP s}; }            \
    template <class T> inline tvec2<T> operator OP(T s, tvec2<T> a) { return {s OP a.x, s OP a.y}; }            \
    template <class T> inline tvec3<T> operator OP(tvec3<T> a, tvec3<T> b) { return {a.x OP b.x, a.y OP b.y, a.z OP b.z}; } \
    template <class T> inline tvec3<T> operator OP(tvec3<T> a, T s) { return {a.x OP s, a.y OP s, a.z OP s}; } \
    template <class T> inline tvec3<T> operator OP(T s, tvec3<T> a) { return {s OP a.x, s OP a.y, s OP a.z}; } \
    template <class T> inline tvec4<T> operator OP(tvec4<T> a, tvec4<T> b) { return {a.x OP b.x, a.y OP b.y, a.z OP b.z, a.w OP b.w}; } \
    template <class T> inline tvec4<T> operator OP(tvec4<T> a, T s) { return {a.x OP s, a.y OP s, a.z OP s, a.w OP s}; }
GLSL_VEC_BINOP(+)
GLSL_VEC_BINOP(-)
GLSL_VEC_BINOP(*)
GLSL_VEC_BINOP(/)
#undef GLSL_VEC_BINOP

template <class T> inline tvec3<T> operator-(tvec3<T> a) { return {-a.x, -a.y, -a.z}; }
template <class T> inline tvec2<T> operator-(tvec2<T> a) { return {-a.x, -a.y}; }

template <class T> inline T dot(tvec2<T> a, tvec2<T> b) { return a.x * b.x + a.y * b.y; }
template <class T> inline T dot(tvec3<T> a, tvec3<T> b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
template <class T> inline T length(tvec2<T> v) { return std::sqrt(dot(v, v)); }
template <class T> inline T length(tvec3<T> v) { return std::sqrt(dot(v, v)); }
template <class T> inline tvec3<T> normalize(tvec3<T> v) { return v / length(v); }
template <class T> inline tvec3<T> cross(tvec3<T> a, tvec3<T> b) {
    return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
}

// Column-major matrices, as GLSL stores them.
template <class T> struct tmat3 {
    tvec3<T> c[3];
    tmat3() {}
    tmat3(tvec3<T> c0, tvec3<T> c1, tvec3<T> c2) { c[0] = c0; c[1] = c1; c[2] = c2; }
};
template <class T> struct tmat4 {
    tvec4<T> c[4];
    tmat4() {}
    // From 16 column-major scalars.
    template <class U> static tmat4 from(const U* m) {
        tmat4 r;
        for (int i = 0; i < 4; ++i) r.c[i] = tvec4<T>(T(m[4 * i]), T(m[4 * i + 1]), T(m[4 * i + 2]), T(m[4 * i + 3]));
        return r;
    }
};
template <class T> inline tmat3<T> transpose(const tmat3<T>& m) {
    return tmat3<T>(tvec3<T>(m.c[0].x, m.c[1].x, m.c[2].x),
                    tvec3<T>(m.c[0].y, m.c[1].y, m.c[2].y),
                    tvec3<T>(m.c[0].z, m.c[1].z, m.c[2].z));
}
template <class T> inline tvec3<T> operator*(const tmat3<T>& m, tvec3<T> v) {
    return m.c[0] * v.x + m.c[1] * v.y + m.c[2] * v.z;
}
template <class T> inline tvec4<T> operator*(const tmat4<T>& m, tvec4<T> v) {
    return ((m.c[0] * v.x + m.c[1] * v.y) + m.c[2] * v.z) + m.c[3] * v.w;
}

// ---- packing built-ins (GLSL 4.3 §8.4) ------------------------------------------------------
// unpackUnorm4x8: component i = float(byte i) / 255.0
template <class T> inline tvec4<T> unpackUnorm4x8(uint p) {
    return tvec4<T>(T(p & 0xFFu) / T(255), T((p >> 8) & 0xFFu) / T(255), T((p >> 16) & 0xFFu) / T(255),
                    T(p >> 24) / T(255));
}

// IEEE binary32 -> binary16, round to nearest even (the conversion CUDA's __float2half_rn uses).
inline uint16_t float_to_half_rne(float f) {
    uint u = floatBitsToUint(f);
    uint sign = (u >> 16) & 0x8000u;
    uint absu = u & 0x7FFFFFFFu;
    if (absu >= 0x7F800000u) return (uint16_t)(sign | 0x7C00u | (absu > 0x7F800000u ? 0x200u : 0u));
    if (absu >= 0x477FF000u) return (uint16_t)(sign | 0x7C00u);  // rounds to inf
    if (absu < 0x38800000u) {                                    // result is subnormal or zero
        if (absu < 0x33000000u) return (uint16_t)sign;           // < 2^-25 -> +-0
        uint e = absu >> 23;
        uint m = (absu & 0x7FFFFFu) | 0x800000u;
        uint shift = 126u - e;  // value / 2^-24 = m * 2^(e-126), with 14 <= shift <= 24
        uint q = m >> shift;
        uint rem = m & ((1u << shift) - 1u);
        uint half = 1u << (shift - 1u);
        if (rem > half || (rem == half && (q & 1u))) q += 1u;
        return (uint16_t)(sign | q);
    }
    uint e = (absu >> 23) - 112u;  // rebias 127 -> 15
    uint m = absu & 0x7FFFFFu;
    uint q = (e << 10) | (m >> 13);
    uint rem = m & 0x1FFFu;
    if (rem > 0x1000u || (rem == 0x1000u && (q & 1u))) q += 1u;  // may carry into exponent: correct
    return (uint16_t)(sign | q);
}
inline float half_to_float(uint16_t h) {
    uint sign = (uint)(h & 0x8000u) << 16;
    uint e = (h >> 10) & 0x1Fu;
    uint m = h & 0x3FFu;
    if (e == 0) {
        float f = std::ldexp((float)m, -24);
        return sign ? -f : f;
    }
    if (e == 31) return uintBitsToFloat(sign | 0x7F800000u | (m << 13));
    return uintBitsToFloat(sign | ((e + 112u) << 23) | (m << 13));
}
// packHalf2x16 takes float inputs; an FP64 caller rounds to binary32 first.
inline uint packHalf2x16(float a, float b) {
    return (uint)float_to_half_rne(a) | ((uint)float_to_half_rne(b) << 16);
}
inline tvec2<float> unpackHalf2x16(uint p) {
    return tvec2<float>(half_to_float((uint16_t)(p & 0xFFFFu)), half_to_float((uint16_t)(p >> 16)));
}

}  // namespace glsl
