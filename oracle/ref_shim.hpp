// GLSL 4.3 shim under which the reference's compute shaders compile as C++ -- TEST
// INFRASTRUCTURE ONLY (built into oracle/_ref by oracle/build_ref.py).
//
// build_ref.py rewrites each shader mechanically (see its docstring) into a C++ struct whose
// members are the shader's globals and whose main() is the shader's main; this header provides
// the GLSL types, operators and built-ins those structs use, with the same evaluation-order
// conventions as oracle/glsl.hpp (dot/length/normalize/cross/mat*vec summed left to right, IEEE
// division and square root, no contraction). Images, samplers and buffers are views of arrays
// the harness (oracle/ref_harness.cpp) owns; a work group's invocations run as fibers so that
// barrier() has its GLSL meaning.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <stdexcept>
#include <type_traits>
#include <utility>
#include <string>
#include <vector>

namespace glslref {

using uint = uint32_t;

template <class T> struct V2;
template <class T> struct V3;
template <class T> struct V4;

// ---- swizzle proxies (lvalue .xy / .xyz / .rgb) ------------------------------------------------
template <class T, int N> struct SwzVec;
template <class T> struct SwzVec<T, 2> { using type = V2<T>; };
template <class T> struct SwzVec<T, 3> { using type = V3<T>; };

template <class T, int N, int A, int B, int C = 0>
struct Swz {
    T* p;
    using VT = typename SwzVec<T, N>::type;
    VT get() const {
        if constexpr (N == 2) return VT(p[A], p[B]);
        else return VT(p[A], p[B], p[C]);
    }
    operator VT() const { return get(); }
    void set(const VT& v) {
        p[A] = v.x;
        p[B] = v.y;
        if constexpr (N == 3) p[C] = v.z;
    }
    Swz& operator=(const VT& v) { set(v); return *this; }
    template <class U> Swz& operator+=(const U& o) { set(VT(get() + unswz(o))); return *this; }
    template <class U> Swz& operator-=(const U& o) { set(VT(get() - unswz(o))); return *this; }
    template <class U> Swz& operator*=(const U& o) { set(VT(get() * unswz(o))); return *this; }
    template <class U> Swz& operator/=(const U& o) { set(VT(get() / unswz(o))); return *this; }
    template <class U> static decltype(auto) unswz(const U& o) {
        if constexpr (requires { o.get(); }) return o.get();
        else return (o);
    }
};

template <class T> struct V2 {
    T x, y;
    V2() : x(0), y(0) {}
    V2(T a, T b) : x(a), y(b) {}
    template <class A, class B, class = std::enable_if_t<std::is_arithmetic_v<A> && std::is_arithmetic_v<B>>>
    V2(A a, B b) : x(T(a)), y(T(b)) {}
    explicit V2(T s) : x(s), y(s) {}
    template <class U> explicit V2(const V2<U>& o) : x(T(o.x)), y(T(o.y)) {}
    template <class S, class = decltype(std::declval<S>().get().y)> explicit V2(const S& s) : V2(s.get()) {}
    T& operator[](int i) { return (&x)[i]; }
    T operator[](int i) const { return (&x)[i]; }
    Swz<T, 2, 0, 1> xy() { return {&x}; }
    V2 xy() const { return *this; }
    V2 rg() const { return *this; }
};
template <class T> struct V3 {
    T x, y, z;
    V3() : x(0), y(0), z(0) {}
    V3(T a, T b, T c) : x(a), y(b), z(c) {}
    template <class A, class B, class C,
              class = std::enable_if_t<std::is_arithmetic_v<A> && std::is_arithmetic_v<B> && std::is_arithmetic_v<C>>>
    V3(A a, B b, C c) : x(T(a)), y(T(b)), z(T(c)) {}
    template <class U, class C> V3(const V2<U>& v, C c) : x(T(v.x)), y(T(v.y)), z(T(c)) {}
    explicit V3(T s) : x(s), y(s), z(s) {}
    template <class U> explicit V3(const V3<U>& o) : x(T(o.x)), y(T(o.y)), z(T(o.z)) {}
    T& operator[](int i) { return (&x)[i]; }
    T operator[](int i) const { return (&x)[i]; }
    Swz<T, 2, 0, 1> xy() { return {&x}; }
    V2<T> xy() const { return V2<T>(x, y); }
    Swz<T, 3, 0, 1, 2> xyz() { return {&x}; }
    V3 xyz() const { return *this; }
    V3 rgb() const { return *this; }
};
template <class T> struct V4 {
    T x, y, z, w;
    V4() : x(0), y(0), z(0), w(0) {}
    V4(T a, T b, T c, T d) : x(a), y(b), z(c), w(d) {}
    template <class A, class B, class C, class D,
              class = std::enable_if_t<std::is_arithmetic_v<A> && std::is_arithmetic_v<B> &&
                                       std::is_arithmetic_v<C> && std::is_arithmetic_v<D>>>
    V4(A a, B b, C c, D d) : x(T(a)), y(T(b)), z(T(c)), w(T(d)) {}
    template <class D> V4(const V3<T>& v, D d) : x(v.x), y(v.y), z(v.z), w(T(d)) {}
    template <class C, class D> V4(const V2<T>& v, C c, D d) : x(v.x), y(v.y), z(T(c)), w(T(d)) {}
    explicit V4(T s) : x(s), y(s), z(s), w(s) {}
    T& operator[](int i) { return (&x)[i]; }
    T operator[](int i) const { return (&x)[i]; }
    Swz<T, 2, 0, 1> xy() { return {&x}; }
    V2<T> xy() const { return V2<T>(x, y); }
    Swz<T, 3, 0, 1, 2> xyz() { return {&x}; }
    V3<T> xyz() const { return V3<T>(x, y, z); }
    Swz<T, 3, 0, 1, 2> rgb() { return {&x}; }
    V3<T> rgb() const { return V3<T>(x, y, z); }
    V2<T> rg() const { return V2<T>(x, y); }
};

using vec2 = V2<float>;
using vec3 = V3<float>;
using vec4 = V4<float>;
using ivec2 = V2<int32_t>;
using ivec3 = V3<int32_t>;
using uvec2 = V2<uint32_t>;
using uvec3 = V3<uint32_t>;
using uvec4 = V4<uint32_t>;
using bvec2 = V2<bool>;

// GLSL implicit conversions for mixed operands: the result type of a op b.
template <class A, class B> using Arith = decltype(A() + B());
template <class T> struct Scal { using type = T; };
template <> struct Scal<int32_t> { using type = int32_t; };

#define GLSLREF_BINOP(OP)                                                                                      \
    template <class A, class B> auto operator OP(const V2<A>& a, const V2<B>& b) {                              \
        using R = std::conditional_t<std::is_floating_point_v<A> || std::is_floating_point_v<B>, float,        \
                                     std::conditional_t<std::is_unsigned_v<A> || std::is_unsigned_v<B>, uint32_t, A>>; \
        return V2<R>(R(a.x) OP R(b.x), R(a.y) OP R(b.y));                                                      \
    }                                                                                                          \
    template <class A, class S, class = std::enable_if_t<std::is_arithmetic_v<S>>>                             \
    auto operator OP(const V2<A>& a, S s) {                                                                     \
        using R = std::conditional_t<std::is_floating_point_v<A> || std::is_floating_point_v<S>, float,        \
                                     std::conditional_t<std::is_unsigned_v<A> || std::is_unsigned_v<S>, uint32_t, A>>; \
        return V2<R>(R(a.x) OP R(s), R(a.y) OP R(s));                                                          \
    }                                                                                                          \
    template <class A, class S, class = std::enable_if_t<std::is_arithmetic_v<S>>>                             \
    auto operator OP(S s, const V2<A>& a) {                                                                     \
        using R = std::conditional_t<std::is_floating_point_v<A> || std::is_floating_point_v<S>, float, A>;    \
        return V2<R>(R(s) OP R(a.x), R(s) OP R(a.y));                                                          \
    }                                                                                                          \
    template <class A, class B> auto operator OP(const V3<A>& a, const V3<B>& b) {                              \
        using R = std::conditional_t<std::is_floating_point_v<A> || std::is_floating_point_v<B>, float, A>;    \
        return V3<R>(R(a.x) OP R(b.x), R(a.y) OP R(b.y), R(a.z) OP R(b.z));                                    \
    }                                                                                                          \
    template <class A, class S, class = std::enable_if_t<std::is_arithmetic_v<S>>>                             \
    auto operator OP(const V3<A>& a, S s) {                                                                     \
        using R = std::conditional_t<std::is_floating_point_v<A> || std::is_floating_point_v<S>, float, A>;    \
        return V3<R>(R(a.x) OP R(s), R(a.y) OP R(s), R(a.z) OP R(s));                                          \
    }                                                                                                          \
    template <class A, class S, class = std::enable_if_t<std::is_arithmetic_v<S>>>                             \
    auto operator OP(S s, const V3<A>& a) {                                                                     \
        using R = std::conditional_t<std::is_floating_point_v<A> || std::is_floating_point_v<S>, float, A>;    \
        return V3<R>(R(s) OP R(a.x), R(s) OP R(a.y), R(s) OP R(a.z));                                          \
    }                                                                                                          \
    template <class A, class B> auto operator OP(const V4<A>& a, const V4<B>& b) {                              \
        using R = std::conditional_t<std::is_floating_point_v<A> || std::is_floating_point_v<B>, float, A>;    \
        return V4<R>(R(a.x) OP R(b.x), R(a.y) OP R(b.y), R(a.z) OP R(b.z), R(a.w) OP R(b.w));                  \
    }                                                                                                          \
    template <class A, class S, class = std::enable_if_t<std::is_arithmetic_v<S>>>                             \
    auto operator OP(const V4<A>& a, S s) {                                                                     \
        using R = std::conditional_t<std::is_floating_point_v<A> || std::is_floating_point_v<S>, float, A>;    \
        return V4<R>(R(a.x) OP R(s), R(a.y) OP R(s), R(a.z) OP R(s), R(a.w) OP R(s));                          \
    }
GLSLREF_BINOP(+)
GLSLREF_BINOP(-)
GLSLREF_BINOP(*)
GLSLREF_BINOP(/)
#undef GLSLREF_BINOP

// swizzle proxies in arithmetic: convert to the vector first
template <class T, int N, int A, int B, int C, class U>
auto operator+(const Swz<T, N, A, B, C>& s, const U& u) { return s.get() + u; }
template <class T, int N, int A, int B, int C, class U>
auto operator-(const Swz<T, N, A, B, C>& s, const U& u) { return s.get() - u; }
template <class T, int N, int A, int B, int C, class U>
auto operator*(const Swz<T, N, A, B, C>& s, const U& u) { return s.get() * u; }
template <class T, int N, int A, int B, int C, class U>
auto operator/(const Swz<T, N, A, B, C>& s, const U& u) { return s.get() / u; }

template <class X> struct is_swz : std::false_type {};
template <class T, int N, int A, int B, int C> struct is_swz<Swz<T, N, A, B, C>> : std::true_type {};
template <class X> decltype(auto) val(const X& x) {
    if constexpr (is_swz<X>::value) return x.get();
    else return (x);
}
template <class X, class Y, class = std::enable_if_t<is_swz<Y>::value && !is_swz<X>::value>>
auto operator*(const X& a, const Y& b) { return a * b.get(); }
template <class X, class Y, class = std::enable_if_t<is_swz<Y>::value && !is_swz<X>::value>>
auto operator+(const X& a, const Y& b) { return a + b.get(); }
template <class X, class Y, class = std::enable_if_t<is_swz<Y>::value && !is_swz<X>::value>>
auto operator-(const X& a, const Y& b) { return a - b.get(); }
template <class X, class Y, class = std::enable_if_t<is_swz<Y>::value && !is_swz<X>::value>>
auto operator/(const X& a, const Y& b) { return a / b.get(); }
template <class T, int N, int A, int B, int C, class S>
auto operator>>(const Swz<T, N, A, B, C>& s, S k) { return s.get() >> k; }
template <class T, int N, int A, int B, int C, class S>
auto operator&(const Swz<T, N, A, B, C>& s, S k) { return s.get() & k; }

template <class T> V2<T>& operator+=(V2<T>& a, const V2<T>& b) { a = a + b; return a; }
template <class T> V3<T>& operator+=(V3<T>& a, const V3<T>& b) { a = a + b; return a; }
template <class T, int A, int B, int C> V3<T>& operator+=(V3<T>& a, const Swz<T, 3, A, B, C>& b) {
    a = a + b.get();
    return a;
}
template <class T> V4<T>& operator+=(V4<T>& a, const V4<T>& b) { a = a + b; return a; }
template <class T, class S> V3<T>& operator*=(V3<T>& a, S s) { a = V3<T>(a * s); return a; }

template <class T> V2<T> operator-(const V2<T>& a) { return V2<T>(-a.x, -a.y); }
template <class T> V3<T> operator-(const V3<T>& a) { return V3<T>(-a.x, -a.y, -a.z); }

// integer vector shifts / masks / comparisons
template <class T, class S> V2<T> operator>>(const V2<T>& a, S s) { return V2<T>(a.x >> s, a.y >> s); }
template <class T, class S> V2<T> operator&(const V2<T>& a, S s) { return V2<T>(a.x & s, a.y & s); }
template <class T> bool operator!=(const V2<T>& a, const V2<T>& b) { return a.x != b.x || a.y != b.y; }
template <class T> bool operator==(const V2<T>& a, const V2<T>& b) { return a.x == b.x && a.y == b.y; }

// ---- scalar built-ins --------------------------------------------------------------------------
inline float sqrt(float x) { return std::sqrt(x); }
inline float ceil(float x) { return std::ceil(x); }
inline float floor(float x) { return std::floor(x); }
inline float log2(float x) { return std::log2(x); }
inline float pow(float x, float y) { return std::pow(x, y); }
inline float sin(float x) { return std::sin(x); }
inline float fract(float x) { return x - std::floor(x); }
inline float mod(float x, float y) { return x - y * std::floor(x / y); }
inline float min(float x, float y) { return y < x ? y : x; }
inline float max(float x, float y) { return x < y ? y : x; }
inline float max(float x, int y) { return max(x, float(y)); }
inline float max(int x, float y) { return max(float(x), y); }
inline float min(float x, int y) { return min(x, float(y)); }
inline int min(int x, int y) { return y < x ? y : x; }
inline float clamp(float x, float a, float b) { return min(max(x, a), b); }
inline float step(float e, float x) { return x < e ? 0.0f : 1.0f; }
inline float sign(float x) { return x > 0.f ? 1.f : (x < 0.f ? -1.f : 0.f); }
inline float smoothstep(float e0, float e1, float x) {
    float t = clamp((x - e0) / (e1 - e0), 0.0f, 1.0f);
    return t * t * (3.0f - 2.0f * t);
}
inline float dot(float a, float b) { return a * b; }
inline float dot(vec2 a, vec2 b) { return a.x * b.x + a.y * b.y; }
inline float dot(vec3 a, vec3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline float length(vec2 v) { return std::sqrt(dot(v, v)); }
inline float length(vec3 v) { return std::sqrt(dot(v, v)); }
inline vec3 normalize(vec3 v) { return v / length(v); }
inline vec3 cross(vec3 a, vec3 b) { return vec3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y); }

inline uint floatBitsToUint(float f) { uint u; std::memcpy(&u, &f, 4); return u; }
inline float uintBitsToFloat(uint u) { float f; std::memcpy(&f, &u, 4); return f; }
inline uvec2 floatBitsToUint(vec2 v) { return uvec2(floatBitsToUint(v.x), floatBitsToUint(v.y)); }
inline uvec3 floatBitsToUint(vec3 v) { return uvec3(floatBitsToUint(v.x), floatBitsToUint(v.y), floatBitsToUint(v.z)); }
inline uvec4 floatBitsToUint(vec4 v) {
    return uvec4(floatBitsToUint(v.x), floatBitsToUint(v.y), floatBitsToUint(v.z), floatBitsToUint(v.w));
}

// ---- matrices (column-major) -------------------------------------------------------------------
struct mat3 {
    vec3 c[3];
    mat3() {}
    mat3(vec3 a, vec3 b, vec3 d) { c[0] = a; c[1] = b; c[2] = d; }
    vec3& operator[](int i) { return c[i]; }
};
struct mat4 {
    vec4 c[4];
    vec4& operator[](int i) { return c[i]; }
    const vec4& operator[](int i) const { return c[i]; }
};
inline mat3 transpose(const mat3& m) {
    return mat3(vec3(m.c[0].x, m.c[1].x, m.c[2].x), vec3(m.c[0].y, m.c[1].y, m.c[2].y),
                vec3(m.c[0].z, m.c[1].z, m.c[2].z));
}
inline vec3 operator*(const mat3& m, vec3 v) { return m.c[0] * v.x + m.c[1] * v.y + m.c[2] * v.z; }
inline vec4 operator*(const mat4& m, vec4 v) { return ((m.c[0] * v.x + m.c[1] * v.y) + m.c[2] * v.z) + m.c[3] * v.w; }

// ---- packing built-ins -------------------------------------------------------------------------
uint16_t f2h_rne(float f);
float h2f(uint16_t h);
inline uint packUnorm4x8(vec4 c) {
    auto q = [](float v) { return (uint)std::nearbyint(clamp(v, 0.f, 1.f) * 255.0f); };
    return q(c.x) | (q(c.y) << 8) | (q(c.z) << 16) | (q(c.w) << 24);
}
inline vec4 unpackUnorm4x8(uint p) {
    return vec4(float(p & 0xFFu) / 255.0f, float((p >> 8) & 0xFFu) / 255.0f, float((p >> 16) & 0xFFu) / 255.0f,
                float(p >> 24) / 255.0f);
}
inline uint packHalf2x16(vec2 v) { return (uint)f2h_rne(v.x) | ((uint)f2h_rne(v.y) << 16); }
inline vec2 unpackHalf2x16(uint p) { return vec2(h2f((uint16_t)(p & 0xFFFFu)), h2f((uint16_t)(p >> 16))); }
inline uint packUnorm2x16(vec2 c) {
    auto q = [](float v) { return (uint)std::nearbyint(clamp(v, 0.f, 1.f) * 65535.0f); };
    return q(c.x) | (q(c.y) << 16);
}
inline vec2 unpackUnorm2x16(uint p) { return vec2(float(p & 0xFFFFu) / 65535.0f, float(p >> 16) / 65535.0f); }

// ---- images, samplers, buffers -----------------------------------------------------------------
// Texel storage is always 4 components of float or uint; the harness converts formats.
struct Image2D {
    float* f = nullptr;
    uint* u = nullptr;
    int w = 0, h = 0;
    int comps = 4;
};
struct Image3D {
    uint* u = nullptr;
    int w = 0, h = 0, d = 0;
};
struct ImageBuffer {
    float* f = nullptr;
    int n = 0;
};
struct UImage2D {
    uint* u = nullptr;
    int w = 0, h = 0;
    int comps = 1;
};
using image2D = Image2D;
using uimage2D = UImage2D;
using uimage1D = UImage2D;
using uimage3D = Image3D;
using imageBuffer = ImageBuffer;
struct Sampler2D {
    const float* f = nullptr;  // 4 floats per texel
    const uint* u = nullptr;   // 4 uints per texel (usampler)
    int w = 0, h = 0;
    bool repeat = true;
};
struct USampler2D {
    const uint* u = nullptr;  // one uint per texel
    int w = 0, h = 0;
};
using sampler2D = Sampler2D;
using usampler2D = USampler2D;
struct sampler3D {};

struct IntScalar {  // imageSize of a buffer image: an int that also answers .x
    int x;
    operator int() const { return x; }
};

inline vec4 imageLoad(const Image2D& im, ivec2 p) {
    if (p.x < 0 || p.y < 0 || p.x >= im.w || p.y >= im.h) return vec4();
    const float* t = im.f + (size_t)im.comps * ((size_t)p.y * im.w + p.x);
    if (im.comps == 1) return vec4(t[0], 0.f, 0.f, 1.f);
    return vec4(t[0], t[1], t[2], t[3]);
}
inline uvec4 imageLoad(const UImage2D& im, ivec2 p) {
    if (p.x < 0 || p.y < 0 || p.x >= im.w || p.y >= im.h) return uvec4();
    return uvec4(im.u[(size_t)p.y * im.w + p.x], 0u, 0u, 1u);
}
inline uvec4 imageLoad(const Image3D& im, ivec3 p) {
    if (p.x < 0 || p.y < 0 || p.z < 0 || p.x >= im.w || p.y >= im.h || p.z >= im.d) return uvec4();
    return uvec4(im.u[((size_t)p.z * im.h + p.y) * im.w + p.x], 0u, 0u, 1u);
}
inline vec4 imageLoad(const ImageBuffer& im, int i) {
    if (i < 0 || i >= im.n) return vec4();
    const float* t = im.f + 4 * (size_t)i;
    return vec4(t[0], t[1], t[2], t[3]);
}
inline void imageStore(Image2D& im, ivec2 p, vec4 v) {
    if (p.x < 0 || p.y < 0 || p.x >= im.w || p.y >= im.h) return;
    float* t = im.f + (size_t)im.comps * ((size_t)p.y * im.w + p.x);
    t[0] = v.x;
    if (im.comps == 4) { t[1] = v.y; t[2] = v.z; t[3] = v.w; }
}
inline void imageStore(UImage2D& im, ivec2 p, uvec4 v) {
    if (p.x < 0 || p.y < 0 || p.x >= im.w || p.y >= im.h) return;
    im.u[(size_t)p.y * im.w + p.x] = v.x;
}
inline void imageStore(ImageBuffer& im, int i, vec4 v) {
    if (i < 0 || i >= im.n) return;
    float* t = im.f + 4 * (size_t)i;
    t[0] = v.x; t[1] = v.y; t[2] = v.z; t[3] = v.w;
}
inline uint imageAtomicMin(UImage2D& im, ivec2 p, uint v) {
    if (p.x < 0 || p.y < 0 || p.x >= im.w || p.y >= im.h) return 0;
    uint* t = im.u + ((size_t)p.y * im.w + p.x);
    uint cur = __atomic_load_n(t, __ATOMIC_RELAXED);
    while (v < cur && !__atomic_compare_exchange_n(t, &cur, v, true, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) {
    }
    return cur;
}
// 1-D images (uimage1D shares UImage2D's storage, one row) and 3-D integer images
inline uvec4 imageLoad(const UImage2D& im, int i) { return imageLoad(im, ivec2(i, 0)); }
inline void imageStore(UImage2D& im, int i, uvec4 v) { imageStore(im, ivec2(i, 0), v); }
inline void imageStore(Image3D& im, ivec3 p, uvec4 v) {
    if (p.x < 0 || p.y < 0 || p.z < 0 || p.x >= im.w || p.y >= im.h || p.z >= im.d) return;
    im.u[((size_t)p.z * im.h + p.y) * im.w + p.x] = v.x;
}
// atomicAdd on shared variables (a work group's invocations run as fibers on one thread) and on
// buffer members (work groups run on several threads)
inline int32_t atomicAdd(int32_t& m, int32_t v) { return __atomic_fetch_add(&m, v, __ATOMIC_RELAXED); }
inline uint atomicAdd(uint& m, uint v) { return __atomic_fetch_add(&m, v, __ATOMIC_RELAXED); }
inline uint atomicAdd(uint& m, int32_t v) { return atomicAdd(m, (uint)v); }
template <class A, class B> bvec2 lessThan(const A& a, const B& b) {
    const auto x = val(a);
    const auto y = val(b);
    return bvec2(x.x < y.x, x.y < y.y);
}
inline bool all(bvec2 b) { return b.x && b.y; }

inline ivec2 imageSize(const Image2D& im) { return ivec2(im.w, im.h); }
inline ivec2 imageSize(const UImage2D& im) { return ivec2(im.w, im.h); }
inline IntScalar imageSize(const ImageBuffer& im) { return IntScalar{im.n}; }

inline vec4 texelFetch(const Sampler2D& s, ivec2 p, int) {
    if (p.x < 0 || p.y < 0 || p.x >= s.w || p.y >= s.h) return vec4();
    const float* t = s.f + 4 * ((size_t)p.y * s.w + p.x);
    return vec4(t[0], t[1], t[2], t[3]);
}
inline uvec4 texelFetch(const USampler2D& s, ivec2 p, int) {
    if (p.x < 0 || p.y < 0 || p.x >= s.w || p.y >= s.h) return uvec4();
    return uvec4(s.u[(size_t)p.y * s.w + p.x], 0u, 0u, 1u);
}
inline ivec2 textureSize(const Sampler2D& s, int) { return ivec2(s.w, s.h); }
// Nearest filtering with GL_REPEAT wrap (the default wrap of the reference's ISM result texture).
inline vec4 textureLod(const Sampler2D& s, vec2 uv, float) {
    long x = (long)std::floor(uv.x * float(s.w)), y = (long)std::floor(uv.y * float(s.h));
    x = ((x % s.w) + s.w) % s.w;
    y = ((y % s.h) + s.h) % s.h;
    return texelFetch(s, ivec2((int)x, (int)y), 0);
}
inline vec4 texture(const Sampler2D& s, vec2 uv, float = 0) { return textureLod(s, uv, 0); }
inline vec4 texture(const sampler3D&, vec3) { return vec4(); }
inline vec2 floor(vec2 v) { return vec2(std::floor(v.x), std::floor(v.y)); }

// ---- bindings, per-invocation built-ins and the work-group scheduler hook ---------------------
struct Bindings {
    std::map<std::string, std::vector<unsigned char>> values;  // uniforms (raw bytes of the C++ type)
    std::map<std::string, void*> buffers;                      // interface-block members
    uvec3 local_size, num_groups;
    template <class T> void set(const std::string& n, const T& v) {
        auto& b = values[n];
        b.resize(sizeof(T));
        std::memcpy(b.data(), &v, sizeof(T));
    }
    template <class T> bool get(const std::string& n, T& v) const {
        auto it = values.find(n);
        if (it == values.end() || it->second.size() != sizeof(T)) return false;
        std::memcpy(&v, it->second.data(), sizeof(T));
        return true;
    }
};

// The work group's shared arena, owned by the worker thread that runs the group.
extern thread_local std::map<std::string, std::vector<unsigned char>>* tl_shared_arena;

struct RefShaderBase {
    Bindings* B;
    uvec3 gl_WorkGroupID, gl_LocalInvocationID, gl_NumWorkGroups, gl_WorkGroupSize;
    vec4 gl_FragCoord;  // fragment shaders: the pixel centre the harness runs
    explicit RefShaderBase(Bindings* b) : B(b), gl_NumWorkGroups(b->num_groups), gl_WorkGroupSize(b->local_size) {}
    template <class T> T uni(const char* n) const {
        T v{};
        if (!B->get(n, v)) throw std::runtime_error(std::string("unbound uniform ") + n);
        return v;
    }
    template <class T, class D> T uni(const char* n, const D& def) const {
        T v{};
        if (!B->get(n, v)) v = T(def);
        return v;
    }
    template <class T> T* buf(const char* n) const {
        auto it = B->buffers.find(n);
        if (it == B->buffers.end()) throw std::runtime_error(std::string("unbound buffer ") + n);
        return static_cast<T*>(it->second);
    }
    template <class T> T* shared_mem(const char* n, size_t count) const {
        // 64 bytes beyond the declared size: clustering.comp's slice index reaches 16 at the far
        // plane and writes one past its 16-entry array (the pin's scenes stay in front of it)
        auto& v = (*tl_shared_arena)[n];
        if (v.size() < count * sizeof(T) + 64) v.resize(count * sizeof(T) + 64);
        return reinterpret_cast<T*>(v.data());
    }
};

void barrier();  // yields the current invocation's fiber until every invocation reached it
inline void memoryBarrierShared() {}

}  // namespace glslref
