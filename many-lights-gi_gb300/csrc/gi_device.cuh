// Device-side math for the GI kernels, written to the GLSL evaluation order of the reference
// shaders. Translation units that must be bit-exact with the reference's FP32 arithmetic
// (VPL processing, ISM splat, pull-push) are compiled with -fmad=false, so every product and sum
// below rounds separately, and use IEEE division and square root.
//   dot(a,b)      ((a.x*b.x + a.y*b.y) + a.z*b.z)
//   length(v)     sqrtf(dot(v,v))
//   normalize(v)  v / length(v)                                (three divides, GLSL definition)
//   cross(a,b)    (a.y*b.z - b.y*a.z, a.z*b.x - b.z*a.x, a.x*b.y - b.x*a.y)
//   min(x,y)      y < x ? y : x          max(x,y)  x < y ? y : x
#pragma once

#include <cstdint>
#include <cuda_fp16.h>
#include <cuda_bf16.h>

namespace mlgi {

struct v3 {
    float x, y, z;
};
__device__ __forceinline__ v3 mk(float x, float y, float z) { return {x, y, z}; }
__device__ __forceinline__ v3 operator+(v3 a, v3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ v3 operator-(v3 a, v3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ v3 operator-(v3 a) { return {-a.x, -a.y, -a.z}; }
__device__ __forceinline__ v3 operator*(v3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ v3 operator*(v3 a, v3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
__device__ __forceinline__ v3 operator/(v3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
__device__ __forceinline__ float dot(v3 a, v3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__device__ __forceinline__ float length(v3 a) { return sqrtf(dot(a, a)); }
__device__ __forceinline__ v3 normalize(v3 a) { return a / length(a); }
__device__ __forceinline__ v3 cross(v3 a, v3 b) {
    return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
}
__device__ __forceinline__ float gmin(float x, float y) { return y < x ? y : x; }
__device__ __forceinline__ float gmax(float x, float y) { return x < y ? y : x; }
__device__ __forceinline__ float gsign(float x) { return x > 0.f ? 1.f : (x < 0.f ? -1.f : 0.f); }

// float -> uint / int with truncation toward zero and saturation (NaN -> 0), the semantics of
// GLSL uint()/int() on the GPU and of cvt.rzi.
__device__ __forceinline__ uint32_t f2u(float x) { return __float2uint_rz(x); }
__device__ __forceinline__ int32_t f2i(float x) { return __float2int_rz(x); }

// unpack3SNFromFloat (floatpacking.glsl:46-66)
__device__ __forceinline__ v3 unpack3SN(uint32_t u) {
    float a = float(u & 0x3FFu) / 1023.0f;
    float b = float((u >> 10) & 0x3FFu) / 1023.0f;
    float c = (float((u >> 20) & 0x3FFu) - 1.5f) / 1021.0f;
    return mk(a * 2.0f - 1.0f, b * 2.0f - 1.0f, c * 2.0f - 1.0f);
}
// pack3SNToFloat (floatpacking.glsl:26-44)
__device__ __forceinline__ uint32_t pack3SN(v3 n) {
    v3 c = mk(n.x * 0.5f + 0.5f, n.y * 0.5f + 0.5f, n.z * 0.5f + 0.5f);
    uint32_t u = f2u(c.x * 1023.0f + 0.5f);
    u |= f2u(c.y * 1023.0f + 0.5f) << 10;
    u |= f2u(c.z * 1021.0f + 1.5f) << 20;
    return u;
}

// lookAtRH (ism_utils.glsl:5-13) rows s and u; the third row is -n.
__device__ __forceinline__ void look_at_rows(v3 n, v3& s, v3& u) {
    const v3 up = mk(0.0f, 1.0f, 0.01f);
    s = normalize(cross(n, up));
    u = cross(s, n);
}

// packHalf2x16 / unpackHalf2x16 with round-to-nearest-even conversion.
__device__ __forceinline__ uint32_t pack_half2(float a, float b) {
    return (uint32_t)__half_as_ushort(__float2half_rn(a)) | ((uint32_t)__half_as_ushort(__float2half_rn(b)) << 16);
}
__device__ __forceinline__ float2 unpack_half2(uint32_t p) {
    return make_float2(__half2float(__ushort_as_half((unsigned short)(p & 0xFFFFu))),
                       __half2float(__ushort_as_half((unsigned short)(p >> 16))));
}

}  // namespace mlgi
