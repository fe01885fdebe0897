// After the gathering: the R11G11B10F GI buffer format, the separable bilateral blur and the GI
// part of the deferred composite.
//
// This translation unit is compiled with -fmad=false and IEEE division and square root. The blur
// performs the shader's operations in the shader's order (normalize as v / length(v), sums from
// +0), so its output equals the oracle's bit for bit. The composite takes its powers with the fast
// __powf (the accurate powf cost 2.5 times the pass's time and still is not the oracle's pow), within
// a stated tolerance of the oracle; the R11G11B10F conversions are exact bit manipulations:
//   gi_blur_kernel    <- data/shaders/gi/gi_blur.frag:24-72 driven by GIStage::blur (GIStage.cpp:308-344)
//   composite_kernel  <- data/shaders/deferredshading.frag:39-44, 69-80 (GI ambient term, Reinhard, toSRGB)
//   R11G11B10F        <- the GI buffers' GL_R11F_G11F_B10F (GIStage.cpp:470)
#include <algorithm>

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "checks.cuh"
#include "gi_device.cuh"
#include "kernels.h"

namespace mlgi {

// ---- R11G11B10F ------------------------------------------------------------------------------
// One unsigned float channel with a 5-bit exponent (bias 15) and `mb` mantissa bits (6 or 5):
// rounded to nearest even, negatives and -0 to 0, overflow to the largest finite value, +Inf to
// Inf, NaN to NaN, denormals kept. In the normal range the FP32 word is rounded at bit 23 - mb by
// one integer add (half minus one, plus the kept lsb: ties to even, a carry moves into the
// exponent) and re-biased by (127 - 15) exponent steps; below 2^-14 the value times 2^(14 + mb)
// (exact) is rounded to an integer.
template <int mb>
__device__ __forceinline__ uint32_t uf_pack(const float x) {
    constexpr int shift = 23 - mb;
    constexpr uint32_t nan_code = (31u << mb) | (1u << (mb - 1)), inf_code = 31u << mb;
    constexpr uint32_t max_code = (30u << mb) | ((1u << mb) - 1u);
    const uint32_t u = __float_as_uint(x);
    const uint32_t t = u + ((1u << (shift - 1)) - 1u) + ((u >> shift) & 1u);
    const uint32_t normal = min((t >> shift) - (112u << mb), max_code);
    const uint32_t denormal = __float2uint_rn(x * float(1 << (14 + mb)));
    uint32_t code = u < 0x38800000u ? denormal : normal;  // 0x38800000 = 2^-14
    code = u == 0x7F800000u ? inf_code : code;
    code = (u >> 31) ? 0u : code;                                  // negative, -0, -Inf
    return (u & 0x7FFFFFFFu) > 0x7F800000u ? nan_code : code;      // NaN of either sign
}

template <int mb>
__device__ __forceinline__ float uf_unpack(const uint32_t v) {  // v: the channel's 11 or 10 bits
    const uint32_t e = v >> mb, m = v & ((1u << mb) - 1u);
    const float normal = __uint_as_float((v << (23 - mb)) + (112u << 23));
    const float denormal = float(m) * (1.0f / float(1 << (14 + mb)));
    const float special = __uint_as_float(m ? 0x7FC00000u : 0x7F800000u);
    return e == 0u ? denormal : (e == 31u ? special : normal);
}

__device__ __forceinline__ uint32_t pack_r11g11b10f(const v3 c) {
    return uf_pack<6>(c.x) | (uf_pack<6>(c.y) << 11) | (uf_pack<5>(c.z) << 22);
}

__device__ __forceinline__ v3 unpack_r11g11b10f(const uint32_t w) {
    return mk(uf_unpack<6>(w & 0x7FFu), uf_unpack<6>((w >> 11) & 0x7FFu), uf_unpack<5>(w >> 22));
}

// Four pixels per thread (three float4 loads, one uint4 store) where the buffers allow it.
__global__ void pack_r11_kernel(const float* rgb, uint32_t* words, int64_t n) {
    const bool vec = ((reinterpret_cast<uintptr_t>(rgb) | reinterpret_cast<uintptr_t>(words)) & 15) == 0;
    const int64_t n4 = vec ? n / 4 : 0;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n4; q += stride) {
        const float4* src = reinterpret_cast<const float4*>(rgb) + 3 * q;
        const float4 f0 = __ldg(src), f1 = __ldg(src + 1), f2 = __ldg(src + 2);
        reinterpret_cast<uint4*>(words)[q] =
            make_uint4(pack_r11g11b10f(mk(f0.x, f0.y, f0.z)), pack_r11g11b10f(mk(f0.w, f1.x, f1.y)),
                       pack_r11g11b10f(mk(f1.z, f1.w, f2.x)), pack_r11g11b10f(mk(f2.y, f2.z, f2.w)));
    }
    for (int64_t i = 4 * n4 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride)
        words[i] = pack_r11g11b10f(mk(rgb[3 * i], rgb[3 * i + 1], rgb[3 * i + 2]));
}

__global__ void unpack_r11_kernel(const uint32_t* words, float* rgb, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const v3 c = unpack_r11g11b10f(words[i]);
        rgb[3 * i] = c.x;
        rgb[3 * i + 1] = c.y;
        rgb[3 * i + 2] = c.z;
    }
}

cudaError_t launch_pack_r11(const float* rgb, uint32_t* words, int64_t n, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    pack_r11_kernel<<<(int)std::min<int64_t>((n + 255) / 256, 152 * 16), 256, 0, s>>>(rgb, words, n);
    return cudaGetLastError();
}

cudaError_t launch_unpack_r11(const uint32_t* words, float* rgb, int64_t n, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    unpack_r11_kernel<<<(int)std::min<int64_t>((n + 255) / 256, 152 * 16), 256, 0, s>>>(words, rgb, n);
    return cudaGetLastError();
}

// ---- bilateral blur ------------------------------------------------------------------------
// One block of 256 threads filters a 32 x 16 tile: the tile and its 3-pixel halo are read once
// into shared memory (normal and linear depth in one float4, GI and an in-image flag in another),
// the X pass runs over the tile's columns for every halo row, and the Y pass over the tile.
constexpr int kBlurTx = 32, kBlurTy = 16, kBlurR = 3;  // KERNEL_RADIUS (gi_blur.frag:21)
constexpr int kBlurThreads = 256;
constexpr int kRegW = kBlurTx + 2 * kBlurR, kRegH = kBlurTy + 2 * kBlurR;

// the gathering's octahedral decode (fg_kernels.cu), normalised as GLSL's normalize: v / length(v)
__device__ __forceinline__ v3 blur_oct_decode(float ex, float ey) {
    v3 n = mk(ex, ey, 1.0f - fabsf(ex) - fabsf(ey));
    if (n.z < 0.f) {
        const float sx = ex >= 0.f ? 1.f : -1.f, sy = ey >= 0.f ? 1.f : -1.f;
        n.x = (1.0f - fabsf(ey)) * sx;
        n.y = (1.0f - fabsf(ex)) * sy;
    }
    const float len = sqrtf(dot(n, n));
    return mk(n.x / len, n.y / len, n.z / len);
}

struct BlurSmem {
    float4 nl[kRegH][kRegW];   // normal xyz, linear depth
    float4 gi[kRegH][kRegW];   // GI rgb, 1 inside the image / 0 outside
    float4 tx[kRegH][kBlurTx]; // X pass rgb
};

// processSample() of gi_blur.frag:37-49 with weight() of :24-35 (the exp2 variant is commented
// out there); `c` is the center's normal and linear depth, `s` the sample's, g its GI.
__device__ __forceinline__ void blur_sample(const float4 c, const float4 s, const float4 g, const float r, v3& acc,
                                            float& factorAcc) {
    const float normalFactor = 1.0f - gmax(0.0f, c.x * s.x + c.y * s.y + c.z * s.z);
    const float depthDiff = s.w - c.w;  // (depthSample - centerDepth) / 1
    const float normalDiff = normalFactor * 5.0f;
    const float factor = gmax(0.0f, (float(kBlurR) - r + 1.0f) * 0.25f - depthDiff * depthDiff - normalDiff * normalDiff);
    factorAcc += factor;
    acc = acc + mk(g.x, g.y, g.z) * factor;
}

__global__ void __launch_bounds__(kBlurThreads) gi_blur_kernel(BlurArgs a) {
    __shared__ BlurSmem S;
    const int x0 = blockIdx.x * kBlurTx, y0 = blockIdx.y * kBlurTy;
    const int tid = threadIdx.x;
    for (int k = tid; k < kRegW * kRegH; k += kBlurThreads) {
        const int ry = k / kRegW, rx = k - ry * kRegW;
        const int gx = x0 - kBlurR + rx, gy = y0 - kBlurR + ry;
        if (gx < 0 || gy < 0 || gx >= a.width || gy >= a.height) {
            S.gi[ry][rx] = make_float4(0.f, 0.f, 0.f, 0.f);
            continue;
        }
        const size_t p = MLGI_IX((size_t)gy * a.width + gx, (size_t)a.width * a.height);
        // linearDepth (reprojection.glsl:6-14)
        const float z_n = 2.0f * __ldg(a.depth + p) - 1.0f;
        const float lin = -a.proj_b / (a.proj_a + z_n);
        float ex, ey;
        if (a.normal_f16) {
            const __half2 h = reinterpret_cast<const __half2*>(a.normal)[p];
            ex = __low2float(h);
            ey = __high2float(h);
        } else {
            const float2 e = reinterpret_cast<const float2*>(a.normal)[p];
            ex = e.x;
            ey = e.y;
        }
        const v3 n = blur_oct_decode(ex, ey);
        S.nl[ry][rx] = make_float4(n.x, n.y, n.z, lin);
        const v3 g = a.packed ? unpack_r11g11b10f(__ldg(reinterpret_cast<const uint32_t*>(a.gi_in) + p))
                              : mk(__ldg(reinterpret_cast<const float*>(a.gi_in) + 3 * p),
                                   __ldg(reinterpret_cast<const float*>(a.gi_in) + 3 * p + 1),
                                   __ldg(reinterpret_cast<const float*>(a.gi_in) + 3 * p + 2));
        S.gi[ry][rx] = make_float4(g.x, g.y, g.z, 1.f);
    }
    __syncthreads();
    // X pass (DIRECTION (1,0)) for every region row over the tile's columns
    for (int k = tid; k < kRegH * kBlurTx; k += kBlurThreads) {
        const int ry = k / kBlurTx, tx = k - ry * kBlurTx, cx = tx + kBlurR;
        const float4 cg = S.gi[ry][cx];
        if (cg.w == 0.f) continue;  // outside the image: never read by an output inside it
        const float4 c = S.nl[ry][cx];
        v3 acc = mk(0.0f + cg.x, 0.0f + cg.y, 0.0f + cg.z);  // the shader's sums start at +0
        float factorAcc = 1.0f;
#pragma unroll
        for (int side = -1; side <= 1; side += 2)
#pragma unroll
            for (int i = 1; i <= kBlurR; ++i) {
                const float4 g = S.gi[ry][cx + side * i];
                if (g.w != 0.f) blur_sample(c, S.nl[ry][cx + side * i], g, float(i), acc, factorAcc);
            }
        v3 o = mk(acc.x / factorAcc, acc.y / factorAcc, acc.z / factorAcc);
        if (a.packed) o = unpack_r11g11b10f(pack_r11g11b10f(o));  // the temp buffer is R11G11B10F
        S.tx[ry][tx] = make_float4(o.x, o.y, o.z, 0.f);
    }
    __syncthreads();
    // Y pass (DIRECTION (0,1)) for the tile
    for (int k = tid; k < kBlurTx * kBlurTy; k += kBlurThreads) {
        const int ty = k / kBlurTx, tx = k - ty * kBlurTx;
        const int gx = x0 + tx, gy = y0 + ty;
        if (gx >= a.width || gy >= a.height) continue;
        const int cy = ty + kBlurR, cx = tx + kBlurR;
        const float4 c = S.nl[cy][cx];
        const float4 ct = S.tx[cy][tx];
        v3 acc = mk(0.0f + ct.x, 0.0f + ct.y, 0.0f + ct.z);
        float factorAcc = 1.0f;
#pragma unroll
        for (int side = -1; side <= 1; side += 2)
#pragma unroll
            for (int i = 1; i <= kBlurR; ++i)
                if (S.gi[cy + side * i][cx].w != 0.f)
                    blur_sample(c, S.nl[cy + side * i][cx], S.tx[cy + side * i][tx], float(i), acc, factorAcc);
        const v3 o = mk(acc.x / factorAcc, acc.y / factorAcc, acc.z / factorAcc);
        const size_t p = MLGI_IX((size_t)gy * a.width + gx, (size_t)a.width * a.height);
        if (a.packed) {
            reinterpret_cast<uint32_t*>(a.gi_out)[p] = pack_r11g11b10f(o);
        } else {
            float* out = reinterpret_cast<float*>(a.gi_out);
            out[3 * p] = o.x;
            out[3 * p + 1] = o.y;
            out[3 * p + 2] = o.z;
        }
    }
}

cudaError_t launch_gi_blur(const BlurArgs& a, cudaStream_t s) {
    if (a.width <= 0 || a.height <= 0) return cudaSuccess;
    const dim3 grid((a.width + kBlurTx - 1) / kBlurTx, (a.height + kBlurTy - 1) / kBlurTy);
    gi_blur_kernel<<<grid, kBlurThreads, 0, s>>>(a);
    return cudaGetLastError();
}

// ---- composite --------------------------------------------------------------------------------
__device__ __forceinline__ v3 composite_pixel(const CompositeArgs& a, const v3 gi, const uint32_t al, const float occlusion,
                                             const v3 direct) {
    const float gamma = 2.2f;  // srgb_utils.glsl:6 (linearRendering)
    const float inv_gamma = 1.0f / gamma;
    // toLinear(texture(diffuseSampler).xyz): RGBA8 UNORM, then pow(v, gamma)
    const v3 diffuse = mk(__powf(float(al & 0xFFu) / 255.0f, gamma), __powf(float((al >> 8) & 0xFFu) / 255.0f, gamma),
                          __powf(float((al >> 16) & 0xFFu) / 255.0f, gamma));
    v3 c = gi * diffuse * occlusion + direct;  // ambientTerm + (diffuseTerm + specularTerm)
    // tonemap (deferredshading.frag:39-44)
    c = c * a.exposure;
    c = mk(c.x / (1.0f + c.x), c.y / (1.0f + c.y), c.z / (1.0f + c.z));
    // toSRGB
    return mk(__powf(c.x, inv_gamma), __powf(c.y, inv_gamma), __powf(c.z, inv_gamma));
}

__device__ __forceinline__ uint32_t rgba8(const v3 c) {
    auto unorm = [](float v) { return f2u(gmin(gmax(v, 0.0f), 1.0f) * 255.0f + 0.5f); };
    return unorm(c.x) | (unorm(c.y) << 8) | (unorm(c.z) << 16) | 0xFF000000u;
}

__device__ __forceinline__ v3 composite_gi(const CompositeArgs& a, int64_t p) {
    return a.gi_packed ? unpack_r11g11b10f(__ldg(reinterpret_cast<const uint32_t*>(a.gi) + p))
                       : mk(__ldg(reinterpret_cast<const float*>(a.gi) + 3 * p),
                            __ldg(reinterpret_cast<const float*>(a.gi) + 3 * p + 1),
                            __ldg(reinterpret_cast<const float*>(a.gi) + 3 * p + 2));
}

// One pixel per iteration; for packed GI and RGBA8 output with 16-byte aligned buffers, four.
__global__ void composite_kernel(CompositeArgs a) {
    const int64_t n = (int64_t)a.width * a.height;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const uintptr_t al16 = reinterpret_cast<uintptr_t>(a.gi) | reinterpret_cast<uintptr_t>(a.albedo) |
                           reinterpret_cast<uintptr_t>(a.out) | reinterpret_cast<uintptr_t>(a.occlusion) |
                           reinterpret_cast<uintptr_t>(a.direct);
    const bool vec = a.gi_packed && a.out_rgba8 && (al16 & 15) == 0;
    const int64_t n4 = vec ? n / 4 : 0;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n4; q += stride) {
        const uint4 g = __ldg(reinterpret_cast<const uint4*>(a.gi) + q);
        const uint4 al = __ldg(reinterpret_cast<const uint4*>(a.albedo) + q);
        const float4 occ = a.occlusion ? __ldg(reinterpret_cast<const float4*>(a.occlusion) + q)
                                       : make_float4(1.f, 1.f, 1.f, 1.f);
        float d[12] = {};
        if (a.direct) {
            const float4* dp = reinterpret_cast<const float4*>(a.direct) + 3 * q;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const float4 t = __ldg(dp + k);
                d[4 * k] = t.x;
                d[4 * k + 1] = t.y;
                d[4 * k + 2] = t.z;
                d[4 * k + 3] = t.w;
            }
        }
        reinterpret_cast<uint4*>(a.out)[q] =
            make_uint4(rgba8(composite_pixel(a, unpack_r11g11b10f(g.x), al.x, occ.x, mk(d[0], d[1], d[2]))),
                       rgba8(composite_pixel(a, unpack_r11g11b10f(g.y), al.y, occ.y, mk(d[3], d[4], d[5]))),
                       rgba8(composite_pixel(a, unpack_r11g11b10f(g.z), al.z, occ.z, mk(d[6], d[7], d[8]))),
                       rgba8(composite_pixel(a, unpack_r11g11b10f(g.w), al.w, occ.w, mk(d[9], d[10], d[11]))));
    }
    for (int64_t p = 4 * n4 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += stride) {
        const v3 dir = a.direct ? mk(__ldg(a.direct + 3 * p), __ldg(a.direct + 3 * p + 1), __ldg(a.direct + 3 * p + 2))
                                : mk(0.f, 0.f, 0.f);
        const v3 c = composite_pixel(a, composite_gi(a, p), __ldg(a.albedo + p),
                                     a.occlusion ? __ldg(a.occlusion + p) : 1.0f, dir);
        if (a.out_rgba8) {
            reinterpret_cast<uint32_t*>(a.out)[p] = rgba8(c);
        } else {
            float* o = reinterpret_cast<float*>(a.out);
            o[3 * p] = c.x;
            o[3 * p + 1] = c.y;
            o[3 * p + 2] = c.z;
        }
    }
}

cudaError_t launch_composite(const CompositeArgs& a, cudaStream_t s) {
    const int64_t n = (int64_t)a.width * a.height;
    if (n <= 0) return cudaSuccess;
    composite_kernel<<<(int)std::min<int64_t>((n + 255) / 256, 152 * 16), 256, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace mlgi

MLGI_CHECK_UNIT(post_kernels)
