// Final gathering: interleaved-sampling VPL accumulation with ISM visibility
// (data/shaders/gi/final_gathering.comp:63-135, dispatched by GIStage::compute_final_gathering,
// GIStage.cpp:261-306).
//
// Work mapping. Pixel (x, y) belongs to interleave class c = (x % I) + (y % I) * I and gathers
// the class's VPL slice [c*N/I^2, (c+1)*N/I^2). A block is a T x T tile of one class in the
// de-interleaved sub-image (pixels (i*I + cx, j*I + cy)), so every thread of a block walks the
// same VPL list and reads each VPL from shared memory as a broadcast. The slice is staged with
// a 1-D bulk TMA copy (cp.async.bulk) completed on an mbarrier whose wait is bounded; per-VPL
// derived data (lookAtRH rows, ISM tile origin) is computed once per block. With culling on,
// the block reduces its pixels' world-space bounding box and drops VPLs whose front half-space
// misses the box (lossless: those pairs have a zero angle factor) and, when an influence cutoff
// is given, VPLs farther from the box than (maxflux / cutoff)^(1/4) (lossy, error stated).
// Accumulation order is ascending VPL index for every pixel, so results are deterministic.
#include <cuda_runtime.h>

#include "batch_items.cuh"
#include "gi_device.cuh"
#include "kernels.h"

namespace mlgi {

constexpr int kMaxVplChunk = 128;
// pixel-VPL pairs evaluated per iteration of the gather loop (3 measured best: 4 spills at the
// 64-register budget of four blocks per SM, and fewer blocks cost more than they gain)
constexpr int kPairs = 3;

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void tma_bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}
// Bounded wait on an mbarrier phase: gives up after ~2^31 SM cycles (about a second) and
// returns false, so a lost transfer can never hang the GPU.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    const long long t0 = clock64();
    for (;;) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(smem_addr(bar)), "r"(parity)
            : "memory");
        if (done) return true;
        if (clock64() - t0 > (1ll << 31)) return false;
    }
}

template <bool kReduced>
__device__ __forceinline__ void decode_vpl(const unsigned char* rec, v3& p, v3& n, v3& f) {
    if (!kReduced) {
        const float4* r = reinterpret_cast<const float4*>(rec);
        const float4 a = r[0], b = r[1], c = r[2];
        p = mk(a.x, a.y, a.z);
        n = mk(b.x, b.y, b.z);
        f = mk(c.x, c.y, c.z);
    } else {
        const uint2* r = reinterpret_cast<const uint2*>(rec);
        const uint2 a = r[0], b = r[1], c = r[2];
        p = mk(__uint_as_float(a.x), __uint_as_float(a.y), __uint_as_float(b.x));
        n = mk(__half2float(__ushort_as_half((unsigned short)(b.y & 0xFFFFu))),
               __half2float(__ushort_as_half((unsigned short)(b.y >> 16))),
               __half2float(__ushort_as_half((unsigned short)(c.x & 0xFFFFu))));
        f = mk(__bfloat162float(__ushort_as_bfloat16((unsigned short)(c.x >> 16))),
               __bfloat162float(__ushort_as_bfloat16((unsigned short)(c.y & 0xFFFFu))),
               __bfloat162float(__ushort_as_bfloat16((unsigned short)(c.y >> 16))));
    }
}

// ---- compensated ("double-float") arithmetic for the world-position reconstruction ----------
// inv_vp * ndc followed by the w divide cancels badly near the far plane (w is a small difference
// of two ~0.5 terms), which makes a plain FP32 evaluation drift ~1e-4 world units from the exact
// value -- enough to flip the clamped 1/d^4 term of near-coplanar VPLs. Each quantity is kept as an
// unevaluated sum hi + lo using the error-free transformations TwoSum (Knuth) and TwoProduct via
// FMA (Ogita, Rump and Oishi, "Accurate sum and dot product", SIAM J. Sci. Comput. 2005); the
// result is rounded once to FP32. Intrinsics keep the compiler from contracting or reordering.
struct df {
    float hi, lo;
};
__device__ __forceinline__ df two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}
__device__ __forceinline__ df fast_two_sum(float a, float b) {  // |a| >= |b|
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ df df_add(df a, df b) {
    const df s = two_sum(a.hi, b.hi);
    return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ df df_mul_f(df a, float b) {
    const float p = __fmul_rn(a.hi, b);
    const float e = __fmaf_rn(a.lo, b, __fmaf_rn(a.hi, b, -p));
    return fast_two_sum(p, e);
}
// a / b rounded to FP32 from double-float operands, given rb ~ 1/b.hi (within a few ulps): the
// quotient a.hi * rb, then one correction by the remainder a - q b (the FMA part a.hi - q b.hi is
// exact); the error left is the square of rb's relative error plus the final rounding.
__device__ __forceinline__ float df_div(df a, df b, float rb) {
    const float q = __fmul_rn(a.hi, rb);
    const float r = __fadd_rn(__fmaf_rn(-q, b.hi, a.hi), __fmaf_rn(-q, b.lo, a.lo));
    return __fmaf_rn(r, rb, q);
}
// 2*k/n - 1 as double-float (k, n small integers, rn = RN(1/n)): the pixel-corner NDC coordinate.
// q = k rn is within an ulp of k/n; the remainder k - q n is exact, and its quotient is the low part.
__device__ __forceinline__ df ndc_coord(int k, int n, float rn) {
    const float fk = float(k), fn = float(n);
    const float q = __fmul_rn(fk, rn);
    const float ql = __fmul_rn(__fmaf_rn(-q, fn, fk), rn);
    const df t = two_sum(__fmul_rn(q, 2.0f), -1.0f);
    return fast_two_sum(t.hi, __fadd_rn(t.lo, __fmul_rn(ql, 2.0f)));
}
// world = (inv_vp * (ndc, 1)).xyz / w, each row summed in double-float.
__device__ __forceinline__ v3 reconstruct_world(const float* m, int x, int y, int w, int h, float rw, float rh,
                                                float d) {
    const df nx = ndc_coord(x, w, rw), ny = ndc_coord(y, h, rh);
    const df nz = two_sum(__fmul_rn(d, 2.0f), -1.0f);
    df r[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        df acc = df_mul_f(nx, m[k]);
        acc = df_add(acc, df_mul_f(ny, m[4 + k]));
        acc = df_add(acc, df_mul_f(nz, m[8 + k]));
        acc = df_add(acc, df{m[12 + k], 0.0f});
        r[k] = acc;
    }
    // one reciprocal of w for the three divides (the hardware approximation); each quotient is
    // corrected by its remainder, as in double-float division (Dekker 1971)
    float rb;
    asm("rcp.approx.f32 %0, %1;" : "=f"(rb) : "f"(r[3].hi));
    return mk(df_div(r[0], r[3], rb), df_div(r[1], r[3], rb), df_div(r[2], r[3], rb));
}

// normalize(v) with the hardware reciprocal square root (about 2 ulps; the gathering's bar is a
// relative L2 of 1e-3).
__device__ __forceinline__ v3 normalize_fast(v3 v) { return v * rsqrtf(dot(v, v)); }

__device__ __forceinline__ v3 oct_decode(float ex, float ey) {
    v3 n = mk(ex, ey, 1.0f - fabsf(ex) - fabsf(ey));
    if (n.z < 0.f) {
        const float sx = ex >= 0.f ? 1.f : -1.f, sy = ey >= 0.f ? 1.f : -1.f;
        n.x = (1.0f - fabsf(ey)) * sx;
        n.y = (1.0f - fabsf(ex)) * sy;
    }
    return normalize_fast(n);
}

// Shared memory of one final-gathering block (one tile of one interleave class).
template <int NT>
struct FgSmem {
    __align__(128) unsigned char raw[kMaxVplChunk * 48];  // VPL records staged by the bulk copy
    float4 a[kMaxVplChunk], b[kMaxVplChunk], c[kMaxVplChunk], d[kMaxVplChunk];
    float2 org[kMaxVplChunk];  // ISM tile origin (texels) + half ISM size folded in
    int list[kMaxVplChunk];
    unsigned char flag[kMaxVplChunk];
    float box[6][NT / 32];
    int n;
    __align__(8) uint64_t bar;
};

// One T x T tile of interleave class c. The caller initialises S.bar once and keeps `parity`
// across calls. Returns false (block-uniform) when the VPL staging wait timed out.
// kClusters: compile the clustered-culling path (cull == 2), which batched views do not use
template <int T, bool kReduced, bool kAtlasF16, bool kNormalF16, bool kClusters = true>
__device__ __forceinline__ bool fg_tile(const FgArgs& a, const int tile, const int c, FgSmem<T * T>& S,
                                        uint32_t& parity) {
    constexpr int NT = T * T;
    constexpr int kRec = kReduced ? 24 : 48;
    const int tid = threadIdx.x;
    const int I = a.interleave;
    const int cx = c % I, cy = c / I;
    // the first VPL chunk's bulk copy starts now and completes behind the pixel setup (the
    // previous tile's use of S.raw ended at its last barrier)
    const int vbase = c * a.per_class;
    const bool use_tma = ((size_t)vbase * kRec) % 16 == 0;
    const unsigned char* src = kReduced ? a.reduced : reinterpret_cast<const unsigned char*>(a.vpl);
    const size_t bytes0 = (size_t)min(kMaxVplChunk, a.per_class) * kRec;
    const bool early = use_tma && bytes0 % 16 == 0;
    if (early && tid == 0) {
        mbar_expect_tx(&S.bar, (uint32_t)bytes0);
        tma_bulk_g2s(S.raw, src + (size_t)vbase * kRec, (uint32_t)bytes0, &S.bar);
    }
    const int sw = (a.width + I - 1) / I;
    const int ntx = (sw + T - 1) / T;
    const int tix = tile % ntx, tiy = tile / ntx;
    const int x = (tix * T + tid % T) * I + cx;
    const int y = (tiy * T + tid / T) * I + cy;
    const bool valid = x < a.width && y < a.height;

    // ---- pixel setup: world position from depth (final_gathering.comp:70-76, evaluated with
    // compensated arithmetic) and the octahedral normal ----
    v3 fw = mk(0.f, 0.f, 0.f), fn = mk(0.f, 0.f, 1.f);
    const uint32_t* cl_row = nullptr;  // cull == 2: the keep bits of the pixel's cluster
    if (valid) {
        const size_t pix = (size_t)y * a.width + x;
        const float d = __ldg(a.depth + pix);
        fw = reconstruct_world(a.inv_vp, x, y, a.width, a.height, a.inv_w, a.inv_h, d);
        float ex, ey;
        if (kNormalF16) {
            const __half2 h = reinterpret_cast<const __half2*>(a.normal)[pix];
            ex = __low2float(h);
            ey = __high2float(h);
        } else {
            const float2 e = reinterpret_cast<const float2*>(a.normal)[pix];
            ex = e.x;
            ey = e.y;
        }
        fn = oct_decode(ex, ey);
        if (kClusters && a.cull == 2) {
            const int cluster = ((y / kClusterPixels) * a.cl_tiles_x + x / kClusterPixels) * kClusterSlices + a.cl_slice[pix];
            cl_row = a.cl_masks + (size_t)cluster * a.cl_words;
        }
    }

    // ---- per-tile bounds for culling ----
    v3 bmin = mk(0.f, 0.f, 0.f), bmax = mk(0.f, 0.f, 0.f);
    if (a.cull == 1) {
        const float inf = __int_as_float(0x7f800000);
        float b[6] = {valid ? fw.x : inf,  valid ? fw.y : inf,  valid ? fw.z : inf,
                      valid ? -fw.x : inf, valid ? -fw.y : inf, valid ? -fw.z : inf};
#pragma unroll
        for (int k = 0; k < 6; ++k) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) b[k] = fminf(b[k], __shfl_xor_sync(0xffffffffu, b[k], o));
        }
        if ((tid & 31) == 0)
#pragma unroll
            for (int k = 0; k < 6; ++k) S.box[k][tid >> 5] = b[k];
        __syncthreads();
        float r[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            r[k] = S.box[k][0];
            for (int w = 1; w < NT / 32; ++w) r[k] = fminf(r[k], S.box[k][w]);
        }
        bmin = mk(r[0], r[1], r[2]);
        bmax = mk(-r[3], -r[4], -r[5]);
    }

    __syncthreads();  // the previous tile's use of S is over

    const float hs = float(a.ism_size) * 0.5f;
    const float inv_zfar = 1.0f / a.z_far;
    float accx = 0.f, accy = 0.f, accz = 0.f;

    for (int base = 0; base < a.per_class; base += kMaxVplChunk) {
        const int cnt = min(kMaxVplChunk, a.per_class - base);
        const size_t bytes = (size_t)cnt * kRec;
        if (use_tma && bytes % 16 == 0) {
            if (tid == 0 && !(base == 0 && early)) {  // the first chunk's copy was issued at the start
                mbar_expect_tx(&S.bar, (uint32_t)bytes);
                tma_bulk_g2s(S.raw, src + (size_t)(vbase + base) * kRec, (uint32_t)bytes, &S.bar);
            }
            const bool ok = __syncthreads_and(mbar_wait(&S.bar, parity));
            if (!ok) {  // block-uniform: flag the error, give the copy one more bounded wait, leave
                if (tid == 0) {
                    atomicOr(a.status, kStatusTmaTimeout);
                    mbar_wait(&S.bar, parity);
                }
                return false;
            }
            parity ^= 1u;
        } else {
            for (size_t k = tid * 4; k < bytes; k += NT * 4)
                *reinterpret_cast<uint32_t*>(S.raw + k) =
                    __ldg(reinterpret_cast<const uint32_t*>(src + (size_t)(vbase + base) * kRec + k));
            __syncthreads();
        }
        // derive per-VPL data and the cull flag
        for (int k = tid; k < cnt; k += NT) {
            v3 p, n, f;
            decode_vpl<kReduced>(S.raw + (size_t)k * kRec, p, n, f);
            // lookAtRH rows (ism_utils.glsl:5-13) with the fast normalisation
            const v3 s = normalize_fast(cross(n, mk(0.0f, 1.0f, 0.01f)));
            const v3 u = cross(s, n);
            const int vid = vbase + base + k;
            // int(ismIndex / gx) of small non-negative integers equals the integer quotient
            const int ism = vid - a.ism_index_offset;
            const int ty = ism / a.gx;
            const int tx = ism - ty * a.gx;
            // the lookAtRH rows scaled by half the ISM size (the texel offset from the ISM centre is
            // hs * s.d / (1 + a1)); d.w = 1 marks an ISM on or beyond the atlas border (a scaled
            // layout gives VPLs outside the range ISM indices off the grid), the only ones whose
            // texel can leave the atlas: |x| < 1 for every pair that reaches the lookup
            const bool border = tx <= 0 || ty <= 0 || tx >= a.gx - 1 || ty >= a.gy - 1;
            S.a[k] = make_float4(p.x, p.y, p.z, f.x);
            S.b[k] = make_float4(n.x, n.y, n.z, f.y);
            S.c[k] = make_float4(s.x * hs, s.y * hs, s.z * hs, f.z);
            S.d[k] = make_float4(u.x * hs, u.y * hs, u.z * hs, border ? 1.0f : 0.0f);
            S.org[k] = make_float2(float(tx * a.ism_size) + hs, float(ty * a.ism_size) + hs);
            bool keep = true;
            if (a.cull == 1) {
                // front half-space of the VPL against the box corner farthest along its normal
                const v3 sup = mk(n.x > 0.f ? bmax.x : bmin.x, n.y > 0.f ? bmax.y : bmin.y, n.z > 0.f ? bmax.z : bmin.z);
                if (dot(n, sup - p) < -1e-3f) keep = false;
                if (keep && a.influence_cutoff > 0.f) {
                    const float fl = fmaxf(f.x, fmaxf(f.y, f.z));
                    const float r = sqrtf(sqrtf(fl / a.influence_cutoff));
                    const v3 q = mk(fminf(fmaxf(p.x, bmin.x), bmax.x), fminf(fmaxf(p.y, bmin.y), bmax.y),
                                    fminf(fmaxf(p.z, bmin.z), bmax.z));
                    const v3 dq = q - p;
                    if (dot(dq, dq) > r * r) keep = false;
                }
            }
            S.flag[k] = keep ? 1 : 0;
        }
        __syncthreads();
        // order-preserving compaction of the kept indices by warp 0
        if (tid < 32) {
            int run = 0;
            for (int w = 0; w < cnt; w += 32) {
                const int k = w + tid;
                const bool keep = k < cnt && S.flag[k];
                const unsigned ballot = __ballot_sync(0xffffffffu, keep);
                if (keep) S.list[run + __popc(ballot & ((1u << tid) - 1u))] = k;
                run += __popc(ballot);
            }
            if (tid == 0) S.n = run;
        }
        __syncthreads();

        // ---- gather over the kept list (final_gathering.comp:97-130) ----
        const int nk = S.n;
        if (valid) {
            const float* atlas32 = reinterpret_cast<const float*>(a.atlas);
            const __half* atlas16 = reinterpret_cast<const __half*>(a.atlas);
            // per-pair parameters in registers (a may live in shared memory in the batched form)
            const float clampv = a.clamp_value;
            const bool shadow = a.shadowing != 0;
            const int aw = a.atlas_w, ah = a.atlas_h;
            // One pair: fG = flux * G (the geometry term G clamped as in the shader), the ISM texel
            // index t and the pixel's normalised distance vz for the shadow test.
            auto prepare = [&](int k, float3& fG, float& vz, uint32_t& t) -> bool {
                if (kClusters && cl_row) {  // outside the pixel's cluster list
                    const int vid = vbase + base + k;
                    if (!((__ldg(cl_row + (vid >> 5)) >> (vid & 31)) & 1u)) return false;
                }
                const float4 A = S.a[k], B = S.b[k];
                const float dx = fw.x - A.x, dy = fw.y - A.y, dz = fw.z - A.z;
                // the cosine terms have the signs of these dot products with the unnormalised
                // direction: most pairs end here, before the square root (max(0, a1) *
                // max(0, a2) > 0 needs a1 > 0 and a2 > 0)
                const float e1 = B.x * dx + B.y * dy + B.z * dz;
                const float e2 = fn.x * dx + fn.y * dy + fn.z * dz;
                if (!(e1 > 0.f && e2 < 0.f)) return false;
                const float d2 = dx * dx + dy * dy + dz * dz;
                const float inv = rsqrtf(d2);
                const float a1 = e1 * inv, a2 = -e2 * inv;
                const float att = (inv * inv) * (inv * inv);
                const float G = fminf((a1 * a2) * att, clampv);
                const float4 C = S.c[k];
                fG = make_float3(A.w * G, B.w * G, C.w * G);
                if (shadow) {
                    const float4 D = S.d[k];
                    const float2 org = S.org[k];
                    // paraboloid_project(diff, dist, n, zFar, ismIndex, grid, false):
                    // x = s.d / (1 - (-n).d), texel = floor(((x + 1)/2 + tile) * ismSize), d the
                    // normalised direction: s.d = (s.(p - v)) / |p - v|
                    const float rz = __fdividef(inv, 1.0f + a1);
                    int ix = __float2int_rd(fmaf(C.x * dx + C.y * dy + C.z * dz, rz, org.x));
                    int iy = __float2int_rd(fmaf(D.x * dx + D.y * dy + D.z * dz, rz, org.y));
                    if (D.w != 0.f) {  // GL_REPEAT, for border ISMs only (uniform over the block)
                        ix %= aw;
                        if (ix < 0) ix += aw;
                        iy %= ah;
                        if (iy < 0) iy += ah;
                    }
                    t = (uint32_t)iy * (uint32_t)aw + (uint32_t)ix;  // atlas sides <= 65535
                    vz = (d2 * inv) * inv_zfar;
                }
                return true;
            };
            auto occluder = [&](uint32_t t) -> float {
                return kAtlasF16 ? __half2float(__ldg(atlas16 + t)) : __ldg(atlas32 + t);
            };
            auto visibility = [&](float vz, float occ) -> float {  // smoothstep(0.98, 1, 1 - (vz - occ))
                if (!shadow) return 1.0f;
                const float sv0 = 1.0f - (vz - occ);
                const float tt = __saturatef((sv0 - 0.98f) * 50.0f);
                return tt * tt * (3.0f - 2.0f * tt);
            };
            // kPairs pairs per iteration so that their ISM texel loads are in flight together;
            // accumulation stays in ascending list order
            int q = 0;
            for (; q + kPairs - 1 < nk; q += kPairs) {
                float3 fG[kPairs];
                float vz[kPairs], o[kPairs];
                uint32_t t[kPairs];
                bool ok[kPairs];
#pragma unroll
                for (int j = 0; j < kPairs; ++j) {
                    vz[j] = 0.f;
                    t[j] = 0;
                    ok[j] = prepare(S.list[q + j], fG[j], vz[j], t[j]);
                }
#pragma unroll
                for (int j = 0; j < kPairs; ++j) o[j] = (ok[j] && shadow) ? occluder(t[j]) : 0.f;
#pragma unroll
                for (int j = 0; j < kPairs; ++j) {
                    if (!ok[j]) continue;
                    const float v = visibility(vz[j], o[j]);
                    accx = fmaf(fG[j].x, v, accx);
                    accy = fmaf(fG[j].y, v, accy);
                    accz = fmaf(fG[j].z, v, accz);
                }
            }
            for (; q < nk; ++q) {
                float3 fG;
                float vz = 0.f;
                uint32_t t = 0;
                if (prepare(S.list[q], fG, vz, t)) {
                    const float v = visibility(vz, shadow ? occluder(t) : 0.f);
                    accx = fmaf(fG.x, v, accx);
                    accy = fmaf(fG.y, v, accy);
                    accz = fmaf(fG.z, v, accz);
                }
            }
        }
        __syncthreads();
    }
    if (valid) {
        const size_t pix = (size_t)y * a.width + x;
        // vec3(acc * giIntensityFactor / vplCount) * interleavedPixels
        a.out[3 * pix + 0] = accx * a.gi_scale;
        a.out[3 * pix + 1] = accy * a.gi_scale;
        a.out[3 * pix + 2] = accz * a.gi_scale;
    }
    return true;
}

template <int T, bool kReduced, bool kAtlasF16, bool kNormalF16>
__global__ void __launch_bounds__(T* T, T == 16 ? 4 : 16) fg_kernel(FgArgs a) {
    __shared__ FgSmem<T * T> S;
    if (threadIdx.x == 0) mbar_init(&S.bar, 1);
    uint32_t parity = 0;
    fg_tile<T, kReduced, kAtlasF16, kNormalF16>(a, a.tile0 + blockIdx.x, blockIdx.y, S, parity);
}

// Tile rows [tr0, tr1): tiles are numbered row by row, so a band of tile rows is a contiguous
// range of tile indices starting at tile0.
template <int T>
static cudaError_t launch_fg_t(const FgArgs& args, cudaStream_t s, int tr0, int tr1) {
    const int I = args.interleave;
    const int sw = (args.width + I - 1) / I;
    const int ntx = (sw + T - 1) / T;
    if (tr1 <= tr0) return cudaSuccess;
    FgArgs a = args;
    a.tile0 = tr0 * ntx;
    const dim3 grid(ntx * (tr1 - tr0), I * I);
    const int sel = (a.reduced ? 4 : 0) | (a.atlas_f16 ? 2 : 0) | (a.normal_f16 ? 1 : 0);
    switch (sel) {
        case 0: fg_kernel<T, false, false, false><<<grid, T * T, 0, s>>>(a); break;
        case 1: fg_kernel<T, false, false, true><<<grid, T * T, 0, s>>>(a); break;
        case 2: fg_kernel<T, false, true, false><<<grid, T * T, 0, s>>>(a); break;
        case 3: fg_kernel<T, false, true, true><<<grid, T * T, 0, s>>>(a); break;
        case 4: fg_kernel<T, true, false, false><<<grid, T * T, 0, s>>>(a); break;
        case 5: fg_kernel<T, true, false, true><<<grid, T * T, 0, s>>>(a); break;
        case 6: fg_kernel<T, true, true, false><<<grid, T * T, 0, s>>>(a); break;
        default: fg_kernel<T, true, true, true><<<grid, T * T, 0, s>>>(a); break;
    }
    return cudaGetLastError();
}

cudaError_t launch_final_gather(const FgArgs& a, cudaStream_t s, int tile_row0, int tile_row1) {
    if (a.width <= 0 || a.height <= 0) return cudaSuccess;
    const int rows = fg_tile_rows(a);
    const int tr0 = tile_row0 < 0 ? 0 : tile_row0, tr1 = tile_row1 < 0 || tile_row1 > rows ? rows : tile_row1;
    if (a.tile == 8) return launch_fg_t<8>(a, s, tr0, tr1);
    return launch_fg_t<16>(a, s, tr0, tr1);
}

// Persistent final gathering over a view table (16 x 16 tiles). Views are FP32 or fully reduced.
// One pass per precision (FP32 views in pass kBpFg, reduced views in kBpFg16), so that each
// kernel holds one variant of the tile body, as the single-view kernels do.
template <bool kReduced>
__global__ void __launch_bounds__(256, 4) batch_fg_kernel(BatchTable t) {
    __shared__ FgSmem<256> S;
    __shared__ FgArgs args;  // the item's view arguments, staged when the block changes views
    __shared__ int tpc;
    if (threadIdx.x == 0) mbar_init(&S.bar, 1);
    uint32_t parity = 0;
    __shared__ int s_pre[kBatchPrefixCache + 1];
    ItemWalk w;
    w.init(t.prefix + (kReduced ? kBpFg16 : kBpFg) * (t.n_views + 1), t.n_views, s_pre);
    int cur = -1;
    for (int item = blockIdx.x; item < w.total; item += gridDim.x) {
        const int lo = w.view(item);
        if (lo != cur) {  // lo is uniform over the block
            __syncthreads();
            if (threadIdx.x == 0) {
                args = t.views[lo].fg;
                tpc = t.views[lo].fg_tiles_per_class;
            }
            __syncthreads();
            cur = lo;
        }
        const int local = w.local(item);
        const int tile = local % tpc, cls = local / tpc;
        if (!fg_tile<16, kReduced, kReduced, kReduced, false>(args, tile, cls, S, parity))
            return;  // block-uniform: the staging wait timed out (status word already set)
    }
}

cudaError_t launch_batch_fg(const BatchTable& t, int pass, int grid, cudaStream_t s) {
    if (grid <= 0) return cudaSuccess;
    if (pass == kBpFg16)
        batch_fg_kernel<true><<<grid, 256, 0, s>>>(t);
    else
        batch_fg_kernel<false><<<grid, 256, 0, s>>>(t);
    return cudaGetLastError();
}

}  // namespace mlgi
