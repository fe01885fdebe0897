// Final gathering: interleaved-sampling VPL accumulation with ISM visibility
// (data/shaders/gi/final_gathering.comp:63-135, dispatched by GIStage::compute_final_gathering,
// GIStage.cpp:261-306).
//
// Work mapping. Pixel (x, y) belongs to interleave class c = (x % I) + (y % I) * I and gathers
// the class's VPL slice [c*N/I^2, (c+1)*N/I^2). A block is a T x T tile of one class in the
// de-interleaved sub-image (pixels (i*I + cx, j*I + cy)), so every thread of a block walks the
// same VPL list and reads each VPL from shared memory as a broadcast. A thread owns two
// horizontally adjacent pixels of the tile and evaluates a VPL for both with packed FP32x2
// arithmetic (T*T/2 threads a block). The slice is staged with
// a 1-D bulk TMA copy (cp.async.bulk) completed on an mbarrier whose wait is bounded; per-VPL
// derived data (lookAtRH rows, ISM tile origin) is computed once per block. With culling on,
// the block reduces its pixels' world-space bounding box and drops VPLs whose front half-space
// misses the box (lossless: those pairs have a zero angle factor) and, when an influence cutoff
// is given, VPLs farther from the box than (maxflux / cutoff)^(1/4) (lossy, error stated).
// Accumulation order is ascending VPL index for every pixel, so results are deterministic.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>

#include "batch_items.cuh"
#include "checks.cuh"
#include "gi_device.cuh"
#include "kernels.h"

namespace mlgi {

// VPLs staged per chunk: 64 for 16 x 16 tiles (13 KB of shared memory a block; with 128 the
// gathering ran 5 % slower at 1080p, the larger carve-out leaving less L1 for the atlas and
// G-buffer loads) and 32 for 8 x 8 tiles (one-warp blocks, many resident)
template <int T>
__host__ __device__ constexpr int fg_chunk() {
    return T == 16 ? 64 : 32;
}

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
// Retires `bytes` of an mbarrier's expected transaction count without a copy.
__device__ __forceinline__ void mbar_complete_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.complete_tx.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
// Bounded wait on an mbarrier phase: gives up after `limit` SM cycles (by default ~2^31, about a
// second) and returns false, so a lost transfer can never hang the GPU.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, long long limit = 1ll << 31) {
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
        if (clock64() - t0 > limit) return false;
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

// ---- two pixels per thread on packed FP32x2 arithmetic ---------------------------------------
// Blackwell's add/sub/mul/fma.f32x2 perform two FP32 operations in one instruction. A thread owns
// two horizontally adjacent pixels of the de-interleaved tile (lane 0 and lane 1 of every packed
// value), and every value of a VPL is stored twice in shared memory, so that one 128-bit load
// yields two packed operands that apply to both pixels. Each pixel still accumulates its VPLs in
// ascending list order.
struct f2 {
    unsigned long long v;
};
__device__ __forceinline__ f2 pk(float a, float b) {
    f2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r.v) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ f2 pk(float a) { return pk(a, a); }
__device__ __forceinline__ void split(f2 a, float& x, float& y) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(x), "=f"(y) : "l"(a.v));
}
__device__ __forceinline__ f2 operator+(f2 a, f2 b) {
    f2 r;
    asm("add.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
    return r;
}
__device__ __forceinline__ f2 operator-(f2 a, f2 b) {
    f2 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
    return r;
}
__device__ __forceinline__ f2 operator*(f2 a, f2 b) {
    f2 r;
    asm("mul.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
    return r;
}
__device__ __forceinline__ f2 fma2(f2 a, f2 b, f2 c) {  // a * b + c
    f2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r.v) : "l"(a.v), "l"(b.v), "l"(c.v));
    return r;
}
__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// ---- compensated ("double-float") world-position reconstruction, for both pixels at once ------
// inv_vp * ndc followed by the w divide cancels badly near the far plane (w is a small difference
// of two ~0.5 terms), which makes a plain FP32 evaluation drift ~1e-4 world units from the exact
// value -- enough to flip the clamped 1/d^4 term of near-coplanar VPLs. Each quantity is kept as an
// unevaluated sum hi + lo using the error-free transformations TwoSum (Knuth) and TwoProduct via
// FMA (Ogita, Rump and Oishi, "Accurate sum and dot product", SIAM J. Sci. Comput. 2005); the
// result is rounded once to FP32. A product that TwoProduct needs rounded on its own is formed as
// fma(a, b, z), z a zero the compiler cannot see, so that it is never fused into the add that
// follows (packed multiplies feeding packed adds may be fused); the other products it could fuse
// are exact (doublings) or add an exact zero.
struct df2 {
    f2 hi, lo;
};
__device__ __forceinline__ df2 two_sum2(f2 a, f2 b) {
    const f2 s = a + b;
    const f2 bb = s - a;
    return {s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ df2 fast_two_sum2(f2 a, f2 b) {  // |a| >= |b|
    const f2 s = a + b;
    return {s, b - (s - a)};
}
__device__ __forceinline__ df2 df_add2(df2 a, df2 b) {
    const df2 s = two_sum2(a.hi, b.hi);
    return fast_two_sum2(s.hi, s.lo + (a.lo + b.lo));
}
__device__ __forceinline__ df2 df_add2(df2 a, f2 b) {  // b exact (low part zero)
    const df2 s = two_sum2(a.hi, b);
    return fast_two_sum2(s.hi, s.lo + a.lo);
}
__device__ __forceinline__ df2 df_mul_f2(df2 a, f2 b, f2 z) {
    const f2 p = fma2(a.hi, b, z);
    const f2 e = fma2(a.lo, b, fma2(a.hi, b, z - p));
    return fast_two_sum2(p, e);
}
// a / b rounded to FP32 from double-float operands, given rb ~ 1/b.hi (within a few ulps): the
// quotient a.hi * rb, then one correction by the remainder a - q b (the FMA part a.hi - q b.hi is
// exact), as in double-float division (Dekker 1971)
__device__ __forceinline__ f2 df_div2(df2 a, df2 b, f2 rb, f2 z) {
    const f2 q = fma2(a.hi, rb, z);
    const f2 nq = z - q;
    const f2 r = fma2(nq, b.hi, a.hi) + fma2(nq, b.lo, a.lo);
    return fma2(r, rb, q);
}
// 2*k/n - 1 as double-float (k, n small integers, rn = RN(1/n)): the pixel-corner NDC coordinate.
// q = k rn is within an ulp of k/n; the remainder k - q n is exact, and its quotient is the low part.
__device__ __forceinline__ df2 ndc_coord2(f2 k, f2 n, f2 rn, f2 z) {
    const f2 q = fma2(k, rn, z);
    const f2 ql = fma2(z - q, n, k) * rn;
    const df2 t = two_sum2(q * pk(2.0f), pk(-1.0f));
    return fast_two_sum2(t.hi, t.lo + ql * pk(2.0f));
}
// world = (inv_vp * (ndc, 1)).xyz / w for pixels (x0, y) and (x1, y) with window depths d0 and d1,
// each row summed in double-float; one hardware reciprocal of w serves the three divides
__device__ __forceinline__ void reconstruct_world2(const float* m, int x0, int x1, int y, int w, int h, float rw,
                                                   float rh, float d0, float d1, f2 z, v3& p0, v3& p1) {
    const df2 nx = ndc_coord2(pk(float(x0), float(x1)), pk(float(w)), pk(rw), z);
    const df2 ny = ndc_coord2(pk(float(y)), pk(float(h)), pk(rh), z);
    const df2 nz = two_sum2(pk(d0, d1) * pk(2.0f), pk(-1.0f));
    df2 r[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        df2 acc = df_mul_f2(nx, pk(m[k]), z);
        acc = df_add2(acc, df_mul_f2(ny, pk(m[4 + k]), z));
        acc = df_add2(acc, df_mul_f2(nz, pk(m[8 + k]), z));
        r[k] = df_add2(acc, pk(m[12 + k]));
    }
    float w0, w1;
    split(r[3].hi, w0, w1);
    const f2 rb = pk(rcp_approx(w0), rcp_approx(w1));
    float ax, bx, ay, by, az, bz;
    split(df_div2(r[0], r[3], rb, z), ax, bx);
    split(df_div2(r[1], r[3], rb, z), ay, by);
    split(df_div2(r[2], r[3], rb, z), az, bz);
    p0 = mk(ax, ay, az);
    p1 = mk(bx, by, bz);
}

// One VPL with every value twice, as (v, v) 64-bit pairs: position, normal, the lookAtRH rows
// scaled by half the ISM size, the ISM tile origin, flux and the border flag.
struct VplPk {
    ulonglong2 r[9];  // (p.x, p.y) (p.z, n.x) (n.y, n.z) (s.x, s.y) (s.z, u.x) (u.y, u.z) (org) (f.x, f.y) (f.z, border)
};

// Shared memory of one final-gathering block (one T x T tile of one interleave class).
template <int T>
struct FgSmem {
    static constexpr int kChunk = fg_chunk<T>(), kThreads = T * T / 2;
    __align__(128) unsigned char raw[kChunk * 48];  // VPL records staged by the bulk copy
    VplPk v[kChunk];
    int list[kChunk];
    unsigned char flag[kChunk];
    float box[6][(kThreads + 31) / 32];
    int n;
    __align__(8) uint64_t bar;
};

// Per-VPL data of the gathering from its staged record: the packed rows (see VplPk) and the
// decoded position, normal and flux. vid is the VPL's index in the VPL buffer.
template <bool kReduced>
__device__ __forceinline__ void derive_vpl(const unsigned char* rec, const int vid, const FgArgs& a, const float hs,
                                           VplPk& R, v3& p, v3& n, v3& f) {
    decode_vpl<kReduced>(rec, p, n, f);
    // lookAtRH rows (ism_utils.glsl:5-13) with the fast normalisation
    const v3 s = normalize_fast(cross(n, mk(0.0f, 1.0f, 0.01f)));
    const v3 u = cross(s, n);
    // int(ismIndex / gx) of small non-negative integers equals the integer quotient
    const int ism = vid - a.ism_index_offset;
    const int ty = ism / a.gx;
    const int tx = ism - ty * a.gx;
    // the lookAtRH rows are scaled by half the ISM size (the texel offset from the ISM centre is
    // hs * s.d / (1 + a1)); border = 1 marks an ISM on or beyond the atlas border (a scaled layout
    // gives VPLs outside the range ISM indices off the grid), the only ones whose texel can leave
    // the atlas: |x| < 1 for every pair that reaches the lookup
    const bool border = tx <= 0 || ty <= 0 || tx >= a.gx - 1 || ty >= a.gy - 1;
    R.r[0] = make_ulonglong2(pk(p.x).v, pk(p.y).v);
    R.r[1] = make_ulonglong2(pk(p.z).v, pk(n.x).v);
    R.r[2] = make_ulonglong2(pk(n.y).v, pk(n.z).v);
    R.r[3] = make_ulonglong2(pk(s.x * hs).v, pk(s.y * hs).v);
    R.r[4] = make_ulonglong2(pk(s.z * hs).v, pk(u.x * hs).v);
    R.r[5] = make_ulonglong2(pk(u.y * hs).v, pk(u.z * hs).v);
    R.r[6] = make_ulonglong2(pk(float(tx * a.ism_size) + hs).v, pk(float(ty * a.ism_size) + hs).v);
    R.r[7] = make_ulonglong2(pk(f.x).v, pk(f.y).v);
    R.r[8] = make_ulonglong2(pk(f.z).v, pk(border ? 1.0f : 0.0f).v);
}

// Squared influence radius of a VPL with flux f: every pixel farther than r = (max flux /
// cutoff)^(1/4) receives flux * cos / d^4 below the cutoff from it (+Inf without a cutoff).
__device__ __forceinline__ float vpl_influence_r2(const v3 f, const float cutoff) {
    if (!(cutoff > 0.f)) return __int_as_float(0x7f800000);
    const float fl = fmaxf(f.x, fmaxf(f.y, f.z));
    const float r = sqrtf(sqrtf(fl / cutoff));
    return r * r;
}

// Culling of one VPL against a box [bmin, bmax] of world positions. vpl_front: the VPL's front
// half-space reaches the box corner farthest along its normal (with a -1e-3 margin, so a VPL it
// drops has a negative cosine at every position in the box: it adds exactly nothing there).
// vpl_near: the box's squared distance is within the influence radius r2 (vpl_influence_r2).
__device__ __forceinline__ bool vpl_front(const v3 p, const v3 n, const v3 bmin, const v3 bmax) {
    const v3 sup = mk(n.x > 0.f ? bmax.x : bmin.x, n.y > 0.f ? bmax.y : bmin.y, n.z > 0.f ? bmax.z : bmin.z);
    return !(dot(n, sup - p) < -1e-3f);
}
__device__ __forceinline__ bool vpl_near(const v3 p, const float r2, const v3 bmin, const v3 bmax) {
    const v3 q = mk(fminf(fmaxf(p.x, bmin.x), bmax.x), fminf(fmaxf(p.y, bmin.y), bmax.y),
                    fminf(fmaxf(p.z, bmin.z), bmax.z));
    const v3 dq = q - p;
    return !(dot(dq, dq) > r2);
}
// Per-tile culling: both tests against the tile's box.
__device__ __forceinline__ bool vpl_keep(const v3 p, const v3 n, const float r2, const v3 bmin, const v3 bmax) {
    return vpl_front(p, n, bmin, bmax) && vpl_near(p, r2, bmin, bmax);
}

// Pixel (x, y) of the G-buffer: window depth and decoded octahedral normal (a pixel outside the
// image gets depth 0.5 and normal +z, finite dummies).
template <bool kNormalF16>
__device__ __forceinline__ void fg_pixel_setup(const FgArgs& a, const int x, const int y, const bool valid, float& d,
                                               v3& fn) {
    d = 0.5f;
    fn = mk(0.f, 0.f, 1.f);
    if (!valid) return;
    const size_t pix = MLGI_IX((size_t)y * a.width + x, (size_t)a.width * a.height);
    d = __ldg(a.depth + pix);
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
}

// World-space bounding box of a warp's pixels (both of each thread's, the valid ones) as six
// minima (x, y, z, -x, -y, -z), in every lane.
__device__ __forceinline__ void fg_warp_box(const v3 w0, const v3 w1, const bool v0, const bool v1, float (&b)[6]) {
    const float inf = __int_as_float(0x7f800000);
    b[0] = fminf(v0 ? w0.x : inf, v1 ? w1.x : inf);
    b[1] = fminf(v0 ? w0.y : inf, v1 ? w1.y : inf);
    b[2] = fminf(v0 ? w0.z : inf, v1 ? w1.z : inf);
    b[3] = fminf(v0 ? -w0.x : inf, v1 ? -w1.x : inf);
    b[4] = fminf(v0 ? -w0.y : inf, v1 ? -w1.y : inf);
    b[5] = fminf(v0 ? -w0.z : inf, v1 ? -w1.z : inf);
#pragma unroll
    for (int k = 0; k < 6; ++k) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) b[k] = fminf(b[k], __shfl_xor_sync(0xffffffffu, b[k], o));
    }
}

// World-space bounding box of a block's pixels, through `box` (6 x NW floats of shared memory)
// and one barrier; wmin/wmax (optional) receive the calling warp's own box.
template <int NW>
__device__ __forceinline__ void fg_tile_box(const v3 w0, const v3 w1, const bool v0, const bool v1,
                                            float (&box)[6][NW], v3& bmin, v3& bmax, v3* wmin = nullptr,
                                            v3* wmax = nullptr) {
    float b[6];
    fg_warp_box(w0, w1, v0, v1, b);
    if (wmin) {
        *wmin = mk(b[0], b[1], b[2]);
        *wmax = mk(-b[3], -b[4], -b[5]);
    }
    if ((threadIdx.x & 31) == 0)
#pragma unroll
        for (int k = 0; k < 6; ++k) box[k][threadIdx.x >> 5] = b[k];
    __syncthreads();
    float r[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        r[k] = box[k][0];
        for (int w = 1; w < NW; ++w) r[k] = fminf(r[k], box[k][w]);
    }
    bmin = mk(r[0], r[1], r[2]);
    bmax = mk(-r[3], -r[4], -r[5]);
}

// VPLs a thread evaluates per gather iteration (for both its pixels): 2 measured best at 1080p,
// 0.0942 ms against 0.0953 with 1 and 0.1009 with 3 (64 bytes of spill at the 64-register budget)
constexpr int kVpls = 2;

// One thread's two pixels of a gathering tile: their world positions and normals as packed pairs,
// the accumulated radiance, and the evaluation of one VPL for both (final_gathering.comp:97-130).
template <bool kAtlasF16, bool kClusters>
struct GatherPair {
    f2 fwx, fwy, fwz, fnx, fny, fnz;
    f2 accx, accy, accz;
    bool v0, v1;
    const uint32_t *cl0, *cl1;
    const void* atlas;
    float clampv;
    bool shadow, clustered;
    int aw, ah;
    f2 izf;

    __device__ __forceinline__ void init(const FgArgs& a, const v3 w0, const v3 n0, const v3 w1, const v3 n1,
                                         const bool pv0, const bool pv1, const uint32_t* c0, const uint32_t* c1) {
        fwx = pk(w0.x, w1.x);
        fwy = pk(w0.y, w1.y);
        fwz = pk(w0.z, w1.z);
        fnx = pk(n0.x, n1.x);
        fny = pk(n0.y, n1.y);
        fnz = pk(n0.z, n1.z);
        accx = accy = accz = pk(0.f);
        v0 = pv0;
        v1 = pv1;
        cl0 = c0;
        cl1 = c1;
        atlas = a.atlas;
        clampv = a.clamp_value;
        shadow = a.shadowing != 0;
        clustered = kClusters && a.cull == 2;
        aw = a.atlas_w;
        ah = a.atlas_h;
        izf = pk(1.0f / a.z_far);
    }

    // One VPL against both pixels: G the clamped geometry term per pixel (0 for a pixel the pair
    // does not reach), the ISM texel index per pixel and the normalised distance vz.
    __device__ __forceinline__ bool prepare(const VplPk& R, const int vid, f2& G, f2& vz, uint32_t& t0, uint32_t& t1,
                                            bool& ok0, bool& ok1) const {
        ok0 = v0;
        ok1 = v1;
        if (kClusters && clustered) {  // outside the pixel's cluster list
            if (cl0) ok0 = ok0 && ((__ldg(cl0 + (vid >> 5)) >> (vid & 31)) & 1u);
            if (cl1) ok1 = ok1 && ((__ldg(cl1 + (vid >> 5)) >> (vid & 31)) & 1u);
        }
        const ulonglong2 R0 = R.r[0], R1 = R.r[1], R2 = R.r[2];
        const f2 dx = fwx - f2{R0.x}, dy = fwy - f2{R0.y}, dz = fwz - f2{R1.x};
        // the cosine terms have the signs of these dot products with the unnormalised direction:
        // most pairs end here, before the square root (max(0, a1) * max(0, a2) > 0 needs a1 > 0 and
        // a2 > 0)
        const f2 e1 = fma2(f2{R1.y}, dx, fma2(f2{R2.x}, dy, f2{R2.y} * dz));
        const f2 e2 = fma2(fnx, dx, fma2(fny, dy, fnz * dz));
        float e1a, e1b, e2a, e2b;
        split(e1, e1a, e1b);
        split(e2, e2a, e2b);
        ok0 = ok0 && e1a > 0.f && e2a < 0.f;
        ok1 = ok1 && e1b > 0.f && e2b < 0.f;
        if (!(ok0 || ok1)) return false;
        const f2 d2 = fma2(dx, dx, fma2(dy, dy, dz * dz));
        float d2a, d2b;
        split(d2, d2a, d2b);
        const f2 inv = pk(rsqrtf(d2a), rsqrtf(d2b));
        const f2 a1 = e1 * inv, a2n = e2 * inv;  // a2 = -a2n
        const f2 i2 = inv * inv;
        float ga, gb;  // -(a1 * a2) / d^4
        split((a1 * a2n) * (i2 * i2), ga, gb);
        G = pk(ok0 ? fminf(-ga, clampv) : 0.f, ok1 ? fminf(-gb, clampv) : 0.f);
        if (shadow) {
            const ulonglong2 R3 = R.r[3], R4 = R.r[4], R5 = R.r[5], R6 = R.r[6];
            float qa, qb;
            split(a1 + pk(1.0f), qa, qb);
            const f2 rz = inv * pk(rcp_approx(qa), rcp_approx(qb));
            const f2 sx = fma2(fma2(f2{R3.x}, dx, fma2(f2{R3.y}, dy, f2{R4.x} * dz)), rz, f2{R6.x});
            const f2 sy = fma2(fma2(f2{R4.y}, dx, fma2(f2{R5.x}, dy, f2{R5.y} * dz)), rz, f2{R6.y});
            float sxa, sxb, sya, syb;
            split(sx, sxa, sxb);
            split(sy, sya, syb);
            int ix0 = __float2int_rd(sxa), ix1 = __float2int_rd(sxb);
            int iy0 = __float2int_rd(sya), iy1 = __float2int_rd(syb);
            float bf, unused;
            split(f2{R.r[8].y}, bf, unused);
            if (bf != 0.f) {  // GL_REPEAT, for border ISMs only (uniform over the block)
                ix0 %= aw;
                if (ix0 < 0) ix0 += aw;
                ix1 %= aw;
                if (ix1 < 0) ix1 += aw;
                iy0 %= ah;
                if (iy0 < 0) iy0 += ah;
                iy1 %= ah;
                if (iy1 < 0) iy1 += ah;
            }
            t0 = ok0 ? (uint32_t)iy0 * (uint32_t)aw + (uint32_t)ix0 : 0u;
            t1 = ok1 ? (uint32_t)iy1 * (uint32_t)aw + (uint32_t)ix1 : 0u;
            vz = (d2 * inv) * izf;
        }
        return true;
    }

    __device__ __forceinline__ float occluder(const uint32_t t) const {
        const uint32_t i = MLGI_IX(t, (uint32_t)aw * (uint32_t)ah);
        return kAtlasF16 ? __half2float(__ldg(reinterpret_cast<const __half*>(atlas) + i))
                         : __ldg(reinterpret_cast<const float*>(atlas) + i);
    }

    // acc += flux * G * smoothstep(0.98, 1, 1 - (vz - occ)) for both pixels
    __device__ __forceinline__ void accumulate(const VplPk& R, const f2 G, const f2 vz, const float o0, const float o1) {
        f2 w = G;
        if (shadow) {
            const f2 sv0 = pk(1.0f) - (vz - pk(o0, o1));
            float sa, sb;
            split(fma2(sv0, pk(50.0f), pk(-49.0f)), sa, sb);
            const f2 tt = pk(__saturatef(sa), __saturatef(sb));
            w = G * ((tt * tt) * fma2(tt, pk(-2.0f), pk(3.0f)));
        }
        const ulonglong2 R7 = R.r[7], R8 = R.r[8];
        accx = fma2(f2{R7.x}, w, accx);
        accy = fma2(f2{R7.y}, w, accy);
        accz = fma2(f2{R8.x}, w, accz);
    }

    // The nk VPLs whose indices into V (ascending) `next()` yields, kVpls per iteration so that
    // their texel loads are in flight together; each pixel accumulates in ascending order. vid0:
    // the VPL index of V[0].
    template <class Next>
    __device__ __forceinline__ void gather(const VplPk* V, const int vid0, const int nk, Next next) {
        int q = 0;
        for (; q + kVpls - 1 < nk; q += kVpls) {
            int kk[kVpls];
            f2 G[kVpls], vz[kVpls];
            uint32_t t[kVpls][2];
            bool ok[kVpls][2], any[kVpls];
#pragma unroll
            for (int j = 0; j < kVpls; ++j) {
                kk[j] = next();
                G[j] = pk(0.f);
                vz[j] = pk(0.f);
                t[j][0] = t[j][1] = 0u;
                any[j] = prepare(V[kk[j]], vid0 + kk[j], G[j], vz[j], t[j][0], t[j][1], ok[j][0], ok[j][1]);
            }
            float o[kVpls][2];
#pragma unroll
            for (int j = 0; j < kVpls; ++j) {
                o[j][0] = (any[j] && shadow && ok[j][0]) ? occluder(t[j][0]) : 0.f;
                o[j][1] = (any[j] && shadow && ok[j][1]) ? occluder(t[j][1]) : 0.f;
            }
#pragma unroll
            for (int j = 0; j < kVpls; ++j)
                if (any[j]) accumulate(V[kk[j]], G[j], vz[j], o[j][0], o[j][1]);
        }
        for (; q < nk; ++q) {
            const int k = next();
            f2 G = pk(0.f), vz = pk(0.f);
            uint32_t t0 = 0u, t1 = 0u;
            bool ok0, ok1;
            if (prepare(V[k], vid0 + k, G, vz, t0, t1, ok0, ok1))
                accumulate(V[k], G, vz, (shadow && ok0) ? occluder(t0) : 0.f, (shadow && ok1) ? occluder(t1) : 0.f);
        }
    }

    __device__ __forceinline__ void store(const FgArgs& a, const int y, const int x0, const int x1) const {
        float ax0, ax1, ay0, ay1, az0, az1;
        split(accx, ax0, ax1);
        split(accy, ay0, ay1);
        split(accz, az0, az1);
        if (v0) {
            const size_t pix = MLGI_IX((size_t)y * a.width + x0, (size_t)a.width * a.height);
            a.out[3 * pix + 0] = ax0 * a.gi_scale;
            a.out[3 * pix + 1] = ay0 * a.gi_scale;
            a.out[3 * pix + 2] = az0 * a.gi_scale;
        }
        if (v1) {
            const size_t pix = MLGI_IX((size_t)y * a.width + x1, (size_t)a.width * a.height);
            a.out[3 * pix + 0] = ax1 * a.gi_scale;
            a.out[3 * pix + 1] = ay1 * a.gi_scale;
            a.out[3 * pix + 2] = az1 * a.gi_scale;
        }
    }
};

// One T x T tile of interleave class c with T*T/2 threads. The caller initialises S.bar once and
// keeps `parity` across calls. Returns false (block-uniform) when the VPL staging wait timed out.
// kClusters: compile the clustered-culling path (cull == 2), which batched views do not use.

template <int T, bool kReduced, bool kAtlasF16, bool kNormalF16, bool kClusters = true>
__device__ __forceinline__ bool fg_tile(const FgArgs& a, const int tile, const int c, FgSmem<T>& S,
                                        uint32_t& parity) {
    constexpr int NT = T * T / 2, HT = T / 2, NW = (NT + 31) / 32, kChunk = fg_chunk<T>();
    constexpr int kRec = kReduced ? 24 : 48;
    const int tid = threadIdx.x;
    const int I = a.interleave;
    const int cx = c % I, cy = c / I;
    const int vbase = c * a.per_class;
    // checked build: a class slice outside the VPL buffer or a chunk larger than the staging
    // buffer skips the tile (block-uniform, before any copy is issued)
    if (!MLGI_RANGE_OK(vbase, a.per_class, a.n_vpl) || !MLGI_RANGE_OK(0, (size_t)min(kChunk, a.per_class) * kRec, sizeof(S.raw)))
        return true;
    const bool use_tma = ((size_t)vbase * kRec) % 16 == 0;
    const unsigned char* src = kReduced ? a.reduced : reinterpret_cast<const unsigned char*>(a.vpl);
    const size_t bytes0 = (size_t)min(kChunk, a.per_class) * kRec;
    const bool early = use_tma && bytes0 % 16 == 0;
    if (early && tid == 0) {
        mbar_expect_tx(&S.bar, (uint32_t)bytes0 + a.test_extra_tx);
        tma_bulk_g2s(S.raw, src + (size_t)vbase * kRec, (uint32_t)bytes0, &S.bar);
    }
    const int sw = (a.width + I - 1) / I;
    const int ntx = (sw + T - 1) / T;
    const int tix = tile % ntx, tiy = tile / ntx;
    // a warp takes a band of adjacent tile rows: its pixels' ISM texels for one VPL are close
    // together (rows interleaved over the warps ran 2 % slower)
    const int y = (tiy * T + tid / HT) * I + cy;
    const int x0 = (tix * T + 2 * (tid % HT)) * I + cx, x1 = x0 + I;
    const bool v0 = x0 < a.width && y < a.height, v1 = x1 < a.width && y < a.height;

    // ---- pixel setup: world position from depth (final_gathering.comp:70-76, evaluated with
    // compensated arithmetic) and the octahedral normal ----
    auto setup = [&](int x, bool valid, float& d, v3& fn, const uint32_t*& cl_row) {
        fg_pixel_setup<kNormalF16>(a, x, y, valid, d, fn);
        cl_row = nullptr;
        if (valid && kClusters && a.cull == 2) {
            const size_t pix = MLGI_IX((size_t)y * a.width + x, (size_t)a.width * a.height);
            const int cluster = ((y / kClusterPixels) * a.cl_tiles_x + x / kClusterPixels) * kClusterSlices + a.cl_slice[pix];
            cl_row = a.cl_masks + (size_t)cluster * a.cl_words;
        }
    };
    v3 w0, n0, w1, n1;
    float d0, d1;
    const uint32_t *cl0, *cl1;
    setup(x0, v0, d0, n0, cl0);
    setup(x1, v1, d1, n1, cl1);
    // both pixels' world positions at once (a pixel outside the image gets a finite dummy)
    reconstruct_world2(a.inv_vp, x0, x1, y, a.width, a.height, a.inv_w, a.inv_h, d0, d1, pk(a.z_far * 0.0f), w0, w1);
    if (!v0) w0 = mk(0.f, 0.f, 0.f);
    if (!v1) w1 = mk(0.f, 0.f, 0.f);

    // ---- per-tile bounds for culling ----
    v3 bmin = mk(0.f, 0.f, 0.f), bmax = mk(0.f, 0.f, 0.f);
    if (a.cull == 1) fg_tile_box<NW>(w0, w1, v0, v1, S.box, bmin, bmax);

    __syncthreads();  // the previous tile's use of S is over

    const float hs = float(a.ism_size) * 0.5f;
    GatherPair<kAtlasF16, kClusters> gp;
    gp.init(a, w0, n0, w1, n1, v0, v1, cl0, cl1);

    for (int base = 0; base < a.per_class; base += kChunk) {
        const int cnt = min(kChunk, a.per_class - base);
        const size_t bytes = (size_t)cnt * kRec;
        if (use_tma && bytes % 16 == 0) {
            if (tid == 0 && !(base == 0 && early)) {  // the first chunk's copy was issued at the start
                mbar_expect_tx(&S.bar, (uint32_t)bytes + (base == 0 ? a.test_extra_tx : 0u));
                tma_bulk_g2s(S.raw, src + (size_t)(vbase + base) * kRec, (uint32_t)bytes, &S.bar);
            }
            const long long limit = a.wait_cycles > 0 ? a.wait_cycles : 1ll << 31;
            const bool ok = __syncthreads_and(mbar_wait(&S.bar, parity, limit));
            if (!ok) {  // block-uniform: flag the error, let the copy land (one more bounded wait), leave
                if (tid == 0) {
                    atomicOr(a.status, kStatusTmaTimeout);
                    // a test surplus of expected bytes (never delivered) is retired first, so that
                    // the phase completes once the real copy has landed
                    if (base == 0 && a.test_extra_tx) mbar_complete_tx(&S.bar, a.test_extra_tx);
                    mbar_wait(&S.bar, parity, 1ll << 31);
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
        // derive per-VPL data (every value stored twice) and the cull flag
        for (int k = tid; k < cnt; k += NT) {
            v3 p, n, f;
            derive_vpl<kReduced>(S.raw + (size_t)k * kRec, vbase + base + k, a, hs, S.v[k], p, n, f);
            const bool keep = a.cull != 1 || vpl_keep(p, n, vpl_influence_r2(f, a.influence_cutoff), bmin, bmax);
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

        // ---- gather over the kept list (final_gathering.comp:97-130), two pixels per thread ----
        if (v0 || v1) {
            int q = 0;
            gp.gather(S.v, vbase + base, S.n, [&]() { return S.list[q++]; });
        }
        __syncthreads();
    }
    gp.store(a, y, x0, x1);
    return true;
}

// Eight 128-thread blocks (or 32 one-warp blocks) per SM: 64 registers a thread.
template <int T, bool kReduced, bool kAtlasF16, bool kNormalF16>
__global__ void __launch_bounds__(T* T / 2, T == 16 ? 8 : 32) fg_kernel(FgArgs a) {
    __shared__ FgSmem<T> S;
    if (threadIdx.x == 0) mbar_init(&S.bar, 1);
    uint32_t parity = 0;
    fg_tile<T, kReduced, kAtlasF16, kNormalF16>(a, a.tile0 + blockIdx.x, blockIdx.y, S, parity);
}

// ---- class-persistent gathering ----------------------------------------------------------------
// Block (b, c) stages and derives interleave class c's VPL slice once (one bulk copy, one bounded
// wait), then gathers tiles b, b + gridDim.x, ... of the launch's tile range for that class. Per
// tile it reduces the tile's world-space box (one barrier: the box slots alternate between tiles),
// and every warp culls the whole slice against it itself, one VPL a lane, keeping the survivors
// as ballot masks: no per-tile staging, derivation or list compaction. Used for 16 x 16 tiles when
// a class slice fits one staging chunk (N / I^2 <= 64) and culling is off or per tile; the tile
// arithmetic (derive_vpl, vpl_keep, GatherPair) is fg_tile's, so results are the same bit for bit.
constexpr int kClassMaxVpls = 64;
constexpr int kFgClassBlocksPerSm = 32;  // C2: 0.0844 ms; 8: 0.0923, 16: 0.0891; per-tile kernel 0.0918

struct FgClassSmem {
    __align__(128) unsigned char raw[kClassMaxVpls * 48];
    VplPk v[kClassMaxVpls];
    float4 cp[kClassMaxVpls], cn[kClassMaxVpls];  // (position, squared influence radius), normal
    float box[2][6][4];
    __align__(8) uint64_t bar;
};

template <bool kReduced, bool kAtlasF16, bool kNormalF16>
__global__ void __launch_bounds__(128, 8) fg_class_kernel(FgArgs a, int tile_begin, int n_tiles) {
    constexpr int T = 16, NT = 128, HT = 8, NW = 4, kRec = kReduced ? 24 : 48;
    __shared__ FgClassSmem S;
    const int tid = threadIdx.x;
    const int c = blockIdx.y;
    const int I = a.interleave, cx = c % I, cy = c / I;
    const int vbase = c * a.per_class, cnt = a.per_class;
    const float hs = float(a.ism_size) * 0.5f;
    const unsigned char* src = kReduced ? a.reduced : reinterpret_cast<const unsigned char*>(a.vpl);
    const size_t bytes = (size_t)cnt * kRec;
    // checked build: a class slice outside the VPL buffer or larger than the staging buffer skips
    // the block (block-uniform, before any copy is issued)
    if (!MLGI_RANGE_OK(vbase, cnt, a.n_vpl) || !MLGI_RANGE_OK(0, bytes, sizeof(S.raw))) return;
    const bool use_tma = ((size_t)vbase * kRec) % 16 == 0 && bytes % 16 == 0;
    if (tid == 0) {
        mbar_init(&S.bar, 1);
        if (use_tma) {
            mbar_expect_tx(&S.bar, (uint32_t)bytes + a.test_extra_tx);
            tma_bulk_g2s(S.raw, src + (size_t)vbase * kRec, (uint32_t)bytes, &S.bar);
        }
    }
    if (!use_tma)
        for (size_t k = tid * 4; k < bytes; k += NT * 4)
            *reinterpret_cast<uint32_t*>(S.raw + k) = __ldg(reinterpret_cast<const uint32_t*>(src + (size_t)vbase * kRec + k));
    __syncthreads();
    if (use_tma) {
        const long long limit = a.wait_cycles > 0 ? a.wait_cycles : 1ll << 31;
        if (!__syncthreads_and(mbar_wait(&S.bar, 0, limit))) {  // block-uniform: flag, let the copy land, leave
            if (tid == 0) {
                atomicOr(a.status, kStatusTmaTimeout);
                if (a.test_extra_tx) mbar_complete_tx(&S.bar, a.test_extra_tx);
                mbar_wait(&S.bar, 0, 1ll << 31);
            }
            return;
        }
    }
    for (int k = tid; k < cnt; k += NT) {
        v3 p, n, f;
        derive_vpl<kReduced>(S.raw + (size_t)k * kRec, vbase + k, a, hs, S.v[k], p, n, f);
        S.cp[k] = make_float4(p.x, p.y, p.z, vpl_influence_r2(f, a.influence_cutoff));
        S.cn[k] = make_float4(n.x, n.y, n.z, 0.f);
    }
    __syncthreads();

    const int sw = (a.width + I - 1) / I, ntx = (sw + T - 1) / T;
    const int lane = tid & 31;
    int it = 0;
    for (int tile = tile_begin + blockIdx.x; tile < tile_begin + n_tiles; tile += gridDim.x, ++it) {
        const int tix = tile % ntx, tiy = tile / ntx;
        const int y = (tiy * T + tid / HT) * I + cy;
        const int x0 = (tix * T + 2 * (tid % HT)) * I + cx, x1 = x0 + I;
        const bool v0 = x0 < a.width && y < a.height, v1 = x1 < a.width && y < a.height;
        v3 w0, n0, w1, n1;
        float d0, d1;
        fg_pixel_setup<kNormalF16>(a, x0, y, v0, d0, n0);
        fg_pixel_setup<kNormalF16>(a, x1, y, v1, d1, n1);
        reconstruct_world2(a.inv_vp, x0, x1, y, a.width, a.height, a.inv_w, a.inv_h, d0, d1, pk(a.z_far * 0.0f), w0, w1);
        if (!v0) w0 = mk(0.f, 0.f, 0.f);
        if (!v1) w1 = mk(0.f, 0.f, 0.f);
        unsigned m0 = 0xFFFFFFFFu, m1 = 0xFFFFFFFFu;
        if (a.cull == 1) {
            // the half-space test against the warp's own box (a VPL it drops adds exactly nothing
            // to any of the warp's pixels, so the radiance is the per-tile cull's bit for bit), the
            // influence test against the tile's box (the culling rule the oracle restates)
            v3 bmin, bmax, wmin, wmax;
            fg_tile_box<NW>(w0, w1, v0, v1, S.box[it & 1], bmin, bmax, &wmin, &wmax);
            auto keep = [&](const int k) {
                if (k >= cnt) return false;
                const float4 cp = S.cp[k], cn = S.cn[k];
                const v3 p = mk(cp.x, cp.y, cp.z);
                return vpl_front(p, mk(cn.x, cn.y, cn.z), wmin, wmax) && vpl_near(p, cp.w, bmin, bmax);
            };
            m0 = __ballot_sync(0xffffffffu, keep(lane));
            m1 = cnt > 32 ? __ballot_sync(0xffffffffu, keep(32 + lane)) : 0u;
        }
        m0 &= cnt >= 32 ? 0xFFFFFFFFu : (1u << cnt) - 1u;
        m1 &= cnt >= 64 ? 0xFFFFFFFFu : cnt > 32 ? (1u << (cnt - 32)) - 1u : 0u;
        GatherPair<kAtlasF16, false> gp;
        gp.init(a, w0, n0, w1, n1, v0, v1, nullptr, nullptr);
        if (v0 || v1) {
            unsigned r0 = m0, r1 = m1;
            gp.gather(S.v, vbase, __popc(m0) + __popc(m1), [&]() {
                int k;
                if (r0) {
                    k = __ffs(r0) - 1;
                    r0 &= r0 - 1u;
                } else {
                    k = 32 + __ffs(r1) - 1;
                    r1 &= r1 - 1u;
                }
                return k;
            });
        }
        gp.store(a, y, x0, x1);
    }
}

// Tile rows [tr0, tr1): tiles are numbered row by row, so a band of tile rows is a contiguous
// range of tile indices starting at tile0.
static int sm_count() {
    static std::atomic<int> n[64];  // contexts on other threads may ask at the same time
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
    int v = n[dev].load(std::memory_order_relaxed);
    if (!v) {
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) cudaGetLastError();
        n[dev].store(v, std::memory_order_relaxed);
    }
    return v > 0 ? v : 152;
}

static cudaError_t launch_fg_class(const FgArgs& a, cudaStream_t s, int tr0, int tr1) {
    const int I = a.interleave;
    const int ntx = ((a.width + I - 1) / I + 15) / 16;
    const int tile_begin = tr0 * ntx, n_tiles = (tr1 - tr0) * ntx;
    // kFgClassBlocksPerSm 128-thread blocks per SM, spread evenly over the classes
    const int per_class = std::max(1, std::min(n_tiles, (kFgClassBlocksPerSm * sm_count() + I * I - 1) / (I * I)));
    const dim3 grid(per_class, I * I);
    const int sel = (a.reduced ? 4 : 0) | (a.atlas_f16 ? 2 : 0) | (a.normal_f16 ? 1 : 0);
    switch (sel) {
        case 0: fg_class_kernel<false, false, false><<<grid, 128, 0, s>>>(a, tile_begin, n_tiles); break;
        case 1: fg_class_kernel<false, false, true><<<grid, 128, 0, s>>>(a, tile_begin, n_tiles); break;
        case 2: fg_class_kernel<false, true, false><<<grid, 128, 0, s>>>(a, tile_begin, n_tiles); break;
        case 3: fg_class_kernel<false, true, true><<<grid, 128, 0, s>>>(a, tile_begin, n_tiles); break;
        case 4: fg_class_kernel<true, false, false><<<grid, 128, 0, s>>>(a, tile_begin, n_tiles); break;
        case 5: fg_class_kernel<true, false, true><<<grid, 128, 0, s>>>(a, tile_begin, n_tiles); break;
        case 6: fg_class_kernel<true, true, false><<<grid, 128, 0, s>>>(a, tile_begin, n_tiles); break;
        default: fg_class_kernel<true, true, true><<<grid, 128, 0, s>>>(a, tile_begin, n_tiles); break;
    }
    return cudaGetLastError();
}

template <int T>
static cudaError_t launch_fg_t(const FgArgs& args, cudaStream_t s, int tr0, int tr1) {
    const int I = args.interleave;
    const int sw = (args.width + I - 1) / I;
    const int ntx = (sw + T - 1) / T;
    if (tr1 <= tr0) return cudaSuccess;
    if (T == 16 && args.cull != 2 && args.per_class >= 1 && args.per_class <= kClassMaxVpls)
        return launch_fg_class(args, s, tr0, tr1);
    FgArgs a = args;
    a.tile0 = tr0 * ntx;
    const dim3 grid(ntx * (tr1 - tr0), I * I);
    const int sel = (a.reduced ? 4 : 0) | (a.atlas_f16 ? 2 : 0) | (a.normal_f16 ? 1 : 0);
    switch (sel) {
        case 0: fg_kernel<T, false, false, false><<<grid, T * T / 2, 0, s>>>(a); break;
        case 1: fg_kernel<T, false, false, true><<<grid, T * T / 2, 0, s>>>(a); break;
        case 2: fg_kernel<T, false, true, false><<<grid, T * T / 2, 0, s>>>(a); break;
        case 3: fg_kernel<T, false, true, true><<<grid, T * T / 2, 0, s>>>(a); break;
        case 4: fg_kernel<T, true, false, false><<<grid, T * T / 2, 0, s>>>(a); break;
        case 5: fg_kernel<T, true, false, true><<<grid, T * T / 2, 0, s>>>(a); break;
        case 6: fg_kernel<T, true, true, false><<<grid, T * T / 2, 0, s>>>(a); break;
        default: fg_kernel<T, true, true, true><<<grid, T * T / 2, 0, s>>>(a); break;
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
__global__ void __launch_bounds__(128, 8) batch_fg_kernel(BatchTable t) {
    __shared__ FgSmem<16> S;
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
        batch_fg_kernel<true><<<grid, 128, 0, s>>>(t);
    else
        batch_fg_kernel<false><<<grid, 128, 0, s>>>(t);
    return cudaGetLastError();
}

}  // namespace mlgi

MLGI_CHECK_UNIT(fg_kernels)
