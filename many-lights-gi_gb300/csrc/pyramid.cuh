// The fused pull-push pyramid: one block per ISM runs the ISM's whole pull-push with levels 1..L
// in shared memory, so that no pyramid level goes through global memory; the block reads the ISM's
// keys (the second time from L2) and writes its final depth once.
//   phase 1  a thread per level-2 texel loads the 4x4 keys below it (four 16-byte rows), pulls the
//            four level-1 texels and, from those in registers, the level-2 texel
//   phase 2  pull levels 3..L, then push L-1..1 in place, a level at a time
//   phase 3  push level 0 by 2x2 quads from level 1 and the keys into the output
// Follows pull.comp:20-126 and push.comp:44-165 as ImperfectShadowmap::pullpush
// (ImperfectShadowmap.cpp:121-182) drives them level by level. The coordinates that enter the
// displacement arithmetic are global coordinates of their level, as in the level-by-level passes,
// so every texel is bit-identical to theirs.
//
// The per-texel arithmetic is the same operations in the same order as pull_combine / push_output,
// arranged so that a warp issues few instructions per texel:
//  * Selects instead of branches. Adding a zero in place of a skipped term leaves every sum as the
//    shader's skip leaves it: a sum that starts at +0 never holds -0, and x + (+-0) == x otherwise.
//  * The fused pyramid runs only for far planes in [2^-20, 2^20] (else the four launches do), so
//    every sum it divides by a sample count or weight sum is +0, NaN or of magnitude within
//    [2^-100, 2^100], where the corrected reciprocal needs no range check, and the quotients of
//    pull level 1 are 0, Inf, NaN or normal.
//  * The push's radius test compares d2 = dx^2 + dy^2 with thresholds 2^-20 (relative) away from
//    the radius squared (sqrt_gt). A d2 within 2^-22 (relative) of the reference's d2 therefore
//    decides it the same way outside that band, so the fast test may form d2 with an FMA; inside
//    the band the quad is redone with the exact per-output code (push_output), which a warp meets
//    rarely.
// This file is part of ism_kernels.cu's translation unit (-fmad=false, IEEE division and square
// root) and uses its helpers.
#pragma once

// Shared tables of the fused pyramid, ahead of its levels.
struct PyramidTables {
    float2 key[256];     // per key radius byte b: (float(b) / 10, ((float(b) / 10) * 2) / zFar * 0.6)
    float rcp[20];       // RN(1 / n), n = 0..16 (0 for n = 0)
    uint32_t disp1[16];  // pull level 1: packHalf2x16 of the mean displacement of the valid samples of mask m
};
constexpr size_t kPyramidTableBytes = (sizeof(PyramidTables) + 15) & ~size_t(15);
// A block's shared memory at most: two blocks per SM (ISM edges up to 128).
constexpr size_t kPyramidSmemMax = 113 * 1024;

__device__ __forceinline__ int pyramid_offset(const int s, const int l) {  // float4s before level l >= 1
    int off = 0;
    for (int k = 1; k < l; ++k) off += (s >> k) * (s >> k);
    return off;
}

size_t pyramid_smem_bytes(int ism_size, int levels) {
    if (ism_size <= 0 || levels < 1 || levels > 16) return ~(size_t)0;
    size_t b = kPyramidTableBytes;
    for (int l = 1; l <= levels; ++l) b += (size_t)(ism_size >> l) * (ism_size >> l) * 16;
    return b;
}

bool pyramid_fits(int ism_size, int levels, float z_far) {
    return levels >= 2 && ism_size % 4 == 0 && pyramid_smem_bytes(ism_size, levels) <= kPyramidSmemMax &&
           z_far >= 0x1p-20f && z_far <= 0x1p+20f;
}

// ISM blocks the GPU holds at once: three per SM for edges up to 64, else two (the kernel forms
// below), times the current device's SMs (152 when it cannot be asked).
long long pyramid_wave(int ism_size) {
    constexpr int kMaxDevices = 64;
    static std::atomic<int> sms[kMaxDevices];  // contexts on other threads may ask at the same time
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        n = 152;
    } else if (!(n = sms[dev].load(std::memory_order_relaxed))) {
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) {
            cudaGetLastError();
            n = 152;
        }
        sms[dev].store(n, std::memory_order_relaxed);
    }
    return (long long)n * (ism_size > 64 ? 2 : 3);
}

// One block per ISM runs a launch of n_isms ISMs when the pyramid fits and the ISMs make at most
// one wave of blocks. Beyond a wave the per-level launches are faster, its middle levels being a
// chain of barrier-separated steps with few threads busy (GB300, ms for fused / per level:
// 64^2 ISMs 256: 0.035 / 0.045, 512: 0.058 / 0.057, 1024: 0.095 / 0.085, 4096: 0.366 / 0.262;
// 128^2 ISMs 256: 0.080 / 0.086, 1024: 0.253 / 0.245; 96^2 ISMs 1024: 0.158 / 0.150).
bool pyramid_fused(int ism_size, int levels, float z_far, long long n_isms) {
    return pyramid_fits(ism_size, levels, z_far) && n_isms <= pyramid_wave(ism_size);
}

// The form of a launch: one block per ISM wherever it fits (kPyrWhereFits), never
// (kPyrPerLevel), or by pyramid_fused for the launch's ISMs (kPyrByCount).
bool pyramid_launch_fused(const PullPushArgs& a) {
    if (a.pyr_form == kPyrPerLevel) return false;
    return a.pyr_form == kPyrWhereFits ? pyramid_fits(a.ism_size, a.levels, a.z_far)
                                       : pyramid_fused(a.ism_size, a.levels, a.z_far,
                                                       (long long)(a.row1 - a.row0) * a.grid_x);
}

__device__ __forceinline__ void fill_pyramid_tables(PyramidTables& T, const float z_far) {
    for (int b = threadIdx.x; b < 256; b += blockDim.x) {
        const float r = float(b) / 10.0f;
        T.key[b] = make_float2(r, (r * 2.0f) / z_far * 0.6f);
    }
    if (threadIdx.x < 20) T.rcp[threadIdx.x] = threadIdx.x == 0 || threadIdx.x > 16 ? 0.f : 1.0f / float(threadIdx.x);
    if (threadIdx.x < 16) {
        const unsigned m = threadIdx.x;
        float dax = 0.f, day = 0.f;
        int n = 0;
        for (int k = 0; k < 4; ++k) {
            if (!((m >> k) & 1u)) continue;
            dax = dax + (kPullOff[k][0] ? 0.25f : -0.25f);
            day = day + (kPullOff[k][1] ? 0.25f : -0.25f);
            ++n;
        }
        T.disp1[m] = n ? pack_half2(dax / float(n), day / float(n)) : 0u;  // IEEE quotients, as div_count4's
    }
}

// x / n for x in {+0, NaN} or 2^-100 <= |x| <= 2^100 and n = 1..16 with R = RN(1/n): the residual
// correction of div_corrected without its range check.
__device__ __forceinline__ float div_n_fast(const float x, const float n, const float R) {
    const float q = x * R;
    return fmaf(fmaf(-q, n, x), R, q);
}

// x / 3.14 for x in {0, Inf, NaN} or 2^-100 <= |x| <= 2^100 (div_314 without its range check).
__device__ __forceinline__ float div_314_fast(const float x) {
    const float R = 1.0f / 3.14f;
    const float q = x * R;
    const float r = fmaf(fmaf(-q, 3.14f, x), R, q);
    return x == __int_as_float(0x7f800000) ? x : r;
}

__device__ __forceinline__ uint32_t pack_half2_rn(const float a, const float b) {
    const __half2 h = __floats2half2_rn(a, b);  // a in the low half, b in the high, each rounded to nearest even
    return *reinterpret_cast<const uint32_t*>(&h);
}

#define MLGI_INF __int_as_float(0x7f800000)

// The combine of pull.comp:60-120 for samples with valid[k] set; kLevel1: the displacements are the
// level-1 constants (their mean comes from the table by the final valid mask).
template <bool kLevel1>
__device__ __forceinline__ float4 pull_combine_lean(const float (&d)[4], const float (&md)[4], const float (&r)[4],
                                                    const float (&dx)[4], const float (&dy)[4], const bool (&valid)[4],
                                                    const PyramidTables& T) {
    float m = MLGI_INF, maxDepth = 0.f;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        // an invalid sample enters as +Inf: it lowers no minimum, and any maxDepth it sets while the
        // minimum is still +Inf is replaced by the first valid sample's (depths are finite and not -0)
        const float dd = valid[k] ? d[k] : MLGI_INF;
        m = fminf(dd, m);
        maxDepth = m == dd ? md[k] : maxDepth;
    }
    float dAcc = 0.f, rAcc = 0.f, xAcc = 0.f, yAcc = 0.f, mv = 0.f;
    int n = 0;
    unsigned mask = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const bool v = valid[k] && !(d[k] > maxDepth);
        dAcc = dAcc + (v ? d[k] : 0.f);
        rAcc = rAcc + (v ? r[k] : 0.f);
        if (!kLevel1) {
            xAcc = xAcc + (v ? dx[k] : 0.f);
            yAcc = yAcc + (v ? dy[k] : 0.f);
        }
        mv = v ? fmaxf(mv, md[k]) : mv;  // gmax(mv, md): both finite and >= +0
        n += v;
        mask |= (unsigned)v << k;
    }
    const float fn = float(n), R = T.rcp[n];
    const uint32_t disp = kLevel1 ? T.disp1[mask] : pack_half2_rn(div_n_fast(xAcc, fn, R), div_n_fast(yAcc, fn, R));
    return n ? make_float4(div_n_fast(dAcc, fn, R), mv, div_n_fast(rAcc, fn, R), __uint_as_float(disp))
             : make_float4(1.0f, 0.f, 0.f, 0.f);
}

// Pull level 1 from four keys in kPullOff order (pull.comp's LEVEL_ZERO branch).
__device__ __forceinline__ float4 pull1_lean(const uint32_t (&key)[4], const PyramidTables& T, const float z_far,
                                             const float fs) {
    float d[4], md[4], r[4];
    bool valid[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float depth = float(key[k] >> 8) * 0x1p-24f;  // float(key >> 8) / (1 << 24), exactly
        const float2 t = T.key[key[k] & 0xFFu];
        d[k] = depth;
        md[k] = depth + t.y;
        const float distToCamera = depth * z_far;
        float radius = div_314_fast(t.x / distToCamera) * fs;
        radius = radius * 1.3f;
        r[k] = gmin(radius, 15.0f);
        // a key's depth is below 1; every sample's displacement length is RN(sqrt(0.125)), and
        // radius * 0.5 is exact
        valid[k] = !(0.3535533845424652f > r[k] * 0.5f);
    }
    return pull_combine_lean<true>(d, md, r, d, d, valid, T);
}

// Pull level l >= 2 at global texel (gox, goy) from its four level-(l-1) texels t[k] (kPullOff order).
__device__ __forceinline__ float4 pull_lean(const float4 (&t)[4], const int gox, const int goy, const float scale,
                                            const PyramidTables& T) {
    float d[4], md[4], r[4], dx[4], dy[4];
    bool valid[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float2 h = unpack_half2(__float_as_uint(t[k].w));
        d[k] = t[k].x;
        md[k] = t[k].y;
        r[k] = t[k].z;
        dx[k] = (float(2 * gox + kPullOff[k][0]) + 0.5f + h.x) / 2.0f - (float(gox) + 0.5f);
        dy[k] = (float(2 * goy + kPullOff[k][1]) + 0.5f + h.y) / 2.0f - (float(goy) + 0.5f);
        valid[k] = d[k] != 1.0f && !sqrt_gt(dx[k] * dx[k] + dy[k] * dy[k], r[k] * scale);
    }
    return pull_combine_lean<false>(d, md, r, dx, dy, valid, T);
}

// Per-coarse-texel terms of a push quad (see push_coarse).
struct PushTerm {
    float d, md, r, ax, ay, hi, lo;
    bool usable;  // depth != 1 (push.comp:88-93)
};

__device__ __forceinline__ PushTerm push_term(const float4 t, const float scale) {
    PushTerm c;
    const float2 h = unpack_half2(__float_as_uint(t.w));
    c.d = t.x;
    c.md = t.y;
    c.r = t.z;
    c.ax = h.x * 2.0f;
    c.ay = h.y * 2.0f;
    c.usable = t.x != 1.0f;
    const float rs = t.z * scale, p = rs * rs;
    const bool fast = rs > 0.f && p >= 1e-30f;  // else NaN thresholds: the band, decided exactly
    c.hi = fast ? p * 1.00000095367431640625f : __int_as_float(0x7fc00000);
    c.lo = fast ? p * 0.99999904632568359375f : __int_as_float(0x7fc00000);
    return c;
}

// Output (qx, qy) of a quad from its pull value `orig` (push.comp:95-161), with the fast radius
// test; `band` collects whether any usable coarse texel inside the output's ISM fell in the band
// (the caller then redoes the quad exactly). bx, by: the quad straddles the ISM's border in x, y.
template <bool kFull, int qx, int qy>
__device__ __forceinline__ float4 push_out_lean(const PushTerm (&c)[4], const bool bx, const bool by,
                                                const float4 orig, bool& band, const PyramidTables& T) {
    float w[4], dvx[4], dvy[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int kx = kPushOff[k][0], ky = kPushOff[k][1];
        const bool in = (kx == qx || !bx) && (ky == qy || !by) && c[k].usable;
        dvx[k] = (float(2 * kx - qx) - 0.5f) + c[k].ax;  // (ctx - (px + 0.5)) + 2 dx, see push_texel
        dvy[k] = (float(2 * ky - qy) - 0.5f) + c[k].ay;
        const float d2 = fmaf(dvx[k], dvx[k], dvy[k] * dvy[k]);  // within 2^-22 of the reference's d2
        const bool far = d2 > c[k].hi;
        band = band || (in && !far && !(d2 < c[k].lo));
        w[k] = in && !far ? float((kx == qx ? 3 : 1) * (ky == qy ? 3 : 1)) : 0.f;
    }
    float m = 9001.0f, maxDepth = 0.f;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float dd = w[k] != 0.f ? c[k].d : MLGI_INF;  // a zero weight takes no part (depths are finite)
        m = fminf(dd, m);
        maxDepth = m == dd ? c[k].md : maxDepth;
    }
    float wsum = 0.f;
    bool occluded = false;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        w[k] = c[k].d > maxDepth ? 0.f : w[k];
        wsum = wsum + w[k];
        occluded = occluded || (w[k] != 0.f && orig.x > c[k].md);
    }
    // the sums start with their first term: +0 plus a term that is not -0 is that term, and a
    // -0 term (a negative displacement times a zero weight) only matters when every weight is 0
    float depthAcc = c[0].d * w[0], maxDepthAcc = 0.f, radiusAcc = 0.f, dax = 0.f, day = 0.f;
    if (kFull) {
        maxDepthAcc = c[0].md * w[0];
        radiusAcc = c[0].r * w[0];
        dax = dvx[0] * w[0];
        day = dvy[0] * w[0];
    }
#pragma unroll
    for (int k = 1; k < 4; ++k) {
        depthAcc = depthAcc + c[k].d * w[k];
        if (kFull) {
            maxDepthAcc = maxDepthAcc + c[k].md * w[k];
            radiusAcc = radiusAcc + c[k].r * w[k];
            dax = dax + dvx[k] * w[k];
            day = day + dvy[k] * w[k];
        }
    }
    const bool replace = wsum > 0.f && (orig.x == 1.0f || occluded);
    const float R = T.rcp[(int)wsum];
    float4 r = orig;
    r.x = replace ? div_n_fast(depthAcc, wsum, R) : orig.x;
    if (kFull) {
        r.y = replace ? div_n_fast(maxDepthAcc, wsum, R) : orig.y;
        r.z = replace ? div_n_fast(radiusAcc, wsum, R) : orig.z;
        r.w = replace ? __uint_as_float(pack_half2_rn(div_n_fast(dax, wsum, R), div_n_fast(day, wsum, R))) : orig.w;
    }
    return r;
}

// The exact per-output push of a quad (push_coarse + push_output), for quads whose fast radius test
// met the band. Out of line, so that only this rare path pays for the registers it needs.
__device__ __noinline__ void push_quad_exact_smem(float4* same, const float4* coarse, const int el, const int gx,
                                                  const int gy, const float scale) {
    const int sc = el >> 1;
    PushCoarse C;
    push_coarse(coarse, sc, sc, sc, gx, gy, scale, C);
    const bool bx = gx == 0 || gx == sc, by = gy == 0 || gy == sc;
    const int x0 = 2 * gx - 1, y0 = 2 * gy - 1;
    const int n = el * el, i0 = y0 * el + x0, i1 = (y0 + 1) * el + x0;  // used only where inside
    if (y0 >= 0 && x0 >= 0) same[MLGI_IX(i0, n)] = push_output<true, 0, 0>(C, bx, by, same[MLGI_IX(i0, n)]);
    if (y0 >= 0 && x0 + 1 < el) same[MLGI_IX(i0 + 1, n)] = push_output<true, 1, 0>(C, bx, by, same[MLGI_IX(i0 + 1, n)]);
    if (y0 + 1 < el && x0 >= 0) same[MLGI_IX(i1, n)] = push_output<true, 0, 1>(C, bx, by, same[MLGI_IX(i1, n)]);
    if (y0 + 1 < el && x0 + 1 < el)
        same[MLGI_IX(i1 + 1, n)] = push_output<true, 1, 1>(C, bx, by, same[MLGI_IX(i1 + 1, n)]);
}

__device__ __noinline__ float4 push_quad_exact_l0(const float4* lv1, const int e1, const int gx, const int gy,
                                                  const float4 keyd) {
    PushCoarse C;
    push_coarse(lv1, e1, e1, e1, gx, gy, 1.0f, C);
    const bool bx = gx == 0 || gx == e1, by = gy == 0 || gy == e1;
    return make_float4(push_output<false, 0, 0>(C, bx, by, make_float4(keyd.x, 0.f, 0.f, 0.f)).x,
                       push_output<false, 1, 0>(C, bx, by, make_float4(keyd.y, 0.f, 0.f, 0.f)).x,
                       push_output<false, 0, 1>(C, bx, by, make_float4(keyd.z, 0.f, 0.f, 0.f)).x,
                       push_output<false, 1, 1>(C, bx, by, make_float4(keyd.w, 0.f, 0.f, 0.f)).x);
}

// Push level l >= 1 of quad (gx, gy) of an ISM in shared memory, in place: `same` is the level
// (edge el, pull values in, push values out), `coarse` the pushed level l + 1 (edge el / 2). A quad
// on the ISM's border (gx or gy 0 or el / 2) has outputs in this ISM on one side only.
__device__ __forceinline__ void push_quad_smem(float4* same, const float4* coarse, const int el, const int gx,
                                               const int gy, const float scale, const PyramidTables& T) {
    const int sc = el >> 1;
    PushTerm c[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int cx = min(max(gx - 1 + kPushOff[k][0], 0), sc - 1), cy = min(max(gy - 1 + kPushOff[k][1], 0), sc - 1);
        c[k] = push_term(coarse[MLGI_IX(cy * sc + cx, sc * sc)], scale);
    }
    const bool bx = gx == 0 || gx == sc, by = gy == 0 || gy == sc;
    const int x0 = 2 * gx - 1, y0 = 2 * gy - 1;
    const bool ok00 = y0 >= 0 && x0 >= 0, ok10 = y0 >= 0 && x0 + 1 < el, ok01 = y0 + 1 < el && x0 >= 0,
               ok11 = y0 + 1 < el && x0 + 1 < el;
    // clamped indices: an output outside the ISM is neither stored nor lets its value matter
    const int i00 = max(y0, 0) * el + max(x0, 0), i10 = max(y0, 0) * el + min(x0 + 1, el - 1),
              i01 = min(y0 + 1, el - 1) * el + max(x0, 0), i11 = min(y0 + 1, el - 1) * el + min(x0 + 1, el - 1);
    const int n = el * el;
    const float4 o00 = same[MLGI_IX(i00, n)], o10 = same[MLGI_IX(i10, n)], o01 = same[MLGI_IX(i01, n)],
                 o11 = same[MLGI_IX(i11, n)];
    bool band = false;
    const float4 r00 = push_out_lean<true, 0, 0>(c, bx, by, o00, band, T);
    const float4 r10 = push_out_lean<true, 1, 0>(c, bx, by, o10, band, T);
    const float4 r01 = push_out_lean<true, 0, 1>(c, bx, by, o01, band, T);
    const float4 r11 = push_out_lean<true, 1, 1>(c, bx, by, o11, band, T);
    if (band) {  // a radius test within 2^-20 of the radius: the exact per-output form
        push_quad_exact_smem(same, coarse, el, gx, gy, scale);
        return;
    }
    if (ok00) same[MLGI_IX(i00, n)] = r00;
    if (ok10) same[MLGI_IX(i10, n)] = r10;
    if (ok01) same[MLGI_IX(i01, n)] = r01;
    if (ok11) same[MLGI_IX(i11, n)] = r11;
}

template <int NT>
__device__ __forceinline__ void pyramid_ism(const PullPushArgs& a, const int ism, unsigned char* smem) {
    PyramidTables& T = *reinterpret_cast<PyramidTables*>(smem);
    float4* pyr = reinterpret_cast<float4*>(smem + kPyramidTableBytes);
    const int s = a.ism_size, L = a.levels, e1 = s >> 1, e2 = s >> 2;
    const int im = MLGI_IX(ism, a.grid_x * a.grid_y), ix = im % a.grid_x, iy = im / a.grid_x;
    const int tid = threadIdx.x;
    fill_pyramid_tables(T, a.z_far);
    __syncthreads();
    float4* const lv1 = pyr;
    float4* const lv2 = pyr + e1 * e1;
    const float fs = float(s), z_far = a.z_far;
    const int aw = a.atlas_w;
#ifdef MLGI_CHECKS
    {  // the whole pyramid inside the block's shared memory: its last texel
        uint32_t dyn;
        asm volatile("mov.u32 %0, %%dynamic_smem_size;" : "=r"(dyn));
        (void)MLGI_IX(pyramid_offset(s, L + 1) - 1, dyn > kPyramidTableBytes ? (dyn - kPyramidTableBytes) / 16 : 0);
    }
#endif
    const size_t nk = (size_t)aw * a.atlas_h - 3;  // a row of four keys: its first

    // phase 1: a thread per level-2 texel, in row-major order
    for (int uy = tid / e2, ux = tid - (tid / e2) * e2; uy < e2;) {
        const int gx2 = ix * e2 + ux, gy2 = iy * e2 + uy;  // global level-2 texel
        const size_t kr = (size_t)(4 * gy2) * aw + 4 * gx2;
        uint4 r[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) r[j] = __ldg(reinterpret_cast<const uint4*>(a.keys + MLGI_IX(kr + (size_t)j * aw, nk)));
        float4 t[4];  // level-1 texels (2 gx2, 2 gy2) + kPullOff[k]
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int kx = kPullOff[k][0], ky = kPullOff[k][1];
            const uint4 ra = r[2 * ky], rb = r[2 * ky + 1];
            const uint32_t key[4] = {kx ? ra.z : ra.x, kx ? rb.z : rb.x, kx ? ra.w : ra.y, kx ? rb.w : rb.y};
            t[k] = pull1_lean(key, T, z_far, fs);
            lv1[MLGI_IX((2 * uy + ky) * e1 + 2 * ux + kx, e1 * e1)] = t[k];
        }
        lv2[MLGI_IX(uy * e2 + ux, e2 * e2)] = pull_lean(t, gx2, gy2, 0.25f, T);
        ux += NT;  // the texel NT further in row-major order (NT may exceed e2)
        while (ux >= e2) {
            ux -= e2;
            ++uy;
        }
    }
    __syncthreads();

    // phase 2: pull 3..L, push L-1..1 (in place: a texel reads only its own pull value)
    for (int l = 3; l <= L; ++l) {
        const int el = s >> l;
        const float4* in = pyr + pyramid_offset(s, l - 1);
        float4* out = pyr + pyramid_offset(s, l);
        const float scale = pow2neg(l);
        for (int i = tid; i < el * el; i += NT) {
            const int ly = i / el, lx = i - ly * el;
            float4 t4[4];
#pragma unroll
            for (int k = 0; k < 4; ++k)
                t4[k] = in[MLGI_IX((2 * ly + kPullOff[k][1]) * 2 * el + 2 * lx + kPullOff[k][0], 4 * el * el)];
            out[i] = pull_lean(t4, el * ix + lx, el * iy + ly, scale, T);
        }
        __syncthreads();
    }
    for (int l = L - 1; l >= 1; --l) {
        const int el = s >> l, nq = (el >> 1) + 1;
        const float4* coarse_lvl = pyr + pyramid_offset(s, l + 1);
        float4* same = pyr + pyramid_offset(s, l);
        const float scale = pow2neg(l);
        for (int i = tid; i < nq * nq; i += NT) {
            const int gy = i / nq, gx = i - gy * nq;
            push_quad_smem(same, coarse_lvl, el, gx, gy, scale, T);
        }
        __syncthreads();
    }

    // phase 3: level 0 by quads (e1 + 1 per axis, ISM-local)
    const int nq = e1 + 1;
    for (int gy = tid / nq, gx = tid - (tid / nq) * nq; gy < nq;) {
        PushTerm c[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int cx = min(max(gx - 1 + kPushOff[k][0], 0), e1 - 1), cy = min(max(gy - 1 + kPushOff[k][1], 0), e1 - 1);
            c[k] = push_term(lv1[MLGI_IX(cy * e1 + cx, e1 * e1)], 1.0f);
        }
        const bool bx = gx == 0 || gx == e1, by = gy == 0 || gy == e1;
        const int x0 = 2 * gx - 1, y0 = 2 * gy - 1;  // ISM-local
        const bool okx0 = x0 >= 0, okx1 = x0 + 1 < s, oky0 = y0 >= 0, oky1 = y0 + 1 < s;
        // global texel offsets of the four outputs, clamped into the ISM (a clamped one is not stored)
        const uint32_t cx0 = (uint32_t)(ix * s + max(x0, 0)), cx1 = (uint32_t)(ix * s + min(x0 + 1, s - 1));
        const uint32_t ry0 = (uint32_t)(iy * s + max(y0, 0)) * (uint32_t)aw;
        const uint32_t ry1 = (uint32_t)(iy * s + min(y0 + 1, s - 1)) * (uint32_t)aw;
        const float k00 = key_depth(a, ry0 + cx0), k10 = key_depth(a, ry0 + cx1);
        const float k01 = key_depth(a, ry1 + cx0), k11 = key_depth(a, ry1 + cx1);
        bool band = false;
        float r00 = push_out_lean<false, 0, 0>(c, bx, by, make_float4(k00, 0.f, 0.f, 0.f), band, T).x;
        float r10 = push_out_lean<false, 1, 0>(c, bx, by, make_float4(k10, 0.f, 0.f, 0.f), band, T).x;
        float r01 = push_out_lean<false, 0, 1>(c, bx, by, make_float4(k01, 0.f, 0.f, 0.f), band, T).x;
        float r11 = push_out_lean<false, 1, 1>(c, bx, by, make_float4(k11, 0.f, 0.f, 0.f), band, T).x;
        if (band) {  // a radius test within 2^-20 of the radius: the exact per-output form
            const float4 e = push_quad_exact_l0(lv1, e1, gx, gy, make_float4(k00, k10, k01, k11));
            r00 = e.x;
            r10 = e.y;
            r01 = e.z;
            r11 = e.w;
        }
        if (oky0 && okx0) store_depth(a, ry0 + cx0, r00);
        if (oky0 && okx1) store_depth(a, ry0 + cx1, r10);
        if (oky1 && okx0) store_depth(a, ry1 + cx0, r01);
        if (oky1 && okx1) store_depth(a, ry1 + cx1, r11);
        gx += NT;
        while (gx >= nq) {
            gx -= nq;
            ++gy;
        }
    }
}

// Bounds-checked build: the lean middle pass's last level texel (float4 index `last` after the
// tables) lies inside the block's dynamic shared memory.
__device__ __forceinline__ void check_lean_smem(const int last) {
#ifdef MLGI_CHECKS
    uint32_t dyn;
    asm volatile("mov.u32 %0, %%dynamic_smem_size;" : "=r"(dyn));
    (void)MLGI_IX(last, dyn > kPyramidTableBytes ? (dyn - kPyramidTableBytes) / 16 : 0);
#else
    (void)last;
#endif
}

// Far planes for which the lean arithmetic above is exact (its range argument, in the header).
__host__ __device__ __forceinline__ bool pyramid_lean_range(const float z_far) {
    return z_far >= 0x1p-20f && z_far <= 0x1p+20f;
}

// The per-level form's middle pass (pullmid_kernel) with the lean arithmetic: ISM `ism`'s levels
// 2..L in shared memory after the tables; level 2 pulled from the lv1 scratch, levels 3..L pulled,
// L-1..2 pushed back by 2x2 quads, and the pushed level 2 written to the lv2 scratch. Bit-identical
// to pullmid_ism's per-texel forms (the same operations in the same order, see the header), in
// fewer instructions: the quad's four coarse texels and their terms serve its four outputs. Far
// planes in pyramid_lean_range only.
__device__ __forceinline__ void pullmid_lean_ism(const PullPushArgs& a, const int ism, unsigned char* smem) {
    PyramidTables& T = *reinterpret_cast<PyramidTables*>(smem);
    float4* const base = reinterpret_cast<float4*>(smem + kPyramidTableBytes);
    __syncthreads();  // the previous ISM's use of smem is over
    // levels >= 2 read only the reciprocal table (the key and displacement tables serve level 1)
    if (threadIdx.x < 20) T.rcp[threadIdx.x] = threadIdx.x == 0 || threadIdx.x > 16 ? 0.f : 1.0f / float(threadIdx.x);
    __syncthreads();
    const int s = a.ism_size, L = a.levels, nt = blockDim.x, tid = threadIdx.x;
    const int im = MLGI_IX(ism, a.grid_x * a.grid_y), ix = im % a.grid_x, iy = im / a.grid_x;
    auto lvl = [&](const int l) { return base + (pyramid_offset(s, l) - pyramid_offset(s, 2)); };  // l >= 2
    check_lean_smem(pyramid_offset(s, L + 1) - pyramid_offset(s, 2) - 1);
    {  // level 2 from lv1
        const int e2 = s >> 2, w1 = a.atlas_w >> 1;
        const size_t n1 = (size_t)w1 * (a.atlas_h >> 1);
        float4* const out = lvl(2);
        for (int i = tid; i < e2 * e2; i += nt) {
            const int ly = i / e2, lx = i - ly * e2, gox = ix * e2 + lx, goy = iy * e2 + ly;
            float4 t4[4];
#pragma unroll
            for (int k = 0; k < 4; ++k)
                t4[k] = a.lv1[MLGI_IX((size_t)(2 * goy + kPullOff[k][1]) * w1 + 2 * gox + kPullOff[k][0], n1)];
            out[i] = pull_lean(t4, gox, goy, 0.25f, T);
        }
        __syncthreads();
    }
    for (int l = 3; l <= L; ++l) {
        const int el = s >> l;
        const float4* in = lvl(l - 1);
        float4* out = lvl(l);
        const float scale = pow2neg(l);
        for (int i = tid; i < el * el; i += nt) {
            const int ly = i / el, lx = i - ly * el;
            float4 t4[4];
#pragma unroll
            for (int k = 0; k < 4; ++k)
                t4[k] = in[MLGI_IX((2 * ly + kPullOff[k][1]) * 2 * el + 2 * lx + kPullOff[k][0], 4 * el * el)];
            out[i] = pull_lean(t4, el * ix + lx, el * iy + ly, scale, T);
        }
        __syncthreads();
    }
    for (int l = L - 1; l >= 2; --l) {
        const int el = s >> l, nq = (el >> 1) + 1;
        const float4* coarse_lvl = lvl(l + 1);
        float4* same = lvl(l);
        const float scale = pow2neg(l);
        for (int i = tid; i < nq * nq; i += nt) {
            const int gy = i / nq, gx = i - gy * nq;
            push_quad_smem(same, coarse_lvl, el, gx, gy, scale, T);
        }
        __syncthreads();
    }
    const int e2 = s >> 2, w2 = a.atlas_w >> 2;
    const float4* l2 = lvl(2);
    for (int i = tid; i < e2 * e2; i += nt)
        a.lv2[MLGI_IX((size_t)(iy * e2 + i / e2) * w2 + ix * e2 + i % e2, (size_t)w2 * (a.atlas_h >> 2))] = l2[i];
}

// Threads per block: kPyrBigThreads for ISM edges above 64 (two blocks per SM, as their shared
// memory allows; 384 threads leave 80 registers a thread, measured at C2: 0.256 ms against 0.274 ms
// with 512 threads at 64 registers and 0.276 ms with 256), kPyrSmallThreads for smaller ones with
// at least three blocks per SM (85 registers: 64^2 ISMs in 0.0945 ms against 0.0955 with four
// blocks at 64 registers and 0.108 with two).
constexpr int kPyrBigThreads = 384, kPyrSmallThreads = 256;

template <int NT, int kMinBlocks>
__global__ void __launch_bounds__(NT, kMinBlocks) pyramid_kernel(PullPushArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    pyramid_ism<NT>(a, a.row0 * a.grid_x + blockIdx.x, smem);
}

// Raises the kernels' dynamic shared-memory limit on the current device (once per device).
static cudaError_t pyramid_prepare() {
    constexpr int kMaxDevices = 64;
    static bool done[kMaxDevices] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess && dev >= 0 && dev < kMaxDevices && done[dev]) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(pyramid_kernel<kPyrBigThreads, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kPyramidSmemMax);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(pyramid_kernel<kPyrSmallThreads, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kPyramidSmemMax);
    if (e == cudaSuccess && dev >= 0 && dev < kMaxDevices) done[dev] = true;
    return e;
}

static void launch_pyramid(const PullPushArgs& a, cudaStream_t s) {
    const int isms = (a.row1 - a.row0) * a.grid_x;
    const size_t smem = pyramid_smem_bytes(a.ism_size, a.levels);
    if (a.ism_size > 64)
        pyramid_kernel<kPyrBigThreads, 2><<<isms, kPyrBigThreads, smem, s>>>(a);
    else
        pyramid_kernel<kPyrSmallThreads, 3><<<isms, kPyrSmallThreads, smem, s>>>(a);
}
