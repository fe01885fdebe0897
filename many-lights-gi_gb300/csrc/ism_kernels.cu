// VPL processing, ISM point splat and the fused pull-push pyramid.
//
// This translation unit is compiled with -fmad=false and IEEE division/square root so that its
// FP32 results are word-for-word those of the reference shaders' arithmetic in GLSL order:
//   vpl_process_kernel  <- data/shaders/gi/vpl_processor.comp:41-72
//   ism_splat_kernel    <- data/shaders/ism/ism.comp:54-139
//   pullpush_kernel     <- data/shaders/ism/pull.comp:20-126 and push.comp:44-165, as driven by
//                          ImperfectShadowmap::pullpush (ImperfectShadowmap.cpp:121-182)
#include <cuda_runtime.h>

#include "gi_device.cuh"
#include "kernels.h"

namespace mlgi {

// ---------------------------------------------------------------------------------------------
// VPL processor: one thread per VPL. Regular RSM sample -> unproject -> flux -> 10:10:10 normal
// round trip -> optional shuffled slot.
__device__ __forceinline__ void vpl_one(const VplArgs& a, const uint32_t idx) {
    if (idx >= (uint32_t)a.n) return;
    const uint32_t tcx = (idx % a.ax) * (uint32_t)a.rsm_w / a.ax;
    const uint32_t tcy = (idx / a.ax) * (uint32_t)a.rsm_h / a.ay;
    const float tfx = float(tcx) / float(a.rsm_w);
    const float tfy = float(tcy) / float(a.rsm_h);
    v3 diffuse = mk(0.f, 0.f, 0.f);
    uint32_t nb = 0;
    float d = 0.f;
    if (tcx < (uint32_t)a.rsm_w && tcy < (uint32_t)a.rsm_h) {  // texelFetch out of range reads zero
        const size_t t = (size_t)tcy * a.rsm_w + tcx;
        const uint32_t dw = __ldg(a.diffuse + t);
        diffuse = mk(float(dw & 0xFFu) / 255.0f, float((dw >> 8) & 0xFFu) / 255.0f, float((dw >> 16) & 0xFFu) / 255.0f);
        nb = __ldg(a.normal + t);
        d = __ldg(a.depth + t);
    }
    const v3 normal = mk(float(nb & 0x3FFu) / 1023.0f * 2.0f - 1.0f, float((nb >> 10) & 0x3FFu) / 1023.0f * 2.0f - 1.0f,
                         float((nb >> 20) & 0x3FFu) / 1023.0f * 2.0f - 1.0f);
    // mat4 * vec4(tfx, tfy, d, 1): ((c0*x + c1*y) + c2*z) + c3*w
    const float* m = a.inv_bpv;
    float w4[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) w4[r] = ((m[r] * tfx + m[4 + r] * tfy) + m[8 + r] * d) + m[12 + r] * 1.0f;
    const v3 pos = mk(w4[0] / w4[3], w4[1] / w4[3], w4[2] / w4[3]);
    const v3 color = diffuse * a.intensity;
    const uint32_t ri = a.perm ? (uint32_t)__ldg(a.perm + idx) : idx;
    const uint32_t pn = pack3SN(normal);
    const v3 un = unpack3SN(pn);
    a.vpl[3 * ri + 0] = make_float4(pos.x, pos.y, pos.z, 0.f);
    a.vpl[3 * ri + 1] = make_float4(un.x, un.y, un.z, 0.f);
    a.vpl[3 * ri + 2] = make_float4(color.x, color.y, color.z, 0.f);
    a.packed[ri] = make_float4(pos.x, pos.y, pos.z, __uint_as_float(pn));
    if (a.reduced) {
        // float pos[3], half normal[3], bfloat16 flux[3]
        uint32_t* r = reinterpret_cast<uint32_t*>(a.reduced + 24 * (size_t)ri);
        const uint32_t hx = __half_as_ushort(__float2half_rn(un.x));
        const uint32_t hy = __half_as_ushort(__float2half_rn(un.y));
        const uint32_t hz = __half_as_ushort(__float2half_rn(un.z));
        const uint32_t br = __bfloat16_as_ushort(__float2bfloat16_rn(color.x));
        const uint32_t bg = __bfloat16_as_ushort(__float2bfloat16_rn(color.y));
        const uint32_t bb = __bfloat16_as_ushort(__float2bfloat16_rn(color.z));
        reinterpret_cast<uint2*>(r)[0] = make_uint2(__float_as_uint(pos.x), __float_as_uint(pos.y));
        reinterpret_cast<uint2*>(r)[1] = make_uint2(__float_as_uint(pos.z), hx | (hy << 16));
        reinterpret_cast<uint2*>(r)[2] = make_uint2(hz | (br << 16), bg | (bb << 16));
    }
}

__global__ void __launch_bounds__(64) vpl_process_kernel(VplArgs a) { vpl_one(a, blockIdx.x * 64u + threadIdx.x); }

cudaError_t launch_vpl_process(const VplArgs& a, cudaStream_t s) {
    if (a.n <= 0) return cudaSuccess;
    vpl_process_kernel<<<(a.n + 63) / 64, 64, 0, s>>>(a);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------
// Atlas clear to 0xFFFFFFFF (ImperfectShadowmap.cpp:212), 16-byte stores.
__global__ void ism_clear_kernel(uint4* p, size_t n4) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (; i < n4; i += stride) p[i] = make_uint4(0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu);
}

cudaError_t launch_ism_clear(uint32_t* keys, size_t n, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    if ((n & 3) || (reinterpret_cast<uintptr_t>(keys) & 15)) return cudaMemsetAsync(keys, 0xFF, n * 4, s);
    const size_t n4 = n / 4;
    int blocks = (int)std::min<size_t>((n4 + 255) / 256, 152 * 16);
    ism_clear_kernel<<<blocks, 256, 0, s>>>(reinterpret_cast<uint4*>(keys), n4);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------
// ISM splat: one block per bucket. The 16 VPLs the bucket tests (ids wg..wg+15 mod N) are cached
// in shared memory together with their unpacked normals and lookAtRH rows, which are computed
// once per block with the same operations the shader repeats per point (so the values are
// identical). Each point keeps the first <= 4 VPLs that pass the two-sided hemisphere cull and
// atomicMin's its key into their paraboloid ISMs.
constexpr int kSplatThreads = 256;

struct SplatSmem {
    float4 pos[16], n[16];  // xyz used; float4 for 16-byte shared loads
    v3 s[16], u[16];
    float ism[16];
};

// Bucket wg (one block of kSplatThreads threads).
__device__ __forceinline__ void splat_bucket(const SplatArgs& a, const int wg, SplatSmem& S) {
    __syncthreads();  // the previous bucket's use of S is over
    const int vplCount = a.vpl_end - a.vpl_start;
    if (a.points_only_scaled && wg > vplCount) return;
    if (threadIdx.x < 16) {
        int index = (wg + (int)threadIdx.x) % a.n_vpl;
        if (a.points_only_scaled) {
            index %= vplCount;
            index += a.vpl_start;
        }
        const float4 pk = a.packed[index];
        const v3 n = unpack3SN(__float_as_uint(pk.w));
        v3 s, u;
        look_at_rows(n, s, u);
        S.pos[threadIdx.x] = make_float4(pk.x, pk.y, pk.z, 0.f);
        S.n[threadIdx.x] = make_float4(n.x, n.y, n.z, 0.f);
        S.s[threadIdx.x] = s;
        S.u[threadIdx.x] = u;
        S.ism[threadIdx.x] = a.scale_isms ? float(index) - float(a.vpl_start) : float(index);
    }
    __syncthreads();

    const uint32_t cnt = __ldg(a.counts + wg);
    const float4* bucket = a.points + (int64_t)wg * a.bucket_stride;
    const float fw = float(a.atlas_w), fh = float(a.atlas_h), fgx = float(a.gx), fgy = float(a.gy);
    for (uint32_t j = threadIdx.x; j < cnt; j += kSplatThreads) {
        const float4 pt = __ldg(bucket + j);
        const v3 position = mk(pt.x, pt.y, pt.z);
        const uint32_t nr = __float_as_uint(pt.w);
        const v3 pn = mk(float(nr & 0xFFu) / 255.0f * 2.0f - 1.0f, float((nr >> 8) & 0xFFu) / 255.0f * 2.0f - 1.0f,
                         float((nr >> 16) & 0xFFu) / 255.0f * 2.0f - 1.0f);
        const float pointRadius = float(nr >> 24) / 255.0f * 25.0f;
        const uint32_t rbyte = f2u(pointRadius * 10.0f / 2.0f);  // / sqrt(maxVplCollectCount)
        // gather up to 4 VPLs that pass the two-sided cull (ism.comp:93-107), as 4-bit indices
        uint32_t used = 0;
        int found = 0;
#pragma unroll
        for (int i = 0; i < 16; ++i) {
            const float4 vp = S.pos[i], vn = S.n[i];
            const v3 rel = position - mk(vp.x, vp.y, vp.z);
            const bool cull = dot(mk(vn.x, vn.y, vn.z), rel) < 0.0f || dot(pn, -rel) < 0.0f;
            if (!cull && found < 4) {
                used |= (uint32_t)i << (4 * found);
                ++found;
            }
        }
        // for each found VPL, project and atomicMin (ism.comp:112-137)
        for (int k = 0; k < found; ++k) {
            const int i = (used >> (4 * k)) & 15;
            const float4 vp = S.pos[i], vn = S.n[i];
            const v3 rel = position - mk(vp.x, vp.y, vp.z);
            // paraboloid_project(rel, length(rel), n, zFar, ismIndex, grid, preserveSign = true)
            const float dist = length(rel);
            const v3 n = mk(vn.x, vn.y, vn.z);
            float vx = dot(S.s[i], rel);
            float vy = dot(S.u[i], rel);
            float vz = ((-n.x) * rel.x + (-n.y) * rel.y) + (-n.z) * rel.z;
            const float signOfV = gsign(vz);
            vx = vx / dist;
            vy = vy / dist;
            vz = vz / dist;
            vz = 1.0f - vz;
            vx = vx / vz;
            vy = vy / vz;
            vz = dist / a.z_far;
            vz = vz * -signOfV;
            vx = (vx + 1.0f) / 2.0f;
            vy = (vy + 1.0f) / 2.0f;
            const float ismIndex = S.ism[i];
            const float ty = float(f2i(ismIndex / fgx));
            const int tx = f2i(ismIndex - ty * fgx);
            vx = vx + float(tx);
            vy = vy + float(f2i(ty));
            vx = vx / fgx;
            vy = vy / fgy;
            vx = vx * fw;
            vy = vy * fh;
            vz = vz * 16777216.0f;
            const uint32_t key = (f2u(vz) << 8) | rbyte;
            const int px = f2i(vx), py = f2i(vy);
            if (px < 0 || py < 0 || px >= a.atlas_w || py >= a.atlas_h) continue;  // image op out of range: no-op
            atomicMin(a.keys + (size_t)py * a.atlas_w + px, key);
        }
    }
}

__global__ void __launch_bounds__(kSplatThreads) ism_splat_kernel(SplatArgs a) {
    __shared__ SplatSmem S;
    splat_bucket(a, blockIdx.x, S);
}

cudaError_t launch_ism_splat(const SplatArgs& a, cudaStream_t s) {
    if (a.n_groups <= 0) return cudaSuccess;
    ism_splat_kernel<<<a.n_groups, kSplatThreads, 0, s>>>(a);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------
// Fused pull-push: one block per ISM. Pull levels and push levels never mix texels of different
// ISMs (2x2 pulls stay inside an ISM because its edge is divisible by 2^levels, and push gives
// weight 0 to every coarse texel across an ISM border), so a whole ISM's pyramid lives in shared
// memory: keys (level 0) plus RGBA texels of levels 1..L. Push level l overwrites pull level l
// in place (a push texel reads only its own pull texel at that level). Coordinates entering the
// displacement arithmetic are global atlas coordinates, as in the level-by-level shaders.
constexpr int kPullPushThreads = 512;
constexpr size_t kPullPushTableBytes = 2 * 256 * sizeof(float);  // key-byte tables, see below

__device__ __forceinline__ float pow2neg(int level) { return __int_as_float((127 - level) << 23); }

// x / n for the sample counts and weight sums that occur (n >= 1). Division by a power of two is
// exact, so it equals the multiply by the reciprocal bit for bit; other n use IEEE division.
__device__ __forceinline__ float div_count(float x, int n) {
    switch (n) {
        case 1: return x;
        case 2: return x * 0.5f;
        case 4: return x * 0.25f;
        case 8: return x * 0.125f;
        case 16: return x * 0.0625f;
        default: return x / float(n);
    }
}

// Shared memory: two 256-entry tables indexed by the key's radius byte b, then levels 1..L.
//   s_rad[b] = float(b) / 10                          (pull.comp:39)
//   s_mdo[b] = ((float(b) / 10) * 2) / zFar * 0.6     (the maxDepth offset of pull.comp:57)
// Each entry is computed with the shader's own operations, so lookups are bit-identical.
// One ISM (one block of kPullPushThreads threads; smem of pullpush_smem_bytes()).
__device__ __forceinline__ void pullpush_ism(const PullPushArgs& a, const int ism, unsigned char* smem) {
    __syncthreads();  // the previous ISM's use of smem is over
    const int s = a.ism_size, L = a.levels;
    // Level-0 keys are read straight from the atlas (each is read once by pull level 1 and once by
    // push level 0, both coalesced), so shared memory holds only the tables and levels 1..L.
    const uint32_t* keys = a.keys;
    float* s_rad = reinterpret_cast<float*>(smem);
    float* s_mdo = s_rad + 256;
    float4* lvl_base = reinterpret_cast<float4*>(smem + kPullPushTableBytes);
    const int bx = (ism % a.grid_x) * s, by = (ism / a.grid_x) * s;
    const int nt = blockDim.x, tid = threadIdx.x;
    for (int b = tid; b < 256; b += nt) {
        const float r = float(b) / 10.0f;
        s_rad[b] = r;
        s_mdo[b] = (r * 2.0f) / a.z_far * 0.6f;
    }
    __syncthreads();

    // level l data starts at lvl_off(l) texels from lvl_base
    auto lvl = [&](int l) {
        size_t off = 0;
        for (int k = 1; k < l; ++k) off += (size_t)(s >> k) * (s >> k);
        return lvl_base + off;
    };

    // ---- pull, levels 1..L (pull.comp) ----
    const int poff[4][2] = {{0, 0}, {0, 1}, {1, 0}, {1, 1}};
    for (int l = 1; l <= L; ++l) {
        const int sl = s >> l, si = s >> (l - 1);
        const int ox0 = bx >> l, oy0 = by >> l;
        const float4* in = l == 1 ? nullptr : lvl(l - 1);
        float4* out = lvl(l);
        const float scale = pow2neg(l);
        for (int i = tid; i < sl * sl; i += nt) {
            const int lx = i % sl, ly = i / sl;
            const int gox = ox0 + lx, goy = oy0 + ly;
            float depthSamples[4], maxDepths[4], radiuses[4], dvx[4], dvy[4];
            bool valid[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int lix = 2 * lx + poff[k][0], liy = 2 * ly + poff[k][1];
                const int gix = 2 * gox + poff[k][0], giy = 2 * goy + poff[k][1];
                float depthSample, radius, maxDepth, dx, dy;
                if (l == 1) {
                    const uint32_t key = __ldg(keys + (size_t)(by + liy) * a.atlas_w + bx + lix);
                    depthSample = float(key >> 8) / 16777216.0f;
                    dx = 0.f;
                    dy = 0.f;
                    maxDepth = depthSample + s_mdo[key & 0xFFu];
                    const float distToCamera = depthSample * a.z_far;
                    radius = s_rad[key & 0xFFu] / distToCamera / 3.14f * float(s);
                    radius = radius * 1.3f;
                    radius = gmin(radius, 15.0f);
                } else {
                    const float4 t = in[liy * si + lix];
                    depthSample = t.x;
                    maxDepth = t.y;
                    radius = t.z;
                    const float2 d = unpack_half2(__float_as_uint(t.w));
                    dx = d.x;
                    dy = d.y;
                }
                const float ndx = (float(gix) + 0.5f + dx) / 2.0f - (float(gox) + 0.5f);
                const float ndy = (float(giy) + 0.5f + dy) / 2.0f - (float(goy) + 0.5f);
                const float dist = sqrtf(ndx * ndx + ndy * ndy);
                const bool pass = dist <= radius * scale;
                depthSamples[k] = depthSample;
                maxDepths[k] = maxDepth;
                radiuses[k] = radius;
                dvx[k] = ndx;
                dvy[k] = ndy;
                valid[k] = depthSample != 1.0f && pass;
            }
            float minimum = __int_as_float(0x7f800000);
            float maxDepth = 0.f;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                if (!valid[k]) continue;
                minimum = gmin(depthSamples[k], minimum);
                if (minimum == depthSamples[k]) maxDepth = maxDepths[k];
            }
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if (depthSamples[k] > maxDepth) valid[k] = false;
            float depthAcc = 0.f, radiusAcc = 0.f, maxValid = 0.f, dax = 0.f, day = 0.f;
            int numValid = 0;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                if (!valid[k]) continue;
                depthAcc = depthAcc + depthSamples[k];
                dax = dax + dvx[k];
                day = day + dvy[k];
                radiusAcc = radiusAcc + radiuses[k];
                maxValid = gmax(maxValid, maxDepths[k]);
                numValid++;
            }
            float4 r;
            if (numValid > 0) {
                r = make_float4(div_count(depthAcc, numValid), maxValid, div_count(radiusAcc, numValid),
                                __uint_as_float(pack_half2(div_count(dax, numValid), div_count(day, numValid))));
            } else {
                r = make_float4(1.0f, 0.f, 0.f, 0.f);
            }
            out[i] = r;
        }
        __syncthreads();
    }

    // ---- push, levels L-1..0 (push.comp): one thread per 2x2 output quad sharing the same four
    // coarse texels, as in the shader; outputs outside this ISM are skipped ----
    const int qoff[4][2] = {{0, 0}, {0, 1}, {1, 1}, {1, 0}};
    const int weightsX[4] = {9, 3, 1, 3};
    for (int l = L - 1; l >= 0; --l) {
        const int sl = s >> l, sc = s >> (l + 1), nq = sc + 1;
        const int o0x = bx >> l, o0y = by >> l;              // this ISM's origin at level l
        const int c0x = bx >> (l + 1), c0y = by >> (l + 1);  // and at level l+1
        const float4* coarse = lvl(l + 1);
        float4* same = l == 0 ? nullptr : lvl(l);
        const float scale = pow2neg(l);
        for (int q = tid; q < nq * nq; q += nt) {
            const int gidx = c0x + q % nq, gidy = c0y + q / nq;  // global gid of the quad
            const int cllx = gidx - 1, clly = gidy - 1;
            float depths[4], maxDepths[4], radiuses[4], dcx[4], dcy[4], rs[4];
            bool usable[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int cx = cllx + qoff[k][0] - c0x, cy = clly + qoff[k][1] - c0y;
                if (cx >= 0 && cy >= 0 && cx < sc && cy < sc) {
                    const float4 t = coarse[cy * sc + cx];
                    depths[k] = t.x;
                    maxDepths[k] = t.y;
                    radiuses[k] = t.z;
                    const float2 d = unpack_half2(__float_as_uint(t.w));
                    dcx[k] = d.x;
                    dcy[k] = d.y;
                    // weight 0 for invalid depth (push.comp:88-93)
                    usable[k] = depths[k] != 1.0f;
                } else {  // across the ISM border: weight 0 (push.comp:77-86)
                    depths[k] = maxDepths[k] = radiuses[k] = dcx[k] = dcy[k] = 0.f;
                    usable[k] = false;
                }
                rs[k] = radiuses[k] * scale;
            }
#pragma unroll
            for (int op = 0; op < 4; ++op) {
                const int px = gidx * 2 - 1 + qoff[op][0], py = gidy * 2 - 1 + qoff[op][1];
                const int lpx = px - o0x, lpy = py - o0y;
                if (lpx < 0 || lpy < 0 || lpx >= sl || lpy >= sl) continue;
                int w[4];
                float dvx[4], dvy[4];
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    w[k] = usable[k] ? weightsX[(k - op + 4) & 3] : 0;
                    const float ctx = (float(cllx + qoff[k][0]) + 0.5f) * 2.0f;
                    const float cty = (float(clly + qoff[k][1]) + 0.5f) * 2.0f;
                    dvx[k] = ctx - (float(px) + 0.5f) + dcx[k] * 2.0f;
                    dvy[k] = cty - (float(py) + 0.5f) + dcy[k] * 2.0f;
                    if (w[k] != 0 && sqrtf(dvx[k] * dvx[k] + dvy[k] * dvy[k]) > rs[k]) w[k] = 0;
                }
                float minimum = 9001.0f, maxDepth = 0.f;
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    if (w[k] == 0) continue;
                    minimum = gmin(depths[k], minimum);
                    if (minimum == depths[k]) maxDepth = maxDepths[k];
                }
                int weightAcc = 0;
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    if (depths[k] > maxDepth) w[k] = 0;
                    weightAcc += w[k];
                }
                const int lp = lpy * sl + lpx;
                float4 orig;
                if (l == 0) {
                    orig = make_float4(float(__ldg(keys + (size_t)py * a.atlas_w + px) >> 8) / 16777216.0f, 0.f, 0.f, 0.f);
                } else {
                    orig = same[lp];
                }
                const bool invalid = orig.x == 1.0f;
                bool occluded = false;
#pragma unroll
                for (int k = 0; k < 4; ++k) occluded = occluded || (w[k] > 0 && orig.x > maxDepths[k]);
                float4 r = orig;
                // the weighted mean is only needed when it replaces the texel (push.comp:158-161);
                // zero-weight terms add +0 and are skipped
                if (!(weightAcc <= 0 || (!invalid && !occluded))) {
                    float depthAcc = 0.f, maxDepthAcc = 0.f, radiusAcc = 0.f, dax = 0.f, day = 0.f;
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        if (w[k] == 0) continue;
                        const float wf = float(w[k]);
                        depthAcc = depthAcc + depths[k] * wf;
                        if (l > 0) {
                            maxDepthAcc = maxDepthAcc + maxDepths[k] * wf;
                            radiusAcc = radiusAcc + radiuses[k] * wf;
                            dax = dax + dvx[k] * wf;
                            day = day + dvy[k] * wf;
                        }
                    }
                    r.x = div_count(depthAcc, weightAcc);
                    if (l > 0) {  // level 0 writes only the depth channel (push.comp:33-37)
                        r.y = div_count(maxDepthAcc, weightAcc);
                        r.z = div_count(radiusAcc, weightAcc);
                        r.w = __uint_as_float(pack_half2(div_count(dax, weightAcc), div_count(day, weightAcc)));
                    }
                }
                if (l == 0) {
                    const size_t o = (size_t)py * a.atlas_w + px;
                    if (a.out_f16)
                        reinterpret_cast<__half*>(a.out)[o] = __float2half_rn(r.x);
                    else
                        reinterpret_cast<float*>(a.out)[o] = r.x;
                } else {
                    same[lp] = r;
                }
            }
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kPullPushThreads, 2) pullpush_kernel(PullPushArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    pullpush_ism(a, blockIdx.x, smem);
}

size_t pullpush_smem_bytes(int ism_size, int levels) {
    size_t b = kPullPushTableBytes;
    for (int l = 1; l <= levels; ++l) b += (size_t)(ism_size >> l) * (ism_size >> l) * 16;
    return b;
}

cudaError_t launch_pullpush(const PullPushArgs& a, cudaStream_t s) {
    const size_t smem = pullpush_smem_bytes(a.ism_size, a.levels);
    cudaError_t e = cudaFuncSetAttribute(pullpush_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    pullpush_kernel<<<a.grid_x * a.grid_y, kPullPushThreads, smem, s>>>(a);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------
// Persistent forms over a view table: block b takes work items b, b + gridDim.x, ... of the pass;
// an item is (view, index inside the view) found from the pass's running item counts. Each item
// runs exactly the single-view body, so batched results equal single-frame results bit for bit.
__device__ __forceinline__ int find_view(const int* prefix, int n_views, int item) {
    int lo = 0, hi = n_views - 1;  // last view whose first item <= item
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(prefix + mid) <= item) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__global__ void __launch_bounds__(256) batch_clear_kernel(BatchTable t) {
    const int* pre = t.prefix + kBpClear * (t.n_views + 1);
    for (int item = blockIdx.x; item < __ldg(pre + t.n_views); item += gridDim.x) {
        const int v = find_view(pre, t.n_views, item);
        const BatchView& V = t.views[v];
        const size_t first = (size_t)(item - __ldg(pre + v)) * kBatchClearTexels;
        uint32_t* keys = V.keys;
        const size_t n = V.atlas_texels;
        for (size_t i = first + threadIdx.x * 4; i < first + kBatchClearTexels && i < n; i += 256 * 4) {
            if (i + 4 <= n)
                *reinterpret_cast<uint4*>(keys + i) = make_uint4(0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu);
            else
                for (size_t k = i; k < n; ++k) keys[k] = 0xFFFFFFFFu;
        }
    }
}

__global__ void __launch_bounds__(kBatchVplPerItem) batch_vpl_kernel(BatchTable t) {
    const int* pre = t.prefix + kBpVpl * (t.n_views + 1);
    for (int item = blockIdx.x; item < __ldg(pre + t.n_views); item += gridDim.x) {
        const int v = find_view(pre, t.n_views, item);
        vpl_one(t.views[v].vpl, (uint32_t)(item - __ldg(pre + v)) * kBatchVplPerItem + threadIdx.x);
    }
}

__global__ void __launch_bounds__(kSplatThreads) batch_splat_kernel(BatchTable t) {
    __shared__ SplatSmem S;
    __shared__ SplatArgs args;  // the item's view arguments, staged once per item
    const int* pre = t.prefix + kBpSplat * (t.n_views + 1);
    for (int item = blockIdx.x; item < __ldg(pre + t.n_views); item += gridDim.x) {
        const int v = find_view(pre, t.n_views, item);
        __syncthreads();
        if (threadIdx.x == 0) args = t.views[v].splat;
        __syncthreads();
        splat_bucket(args, item - __ldg(pre + v), S);
    }
}

__global__ void __launch_bounds__(kPullPushThreads, 2) batch_pullpush_kernel(BatchTable t) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ PullPushArgs args;
    const int* pre = t.prefix + kBpPullPush * (t.n_views + 1);
    for (int item = blockIdx.x; item < __ldg(pre + t.n_views); item += gridDim.x) {
        const int v = find_view(pre, t.n_views, item);
        __syncthreads();
        if (threadIdx.x == 0) args = t.views[v].pp;
        __syncthreads();
        pullpush_ism(args, item - __ldg(pre + v), smem);
    }
}

cudaError_t launch_batch_ism(const BatchTable& t, int pass, int grid, size_t smem, cudaStream_t s) {
    if (grid <= 0) return cudaSuccess;
    switch (pass) {
        case kBpClear: batch_clear_kernel<<<grid, 256, 0, s>>>(t); break;
        case kBpVpl: batch_vpl_kernel<<<grid, kBatchVplPerItem, 0, s>>>(t); break;
        case kBpSplat: batch_splat_kernel<<<grid, kSplatThreads, 0, s>>>(t); break;
        case kBpPullPush:  // the dynamic shared-memory limit was raised by batch_blocks_per_sm()
            batch_pullpush_kernel<<<grid, kPullPushThreads, smem, s>>>(t);
            break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

int batch_blocks_per_sm(int pass, size_t smem) {
    int n = 1;
    switch (pass) {
        case kBpClear: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_clear_kernel, 256, 0); break;
        case kBpVpl: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_vpl_kernel, kBatchVplPerItem, 0); break;
        case kBpSplat: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_splat_kernel, kSplatThreads, 0); break;
        case kBpPullPush:
            cudaFuncSetAttribute(batch_pullpush_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_pullpush_kernel, kPullPushThreads, smem);
            break;
        default: break;
    }
    return n > 0 ? n : 1;
}

}  // namespace mlgi
