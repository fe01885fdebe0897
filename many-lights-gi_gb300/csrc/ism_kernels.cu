// VPL processing, ISM point splat and the pull-push pyramid.
//
// This translation unit is compiled with -fmad=false and IEEE division/square root so that its
// FP32 results are word-for-word those of the reference shaders' arithmetic in GLSL order:
//   vpl_process_kernel  <- data/shaders/gi/vpl_processor.comp:41-72
//   ism_splat_kernel    <- data/shaders/ism/ism.comp:54-139
//   pyramid_kernel      <- data/shaders/ism/pull.comp:20-126 and push.comp:44-165, as driven by
//                          ImperfectShadowmap::pullpush (ImperfectShadowmap.cpp:121-182): an
//                          ISM's whole pyramid in one block (pyramid.cuh); pull1_kernel,
//                          pullmid_kernel, push1_kernel and push0_kernel run it level by level
//                          for launches of more than a wave of ISMs (pull1_lean_kernel,
//                          pullmid_kernel<., true> and push1_lean_kernel: the same results on
//                          the one-block pyramid's leaner arithmetic, where it is faster)
#include <cuda_runtime.h>

#include <atomic>

#include "batch_items.cuh"
#include "checks.cuh"
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
        const size_t t = MLGI_IX((size_t)tcy * a.rsm_w + tcx, (size_t)a.rsm_w * a.rsm_h);
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
    const uint32_t ri = MLGI_IX(a.perm ? (uint32_t)__ldg(a.perm + idx) : idx, (uint32_t)a.n);
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

// The VPL pass and the atlas clear in one launch, for the frames: blocks [0, vpl_blocks) run the
// VPLs (256 a block), the rest clear the key atlas. The two write disjoint buffers, and the VPL
// pass's few blocks run beside the clear's instead of before them.
__global__ void __launch_bounds__(256) vpl_clear_kernel(VplArgs va, uint4* p, size_t n4, int vpl_blocks) {
    if ((int)blockIdx.x < vpl_blocks) {
        vpl_one(va, blockIdx.x * 256u + threadIdx.x);
        return;
    }
    size_t i = (blockIdx.x - (unsigned)vpl_blocks) * (size_t)blockDim.x + threadIdx.x;
    const size_t stride = (size_t)(gridDim.x - (unsigned)vpl_blocks) * blockDim.x;
    for (; i < n4; i += stride) p[i] = make_uint4(0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu);
}

cudaError_t launch_vpl_clear(const VplArgs& va, uint32_t* keys, size_t n, cudaStream_t s) {
    if (va.n <= 0 || n == 0 || (n & 3) || (reinterpret_cast<uintptr_t>(keys) & 15)) {
        cudaError_t e = launch_vpl_process(va, s);
        return e == cudaSuccess ? launch_ism_clear(keys, n, s) : e;
    }
    const size_t n4 = n / 4;
    const int vpl_blocks = (va.n + 255) / 256;
    const int clear_blocks = (int)std::min<size_t>((n4 + 255) / 256, 152 * 16);
    vpl_clear_kernel<<<vpl_blocks + clear_blocks, 256, 0, s>>>(va, reinterpret_cast<uint4*>(keys), n4, vpl_blocks);
    return cudaGetLastError();
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
constexpr int kSplatTaskCap = 31 + 4 * 32;

struct SplatSmem {
    // per VPL, 16-byte rows: (position, ISM tile x), (normal, ISM tile y), (lookAtRH s, 0),
    // (lookAtRH u, 0); the tile offsets are float(x) and float(y) of ism_utils.glsl:35-37
    float4 pos[16], n[16], s[16], u[16];
    // the cull's operands by VPL pairs (2j, 2j + 1), each value for both VPLs of the pair side by
    // side for packed FP32x2 arithmetic: (-x, -y), (-z, normal x), (normal y, normal z)
    float4 cull[8][3];
    // per warp: (point xyz, VPL slot << 8 | radius byte); up to 31 carried over from the previous
    // group of points plus 4 for each of 32 new points
    float4 tasks[kSplatThreads / 32][kSplatTaskCap];
    // per byte value b of a point's packed word, computed with the shader's own operations:
    float unorm[256];       // float(b) / 255 * 2 - 1, a normal component (ism.comp:81-85)
    uint8_t rbyte[256];     // uint(float(b) / 255 * 25 * 10 / 2), the key's radius byte (ism.comp:87, 131-136)
};

// 1/x when x is a power of two (then v / x == v * (1/x) bit for bit: both are the rounding of the
// same real number), else 0.
__device__ __forceinline__ float pow2_recip(int x) {
    if (x <= 0 || (x & (x - 1))) return 0.f;
    return __int_as_float((127 - (31 - __clz(x))) << 23);
}

// Bucket wg (one block of kSplatThreads threads).
// Work item `item` of a splat: chunk item % chunks of bucket item / chunks, i.e. the bucket's
// points [chunk * kSplatChunk, (chunk + 1) * kSplatChunk), the last chunk up to the bucket's count
// (one block each).
// kCount: count the atomics the splat would issue (into *atomics) instead of issuing them.
template <bool kCount = false>
__device__ __forceinline__ void splat_bucket(const SplatArgs& a, const int item, SplatSmem& S,
                                             unsigned long long* atomics = nullptr) {
    const int local = item / a.chunks, chunk = item - local * a.chunks;
    const int wg = a.bucket0 + local;
    __syncthreads();  // the previous bucket's use of S is over
    const int vplCount = a.vpl_end - a.vpl_start;
    if (a.points_only_scaled && wg > vplCount) return;
    if (threadIdx.x < 16) {
        int index = (wg + (int)threadIdx.x) % a.n_vpl;
        if (a.points_only_scaled) {
            index %= vplCount;
            index += a.vpl_start;
        }
        const float4 pk = a.packed[MLGI_IX(index, a.n_vpl)];
        const v3 n = unpack3SN(__float_as_uint(pk.w));
        v3 s, u;
        look_at_rows(n, s, u);
        S.s[threadIdx.x] = make_float4(s.x, s.y, s.z, 0.f);
        S.u[threadIdx.x] = make_float4(u.x, u.y, u.z, 0.f);
        const float ismIndex = a.scale_isms ? float(index) - float(a.vpl_start) : float(index);
        const float fgx = float(a.gx);
        const float ty = float(f2i(ismIndex / fgx));
        S.pos[threadIdx.x] = make_float4(pk.x, pk.y, pk.z, float(f2i(ismIndex - ty * fgx)));
        S.n[threadIdx.x] = make_float4(n.x, n.y, n.z, float(f2i(ty)));
        float* c = reinterpret_cast<float*>(S.cull[threadIdx.x >> 1]) + (threadIdx.x & 1);
        c[0] = -pk.x, c[2] = -pk.y, c[4] = -pk.z, c[6] = n.x, c[8] = n.y, c[10] = n.z;
    }
    for (int b = threadIdx.x; b < 256; b += kSplatThreads) {
        const float f = float(b) / 255.0f;
        S.unorm[b] = f * 2.0f - 1.0f;
        S.rbyte[b] = (uint8_t)f2u(f * 25.0f * 10.0f / 2.0f);  // / sqrt(maxVplCollectCount)
    }
    __syncthreads();

    const uint32_t first = (uint32_t)chunk * kSplatChunk;
    // A counter may run past its bucket (ism.geom:65-67 does not bound it): the shader then reads
    // the next buckets' entries, and past the end of the buffer its imageLoad returns zero. All
    // such points are the same zero point, and splatting it again changes no key (atomicMin), so
    // the count stops one past the buffer's entries; that also bounds the block's work.
    const int64_t in_buffer = max((int64_t)0, a.n_entries - (int64_t)wg * a.bucket_stride);
    const uint32_t avail = (uint32_t)min(in_buffer, (int64_t)0xFFFFFFFE);
    // the last chunk takes any points beyond the stride (the counts hold at least the launch's buckets)
    uint32_t count = __ldg(a.counts + MLGI_IX(wg, a.bucket0 + a.n_groups));
    if (count > avail) count = avail + 1;
    const uint32_t cnt = chunk == a.chunks - 1 ? count : min(count, first + kSplatChunk);
    const float fw = float(a.atlas_w), fh = float(a.atlas_h), fgx = float(a.gx), fgy = float(a.gy);
    const float rgx = pow2_recip(a.gx), rgy = pow2_recip(a.gy);
    // per-task parameters in registers (a may live in shared memory in the batched form)
    const float z_far = a.z_far;
    const int atlas_w = a.atlas_w, atlas_h = a.atlas_h;
    uint32_t* const keys = a.keys;
    const int lane = threadIdx.x & 31;
    float4* tasks = S.tasks[threadIdx.x >> 5];
    unsigned issued = 0;  // kCount: this thread's in-range projections
    // Each warp takes 32 points at a time; a point's projections into its <= 4 VPLs become tasks
    // in the warp's list, and the warp runs them 32 at a time with all lanes. Fewer than 32 left
    // over wait for the next group's tasks, so that only the warp's last round runs partly empty.
    // atomicMin is order-independent, so the keys do not depend on when a task runs.
    int pending = 0;  // tasks in the list (warp-uniform)
    auto run_task = [&](const float4 task) {
        const uint32_t tw = __float_as_uint(task.w);
        const int i = (int)(tw >> 8);
        const uint32_t rbyte = tw & 0xFFu;
        const float4 vp = S.pos[MLGI_IX(i, 16)], vn = S.n[MLGI_IX(i, 16)];
        const v3 rel = mk(task.x, task.y, task.z) - mk(vp.x, vp.y, vp.z);
        // paraboloid_project(rel, length(rel), n, zFar, ismIndex, grid, preserveSign = true)
        const float dist = length(rel);
        const v3 n = mk(vn.x, vn.y, vn.z);
        const float4 vs = S.s[MLGI_IX(i, 16)], vu = S.u[MLGI_IX(i, 16)];
        float vx = dot(mk(vs.x, vs.y, vs.z), rel);
        float vy = dot(mk(vu.x, vu.y, vu.z), rel);
        float vz = ((-n.x) * rel.x + (-n.y) * rel.y) + (-n.z) * rel.z;
        const float signOfV = gsign(vz);
        vx = vx / dist;
        vy = vy / dist;
        vz = vz / dist;
        vz = 1.0f - vz;
        vx = vx / vz;
        vy = vy / vz;
        vz = dist / z_far;
        vz = vz * -signOfV;
        vx = (vx + 1.0f) / 2.0f;
        vy = (vy + 1.0f) / 2.0f;
        vx = vx + vp.w;  // ISM tile x
        vy = vy + vn.w;  // ISM tile y
        vx = rgx != 0.f ? vx * rgx : vx / fgx;
        vy = rgy != 0.f ? vy * rgy : vy / fgy;
        vx = vx * fw;
        vy = vy * fh;
        vz = vz * 16777216.0f;
        const uint32_t key = (f2u(vz) << 8) | rbyte;
        const int px = f2i(vx), py = f2i(vy);
        if (px < 0 || py < 0 || px >= atlas_w || py >= atlas_h) return;  // image op out of range: no-op
        if (kCount)
            ++issued;
        else
            atomicMin(keys + MLGI_IX((size_t)py * atlas_w + px, (size_t)atlas_w * atlas_h), key);
    };
    for (uint32_t base = first + threadIdx.x - lane; base < cnt; base += kSplatThreads) {
        const uint32_t j = base + lane;
        float4 pt = make_float4(0.f, 0.f, 0.f, 0.f);
        int found = 0;
        uint32_t used = 0;
        if (j < cnt) {
            if (j < avail) pt = __ldg(a.points + MLGI_IX((int64_t)wg * a.bucket_stride + j, a.n_entries));  // else the zero point
            const v3 position = mk(pt.x, pt.y, pt.z);
            const uint32_t nr = __float_as_uint(pt.w);
            const v3 pn = mk(S.unorm[nr & 0xFFu], S.unorm[(nr >> 8) & 0xFFu], S.unorm[(nr >> 16) & 0xFFu]);
            // gather up to 4 VPLs that pass the two-sided cull (ism.comp:93-107), as 4-bit indices.
            // Two VPLs at a time on packed FP32x2 operations with explicit rounding, which are never
            // contracted: per VPL, rel = position - vpl (added as position + (-vpl)), then
            // dot(n_vpl, rel) < 0 and dot(pn, -rel) < 0, each dot (x*x + y*y) + z*z. The second is
            // tested as dot(pn, rel) > 0: rounding to nearest is symmetric, so the two dots are
            // negatives of each other up to the sign of a zero, which neither comparison sees.
            const float2 p2x = make_float2(position.x, position.x), p2y = make_float2(position.y, position.y),
                         p2z = make_float2(position.z, position.z);
            const float2 n2x = make_float2(pn.x, pn.x), n2y = make_float2(pn.y, pn.y), n2z = make_float2(pn.z, pn.z);
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                if (found == 4) break;  // later VPLs are not used (ism.comp:103-106)
                const float4 c0 = S.cull[j][0], c1 = S.cull[j][1], c2 = S.cull[j][2];
                const float2 rx = __fadd2_rn(p2x, make_float2(c0.x, c0.y));
                const float2 ry = __fadd2_rn(p2y, make_float2(c0.z, c0.w));
                const float2 rz = __fadd2_rn(p2z, make_float2(c1.x, c1.y));
                const float2 dv = __fadd2_rn(__fadd2_rn(__fmul2_rn(make_float2(c1.z, c1.w), rx),
                                                        __fmul2_rn(make_float2(c2.x, c2.y), ry)),
                                             __fmul2_rn(make_float2(c2.z, c2.w), rz));
                const float2 dp = __fadd2_rn(__fadd2_rn(__fmul2_rn(n2x, rx), __fmul2_rn(n2y, ry)), __fmul2_rn(n2z, rz));
                if (!(dv.x < 0.0f || dp.x > 0.0f)) {
                    used |= (uint32_t)(2 * j) << (4 * found);
                    ++found;
                }
                if (!(dv.y < 0.0f || dp.y > 0.0f) && found < 4) {
                    used |= (uint32_t)(2 * j + 1) << (4 * found);
                    ++found;
                }
            }
        }
        // exclusive prefix of `found` over the warp
        int pre = found;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, pre, o);
            if (lane >= o) pre += t;
        }
        const int total = __shfl_sync(0xffffffffu, pre, 31);
        pre -= found;
        if (found > 0) {
            const uint32_t rbyte = S.rbyte[__float_as_uint(pt.w) >> 24];
            for (int k = 0; k < found; ++k)
                tasks[MLGI_IX(pending + pre + k, kSplatTaskCap)] =
                    make_float4(pt.x, pt.y, pt.z, __uint_as_float((((used >> (4 * k)) & 15u) << 8) | rbyte));
        }
        pending += total;
        __syncwarp();
        // full rounds of 32 tasks (ism.comp:112-137 for each)
        const int full = pending & ~31;
        for (int t = lane; t < full; t += 32) run_task(tasks[t]);
        // the remainder (< 32) moves to the front of the list
        const int rem = pending - full;
        float4 keep = make_float4(0.f, 0.f, 0.f, 0.f);
        if (lane < rem) keep = tasks[full + lane];
        __syncwarp();
        if (lane < rem) tasks[lane] = keep;
        pending = rem;
        __syncwarp();
    }
    if (lane < pending) run_task(tasks[lane]);  // the last, partly empty round
    if (kCount) {
        for (int o = 16; o > 0; o >>= 1) issued += __shfl_xor_sync(0xffffffffu, issued, o);
        if (lane == 0 && issued) atomicAdd(atomics, (unsigned long long)issued);
    }
}

// Seven blocks a SM (32 registers, no spill; shared memory would allow nine): splat 0.0466 ->
// 0.0427 ms at CREF and 0.277 -> 0.271 at C3-B against six, C2 unchanged; eight measured the same.
__global__ void __launch_bounds__(kSplatThreads, 7) ism_splat_kernel(SplatArgs a) {
    __shared__ SplatSmem S;
    splat_bucket(a, blockIdx.x, S);
}

cudaError_t launch_ism_splat(const SplatArgs& a, cudaStream_t s) {
    if (a.n_groups <= 0) return cudaSuccess;
    ism_splat_kernel<<<a.n_groups * a.chunks, kSplatThreads, 0, s>>>(a);
    return cudaGetLastError();
}

__global__ void __launch_bounds__(kSplatThreads) ism_splat_count_kernel(SplatArgs a, unsigned long long* count) {
    __shared__ SplatSmem S;
    splat_bucket<true>(a, blockIdx.x, S, count);
}

cudaError_t launch_ism_splat_count(const SplatArgs& a, unsigned long long* count, cudaStream_t s) {
    if (a.n_groups <= 0) return cudaSuccess;
    ism_splat_count_kernel<<<a.n_groups * a.chunks, kSplatThreads, 0, s>>>(a, count);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------
// Pull-push in up to four launches. Pull and push never mix texels of different ISMs (2x2 pulls
// stay inside an ISM because its edge is divisible by 2^levels, and push gives weight 0 to every
// coarse texel across an ISM border), and each texel of a level depends only on texels of the
// next finer (pull) or next coarser (push) level of its own ISM:
//   pull1_kernel    level 1 from the keys, one thread per level-1 texel            -> lv1
//   pullmid_kernel  one block per ISM: pull 2..L, push L-1..2 in shared memory     -> lv2
//   push1_kernel    push level 1 from lv2 onto lv1 in place, one thread per 2x2 quad
//   push0_kernel    push level 0 (depth only) from lv1 and the keys, one thread per 2x2 quad -> out
// Texels of levels >= 1 are (depth, maxDepth, radius, packHalf2x16(dx, dy)), the reference's
// RGBA32F pyramid. Coordinates entering the displacement arithmetic are global coordinates of the
// level, as in the level-by-level shaders.
constexpr int kPpTileW = 32, kPpTileH = 8;  // texel tile of the per-texel kernels (256 threads)
constexpr int kPullMidThreads = 128;  // one wave of ISM blocks at the usual atlas sizes
constexpr int kPpBatchTiles = 4;  // texel tiles per work item of the batched per-texel passes
constexpr size_t kPullPushTableBytes = 2 * 256 * sizeof(float);  // key-byte tables, see below

__device__ __forceinline__ float pow2neg(int level) { return __int_as_float((127 - level) << 23); }

// sqrt(d2) > r with sqrt correctly rounded, for finite d2 >= 0 and finite r. RN(sqrt(d2)) > r
// exactly when sqrt(d2) exceeds the midpoint between r and the next float up (a square root of a
// float is never such a midpoint), i.e. when d2 > r^2 (1 + 2^-24)^2 at most. With p = RN(r*r):
// d2 > RN(p (1 + 2^-20)) implies d2 > r^2 (1 + 2^-21), above that threshold; d2 < RN(p (1 - 2^-20))
// implies d2 < r^2, so sqrt(d2) < r and RN(sqrt(d2)) <= r. Only the band in between takes sqrtf,
// out of line so that the unrolled callers stay small.
__device__ __noinline__ bool sqrt_gt_band(float d2, float r) { return sqrtf(d2) > r; }

__device__ __forceinline__ bool sqrt_gt(float d2, float r) {
    const float p = r * r;
    if (r > 0.f && p >= 1e-30f) {
        if (d2 > p * 1.00000095367431640625f) return true;
        if (d2 < p * 0.99999904632568359375f) return false;
    }
    return sqrt_gt_band(d2, r);
}

// RN(1/n) for n = 1..16 (entry 0 unused), folded by the compiler in IEEE single precision.
__device__ const float kRcpSmall[17] = {0.0f,        1.0f,        1.0f / 2.0f,  1.0f / 3.0f,  1.0f / 4.0f,  1.0f / 5.0f,
                                        1.0f / 6.0f, 1.0f / 7.0f, 1.0f / 8.0f,  1.0f / 9.0f,  1.0f / 10.0f, 1.0f / 11.0f,
                                        1.0f / 12.0f, 1.0f / 13.0f, 1.0f / 14.0f, 1.0f / 15.0f, 1.0f / 16.0f};

// x / n rounded to nearest for the sample counts and weight sums that occur (1 <= n <= 16), from
// R = RN(1/n) and one correction by the exact residual (Markstein's division): q = RN(x R),
// r = x - q n (exact by FMA), result RN(q + r R). That equals IEEE x / n for every float
// significand and every n <= 16 (checked exhaustively in tests/test_small_division.py); scaling by
// a power of two is exact, so it holds for every x whose intermediates stay normal. Zero, tiny,
// huge and non-finite x take the IEEE division.
__device__ __forceinline__ float div_corrected(float x, float d, float R) {
    const float ax = fabsf(x);
    if (!(ax >= 0x1p-100f && ax <= 0x1p+100f)) return x / d;
    const float q = x * R;
    const float r = fmaf(-q, d, x);
    return fmaf(r, R, q);
}

// The push's weight sums 1..16, without branches (for a power of two R is exact and the
// correction adds 0).
__device__ __forceinline__ float div_count(float x, int n) {
    return n <= 16 ? div_corrected(x, float(n), __ldg(kRcpSmall + n)) : x / float(n);
}

// The pull's valid-sample counts 1..4: only 3 needs a division; the others are exact multiplies.
__device__ __forceinline__ float div_count4(float x, int n) {
    switch (n) {
        case 1: return x;
        case 2: return x * 0.5f;
        case 3: return div_corrected(x, 3.0f, 1.0f / 3.0f);
        default: return x * 0.25f;
    }
}

// x / 3.14f rounded to nearest by the same correction (checked exhaustively for this
// divisor in tests/test_small_division.py).
__device__ __forceinline__ float div_314(float x) { return div_corrected(x, 3.14f, 1.0f / 3.14f); }

// Two 256-entry tables indexed by a key's radius byte b, each entry computed with the shader's own
// operations so that lookups are bit-identical:
//   s_rad[b] = float(b) / 10                          (pull.comp:39)
//   s_mdo[b] = ((float(b) / 10) * 2) / zFar * 0.6     (the maxDepth offset of pull.comp:57)
__device__ __forceinline__ void fill_key_tables(float* s_rad, float* s_mdo, float z_far) {
    for (int b = threadIdx.x; b < 256; b += blockDim.x) {
        const float r = float(b) / 10.0f;
        s_rad[b] = r;
        s_mdo[b] = (r * 2.0f) / z_far * 0.6f;
    }
}

struct PullSample {
    float depth, maxDepth, radius, ndx, ndy;
};

// One pull output from its four samples in the order (0,0), (0,1), (1,0), (1,1) (pull.comp:60-120).
// dist1 >= 0: every sample's displacement length is this value (already rounded as sqrt rounds it).
__device__ __forceinline__ float4 pull_combine(const PullSample (&q)[4], const float scale, const float dist1 = -1.0f) {
    bool valid[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {  // dist <= radius * scale, dist = length(displacement)
        const bool far = dist1 >= 0.f ? dist1 > q[k].radius * scale
                                      : sqrt_gt(q[k].ndx * q[k].ndx + q[k].ndy * q[k].ndy, q[k].radius * scale);
        valid[k] = q[k].depth != 1.0f && !far;
    }
    float minimum = __int_as_float(0x7f800000);
    float maxDepth = 0.f;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (!valid[k]) continue;
        minimum = gmin(q[k].depth, minimum);
        if (minimum == q[k].depth) maxDepth = q[k].maxDepth;
    }
#pragma unroll
    for (int k = 0; k < 4; ++k)
        if (q[k].depth > maxDepth) valid[k] = false;
    float depthAcc = 0.f, radiusAcc = 0.f, maxValid = 0.f, dax = 0.f, day = 0.f;
    int numValid = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (!valid[k]) continue;
        depthAcc = depthAcc + q[k].depth;
        dax = dax + q[k].ndx;
        day = day + q[k].ndy;
        radiusAcc = radiusAcc + q[k].radius;
        maxValid = gmax(maxValid, q[k].maxDepth);
        numValid++;
    }
    if (numValid == 0) return make_float4(1.0f, 0.f, 0.f, 0.f);
    return make_float4(div_count4(depthAcc, numValid), maxValid, div_count4(radiusAcc, numValid),
                       __uint_as_float(pack_half2(div_count4(dax, numValid), div_count4(day, numValid))));
}

__device__ constexpr int kPullOff[4][2] = {{0, 0}, {0, 1}, {1, 0}, {1, 1}};

// Pull level 1 at global level-1 texel (gox, goy) from the four keys below it. The displacement
// of a key sample is exactly (+-0.25, +-0.25) (dx = dy = 0 at level 0).
__device__ __forceinline__ float4 pull1_texel(const PullPushArgs& a, const float* s_rad, const float* s_mdo,
                                              const int gox, const int goy) {
    const size_t nk = (size_t)a.atlas_w * a.atlas_h - 1;  // a pair's first key
    const uint2 r0 = __ldg(reinterpret_cast<const uint2*>(a.keys + MLGI_IX((size_t)(2 * goy) * a.atlas_w + 2 * gox, nk)));
    const uint2 r1 = __ldg(reinterpret_cast<const uint2*>(a.keys + MLGI_IX((size_t)(2 * goy + 1) * a.atlas_w + 2 * gox, nk)));
    const uint32_t key[4] = {r0.x, r1.x, r0.y, r1.y};  // (0,0), (0,1), (1,0), (1,1)
    const float fs = float(a.ism_size);
    PullSample q[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float depthSample = float(key[k] >> 8) / 16777216.0f;
        q[k].depth = depthSample;
        q[k].maxDepth = depthSample + s_mdo[key[k] & 0xFFu];
        const float distToCamera = depthSample * a.z_far;
        float radius = div_314(s_rad[key[k] & 0xFFu] / distToCamera) * fs;
        radius = radius * 1.3f;
        q[k].radius = gmin(radius, 15.0f);
        q[k].ndx = kPullOff[k][0] ? 0.25f : -0.25f;
        q[k].ndy = kPullOff[k][1] ? 0.25f : -0.25f;
    }
    // |(+-0.25, +-0.25)|^2 = 0.125 exactly, so every sample's length is RN(sqrt(0.125))
    return pull_combine(q, 0.5f, sqrtf(0.125f));
}

// Pull level l >= 2 at global level-l texel (gox, goy); `in` is level l-1 (n texels) with row
// pitch `pin` and origin (ix0, iy0) in global level-(l-1) coordinates.
__device__ __forceinline__ float4 pull_texel(const float4* in, const size_t n, const int pin, const int ix0,
                                             const int iy0, const int gox, const int goy, const float scale) {
    PullSample q[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int gix = 2 * gox + kPullOff[k][0], giy = 2 * goy + kPullOff[k][1];
        const float4 t = in[MLGI_IX((giy - iy0) * pin + (gix - ix0), n)];
        const float2 d = unpack_half2(__float_as_uint(t.w));
        q[k].depth = t.x;
        q[k].maxDepth = t.y;
        q[k].radius = t.z;
        q[k].ndx = (float(gix) + 0.5f + d.x) / 2.0f - (float(gox) + 0.5f);
        q[k].ndy = (float(giy) + 0.5f + d.y) / 2.0f - (float(goy) + 0.5f);
    }
    return pull_combine(q, scale);
}

__device__ constexpr int kPushOff[4][2] = {{0, 0}, {0, 1}, {1, 1}, {1, 0}};

// floor(n / d) for n < 2^16 and 2 <= d < 2^16 from m = ceil(2^32 / d): the error of n * m / 2^32
// is below n / 2^32 < 1 / d, too small to cross an integer.
__device__ __forceinline__ int div_small(int n, uint32_t m) { return (int)__umulhi((uint32_t)n, m); }

// Push at level l for a level-l texel at position (qx, qy) = ((px + 1) & 1, (py + 1) & 1) of its
// 2x2 quad gid = ((px + 1) >> 1, (py + 1) >> 1) (push.comp:44-165). Coarse texel k is
// gid - 1 + kPushOff[k] at level l+1, zero when it lies outside this ISM (`inside[k]` false:
// weight 0, push.comp:77-86). The shader's weight of coarse texel k for quad output op,
// {9, 3, 1, 3}[(k - op) & 3], is 3 per coordinate that k shares with the output's quad position
// times 1 per coordinate it does not. `orig` is the texel's pull value; kFull: all four channels
// (levels >= 1), else the depth channel only (level 0, push.comp:33-37).
template <bool kFull>
__device__ __forceinline__ float4 push_texel(const float4 (&coarse)[4], const bool (&inside)[4], const int qx,
                                             const int qy, const float4 orig, const float scale) {
    float depths[4], maxDepths[4], radiuses[4], dvx[4], dvy[4];
    int w[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int kx = kPushOff[k][0], ky = kPushOff[k][1];
        const float4 t = coarse[k];
        const float2 d = unpack_half2(__float_as_uint(t.w));
        depths[k] = t.x;
        maxDepths[k] = t.y;
        radiuses[k] = t.z;
        // weight 0 for invalid depth (push.comp:88-93)
        w[k] = inside[k] && t.x != 1.0f ? (kx == qx ? 3 : 1) * (ky == qy ? 3 : 1) : 0;
        // (ctx - (px + 0.5)) with ctx = (gid - 1 + kx + 0.5) * 2 and px = 2 gid - 1 + qx is exactly
        // 2 kx - qx - 0.5 (all integers below 2^24)
        const float ox = qx ? float(2 * kx) - 1.5f : float(2 * kx) - 0.5f;
        const float oy = qy ? float(2 * ky) - 1.5f : float(2 * ky) - 0.5f;
        dvx[k] = ox + d.x * 2.0f;
        dvy[k] = oy + d.y * 2.0f;
        if (w[k] != 0 && sqrt_gt(dvx[k] * dvx[k] + dvy[k] * dvy[k], radiuses[k] * scale)) w[k] = 0;
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
            if (kFull) {
                maxDepthAcc = maxDepthAcc + maxDepths[k] * wf;
                radiusAcc = radiusAcc + radiuses[k] * wf;
                dax = dax + dvx[k] * wf;
                day = day + dvy[k] * wf;
            }
        }
        r.x = div_count(depthAcc, weightAcc);
        if (kFull) {
            r.y = div_count(maxDepthAcc, weightAcc);
            r.z = div_count(radiusAcc, weightAcc);
            r.w = __uint_as_float(pack_half2(div_count(dax, weightAcc), div_count(day, weightAcc)));
        }
    }
    return r;
}

// Push levels 1 and 0 by 2x2 quads: the thread of quad gid = (gx, gy) of level l loads the four
// coarse texels gid - 1 + kPushOff[k] of level l+1 once and derives their per-texel terms once,
// then produces the quad's outputs (2 gx - 1 + qx, 2 gy - 1 + qy) -- those inside the atlas --
// with the shader's per-output arithmetic. A quad straddles two ISMs in x exactly when gx is a
// multiple of the ISM edge sc at level l+1 (then its left output is the last column of one ISM
// and its right output the first of the next); coarse column gx - 1 + kx belongs to the ISM of
// output qx unless the quad straddles and kx != qx. The same holds in y.
struct PushCoarse {
    float depth[4], maxDepth[4], radius[4], ax[4], ay[4], rs[4], hi[4], lo[4];
    bool usable[4];
};

__device__ __forceinline__ void push_coarse(const float4* c, const int pc, const int cw, const int ch, const int gx,
                                            const int gy, const float scale, PushCoarse& C) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        // coordinates off the level are clamped: such texels are never inside an output's ISM
        const int cx = min(max(gx - 1 + kPushOff[k][0], 0), cw - 1);
        const int cy = min(max(gy - 1 + kPushOff[k][1], 0), ch - 1);
        const float4 t = c[MLGI_IX((uint32_t)cy * (uint32_t)pc + (uint32_t)cx, (uint32_t)pc * (uint32_t)ch)];
        const float2 d = unpack_half2(__float_as_uint(t.w));
        C.depth[k] = t.x;
        C.maxDepth[k] = t.y;
        C.radius[k] = t.z;
        C.usable[k] = t.x != 1.0f;  // weight 0 for invalid depth (push.comp:88-93)
        C.ax[k] = d.x * 2.0f;
        C.ay[k] = d.y * 2.0f;
        const float r = t.z * scale;
        const float p = r * r;
        const bool fast = r > 0.f && p >= 1e-30f;  // the thresholds of sqrt_gt; NaN sends to sqrtf
        C.rs[k] = r;
        C.hi[k] = fast ? p * 1.00000095367431640625f : __int_as_float(0x7fc00000);
        C.lo[k] = fast ? p * 0.99999904632568359375f : __int_as_float(0x7fc00000);
    }
}

// Output (qx, qy) of the quad (push.comp:95-161); `orig` is its pull value.
template <bool kFull, int qx, int qy>
__device__ __forceinline__ float4 push_output(const PushCoarse& C, const bool bx, const bool by, const float4 orig) {
    float dvx[4], dvy[4];
    int w[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int kx = kPushOff[k][0], ky = kPushOff[k][1];
        const bool inside = (kx == qx || !bx) && (ky == qy || !by);  // weight 0 across the border (push.comp:77-86)
        w[k] = inside && C.usable[k] ? (kx == qx ? 3 : 1) * (ky == qy ? 3 : 1) : 0;
        // (ctx - (px + 0.5)) is exactly 2 kx - qx - 0.5 (see push_texel)
        dvx[k] = (float(2 * kx - qx) - 0.5f) + C.ax[k];
        dvy[k] = (float(2 * ky - qy) - 0.5f) + C.ay[k];
        if (w[k] != 0) {
            const float d2 = dvx[k] * dvx[k] + dvy[k] * dvy[k];
            const bool gt = d2 > C.hi[k] || (!(d2 < C.lo[k]) && sqrt_gt_band(d2, C.rs[k]));
            if (gt) w[k] = 0;
        }
    }
    float minimum = 9001.0f, maxDepth = 0.f;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (w[k] == 0) continue;
        minimum = gmin(C.depth[k], minimum);
        if (minimum == C.depth[k]) maxDepth = C.maxDepth[k];
    }
    int weightAcc = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (C.depth[k] > maxDepth) w[k] = 0;
        weightAcc += w[k];
    }
    const bool invalid = orig.x == 1.0f;
    bool occluded = false;
#pragma unroll
    for (int k = 0; k < 4; ++k) occluded = occluded || (w[k] > 0 && orig.x > C.maxDepth[k]);
    float4 r = orig;
    if (!(weightAcc <= 0 || (!invalid && !occluded))) {
        float depthAcc = 0.f, maxDepthAcc = 0.f, radiusAcc = 0.f, dax = 0.f, day = 0.f;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (w[k] == 0) continue;
            const float wf = float(w[k]);
            depthAcc = depthAcc + C.depth[k] * wf;
            if (kFull) {
                maxDepthAcc = maxDepthAcc + C.maxDepth[k] * wf;
                radiusAcc = radiusAcc + C.radius[k] * wf;
                dax = dax + dvx[k] * wf;
                day = day + dvy[k] * wf;
            }
        }
        r.x = div_count(depthAcc, weightAcc);
        if (kFull) {
            r.y = div_count(maxDepthAcc, weightAcc);
            r.z = div_count(radiusAcc, weightAcc);
            r.w = __uint_as_float(pack_half2(div_count(dax, weightAcc), div_count(day, weightAcc)));
        }
    }
    return r;
}

// x is a multiple of d (d >= 1, x < 2^16; m = ceil(2^32 / d) when d >= 2)
__device__ __forceinline__ bool multiple_of(const int x, const int d, const uint32_t m) {
    return d == 1 || x == div_small(x, m) * d;
}

// Per-texel pass on a kPpTileW x kPpTileH tile (tx, ty) of level 1, tile rows counted from the
// launch's first ISM row.
__device__ __forceinline__ void pull1_tile(const PullPushArgs& a, const int tx, const int ty, const float* s_rad,
                                           const float* s_mdo) {
    const int s1 = a.ism_size >> 1;
    const int x = tx * kPpTileW + (threadIdx.x % kPpTileW), y = a.row0 * s1 + ty * kPpTileH + (threadIdx.x / kPpTileW);
    const int w1 = a.atlas_w >> 1;
    if (x < w1 && y < a.row1 * s1)
        a.lv1[MLGI_IX((uint32_t)y * w1 + x, (uint32_t)w1 * (a.atlas_h >> 1))] = pull1_texel(a, s_rad, s_mdo, x, y);
}

// Quad passes on a kPpTileW x kPpTileH tile (tx, ty) of quads: level l has (w_l / 2 + 1) x
// (h_l / 2 + 1) quads. A launch over ISM rows [row0, row1) writes the level's rows [Y0, Y1) =
// [row0, row1) * edge, from quad rows Y0 / 2 .. Y1 / 2 (quad gy writes rows 2 gy - 1 and 2 gy);
// a quad on the range's border also reads coarse texels of the neighbouring ISM row, with weight
// 0 for the outputs written here, so their values do not matter.
__device__ __forceinline__ void push1_quads(const PullPushArgs& a, const int tx, const int ty) {
    const int w1 = a.atlas_w >> 1, h1 = a.atlas_h >> 1, w2 = a.atlas_w >> 2, h2 = a.atlas_h >> 2;
    const int s1 = a.ism_size >> 1, Y0 = a.row0 * s1, Y1 = a.row1 * s1;
    const int gx = tx * kPpTileW + (threadIdx.x % kPpTileW), gy = (Y0 >> 1) + ty * kPpTileH + (threadIdx.x / kPpTileW);
    if (gx > w2 || gy > (Y1 >> 1)) return;
    const int sc = a.ism_size >> 2;  // ISM edge at level 2
    PushCoarse C;
    push_coarse(a.lv2, w2, w2, h2, gx, gy, 0.5f, C);
    const bool bx = multiple_of(gx, sc, a.m_c1), by = multiple_of(gy, sc, a.m_c1);
    const int x0 = 2 * gx - 1, y0 = 2 * gy - 1;
    const bool okx0 = x0 >= 0, okx1 = x0 + 1 < w1, oky0 = y0 >= Y0, oky1 = y0 + 1 < Y1;
    const uint32_t n1 = (uint32_t)w1 * h1;
    const uint32_t o0 = (uint32_t)max(y0, 0) * w1 + x0, o1 = (uint32_t)min(y0 + 1, h1 - 1) * w1 + x0;  // x0 < 0: unused
    float4* lv1 = a.lv1;
    if (oky0 && okx0) lv1[MLGI_IX(o0, n1)] = push_output<true, 0, 0>(C, bx, by, lv1[MLGI_IX(o0, n1)]);
    if (oky0 && okx1) lv1[MLGI_IX(o0 + 1, n1)] = push_output<true, 1, 0>(C, bx, by, lv1[MLGI_IX(o0 + 1, n1)]);
    if (oky1 && okx0) lv1[MLGI_IX(o1, n1)] = push_output<true, 0, 1>(C, bx, by, lv1[MLGI_IX(o1, n1)]);
    if (oky1 && okx1) lv1[MLGI_IX(o1 + 1, n1)] = push_output<true, 1, 1>(C, bx, by, lv1[MLGI_IX(o1 + 1, n1)]);
}

__device__ __forceinline__ void store_depth(const PullPushArgs& a, uint32_t o, const float d) {
    o = MLGI_IX(o, (uint32_t)a.atlas_w * (uint32_t)a.atlas_h);
    if (a.out_f16)
        reinterpret_cast<__half*>(a.out)[o] = __float2half_rn(d);
    else
        reinterpret_cast<float*>(a.out)[o] = d;
}

__device__ __forceinline__ float key_depth(const PullPushArgs& a, const uint32_t o) {
    return float(__ldg(a.keys + MLGI_IX(o, (uint32_t)a.atlas_w * (uint32_t)a.atlas_h)) >> 8) / 16777216.0f;
}

__device__ __forceinline__ void push0_quads(const PullPushArgs& a, const int tx, const int ty) {
    const int w = a.atlas_w, h = a.atlas_h, w1 = w >> 1, h1 = h >> 1;
    const int Y0 = a.row0 * a.ism_size, Y1 = a.row1 * a.ism_size;
    const int gx = tx * kPpTileW + (threadIdx.x % kPpTileW), gy = (Y0 >> 1) + ty * kPpTileH + (threadIdx.x / kPpTileW);
    if (gx > w1 || gy > (Y1 >> 1)) return;
    const int sc = a.ism_size >> 1;  // ISM edge at level 1
    PushCoarse C;
    push_coarse(a.lv1, w1, w1, h1, gx, gy, 1.0f, C);
    const bool bx = multiple_of(gx, sc, a.m_c0), by = multiple_of(gy, sc, a.m_c0);
    const int x0 = 2 * gx - 1, y0 = 2 * gy - 1;
    const bool okx0 = x0 >= 0, okx1 = x0 + 1 < w, oky0 = y0 >= Y0, oky1 = y0 + 1 < Y1;
    const uint32_t r0 = (uint32_t)y0 * w, r1 = (uint32_t)(y0 + 1) * w;
    // the four keys first, so that their loads overlap each other and the coarse terms
    const float k00 = oky0 && okx0 ? key_depth(a, r0 + x0) : 0.f;
    const float k10 = oky0 && okx1 ? key_depth(a, r0 + x0 + 1) : 0.f;
    const float k01 = oky1 && okx0 ? key_depth(a, r1 + x0) : 0.f;
    const float k11 = oky1 && okx1 ? key_depth(a, r1 + x0 + 1) : 0.f;
    // level 0 writes only the depth channel (push.comp:33-37)
    if (oky0 && okx0) store_depth(a, r0 + x0, push_output<false, 0, 0>(C, bx, by, make_float4(k00, 0.f, 0.f, 0.f)).x);
    if (oky0 && okx1) store_depth(a, r0 + x0 + 1, push_output<false, 1, 0>(C, bx, by, make_float4(k10, 0.f, 0.f, 0.f)).x);
    if (oky1 && okx0) store_depth(a, r1 + x0, push_output<false, 0, 1>(C, bx, by, make_float4(k01, 0.f, 0.f, 0.f)).x);
    if (oky1 && okx1) store_depth(a, r1 + x0 + 1, push_output<false, 1, 1>(C, bx, by, make_float4(k11, 0.f, 0.f, 0.f)).x);
}

// Levels 2..L of one ISM in shared memory (tables first, then level 2, 3, ...): pull from lv1,
// push back down to level 2, which is written to lv2.
__device__ __forceinline__ void pullmid_ism(const PullPushArgs& a, const int ism, unsigned char* smem) {
    __syncthreads();  // the previous ISM's use of smem is over
    const int s = a.ism_size, L = a.levels;
    float4* lvl_base = reinterpret_cast<float4*>(smem + kPullPushTableBytes);
    auto lvl = [&](int l) {  // level l >= 2 in shared memory, row pitch s >> l
        size_t off = 0;
        for (int k = 2; k < l; ++k) off += (size_t)(s >> k) * (s >> k);
        return lvl_base + off;
    };
#ifdef MLGI_CHECKS
    {  // levels 2..L inside the block's shared memory: their last texel
        uint32_t dyn;
        asm volatile("mov.u32 %0, %%dynamic_smem_size;" : "=r"(dyn));
        (void)MLGI_IX((lvl(L + 1) - lvl_base) - 1, dyn > kPullPushTableBytes ? (dyn - kPullPushTableBytes) / 16 : 0);
    }
#endif
    const int im = MLGI_IX(ism, a.grid_x * a.grid_y), ix = im % a.grid_x, iy = im / a.grid_x;
    const int nt = blockDim.x, tid = threadIdx.x;
    for (int l = 2; l <= L; ++l) {  // pull
        const int sl = s >> l;
        const int ox0 = ix * sl, oy0 = iy * sl;
        float4* out = lvl(l);
        const float scale = pow2neg(l);
        for (int i = tid; i < sl * sl; i += nt) {
            const int gox = ox0 + i % sl, goy = oy0 + i / sl;
            out[i] = l == 2 ? pull_texel(a.lv1, (size_t)(a.atlas_w >> 1) * (a.atlas_h >> 1), a.atlas_w >> 1, 0, 0, gox,
                                         goy, scale)
                            : pull_texel(lvl(l - 1), (size_t)4 * sl * sl, 2 * sl, 2 * ox0, 2 * oy0, gox, goy, scale);
        }
        __syncthreads();
    }
    for (int l = L - 1; l >= 2; --l) {  // push in place: a texel reads only its own pull value
        const int sl = s >> l;
        const int ox0 = ix * sl, oy0 = iy * sl;
        const float4* coarse_lvl = lvl(l + 1);
        float4* same = lvl(l);
        const float scale = pow2neg(l);
        const int sc = sl >> 1;
        for (int i = tid; i < sl * sl; i += nt) {
            const int px = ox0 + i % sl, py = oy0 + i / sl;
            // the coarse texels of the texel's quad, on the ISM-local level in shared memory
            float4 coarse[4];
            bool inside[4];
            const int gidx = (px + 1) >> 1, gidy = (py + 1) >> 1;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int cx = gidx - 1 + kPushOff[k][0] - ix * sc, cy = gidy - 1 + kPushOff[k][1] - iy * sc;
                inside[k] = cx >= 0 && cy >= 0 && cx < sc && cy < sc;
                coarse[k] = inside[k] ? coarse_lvl[MLGI_IX(cy * sc + cx, sc * sc)] : make_float4(0.f, 0.f, 0.f, 0.f);
            }
            same[i] = push_texel<true>(coarse, inside, (px + 1) & 1, (py + 1) & 1, same[i], scale);
        }
        __syncthreads();
    }
    const int s2 = s >> 2, w2 = a.atlas_w >> 2;
    const float4* l2 = lvl(2);
    for (int i = tid; i < s2 * s2; i += nt)
        a.lv2[MLGI_IX((size_t)(iy * s2 + i / s2) * w2 + ix * s2 + i % s2, (size_t)w2 * (a.atlas_h >> 2))] = l2[i];
}

// kPull1Rows tile rows per block, so that the key tables are filled once for several tiles.
constexpr int kPull1Rows = 4;  // 2 and 8 (lean kernel, eight blocks a SM): C2 pass 0.2307 / 0.2235 ms, CREF 0.0748 / 0.0730, against 0.2245 / 0.0719
__global__ void __launch_bounds__(kPpTileW * kPpTileH) pull1_kernel(PullPushArgs a) {
    __shared__ float s_tab[512];
    fill_key_tables(s_tab, s_tab + 256, a.z_far);
    __syncthreads();
#pragma unroll 1
    for (int j = 0; j < kPull1Rows; ++j) pull1_tile(a, blockIdx.x, blockIdx.y * kPull1Rows + j, s_tab, s_tab + 256);
}

// NT threads per ISM: kPullMidThreads when the launch fills the GPU with ISM blocks, more when a
// launch over a few ISM rows would leave most SMs idle (the pass is then bound by one block's time).
__host__ __device__ __forceinline__ bool pyramid_lean_range(float z_far);
__device__ __forceinline__ void pullmid_lean_ism(const PullPushArgs& a, int ism, unsigned char* smem);

// kLean: the one-block pyramid's arithmetic (pullmid_lean_ism), for ISM edges of at least
// kPullMidLeanEdge (fewer instructions at 84 registers a thread; C2 0.244 -> 0.236 ms a pass,
// while 96^2 and 64^2 ISMs, whose pass is bound by latency and residency, took 0.259 -> 0.261 and
// 0.075 -> 0.081 ms with it).
template <int NT, bool kLean>
__global__ void __launch_bounds__(NT) pullmid_kernel(PullPushArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    if (kLean)
        pullmid_lean_ism(a, a.row0 * a.grid_x + blockIdx.x, smem);
    else
        pullmid_ism(a, a.row0 * a.grid_x + blockIdx.x, smem);
}
constexpr int kPullMidLeanEdge = 128;
constexpr int kPullMidWideThreads = 512;
constexpr int kPullMidWideBelow = 2 * 152;  // ISMs per launch under which the wide form is used

__global__ void __launch_bounds__(kPpTileW * kPpTileH) push1_kernel(PullPushArgs a) {
    push1_quads(a, blockIdx.x, blockIdx.y);
}

__global__ void __launch_bounds__(kPpTileW * kPpTileH, 5) push0_kernel(PullPushArgs a) {
    push0_quads(a, blockIdx.x, blockIdx.y);
}

#include "pyramid.cuh"

// pull1_kernel on the one-block pyramid's arithmetic (pull1_lean: selects instead of branches, the
// displacement mean from a table), for far planes in pyramid_lean_range; bit-identical. Eight
// blocks a SM (32 registers, no spill): the pass 0.2267 -> 0.2243 ms at C2, 0.0740 -> 0.0714 at
// CREF, against the compiler's 34 registers and seven blocks. (Push level 0 at six blocks, 40
// registers with a spill, took 0.2310 ms against 0.2267.)
__global__ void __launch_bounds__(kPpTileW * kPpTileH, 8) pull1_lean_kernel(PullPushArgs a) {
    __shared__ PyramidTables T;
    fill_pyramid_tables(T, a.z_far);
    __syncthreads();
    const int s1 = a.ism_size >> 1, w1 = a.atlas_w >> 1;
    const float fs = float(a.ism_size);
    const size_t nk = (size_t)a.atlas_w * a.atlas_h - 1;  // a pair's first key
#pragma unroll 1
    for (int j = 0; j < kPull1Rows; ++j) {
        const int x = blockIdx.x * kPpTileW + (threadIdx.x % kPpTileW);
        const int y = a.row0 * s1 + (blockIdx.y * kPull1Rows + j) * kPpTileH + (threadIdx.x / kPpTileW);
        if (x >= w1 || y >= a.row1 * s1) continue;
        const uint2 r0 = __ldg(reinterpret_cast<const uint2*>(a.keys + MLGI_IX((size_t)(2 * y) * a.atlas_w + 2 * x, nk)));
        const uint2 r1 = __ldg(reinterpret_cast<const uint2*>(a.keys + MLGI_IX((size_t)(2 * y + 1) * a.atlas_w + 2 * x, nk)));
        const uint32_t key[4] = {r0.x, r1.x, r0.y, r1.y};  // kPullOff order
        a.lv1[MLGI_IX((uint32_t)y * w1 + x, (uint32_t)w1 * (a.atlas_h >> 1))] = pull1_lean(key, T, a.z_far, fs);
    }
}

// push1_kernel on the one-block pyramid's arithmetic (push_term, push_out_lean) for far planes in
// pyramid_lean_range and ISM edges above 64: a quad's four coarse level-2 texels and their terms
// serve its four outputs; a quad whose radius test meets the band is redone with push1_quads'
// exact per-output code. Three blocks a SM (80 registers): C2's pass 0.2315 -> 0.2264 ms, C3-B's
// 0.2536 -> 0.2483; 64^2 ISMs (CREF) took 0.0743 -> 0.0754, so they keep push1_kernel. As
// compiled (105 registers, two blocks) it was slower everywhere.
__global__ void __launch_bounds__(kPpTileW * kPpTileH, 3) push1_lean_kernel(PullPushArgs a) {
    __shared__ PyramidTables T;  // levels >= 1 read only the reciprocal table
    if (threadIdx.x < 20) T.rcp[threadIdx.x] = threadIdx.x == 0 || threadIdx.x > 16 ? 0.f : 1.0f / float(threadIdx.x);
    __syncthreads();
    const int w1 = a.atlas_w >> 1, h1 = a.atlas_h >> 1, w2 = a.atlas_w >> 2, h2 = a.atlas_h >> 2;
    const int s1 = a.ism_size >> 1, Y0 = a.row0 * s1, Y1 = a.row1 * s1;
    const int gx = blockIdx.x * kPpTileW + (threadIdx.x % kPpTileW);
    const int gy = (Y0 >> 1) + blockIdx.y * kPpTileH + (threadIdx.x / kPpTileW);
    if (gx > w2 || gy > (Y1 >> 1)) return;
    const int sc = a.ism_size >> 2;  // ISM edge at level 2
    PushTerm c[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {  // coordinates off the level are clamped, as push_coarse does
        const int cx = min(max(gx - 1 + kPushOff[k][0], 0), w2 - 1), cy = min(max(gy - 1 + kPushOff[k][1], 0), h2 - 1);
        c[k] = push_term(a.lv2[MLGI_IX((uint32_t)cy * (uint32_t)w2 + (uint32_t)cx, (uint32_t)w2 * (uint32_t)h2)], 0.5f);
    }
    const bool bx = multiple_of(gx, sc, a.m_c1), by = multiple_of(gy, sc, a.m_c1);
    const int x0 = 2 * gx - 1, y0 = 2 * gy - 1;
    const bool okx0 = x0 >= 0, okx1 = x0 + 1 < w1, oky0 = y0 >= Y0, oky1 = y0 + 1 < Y1;
    const uint32_t n1 = (uint32_t)w1 * h1;
    const uint32_t o0 = (uint32_t)max(y0, 0) * w1 + x0, o1 = (uint32_t)min(y0 + 1, h1 - 1) * w1 + x0;  // x0 < 0: unused
    float4* lv1 = a.lv1;
    const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 p00 = oky0 && okx0 ? lv1[MLGI_IX(o0, n1)] : z, p10 = oky0 && okx1 ? lv1[MLGI_IX(o0 + 1, n1)] : z;
    const float4 p01 = oky1 && okx0 ? lv1[MLGI_IX(o1, n1)] : z, p11 = oky1 && okx1 ? lv1[MLGI_IX(o1 + 1, n1)] : z;
    bool band = false;
    const float4 r00 = push_out_lean<true, 0, 0>(c, bx, by, p00, band, T);
    const float4 r10 = push_out_lean<true, 1, 0>(c, bx, by, p10, band, T);
    const float4 r01 = push_out_lean<true, 0, 1>(c, bx, by, p01, band, T);
    const float4 r11 = push_out_lean<true, 1, 1>(c, bx, by, p11, band, T);
    if (band) {  // a radius test within 2^-20 of the radius: the exact per-output form
        push1_quads(a, blockIdx.x, blockIdx.y);
        return;
    }
    if (oky0 && okx0) lv1[MLGI_IX(o0, n1)] = r00;
    if (oky0 && okx1) lv1[MLGI_IX(o0 + 1, n1)] = r10;
    if (oky1 && okx0) lv1[MLGI_IX(o1, n1)] = r01;
    if (oky1 && okx1) lv1[MLGI_IX(o1 + 1, n1)] = r11;
}

static void launch_push1(const PullPushArgs& a, const dim3 grid, cudaStream_t s) {
    if (a.ism_size > 64 && pyramid_lean_range(a.z_far))
        push1_lean_kernel<<<grid, kPpTileW * kPpTileH, 0, s>>>(a);
    else
        push1_kernel<<<grid, kPpTileW * kPpTileH, 0, s>>>(a);
}

static void launch_pull1(const PullPushArgs& a, const dim3 grid, cudaStream_t s) {
    if (pyramid_lean_range(a.z_far))
        pull1_lean_kernel<<<grid, kPpTileW * kPpTileH, 0, s>>>(a);
    else
        pull1_kernel<<<grid, kPpTileW * kPpTileH, 0, s>>>(a);
}

// The tables of either middle pass (pullmid_ism's key tables, the lean pass's PyramidTables), then
// levels 2..L.
size_t pullmid_smem_bytes(int ism_size, int levels) {
    size_t b = std::max(kPullPushTableBytes, kPyramidTableBytes);
    for (int l = 2; l <= levels; ++l) b += (size_t)(ism_size >> l) * (ism_size >> l) * 16;
    return b;
}

size_t pullpush_scratch_bytes(int atlas_w, int atlas_h, int levels, size_t* lv2_offset) {
    const size_t lv1 = (size_t)(atlas_w >> 1) * (atlas_h >> 1) * 16;
    const size_t lv2 = levels >= 2 ? (size_t)(atlas_w >> 2) * (atlas_h >> 2) * 16 : 0;
    if (lv2_offset) *lv2_offset = (lv1 + 255) & ~(size_t)255;
    return ((lv1 + 255) & ~(size_t)255) + lv2;
}

__host__ __device__ __forceinline__ int tiles_x(int w) { return (w + kPpTileW - 1) / kPpTileW; }
__host__ __device__ __forceinline__ int tiles_y(int h) { return (h + kPpTileH - 1) / kPpTileH; }
// Work items of the batched per-texel passes: runs of kPpBatchTiles tiles along a tile row.
__host__ __device__ __forceinline__ int row_items(int w) { return (tiles_x(w) + kPpBatchTiles - 1) / kPpBatchTiles; }

cudaError_t pullpush_prepare(size_t smem) {
    cudaError_t e = cudaFuncSetAttribute(pullmid_kernel<kPullMidThreads, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(pullmid_kernel<kPullMidThreads, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(pullmid_kernel<kPullMidWideThreads, false>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess) e = pyramid_prepare();
    return e;
}

static void launch_pullmid(const PullPushArgs& a, int isms, size_t smem, cudaStream_t s) {
    if (isms < kPullMidWideBelow)
        pullmid_kernel<kPullMidWideThreads, false><<<isms, kPullMidWideThreads, smem, s>>>(a);
    else if (a.ism_size >= kPullMidLeanEdge && pyramid_lean_range(a.z_far))
        pullmid_kernel<kPullMidThreads, true><<<isms, kPullMidThreads, smem, s>>>(a);
    else
        pullmid_kernel<kPullMidThreads, false><<<isms, kPullMidThreads, smem, s>>>(a);
}

// Grids of the four launches over ISM rows [a.row0, a.row1).
struct PullPushGrids {
    dim3 g1, q1, q0;
    int isms;
};

static PullPushGrids pullpush_grids(const PullPushArgs& a) {
    const int w1 = a.atlas_w >> 1, rows = a.row1 - a.row0;
    const int s1 = a.ism_size >> 1, s0 = a.ism_size;
    PullPushGrids g;
    g.g1 = dim3(tiles_x(w1), (tiles_y(rows * s1) + kPull1Rows - 1) / kPull1Rows);
    g.q1 = dim3(tiles_x(w1 / 2 + 1), tiles_y(((a.row1 * s1) >> 1) - ((a.row0 * s1) >> 1) + 1));
    g.q0 = dim3(tiles_x(w1 + 1), tiles_y(((a.row1 * s0) >> 1) - ((a.row0 * s0) >> 1) + 1));
    g.isms = rows * a.grid_x;
    return g;
}

cudaError_t launch_pullpush_captured(const PullPushArgs& a, cudaStream_t s) {
    if (a.row1 <= a.row0) return cudaSuccess;
    if (pyramid_launch_fused(a)) {
        launch_pyramid(a, s);
        return cudaGetLastError();
    }
    const PullPushGrids g = pullpush_grids(a);
    launch_pull1(a, g.g1, s);
    if (a.levels >= 2) {
        launch_pullmid(a, g.isms, pullmid_smem_bytes(a.ism_size, a.levels), s);
        launch_push1(a, g.q1, s);
    }
    push0_kernel<<<g.q0, kPpTileW * kPpTileH, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_pullpush(const PullPushArgs& a, cudaStream_t s, cudaEvent_t* marks) {
    if (a.row1 <= a.row0) return cudaSuccess;
    if (pyramid_launch_fused(a)) {
        const cudaError_t e = pyramid_prepare();
        if (e != cudaSuccess) return e;
        if (marks)  // one launch: the pass's time lands in the last of the four slots
            for (int k = 0; k < 3; ++k) cudaEventRecord(marks[k], s);
        launch_pyramid(a, s);
        return cudaGetLastError();
    }
    const PullPushGrids g = pullpush_grids(a);
    launch_pull1(a, g.g1, s);
    if (marks) cudaEventRecord(marks[0], s);
    if (a.levels >= 2) {
        const size_t smem = pullmid_smem_bytes(a.ism_size, a.levels);
        cudaError_t e = pullpush_prepare(smem);
        if (e != cudaSuccess) return e;
        launch_pullmid(a, g.isms, smem, s);
        if (marks) cudaEventRecord(marks[1], s);
        launch_push1(a, g.q1, s);
    } else if (marks) {
        cudaEventRecord(marks[1], s);
    }
    if (marks) cudaEventRecord(marks[2], s);
    push0_kernel<<<g.q0, kPpTileW * kPpTileH, 0, s>>>(a);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------
// Persistent forms over a view table: block b takes work items b, b + gridDim.x, ... of the pass;
// their register budgets (launch bounds) keep the occupancy of the single-view kernels, which the
// loop state would otherwise lower;
// an item is (view, index inside the view) found from the pass's running item counts. Each item
// runs exactly the single-view body, so batched results equal single-frame results bit for bit.

__global__ void __launch_bounds__(256) batch_clear_kernel(BatchTable t) {
    __shared__ int s_pre[kBatchPrefixCache + 1];
    ItemWalk w;
    w.init(t.prefix + kBpClear * (t.n_views + 1), t.n_views, s_pre);
    for (int item = blockIdx.x; item < w.total; item += gridDim.x) {
        const BatchView& V = t.views[w.view(item)];
        const size_t first = (size_t)w.local(item) * kBatchClearTexels;
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
    __shared__ int s_pre[kBatchPrefixCache + 1];
    ItemWalk w;
    w.init(t.prefix + kBpVpl * (t.n_views + 1), t.n_views, s_pre);
    for (int item = blockIdx.x; item < w.total; item += gridDim.x) {
        const int v = w.view(item);
        vpl_one(t.views[v].vpl, (uint32_t)w.local(item) * kBatchVplPerItem + threadIdx.x);
    }
}

__global__ void __launch_bounds__(kSplatThreads, 6) batch_splat_kernel(BatchTable t) {
    __shared__ SplatSmem S;
    __shared__ SplatArgs args;  // the item's view arguments, staged once per item
    __shared__ int s_pre[kBatchPrefixCache + 1];
    ItemWalk w;
    w.init(t.prefix + kBpSplat * (t.n_views + 1), t.n_views, s_pre);
    int cur = -1;
    for (int item = blockIdx.x; item < w.total; item += gridDim.x) {
        const int v = w.view(item);
        if (v != cur) {  // v is uniform over the block
            __syncthreads();
            if (threadIdx.x == 0) args = t.views[v].splat;
            __syncthreads();
            cur = v;
        }
        splat_bucket(args, w.local(item), S);
    }
}

// Pull-push passes over the view table. An item is kPpBatchTiles texel tiles (or one ISM for the
// middle pass); the view's arguments (and the key tables of pull level 1) are staged in shared
// memory when a block moves to another view.
__device__ __forceinline__ bool stage_pp_args(const BatchTable& t, const int v, int& cur, PullPushArgs& args) {
    if (v == cur) return false;  // v is uniform over the block
    __syncthreads();
    if (threadIdx.x == 0) args = t.views[v].pp;
    __syncthreads();
    cur = v;
    return true;
}

__global__ void __launch_bounds__(kPpTileW * kPpTileH, 6) batch_pull1_kernel(BatchTable t) {
    __shared__ float s_tab[512];
    __shared__ PullPushArgs args;
    __shared__ int s_pre[kBatchPrefixCache + 1];
    ItemWalk w;
    w.init(t.prefix + kBpPull1 * (t.n_views + 1), t.n_views, s_pre);
    int cur = -1;
    for (int item = blockIdx.x; item < w.total; item += gridDim.x) {
        const int v = w.view(item);
        if (stage_pp_args(t, v, cur, args)) {
            fill_key_tables(s_tab, s_tab + 256, args.z_far);
            __syncthreads();
        }
        const int w1 = args.atlas_w >> 1, per_row = row_items(w1), i = w.local(item);
        const int ty = i / per_row, tx0 = (i - ty * per_row) * kPpBatchTiles;
        for (int tx = tx0; tx < tx0 + kPpBatchTiles && tx < tiles_x(w1); ++tx) pull1_tile(args, tx, ty, s_tab, s_tab + 256);
    }
}

__global__ void __launch_bounds__(kPullMidThreads, 8) batch_pullmid_kernel(BatchTable t) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ PullPushArgs args;
    __shared__ int s_pre[kBatchPrefixCache + 1];
    ItemWalk w;
    w.init(t.prefix + kBpPullMid * (t.n_views + 1), t.n_views, s_pre);
    int cur = -1;
    for (int item = blockIdx.x; item < w.total; item += gridDim.x) {
        const int v = w.view(item);
        stage_pp_args(t, v, cur, args);
        pullmid_ism(args, w.local(item), smem);
    }
}

__global__ void __launch_bounds__(kPpTileW * kPpTileH, 4) batch_push1_kernel(BatchTable t) {
    __shared__ PullPushArgs args;
    __shared__ int s_pre[kBatchPrefixCache + 1];
    ItemWalk w;
    w.init(t.prefix + kBpPush1 * (t.n_views + 1), t.n_views, s_pre);
    int cur = -1;
    for (int item = blockIdx.x; item < w.total; item += gridDim.x) {
        const int v = w.view(item);
        stage_pp_args(t, v, cur, args);
        const int qw = (args.atlas_w >> 2) + 1, per_row = row_items(qw), i = w.local(item);
        const int ty = i / per_row, tx0 = (i - ty * per_row) * kPpBatchTiles;
        for (int tx = tx0; tx < tx0 + kPpBatchTiles && tx < tiles_x(qw); ++tx) push1_quads(args, tx, ty);
    }
}

__global__ void __launch_bounds__(kPpTileW * kPpTileH, 5) batch_push0_kernel(BatchTable t) {
    __shared__ PullPushArgs args;
    __shared__ int s_pre[kBatchPrefixCache + 1];
    ItemWalk w;
    w.init(t.prefix + kBpPush0 * (t.n_views + 1), t.n_views, s_pre);
    int cur = -1;
    for (int item = blockIdx.x; item < w.total; item += gridDim.x) {
        const int v = w.view(item);
        stage_pp_args(t, v, cur, args);
        const int qw = (args.atlas_w >> 1) + 1, per_row = row_items(qw), i = w.local(item);
        const int ty = i / per_row, tx0 = (i - ty * per_row) * kPpBatchTiles;
        for (int tx = tx0; tx < tx0 + kPpBatchTiles && tx < tiles_x(qw); ++tx) push0_quads(args, tx, ty);
    }
}

int pullpush_batch_items(int pass, int atlas_w, int atlas_h, int ism_count, int levels) {
    const int w1 = atlas_w >> 1, h1 = atlas_h >> 1;
    switch (pass) {
        case kBpPull1: return row_items(w1) * tiles_y(h1);
        case kBpPullMid: return levels >= 2 ? ism_count : 0;
        case kBpPush1: return levels >= 2 ? row_items(w1 / 2 + 1) * tiles_y(h1 / 2 + 1) : 0;
        case kBpPush0: return row_items(w1 + 1) * tiles_y(h1 + 1);
        default: return 0;
    }
}

cudaError_t launch_batch_ism(const BatchTable& t, int pass, int grid, size_t smem, cudaStream_t s) {
    if (grid <= 0) return cudaSuccess;
    switch (pass) {
        case kBpClear: batch_clear_kernel<<<grid, 256, 0, s>>>(t); break;
        case kBpVpl: batch_vpl_kernel<<<grid, kBatchVplPerItem, 0, s>>>(t); break;
        case kBpSplat: batch_splat_kernel<<<grid, kSplatThreads, 0, s>>>(t); break;
        case kBpPull1: batch_pull1_kernel<<<grid, kPpTileW * kPpTileH, 0, s>>>(t); break;
        case kBpPullMid:  // the dynamic shared-memory limit was raised by batch_blocks_per_sm()
            batch_pullmid_kernel<<<grid, kPullMidThreads, smem, s>>>(t);
            break;
        case kBpPush1: batch_push1_kernel<<<grid, kPpTileW * kPpTileH, 0, s>>>(t); break;
        case kBpPush0: batch_push0_kernel<<<grid, kPpTileW * kPpTileH, 0, s>>>(t); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

int batch_blocks_per_sm(int pass, size_t smem) {
    int n = 1;
    const int tt = kPpTileW * kPpTileH;
    switch (pass) {
        case kBpClear: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_clear_kernel, 256, 0); break;
        case kBpVpl: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_vpl_kernel, kBatchVplPerItem, 0); break;
        case kBpSplat: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_splat_kernel, kSplatThreads, 0); break;
        case kBpPull1: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_pull1_kernel, tt, 0); break;
        case kBpPullMid:
            cudaFuncSetAttribute(batch_pullmid_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_pullmid_kernel, kPullMidThreads, smem);
            break;
        case kBpPush1: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_push1_kernel, tt, 0); break;
        case kBpPush0: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_push0_kernel, tt, 0); break;
        default: break;
    }
    return n > 0 ? n : 1;
}

}  // namespace mlgi

MLGI_CHECK_UNIT(ism_kernels)
