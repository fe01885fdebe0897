// Device-side scene fixture: the seeded room ray-cast on the GPU into the camera G-buffer and the
// light's RSM, and its surface points sampled and bucketed on the GPU. This replaces, for served
// and batched frames, the host ray caster of host/scene.cpp (itself the stand-in for the
// reference's RasterizationStage::render, RasterizationStage.cpp:151-277, and its tessellation
// point generator, ism.geom:49-70), so that a frame needs no per-frame upload. The room
// description (objects, sampling table, matrices) is one kernel parameter (host/room.h). FP32
// math: values match the host fixture to rounding, not bit for bit.
#include <cuda_runtime.h>
#include <cuda_fp16.h>

#include "../host/room.h"
#include "checks.cuh"
#include "kernels.h"
#include "mlgi.h"

namespace mlgi {
namespace {

struct Ray {
    float ox, oy, oz, dx, dy, dz;
};
struct Hit {
    float t, nx, ny, nz;
    const float* albedo;
};

__device__ __forceinline__ void xform(const float* m, float x, float y, float z, float w, float* o) {
#pragma unroll
    for (int r = 0; r < 4; ++r) o[r] = m[r] * x + m[4 + r] * y + m[8 + r] * z + m[12 + r] * w;
}

// Ray through the centre of pixel (x, y) of a w x h view with inverse view-projection `inv`.
__device__ Ray pixel_ray(const float* inv, int x, int y, int w, int h) {
    const float nx = (x + 0.5f) / w * 2.f - 1.f, ny = (y + 0.5f) / h * 2.f - 1.f;
    float a[4], b[4];
    xform(inv, nx, ny, -1.f, 1.f, a);
    xform(inv, nx, ny, 1.f, 1.f, b);
    Ray r;
    r.ox = a[0] / a[3];
    r.oy = a[1] / a[3];
    r.oz = a[2] / a[3];
    float dx = b[0] / b[3] - r.ox, dy = b[1] / b[3] - r.oy, dz = b[2] / b[3] - r.oz;
    const float il = rsqrtf(dx * dx + dy * dy + dz * dz);
    r.dx = dx * il;
    r.dy = dy * il;
    r.dz = dz * il;
    return r;
}

__device__ bool trace(const RoomGPU& R, const Ray& ray, Hit& h) {
    constexpr float kRoom = 100.f;
    h.t = 3.0e38f;
    bool any = false;
    const float o[3] = {ray.ox, ray.oy, ray.oz}, d[3] = {ray.dx, ray.dy, ray.dz};
    const int axis[5] = {1, 1, 2, 0, 0};
    const float val[5] = {0.f, kRoom, 0.f, 0.f, kRoom};
    const float nrm[5] = {1.f, -1.f, 1.f, 1.f, -1.f};
#pragma unroll
    for (int w = 0; w < 5; ++w) {
        const int ax = axis[w];
        if (fabsf(d[ax]) < 1e-30f) continue;
        const float t = (val[w] - o[ax]) / d[ax];
        if (t <= 0.f || t >= h.t) continue;
        bool inside = true;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            if (k == ax) continue;
            const float c = o[k] + d[k] * t;
            if (c < 0.f || c > kRoom) inside = false;
        }
        if (!inside) continue;
        h.t = t;
        h.nx = ax == 0 ? nrm[w] : 0.f;
        h.ny = ax == 1 ? nrm[w] : 0.f;
        h.nz = ax == 2 ? nrm[w] : 0.f;
        h.albedo = R.wall_albedo[w];
        any = true;
    }
    for (int i = 0; i < R.n_boxes; ++i) {
        float t0 = 0.f, t1 = h.t, es = 0.f;
        int ea = -1;
        bool miss = false;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float lo = R.box_lo[i][k], hi = R.box_hi[i][k];
            if (fabsf(d[k]) < 1e-30f) {
                if (o[k] < lo || o[k] > hi) miss = true;
                continue;
            }
            float ta = (lo - o[k]) / d[k], tb = (hi - o[k]) / d[k], sg = -1.f;
            if (ta > tb) {
                const float tmp = ta;
                ta = tb;
                tb = tmp;
                sg = 1.f;
            }
            if (ta > t0) {
                t0 = ta;
                ea = k;
                es = sg;
            }
            t1 = fminf(t1, tb);
        }
        if (miss || ea < 0 || t0 > t1 || t0 <= 0.f || t0 >= h.t) continue;
        h.t = t0;
        h.nx = ea == 0 ? es : 0.f;
        h.ny = ea == 1 ? es : 0.f;
        h.nz = ea == 2 ? es : 0.f;
        h.albedo = R.box_albedo[i];
        any = true;
    }
    for (int i = 0; i < R.n_spheres; ++i) {
        const float cx = o[0] - R.sph_c[i][0], cy = o[1] - R.sph_c[i][1], cz = o[2] - R.sph_c[i][2];
        const float b = cx * d[0] + cy * d[1] + cz * d[2];
        const float c = cx * cx + cy * cy + cz * cz - R.sph_r[i] * R.sph_r[i];
        const float disc = b * b - c;
        if (disc < 0.f) continue;
        const float t = -b - sqrtf(disc);
        if (t <= 0.f || t >= h.t) continue;
        h.t = t;
        const float inv_r = 1.f / R.sph_r[i];
        h.nx = (o[0] + d[0] * t - R.sph_c[i][0]) * inv_r;
        h.ny = (o[1] + d[1] * t - R.sph_c[i][1]) * inv_r;
        h.nz = (o[2] + d[2] * t - R.sph_c[i][2]) * inv_r;
        h.albedo = R.sph_albedo[i];
        any = true;
    }
    return any;
}

__device__ __forceinline__ uint32_t unorm8(float v) {
    return (uint32_t)__float2int_rn(fminf(fmaxf(v, 0.f), 1.f) * 255.f);
}
__device__ __forceinline__ uint32_t rgba8(float r, float g, float b) {
    return unorm8(r) | (unorm8(g) << 8) | (unorm8(b) << 16) | (255u << 24);
}
__device__ __forceinline__ uint32_t unorm10(float v) {
    return (uint32_t)__float2int_rn(fminf(fmaxf(v * 0.5f + 0.5f, 0.f), 1.f) * 1023.f);
}

__device__ float window_depth(const float* vp, float x, float y, float z) {
    float c[4];
    xform(vp, x, y, z, 1.f, c);
    return c[2] / c[3] * 0.5f + 0.5f;
}

__global__ void raster_camera_kernel(const RoomGPU R, int w, int h, float* depth, void* normal, int normal_f16,
                                     uint32_t* albedo) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h) return;
    const size_t i = MLGI_IX((size_t)y * w + x, (size_t)w * h);
    const Ray ray = pixel_ray(R.inv_vp, x, y, w, h);
    Hit hit;
    float d = 1.f, ex = 0.f, ey = 0.f;
    uint32_t alb = 0u;
    if (trace(R, ray, hit)) {
        const float px = ray.ox + ray.dx * hit.t, py = ray.oy + ray.dy * hit.t, pz = ray.oz + ray.dz * hit.t;
        d = window_depth(R.vp, px, py, pz);
        const float l1 = fabsf(hit.nx) + fabsf(hit.ny) + fabsf(hit.nz);
        ex = hit.nx / l1;
        ey = hit.ny / l1;
        if (hit.nz < 0.f) {  // octahedral fold
            const float sx = ex >= 0.f ? 1.f : -1.f, sy = ey >= 0.f ? 1.f : -1.f;
            const float fx = (1.f - fabsf(ey)) * sx, fy = (1.f - fabsf(ex)) * sy;
            ex = fx;
            ey = fy;
        }
        alb = rgba8(hit.albedo[0], hit.albedo[1], hit.albedo[2]);
    }
    if (depth) depth[i] = d;
    if (normal) {
        if (normal_f16)
            reinterpret_cast<__half2*>(normal)[i] = __floats2half2_rn(ex, ey);
        else
            reinterpret_cast<float2*>(normal)[i] = make_float2(ex, ey);
    }
    if (albedo) albedo[i] = alb;
}

__global__ void raster_light_kernel(const RoomGPU R, int w, int h, float* depth, uint32_t* normal, uint32_t* diffuse) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h) return;
    const size_t i = MLGI_IX((size_t)y * w + x, (size_t)w * h);
    const Ray ray = pixel_ray(R.inv_lvp, x, y, w, h);
    Hit hit;
    float d = 1.f;
    uint32_t n10 = 0u, dif = 0u;
    if (trace(R, ray, hit)) {
        const float px = ray.ox + ray.dx * hit.t, py = ray.oy + ray.dy * hit.t, pz = ray.oz + ray.dz * hit.t;
        d = window_depth(R.lvp, px, py, pz);
        n10 = unorm10(hit.nx) | (unorm10(hit.ny) << 10) | (unorm10(hit.nz) << 20) | (3u << 30);
        const float cosr = fmaxf(0.f, -(hit.nx * ray.dx + hit.ny * ray.dy + hit.nz * ray.dz));
        const float cone = (ray.dx * R.light_dir[0] + ray.dy * R.light_dir[1] + ray.dz * R.light_dir[2]) >= R.cos_cone
                               ? 1.f : 0.f;
        const float s = cosr * cone;
        dif = rgba8(hit.albedo[0] * s, hit.albedo[1] * s, hit.albedo[2] * s);
    }
    if (depth) depth[i] = d;
    if (normal) normal[i] = n10;
    if (diffuse) diffuse[i] = dif;
}

__device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}
__device__ __forceinline__ float u01(uint64_t& s) {
    s = splitmix64(s);
    return (float)(s >> 40) * (1.0f / 16777216.0f);
}

// One point per thread: area-uniform surface sample, bucketed round-robin (bucket k % B, slot k / B).
__global__ void points_kernel(const RoomGPU R, int64_t n_points, int n_buckets, int64_t stride, float4* points) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= n_points) return;
    uint64_t st = R.point_seed ^ ((uint64_t)k * 0xD1B54A32D192ED03ull);
    const float u0 = u01(st) * R.total_area, u1 = u01(st), u2 = u01(st);
    int lo = 0, hi = R.n_patches - 1;  // first patch whose running area >= u0
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (R.cdf[mid] < u0) lo = mid + 1; else hi = mid;
    }
    float px, py, pz, nx, ny, nz;
    lo = MLGI_IX(lo, R.n_patches < kRoomMaxPatches ? R.n_patches : kRoomMaxPatches);
    if (R.patch_kind[lo] == 0) {
        px = R.patch_o[lo][0] + R.patch_a[lo][0] * u1 + R.patch_b[lo][0] * u2;
        py = R.patch_o[lo][1] + R.patch_a[lo][1] * u1 + R.patch_b[lo][1] * u2;
        pz = R.patch_o[lo][2] + R.patch_a[lo][2] * u1 + R.patch_b[lo][2] * u2;
        nx = R.patch_n[lo][0];
        ny = R.patch_n[lo][1];
        nz = R.patch_n[lo][2];
    } else {  // Marsaglia: a point of the unit disk by rejection (bounded), lifted to the sphere
        float a = 2.f * u1 - 1.f, b = 2.f * u2 - 1.f, q = a * a + b * b;
        for (int tries = 0; (q >= 1.f || q == 0.f) && tries < 64; ++tries) {
            a = 2.f * u01(st) - 1.f;
            b = 2.f * u01(st) - 1.f;
            q = a * a + b * b;
        }
        if (q >= 1.f || q == 0.f) {
            a = 0.f;
            b = 0.f;
            q = 0.f;
        }
        const float r2 = 2.f * sqrtf(1.f - q);
        nx = a * r2;
        ny = b * r2;
        nz = 1.f - 2.f * q;
        px = R.patch_o[lo][0] + nx * R.patch_r[lo];
        py = R.patch_o[lo][1] + ny * R.patch_r[lo];
        pz = R.patch_o[lo][2] + nz * R.patch_r[lo];
    }
    const uint32_t w = unorm8(nx * 0.5f + 0.5f) | (unorm8(ny * 0.5f + 0.5f) << 8) | (unorm8(nz * 0.5f + 0.5f) << 16) |
                       (unorm8(R.r_boost / 25.f) << 24);
    const int64_t b = k % n_buckets, slot = k / n_buckets;
    points[MLGI_IX(b * stride + slot, (int64_t)n_buckets * stride)] = make_float4(px, py, pz, __uint_as_float(w));
}

__global__ void counts_kernel(int64_t n_points, int n_buckets, uint32_t* counts) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n_buckets) return;
    counts[b] = (uint32_t)(n_points / n_buckets + (b < n_points % n_buckets ? 1 : 0));
}

}  // namespace
}  // namespace mlgi

extern "C" mlgi_status mlgi_scene_generate_device(const mlgi_scene_desc* desc, mlgi_scene_info* info, float* gbuf_depth,
                                                  void* gbuf_normal, int gbuf_normal_format, uint32_t* gbuf_albedo,
                                                  float* rsm_depth, uint32_t* rsm_normal, uint32_t* rsm_diffuse,
                                                  float* points, uint32_t* counts, mlgi_stream stream) {
    using namespace mlgi;
    if (!desc) return MLGI_EINVAL;
    if (gbuf_normal_format != MLGI_F32 && gbuf_normal_format != MLGI_F16) return MLGI_EINVAL;
    RoomGPU room;
    mlgi_scene_info local;
    const mlgi_status st = build_room(*desc, &room, info ? info : &local);
    if (st != MLGI_OK) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const dim3 blk(16, 16);
    if ((gbuf_depth || gbuf_normal || gbuf_albedo) && desc->width > 0 && desc->height > 0) {
        const dim3 grid((desc->width + 15) / 16, (desc->height + 15) / 16);
        raster_camera_kernel<<<grid, blk, 0, s>>>(room, desc->width, desc->height, gbuf_depth, gbuf_normal,
                                                  gbuf_normal_format == MLGI_F16, gbuf_albedo);
    }
    if ((rsm_depth || rsm_normal || rsm_diffuse) && desc->rsm_width > 0 && desc->rsm_height > 0) {
        const dim3 grid((desc->rsm_width + 15) / 16, (desc->rsm_height + 15) / 16);
        raster_light_kernel<<<grid, blk, 0, s>>>(room, desc->rsm_width, desc->rsm_height, rsm_depth, rsm_normal,
                                                 rsm_diffuse);
    }
    const int64_t stride = (desc->n_points + desc->n_buckets - 1) / desc->n_buckets;
    if (points && desc->n_points > 0) {
        if (reinterpret_cast<uintptr_t>(points) & 15) return MLGI_EINVAL;
        points_kernel<<<(unsigned)((desc->n_points + 255) / 256), 256, 0, s>>>(room, desc->n_points, desc->n_buckets,
                                                                               stride, reinterpret_cast<float4*>(points));
    }
    if (counts) counts_kernel<<<(desc->n_buckets + 255) / 256, 256, 0, s>>>(desc->n_points, desc->n_buckets, counts);
    return cudaGetLastError() == cudaSuccess ? MLGI_OK : MLGI_ECUDA;
}

MLGI_CHECK_UNIT(scene_kernels)
