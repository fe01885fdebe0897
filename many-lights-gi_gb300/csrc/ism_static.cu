// Allocation-free ISM rendering: splat + pull-push with the softrender key atlas held in a
// fixed, statically allocated device array instead of caller- or context-owned memory.
//
// Who needs it: code that must not call cudaMalloc -- e.g. a renderer running inside a host
// process whose device memory is fully reserved up front by another allocator, a plugin that is
// only handed pre-allocated buffers, or a callback that runs while the CUDA allocator is locked.
// Such callers still pass their own input (points, VPLs) and output (final depth atlas) buffers;
// only the intermediates -- the key atlas and pull-push pyramid levels 1 and 2 -- live here. (The
// pyramid levels are used only by the per-level pull-push form; where an ISM's pyramid runs in
// one block, its levels stay in that block's shared memory.)
//
// Limits and behaviour:
//   * The key atlas holds at most kStaticKeyTexels = 1,048,576 texels (a 1024 x 1024 atlas,
//     4 MiB), the pyramid levels a quarter and a sixteenth of that as float4 (5 MiB). Larger
//     atlases are rejected with MLGI_EINVAL, and so is any geometry the allocating entry points
//     refuse (the same checks, e.g. at most 65535 texels a side).
//   * When the 9 MiB are reserved: the arrays belong to this file's module. Under the CUDA
//     runtime's default lazy module loading, a device creates the module -- and reserves the
//     9 MiB -- at the first call on that device, when the call looks the arrays up
//     (cudaGetSymbolAddress) with the device current; with CUDA_MODULE_LOADING=EAGER it happens
//     when the context is created. A caller whose other allocator reserves the device's memory
//     up front should make its first call before that reservation (or load eagerly); if the
//     reservation leaves no room, the first call returns MLGI_ENOMEM. From then on the arrays stay
//     until the process exits. Make the first call before any stream capture.
//   * The looked-up addresses are kept per device for the life of the process, so the entry
//     point must not be used on a device after cudaDeviceReset of that device.
//   * All calls share the one set of arrays. Each call clears it to the empty key (0xFFFFFFFF) before
//     splatting, so nothing of a previous call leaks into the result, but calls whose work
//     overlaps on the GPU (different streams, or different host threads) race on it.
//   * No cudaMalloc, cudaFree or allocating library call is made.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>

#include "kernels.h"
#include "mlgi.h"

namespace {

constexpr size_t kStaticKeyTexels = size_t(1) << 20;

// levels 1 and 2 of a kStaticKeyTexels atlas, laid out as pullpush_scratch_bytes() describes
constexpr size_t kStaticPyramidFloat4 = (kStaticKeyTexels / 4) + 16 + kStaticKeyTexels / 16;

__device__ __align__(256) uint32_t g_static_keys[kStaticKeyTexels];
__device__ __align__(256) float4 g_static_pyramid[kStaticPyramidFloat4];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
uint32_t* g_static_keys_dev[kMaxDevices] = {};
void* g_static_pyramid_dev[kMaxDevices] = {};

// Device addresses of g_static_keys and g_static_pyramid on the current device (resolved once
// per device).
mlgi_status static_addresses(uint32_t** keys, void** pyramid) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return MLGI_ECUDA;
    }
    if (dev < 0 || dev >= kMaxDevices) return MLGI_EINVAL;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_static_keys_dev[dev]) {
        void *p = nullptr, *q = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_static_keys);
        if (e == cudaSuccess) e = cudaGetSymbolAddress(&q, g_static_pyramid);
        if (e != cudaSuccess || !p || !q) {
            cudaGetLastError();
            // loading the module reserves the arrays; no room for them is an allocation failure
            return e == cudaErrorMemoryAllocation ? MLGI_ENOMEM : MLGI_ECUDA;
        }
        g_static_pyramid_dev[dev] = q;
        g_static_keys_dev[dev] = static_cast<uint32_t*>(p);
    }
    *keys = g_static_keys_dev[dev];
    *pyramid = g_static_pyramid_dev[dev];
    return MLGI_OK;
}

}  // namespace

extern "C" mlgi_status mlgi_ism_render_static(const mlgi_points* pts, const mlgi_vpl_buf* vpls, int n_vpl,
                                              const mlgi_ism_params* p, void* depth_out, int depth_format,
                                              mlgi_stream stream) {
    if (!pts || !vpls || !p || !depth_out) return MLGI_EINVAL;
    if (depth_format != MLGI_F32 && depth_format != MLGI_F16) return MLGI_EINVAL;
    char why[160];
    if (!mlgi::ism_params_valid(p, why, sizeof(why))) return MLGI_EINVAL;  // the allocating path's checks
    const size_t aw = (size_t)p->grid_x * p->ism_size, ah = (size_t)p->grid_y * p->ism_size;
    if (aw * ah > kStaticKeyTexels) return MLGI_EINVAL;  // beyond the static key atlas
    if (n_vpl <= 0 || n_vpl > vpls->capacity || p->vpl_end > n_vpl)
        return MLGI_EINVAL;
    const int vplCount = p->vpl_end - p->vpl_start;
    if ((p->scale_isms ? vplCount : n_vpl) > p->grid_x * p->grid_y) return MLGI_EINVAL;
    if (pts->n_buckets != (p->points_only_scaled ? vplCount : n_vpl)) return MLGI_EINVAL;
    if (pts->n_buckets > 0 && (!pts->points || !pts->counts || pts->bucket_stride < 0)) return MLGI_EINVAL;
    if (!vpls->packed || (reinterpret_cast<uintptr_t>(vpls->packed) & 15) ||
        (reinterpret_cast<uintptr_t>(pts->points) & 15))
        return MLGI_EINVAL;
    if (mlgi::pullmid_smem_bytes(p->ism_size, p->levels) > 227 * 1024) return MLGI_EINVAL;
    size_t lv2_off = 0;
    if (mlgi::pullpush_scratch_bytes((int)aw, (int)ah, p->levels, &lv2_off) > kStaticPyramidFloat4 * sizeof(float4))
        return MLGI_EINVAL;

    uint32_t* keys = nullptr;
    void* pyramid = nullptr;
    const mlgi_status st = static_addresses(&keys, &pyramid);
    if (st != MLGI_OK) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);

    if (mlgi::launch_ism_clear(keys, aw * ah, s) != cudaSuccess) return MLGI_ECUDA;
    mlgi::SplatArgs a{};
    a.points = reinterpret_cast<const float4*>(pts->points);
    a.counts = pts->counts;
    a.bucket_stride = pts->bucket_stride;
    a.n_entries = (int64_t)pts->n_buckets * pts->bucket_stride;
    a.n_groups = pts->n_buckets;
    a.chunks = (int)std::max<int64_t>(1, (pts->bucket_stride + mlgi::kSplatChunk - 1) / mlgi::kSplatChunk);
    a.packed = reinterpret_cast<const float4*>(vpls->packed);
    a.n_vpl = n_vpl;
    a.vpl_start = p->vpl_start;
    a.vpl_end = p->vpl_end;
    a.scale_isms = p->scale_isms;
    a.points_only_scaled = p->points_only_scaled;
    a.gx = p->grid_x;
    a.gy = p->grid_y;
    a.atlas_w = (int)aw;
    a.atlas_h = (int)ah;
    a.z_far = p->z_far;
    a.keys = keys;
    if (mlgi::launch_ism_splat(a, s) != cudaSuccess) return MLGI_ECUDA;
    mlgi::PullPushArgs q{};
    q.keys = keys;
    q.out = depth_out;
    q.out_f16 = depth_format == MLGI_F16;
    q.atlas_w = (int)aw;
    q.atlas_h = (int)ah;
    q.ism_size = p->ism_size;
    q.levels = p->levels;
    q.grid_x = p->grid_x;
    q.grid_y = p->grid_y;
    q.z_far = p->z_far;
    q.m_c0 = mlgi::small_div_magic(p->ism_size >> 1);
    q.m_c1 = mlgi::small_div_magic(p->ism_size >> 2);
    q.lv1 = static_cast<float4*>(pyramid);
    q.lv2 = p->levels >= 2 ? reinterpret_cast<float4*>(static_cast<char*>(pyramid) + lv2_off) : nullptr;
    q.row0 = 0;
    q.row1 = p->grid_y;
    if (mlgi::launch_pullpush(q, s) != cudaSuccess) return MLGI_ECUDA;
    return MLGI_OK;
}
