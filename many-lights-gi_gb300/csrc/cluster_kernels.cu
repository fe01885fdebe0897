// Reference-style clustered light culling: ClusteredShading::process (ClusteredShading.cpp:70-112)
// with clustering.comp:30-86 and light_lists.comp:50-126, an alternative to the gathering's own
// per-tile culler for parity studies.
//
// Clusters are 128 x 128-pixel screen tiles times 16 logarithmic depth slices. cluster_mark_kernel
// records the slice of every pixel and the slices each tile uses; cluster_lists_kernel keeps, for
// every used cluster, the VPLs for which any of the cluster's corners lies on the front side of the
// VPL's plane, as a bitmask over the VPLs (the reference writes 16-bit index lists in atomic order;
// the set is the same, the order here is the index order, so the gathering is deterministic).
// Kept as the reference has them: slice 0's front plane at view z = +0.05 (sliceToZ), and the
// corner list with (left, top) twice in place of (right, top) (light_lists.comp:82-83).
// Deviations, each because the reference's behaviour is undefined or inconsistent:
//   * the slice index is clamped to 15: at the far plane the formula gives 16 (clustering.comp:50
//     then writes usedDepthSlices[16], past its 16 entries);
//   * the gathering finds its cluster with the clustering pass's scale log2(zFar)
//     (final_gathering.comp:83 hard-codes log2(50), which agrees only for zFar = 50).
// Compiled with -fmad=false and IEEE division/square root, so the cull decisions follow the
// shaders' FP32 operation order word for word.
#include <cuda_runtime.h>

#include "checks.cuh"
#include "gi_device.cuh"
#include "kernels.h"

namespace mlgi {

// reprojection.glsl:6-24
__device__ __forceinline__ float linear_depth(float z_b, float A, float B) {
    const float z_n = 2.0f * z_b - 1.0f;
    return -B / (A + z_n);
}

__device__ __forceinline__ float log_depth(float z_e, float A, float B) {
    const float z_n = (1.0f / z_e * -B) - A;
    return (z_n + 1.0f) / 2.0f;
}

// clustering.comp:24, 50 (clamped, see above)
__device__ __forceinline__ int depth_slice(float lin, float scale) {
    const float s = gmax(log2f(-lin) * scale - float(kClusterSlicesIntoFirst), 0.0f);
    return min(f2i(s), kClusterSlices - 1);
}

// A block covers kClusterPixels columns (one tile) of kMarkRows rows, all in one tile; its slice
// bits are OR-reduced in the block and set with one atomic (a per-pixel atomic on the tile's word
// serialises on the few tile words: 1.13 ms at 1080p against microseconds reduced).
constexpr int kMarkRows = 8;
static_assert(kClusterPixels % kMarkRows == 0, "a block's rows lie in one tile");
__global__ void __launch_bounds__(kClusterPixels) cluster_mark_kernel(ClusterArgs a) {
    const int x = blockIdx.x * kClusterPixels + threadIdx.x;
    uint32_t bits = 0;
#pragma unroll 1
    for (int r = 0; r < kMarkRows; ++r) {
        const int y = blockIdx.y * kMarkRows + r;
        if (x < a.width && y < a.height) {
            const size_t p = MLGI_IX((size_t)y * a.width + x, (size_t)a.width * a.height);
            const int slice = depth_slice(linear_depth(__ldg(a.depth + p), a.proj_a, a.proj_b), a.scale);
            a.pixel_slice[p] = (uint8_t)slice;
            bits |= 1u << slice;
        }
    }
    bits = __reduce_or_sync(0xffffffffu, bits);
    __shared__ uint32_t s_bits[kClusterPixels / 32];
    if ((threadIdx.x & 31) == 0) s_bits[threadIdx.x >> 5] = bits;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t v = 0;
        for (int w = 0; w < kClusterPixels / 32; ++w) v |= s_bits[w];
        if (v) atomicOr(a.used + MLGI_IX((blockIdx.y * kMarkRows / kClusterPixels) * a.tiles_x + blockIdx.x, a.tiles_x * a.tiles_y), v);
    }
}

// light_lists.comp:42-47
__device__ __forceinline__ float slice_to_z(int slice, float scale) {
    if (slice == 0) return 0.05f;  // nearPlane
    return -powf(2.0f, float(slice + kClusterSlicesIntoFirst) / scale);
}

// One block per cluster (tile-major, 16 slices per tile); each warp takes 32 consecutive VPLs and
// writes their keep bits as one mask word.
__global__ void __launch_bounds__(128) cluster_lists_kernel(ClusterArgs a) {
    const int cl = MLGI_IX((int)blockIdx.x, a.tiles_x * a.tiles_y * kClusterSlices);
    const int tile = cl / kClusterSlices, slice = cl - tile * kClusterSlices;
    if (!((__ldg(a.used + tile) >> slice) & 1u)) return;  // unused: never read
    const int cx = tile % a.tiles_x, cy = tile / a.tiles_x;
    __shared__ float corner[8][3];
    if (threadIdx.x < 8) {
        const float zFront = slice_to_z(slice, a.scale), zBack = slice_to_z(slice + 1, a.scale);
        const float ndcL = float(cx) * float(kClusterPixels) / float(a.width);
        const float ndcR = float(cx + 1) * float(kClusterPixels) / float(a.width);
        const float ndcB = float(cy) * float(kClusterPixels) / float(a.height);
        const float ndcT = float(cy + 1) * float(kClusterPixels) / float(a.height);
        const float ndcFront = log_depth(zFront, a.proj_a, a.proj_b), ndcBack = log_depth(zBack, a.proj_a, a.proj_b);
        // light_lists.comp:76-83, corners 6 and 7 as the reference has them
        const float cs[8][3] = {{ndcL, ndcB, ndcFront}, {ndcL, ndcB, ndcBack}, {ndcR, ndcB, ndcFront},
                                {ndcR, ndcB, ndcBack},  {ndcL, ndcT, ndcFront}, {ndcL, ndcT, ndcBack},
                                {ndcL, ndcT, ndcFront}, {ndcL, ndcT, ndcBack}};
        const int i = threadIdx.x;
        const float v[4] = {cs[i][0] * 2.0f - 1.0f, cs[i][1] * 2.0f - 1.0f, cs[i][2] * 2.0f - 1.0f, 1.0f * 2.0f - 1.0f};
        const float* m = a.inv_vp;
        float r[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) r[k] = ((m[k] * v[0] + m[4 + k] * v[1]) + m[8 + k] * v[2]) + m[12 + k] * v[3];
        corner[i][0] = r[0] / r[3];
        corner[i][1] = r[1] / r[3];
        corner[i][2] = r[2] / r[3];
    }
    __syncthreads();
    uint32_t* mask = a.masks + (size_t)cl * a.mask_words;
    for (int base = (threadIdx.x & ~31); base < a.n_vpl; base += blockDim.x) {
        const int v = base + (threadIdx.x & 31);
        bool found = false;
        if (v < a.n_vpl) {
            const float4 pk = __ldg(a.packed + MLGI_IX(v, a.n_vpl));
            const v3 n = unpack3SN(__float_as_uint(pk.w));
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const v3 vplToCorner = mk(corner[j][0], corner[j][1], corner[j][2]) - mk(pk.x, pk.y, pk.z);
                found = found || (dot(vplToCorner, n) >= 0.0f);
            }
        }
        const unsigned bits = __ballot_sync(0xffffffffu, found);
        if ((threadIdx.x & 31) == 0) mask[MLGI_IX(base >> 5, a.mask_words)] = bits;
    }
}

cudaError_t launch_cluster_lights(const ClusterArgs& a, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(a.used, 0, sizeof(uint32_t) * a.tiles_x * a.tiles_y, s);
    if (e != cudaSuccess) return e;
    cluster_mark_kernel<<<dim3((a.width + kClusterPixels - 1) / kClusterPixels, (a.height + kMarkRows - 1) / kMarkRows),
                          kClusterPixels, 0, s>>>(a);
    cluster_lists_kernel<<<a.tiles_x * a.tiles_y * kClusterSlices, 128, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace mlgi

MLGI_CHECK_UNIT(cluster_kernels)
