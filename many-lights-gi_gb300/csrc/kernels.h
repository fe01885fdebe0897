// Launch interface between the C ABI (mlgi_api.cu) and the kernel translation units.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "mlgi.h"

namespace mlgi {

// The ISM geometry checks every entry point that takes mlgi_ism_params applies (sizes, level count,
// atlas at most 65535 texels a side, far plane, VPL range); on failure `why` (n bytes) says why.
bool ism_params_valid(const mlgi_ism_params* p, char* why, size_t n);

// Every device and pinned host allocation of the library goes through these. Once the allocations
// that mlgi_set_alloc_fault allows are used up they fail with cudaErrorMemoryAllocation without
// asking CUDA (the simulated out-of-memory of the allocation-failure tests).
cudaError_t dev_alloc(void** p, size_t bytes);
cudaError_t dev_alloc_async(void** p, size_t bytes, cudaStream_t s);
cudaError_t pinned_alloc(void** p, size_t bytes);

#ifdef MLGI_CHECKS
// The bounds-checked build: each kernel translation unit's first index violation since the last
// call, read and cleared (checks.cuh).
cudaError_t checks_take_ism_kernels(unsigned long long* rec);
cudaError_t checks_take_fg_kernels(unsigned long long* rec);
cudaError_t checks_take_scene_kernels(unsigned long long* rec);
cudaError_t checks_take_post_kernels(unsigned long long* rec);
cudaError_t checks_take_cluster_kernels(unsigned long long* rec);
cudaError_t checks_take_mlgi_api(unsigned long long* rec);
#endif

struct VplArgs {
    int n;                 // VPL count (work items)
    uint32_t ax, ay;       // lightsOnAxis
    int rsm_w, rsm_h;
    const float* depth;
    const uint32_t* normal;
    const uint32_t* diffuse;
    float inv_bpv[16];
    float intensity;
    const int32_t* perm;   // nullptr: no shuffle
    float4* vpl;           // 3 float4 per VPL
    float4* packed;
    uint8_t* reduced;      // 24 bytes per VPL, or nullptr
};

constexpr int kSplatChunk = 1024;  // points of a bucket per splat work item

struct SplatArgs {
    const float4* points;
    const uint32_t* counts;
    int64_t bucket_stride;
    int64_t n_entries;     // entries in the point buffer (n_buckets * bucket_stride)
    int n_groups;          // buckets of this launch: bucket0 .. bucket0 + n_groups - 1
    int chunks;            // work items per bucket: ceil(bucket_stride / kSplatChunk), at least 1
    int bucket0;           // first bucket of this launch (0 for a whole splat)
    const float4* packed;  // packedVplBuffer
    int n_vpl;
    int vpl_start, vpl_end;
    int scale_isms, points_only_scaled;
    int gx, gy, atlas_w, atlas_h;
    float z_far;
    uint32_t* keys;
};

// ceil(2^32 / d) for 2 <= d < 2^16 (exact floor(n / d) for n < 2^16 by a high multiply), else 0.
inline uint32_t small_div_magic(int d) { return d >= 2 ? (uint32_t)((0x100000000ull + d - 1) / d) : 0u; }

struct PullPushArgs {
    const uint32_t* keys;
    void* out;            // final depth (FP32 or FP16)
    int out_f16;
    int atlas_w, atlas_h;
    int ism_size, levels;
    int grid_x, grid_y;
    float z_far;
    float4* lv1;          // scratch: pyramid level 1, (atlas_w/2) x (atlas_h/2)
    float4* lv2;          // scratch: pyramid level 2, (atlas_w/4) x (atlas_h/4), when levels >= 2
    uint32_t m_c0, m_c1;  // ceil(2^32 / d) for d = ism_size / 2 and ism_size / 4 when d >= 2, else 0
    int row0, row1;       // the launch covers ISM rows [row0, row1) of the grid (0, grid_y: all)
    int pyr_form;         // kPyrByCount, kPyrWhereFits or kPyrPerLevel (see pyramid_launch_fused)
};
constexpr int kPyrByCount = 0, kPyrWhereFits = 1, kPyrPerLevel = 2;

struct FgArgs {
    int width, height;
    const float* depth;
    const void* normal;
    int normal_f16;
    float inv_vp[16];
    const float4* vpl;        // 48-byte records (3 float4), or nullptr when reduced is used
    const uint8_t* reduced;   // 24-byte records, or nullptr
    const void* atlas;
    int atlas_f16;
    int atlas_w, atlas_h;
    int gx, gy, ism_size;
    int n_vpl, per_class;
    int interleave;
    int shadowing;
    int ism_index_offset;
    float z_far;
    float gi_scale;           // giIntensity / vplCount * I^2 (final_gathering.comp:133), folded on the host
    float inv_w, inv_h;       // 1 / width, 1 / height
    float clamp_value;
    int tile;                 // tile edge (threads = tile*tile/2, two pixels each)
    int cull;                 // per-tile culling on/off
    float influence_cutoff;   // 0: off
    float* out;               // width*height*3
    uint32_t* status;         // device error word (bit 0: VPL staging wait timed out)
    long long wait_cycles;    // limit of the VPL staging wait in SM cycles (0: about 2^31)
    uint32_t test_extra_tx;   // test only: bytes the first staging wait expects beyond its copy (0)
    // cull == 2: clustered culling; a pixel keeps the VPLs of its cluster's mask
    const uint32_t* cl_masks;     // (tiles_x * tiles_y * 16) x cl_words
    const uint8_t* cl_slice;      // per pixel
    int cl_tiles_x, cl_words;
    int tile0;                    // tile index of the launch's first block column (tile-row bands)
};

// Tile rows of the gathering (each covers tile * interleave image rows, all interleave classes).
inline int fg_tile_rows(const FgArgs& a) {
    const int T = a.tile == 8 ? 8 : 16, sh = (a.height + a.interleave - 1) / a.interleave;
    return (sh + T - 1) / T;
}
inline int fg_rows_per_tile_row(const FgArgs& a) { return (a.tile == 8 ? 8 : 16) * a.interleave; }

// ---- clustered culling (reference style) ---------------------------------------------------
constexpr int kClusterPixels = 128, kClusterSlices = 16, kClusterSlicesIntoFirst = 3;

struct ClusterArgs {
    int width, height, tiles_x, tiles_y;
    const float* depth;
    float inv_vp[16];
    float proj_a, proj_b;
    float scale;              // (16 + 3) / log2(zFar)
    const float4* packed;     // packed VPL records
    int n_vpl, mask_words;
    uint32_t* used;           // per tile: bit s set when slice s is used
    uint32_t* masks;          // per cluster (tile * 16 + slice): mask_words words
    uint8_t* pixel_slice;     // per pixel
};

cudaError_t launch_cluster_lights(const ClusterArgs& a, cudaStream_t s);

// ---- after the gathering -------------------------------------------------------------------
struct BlurArgs {
    int width, height;
    const float* depth;
    const void* normal;  // octahedral, 2 x f32 or 2 x f16 per pixel
    int normal_f16;
    const void* gi_in;   // RGB floats or R11G11B10F words
    void* gi_out;
    int packed;          // 1: R11G11B10F input, intermediate and output
    float proj_a, proj_b;
};

struct CompositeArgs {
    int width, height;
    const void* gi;
    int gi_packed;
    const uint32_t* albedo;    // RGBA8 UNORM
    const float* occlusion;    // or nullptr
    const float* direct;       // RGB floats, or nullptr
    void* out;
    int out_rgba8;
    float exposure;
};

cudaError_t launch_pack_r11(const float* rgb, uint32_t* words, int64_t n, cudaStream_t s);
cudaError_t launch_unpack_r11(const uint32_t* words, float* rgb, int64_t n, cudaStream_t s);
cudaError_t launch_gi_blur(const BlurArgs& a, cudaStream_t s);
cudaError_t launch_composite(const CompositeArgs& a, cudaStream_t s);

// ---- batched frames: one persistent launch per pass over a device-resident view table -------
struct BatchView {
    VplArgs vpl;
    SplatArgs splat;
    PullPushArgs pp;
    FgArgs fg;
    uint32_t* keys;
    size_t atlas_texels;
    int fg_tiles_per_class;
    int fg_mode;  // 0: FP32 records/atlas/normals, 1: reduced (24-byte records, FP16 atlas and normals)
};

enum BatchPass { kBpClear = 0, kBpVpl, kBpSplat, kBpPull1, kBpPullMid, kBpPush1, kBpPush0, kBpFg, kBpFg16, kBpCount };

struct BatchTable {
    const BatchView* views;  // device
    const int* prefix;       // device, kBpCount x (n_views + 1) running work-item counts
    int n_views;
};

constexpr int kBatchClearTexels = 4096;  // atlas texels cleared per work item
constexpr int kBatchVplPerItem = 256;

cudaError_t launch_batch_ism(const BatchTable& t, int pass, int grid, size_t smem, cudaStream_t s);
cudaError_t launch_batch_fg(const BatchTable& t, int pass, int grid, cudaStream_t s);  // pass kBpFg or kBpFg16
int batch_blocks_per_sm(int pass, size_t smem);

// Error bits written to the device status word.
constexpr uint32_t kStatusTmaTimeout = 1u;

cudaError_t launch_vpl_process(const VplArgs& a, cudaStream_t s);
cudaError_t launch_ism_clear(uint32_t* keys, size_t n, cudaStream_t s);
// launch_vpl_process and launch_ism_clear in one launch (separate launches when the atlas is not
// a whole number of aligned 16-byte rows).
cudaError_t launch_vpl_clear(const VplArgs& va, uint32_t* keys, size_t n, cudaStream_t s);
cudaError_t launch_ism_splat(const SplatArgs& a, cudaStream_t s);
// The atomics launch_ism_splat would issue (projections that land inside the atlas), added to *count.
cudaError_t launch_ism_splat_count(const SplatArgs& a, unsigned long long* count, cudaStream_t s);
// The pyramid of ISM rows [a.row0, a.row1). marks (optional): three events recorded after level
// 1, the middle levels and push level 1.
cudaError_t launch_pullpush(const PullPushArgs& a, cudaStream_t s, cudaEvent_t* marks = nullptr);
// Raise the middle pass's dynamic shared-memory limit to `smem` outside any stream capture; then
// launch_pullpush_captured issues the same launches as launch_pullpush without that attribute call.
cudaError_t pullpush_prepare(size_t smem);
cudaError_t launch_pullpush_captured(const PullPushArgs& a, cudaStream_t s);
// Shared memory of the per-ISM middle pass (levels 2..L), and the lv1 + lv2 scratch in bytes
// (lv2 starts at *lv2_offset).
size_t pullmid_smem_bytes(int ism_size, int levels);
// Whether launch_pullpush runs an ISM's whole pyramid in one block (pyramid_kernel, no scratch;
// ISM edges up to 128, far plane in [2^-20, 2^20]) rather than in four launches over the lv1/lv2
// scratch; its shared memory per block.
bool pyramid_fits(int ism_size, int levels, float z_far);
bool pyramid_fused(int ism_size, int levels, float z_far, long long n_isms);
bool pyramid_launch_fused(const PullPushArgs& a);
size_t pyramid_smem_bytes(int ism_size, int levels);
size_t pullpush_scratch_bytes(int atlas_w, int atlas_h, int levels, size_t* lv2_offset);
int pullpush_batch_items(int pass, int atlas_w, int atlas_h, int ism_count, int levels);
// Tile rows [tile_row0, tile_row1) of the gathering (tile_row1 < 0: through the last).
cudaError_t launch_final_gather(const FgArgs& a, cudaStream_t s, int tile_row0 = 0, int tile_row1 = -1);

}  // namespace mlgi
