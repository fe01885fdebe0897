// Flat description of one seeded room (objects, sampling table, camera and light matrices),
// built on the host by build_room() and passed by value as a kernel parameter to the device-side
// ray caster and point sampler (csrc/scene_kernels.cu). Plain data: no CUDA types.
#pragma once

#include <cstdint>

#include "mlgi.h"

namespace mlgi {

constexpr int kRoomMaxBoxes = 32;
constexpr int kRoomMaxSpheres = 16;
constexpr int kRoomMaxPatches = 5 + 6 * kRoomMaxBoxes + kRoomMaxSpheres;

struct RoomGPU {
    float wall_albedo[5][3];  // floor, ceiling, back, left, right
    int n_boxes, n_spheres, n_patches, pad0;
    float box_lo[kRoomMaxBoxes][3], box_hi[kRoomMaxBoxes][3], box_albedo[kRoomMaxBoxes][3];
    float sph_c[kRoomMaxSpheres][3], sph_r[kRoomMaxSpheres], sph_albedo[kRoomMaxSpheres][3];
    // area-uniform sampling table: rectangle (o, a, b, n) or sphere (o = centre, r)
    float patch_o[kRoomMaxPatches][3], patch_a[kRoomMaxPatches][3], patch_b[kRoomMaxPatches][3];
    float patch_n[kRoomMaxPatches][3], patch_r[kRoomMaxPatches];
    int patch_kind[kRoomMaxPatches];
    float cdf[kRoomMaxPatches];  // running area
    float vp[16], inv_vp[16];    // camera, column-major
    float lvp[16], inv_lvp[16];  // light
    float light_dir[3], cos_cone;
    float total_area, r_boost;
    uint64_t point_seed;
};

// Host: the room of `d` (same objects and matrices as mlgi_scene_generate) in device layout.
mlgi_status build_room(const mlgi_scene_desc& d, RoomGPU* room, mlgi_scene_info* info);

}  // namespace mlgi
