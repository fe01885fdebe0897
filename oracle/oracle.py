"""ctypes wrapper of the CPU oracle (oracle/oracle.cpp) -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this module, as the
checker or the timed CPU baseline; the product never imports it. Inputs are numpy arrays.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            import importlib.util
            spec = importlib.util.spec_from_file_location("oracle_build", os.path.join(HERE, "build.py"))
            mod = importlib.util.module_from_spec(spec)
            spec.loader.exec_module(mod)
            mod.build()
        _lib = C.CDLL(LIB_PATH)
        _lib.oracle_max_threads.restype = C.c_int
        _lib.oracle_ism_splat_count_f32.restype = C.c_int64
    return _lib


class _Arg:
    """A pointer argument that holds its array: ctypes passes `_as_parameter_`, and the array lives
    as long as the call's argument list, also when it is a temporary conversion."""

    def __init__(self, a):
        self.a = a
        self._as_parameter_ = C.c_void_p(0 if a is None else a.ctypes.data)


def _p(a):
    return _Arg(a)


def _f(t):
    return C.c_float if t == np.float32 else C.c_double


def max_threads() -> int:
    return lib().oracle_max_threads()


def vpl_process(rsm_depth, rsm_normal, rsm_diffuse, n, inv_bpv, intensity, shuffle, perm, dtype=np.float32):
    """vpl_processor.comp:41-72. Returns (pos[N,3], normal[N,3], color[N,3], packed_normal[N] uint32)."""
    h, w = rsm_depth.shape
    pos = np.zeros((n, 3), dtype)
    nrm = np.zeros((n, 3), dtype)
    col = np.zeros((n, 3), dtype)
    pn = np.zeros(n, np.uint32)
    m = np.ascontiguousarray(np.asarray(inv_bpv, dtype).reshape(16))
    perm = np.ascontiguousarray(perm, np.int32) if perm is not None else np.arange(n, dtype=np.int32)
    fn = lib().oracle_vpl_process_f32 if dtype == np.float32 else lib().oracle_vpl_process_f64
    fn(w, h, _p(np.ascontiguousarray(rsm_depth, np.float32)), _p(np.ascontiguousarray(rsm_normal, np.uint32)),
       _p(np.ascontiguousarray(rsm_diffuse, np.uint32)), n, _p(m), _f(dtype)(intensity), int(shuffle), _p(perm),
       _p(pos), _p(nrm), _p(col), _p(pn))
    return pos, nrm, col, pn


def ism_splat(points, counts, bucket_stride, vpl_pos, vpl_pn, n_vpl, ism_size, grid_x, grid_y, z_far,
              vpl_start=0, vpl_end=None, scale_isms=0, points_only=0, threads=0, dtype=np.float32, count=False):
    """ism.comp:54-139 after the atlas clear of ImperfectShadowmap.cpp:212. Returns uint32 keys (H, W);
    with count=True (FP32 only) also the number of atomicMin calls that land inside the atlas."""
    vpl_end = n_vpl if vpl_end is None else vpl_end
    aw, ah = grid_x * ism_size, grid_y * ism_size
    atlas = np.full((ah, aw), 0xFFFFFFFF, np.uint32)
    n_groups = (vpl_end - vpl_start) if points_only else n_vpl
    if count:
        assert dtype == np.float32
        fn = lib().oracle_ism_splat_count_f32
    else:
        fn = lib().oracle_ism_splat_f32 if dtype == np.float32 else lib().oracle_ism_splat_f64
    points = np.ascontiguousarray(points, np.float32)
    # imageSize(pointBuffer): entries past it read as zero (a bucket's counter may run past its stride)
    n_entries = points.size // 4
    issued = fn(_p(points), _p(np.ascontiguousarray(counts, np.uint32)), n_groups,
                C.c_int64(bucket_stride), C.c_int64(n_entries), _p(np.ascontiguousarray(vpl_pos, dtype)),
                _p(np.ascontiguousarray(vpl_pn, np.uint32)), n_vpl, vpl_start, vpl_end, scale_isms, points_only,
                grid_x, grid_y, aw, ah, _f(dtype)(z_far), _p(atlas), threads)
    return (atlas, int(issued)) if count else atlas


def pullpush(keys, ism_size, levels, z_far, threads=0, dtype=np.float32):
    """ImperfectShadowmap::pullpush (pull.comp + push.comp level by level). Returns the final depth."""
    h, w = keys.shape
    out = np.zeros((h, w), dtype)
    fn = lib().oracle_pullpush_f32 if dtype == np.float32 else lib().oracle_pullpush_f64
    fn(_p(np.ascontiguousarray(keys, np.uint32)), w, h, ism_size, levels, _f(dtype)(z_far), _p(out), threads)
    return out


def pull_level(level, keys, inp, out_w, out_h, z_far, ism_pixel_size):
    """One pull.comp pass; texel planes are uint32 (h, w, 4): r, g, b float bits and half2 bits."""
    out = np.zeros((out_h, out_w, 4), np.uint32)
    in_w = keys.shape[1] if level == 1 else inp.shape[1]
    lib().oracle_pull_level_f32(level, _p(np.ascontiguousarray(keys, np.uint32) if keys is not None else None),
                                _p(np.ascontiguousarray(inp, np.uint32) if inp is not None else None), in_w, _p(out),
                                out_w, out_h, C.c_float(z_far), ism_pixel_size)
    return out


def push_level(level, keys, same, coarse, out_w, out_h, ism_size):
    """One push.comp pass. Returns (texel plane, final depth plane); level 0 writes only the latter."""
    out = np.zeros((out_h, out_w, 4), np.uint32)
    fin = np.zeros((out_h, out_w), np.float32)
    ch, cw = coarse.shape[:2]
    lib().oracle_push_level_f32(level, _p(np.ascontiguousarray(keys, np.uint32) if keys is not None else None),
                                _p(np.ascontiguousarray(same, np.uint32) if same is not None else None),
                                _p(np.ascontiguousarray(coarse, np.uint32)), cw, ch, _p(out), _p(fin), out_w, out_h,
                                ism_size)
    return out, fin


def final_gather(depth, normal_oct, inv_vp, vpl_pos, vpl_nrm, vpl_col, atlas, ism_size, grid_x, grid_y, z_far,
                 gi_intensity, clamp_value, interleave, shadowing=1, tile=0, cutoff=0.0, vpl_count=None,
                 ism_offset=0, threads=0, dtype=np.float32, accurate_world=False):
    """final_gathering.comp:63-135 (class slices; optional per-tile culling). Returns (H, W, 3).

    accurate_world (FP32 only): world positions exactly rounded instead of evaluated in FP32."""
    h, w = depth.shape
    n = vpl_pos.shape[0]
    vpl_count = n if vpl_count is None else vpl_count
    out = np.zeros((h, w, 3), dtype)
    ah, aw = atlas.shape
    m = np.ascontiguousarray(np.asarray(inv_vp, dtype).reshape(16))
    fn = lib().oracle_final_gather_f32 if dtype == np.float32 else lib().oracle_final_gather_f64
    if accurate_world and dtype == np.float32:
        fn = lib().oracle_final_gather_f32_accurate_world
    d, nm = np.ascontiguousarray(depth, np.float32), np.ascontiguousarray(normal_oct, np.float32)
    vp, vn = np.ascontiguousarray(vpl_pos, dtype), np.ascontiguousarray(vpl_nrm, dtype)
    vc, at = np.ascontiguousarray(vpl_col, dtype), np.ascontiguousarray(atlas, np.float32)
    fn(w, h, _p(d), _p(nm), _p(m), n, vpl_count, ism_offset, _p(vp), _p(vn), _p(vc), _p(at), aw, ah, grid_x, grid_y,
       _f(dtype)(z_far), _f(dtype)(gi_intensity), _f(dtype)(clamp_value), interleave, shadowing, tile,
       C.c_double(cutoff), _p(out), threads)
    return out


def pack3sn(x, y, z) -> int:
    lib().oracle_pack3sn_f32.restype = C.c_uint32
    return lib().oracle_pack3sn_f32(C.c_float(x), C.c_float(y), C.c_float(z))


def unpack3sn(u: int) -> np.ndarray:
    out = np.zeros(3, np.float32)
    lib().oracle_unpack3sn_f32(C.c_uint32(u), _p(out))
    return out


def pack_half2x16(a, b) -> int:
    lib().oracle_pack_half2x16.restype = C.c_uint32
    return lib().oracle_pack_half2x16(C.c_float(a), C.c_float(b))


def paraboloid_project(rel, dist, n, z_far, ism_index, gx, gy, preserve_sign):
    out = np.zeros(3, np.float32)
    lib().oracle_paraboloid_project_f32(_p(np.asarray(rel, np.float32)), C.c_float(dist), _p(np.asarray(n, np.float32)),
                                        C.c_float(z_far), C.c_float(ism_index), gx, gy, int(preserve_sign), _p(out))
    return out


def pack_r11g11b10f(rgb) -> np.ndarray:
    """GL_R11F_G11F_B10F words of RGB triples (rgb: [..., 3] float32)."""
    a = np.ascontiguousarray(rgb, np.float32).reshape(-1, 3)
    out = np.zeros(len(a), np.uint32)
    lib().oracle_pack_r11g11b10f(_p(a), _p(out), C.c_int64(len(a)))
    return out


def unpack_r11g11b10f(words) -> np.ndarray:
    w = np.ascontiguousarray(words, np.uint32).reshape(-1)
    out = np.zeros((len(w), 3), np.float32)
    lib().oracle_unpack_r11g11b10f(_p(w), _p(out), C.c_int64(len(w)))
    return out


def gi_blur(depth, normal_oct, gi, proj_a, proj_b, packed=False, threads=0):
    """gi_blur.frag's X then Y pass (GIStage.cpp:308-344). gi: [H, W, 3] float32, or [H, W] uint32
    R11G11B10F words with packed=True; returns the same layout."""
    depth = np.ascontiguousarray(depth, np.float32)
    h, w = depth.shape
    n = np.ascontiguousarray(normal_oct, np.float32)
    g = np.ascontiguousarray(gi, np.uint32 if packed else np.float32)
    out = np.zeros_like(g)
    lib().oracle_gi_blur(w, h, _p(depth), _p(n), _p(g), int(packed), C.c_float(proj_a), C.c_float(proj_b), _p(out),
                         threads)
    return out


def gi_blur_rgb_normals(depth, normal_rgb, gi, proj_a, proj_b, threads=0):
    """gi_blur with the normals given as n*0.5+0.5 RGB [H, W, 3] (the reference G-buffer's format,
    decoded rgb * 2 - 1 as gi_blur.frag does); FP32 RGB in and out."""
    depth = np.ascontiguousarray(depth, np.float32)
    h, w = depth.shape
    g = np.ascontiguousarray(gi, np.float32)
    out = np.zeros_like(g)
    lib().oracle_gi_blur_rgb_normals(w, h, _p(depth), _p(np.ascontiguousarray(normal_rgb, np.float32)), _p(g),
                                     C.c_float(proj_a), C.c_float(proj_b), _p(out), threads)
    return out


def composite(gi, albedo, exposure, occlusion=None, direct=None, packed=False):
    """deferredshading.frag's GI ambient term, Reinhard and toSRGB. Returns (rgb float32 [H, W, 3],
    rgba8 uint32 [H, W])."""
    albedo = np.ascontiguousarray(albedo, np.uint32)
    h, w = albedo.shape
    g = np.ascontiguousarray(gi, np.uint32 if packed else np.float32)
    occ = None if occlusion is None else np.ascontiguousarray(occlusion, np.float32)
    d = None if direct is None else np.ascontiguousarray(direct, np.float32)
    rgb = np.zeros((h, w, 3), np.float32)
    words = np.zeros((h, w), np.uint32)
    lib().oracle_composite(w, h, _p(g), int(packed), _p(albedo), _p(occ), _p(d), C.c_float(exposure), _p(rgb),
                           _p(words))
    return rgb, words


def cluster_lights(depth, inv_vp, proj_a, proj_b, z_far, vpl_pos, vpl_pn, n_vpl):
    """clustering.comp + light_lists.comp: (used [tiles] uint32, masks [tiles*16, words] uint32,
    pixel_slice [H, W] uint8)."""
    depth = np.ascontiguousarray(depth, np.float32)
    h, w = depth.shape
    tiles = ((w + 127) // 128) * ((h + 127) // 128)
    words = (n_vpl + 31) // 32
    used = np.zeros(tiles, np.uint32)
    masks = np.zeros((tiles * 16, words), np.uint32)
    sl = np.zeros((h, w), np.uint8)
    m = np.ascontiguousarray(np.asarray(inv_vp, np.float32).reshape(16))
    vp = np.ascontiguousarray(vpl_pos, np.float32)
    vn = np.ascontiguousarray(vpl_pn, np.uint32)
    lib().oracle_cluster_lights(w, h, _p(depth), _p(m), C.c_float(proj_a), C.c_float(proj_b), C.c_float(z_far),
                                _p(vp), _p(vn), n_vpl, _p(used), _p(masks), _p(sl))
    return used, masks, sl


def final_gather_clustered(depth, normal_oct, inv_vp, vpl_pos, vpl_nrm, vpl_col, atlas, ism_size, grid_x, grid_y,
                           z_far, gi_intensity, clamp_value, interleave, masks, pixel_slice, shadowing=True,
                           threads=0):
    """final_gathering.comp in FP64 with each pixel restricted to its cluster's VPL mask."""
    h, w = depth.shape
    n = len(vpl_pos)
    out = np.zeros((h, w, 3), np.float64)
    # every converted array is bound to a name, so that it outlives the call
    keep = [np.ascontiguousarray(depth, np.float32), np.ascontiguousarray(normal_oct, np.float32),
            np.ascontiguousarray(np.asarray(inv_vp, np.float64).reshape(16)), np.ascontiguousarray(vpl_pos, np.float64),
            np.ascontiguousarray(vpl_nrm, np.float64), np.ascontiguousarray(vpl_col, np.float64),
            np.ascontiguousarray(atlas, np.float32), np.ascontiguousarray(masks, np.uint32),
            np.ascontiguousarray(pixel_slice, np.uint8)]
    d, nm, m, vp, vn, vc, at, mk, sl = keep
    lib().oracle_final_gather_f64_clustered(
        w, h, _p(d), _p(nm), _p(m), n, n, 0, _p(vp), _p(vn), _p(vc), _p(at), at.shape[1], at.shape[0], grid_x, grid_y,
        C.c_double(z_far), C.c_double(gi_intensity), C.c_double(clamp_value), interleave, int(shadowing), _p(mk), _p(sl),
        _p(out), threads)
    return out
