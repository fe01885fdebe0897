"""ctypes wrapper of oracle/_ref/libref.so: the reference's own compute shaders compiled as C++
(see oracle/build_ref.py) -- TEST INFRASTRUCTURE ONLY, used to pin the oracle restatement and as
the CPU implementation timed by bench.py's reference arm."""
from __future__ import annotations

import ctypes as C
import importlib.util
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_lib = None


def available() -> bool:
    try:
        lib()
        return True
    except Exception:
        return False


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        spec = importlib.util.spec_from_file_location("oracle_build_ref", os.path.join(HERE, "build_ref.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        path = mod.build_if_reference_present()
        if not path:
            raise RuntimeError("oracle/_ref is not buildable here (no reference shaders, no generated sources)")
        _lib = C.CDLL(path)
    return _lib


def _p(a):
    return C.c_void_p(0 if a is None else a.ctypes.data)


def vpl_process(rsm_depth, rsm_normal, rsm_diffuse, n, inv_bpv, intensity, shuffle, perm, threads=0):
    """vpl_processor.comp (N must be 1024). Returns (pos, normal, color [N,3]) and packed [N,4]."""
    h, w = rsm_depth.shape
    vpl = np.zeros((n, 9), np.float32)
    packed = np.zeros((n, 4), np.float32)
    lib().ref_vpl_process(w, h, _p(np.ascontiguousarray(rsm_depth, np.float32)),
                          _p(np.ascontiguousarray(rsm_normal, np.uint32)), _p(np.ascontiguousarray(rsm_diffuse, np.uint32)),
                          n, _p(np.ascontiguousarray(inv_bpv, np.float32).reshape(16)), C.c_float(intensity),
                          int(shuffle), _p(np.ascontiguousarray(perm, np.int32)), _p(vpl), _p(packed), threads)
    return vpl[:, 0:3].copy(), vpl[:, 3:6].copy(), vpl[:, 6:9].copy(), packed


def ism_splat(points, counts, packed_vpls, n_vpl, atlas_w, atlas_h, z_far, vpl_start=0, vpl_end=None, scale_isms=0,
              points_only=0, threads=0):
    """ism.comp after the atlas clear (ImperfectShadowmap::render). Returns uint32 keys (H, W)."""
    vpl_end = n_vpl if vpl_end is None else vpl_end
    keys = np.zeros((atlas_h, atlas_w), np.uint32)
    pts = np.ascontiguousarray(points, np.float32)
    lib().ref_ism_splat(_p(pts), C.c_int64(pts.shape[0]), _p(np.ascontiguousarray(counts, np.uint32)), len(counts),
                        _p(np.ascontiguousarray(packed_vpls, np.float32)), n_vpl, vpl_start, vpl_end, scale_isms,
                        points_only, atlas_w, atlas_h, C.c_float(z_far), _p(keys), threads)
    return keys


def pullpush(keys, ism_pixel_size, levels, z_far, threads=0):
    h, w = keys.shape
    out = np.zeros((h, w), np.float32)
    lib().ref_pullpush(_p(np.ascontiguousarray(keys, np.uint32)), w, h, ism_pixel_size, levels, C.c_float(z_far),
                       _p(out), threads)
    return out


def final_gather(depth, normal_rgb, inv_vp, proj, vpl9, n_vpl, vpl_start, vpl_end, atlas, z_far, z_near, gi, clampv,
                 per_class, threads=0):
    h, w = depth.shape
    out = np.zeros((h, w, 3), np.float32)
    ah, aw = atlas.shape
    lib().ref_final_gather(w, h, _p(np.ascontiguousarray(depth, np.float32)),
                           _p(np.ascontiguousarray(normal_rgb, np.float32)),
                           _p(np.ascontiguousarray(inv_vp, np.float32).reshape(16)),
                           _p(np.ascontiguousarray(proj, np.float32).reshape(16)),
                           _p(np.ascontiguousarray(vpl9, np.float32)), n_vpl, vpl_start, vpl_end,
                           _p(np.ascontiguousarray(atlas, np.float32)), aw, ah, C.c_float(z_far), C.c_float(z_near),
                           C.c_float(gi), C.c_float(clampv), per_class, _p(out), threads)
    return out


def cluster_lights(depth, inv_vp, proj_a, proj_b, z_far, packed_vpls):
    """clustering.comp + light_lists.comp as ClusteredShading::process drives them (1024 VPLs).
    Returns, per used cluster in the atomic counter's order, (x, y, slice) and its 1024-entry
    light-list column (entry 64 s: sub-list s's count + 1; its VPL ids follow)."""
    h, w = depth.shape
    nclusters = ((w + 127) // 128) * ((h + 127) // 128) * 16
    n_used = C.c_int(0)
    words = np.zeros(nclusters, np.uint32)
    lists = np.zeros((nclusters, 1024), np.uint32)
    pk = np.ascontiguousarray(packed_vpls, np.float32)
    lib().ref_cluster_lights(w, h, _p(np.ascontiguousarray(depth, np.float32)),
                             _p(np.ascontiguousarray(inv_vp, np.float32).reshape(16)), C.c_float(proj_a),
                             C.c_float(proj_b), C.c_float(z_far), _p(pk), pk.shape[0], C.byref(n_used), _p(words),
                             _p(lists))
    n = n_used.value
    xyz = [(int(wd & 0xFF), int((wd >> 8) & 0xFF), int((wd >> 16) & 0xFF)) for wd in words[:n]]
    return xyz, lists[:n]


def gi_blur(depth, normal_rgb, gi, proj_a, proj_b, threads=0):
    """gi_blur.frag's X program then its Y program (GIStage::blur) on float RGB buffers; normal_rgb
    is n*0.5+0.5. Returns [H, W, 3] float32."""
    h, w = depth.shape
    out = np.zeros((h, w, 3), np.float32)
    lib().ref_gi_blur(w, h, _p(np.ascontiguousarray(depth, np.float32)),
                      _p(np.ascontiguousarray(normal_rgb, np.float32)), _p(np.ascontiguousarray(gi, np.float32)),
                      C.c_float(proj_a), C.c_float(proj_b), _p(out), threads)
    return out
