"""ctypes binding of libmlgi.so (include/mlgi.h) plus the workload configurations.

This module is a thin caller of the C ABI: every device computation goes through the CUDA
kernels in libmlgi.so. Loading fails loudly when the library has not been built; there is no
fallback implementation. With MLGI_CHECKED=1 in the environment it loads the bounds-checked
variant, libmlgi_checked.so, instead.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(_HERE)
LIB_PATH_NORMAL = os.path.join(PKG, "_build", "libmlgi.so")
LIB_PATH_CHECKED = os.path.join(PKG, "_build_checked", "libmlgi_checked.so")
LIB_PATH = LIB_PATH_CHECKED if os.environ.get("MLGI_CHECKED") == "1" else LIB_PATH_NORMAL

OK, EINVAL, ENOMEM, ETIMEDOUT, ECUDA, ECANCELED, EBOUNDS = 0, 1, 2, 3, 4, 5, 6
F32, F16, BF16, R11G11B10F, RGBA8 = 0, 1, 2, 3, 4

_p = C.c_void_p
_f16 = C.c_float * 16


class RsmView(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("depth", _p), ("normal", _p), ("diffuse", _p)]


class VplParams(C.Structure):
    _fields_ = [("count", C.c_int), ("light_intensity", C.c_float), ("shuffle", C.c_int),
                ("inv_biased_light_vp", _f16)]


class VplBuf(C.Structure):
    _fields_ = [("capacity", C.c_int), ("vpl", _p), ("packed", _p), ("reduced", _p)]


class Points(C.Structure):
    _fields_ = [("points", _p), ("counts", _p), ("n_buckets", C.c_int), ("bucket_stride", C.c_int64)]


class IsmParams(C.Structure):
    _fields_ = [("vpl_start", C.c_int), ("vpl_end", C.c_int), ("scale_isms", C.c_int),
                ("points_only_scaled", C.c_int), ("ism_size", C.c_int), ("grid_x", C.c_int),
                ("grid_y", C.c_int), ("levels", C.c_int), ("z_far", C.c_float)]


class Atlas(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("keys", _p), ("depth", _p), ("format", C.c_int)]


class GBufferView(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("depth", _p), ("normal", _p), ("normal_format", C.c_int)]


class FgParams(C.Structure):
    _fields_ = [("inv_view_proj", _f16), ("z_far", C.c_float), ("gi_intensity", C.c_float),
                ("clamp_value", C.c_float), ("vpl_count", C.c_int), ("vpl_start", C.c_int), ("vpl_end", C.c_int),
                ("scale_isms", C.c_int), ("ism_size", C.c_int), ("grid_x", C.c_int), ("grid_y", C.c_int),
                ("interleave", C.c_int), ("shadowing", C.c_int), ("tile", C.c_int), ("cull", C.c_int),
                ("influence_cutoff", C.c_float), ("vpl_format", C.c_int), ("proj_a", C.c_float),
                ("proj_b", C.c_float), ("camera_z_far", C.c_float)]


class Radiance(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("rgb", _p)]


class FrameDesc(C.Structure):
    _fields_ = [("rsm", RsmView), ("vpl", VplParams), ("points", Points), ("ism", IsmParams),
                ("atlas_format", C.c_int), ("gbuffer", GBufferView), ("fg", FgParams)]


class FrameHostSizes(C.Structure):
    _fields_ = [(n, C.c_size_t) for n in ("rsm_depth", "rsm_normal", "rsm_diffuse", "points", "counts",
                                           "gbuf_depth", "gbuf_normal", "radiance")]


class AutotuneQuery(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("n_vpl", C.c_int), ("n_points", C.c_int64),
                ("reduced", C.c_int), ("rsm_size", C.c_int), ("min_vpls_per_pixel", C.c_int),
                ("min_ism_size", C.c_int), ("batched", C.c_int), ("budget_ms", C.c_float), ("seed", C.c_uint64)]


class AutotuneResult(C.Structure):
    _fields_ = [("interleave", C.c_int), ("ism_size", C.c_int), ("grid_x", C.c_int), ("grid_y", C.c_int),
                ("levels", C.c_int), ("tile", C.c_int), ("ms", C.c_float), ("candidates_timed", C.c_int)]


class CtxDesc(C.Structure):
    _fields_ = [("device", C.c_int), ("flags", C.c_uint32)]


class SceneDesc(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("n_boxes", C.c_int), ("n_spheres", C.c_int), ("width", C.c_int),
                ("height", C.c_int), ("rsm_width", C.c_int), ("rsm_height", C.c_int), ("n_points", C.c_int64),
                ("n_buckets", C.c_int), ("ism_count", C.c_int), ("light_yaw_deg", C.c_float),
                ("light_pitch_deg", C.c_float), ("camera_orbit_deg", C.c_float), ("z_near", C.c_float),
                ("z_far", C.c_float)]


class SceneInfo(C.Structure):
    _fields_ = [("view", _f16), ("proj", _f16), ("inv_view_proj", _f16), ("light_view", _f16),
                ("light_proj", _f16), ("inv_biased_light_vp", _f16), ("eye", C.c_float * 3),
                ("light_pos", C.c_float * 3), ("light_dir", C.c_float * 3), ("z_near", C.c_float),
                ("z_far", C.c_float), ("total_area", C.c_float), ("point_radius", C.c_float),
                ("bucket_stride", C.c_int64)]


class ClusterParams(C.Structure):
    _fields_ = [("inv_view_proj", _f16), ("proj_a", C.c_float), ("proj_b", C.c_float), ("z_far", C.c_float)]


class BlurParams(C.Structure):
    _fields_ = [("proj_a", C.c_float), ("proj_b", C.c_float), ("format", C.c_int)]


class CompositeParams(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("exposure", C.c_float), ("gi_format", C.c_int),
                ("out_format", C.c_int)]


BATCH_PERSISTENT, BATCH_CONCURRENT = 0, 1


class BatchOpts(C.Structure):
    _fields_ = [("form", C.c_int), ("streams", C.c_int)]


class ServerDesc(C.Structure):
    _fields_ = [("device", C.c_int), ("slots", C.c_int), ("max_width", C.c_int), ("max_height", C.c_int),
                ("rsm_size", C.c_int), ("hbm_budget", C.c_size_t)]


class Request(C.Structure):
    _fields_ = [("id", C.c_uint64), ("room_seed", C.c_uint64), ("width", C.c_int), ("height", C.c_int),
                ("n_vpl", C.c_int), ("n_points", C.c_int64), ("reduced", C.c_int), ("light_yaw_deg", C.c_float),
                ("light_pitch_deg", C.c_float), ("camera_orbit_deg", C.c_float), ("arrival_s", C.c_double),
                ("out_host", _p)]


class Completion(C.Structure):
    _fields_ = [("id", C.c_uint64), ("status", C.c_int32), ("latency_ms", C.c_double), ("queue_ms", C.c_double),
                ("digest", C.c_uint64), ("sum", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [("queued", C.c_int64), ("inflight", C.c_int64), ("admitted", C.c_int64),
                ("rooms_resident", C.c_int64), ("budget_waits", C.c_int64), ("evictions", C.c_int64),
                ("room_bytes", C.c_size_t),
                ("slot_bytes", C.c_size_t)]


class PoissonDesc(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("rate_hz", C.c_double), ("duration_s", C.c_double), ("shapes", _p),
                ("n_shapes", C.c_int), ("n_rooms", C.c_int), ("room_seed_base", C.c_uint64),
                ("light_jitter_deg", C.c_float), ("orbit_step_deg", C.c_float), ("drain_timeout_s", C.c_double),
                ("mode", C.c_int)]


# Every entry point of include/mlgi.h with its ctypes signature.
_SIGS = {
    "mlgi_create": (C.c_int32, [C.POINTER(C.c_void_p), C.POINTER(CtxDesc)]),
    "mlgi_destroy": (None, [_p]),
    "mlgi_last_error": (C.c_char_p, [_p]),
    "mlgi_status_string": (C.c_char_p, [C.c_int32]),
    "mlgi_ctx_stream": (_p, [_p]),
    "mlgi_vpl_process": (C.c_int32, [_p, C.POINTER(RsmView), C.POINTER(VplParams), C.POINTER(VplBuf), _p]),
    "mlgi_shuffle_table": (C.c_int32, [C.c_int, _p]),
    "mlgi_ism_splat": (C.c_int32, [_p, C.POINTER(Points), C.POINTER(VplBuf), C.c_int, C.POINTER(IsmParams),
                                   C.POINTER(Atlas), _p]),
    "mlgi_pullpush": (C.c_int32, [_p, C.POINTER(Atlas), C.POINTER(IsmParams), _p]),
    "mlgi_ism_clear": (C.c_int32, [_p, C.POINTER(Atlas), _p]),
    "mlgi_ism_splat_count": (C.c_int32, [_p, C.POINTER(Points), C.POINTER(VplBuf), C.c_int, C.POINTER(IsmParams),
                                         C.POINTER(Atlas), C.POINTER(C.c_uint64)]),
    "mlgi_ism_splat_range": (C.c_int32, [_p, C.POINTER(Points), C.POINTER(VplBuf), C.c_int, C.POINTER(IsmParams),
                                         C.POINTER(Atlas), C.c_int, C.c_int, _p]),
    "mlgi_pullpush_rows": (C.c_int32, [_p, C.POINTER(Atlas), C.POINTER(IsmParams), C.c_int, C.c_int, _p]),
    "mlgi_pullpush_launches": (C.c_int, [C.POINTER(IsmParams)]),
    "mlgi_ism_render_static": (C.c_int32, [C.POINTER(Points), C.POINTER(VplBuf), C.c_int, C.POINTER(IsmParams), _p,
                                           C.c_int, _p]),
    "mlgi_final_gather": (C.c_int32, [_p, C.POINTER(GBufferView), C.POINTER(VplBuf), C.POINTER(Atlas),
                                      C.POINTER(FgParams), C.POINTER(Radiance), _p]),
    "mlgi_gi_frame": (C.c_int32, [_p, C.POINTER(FrameDesc), C.POINTER(Radiance), _p]),
    "mlgi_batch_create": (C.c_int32, [_p, C.c_int, _p, _p, C.POINTER(C.c_void_p)]),
    "mlgi_batch_update_view": (C.c_int32, [_p, C.c_int, C.POINTER(FrameDesc), C.POINTER(Radiance)]),
    "mlgi_batch_launch": (C.c_int32, [_p, _p]),
    "mlgi_batch_destroy": (None, [_p]),
    "mlgi_batch_create_ex": (C.c_int32, [_p, C.c_int, _p, _p, C.POINTER(BatchOpts), C.POINTER(C.c_void_p)]),
    "mlgi_batch_kernel_launches": (C.c_int, [_p]),
    "mlgi_autotune": (C.c_int32, [_p, C.POINTER(AutotuneQuery), C.POINTER(AutotuneResult)]),
    "mlgi_ctx_reserve": (C.c_int32, [_p, C.c_int, C.c_size_t]),
    "mlgi_server_create": (C.c_int32, [C.POINTER(ServerDesc), C.POINTER(C.c_void_p)]),
    "mlgi_server_prepare": (C.c_int32, [_p, _p, C.c_int]),
    "mlgi_server_submit": (C.c_int32, [_p, C.POINTER(Request)]),
    "mlgi_server_cancel": (C.c_int32, [_p, C.c_uint64]),
    "mlgi_server_poll": (C.c_int, [_p, _p, C.c_int]),
    "mlgi_server_drain": (C.c_int32, [_p, C.c_double]),
    "mlgi_server_stats_get": (C.c_int32, [_p, C.POINTER(ServerStats)]),
    "mlgi_server_destroy": (None, [_p]),
    "mlgi_server_run_poisson": (C.c_int32, [_p, C.POINTER(PoissonDesc), _p, C.c_int, C.POINTER(C.c_int),
                                            C.POINTER(C.c_double)]),
    "mlgi_frame_host_sizes_get": (C.c_int32, [C.POINTER(FrameDesc), C.POINTER(FrameHostSizes)]),
    "mlgi_gi_frame_host": (C.c_int32, [_p, C.POINTER(FrameDesc), _p]),
    "mlgi_cluster_lights": (C.c_int32, [_p, C.POINTER(GBufferView), C.POINTER(VplBuf), C.c_int,
                                        C.POINTER(ClusterParams), _p, _p, _p, _p]),
    "mlgi_pack_r11g11b10f": (C.c_int32, [_p, _p, _p, C.c_int64, _p]),
    "mlgi_unpack_r11g11b10f": (C.c_int32, [_p, _p, _p, C.c_int64, _p]),
    "mlgi_gi_blur": (C.c_int32, [_p, C.POINTER(GBufferView), _p, _p, C.POINTER(BlurParams), _p]),
    "mlgi_composite": (C.c_int32, [_p, _p, _p, _p, _p, _p, C.POINTER(CompositeParams), _p]),
    "mlgi_set_timing": (C.c_int32, [_p, C.c_int]),
    "mlgi_last_timings": (C.c_int32, [_p, _p, C.c_int]),
    "mlgi_check_device_status": (C.c_int32, [_p, _p]),
    "mlgi_set_gather_wait_test": (C.c_int32, [_p, C.c_int64, C.c_uint32]),
    "mlgi_set_alloc_fault": (C.c_int32, [C.c_int64]),
    "mlgi_checks_enabled": (C.c_int, []),
    "mlgi_check_index_selftest": (C.c_int32, [_p, C.c_int64, C.c_int64]),
    "mlgi_scene_generate": (C.c_int32, [C.POINTER(SceneDesc), C.POINTER(SceneInfo), _p, _p, _p, _p, _p, _p, _p, _p]),
    "mlgi_scene_generate_device": (C.c_int32, [C.POINTER(SceneDesc), C.POINTER(SceneInfo), _p, _p, C.c_int, _p, _p, _p,
                                               _p, _p, _p, _p]),
}

_lib = None


def load(path: str) -> C.CDLL:
    """Load a build of the library at `path` with the ctypes signature of every entry point."""
    if not os.path.exists(path):
        raise RuntimeError(f"{os.path.basename(path)} is not built ({path}); run __graft_entry__.build()")
    L = C.CDLL(path)
    for name, (res, args) in _SIGS.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    return L


def lib() -> C.CDLL:
    """Load libmlgi.so, or libmlgi_checked.so under MLGI_CHECKED=1 (raises if it was not built)."""
    global _lib
    if _lib is None:
        _lib = load(LIB_PATH)
    return _lib


def declared_symbols() -> list[str]:
    return list(_SIGS)


class MlgiError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"mlgi status {status}: {msg}")
        self.status = status


def ptr(x) -> int:
    """Device or host address of a torch tensor / numpy array (None -> NULL)."""
    if x is None:
        return 0
    if isinstance(x, np.ndarray):
        return x.ctypes.data
    return x.data_ptr()


def mat16(m) -> "C.Array":
    a = np.asarray(m, dtype=np.float32).reshape(16)
    return _f16(*a.tolist())


class Context:
    """Owns an mlgi_ctx; each method calls one C-ABI entry point and raises on failure."""

    def __init__(self, device: int = 0):
        self.h = C.c_void_p()
        d = CtxDesc(device, 0)
        st = lib().mlgi_create(C.byref(self.h), C.byref(d))
        if st != OK:
            raise MlgiError(st, "mlgi_create failed")

    def close(self):
        if self.h:
            lib().mlgi_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, st: int):
        if st != OK:
            raise MlgiError(st, lib().mlgi_last_error(self.h).decode())
        return st

    def stream(self) -> int:
        return lib().mlgi_ctx_stream(self.h) or 0

    def vpl_process(self, rsm: RsmView, params: VplParams, out: VplBuf, stream: int = 0):
        return self._chk(lib().mlgi_vpl_process(self.h, C.byref(rsm), C.byref(params), C.byref(out), stream))

    def ism_splat(self, pts: Points, vpls: VplBuf, n_vpl: int, params: IsmParams, atlas: Atlas, stream: int = 0):
        return self._chk(lib().mlgi_ism_splat(self.h, C.byref(pts), C.byref(vpls), n_vpl, C.byref(params),
                                              C.byref(atlas), stream))

    def pullpush(self, atlas: Atlas, params: IsmParams, stream: int = 0):
        return self._chk(lib().mlgi_pullpush(self.h, C.byref(atlas), C.byref(params), stream))

    def ism_splat_count(self, pts: Points, vpls: VplBuf, n_vpl: int, params: IsmParams, atlas: Atlas) -> int:
        n = C.c_uint64(0)
        self._chk(lib().mlgi_ism_splat_count(self.h, C.byref(pts), C.byref(vpls), n_vpl, C.byref(params),
                                             C.byref(atlas), C.byref(n)))
        return int(n.value)

    def ism_clear(self, atlas: Atlas, stream: int = 0):
        return self._chk(lib().mlgi_ism_clear(self.h, C.byref(atlas), stream))

    def ism_splat_range(self, pts: Points, vpls: VplBuf, n_vpl: int, params: IsmParams, atlas: Atlas, bucket0: int,
                        n_buckets: int, stream: int = 0):
        return self._chk(lib().mlgi_ism_splat_range(self.h, C.byref(pts), C.byref(vpls), n_vpl, C.byref(params),
                                                    C.byref(atlas), bucket0, n_buckets, stream))

    def pullpush_rows(self, atlas: Atlas, params: IsmParams, row0: int, row1: int, stream: int = 0):
        return self._chk(lib().mlgi_pullpush_rows(self.h, C.byref(atlas), C.byref(params), row0, row1, stream))

    def final_gather(self, g: GBufferView, vpls: VplBuf, atlas: Atlas, params: FgParams, out: Radiance,
                     stream: int = 0):
        return self._chk(lib().mlgi_final_gather(self.h, C.byref(g), C.byref(vpls), C.byref(atlas),
                                                 C.byref(params), C.byref(out), stream))

    def gi_frame(self, f: FrameDesc, out: Radiance, stream: int = 0):
        return self._chk(lib().mlgi_gi_frame(self.h, C.byref(f), C.byref(out), stream))

    def gi_frame_host(self, f: FrameDesc, rgb_host: np.ndarray):
        return self._chk(lib().mlgi_gi_frame_host(self.h, C.byref(f), ptr(rgb_host)))

    def set_timing(self, on: bool):
        return self._chk(lib().mlgi_set_timing(self.h, int(on)))

    def last_timings(self) -> np.ndarray:
        """Per-pass ms of the last timed frame: VPLP, ISM clear, splat, pull-push, FG, H2D, D2H, then
        pull level 1, middle levels, push level 1, push level 0."""
        ms = np.zeros(11, np.float32)
        self._chk(lib().mlgi_last_timings(self.h, ms.ctypes.data, 11))
        return ms

    def cluster_lights(self, g: GBufferView, vpls: VplBuf, n_vpl: int, params: ClusterParams, used, masks,
                       pixel_slice, stream: int = 0):
        return self._chk(lib().mlgi_cluster_lights(self.h, C.byref(g), C.byref(vpls), n_vpl, C.byref(params),
                                                   ptr(used), ptr(masks), ptr(pixel_slice), stream))

    def pack_r11g11b10f(self, rgb, words, n: int, stream: int = 0):
        return self._chk(lib().mlgi_pack_r11g11b10f(self.h, ptr(rgb), ptr(words), n, stream))

    def unpack_r11g11b10f(self, words, rgb, n: int, stream: int = 0):
        return self._chk(lib().mlgi_unpack_r11g11b10f(self.h, ptr(words), ptr(rgb), n, stream))

    def gi_blur(self, g: GBufferView, gi_in, gi_out, proj_a: float, proj_b: float, fmt: int = F32, stream: int = 0):
        p = BlurParams(proj_a, proj_b, fmt)
        return self._chk(lib().mlgi_gi_blur(self.h, C.byref(g), ptr(gi_in), ptr(gi_out), C.byref(p), stream))

    def composite(self, gi, albedo, out, width: int, height: int, exposure: float, gi_format: int = F32,
                  out_format: int = F32, occlusion=None, direct=None, stream: int = 0):
        p = CompositeParams(width, height, exposure, gi_format, out_format)
        return self._chk(lib().mlgi_composite(self.h, ptr(gi), ptr(albedo), ptr(occlusion), ptr(direct), ptr(out),
                                              C.byref(p), stream))

    def check_device_status(self, stream: int = 0):
        return self._chk(lib().mlgi_check_device_status(self.h, stream))

    def autotune(self, width, height, n_vpl, n_points, reduced=False, min_vpls_per_pixel=16, min_ism_size=64,
                 batched=False, budget_ms=0.0, seed=1, rsm_size=512) -> AutotuneResult:
        q = AutotuneQuery(width, height, n_vpl, n_points, int(reduced), rsm_size, min_vpls_per_pixel, min_ism_size,
                          int(batched), budget_ms, seed)
        r = AutotuneResult()
        self._chk(lib().mlgi_autotune(self.h, C.byref(q), C.byref(r)))
        return r


def shuffle_table(n: int) -> np.ndarray:
    out = np.zeros(n, np.int32)
    st = lib().mlgi_shuffle_table(n, out.ctypes.data)
    if st != OK:
        raise MlgiError(st, "mlgi_shuffle_table")
    return out


# ---- workload configurations ------------------------------------------------------------------

@dataclasses.dataclass(frozen=True)
class Config:
    """One GI workload: scene, buffer sizes and the GI parameters of GIStage (GIStage.cpp:213-232)."""
    name: str
    width: int
    height: int
    rsm: int
    n_vpl: int
    n_points: int
    ism_size: int
    grid_x: int
    grid_y: int
    levels: int
    interleave: int
    n_boxes: int
    n_spheres: int
    tile: int = 16
    cull: int = 0
    influence_cutoff: float = 0.0
    reduced: bool = False          # FP16 atlas, BF16/FP16 VPL records, FP16 G-buffer normals
    seed: int = 1
    light_intensity: float = 5.0   # GIStage.cpp:215
    gi_intensity: float = 3000.0   # GIStage.cpp:217
    clamp_value: float = 0.001     # GIStage.cpp:218
    shuffle: bool = True           # GIStage.cpp:232
    z_near: float = 1.0
    z_far: float = 400.0
    light_yaw_deg: float = 0.0
    light_pitch_deg: float = 0.0
    camera_orbit_deg: float = 0.0

    @property
    def atlas_w(self) -> int:
        return self.grid_x * self.ism_size

    @property
    def atlas_h(self) -> int:
        return self.grid_y * self.ism_size

    @property
    def pairs(self) -> int:
        """Evaluated pixel-VPL pairs per frame: W*H*N/I^2."""
        return self.width * self.height * self.n_vpl // (self.interleave ** 2)

    def replace(self, **kw) -> "Config":
        return dataclasses.replace(self, **kw)


# Plain method, small, FP32, one frame (640x360, 256 VPLs, 2^18 points, 64^2 ISMs, 4 levels, I=4).
C1 = Config("c1_640x360_n256", 640, 360, 256, 256, 1 << 18, 64, 16, 16, 4, 4, 4, 2, tile=16, cull=0)
# Plain method, full size (1080p, 1024 VPLs, 2^22 points, 128^2 ISMs in a 4096^2 atlas, 6 levels, I=8,
# 16x16 tiles with per-tile culling: the VPL's half-space against the tile's box, and an influence
# radius from flux, (max flux / cutoff)^(1/4); the cutoff 1e-8 is 1e-5 of the per-pair clamp).
C2 = Config("c2_1920x1080_n1024", 1920, 1080, 512, 1024, 1 << 22, 128, 32, 32, 6, 8, 16, 8, tile=16, cull=1,
            influence_cutoff=1e-8)
# Reduced-precision form of C1 (FP16 atlas, FP16 normals, BF16 flux).
C3 = C1.replace(name="c3_640x360_n256_fp16", reduced=True)
# Reduced precision with 2048 VPLs at 96^2 ISMs on a 64x32 grid (6144x3072 atlas), 2^23 points.
C3B = C1.replace(name="c3b_640x360_n2048_ism96_fp16", n_vpl=2048, n_points=1 << 23, ism_size=96, grid_x=64,
                 grid_y=32, levels=5, reduced=True)
# The reference's own defaults where its shaders hard-code them: 1024 VPLs, 64^2 ISMs in a 2048^2
# atlas (ImperfectShadowmap.cpp:34), 6 pull-push levels, interleave 4 (final_gathering.comp:53);
# only axis-aligned geometry, so G-buffer normals are exact in every encoding.
CREF = Config("cref_640x360_n1024_ism64", 640, 360, 512, 1024, 1 << 20, 64, 32, 32, 6, 4, 8, 0, tile=16, cull=0)
# A tiny case for unit-sized parity checks.
C0 = Config("c0_160x96_n64", 160, 96, 64, 64, 1 << 14, 32, 8, 8, 3, 4, 3, 1, tile=8, cull=0)

CONFIGS = {c.name: c for c in (C0, C1, C2, C3, C3B, CREF)}


@dataclasses.dataclass
class Scene:
    """Host arrays of one seeded room (numpy), as mlgi_scene_generate writes them."""
    cfg: Config
    info: SceneInfo
    gbuf_depth: np.ndarray
    gbuf_normal: np.ndarray   # float32 (H, W, 2) octahedral
    gbuf_albedo: np.ndarray
    rsm_depth: np.ndarray
    rsm_normal: np.ndarray
    rsm_diffuse: np.ndarray
    points: np.ndarray        # float32 (n_buckets*stride, 4)
    counts: np.ndarray
    bucket_stride: int

    def mat(self, name: str) -> np.ndarray:
        return np.array(getattr(self.info, name), dtype=np.float32)


def make_scene(cfg: Config, points: bool = True) -> Scene:
    """Generate a seeded room on the host through mlgi_scene_generate."""
    d = SceneDesc(cfg.seed, cfg.n_boxes, cfg.n_spheres, cfg.width, cfg.height, cfg.rsm, cfg.rsm, cfg.n_points,
                  cfg.n_vpl, cfg.n_vpl, cfg.light_yaw_deg, cfg.light_pitch_deg, cfg.camera_orbit_deg,
                  cfg.z_near, cfg.z_far)
    info = SceneInfo()
    stride = (cfg.n_points + cfg.n_vpl - 1) // cfg.n_vpl
    W, H, R = cfg.width, cfg.height, cfg.rsm
    gd = np.empty((H, W), np.float32)
    gn = np.empty((H, W, 2), np.float32)
    ga = np.empty((H, W), np.uint32)
    rd = np.empty((R, R), np.float32)
    rn = np.empty((R, R), np.uint32)
    rf = np.empty((R, R), np.uint32)
    pts = np.empty((cfg.n_vpl * stride, 4), np.float32) if points else None
    cnt = np.empty(cfg.n_vpl, np.uint32)
    st = lib().mlgi_scene_generate(C.byref(d), C.byref(info), ptr(gd), ptr(gn), ptr(ga), ptr(rd), ptr(rn), ptr(rf),
                                   ptr(pts), ptr(cnt))
    if st != OK:
        raise MlgiError(st, "mlgi_scene_generate")
    return Scene(cfg, info, gd, gn, ga, rd, rn, rf, pts, cnt, int(info.bucket_stride))


def depth_terms(scene: "Scene") -> tuple[float, float]:
    """projectionMatrix[2][2] and [3][2] of the camera (reprojection.glsl's linearDepth A and B)."""
    p = scene.mat("proj")
    return float(p[10]), float(p[14])


def ism_params(cfg: Config) -> IsmParams:
    return IsmParams(0, cfg.n_vpl, 0, 0, cfg.ism_size, cfg.grid_x, cfg.grid_y, cfg.levels, cfg.z_far)


def pullpush_launches(cfg: Config) -> int:
    """Kernel launches of mlgi_pullpush for the configuration: 1 when each ISM's whole pyramid runs in
    one block, 4 (2 for a single level) for the per-level form."""
    return lib().mlgi_pullpush_launches(C.byref(ism_params(cfg)))


def vpl_params(cfg: Config, scene: Scene) -> VplParams:
    return VplParams(cfg.n_vpl, cfg.light_intensity, int(cfg.shuffle), mat16(scene.mat("inv_biased_light_vp")))


def fg_params(cfg: Config, scene: Scene) -> FgParams:
    a, b = depth_terms(scene) if scene.info is not None else (0.0, 0.0)
    return FgParams(mat16(scene.mat("inv_view_proj")), cfg.z_far, cfg.gi_intensity, cfg.clamp_value, cfg.n_vpl, 0,
                    cfg.n_vpl, 0, cfg.ism_size, cfg.grid_x, cfg.grid_y, cfg.interleave, 1, cfg.tile, cfg.cull,
                    cfg.influence_cutoff, F16 if cfg.reduced else F32, a, b, cfg.z_far)
