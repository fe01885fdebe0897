"""Device-resident buffers of one GI frame, allocated with torch and handed to the C ABI.

torch is used only for device memory, pinned host memory and streams; every computation is a
libmlgi.so kernel.
"""
from __future__ import annotations

import numpy as np

from . import (F16, F32, Atlas, Config, FgParams, FrameDesc, GBufferView, Points, Radiance, RsmView, Scene,
               VplBuf, fg_params, ism_params, ptr, vpl_params)


def _t(a: np.ndarray, device):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a)).to(device)


class DeviceFrame:
    """Inputs, intermediate buffers and output of one frame on the GPU."""

    def __init__(self, scene: Scene, device: str = "cuda", generated: bool = False, intermediates: bool = True):
        import torch

        cfg: Config = scene.cfg
        self.cfg, self.scene, self.device = cfg, scene, device
        if generated:  # inputs produced on the GPU by mlgi_scene_generate_device
            R, px = cfg.rsm, cfg.width * cfg.height
            self.rsm_depth = torch.empty(R * R, dtype=torch.float32, device=device)
            self.rsm_normal = torch.empty(R * R, dtype=torch.int32, device=device)
            self.rsm_diffuse = torch.empty(R * R, dtype=torch.int32, device=device)
            self.points = torch.zeros(cfg.n_vpl * scene.bucket_stride * 4, dtype=torch.float32, device=device)
            self.counts = torch.empty(cfg.n_vpl, dtype=torch.int32, device=device)
            self.gbuf_depth = torch.empty(px, dtype=torch.float32, device=device)
            self.gbuf_normal = torch.empty(px * 2, dtype=torch.float16 if cfg.reduced else torch.float32, device=device)
        else:
            self.rsm_depth = _t(scene.rsm_depth, device)
            self.rsm_normal = _t(scene.rsm_normal.view(np.int32), device)
            self.rsm_diffuse = _t(scene.rsm_diffuse.view(np.int32), device)
            self.points = _t(scene.points, device)
            self.counts = _t(scene.counts.view(np.int32), device)
            self.gbuf_depth = _t(scene.gbuf_depth, device)
            gn = scene.gbuf_normal.astype(np.float16) if cfg.reduced else scene.gbuf_normal
            self.gbuf_normal = _t(gn, device)
        n = cfg.n_vpl if intermediates else 1
        self.vpl = torch.zeros(n * 12, dtype=torch.float32, device=device)
        self.packed = torch.zeros(n * 4, dtype=torch.float32, device=device)
        self.reduced = torch.zeros(n * 24, dtype=torch.uint8, device=device)
        texels = cfg.atlas_h * cfg.atlas_w if intermediates else 1
        self.keys = torch.zeros(texels, dtype=torch.int32, device=device)
        self.atlas = torch.zeros(texels, dtype=torch.float16 if cfg.reduced else torch.float32, device=device)
        self.rgb = torch.zeros(cfg.height * cfg.width * 3, dtype=torch.float32, device=device)
        if generated:
            self.generate()
        # the library works on its own (non-blocking) streams: the uploads above must be complete
        torch.cuda.synchronize(device)

    @classmethod
    def generated(cls, cfg: Config, device: str = "cuda", intermediates: bool = True) -> "DeviceFrame":
        """A frame whose inputs are generated on the GPU (no host-side scene arrays)."""
        from . import SceneInfo

        stride = (cfg.n_points + cfg.n_vpl - 1) // cfg.n_vpl
        scene = Scene(cfg, SceneInfo(), None, None, None, None, None, None, None, None, stride)
        return cls(scene, device, generated=True, intermediates=intermediates)

    def generate(self, stream: int = 0):
        """(Re)generate this frame's inputs on the GPU from cfg (room seed, light and camera pose)."""
        import ctypes as C

        from . import SceneDesc, lib

        c = self.cfg
        d = SceneDesc(c.seed, c.n_boxes, c.n_spheres, c.width, c.height, c.rsm, c.rsm, c.n_points, c.n_vpl, c.n_vpl,
                      c.light_yaw_deg, c.light_pitch_deg, c.camera_orbit_deg, c.z_near, c.z_far)
        st = lib().mlgi_scene_generate_device(C.byref(d), C.byref(self.scene.info), ptr(self.gbuf_depth),
                                              ptr(self.gbuf_normal), F16 if c.reduced else F32, None,
                                              ptr(self.rsm_depth), ptr(self.rsm_normal), ptr(self.rsm_diffuse),
                                              ptr(self.points), ptr(self.counts), stream or None)
        if st != 0:
            raise RuntimeError(f"mlgi_scene_generate_device failed: {st}")

    # -- C structs ---------------------------------------------------------------------------
    def rsm_view(self) -> RsmView:
        c = self.cfg
        return RsmView(c.rsm, c.rsm, ptr(self.rsm_depth), ptr(self.rsm_normal), ptr(self.rsm_diffuse))

    def vpl_buf(self) -> VplBuf:
        return VplBuf(self.cfg.n_vpl, ptr(self.vpl), ptr(self.packed), ptr(self.reduced))

    def points_view(self) -> Points:
        return Points(ptr(self.points), ptr(self.counts), self.cfg.n_vpl, self.scene.bucket_stride)

    def atlas_view(self) -> Atlas:
        c = self.cfg
        return Atlas(c.atlas_w, c.atlas_h, ptr(self.keys), ptr(self.atlas), F16 if c.reduced else F32)

    def gbuffer_view(self) -> GBufferView:
        c = self.cfg
        return GBufferView(c.width, c.height, ptr(self.gbuf_depth), ptr(self.gbuf_normal), F16 if c.reduced else F32)

    def radiance(self) -> Radiance:
        return Radiance(self.cfg.width, self.cfg.height, ptr(self.rgb))

    def fg(self) -> FgParams:
        return fg_params(self.cfg, self.scene)

    def frame_desc(self) -> FrameDesc:
        c = self.cfg
        return FrameDesc(self.rsm_view(), vpl_params(c, self.scene), self.points_view(), ism_params(c),
                         F16 if c.reduced else F32, self.gbuffer_view(), self.fg())

    # -- host copies -----------------------------------------------------------------------
    def vpl_records(self):
        """(pos[N,3], normal[N,3], flux[N,3], packed_normal_bits[N]) as numpy."""
        v = self.vpl.view(-1, 12).cpu().numpy()
        p = self.packed.view(-1, 4).cpu().numpy()
        return v[:, 0:3].copy(), v[:, 4:7].copy(), v[:, 8:11].copy(), p[:, 3].view(np.uint32).copy()

    def keys_np(self) -> np.ndarray:
        return self.keys.cpu().numpy().view(np.uint32).reshape(self.cfg.atlas_h, self.cfg.atlas_w)

    def atlas_np(self) -> np.ndarray:
        return self.atlas.float().cpu().numpy().reshape(self.cfg.atlas_h, self.cfg.atlas_w)

    def rgb_np(self) -> np.ndarray:
        return self.rgb.cpu().numpy().reshape(self.cfg.height, self.cfg.width, 3)


def host_frame_desc(scene: Scene, pinned: dict) -> FrameDesc:
    """FrameDesc whose pointers are the HOST arrays in `pinned` (for mlgi_gi_frame_host)."""
    c = scene.cfg
    fd = FrameDesc(RsmView(c.rsm, c.rsm, ptr(pinned["rsm_depth"]), ptr(pinned["rsm_normal"]),
                           ptr(pinned["rsm_diffuse"])),
                   vpl_params(c, scene),
                   Points(ptr(pinned["points"]), ptr(pinned["counts"]), c.n_vpl, scene.bucket_stride),
                   ism_params(c), F16 if c.reduced else F32,
                   GBufferView(c.width, c.height, ptr(pinned["gbuf_depth"]), ptr(pinned["gbuf_normal"]),
                               F16 if c.reduced else F32),
                   fg_params(c, scene))
    return fd


def pinned_inputs(scene: Scene) -> dict:
    """Copies of the frame's host inputs in page-locked memory (torch pin_memory)."""
    import torch

    c = scene.cfg
    gn = scene.gbuf_normal.astype(np.float16) if c.reduced else scene.gbuf_normal
    arrs = {"rsm_depth": scene.rsm_depth, "rsm_normal": scene.rsm_normal.view(np.int32),
            "rsm_diffuse": scene.rsm_diffuse.view(np.int32), "points": scene.points,
            "counts": scene.counts.view(np.int32), "gbuf_depth": scene.gbuf_depth, "gbuf_normal": gn}
    out = {k: torch.from_numpy(np.ascontiguousarray(v)).pin_memory() for k, v in arrs.items()}
    out["rgb"] = torch.zeros(c.height * c.width * 3, dtype=torch.float32).pin_memory()
    return out


class Batch:
    """mlgi_batch over DeviceFrames, replayed from a CUDA graph: one persistent launch per pass
    (form BATCH_PERSISTENT) or each view's kernels spread over `streams` streams (BATCH_CONCURRENT)."""

    def __init__(self, ctx, frames, form: int = 0, streams: int = 0):
        import ctypes as C

        from . import BatchOpts, FrameDesc, Radiance, lib

        self.ctx, self.frames = ctx, list(frames)
        self.descs = (FrameDesc * len(self.frames))(*[f.frame_desc() for f in self.frames])
        self.outs = (Radiance * len(self.frames))(*[f.radiance() for f in self.frames])
        self.h = C.c_void_p()
        opts = BatchOpts(form, streams)
        ctx._chk(lib().mlgi_batch_create_ex(ctx.h, len(self.frames), C.cast(self.descs, C.c_void_p),
                                            C.cast(self.outs, C.c_void_p), C.byref(opts), C.byref(self.h)))

    def launch(self, stream: int = 0):
        from . import lib

        return self.ctx._chk(lib().mlgi_batch_launch(self.h, stream))

    def update(self, i: int):
        """Re-read frame i's parameters (e.g. after changing its scene matrices)."""
        import ctypes as C

        from . import lib

        self.descs[i] = self.frames[i].frame_desc()
        return self.ctx._chk(lib().mlgi_batch_update_view(self.h, i, C.byref(self.descs[i]), C.byref(self.outs[i])))

    def kernel_launches(self) -> int:
        from . import lib

        return lib().mlgi_batch_kernel_launches(self.h)

    def close(self):
        from . import lib

        if self.h:
            lib().mlgi_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
