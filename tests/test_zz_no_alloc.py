"""The allocation-free ISM entry point (mlgi_ism_render_static) against the allocating path.

Some callers cannot allocate device memory at all: their device memory is reserved up front by
another allocator, or they run inside a callback or plugin that is only handed pre-allocated
buffers. mlgi_ism_render_static serves them by keeping its one intermediate buffer (the
softrender key atlas) in a fixed device array inside the library. This file checks, through the
C ABI, that two calls in a row produce exactly what mlgi_ism_splat + mlgi_pullpush produce
(bit-exact, the same bar as the other ISM tests), and that an atlas beyond the array's 1024 x 1024
texels is refused. It is collected last on purpose and also passes on its own.
"""
import ctypes as C

import numpy as np
import pytest

import mlgi
from mlgi.device import DeviceFrame

pytestmark = pytest.mark.gpu


def _render_static(df, cfg):
    import torch

    out = torch.zeros_like(df.atlas)
    pts, vb, ip = df.points_view(), df.vpl_buf(), mlgi.ism_params(cfg)
    st = mlgi.lib().mlgi_ism_render_static(C.byref(pts), C.byref(vb), cfg.n_vpl, C.byref(ip), mlgi.ptr(out),
                                           mlgi.F16 if cfg.reduced else mlgi.F32, None)
    torch.cuda.synchronize()
    return st, out


def test_static_ism_matches_allocating_path_twice():
    import torch

    ctx = mlgi.Context(0)
    # two calls in a row with different atlas sizes: the second must not see the first's keys
    for cfg in (mlgi.C1, mlgi.C0):
        df = DeviceFrame(mlgi.make_scene(cfg))
        ctx.vpl_process(df.rsm_view(), mlgi.vpl_params(cfg, df.scene), df.vpl_buf())
        ctx.ism_splat(df.points_view(), df.vpl_buf(), cfg.n_vpl, mlgi.ism_params(cfg), df.atlas_view())
        ctx.pullpush(df.atlas_view(), mlgi.ism_params(cfg))
        torch.cuda.synchronize()
        ref = df.atlas.cpu().numpy().copy()
        st, out = _render_static(df, cfg)
        assert st == mlgi.OK
        got = out.cpu().numpy()
        assert (got.view(np.uint32) == ref.view(np.uint32)).all()
        assert (got < 0.99).any()
    ctx.close()


def test_static_ism_rejects_atlas_beyond_its_array():
    cfg = mlgi.C2  # 4096 x 4096 texels > 1024 x 1024
    ip = mlgi.ism_params(cfg)
    pts = mlgi.Points(None, None, cfg.n_vpl, 1)
    vb = mlgi.VplBuf(cfg.n_vpl, None, None, None)
    st = mlgi.lib().mlgi_ism_render_static(C.byref(pts), C.byref(vb), cfg.n_vpl, C.byref(ip), 16, mlgi.F32, None)
    assert st == mlgi.EINVAL
