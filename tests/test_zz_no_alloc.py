"""The allocation-free ISM entry point (mlgi_ism_render_static) against the allocating path.

Some callers cannot allocate device memory at all: their device memory is reserved up front by
another allocator, or they run inside a callback or plugin that is only handed pre-allocated
buffers. mlgi_ism_render_static serves them by keeping its intermediates in two fixed device
arrays inside the library: the softrender key atlas (4 MiB) and pull-push pyramid levels 1 and 2
(5 MiB), 9 MiB in all. This file checks, through the C ABI, that calls in a row produce exactly
what mlgi_ism_splat + mlgi_pullpush produce (bit-exact, the same bar as the other ISM tests), also
for the FP16 atlas and for ScaleISMs over a VPL subrange, and that an atlas beyond the arrays'
1024 x 1024 texels, or one the allocating path refuses, is refused with otherwise valid buffers.
It is collected last on purpose and also passes on its own.
"""
import ctypes as C

import numpy as np
import pytest

import mlgi
from mlgi.device import DeviceFrame

pytestmark = pytest.mark.gpu


def _render_static(df, cfg, ip):
    import torch

    out = torch.zeros_like(df.atlas)
    pts, vb = df.points_view(), df.vpl_buf()
    st = mlgi.lib().mlgi_ism_render_static(C.byref(pts), C.byref(vb), cfg.n_vpl, C.byref(ip), mlgi.ptr(out),
                                           mlgi.F16 if cfg.reduced else mlgi.F32, None)
    torch.cuda.synchronize()
    return st, out


def _scaled(cfg):
    ip = mlgi.ism_params(cfg)
    ip.vpl_start, ip.vpl_end, ip.scale_isms = 16, cfg.n_vpl // 2, 1
    return ip


def test_static_ism_matches_allocating_path_twice():
    import torch

    ctx = mlgi.Context(0)
    # calls in a row with different atlas sizes and formats: none may see an earlier call's keys
    cases = [(mlgi.C1, mlgi.ism_params), (mlgi.C3, mlgi.ism_params), (mlgi.C1, _scaled), (mlgi.C0, mlgi.ism_params)]
    for cfg, params in cases:
        df = DeviceFrame(mlgi.make_scene(cfg))
        ip = params(cfg)
        ctx.vpl_process(df.rsm_view(), mlgi.vpl_params(cfg, df.scene), df.vpl_buf())
        ctx.ism_splat(df.points_view(), df.vpl_buf(), cfg.n_vpl, ip, df.atlas_view())
        ctx.pullpush(df.atlas_view(), ip)
        torch.cuda.synchronize()
        ref = df.atlas.cpu().numpy().copy()
        st, out = _render_static(df, cfg, ip)
        assert st == mlgi.OK, (cfg.name, params.__name__)
        got = out.cpu().numpy()
        bits = np.uint16 if cfg.reduced else np.uint32
        assert (got.view(bits) == ref.view(bits)).all(), (cfg.name, params.__name__)
        assert (got < 0.99).any()
    ctx.close()


def test_static_ism_rejects_atlas_beyond_its_array():
    cfg = mlgi.C1  # 16 x 16 ISMs of 64^2: exactly the 1024 x 1024 the arrays hold
    df = DeviceFrame(mlgi.make_scene(cfg))
    ctx = mlgi.Context(0)
    ctx.vpl_process(df.rsm_view(), mlgi.vpl_params(cfg, df.scene), df.vpl_buf())
    ctx.close()
    st, _ = _render_static(df, cfg, mlgi.ism_params(cfg))
    assert st == mlgi.OK
    # one ISM column more: 1088 x 1024 texels, every other argument as in the accepted call
    ip = mlgi.ism_params(cfg)
    ip.grid_x += 1
    assert _render_static(df, cfg, ip)[0] == mlgi.EINVAL
    # a long thin atlas within the texel count but wider than 65535 texels, which the allocating
    # entry points refuse too
    ip = mlgi.ism_params(cfg)
    ip.ism_size, ip.levels, ip.grid_x, ip.grid_y = 2, 1, 32768, 1
    assert 2 * 32768 * 2 <= 1 << 20
    assert _render_static(df, cfg, ip)[0] == mlgi.EINVAL
