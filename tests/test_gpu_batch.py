"""Batched views (mlgi_batch_*): one persistent launch per pass over mixed views (or over each of
several view groups on their own streams), or each view's kernels on several streams, replayed
from a CUDA graph, must give each view exactly its single-frame (mlgi_gi_frame) result."""
import numpy as np
import pytest

import mlgi
from mlgi.device import Batch, DeviceFrame

pytestmark = pytest.mark.gpu

VIEWS = [mlgi.C0, mlgi.C1.replace(seed=2), mlgi.C3.replace(seed=3),
         mlgi.C1.replace(seed=4, interleave=8, tile=8, name="c1_i8"),
         mlgi.C0.replace(seed=7, reduced=True, name="c0_fp16"), mlgi.C2.replace(seed=5)]


@pytest.fixture(scope="module")
def ctx():
    c = mlgi.Context(0)
    yield c
    c.close()


def single(ctx, df):
    import torch

    ctx.gi_frame(df.frame_desc(), df.radiance())
    torch.cuda.synchronize()
    return df.rgb_np().copy()


@pytest.mark.parametrize("form,streams", [(mlgi.BATCH_PERSISTENT, 0), (mlgi.BATCH_PERSISTENT, 2),
                                          (mlgi.BATCH_PERSISTENT, 4), (mlgi.BATCH_CONCURRENT, 3)],
                         ids=["persistent", "persistent_2groups", "persistent_4groups", "concurrent"])
def test_batch_equals_single_frames_and_replays(ctx, form, streams):
    import torch

    frames = [DeviceFrame(mlgi.make_scene(c)) for c in VIEWS]
    ref = [single(ctx, f) for f in frames]
    for f in frames:
        f.rgb.zero_()
    torch.cuda.synchronize()  # the batch runs on its own stream
    b = Batch(ctx, frames, form, streams)
    # persistent: per view group, clear, VPLs, splat, the four pull-push levels' passes and a
    # gathering pass per precision the group holds (a pass with no items is not launched);
    # concurrent: each view's own kernels
    if form == mlgi.BATCH_PERSISTENT:
        assert b.kernel_launches() == 9 if streams == 0 else 7 * streams < b.kernel_launches() <= 9 * streams
    else:
        # a view's own kernels: the VPL pass with the atlas clear, the splat, one pull-push sequence
        # (one block per ISM, or the per-level launches) and the gathering
        one_seq = [1 if mlgi.pullpush_launches(f.cfg) == 1 else 4 if f.cfg.levels >= 2 else 2 for f in frames]
        assert b.kernel_launches() == sum(2 + n + 1 for n in one_seq)
    for _ in range(2):  # the graph replays
        b.launch()
        torch.cuda.synchronize()
        for f, r in zip(frames, ref):
            got = f.rgb_np()
            assert (got.view(np.uint32) == r.view(np.uint32)).all(), f.cfg.name
            f.rgb.zero_()
        torch.cuda.synchronize()
    ctx.check_device_status()
    # a parameter update takes effect at the next launch
    frames[1].cfg = frames[1].cfg.replace(light_intensity=2.5)
    b.update(1)
    b.launch()
    torch.cuda.synchronize()
    got = frames[1].rgb_np().copy()
    assert (got.view(np.uint32) == single(ctx, frames[1]).view(np.uint32)).all()
    assert not (got == ref[1]).all()
    b.close()


def test_batch_rejects_mixed_precision_view(ctx):
    df = DeviceFrame(mlgi.make_scene(mlgi.C0))
    fd = df.frame_desc()
    fd.atlas_format = mlgi.F16  # FP32 records and normals with an FP16 atlas
    import ctypes as C

    descs = (mlgi.FrameDesc * 1)(fd)
    outs = (mlgi.Radiance * 1)(df.radiance())
    h = C.c_void_p()
    st = mlgi.lib().mlgi_batch_create(ctx.h, 1, C.cast(descs, C.c_void_p), C.cast(outs, C.c_void_p), C.byref(h))
    assert st == mlgi.EINVAL


def test_autotune_picks_measured_candidates(ctx):
    r = ctx.autotune(640, 360, 256, 1 << 18)
    assert 256 // (r.interleave ** 2) >= 16 and r.ism_size in (64, 96, 128) and r.tile in (8, 16)
    assert r.ms > 0 and r.candidates_timed > 4
    again = ctx.autotune(640, 360, 256, 1 << 18)  # cached
    assert (again.interleave, again.ism_size, again.tile, again.ms) == (r.interleave, r.ism_size, r.tile, r.ms)
    # a generous budget buys the highest quality: every VPL at every pixel, the largest ISMs
    best = ctx.autotune(640, 360, 256, 1 << 18, budget_ms=1000.0)
    assert best.interleave == 1 and best.ism_size == 128
    batched = ctx.autotune(640, 360, 256, 1 << 18, batched=True)
    assert batched.tile == 16
