"""The gathering's bounded device wait runs out, is reported, and leaves the context usable.

The final gathering stages each tile's VPL slice with a bulk copy completed on an mbarrier and
waits for it a bounded number of SM cycles. mlgi_set_gather_wait_test shortens that limit and
makes each block's first wait expect 16 bytes more than its copy delivers, so the phase never
completes and every wait runs out: no GPU fault, trap or unbounded spin is involved. The blocks set
the device status word, retire the surplus, let their copies land and return; then
mlgi_check_device_status reports MLGI_ETIMEDOUT, and the same context renders the frame again,
bit for bit as before.
"""
import ctypes as C

import numpy as np
import pytest

import mlgi
from mlgi.device import DeviceFrame

pytestmark = pytest.mark.gpu


def _gather(ctx, df):
    import torch

    df.rgb.zero_()
    ctx.final_gather(df.gbuffer_view(), df.vpl_buf(), df.atlas_view(), df.fg(), df.radiance())
    torch.cuda.synchronize()
    return df.rgb_np().copy()


@pytest.mark.parametrize("cfg", [mlgi.C1, mlgi.C2], ids=lambda c: c.name)
def test_staging_wait_times_out_and_the_context_recovers(cfg):
    ctx = mlgi.Context(0)
    df = DeviceFrame(mlgi.make_scene(cfg))
    ip = mlgi.ism_params(cfg)
    ctx.vpl_process(df.rsm_view(), mlgi.vpl_params(cfg, df.scene), df.vpl_buf())
    ctx.ism_splat(df.points_view(), df.vpl_buf(), cfg.n_vpl, ip, df.atlas_view())
    ctx.pullpush(df.atlas_view(), ip)
    ref = _gather(ctx, df)
    ctx.check_device_status()
    assert np.abs(ref).max() > 0

    # a short limit alone changes nothing
    assert mlgi.lib().mlgi_set_gather_wait_test(ctx.h, 2_000_000, 0) == mlgi.OK
    assert (_gather(ctx, df) == ref).all()
    ctx.check_device_status()

    # 16 bytes expected beyond each first copy: every block's wait runs out after ~0.1 ms
    assert mlgi.lib().mlgi_set_gather_wait_test(ctx.h, 200_000, 16) == mlgi.OK
    _gather(ctx, df)
    with pytest.raises(mlgi.MlgiError) as e:
        ctx.check_device_status()
    assert e.value.status == mlgi.ETIMEDOUT
    ctx.check_device_status()  # the word was cleared when it was reported

    # back to normal: the same context renders the same frame
    assert mlgi.lib().mlgi_set_gather_wait_test(ctx.h, 0, 0) == mlgi.OK
    assert (_gather(ctx, df) == ref).all()
    ctx.check_device_status()

    # out-of-range settings are refused
    assert mlgi.lib().mlgi_set_gather_wait_test(ctx.h, 10, 0) == mlgi.EINVAL
    assert mlgi.lib().mlgi_set_gather_wait_test(ctx.h, -1, 0) == mlgi.EINVAL
    assert mlgi.lib().mlgi_set_gather_wait_test(ctx.h, 0, 1 << 20) == mlgi.EINVAL
    ctx.close()
