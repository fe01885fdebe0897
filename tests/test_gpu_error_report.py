"""Radiance error of each precision form against the FP64 oracle of the full-precision chain on
the same scene: FP32 (C1, and C2 with per-tile culling) and reduced precision (C3: FP16 atlas, FP16
normals, BF16 flux; C3-B: 2048 VPLs at 96^2). Each value is asserted against its bar and, when
MLGI_ERROR_REPORT names a file, written there as JSON."""
import json
import os

import numpy as np
import pytest

import mlgi
from oracle import oracle as O

pytestmark = pytest.mark.gpu

REPORT = {}


@pytest.fixture(scope="module")
def ctx():
    c = mlgi.Context(0)
    yield c
    path = os.environ.get("MLGI_ERROR_REPORT")
    if path and REPORT:
        with open(path, "w") as f:
            json.dump(REPORT, f, indent=1, sort_keys=True)
    c.close()


def chain(ctx, cfg):
    """VPLs, ISM keys, pull-push and gathering of cfg on the GPU; returns (scene, frame)."""
    import torch

    from mlgi.device import DeviceFrame

    sc = mlgi.make_scene(cfg)
    df = DeviceFrame(sc)
    ctx.vpl_process(df.rsm_view(), mlgi.vpl_params(cfg, sc), df.vpl_buf())
    ctx.ism_splat(df.points_view(), df.vpl_buf(), cfg.n_vpl, mlgi.ism_params(cfg), df.atlas_view())
    ctx.pullpush(df.atlas_view(), mlgi.ism_params(cfg))
    ctx.final_gather(df.gbuffer_view(), df.vpl_buf(), df.atlas_view(), df.fg(), df.radiance())
    ctx.check_device_status()
    torch.cuda.synchronize()
    return sc, df


def fp64_reference(cfg32, sc, df):
    """The FP64 oracle gather on the full-precision chain's VPL records and atlas."""
    pos, nrm, col, _ = df.vpl_records()
    return O.final_gather(sc.gbuf_depth, sc.gbuf_normal, sc.mat("inv_view_proj").astype(np.float64),
                          pos.astype(np.float64), nrm.astype(np.float64), col.astype(np.float64), df.atlas_np(),
                          cfg32.ism_size, cfg32.grid_x, cfg32.grid_y, cfg32.z_far, cfg32.gi_intensity,
                          cfg32.clamp_value, cfg32.interleave, dtype=np.float64)


@pytest.mark.parametrize("cfg,bar", [(mlgi.C1, 1e-3), (mlgi.C2, 1e-3), (mlgi.C3, 2e-2), (mlgi.C3B, 2e-2)],
                         ids=lambda v: getattr(v, "name", str(v)))
def test_radiance_error_against_fp64(ctx, cfg, bar):
    cfg32 = cfg.replace(reduced=False, name=cfg.name + "_fp32")
    sc32, df32 = chain(ctx, cfg32)
    ref = fp64_reference(cfg32, sc32, df32)
    if cfg.reduced:
        _, df = chain(ctx, cfg)
    else:
        df = df32
    rgb = df.rgb_np().astype(np.float64)
    rel = float(np.linalg.norm(rgb - ref) / np.linalg.norm(ref))
    max_abs = float(np.abs(rgb - ref).max())
    REPORT[cfg.name] = {"rel_l2": rel, "max_abs": max_abs, "max_ref": float(np.abs(ref).max()), "bar": bar}
    print(f"{cfg.name}: rel L2 {rel:.3e}, max abs {max_abs:.3e} (max radiance {np.abs(ref).max():.3e})")
    assert rel < bar
