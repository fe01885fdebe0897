"""Reference-style clustered culling (mlgi_cluster_lights; mlgi_final_gather with cull == 2) on
the GPU against the oracle, and the parity study: its radiance against the unculled FP64 gather
and against the per-tile culler's."""
import json
import os

import numpy as np
import pytest

import mlgi
from oracle import oracle as O

pytestmark = pytest.mark.gpu

STUDY = {}


@pytest.fixture(scope="module")
def ctx():
    c = mlgi.Context(0)
    yield c
    path = os.environ.get("MLGI_CLUSTER_REPORT")
    if path and STUDY:
        with open(path, "w") as f:
            json.dump(STUDY, f, indent=1, sort_keys=True)
    c.close()


def _ms(ctx, fn, reps=20):
    """Mean device time of fn (calls on the context's stream), after warm-up."""
    import torch

    st = torch.cuda.ExternalStream(ctx.stream())
    for _ in range(3):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(reps):
        fn()
    e1.record(st)
    e1.synchronize()
    return e0.elapsed_time(e1) / reps


def frame(ctx, cfg):
    import torch

    from mlgi.device import DeviceFrame

    sc = mlgi.make_scene(cfg)
    df = DeviceFrame(sc)
    ctx.vpl_process(df.rsm_view(), mlgi.vpl_params(cfg, sc), df.vpl_buf())
    ctx.ism_splat(df.points_view(), df.vpl_buf(), cfg.n_vpl, mlgi.ism_params(cfg), df.atlas_view())
    ctx.pullpush(df.atlas_view(), mlgi.ism_params(cfg))
    torch.cuda.synchronize()
    return sc, df


@pytest.mark.parametrize("cfg", [mlgi.C1, mlgi.C2], ids=lambda c: c.name)
def test_cluster_masks_match_oracle(ctx, cfg):
    import torch

    sc, df = frame(ctx, cfg)
    w, h = cfg.width, cfg.height
    tiles = ((w + 127) // 128) * ((h + 127) // 128)
    words = (cfg.n_vpl + 31) // 32
    used = torch.zeros(tiles, dtype=torch.int32, device="cuda")
    masks = torch.zeros(tiles * 16 * words, dtype=torch.int32, device="cuda")
    sl = torch.zeros(h * w, dtype=torch.uint8, device="cuda")
    a, b = mlgi.depth_terms(sc)
    p = mlgi.ClusterParams(mlgi.mat16(sc.mat("inv_view_proj")), a, b, cfg.z_far)
    ctx.cluster_lights(df.gbuffer_view(), df.vpl_buf(), cfg.n_vpl, p, used, masks, sl)
    torch.cuda.synchronize()
    pos, _, _, pn = df.vpl_records()
    ru, rm, rs = O.cluster_lights(sc.gbuf_depth, sc.mat("inv_view_proj"), a, b, cfg.z_far, pos, pn, cfg.n_vpl)
    gu = used.cpu().numpy().view(np.uint32)
    assert (sl.cpu().numpy().reshape(h, w) == rs).all()
    assert (gu == ru).all()
    gm = masks.cpu().numpy().view(np.uint32).reshape(tiles * 16, words)
    rows = np.array([(ru[r // 16] >> (r % 16)) & 1 for r in range(tiles * 16)], bool)  # used clusters only
    assert (gm[rows] == rm[rows]).all()
    kept = np.unpackbits(gm[rows].view(np.uint8)).mean()
    assert 0 < kept < 1  # the culler keeps some VPLs and drops others


@pytest.mark.parametrize("cfg", [mlgi.C1, mlgi.C2], ids=lambda c: c.name)
def test_clustered_gather_matches_oracle_and_study(ctx, cfg):
    import torch

    sc, df = frame(ctx, cfg)
    pos, nrm, col, pn = df.vpl_records()
    a, b = mlgi.depth_terms(sc)
    fp = mlgi.fg_params(cfg.replace(cull=2), sc)
    ctx.final_gather(df.gbuffer_view(), df.vpl_buf(), df.atlas_view(), fp, df.radiance())
    ctx.check_device_status()
    torch.cuda.synchronize()
    got = df.rgb_np().astype(np.float64)
    _, masks, sl = O.cluster_lights(sc.gbuf_depth, sc.mat("inv_view_proj"), a, b, cfg.z_far, pos, pn, cfg.n_vpl)
    atlas = df.atlas_np()
    args = (sc.gbuf_depth, sc.gbuf_normal, sc.mat("inv_view_proj").astype(np.float64), pos, nrm, col, atlas,
            cfg.ism_size, cfg.grid_x, cfg.grid_y, cfg.z_far, cfg.gi_intensity, cfg.clamp_value, cfg.interleave)
    ref = O.final_gather_clustered(*args, masks, sl)
    rel = lambda x, y: float(np.linalg.norm(x - y) / np.linalg.norm(y))
    assert rel(got, ref) < 1e-3
    # the study: the reference-style culler against no culling and against the per-tile culler
    full = O.final_gather(*args, dtype=np.float64)
    fp1 = mlgi.fg_params(cfg.replace(cull=1, tile=16), sc)
    ctx.final_gather(df.gbuffer_view(), df.vpl_buf(), df.atlas_view(), fp1, df.radiance())
    torch.cuda.synchronize()
    tiled = df.rgb_np().astype(np.float64)
    lost = float(np.mean(np.abs(got - full).max(-1) > 1e-3 * np.abs(full).max()))
    g, vb, at, out = df.gbuffer_view(), df.vpl_buf(), df.atlas_view(), df.radiance()
    tiles = ((cfg.width + 127) // 128) * ((cfg.height + 127) // 128)
    used = torch.zeros(tiles, dtype=torch.int32, device="cuda")
    cmasks = torch.zeros(tiles * 16 * ((cfg.n_vpl + 31) // 32), dtype=torch.int32, device="cuda")
    csl = torch.zeros(cfg.width * cfg.height, dtype=torch.uint8, device="cuda")
    cp = mlgi.ClusterParams(mlgi.mat16(sc.mat("inv_view_proj")), a, b, cfg.z_far)
    STUDY[cfg.name] = {"clustered_vs_unculled_rel_l2": rel(got, full), "per_tile_vs_unculled_rel_l2": rel(tiled, full),
                       "pixels_off_by_more_than_1e-3_of_max": lost,
                       "cluster_passes_ms": _ms(ctx, lambda: ctx.cluster_lights(g, vb, cfg.n_vpl, cp, used, cmasks, csl)),
                       "clustered_gather_ms": _ms(ctx, lambda: ctx.final_gather(g, vb, at, fp, out)),
                       "per_tile_gather_ms": _ms(ctx, lambda: ctx.final_gather(g, vb, at, fp1, out))}
    print(cfg.name, STUDY[cfg.name])
    assert rel(tiled, full) < 1e-3
