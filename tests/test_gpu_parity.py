"""GPU parity: each CUDA pass, called through the C ABI, against the CPU oracle.

Bar (stated per test): VPL records, ISM keys and the FP32 pull-push atlas are bit-exact with the
oracle's FP32 restatement of the reference shaders; gathered radiance is within a relative L2 of
1e-3 of the FP64 oracle on identical inputs (max-abs reported in the failure message).
"""
import numpy as np
import pytest

import mlgi
from mlgi.device import DeviceFrame, host_frame_desc, pinned_inputs
from oracle import oracle as O

pytestmark = pytest.mark.gpu

FG_REL_L2 = 1e-3  # FP32 gather vs FP64 oracle, relative L2 over the image


@pytest.fixture(scope="module")
def ctx():
    c = mlgi.Context(0)
    yield c
    c.close()


_scenes = {}


def scene(cfg):
    if cfg.name not in _scenes:
        _scenes[cfg.name] = mlgi.make_scene(cfg)
    return _scenes[cfg.name]


def rel_l2(a, b):
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-30))


def oracle_vpls(cfg, sc, dtype=np.float32):
    perm = mlgi.shuffle_table(cfg.n_vpl) if cfg.shuffle else None
    return O.vpl_process(sc.rsm_depth, sc.rsm_normal, sc.rsm_diffuse, cfg.n_vpl, sc.mat("inv_biased_light_vp"),
                         cfg.light_intensity, int(cfg.shuffle), perm, dtype=dtype)


def run_vpl(ctx, df):
    import torch

    ctx.vpl_process(df.rsm_view(), mlgi.vpl_params(df.cfg, df.scene), df.vpl_buf())
    torch.cuda.synchronize()


CFGS_SMALL = [mlgi.C0, mlgi.C1]


@pytest.mark.parametrize("cfg", CFGS_SMALL + [mlgi.C2, mlgi.C1.replace(shuffle=False, name="c1_noshuffle")],
                         ids=lambda c: c.name)
def test_vpl_process_bit_exact(ctx, cfg):
    sc = scene(cfg)
    df = DeviceFrame(sc)
    run_vpl(ctx, df)
    pos, nrm, col, pn = df.vpl_records()
    opos, onrm, ocol, opn = oracle_vpls(cfg, sc)
    assert (pn == opn).all()
    assert (pos.view(np.uint32) == opos.view(np.uint32)).all()
    assert (nrm.view(np.uint32) == onrm.view(np.uint32)).all()
    assert (col.view(np.uint32) == ocol.view(np.uint32)).all()


@pytest.mark.parametrize("cfg", CFGS_SMALL + [mlgi.C2, mlgi.C3B.replace(reduced=False, name="c3b_fp32")],
                         ids=lambda c: c.name)
def test_ism_splat_bit_exact(ctx, cfg):
    """The splat's key atlas against the oracle's, word for word (the cull runs on packed FP32x2,
    the projections on scalar IEEE arithmetic)."""
    import torch

    sc = scene(cfg)
    df = DeviceFrame(sc)
    run_vpl(ctx, df)
    ctx.ism_splat(df.points_view(), df.vpl_buf(), cfg.n_vpl, mlgi.ism_params(cfg), df.atlas_view())
    torch.cuda.synchronize()
    opos, _, _, opn = oracle_vpls(cfg, sc)
    okeys = O.ism_splat(sc.points, sc.counts, sc.bucket_stride, opos, opn, cfg.n_vpl, cfg.ism_size, cfg.grid_x,
                        cfg.grid_y, cfg.z_far)
    keys = df.keys_np()
    assert (okeys != 0xFFFFFFFF).mean() > 0.05  # the case does splat something
    mism = int((keys != okeys).sum())
    assert mism == 0, f"{mism} of {keys.size} atlas words differ"


@pytest.mark.parametrize("cfg", CFGS_SMALL + [mlgi.C2], ids=lambda c: c.name)
def test_ism_splat_atomics_count(ctx, cfg):
    """mlgi_ism_splat_count: the atomics the splat issues, equal to the oracle's count of
    imageAtomicMin calls that land inside the atlas."""
    sc = scene(cfg)
    df = DeviceFrame(sc)
    run_vpl(ctx, df)
    n = ctx.ism_splat_count(df.points_view(), df.vpl_buf(), cfg.n_vpl, mlgi.ism_params(cfg), df.atlas_view())
    opos, _, _, opn = oracle_vpls(cfg, sc)
    _, want = O.ism_splat(sc.points, sc.counts, sc.bucket_stride, opos, opn, cfg.n_vpl, cfg.ism_size, cfg.grid_x,
                          cfg.grid_y, cfg.z_far, count=True)
    assert n == want and 0 < n <= 4 * int(sc.counts.sum())


def _overflowing_counts(sc):
    """Bucket counters past their stride, which the reference's point producer does not bound:
    one bucket reads 37 entries of the next, the last reads past the end of the buffer (zero
    points there), and one counter is 2^32 - 1."""
    c = sc.counts.astype(np.uint32).copy()
    c[3] = sc.bucket_stride + 37
    c[5] = 0xFFFFFFFF
    c[-1] = 3 * sc.bucket_stride
    return c


def test_ism_splat_counts_past_the_stride(ctx):
    import torch

    cfg = mlgi.C0
    sc = scene(cfg)
    df = DeviceFrame(sc)
    run_vpl(ctx, df)
    c = _overflowing_counts(sc)
    df.counts.copy_(torch.from_numpy(c.view(np.int32)))
    ctx.ism_splat(df.points_view(), df.vpl_buf(), cfg.n_vpl, mlgi.ism_params(cfg), df.atlas_view())
    torch.cuda.synchronize()
    opos, _, _, opn = oracle_vpls(cfg, sc)
    assert sc.points.shape[0] == cfg.n_vpl * sc.bucket_stride  # the oracle's imageSize
    okeys = O.ism_splat(sc.points, c, sc.bucket_stride, opos, opn, cfg.n_vpl, cfg.ism_size, cfg.grid_x, cfg.grid_y,
                        cfg.z_far)
    plain = O.ism_splat(sc.points, sc.counts, sc.bucket_stride, opos, opn, cfg.n_vpl, cfg.ism_size, cfg.grid_x,
                        cfg.grid_y, cfg.z_far)
    assert (okeys != plain).any()  # the overflowing counters do change the atlas
    assert (df.keys_np() == okeys).all()


def test_host_frame_counts_past_the_stride(ctx):
    """Counters past the stride make a bucket read the next buckets' entries: the host-buffer frame
    then uploads every point before splatting, and still equals the device frame bit for bit."""
    import torch

    cfg = mlgi.C2
    sc = scene(cfg)
    df = DeviceFrame(sc)
    c = _overflowing_counts(sc)
    df.counts.copy_(torch.from_numpy(c.view(np.int32)))
    ctx.gi_frame(df.frame_desc(), df.radiance())
    torch.cuda.synchronize()
    dev = df.rgb_np().copy()
    pinned = pinned_inputs(sc)
    pinned["counts"].copy_(torch.from_numpy(c.view(np.int32)))
    ctx.gi_frame_host(host_frame_desc(sc, pinned), pinned["rgb"].numpy())
    host = pinned["rgb"].numpy().reshape(dev.shape)
    assert np.abs(dev).max() > 0
    assert (dev.view(np.uint32) == host.view(np.uint32)).all()


def test_ism_splat_vpl_subrange_and_scaled_isms(ctx):
    """VPLStartIndex/EndIndex with ScaleISMs and PointsOnlyToScaledISMs (ism.comp:31-40,56-66)."""
    import torch

    cfg = mlgi.C0
    sc = scene(cfg)
    df = DeviceFrame(sc)
    run_vpl(ctx, df)
    start, end = 16, 48
    ip = mlgi.ism_params(cfg)
    ip.vpl_start, ip.vpl_end, ip.scale_isms, ip.points_only_scaled = start, end, 1, 1
    pts = df.points_view()
    pts.n_buckets = end - start
    ctx.ism_splat(pts, df.vpl_buf(), cfg.n_vpl, ip, df.atlas_view())
    torch.cuda.synchronize()
    opos, _, _, opn = oracle_vpls(cfg, sc)
    okeys = O.ism_splat(sc.points, sc.counts, sc.bucket_stride, opos, opn, cfg.n_vpl, cfg.ism_size, cfg.grid_x,
                        cfg.grid_y, cfg.z_far, vpl_start=start, vpl_end=end, scale_isms=1, points_only=1)
    assert (df.keys_np() == okeys).all()


def test_ism_splat_empty_buckets(ctx):
    import torch

    cfg = mlgi.C0
    sc = scene(cfg)
    df = DeviceFrame(sc)
    run_vpl(ctx, df)
    df.counts.zero_()
    ctx.ism_splat(df.points_view(), df.vpl_buf(), cfg.n_vpl, mlgi.ism_params(cfg), df.atlas_view())
    torch.cuda.synchronize()
    assert (df.keys_np() == 0xFFFFFFFF).all()


@pytest.mark.parametrize("cfg", CFGS_SMALL + [mlgi.C2, mlgi.C3B.replace(reduced=False, name="c3b_fp32")],
                         ids=lambda c: c.name)
def test_pullpush_bit_exact(ctx, cfg):
    """mlgi_pullpush vs the level-by-level restatement of pull.comp/push.comp: one block per ISM
    where the atlas's ISMs make at most one wave of blocks (C0, C1, C3), else the per-level launches
    (C2, C3-B)."""
    import torch

    sc = scene(cfg)
    opos, _, _, opn = oracle_vpls(cfg, sc)
    okeys = O.ism_splat(sc.points, sc.counts, sc.bucket_stride, opos, opn, cfg.n_vpl, cfg.ism_size, cfg.grid_x,
                        cfg.grid_y, cfg.z_far)
    ofin = O.pullpush(okeys, cfg.ism_size, cfg.levels, cfg.z_far)
    df = DeviceFrame(sc)
    df.keys.copy_(torch.from_numpy(okeys.view(np.int32).ravel()))
    ctx.pullpush(df.atlas_view(), mlgi.ism_params(cfg))
    torch.cuda.synchronize()
    fin = df.atlas_np()
    assert (ofin < 0.99).mean() > (okeys >> 8 < 0.99 * 2 ** 24).mean()  # the pyramid fills holes
    mism = int((fin.view(np.uint32) != ofin.view(np.uint32)).sum())
    assert mism == 0, f"{mism} of {fin.size} atlas texels differ"


@pytest.mark.parametrize("cfg", [mlgi.C2, mlgi.C3B.replace(reduced=False, name="c3b_fp32")], ids=lambda c: c.name)
def test_one_block_pyramid_on_large_atlases_bit_exact(ctx, cfg):
    """The one-block-per-ISM pyramid on atlases of several waves of ISMs, run as mlgi_pullpush_rows
    over row runs of at most one wave each (152 SMs x 2 blocks of 128^2 or 96^2 ISMs: 304, so runs of
    8 rows of 32 or 4 rows of 64 ISMs), against the oracle."""
    import torch

    sc = scene(cfg)
    opos, _, _, opn = oracle_vpls(cfg, sc)
    okeys = O.ism_splat(sc.points, sc.counts, sc.bucket_stride, opos, opn, cfg.n_vpl, cfg.ism_size, cfg.grid_x,
                        cfg.grid_y, cfg.z_far)
    ofin = O.pullpush(okeys, cfg.ism_size, cfg.levels, cfg.z_far)
    assert mlgi.pullpush_launches(cfg) == 8  # the whole atlas: several waves, level by level in two halves
    df = DeviceFrame(sc)
    df.keys.copy_(torch.from_numpy(okeys.view(np.int32).ravel()))
    ip = mlgi.ism_params(cfg)
    rows = max(1, 256 // cfg.grid_x)
    for r0 in range(0, cfg.grid_y, rows):
        ctx.pullpush_rows(df.atlas_view(), ip, r0, min(cfg.grid_y, r0 + rows))
    torch.cuda.synchronize()
    fin = df.atlas_np()
    mism = int((fin.view(np.uint32) != ofin.view(np.uint32)).sum())
    assert mism == 0, f"{mism} of {fin.size} atlas texels differ"


@pytest.mark.parametrize("geom", [(mlgi.C1, 256, 4, 4, 4), (mlgi.C1, 256, 4, 3, 4), (mlgi.C0, 32, 8, 8, 1)],
                         ids=["c1_keys_as_256px_isms", "c1_keys_as_3_rows_of_256px_isms", "c0_one_level"])
def test_pullpush_per_level_form_bit_exact(ctx, geom):
    """The per-level pull-push (four launches, two for one level, over each half of the ISM rows
    side by side) that serves ISMs whose pyramid does not fit one block's shared memory, against the
    level-by-level restatement: a splatted atlas read as 4 x 4 ISMs of 256^2 texels with 4 levels,
    its first 768 rows as 4 x 3 such ISMs (halves of one and two rows), and C0's atlas with a single
    level."""
    import torch

    cfg, ism, gx, gy, levels = geom
    sc = scene(cfg)
    opos, _, _, opn = oracle_vpls(cfg, sc)
    okeys = O.ism_splat(sc.points, sc.counts, sc.bucket_stride, opos, opn, cfg.n_vpl, cfg.ism_size, cfg.grid_x,
                        cfg.grid_y, cfg.z_far)
    g = cfg.replace(ism_size=ism, grid_x=gx, grid_y=gy, levels=levels, name="per_level")
    assert g.atlas_w == cfg.atlas_w and g.atlas_h <= cfg.atlas_h
    okeys = np.ascontiguousarray(okeys[: g.atlas_h])
    assert mlgi.pullpush_launches(g) == (4 if levels >= 2 else 2) * 2  # two halves of the ISM rows
    ofin = O.pullpush(okeys, ism, levels, cfg.z_far)
    df = DeviceFrame(sc)
    df.keys[: okeys.size].copy_(torch.from_numpy(okeys.view(np.int32).ravel()))
    ctx.pullpush(mlgi.Atlas(g.atlas_w, g.atlas_h, mlgi.ptr(df.keys), mlgi.ptr(df.atlas), mlgi.F32), mlgi.ism_params(g))
    torch.cuda.synchronize()
    fin = df.atlas.float().cpu().numpy()[: okeys.size].reshape(g.atlas_h, g.atlas_w)
    mism = int((fin.view(np.uint32) != ofin.view(np.uint32)).sum())
    assert mism == 0, f"{mism} of {fin.size} atlas texels differ"


@pytest.mark.parametrize("cfg,z_far", [(mlgi.C1, 3.0e6), (mlgi.C1, 1.0e-7), (mlgi.C2, 3.0e6)],
                         ids=["c1_far_3e6", "c1_far_1e-7", "c2_far_3e6"])
def test_pullpush_far_planes_outside_the_lean_range(ctx, cfg, z_far):
    """A far plane outside [2^-20, 2^20] takes the per-level kernels' general arithmetic (pull1_kernel,
    pullmid_kernel's per-texel forms, push1_kernel) instead of the one-block pyramid's lean forms,
    in two halves of the ISM rows: bit for bit the level-by-level restatement with that far plane."""
    import torch

    sc = scene(cfg)
    opos, _, _, opn = oracle_vpls(cfg, sc)
    okeys = O.ism_splat(sc.points, sc.counts, sc.bucket_stride, opos, opn, cfg.n_vpl, cfg.ism_size, cfg.grid_x,
                        cfg.grid_y, cfg.z_far)
    g = cfg.replace(z_far=z_far, name=cfg.name + "_far")
    assert mlgi.pullpush_launches(g) == (4 if cfg.levels >= 2 else 2) * 2
    ofin = O.pullpush(okeys, cfg.ism_size, cfg.levels, z_far)
    df = DeviceFrame(sc)
    df.keys.copy_(torch.from_numpy(okeys.view(np.int32).ravel()))
    ctx.pullpush(df.atlas_view(), mlgi.ism_params(g))
    torch.cuda.synchronize()
    fin = df.atlas_np()
    mism = int((fin.view(np.uint32) != ofin.view(np.uint32)).sum())
    assert mism == 0, f"{mism} of {fin.size} atlas texels differ"


@pytest.mark.parametrize("cfg", [mlgi.C0, mlgi.C2, mlgi.C3B.replace(reduced=False, name="c3b_fp32")],
                         ids=lambda c: c.name)
def test_splat_ranges_and_pullpush_rows_equal_whole_passes(ctx, cfg):
    """mlgi_ism_splat_range over a shuffled partition of the buckets after one clear, then
    mlgi_pullpush_rows over a shuffled partition of the ISM rows spread over two streams, give
    mlgi_ism_splat's keys and mlgi_pullpush's atlas bit for bit."""
    import torch

    sc = scene(cfg)
    df = DeviceFrame(sc)
    run_vpl(ctx, df)
    ip = mlgi.ism_params(cfg)
    ctx.ism_splat(df.points_view(), df.vpl_buf(), cfg.n_vpl, ip, df.atlas_view())
    ctx.pullpush(df.atlas_view(), ip)
    torch.cuda.synchronize()
    keys, fin = df.keys_np().copy(), df.atlas_np().copy()
    rng = np.random.default_rng(11)
    cuts = np.unique(np.concatenate([[0, cfg.n_vpl], rng.integers(0, cfg.n_vpl, 9)]))
    parts = list(zip(cuts[:-1], cuts[1:]))
    rng.shuffle(parts)
    df.atlas.zero_()
    ctx.ism_clear(df.atlas_view())
    for b0, b1 in parts:
        ctx.ism_splat_range(df.points_view(), df.vpl_buf(), cfg.n_vpl, ip, df.atlas_view(), int(b0), int(b1 - b0))
    torch.cuda.synchronize()
    assert (df.keys_np() == keys).all()
    cuts = np.unique(np.concatenate([[0, cfg.grid_y], rng.integers(0, cfg.grid_y, 4)]))
    rows = list(zip(cuts[:-1], cuts[1:]))
    rng.shuffle(rows)
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    streams = [ctx.stream(), side.cuda_stream]
    torch.cuda.synchronize()
    for i, (r0, r1) in enumerate(rows):
        ctx.pullpush_rows(df.atlas_view(), ip, int(r0), int(r1), streams[i % 2])
    torch.cuda.synchronize()
    assert (df.atlas_np().view(np.uint32) == fin.view(np.uint32)).all()
    with pytest.raises(mlgi.MlgiError):
        ctx.pullpush_rows(df.atlas_view(), ip, 0, cfg.grid_y + 1)
    with pytest.raises(mlgi.MlgiError):
        ctx.ism_splat_range(df.points_view(), df.vpl_buf(), cfg.n_vpl, ip, df.atlas_view(), cfg.n_vpl - 1, 2)


def test_pullpush_fp16_atlas_is_rounded_fp32(ctx):
    import torch

    cfg = mlgi.C3
    sc = scene(cfg)
    opos, _, _, opn = oracle_vpls(cfg, sc)
    okeys = O.ism_splat(sc.points, sc.counts, sc.bucket_stride, opos, opn, cfg.n_vpl, cfg.ism_size, cfg.grid_x,
                        cfg.grid_y, cfg.z_far)
    ofin = O.pullpush(okeys, cfg.ism_size, cfg.levels, cfg.z_far)
    df = DeviceFrame(sc)
    df.keys.copy_(torch.from_numpy(okeys.view(np.int32).ravel()))
    ctx.pullpush(df.atlas_view(), mlgi.ism_params(cfg))
    torch.cuda.synchronize()
    assert (df.atlas.cpu().numpy().reshape(ofin.shape) == ofin.astype(np.float16)).all()


def _fg_inputs(ctx, cfg):
    """Run the GPU chain up to the atlas; return the frame and oracle-side copies of its inputs."""
    import torch

    sc = scene(cfg)
    df = DeviceFrame(sc)
    run_vpl(ctx, df)
    ctx.ism_splat(df.points_view(), df.vpl_buf(), cfg.n_vpl, mlgi.ism_params(cfg), df.atlas_view())
    ctx.pullpush(df.atlas_view(), mlgi.ism_params(cfg))
    torch.cuda.synchronize()
    return sc, df


def _oracle_fg(cfg, sc, df, dtype, tile=0, cutoff=0.0, reduced_inputs=False):
    pos, nrm, col, _ = df.vpl_records()
    gn = sc.gbuf_normal
    if reduced_inputs:  # the reduced path's stored values, widened back
        rec = df.reduced.cpu().numpy().view(np.uint8).reshape(-1, 24)
        pos = rec[:, 0:12].copy().view(np.float32).reshape(-1, 3)
        nrm = rec[:, 12:18].copy().view(np.float16).astype(np.float32).reshape(-1, 3)
        fl = rec[:, 18:24].copy().view(np.uint16).astype(np.uint32) << 16
        col = fl.view(np.float32).reshape(-1, 3)
        gn = sc.gbuf_normal.astype(np.float16).astype(np.float32)
    atlas = df.atlas_np()
    return O.final_gather(sc.gbuf_depth, gn, sc.mat("inv_view_proj").astype(dtype), pos.astype(dtype),
                          nrm.astype(dtype), col.astype(dtype), atlas, cfg.ism_size, cfg.grid_x, cfg.grid_y,
                          cfg.z_far, cfg.gi_intensity, cfg.clamp_value, cfg.interleave, tile=tile, cutoff=cutoff,
                          dtype=dtype)


@pytest.mark.parametrize("cfg", CFGS_SMALL + [mlgi.C1.replace(interleave=8, tile=8, name="c1_i8_t8"),
                                              mlgi.C1.replace(interleave=1, name="c1_i1"),
                                              mlgi.C1.replace(width=637, height=357, cull=1, name="c1_ragged_cull"),
                                              # one-warp 8x8 tiles with culling; 64 VPLs a class in
                                              # two staging chunks
                                              mlgi.C1.replace(interleave=8, tile=8, cull=1, name="c1_i8_t8_cull"),
                                              mlgi.C1.replace(interleave=2, tile=8, cull=1, name="c1_i2_t8_cull")],
                         ids=lambda c: c.name)
def test_final_gather_matches_fp64_oracle(ctx, cfg):
    import torch

    sc, df = _fg_inputs(ctx, cfg)
    ctx.final_gather(df.gbuffer_view(), df.vpl_buf(), df.atlas_view(), df.fg(), df.radiance())
    ctx.check_device_status()
    torch.cuda.synchronize()
    rgb = df.rgb_np()
    ref = _oracle_fg(cfg, sc, df, np.float64)
    e = rel_l2(rgb, ref)
    assert e < FG_REL_L2, f"rel L2 {e:.3e}, max abs {np.abs(rgb - ref).max():.3e}"
    assert np.abs(ref).max() > 0


def test_final_gather_scaled_isms_wrap_off_the_grid(ctx):
    """ScaleISMs with vplStart 192 of 256 VPLs on an 8x8 grid: VPLs below the range have ISM
    indices far off the grid (down to -192, tile rows down to -24), whose texels wrap around the
    atlas (GL_REPEAT, a true modulo). Against the FP64 oracle with the same layout."""
    import torch

    cfg = mlgi.C1.replace(grid_x=8, grid_y=8, name="c1_grid8")
    sc = scene(cfg)
    df = DeviceFrame(sc)
    run_vpl(ctx, df)
    start, end = 192, 256
    ip = mlgi.ism_params(cfg)
    ip.vpl_start, ip.vpl_end, ip.scale_isms, ip.points_only_scaled = start, end, 1, 1
    pts = df.points_view()
    pts.n_buckets = end - start
    ctx.ism_splat(pts, df.vpl_buf(), cfg.n_vpl, ip, df.atlas_view())
    ctx.pullpush(df.atlas_view(), ip)
    fp = df.fg()
    fp.vpl_start, fp.vpl_end, fp.scale_isms = start, end, 1
    ctx.final_gather(df.gbuffer_view(), df.vpl_buf(), df.atlas_view(), fp, df.radiance())
    ctx.check_device_status()
    torch.cuda.synchronize()
    pos, nrm, col, _ = df.vpl_records()
    ref = O.final_gather(sc.gbuf_depth, sc.gbuf_normal, sc.mat("inv_view_proj").astype(np.float64),
                         pos.astype(np.float64), nrm.astype(np.float64), col.astype(np.float64), df.atlas_np(),
                         cfg.ism_size, cfg.grid_x, cfg.grid_y, cfg.z_far, cfg.gi_intensity, cfg.clamp_value,
                         cfg.interleave, vpl_count=end - start, ism_offset=start, dtype=np.float64)
    got = df.rgb_np()
    assert np.abs(ref).max() > 0
    e = rel_l2(got, ref)
    assert e < FG_REL_L2, f"rel L2 {e:.3e}"


def test_final_gather_culling_c2(ctx):
    """C2: 16x16 same-class tiles with culling: the lossless half-space cull and the influence
    radius from flux (cutoff 1e-8). The result must match the FP64 oracle that applies the same
    rules, and the no-cull FP64 oracle, within the same bar."""
    import torch

    cfg = mlgi.C2
    assert cfg.cull == 1 and cfg.influence_cutoff > 0
    sc, df = _fg_inputs(ctx, cfg)
    ctx.final_gather(df.gbuffer_view(), df.vpl_buf(), df.atlas_view(), df.fg(), df.radiance())
    torch.cuda.synchronize()
    rgb = df.rgb_np()
    ref_cull = _oracle_fg(cfg, sc, df, np.float64, tile=cfg.tile, cutoff=cfg.influence_cutoff)
    e = rel_l2(rgb, ref_cull)
    assert e < FG_REL_L2, f"C2 culled vs culled FP64: rel L2 {e:.3e}"
    ref_nocull = _oracle_fg(cfg, sc, df, np.float64)
    e = rel_l2(rgb, ref_nocull)
    assert e < FG_REL_L2, f"C2 culled vs unculled FP64: rel L2 {e:.3e}"


def test_reduced_precision_error_c3(ctx):
    """C3: FP16 atlas, FP16 normals, BF16 flux. FG on the stored reduced values matches the FP64
    oracle on the same widened values; the end-to-end error against the FP32 chain is stated."""
    import torch

    cfg = mlgi.C3
    sc, df = _fg_inputs(ctx, cfg)
    ctx.final_gather(df.gbuffer_view(), df.vpl_buf(), df.atlas_view(), df.fg(), df.radiance())
    torch.cuda.synchronize()
    rgb = df.rgb_np()
    same_inputs = _oracle_fg(cfg, sc, df, np.float64, reduced_inputs=True)
    assert rel_l2(rgb, same_inputs) < FG_REL_L2
    full = mlgi.C1
    sc32, df32 = _fg_inputs(ctx, full)
    ref32 = _oracle_fg(full, sc32, df32, np.float64)
    e = rel_l2(rgb, ref32)
    assert e < 2e-2, f"reduced-precision chain vs FP64 oracle: rel L2 {e:.3e}"


def test_frame_chain_and_host_frame_agree(ctx):
    import torch

    cfg = mlgi.C1
    sc = scene(cfg)
    df = DeviceFrame(sc)
    ctx.gi_frame(df.frame_desc(), df.radiance())
    torch.cuda.synchronize()
    dev = df.rgb_np().copy()
    pinned = pinned_inputs(sc)
    ctx.gi_frame_host(host_frame_desc(sc, pinned), pinned["rgb"].numpy())
    host = pinned["rgb"].numpy().reshape(dev.shape)
    assert (dev == host).all()
    # and the chain equals the stage-by-stage oracle within the FG bar
    opos, onrm, ocol, opn = oracle_vpls(cfg, sc)
    okeys = O.ism_splat(sc.points, sc.counts, sc.bucket_stride, opos, opn, cfg.n_vpl, cfg.ism_size, cfg.grid_x,
                        cfg.grid_y, cfg.z_far)
    ofin = O.pullpush(okeys, cfg.ism_size, cfg.levels, cfg.z_far)
    ref = O.final_gather(sc.gbuf_depth, sc.gbuf_normal, sc.mat("inv_view_proj").astype(np.float64),
                         opos.astype(np.float64), onrm.astype(np.float64), ocol.astype(np.float64), ofin,
                         cfg.ism_size, cfg.grid_x, cfg.grid_y, cfg.z_far, cfg.gi_intensity, cfg.clamp_value,
                         cfg.interleave, dtype=np.float64)
    assert rel_l2(dev, ref) < FG_REL_L2


@pytest.mark.parametrize("cfg", [mlgi.C1, mlgi.C2, mlgi.C1.replace(cull=2, name="c1_clustered")], ids=lambda c: c.name)
def test_repeated_device_frames_replay_the_same_frame(cfg):
    """mlgi_gi_frame called again with the same arguments captures the frame into a CUDA graph (the
    second call) and replays it (later calls): every such frame equals the first, issued call by
    call, bit for bit; new arguments run directly again; so do frames with per-pass timing."""
    import torch

    ctx = mlgi.Context(0)
    df = DeviceFrame(scene(cfg))
    fd, out = df.frame_desc(), df.radiance()

    def frame(f):
        df.rgb.zero_()
        torch.cuda.synchronize()
        ctx.gi_frame(f, out)
        torch.cuda.synchronize()
        return df.rgb_np().copy()

    first = frame(fd)
    assert np.abs(first).max() > 0
    for _ in range(3):
        assert (frame(fd).view(np.uint32) == first.view(np.uint32)).all()
    brighter = df.frame_desc()
    brighter.vpl.light_intensity *= 2.0
    other = frame(brighter)
    assert not (other == first).all()
    for _ in range(2):
        assert (frame(brighter).view(np.uint32) == other.view(np.uint32)).all()
    assert (frame(fd).view(np.uint32) == first.view(np.uint32)).all()
    ctx.set_timing(True)
    assert (frame(fd).view(np.uint32) == first.view(np.uint32)).all()
    ctx.set_timing(False)
    ctx.check_device_status()
    ctx.close()


@pytest.mark.parametrize("cfg", [mlgi.C0, mlgi.CREF, mlgi.C2, mlgi.C3B, mlgi.C1.replace(cull=2, name="c1_clustered")],
                         ids=lambda c: c.name)
def test_host_frame_equals_device_frame(ctx, cfg):
    """The host-buffer frame splats point ranges as they arrive, pulls and pushes the ISM rows each
    range completes, and gathers and downloads in bands of rows: bit for bit the device frame."""
    import torch

    sc = scene(cfg)
    df = DeviceFrame(sc)
    ctx.gi_frame(df.frame_desc(), df.radiance())
    torch.cuda.synchronize()
    dev = df.rgb_np().copy()
    pinned = pinned_inputs(sc)
    for _ in range(3):  # runs directly, then captures the frame into a graph, then replays it
        pinned["rgb"].zero_()
        ctx.gi_frame_host(host_frame_desc(sc, pinned), pinned["rgb"].numpy())
        host = pinned["rgb"].numpy().reshape(dev.shape)
        assert np.abs(dev).max() > 0
        assert (dev.view(np.uint32) == host.view(np.uint32)).all()


def test_host_frame_replay_reads_new_inputs(ctx):
    """A repeated call replays the captured frame, which copies whatever the host buffers hold at the
    time: new contents of the same buffers give the new frame's result."""
    import torch

    cfg = mlgi.C0
    sa, sb = scene(cfg), scene(cfg.replace(seed=cfg.seed + 11, name="c0_b"))
    pinned = pinned_inputs(sa)
    hfd = host_frame_desc(sa, pinned)
    for _ in range(3):  # direct, captured, replayed
        ctx.gi_frame_host(hfd, pinned["rgb"].numpy())
    for k, v in pinned_inputs(sb).items():  # same shapes, new contents, same buffers
        pinned[k].copy_(v)
    pinned["rgb"].zero_()
    ctx.gi_frame_host(hfd, pinned["rgb"].numpy())
    df = DeviceFrame(sb)
    ctx.gi_frame(df.frame_desc(), df.radiance())
    torch.cuda.synchronize()
    dev = df.rgb_np()
    host = pinned["rgb"].numpy().reshape(dev.shape)
    assert np.abs(dev).max() > 0
    assert (dev.view(np.uint32) == host.view(np.uint32)).all()


def test_host_frame_vpl_subrange_scaled_isms(ctx):
    """A layout the overlapped schedule does not split (VPL subrange, scaled ISMs, points only into
    them): every ISM row is pulled and pushed after the last point range; still the device frame's
    result bit for bit."""
    import torch

    cfg = mlgi.C2
    sc = scene(cfg)
    df = DeviceFrame(sc)
    start, end = 256, 768
    fd = df.frame_desc()
    fd.ism.vpl_start, fd.ism.vpl_end, fd.ism.scale_isms, fd.ism.points_only_scaled = start, end, 1, 1
    fd.points.n_buckets = end - start
    fd.fg.vpl_start, fd.fg.vpl_end, fd.fg.scale_isms = start, end, 1
    ctx.gi_frame(fd, df.radiance())
    torch.cuda.synchronize()
    dev = df.rgb_np().copy()
    pinned = pinned_inputs(sc)
    hfd = host_frame_desc(sc, pinned)
    hfd.ism.vpl_start, hfd.ism.vpl_end, hfd.ism.scale_isms, hfd.ism.points_only_scaled = start, end, 1, 1
    hfd.points.n_buckets = end - start
    hfd.fg.vpl_start, hfd.fg.vpl_end, hfd.fg.scale_isms = start, end, 1
    ctx.gi_frame_host(hfd, pinned["rgb"].numpy())
    host = pinned["rgb"].numpy().reshape(dev.shape)
    assert np.abs(dev).max() > 0
    assert (dev.view(np.uint32) == host.view(np.uint32)).all()


def test_frame_is_deterministic(ctx):
    import torch

    cfg = mlgi.C1
    df = DeviceFrame(scene(cfg))
    outs = []
    for _ in range(3):
        ctx.gi_frame(df.frame_desc(), df.radiance())
        torch.cuda.synchronize()
        outs.append(df.rgb_np().copy())
    assert all((o == outs[0]).all() for o in outs[1:])


def test_invalid_arguments_are_rejected(ctx):
    cfg = mlgi.C0
    df = DeviceFrame(scene(cfg))
    vp = mlgi.vpl_params(cfg, df.scene)
    vp.count = 100  # not a multiple of 64
    with pytest.raises(mlgi.MlgiError) as e:
        ctx.vpl_process(df.rsm_view(), vp, df.vpl_buf())
    assert e.value.status == mlgi.EINVAL
    ip = mlgi.ism_params(cfg)
    ip.ism_size = 30  # not divisible by 2^levels and mismatching the atlas
    with pytest.raises(mlgi.MlgiError):
        ctx.pullpush(df.atlas_view(), ip)
    fp = df.fg()
    fp.interleave = 3  # 64 VPLs are not a multiple of 9
    with pytest.raises(mlgi.MlgiError):
        ctx.final_gather(df.gbuffer_view(), df.vpl_buf(), df.atlas_view(), fp, df.radiance())


def _rejected(fn):
    with pytest.raises(mlgi.MlgiError) as e:
        fn()
    assert e.value.status == mlgi.EINVAL, e.value


def test_limits_and_inconsistent_layouts_are_rejected(ctx):
    """Sizes past the kernels' limits and inconsistent layouts fail with EINVAL before any launch;
    the context stays usable."""
    import torch

    cfg = mlgi.C0
    df = DeviceFrame(scene(cfg))
    run_vpl(ctx, df)
    pts, vb, at = df.points_view(), df.vpl_buf(), df.atlas_view()

    def ism(**kw):
        ip = mlgi.ism_params(cfg)
        for k, v in kw.items():
            setattr(ip, k, v)
        return ip

    big = mlgi.Atlas(8 * 8192, 8 * 32, at.keys, at.depth, at.format)  # 65536 texels wide
    _rejected(lambda: ctx.ism_splat(pts, vb, cfg.n_vpl, ism(ism_size=8192, grid_x=8, grid_y=8, levels=3), big))
    _rejected(lambda: ctx.pullpush(at, ism(levels=0)))
    _rejected(lambda: ctx.pullpush(at, ism(levels=11)))
    _rejected(lambda: ctx.ism_splat(pts, vb, cfg.n_vpl, ism(grid_x=4, grid_y=4),
                                    mlgi.Atlas(4 * cfg.ism_size, 4 * cfg.ism_size, at.keys, at.depth, at.format)))
    bad_pts = df.points_view()
    bad_pts.n_buckets = cfg.n_vpl - 1  # the splat samples one bucket per VPL
    _rejected(lambda: ctx.ism_splat(bad_pts, vb, cfg.n_vpl, ism(), at))
    _rejected(lambda: ctx.ism_splat(pts, vb, cfg.n_vpl, ism(vpl_start=8, vpl_end=8), at))
    _rejected(lambda: ctx.ism_splat(pts, vb, cfg.n_vpl, ism(z_far=0.0), at))
    for field, value in (("tile", 12), ("cull", 3), ("vpl_format", 7)):
        fp = df.fg()
        setattr(fp, field, value)
        _rejected(lambda: ctx.final_gather(df.gbuffer_view(), vb, at, fp, df.radiance()))
    # reduced VPL records off a 16-byte boundary: written by the VPL pass, bulk-copied by the gathering
    odd = mlgi.VplBuf(vb.capacity, vb.vpl, vb.packed, vb.reduced + 8)
    _rejected(lambda: ctx.vpl_process(df.rsm_view(), mlgi.vpl_params(cfg, df.scene), odd))
    fp = df.fg()
    fp.vpl_format = mlgi.F16
    _rejected(lambda: ctx.final_gather(df.gbuffer_view(), odd, at, fp, df.radiance()))
    # a NULL host input of the host-buffer frame
    pinned = pinned_inputs(scene(cfg))
    hfd = host_frame_desc(scene(cfg), pinned)
    hfd.gbuffer.depth = None
    _rejected(lambda: ctx.gi_frame_host(hfd, pinned["rgb"].numpy()))
    # still usable: a valid frame runs after the rejections
    ctx.gi_frame(df.frame_desc(), df.radiance())
    ctx.check_device_status()
    torch.cuda.synchronize()
    assert np.abs(df.rgb_np()).max() > 0
