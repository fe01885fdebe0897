"""Pin the oracle restatement to the reference's own shader source.

oracle/_ref/libref.so is the reference's five GLSL compute shaders compiled as C++ (mechanical
rewrite in oracle/build_ref.py) and driven with the reference's host dispatch geometry. On the
reference's own configuration (CREF: 1024 VPLs, 64^2 ISMs in a 2048^2 atlas, 6 pull-push levels,
interleave 4) every stage of the restatement must agree with it word for word.
"""
import numpy as np
import pytest

import mlgi
from oracle import oracle as O
from oracle import ref as R

pytestmark = pytest.mark.skipif(not R.available(), reason="reference shaders not available to compile")


@pytest.fixture(scope="module")
def case():
    cfg = mlgi.CREF
    sc = mlgi.make_scene(cfg)
    perm = mlgi.shuffle_table(cfg.n_vpl)
    return cfg, sc, perm


def octahedral_to_rgb(e):
    """n*0.5+0.5 of the decoded octahedral normal (the reference G-buffer's normal encoding)."""
    e = e.astype(np.float64)
    n = np.stack([e[..., 0], e[..., 1], 1 - np.abs(e[..., 0]) - np.abs(e[..., 1])], -1)
    neg = n[..., 2] < 0
    sx, sy = np.where(e[..., 0] >= 0, 1, -1), np.where(e[..., 1] >= 0, 1, -1)
    nx = np.where(neg, (1 - np.abs(e[..., 1])) * sx, n[..., 0])
    ny = np.where(neg, (1 - np.abs(e[..., 0])) * sy, n[..., 1])
    n = np.stack([nx, ny, n[..., 2]], -1)
    n /= np.linalg.norm(n, axis=-1, keepdims=True)
    return (n * 0.5 + 0.5).astype(np.float32)


def test_vpl_processor(case):
    cfg, sc, perm = case
    rp, rn, rc, rpk = R.vpl_process(sc.rsm_depth, sc.rsm_normal, sc.rsm_diffuse, cfg.n_vpl,
                                    sc.mat("inv_biased_light_vp"), cfg.light_intensity, 1, perm)
    op, on, oc, opn = O.vpl_process(sc.rsm_depth, sc.rsm_normal, sc.rsm_diffuse, cfg.n_vpl,
                                    sc.mat("inv_biased_light_vp"), cfg.light_intensity, 1, perm)
    for a, b in ((rp, op), (rn, on), (rc, oc)):
        assert (a.view(np.uint32) == b.view(np.uint32)).all()
    assert (rpk[:, 3].view(np.uint32) == opn).all()


def test_ism_splat_and_pullpush(case):
    cfg, sc, perm = case
    op, _, _, opn = O.vpl_process(sc.rsm_depth, sc.rsm_normal, sc.rsm_diffuse, cfg.n_vpl,
                                  sc.mat("inv_biased_light_vp"), cfg.light_intensity, 1, perm)
    packed = np.concatenate([op, opn.view(np.float32)[:, None]], 1)
    rk = R.ism_splat(sc.points, sc.counts, packed, cfg.n_vpl, cfg.atlas_w, cfg.atlas_h, cfg.z_far)
    ok = O.ism_splat(sc.points, sc.counts, sc.bucket_stride, op, opn, cfg.n_vpl, cfg.ism_size, cfg.grid_x,
                     cfg.grid_y, cfg.z_far)
    assert (ok != 0xFFFFFFFF).mean() > 0.1
    assert (rk == ok).all()
    rf = R.pullpush(rk, cfg.ism_size, cfg.levels, cfg.z_far)
    of = O.pullpush(ok, cfg.ism_size, cfg.levels, cfg.z_far)
    assert (rf.view(np.uint32) == of.view(np.uint32)).all()


def test_ism_splat_scaled_subrange(case):
    """ScaleISMs + PointsOnlyToScaledISMs over VPLs [0, 512) (ism.comp:31-40,56-66)."""
    cfg, sc, perm = case
    op, _, _, opn = O.vpl_process(sc.rsm_depth, sc.rsm_normal, sc.rsm_diffuse, cfg.n_vpl,
                                  sc.mat("inv_biased_light_vp"), cfg.light_intensity, 1, perm)
    packed = np.concatenate([op, opn.view(np.float32)[:, None]], 1)
    counts = sc.counts[:512]
    rk = R.ism_splat(sc.points[: 512 * sc.bucket_stride], counts, packed, cfg.n_vpl, cfg.atlas_w, cfg.atlas_h,
                     cfg.z_far, 0, 512, 1, 1)
    ok = O.ism_splat(sc.points, counts, sc.bucket_stride, op, opn, cfg.n_vpl, cfg.ism_size, cfg.grid_x, cfg.grid_y,
                     cfg.z_far, vpl_start=0, vpl_end=512, scale_isms=1, points_only=1)
    assert (rk == ok).all()


def test_final_gathering(case):
    """final_gathering.comp with light lists of 32 VPLs per interleave class (the most the
    reference's 64-entry sub-lists hold without their last entry colliding with the next count)."""
    cfg, sc, perm = case
    op, on, oc, opn = O.vpl_process(sc.rsm_depth, sc.rsm_normal, sc.rsm_diffuse, cfg.n_vpl,
                                    sc.mat("inv_biased_light_vp"), cfg.light_intensity, 1, perm)
    ok = O.ism_splat(sc.points, sc.counts, sc.bucket_stride, op, opn, cfg.n_vpl, cfg.ism_size, cfg.grid_x,
                     cfg.grid_y, cfg.z_far)
    atlas = O.pullpush(ok, cfg.ism_size, cfg.levels, cfg.z_far)
    n = 512
    vpl9 = np.concatenate([op, on, oc], 1)
    rr = R.final_gather(sc.gbuf_depth, octahedral_to_rgb(sc.gbuf_normal), sc.mat("inv_view_proj"), sc.mat("proj"),
                        vpl9[:n], n, 0, n, atlas, cfg.z_far, cfg.z_near, cfg.gi_intensity, cfg.clamp_value, 32)
    orr = O.final_gather(sc.gbuf_depth, sc.gbuf_normal, sc.mat("inv_view_proj"), op[:n], on[:n], oc[:n], atlas,
                         cfg.ism_size, cfg.grid_x, cfg.grid_y, cfg.z_far, cfg.gi_intensity, cfg.clamp_value,
                         cfg.interleave)
    assert np.abs(orr).max() > 0
    assert (rr.view(np.uint32) == orr.view(np.uint32)).all()


def test_clustered_culling_lists(case):
    """clustering.comp + light_lists.comp against the restatement (O.cluster_lights) on CREF: the
    same used clusters, and in each cluster's sub-list s the same VPLs of [64 s, 64 s + 64), as
    sets (the reference's list order is atomic order). A sub-list that keeps all 64 VPLs loses its
    last entry to the next sub-list's count slot (light_lists.comp:117-126), so for such lists the
    reference's 63 entries must be a subset of the restatement's 64."""
    cfg, sc, perm = case
    op, _, _, opn = O.vpl_process(sc.rsm_depth, sc.rsm_normal, sc.rsm_diffuse, cfg.n_vpl,
                                  sc.mat("inv_biased_light_vp"), cfg.light_intensity, 1, perm)
    a, b = mlgi.depth_terms(sc)
    packed = np.concatenate([op, opn.view(np.float32)[:, None]], 1)
    xyz, lists = R.cluster_lights(sc.gbuf_depth, sc.mat("inv_view_proj"), a, b, cfg.z_far, packed)
    used, masks, _ = O.cluster_lights(sc.gbuf_depth, sc.mat("inv_view_proj"), a, b, cfg.z_far, op, opn, cfg.n_vpl)
    ncx = (cfg.width + 127) // 128
    ours = {(t % ncx, t // ncx, s) for t in range(len(used)) for s in range(16) if (int(used[t]) >> s) & 1}
    assert set(xyz) == ours and len(xyz) == len(ours) > 0
    full = partial = 0
    for (x, y, s_), col in zip(xyz, lists):
        row = masks[(y * ncx + x) * 16 + s_]
        for sub in range(16):
            mine = {k for k in range(64 * sub, 64 * sub + 64) if (int(row[k // 32]) >> (k % 32)) & 1}
            n = int(col[64 * sub]) - 1
            ref = {int(v) for v in col[64 * sub + 1: 64 * sub + 1 + min(n, 63)]}
            assert n == len(mine), (x, y, s_, sub)
            if n <= 63:
                assert ref == mine, (x, y, s_, sub)
                partial += 1
            else:
                assert ref <= mine and len(ref) == 63, (x, y, s_, sub)
                full += 1
    assert partial > 0


def test_gi_blur(case):
    """gi_blur.frag's X and Y programs against the restatement, with the normals in the reference's
    RGB G-buffer format on both sides; bit for bit away from the image border, where the shader's
    texelFetch outside the image is undefined and the restatement skips the sample."""
    cfg, sc, perm = case
    a, b = mlgi.depth_terms(sc)
    rgb = octahedral_to_rgb(sc.gbuf_normal)
    gi = np.random.default_rng(3).random((cfg.height, cfg.width, 3)).astype(np.float32)
    rr = R.gi_blur(sc.gbuf_depth, rgb, gi, a, b)
    orr = O.gi_blur_rgb_normals(sc.gbuf_depth, rgb, gi, a, b)
    inner = (slice(3, cfg.height - 3), slice(3, cfg.width - 3))
    assert (rr[inner].view(np.uint32) == orr[inner].view(np.uint32)).all()
    assert np.abs(rr[inner] - gi[inner]).max() > 1e-3  # the filter did change the image
