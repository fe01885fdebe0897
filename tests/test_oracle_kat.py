"""Known-answer tests that pin the CPU oracle to the reference shaders' rules.

The reference ships no tests or golden vectors for this path, so each case here is derived by
hand from the shader source it names (paths inside the reference project) and checked against
the oracle's FP32 restatement word for word.
"""
import numpy as np
import pytest

from oracle import oracle as O

f32 = np.float32


def bits(x):
    return int(np.asarray(x, np.float32).view(np.uint32))


# ---- floatpacking.glsl ------------------------------------------------------------------------

def test_pack3sn_axis_normals():
    # floatpacking.glsl:26-44: x*1023+.5, y*1023+.5, z*1021+1.5 into 10-bit fields of n*0.5+0.5
    assert O.pack3sn(0.0, 0.0, 1.0) == 512 | (512 << 10) | (1022 << 20)
    assert O.pack3sn(-1.0, 0.0, 0.0) == 0 | (512 << 10) | (512 << 20)
    assert O.pack3sn(1.0, -1.0, -1.0) == 1023 | (0 << 10) | (1 << 20)


def test_unpack3sn_values():
    # floatpacking.glsl:46-66: a = f/1023, c = (f - 1.5)/1021, then *2 - 1
    u = 512 | (512 << 10) | (1022 << 20)
    v = O.unpack3sn(u)
    ex = f32(512) / f32(1023) * f32(2) - f32(1)
    ez = (f32(1022) - f32(1.5)) / f32(1021) * f32(2) - f32(1)
    assert bits(v[0]) == bits(ex) and bits(v[1]) == bits(ex) and bits(v[2]) == bits(ez)
    # z field 512 decodes to exactly 0 ((512-1.5)/1021 = 0.5)
    assert O.unpack3sn(512 << 20)[2] == 0.0


def test_pack_half2x16_round_to_nearest_even():
    assert O.pack_half2x16(1.0, -2.0) == 0x3C00 | (0xC000 << 16)
    assert O.pack_half2x16(1.0 + 2.0 ** -11, 0.0) & 0xFFFF == 0x3C00          # tie -> even
    assert O.pack_half2x16(1.0 + 3 * 2.0 ** -11, 0.0) & 0xFFFF == 0x3C02      # tie -> even
    assert O.pack_half2x16(2.0 ** -24, 0.0) & 0xFFFF == 0x0001                # smallest subnormal
    assert O.pack_half2x16(65520.0, 0.0) & 0xFFFF == 0x7C00                   # overflow -> inf
    rng = np.random.default_rng(3)
    for x in rng.normal(0, 30, 2000).astype(np.float32):
        assert O.pack_half2x16(float(x), 0.0) & 0xFFFF == int(np.float16(x).view(np.uint16))


# ---- ism_utils.glsl ---------------------------------------------------------------------------

def test_paraboloid_project_on_axis():
    # lookAtRH((0,0,1)) has rows s=(-1,0,0), u=(0,1,0), -f=(0,0,-1); a point 10 units along the
    # normal projects to the ISM centre with depth 10/zFar (sign preserved positive).
    v = O.paraboloid_project([0, 0, 10], 10.0, [0, 0, 1], 400.0, 5.0, 4, 4, True)
    assert v[0] == f32(0.375) and v[1] == f32(0.375)          # ((0+1)/2 + 1) / 4, tile (1,1) of 5
    assert bits(v[2]) == bits(f32(10) / f32(400))
    v = O.paraboloid_project([0, 0, 10], 10.0, [0, 0, 1], 400.0, 5.0, 4, 4, False)
    assert bits(v[2]) == bits(f32(10) / f32(400))


def test_paraboloid_project_45_degrees_and_rect_grid():
    k = f32(7.0)
    rel = np.array([k, 0, k], np.float32)
    d = np.sqrt(np.float32(k * k + k * k), dtype=np.float32)
    v = O.paraboloid_project(rel, float(d), [0, 0, 1], 400.0, 9.0, 8, 2, True)
    # x = -1/sqrt2 / (1 + 1/sqrt2) = 1 - sqrt2 ; tile of index 9 on an 8-wide grid is (1, 1)
    assert abs(float(v[0]) - ((1 - np.sqrt(2) + 1) / 2 + 1) / 8) < 2e-7
    assert abs(float(v[1]) - (0.5 + 1) / 2) < 2e-7


# ---- ism.comp -----------------------------------------------------------------------------------

def _point(pos, nrm, radius_unorm):
    n = (np.asarray(nrm, np.float64) * 0.5 + 0.5)
    b = [int(round(c * 255)) for c in n] + [radius_unorm]
    w = b[0] | (b[1] << 8) | (b[2] << 16) | (b[3] << 24)
    return np.array([pos[0], pos[1], pos[2], np.uint32(w).view(np.float32)], np.float32)


def test_splat_single_point_key():
    # One VPL at the origin facing +z; a point 10 units in front facing it.
    vpos = np.zeros((1, 3), np.float32)
    vpn = np.array([O.pack3sn(0.0, 0.0, 1.0)], np.uint32)
    n_unpacked = O.unpack3sn(int(vpn[0]))
    pts = np.stack([_point([0, 0, 10], [0, 0, -1], 51)])
    keys = O.ism_splat(pts, np.array([1], np.uint32), 1, vpos, vpn, 1, 8, 1, 1, 400.0)
    # ism.comp:121-136 (the VPL normal is the 10:10:10-decoded one, so the texel is near centre)
    v = O.paraboloid_project([0, 0, 10], 10.0, n_unpacked, 400.0, 0.0, 1, 1, True)
    depth_key = int(np.float32(v[2]) * np.float32(1 << 24))
    radius = np.float32(51) / np.float32(255) * np.float32(25)
    key = (depth_key << 8) | int(radius * np.float32(10) / np.float32(2))
    tx, ty = int(v[0] * f32(8)), int(v[1] * f32(8))
    assert keys[ty, tx] == key
    assert (keys != 0xFFFFFFFF).sum() == 1


def test_splat_two_sided_cull():
    vpos = np.zeros((1, 3), np.float32)
    vpn = np.array([O.pack3sn(0.0, 0.0, 1.0)], np.uint32)
    behind = _point([0, 0, -10], [0, 0, 1], 40)      # behind the VPL: dot(n_vpl, rel) < 0
    facing_away = _point([0, 0, 10], [0, 0, 1], 40)  # point normal faces away: dot(n_p, -rel) < 0
    keys = O.ism_splat(np.stack([behind, facing_away]), np.array([2], np.uint32), 2, vpos, vpn, 1, 8, 1, 1, 400.0)
    assert (keys == 0xFFFFFFFF).all()


def test_splat_keeps_first_four_of_sixteen():
    # 16 VPLs all facing +z at distinct x; one point sees all of them; only the first four (in the
    # bucket's cache order wg, wg+1, ...) receive it (ism.comp:93-107).
    n = 16
    vpos = np.zeros((n, 3), np.float32)
    vpos[:, 0] = np.arange(n, dtype=np.float32)
    vpn = np.full(n, O.pack3sn(0.0, 0.0, 1.0), np.uint32)
    pts = np.zeros((n, 4), np.float32)  # one bucket per VPL, stride 1; only bucket 0 holds a point
    pts[0] = _point([7.5, 0, 30], [0, 0, -1], 40)
    counts = np.zeros(n, np.uint32)
    counts[0] = 1
    keys = O.ism_splat(pts, counts, 1, vpos, vpn, n, 8, 4, 4, 400.0)
    hit_isms = sorted({(y // 8) * 4 + (x // 8) for y, x in zip(*np.nonzero(keys != 0xFFFFFFFF))})
    assert hit_isms == [0, 1, 2, 3]


# ---- pull.comp / push.comp ---------------------------------------------------------------------

EMPTY = 0xFFFFFFFF


def test_pull_treats_clear_value_as_far_valid_sample():
    # pull.comp:37-39: the clear key decodes to depth (2^24-1)/2^24 != 1.0, radius 25.5, so after
    # projection (radius / (d*zFar) / 3.14 * ismPixelSize * 1.3 = 1.69 px) it passes the level-1
    # radius test and counts as a *valid* far sample -- a reference quirk that the restatement
    # keeps. Four empty keys average to that depth and radius.
    keys = np.full((2, 2), EMPTY, np.uint32)
    out = O.pull_level(1, keys, None, 1, 1, 400.0, 64)
    d = f32(16777215) / f32(16777216)
    r = f32(255) / f32(10)
    r = r / (d * f32(400)) / f32(3.14) * f32(64)
    r = r * f32(1.3)
    assert out[0, 0, 0] == bits(d)
    assert out[0, 0, 2] == bits(r)


def test_pull_small_radius_sample_is_rejected():
    # A point at depth 0.25 with world radius 2 projects to 2/100/3.14*64*1.3 = 0.53 px, which fails
    # the level-1 radius test (dist = 0.354 > 0.53 * 2^-1); the three empty samples (1.69 px) pass,
    # so the output is their average depth (2^24-1)/2^24.
    keys = np.full((2, 2), EMPTY, np.uint32)
    keys[0, 0] = (4194304 << 8) | 20
    out = O.pull_level(1, keys, None, 1, 1, 400.0, 64)
    assert out[0, 0, 0] == bits(f32(16777215) / f32(16777216))
    # With 4-texel ISMs every projected radius is below 0.354*2 px: nothing is valid and the
    # texel gets the sentinel (1, 0, 0, 0) of pull.comp:121-123.
    out = O.pull_level(1, keys, None, 1, 1, 400.0, 4)
    assert list(out[0, 0]) == [bits(f32(1)), 0, 0, 0]


def test_pull_depth_range_rejects_far_samples():
    # Two near points with big radii and two empty texels: the empties' depth exceeds the
    # nearest sample's maxDepth (pull.comp:84-97), so only the near pair is averaged.
    keys = np.full((2, 2), EMPTY, np.uint32)
    keys[0, 0] = (4194304 << 8) | 200  # depth 0.25, radius 20
    keys[1, 1] = (4194304 << 8) | 200
    out = O.pull_level(1, keys, None, 1, 1, 400.0, 64)
    assert out[0, 0, 0] == bits(f32(0.25))
    max_depth = f32(0.25) + (f32(20) * f32(2)) / f32(400) * f32(0.6)
    assert out[0, 0, 1] == bits(max_depth)


def test_pull_all_invalid_writes_sentinel():
    inp = np.zeros((2, 2, 4), np.uint32)
    inp[..., 0] = bits(f32(1.0))  # depth 1.0 exactly is invalid at levels >= 2
    out = O.pull_level(2, None, inp, 1, 1, 400.0, 64)
    assert list(out[0, 0]) == [bits(f32(1)), 0, 0, 0]


def test_push_keeps_valid_unoccluded_sample_and_fills_occluded():
    # 4x4 level-0 keys of one 4x4 ISM; the coarse level (2x2) is uniformly depth 0.5 with a large
    # radius. Level-0 texel (1,1) holds a nearer point (kept: valid and not occluded); the empty
    # texels are "occluded" by the coarse maxDepth and get the weighted coarse depth 0.5.
    keys = np.full((4, 4), EMPTY, np.uint32)
    keys[1, 1] = (2097152 << 8) | 30  # depth 0.125
    coarse = np.zeros((2, 2, 4), np.uint32)
    coarse[..., 0] = bits(f32(0.5))
    coarse[..., 1] = bits(f32(0.6))
    coarse[..., 2] = bits(f32(10))
    _, fin = O.push_level(0, keys, None, coarse, 4, 4, 4)
    assert fin[1, 1] == f32(0.125)
    assert fin[0, 0] == f32(0.5) and fin[3, 3] == f32(0.5)


def test_push_zero_weight_across_ism_border():
    # Two 2x2 ISMs side by side at level 0; the right ISM's coarse texel is near, the left one far.
    # Texel (1,0) of the left ISM must not take weight from the right ISM (push.comp:77-86).
    keys = np.full((2, 4), EMPTY, np.uint32)
    coarse = np.zeros((1, 2, 4), np.uint32)
    coarse[0, 0, 0], coarse[0, 0, 1], coarse[0, 0, 2] = bits(f32(0.9)), bits(f32(0.95)), bits(f32(10))
    coarse[0, 1, 0], coarse[0, 1, 1], coarse[0, 1, 2] = bits(f32(0.1)), bits(f32(0.15)), bits(f32(10))
    _, fin = O.push_level(0, keys, None, coarse, 4, 2, 2)
    # each side is the weighted mean of its own coarse texel only (w*d/w, one FP32 rounding each)
    assert abs(float(fin[0, 1]) - 0.9) < 2e-7 and abs(float(fin[0, 2]) - 0.1) < 2e-7


# ---- final_gathering.comp ----------------------------------------------------------------------

def test_final_gather_single_pair():
    # One pixel, one VPL, no shadowing: acc = flux * min(cos*cos/d^4, clamp); out = acc*gi/N*I^2.
    depth = np.array([[0.5]], np.float32)
    inv_vp = np.eye(4, dtype=np.float32)  # world = ndc: pixel (0,0) -> (-1, -1, 0)
    nrm = np.array([[[1.0, 1.0]]], np.float32)  # octahedral (1,1) -> -z, facing the VPL
    vpos = np.array([[-1.0, -1.0, -4.0]], np.float32)
    vn = np.array([[0.0, 0.0, 1.0]], np.float32)
    vc = np.array([[1.0, 2.0, 3.0]], np.float32)
    atlas = np.ones((8, 8), np.float32)
    out = O.final_gather(depth, nrm, inv_vp, vpos, vn, vc, atlas, 8, 1, 1, 400.0, 3000.0, 1e6, 1, shadowing=0)
    g = 1.0 / 4.0 ** 4
    np.testing.assert_allclose(out[0, 0], np.array([1, 2, 3]) * g * 3000.0, rtol=1e-6)
    out = O.final_gather(depth, nrm, inv_vp, vpos, vn, vc, atlas, 8, 1, 1, 400.0, 3000.0, 1e-4, 1, shadowing=0)
    np.testing.assert_allclose(out[0, 0], np.array([1, 2, 3]) * 1e-4 * 3000.0, rtol=1e-6)  # clamped


def test_final_gather_occluded_pair_is_dark():
    depth = np.array([[0.5]], np.float32)
    inv_vp = np.eye(4, dtype=np.float32)
    nrm = np.array([[[1.0, 1.0]]], np.float32)
    vpos = np.array([[-1.0, -1.0, -4.0]], np.float32)
    vn = np.array([[0.0, 0.0, 1.0]], np.float32)
    vc = np.ones((1, 3), np.float32)
    occluder = np.zeros((8, 8), np.float32)  # occluder at depth 0: 1 - (4/400 - 0) = 0.99 -> half lit
    lit = O.final_gather(depth, nrm, inv_vp, vpos, vn, vc, np.ones((8, 8), np.float32), 8, 1, 1, 400.0, 1.0, 1e6, 1)
    dark = O.final_gather(depth, nrm, inv_vp, vpos, vn, vc, occluder, 8, 1, 1, 400.0, 1.0, 1e6, 1)
    t = (0.99 - 0.98) / 0.02
    np.testing.assert_allclose(dark[0, 0], lit[0, 0] * t * t * (3 - 2 * t), rtol=1e-4)
    far = np.full((8, 8), -1.0, np.float32)  # 1 - (0.01 + 1) < 0.98 -> fully shadowed
    assert (O.final_gather(depth, nrm, inv_vp, vpos, vn, vc, far, 8, 1, 1, 400.0, 1.0, 1e6, 1) == 0).all()


def test_fp32_and_fp64_oracles_agree_on_small_frame():
    import mlgi

    cfg = mlgi.C0
    sc = mlgi.make_scene(cfg)
    perm = mlgi.shuffle_table(cfg.n_vpl)
    pos, nrm, col, pn = O.vpl_process(sc.rsm_depth, sc.rsm_normal, sc.rsm_diffuse, cfg.n_vpl,
                                      sc.mat("inv_biased_light_vp"), cfg.light_intensity, 1, perm)
    keys = O.ism_splat(sc.points, sc.counts, sc.bucket_stride, pos, pn, cfg.n_vpl, cfg.ism_size, cfg.grid_x,
                       cfg.grid_y, cfg.z_far)
    fin = O.pullpush(keys, cfg.ism_size, cfg.levels, cfg.z_far)
    args = (fin, cfg.ism_size, cfg.grid_x, cfg.grid_y, cfg.z_far, cfg.gi_intensity, cfg.clamp_value, cfg.interleave)
    r32 = O.final_gather(sc.gbuf_depth, sc.gbuf_normal, sc.mat("inv_view_proj"), pos, nrm, col, *args)
    r64 = O.final_gather(sc.gbuf_depth, sc.gbuf_normal, sc.mat("inv_view_proj").astype(np.float64),
                         pos.astype(np.float64), nrm.astype(np.float64), col.astype(np.float64), *args,
                         dtype=np.float64)
    assert np.linalg.norm(r32 - r64) / np.linalg.norm(r64) < 1e-3
    # the threaded and single-threaded oracles are identical (order-independent atomicMin)
    keys1 = O.ism_splat(sc.points, sc.counts, sc.bucket_stride, pos, pn, cfg.n_vpl, cfg.ism_size, cfg.grid_x,
                        cfg.grid_y, cfg.z_far, threads=1)
    assert (keys1 == keys).all()
    assert (O.pullpush(keys, cfg.ism_size, cfg.levels, cfg.z_far, threads=1) == fin).all()


@pytest.mark.parametrize("n", [256, 1024])
def test_shuffle_table_is_a_permutation(n):
    import mlgi

    p = mlgi.shuffle_table(n)
    assert sorted(p.tolist()) == list(range(n))
    assert (p != np.arange(n)).mean() > 0.9
