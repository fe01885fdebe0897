"""Known answers of the oracle's post-gathering restatements: the R11G11B10F format of the GI
buffers (GIStage.cpp:470), the bilateral blur (gi_blur.frag) and the composite
(deferredshading.frag). CPU only."""
import numpy as np

from oracle import oracle as O


def words(rgb):
    return O.pack_r11g11b10f(np.asarray(rgb, np.float32).reshape(-1, 3))


def test_r11g11b10f_known_words():
    one = (15 << 6) | ((15 << 6) << 11) | ((15 << 5) << 22)
    assert words([1, 1, 1])[0] == one
    assert words([65024, 65024, 64512])[0] == 0x7BF | (0x7BF << 11) | (0x3DF << 22)  # largest finite
    assert words([1e9, 1e30, 70000])[0] == 0x7BF | (0x7BF << 11) | (0x3DF << 22)  # saturates
    assert words([np.inf, 0, 0])[0] == 0x7C0
    assert words([np.nan, 0, 0])[0] == 0x7E0
    assert words([-1, -0.0, -np.inf])[0] == 0
    # ties round to even: 1 + 2^-7 is halfway between mantissas 0 and 1 (6 bits) -> 0
    assert words([1 + 2 ** -7, 1 + 3 * 2 ** -7, 1 + 2 ** -6])[0] & 0x7FF == 15 << 6
    assert (words([0, 1 + 3 * 2 ** -7, 0])[0] >> 11) & 0x7FF == (15 << 6) | 2
    # denormals: the unit of an 11-bit channel is 2^-20, of the 10-bit one 2^-19
    assert words([2.0 ** -20, 0, 2.0 ** -19])[0] == 1 | (1 << 22)
    assert words([2.0 ** -21, 1.5 * 2.0 ** -20, 0])[0] == (2 << 11)  # 0.5 -> 0 (even), 1.5 -> 2 (even)


def test_r11g11b10f_every_code_round_trips():
    r = np.arange(0x7C0, dtype=np.uint32)  # all finite 11-bit codes
    b = np.arange(0x3E0, dtype=np.uint32)  # all finite 10-bit codes
    w = np.concatenate([r, r << 11, b << 22])
    vals = O.unpack_r11g11b10f(w)
    assert (O.pack_r11g11b10f(vals) == w).all()
    # monotone, exact powers of two at the normal codes
    assert (np.diff(vals[: len(r), 0]) > 0).all()
    assert vals[15 << 6, 0] == 1.0 and vals[1 << 6, 0] == 2.0 ** -14


def flat_scene(h=16, w=20, depth=0.5):
    d = np.full((h, w), depth, np.float32)
    n = np.zeros((h, w, 2), np.float32)  # octahedral (0, 0) = +z
    return d, n


def test_blur_of_flat_surface_spreads_with_the_tent_weights():
    d, n = flat_scene()
    gi = np.zeros((16, 20, 3), np.float32)
    gi[6, 10] = 1.0  # three pixels or more from every border
    out = O.gi_blur(d, n, gi, proj_a=-1.0, proj_b=-2.0)
    # X then Y: weights 1, .75, .5, .25 on each axis (sum 4) -> separable tent / 16
    t = np.array([0.25, 0.5, 0.75, 1.0, 0.75, 0.5, 0.25], np.float64) / 4.0
    ref = np.outer(t, t)
    got = out[3:10, 7:14, 0].astype(np.float64)
    assert np.abs(got - ref).max() < 1e-6
    assert np.abs(out.sum() / 3 - 1.0) < 1e-5


def test_blur_stops_at_depth_and_normal_edges():
    d, n = flat_scene()
    d[:, 10:] = 0.9  # linear depth jumps by far more than 1 unit
    gi = np.zeros((16, 20, 3), np.float32)
    gi[:, :10] = 1.0
    out = O.gi_blur(d, n, gi, proj_a=-1.0, proj_b=-2.0)
    assert (out[:, 10:] == 0).all() and np.allclose(out[:, :10], 1.0, atol=1e-6)
    d, n = flat_scene()
    n[:, 10:] = [1.0, 0.0]  # +x: dot with +z is 0, weight (4-i)/4 - 25 < 0
    out = O.gi_blur(d, n, gi, proj_a=-1.0, proj_b=-2.0)
    assert (out[:, 10:] == 0).all()


def test_packed_blur_rounds_every_buffer():
    rng = np.random.default_rng(1)
    d, n = flat_scene()
    gi = rng.uniform(0, 4, (16, 20, 3)).astype(np.float32)
    w = O.pack_r11g11b10f(gi).reshape(16, 20)
    out = O.gi_blur(d, n, w, -1.0, -2.0, packed=True)
    f = O.gi_blur(d, n, O.unpack_r11g11b10f(w).reshape(16, 20, 3), -1.0, -2.0)
    back = O.unpack_r11g11b10f(out).reshape(16, 20, 3)
    assert np.abs(back - f).max() / 4.0 < 2 ** -5  # within the format's rounding of both passes


def test_composite_known_values():
    albedo = np.full((2, 2), 0xFFFFFFFF, np.uint32)  # white: toLinear(1) = 1
    gi = np.full((2, 2, 3), 1.0, np.float32)
    rgb, words8 = O.composite(gi, albedo, exposure=1.0)
    assert np.allclose(rgb, 0.5 ** (1 / 2.2), rtol=1e-6)  # Reinhard 1 -> 0.5, then gamma
    assert (words8 == (0xFF000000 | (186 << 16) | (186 << 8) | 186)).all()  # round(0.7297 * 255)
    rgb0, _ = O.composite(np.zeros_like(gi), albedo, 1.0)
    assert (rgb0 == 0).all()
    rgbd, _ = O.composite(np.zeros_like(gi), albedo, 1.0, occlusion=np.zeros((2, 2)), direct=np.ones((2, 2, 3)))
    assert np.allclose(rgbd, rgb)
