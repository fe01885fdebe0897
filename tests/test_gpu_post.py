"""After the gathering, on the GPU against the oracle: the R11G11B10F GI buffer format and the
fused bilateral blur on FP32 and on R11G11B10F buffers, bit-exact; the composite, whose powers are
the fast __powf, within 1e-5 of the image's largest value and RGBA8 codes equal or one apart."""
import numpy as np
import pytest

import mlgi
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = mlgi.Context(0)
    yield c
    c.close()


def dev(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t, dtype):
    return t.cpu().numpy().view(dtype)


@pytest.fixture(scope="module")
def c1_frame(ctx):
    """The C1 scene and its gathered radiance (device frame)."""
    import torch

    from mlgi.device import DeviceFrame

    sc = mlgi.make_scene(mlgi.C1)
    df = DeviceFrame(sc)
    ctx.gi_frame(df.frame_desc(), df.radiance())
    torch.cuda.synchronize()
    return sc, df


def test_pack_unpack_r11g11b10f_bit_exact(ctx):
    import torch

    rng = np.random.default_rng(3)
    vals = np.concatenate([rng.uniform(0, 8, 3000), rng.lognormal(0, 6, 3000), -rng.uniform(0, 1, 300),
                           np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 65024, 65535, 70000, 64512, 2 ** -20,
                                     2 ** -21, 1.5 * 2 ** -20, 2 ** -14, 1 + 2 ** -7, 1 + 3 * 2 ** -7, 1e-30, 3e38])])
    vals = np.resize(vals, (len(vals) // 3 + 1) * 3).astype(np.float32).reshape(-1, 3)
    n = len(vals)
    w = torch.zeros(n, dtype=torch.int32, device="cuda")
    ctx.pack_r11g11b10f(dev(vals), w, n)
    torch.cuda.synchronize()
    assert (host(w, np.uint32) == O.pack_r11g11b10f(vals)).all()
    codes = np.concatenate([np.arange(0x800, dtype=np.uint32), np.arange(0x800, dtype=np.uint32) << 11,
                            np.arange(0x400, dtype=np.uint32) << 22])
    back = torch.zeros(len(codes) * 3, dtype=torch.float32, device="cuda")
    ctx.unpack_r11g11b10f(dev(codes.view(np.int32)), back, len(codes))
    torch.cuda.synchronize()
    got, ref = host(back, np.uint32), O.unpack_r11g11b10f(codes).reshape(-1).view(np.uint32)
    nan = np.isnan(O.unpack_r11g11b10f(codes).reshape(-1))
    assert (got[~nan] == ref[~nan]).all() and np.isnan(back.cpu().numpy()[nan]).all()


@pytest.mark.parametrize("crop", [(360, 640), (357, 637), (41, 29)], ids=["c1", "ragged", "small"])
def test_blur_bit_exact_fp32_and_packed(ctx, c1_frame, crop):
    import torch

    sc, df = c1_frame
    h, w = crop
    depth = sc.gbuf_depth[:h, :w].copy()
    nrm = sc.gbuf_normal[:h, :w].copy()
    gi = df.rgb_np()[:h, :w].copy()
    a, b = mlgi.depth_terms(sc)
    g = mlgi.GBufferView(w, h, mlgi.ptr(dev_d := dev(depth)), mlgi.ptr(dev_n := dev(nrm)), mlgi.F32)
    out = torch.zeros(h * w * 3, dtype=torch.float32, device="cuda")
    ctx.gi_blur(g, dev_gi := dev(gi), out, a, b, mlgi.F32)
    torch.cuda.synchronize()
    ref = O.gi_blur(depth, nrm, gi, a, b)
    got = out.cpu().numpy().reshape(h, w, 3)
    assert (got.view(np.uint32) == ref.view(np.uint32)).all()
    assert np.abs(ref - gi).max() > 1e-3 * np.abs(ref).max()  # the filter did something
    # R11G11B10F buffers, as GIStage's
    words = torch.zeros(h * w, dtype=torch.int32, device="cuda")
    ctx.pack_r11g11b10f(dev_gi, words, h * w)
    out_w = torch.zeros(h * w, dtype=torch.int32, device="cuda")
    ctx.gi_blur(g, words, out_w, a, b, mlgi.R11G11B10F)
    torch.cuda.synchronize()
    ref_w = O.gi_blur(depth, nrm, O.pack_r11g11b10f(gi).reshape(h, w), a, b, packed=True)
    got_w = host(out_w, np.uint32).reshape(h, w)
    assert (got_w == ref_w).all()
    del dev_d, dev_n


def test_blur_rejects_bad_arguments(ctx, c1_frame):
    sc, df = c1_frame
    g = df.gbuffer_view()
    with pytest.raises(mlgi.MlgiError):
        ctx.gi_blur(g, df.rgb, df.rgb, 0.0, 0.0)  # in place
    with pytest.raises(mlgi.MlgiError):
        ctx.gi_blur(g, df.rgb, df.atlas, 0.0, 0.0, fmt=mlgi.F16)


@pytest.mark.parametrize("packed", [False, True], ids=["fp32_gi", "r11g11b10f_gi"])
def test_composite_matches_oracle(ctx, c1_frame, packed):
    import torch

    sc, df = c1_frame
    h, w = mlgi.C1.height, mlgi.C1.width
    gi = df.rgb_np()
    rng = np.random.default_rng(5)
    occ = rng.uniform(0.5, 1.0, (h, w)).astype(np.float32)
    direct = rng.uniform(0, 0.2, (h, w, 3)).astype(np.float32)
    if packed:
        gi_in = O.pack_r11g11b10f(gi).reshape(h, w)
        g_dev = dev(gi_in.view(np.int32))
    else:
        gi_in = gi
        g_dev = dev(gi)
    alb = dev(sc.gbuf_albedo.view(np.int32))
    out_f = torch.zeros(h * w * 3, dtype=torch.float32, device="cuda")
    out_8 = torch.zeros(h * w, dtype=torch.int32, device="cuda")
    fmt = mlgi.R11G11B10F if packed else mlgi.F32
    ctx.composite(g_dev, alb, out_f, w, h, 1.5, fmt, mlgi.F32, occlusion=dev(occ), direct=dev(direct))
    ctx.composite(g_dev, alb, out_8, w, h, 1.5, fmt, mlgi.RGBA8, occlusion=dev(occ), direct=dev(direct))
    torch.cuda.synchronize()
    ref_f, ref_8 = O.composite(gi_in, sc.gbuf_albedo, 1.5, occ, direct, packed=packed)
    got_f = out_f.cpu().numpy().reshape(h, w, 3)
    assert np.abs(got_f - ref_f).max() <= 1e-5 * max(1.0, np.abs(ref_f).max())
    got_8 = host(out_8, np.uint32).reshape(h, w)
    diff = np.abs(np.stack([(got_8 >> s) & 255 for s in (0, 8, 16)]).astype(int) -
                  np.stack([(ref_8 >> s) & 255 for s in (0, 8, 16)]).astype(int))
    assert diff.max() <= 1 and (diff == 0).mean() > 0.999
    assert ((got_8 >> 24) == 255).all()
