"""The oracle and the scene fixture reproduce the committed golden vectors (tests/golden/),
on this machine and on the GPU host alike."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import make_golden  # noqa: E402
import mlgi  # noqa: E402

GOLDEN = os.path.join(HERE, "golden", "c0_golden.npz")


@pytest.fixture(scope="module")
def golden():
    return dict(np.load(GOLDEN))


@pytest.fixture(scope="module")
def fresh():
    return make_golden.compute(mlgi.C0)


def test_scene_fixture_matches_golden(golden, fresh):
    assert str(fresh["scene_sha"]) == str(golden["scene_sha"])


@pytest.mark.parametrize("key", ["perm", "vpl_pn", "vpl_pos", "vpl_nrm", "vpl_col", "keys", "atlas", "radiance"])
def test_oracle_fp32_matches_golden_bit_exact(golden, fresh, key):
    a, b = fresh[key], golden[key]
    assert a.shape == b.shape
    assert (a.view(np.uint8) == b.view(np.uint8)).all()


def test_oracle_fp64_matches_golden(golden, fresh):
    a, b = fresh["radiance64"], golden["radiance64"]
    assert np.linalg.norm(a - b) / np.linalg.norm(b) < 1e-6


@pytest.mark.gpu
def test_gpu_chain_matches_golden(golden):
    import torch

    from mlgi.device import DeviceFrame

    cfg = mlgi.C0
    ctx = mlgi.Context(0)
    df = DeviceFrame(mlgi.make_scene(cfg))
    ctx.vpl_process(df.rsm_view(), mlgi.vpl_params(cfg, df.scene), df.vpl_buf())
    ctx.ism_splat(df.points_view(), df.vpl_buf(), cfg.n_vpl, mlgi.ism_params(cfg), df.atlas_view())
    ctx.pullpush(df.atlas_view(), mlgi.ism_params(cfg))
    ctx.final_gather(df.gbuffer_view(), df.vpl_buf(), df.atlas_view(), df.fg(), df.radiance())
    torch.cuda.synchronize()
    pos, nrm, col, pn = df.vpl_records()
    assert (pn == golden["vpl_pn"]).all() and (pos == golden["vpl_pos"]).all()
    assert (df.keys_np() == golden["keys"]).all()
    assert (df.atlas_np().view(np.uint32) == golden["atlas"].view(np.uint32)).all()
    rad = df.rgb_np()
    assert np.linalg.norm(rad - golden["radiance64"]) / np.linalg.norm(golden["radiance64"]) < 1e-3
    ctx.close()


def _cref_oracle_outputs():
    import hashlib
    import json

    from oracle import oracle as O

    cfg = mlgi.CREF
    sc = mlgi.make_scene(cfg)
    perm = mlgi.shuffle_table(cfg.n_vpl)
    pos, nrm, col, pn = O.vpl_process(sc.rsm_depth, sc.rsm_normal, sc.rsm_diffuse, cfg.n_vpl,
                                      sc.mat("inv_biased_light_vp"), cfg.light_intensity, 1, perm)
    keys = O.ism_splat(sc.points, sc.counts, sc.bucket_stride, pos, pn, cfg.n_vpl, cfg.ism_size, cfg.grid_x,
                       cfg.grid_y, cfg.z_far)
    atlas = O.pullpush(keys, cfg.ism_size, cfg.levels, cfg.z_far)
    n = 512
    rad = O.final_gather(sc.gbuf_depth, sc.gbuf_normal, sc.mat("inv_view_proj"), pos[:n], nrm[:n], col[:n], atlas,
                         cfg.ism_size, cfg.grid_x, cfg.grid_y, cfg.z_far, cfg.gi_intensity, cfg.clamp_value,
                         cfg.interleave)
    sha = lambda a: hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()
    golden = json.load(open(os.path.join(HERE, "golden", "cref_ref.json")))
    return sc, golden, {"scene": make_golden.scene_sha(sc), "vpl_pos": sha(pos), "vpl_nrm": sha(nrm),
                        "vpl_col": sha(col), "keys": sha(keys), "atlas": sha(atlas), "radiance_512": sha(rad)}


def test_oracle_reproduces_reference_shader_checksums():
    """The reference's own shaders (compiled as C++ where its sources are) produced
    tests/golden/cref_ref.json; the restatement must reproduce every checksum on any host."""
    _, golden, got = _cref_oracle_outputs()
    for k, v in got.items():
        assert v == golden[k], k


@pytest.mark.gpu
def test_gpu_stages_reproduce_reference_shader_checksums():
    """VPL records, ISM keys and the pull-push atlas computed by the CUDA kernels on CREF equal,
    word for word, what the reference's own shaders produce (checksums in cref_ref.json)."""
    import hashlib
    import json

    import torch

    from mlgi.device import DeviceFrame

    sha = lambda a: hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()
    golden = json.load(open(os.path.join(HERE, "golden", "cref_ref.json")))
    cfg = mlgi.CREF
    sc = mlgi.make_scene(cfg)
    assert make_golden.scene_sha(sc) == golden["scene"]
    ctx = mlgi.Context(0)
    df = DeviceFrame(sc)
    ctx.vpl_process(df.rsm_view(), mlgi.vpl_params(cfg, sc), df.vpl_buf())
    ctx.ism_splat(df.points_view(), df.vpl_buf(), cfg.n_vpl, mlgi.ism_params(cfg), df.atlas_view())
    ctx.pullpush(df.atlas_view(), mlgi.ism_params(cfg))
    torch.cuda.synchronize()
    pos, nrm, col, _ = df.vpl_records()
    assert sha(pos) == golden["vpl_pos"] and sha(nrm) == golden["vpl_nrm"] and sha(col) == golden["vpl_col"]
    assert sha(df.keys_np()) == golden["keys"]
    assert sha(df.atlas_np()) == golden["atlas"]
    ctx.close()
