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
