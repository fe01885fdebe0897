"""Locality of the ISM splat, which the overlapped host frame relies on when it pulls and pushes the
ISM rows a point range has completed: the keys of bucket b land only in the ISMs of VPLs
b..b+15 (mod N), in the ISMs next to those (rounding at a paraboloid's rim), or on texel (0, 0)
(a point on a VPL's position). Checked bucket by bucket with the oracle (the CPU restatement of
ism.comp) on the small workloads."""
import numpy as np
import pytest

import mlgi
from oracle import oracle as O


def _vpls(cfg, sc):
    perm = mlgi.shuffle_table(cfg.n_vpl) if cfg.shuffle else None
    return O.vpl_process(sc.rsm_depth, sc.rsm_normal, sc.rsm_diffuse, cfg.n_vpl, sc.mat("inv_biased_light_vp"),
                         cfg.light_intensity, int(cfg.shuffle), perm)


@pytest.mark.parametrize("cfg", [mlgi.C0, mlgi.C1], ids=lambda c: c.name)
def test_bucket_keys_stay_near_their_isms(cfg):
    sc = mlgi.make_scene(cfg)
    opos, _, _, opn = _vpls(cfg, sc)
    S, gx, gy, N = cfg.ism_size, cfg.grid_x, cfg.grid_y, cfg.n_vpl
    splatted = spilled = 0
    for b in range(N):
        counts = np.zeros_like(sc.counts)
        counts[b] = sc.counts[b]
        keys = O.ism_splat(sc.points, counts, sc.bucket_stride, opos, opn, N, S, gx, gy, cfg.z_far)
        ys, xs = np.nonzero(keys != 0xFFFFFFFF)
        splatted += len(ys)
        touched = set(zip((xs // S).tolist(), (ys // S).tolist()))
        own = {((b + i) % N % gx, (b + i) % N // gx) for i in range(16)}
        near = {(x + dx, y + dy) for x, y in own for dx in (-1, 0, 1) for dy in (-1, 0, 1)}
        stray = touched - near
        assert stray <= {(0, 0)}, (b, sorted(stray))
        if (0, 0) in stray:  # only texel (0, 0) of ISM 0
            assert all((x, y) == (0, 0) or (x // S, y // S) in near for x, y in zip(xs.tolist(), ys.tolist()))
        spilled += sum((x // S, y // S) not in own for x, y in zip(xs.tolist(), ys.tolist()))
    assert splatted > 0
    if cfg.n_vpl >= 256:  # rim rounding does put keys into neighbouring ISMs: the rule is needed
        assert spilled > 0
