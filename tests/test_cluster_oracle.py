"""Known answers of the oracle's reference-style clustered culling (clustering.comp,
light_lists.comp). CPU only."""
import numpy as np

import mlgi
from oracle import oracle as O


def test_slices_and_masks_of_an_identity_camera():
    # inv_vp = identity: a corner (u, v, z_b) maps to world (2u-1, 2v-1, 2z_b-1); A, B of a GL
    # projection with near 1 and far 100
    n, f = 1.0, 100.0
    A, B = -(f + n) / (f - n), -2 * f * n / (f - n)
    h, w = 130, 260  # 3 x 2 tiles, the last ones partial
    z_b = np.full((h, w), 0.5, np.float32)
    z_b[:, 128:] = 0.999  # far
    used, masks, sl = O.cluster_lights(z_b, np.eye(4, dtype=np.float32).T.reshape(16), A, B, f,
                                       np.zeros((64, 3), np.float32), np.zeros(64, np.uint32), 64)
    lin = -B / (A + (2 * 0.5 - 1))
    s_near = int(max(np.log2(-lin) * 19 / np.log2(f) - 3, 0))
    assert (sl[:, :128] == s_near).all()
    assert (sl[:, 128:] == min(int(max(np.log2(-(-B / (A + (2 * 0.999 - 1)))) * 19 / np.log2(f) - 3, 0)), 15)).all()
    assert used[0] == 1 << s_near and used[3] == 1 << s_near  # tiles (0,0) and (0,1)
    assert bin(int(used[1])).count("1") == 1 and used[1] == used[2]
    # 64 VPLs on the z axis with normals -z (even) and +z (odd): with the identity matrix a corner's
    # world z is 2 * logDepth(sliceZ) - 1, so the keep rule dot(corner - p, n) >= 0 is a z comparison
    vz = np.linspace(-2, 2, 64).astype(np.float32)
    pos = np.stack([np.zeros(64), np.zeros(64), vz], -1).astype(np.float32)
    pn = np.array([mlgi_pack(0.0, 0.0, -1.0 if i % 2 == 0 else 1.0) for i in range(64)], np.uint32)
    used, masks, sl = O.cluster_lights(z_b, np.eye(4, dtype=np.float32).T.reshape(16), A, B, f, pos, pn, 64)
    scale = 19 / np.log2(f)

    def corner_z(slice_):
        z = 0.05 if slice_ == 0 else -2 ** ((slice_ + 3) / scale)
        return 2 * (((1 / z * -B) - A + 1) / 2) - 1

    rows = masks.reshape(-1, 16, 2)
    checked = 0
    for t in range(6):
        for s_ in range(16):
            if not (used[t] >> s_) & 1:
                continue
            zs = [corner_z(s_), corner_z(s_ + 1)]
            for i in range(64):
                keep = max(zs) >= vz[i] if i % 2 else min(zs) <= vz[i]
                assert bool((rows[t, s_, i // 32] >> (i % 32)) & 1) == keep, (t, s_, i)
                checked += 1
    assert checked == 64 * sum(bin(int(u)).count("1") for u in used)


def mlgi_pack(x, y, z):
    return O.pack3sn(x, y, z)


def test_clustered_gather_stays_close_to_the_unculled_one():
    cfg = mlgi.C0
    sc = mlgi.make_scene(cfg)
    perm = mlgi.shuffle_table(cfg.n_vpl)
    pos, nrm, col, pn = O.vpl_process(sc.rsm_depth, sc.rsm_normal, sc.rsm_diffuse, cfg.n_vpl,
                                      sc.mat("inv_biased_light_vp"), cfg.light_intensity, 1, perm)
    keys = O.ism_splat(sc.points, sc.counts, sc.bucket_stride, pos, pn, cfg.n_vpl, cfg.ism_size, cfg.grid_x,
                       cfg.grid_y, cfg.z_far)
    atlas = O.pullpush(keys, cfg.ism_size, cfg.levels, cfg.z_far)
    a, b = mlgi.depth_terms(sc)
    used, masks, sl = O.cluster_lights(sc.gbuf_depth, sc.mat("inv_view_proj"), a, b, cfg.z_far, pos, pn, cfg.n_vpl)
    args = (sc.gbuf_depth, sc.gbuf_normal, sc.mat("inv_view_proj").astype(np.float64), pos, nrm, col, atlas,
            cfg.ism_size, cfg.grid_x, cfg.grid_y, cfg.z_far, cfg.gi_intensity, cfg.clamp_value, cfg.interleave)
    full = O.final_gather(*args, dtype=np.float64)
    clu = O.final_gather_clustered(*args, masks, sl)
    assert (masks != 0).any() and np.abs(clu).max() > 0
    assert np.linalg.norm(clu - full) / np.linalg.norm(full) < 0.05
