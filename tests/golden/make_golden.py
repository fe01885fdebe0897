"""Regenerate the golden fixtures in tests/golden/.

    python tests/golden/make_golden.py

shuffle_1024.npy   the VPL shuffle table of VPLProcessor.cpp:58-65 (std::iota + std::shuffle with
                   std::mt19937(1979982), libstdc++), produced through mlgi_shuffle_table.
c0_golden.npz      the tiny C0 workload (160x96, 64 VPLs, 2^14 points, 32^2 ISMs on an 8x8 grid,
                   3 pull-push levels, I=4): scene checksums, and the FP32 oracle's VPL records,
                   ISM keys, pull-push atlas and gathered radiance, plus the FP64 oracle's radiance.
cref_ref.json      sha256 checksums of the reference's own shaders (oracle/_ref, the GLSL compiled
                   as C++) on the CREF workload (1024 VPLs, 2048^2 atlas of 64^2 ISMs, 6 levels,
                   I=4): the scene, the VPL records, ISM keys, pull-push atlas and gathered radiance
                   (512 VPLs, 32 per interleave class). A host without the reference sources checks
                   its oracle and GPU stages against these.
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "many-lights-gi_gb300")]

import mlgi  # noqa: E402
from oracle import oracle as O  # noqa: E402


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def compute(cfg):
    sc = mlgi.make_scene(cfg)
    perm = mlgi.shuffle_table(cfg.n_vpl)
    pos, nrm, col, pn = O.vpl_process(sc.rsm_depth, sc.rsm_normal, sc.rsm_diffuse, cfg.n_vpl,
                                      sc.mat("inv_biased_light_vp"), cfg.light_intensity, 1, perm)
    keys = O.ism_splat(sc.points, sc.counts, sc.bucket_stride, pos, pn, cfg.n_vpl, cfg.ism_size, cfg.grid_x,
                       cfg.grid_y, cfg.z_far)
    fin = O.pullpush(keys, cfg.ism_size, cfg.levels, cfg.z_far)
    args = (fin, cfg.ism_size, cfg.grid_x, cfg.grid_y, cfg.z_far, cfg.gi_intensity, cfg.clamp_value, cfg.interleave)
    rad = O.final_gather(sc.gbuf_depth, sc.gbuf_normal, sc.mat("inv_view_proj"), pos, nrm, col, *args)
    rad64 = O.final_gather(sc.gbuf_depth, sc.gbuf_normal, sc.mat("inv_view_proj").astype(np.float64),
                           pos.astype(np.float64), nrm.astype(np.float64), col.astype(np.float64), *args,
                           dtype=np.float64)
    scene_sha = sha(np.concatenate([sc.gbuf_depth.ravel().view(np.uint32), sc.gbuf_normal.ravel().view(np.uint32),
                                    sc.rsm_depth.ravel().view(np.uint32), sc.rsm_normal.ravel(),
                                    sc.rsm_diffuse.ravel(), sc.points.ravel().view(np.uint32), sc.counts]))
    return dict(scene_sha=np.array(scene_sha), perm=perm, vpl_pos=pos, vpl_nrm=nrm, vpl_col=col, vpl_pn=pn,
                keys=keys, atlas=fin, radiance=rad, radiance64=rad64.astype(np.float32))


def scene_sha(sc):
    return sha(np.concatenate([sc.gbuf_depth.ravel().view(np.uint32), sc.gbuf_normal.ravel().view(np.uint32),
                               sc.rsm_depth.ravel().view(np.uint32), sc.rsm_normal.ravel(), sc.rsm_diffuse.ravel(),
                               sc.points.ravel().view(np.uint32), sc.counts]))


def cref_reference_hashes():
    """Run the reference's shaders (oracle/_ref) on CREF; return the checksums of each stage."""
    from oracle import ref as R
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from test_ref_pin import octahedral_to_rgb

    cfg = mlgi.CREF
    sc = mlgi.make_scene(cfg)
    perm = mlgi.shuffle_table(cfg.n_vpl)
    rp, rn, rc, rpk = R.vpl_process(sc.rsm_depth, sc.rsm_normal, sc.rsm_diffuse, cfg.n_vpl,
                                    sc.mat("inv_biased_light_vp"), cfg.light_intensity, 1, perm)
    keys = R.ism_splat(sc.points, sc.counts, rpk, cfg.n_vpl, cfg.atlas_w, cfg.atlas_h, cfg.z_far)
    atlas = R.pullpush(keys, cfg.ism_size, cfg.levels, cfg.z_far)
    n = 512
    vpl9 = np.concatenate([rp, rn, rc], 1)
    rad = R.final_gather(sc.gbuf_depth, octahedral_to_rgb(sc.gbuf_normal), sc.mat("inv_view_proj"), sc.mat("proj"),
                         vpl9[:n], n, 0, n, atlas, cfg.z_far, cfg.z_near, cfg.gi_intensity, cfg.clamp_value, 32)
    return {"config": cfg.name, "scene": scene_sha(sc), "vpl_pos": sha(rp), "vpl_nrm": sha(rn), "vpl_col": sha(rc),
            "vpl_packed": sha(rpk), "keys": sha(keys), "atlas": sha(atlas), "radiance_512": sha(rad),
            "keys_filled_fraction": float((keys != 0xFFFFFFFF).mean())}


def main():
    import json

    os.makedirs(HERE, exist_ok=True)
    np.save(os.path.join(HERE, "shuffle_1024.npy"), mlgi.shuffle_table(1024))
    g = compute(mlgi.C0)
    np.savez_compressed(os.path.join(HERE, "c0_golden.npz"), **g)
    print("wrote", sorted(g))
    from oracle import ref as R
    if R.available():
        h = cref_reference_hashes()
        with open(os.path.join(HERE, "cref_ref.json"), "w") as f:
            json.dump(h, f, indent=1)
        print("wrote cref_ref.json")


if __name__ == "__main__":
    main()
