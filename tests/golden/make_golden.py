"""Regenerate the golden fixtures in tests/golden/.

    python tests/golden/make_golden.py

shuffle_1024.npy   the VPL shuffle table of VPLProcessor.cpp:58-65 (std::iota + std::shuffle with
                   std::mt19937(1979982), libstdc++), produced through mlgi_shuffle_table.
c0_golden.npz      the tiny C0 workload (160x96, 64 VPLs, 2^14 points, 32^2 ISMs on an 8x8 grid,
                   3 pull-push levels, I=4): scene checksums, and the FP32 oracle's VPL records,
                   ISM keys, pull-push atlas and gathered radiance, plus the FP64 oracle's radiance.
                   When oracle/_ref (the reference shaders compiled as C++) is built, its outputs
                   for the same inputs are stored too and must equal the FP32 oracle's.
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


def main():
    os.makedirs(HERE, exist_ok=True)
    np.save(os.path.join(HERE, "shuffle_1024.npy"), mlgi.shuffle_table(1024))
    g = compute(mlgi.C0)
    np.savez_compressed(os.path.join(HERE, "c0_golden.npz"), **g)
    print("wrote", sorted(g))


if __name__ == "__main__":
    main()
