"""CPU-side checks of the C ABI: the library loads, exports every declared symbol, and the host
entry points (scene fixture, shuffle table, host sizes, status strings) behave."""
import ctypes as C
import os
import re

import numpy as np

import mlgi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    src = open(os.path.join(ROOT, "include", "mlgi.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(mlgi_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    lib = mlgi.lib()
    names = header_functions()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert sorted(mlgi.declared_symbols()) == names


# ctypes mirror of every struct in include/mlgi.h
STRUCTS = {"mlgi_ctx_desc": "CtxDesc", "mlgi_rsm_view": "RsmView", "mlgi_vpl_params": "VplParams",
           "mlgi_vpl_buf": "VplBuf", "mlgi_points": "Points", "mlgi_ism_params": "IsmParams", "mlgi_atlas": "Atlas",
           "mlgi_gbuffer_view": "GBufferView", "mlgi_fg_params": "FgParams", "mlgi_radiance": "Radiance",
           "mlgi_frame_desc": "FrameDesc", "mlgi_autotune_query": "AutotuneQuery",
           "mlgi_autotune_result": "AutotuneResult", "mlgi_frame_host_sizes": "FrameHostSizes",
           "mlgi_scene_desc": "SceneDesc", "mlgi_scene_info": "SceneInfo", "mlgi_server_desc": "ServerDesc",
           "mlgi_request": "Request", "mlgi_completion": "Completion", "mlgi_server_stats": "ServerStats",
           "mlgi_poisson_desc": "PoissonDesc", "mlgi_batch_opts": "BatchOpts", "mlgi_blur_params": "BlurParams",
           "mlgi_composite_params": "CompositeParams", "mlgi_cluster_params": "ClusterParams"}


def test_struct_layouts_match_the_header(tmp_path):
    """sizeof of every header struct (from the C compiler) equals its ctypes mirror's size."""
    import subprocess

    src = open(os.path.join(ROOT, "include", "mlgi.h")).read()
    declared = set(re.findall(r"\}\s*(mlgi_[a-z0-9_]+)\s*;", src))
    assert declared == set(STRUCTS), declared ^ set(STRUCTS)
    prog = tmp_path / "sizes.c"
    prog.write_text('#include <stdio.h>\n#include "mlgi.h"\nint main(void){\n' +
                    "".join(f'printf("{k} %zu\\n", sizeof({k}));\n' for k in STRUCTS) + "return 0;}\n")
    exe = tmp_path / "sizes"
    subprocess.run(["gcc", "-std=c99", f"-I{os.path.join(ROOT, 'include')}", str(prog), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    sizes = dict(zip(out[0::2], map(int, out[1::2])))
    for k, py in STRUCTS.items():
        assert C.sizeof(getattr(mlgi, py)) == sizes[k], (k, C.sizeof(getattr(mlgi, py)), sizes[k])


def test_status_strings():
    L = mlgi.lib()
    assert L.mlgi_status_string(mlgi.OK) == b"ok"
    assert L.mlgi_status_string(mlgi.ETIMEDOUT) == b"device wait timed out"
    assert L.mlgi_status_string(mlgi.EBOUNDS) == b"index out of bounds"


def test_checked_library_exports_every_declared_symbol_and_says_it_checks():
    normal = mlgi.load(mlgi.LIB_PATH_NORMAL)
    checked = mlgi.load(mlgi.LIB_PATH_CHECKED)
    missing = [n for n in header_functions() if not hasattr(checked, n)]
    assert not missing, missing
    assert normal.mlgi_checks_enabled() == 0 and checked.mlgi_checks_enabled() == 1


def test_allocation_hook_arguments():
    L = mlgi.lib()
    assert L.mlgi_set_alloc_fault(-2) == mlgi.EINVAL
    assert L.mlgi_set_alloc_fault(3) == mlgi.OK
    assert L.mlgi_set_alloc_fault(-1) == mlgi.OK


def test_null_context_is_rejected():
    L = mlgi.lib()
    assert L.mlgi_vpl_process(None, None, None, None, None) == mlgi.EINVAL
    assert L.mlgi_gi_frame(None, None, None, None) == mlgi.EINVAL


def test_shuffle_table_matches_std_shuffle_prefix():
    # VPLProcessor.cpp:58-65 with libstdc++: pinned prefix of the 1024-entry permutation.
    p = mlgi.shuffle_table(1024)
    assert sorted(p.tolist()) == list(range(1024))
    golden = np.load(os.path.join(ROOT, "tests", "golden", "shuffle_1024.npy"))
    assert (p == golden).all()


def test_scene_is_deterministic_and_well_formed():
    cfg = mlgi.C0
    a = mlgi.make_scene(cfg)
    b = mlgi.make_scene(cfg)
    for k in ("gbuf_depth", "gbuf_normal", "rsm_depth", "rsm_normal", "rsm_diffuse", "points", "counts"):
        assert (getattr(a, k) == getattr(b, k)).all(), k
    assert a.counts.sum() == cfg.n_points
    assert (a.gbuf_depth > 0).all() and (a.gbuf_depth <= 1).all()
    assert np.abs(a.gbuf_normal).max() <= 1.0
    # points inside the room, radius byte as packed from the area per point
    p = a.points[: a.counts[0]]
    assert (p[:, :3] >= -1e-3).all() and (p[:, :3] <= 100 + 1e-3).all()
    rbyte = p[:, 3].view(np.uint32) >> 24
    r = np.sqrt(a.info.total_area / (cfg.n_points * np.pi)) * np.sqrt(cfg.n_vpl)
    assert (rbyte == round(r / 25 * 255)).all()
    c = mlgi.make_scene(cfg.replace(seed=2))
    assert not (c.gbuf_depth == a.gbuf_depth).all()


def test_frame_host_sizes():
    cfg = mlgi.C1
    sc = mlgi.make_scene(cfg, points=False)
    fd = mlgi.FrameDesc()
    fd.rsm.width = fd.rsm.height = cfg.rsm
    fd.points.n_buckets = cfg.n_vpl
    fd.points.bucket_stride = sc.bucket_stride
    fd.gbuffer.width, fd.gbuffer.height = cfg.width, cfg.height
    z = mlgi.FrameHostSizes()
    assert mlgi.lib().mlgi_frame_host_sizes_get(C.byref(fd), C.byref(z)) == mlgi.OK
    assert z.points == cfg.n_vpl * sc.bucket_stride * 16
    assert z.radiance == cfg.width * cfg.height * 12
    assert z.gbuf_normal == cfg.width * cfg.height * 8


def test_pullpush_form_selection():
    """mlgi_pullpush_launches: one launch (each ISM's pyramid in one block) while the ISMs make at most
    one wave of such blocks (152 SMs here, the GB300's count, as no GPU answers: three blocks a SM for
    ISM edges up to 64, else two) and the far plane lies in [2^-20, 2^20]; else the per-level
    launches, four per sequence (two for a single level), in two halves of the ISM rows."""
    cases = [(mlgi.C0, 1), (mlgi.C1, 1), (mlgi.C2, 8), (mlgi.CREF, 8), (mlgi.C3B, 8),
             (mlgi.C2.replace(z_far=3.0e6, name="c2_far"), 8), (mlgi.C1.replace(z_far=1.0e-7, name="c1_near"), 8),
             (mlgi.C1.replace(levels=1, name="c1_one_level"), 4)]
    for cfg, launches in cases:
        assert mlgi.pullpush_launches(cfg) == launches, cfg.name
