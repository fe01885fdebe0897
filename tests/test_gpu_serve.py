"""The request server (mlgi_server_*): every request's result is the same alone and in the mix,
equals the single-frame path on the same inputs, and matches the oracle; admission under the HBM
budget, cancellation and malformed requests."""
import numpy as np
import pytest

import mlgi
from mlgi.serve import Server, request, shape_set

pytestmark = pytest.mark.gpu

SMALL = [(640, 360), (854, 480)]


def small_shapes():
    return shape_set(resolutions=SMALL, vpls=(256, 512), points=(1 << 18, 1 << 19))


def requests(n, seed=0, rooms=3):
    rng = np.random.default_rng(seed)
    shapes = small_shapes()
    out = []
    for i in range(n):
        s = shapes[rng.integers(len(shapes))]
        out.append(request(s.width, s.height, s.n_vpl, s.n_points, bool(s.reduced), room_seed=100 + rng.integers(rooms),
                           light_yaw_deg=float(rng.uniform(-5, 5)), light_pitch_deg=float(rng.uniform(-5, 5)),
                           camera_orbit_deg=float(rng.uniform(-10, 10)), id=i))
    return out


def serve_all(sv, reqs):
    for r in reqs:
        assert sv.submit(r) == mlgi.OK
    sv.drain(120)
    c = sv.poll()
    assert len(c) == len(reqs)
    return {int(x["id"]): x for x in c}


def serve_one_by_one(sv, reqs):
    res = {}
    for r in reqs:
        assert sv.submit(r) == mlgi.OK
        sv.drain(60)
        (x,) = sv.poll()
        res[int(x["id"])] = x
    return res


def test_results_are_the_same_alone_and_in_the_mix():
    reqs = requests(40)
    mix = Server(slots=6, max_width=854, max_height=480, hbm_budget=8 << 30)
    mix.prepare(small_shapes())
    a = serve_all(mix, reqs)
    st = mix.stats()
    mix.close()
    alone = Server(slots=1, max_width=854, max_height=480, hbm_budget=8 << 30)
    alone.prepare(small_shapes())
    b = serve_one_by_one(alone, reqs)
    alone.close()
    assert all(a[i]["status"] == mlgi.OK for i in a)
    assert all(a[i]["digest"] == b[i]["digest"] and a[i]["sum"] == b[i]["sum"] for i in a)
    # different poses give different frames
    assert len({int(a[i]["digest"]) for i in a}) == len(reqs)
    assert st["rooms_resident"] <= 3 * 2 * 2 and st["admitted"] == len(reqs)


def test_served_frame_equals_the_single_frame_path_and_the_oracle():
    """One FP32 request through the server, copied out, against DeviceFrame + mlgi_gi_frame on the
    same device-generated inputs with the same autotuned configuration (bit-exact), and against the
    FP64 oracle on those inputs (relative L2 <= 1e-3)."""
    import torch

    from mlgi.device import DeviceFrame
    from oracle import oracle as O

    W, H, N, P = 640, 360, 256, 1 << 18
    out = np.zeros(W * H * 3, np.float32)
    sv = Server(slots=2, max_width=W, max_height=H, hbm_budget=4 << 30)
    sv.prepare([request(W, H, N, P)])
    r = request(W, H, N, P, room_seed=7, light_yaw_deg=3.0, light_pitch_deg=-2.0, camera_orbit_deg=4.5, id=1,
                out_host=out)
    assert sv.submit(r) == mlgi.OK
    sv.drain(60)
    (c,) = sv.poll()
    sv.close()
    assert c["status"] == mlgi.OK
    # the digest is that of the copied radiance
    bits = out.view(np.uint32).astype(np.uint64)
    i = np.arange(1, out.size + 1, dtype=np.uint64)
    with np.errstate(over="ignore"):
        x = bits + np.uint64(0x9E3779B97F4A7C15) * i
        x = (x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        x = (x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        x = x ^ (x >> np.uint64(31))
        digest = int(np.sum(x, dtype=np.uint64))
    assert digest == int(c["digest"])

    ctx = mlgi.Context(0)
    tu = ctx.autotune(W, H, N, P)  # the server's query: 16 VPLs/pixel floor, 64^2 ISM floor, seed 1
    cfg = mlgi.Config("served", W, H, 512, N, P, tu.ism_size, tu.grid_x, tu.grid_y, tu.levels, tu.interleave, 16, 8,
                      tile=tu.tile, cull=1, seed=7, light_yaw_deg=3.0, light_pitch_deg=-2.0, camera_orbit_deg=4.5)
    df = DeviceFrame.generated(cfg)
    ctx.gi_frame(df.frame_desc(), df.radiance())
    torch.cuda.synchronize()
    rgb = df.rgb_np()
    assert (rgb.reshape(-1).view(np.uint32) == out.view(np.uint32)).all()

    sc = df.scene
    rd = df.rsm_depth.cpu().numpy().reshape(512, 512)
    rn = df.rsm_normal.cpu().numpy().view(np.uint32).reshape(512, 512)
    rf = df.rsm_diffuse.cpu().numpy().view(np.uint32).reshape(512, 512)
    gd = df.gbuf_depth.cpu().numpy().reshape(H, W)
    gn = df.gbuf_normal.cpu().numpy().reshape(H, W, 2)
    pts = df.points.cpu().numpy().reshape(-1, 4)
    counts = df.counts.cpu().numpy().view(np.uint32)
    perm = mlgi.shuffle_table(N)
    pos, nrm, col, pn = O.vpl_process(rd, rn, rf, N, sc.mat("inv_biased_light_vp"), cfg.light_intensity, 1, perm)
    keys = O.ism_splat(pts, counts, sc.bucket_stride, pos, pn, N, cfg.ism_size, cfg.grid_x, cfg.grid_y, cfg.z_far)
    assert (keys != 0xFFFFFFFF).mean() > 0.05
    fin = O.pullpush(keys, cfg.ism_size, cfg.levels, cfg.z_far)
    ref = O.final_gather(gd, gn, sc.mat("inv_view_proj").astype(np.float64), pos.astype(np.float64),
                         nrm.astype(np.float64), col.astype(np.float64), fin, cfg.ism_size, cfg.grid_x, cfg.grid_y,
                         cfg.z_far, cfg.gi_intensity, cfg.clamp_value, cfg.interleave, dtype=np.float64)
    assert np.linalg.norm(rgb - ref) / np.linalg.norm(ref) < 1e-3
    ctx.close()


def test_admission_under_a_small_budget_evicts_rooms_and_keeps_results():
    reqs = requests(24, seed=3, rooms=4)
    room_bytes = max(r.n_vpl * -(-r.n_points // r.n_vpl) * 16 + r.n_vpl * 4 for r in reqs)
    big = Server(slots=2, max_width=854, max_height=480, hbm_budget=8 << 30)
    big.prepare(small_shapes())
    a = serve_all(big, reqs)
    slot_bytes = big.stats()["slot_bytes"]
    big.close()
    # room for the slots and two rooms: later rooms evict earlier ones
    tight = Server(slots=2, max_width=854, max_height=480, hbm_budget=slot_bytes + 2 * room_bytes + (1 << 20))
    tight.prepare(small_shapes())
    b = serve_all(tight, reqs)
    st = tight.stats()
    tight.close()
    assert st["evictions"] > 0 and st["room_bytes"] + st["slot_bytes"] <= slot_bytes + 2 * room_bytes + (1 << 20)
    assert all(b[i]["status"] == mlgi.OK and b[i]["digest"] == a[i]["digest"] for i in a)
    # a room that cannot fit even in an empty server completes with ENOMEM
    tiny = Server(slots=1, max_width=854, max_height=480, hbm_budget=64 << 20)
    tiny.prepare([request(640, 360, 256, 1 << 18)])
    c = serve_all(tiny, [request(640, 360, 256, 1 << 22, id=5)])
    tiny.close()
    assert c[5]["status"] == mlgi.ENOMEM


def test_cancel_and_malformed_requests():
    sv = Server(slots=1, max_width=854, max_height=480, hbm_budget=8 << 30)
    sv.prepare(small_shapes())
    assert sv.submit(request(640, 360, 100, 1 << 18)) == mlgi.EINVAL  # VPL count not a multiple of 64
    reqs = requests(12, seed=9)
    for r in reqs:
        assert sv.submit(r) == mlgi.OK
    cancelled = sv.cancel(11)
    assert sv.submit(request(1920, 1080, 256, 1 << 18, id=99)) == mlgi.OK  # larger than the server's frames
    sv.drain(60)
    c = {int(x["id"]): x for x in sv.poll()}
    sv.close()
    assert c[99]["status"] == mlgi.EINVAL
    if cancelled == mlgi.OK:
        assert c[11]["status"] == mlgi.ECANCELED
    assert all(c[i]["status"] == mlgi.OK for i in range(11))


def test_poisson_served_and_plain_runs_agree_per_request():
    shapes = small_shapes()
    sv = Server(slots=4, max_width=854, max_height=480, hbm_budget=8 << 30)
    sv.prepare(shapes)
    served, wall_s = sv.run_poisson(shapes, rate_hz=400, duration_s=0.5, seed=11, n_rooms=3)
    plain, wall_p = sv.run_poisson(shapes, rate_hz=400, duration_s=0.5, seed=11, n_rooms=3, plain=True)
    sv.close()
    assert len(served) == len(plain) > 100
    a = {int(x["id"]): x for x in served}
    b = {int(x["id"]): x for x in plain}
    assert a.keys() == b.keys()
    assert all(a[i]["status"] == mlgi.OK and a[i]["digest"] == b[i]["digest"] for i in a)
    assert (served["latency_ms"] > 0).all() and (plain["latency_ms"] > 0).all()
