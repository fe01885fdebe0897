"""Allocation failures, simulated with the library's allocation hook (mlgi_set_alloc_fault), are
reported as MLGI_ENOMEM at every allocation a context, a device frame, a host-buffer frame, a batch
and a server make. Nothing leaks, and a context that met a failure then renders the frame bit for
bit. No GPU fault is involved: a failing allocation is refused before CUDA is asked."""
import ctypes as C

import numpy as np
import pytest

import mlgi
from mlgi.device import DeviceFrame, host_frame_desc, pinned_inputs
from mlgi.serve import Server, request

pytestmark = pytest.mark.gpu

MiB = 1 << 20


@pytest.fixture(autouse=True)
def _hook_off():
    mlgi.lib().mlgi_set_alloc_fault(-1)
    yield
    mlgi.lib().mlgi_set_alloc_fault(-1)


def _create():
    h = C.c_void_p()
    st = mlgi.lib().mlgi_create(C.byref(h), C.byref(mlgi.CtxDesc(0, 0)))
    return st, h


def _free_bytes():
    import torch

    torch.cuda.synchronize()
    return torch.cuda.mem_get_info()[0]


def test_context_creation_fails_cleanly():
    L = mlgi.lib()
    for k in (0, 1):  # the status word, then its pinned host copy
        assert L.mlgi_set_alloc_fault(k) == mlgi.OK
        st, h = _create()
        assert st == mlgi.ENOMEM and not h.value
    assert L.mlgi_set_alloc_fault(-1) == mlgi.OK
    st, h = _create()
    assert st == mlgi.OK
    L.mlgi_destroy(h)
    assert L.mlgi_set_alloc_fault(-2) == mlgi.EINVAL


def _sweep(run, ref, check):
    """Fresh contexts whose allocations fail from the k-th on, for k = 0, 1, ...: each failing call
    returns ENOMEM, then the same context renders the frame once the hook is off. Returns the
    number of failure points met before a call went through."""
    L = mlgi.lib()
    failures = 0
    for k in range(64):
        L.mlgi_set_alloc_fault(k)
        st, h = _create()
        if st != mlgi.OK:
            L.mlgi_set_alloc_fault(-1)
            assert st == mlgi.ENOMEM
            failures += 1
            continue
        st = run(h)
        L.mlgi_set_alloc_fault(-1)
        if st == mlgi.OK:
            check(ref)
            L.mlgi_destroy(h)
            return failures
        assert st == mlgi.ENOMEM, (k, st, L.mlgi_last_error(h))
        failures += 1
        assert run(h) == mlgi.OK, L.mlgi_last_error(h)
        check(ref)
        L.mlgi_destroy(h)
    raise AssertionError("the call never went through")


def test_device_frame_allocations_fail_cleanly_and_leak_nothing():
    import torch

    cfg = mlgi.C1
    df = DeviceFrame(mlgi.make_scene(cfg))
    fd, out = df.frame_desc(), df.radiance()
    ctx = mlgi.Context(0)
    ctx.gi_frame(fd, out)
    torch.cuda.synchronize()
    ref = df.rgb_np().copy()
    ctx.close()
    assert np.abs(ref).max() > 0

    def run(h):
        df.rgb.zero_()
        torch.cuda.synchronize()
        return mlgi.lib().mlgi_gi_frame(h, C.byref(fd), C.byref(out), None)

    def check(r):
        torch.cuda.synchronize()
        assert (df.rgb_np() == r).all()

    free0 = _free_bytes()
    failures = _sweep(run, ref, check)
    assert failures >= 6  # two in the context, then the frame's shuffle table and buffers
    assert abs(_free_bytes() - free0) < 16 * MiB


def test_host_frame_allocations_fail_cleanly():
    import torch

    cfg = mlgi.C1
    sc = mlgi.make_scene(cfg)
    pinned = pinned_inputs(sc)
    fd = host_frame_desc(sc, pinned)
    ctx = mlgi.Context(0)
    rgb = pinned["rgb"]
    ctx.gi_frame_host(fd, rgb)
    ref = rgb.numpy().copy()
    ctx.close()

    def run(h):
        rgb.zero_()
        return mlgi.lib().mlgi_gi_frame_host(h, C.byref(fd), mlgi.ptr(rgb))

    def check(r):
        torch.cuda.synchronize()
        assert (rgb.numpy() == r).all()

    free0 = _free_bytes()
    failures = _sweep(run, ref, check)
    assert failures >= 10  # the staging buffers of the host inputs fail too
    assert abs(_free_bytes() - free0) < 16 * MiB


def test_batch_creation_fails_cleanly():
    L = mlgi.lib()
    ctx = mlgi.Context(0)
    frames = [DeviceFrame(mlgi.make_scene(c)) for c in (mlgi.C0, mlgi.C1)]
    descs = (mlgi.FrameDesc * 2)(*[f.frame_desc() for f in frames])
    outs = (mlgi.Radiance * 2)(*[f.radiance() for f in frames])
    failures = 0
    for k in range(32):
        L.mlgi_set_alloc_fault(k)
        b = C.c_void_p()
        st = L.mlgi_batch_create_ex(ctx.h, 2, C.cast(descs, C.c_void_p), C.cast(outs, C.c_void_p),
                                    C.byref(mlgi.BatchOpts(0, 0)), C.byref(b))
        L.mlgi_set_alloc_fault(-1)
        if st == mlgi.OK:
            assert L.mlgi_batch_launch(b, None) == mlgi.OK
            L.mlgi_batch_destroy(b)
            break
        assert st == mlgi.ENOMEM and not b.value
        failures += 1
    assert failures >= 4  # arena, host and device view tables, running counts
    ctx.check_device_status()
    ctx.close()


def test_server_creation_and_room_allocation_fail_cleanly():
    L = mlgi.lib()
    failures = 0
    for k in range(64):
        L.mlgi_set_alloc_fault(k)
        try:
            sv = Server(slots=1, max_width=640, max_height=360, hbm_budget=2 << 30)
        except mlgi.MlgiError as e:
            L.mlgi_set_alloc_fault(-1)
            assert e.status == mlgi.ENOMEM
            failures += 1
            continue
        L.mlgi_set_alloc_fault(-1)
        break
    assert failures >= 8  # the tuning context, then the slot's context, frame buffers and pinned word
    sv.prepare([request(640, 360, 256, 1 << 18)])
    # the room of the next request cannot be allocated: it completes with ENOMEM
    L.mlgi_set_alloc_fault(0)
    assert sv.submit(request(640, 360, 256, 1 << 18, room_seed=7, id=1)) == mlgi.OK
    sv.drain(60)
    (c,) = sv.poll()
    L.mlgi_set_alloc_fault(-1)
    assert int(c["id"]) == 1 and c["status"] == mlgi.ENOMEM
    # and the server goes on
    assert sv.submit(request(640, 360, 256, 1 << 18, room_seed=7, id=2)) == mlgi.OK
    sv.drain(60)
    (c,) = sv.poll()
    sv.close()
    assert int(c["id"]) == 2 and c["status"] == mlgi.OK
