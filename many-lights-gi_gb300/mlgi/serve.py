"""Python handle of the request server (mlgi_server_* in include/mlgi.h).

The scheduler, slots, room cache and load generator are native (host/serve.cpp); this class only
marshals requests and completions.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import OK, Completion, MlgiError, PoissonDesc, Request, ServerDesc, ServerStats, lib, ptr

COMPLETION_DTYPE = np.dtype([("id", np.uint64), ("status", np.int32), ("latency_ms", np.float64),
                             ("queue_ms", np.float64), ("digest", np.uint64), ("sum", np.float64)], align=True)
assert COMPLETION_DTYPE.itemsize == C.sizeof(Completion)


def request(width, height, n_vpl, n_points, reduced=False, room_seed=1, light_yaw_deg=0.0, light_pitch_deg=0.0,
            camera_orbit_deg=0.0, id=0, out_host: np.ndarray | None = None) -> Request:
    return Request(id, room_seed, width, height, n_vpl, n_points, int(reduced), light_yaw_deg, light_pitch_deg,
                   camera_orbit_deg, 0.0, ptr(out_host) if out_host is not None else None)


def shape_set(resolutions=((854, 480), (1280, 720), (1920, 1080), (2560, 1440)), vpls=(256, 512, 1024, 2048, 4096),
              points=(1 << 20, 1 << 21, 1 << 22, 1 << 23), precisions=(False, True)) -> list[Request]:
    """Every combination of the given frame sizes, VPL counts, point counts and precisions."""
    return [request(w, h, n, p, r) for (w, h) in resolutions for n in vpls for p in points for r in precisions]


class Server:
    def __init__(self, slots=8, max_width=2560, max_height=1440, rsm_size=512, hbm_budget=150 << 30, device=0):
        self.h = C.c_void_p()
        d = ServerDesc(device, slots, max_width, max_height, rsm_size, hbm_budget)
        st = lib().mlgi_server_create(C.byref(d), C.byref(self.h))
        if st != OK:
            raise MlgiError(st, "mlgi_server_create failed")

    def _chk(self, st, what):
        if st != OK:
            raise MlgiError(st, what)
        return st

    def prepare(self, shapes: list[Request]):
        arr = (Request * len(shapes))(*shapes)
        return self._chk(lib().mlgi_server_prepare(self.h, C.cast(arr, C.c_void_p), len(shapes)),
                         "mlgi_server_prepare")

    def submit(self, req: Request) -> int:
        return lib().mlgi_server_submit(self.h, C.byref(req))

    def cancel(self, id: int) -> int:
        return lib().mlgi_server_cancel(self.h, id)

    def poll(self, max_n: int = 4096) -> np.ndarray:
        out = np.zeros(max_n, COMPLETION_DTYPE)
        n = lib().mlgi_server_poll(self.h, out.ctypes.data, max_n)
        return out[:n]

    def drain(self, timeout_s: float = 600.0):
        return self._chk(lib().mlgi_server_drain(self.h, timeout_s), "mlgi_server_drain")

    def stats(self) -> dict:
        s = ServerStats()
        self._chk(lib().mlgi_server_stats_get(self.h, C.byref(s)), "mlgi_server_stats_get")
        return {k: getattr(s, k) for k, _ in ServerStats._fields_}

    def run_poisson(self, shapes: list[Request], rate_hz: float, duration_s: float, seed: int = 5, n_rooms: int = 8,
                    room_seed_base: int = 1000, light_jitter_deg: float = 5.0, orbit_step_deg: float = 0.5,
                    plain: bool = False, max_out: int | None = None):
        """Open-loop Poisson run; returns (completions, wall seconds)."""
        arr = (Request * len(shapes))(*shapes)
        d = PoissonDesc(seed, rate_hz, duration_s, C.cast(arr, C.c_void_p), len(shapes), n_rooms, room_seed_base,
                        light_jitter_deg, orbit_step_deg, 0.0, int(plain))
        cap = max_out or int(rate_hz * duration_s * 1.5 + 1000)
        out = np.zeros(cap, COMPLETION_DTYPE)
        n, wall = C.c_int(0), C.c_double(0)
        self._chk(lib().mlgi_server_run_poisson(self.h, C.byref(d), out.ctypes.data, cap, C.byref(n), C.byref(wall)),
                  "mlgi_server_run_poisson")
        return out[: n.value], wall.value

    def close(self):
        if self.h:
            lib().mlgi_server_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
