"""The multi-process form of bench.py on CPU with gloo (world size 2): the replicas' timings reduce
to their maximum, and the reference arm under torchrun runs on rank 0 alone and prints one line."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out_dir):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        got = bench.reduce_max([1.0 + rank, 10.0 - rank, 3.5], world)
        with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
            json.dump(got, f)
    finally:
        dist.destroy_process_group()


def test_timings_reduce_to_the_slowest_rank(tmp_path):
    import torch.multiprocessing as mp

    port = _free_port()
    mp.spawn(_rank, args=(2, port, str(tmp_path)), nprocs=2, join=True)  # spawn start method
    got = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(2)]
    assert got[0] == got[1] == [2.0, 10.0, 3.5]


def test_reference_arm_under_torchrun_two_ranks():
    port = _free_port()
    env = dict(os.environ, OMP_NUM_THREADS="2")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference", "--gpus", "2",
           "--config", "c0_160x96_n64", "--steps", "2", "--warmup", "1", "--reference-seconds", "1"]
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(l) for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = lines[0]
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["value"] == d["value"] and d["cpu_baseline"]["kind"] == "port"
    passes = d["cpu_baseline"]["passes_ms"]
    assert set(passes) == {"vpl_process", "ism_clear+ism_splat", "pullpush", "final_gather"}
    assert all(v >= 0 for v in passes.values()) and sum(passes.values()) <= d["value"] * 1.01
