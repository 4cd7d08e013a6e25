"""The multi-GPU form is replicas only: each rank renders its own samples and
the bench reduces one time (max over ranks) with no data-path collective.
These run as gloo ranks on the CPU."""
import json
import os
import pathlib
import socket
import subprocess
import sys

import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = pathlib.Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    sys.path.insert(0, str(ROOT))
    import bench

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        bench.barrier(world)
        t = bench.max_over_ranks(1.0 + rank, world, "cpu")
        _, rays = bench.traversal_inputs(rank, True, rays=64)
        req = bench.served_inputs(4, True, rank)[1]
        out.put((rank, t, rays[:4].tolist(), [round(r.arrival, 9) for r in req]))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_per_rank_inputs():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, out), nprocs=2, start_method="spawn", join=True)
    got = sorted(out.get(timeout=60) for _ in range(2))
    assert [g[1] for g in got] == [2.0, 2.0]  # every rank sees the slowest rank's time
    assert got[0][2] != got[1][2]  # ranks trace different rays
    assert got[0][3] != got[1][3]  # and serve request traces of their own (arrival times differ)


def test_reference_arm_under_torchrun_prints_one_line(oracle):
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), str(ROOT / "bench.py"), "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "1", "--small", "--cpu-seconds", "0.4"]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    res = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=300, env=env)
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [ln for ln in res.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, res.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["value"] == d["value"] and d["cpu_baseline"]["kind"] == "port"
