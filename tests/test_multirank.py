"""The multi-rank (replica) path of bench.py on CPU: two gloo ranks, as
torchrun launches them for --gpus 2.  Ranks share no data; the only
collectives are the barrier and the max over ranks of the step time, and
rank 0 alone prints the JSON line."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, port: int, out: str):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE="2", RANK=str(rank),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    world, r, local = bench.dist_setup()
    bench.barrier(world)
    t = bench.all_max(world, 1.5 if r == 0 else 4.25)   # each rank's own step time
    with open(f"{out}.{r}", "w") as f:
        json.dump({"world": world, "rank": r, "max": t}, f)
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_max_step_time(tmp_path):
    import torch.multiprocessing as mp
    port = free_port()
    out = str(tmp_path / "r")
    mp.start_processes(_rank_main, args=(port, out), nprocs=2, start_method="spawn", join=True)
    got = [json.load(open(f"{out}.{r}")) for r in range(2)]
    assert [g["world"] for g in got] == [2, 2]
    assert [g["max"] for g in got] == [4.25, 4.25]


def test_reference_arm_under_torchrun_prints_one_line():
    port = free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "0", "--edge", "32", "--res", "64", "--spp", "4",
           "--cpu-seconds", "0.3"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"
