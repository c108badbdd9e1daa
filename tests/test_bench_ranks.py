"""The benchmark's multi-process path on CPU: two ranks on the gloo backend
(127.0.0.1), launched with the variables torchrun sets, agree on the slowest
rank's time (bench.max_over_ranks, the all-reduce MAX that the GPU run does
over NCCL) and report the whole job's rate from it (bench.whole_job_rate:
every rank an independent replica, weak scaling).  CPU only."""
import json
import os
import socket
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)

WORKER = r"""
import json, sys
sys.path.insert(0, sys.argv[1])
import torch.distributed as dist
dist.init_process_group("gloo")
import bench
rank, world = dist.get_rank(), dist.get_world_size()
t = bench.max_over_ranks(1.0 + 0.5 * rank, world, "cpu")  # rank r took 1 + r / 2 s
print(json.dumps({"rank": rank, "t": t, "rate": bench.whole_job_rate(world, 1000, 10, t)}))
dist.destroy_process_group()
"""


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_report_the_slowest_time_and_the_whole_job_rate():
    world, port = 2, free_port()
    procs = []
    for rank in range(world):
        env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", WORKER, REPO], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    try:
        for p in procs:
            out, err = p.communicate(timeout=300)
            assert p.returncode == 0, err
            outs.append(json.loads(out.strip().splitlines()[-1]))
    finally:
        for p in procs:
            if p.poll() is None:
                p.kill()
    assert sorted(o["rank"] for o in outs) == [0, 1]
    for o in outs:
        assert o["t"] == 1.5  # every rank holds the slowest rank's time
        assert abs(o["rate"] - 2 * 1000 * 10 / 1.5) < 1e-9


def test_single_process_needs_no_process_group():
    sys.path.insert(0, REPO)
    import bench
    assert bench.max_over_ranks(2.5, 1, "cpu") == 2.5
    assert bench.whole_job_rate(1, 1000, 10, 2.0) == 5000.0
