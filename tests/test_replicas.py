"""The multi-GPU path of bench.py on the CPU: under torchrun every rank runs
an independent replica of the round trip (the path does not shard), the job
time is the slowest rank's (barrier + all-reduce MAX) and the value counts
the round trips of all ranks.  Two gloo ranks stand in for two GPUs; the
reference arm prints from rank 0 only."""
import json
import os
import socket
import subprocess
import sys

import torch.multiprocessing as mp

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, secs, steps, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(ws), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as tdist

    import bench
    tdist.init_process_group("gloo", rank=rank, world_size=ws)
    m = bench.max_over_ranks(secs[rank], True, "cpu")
    q.put((rank, m, bench.whole_job_value(ws, steps, m)))
    tdist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port, secs, steps = _free_port(), [0.5, 0.8], 10
    procs = [ctx.Process(target=_rank, args=(r, 2, port, secs, steps, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, m, v in got:
        assert m == 0.8
        assert abs(v - 2 * steps / 0.8) < 1e-12


def test_reference_arm_prints_from_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                          "--steps", "1", "--warmup", "0"], env=env, capture_output=True, text=True,
                         timeout=120)
    assert out.returncode == 0, out.stderr
    assert out.stdout.strip() == ""


def test_single_process_value():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(1.25, False, "cpu") == 1.25
    assert bench.whole_job_value(1, 20, 0.5) == 40.0
    assert json.loads(json.dumps({"v": bench.whole_job_value(4, 3, 2.0)}))["v"] == 6.0
