"""Replica runs (one independent DNS per rank under torchrun): the host logic on two gloo ranks on the CPU.

* the barrier brackets and the max over ranks of the timed interval (each rank passes its own time; every
  rank gets the slowest);
* the whole-job rate counts every rank's steps over that time (weak scaling);
* `bench.py --impl reference` under two ranks: rank 0 alone prints the line, the other rank exits 0 with no
  output and no work.
"""

import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    from channelflow_gb300.replicas import Replicas
    reps = Replicas(rank, world)
    assert reps.device == "cpu" and reps.dist is not None
    reps.barrier()
    t = reps.max_over_ranks(1.5 + rank)          # rank r took 1.5 + r seconds
    rate = reps.throughput(100, t)               # 100 steps per rank
    reps.barrier()
    reps.close()
    out.put((rank, t, rate))


def test_two_gloo_ranks_max_and_rate():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[0] for r in res] == [0, 1]
    for _, t, rate in res:
        assert t == 2.5                          # the slowest rank's time on every rank
        assert rate == pytest.approx(2 * 100 / 2.5)


def test_single_rank_needs_no_process_group():
    from channelflow_gb300.replicas import Replicas
    reps = Replicas(0, 1)
    assert reps.dist is None
    reps.barrier()
    assert reps.max_over_ranks(3.0) == 3.0
    assert reps.throughput(10, 2.0) == 5.0


def test_reference_arm_other_rank_exits_quietly():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1", MASTER_ADDR="127.0.0.1")
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--gpus", "2", "--steps", "1",
                        "--warmup", "3"], cwd=ROOT, env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
    with pytest.raises(json.JSONDecodeError):
        json.loads(r.stdout or "")
