"""CPU tests of the replica-rank host logic (cosmicblup_gb300/ranks.py) with two gloo
ranks: the barrier, the slowest-rank time, the whole-job rate and the round-robin
sharding of independent problems.  No GPU: the ranks share host scalars only."""
import multiprocessing as mp
import os
import socket

import pytest


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    from cosmicblup_gb300.ranks import Replicas, job_rate
    reps = Replicas()
    try:
        reps.barrier()
        rate, ms = job_rate(5, 100.0 * (rank + 1), reps)
        q.put((rank, rate, ms, reps.shard(list(range(11))), reps.sum(rank + 1)))
    finally:
        reps.close()


def test_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, rate0, ms0, sh0, s0), (r1, rate1, ms1, sh1, s1) = out
    # both ranks see the slowest rank's 200 ms and the job's 10 units in it
    assert ms0 == ms1 == 200.0
    assert rate0 == rate1 == pytest.approx(50.0)
    assert sh0 == [0, 2, 4, 6, 8, 10] and sh1 == [1, 3, 5, 7, 9]
    assert s0 == s1 == 3.0


def test_single_process_defaults(monkeypatch):
    for k in ("RANK", "LOCAL_RANK", "WORLD_SIZE"):
        monkeypatch.delenv(k, raising=False)
    from cosmicblup_gb300.ranks import Replicas, job_rate
    reps = Replicas()
    assert (reps.rank, reps.local_rank, reps.world) == (0, 0, 1)
    reps.barrier()
    assert job_rate(3, 1500.0, reps) == (2.0, 1500.0)
    assert reps.shard([1, 2, 3]) == [1, 2, 3]
