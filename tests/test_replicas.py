"""The multi-GPU form of the benchmark is replicas only (each rank runs the
whole workload on its own GPU, no data-path collective): the host logic --
rank and world from the launcher's environment, the job time as the slowest
rank's, the whole-job rate -- run as two gloo ranks on the CPU."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    r, w = bench._env_rank()
    dist.init_process_group("gloo", rank=r, world_size=w)
    ms_local = 100.0 + 25.0 * rank          # the ranks' own step-loop times
    ms = bench.max_over_ranks(ms_local, dist)
    out.put((r, w, ms, bench.replica_rate(1000, 10, w, ms)))
    dist.destroy_process_group()


def test_replicas_time_is_the_slowest_rank():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[0] for r in res] == [0, 1] and all(r[1] == 2 for r in res)
    assert all(r[2] == 125.0 for r in res)                 # max over the two ranks
    assert res[0][3] == pytest.approx(1000 * 10 * 2 / 0.125)


def test_single_rank_needs_no_process_group():
    import bench
    assert bench.max_over_ranks(42.0, None) == 42.0
    assert bench.replica_rate(4603904, 100, 1, 1000.0) == pytest.approx(460390400.0)
