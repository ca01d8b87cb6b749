"""Multi-GPU is replicas only: each rank runs an independent simulation (seed 777 +
rank) and only the job totals are combined.  This runs that path as two gloo ranks
on the CPU, with the oracle as each rank's simulation, through bench.py's own
aggregation (reduce_replicas)."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist
    import bench
    from oracle.oracle import Oracle, make_params
    dist.init_process_group("gloo", rank=rank, world_size=world)
    p = make_params(max_days=12, people_scaling=0.005, location_scaling=0.005)
    o = Oracle(p, bench.SEED + rank)
    o.setup()
    days = 0
    while True:
        rc, _, _ = o.step_day()
        if rc == 2:
            break
        days += 1
        if rc == 1:
            break
    n = o.view()["N"]
    gp, _ = o.gen_counts()
    o.close()
    ms = 10.0 * (rank + 1)
    ms_max, pd = bench.reduce_replicas(ms, float(n * days), "cpu")
    out.put((rank, n, days, ms_max, pd, gp.tolist()))
    dist.destroy_process_group()


def test_two_replicas_are_independent_and_summed():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for pr in procs:
        pr.start()
    res = sorted(q.get(timeout=180) for _ in range(world))
    for pr in procs:
        pr.join(timeout=60)
        assert pr.exitcode == 0
    total = sum(n * d for _, n, d, *_ in res)
    for rank, n, days, ms_max, pd, _ in res:
        assert ms_max == pytest.approx(20.0)   # slowest rank
        assert pd == pytest.approx(total)       # whole-job person-days
    # different seeds give different populations / epidemics
    assert res[0][5] != res[1][5]
