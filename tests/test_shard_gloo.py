"""Multi-GPU host logic on CPU: two gloo ranks each run their shard of the
event batch (on the oracle: no GPU here), and the reduced verification sum
and timing equal the single-process ones."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from xsbench_gb300.shard import reduce_time_max, reduce_verification, shard_range


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, scaling, n, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import oracle
    from conftest import oracle_config
    first, count = shard_range(rank, world, n, scaling)
    with oracle.Problem(oracle_config("tiny_unionized")) as p:
        v = p.run_event(first=first, n=count, nthreads=2)["verification"]
    total = reduce_verification(v, dist)
    tmax = reduce_time_max(float(rank + 1), dist)
    out[rank] = (total, tmax, first, count)
    dist.destroy_process_group()


@pytest.mark.parametrize("scaling", ["strong", "weak"])
def test_two_gloo_ranks_reduce_to_the_single_process_result(scaling):
    import oracle
    from conftest import oracle_config
    n = 60000
    world = 2
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, scaling, n, out)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    total_events = n if scaling == "strong" else n * world
    with oracle.Problem(oracle_config("tiny_unionized")) as p:
        ref = p.run_event(first=0, n=total_events, nthreads=2)["verification"]
    for r in range(world):
        assert out[r][0] == ref
        assert out[r][1] == 2.0
    ranges = sorted((out[r][2], out[r][3]) for r in range(world))
    assert ranges[0][0] == 0 and ranges[0][0] + ranges[0][1] == ranges[1][0]


def test_shard_range_partitions():
    for world in (1, 2, 3, 8):
        n = 17000000
        parts = [shard_range(r, world, n, "strong") for r in range(world)]
        assert parts[0][0] == 0 and sum(c for _, c in parts) == n
        for (a, c), (b, _) in zip(parts, parts[1:]):
            assert a + c == b
        assert [shard_range(r, world, n, "weak") for r in range(world)] == [(r * n, n) for r in range(world)]
    with pytest.raises(ValueError):
        shard_range(2, 2, 10)
