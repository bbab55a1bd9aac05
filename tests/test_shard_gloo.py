"""Multi-GPU host logic on CPU: two gloo ranks each run their shard of the
event batch (on the oracle: no GPU here), and the reduced verification sum
and timing equal the single-process ones."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from xsbench_gb300.shard import reduce_gradients, reduce_time_max, reduce_verification, shard_range


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


def _grad_worker(rank, world, port, n, out):
    """Rank's shard of an adjoint batch: gradients of its lookups with the
    plain-PyTorch reference (the adjoint's own checker; no GPU here), then the
    rank-order reduction."""
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import numpy as np
    import torch
    import oracle
    from conftest import oracle_config
    from torch_reference import reference_gradients, tables_from_arrays
    first, count = shard_range(rank, world, n, "strong")
    with oracle.Problem(oracle_config("tiny_unionized")) as p:
        arrs = p.arrays()
        r = p.run_event(first=first, n=count, want_samples=True, nthreads=1)
        egrid, xs, concs, mats, nn = tables_from_arrays(arrs, 68, 1000, 34)
    g = np.random.default_rng(77).standard_normal((n, 5))[first:first + count]
    _, _, dc, dx = reference_gradients(r["energy"], r["mat"], g, egrid, xs, concs, mats, nn)
    red = reduce_gradients([torch.from_numpy(dc), torch.from_numpy(dx)], dist)
    out[rank] = (dc, dx, red[0].numpy(), red[1].numpy())
    dist.destroy_process_group()


def test_two_gloo_ranks_reduce_adjoint_gradients_in_rank_order():
    """The ranks' dL/dconcs and dL/dxs, reduced, are the same bits on every
    rank and equal the rank-order sum of the partial gradients; they match
    the single-process gradient of the whole batch within rounding."""
    import numpy as np
    import oracle
    from conftest import oracle_config
    from torch_reference import reference_gradients, tables_from_arrays
    n, world = 6000, 2
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_grad_worker, args=(r, world, port, n, out)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(300)
        assert p.exitcode == 0
    serial_c = out[0][0] + out[1][0]
    serial_x = out[0][1] + out[1][1]
    for r in range(world):
        assert np.array_equal(out[r][2], serial_c)
        assert np.array_equal(out[r][3], serial_x)
    with oracle.Problem(oracle_config("tiny_unionized")) as p:
        arrs = p.arrays()
        s = p.run_event(first=0, n=n, want_samples=True, nthreads=1)
        egrid, xs, concs, mats, nn = tables_from_arrays(arrs, 68, 1000, 34)
    g = np.random.default_rng(77).standard_normal((n, 5))
    _, _, dc, dx = reference_gradients(s["energy"], s["mat"], g, egrid, xs, concs, mats, nn)
    assert np.max(np.abs(serial_c - dc)) <= 1e-12 * np.max(np.abs(dc))
    assert np.max(np.abs(serial_x - dx)) <= 1e-12 * np.max(np.abs(dx))
