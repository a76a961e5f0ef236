"""Products shard across ranks with no data-path collective (one GPU per
rank).  Host logic only: the plan, and a world-size-2 gloo run whose ranks
each compute their share (with the oracle standing in for the GPU) and
gather the results."""
import os
import socket

import numpy as np
import pytest


def test_plan_covers_every_product_once_and_balances():
    import importlib
    shard = importlib.import_module("fherma-bytecrt_gb300.shard")
    costs = [shard.cost(65536, 1747)] * 38 + [shard.cost(32768, 868)] * 58
    for world in (1, 2, 3, 4, 8):
        shares = shard.plan(costs, world)
        flat = sorted(i for s in shares for i in s)
        assert flat == list(range(len(costs)))
        loads = [sum(costs[i] for i in s) for s in shares]
        assert max(loads) - min(loads) <= max(costs)
    assert shard.plan([], 2) == [[], []]
    assert shard.plan([3.0, 1.0, 2.0], 1) == [[0, 1, 2]]
    with pytest.raises(ValueError):
        shard.plan([1.0], 0)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, dst, out_q):
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, os.path.dirname(here))
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        _work(rank, dst, out_q)
    except Exception as e:   # report instead of leaving the parent waiting
        out_q.put((rank, -1, False, repr(e)))
    finally:
        dist.destroy_process_group()


def _work(rank, dst, out_q):
    import importlib
    shard = importlib.import_module("fherma-bytecrt_gb300.shard")
    inputs = importlib.import_module("fherma-bytecrt_gb300.inputs")
    from oracle import oracle as O
    items = []
    for i, (N, W) in enumerate([(64, 100), (128, 40), (16, 200), (64, 100), (32, 64)]):
        q = inputs.modulus(W, 50 + i)
        items.append((N, W, q, inputs.uniform(q, N, 2 * i), inputs.uniform(q, N, 2 * i + 1)))
    computed = []

    def fn(item):
        N, W, q, a, b = item
        computed.append(N)
        return O.Oracle(N, W, q).multiply(a, b)

    res = shard.run_sharded(items, fn, costs=[shard.cost(x[0], x[1]) for x in items], dst=dst)
    ok = None
    if res is not None:
        ok = all(np.array_equal(r, O.schoolbook(x[3], x[4], inputs.q_int(x[2]))) for r, x in zip(res, items))
    out_q.put((rank, len(computed), res is not None, ok))


@pytest.mark.parametrize("dst", [None, 0])
def test_gloo_two_ranks_share_and_gather(dst):
    import multiprocessing as mp
    from oracle import oracle as O
    O.build()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, dst, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert all(r[1] >= 0 for r in results), results
    # Each product computed exactly once across the ranks.
    assert sum(r[1] for r in results) == 5 and all(r[1] > 0 for r in results)
    for rank, _, has, ok in results:
        if dst is None or rank == dst:
            assert has and ok
        else:
            assert not has
