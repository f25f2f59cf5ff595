"""The N>1 path of bench.py on CPU with the gloo backend, world size 2: the
batched and served workloads shard their instances across ranks (bench.shard,
no collective on the data), and the union of the ranks' instances and
results equals the single-rank run; the elapsed time reported is the max over
ranks.  Each rank computes its instances' results with the oracle, the CPU
stand-in for its GPU replica.  No GPU involved."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _oracle_terms(spec):
    import bench
    import oracle as O
    shape, d, a, graded, robin = spec
    out = []
    for ax, n in enumerate(shape):
        dx = bench.batch_grid(n, graded)
        bc = O.robin(bench.ROBIN_L, bench.ROBIN_R, dx, 1) if robin else O.dirichlet(*bench.DIRICHLET_LR)
        out.append((O.centered(d, a, dx, n, axis=ax + 1), bc))
    return out


def _serve_terms(r):
    import oracle as O
    terms = []
    for k, n in enumerate(r.shape):
        terms.append((O.centered(2, 2, 1.0 / (n + 1), n, axis=k + 1).scale(r.nu), O.dirichlet0()))
    terms.append((O.upwind(1, r.approx_order, 1.0 / (r.shape[0] + 1), r.shape[0], -r.c, axis=1), O.dirichlet0()))
    return terms


def _batch_specs():
    import bench
    return bench.batch_specs(40, scale=0.01)


def _requests():
    from deo.serve import poisson_requests
    return poisson_requests(10, 2000.0, seed=5, size_scale=0.02, k_range=(2, 4), grad_frac=0.0)


def _run(rank, ws):
    """One rank's share of both workloads, computed by the oracle."""
    import bench
    import oracle as O
    specs = _batch_specs()
    mine = bench.shard([int(np.prod(s[0])) for s in specs], rank, ws)
    batch = {}
    for i in mine:
        u = np.asfortranarray(np.random.default_rng(1000 + i).standard_normal(specs[i][0]))
        batch[i] = O.apply(_oracle_terms(specs[i]), u)
    reqs = _requests()
    served = {}
    for i in bench.shard([bench._serve_cost(r) for r in reqs], rank, ws):
        r = reqs[i]
        served[r.rid] = O.ssprk3(_serve_terms(r), r.initial(), r.dt(), r.K)
    return batch, served


def _worker(rank, ws, port, out):
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    batch, served = _run(rank, ws)
    parts = bench.gather_objects((batch, served), ws)
    bench.barrier(ws)
    t = bench.max_over_ranks(1.0 + rank, ws)
    out[rank] = (parts, t)
    dist.destroy_process_group()


def test_sharded_workloads_equal_single_rank():
    ws = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    port = _free_port()
    mp.start_processes(_worker, args=(ws, port, out), nprocs=ws, start_method="spawn", join=True)
    one_batch, one_served = _run(0, 1)
    for r in range(ws):
        parts, t = out[r]
        assert t == float(ws)  # max over ranks
        keys_b = [k for b, _ in parts for k in b]
        keys_s = [k for _, s in parts for k in s]
        # a partition: every instance on exactly one rank, none twice
        assert sorted(keys_b) == sorted(one_batch) and len(set(keys_b)) == len(keys_b)
        assert sorted(keys_s) == sorted(one_served) and len(set(keys_s)) == len(keys_s)
        assert all(len(b) > 0 for b, _ in parts)
        for b, s in parts:
            for k, v in b.items():
                assert np.array_equal(v, one_batch[k])
            for k, v in s.items():
                assert np.array_equal(v, one_served[k])


@pytest.mark.parametrize("n,ws", [(0, 2), (5, 3), (4096, 7), (3, 8), (40, 2)])
def test_shard_partition_and_balance(n, ws):
    import bench
    costs = [int(c) for c in np.random.default_rng(n + ws).integers(1, 1000, size=n)]
    parts = [bench.shard(costs, r, ws) for r in range(ws)]
    assert sorted(i for p in parts for i in p) == list(range(n))
    assert all(p == sorted(p) for p in parts)
    loads = [sum(costs[i] for i in p) for p in parts]
    if n:
        # greedy by decreasing cost: no rank exceeds another by more than the largest cost
        assert max(loads) - min(loads) <= max(costs)
