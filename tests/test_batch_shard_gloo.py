"""Sharding a batch of uneven systems across GPUs, on CPU: two ranks over gloo
(127.0.0.1). The systems are independent, so each rank takes one contiguous,
cost-balanced slice (la_batch_partition: cost 2/3 n^3 + 2 n^2 nrhs) and works
it alone; nothing crosses ranks until the answers are gathered. Here each rank
solves its slice with the oracle (no GPU in these tests), the slices are
gathered on rank 0, and the result must equal the one-rank solution bit for
bit; the partition must balance the cost."""
import os
import socket
import sys

import numpy as np
import pytest

torch = pytest.importorskip("torch")

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
PKG = os.path.join(ROOT, "rust-la_gb300")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _batch(count, seed):
    rng = np.random.default_rng(seed)
    ns = rng.integers(8, 97, size=count)
    rs = rng.integers(1, 5, size=count)
    a = [rng.standard_normal((n, n)) + (0.5 * n * np.eye(n) if i % 2 == 0 else 0)
         for i, n in enumerate(ns)]
    b = [rng.standard_normal((n, r)) for n, r in zip(ns, rs)]
    return ns, rs, np.concatenate([m.ravel() for m in a]), np.concatenate([m.ravel() for m in b])


def _solve_slice(oracle, systems, ha, hb, x):
    for s in systems:
        f = oracle.lu_factor(ha[s.a_offset:s.a_offset + s.n * s.n].reshape(s.n, s.n))
        xi = oracle.solve(f, hb[s.b_offset:s.b_offset + s.n * s.nrhs].reshape(s.n, s.nrhs))
        x[s.b_offset:s.b_offset + s.n * s.nrhs] = xi.ravel()


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world),
                      RANK=str(rank), LOCAL_RANK=str(rank))
    for p in (ROOT, PKG):
        sys.path.insert(0, p)
    import torch.distributed as dist
    import la_gpu
    import oracle
    dist.init_process_group("gloo")
    try:
        ns, rs, ha, hb = _batch(97, 5)
        systems, na, nb = la_gpu.batch_systems(ns, rs)
        bounds = la_gpu.batch_partition(systems, world)
        mine, a0, alen, b0, blen = la_gpu.batch_slice(systems, bounds[rank], bounds[rank + 1])
        x = np.zeros(blen)
        _solve_slice(oracle, mine, ha[a0:a0 + alen], hb[b0:b0 + blen], x)
        got = [None] * world
        dist.all_gather_object(got, (rank, b0, x))
        if rank == 0:
            full = np.zeros(nb)
            for _, base, xs in got:
                full[base:base + len(xs)] = xs
            q.put((bounds, full))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_ranks_gather_the_one_rank_solution_bit_for_bit(lagpu, oracle_lib):
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    bounds, full = q.get(timeout=180)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    ns, rs, ha, hb = _batch(97, 5)
    systems, na, nb = lagpu.batch_systems(ns, rs)
    want = np.zeros(nb)
    _solve_slice(oracle_lib, systems, ha, hb, want)
    assert np.array_equal(full, want)
    assert bounds[0] == 0 and bounds[-1] == len(ns) and bounds[0] <= bounds[1] <= bounds[2]


@pytest.mark.parametrize("parts", [1, 2, 3, 8])
def test_partition_balances_the_cost(lagpu, parts):
    rng = np.random.default_rng(parts)
    ns = rng.integers(8, 257, size=2000)
    rs = rng.integers(1, 5, size=2000)
    systems, _, _ = lagpu.batch_systems(ns, rs)
    bounds = lagpu.batch_partition(systems, parts)
    cost = 2.0 / 3.0 * ns.astype(float) ** 3 + 2.0 * ns.astype(float) ** 2 * rs
    total = cost.sum()
    assert bounds[0] == 0 and bounds[-1] == len(ns) and np.all(np.diff(bounds) >= 0)
    for p in range(parts):
        share = cost[bounds[p]:bounds[p + 1]].sum()
        # each slice is within one system's cost of an equal share
        assert abs(share - total / parts) <= 2 * cost.max()
    # slices rebase their offsets and cover the packed buffers exactly
    tot_a = tot_b = 0
    for p in range(parts):
        sl, a0, alen, b0, blen = lagpu.batch_slice(systems, bounds[p], bounds[p + 1])
        assert a0 == tot_a and b0 == tot_b
        if len(sl):
            assert sl[0].a_offset == 0 and sl[0].b_offset == 0
        tot_a += alen
        tot_b += blen
    assert tot_a == sum(int(n) * int(n) for n in ns)
    assert tot_b == sum(int(n) * int(r) for n, r in zip(ns, rs))


def test_partition_rejects_bad_arguments(lagpu):
    systems, _, _ = lagpu.batch_systems([4, 5], [1, 1])
    with pytest.raises(lagpu.LaError):
        lagpu.batch_partition(systems, 0)
    assert lagpu.batch_partition(systems, 4)[-1] == 2  # more parts than systems: empty slices
