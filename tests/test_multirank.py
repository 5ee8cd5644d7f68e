"""Ensembles over several ranks: the member partition and the host-side gather, as world_size-2
gloo process groups on the CPU (no GPU)."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_partition_balances_and_covers(pkg):
    rng = np.random.default_rng(3)
    costs = np.exp(rng.uniform(np.log(2e4), np.log(4e5), 64))   # member sizes log-uniform in [20k, 400k]
    for world in (1, 2, 3, 4, 8):
        parts = pkg.ensemble.partition_members(costs, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(costs)))                    # every member exactly once
        loads = [costs[p].sum() for p in parts]
        # longest-processing-time rule: the heaviest rank exceeds the mean by at most the largest member
        assert max(loads) <= costs.sum() / world + costs.max() + 1e-6
        assert parts == pkg.ensemble.partition_members(list(costs), world)   # deterministic
    assert pkg.ensemble.shard(1, 4, costs) == pkg.ensemble.partition_members(costs, 4)[1]
    with pytest.raises(ValueError):
        pkg.ensemble.shard(4, 4, costs)


def _worker(rank, world, port, costs, out):
    import sys
    import torch.distributed as dist
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import __graft_entry__
    pkg = __graft_entry__.load_package()
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        mine = pkg.ensemble.shard(rank, world, costs)
        # stand-in for each member's solve: a result that names the member and the rank
        results = pkg.ensemble.gather_results({i: {"rank": rank, "value": float(costs[i]) * 2.0} for i in mine})
        slowest = pkg.ensemble.max_over_ranks(float(len(mine)) + 0.5 * rank)
        out.put((rank, sorted(results), {k: v["rank"] for k, v in results.items()}, slowest))
    finally:
        dist.destroy_process_group()


def test_two_ranks_gather_every_member_once(pkg):
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    costs = [5.0, 1.0, 4.0, 2.0, 3.0, 3.0, 1.0]
    port = _free_port()
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, costs, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = [q.get(timeout=120) for _ in range(2)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    parts = pkg.ensemble.partition_members(costs, 2)
    for rank, members, owner, slowest in got:
        assert members == list(range(len(costs)))                  # every rank sees all members
        for r, part in enumerate(parts):
            assert all(owner[i] == r for i in part)                # each solved by its owner only
        assert slowest == max(len(parts[0]), len(parts[1]) + 0.5)  # the max over ranks


def test_mixed_ensemble_members(pkg):
    """The mixed-size DIVA ensemble's generator: 64 sizes log-uniform in [20k, 400k] summing to
    about 8.1M vertices, and a small member with the stated bed statistics and a dome with
    grounded and floating ice."""
    G = pkg.geometry
    sizes = G.mixed_ensemble_sizes()
    assert len(sizes) == 64 and sizes.min() >= 20_000 and sizes.max() <= 400_000
    assert abs(sizes.sum() - 8.1e6) < 0.05e6
    m = G.mixed_ensemble_mesh(6000, seed=2, nz=6)
    assert 5000 < m.nV < 7500
    ice, p = G.mixed_ensemble_member(m, 2)
    bed = ice["Hb"]
    assert abs(bed.mean() + 300.0) < 1e-6 and abs(bed.std() - 800.0) < 1e-6
    on_ice = ice["Hi"] > 0
    assert 0.2 < on_ice.mean() < 0.7
    g = ice["mask_grounded_ice"].astype(bool)
    assert g.any() and (on_ice & ~g).any()     # grounded and floating ice both present
