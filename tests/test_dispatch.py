"""Host-side dispatch of independent jobs over GPUs (reda_erplacer_gb300.dispatch)
and the cross-rank helpers of bench.py, on CPU: the partition's properties, and
a two-rank gloo run (one process per rank, as torchrun starts them) in which
each rank takes its shard and the ranks gather timings and results."""
import os
import socket

import numpy as np
import pytest

from conftest import ROOT


@pytest.fixture(scope="module")
def D(built):
    from reda_erplacer_gb300 import dispatch
    return dispatch


def test_shard_is_a_balanced_partition(D):
    shard, rank_jobs = D.shard, D.rank_jobs
    rng = np.random.default_rng(3)
    costs = list(np.exp(rng.uniform(np.log(2000), np.log(200000), 64)))
    for world in (1, 2, 3, 4, 8):
        parts = shard(costs, world)
        assert len(parts) == world
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(costs)))          # every job once
        loads = [sum(costs[i] for i in p) for p in parts]
        # longest-processing-time-first: within 4/3 of the best makespan
        lower = max(sum(costs) / world, max(costs))
        assert max(loads) <= 4.0 / 3.0 * lower + 1e-6
        assert parts == shard(costs, world)              # deterministic
        for r in range(world):
            assert rank_jobs(costs, world, r) == parts[r]


def test_shard_edge_cases(D):
    shard, rank_jobs, job_cost = D.shard, D.rank_jobs, D.job_cost
    assert shard([], 3) == [[], [], []]
    assert shard([5.0], 4) == [[0], [], [], []]
    assert shard([1.0, 1.0, 1.0, 1.0], 2) == [[0, 2], [1, 3]]   # ties go to the lower rank
    with pytest.raises(ValueError):
        shard([1.0], 0)
    with pytest.raises(ValueError):
        rank_jobs([1.0], 2, 2)
    assert job_cost(1000, 600) == 600000.0


def test_route_stream_least_loaded_on_arrival(D):
    route_stream = D.route_stream
    costs = [10, 1, 1, 1, 10, 1]
    assert route_stream(costs, 1) == [0] * 6
    assert route_stream(costs, 2) == [0, 1, 1, 1, 1, 0]
    rng = np.random.default_rng(5)
    c = list(rng.uniform(1, 100, 500))
    r = route_stream(c, 4)
    loads = [sum(x for x, k in zip(c, r) if k == q) for q in range(4)]
    assert max(loads) - min(loads) <= max(c)   # online greedy: within one job of each other


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import json
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import bench
    from reda_erplacer_gb300.dispatch import job_cost, rank_jobs
    w, r, local = bench.dist_setup()
    costs = [job_cost(c, 600) for c in (16228, 5596, 64128, 7481, 132769, 83363, 15273, 14746, 8436)]
    mine = rank_jobs(costs, w, r)
    # "run" the shard: every job reports (index, rank); each rank's time differs
    done = [(i, r) for i in mine]
    t = 1.0 + r
    res = {
        "world": w, "rank": r,
        "all": bench.gather_items(done, w),
        "tmax": bench.allreduce_max(t, w),
        "tsum": bench.allreduce_sum(t, w),
        "mine": mine,
    }
    bench.barrier(w)
    with open(os.path.join(out_dir, f"rank{r}.json"), "w") as f:
        json.dump(res, f)
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_rank_gloo_sharded_jobs(D, tmp_path):
    torch = pytest.importorskip("torch")
    import json
    import torch.multiprocessing as mp
    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    res = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(world)]
    assert [x["rank"] for x in res] == [0, 1] and all(x["world"] == 2 for x in res)
    # both ranks see the same gathered list: every job exactly once, run by its owner
    assert res[0]["all"] == res[1]["all"]
    jobs = sorted(i for i, _ in res[0]["all"])
    assert jobs == list(range(9))
    for i, r in res[0]["all"]:
        assert i in res[r]["mine"]
    assert not set(res[0]["mine"]) & set(res[1]["mine"])
    # the slowest rank's time, and the sum (capacity) across ranks
    assert res[0]["tmax"] == res[1]["tmax"] == 2.0
    assert res[0]["tsum"] == res[1]["tsum"] == 3.0
