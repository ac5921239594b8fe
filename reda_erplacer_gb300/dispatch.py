"""Host-side dispatch of independent placement jobs over GPUs (one process per
GPU).  Jobs share nothing, so a job stream or a batch is partitioned across the
ranks with no collective on the data path; the only cross-rank traffic is the
final gathering of timings and results.

    shard(costs, world)          -> list of job-index lists, one per rank
    rank_jobs(costs, world, r)   -> the jobs of rank r
    route_stream(costs, world)   -> the rank of each job of an arriving stream
    job_cost(cells, iterations)  -> the cost model the bench uses

The partition is the longest-processing-time-first greedy: jobs in decreasing
cost order (ties by index) each go to the rank with the least total so far
(ties by rank), which is deterministic and within 4/3 of the best makespan.
A stream is routed online instead: each job, in arrival order, goes to the
rank with the least work assigned so far.
"""


def job_cost(cells, iterations=1):
    """Estimated GPU time of a job: proportional to cells x iterations (the step's
    passes are linear in cells, nets and bins, which scale together)."""
    return float(cells) * float(iterations)


def shard(costs, world):
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i))
    load = [0.0] * world
    parts = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        parts[r].append(i)
        load[r] += float(costs[i])
    for p in parts:
        p.sort()
    return parts


def rank_jobs(costs, world, rank):
    if not 0 <= rank < world:
        raise ValueError("rank out of range")
    return shard(costs, world)[rank]


def route_stream(costs, world):
    """Rank of each job of a stream (costs in arrival order), routed on arrival
    to the rank with the least assigned work (ties by rank)."""
    if world < 1:
        raise ValueError("world must be >= 1")
    load = [0.0] * world
    out = []
    for c in costs:
        r = min(range(world), key=lambda k: (load[k], k))
        out.append(r)
        load[r] += float(c)
    return out
