"""Continuous-batching server: jobs that arrive while others run are admitted as
slots and memory free up, overlap on the device, and each result is the same
as the job run alone (identical kernels; only the scheduling differs)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def R(built):
    import reda_erplacer_gb300 as R
    return R


def _jobs(R, count, seed):
    mix = R.workload_batch(count=count, seed=seed, min_cells=1500, max_cells=15000)
    return [(d, b) for d, b in mix]


@pytest.mark.parametrize("form", ["branches", "packed"])
@pytest.mark.parametrize("max_active,count", [(4, 8), (6, 12)])
def test_server_results_equal_alone(R, max_active, count, form):
    """Each job runs its own graph (the default), or, with ERP_SERVER_FORM=packed,
    a round runs the four or more small jobs active as one graph of packed
    launches, rebuilt as the set changes (fewer: each its own graph); jobs then
    move between the two forms as others arrive and retire."""
    import os
    from reda_erplacer_gb300.serving import Server, run_stream
    jobs = _jobs(R, count, seed=91)
    arrivals = np.sort(np.random.default_rng(count).uniform(0.0, 0.15, count))
    arrivals[:2] = 0.0
    os.environ["ERP_SERVER_FORM"] = form
    try:
        sv = Server(max_active=max_active, hbm_budget_gb=8.0, max_iterations=120, stop_overflow=0.5, chunk=8,
                    keep_positions=True)
    finally:
        del os.environ["ERP_SERVER_FORM"]
    res = run_stream(sv, jobs, arrivals)
    assert len(res) == len(jobs) and all(r["status"] == 0 for r in res)
    # work of different jobs overlapped: some job was admitted before another finished
    spans = sorted((r["admit_s"], r["finish_s"]) for r in res)
    assert any(spans[i + 1][0] < spans[i][1] for i in range(len(spans) - 1))
    by_id = {r["job_id"]: r for r in res}
    for i, (d, b) in enumerate(jobs):
        pl = R.Placement(d, b, 1.0, start_mode=1)
        it, last = pl.run(120, stop_overflow=0.5)
        r = by_id[i]
        assert r["iterations"] == it
        assert r["last"]["hpwl"] == last["hpwl"] and r["last"]["overflow"] == last["overflow"]
        xa, ya = pl.positions()
        xb, yb = sv.positions(i)
        assert np.array_equal(xa, xb) and np.array_equal(ya, yb)
        pl.close()
    sv.close()


def test_server_admission_by_footprint(R):
    from reda_erplacer_gb300.serving import Server, estimate_footprint, run_stream
    jobs = _jobs(R, 6, seed=92)
    fps = [estimate_footprint(d, b) for d, b in jobs]
    budget = 2.2 * max(fps)                     # at most two jobs fit at once
    sv = Server(max_active=16, hbm_budget_gb=budget / 2 ** 30, max_iterations=40, stop_overflow=0.0,
                chunk=8)
    res = run_stream(sv, jobs, np.zeros(len(jobs)))
    assert all(r["status"] == 0 and r["iterations"] == 40 for r in res)
    events = sorted([(r["admit_s"], 1, r["footprint_bytes"]) for r in res] +
                    [(r["finish_s"], -1, r["footprint_bytes"]) for r in res], key=lambda e: (e[0], e[1]))
    used = 0
    for _, kind, fp in events:
        used += kind * fp
        assert used <= budget
    sv.close()
    # a job that can never fit is rejected, not queued forever
    sv = Server(max_active=4, hbm_budget_gb=min(fps) / 2 / 2 ** 30, max_iterations=10, chunk=4)
    res = run_stream(sv, jobs[:1], np.zeros(1))
    assert res[0]["status"] == R.lib.ENOMEM
    sv.close()


def test_server_cancel(R):
    """A queued job and a running job withdrawn mid-stream report ECANCELED and
    free their slot; every other job ends with the results it has alone."""
    from reda_erplacer_gb300.serving import Server
    jobs = _jobs(R, 8, seed=93)
    sv = Server(max_active=3, hbm_budget_gb=8.0, max_iterations=80, stop_overflow=0.0, chunk=8,
                keep_positions=True)
    for i, (d, b) in enumerate(jobs):
        sv.submit(i, d, b)
    res = []
    for _ in range(4):   # a few rounds: some jobs running, the rest queued
        sv.pump()
        res += sv.poll()
    sv.cancel(7)                             # still queued (three slots, FIFO)
    running = [j for j in range(7) if j not in {r["job_id"] for r in res}][0]
    sv.cancel(running)
    with pytest.raises(R.lib.ErpError) as e:
        sv.cancel(12345)
    assert e.value.status == R.lib.EINVAL
    while True:
        active, queued = sv.pump()
        res += sv.poll()
        if not active and not queued:
            break
    res += sv.poll()
    by_id = {r["job_id"]: r for r in res}
    assert sorted(by_id) == list(range(8))
    assert by_id[7]["status"] == R.lib.ECANCELED and by_id[7]["iterations"] == 0
    assert by_id[running]["status"] == R.lib.ECANCELED and by_id[running]["iterations"] < 80
    for i, (d, b) in enumerate(jobs):
        if i in (7, running):
            continue
        assert by_id[i]["status"] == 0 and by_id[i]["iterations"] == 80
        pl = R.Placement(d, b, 1.0, start_mode=1)
        pl.run(80)
        xa, ya = pl.positions()
        xb, yb = sv.positions(i)
        assert np.array_equal(xa, xb) and np.array_equal(ya, yb), i
        pl.close()
    sv.close()
