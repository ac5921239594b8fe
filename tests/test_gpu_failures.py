"""Failure handling on the GPU without a fault.

* A non-finite position retires the context through the step's own check on the
  device (non-finite HPWL, overflow or step length): the host reads ERP_ENAN,
  and the context stays retired.  Every index the kernels derive from a
  position is clamped, so NaN coordinates read and write in bounds.
* Positions far outside the die (beyond 2^31 bins, negative, huge) index
  nothing out of bounds: every kernel clamps the bins it derives from a
  position, so the step ends with a status (ERP_OK, or ERP_ENAN if a total
  overflowed), never a CUDA error, and the device stays usable.
* Inside the server a job that cannot be set up (a bin grid the library
  rejects, a non-finite coordinate) fails alone on its admission worker: its
  result carries its status, and the other jobs of the stream finish with the
  results they have alone.
* A bounded device wait that runs out: under ERP_FLAG_EXPIRE_WAITS the row
  pass's wait on its bulk copies gives up at once (no copy stalls: each is
  still drained with the full limit), so the timeout path runs -- the status
  bit, the context's retirement, ERP_ETIMEDOUT on the host -- and the device
  stays usable.
"""
import numpy as np
import pytest

from designs import small_synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def R(built):
    import reda_erplacer_gb300 as R
    return R


def _with_nan(d, cell):
    import copy
    e = copy.deepcopy(d)
    e.x = e.x.copy()
    e.x[cell] = np.nan
    return e


def test_nan_position_retires_with_enan(R):
    d = small_synth(3000, seed=41)
    with R.Placement(d, (64, 64), 1.0, start_mode=1) as pl:
        pl.step()
        x, y = pl.positions()
        x[5] = np.nan
        pl.set_positions(x, y)
        with pytest.raises(R.ErpError) as e:
            for _ in range(3):
                pl.step()
        assert e.value.status == R.lib.ENAN
        assert "non-finite" in str(e.value)
        with pytest.raises(R.ErpError) as e2:   # retired: the next step reports the same
            pl.step()
        assert e2.value.status == R.lib.ENAN
    # a fresh context on the same design is unaffected
    with R.Placement(d, (64, 64), 1.0, start_mode=1) as pl:
        it, last = pl.run(5)
        assert it == 5 and np.isfinite(last["hpwl"])


@pytest.mark.parametrize("bins", [(64, 64), (256, 128), (512, 512)])
def test_bounded_wait_runs_out(R, bins):
    """Row passes of both copy-staged forms (one warp per row up to 256 bins, four
    warps per row from 512): the step reports ERP_ETIMEDOUT, the context stays
    retired, and a context without the flag on the same design runs normally."""
    d = small_synth(3000, seed=42)
    with R.Placement(d, bins, 1.0, start_mode=1, flags=R.lib.FLAG_EXPIRE_WAITS) as pl:
        with pytest.raises(R.ErpError) as e:
            pl.step()
        assert e.value.status == R.lib.ETIMEDOUT
        assert "wait limit" in str(e.value)
        x0, y0 = pl.positions()
        with pytest.raises(R.ErpError) as e2:   # retired: later steps report the same, move nothing
            pl.step()
        assert e2.value.status == R.lib.ETIMEDOUT
        x1, y1 = pl.positions()
        assert np.array_equal(x0, x1) and np.array_equal(y0, y1)
    with R.Placement(d, bins, 1.0, start_mode=1) as pl:
        it, last = pl.run(5)
        assert it == 5 and np.isfinite(last["hpwl"])


def test_unknown_flags_are_rejected(R):
    d = small_synth(500, seed=43)
    with pytest.raises(R.ErpError) as e:
        R.Placement(d, (64, 64), 1.0, flags=2)
    assert e.value.status == R.lib.EINVAL


def test_server_isolates_failed_jobs(R):
    from reda_erplacer_gb300.serving import Server, run_stream
    good = [(R.synth(c, int(1.05 * c), num_io=20, seed=950 + k), (64, 64)) for k, c in enumerate((3000, 5000, 4000))]
    bad_bins = (good[0][0], (100, 100))                 # not a power of two: erp_create rejects it
    nan_job = (_with_nan(good[1][0], 7), (64, 64))     # a NaN coordinate: rejected at set-up
    jobs = [good[0], bad_bins, good[1], nan_job, good[2]]
    sv = Server(max_active=4, hbm_budget_gb=8.0, max_iterations=60, stop_overflow=0.0, chunk=8)
    res = run_stream(sv, jobs, np.array([0.0, 0.0, 0.0, 0.01, 0.02]))
    sv.close()
    by_id = {r["job_id"]: r for r in res}
    assert len(by_id) == 5
    assert by_id[1]["status"] == R.lib.EINVAL
    assert by_id[3]["status"] == R.lib.EINVAL
    for i, (d, b) in ((0, good[0]), (2, good[1]), (4, good[2])):
        r = by_id[i]
        assert r["status"] == 0 and r["iterations"] == 60
        with R.Placement(d, b, 1.0, start_mode=1) as pl:
            it, last = pl.run(60)
        assert r["last"]["hpwl"] == last["hpwl"] and r["last"]["overflow"] == last["overflow"]


def test_out_of_range_positions_stay_in_bounds(R):
    d = small_synth(3000, seed=43)
    with R.Placement(d, (64, 64), 1.0, start_mode=1) as pl:
        pl.step()
        x, y = pl.positions()
        x[3], y[3] = 3.0e9, 5.0            # beyond 2^31 bins of the grid in x
        x[4], y[4] = -4.0e12, -7.0e10      # far below the die
        x[8], y[8] = 1.0e20, 1.0e20        # beyond isize in bin units
        pl.set_positions(x, y)
        try:
            for _ in range(3):
                pl.step()
            status = 0
        except R.ErpError as e:
            status = e.status
        assert status in (0, R.lib.ENAN)
        if status == 0:   # the update clamps every cell back onto the die
            x2, y2 = pl.positions()
            NM = d.num_movable
            assert np.all(np.isfinite(x2[:NM])) and np.all(x2[:NM] >= 0.0) and np.all(x2[:NM] <= d.die_w)
    with R.Placement(d, (64, 64), 1.0, start_mode=1) as pl:
        it, last = pl.run(5)
        assert it == 5 and np.isfinite(last["hpwl"])
