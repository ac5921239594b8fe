"""GPU runs of designs that come in through LEF/DEF: the hand-written ISPD-style
pair (one-pin nets, unplaced and unconnected IO pins, rotated and mirrored
instances) stage by stage against the oracle, the 20k-cell workload written as
LEF/DEF and placed end to end against the oracle, and the command-line driver
against the Python API (same positions, placed DEF, snapshots)."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, rel_l2
from designs import spread_positions

pytestmark = pytest.mark.gpu

GOLD = os.path.join(ROOT, "tests", "golden", "lefdef")
TECH = os.path.join(GOLD, "tiny_tech.lef")
CELLS = os.path.join(GOLD, "tiny_cells.lef")
DEF = os.path.join(GOLD, "tiny.def")
TOL = 1e-5


@pytest.fixture(scope="module")
def R(built):
    import reda_erplacer_gb300 as R
    return R


@pytest.fixture(scope="module")
def O(built):
    from oracle import erp_oracle as O
    return O


@pytest.fixture(scope="module")
def LD(R):
    from reda_erplacer_gb300 import lefdef
    return lefdef


@pytest.fixture(scope="module")
def small_files(R, LD, tmp_path_factory):
    """The 20,000-cell / 21,000-net / 400-IO workload written as LEF/DEF."""
    d, cfg = R.workload_small()
    base = tmp_path_factory.mktemp("small")
    lef, de = str(base / "small.lef"), str(base / "small.def")
    LD.write_lefdef(d, lef, de)
    return lef, de, cfg


@pytest.mark.parametrize("m,n", [(16, 16), (16, 32)])
def test_hand_written_design_stages(R, O, LD, m, n):
    d = LD.read_db([TECH, CELLS], DEF)
    xy = spread_positions(d, seed=5, frac=0.6)
    o = O.Oracle(d, m, n, target_density=1.0, start_mode=O.START_DB, density_mode=O.DENSITY_FIXED, reduce_fp64=1)
    g = R.Placement(d, (m, n), 1.0, start_mode=1)
    o.set_positions(*xy)
    g.set_positions(*xy)
    try:
        assert np.array_equal(g.array("INITIAL"), o.get("initial_map"))
        for gamma in (0.5, 4.0):
            ho = o.compute_hpwl(gamma)
            hg = g.compute_hpwl(gamma)
            assert abs(hg - ho) <= 1e-6 * abs(ho)
            assert rel_l2(g.array("WL_GRAD_X"), o.get("wl_grad_x")) <= TOL
            assert rel_l2(g.array("WL_GRAD_Y"), o.get("wl_grad_y")) <= TOL
            # the one-pin net n6 has zero length on both sides
            assert g.array("NET_HPWL")[5] == 0.0 and o.get("net_hpwl")[5] == 0.0
        _, ovo = o.compute_potential(0)
        _, ovg = g.compute_potential(0)
        assert np.array_equal(g.array("DENSITY_I64"), o.get("density_i64"))
        assert abs(ovg - ovo) <= 1e-6 * max(abs(ovo), 1e-12)
        assert rel_l2(g.array("FIELD_X"), o.get("field_x")) <= TOL
        assert rel_l2(g.array("FIELD_Y"), o.get("field_y")) <= TOL
        # five movable cells on a coarse grid: overflow jumps between bins, so the
        # free-running comparison stays short
        for it in range(3):
            so = o.step()
            g.step()
        sg = g.last_stats
        assert abs(sg["hpwl"] - so["hpwl"]) <= 0.005 * so["hpwl"]
        assert abs(sg["overflow"] - so["overflow"]) <= 0.005
    finally:
        g.close()
        o.close()


def test_small_workload_from_lefdef_end_to_end(R, O, LD, small_files):
    """The 20k-cell workload read from LEF/DEF, 60 iterations from its jittered
    start: HPWL within 0.5 % and overflow within 0.005 of the oracle."""
    lef, de, cfg = small_files
    d = LD.read_db(lef, de)
    o = O.Oracle(d, 256, 256, target_density=1.0, start_mode=O.START_DB, density_mode=O.DENSITY_FIXED,
                 reduce_fp64=1)
    g = R.Placement(d, (256, 256), 1.0, start_mode=1)
    try:
        for i in range(60):
            so = o.step()
            g.step()
        sg = g.last_stats
        assert abs(sg["hpwl"] - so["hpwl"]) <= 0.005 * so["hpwl"]
        assert abs(sg["overflow"] - so["overflow"]) <= 0.005
    finally:
        g.close()
        o.close()


def test_cli_matches_python_api(R, LD, small_files, tmp_path):
    """erplacer_gb300 -l LEF -d DEF --iterations 60: the placed DEF holds the
    positions the Python API reaches on the same design (both runs are
    deterministic), rounded to DEF units; snapshots at 0, 50 and the end."""
    from reda_erplacer_gb300 import build
    lef, de, cfg = small_files
    out = str(tmp_path / "placed.def")
    img = tmp_path / "images"
    img.mkdir()
    r = subprocess.run([build.CLI, "-l", lef, "-d", de, "--iterations", "60", "-v", "--bins", "256x256",
                        "--target-density", "1.0", "--out", out, "--images", str(img)],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    assert "Bins:" in r.stdout and "Placement took" in r.stdout and "wrote" in r.stdout
    assert sorted(os.listdir(img)) == ["solution_0000000.ppm", "solution_0000050.ppm", "solution_0000060.ppm"]
    d = LD.read_db(lef, de)
    with R.Placement(d, (256, 256), 1.0) as g:
        for _ in range(60):
            g.step()
        x, y = g.positions()
        snap = g.snapshot_placement()
    p = LD.read_db(lef, out)
    NM = d.num_movable
    qx = (np.floor(x[:NM].astype(np.float64) * 2000 + 0.5) / 2000).astype(np.float32)   # half away from 0
    qy = (np.floor(y[:NM].astype(np.float64) * 2000 + 0.5) / 2000).astype(np.float32)
    np.testing.assert_array_equal(p.x[:NM], qx)
    np.testing.assert_array_equal(p.y[:NM], qy)
    np.testing.assert_array_equal(p.x[NM:], d.x[NM:])
    with open(img / "solution_0000060.ppm", "rb") as f:
        h, w = snap.shape[:2]
        assert f.read(len(b"P6\n%d %d\n255\n" % (w, h))) == b"P6\n%d %d\n255\n" % (w, h)
        assert np.array_equal(np.frombuffer(f.read(), np.uint8).reshape(h, w, 3), snap)


def test_cli_precision_and_early_stop(R, LD, small_files, tmp_path):
    """--precision tf32 (tensor-core solve), --stop-overflow (retire early) and
    --start db (keep the DEF coordinates) through the command-line driver."""
    from reda_erplacer_gb300 import build
    lef, de, cfg = small_files
    out = str(tmp_path / "placed.def")
    r = subprocess.run([build.CLI, "-l", lef, "-d", de, "--iterations", "450", "--bins", "256x256",
                        "--target-density", "1.0", "--precision", "tf32", "--stop-overflow", "0.5",
                        "--start", "db", "--out", out, "--images", str(tmp_path)],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    line = next(ln for ln in r.stdout.splitlines() if ln.startswith("[INFO] Placement took"))
    ran = int(line.split(":")[1].split("iterations")[0])
    over = float(line.rsplit("overflow", 1)[1])
    assert 0 < ran < 450 and over <= 0.5
    p = LD.read_db(lef, out)
    assert np.isfinite(p.x).all() and np.isfinite(p.y).all()
    # an unsupported precision for the grid is reported, not run
    r = subprocess.run([build.CLI, "-l", lef, "-d", de, "--bins", "64x64", "--precision", "bf16x3"],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 1 and "error" in r.stderr
