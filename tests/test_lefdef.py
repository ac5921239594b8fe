"""LEF/DEF ingest, export and placed-DEF hand-off (host code of the library, no
GPU needed): the database a hand-written ISPD-style LEF/DEF pair yields,
worked out by hand below, the round trip of synthetic designs through
LEF/DEF, the placed DEF, and the reader's errors."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, gpu_available

GOLD = os.path.join(ROOT, "tests", "golden", "lefdef")
TECH = os.path.join(GOLD, "tiny_tech.lef")
CELLS = os.path.join(GOLD, "tiny_cells.lef")
DEF = os.path.join(GOLD, "tiny.def")


@pytest.fixture(scope="module")
def R(built):
    import reda_erplacer_gb300 as R
    return R


@pytest.fixture(scope="module")
def LD(R):
    from reda_erplacer_gb300 import lefdef
    return lefdef


def f32(v):
    return np.asarray(v, np.float64).astype(np.float32)


# --- the hand-written design --------------------------------------------------
# DEF units 2000 / um, LEF grid 1000 / um, die (2000, 4000)-(42000, 44000) -> 20 x 20 um at the origin.
# INV 0.6 x 2.0: A = centre of RECT 0.1 0.4 0.2 0.8 = (0.15, 0.6); Z = bbox of POLYGON x 0.4-0.5,
#   y 0.2-1.6 and RECT 0.3 1.5 0.5 1.8 = x 0.3-0.5, y 0.2-1.8 -> (0.4, 1.0).
# SHIFTED 1.0 x 2.0, ORIGIN 0.1 0.2: Y = (0.1, 0.1) + origin = (0.2, 0.3); NOSHAPE = macro centre (0.5, 1.0).
# RAM 10 x 4: D = (9.9, 1.1) (the VIA point lies inside the RECT).
# Orientations (offset from the oriented footprint's lower-left, footprint w x h):
#   N (px, py); FS (px, h-py); E (py, w-px), footprint swapped; FW (py, px), swapped; S (w-px, h-py);
#   FN (w-px, py).
# Instances: movable u1 u2 u3 u4(UNPLACED) u5, fixed ram0 (FIXED) u6 (COVER), then PINS in1 out1 vdd.
NAMES = ["u1", "u2", "u3", "u4", "u5", "ram0", "u6", "in1", "out1", "vdd"]
X = [1.0, 2.0, 3.0, 0.0, 4.0, 9.0, 14.0, 0.0, 20.0, 0.0]
Y = [2.0, 2.0, 2.0, 0.0, 4.0, 8.0, 13.0, 10.0, 13.0, 0.0]
W = [0.6, 0.6, 2.0, 0.6, 2.0, 10.0, 0.6, 0.0, 0.0, 0.0]
H = [2.0, 2.0, 0.6, 2.0, 1.0, 4.0, 2.0, 0.0, 0.0, 0.0]
# nets: n2 and n4 (two pins) first, then n1 n3 n5 n6 (n5 without the wildcard); "empty" dropped
NETS = ["n2", "n4", "n1", "n3", "n5", "n6"]
NET_PTR = [0, 2, 4, 7, 10, 13, 14]
PIN_INST = [0, 8, 2, 4, 7, 0, 1, 1, 2, 3, 4, 5, 6, 3]
POX = [0.4, 0.05, 1.0, 0.3, 0.1, 0.15, 0.15, 0.4, 0.6, 0.15, 1.0, 0.1, 0.45, 0.4]
POY = [1.0, 0.05, 0.2, 0.2, 0.0, 0.6, 1.4, 1.0, 0.45, 0.6, 0.5, 2.9, 0.6, 1.0]
# in1: LAYER ( -100 0 ) ( 100 400 ) centre (0, 200) DEF units, E about the point -> (200, 0) = (0.1, 0) um
# out1: POLYGON centre (100, 100) -> (0.05, 0.05) um


def test_reads_hand_written_design(LD):
    with LD.Netlist.read([TECH, CELLS], DEF) as nl:
        d = nl.design()
        st = nl.stats()
        assert [nl.node_name(i) for i in range(d.num_nodes)] == NAMES
        assert [nl.net_name(e) for e in range(d.num_nets)] == NETS
    assert (d.num_nodes, d.num_movable, d.num_pins, d.num_nets, d.n_2nets) == (10, 5, 14, 6, 2)
    for k, v in (("x", X), ("y", Y), ("w", W), ("h", H), ("pin_ox", POX), ("pin_oy", POY)):
        np.testing.assert_array_equal(getattr(d, k), f32(v), err_msg=k)
    np.testing.assert_array_equal(d.net_ptr, NET_PTR)
    np.testing.assert_array_equal(d.net_pins, np.arange(14))
    np.testing.assert_array_equal(d.pin_inst, PIN_INST)
    np.testing.assert_array_equal(d.num_pins_f, f32([2, 2, 2, 2, 2, 1, 1, 1, 1, 0]))
    np.testing.assert_array_equal(d.inst_pin_ptr, [0, 2, 4, 6, 8, 10, 11, 12, 13, 14, 14])
    np.testing.assert_array_equal(d.inst_pins, [0, 5, 6, 7, 2, 8, 9, 13, 3, 10, 11, 12, 4, 1])
    assert d.die_w == 20.0 and d.die_h == 20.0
    # movable 4 x 0.6 x 2 + 2 x 1; fixed inside the die: 10 x 4 + 0.6 x 2
    assert d.movable_area == np.float32(6.8)
    assert d.cell_utilization == np.float32(6.8 / (400.0 - 41.2))
    assert st["num_fixed"] == 2 and st["num_io"] == 3 and st["num_macros"] == 3
    assert st["num_dropped_nets"] == 1           # "empty"
    assert st["num_skipped_conns"] == 2          # ( * VSS ) and MUSTJOIN
    assert st["num_unplaced_io"] == 1            # vdd
    assert (st["def_dbu"], st["lef_dbu"]) == (2000, 1000)
    assert st["die"] == (2000, 4000, 42000, 44000)


def test_read_db_matches_netlist_and_one_file_order(LD):
    d1 = LD.read_db([TECH, CELLS], DEF)
    # a later LEF can only add or replace macros: cells first then tech gives the same database
    d2 = LD.read_db([CELLS, TECH], DEF)
    for k in ("x", "y", "w", "h", "pin_ox", "pin_oy", "pin_inst", "net_ptr", "inst_pins"):
        np.testing.assert_array_equal(getattr(d1, k), getattr(d2, k))


def test_placed_def_changes_only_movable_clauses(LD, tmp_path):
    out = str(tmp_path / "placed.def")
    with LD.Netlist.read([TECH, CELLS], DEF) as nl:
        d = nl.design()
        x = d.x.copy()
        y = d.y.copy()
        x[:5] = [1.25, 5.5, 7.0, 8.0005, 12.34567]
        y[:5] = [6.0, 6.0, 2.0, 18.0, 0.5]
        x[5:] = -99.0   # fixed and IO entries are ignored
        nl.write_placed(x, y, out)
    src = open(DEF).read().splitlines()
    got = open(out).read().splitlines()
    assert len(src) == len(got)
    changed = [(a, b) for a, b in zip(src, got) if a != b]
    assert [b for _, b in changed] == [
        "- u1 INV + PLACED ( 4500 16000 ) N ;",
        "- u2 INV + PLACED ( 13000 16000 ) FS ;",
        "- u3 INV + SOURCE NETLIST + PLACED ( 16000 8000 ) E + WEIGHT 2 ;",
        "  + PLACED ( 18001 40000 ) N ;",
        "- u5 SHIFTED + PLACED ( 26691 5000 ) FW ;",
    ]
    p = LD.read_db([TECH, CELLS], out)
    np.testing.assert_array_equal(p.x[:5], f32([1.25, 5.5, 7.0, 8.0005, 12.3455]))
    np.testing.assert_array_equal(p.y[:5], f32([6.0, 6.0, 2.0, 18.0, 0.5]))
    np.testing.assert_array_equal(p.x[5:], d.x[5:])
    for k in ("w", "h", "pin_ox", "pin_oy", "pin_inst", "net_ptr", "inst_pins"):
        np.testing.assert_array_equal(getattr(p, k), getattr(d, k))


def test_placed_def_inserts_a_missing_clause(LD, tmp_path):
    src = open(DEF).read().replace("- u1 INV + PLACED ( 4000 8000 ) N ;", "- u1 INV ;")
    path = tmp_path / "noclause.def"
    path.write_text(src)
    out = str(tmp_path / "placed.def")
    with LD.Netlist.read([TECH, CELLS], str(path)) as nl:
        d = nl.design()
        assert d.x[0] == 0.0 and d.y[0] == 0.0    # no location: the die corner
        nl.write_placed(d.x + 1.0, d.y + 1.0, out)
    assert "- u1 INV + PLACED ( 4000 6000 ) N ;" in open(out).read()
    assert LD.read_db([TECH, CELLS], out).x[0] == 1.0


@pytest.mark.parametrize("seed,cells,macros,io", [(3, 1500, 0, 40), (7, 3000, 4, 60)])
def test_synthetic_round_trip(R, LD, tmp_path, seed, cells, macros, io):
    d = R.synth(cells, int(cells * 1.05), num_io=io, num_macros=macros, macro_area_frac=0.015,
                utilization=0.65, seed=seed)
    a_lef, a_def = str(tmp_path / "a.lef"), str(tmp_path / "a.def")
    q = LD.write_lefdef(d, a_lef, a_def)
    r = LD.read_db(a_lef, a_def)
    # structure survives exactly; coordinates move to the 1/2000 um grid
    for k in ("num_nodes", "num_movable", "num_pins", "num_nets", "n_2nets"):
        assert getattr(r, k) == getattr(d, k), k
    for k in ("net_ptr", "net_pins", "pin_inst", "inst_pin_ptr", "inst_pins", "num_pins_f"):
        np.testing.assert_array_equal(getattr(r, k), getattr(d, k), err_msg=k)
    for k in ("x", "y", "w", "h", "pin_ox", "pin_oy"):
        assert np.abs(getattr(r, k).astype(np.float64) - getattr(d, k)).max() <= 0.5 / 2000 + 1e-5, k
        # the exported design is what the files carry, bit for bit
        np.testing.assert_array_equal(getattr(r, k).view(np.int32), getattr(q, k).view(np.int32), err_msg=k)
    assert abs(r.die_w - d.die_w) <= 0.5 / 2000 + 1e-4
    assert abs(r.cell_utilization - d.cell_utilization) < 1e-4
    assert r.movable_area == q.movable_area
    # a second export of the read design gives the same files byte for byte
    b_lef, b_def = str(tmp_path / "b.lef"), str(tmp_path / "b.def")
    LD.write_lefdef(r, b_lef, b_def)
    assert open(a_lef, "rb").read() == open(b_lef, "rb").read()
    assert open(a_def, "rb").read() == open(b_def, "rb").read()


def test_round_trip_of_the_hand_written_design(LD, tmp_path):
    """Export of a read design keeps its database (names are regenerated)."""
    d = LD.read_db([TECH, CELLS], DEF)
    lef, de = str(tmp_path / "t.lef"), str(tmp_path / "t.def")
    LD.write_lefdef(d, lef, de, dbu=2000, site_w=0.2, row_h=2.0)
    r = LD.read_db(lef, de)
    for k in ("x", "y", "w", "h", "pin_ox", "pin_oy", "num_pins_f"):
        np.testing.assert_array_equal(getattr(r, k), getattr(d, k), err_msg=k)
    for k in ("net_ptr", "net_pins", "pin_inst", "inst_pin_ptr", "inst_pins"):
        np.testing.assert_array_equal(getattr(r, k), getattr(d, k), err_msg=k)
    assert (r.n_2nets, r.num_movable) == (d.n_2nets, d.num_movable)


def test_small_workload_through_lefdef(R, LD, tmp_path):
    """20,000 cells / 21,000 nets / 400 IO pins, written as LEF/DEF and read back."""
    d, cfg = R.workload_small()
    lef, de = str(tmp_path / "s.lef"), str(tmp_path / "s.def")
    q = LD.write_lefdef(d, lef, de)
    r = LD.read_db(lef, de)
    assert (r.num_nodes, r.num_movable, r.num_nets, r.num_pins) == (20400, 20000, 21000, d.num_pins)
    np.testing.assert_array_equal(r.net_pins, d.net_pins)
    np.testing.assert_array_equal(r.x, q.x)
    assert os.path.getsize(de) > 1e6


ERRORS = [
    ("- u1 INV + PLACED", "- u1 NAND9 + PLACED", "component 'u1' of unknown macro 'NAND9'"),
    ("( u1 A ) ( u2 A )", "( u1 Q ) ( u2 A )", "macro 'INV' has no pin 'Q'"),
    ("( u2 Z ) ( u3 A )", "( u2 Z ) ( u9 A )", "unknown component 'u9'"),
    ("( PIN in1 )", "( PIN in9 )", "unknown pin 'in9'"),
    ("+ PLACED ( 6000 8000 ) FS", "+ PLACED ( 6000 8000 ) XX", "bad orientation 'XX'"),
    ("DIEAREA ( 2000 4000 ) ( 42000 4000 ) ( 42000 44000 ) ( 2000 44000 ) ;", "", "no DIEAREA"),
    ("END DESIGN", "NETS 1 ;\n- x ( u1", "unexpected end of file"),
]


@pytest.mark.parametrize("old,new,msg", ERRORS)
def test_reader_errors_name_file_and_line(R, LD, tmp_path, old, new, msg):
    src = open(DEF).read()
    assert old in src
    path = tmp_path / "bad.def"
    path.write_text(src.replace(old, new, 1))
    with pytest.raises(R.ErpError) as e:
        LD.read_db([TECH, CELLS], str(path))
    assert e.value.status == R.lib.EINVAL
    assert msg in str(e.value)
    assert "bad.def" in str(e.value)
    if msg not in ("no DIEAREA", "unexpected end of file"):
        line = src.replace(old, new, 1).splitlines().index(
            next(ln for ln in src.replace(old, new, 1).splitlines() if new.split("\n")[0] in ln)) + 1
        assert f"bad.def:{line}:" in str(e.value)


def test_reader_errors_in_lef_and_missing_files(R, LD, tmp_path):
    bad = tmp_path / "bad.lef"
    bad.write_text(open(CELLS).read().replace("END A\n", "END B\n", 1))
    with pytest.raises(R.ErpError, match=r"bad.lef:\d+: expected 'END A'"):
        LD.read_db([TECH, str(bad)], DEF)
    with pytest.raises(R.ErpError, match="cannot read"):
        LD.read_db([TECH, CELLS], str(tmp_path / "missing.def"))
    with pytest.raises(R.ErpError, match="cannot read"):
        LD.read_db(str(tmp_path / "missing.lef"), DEF)


def test_cli_reads_and_fails_loudly_without_a_gpu(R, built, tmp_path):
    """The command-line driver parses the reference's flags and reads the design;
    with no GPU the placement step fails with ERP_ENODEV (no CPU fallback)."""
    if gpu_available():
        pytest.skip("a GPU is present: covered by the GPU tests")
    from reda_erplacer_gb300 import build
    r = subprocess.run([build.CLI, "-l", TECH, "-l", CELLS, "-d", DEF, "--iterations", "3", "--bins", "16x16"],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 1
    assert "Reading DB took" in r.stdout and "10 instances (5 movable, 2 fixed, 3 IO pins)" in r.stdout
    assert "sm_103" in r.stderr or "no CUDA" in r.stderr or "device" in r.stderr
    r = subprocess.run([build.CLI, "-d", DEF], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2 and "usage" in r.stderr


def test_cli_rejects_bad_arguments_and_inputs(R, built, tmp_path):
    """Flag errors exit 2 with usage; unreadable inputs and parameters the library
    rejects exit 1 with the reason, before any device work (GPU or not)."""
    from reda_erplacer_gb300 import build
    base = [build.CLI, "-l", TECH, "-l", CELLS, "-d", DEF]
    usage = [["--bogus"], ["--precision", "fp16"], ["--bins", "64x"], ["--bins", "64x64x"], ["--iterations"],
             ["--iterations", "-3"], ["--iterations", "12abc"], ["--start", "left"], ["--target-density", "nan"],
             ["--target-density", "abc"], ["--stop-overflow", "0.1x"], ["--device", "one"]]
    for extra in usage:
        r = subprocess.run(base + extra, capture_output=True, text=True, timeout=60)
        assert r.returncode == 2, (extra, r.returncode, r.stderr)
        assert "error" in r.stderr or "usage" in r.stderr, extra
    r = subprocess.run([build.CLI, "-l", TECH, "-l", CELLS, "-d", str(tmp_path / "missing.def")],
                       capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "missing.def" in r.stderr
    for extra, msg in ((["--bins", "30x16"], "powers of two"), (["--target-density", "0"], "target density"),
                       (["--precision", "tf32", "--bins", "64x64"], "multiples of 128")):
        r = subprocess.run(base + extra, capture_output=True, text=True, timeout=60)
        assert r.returncode == 1 and msg in r.stderr, (extra, r.returncode, r.stderr)
