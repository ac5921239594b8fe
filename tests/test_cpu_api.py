"""CPU-only checks of the C ABI library: it loads, exports every symbol that
include/erplacer.h declares, rejects bad designs, fails loudly without a GPU,
and its synthetic netlist generator follows its documented rule."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT, gpu_available
from designs import build_design, edge_design


@pytest.fixture(scope="module")
def R(built):
    import reda_erplacer_gb300 as R
    return R


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "erplacer.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(erp_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol(R):
    lib = C.CDLL(R.lib.LIB_PATH)
    syms = declared_symbols()
    assert len(syms) >= 25
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    # the Python binding covers the whole header as well
    assert set(syms) <= set(R.lib.EXPORTS)


def test_status_strings(R):
    assert R.lib.status_string(0) == "ok"
    assert "sm_103" in R.lib.status_string(7)
    assert R.lib.load().erp_abi_version() == 1


@pytest.mark.skipif(gpu_available(), reason="checks the no-GPU failure path")
def test_no_gpu_fails_loudly(R):
    d = edge_design()
    with pytest.raises(R.ErpError) as e:
        R.Placement(d, (32, 16), 1.0)
    assert e.value.status == R.lib.ENODEV


def test_invalid_designs_rejected(R):
    d = edge_design()
    bad = [("bins not power of two", dict(num_bins=(30, 16))),
           ("bins too small", dict(num_bins=(8, 16)))]
    for _, kw in bad:
        with pytest.raises(R.ErpError) as e:
            R.Placement(d, **kw)
        assert e.value.status == R.lib.EINVAL
    # a pin in two nets
    d2 = edge_design()
    d2.net_pins = d2.net_pins.copy()
    d2.net_pins[1] = d2.net_pins[0]
    with pytest.raises(R.ErpError) as e:
        R.Placement(d2, (32, 16))
    assert e.value.status == R.lib.EINVAL and "more than one net" in str(e.value)
    # n_2nets claims a 3-pin net
    d3 = edge_design()
    d3.n_2nets = d3.n_2nets + 10
    with pytest.raises(R.ErpError) as e:
        R.Placement(d3, (32, 16))
    assert e.value.status == R.lib.EINVAL


def test_non_finite_and_malformed_inputs_rejected(R):
    """Validation runs before the device check, so these fail with ERP_EINVAL
    and a message whether or not a GPU is present."""
    import copy

    def variant(f):
        d = copy.deepcopy(edge_design())
        f(d)
        return d

    def set_item(name, i, v):
        def f(d):
            a = getattr(d, name).copy()
            a[i] = v
            setattr(d, name, a)
        return f

    cases = [
        ("instance width", set_item("w", 1, np.inf), {}, "instance geometry"),
        ("instance height", set_item("h", 0, np.nan), {}, "instance geometry"),
        ("pin offset", set_item("pin_ox", 2, np.nan), {}, "pin offset"),
        ("pin count", set_item("num_pins_f", 0, np.nan), {}, "num_pins_f"),
        ("negative pin count", set_item("num_pins_f", 1, -1.0), {}, "num_pins_f"),
        ("die", lambda d: setattr(d, "die_w", float("inf")), {}, "die"),
        ("movable area", lambda d: setattr(d, "movable_area", float("inf")), {}, "movable_area"),
        ("target density", lambda d: None, {"target_density": float("inf")}, "target density"),
        ("NaN target density", lambda d: None, {"target_density": float("nan")}, "target density"),
        ("cell utilisation", lambda d: setattr(d, "cell_utilization", float("nan")), {"target_density": -1.0},
         "target density"),
        ("pin listed twice", set_item("inst_pins", 1, None), {}, "inst_pins"),
    ]
    for what, f, kw, msg in cases:
        if what == "pin listed twice":
            def f(d):
                a = d.inst_pins.copy()
                i = int(np.argmax(np.diff(d.inst_pin_ptr) >= 2))   # an instance with two pins
                k = d.inst_pin_ptr[i]
                a[k + 1] = a[k]
                d.inst_pins = a
        d = variant(f)
        with pytest.raises(R.ErpError) as e:
            R.Placement(d, (32, 16), **({"target_density": 1.0} | kw))
        assert e.value.status == R.lib.EINVAL, what
        assert msg in str(e.value), (what, str(e.value))


def test_synth_is_deterministic_and_follows_rule(R):
    a = R.synth(5000, 5250, num_io=100, num_macros=4, utilization=0.65, seed=42)
    b = R.synth(5000, 5250, num_io=100, num_macros=4, utilization=0.65, seed=42)
    c = R.synth(5000, 5250, num_io=100, num_macros=4, utilization=0.65, seed=43)
    for k in ("x", "y", "w", "h", "pin_ox", "pin_inst", "net_ptr", "net_pins"):
        assert np.array_equal(getattr(a, k), getattr(b, k)), k
    assert not np.array_equal(a.pin_inst, c.pin_inst)
    NM = a.num_movable
    assert NM == 5000 and a.num_nodes == 5000 + 4 + 100 and a.num_nets == 5250
    deg = np.diff(a.net_ptr)
    # exact class shares; the rounding remainder goes to the two-pin class
    assert abs(a.n_2nets - 0.55 * 5250) <= 2 and np.all(deg[: a.n_2nets] == 2)
    assert np.all(deg[a.n_2nets:] >= 3) and deg.max() <= 128 + 100
    # widths are integer multiples of the 0.2 um site in [2, 16] sites, one row high
    sites = a.w[:NM] / 0.2
    assert np.allclose(sites, np.round(sites), atol=1e-4) and sites.min() >= 2 - 1e-4 and sites.max() <= 16 + 1e-4
    assert np.all(a.h[:NM] == 2.0)
    # distinct cells per net
    for e in range(a.num_nets):
        pins = a.net_pins[a.net_ptr[e]:a.net_ptr[e + 1]]
        insts = a.pin_inst[pins]
        assert len(set(insts.tolist())) == len(insts)
    # IO pins sit on the boundary with zero size
    io = slice(NM + 4, a.num_nodes)
    on_edge = (a.x[io] == 0) | (a.y[io] == 0) | np.isclose(a.x[io], a.die_w) | np.isclose(a.y[io], a.die_h)
    assert np.all(on_edge) and np.all(a.w[io] == 0)
    # utilisation of the free area
    free = a.die_w * a.die_h - np.sum(a.w[NM:NM + 4].astype(np.float64) * a.h[NM:NM + 4])
    assert a.cell_utilization == pytest.approx(a.movable_area / free, rel=1e-5)
    assert a.cell_utilization == pytest.approx(0.65, rel=1e-3)
    # macros do not overlap
    mx = [(a.x[i], a.y[i], a.w[i], a.h[i]) for i in range(NM, NM + 4)]
    for i in range(4):
        for j in range(i + 1, 4):
            xi, yi, wi, hi = mx[i]
            xj, yj, wj, hj = mx[j]
            assert xi + wi <= xj + 1e-3 or xj + wj <= xi + 1e-3 or yi + hi <= yj + 1e-3 or yj + hj <= yi + 1e-3


def test_bins_for_cells_rule(R):
    assert R.bins_for_cells(2000) == 64       # sqrt(2000)/2 = 22 -> 32 -> clamp 64
    assert R.bins_for_cells(200000) == 256    # 223.6 -> 256
    assert R.bins_for_cells(5_000_000) == 1024


def test_design_struct_roundtrip(R):
    d = edge_design()
    s = d.to_struct()
    back = R.Design.from_struct(s)
    for k in ("x", "pin_inst", "net_ptr", "net_pins", "inst_pin_ptr", "inst_pins"):
        assert np.array_equal(getattr(back, k), getattr(d, k))


def _c_struct_fields(txt, name):
    """Field names of `typedef struct <name> { ... } <name>;` in declaration order."""
    body = re.search(r"typedef struct %s \{(.*?)\} %s;" % (name, name), txt, flags=re.S).group(1)
    out = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        decl = re.sub(r"\[[^\]]*\]", "", decl)
        for part in decl.split(","):
            out.append(re.findall(r"[A-Za-z_][A-Za-z0-9_]*", part)[-1])
    return out


def _rust_struct_fields(txt, name):
    body = re.search(r"pub struct %s \{(.*?)\n\}" % name, txt, flags=re.S).group(1)
    return re.findall(r"pub ([a-z_0-9]+):", body)


def test_rust_binding_mirrors_the_header():
    """reda_erplacer_gb300/rust/ffi.rs (the binding the reference crate would
    add; no Rust toolchain here) declares every entry point of the header, and
    its #[repr(C)] structs list the header's fields in the same order."""
    h = open(os.path.join(ROOT, "include", "erplacer.h")).read()
    h = re.sub(r"/\*.*?\*/", "", h, flags=re.S)
    rs = open(os.path.join(ROOT, "reda_erplacer_gb300", "rust", "ffi.rs")).read()
    decl = set(re.findall(r"pub fn (erp_[a-z0-9_]+)\s*\(", rs))
    missing = [s for s in declared_symbols() if s not in decl]
    assert not missing, missing
    for st in ("erp_design", "erp_params", "erp_step_stats", "erp_scalars", "erp_server_params",
               "erp_job_result", "erp_synth_params", "erp_lefdef_stats", "erp_lefdef_params"):
        assert _c_struct_fields(h, st) == _rust_struct_fields(rs, st), st
