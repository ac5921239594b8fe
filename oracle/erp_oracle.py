"""ctypes binding of the oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU legs import this
module, as the checker or the timed CPU baseline.  The product package never
imports it.  Parity of the oracle against the reference binary is unpinned
(see erp_oracle.h); it is pinned against FP64 closed forms in tests/golden.

synth() builds the seeded synthetic netlists through liberp_synth.so, the
package's generator source compiled on its own, so that a CPU leg can make its
input design without loading the product library.
"""
import ctypes as C
import os
from types import SimpleNamespace

import numpy as np

from . import build_oracle

_lib = None
_synth_lib = None

f32p = C.POINTER(C.c_float)
f64p = C.POINTER(C.c_double)
i32p = C.POINTER(C.c_int32)
i64p = C.POINTER(C.c_int64)


class Design(C.Structure):
    _fields_ = [("num_nodes", C.c_int32), ("num_movable", C.c_int32), ("num_pins", C.c_int32),
                ("num_nets", C.c_int32), ("n_2nets", C.c_int32), ("_pad", C.c_int32),
                ("x", f32p), ("y", f32p), ("w", f32p), ("h", f32p), ("num_pins_f", f32p),
                ("pin_ox", f32p), ("pin_oy", f32p), ("pin_inst", i32p), ("net_ptr", i32p),
                ("net_pins", i32p), ("inst_pin_ptr", i32p), ("inst_pins", i32p),
                ("die_w", C.c_float), ("die_h", C.c_float), ("cell_utilization", C.c_float),
                ("movable_area", C.c_float)]


class Params(C.Structure):
    _fields_ = [("num_bins_x", C.c_int32), ("num_bins_y", C.c_int32),
                ("target_density", C.c_float), ("start_mode", C.c_int32),
                ("density_mode", C.c_int32), ("reduce_fp64", C.c_int32),
                ("num_threads", C.c_int32)]


class View(C.Structure):
    _fields_ = [("m", C.c_int32), ("n", C.c_int32), ("bin_w", C.c_float), ("bin_h", C.c_float),
                ("target_density", C.c_float), ("fixed_shift", C.c_int32),
                ("fixed_shift_init", C.c_int32),
                ("x", f32p), ("y", f32p), ("wl_grad_x", f32p), ("wl_grad_y", f32p),
                ("pin_grad_x", f32p), ("pin_grad_y", f32p), ("net_hpwl", f32p),
                ("dens_grad_x", f32p), ("dens_grad_y", f32p),
                ("clamped_w", f32p), ("clamped_h", f32p), ("offset_x", f32p), ("offset_y", f32p),
                ("ratio", f32p), ("initial_map", f32p), ("density_map", f32p),
                ("density_i64", i64p), ("auv", f32p), ("field_x", f32p), ("field_y", f32p),
                ("potential", f32p), ("prev_x", f32p), ("prev_y", f32p), ("prev_gx", f32p),
                ("prev_gy", f32p), ("iteration", C.c_int32), ("gamma", C.c_float),
                ("base_gamma", C.c_float), ("density_weight", C.c_float), ("alpha", C.c_float),
                ("beta", C.c_float), ("hpwl_initial", C.c_float), ("hpwl_current", C.c_float),
                ("hpwl_previous", C.c_float), ("overflow_current", C.c_float),
                ("overflow_previous", C.c_float), ("hpwl_initial_set", C.c_int32)]


class StepStats(C.Structure):
    _fields_ = [("hpwl", C.c_float), ("overflow", C.c_float), ("energy", C.c_float),
                ("density_weight", C.c_float), ("gamma", C.c_float), ("should_stop", C.c_int32)]


START_CENTER, START_DB = 0, 1
DENSITY_REFERENCE, DENSITY_FIXED = 0, 1


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        L = C.CDLL(path)
        L.erpo_create.restype = C.c_void_p
        L.erpo_create.argtypes = [C.POINTER(Design), C.POINTER(Params)]
        L.erpo_destroy.argtypes = [C.c_void_p]
        L.erpo_get_view.argtypes = [C.c_void_p, C.POINTER(View)]
        L.erpo_set_positions.argtypes = [C.c_void_p, f32p, f32p]
        L.erpo_set_nesterov_state.argtypes = [C.c_void_p, f32p, f32p, f32p, f32p, C.c_float, C.c_float]
        L.erpo_set_scheduler.argtypes = [C.c_void_p, C.c_int32, C.c_float, C.c_float]
        L.erpo_set_metrics.argtypes = [C.c_void_p] + [C.c_float] * 5
        L.erpo_compute_hpwl.restype = C.c_float
        L.erpo_compute_hpwl.argtypes = [C.c_void_p, C.c_float]
        L.erpo_compute_potential.restype = C.c_float
        L.erpo_compute_potential.argtypes = [C.c_void_p, C.c_int32, f32p]
        L.erpo_nesterov.argtypes = [C.c_void_p, C.c_int32]
        L.erpo_scheduler_update.argtypes = [C.c_void_p, C.c_float, C.c_float]
        L.erpo_should_stop.restype = C.c_int32
        L.erpo_should_stop.argtypes = [C.c_void_p]
        L.erpo_step.restype = C.c_int32
        L.erpo_step.argtypes = [C.c_void_p, C.POINTER(StepStats)]
        for nm in ("dct2", "idct2", "idct_idxst", "idxst_idct"):
            getattr(L, f"erpo_{nm}_f32").argtypes = [f32p, f32p, C.c_int32, C.c_int32]
            getattr(L, f"erpo_{nm}_f64").argtypes = [f64p, f64p, C.c_int32, C.c_int32]
        L.erpo_poisson_f32.argtypes = [f32p, C.c_int32, C.c_int32, C.c_float, C.c_float, f32p, f32p, f32p]
        L.erpo_poisson_f64.argtypes = [f64p, C.c_int32, C.c_int32, C.c_double, C.c_double, f64p, f64p, f64p]
        L.erpo_fixed_shift.restype = C.c_int32
        L.erpo_fixed_shift.argtypes = [C.c_double]
        _lib = L
    return _lib


def _p(a, t):
    return a.ctypes.data_as(t)


def make_design_struct(d):
    """Build a Design struct from an object with numpy-array attributes (see
    reda_erplacer_gb300.design.Design); keeps references alive on the struct."""
    keep = {}

    def arr(name, dt):
        a = np.ascontiguousarray(getattr(d, name), dtype=dt)
        keep[name] = a
        return a

    s = Design()
    s.num_nodes = int(d.num_nodes)
    s.num_movable = int(d.num_movable)
    s.num_pins = int(d.num_pins)
    s.num_nets = int(d.num_nets)
    s.n_2nets = int(d.n_2nets)
    for nm in ("x", "y", "w", "h", "num_pins_f", "pin_ox", "pin_oy"):
        setattr(s, nm, _p(arr(nm, np.float32), f32p))
    for nm in ("pin_inst", "net_ptr", "net_pins", "inst_pin_ptr", "inst_pins"):
        setattr(s, nm, _p(arr(nm, np.int32), i32p))
    s.die_w = float(d.die_w)
    s.die_h = float(d.die_h)
    s.cell_utilization = float(d.cell_utilization)
    s.movable_area = float(d.movable_area)
    s._keep = keep
    return s


def _arr(ptr, n, dt=np.float32):
    if n == 0:
        return np.zeros(0, dtype=dt)
    return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dt, copy=True)


class Oracle:
    """Oracle placement state mirroring the reference's Placement struct."""

    def __init__(self, design, m, n, target_density=-1.0, start_mode=START_CENTER,
                 density_mode=DENSITY_FIXED, reduce_fp64=1, num_threads=0):
        self.L = lib()
        self.design = design
        self._ds = make_design_struct(design)
        self._p = Params(m, n, float(target_density), start_mode, density_mode, reduce_fp64,
                         num_threads)
        self.h = self.L.erpo_create(C.byref(self._ds), C.byref(self._p))
        if not self.h:
            raise ValueError("oracle: invalid parameters (bin counts must be powers of two >= 4)")
        self.N = int(design.num_nodes)
        self.P = int(design.num_pins)
        self.E = int(design.num_nets)
        self.m, self.n = m, n

    def close(self):
        if self.h:
            self.L.erpo_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def view(self):
        v = View()
        self.L.erpo_get_view(self.h, C.byref(v))
        return v

    def get(self, name):
        v = self.view()
        N, P, E, mn = self.N, self.P, self.E, self.m * self.n
        sizes = {"x": N, "y": N, "wl_grad_x": N, "wl_grad_y": N, "pin_grad_x": P,
                 "pin_grad_y": P, "net_hpwl": E, "dens_grad_x": N, "dens_grad_y": N,
                 "clamped_w": N, "clamped_h": N, "offset_x": N, "offset_y": N, "ratio": N,
                 "initial_map": mn, "density_map": mn, "auv": mn, "field_x": mn,
                 "field_y": mn, "potential": mn, "prev_x": N, "prev_y": N, "prev_gx": N,
                 "prev_gy": N}
        if name == "density_i64":
            return _arr(v.density_i64, mn, np.int64)
        if name in sizes:
            return _arr(getattr(v, name), sizes[name])
        return getattr(v, name)

    def set_positions(self, x, y):
        x = np.ascontiguousarray(x, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        self.L.erpo_set_positions(self.h, _p(x, f32p), _p(y, f32p))

    def set_nesterov_state(self, px, py, pgx, pgy, alpha, beta):
        a = [np.ascontiguousarray(t, np.float32) for t in (px, py, pgx, pgy)]
        self.L.erpo_set_nesterov_state(self.h, *[_p(t, f32p) for t in a], float(alpha), float(beta))

    def set_scheduler(self, iteration, gamma, dw):
        self.L.erpo_set_scheduler(self.h, int(iteration), float(gamma), float(dw))

    def set_metrics(self, hpwl_initial, hpwl_current, hpwl_previous, overflow_current, overflow_previous):
        self.L.erpo_set_metrics(self.h, float(hpwl_initial), float(hpwl_current), float(hpwl_previous),
                                float(overflow_current), float(overflow_previous))

    def load_state(self, g):
        """Copy a GPU placement's whole loop state (positions, Nesterov history,
        scheduler and optimiser scalars) into the oracle, so that both continue
        from the same state."""
        x, y = g.positions()
        self.set_positions(x, y)
        s = g.scalars()
        self.set_nesterov_state(g.array("PREV_X"), g.array("PREV_Y"), g.array("PREV_GX"),
                                g.array("PREV_GY"), s["alpha"], s["beta"])
        self.set_scheduler(s["iteration"], s["gamma"], s["density_weight"])
        self.set_metrics(s["hpwl_initial"], s["hpwl_current"], s["hpwl_previous"], s["overflow_current"],
                         s["overflow_previous"])

    def compute_hpwl(self, gamma):
        return float(self.L.erpo_compute_hpwl(self.h, float(gamma)))

    def compute_potential(self, iteration):
        e = C.c_float(0)
        ovf = self.L.erpo_compute_potential(self.h, int(iteration), C.byref(e))
        return float(e.value), float(ovf)

    def nesterov(self, iteration):
        self.L.erpo_nesterov(self.h, int(iteration))

    def scheduler_update(self, hpwl, overflow):
        self.L.erpo_scheduler_update(self.h, float(hpwl), float(overflow))

    def step(self):
        st = StepStats()
        stop = self.L.erpo_step(self.h, C.byref(st))
        return {"hpwl": st.hpwl, "overflow": st.overflow, "energy": st.energy,
                "density_weight": st.density_weight, "gamma": st.gamma,
                "should_stop": bool(stop)}


def transform(name, x, dtype=np.float32):
    """Run one standalone transform (dct2 / idct2 / idct_idxst / idxst_idct)."""
    L = lib()
    x = np.ascontiguousarray(x, dtype)
    m, n = x.shape
    out = np.zeros_like(x)
    sfx, pt = ("f32", f32p) if dtype == np.float32 else ("f64", f64p)
    getattr(L, f"erpo_{name}_{sfx}")(_p(x, pt), _p(out, pt), m, n)
    return out


def poisson(rho, bin_w, bin_h, dtype=np.float32):
    L = lib()
    rho = np.ascontiguousarray(rho, dtype)
    m, n = rho.shape
    fx, fy, pot = np.zeros_like(rho), np.zeros_like(rho), np.zeros_like(rho)
    sfx, pt = ("f32", f32p) if dtype == np.float32 else ("f64", f64p)
    getattr(L, f"erpo_poisson_{sfx}")(_p(rho, pt), m, n, bin_w, bin_h, _p(fx, pt), _p(fy, pt),
                                      _p(pot, pt))
    return fx, fy, pot


def fixed_shift(total_area):
    return int(lib().erpo_fixed_shift(float(total_area)))


class SynthParams(C.Structure):
    """erp_synth_params of include/erplacer.h."""
    _fields_ = [("seed", C.c_int64), ("num_cells", C.c_int32), ("num_nets", C.c_int32),
                ("num_io", C.c_int32), ("num_macros", C.c_int32), ("macro_area_frac", C.c_float),
                ("utilization", C.c_float), ("site_w", C.c_float), ("row_h", C.c_float),
                ("min_sites", C.c_int32), ("max_sites", C.c_int32), ("jitter_frac", C.c_float)]


def synth_lib():
    global _synth_lib
    if _synth_lib is None:
        build_oracle.build_synth()
        L = C.CDLL(build_oracle.SYNTH_LIB)
        L.erp_synth_create.restype = C.c_int
        L.erp_synth_create.argtypes = [C.POINTER(SynthParams), C.POINTER(C.c_void_p)]
        L.erp_synth_design.restype = C.c_int
        L.erp_synth_design.argtypes = [C.c_void_p, C.POINTER(Design)]
        L.erp_synth_destroy.argtypes = [C.c_void_p]
        _synth_lib = L
    return _synth_lib


def synth(num_cells, num_nets=None, num_io=0, num_macros=0, macro_area_frac=0.015, utilization=0.7,
          seed=1, site_w=0.2, row_h=2.0, min_sites=2, max_sites=16, jitter_frac=0.001):
    """The package's seeded synthetic netlist (same arguments as
    reda_erplacer_gb300.synth, same bits), as a namespace of numpy arrays."""
    L = synth_lib()
    p = SynthParams(int(seed), int(num_cells), int(num_nets if num_nets else round(1.05 * num_cells)),
                    int(num_io), int(num_macros), float(macro_area_frac), float(utilization),
                    float(site_w), float(row_h), int(min_sites), int(max_sites), float(jitter_frac))
    h = C.c_void_p()
    st = L.erp_synth_create(C.byref(p), C.byref(h))
    if st != 0:
        raise ValueError(f"synthetic netlist: invalid parameters (status {st})")
    try:
        d = Design()
        if L.erp_synth_design(h, C.byref(d)) != 0:
            raise ValueError("synthetic netlist: no design")
        N, P, E = d.num_nodes, d.num_pins, d.num_nets
        net_ptr = _arr(d.net_ptr, E + 1, np.int32)
        inst_ptr = _arr(d.inst_pin_ptr, N + 1, np.int32)
        return SimpleNamespace(
            num_nodes=N, num_movable=d.num_movable, num_pins=P, num_nets=E, n_2nets=d.n_2nets,
            x=_arr(d.x, N), y=_arr(d.y, N), w=_arr(d.w, N), h=_arr(d.h, N),
            num_pins_f=_arr(d.num_pins_f, N), pin_ox=_arr(d.pin_ox, P), pin_oy=_arr(d.pin_oy, P),
            pin_inst=_arr(d.pin_inst, P, np.int32), net_ptr=net_ptr,
            net_pins=_arr(d.net_pins, int(net_ptr[-1]), np.int32), inst_pin_ptr=inst_ptr,
            inst_pins=_arr(d.inst_pins, int(inst_ptr[-1]), np.int32), die_w=float(d.die_w),
            die_h=float(d.die_h), cell_utilization=float(d.cell_utilization),
            movable_area=float(d.movable_area))
    finally:
        L.erp_synth_destroy(h)
