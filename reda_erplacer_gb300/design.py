"""Placement database container (the erp_design view of include/erplacer.h) and
the seeded synthetic netlist workloads.

A Design holds numpy arrays in the layout the reference loop reads from
reda-db's DB<T>: movable instances first, per-instance pin counts as float,
pin offsets from the instance's lower-left corner, net CSR with the two-pin
nets first, and the per-instance pin lists (macro_2_pins).
"""
import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import lib as L


@dataclass
class Design:
    num_nodes: int
    num_movable: int
    num_pins: int
    num_nets: int
    n_2nets: int
    x: np.ndarray
    y: np.ndarray
    w: np.ndarray
    h: np.ndarray
    num_pins_f: np.ndarray
    pin_ox: np.ndarray
    pin_oy: np.ndarray
    pin_inst: np.ndarray
    net_ptr: np.ndarray
    net_pins: np.ndarray
    inst_pin_ptr: np.ndarray
    inst_pins: np.ndarray
    die_w: float
    die_h: float
    cell_utilization: float
    movable_area: float

    def to_struct(self):
        """erp_design struct pointing at this design's arrays (kept alive on the struct)."""
        keep = {}
        s = L.Design()
        s.num_nodes, s.num_movable = int(self.num_nodes), int(self.num_movable)
        s.num_pins, s.num_nets, s.n_2nets = int(self.num_pins), int(self.num_nets), int(self.n_2nets)
        for nm in ("x", "y", "w", "h", "num_pins_f", "pin_ox", "pin_oy"):
            a = np.ascontiguousarray(getattr(self, nm), np.float32)
            keep[nm] = a
            setattr(s, nm, a.ctypes.data_as(L.f32p))
        for nm in ("pin_inst", "net_ptr", "net_pins", "inst_pin_ptr", "inst_pins"):
            a = np.ascontiguousarray(getattr(self, nm), np.int32)
            keep[nm] = a
            setattr(s, nm, a.ctypes.data_as(L.i32p))
        s.die_w, s.die_h = float(self.die_w), float(self.die_h)
        s.cell_utilization, s.movable_area = float(self.cell_utilization), float(self.movable_area)
        s._keep = keep
        return s

    @staticmethod
    def from_struct(d):
        def f(p, n):
            return np.ctypeslib.as_array(p, shape=(n,)).astype(np.float32, copy=True) if n else np.zeros(0, np.float32)

        def i(p, n):
            return np.ctypeslib.as_array(p, shape=(n,)).astype(np.int32, copy=True) if n else np.zeros(0, np.int32)

        N, P, E = d.num_nodes, d.num_pins, d.num_nets
        net_ptr = i(d.net_ptr, E + 1)
        inst_ptr = i(d.inst_pin_ptr, N + 1)
        return Design(
            num_nodes=N, num_movable=d.num_movable, num_pins=P, num_nets=E, n_2nets=d.n_2nets,
            x=f(d.x, N), y=f(d.y, N), w=f(d.w, N), h=f(d.h, N), num_pins_f=f(d.num_pins_f, N),
            pin_ox=f(d.pin_ox, P), pin_oy=f(d.pin_oy, P), pin_inst=i(d.pin_inst, P),
            net_ptr=net_ptr, net_pins=i(d.net_pins, int(net_ptr[-1])), inst_pin_ptr=inst_ptr,
            inst_pins=i(d.inst_pins, int(inst_ptr[-1])), die_w=float(d.die_w), die_h=float(d.die_h),
            cell_utilization=float(d.cell_utilization), movable_area=float(d.movable_area))

    def bytes(self):
        return sum(getattr(self, k).nbytes for k in ("x", "y", "w", "h", "num_pins_f", "pin_ox", "pin_oy",
                                                      "pin_inst", "net_ptr", "net_pins",
                                                      "inst_pin_ptr", "inst_pins"))


def synth(num_cells, num_nets=None, num_io=0, num_macros=0, macro_area_frac=0.015,
          utilization=0.7, seed=1, site_w=0.2, row_h=2.0, min_sites=2, max_sites=16,
          jitter_frac=0.001):
    """Seeded synthetic netlist (rule documented in csrc/synth.cpp)."""
    lib = L.load()
    p = L.SynthParams(int(seed), int(num_cells), int(num_nets if num_nets else round(1.05 * num_cells)),
                      int(num_io), int(num_macros), float(macro_area_frac), float(utilization),
                      float(site_w), float(row_h), int(min_sites), int(max_sites), float(jitter_frac))
    h = C.c_void_p()
    L.check(lib.erp_synth_create(C.byref(p), C.byref(h)))
    try:
        d = L.Design()
        L.check(lib.erp_synth_design(h, C.byref(d)))
        return Design.from_struct(d)
    finally:
        lib.erp_synth_destroy(h)


# Workloads (seeded synthetic stand-ins for the reference's ISPD runs): the
# generator's arguments and the run's configuration, as plain data so that a
# CPU-only consumer can rebuild the same design with the generator alone.
WORKLOADS = {
    # 20,000 movable cells, 21,000 nets, 400 IO pins, 70 % utilisation; 256x256 bins,
    # target density 1.0, 450 iterations
    "small": (dict(num_cells=20000, num_nets=21000, num_io=400, num_macros=0, utilization=0.70, seed=1),
              dict(bins=(256, 256), target_density=1.0, iterations=450)),
    # 1,000,000 movable cells, 1,050,000 nets, 16 macros at 1.5 % of the die each, 4,000 IO
    # pins, 65 % utilisation of the free area; 1024x1024 bins, 1,000 iterations
    "large": (dict(num_cells=1000000, num_nets=1050000, num_io=4000, num_macros=16, macro_area_frac=0.015,
                   utilization=0.65, seed=2),
              dict(bins=(1024, 1024), target_density=1.0, iterations=1000)),
}


def workload(name, seed=None):
    args, cfg = WORKLOADS[name]
    args = dict(args)
    if seed is not None:
        args["seed"] = seed
    return synth(**args), dict(cfg)


def workload_small(seed=1):
    """20,000 movable cells, 21,000 nets, 400 IO pins, 70 % utilisation; 256x256 bins,
    target density 1.0, 450 iterations."""
    return workload("small", seed)


def workload_large(seed=2):
    """1,000,000 movable cells, 1,050,000 nets, 16 macros at 1.5 % of the die each,
    4,000 IO pins, 65 % utilisation of the free area; 1024x1024 bins, 1,000 iterations."""
    return workload("large", seed)


def batch_specs(count=64, seed=4000, min_cells=2000, max_cells=200000):
    """Per-instance (cells, macros, seed) of the batched / served mix: cells
    log-uniform in [min, max], macros uniform 0-16, each instance its own seed."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        cells = int(round(np.exp(rng.uniform(np.log(min_cells), np.log(max_cells)))))
        macros = int(rng.integers(0, 17))
        out.append((cells, macros, seed + 1 + i))
    return out


def batch_job(cells, macros, seed):
    """One instance of the mix: nets 1.05 x cells, bin grid = power of two nearest
    sqrt(cells)/2 clamped to 64..1024."""
    d = synth(cells, int(round(1.05 * cells)), num_io=max(4, cells // 250), num_macros=macros,
              macro_area_frac=0.015, utilization=0.65, seed=seed)
    b = bins_for_cells(cells)
    return d, (b, b)


def workload_batch(count=64, seed=4000, min_cells=2000, max_cells=200000):
    """Instance mix of the batched workload (batch_specs, batch_job)."""
    return [batch_job(*sp) for sp in batch_specs(count, seed, min_cells, max_cells)]


def workload_spectral(side, seed=7):
    """Density map of the isolated-solve workload: a uniform 0.7 background plus
    2,000 Gaussian blobs (amplitude uniform 0.1-0.5, sigma uniform 1-20 bins,
    centres uniform; each evaluated within 4 sigma) plus 10 rectangular macro
    blocks (sides uniform side/32..side/8) set to 1.0.  float32 [side, side]."""
    rng = np.random.default_rng(seed)
    rho = np.full((side, side), 0.7, np.float64)
    amp = rng.uniform(0.1, 0.5, 2000)
    sig = rng.uniform(1.0, 20.0, 2000)
    cx = rng.uniform(0, side, 2000)
    cy = rng.uniform(0, side, 2000)
    for a, s_, x0, y0 in zip(amp, sig, cx, cy):
        r = int(np.ceil(4 * s_))
        i0, i1 = max(0, int(x0) - r), min(side, int(x0) + r + 1)
        j0, j1 = max(0, int(y0) - r), min(side, int(y0) + r + 1)
        xi = (np.arange(i0, i1) + 0.5 - x0)[:, None]
        yj = (np.arange(j0, j1) + 0.5 - y0)[None, :]
        rho[i0:i1, j0:j1] += a * np.exp(-(xi * xi + yj * yj) / (2 * s_ * s_))
    for _ in range(10):
        w = int(rng.integers(side // 32, side // 8 + 1))
        h = int(rng.integers(side // 32, side // 8 + 1))
        x0 = int(rng.integers(0, side - w + 1))
        y0 = int(rng.integers(0, side - h + 1))
        rho[x0:x0 + w, y0:y0 + h] = 1.0
    return rho.astype(np.float32)


def bins_for_cells(num_cells):
    """Power of two nearest sqrt(cells)/2, clamped to 64..1024 (batched-instance rule)."""
    t = np.sqrt(num_cells) / 2.0
    b = int(2 ** int(np.round(np.log2(max(t, 1.0)))))
    return int(min(max(b, 64), 1024))
