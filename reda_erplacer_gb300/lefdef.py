"""LEF/DEF ingest, export and the placed-DEF hand-off over the C ABI
(erp_lefdef_*, erp_netlist_* in include/erplacer.h; host code, no GPU needed).

    read_db(lef, def_path) -> Design       reda_db::read_db::<f32> (src/main.rs:69)
    Netlist.read(lef, def_path)            the same, keeping names and the DEF text
    Netlist.from_design(design, ...)       export of an in-memory (e.g. synthetic) design
    Netlist.write(lef_path, def_path)      LEF + DEF text
    Netlist.write_placed(x, y, def_path)   the placed DEF for legalisation

The database rules (instance order, units, pin offsets, two-pin nets first)
are stated in csrc/lefdef.cpp.
"""
import ctypes as C
import os

import numpy as np

from . import lib as L
from .design import Design


def _check(st):
    if st != L.OK:
        msg = L.load().erp_lefdef_last_error()
        raise L.ErpError(st, msg.decode(errors="replace") if msg else "")


def _path(p):
    return os.fsencode(p)


class Netlist:
    """An erp_netlist handle: a LEF/DEF design with its names."""

    def __init__(self, handle):
        self.lib = L.load()
        self.h = handle

    @classmethod
    def read(cls, lef, def_path):
        """lef: one path or a list (technology first, then cells)."""
        lefs = [lef] if isinstance(lef, (str, bytes, os.PathLike)) else list(lef)
        arr = (C.c_char_p * max(1, len(lefs)))(*[_path(p) for p in lefs])
        h = C.c_void_p()
        _check(L.load().erp_lefdef_read(arr, len(lefs), _path(def_path), C.byref(h)))
        return cls(h)

    @classmethod
    def from_design(cls, design, dbu=2000, site_w=0.2, row_h=2.0):
        s = design.to_struct()
        p = L.LefDefParams(int(dbu), float(site_w), float(row_h))
        h = C.c_void_p()
        _check(L.load().erp_netlist_from_design(C.byref(s), C.byref(p), C.byref(h)))
        return cls(h)

    def design(self):
        d = L.Design()
        _check(self.lib.erp_netlist_design(self.h, C.byref(d)))
        return Design.from_struct(d)

    def stats(self):
        s = L.LefDefStats()
        _check(self.lib.erp_netlist_stats(self.h, C.byref(s)))
        return s.as_dict()

    def node_name(self, i):
        r = self.lib.erp_netlist_node_name(self.h, int(i))
        if r is None:
            raise IndexError(i)
        return r.decode(errors="surrogateescape")   # names are bytes in the files

    def net_name(self, e):
        r = self.lib.erp_netlist_net_name(self.h, int(e))
        if r is None:
            raise IndexError(e)
        return r.decode(errors="surrogateescape")

    def write(self, lef_path=None, def_path=None):
        _check(self.lib.erp_lefdef_write(self.h, _path(lef_path) if lef_path else None,
                                         _path(def_path) if def_path else None))

    def write_placed(self, x, y, def_path):
        """Movable instance k (design order) at (x[k], y[k]) microns."""
        x = np.ascontiguousarray(x, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        _check(self.lib.erp_def_write_placed(self.h, x.ctypes.data_as(L.f32p), y.ctypes.data_as(L.f32p),
                                             _path(def_path)))

    def close(self):
        if getattr(self, "h", None):
            self.lib.erp_netlist_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def read_db(lef, def_path):
    """The placement database of a LEF/DEF pair (reda_db::read_db, src/main.rs:69)."""
    with Netlist.read(lef, def_path) as nl:
        return nl.design()


def write_lefdef(design, lef_path, def_path, dbu=2000, site_w=0.2, row_h=2.0):
    """Write a design as LEF/DEF; returns the design as the files carry it
    (coordinates on the 1/dbu micron grid), which read_db gives back exactly."""
    with Netlist.from_design(design, dbu, site_w, row_h) as nl:
        nl.write(lef_path, def_path)
        return nl.design()
