"""GB300-native (sm_103a) electrostatic global-placement loop: a drop-in for
ERPlacer's (giammirove/reda-erplacer) placement step behind the C ABI of
include/erplacer.h.  All compute runs in liberplacer_gb300.so; importing this
package fails if the library has not been built (no fallback)."""
from . import lib
from .lib import ErpError
from .design import (Design, bins_for_cells, synth, workload_batch, workload_large, workload_small,
                     workload_spectral)
from .placement import Batch, Placement, SpectralSolver
from .lefdef import Netlist, read_db, write_lefdef

lib.load()

__all__ = ["Design", "synth", "workload_small", "workload_large", "workload_batch", "workload_spectral",
           "bins_for_cells",
           "Placement", "Batch", "SpectralSolver", "ErpError", "Netlist", "read_db", "write_lefdef"]
