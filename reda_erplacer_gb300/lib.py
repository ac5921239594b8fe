"""ctypes binding of the C ABI in include/erplacer.h (liberplacer_gb300.so).

The library is built in-tree (reda_erplacer_gb300/build.py).  There is no
fallback: if the shared library is missing or cannot be loaded, importing the
binding raises, and every compute entry point fails with ERP_ENODEV when no
sm_103 GPU is present.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
# ERP_LIBRARY names another build of the same ABI (e.g. one compiled elsewhere).
LIB_PATH = os.environ.get("ERP_LIBRARY") or os.path.join(HERE, "liberplacer_gb300.so")

f32p = C.POINTER(C.c_float)
i32p = C.POINTER(C.c_int32)

OK, EINVAL, ENOMEM, ECUDA, ENAN, ETIMEDOUT, ENOTSUP, ENODEV, ESTATE, ECANCELED = range(10)
START_CENTER, START_DB = 0, 1
STAGES = ("wirelength", "wl_gather", "density", "spectral", "force", "nesterov", "scheduler")
PREC_FP32, PREC_TF32_GEMM, PREC_BF16X3_GEMM = 0, 1, 2
FLAG_EXPIRE_WAITS = 1   # erp_params.flags: test hook of the bounded device waits

ARR = dict(WL_GRAD_X=0, WL_GRAD_Y=1, DENS_GRAD_X=2, DENS_GRAD_Y=3, PIN_GRAD_X=4, PIN_GRAD_Y=5,
           DENSITY_I64=6, DENSITY=7, INITIAL=8, FIELD_X=9, FIELD_Y=10, POTENTIAL=11, PREV_X=12,
           PREV_Y=13, PREV_GX=14, PREV_GY=15, NET_HPWL=16)


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
                ("precision", C.c_int32), ("device", C.c_int32), ("stream", C.c_void_p),
                ("flags", C.c_int32)]


class StepStats(C.Structure):
    _fields_ = [("iteration", C.c_int32), ("should_stop", C.c_int32), ("hpwl", C.c_float),
                ("overflow", C.c_float), ("density_weight", C.c_float), ("gamma", C.c_float),
                ("alpha", C.c_float), ("beta", C.c_float)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Scalars(C.Structure):
    _fields_ = [("iteration", C.c_int32), ("gamma", C.c_float), ("base_gamma", C.c_float),
                ("density_weight", C.c_float), ("alpha", C.c_float), ("beta", C.c_float),
                ("hpwl_initial", C.c_float), ("hpwl_current", C.c_float),
                ("hpwl_previous", C.c_float), ("overflow_current", C.c_float),
                ("overflow_previous", C.c_float), ("hpwl_last", C.c_double),
                ("overflow_last", C.c_double), ("energy_last", C.c_double),
                ("fixed_shift", C.c_int32), ("fixed_shift_init", C.c_int32),
                ("num_bins_x", C.c_int32), ("num_bins_y", C.c_int32), ("bin_w", C.c_float),
                ("bin_h", C.c_float), ("target_density", C.c_float), ("graph_kernels", C.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class SynthParams(C.Structure):
    _fields_ = [("seed", C.c_int64), ("num_cells", C.c_int32), ("num_nets", C.c_int32),
                ("num_io", C.c_int32), ("num_macros", C.c_int32), ("macro_area_frac", C.c_float),
                ("utilization", C.c_float), ("site_w", C.c_float), ("row_h", C.c_float),
                ("min_sites", C.c_int32), ("max_sites", C.c_int32), ("jitter_frac", C.c_float)]


class ServerParams(C.Structure):
    _fields_ = [("device", C.c_int32), ("max_active", C.c_int32), ("hbm_budget_bytes", C.c_int64),
                ("max_iterations", C.c_int32), ("stop_overflow", C.c_float), ("chunk", C.c_int32),
                ("keep_positions", C.c_int32)]


class JobResult(C.Structure):
    _fields_ = [("job_id", C.c_int64), ("status", C.c_int32), ("iterations", C.c_int32),
                ("last", StepStats), ("submit_s", C.c_double), ("admit_s", C.c_double),
                ("finish_s", C.c_double), ("footprint_bytes", C.c_int64)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_ if k != "last"}
        d["last"] = self.last.as_dict()
        return d


class LefDefStats(C.Structure):
    _fields_ = [("num_nodes", C.c_int32), ("num_movable", C.c_int32), ("num_fixed", C.c_int32),
                ("num_io", C.c_int32), ("num_nets", C.c_int32), ("num_pins", C.c_int32),
                ("num_macros", C.c_int32), ("num_dropped_nets", C.c_int32),
                ("num_skipped_conns", C.c_int32), ("num_unplaced_io", C.c_int32),
                ("def_dbu", C.c_int32), ("lef_dbu", C.c_int32), ("die", C.c_int64 * 4)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_ if k != "die"}
        d["die"] = tuple(int(v) for v in self.die)
        return d


class LefDefParams(C.Structure):
    _fields_ = [("dbu", C.c_int32), ("site_w", C.c_float), ("row_h", C.c_float)]


EXPORTS = {
    "erp_server_create": (C.c_int, [C.POINTER(ServerParams), C.POINTER(C.c_void_p)]),
    "erp_server_submit": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(Design), C.POINTER(Params)]),
    "erp_server_pump": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "erp_server_cancel": (C.c_int, [C.c_void_p, C.c_int64]),
    "erp_server_poll": (C.c_int, [C.c_void_p, C.POINTER(JobResult), C.c_int32, C.POINTER(C.c_int32)]),
    "erp_server_positions": (C.c_int, [C.c_void_p, C.c_int64, f32p, f32p]),
    "erp_server_now": (C.c_double, [C.c_void_p]),
    "erp_server_last_error": (C.c_char_p, [C.c_void_p]),
    "erp_server_destroy": (None, [C.c_void_p]),
    "erp_estimate_footprint": (C.c_int, [C.POINTER(Design), C.POINTER(Params), C.POINTER(C.c_int64)]),
    "erp_status_string": (C.c_char_p, [C.c_int]),
    "erp_last_error": (C.c_char_p, [C.c_void_p]),
    "erp_abi_version": (C.c_int32, []),
    "erp_create": (C.c_int, [C.POINTER(Design), C.POINTER(Params), C.POINTER(C.c_void_p)]),
    "erp_destroy": (None, [C.c_void_p]),
    "erp_wirelength": (C.c_int, [C.c_void_p, C.c_float, f32p]),
    "erp_potential": (C.c_int, [C.c_void_p, C.c_int32, f32p, f32p]),
    "erp_nesterov": (C.c_int, [C.c_void_p, C.c_int32]),
    "erp_scheduler_update": (C.c_int, [C.c_void_p, C.c_float, C.c_float]),
    "erp_should_stop": (C.c_int, [C.c_void_p, i32p]),
    "erp_step": (C.c_int, [C.c_void_p, C.POINTER(StepStats)]),
    "erp_step_host": (C.c_int, [C.c_void_p, f32p, f32p, C.POINTER(StepStats)]),
    "erp_run": (C.c_int, [C.c_void_p, C.c_int32, C.c_float, i32p, C.POINTER(StepStats)]),
    "erp_get_scalars": (C.c_int, [C.c_void_p, C.POINTER(Scalars)]),
    "erp_set_scalars": (C.c_int, [C.c_void_p, C.c_int32, C.c_float, C.c_float, C.c_float, C.c_float]),
    "erp_get_positions": (C.c_int, [C.c_void_p, f32p, f32p]),
    "erp_set_positions": (C.c_int, [C.c_void_p, f32p, f32p]),
    "erp_set_nesterov_history": (C.c_int, [C.c_void_p, f32p, f32p, f32p, f32p]),
    "erp_get_array": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_size_t]),
    "erp_synchronize": (C.c_int, [C.c_void_p]),
    "erp_snapshot_size": (C.c_int, [C.c_void_p, i32p, i32p]),
    "erp_snapshot_placement": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "erp_snapshot_density": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "erp_checkpoint_size": (C.c_int, [C.c_void_p, C.POINTER(C.c_size_t)]),
    "erp_checkpoint": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "erp_restore": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "erp_profile_stages": (C.c_int, [C.c_void_p, C.c_int32, f32p]),
    "erp_spectral_create": (C.c_int, [C.c_int32, C.c_int32, C.c_float, C.c_float, C.c_int32,
                                      C.c_void_p, C.POINTER(C.c_void_p)]),
    "erp_spectral_solve": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "erp_spectral_destroy": (None, [C.c_void_p]),
    "erp_spectral_solve_noalloc": (C.c_int, [C.c_int32, C.c_int32, C.c_float, C.c_float, C.c_void_p,
                                             C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "erp_batch_create": (C.c_int, [C.POINTER(Design), C.POINTER(Params), C.c_int32, C.POINTER(C.c_void_p)]),
    "erp_batch_run": (C.c_int, [C.c_void_p, C.c_int32, C.c_float, i32p, C.POINTER(StepStats)]),
    "erp_batch_context": (C.c_void_p, [C.c_void_p, C.c_int32]),
    "erp_batch_size": (C.c_int32, [C.c_void_p]),
    "erp_batch_last_error": (C.c_char_p, [C.c_void_p]),
    "erp_batch_destroy": (None, [C.c_void_p]),
    "erp_batch_tuning": (C.c_int, [C.c_void_p, i32p, i32p, f32p, C.c_int32, i32p]),
    "erp_batch_spectral_tuning": (C.c_int, [C.c_void_p, i32p, i32p, f32p, C.c_int32, i32p]),
    "erp_batch_packed": (C.c_int, [C.c_void_p, i32p]),
    "erp_synth_create": (C.c_int, [C.POINTER(SynthParams), C.POINTER(C.c_void_p)]),
    "erp_synth_design": (C.c_int, [C.c_void_p, C.POINTER(Design)]),
    "erp_synth_destroy": (None, [C.c_void_p]),
    "erp_lefdef_read": (C.c_int, [C.POINTER(C.c_char_p), C.c_int32, C.c_char_p, C.POINTER(C.c_void_p)]),
    "erp_lefdef_last_error": (C.c_char_p, []),
    "erp_netlist_design": (C.c_int, [C.c_void_p, C.POINTER(Design)]),
    "erp_netlist_stats": (C.c_int, [C.c_void_p, C.POINTER(LefDefStats)]),
    "erp_netlist_node_name": (C.c_char_p, [C.c_void_p, C.c_int32]),
    "erp_netlist_net_name": (C.c_char_p, [C.c_void_p, C.c_int32]),
    "erp_netlist_from_design": (C.c_int, [C.POINTER(Design), C.POINTER(LefDefParams), C.POINTER(C.c_void_p)]),
    "erp_lefdef_write": (C.c_int, [C.c_void_p, C.c_char_p, C.c_char_p]),
    "erp_def_write_placed": (C.c_int, [C.c_void_p, f32p, f32p, C.c_char_p]),
    "erp_netlist_destroy": (None, [C.c_void_p]),
}

_lib = None


class ErpError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{status_string(status)}: {msg}")
        self.status = status


def load():
    """Load liberplacer_gb300.so (raises if it is missing: there is no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing; build it with reda_erplacer_gb300.build.build()")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in EXPORTS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def status_string(s):
    return load().erp_status_string(int(s)).decode()


def check(status, ctx=None):
    if status != OK:
        msg = load().erp_last_error(ctx)
        raise ErpError(status, msg.decode(errors="replace") if msg else "")
