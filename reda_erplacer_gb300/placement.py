"""Host-side mirror of the reference's placement call surface over the C ABI.

    Placement(design, ...)          Placement::new          (src/placement.rs:159-178)
    .step() -> bool                 Placement::step         (src/placement.rs:180-228)
    .compute_hpwl(gamma) -> hpwl    compute_hpwl            (src/hpwl.rs:139-343)
    .compute_potential(it)          compute_potential       (src/epotential.rs:225-374)
                                    -> (energy, overflow)
    .step_adaptive(it)              Nesterov::step_adaptive (src/nesterov.rs:27-146)
    .scheduler_update(h, o)         Scheduler::update       (src/scheduler.rs:68-73)
    .should_stop() -> bool          Scheduler::should_stop  (src/scheduler.rs:75-81)

Every call runs on the GPU through liberplacer_gb300.so; errors raise ErpError.
"""
import ctypes as C

import numpy as np

from . import lib as L


def write_ppm(path, img):
    """Binary PPM (P6) of an (height, width, 3) uint8 image."""
    h, w, _ = img.shape
    with open(path, "wb") as f:
        f.write(b"P6\n%d %d\n255\n" % (w, h))
        f.write(np.ascontiguousarray(img, np.uint8).tobytes())


class Placement:
    def __init__(self, design, num_bins=(512, 512), target_density=-1.0,
                 start_mode=L.START_CENTER, device=0, stream=None, precision=L.PREC_FP32, flags=0):
        self.lib = L.load()
        self.design = design
        self._ds = design.to_struct()
        m, n = num_bins
        self._params = L.Params(int(m), int(n), float(target_density), int(start_mode),
                                int(precision), int(device), C.c_void_p(stream) if stream else None,
                                int(flags))
        h = C.c_void_p()
        st = self.lib.erp_create(C.byref(self._ds), C.byref(self._params), C.byref(h))
        L.check(st, None)
        self.h = h
        self.N = int(design.num_nodes)
        self.P = int(design.num_pins)
        self.E = int(design.num_nets)
        self.m, self.n = int(m), int(n)

    # -- lifetime --
    def close(self):
        if getattr(self, "h", None):
            self.lib.erp_destroy(self.h)
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

    def _ck(self, st):
        L.check(st, self.h)

    # -- reference stages --
    def compute_hpwl(self, gamma):
        out = C.c_float()
        self._ck(self.lib.erp_wirelength(self.h, float(gamma), C.byref(out)))
        return float(out.value)

    def compute_potential(self, iteration, want_energy=True):
        e, o = C.c_float(), C.c_float()
        self._ck(self.lib.erp_potential(self.h, int(iteration), C.byref(e) if want_energy else None,
                                        C.byref(o)))
        return (float(e.value) if want_energy else None), float(o.value)

    def step_adaptive(self, iteration):
        self._ck(self.lib.erp_nesterov(self.h, int(iteration)))

    def scheduler_update(self, hpwl, overflow):
        self._ck(self.lib.erp_scheduler_update(self.h, float(hpwl), float(overflow)))

    def should_stop(self):
        s = C.c_int32()
        self._ck(self.lib.erp_should_stop(self.h, C.byref(s)))
        return bool(s.value)

    def step(self, stats=True):
        """One Placement::step (CUDA-graph replay).  Returns should_stop, or None
        when stats=False (the call then only enqueues work)."""
        if not stats:
            self._ck(self.lib.erp_step(self.h, None))
            return None
        st = L.StepStats()
        self._ck(self.lib.erp_step(self.h, C.byref(st)))
        self.last_stats = st.as_dict()
        return bool(st.should_stop)

    def step_host(self, x, y):
        """Drop-in step for host-owned coordinates (float32 arrays, updated in place)."""
        assert x.dtype == np.float32 and y.dtype == np.float32 and x.flags.c_contiguous
        st = L.StepStats()
        self._ck(self.lib.erp_step_host(self.h, x.ctypes.data_as(L.f32p), y.ctypes.data_as(L.f32p),
                                        C.byref(st)))
        return st.as_dict()

    def run(self, max_iterations, stop_overflow=0.0):
        it = C.c_int32()
        st = L.StepStats()
        self._ck(self.lib.erp_run(self.h, int(max_iterations), float(stop_overflow), C.byref(it),
                                  C.byref(st)))
        return int(it.value), st.as_dict()

    def synchronize(self):
        self._ck(self.lib.erp_synchronize(self.h))

    def profile_stages(self, reps=10, warm=False):
        """Mean milliseconds per launch of each stage, timed in isolation with an
        L2 flush before every launch (mutates the placement state); warm=True:
        whole steps in graph order with events between the stages, caches warm
        (advances the placement by reps + 1 iterations)."""
        out = (C.c_float * len(L.STAGES))()
        self._ck(self.lib.erp_profile_stages(self.h, -int(reps) if warm else int(reps), out))
        return dict(zip(L.STAGES, [float(v) for v in out]))

    # -- state --
    def scalars(self):
        s = L.Scalars()
        self._ck(self.lib.erp_get_scalars(self.h, C.byref(s)))
        return s.as_dict()

    def set_scalars(self, iteration, gamma, density_weight, alpha, beta):
        self._ck(self.lib.erp_set_scalars(self.h, int(iteration), float(gamma), float(density_weight),
                                          float(alpha), float(beta)))

    def positions(self):
        x = np.empty(self.N, np.float32)
        y = np.empty(self.N, np.float32)
        self._ck(self.lib.erp_get_positions(self.h, x.ctypes.data_as(L.f32p), y.ctypes.data_as(L.f32p)))
        return x, y

    def set_positions(self, x, y):
        x = np.ascontiguousarray(x, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        self._ck(self.lib.erp_set_positions(self.h, x.ctypes.data_as(L.f32p), y.ctypes.data_as(L.f32p)))

    # -- checkpoint / resume --
    def checkpoint(self):
        """The state one step hands to the next, as bytes (erp_checkpoint)."""
        n = C.c_size_t()
        self._ck(self.lib.erp_checkpoint_size(self.h, C.byref(n)))
        buf = (C.c_char * n.value)()
        self._ck(self.lib.erp_checkpoint(self.h, buf, n.value))
        return bytes(buf)

    def restore(self, blob):
        """Continue from a checkpoint of the same design and bin grid (erp_restore)."""
        buf = (C.c_char * len(blob)).from_buffer_copy(blob)
        self._ck(self.lib.erp_restore(self.h, buf, len(blob)))

    # -- headless snapshots --
    def snapshot_placement(self, path=None):
        """draw_placement (src/drawing.rs:7-60) as an (height, width, 3) uint8
        array rasterised on the device; written as a binary PPM when path is given."""
        w, h = C.c_int32(), C.c_int32()
        self._ck(self.lib.erp_snapshot_size(self.h, C.byref(w), C.byref(h)))
        img = np.empty((h.value, w.value, 3), np.uint8)
        self._ck(self.lib.erp_snapshot_placement(self.h, img.ctypes.data_as(C.c_void_p), img.nbytes))
        if path:
            write_ppm(path, img)
        return img

    def snapshot_density(self, path=None):
        """draw_density_map (src/epotential.rs:199-223) of the current positions as an
        (n, m, 3) uint8 array; written as a binary PPM when path is given."""
        img = np.empty((self.n, self.m, 3), np.uint8)
        self._ck(self.lib.erp_snapshot_density(self.h, img.ctypes.data_as(C.c_void_p), img.nbytes))
        if path:
            write_ppm(path, img)
        return img

    def set_nesterov_history(self, px, py, pgx, pgy):
        a = [np.ascontiguousarray(t, np.float32) for t in (px, py, pgx, pgy)]
        self._ck(self.lib.erp_set_nesterov_history(self.h, *[t.ctypes.data_as(L.f32p) for t in a]))

    def array(self, name):
        which = L.ARR[name]
        mn = self.m * self.n
        if name == "DENSITY_I64":
            out = np.empty(mn, np.int64)
        elif name in ("PIN_GRAD_X", "PIN_GRAD_Y"):
            out = np.empty(self.P, np.float32)
        elif name == "NET_HPWL":
            out = np.empty(self.E, np.float32)
        elif name in ("DENSITY", "INITIAL", "FIELD_X", "FIELD_Y", "POTENTIAL"):
            out = np.empty(mn, np.float32)
        else:
            out = np.empty(self.N, np.float32)
        self._ck(self.lib.erp_get_array(self.h, which, out.ctypes.data_as(C.c_void_p), out.nbytes))
        return out


class Batch:
    """Many designs advanced together by one CUDA graph (one branch per design);
    see erp_batch_* in include/erplacer.h."""

    def __init__(self, designs, num_bins, target_density=1.0, start_mode=L.START_CENTER, device=0,
                 precision=L.PREC_FP32, flags=0):
        """precision, flags: one value for every design, or one per design."""
        self.lib = L.load()
        K = len(designs)
        self._structs = [d.to_struct() for d in designs]
        darr = (L.Design * K)(*self._structs)
        bins = num_bins if isinstance(num_bins[0], (tuple, list)) else [num_bins] * K
        precs = list(precision) if isinstance(precision, (tuple, list)) else [precision] * K
        flg = list(flags) if isinstance(flags, (tuple, list)) else [flags] * K
        parr = (L.Params * K)(*[L.Params(int(b[0]), int(b[1]), float(target_density), int(start_mode),
                                         int(pr), int(device), None, int(f))
                                for b, pr, f in zip(bins, precs, flg)])
        h = C.c_void_p()
        st = self.lib.erp_batch_create(darr, parr, K, C.byref(h))
        L.check(st, None)
        self.h = h
        self.K = K
        self.designs = designs

    def run(self, max_iterations, stop_overflow=0.0):
        it = (C.c_int32 * self.K)()
        last = (L.StepStats * self.K)()
        st = self.lib.erp_batch_run(self.h, int(max_iterations), float(stop_overflow), it, last)
        if st != L.OK:
            raise L.ErpError(st, self.lib.erp_batch_last_error(self.h).decode(errors="replace"))
        return [int(v) for v in it], [s.as_dict() for s in last]

    def tuning(self):
        """The autotuned scatter shape: (chosen cells per block, [(candidate, ms), ...])."""
        ch, n = C.c_int32(), C.c_int32()
        cells = (C.c_int32 * 8)()
        ms = (C.c_float * 8)()
        L.check(self.lib.erp_batch_tuning(self.h, C.byref(ch), cells, ms, 8, C.byref(n)))
        return int(ch.value), [(int(cells[i]), float(ms[i])) for i in range(min(n.value, 8))]

    def packed_instances(self):
        """How many instances advance in packed launches (erp_batch_packed)."""
        n = C.c_int32()
        L.check(self.lib.erp_batch_packed(self.h, C.byref(n)))
        return int(n.value)

    def spectral_tuning(self):
        """The autotuned tile shape of the FP32 spectral passes: (chosen sequences
        per block, 0 for the fixed shape, [(candidate, ms), ...])."""
        ch, n = C.c_int32(), C.c_int32()
        seqs = (C.c_int32 * 8)()
        ms = (C.c_float * 8)()
        L.check(self.lib.erp_batch_spectral_tuning(self.h, C.byref(ch), seqs, ms, 8, C.byref(n)))
        return int(ch.value), [(int(seqs[i]), float(ms[i])) for i in range(min(n.value, 8))]

    def positions(self, i):
        ctx = self.lib.erp_batch_context(self.h, int(i))
        N = int(self.designs[i].num_nodes)
        x = np.empty(N, np.float32)
        y = np.empty(N, np.float32)
        L.check(self.lib.erp_get_positions(ctx, x.ctypes.data_as(L.f32p), y.ctypes.data_as(L.f32p)), ctx)
        return x, y

    def close(self):
        if getattr(self, "h", None):
            self.lib.erp_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class SpectralSolver:
    """Standalone Poisson solve (src/epotential.rs:284-343) on device pointers.
    precision: lib.PREC_FP32 (FFT), PREC_TF32_GEMM or PREC_BF16X3_GEMM (DCT
    matrix contractions on the tensor cores; bin counts multiples of 128)."""

    def __init__(self, m, n, bin_w, bin_h, stream=None, precision=L.PREC_FP32):
        self.lib = L.load()
        h = C.c_void_p()
        L.check(self.lib.erp_spectral_create(int(m), int(n), float(bin_w), float(bin_h), int(precision),
                                             C.c_void_p(stream) if stream else None, C.byref(h)))
        self.h = h

    def solve(self, rho_ptr, fx_ptr, fy_ptr, psi_ptr=None):
        L.check(self.lib.erp_spectral_solve(self.h, C.c_void_p(rho_ptr), C.c_void_p(fx_ptr),
                                            C.c_void_p(fy_ptr), C.c_void_p(psi_ptr) if psi_ptr else None))

    def close(self):
        if getattr(self, "h", None):
            self.lib.erp_spectral_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
