//! Rust binding of liberplacer_gb300.so for the ERPlacer crate (src/gb300.rs
//! once added there, with `mod gb300;` in src/main.rs).  The `extern "C"`
//! block mirrors include/erplacer.h one to one; `Gb300Placement` is the thin
//! safe layer that takes the place of `Placement` (src/placement.rs:141-228)
//! in src/main.rs:72-90.  Not built here: this environment has no Rust
//! toolchain.  The same symbols are exercised through ctypes by the Python
//! tests.
#![allow(non_camel_case_types, dead_code)]

use std::ffi::{CStr, CString};
use std::os::raw::{c_char, c_int, c_void};

pub type erp_status = c_int;
pub const ERP_OK: erp_status = 0;
pub const ERP_ETIMEDOUT: erp_status = 5;
pub const ERP_ECANCELED: erp_status = 9;

pub const ERP_START_CENTER: i32 = 0; // src/placement.rs:109-139
pub const ERP_START_DB: i32 = 1;
pub const ERP_PREC_FP32: i32 = 0;
pub const ERP_PREC_TF32_GEMM: i32 = 1;
pub const ERP_PREC_BF16X3_GEMM: i32 = 2;

/// erp_design: the fields of reda-db's DB<f32> that the loop reads.
#[repr(C)]
pub struct erp_design {
    pub num_nodes: i32,
    pub num_movable: i32,
    pub num_pins: i32,
    pub num_nets: i32,
    pub n_2nets: i32,
    pub _pad: i32,
    pub x: *const f32,
    pub y: *const f32,
    pub w: *const f32,
    pub h: *const f32,
    pub num_pins_f: *const f32,
    pub pin_ox: *const f32,
    pub pin_oy: *const f32,
    pub pin_inst: *const i32,
    pub net_ptr: *const i32,
    pub net_pins: *const i32,
    pub inst_pin_ptr: *const i32,
    pub inst_pins: *const i32,
    pub die_w: f32,
    pub die_h: f32,
    pub cell_utilization: f32,
    pub movable_area: f32,
}

#[repr(C)]
pub struct erp_params {
    pub num_bins_x: i32, // 0: 512 (src/placement.rs:50)
    pub num_bins_y: i32,
    pub target_density: f32, // < 0: db.cell_utilization (src/placement.rs:134)
    pub start_mode: i32,
    pub precision: i32,
    pub device: i32,
    pub stream: *mut c_void,
    pub flags: i32,
}

#[repr(C)]
#[derive(Default, Clone, Copy, Debug)]
pub struct erp_step_stats {
    pub iteration: i32,
    pub should_stop: i32,
    pub hpwl: f32,
    pub overflow: f32,
    pub density_weight: f32,
    pub gamma: f32,
    pub alpha: f32,
    pub beta: f32,
}

#[repr(C)]
#[derive(Default, Clone, Copy, Debug)]
pub struct erp_scalars {
    pub iteration: i32,
    pub gamma: f32,
    pub base_gamma: f32,
    pub density_weight: f32,
    pub alpha: f32,
    pub beta: f32,
    pub hpwl_initial: f32,
    pub hpwl_current: f32,
    pub hpwl_previous: f32,
    pub overflow_current: f32,
    pub overflow_previous: f32,
    pub hpwl_last: f64,
    pub overflow_last: f64,
    pub energy_last: f64,
    pub fixed_shift: i32,
    pub fixed_shift_init: i32,
    pub num_bins_x: i32,
    pub num_bins_y: i32,
    pub bin_w: f32,
    pub bin_h: f32,
    pub target_density: f32,
    pub graph_kernels: i32,
}

#[repr(C)]
pub struct erp_server_params {
    pub device: i32,
    pub max_active: i32,
    pub hbm_budget_bytes: i64,
    pub max_iterations: i32,
    pub stop_overflow: f32,
    pub chunk: i32,
    pub keep_positions: i32,
}

#[repr(C)]
#[derive(Default, Clone, Copy, Debug)]
pub struct erp_job_result {
    pub job_id: i64,
    pub status: i32,
    pub iterations: i32,
    pub last: erp_step_stats,
    pub submit_s: f64,
    pub admit_s: f64,
    pub finish_s: f64,
    pub footprint_bytes: i64,
}

#[repr(C)]
pub struct erp_synth_params {
    pub seed: i64,
    pub num_cells: i32,
    pub num_nets: i32,
    pub num_io: i32,
    pub num_macros: i32,
    pub macro_area_frac: f32,
    pub utilization: f32,
    pub site_w: f32,
    pub row_h: f32,
    pub min_sites: i32,
    pub max_sites: i32,
    pub jitter_frac: f32,
}

#[repr(C)]
#[derive(Default, Clone, Copy, Debug)]
pub struct erp_lefdef_stats {
    pub num_nodes: i32,
    pub num_movable: i32,
    pub num_fixed: i32,
    pub num_io: i32,
    pub num_nets: i32,
    pub num_pins: i32,
    pub num_macros: i32,
    pub num_dropped_nets: i32,
    pub num_skipped_conns: i32,
    pub num_unplaced_io: i32,
    pub def_dbu: i32,
    pub lef_dbu: i32,
    pub die: [i64; 4],
}

#[repr(C)]
pub struct erp_lefdef_params {
    pub dbu: i32,
    pub site_w: f32,
    pub row_h: f32,
}

pub const ERP_NUM_STAGES: usize = 7;
pub const ERP_NOALLOC_MAX_BINS: i32 = 512 * 512;

pub enum erp_ctx {}
pub enum erp_batch {}
pub enum erp_server {}
pub enum erp_netlist {}
pub enum erp_spectral {}
pub enum erp_synth {}

extern "C" {
    pub fn erp_status_string(s: erp_status) -> *const c_char;
    pub fn erp_last_error(ctx: *const erp_ctx) -> *const c_char;
    pub fn erp_abi_version() -> i32;

    // Placement::new (src/placement.rs:159-178)
    pub fn erp_create(d: *const erp_design, p: *const erp_params, out: *mut *mut erp_ctx) -> erp_status;
    pub fn erp_destroy(ctx: *mut erp_ctx);
    // compute_hpwl (src/hpwl.rs:139-343)
    pub fn erp_wirelength(ctx: *mut erp_ctx, gamma: f32, hpwl: *mut f32) -> erp_status;
    // compute_potential (src/epotential.rs:225-374)
    pub fn erp_potential(ctx: *mut erp_ctx, iteration: i32, energy: *mut f32, overflow: *mut f32) -> erp_status;
    // Nesterov::step_adaptive (src/nesterov.rs:27-146)
    pub fn erp_nesterov(ctx: *mut erp_ctx, iteration: i32) -> erp_status;
    // Scheduler::update / should_stop (src/scheduler.rs:68-81)
    pub fn erp_scheduler_update(ctx: *mut erp_ctx, hpwl: f32, overflow: f32) -> erp_status;
    pub fn erp_should_stop(ctx: *mut erp_ctx, stop: *mut i32) -> erp_status;
    // Placement::step (src/placement.rs:180-228)
    pub fn erp_step(ctx: *mut erp_ctx, stats: *mut erp_step_stats) -> erp_status;
    pub fn erp_step_host(ctx: *mut erp_ctx, x: *mut f32, y: *mut f32, stats: *mut erp_step_stats) -> erp_status;
    // the loop of src/main.rs:78-90
    pub fn erp_run(ctx: *mut erp_ctx, max_iterations: i32, stop_overflow: f32, iterations_run: *mut i32,
                   last: *mut erp_step_stats) -> erp_status;
    pub fn erp_get_scalars(ctx: *mut erp_ctx, out: *mut erp_scalars) -> erp_status;
    pub fn erp_set_scalars(ctx: *mut erp_ctx, iteration: i32, gamma: f32, density_weight: f32, alpha: f32,
                           beta: f32) -> erp_status;
    pub fn erp_get_positions(ctx: *mut erp_ctx, x: *mut f32, y: *mut f32) -> erp_status;
    pub fn erp_set_positions(ctx: *mut erp_ctx, x: *const f32, y: *const f32) -> erp_status;
    pub fn erp_set_nesterov_history(ctx: *mut erp_ctx, prev_x: *const f32, prev_y: *const f32,
                                    prev_gx: *const f32, prev_gy: *const f32) -> erp_status;
    // device arrays for inspection (which: the erp_array values of the header)
    pub fn erp_get_array(ctx: *mut erp_ctx, which: c_int, dst: *mut c_void, bytes: usize) -> erp_status;
    pub fn erp_synchronize(ctx: *mut erp_ctx) -> erp_status;
    // the reference's time_it phases (src/utils.rs:106-124): ERP_NUM_STAGES means
    pub fn erp_profile_stages(ctx: *mut erp_ctx, reps: i32, ms_out: *mut f32) -> erp_status;

    // draw_placement (src/drawing.rs:7-60), draw_density_map (src/epotential.rs:199-223)
    pub fn erp_snapshot_size(ctx: *mut erp_ctx, width: *mut i32, height: *mut i32) -> erp_status;
    pub fn erp_snapshot_placement(ctx: *mut erp_ctx, rgb: *mut u8, bytes: usize) -> erp_status;
    pub fn erp_snapshot_density(ctx: *mut erp_ctx, rgb: *mut u8, bytes: usize) -> erp_status;

    // checkpoint / resume (no counterpart in the reference)
    pub fn erp_checkpoint_size(ctx: *mut erp_ctx, bytes: *mut usize) -> erp_status;
    pub fn erp_checkpoint(ctx: *mut erp_ctx, buf: *mut c_void, bytes: usize) -> erp_status;
    pub fn erp_restore(ctx: *mut erp_ctx, buf: *const c_void, bytes: usize) -> erp_status;

    // many designs at once (no counterpart in the reference)
    pub fn erp_batch_create(designs: *const erp_design, params: *const erp_params, count: i32,
                            out: *mut *mut erp_batch) -> erp_status;
    pub fn erp_batch_run(b: *mut erp_batch, max_iterations: i32, stop_overflow: f32, iterations: *mut i32,
                         last: *mut erp_step_stats) -> erp_status;
    pub fn erp_batch_context(b: *mut erp_batch, i: i32) -> *mut erp_ctx;
    pub fn erp_batch_size(b: *const erp_batch) -> i32;
    pub fn erp_batch_last_error(b: *const erp_batch) -> *const c_char;
    pub fn erp_batch_tuning(b: *const erp_batch, chosen: *mut i32, cells: *mut i32, ms: *mut f32, cap: i32,
                            count: *mut i32) -> erp_status;
    pub fn erp_batch_spectral_tuning(b: *const erp_batch, chosen: *mut i32, seqs: *mut i32, ms: *mut f32, cap: i32,
                                     count: *mut i32) -> erp_status;
    pub fn erp_batch_packed(b: *const erp_batch, packed_instances: *mut i32) -> erp_status;
    pub fn erp_batch_destroy(b: *mut erp_batch);

    // a stream of jobs: continuous batching under an HBM budget
    pub fn erp_server_create(p: *const erp_server_params, out: *mut *mut erp_server) -> erp_status;
    pub fn erp_server_submit(s: *mut erp_server, job_id: i64, d: *const erp_design,
                             p: *const erp_params) -> erp_status;
    pub fn erp_server_pump(s: *mut erp_server, active: *mut i32, queued: *mut i32) -> erp_status;
    pub fn erp_server_cancel(s: *mut erp_server, job_id: i64) -> erp_status;
    pub fn erp_server_poll(s: *mut erp_server, out: *mut erp_job_result, cap: i32, count: *mut i32) -> erp_status;
    pub fn erp_server_positions(s: *mut erp_server, job_id: i64, x: *mut f32, y: *mut f32) -> erp_status;
    pub fn erp_server_now(s: *const erp_server) -> f64;
    pub fn erp_server_last_error(s: *const erp_server) -> *const c_char;
    pub fn erp_server_destroy(s: *mut erp_server);
    pub fn erp_estimate_footprint(d: *const erp_design, p: *const erp_params, bytes: *mut i64) -> erp_status;

    // read_db::<f32>(lef, def, verbose) (src/main.rs:69) and the placed DEF
    pub fn erp_lefdef_read(lef_paths: *const *const c_char, num_lef: i32, def_path: *const c_char,
                           out: *mut *mut erp_netlist) -> erp_status;
    pub fn erp_lefdef_last_error() -> *const c_char;
    pub fn erp_netlist_design(nl: *const erp_netlist, d: *mut erp_design) -> erp_status;
    pub fn erp_netlist_stats(nl: *const erp_netlist, s: *mut erp_lefdef_stats) -> erp_status;
    pub fn erp_netlist_node_name(nl: *const erp_netlist, instance: i32) -> *const c_char;
    pub fn erp_netlist_net_name(nl: *const erp_netlist, net: i32) -> *const c_char;
    pub fn erp_netlist_from_design(d: *const erp_design, p: *const erp_lefdef_params,
                                   out: *mut *mut erp_netlist) -> erp_status;
    pub fn erp_lefdef_write(nl: *const erp_netlist, lef_path: *const c_char, def_path: *const c_char) -> erp_status;
    pub fn erp_def_write_placed(nl: *const erp_netlist, x: *const f32, y: *const f32,
                                def_path: *const c_char) -> erp_status;
    pub fn erp_netlist_destroy(nl: *mut erp_netlist);

    // seeded synthetic netlists (stand-in for read_db on the ISPD designs)
    pub fn erp_synth_create(p: *const erp_synth_params, out: *mut *mut erp_synth) -> erp_status;
    pub fn erp_synth_design(s: *const erp_synth, d: *mut erp_design) -> erp_status;
    pub fn erp_synth_destroy(s: *mut erp_synth);

    // the Poisson part of compute_potential on device buffers
    pub fn erp_spectral_create(m: i32, n: i32, bin_w: f32, bin_h: f32, precision: i32, stream: *mut c_void,
                               out: *mut *mut erp_spectral) -> erp_status;
    pub fn erp_spectral_solve(sp: *mut erp_spectral, rho: *const f32, field_x: *mut f32, field_y: *mut f32,
                              potential: *mut f32) -> erp_status;
    pub fn erp_spectral_destroy(sp: *mut erp_spectral);
    // allocation-free form of the solve (no counterpart in the reference)
    pub fn erp_spectral_solve_noalloc(m: i32, n: i32, bin_w: f32, bin_h: f32, rho: *const f32,
                                      field_x: *mut f32, field_y: *mut f32, potential: *mut f32,
                                      stream: *mut c_void) -> erp_status;
}

fn message(p: *const c_char) -> String {
    if p.is_null() {
        return String::from("unknown error");
    }
    unsafe { CStr::from_ptr(p) }.to_string_lossy().into_owned()
}

/// The reference panics on failure; the binding returns the library's message.
#[derive(Debug)]
pub struct Gb300Error {
    pub status: erp_status,
    pub message: String,
}

impl std::fmt::Display for Gb300Error {
    fn fmt(&self, f: &mut std::fmt::Formatter<'_>) -> std::fmt::Result {
        write!(f, "erplacer_gb300 status {}: {}", self.status, self.message)
    }
}

impl std::error::Error for Gb300Error {}

/// Borrowed view of a design in the erp_design layout.  Build it from the
/// DB<f32> fields (src/placement.rs:159-178): `macro_2_pins` flattened into
/// `inst_pin_ptr` / `inst_pins`, `nets[i].pin_ids` into `net_ptr` / `net_pins`
/// with the two-pin nets first.
pub struct DesignView<'a> {
    pub num_movable: usize,
    pub n_2nets: usize,
    pub x: &'a [f32],
    pub y: &'a [f32],
    pub w: &'a [f32],
    pub h: &'a [f32],
    pub num_pins_f: &'a [f32],
    pub pin_ox: &'a [f32],
    pub pin_oy: &'a [f32],
    pub pin_inst: &'a [i32],
    pub net_ptr: &'a [i32],
    pub net_pins: &'a [i32],
    pub inst_pin_ptr: &'a [i32],
    pub inst_pins: &'a [i32],
    pub die_w: f32,
    pub die_h: f32,
    pub cell_utilization: f32,
    pub movable_area: f32,
}

impl DesignView<'_> {
    fn raw(&self) -> erp_design {
        erp_design {
            num_nodes: self.x.len() as i32,
            num_movable: self.num_movable as i32,
            num_pins: self.pin_inst.len() as i32,
            num_nets: (self.net_ptr.len() - 1) as i32,
            n_2nets: self.n_2nets as i32,
            _pad: 0,
            x: self.x.as_ptr(),
            y: self.y.as_ptr(),
            w: self.w.as_ptr(),
            h: self.h.as_ptr(),
            num_pins_f: self.num_pins_f.as_ptr(),
            pin_ox: self.pin_ox.as_ptr(),
            pin_oy: self.pin_oy.as_ptr(),
            pin_inst: self.pin_inst.as_ptr(),
            net_ptr: self.net_ptr.as_ptr(),
            net_pins: self.net_pins.as_ptr(),
            inst_pin_ptr: self.inst_pin_ptr.as_ptr(),
            inst_pins: self.inst_pins.as_ptr(),
            die_w: self.die_w,
            die_h: self.die_h,
            cell_utilization: self.cell_utilization,
            movable_area: self.movable_area,
        }
    }
}

/// Stand-in for `Placement` (src/placement.rs:141-228) with the loop on the GPU.
pub struct Gb300Placement {
    ctx: *mut erp_ctx,
    num_nodes: usize,
}

impl Gb300Placement {
    /// Placement::new: bins 512 x 512 and cell_utilization as the target
    /// density unless given; the reference's exact-centre start.
    pub fn new(d: &DesignView, bins: (i32, i32), target_density: Option<f32>) -> Result<Self, Gb300Error> {
        let raw = d.raw();
        let p = erp_params {
            num_bins_x: bins.0,
            num_bins_y: bins.1,
            target_density: target_density.unwrap_or(-1.0),
            start_mode: ERP_START_CENTER,
            precision: ERP_PREC_FP32,
            device: 0,
            stream: std::ptr::null_mut(),
            flags: 0,
        };
        let mut ctx = std::ptr::null_mut();
        let s = unsafe { erp_create(&raw, &p, &mut ctx) };
        if s != ERP_OK {
            return Err(Gb300Error { status: s, message: message(unsafe { erp_last_error(std::ptr::null()) }) });
        }
        Ok(Gb300Placement { ctx, num_nodes: d.x.len() })
    }

    fn check(&self, s: erp_status) -> Result<(), Gb300Error> {
        if s == ERP_OK {
            Ok(())
        } else {
            Err(Gb300Error { status: s, message: message(unsafe { erp_last_error(self.ctx) }) })
        }
    }

    /// Placement::step: returns Scheduler::should_stop, like the reference.
    pub fn step(&mut self) -> Result<bool, Gb300Error> {
        let mut st = erp_step_stats::default();
        self.check(unsafe { erp_step(self.ctx, &mut st) })?;
        Ok(st.should_stop != 0)
    }

    /// The step for a host that keeps `ps.instances` (src/nesterov.rs:39).
    pub fn step_host(&mut self, x: &mut [f32], y: &mut [f32]) -> Result<erp_step_stats, Gb300Error> {
        assert!(x.len() == self.num_nodes && y.len() == self.num_nodes);
        let mut st = erp_step_stats::default();
        self.check(unsafe { erp_step_host(self.ctx, x.as_mut_ptr(), y.as_mut_ptr(), &mut st) })?;
        Ok(st)
    }

    /// Positions of all nodes, movable first (what draw_placement reads).
    pub fn positions(&mut self) -> Result<(Vec<f32>, Vec<f32>), Gb300Error> {
        let mut x = vec![0f32; self.num_nodes];
        let mut y = vec![0f32; self.num_nodes];
        self.check(unsafe { erp_get_positions(self.ctx, x.as_mut_ptr(), y.as_mut_ptr()) })?;
        Ok((x, y))
    }

    pub fn scalars(&mut self) -> Result<erp_scalars, Gb300Error> {
        let mut s = erp_scalars::default();
        self.check(unsafe { erp_get_scalars(self.ctx, &mut s) })?;
        Ok(s)
    }
}

impl Drop for Gb300Placement {
    fn drop(&mut self) {
        unsafe { erp_destroy(self.ctx) };
    }
}

/// read_db::<f32>(&args.lef, &args.def, verbose) in src/main.rs:69: the
/// netlist stays alive while its design view is used.
pub struct Netlist {
    nl: *mut erp_netlist,
}

impl Netlist {
    pub fn read(lefs: &[&str], def: &str) -> Result<Self, Gb300Error> {
        let lef_c: Vec<CString> = lefs.iter().map(|s| CString::new(*s).unwrap()).collect();
        let lef_p: Vec<*const c_char> = lef_c.iter().map(|s| s.as_ptr()).collect();
        let def_c = CString::new(def).unwrap();
        let mut nl = std::ptr::null_mut();
        let s = unsafe { erp_lefdef_read(lef_p.as_ptr(), lef_p.len() as i32, def_c.as_ptr(), &mut nl) };
        if s != ERP_OK {
            return Err(Gb300Error { status: s, message: message(unsafe { erp_lefdef_last_error() }) });
        }
        Ok(Netlist { nl })
    }

    /// The erp_design of the netlist (pointers valid while `self` lives).
    pub fn design(&self) -> Result<erp_design, Gb300Error> {
        let mut d: erp_design = unsafe { std::mem::zeroed() };
        let s = unsafe { erp_netlist_design(self.nl, &mut d) };
        if s != ERP_OK {
            return Err(Gb300Error { status: s, message: message(unsafe { erp_lefdef_last_error() }) });
        }
        Ok(d)
    }

    /// The placed DEF for legalisation (the reference stops at global placement).
    pub fn write_placed(&self, x: &[f32], y: &[f32], path: &str) -> Result<(), Gb300Error> {
        let p = CString::new(path).unwrap();
        let s = unsafe { erp_def_write_placed(self.nl, x.as_ptr(), y.as_ptr(), p.as_ptr()) };
        if s != ERP_OK {
            return Err(Gb300Error { status: s, message: message(unsafe { erp_lefdef_last_error() }) });
        }
        Ok(())
    }
}

impl Drop for Netlist {
    fn drop(&mut self) {
        unsafe { erp_netlist_destroy(self.nl) };
    }
}
