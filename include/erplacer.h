/*
 * erplacer.h — C ABI of the GB300-native (sm_103a) electrostatic global-placement
 * loop, a drop-in for ERPlacer's (giammirove/reda-erplacer) placement step.
 *
 * One context = one placement design resident on one GPU.  All compute runs in
 * hand-written CUDA kernels on the context's stream; there is no CPU fallback:
 * every entry point fails with ERP_ECUDA / ERP_ENODEV when no usable GPU is
 * present.  Host arrays passed in are copied; the caller keeps ownership.
 * Calls on one context must come from one host thread at a time.
 *
 * Each entry point names the reference function it replaces (file:line in the
 * reference crate).  The reference functions are `pub(crate)` Rust; the Rust
 * binding a maintainer adds is reda_erplacer_gb300/rust/ffi.rs (the extern "C"
 * block and a safe Placement stand-in) with reda_erplacer_gb300/rust/build.rs.
 */
#ifndef ERPLACER_H
#define ERPLACER_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ERP_ABI_VERSION 1

typedef enum erp_status {
    ERP_OK = 0,
    ERP_EINVAL = 1,     /* bad argument or design (message in erp_last_error) */
    ERP_ENOMEM = 2,     /* device or host allocation failed */
    ERP_ECUDA = 3,      /* CUDA runtime error */
    ERP_ENAN = 4,       /* non-finite value detected in positions or gradients */
    ERP_ETIMEDOUT = 5,  /* a bounded device wait ran out */
    ERP_ENOTSUP = 6,    /* feature not supported for these parameters */
    ERP_ENODEV = 7,     /* no CUDA device of compute capability 10.3 */
    ERP_ESTATE = 8,     /* call not valid in the current state */
    ERP_ECANCELED = 9   /* the job was cancelled (erp_server_cancel) */
} erp_status;

/* Placement database, structure-of-arrays + CSR (the fields of reda-db's
 * DB<T> that the loop reads; semantics restated from their use sites):
 *  - instances: movable first (src/placement.rs:125); (x, y) lower-left DEF
 *    coordinates; fixed IO pins are zero-size instances;
 *  - num_pins_f: per-instance pin count stored as float (src/nesterov.rs:78);
 *  - pins: offsets from the owning instance's lower-left corner
 *    (src/hpwl.rs:107); pin_inst maps a pin to its instance;
 *  - nets: CSR over pin ids; the first n_2nets nets have exactly two pins
 *    (src/hpwl.rs:159,173);
 *  - inst_pin_ptr / inst_pins: per-instance pin lists (macro_2_pins);
 *  - the die spans [0, die_w] x [0, die_h] (src/nesterov.rs:131). */
typedef struct erp_design {
    int32_t num_nodes;
    int32_t num_movable;
    int32_t num_pins;
    int32_t num_nets;
    int32_t n_2nets;
    int32_t _pad;
    const float *x, *y;
    const float *w, *h;
    const float *num_pins_f;
    const float *pin_ox, *pin_oy;
    const int32_t *pin_inst;
    const int32_t *net_ptr;
    const int32_t *net_pins;
    const int32_t *inst_pin_ptr;
    const int32_t *inst_pins;
    float die_w, die_h;
    float cell_utilization;   /* default target density (src/placement.rs:134) */
    float movable_area;       /* overflow normaliser (src/epotential.rs:277) */
} erp_design;

typedef enum erp_start_mode {
    ERP_START_CENTER = 0,     /* reference rule: movable cells at the die centre (src/placement.rs:109-139) */
    ERP_START_DB = 1          /* keep the design's coordinates (e.g. a jittered start) */
} erp_start_mode;

typedef enum erp_precision {
    ERP_PREC_FP32 = 0,        /* FP32 spectral solve (FFT-based DCT/DST), the parity path */
    ERP_PREC_TF32_GEMM = 1,   /* spectral solve as DCT/IDXST matrix contractions on tcgen05, TF32
                                 operands, FP32 accumulation (erp_spectral_create and placement
                                 contexts; bins multiples of 128); ~2e-3 against FP64 */
    ERP_PREC_BF16X3_GEMM = 2  /* same contractions with bf16 hi/lo split operands, three products
                                 hi.hi + hi.lo + lo.hi, FP32 accumulation; ~1e-5 against FP64 */
} erp_precision;

typedef struct erp_params {
    int32_t num_bins_x;       /* 0: 512 like the reference (src/placement.rs:50); power of two, 16..4096 */
    int32_t num_bins_y;
    float target_density;     /* < 0: design cell_utilization (reference rule) */
    int32_t start_mode;       /* erp_start_mode */
    int32_t precision;        /* erp_precision */
    int32_t device;           /* CUDA device ordinal */
    void *stream;             /* cudaStream_t to run on; NULL: the context creates its own */
    int32_t flags;            /* 0, or ERP_FLAG_EXPIRE_WAITS */
} erp_params;

/* Test hook of the bounded device waits.  Every kernel wait on a bulk copy
 * into shared memory gives up at once instead of after its limit; the kernel
 * then drains the copy with the full limit, records the timeout and retires
 * the context, exactly as when a copy really stalls, and the call returns
 * ERP_ETIMEDOUT.  Nothing on the device is left waiting or in flight.  Only
 * the FP32 spectral path's row pass waits on copies, at bin counts of 64 and
 * more in the row direction; other contexts ignore the flag. */
#define ERP_FLAG_EXPIRE_WAITS 1

/* One Placement::step's scalars (the reference logs these every 10
 * iterations, src/placement.rs:213-223).  gamma and density_weight are the
 * values the step used, before the scheduler update. */
typedef struct erp_step_stats {
    int32_t iteration;        /* iteration index of the step */
    int32_t should_stop;      /* Scheduler::should_stop after the update */
    float hpwl;
    float overflow;
    float density_weight;
    float gamma;
    float alpha;              /* Nesterov step length after the step */
    float beta;
} erp_step_stats;

typedef struct erp_ctx erp_ctx;

const char *erp_status_string(erp_status s);
/* Last error message of a context (NULL ctx: last error of erp_create on this thread). */
const char *erp_last_error(const erp_ctx *ctx);
int32_t erp_abi_version(void);

/* Placement::new (src/placement.rs:159-178): Bins::new, PlacementSolution::new,
 * PotentialComputation::new (incl. the fixed-cell initial density map),
 * HpwlComputation::new, Scheduler::new, Nesterov::new.
 * The context's device arrays are one stream-ordered allocation from the
 * library's own memory pool on the device; erp_destroy returns it to that pool,
 * which keeps up to 8 GiB of freed memory for later contexts (the rest goes
 * back to the system).  Not supported: cudaDeviceReset on a device after its
 * first context (kernel attributes are set once per device and process). */
erp_status erp_create(const erp_design *design, const erp_params *params, erp_ctx **out);
void erp_destroy(erp_ctx *ctx);

/* compute_hpwl (src/hpwl.rs:139-343): WA wirelength gradient (kept on the
 * device) and the HPWL total (double-float reduction in a fixed order, returned as
 * FP64).  hpwl may be NULL (no sync). */
erp_status erp_wirelength(erp_ctx *ctx, float gamma, float *hpwl);

/* compute_potential (src/epotential.rs:225-374): density scatter (int64 fixed
 * point), overflow, spectral Poisson solve, electric force.  energy may be NULL
 * (then the potential map is skipped, as the caller discards it,
 * src/placement.rs:185); overflow may be NULL (no sync). */
erp_status erp_potential(erp_ctx *ctx, int32_t iteration, float *energy, float *overflow);

/* Nesterov::step_adaptive (src/nesterov.rs:27-146) on the gradients of the last
 * erp_wirelength / erp_potential calls, with the context's density weight. */
erp_status erp_nesterov(erp_ctx *ctx, int32_t iteration);

/* Scheduler::update (src/scheduler.rs:68-73) with host-supplied metrics. */
erp_status erp_scheduler_update(erp_ctx *ctx, float hpwl, float overflow);
/* Scheduler::should_stop (src/scheduler.rs:75-81). */
erp_status erp_should_stop(erp_ctx *ctx, int32_t *stop);

/* Placement::step (src/placement.rs:180-228): one whole iteration, replayed from
 * a captured CUDA graph; the scheduler runs on the device.  stats may be NULL:
 * then the call only enqueues work (no host sync). */
erp_status erp_step(erp_ctx *ctx, erp_step_stats *stats);

/* Drop-in form for a host that owns the coordinates (the reference's
 * ps.instances, mutated by step_adaptive, src/nesterov.rs:39): copies x/y
 * (all nodes) to the device, runs one step, copies the new x/y back.  When x
 * and y each lie in one page-locked allocation (cudaHostAlloc or
 * cudaHostRegister) that covers all nodes, the device reads and writes them
 * directly instead; an array whose first or last element is not page-locked
 * goes through copies. */
erp_status erp_step_host(erp_ctx *ctx, float *x, float *y, erp_step_stats *stats);

/* Run up to max_iterations steps (the CLI loop, src/main.rs:78-90), stopping
 * early once overflow <= stop_overflow (stop_overflow <= 0: never).  Returns
 * the number of iterations run and the last step's stats. */
erp_status erp_run(erp_ctx *ctx, int32_t max_iterations, float stop_overflow,
                   int32_t *iterations_run, erp_step_stats *last);

/* Scheduler / optimiser scalars. */
typedef struct erp_scalars {
    int32_t iteration;
    float gamma, base_gamma, density_weight;
    float alpha, beta;
    float hpwl_initial, hpwl_current, hpwl_previous;
    float overflow_current, overflow_previous;
    double hpwl_last;         /* HPWL total of the last wirelength pass (double-float sum) */
    double overflow_last;     /* overflow of the last potential pass (double-float sum) */
    double energy_last;
    int32_t fixed_shift;      /* S: movable density contributions are rint(v * 2^S) */
    int32_t fixed_shift_init; /* S0 for the fixed-cell initial map */
    int32_t num_bins_x, num_bins_y;
    float bin_w, bin_h, target_density;
    int32_t graph_kernels;    /* kernel launches in one captured Placement::step (0 before the first erp_step) */
} erp_scalars;
erp_status erp_get_scalars(erp_ctx *ctx, erp_scalars *out);
erp_status erp_set_scalars(erp_ctx *ctx, int32_t iteration, float gamma, float density_weight,
                           float alpha, float beta);

/* Positions of all nodes (movable first). */
erp_status erp_get_positions(erp_ctx *ctx, float *x, float *y);
erp_status erp_set_positions(erp_ctx *ctx, const float *x, const float *y);
/* Nesterov history (prev coords / prev grads) of all nodes. */
erp_status erp_set_nesterov_history(erp_ctx *ctx, const float *prev_x, const float *prev_y,
                                    const float *prev_gx, const float *prev_gy);

/* Device arrays readable for inspection and tests (copied to host memory). */
typedef enum erp_array {
    ERP_ARR_WL_GRAD_X = 0,    /* float [num_nodes] hc.grad_x */
    ERP_ARR_WL_GRAD_Y = 1,
    ERP_ARR_DENS_GRAD_X = 2,  /* float [num_nodes] pc.grad_x */
    ERP_ARR_DENS_GRAD_Y = 3,
    ERP_ARR_PIN_GRAD_X = 4,   /* float [num_pins] grad_pins_x, original pin order */
    ERP_ARR_PIN_GRAD_Y = 5,
    ERP_ARR_DENSITY_I64 = 6,  /* int64 [m*n] movable fixed-point sums of the last potential pass */
    ERP_ARR_DENSITY = 7,      /* float [m*n] density map scaled by 1/bin_area */
    ERP_ARR_INITIAL = 8,      /* float [m*n] fixed-cell map x target density */
    ERP_ARR_FIELD_X = 9,      /* float [m*n] */
    ERP_ARR_FIELD_Y = 10,
    ERP_ARR_POTENTIAL = 11,   /* float [m*n] (only after erp_potential with energy != NULL) */
    ERP_ARR_PREV_X = 12,
    ERP_ARR_PREV_Y = 13,
    ERP_ARR_PREV_GX = 14,
    ERP_ARR_PREV_GY = 15,
    ERP_ARR_NET_HPWL = 16     /* float [num_nets] per-net HPWL, original net order */
} erp_array;
erp_status erp_get_array(erp_ctx *ctx, erp_array which, void *dst, size_t bytes);

/* Block until the context's stream is idle. */
erp_status erp_synchronize(erp_ctx *ctx);

/* ---- headless snapshots (src/drawing.rs:7-60 draw_placement,
 * src/epotential.rs:199-223 draw_density_map), rasterised on the device into
 * RGB bytes; the caller writes the image file (no graphics API).
 * Placement: width = ceil(die_w), height = ceil(die_h) pixels, one pixel per
 * unit; white background, movable instances blue, fixed red, later instances
 * over earlier ones, zero-size instances skipped, row 0 at the top.
 * Density: m x n pixels (bin (i, j) at column i, row n-1-j) of the density map
 * of the current positions, min-max normalised, blue (low) to red (high). ---- */
erp_status erp_snapshot_size(erp_ctx *ctx, int32_t *width, int32_t *height);
erp_status erp_snapshot_placement(erp_ctx *ctx, uint8_t *rgb, size_t bytes);   /* width*height*3 */
erp_status erp_snapshot_density(erp_ctx *ctx, uint8_t *rgb, size_t bytes);     /* m*n*3 */

/* ---- checkpoint / resume (no counterpart in the reference): the state one
 * Placement::step hands to the next -- positions, the Nesterov history and the
 * scheduler / optimiser scalars -- in a versioned host buffer.  Restoring into
 * a context of the same design and bin grid continues the run bit-identically;
 * other buffers are rejected with ERP_EINVAL. ---- */
erp_status erp_checkpoint_size(erp_ctx *ctx, size_t *bytes);
erp_status erp_checkpoint(erp_ctx *ctx, void *buf, size_t bytes);
erp_status erp_restore(erp_ctx *ctx, const void *buf, size_t bytes);

/* ---- batched instances ----
 * Many designs advance together (the reference drives one design from its CLI
 * loop, src/main.rs:78-90; here that loop runs for a whole table of designs).
 * One CUDA graph holds one branch per instance -- each branch is that
 * instance's whole Placement::step -- so one graph launch moves every unfinished
 * instance by one iteration and independent instances overlap on the GPU.  An
 * instance retires on the device once its overflow <= stop_overflow or its
 * iteration budget is spent; its kernels then return at entry. */
typedef struct erp_batch erp_batch;
erp_status erp_batch_create(const erp_design *designs, const erp_params *params, int32_t count,
                            erp_batch **out);
/* Run every instance for up to max_iterations more steps (stop_overflow <= 0:
 * never early).  iterations[i] and last[i] (either may be NULL) receive each
 * instance's step count and final step record. */
erp_status erp_batch_run(erp_batch *b, int32_t max_iterations, float stop_overflow,
                         int32_t *iterations, erp_step_stats *last);
/* The context of instance i (owned by the batch: do not destroy it). */
erp_ctx *erp_batch_context(erp_batch *b, int32_t i);
int32_t erp_batch_size(const erp_batch *b);
const char *erp_batch_last_error(const erp_batch *b);
void erp_batch_destroy(erp_batch *b);
/* The batch's autotuned shape of the density scatter (no counterpart in the
 * reference).  erp_batch_create times candidate block shapes -- movable cells per
 * scatter block, 0 meaning the rule of a context run alone -- on all instances'
 * scatters running together, and keeps, among the candidates within 10 % of the
 * fastest, the one with the fewest blocks.  The shape decides no bit of the
 * results.  *chosen receives it; cells[i] / ms[i] (up to cap entries) each
 * candidate and its time; *count the number of candidates.  The environment variable ERP_BATCH_SCATTER_CELLS
 * fixes the shape instead (count 0). */
erp_status erp_batch_tuning(const erp_batch *b, int32_t *chosen, int32_t *cells, float *ms, int32_t cap,
                            int32_t *count);
/* The batch's autotuned tile shape of the FP32 spectral passes (no counterpart in
 * the reference): the sequences -- rows or columns -- per block of the passes that
 * serve sides 64..256, 0 meaning the fixed shape (four), else 2 or 8.
 * erp_batch_create times the candidates on all FP32 instances' three passes
 * running together and keeps the fastest; instances on the tensor-core solve
 * and instances without such a side keep the fixed shape.  The shape decides no
 * bit of the results.  *chosen receives it; seqs[i] / ms[i] (up to cap entries)
 * each candidate and its time; *count the number of candidates (0 when no
 * instance had such a side).  The environment variable ERP_BATCH_SPECTRAL_SEQS
 * (2 or 8; anything else: the fixed shape) fixes the shape instead (count 0). */
erp_status erp_batch_spectral_tuning(const erp_batch *b, int32_t *chosen, int32_t *seqs, float *ms, int32_t cap,
                                     int32_t *count);
/* How many of the batch's instances advance in packed launches (no counterpart
 * in the reference): every FP32 instance whose bin grid is 64..256 on both axes,
 * with movable cells and nets and at most 100,000 movable cells (the environment
 * variable ERP_BATCH_PACK_MAX_CELLS sets that cap), runs each stage of its step inside one
 * launch per stage and kernel variant that covers all such instances -- each
 * block finds its instance in a packed table of their arguments -- instead of a
 * graph branch of its own kernels; the rest keep a branch each.  The results are
 * those of each instance run alone, bit for bit.  With fewer than four such
 * instances every instance keeps a branch (count 0), and the same rule applies
 * whenever retirements leave fewer than four active.  The environment variable
 * ERP_BATCH_FORM=branches gives every instance a branch instead (count 0). */
erp_status erp_batch_packed(const erp_batch *b, int32_t *packed_instances);

/* ---- serving: continuous batching of placement jobs ----
 * Jobs are submitted as they arrive and wait in a FIFO queue.  Each
 * erp_server_pump round admits queued jobs while their device footprint fits
 * the HBM budget (and the active-job cap), runs `chunk` iterations of every
 * active job -- each job replays its own captured step graph on its own stream;
 * with the environment variable ERP_SERVER_FORM=packed, four or more active
 * jobs of the kind batches pack run as one graph of packed launches instead,
 * rebuilt when that set changes -- and retires jobs whose overflow <=
 * stop_overflow or whose iteration budget is spent, freeing their memory for
 * the next admissions.  Results are each job's alone, bit for bit, in either
 * form.  Times are seconds on the server's steady clock. */
typedef struct erp_server_params {
    int32_t device;
    int32_t max_active;         /* jobs on the GPU at once (1: one job at a time) */
    int64_t hbm_budget_bytes;   /* admission budget for the jobs' device memory */
    int32_t max_iterations;     /* per job */
    float stop_overflow;        /* retire threshold (<= 0: run max_iterations) */
    int32_t chunk;              /* iterations per scheduling round */
    int32_t keep_positions;     /* 1: keep each retired job's final positions */
} erp_server_params;

typedef struct erp_job_result {
    int64_t job_id;
    int32_t status;             /* erp_status of the job */
    int32_t iterations;
    erp_step_stats last;
    double submit_s, admit_s, finish_s;
    int64_t footprint_bytes;
} erp_job_result;

typedef struct erp_server erp_server;
erp_status erp_server_create(const erp_server_params *p, erp_server **out);
/* Queue a job (the design's arrays are copied).  params may be NULL. */
erp_status erp_server_submit(erp_server *s, int64_t job_id, const erp_design *design,
                             const erp_params *params);
/* One scheduling round; reports the active and queued job counts. */
erp_status erp_server_pump(erp_server *s, int32_t *active, int32_t *queued);
/* Withdraw a job: a queued one leaves the queue; a running one retires at once
 * (the iterations already launched for it finish on the device, and its memory
 * is released when they have); one still being set up retires when the set-up
 * ends.  Its result carries ERP_ECANCELED and the state it reached.  The other
 * jobs are not affected.  ERP_EINVAL if no queued or running job has this id. */
erp_status erp_server_cancel(erp_server *s, int64_t job_id);
/* Move up to `cap` finished jobs into out[]; *count receives how many. */
erp_status erp_server_poll(erp_server *s, erp_job_result *out, int32_t cap, int32_t *count);
/* Final positions of a retired job (keep_positions = 1). */
erp_status erp_server_positions(erp_server *s, int64_t job_id, float *x, float *y);
double erp_server_now(const erp_server *s);
const char *erp_server_last_error(const erp_server *s);
void erp_server_destroy(erp_server *s);
/* Device bytes a context for this design would allocate. */
erp_status erp_estimate_footprint(const erp_design *design, const erp_params *params, int64_t *bytes);

/* ---- profiling (the reference's time_it phases, src/utils.rs:106-124) ----
 * Times each stage of one step in isolation: `reps` launches, each preceded by
 * an L2 flush (a 256 MiB device write, untimed), bracketed by CUDA events on
 * the context's stream.  ms_out[ERP_NUM_STAGES] receives the mean per launch.
 * Mutates the placement state (positions, scheduler): call it after the
 * measured run. */
typedef enum erp_stage {
    ERP_STAGE_WIRELENGTH = 0, /* WA nets + HPWL reduction (pin gradients) */
    ERP_STAGE_WL_GATHER = 1,  /* instance gradients from the pin gradients */
    ERP_STAGE_DENSITY = 2,    /* map clear + density scatter */
    ERP_STAGE_SPECTRAL = 3,   /* map conversion + overflow + Poisson solve (3 passes) */
    ERP_STAGE_FORCE = 4,      /* electric force gather (+ the iteration-0 density-weight rescale) */
    ERP_STAGE_NESTEROV = 5,   /* preconditioned gradient / Lipschitz + update */
    ERP_STAGE_SCHEDULER = 6,
    ERP_NUM_STAGES = 7
} erp_stage;
/* reps > 0: each stage alone, L2 flushed before every launch (mutates the
 * state).  reps < 0: -reps whole steps launched in graph order with an event
 * between the stages and warm caches (advances the placement by -reps + 1
 * iterations).  ms_out receives ERP_NUM_STAGES mean milliseconds. */
erp_status erp_profile_stages(erp_ctx *ctx, int32_t reps, float *ms_out);

/* ---- standalone spectral solve (the Poisson part of compute_potential,
 * src/epotential.rs:284-343) on device buffers, for the isolated-solve
 * workload.  All pointers are device pointers of m*n floats; potential may be
 * NULL. ---- */
typedef struct erp_spectral erp_spectral;
erp_status erp_spectral_create(int32_t m, int32_t n, float bin_w, float bin_h, int32_t precision,
                               void *stream, erp_spectral **out);
erp_status erp_spectral_solve(erp_spectral *sp, const float *rho_dev, float *field_x_dev,
                              float *field_y_dev, float *potential_dev);
void erp_spectral_destroy(erp_spectral *sp);

/* Allocation-free form of erp_spectral_create + erp_spectral_solve, for callers
 * that cannot call cudaMalloc: hosts whose device memory belongs to another
 * allocator's pool (a framework caching allocator, a pre-reserved arena) and
 * loops that must not stall on cudaFree's device-wide synchronisation.  It has
 * no counterpart in the reference.  All intermediates live in one file-scope
 * device array of about 4.1 MiB that every GPU loading the library holds until
 * exit; grids above ERP_NOALLOC_MAX_BINS (the reference's 512 x 512) are
 * rejected with ERP_EINVAL.  The caller passes device buffers of m*n floats
 * (potential may be NULL) and a stream (NULL: the legacy default stream).
 * The first call on a device looks up the array's address and sets kernel
 * limits: make it before any stream capture.  That address is kept for the
 * life of the process: cudaDeviceReset after the first call is not supported.
 * Every call reuses the array, so calls that overlap on the GPU race;
 * sequential calls are independent.  Results agree with erp_spectral_solve
 * within FP32 rounding (its twiddle tables are built on the device), not bit
 * for bit. */
#define ERP_NOALLOC_MAX_BINS (512 * 512)
erp_status erp_spectral_solve_noalloc(int32_t m, int32_t n, float bin_w, float bin_h,
                                      const float *rho_dev, float *field_x_dev,
                                      float *field_y_dev, float *potential_dev, void *stream);

/* ---- seeded synthetic netlists (stand-in for reda-db's read_db on the
 * LEF/DEF benchmarks, which are not shipped) ---- */
typedef struct erp_synth_params {
    int64_t seed;
    int32_t num_cells;        /* movable standard cells */
    int32_t num_nets;
    int32_t num_io;           /* fixed IO pins on the die boundary */
    int32_t num_macros;       /* fixed rectangular macros */
    float macro_area_frac;    /* each macro's share of the die area (e.g. 0.015) */
    float utilization;        /* movable area / free area */
    float site_w, row_h;      /* 0.2 / 2.0 um */
    int32_t min_sites, max_sites; /* cell width range in sites (2..16) */
    float jitter_frac;        /* start jitter sigma as a fraction of die width (0.001) */
} erp_synth_params;
typedef struct erp_synth erp_synth;
erp_status erp_synth_create(const erp_synth_params *p, erp_synth **out);
/* Fills *d with pointers into the generator's host arrays (valid until destroy). */
erp_status erp_synth_design(const erp_synth *s, erp_design *d);
void erp_synth_destroy(erp_synth *s);

/* ---- LEF/DEF: ingest (replaces reda_db::read_db::<f32>(lef, def, verbose),
 * src/main.rs:69), export, and the placed-DEF hand-off to legalisation (the
 * step after global placement, which the reference does not write,
 * README.md:23).  Host code only: these calls need no GPU.
 *
 * The design a netlist exposes (erp_netlist_design) follows the erp_design
 * rules above: movable components (DEF status PLACED / UNPLACED) first in DEF
 * order, then FIXED / COVER components, then the DEF PINS as zero-size fixed
 * instances; microns with the DIEAREA's lower-left corner at the origin; a
 * pin's offset is the centre of its LEF port shapes after ORIGIN and the
 * component orientation; nets with at least one connection, the two-pin nets
 * first; LEF geometry snapped to the LEF database grid.  Errors are ERP_EINVAL
 * (ERP_ENOMEM) with "file:line: message" in erp_lefdef_last_error(). ---- */
typedef struct erp_netlist erp_netlist;
typedef struct erp_lefdef_stats {
    int32_t num_nodes, num_movable, num_fixed, num_io;
    int32_t num_nets, num_pins, num_macros;
    int32_t num_dropped_nets;    /* NETS entries without a connection */
    int32_t num_skipped_conns;   /* "( * pin )" wildcards and MUSTJOIN entries */
    int32_t num_unplaced_io;     /* DEF PINS without a location (placed at the die corner) */
    int32_t def_dbu, lef_dbu;    /* DEF UNITS DISTANCE MICRONS; the LEF snap grid */
    int64_t die[4];              /* DIEAREA bounding box, DEF units: x0 y0 x1 y1 */
} erp_lefdef_stats;

/* Read LEF files in order (technology, then cells; a later MACRO of the same
 * name replaces an earlier one), then the DEF.  The netlist keeps the DEF text
 * for erp_def_write_placed. */
erp_status erp_lefdef_read(const char *const *lef_paths, int32_t num_lef, const char *def_path, erp_netlist **out);
/* The message of the last failed LEF/DEF call on this thread. */
const char *erp_lefdef_last_error(void);
/* Fills *d with pointers into the netlist's arrays (valid until destroy). */
erp_status erp_netlist_design(const erp_netlist *nl, erp_design *d);
erp_status erp_netlist_stats(const erp_netlist *nl, erp_lefdef_stats *s);
/* Names in design order (NULL when out of range). */
const char *erp_netlist_node_name(const erp_netlist *nl, int32_t instance);
const char *erp_netlist_net_name(const erp_netlist *nl, int32_t net);

/* A netlist of an in-memory design (e.g. erp_synth_design), for export:
 * movable instances become PLACED components c<i>, sized fixed instances FIXED
 * components m<i> of CLASS BLOCK macros, zero-size fixed instances with at most
 * one pin DEF PINS p<k>; nets n<e>; one macro per distinct (size, pin offsets),
 * pins P<j> in inst_pins order.  Coordinates snap to 1/dbu micron, so the
 * netlist's own design (erp_netlist_design) is the design as LEF/DEF carries it,
 * and reading the written files back gives that design exactly. */
typedef struct erp_lefdef_params {
    int32_t dbu;              /* database units per micron (0: 2000) */
    float site_w, row_h;      /* core site for the SITE and ROW statements (0: none) */
} erp_lefdef_params;
erp_status erp_netlist_from_design(const erp_design *d, const erp_lefdef_params *p, erp_netlist **out);
/* Write the netlist as LEF and/or DEF (either path may be NULL). */
erp_status erp_lefdef_write(const erp_netlist *nl, const char *lef_path, const char *def_path);
/* The placed DEF: movable instance k (design order, k < num_movable) at
 * (x[k], y[k]) microns, written as "PLACED ( X Y ) orient" in DEF units (rounded
 * to nearest).  For a netlist read from a DEF, the source text is copied
 * byte for byte except those clauses (ROW, TRACKS, SPECIALNETS, routing ...
 * are kept for the legaliser); for one made from a design, the DEF is written
 * anew. */
erp_status erp_def_write_placed(const erp_netlist *nl, const float *x, const float *y, const char *def_path);
void erp_netlist_destroy(erp_netlist *nl);

#ifdef __cplusplus
}
#endif
#endif
