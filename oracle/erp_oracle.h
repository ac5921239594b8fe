/*
 * erp_oracle.h — CPU restatement of ERPlacer's electrostatic global-placement
 * loop (giammirove/reda-erplacer, Rust crate `reda-erplacer`).
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the correctness oracle and the
 * timed CPU baseline.  Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline / reference legs load it.  The product library
 * (liberplacer_gb300.so) never links, calls or falls back to it.
 *
 * Parity status: UNPINNED against the reference binary.  The reference is Rust
 * (no cargo/rustc here) and depends on un-vendored git crates (reda-db,
 * reda-lefdef) with no Cargo.lock, and its known-answer fixtures
 * (tests/fft2/..., tests/density/...) are not shipped.  The restatement is
 * pinned instead against closed-form definitions computed independently in
 * FP64 (tests/golden/, generated by tests/golden/make_golden.py): the 2-D
 * DCT-II / DCT-III / DXST transforms, the weighted-average wirelength gradient
 * and the bin-overlap density of single cells.
 *
 * Every function cites the reference file:line it follows.  Arithmetic is
 * FP32 (the reference instantiates T = f32, src/main.rs:69) unless a mode flag
 * below selects the documented FP64 / fixed-point variants that the GPU path
 * uses.  Compile with -ffp-contract=off: the reference never fuses a*b+c.
 */
#ifndef ERP_ORACLE_H
#define ERP_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Placement database view (the fields of reda-db's DB<T> that the loop reads,
 * restated from their use sites: src/placement.rs:109-139, src/hpwl.rs:24-135,
 * src/epotential.rs:58-171, src/nesterov.rs:27-146).
 *  - instances: movable first (src/placement.rs:125), lower-left coordinates;
 *  - pins: offsets from the owning instance's lower-left corner (src/hpwl.rs:107);
 *  - nets: CSR over pin ids, the first n_2nets nets have exactly two pins
 *    (src/hpwl.rs:159,173);
 *  - inst_pin_ptr/inst_pins: the per-instance pin lists (macro_2_pins). */
typedef struct erpo_design {
    int32_t num_nodes;
    int32_t num_movable;
    int32_t num_pins;
    int32_t num_nets;
    int32_t n_2nets;
    int32_t _pad;
    const float *x, *y;          /* [num_nodes] DEF coordinates */
    const float *w, *h;          /* [num_nodes] sizes */
    const float *num_pins_f;     /* [num_nodes] pin count stored as T */
    const float *pin_ox, *pin_oy;/* [num_pins] */
    const int32_t *pin_inst;     /* [num_pins] */
    const int32_t *net_ptr;      /* [num_nets+1] */
    const int32_t *net_pins;     /* [net_ptr[num_nets]] */
    const int32_t *inst_pin_ptr; /* [num_nodes+1] */
    const int32_t *inst_pins;    /* [inst_pin_ptr[num_nodes]] */
    float die_w, die_h;          /* die at the origin (src/nesterov.rs:131) */
    float cell_utilization;      /* reference target density (src/placement.rs:134) */
    float movable_area;          /* overflow normaliser (src/epotential.rs:277) */
} erpo_design;

enum {
    ERPO_START_CENTER = 0,   /* reference rule: movable cells at the die centre */
    ERPO_START_DB = 1        /* keep the DB (DEF) coordinates */
};
enum {
    ERPO_DENSITY_REFERENCE = 0, /* FP32 sums: sequential below iteration 200, per-bin atomic after */
    ERPO_DENSITY_FIXED = 1      /* int64 fixed-point replay of the GPU rule (order independent) */
};

typedef struct erpo_params {
    int32_t num_bins_x;      /* m: the reference hard-codes 512 (src/placement.rs:50) */
    int32_t num_bins_y;      /* n */
    float target_density;    /* < 0: use cell_utilization like the reference */
    int32_t start_mode;      /* ERPO_START_* */
    int32_t density_mode;    /* ERPO_DENSITY_* */
    int32_t reduce_fp64;     /* 1: FP64 accumulators for HPWL, overflow, energy,
                                Lipschitz sums and the scheduler; 0: the
                                reference's FP32 accumulators */
    int32_t num_threads;     /* OpenMP threads, 0 = all */
} erpo_params;

typedef struct erpo_state erpo_state;

/* Read-only view of the oracle state (pointers stay valid until destroy). */
typedef struct erpo_view {
    int32_t m, n;
    float bin_w, bin_h;
    float target_density;
    int32_t fixed_shift;         /* S: movable contributions are llrint(v * 2^S) */
    int32_t fixed_shift_init;    /* S0 for the fixed-cell initial map */
    const float *x, *y;          /* current positions [num_nodes] */
    const float *wl_grad_x, *wl_grad_y;      /* hc.grad_x/y [num_nodes] */
    const float *pin_grad_x, *pin_grad_y;    /* [num_pins] */
    const float *net_hpwl;                   /* [num_nets] */
    const float *dens_grad_x, *dens_grad_y;  /* pc.grad_x/y [num_nodes] */
    const float *clamped_w, *clamped_h, *offset_x, *offset_y, *ratio;
    const float *initial_map;    /* [m*n] fixed cells, scaled by target density */
    const float *density_map;    /* [m*n] after compute_potential: scaled by 1/bin_area */
    const int64_t *density_i64;  /* [m*n] fixed-point movable sums (fixed mode) */
    const float *auv;            /* DCT2 of the scaled map */
    const float *field_x, *field_y, *potential;
    const float *prev_x, *prev_y, *prev_gx, *prev_gy;
    /* scheduler / optimiser scalars */
    int32_t iteration;
    float gamma, base_gamma, density_weight;
    float alpha, beta;
    float hpwl_initial, hpwl_current, hpwl_previous;
    float overflow_current, overflow_previous;
    int32_t hpwl_initial_set;
} erpo_view;

typedef struct erpo_step_stats {
    float hpwl, overflow, energy, density_weight, gamma;
    int32_t should_stop;
} erpo_step_stats;

erpo_state *erpo_create(const erpo_design *d, const erpo_params *p);
void erpo_destroy(erpo_state *s);
void erpo_get_view(const erpo_state *s, erpo_view *v);

/* Overwrite current positions (all nodes) — lets tests feed identical inputs. */
void erpo_set_positions(erpo_state *s, const float *x, const float *y);
/* Overwrite the Nesterov history (prev coords, prev grads) and alpha/beta. */
void erpo_set_nesterov_state(erpo_state *s, const float *px, const float *py,
                             const float *pgx, const float *pgy, float alpha, float beta);
void erpo_set_scheduler(erpo_state *s, int32_t iteration, float gamma, float density_weight);
/* HPWL / overflow metrics of the scheduler (initial, current, previous). */
void erpo_set_metrics(erpo_state *s, float hpwl_init, float hpwl_cur, float hpwl_prev, float ovf_cur,
                      float ovf_prev);

/* src/hpwl.rs:139-343 */
float erpo_compute_hpwl(erpo_state *s, float gamma);
/* src/epotential.rs:225-374; returns overflow, writes energy */
float erpo_compute_potential(erpo_state *s, int32_t iteration, float *energy);
/* src/nesterov.rs:27-158 */
void erpo_nesterov(erpo_state *s, int32_t iteration);
/* src/scheduler.rs:68-73 / 75-81 */
void erpo_scheduler_update(erpo_state *s, float hpwl, float overflow);
int32_t erpo_should_stop(const erpo_state *s);
/* src/placement.rs:180-228 */
int32_t erpo_step(erpo_state *s, erpo_step_stats *st);

/* Standalone spectral transforms (same pipelines as the loop) in FP32 and FP64.
 * x, out: m*n row-major (row index = x-bin, src/epotential.rs:237-238). */
void erpo_dct2_f32(const float *x, float *out, int32_t m, int32_t n);
void erpo_idct2_f32(const float *x, float *out, int32_t m, int32_t n);
void erpo_idct_idxst_f32(const float *x, float *out, int32_t m, int32_t n);
void erpo_idxst_idct_f32(const float *x, float *out, int32_t m, int32_t n);
void erpo_dct2_f64(const double *x, double *out, int32_t m, int32_t n);
void erpo_idct2_f64(const double *x, double *out, int32_t m, int32_t n);
void erpo_idct_idxst_f64(const double *x, double *out, int32_t m, int32_t n);
void erpo_idxst_idct_f64(const double *x, double *out, int32_t m, int32_t n);

/* Full Poisson solve on a density map that is already scaled by 1/bin_area
 * (src/epotential.rs:287-343) in FP32 or FP64. */
void erpo_poisson_f32(const float *rho, int32_t m, int32_t n, float bin_w, float bin_h,
                      float *field_x, float *field_y, float *potential);
void erpo_poisson_f64(const double *rho, int32_t m, int32_t n, double bin_w, double bin_h,
                      double *field_x, double *field_y, double *potential);

/* Fixed-point shift rule shared with the GPU path: the largest S with
 * total_area * 2^S < 2^61, clamped to [-64, 100]. */
int32_t erpo_fixed_shift(double total_area);

#ifdef __cplusplus
}
#endif
#endif
