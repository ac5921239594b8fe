/*
 * erp_oracle.c — TEST INFRASTRUCTURE ONLY (see erp_oracle.h).
 * CPU restatement of ERPlacer's global-placement loop.  Parity unpinned
 * against the reference binary; pinned against FP64 closed forms in
 * tests/golden.  Build: oracle/build_oracle.py (gcc -O2 -fopenmp
 * -ffp-contract=off).
 */
#define _GNU_SOURCE
#include "erp_oracle.h"

#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ---- spectral transforms, FP32 and FP64 instantiations ---- */
#define REAL float
#define SFX f32
#define COS cosf
#define SIN sinf
#define PI_VALUE 3.14159265358979323846f /* std::f32::consts::PI (src/utils.rs:3) */
#include "spectral_impl.h"
#undef REAL
#undef SFX
#undef COS
#undef SIN
#undef PI_VALUE

#define REAL double
#define SFX f64
#define COS cos
#define SIN sin
#define PI_VALUE M_PI
#include "spectral_impl.h"
#undef REAL
#undef SFX
#undef COS
#undef SIN
#undef PI_VALUE

/* ------------------------------------------------------------------ */

struct erpo_state {
    erpo_design d;
    erpo_params p;
    int m, n;
    float bin_w, bin_h;            /* Bins::new (src/placement.rs:49-66) */
    float *bin_cx, *bin_cy;        /* bin_centers (src/placement.rs:81-94) */
    float target_density;
    /* PlacementSolution (src/placement.rs:96-140) */
    float *x, *y;
    /* HpwlComputation (src/hpwl.rs:7-19) */
    float *pins_x, *pins_y, *hpwls, *gpx, *gpy, *wlgx, *wlgy;
    /* PotentialComputation (src/epotential.rs:21-52) */
    float *initial_map, *density_map, *cw, *ch, *offx, *offy, *ratio;
    int64_t *dens_i64;
    int32_t shift, shift0;
    cx_f32 *expk_m, *expk_n;
    float *wu_half, *wv_half, *inv_w, *auv, *tmp, *fx, *fy, *pot, *dgx, *dgy;
    /* Nesterov (src/nesterov.rs:6-24) */
    float *prev_x, *prev_y, *prev_gx, *prev_gy, *g_x, *g_y;
    float alpha, beta;
    /* Scheduler (src/scheduler.rs:37-66) */
    int32_t iteration;
    float gamma, base_gamma, dw;
    int32_t hpwl_init_set, ovf_init_set;
    float hpwl_init, hpwl_cur, hpwl_prev, ovf_init, ovf_cur, ovf_prev;
};

static float *falloc(size_t n) { return (float *)calloc(n ? n : 1, sizeof(float)); }

int32_t erpo_fixed_shift(double total_area) {
    int e = 0;
    if (total_area > 0) frexp(total_area, &e); /* total < 2^e */
    int s = 61 - e;
    if (s < -64) s = -64;
    if (s > 100) s = 100;
    return s;
}

/* llrint(v * 2^shift) with v*2^shift formed in float (exact: power of two) */
static inline int64_t to_fixed(float v, float scale) { return llrintf(v * scale); }

static float pow2f(int e) { return ldexpf(1.0f, e); }

/* compute_density_overflow (src/density.rs:16-23) */
static inline float overlap_center(float x, float s, float c, float bs) {
    float two = 1.0f + 1.0f;
    float v = fminf(x + s, c + bs / two) - fmaxf(x, c - bs / two);
    return v > 0.0f ? v : 0.0f;
}

/* Rust's f32::min/max return the non-NaN operand like fminf/fmaxf. */

/* triangle_density_function with the max(0) clamp (src/density.rs:7-13) */
static inline float tri_clamped(float x, float s, float xl, int k, float bs) {
    float bin_xl = xl + (float)k * bs;
    float v = fminf(x + s, bin_xl + bs) - fmaxf(x, bin_xl);
    return v > 0.0f ? v : 0.0f;
}

/* compute_exact_density_overflow_map_parallel (src/density.rs:26-99) for the
 * fixed cells [num_movable, num_nodes).  Reference mode sums per thread chunk
 * then adds chunks in order; with one chunk this is the cell-order sum.
 * Fixed mode accumulates llrint(px*py*2^S0) in int64. */
static void initial_density(erpo_state *s) {
    const erpo_design *d = &s->d;
    int m = s->m, n = s->n;
    float inv_bx = 1.0f / s->bin_w, inv_by = 1.0f / s->bin_h;
    size_t mn = (size_t)m * n;
    int64_t *acc = NULL;
    float scale = 1.0f;
    if (s->p.density_mode == ERPO_DENSITY_FIXED) {
        double tot = 0;
        for (int i = d->num_movable; i < d->num_nodes; ++i) tot += (double)d->w[i] * d->h[i];
        s->shift0 = erpo_fixed_shift(tot);
        scale = pow2f(s->shift0);
        acc = (int64_t *)calloc(mn, sizeof(int64_t));
    }
    for (int i = d->num_movable; i < d->num_nodes; ++i) {
        float xi = d->x[i], yi = d->y[i], sxi = d->w[i], syi = d->h[i];
        long bxl = (long)floorf((xi - 0.0f) * inv_bx);
        long bxh = (long)ceilf((xi - 0.0f + sxi) * inv_bx) + 1;
        if (bxl < 0) bxl = 0; /* to_usize().unwrap() would panic: inputs are on the die */
        if (bxh > m - 1) bxh = m - 1;
        long byl = (long)floorf((yi - 0.0f) * inv_by);
        long byh = (long)ceilf((yi - 0.0f + syi) * inv_by) + 1;
        if (byl < 0) byl = 0;
        if (byh > n - 1) byh = n - 1;
        for (long bx = bxl; bx < bxh; ++bx) {
            float px = overlap_center(xi, sxi, s->bin_cx[bx], s->bin_w);
            for (long by = byl; by < byh; ++by) {
                float py = overlap_center(yi, syi, s->bin_cy[by], s->bin_h);
                size_t k = (size_t)bx * n + by;
                if (acc) acc[k] += to_fixed(px * py, scale);
                else s->initial_map[k] += px * py;
            }
        }
    }
    if (acc) {
        float inv = pow2f(-s->shift0);
        for (size_t k = 0; k < mn; ++k) s->initial_map[k] = (float)acc[k] * inv;
        free(acc);
    }
    /* src/epotential.rs:138-140 */
    for (size_t k = 0; k < mn; ++k) s->initial_map[k] = s->initial_map[k] * s->target_density;
}

/* The state's thread count for the parallel regions that follow (num_threads
 * <= 0: every processor).  OpenMP's thread count is one setting of the calling
 * thread, so each entry point sets it again: two oracles with different counts
 * can be used in turn. */
static void use_threads(const erpo_state *s) {
    omp_set_num_threads(s->p.num_threads > 0 ? s->p.num_threads : omp_get_num_procs());
}

erpo_state *erpo_create(const erpo_design *d, const erpo_params *p) {
    if (!d || !p) return NULL;
    int m = p->num_bins_x, n = p->num_bins_y;
    if (m < 4 || n < 4 || (m & (m - 1)) || (n & (n - 1))) return NULL;
    erpo_state *s = (erpo_state *)calloc(1, sizeof(erpo_state));
    s->d = *d;
    s->p = *p;
    use_threads(s);
    s->m = m; s->n = n;
    size_t N = (size_t)d->num_nodes, P = (size_t)d->num_pins, E = (size_t)d->num_nets;
    size_t mn = (size_t)m * n;
    /* Bins::new */
    s->bin_w = d->die_w / (float)m;
    s->bin_h = d->die_h / (float)n;
    s->bin_cx = falloc((size_t)m);
    s->bin_cy = falloc((size_t)n);
    for (int i = 0; i < m; ++i) {
        float l = 0.0f + (float)i * s->bin_w, h = fminf(l + s->bin_w, d->die_w);
        s->bin_cx[i] = (l + h) / 2.0f;
    }
    for (int i = 0; i < n; ++i) {
        float l = 0.0f + (float)i * s->bin_h, h = fminf(l + s->bin_h, d->die_h);
        s->bin_cy[i] = (l + h) / 2.0f;
    }
    /* PlacementSolution::new */
    s->target_density = p->target_density >= 0 ? p->target_density : d->cell_utilization;
    s->x = falloc(N); s->y = falloc(N);
    float cxm = d->die_w / 2.0f, cym = d->die_h / 2.0f;
    for (size_t i = 0; i < N; ++i) {
        if ((int)i >= d->num_movable || p->start_mode == ERPO_START_DB) {
            s->x[i] = d->x[i]; s->y[i] = d->y[i];
        } else {
            s->x[i] = cxm - d->w[i] / 2.0f;
            s->y[i] = cym - d->h[i] / 2.0f;
        }
    }
    /* PotentialComputation::new (src/epotential.rs:58-171) */
    s->cw = falloc(N); s->ch = falloc(N); s->offx = falloc(N); s->offy = falloc(N); s->ratio = falloc(N);
    float sqrt2 = 1.41421356237309504880f; /* std::f32::consts::SQRT_2 */
    double mov_tot = 0;
    for (size_t i = 0; i < N; ++i) {
        float w = d->w[i], h = d->h[i];
        float cw = fmaxf(w, s->bin_w * sqrt2), ch = fmaxf(h, s->bin_h * sqrt2);
        float r = (w * h) / (cw * ch);
        if ((int)i >= d->num_movable) r = s->target_density;
        s->cw[i] = cw; s->ch[i] = ch;
        s->offx[i] = (w - cw) * 0.5f;
        s->offy[i] = (h - ch) * 0.5f;
        s->ratio[i] = r;
        if ((int)i < d->num_movable) mov_tot += (double)w * (double)h;
    }
    s->shift = erpo_fixed_shift(mov_tot);
    s->expk_m = (cx_f32 *)malloc(sizeof(cx_f32) * (size_t)m);
    s->expk_n = (cx_f32 *)malloc(sizeof(cx_f32) * (size_t)n);
    make_expk_f32(m, s->expk_m);
    make_expk_f32(n, s->expk_n);
    s->wu_half = falloc(mn); s->wv_half = falloc(mn); s->inv_w = falloc(mn);
    frequency_matrices_f32(m, n, s->bin_w, s->bin_h, s->wu_half, s->wv_half, s->inv_w);
    s->initial_map = falloc(mn); s->density_map = falloc(mn);
    s->dens_i64 = (int64_t *)calloc(mn, sizeof(int64_t));
    s->auv = falloc(mn); s->tmp = falloc(mn);
    s->fx = falloc(mn); s->fy = falloc(mn); s->pot = falloc(mn);
    s->dgx = falloc(N); s->dgy = falloc(N);
    initial_density(s);
    /* HpwlComputation::new */
    s->pins_x = falloc(P); s->pins_y = falloc(P);
    s->hpwls = falloc(E); s->gpx = falloc(P); s->gpy = falloc(P);
    s->wlgx = falloc(N); s->wlgy = falloc(N);
    for (size_t i = 0; i < N; ++i)
        for (int k = d->inst_pin_ptr[i]; k < d->inst_pin_ptr[i + 1]; ++k) {
            int pid = d->inst_pins[k];
            s->pins_x[pid] = d->x[i] + d->pin_ox[pid];
            s->pins_y[pid] = d->y[i] + d->pin_oy[pid];
        }
    /* Scheduler::new (src/scheduler.rs:52-66) */
    s->gamma = 4.0f * (s->bin_w + s->bin_h);
    s->base_gamma = s->gamma;
    s->dw = 8e-5f;
    /* Nesterov::new: prev coords = DB coordinates (src/nesterov.rs:15-24) */
    s->prev_x = falloc(N); s->prev_y = falloc(N);
    memcpy(s->prev_x, d->x, sizeof(float) * N);
    memcpy(s->prev_y, d->y, sizeof(float) * N);
    s->prev_gx = falloc(N); s->prev_gy = falloc(N);
    s->g_x = falloc(N); s->g_y = falloc(N);
    s->alpha = 1.0f; s->beta = 0.0f;
    return s;
}

void erpo_destroy(erpo_state *s) {
    if (!s) return;
    float *fl[] = {s->bin_cx, s->bin_cy, s->x, s->y, s->pins_x, s->pins_y, s->hpwls, s->gpx,
                   s->gpy, s->wlgx, s->wlgy, s->initial_map, s->density_map, s->cw, s->ch,
                   s->offx, s->offy, s->ratio, s->wu_half, s->wv_half, s->inv_w, s->auv,
                   s->tmp, s->fx, s->fy, s->pot, s->dgx, s->dgy, s->prev_x, s->prev_y,
                   s->prev_gx, s->prev_gy, s->g_x, s->g_y};
    for (size_t i = 0; i < sizeof(fl) / sizeof(fl[0]); ++i) free(fl[i]);
    free(s->dens_i64); free(s->expk_m); free(s->expk_n);
    free(s);
}

void erpo_get_view(const erpo_state *s, erpo_view *v) {
    memset(v, 0, sizeof(*v));
    v->m = s->m; v->n = s->n; v->bin_w = s->bin_w; v->bin_h = s->bin_h;
    v->target_density = s->target_density;
    v->fixed_shift = s->shift; v->fixed_shift_init = s->shift0;
    v->x = s->x; v->y = s->y;
    v->wl_grad_x = s->wlgx; v->wl_grad_y = s->wlgy;
    v->pin_grad_x = s->gpx; v->pin_grad_y = s->gpy; v->net_hpwl = s->hpwls;
    v->dens_grad_x = s->dgx; v->dens_grad_y = s->dgy;
    v->clamped_w = s->cw; v->clamped_h = s->ch; v->offset_x = s->offx; v->offset_y = s->offy;
    v->ratio = s->ratio;
    v->initial_map = s->initial_map; v->density_map = s->density_map;
    v->density_i64 = s->dens_i64; v->auv = s->auv;
    v->field_x = s->fx; v->field_y = s->fy; v->potential = s->pot;
    v->prev_x = s->prev_x; v->prev_y = s->prev_y; v->prev_gx = s->prev_gx; v->prev_gy = s->prev_gy;
    v->iteration = s->iteration; v->gamma = s->gamma; v->base_gamma = s->base_gamma;
    v->density_weight = s->dw; v->alpha = s->alpha; v->beta = s->beta;
    v->hpwl_initial = s->hpwl_init; v->hpwl_current = s->hpwl_cur; v->hpwl_previous = s->hpwl_prev;
    v->overflow_current = s->ovf_cur; v->overflow_previous = s->ovf_prev;
    v->hpwl_initial_set = s->hpwl_init_set;
}

void erpo_set_positions(erpo_state *s, const float *x, const float *y) {
    memcpy(s->x, x, sizeof(float) * (size_t)s->d.num_nodes);
    memcpy(s->y, y, sizeof(float) * (size_t)s->d.num_nodes);
}

void erpo_set_nesterov_state(erpo_state *s, const float *px, const float *py, const float *pgx,
                             const float *pgy, float alpha, float beta) {
    size_t N = (size_t)s->d.num_nodes;
    memcpy(s->prev_x, px, sizeof(float) * N); memcpy(s->prev_y, py, sizeof(float) * N);
    memcpy(s->prev_gx, pgx, sizeof(float) * N); memcpy(s->prev_gy, pgy, sizeof(float) * N);
    s->alpha = alpha; s->beta = beta;
}

void erpo_set_scheduler(erpo_state *s, int32_t iteration, float gamma, float dw) {
    s->iteration = iteration; s->gamma = gamma; s->dw = dw;
}

/* the scheduler's HpwlMetrics / OverflowMetrics (src/scheduler.rs:6-35) */
void erpo_set_metrics(erpo_state *s, float hpwl_init, float hpwl_cur, float hpwl_prev, float ovf_cur,
                      float ovf_prev) {
    s->hpwl_init = hpwl_init; s->hpwl_cur = hpwl_cur; s->hpwl_prev = hpwl_prev;
    s->ovf_cur = ovf_cur; s->ovf_prev = ovf_prev;
    s->hpwl_init_set = 1; s->ovf_init_set = 1;
}

/* ---------------- wirelength: src/hpwl.rs ---------------- */

/* one net, general path (src/hpwl.rs:248-334); the two-pin fast path
 * (src/hpwl.rs:172-246) produces the same bits (sums start at 0). */
static float wa_net(erpo_state *s, int e, float inv_gamma, float def_min_x, float def_min_y) {
    const erpo_design *d = &s->d;
    const int *pl = d->net_pins + d->net_ptr[e];
    int deg = d->net_ptr[e + 1] - d->net_ptr[e];
    const float *px = s->pins_x, *py = s->pins_y;
    float one = 1.0f;
    if (e < d->n_2nets) {
        int p0 = pl[0], p1 = pl[1];
        float x0 = px[p0], y0 = py[p0], x1 = px[p1], y1 = py[p1];
        float min_x = fminf(x0, x1), max_x = fmaxf(x0, x1);
        float min_y = fminf(y0, y1), max_y = fmaxf(y0, y1);
        float hp = (max_x - min_x) + (max_y - min_y);
        float ex0 = expf((x0 - max_x) * inv_gamma), ex1 = expf((x1 - max_x) * inv_gamma);
        float enx0 = expf((min_x - x0) * inv_gamma), enx1 = expf((min_x - x1) * inv_gamma);
        float exs = ex0 + ex1, enxs = enx0 + enx1;
        float xexs = x0 * ex0 + x1 * ex1, xenxs = x0 * enx0 + x1 * enx1;
        float ey0 = expf((y0 - max_y) * inv_gamma), ey1 = expf((y1 - max_y) * inv_gamma);
        float eny0 = expf((min_y - y0) * inv_gamma), eny1 = expf((min_y - y1) * inv_gamma);
        float eys = ey0 + ey1, enys = eny0 + eny1;
        float yeys = y0 * ey0 + y1 * ey1, yenys = y0 * eny0 + y1 * eny1;
        float b_x = inv_gamma / exs, a_x = (one - b_x * xexs) / exs;
        float b_nx = -inv_gamma / enxs, a_nx = (one - b_nx * xenxs) / enxs;
        float b_y = inv_gamma / eys, a_y = (one - b_y * yeys) / eys;
        float b_ny = -inv_gamma / enys, a_ny = (one - b_ny * yenys) / enys;
        s->gpx[p0] = (a_x + b_x * x0) * ex0 - (a_nx + b_nx * x0) * enx0;
        s->gpx[p1] = (a_x + b_x * x1) * ex1 - (a_nx + b_nx * x1) * enx1;
        s->gpy[p0] = (a_y + b_y * y0) * ey0 - (a_ny + b_ny * y0) * eny0;
        s->gpy[p1] = (a_y + b_y * y1) * ey1 - (a_ny + b_ny * y1) * eny1;
        return hp;
    }
    float min_x = def_min_x, max_x = 0.0f, min_y = def_min_y, max_y = 0.0f;
    for (int k = 0; k < deg; ++k) {
        float x = px[pl[k]], y = py[pl[k]];
        min_x = fminf(min_x, x); max_x = fmaxf(max_x, x);
        min_y = fminf(min_y, y); max_y = fmaxf(max_y, y);
    }
    float xexs = 0, xenxs = 0, exs = 0, enxs = 0, yeys = 0, yenys = 0, eys = 0, enys = 0;
    for (int k = 0; k < deg; ++k) {
        float x = px[pl[k]], y = py[pl[k]];
        float ex = expf((x - max_x) * inv_gamma), enx = expf((min_x - x) * inv_gamma);
        xexs += x * ex; xenxs += x * enx; exs += ex; enxs += enx;
        float ey = expf((y - max_y) * inv_gamma), eny = expf((min_y - y) * inv_gamma);
        yeys += y * ey; yenys += y * eny; eys += ey; enys += eny;
    }
    float hp = (max_x - min_x) + (max_y - min_y);
    float b_x = inv_gamma / exs, a_x = (one - b_x * xexs) / exs;
    float b_nx = -inv_gamma / enxs, a_nx = (one - b_nx * xenxs) / enxs;
    float b_y = inv_gamma / eys, a_y = (one - b_y * yeys) / eys;
    float b_ny = -inv_gamma / enys, a_ny = (one - b_ny * yenys) / enys;
    for (int k = 0; k < deg; ++k) {
        int pid = pl[k];
        float x = px[pid], y = py[pid];
        float ex = expf((x - max_x) * inv_gamma), enx = expf((min_x - x) * inv_gamma);
        s->gpx[pid] = (a_x + b_x * x) * ex - (a_nx + b_nx * x) * enx;
        float ey = expf((y - max_y) * inv_gamma), eny = expf((min_y - y) * inv_gamma);
        s->gpy[pid] = (a_y + b_y * y) * ey - (a_ny + b_ny * y) * eny;
    }
    return hp;
}

float erpo_compute_hpwl(erpo_state *s, float gamma) {
    use_threads(s);
    const erpo_design *d = &s->d;
    long N = d->num_nodes, P = d->num_pins, E = d->num_nets, NM = d->num_movable;
    /* reset (src/hpwl.rs:77-84) */
    memset(s->hpwls, 0, sizeof(float) * (size_t)E);
    memset(s->gpx, 0, sizeof(float) * (size_t)P);
    memset(s->gpy, 0, sizeof(float) * (size_t)P);
    memset(s->wlgx, 0, sizeof(float) * (size_t)N);
    memset(s->wlgy, 0, sizeof(float) * (size_t)N);
    /* compute_pins_position (src/hpwl.rs:86-111): movable only */
#pragma omp parallel for schedule(static)
    for (long i = 0; i < NM; ++i)
        for (int k = d->inst_pin_ptr[i]; k < d->inst_pin_ptr[i + 1]; ++k) {
            int pid = d->inst_pins[k];
            s->pins_x[pid] = s->x[i] + d->pin_ox[pid];
            s->pins_y[pid] = s->y[i] + d->pin_oy[pid];
        }
    float one = 1.0f;
    float def_min_x = d->die_w + one, def_min_y = d->die_h + one;
    float inv_gamma = one / gamma;
#pragma omp parallel for schedule(dynamic, 1024)
    for (long e = 0; e < E; ++e) s->hpwls[e] = wa_net(s, (int)e, inv_gamma, def_min_x, def_min_y);
    /* compute_gradients (src/hpwl.rs:113-135) */
#pragma omp parallel for schedule(static)
    for (long i = 0; i < NM; ++i) {
        float gx = 0.0f, gy = 0.0f;
        for (int k = d->inst_pin_ptr[i]; k < d->inst_pin_ptr[i + 1]; ++k) {
            gx += s->gpx[d->inst_pins[k]];
            gy += s->gpy[d->inst_pins[k]];
        }
        s->wlgx[i] = gx; s->wlgy[i] = gy;
    }
    /* src/hpwl.rs:341-342 (reduction order unspecified in the reference) */
    if (s->p.reduce_fp64) {
        double t = 0;
#pragma omp parallel for reduction(+ : t) schedule(static)
        for (long e = 0; e < E; ++e) t += (double)s->hpwls[e];
        return (float)t;
    }
    float t = 0.0f;
    for (long e = 0; e < E; ++e) t += s->hpwls[e];
    return t;
}

/* ---------------- density: src/density.rs ---------------- */

static void movable_density(erpo_state *s, int iteration) {
    const erpo_design *d = &s->d;
    int m = s->m, n = s->n;
    long NM = d->num_movable;
    size_t mn = (size_t)m * n;
    float inv_bx = 1.0f / s->bin_w, inv_by = 1.0f / s->bin_h;
    float *map = s->density_map;
    memset(map, 0, sizeof(float) * mn); /* pc.reset (src/epotential.rs:173-180) */
    if (s->p.density_mode == ERPO_DENSITY_FIXED) {
        float scale = pow2f(s->shift);
        memset(s->dens_i64, 0, sizeof(int64_t) * mn);
        int64_t *acc = s->dens_i64;
#pragma omp parallel for schedule(static)
        for (long i = 0; i < NM; ++i) {
            float xi = s->x[i] + s->offx[i], yi = s->y[i] + s->offy[i];
            float sxi = s->cw[i], syi = s->ch[i], r = s->ratio[i];
            /* bin range of src/density.rs:202-218 (floor / ceil+1, clamp [0, bins-1)) */
            long bxl = (long)floorf((xi - 0.0f) * inv_bx);
            long bxh = (long)ceilf((xi - 0.0f + sxi) * inv_bx) + 1;
            if (bxl < 0) bxl = 0;
            if (bxh > m - 1) bxh = m - 1;
            long byl = (long)floorf((yi - 0.0f) * inv_by);
            long byh = (long)ceilf((yi - 0.0f + syi) * inv_by) + 1;
            if (byl < 0) byl = 0;
            if (byh > n - 1) byh = n - 1;
            for (long bx = bxl; bx < bxh; ++bx) {
                float px = r * tri_clamped(xi, sxi, 0.0f, (int)bx, s->bin_w);
                for (long by = byl; by < byh; ++by) {
                    float py = tri_clamped(yi, syi, 0.0f, (int)by, s->bin_h);
                    int64_t c = to_fixed(px * py, scale);
                    if (c) {
#pragma omp atomic
                        acc[(size_t)bx * n + by] += c;
                    }
                }
            }
        }
        float inv = pow2f(-s->shift);
#pragma omp parallel for schedule(static)
        for (size_t k = 0; k < mn; ++k) map[k] = (float)acc[k] * inv + s->initial_map[k];
        return;
    }
    if (iteration < 200) {
        /* compute_density_overflow_map_sequential (src/density.rs:174-237) */
        for (long i = 0; i < NM; ++i) {
            float xi = s->x[i] + s->offx[i], yi = s->y[i] + s->offy[i];
            float sxi = s->cw[i], syi = s->ch[i], r = s->ratio[i];
            long bxl = (long)floorf((xi - 0.0f) * inv_bx);
            long bxh = (long)ceilf((xi - 0.0f + sxi) * inv_bx) + 1;
            if (bxl < 0) bxl = 0;
            if (bxh > m - 1) bxh = m - 1;
            long byl = (long)floorf((yi - 0.0f) * inv_by);
            long byh = (long)ceilf((yi - 0.0f + syi) * inv_by) + 1;
            if (byl < 0) byl = 0;
            if (byh > n - 1) byh = n - 1;
            for (long bx = bxl; bx < bxh; ++bx) {
                float px = r * tri_clamped(xi, sxi, 0.0f, (int)bx, s->bin_w);
                for (long by = byl; by < byh; ++by)
                    map[(size_t)bx * n + by] += px * tri_clamped(yi, syi, 0.0f, (int)by, s->bin_h);
            }
        }
    } else {
        /* compute_density_overflow_map_parallel (src/density.rs:102-171): truncating
         * ranges and one lock per (cell, bin) contribution; here an atomic add. */
#pragma omp parallel for schedule(static)
        for (long i = 0; i < NM; ++i) {
            float xi = s->x[i] + s->offx[i], yi = s->y[i] + s->offy[i];
            float sxi = s->cw[i], syi = s->ch[i], r = s->ratio[i];
            long bxl = (long)((xi - 0.0f) * inv_bx);
            long bxh = (long)((xi - 0.0f + sxi) * inv_bx) + 1;
            if (bxl < 0) bxl = 0;
            if (bxh > m - 1) bxh = m - 1;
            long byl = (long)((yi - 0.0f) * inv_by);
            long byh = (long)((yi - 0.0f + syi) * inv_by) + 1;
            if (byl < 0) byl = 0;
            if (byh > n - 1) byh = n - 1;
            for (long bx = bxl; bx < bxh; ++bx) {
                float px = r * tri_clamped(xi, sxi, 0.0f, (int)bx, s->bin_w);
                for (long by = byl; by < byh; ++by) {
                    float v = px * tri_clamped(yi, syi, 0.0f, (int)by, s->bin_h);
#pragma omp atomic
                    map[(size_t)bx * n + by] += v;
                }
            }
        }
    }
#pragma omp parallel for schedule(static)
    for (size_t k = 0; k < mn; ++k) map[k] += s->initial_map[k];
}

/* triangle_density_function without the clamp (src/eforce.rs:6-13) */
static inline float tri_raw(float x, float sz, float xl, long k, float bs) {
    float bin_xl = xl + (float)k * bs;
    return fminf(x + sz, bin_xl + bs) - fmaxf(x, bin_xl);
}

/* Rust `f.to_isize().unwrap_or(0)`: truncation, NaN / out of range -> 0 */
static inline long to_isize0(float v) {
    if (!(v == v) || v >= 9.2e18f || v <= -9.2e18f) return 0;
    return (long)v;
}

/* compute_electric_force (src/eforce.rs:15-91) */
static void electric_force(erpo_state *s) {
    const erpo_design *d = &s->d;
    long NM = d->num_movable;
    int m = s->m, n = s->n;
    float inv_bx = 1.0f / s->bin_w, inv_by = 1.0f / s->bin_h;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < NM; ++i) {
        float sx = s->cw[i], sy = s->ch[i];
        float nx = s->x[i] + s->offx[i], ny = s->y[i] + s->offy[i], r = s->ratio[i];
        long xl = to_isize0((nx - 0.0f) * inv_bx); if (xl < 0) xl = 0;
        long xh = to_isize0((nx + sx - 0.0f) * inv_bx) + 1;
        if (xh < 0 || xh > m) xh = m; /* negative wraps to usize::MAX, then min */
        long yl = to_isize0((ny - 0.0f) * inv_by); if (yl < 0) yl = 0;
        long yh = to_isize0((ny + sy - 0.0f) * inv_by) + 1;
        if (yh < 0 || yh > n) yh = n;
        float gx = 0.0f, gy = 0.0f;
        for (long k = xl; k < xh; ++k) {
            float px = tri_raw(nx, sx, 0.0f, k, s->bin_w);
            for (long h = yl; h < yh; ++h) {
                float py = tri_raw(ny, sy, 0.0f, h, s->bin_h);
                float area = px * py;
                size_t idx = (size_t)k * n + h;
                gx += area * s->fx[idx];
                gy += area * s->fy[idx];
            }
        }
        s->dgx[i] = -gx * r;
        s->dgy[i] = -gy * r;
    }
}

float erpo_compute_potential(erpo_state *s, int32_t iteration, float *energy_out) {
    use_threads(s);
    int m = s->m, n = s->n;
    size_t mn = (size_t)m * n;
    movable_density(s, iteration);
    /* overflow (src/epotential.rs:271-277) */
    float bin_area = s->bin_w * s->bin_h;
    float coef = s->target_density * bin_area;
    float overflow;
    if (s->p.reduce_fp64) {
        double o = 0;
#pragma omp parallel for reduction(+ : o) schedule(static)
        for (size_t k = 0; k < mn; ++k) {
            float v = s->density_map[k] - coef;
            o += (double)(v > 0.0f ? v : 0.0f);
        }
        overflow = (float)(o / (double)s->d.movable_area);
    } else {
        float o = 0.0f;
        for (size_t k = 0; k < mn; ++k) {
            float v = s->density_map[k] - coef;
            o += v > 0.0f ? v : 0.0f;
        }
        overflow = o / s->d.movable_area;
    }
    /* src/epotential.rs:284-285 */
    float kk = 1.0f / bin_area;
#pragma omp parallel for schedule(static)
    for (size_t k = 0; k < mn; ++k) s->density_map[k] = s->density_map[k] * kk;
    /* src/epotential.rs:287-343 */
    dct2_fft2_forward_f32(s->density_map, s->expk_m, s->expk_n, s->auv, m, n);
    for (size_t k = 0; k < mn; ++k) s->tmp[k] = s->auv[k] * s->wu_half[k];
    inverse_forward_f32(s->tmp, s->expk_m, s->expk_n, s->fx, m, n, 2);
    for (size_t k = 0; k < mn; ++k) s->tmp[k] = s->auv[k] * s->wv_half[k];
    inverse_forward_f32(s->tmp, s->expk_m, s->expk_n, s->fy, m, n, 1);
    for (size_t k = 0; k < mn; ++k) s->tmp[k] = s->auv[k] * s->inv_w[k];
    inverse_forward_f32(s->tmp, s->expk_m, s->expk_n, s->pot, m, n, 0);
    /* energy (src/epotential.rs:344-346) */
    if (energy_out) {
        double e = 0;
        for (size_t k = 0; k < mn; ++k) e += (double)(s->pot[k] * s->density_map[k]);
        *energy_out = (float)e;
    }
    electric_force(s);
    return overflow;
}

/* ---------------- optimiser: src/nesterov.rs ---------------- */

void erpo_nesterov(erpo_state *s, int32_t iteration) {
    use_threads(s);
    const erpo_design *d = &s->d;
    long NM = d->num_movable;
    float one = 1.0f, two = one + one, four = two + two;
    /* update_momentum (src/nesterov.rs:148-158) */
    float a_prev = s->alpha;
    float na = (one + sqrtf(four * a_prev * a_prev + one)) / two;
    s->beta = (a_prev - one) / na;
    s->alpha = na;
    /* src/nesterov.rs:47-55 */
    if (iteration == 0) {
        if (s->p.reduce_fp64) {
            double num = 0, den = 0;
            for (long i = 0; i < NM; ++i) {
                num += (double)fabsf(s->wlgx[i]) + (double)fabsf(s->wlgy[i]);
                den += (double)fabsf(s->dgx[i]) + (double)fabsf(s->dgy[i]);
            }
            s->dw = (float)((double)s->dw * (num / den));
        } else {
            float num = 0, den = 0;
            for (long i = 0; i < NM; ++i) {
                num = num + fabsf(s->wlgx[i]) + fabsf(s->wlgy[i]);
                den = den + fabsf(s->dgx[i]) + fabsf(s->dgy[i]);
            }
            s->dw = s->dw * (num / den);
        }
    }
    float dw = s->dw;
    /* src/nesterov.rs:74-95 */
    double dnum = 0, dden = 0;
    float fnum = 0, fden = 0;
    for (long i = 0; i < NM; ++i) {
        float area = d->w[i] * d->h[i];
        float npins = d->num_pins_f[i];
        float inv_pre = one / fminf(npins + dw * area, one);
        float gx = (s->wlgx[i] + dw * s->dgx[i]) * inv_pre;
        float gy = (s->wlgy[i] + dw * s->dgy[i]) * inv_pre;
        s->g_x[i] = gx; s->g_y[i] = gy;
        float dx = s->x[i] - s->prev_x[i], dy = s->y[i] - s->prev_y[i];
        float dgx = gx - s->prev_gx[i], dgy = gy - s->prev_gy[i];
        if (s->p.reduce_fp64) {
            dnum += (double)(dx * dx) + (double)(dy * dy);
            dden += (double)(dgx * dgx) + (double)(dgy * dgy);
        } else {
            fnum = fnum + dx * dx + dy * dy;
            fden = fden + dgx * dgx + dgy * dgy;
        }
    }
    /* src/nesterov.rs:98-100 */
    if (s->p.reduce_fp64) {
        if (iteration > 0 && dden > 0) s->alpha = (float)sqrt(dnum / dden);
    } else {
        if (iteration > 0 && fden > 0) s->alpha = sqrtf(fnum / fden);
    }
    /* src/nesterov.rs:111-145 */
    float alpha = s->alpha, beta = s->beta;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < NM; ++i) {
        float w = d->w[i], h = d->h[i];
        float xo = s->x[i], yo = s->y[i];
        float xh = s->x[i] + beta * (s->x[i] - s->prev_x[i]);
        float yh = s->y[i] + beta * (s->y[i] - s->prev_y[i]);
        float hx = d->die_w - w - one, hy = d->die_h - h - one;
        float nx = xh - alpha * s->g_x[i], ny = yh - alpha * s->g_y[i];
        nx = nx < 0.0f ? 0.0f : (nx > hx ? hx : nx);
        ny = ny < 0.0f ? 0.0f : (ny > hy ? hy : ny);
        s->prev_x[i] = xo; s->prev_y[i] = yo;
        s->x[i] = nx; s->y[i] = ny;
        s->prev_gx[i] = s->g_x[i]; s->prev_gy[i] = s->g_y[i];
    }
}

/* ---------------- scheduler: src/scheduler.rs ---------------- */

void erpo_scheduler_update(erpo_state *s, float hpwl, float overflow) {
    s->iteration += 1;                                   /* :83-85 */
    if (!s->hpwl_init_set) { s->hpwl_init = hpwl; s->hpwl_init_set = 1; }
    s->hpwl_prev = s->hpwl_cur; s->hpwl_cur = hpwl;      /* Metric::update :27-33 */
    if (!s->ovf_init_set) { s->ovf_init = overflow; s->ovf_init_set = 1; }
    s->ovf_prev = s->ovf_cur; s->ovf_cur = overflow;
    /* update_density_weight (:92-116) */
    float ref = s->hpwl_init_set ? s->hpwl_init : 350000.0f;
    float lower = 0.95f, upper = 1.05f;
    float delta = s->hpwl_cur - s->hpwl_prev;
    if (s->p.reduce_fp64) {
        /* the FP64 form: b^e of the constant bases as exp(e * ln b) */
        double power;
        if (delta < 0.0f) {
            power = exp((double)s->iteration * log(0.9999));
            if (power < 0.98) power = 0.98;
        } else {
            power = exp(-(double)delta / (double)ref * log(1.05));
            power = power < 0.95 ? 0.95 : (power > 1.05 ? 1.05 : power);
        }
        s->dw = (float)((double)s->dw * (1.05 * power));
        double ovf = (double)s->ovf_cur;
        double coef = exp(((ovf - 0.1) * 20.0 / 9.0 - 1.0) * log(10.0));
        coef = coef < 0.05 ? 0.05 : (coef > 10.0 ? 10.0 : coef);
        s->gamma = (float)((double)s->base_gamma * coef);
        return;
    }
    float power;
    if (delta < 0.0f) {
        /* f32::powi lowers to binary exponentiation (compiler-rt __powisf2) */
        float pw = 1.0f, b = 0.9999f;
        for (int e = s->iteration;;) {
            if (e & 1) pw *= b;
            e /= 2;
            if (e == 0) break;
            b *= b;
        }
        power = fmaxf(pw, 0.98f);
    } else {
        power = powf(upper, -delta / ref);
        power = power < lower ? lower : (power > upper ? upper : power);
    }
    s->dw = s->dw * (upper * power);
    /* update_gamma (:118-130) */
    float coef = powf(10.0f, (s->ovf_cur - 0.1f) * 20.0f / 9.0f - 1.0f);
    coef = coef < 0.05f ? 0.05f : (coef > 10.0f ? 10.0f : coef);
    s->gamma = s->base_gamma * coef;
}

int32_t erpo_should_stop(const erpo_state *s) {
    float cur = s->hpwl_cur, prev = s->hpwl_prev;
    return prev != 0.0f && cur != 0.0f && prev > cur * 1.5f;
}

int32_t erpo_step(erpo_state *s, erpo_step_stats *st) {
    use_threads(s);
    float hp = erpo_compute_hpwl(s, s->gamma);
    float energy = 0;
    float ovf = erpo_compute_potential(s, s->iteration, &energy);
    erpo_nesterov(s, s->iteration);
    float dw = s->dw, g = s->gamma;
    erpo_scheduler_update(s, hp, ovf);
    int32_t stop = erpo_should_stop(s);
    if (st) {
        st->hpwl = hp; st->overflow = ovf; st->energy = energy;
        st->density_weight = dw; st->gamma = g; st->should_stop = stop;
    }
    return stop;
}

/* ---------------- standalone transforms ---------------- */

#define STANDALONE(SUF, REALT, CXT, VAR, BODY)                                                   \
    void erpo_##VAR##_##SUF(const REALT *x, REALT *out, int32_t m, int32_t n) {                \
        CXT *em = (CXT *)malloc(sizeof(CXT) * (size_t)m), *en = (CXT *)malloc(sizeof(CXT) * (size_t)n); \
        make_expk_##SUF(m, em);                                                                  \
        make_expk_##SUF(n, en);                                                                  \
        BODY;                                                                                    \
        free(em); free(en);                                                                      \
    }

STANDALONE(f32, float, cx_f32, dct2, dct2_fft2_forward_f32(x, em, en, out, m, n))
STANDALONE(f32, float, cx_f32, idct2, inverse_forward_f32(x, em, en, out, m, n, 0))
STANDALONE(f32, float, cx_f32, idct_idxst, inverse_forward_f32(x, em, en, out, m, n, 1))
STANDALONE(f32, float, cx_f32, idxst_idct, inverse_forward_f32(x, em, en, out, m, n, 2))
STANDALONE(f64, double, cx_f64, dct2, dct2_fft2_forward_f64(x, em, en, out, m, n))
STANDALONE(f64, double, cx_f64, idct2, inverse_forward_f64(x, em, en, out, m, n, 0))
STANDALONE(f64, double, cx_f64, idct_idxst, inverse_forward_f64(x, em, en, out, m, n, 1))
STANDALONE(f64, double, cx_f64, idxst_idct, inverse_forward_f64(x, em, en, out, m, n, 2))

void erpo_poisson_f32(const float *rho, int32_t m, int32_t n, float bw, float bh, float *fx,
                      float *fy, float *pot) {
    cx_f32 *em = (cx_f32 *)malloc(sizeof(cx_f32) * (size_t)m), *en = (cx_f32 *)malloc(sizeof(cx_f32) * (size_t)n);
    make_expk_f32(m, em); make_expk_f32(n, en);
    float *auv = falloc((size_t)m * n);
    poisson_f32(rho, m, n, bw, bh, em, en, auv, fx, fy, pot);
    free(auv); free(em); free(en);
}

void erpo_poisson_f64(const double *rho, int32_t m, int32_t n, double bw, double bh, double *fx,
                      double *fy, double *pot) {
    cx_f64 *em = (cx_f64 *)malloc(sizeof(cx_f64) * (size_t)m), *en = (cx_f64 *)malloc(sizeof(cx_f64) * (size_t)n);
    make_expk_f64(m, em); make_expk_f64(n, en);
    double *auv = (double *)calloc((size_t)m * n, sizeof(double));
    poisson_f64(rho, m, n, bw, bh, em, en, auv, fx, fy, pot);
    free(auv); free(em); free(en);
}
