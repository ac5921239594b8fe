// Internal definitions shared by the CUDA translation units of
// liberplacer_gb300.so: the device-resident context layout, the scalar state
// the whole iteration keeps on the device, and the kernel launchers.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <string>
#include <vector>

#include "erplacer.h"
#include "packed.h"

namespace erp {

constexpr int kThreads = 256;

// Device-resident scalars.  Every quantity the reference keeps in Scheduler /
// Nesterov (src/scheduler.rs:37-50, src/nesterov.rs:6-13) plus the reductions
// of the current step, so that a whole Placement::step runs without a host
// round trip (the HPWL / overflow totals and the Lipschitz sums are double-float
// sums stored as FP64; the density-weight update is FP64).
struct DevState {
    // scheduler
    int32_t iteration;
    int32_t hpwl_init_set;
    float gamma, base_gamma, dw;
    float hpwl_init, hpwl_cur, hpwl_prev;
    float ovf_init, ovf_cur, ovf_prev;
    int32_t ovf_init_set;
    // optimiser
    float alpha, beta;
    // this step's reductions
    double hpwl;
    double overflow;
    double energy;
    double lip_num, lip_den;
    double abs_wl, abs_dens;
    float hpwl_f, overflow_f;
    // step bookkeeping
    int32_t done;          // set once overflow <= stop threshold: kernels become no-ops
    int32_t status;        // bit 0: non-finite value seen; bit 1: a bounded wait ran out
    float stop_overflow;   // <= 0: never stop
    int32_t stop_iter;     // > 0: retire once iteration reaches it
    int32_t last_iter;     // iteration index of the last completed step
    erp_step_stats last;   // stats of the last completed step
    // 1 under ERP_FLAG_EXPIRE_WAITS: a kernel's mbarrier wait gives up at once
    // instead of after kWaitTries tries (the copy is then still drained with
    // the full limit before the shared area is reused); 0 otherwise
    uint32_t expire_waits;
    // last-block counters of the deterministic reductions
    uint32_t ctr[8];
};

constexpr int32_t kStatusWaitTimeout = 2;   // DevState::status bit 1

enum Counter { CTR_HPWL = 0, CTR_OVF = 1, CTR_ABS = 2, CTR_LIP = 3, CTR_ENERGY = 4 };

// Net degree classes processed by one thread group of width W each.
// Classes 0..7 hold nets of one exact degree -- class 0 the leading 2-pin nets
// (the reference's fast path), classes 1..7 the other nets of degree 2..8 --
// whose pin slots are stored pin-major: pin q of the class's net g sits at slot
// slot0 + q * count + g, so one thread per net reads and writes coalesced.
// Classes 8..10 hold the remaining nets (degree <= 16, <= 32, > 32) with each
// net's slots contiguous (net_ptr), served by lane groups.
constexpr int kNumExact = 8;
constexpr int kNumClasses = 11;
struct NetClass {
    int32_t begin, count;  // range in the internal net order
    int32_t width;         // lanes per net
    int32_t general;       // 1: general path (min/max initialised to die+1 / 0)
    int32_t degree;        // exact degree (classes 0..7), else 0
    int32_t slot0;         // first pin slot of the class
};

struct DctGemmPlan;   // tensor-core spectral solve (k_dctgemm.cu)

struct Ctx {
    // --- sizes ---
    int32_t N, NM, P, E, NS;   // nodes, movable, pins, nets, pin slots (= P)
    int32_t m, n, logm, logn;
    float die_w, die_h, bin_w, bin_h, inv_bw, inv_bh, bin_area, inv_bin_area;
    float target_density, movable_area;
    int32_t shift, shift0;
    float fixed_scale, fixed_inv;
    int device;
    cudaStream_t stream;
    bool own_stream;
    uint32_t expire_waits;   // DevState::expire_waits of this context
    std::string err;
    // --- cells [N] ---
    float *x, *y, *w, *h, *npins, *cw, *ch, *offx, *offy, *ratio;
    float2 *xy;                // (x, y) interleaved: one 8-byte gather per pin in the wirelength pass
    float *wlgx, *wlgy;
    float *prev_x, *prev_y, *prev_gx, *prev_gy;
    // --- pins in internal slot order [NS] ---
    int32_t *slot_cell;
    float2 *slot_off;
    float2 *slot_grad;
    int32_t *net_ptr;          // [E+1] internal order
    float *net_hpwl;           // [E] internal order
    NetClass cls[kNumClasses];
    int32_t *cell_slot_ptr;    // [NM+1]
    int32_t *cell_slots;
    // --- scatter order [NM] (k_density_scatter; refreshed every kSortEvery steps) ---
    int32_t *perm, *skey;      // cell at each scatter position, its sort tile
    int32_t *pos;              // scatter position of each movable cell (perm's inverse)
    float2 *dgp;               // density gradient in scatter order (k_force writes it coalesced)
    float4 *soff;              // offx, offy, cw, ch in scatter order
    float *sratio;
    int32_t *sort_key, *sort_rank, *sort_hist, *sort_start;   // counting-sort scratch ([NM], [NM], tiles, tiles)
    int32_t sort_age;          // steps since the order was computed
    int32_t scatter_cells;     // movable cells per scatter block; 0: the rule for a context run alone
    int32_t scatter_planes;    // 21-bit pieces per contribution in the scatter's window: 2 or 3
    int32_t spectral_seqs;     // sequences per block of the warp-form spectral passes; 0: the fixed shape
    // host-side permutations for test hooks
    int32_t *h_slot_of_pin;    // [P]
    int32_t *h_net_of_internal;// [E]
    // --- maps [m*n] ---
    unsigned long long *dmap;  // int64 fixed-point movable density
    float *initial, *rho, *t1, *tx, *ty, *tp, *fx, *fy, *psi;
    float2 *tw_m, *tw_n, *ek_m, *ek_n;   // FFT twiddles and DCT post-twiddles
    float *wu, *wv;            // frequency vectors [m], [n]
    bool map_dirty;
    bool psi_valid;
    // --- reductions ---
    double *partials;          // kMaxPartials
    int32_t max_partials;
    DevState *st;
    DevState *h_st;            // pinned host mirror
    void *arena;               // the one allocation that holds every device array above
    DctGemmPlan *gemm;         // tensor-core spectral solve (precision TF32 / BF16x3), else nullptr
    // --- graph ---
    cudaGraphExec_t graph;
    bool graph_ready;
    int32_t graph_kernels;
    // --- timing hooks (bench): events around the dominant kernel ---
};

constexpr int kMaxPartials = 8192;

// ---------------- launchers (stream = ctx.stream) ----------------
// wirelength (src/hpwl.rs)
void launch_wirelength(Ctx &c, float gamma_arg);          // gamma_arg < 0: read DevState.gamma
void launch_pack_xy(Ctx &c);                               // xy from x, y after a host write
// headless snapshots (k_snapshot.cu): RGB bytes on the device
cudaError_t launch_snapshot_placement(Ctx &c, int W, int H, unsigned char *d_rgb, int *d_top);
cudaError_t launch_snapshot_density(Ctx &c, const float *map, unsigned char *d_rgb, unsigned *d_mm);
void launch_wl_gather(Ctx &c);
// density + spectral + force (src/density.rs, src/epotential.rs, src/eforce.rs)
void launch_initial_density(Ctx &c, const float *hx, const float *hy, const float *hw,
                            const float *hh);               // setup, on device
void launch_density_scatter(Ctx &c);
void launch_spectral(Ctx &c, bool zero_map, bool store_rho, bool want_psi);
void launch_scatter_order(Ctx &c, cudaStream_t s);   // recompute the scatter order from the current positions
int scatter_tiles(int m, int n);
void launch_xy_from_host(Ctx &c, const float *hx, const float *hy);   // device-mapped host x, y -> x, y, xy
void launch_xy_to_host(Ctx &c, float *hx, float *hy);                 // xy -> device-mapped host x, y
cudaError_t place_occupancy();                        // resident block counts of the streaming kernels
constexpr int kSortEvery = 16;                          // steps between scatter-order refreshes
void launch_force(Ctx &c, int rescale);                   // rescale 1: also the iteration-0 density-weight rescale (step graph)
void launch_energy(Ctx &c);
// optimiser + scheduler (src/nesterov.rs, src/scheduler.rs)
void launch_nesterov(Ctx &c, int iter_arg);                // iter_arg < 0: read DevState.iteration
void launch_scheduler(Ctx &c, int use_args, float hpwl, float overflow);
// One whole Placement::step on the context's stream (the graph's content).
void enqueue_step_kernels(Ctx &c);
// Gather the retire flags of several contexts into out[i] (device pointers).
void launch_gather_done(DevState *const *states, int count, int32_t *out, cudaStream_t s);

// ---- packed launches (batches) ----
// The packed form of a kernel whose body is BODY(args, block, grid).
template <typename P, void (*BODY)(const P &, int, int), int THREADS, int MINB>
__global__ void __launch_bounds__(THREADS, MINB) k_packed(const __grid_constant__ Packed<P> pk) {
    const int b = (int)blockIdx.x;
    const int i = packed_instance(pk.block0, pk.n, b);
    const int b0 = pk.block0[i];
    BODY(pk.tab[i], b - b0, pk.block0[i + 1] - b0);
}
// The argument tables of a batch's packed step, built on the host (one buffer,
// copied once to one device buffer), and its launches in stage order.
struct PackedArena {
    std::vector<unsigned char> host;
    size_t put(const void *p, size_t bytes) {
        const size_t off = (host.size() + 255) & ~size_t(255);
        host.resize(off + bytes);
        if (bytes) memcpy(host.data() + off, p, bytes);
        return off;
    }
};
struct PackedLaunch {
    int kind;        // PackKind
    int variant;     // template variant of the kernel (scatter planes; spectral E and NW)
    size_t tab, block0;   // offsets of the argument table and the block prefix in the arena
    int n, blocks, threads;
    size_t smem;
};
template <typename P>
inline Packed<P> packed_args(const PackedLaunch &l, const unsigned char *dev) {
    return Packed<P>{reinterpret_cast<const P *>(dev + l.tab), reinterpret_cast<const int32_t *>(dev + l.block0),
                     l.n};
}
enum PackKind { PK_WA, PK_GATHER, PK_SCATTER, PK_ROWS_DCT_W, PK_COLS_W, PK_ROWS_INV_W, PK_FORCE, PK_GRAD, PK_UPDATE,
                PK_SCHED };
// Appends one packed launch of the given kind over the contexts xs (k_place.cu:
// wirelength, gather, scatter, force, Nesterov, scheduler; the scatter one per
// plane count in use), and issues a planned launch with the arena at dev (false:
// not one of its kinds).
void packed_place_stage(PackKind k, const std::vector<Ctx *> &xs, PackedArena &ar, std::vector<PackedLaunch> &out);
bool packed_place_launch(const PackedLaunch &l, const unsigned char *dev, cudaStream_t s);

// A stream-ordered allocation for a context's arrays, from the library's pool on
// the current device (freed with cudaFreeAsync; erp_api.cu).
cudaError_t ctx_alloc(void **p, size_t bytes, cudaStream_t s);

// spectral engine for the standalone solve
// The sequences-per-block alternatives of the warp-form spectral passes (sides
// 64..256) that a batch's autotuner times against the fixed shape (four).
constexpr int kSeqCandidates[2] = {2, 8};
struct SpectralPlan {
    int32_t m, n, logm, logn;
    float bin_w, bin_h;
    float2 *tw_m, *tw_n, *ek_m, *ek_n;
    float *wu, *wv;
    float *t1, *tx, *ty, *tp;
    double *partials;
    DevState *st;
    cudaStream_t stream;
    // sequences per block of the warp-form passes (sides 64..256): 0 for the
    // fixed shape, else one a batch's autotuner chose (2 or 8)
    int32_t seqs = 0;
};
void spectral_tables(int m, int n, float bin_w, float bin_h, float2 **tw_m, float2 **tw_n,
                     float2 **ek_m, float2 **ek_n, float **wu, float **wv, cudaStream_t s);
// The same tables into arrays the caller allocated (m / 2, n / 2, m, n, m, n elements).
void spectral_tables_fill(int m, int n, float bin_w, float bin_h, float2 *tw_m, float2 *tw_n, float2 *ek_m,
                          float2 *ek_n, float *wu, float *wv, cudaStream_t s);
struct SpectralArgs {
    const float *rho_in = nullptr;          // standalone: rho given directly
    unsigned long long *dmap = nullptr;     // loop: int64 fixed-point movable map
    const float *initial = nullptr;         // loop: fixed-cell map
    float fixed_inv = 0.f, coef = 0.f, inv_bin_area = 0.f;
    double movable_area = 1.0;
    bool zero_map = false;
    float *rho_out = nullptr;
    float *fx = nullptr, *fy = nullptr, *psi = nullptr;
    double *partials = nullptr;
    DevState *st = nullptr;
};
void launch_spectral_plan(const SpectralPlan &p, const SpectralArgs &a);
// The warp-form passes (sides 64..256) of many solves as packed launches, one
// per template variant in use (k_spectral.cu): kind PK_ROWS_DCT_W, PK_COLS_W or
// PK_ROWS_INV_W.
struct SpectralJob {
    SpectralPlan p;
    SpectralArgs a;
};
void packed_spectral_stage(PackKind k, const std::vector<SpectralJob> &v, PackedArena &ar,
                           std::vector<PackedLaunch> &out);
bool packed_spectral_launch(const PackedLaunch &l, const unsigned char *dev, cudaStream_t s);
// the map -> rho conversion, overflow and zeroing of R1 alone (tensor-core precisions)
void launch_map_rho(const SpectralArgs &a, size_t mn, float *rho, cudaStream_t s);
cudaError_t spectral_prepare();
// tensor-core form of the spectral solve (k_dctgemm.cu): kind 0 TF32, 1 BF16x3
DctGemmPlan *dctgemm_create(int m, int n, float bin_w, float bin_h, int kind, cudaStream_t stream,
                            std::string &err);
cudaError_t dctgemm_solve(DctGemmPlan &P, const float *rho, float *fx, float *fy, float *psi, int *status);
void dctgemm_destroy(DctGemmPlan *P);
cudaError_t place_prepare();   // opt the density scatter into its dynamic shared memory
size_t spectral_smem_bytes(int m, int n);

int ilog2(int v);

// Message returned by erp_last_error(NULL) on this host thread.
void set_thread_error(const std::string &msg);

}  // namespace erp

#define ERP_CUDA_CHECK_RET(c, expr)                                                  \
    do {                                                                             \
        cudaError_t _e = (expr);                                                     \
        if (_e != cudaSuccess) {                                                     \
            (c).err = std::string(#expr) + ": " + cudaGetErrorString(_e);           \
            return ERP_ECUDA;                                                        \
        }                                                                            \
    } while (0)
