// C ABI of liberplacer_gb300.so (include/erplacer.h): context set-up
// (Placement::new, src/placement.rs:159-178), the reference's stage entry
// points, the CUDA-graph Placement::step, the run loop and accessors.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "erp_internal.cuh"
#include "arena.h"

using namespace erp;

struct erp_ctx {
    Ctx c;
};

struct erp_spectral {
    SpectralPlan p;
    DevState *st;
    std::string err;
    DctGemmPlan *gemm = nullptr;   // tensor-core precisions
};

static thread_local std::string g_create_err;

void erp::set_thread_error(const std::string &msg) { g_create_err = msg; }

extern "C" const char *erp_status_string(erp_status s) {
    switch (s) {
    case ERP_OK: return "ok";
    case ERP_EINVAL: return "invalid argument";
    case ERP_ENOMEM: return "out of memory";
    case ERP_ECUDA: return "CUDA error";
    case ERP_ENAN: return "non-finite value";
    case ERP_ETIMEDOUT: return "device wait timed out";
    case ERP_ENOTSUP: return "not supported";
    case ERP_ENODEV: return "no sm_103 CUDA device";
    case ERP_ESTATE: return "invalid state";
    case ERP_ECANCELED: return "cancelled";
    }
    return "unknown";
}

extern "C" const char *erp_last_error(const erp_ctx *ctx) {
    return ctx ? ctx->c.err.c_str() : g_create_err.c_str();
}

extern "C" int32_t erp_abi_version(void) { return ERP_ABI_VERSION; }

namespace erp {
// A named range on the host timeline of a profiler (NVTX, header-only; no cost
// without a profiler attached): one per public call that does device work.
struct HostRange {
    explicit HostRange(const char *name) { nvtxRangePushA(name); }
    ~HostRange() { nvtxRangePop(); }
    HostRange(const HostRange &) = delete;
    HostRange &operator=(const HostRange &) = delete;
};

// Stream-ordered allocations on the context's stream: creating or destroying a
// context never synchronises the device, so jobs can be admitted and retired
// while other contexts' work runs.  The contexts' arrays come from one pool per
// device that keeps up to kPoolKeep bytes of freed memory for the next contexts
// (the device's default pool returns freed memory to the system at every
// synchronisation), so the next batch or a server admission after a retirement
// reuses the memory of the contexts that went before instead of mapping it again.
constexpr unsigned long long kPoolKeep = 8ull << 30;

cudaError_t ctx_alloc(void **p, size_t bytes, cudaStream_t s) {
    static std::mutex mu;
    static std::vector<cudaMemPool_t> pools;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    cudaMemPool_t pool = nullptr;
    {
        std::lock_guard<std::mutex> lock(mu);
        if ((size_t)dev >= pools.size()) pools.resize((size_t)dev + 1, nullptr);
        if (!pools[dev]) {
            cudaMemPoolProps props;
            memset(&props, 0, sizeof props);
            props.allocType = cudaMemAllocationTypePinned;
            props.handleTypes = cudaMemHandleTypeNone;
            props.location.type = cudaMemLocationTypeDevice;
            props.location.id = dev;
            cudaMemPool_t np = nullptr;
            e = cudaMemPoolCreate(&np, &props);
            if (e != cudaSuccess) return e;
            unsigned long long keep = kPoolKeep;
            e = cudaMemPoolSetAttribute(np, cudaMemPoolAttrReleaseThreshold, &keep);
            if (e != cudaSuccess) {
                cudaMemPoolDestroy(np);
                return e;
            }
            pools[dev] = np;
        }
        pool = pools[dev];
    }
    return cudaMallocFromPoolAsync(p, bytes, pool, s);
}
}  // namespace erp

namespace {

bool pow2_ok(int v) { return v >= 16 && v <= 4096 && (v & (v - 1)) == 0; }

cudaError_t upload(void *dst, const void *src, size_t bytes, cudaStream_t s) {
    if (!bytes) return cudaSuccess;
    return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s);
}

int32_t fixed_shift(double total_area) {
    int e = 0;
    if (total_area > 0) frexp(total_area, &e);
    int s = 61 - e;
    return s < -64 ? -64 : (s > 100 ? 100 : s);
}

erp_status check_device(int dev, std::string &err) {
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        err = "no CUDA device available";
        return ERP_ENODEV;
    }
    if (dev < 0 || dev >= count) {
        err = "device ordinal out of range";
        return ERP_EINVAL;
    }
    int major = 0, minor = 0;   // two attributes, not the whole property set (milliseconds per call)
    if (cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev) != cudaSuccess) {
        cudaGetLastError();
        err = "cudaDeviceGetAttribute failed";
        return ERP_ECUDA;
    }
    if (major != 10 || minor != 3) {
        char buf[128];
        snprintf(buf, sizeof buf, "device %d is sm_%d%d; this library is built for sm_103a only", dev, major, minor);
        err = buf;
        return ERP_ENODEV;
    }
    if (cudaSetDevice(dev) != cudaSuccess) {
        err = "cudaSetDevice failed";
        return ERP_ECUDA;
    }
    return ERP_OK;
}

// The kernels' shared-memory attributes and the resident block counts that size
// the streaming grids belong to the device (its primary context), so they are
// set once per device and process, not per context: a batch creates its
// contexts on several threads at once.  (cudaDeviceReset after the first
// context on a device is not supported: it would clear the attributes.)
erp_status prepare_device(int dev, std::string &err) {
    static std::mutex mu;
    static std::vector<char> ready;
    std::lock_guard<std::mutex> lock(mu);
    if ((size_t)dev < ready.size() && ready[dev]) return ERP_OK;
    cudaError_t e = spectral_prepare();
    if (e == cudaSuccess) e = place_prepare();
    if (e == cudaSuccess) e = place_occupancy();
    if (e != cudaSuccess) {
        cudaGetLastError();
        err = std::string("kernel set-up: ") + cudaGetErrorString(e);
        return ERP_ECUDA;
    }
    if ((size_t)dev >= ready.size()) ready.resize((size_t)dev + 1, 0);
    ready[dev] = 1;
    return ERP_OK;
}

erp_status validate(const erp_design *d, std::string &err) {
#define REQ(cond, msg)        \
    if (!(cond)) {            \
        err = msg;            \
        return ERP_EINVAL;    \
    }
    REQ(d, "design is NULL");
    REQ(d->num_nodes >= 0 && d->num_movable >= 0 && d->num_movable <= d->num_nodes, "bad node counts");
    REQ(d->num_pins >= 0 && d->num_nets >= 0 && d->n_2nets >= 0 && d->n_2nets <= d->num_nets, "bad pin/net counts");
    REQ(d->num_nodes == 0 || (d->x && d->y && d->w && d->h && d->num_pins_f), "instance arrays missing");
    REQ(d->num_pins == 0 || (d->pin_ox && d->pin_oy && d->pin_inst), "pin arrays missing");
    REQ(d->net_ptr && d->inst_pin_ptr, "CSR pointers missing");
    REQ(d->die_w > 0 && d->die_h > 0 && isfinite(d->die_w) && isfinite(d->die_h), "die must have positive, finite size");
    REQ(d->net_ptr[0] == 0, "net_ptr[0] must be 0");
    for (int e = 0; e < d->num_nets; ++e) REQ(d->net_ptr[e + 1] >= d->net_ptr[e], "net_ptr not monotone");
    REQ(d->net_ptr[d->num_nets] == 0 || d->net_pins, "net_pins missing");
    for (int e = 0; e < d->n_2nets; ++e) REQ(d->net_ptr[e + 1] - d->net_ptr[e] == 2, "first n_2nets nets must have 2 pins");
    std::vector<char> seen(d->num_pins, 0);
    for (int k = 0; k < d->net_ptr[d->num_nets]; ++k) {
        int p = d->net_pins[k];
        REQ(p >= 0 && p < d->num_pins, "net pin id out of range");
        REQ(!seen[p], "a pin belongs to more than one net");
        seen[p] = 1;
    }
    for (int p = 0; p < d->num_pins; ++p) {
        REQ(d->pin_inst[p] >= 0 && d->pin_inst[p] < d->num_nodes, "pin_inst out of range");
        REQ(isfinite(d->pin_ox[p]) && isfinite(d->pin_oy[p]), "non-finite pin offset");
    }
    REQ(d->inst_pin_ptr[0] == 0, "inst_pin_ptr[0] must be 0");
    for (int i = 0; i < d->num_nodes; ++i) REQ(d->inst_pin_ptr[i + 1] >= d->inst_pin_ptr[i], "inst_pin_ptr not monotone");
    REQ(d->inst_pin_ptr[d->num_nodes] == 0 || d->inst_pins, "inst_pins missing");
    std::fill(seen.begin(), seen.end(), 0);
    for (int k = 0; k < d->inst_pin_ptr[d->num_nodes]; ++k) {   // macro_2_pins lists each pin once
        const int p = d->inst_pins[k];
        REQ(p >= 0 && p < d->num_pins, "inst pin id out of range");
        REQ(!seen[p], "a pin is listed twice in inst_pins");
        seen[p] = 1;
    }
    for (int i = 0; i < d->num_nodes; ++i) {
        REQ(isfinite(d->x[i]) && isfinite(d->y[i]) && d->w[i] >= 0 && d->h[i] >= 0 && isfinite(d->w[i]) &&
                isfinite(d->h[i]),
            "non-finite or negative instance geometry");
        REQ(d->num_pins_f[i] >= 0 && isfinite(d->num_pins_f[i]), "non-finite or negative num_pins_f");
        for (int k = d->inst_pin_ptr[i]; k < d->inst_pin_ptr[i + 1]; ++k)
            REQ(d->pin_inst[d->inst_pins[k]] == i, "inst_pins disagrees with pin_inst");
    }
    return ERP_OK;
#undef REQ
}

void free_ctx(Ctx &c) {
    if (c.arena) {   // stream-ordered, on the stream it was allocated on
        if (c.stream) cudaFreeAsync(c.arena, c.stream);
        else cudaFree(c.arena);
    }
    if (c.h_st) cudaFreeHost(c.h_st);
    if (c.gemm) dctgemm_destroy(c.gemm);   // synchronises the stream before freeing
    if (c.graph_ready) cudaGraphExecDestroy(c.graph);
    if (c.own_stream && c.stream) cudaStreamDestroy(c.stream);
    delete[] c.h_slot_of_pin;
    delete[] c.h_net_of_internal;
}

SpectralPlan plan_of(Ctx &c) {
    SpectralPlan p;
    p.m = c.m; p.n = c.n; p.logm = c.logm; p.logn = c.logn;
    p.bin_w = c.bin_w; p.bin_h = c.bin_h;
    p.tw_m = c.tw_m; p.tw_n = c.tw_n; p.ek_m = c.ek_m; p.ek_n = c.ek_n;
    p.wu = c.wu; p.wv = c.wv;
    p.t1 = c.t1; p.tx = c.tx; p.ty = c.ty; p.tp = c.tp;
    p.partials = c.partials; p.st = c.st; p.stream = c.stream;
    p.seqs = c.spectral_seqs;
    return p;
}

}  // namespace

namespace erp {
static SpectralArgs spectral_args(Ctx &c, bool zero_map, bool store_rho, bool want_psi) {
    SpectralArgs a;
    a.dmap = c.dmap;
    a.initial = c.initial;
    a.fixed_inv = c.fixed_inv;
    a.coef = c.target_density * c.bin_area;           // src/epotential.rs:272-273
    a.inv_bin_area = c.inv_bin_area;
    a.movable_area = (double)c.movable_area;
    a.zero_map = zero_map;
    a.rho_out = store_rho ? c.rho : nullptr;
    a.fx = c.fx;
    a.fy = c.fy;
    a.psi = want_psi ? c.psi : nullptr;
    a.partials = c.partials;
    a.st = c.st;
    return a;
}

void launch_spectral(Ctx &c, bool zero_map, bool store_rho, bool want_psi) {
    const SpectralArgs a = spectral_args(c, zero_map, store_rho, want_psi);
    if (c.gemm) {   // tensor-core precisions: rho, then the contractions (rho_out is c.rho itself)
        launch_map_rho(a, (size_t)c.m * c.n, c.rho, c.stream);
        dctgemm_solve(*c.gemm, c.rho, c.fx, c.fy, a.psi, &c.st->status);
        return;
    }
    launch_spectral_plan(plan_of(c), a);
}
}  // namespace erp

#define CK(expr)                                                               \
    do {                                                                       \
        cudaError_t _e = (expr);                                               \
        if (_e != cudaSuccess) {                                               \
            c.err = std::string(#expr) + ": " + cudaGetErrorString(_e);       \
            return _e == cudaErrorMemoryAllocation ? ERP_ENOMEM : ERP_ECUDA;  \
        }                                                                      \
    } while (0)

static erp_status create_impl(const erp_design *d, const erp_params *pp, Ctx &c) {
    erp_params prm;
    memset(&prm, 0, sizeof prm);
    if (pp) prm = *pp;
    if (prm.num_bins_x == 0) prm.num_bins_x = 512;
    if (prm.num_bins_y == 0) prm.num_bins_y = 512;
    if (!pow2_ok(prm.num_bins_x) || !pow2_ok(prm.num_bins_y)) {
        c.err = "bin counts must be powers of two in [16, 4096]";
        return ERP_EINVAL;
    }
    if (prm.precision != ERP_PREC_FP32 && prm.precision != ERP_PREC_TF32_GEMM &&
        prm.precision != ERP_PREC_BF16X3_GEMM) {
        c.err = "unsupported precision";
        return ERP_ENOTSUP;
    }
    if (prm.flags & ~ERP_FLAG_EXPIRE_WAITS) {
        c.err = "unknown flags";
        return ERP_EINVAL;
    }
    c.expire_waits = (prm.flags & ERP_FLAG_EXPIRE_WAITS) ? 1u : 0u;
    if (prm.precision != ERP_PREC_FP32 && (prm.num_bins_x % 128 || prm.num_bins_y % 128)) {
        c.err = "the tensor-core spectral solve needs bin counts that are multiples of 128";
        return ERP_EINVAL;
    }
    erp_status s = validate(d, c.err);
    if (s != ERP_OK) return s;
    // target_density < 0 selects the design's cell_utilization; NaN is an error
    c.target_density = prm.target_density >= 0 ? prm.target_density : d->cell_utilization;
    if (isnan(prm.target_density) || !(c.target_density > 0) || !isfinite(c.target_density)) {
        c.err = "target density (or the design's cell_utilization) must be positive and finite";
        return ERP_EINVAL;
    }
    c.movable_area = d->movable_area;
    if (!(c.movable_area > 0) || !isfinite(c.movable_area)) {
        c.err = "movable_area must be positive and finite";
        return ERP_EINVAL;
    }
    s = check_device(prm.device, c.err);
    if (s != ERP_OK) return s;
    c.device = prm.device;
    s = prepare_device(c.device, c.err);
    if (s != ERP_OK) return s;
    const int N = d->num_nodes, NM = d->num_movable, P = d->num_pins, E = d->num_nets;
    c.N = N; c.NM = NM; c.P = P; c.E = E; c.NS = P;
    c.m = prm.num_bins_x; c.n = prm.num_bins_y;
    c.logm = ilog2(c.m); c.logn = ilog2(c.n);
    c.die_w = d->die_w; c.die_h = d->die_h;
    // Bins::new (src/placement.rs:49-66)
    c.bin_w = d->die_w / (float)c.m;
    c.bin_h = d->die_h / (float)c.n;
    c.inv_bw = 1.0f / c.bin_w;
    c.inv_bh = 1.0f / c.bin_h;
    c.bin_area = c.bin_w * c.bin_h;
    c.inv_bin_area = 1.0f / c.bin_area;
    if (prm.stream) {
        c.stream = (cudaStream_t)prm.stream;
        c.own_stream = false;
    } else {
        CK(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
        c.own_stream = true;
    }
    // --- cells: PlacementSolution::new + PotentialComputation::new sizes ---
    std::vector<float> hx(N), hy(N), hcw(N), hch(N), hox(N), hoy(N), hr(N);
    const float cxm = d->die_w / 2.0f, cym = d->die_h / 2.0f;
    const float sqrt2 = 1.41421356237309504880f;
    double mov_tot = 0, fix_tot = 0;
    for (int i = 0; i < N; ++i) {
        const float w = d->w[i], h = d->h[i];
        if (i >= NM || prm.start_mode == ERP_START_DB) {
            hx[i] = d->x[i]; hy[i] = d->y[i];
        } else {
            hx[i] = cxm - w / 2.0f;                       // src/placement.rs:129-130
            hy[i] = cym - h / 2.0f;
        }
        const float cw = fmaxf(w, c.bin_w * sqrt2), ch = fmaxf(h, c.bin_h * sqrt2);   // src/epotential.rs:88-92
        float r = (w * h) / (cw * ch);
        if (i >= NM) r = c.target_density;
        hcw[i] = cw; hch[i] = ch;
        hox[i] = (w - cw) * 0.5f; hoy[i] = (h - ch) * 0.5f;
        hr[i] = r;
        if (i < NM) mov_tot += (double)w * (double)h;
        else fix_tot += (double)w * (double)h;
    }
    c.shift = fixed_shift(mov_tot);
    c.shift0 = fixed_shift(fix_tot);
    c.fixed_scale = ldexpf(1.0f, c.shift);
    c.fixed_inv = ldexpf(1.0f, -c.shift);
    {
        // The scatter keeps each contribution rint((px * py) * 2^S) in 21-bit
        // pieces; two pieces suffice when no contribution reaches 2^42.  A
        // contribution is at most ratio * x-overlap * y-overlap * 2^S, an overlap
        // at most the bin size plus the rounding of a bin edge (a few ulps of the
        // die), the ratio of a movable cell at most 1 (checked here).
        double rmax = 0;
        for (int i = 0; i < NM; ++i) rmax = std::max(rmax, (double)hr[i]);
        const double ex = ldexp((double)d->die_w + c.bin_w, -20), ey = ldexp((double)d->die_h + c.bin_h, -20);
        const double cmax = std::max(rmax, 1.0) * ((double)c.bin_w + ex) * ((double)c.bin_h + ey) *
                            ldexp(1.0, c.shift) * (1.0 + ldexp(1.0, -16));
        c.scatter_planes = cmax < ldexp(1.0, 42) ? 2 : 3;
    }
    // --- nets: degree classes, internal order, pin slots ---
    std::vector<int> cls_of(E);
    int counts[kNumClasses] = {0};
    for (int e = 0; e < E; ++e) {
        const int deg = d->net_ptr[e + 1] - d->net_ptr[e];
        int k;
        if (e < d->n_2nets) k = 0;                       // validated: exactly 2 pins
        else if (deg >= 2 && deg <= kNumExact) k = deg - 1;
        else if (deg <= 16) k = kNumExact;
        else if (deg <= 32) k = kNumExact + 1;
        else k = kNumExact + 2;
        cls_of[e] = k;
        counts[k]++;
    }
    const int widths[kNumClasses] = {1, 1, 1, 1, 1, 1, 1, 1, 2, 4, 32};   // lanes per net (k_wa's dispatch)
    int begin = 0;
    for (int k = 0; k < kNumClasses; ++k) {
        c.cls[k].begin = begin;
        c.cls[k].count = counts[k];
        c.cls[k].width = widths[k];
        c.cls[k].general = k == 0 ? 0 : 1;
        c.cls[k].degree = k == 0 ? 2 : (k < kNumExact ? k + 1 : 0);
        begin += counts[k];
    }
    std::vector<int> fill(kNumClasses);
    for (int k = 0; k < kNumClasses; ++k) fill[k] = c.cls[k].begin;
    c.h_net_of_internal = new int32_t[E > 0 ? E : 1];
    for (int e = 0; e < E; ++e) c.h_net_of_internal[fill[cls_of[e]]++] = e;
    for (int k = 0; k < kNumClasses; ++k)   // degree order within a class: warp-uniform pin loops
        std::stable_sort(c.h_net_of_internal + c.cls[k].begin, c.h_net_of_internal + c.cls[k].begin + c.cls[k].count,
                         [&](int32_t a, int32_t b) {
                             return d->net_ptr[a + 1] - d->net_ptr[a] < d->net_ptr[b + 1] - d->net_ptr[b];
                         });
    std::vector<int32_t> hnet_ptr(E + 1, 0), hslot_cell(P), hcell_ptr(NM + 1, 0);
    std::vector<float2> hslot_off(P);
    c.h_slot_of_pin = new int32_t[P > 0 ? P : 1];
    for (int p = 0; p < P; ++p) c.h_slot_of_pin[p] = -1;
    int slot = 0;
    for (int k = 0; k < kNumClasses; ++k) {
        NetClass &nc = c.cls[k];
        nc.slot0 = slot;
        for (int g = 0; g < nc.count; ++g) {
            const int ie = nc.begin + g, e = c.h_net_of_internal[ie];
            if (nc.degree) {   // pin-major: pin q of net g at slot0 + q * count + g
                hnet_ptr[ie] = nc.slot0 + g;
                for (int q = 0; q < nc.degree; ++q)
                    c.h_slot_of_pin[d->net_pins[d->net_ptr[e] + q]] = nc.slot0 + q * nc.count + g;
            } else {
                hnet_ptr[ie] = slot;
                for (int p = d->net_ptr[e]; p < d->net_ptr[e + 1]; ++p) c.h_slot_of_pin[d->net_pins[p]] = slot++;
            }
        }
        if (nc.degree) slot += nc.degree * nc.count;
    }
    hnet_ptr[E] = slot;
    for (int p = 0; p < P; ++p)
        if (c.h_slot_of_pin[p] < 0) c.h_slot_of_pin[p] = slot++;   // unconnected pins: gradient stays 0
    for (int p = 0; p < P; ++p) {
        const int sl = c.h_slot_of_pin[p];
        hslot_cell[sl] = d->pin_inst[p];
        hslot_off[sl] = make_float2(d->pin_ox[p], d->pin_oy[p]);
    }
    for (int i = 0; i < NM; ++i) hcell_ptr[i + 1] = hcell_ptr[i] + (d->inst_pin_ptr[i + 1] - d->inst_pin_ptr[i]);
    std::vector<int32_t> hcell_slots(hcell_ptr[NM]);
    for (int i = 0; i < NM; ++i)
        for (int k = d->inst_pin_ptr[i], o = hcell_ptr[i]; k < d->inst_pin_ptr[i + 1]; ++k, ++o)
            hcell_slots[o] = c.h_slot_of_pin[d->inst_pins[k]];
    // --- device allocations ---
    const size_t mn = (size_t)c.m * c.n;
    float **cellarr[] = {&c.x, &c.y, &c.w, &c.h, &c.npins, &c.cw, &c.ch, &c.offx, &c.offy, &c.ratio,
                         &c.wlgx, &c.wlgy, &c.prev_x, &c.prev_y, &c.prev_gx, &c.prev_gy};
    ArenaPlan ap;
    for (float **a : cellarr) ap.add(a, (size_t)N + 4);
    ap.add(&c.xy, (size_t)N + 4);
    ap.add(&c.slot_cell, P);
    ap.add(&c.slot_off, P);
    ap.add(&c.slot_grad, P);
    ap.add(&c.net_ptr, (size_t)E + 1);
    ap.add(&c.net_hpwl, E);
    ap.add(&c.cell_slot_ptr, (size_t)NM + 1);
    ap.add(&c.cell_slots, hcell_slots.size());
    ap.add(&c.perm, NM);
    ap.add(&c.pos, (size_t)NM + 4);
    ap.add(&c.dgp, (size_t)NM + 4);
    ap.add(&c.skey, NM);
    ap.add(&c.soff, NM);
    ap.add(&c.sratio, NM);
    ap.add(&c.sort_key, NM);
    ap.add(&c.sort_rank, NM);
    ap.add(&c.sort_hist, scatter_tiles(c.m, c.n));
    ap.add(&c.sort_start, scatter_tiles(c.m, c.n));
    ap.add(&c.dmap, mn);
    float **maps[] = {&c.initial, &c.rho, &c.t1, &c.tx, &c.ty, &c.tp, &c.fx, &c.fy, &c.psi};
    for (float **a : maps) ap.add(a, mn);
    ap.add(&c.partials, kMaxPartials);
    c.max_partials = kMaxPartials;
    ap.add(&c.st, 1);
    ap.add(&c.tw_m, (size_t)c.m / 2);
    ap.add(&c.tw_n, (size_t)c.n / 2);
    ap.add(&c.ek_m, c.m);
    ap.add(&c.ek_n, c.n);
    ap.add(&c.wu, c.m);
    ap.add(&c.wv, c.n);
    // Every array in one pool allocation (arena.h).  Fifty pool operations per
    // context became one; the pool's time per operation grew with the
    // allocations and frees of earlier contexts, and a batch of 64 small designs
    // created after another in the same process took 80-89 ms, 11.5 ms now
    // (fixed tile shapes; 20 ms with the autotuning).
    CK(ctx_alloc(&c.arena, ap.bytes(), c.stream));
    ap.place(c.arena);
    CK(cudaMallocHost((void **)&c.h_st, sizeof(DevState)));
    spectral_tables_fill(c.m, c.n, c.bin_w, c.bin_h, c.tw_m, c.tw_n, c.ek_m, c.ek_n, c.wu, c.wv, c.stream);
    CK(cudaGetLastError());
    if (prm.precision != ERP_PREC_FP32) {
        c.gemm = dctgemm_create(c.m, c.n, c.bin_w, c.bin_h, prm.precision == ERP_PREC_TF32_GEMM ? 0 : 1, c.stream,
                                c.err);
        if (!c.gemm) return ERP_ECUDA;
    }
    // --- uploads ---
    CK(upload(c.x, hx.data(), sizeof(float) * N, c.stream));
    CK(upload(c.y, hy.data(), sizeof(float) * N, c.stream));
    CK(upload(c.w, d->w, sizeof(float) * N, c.stream));
    CK(upload(c.h, d->h, sizeof(float) * N, c.stream));
    CK(upload(c.npins, d->num_pins_f, sizeof(float) * N, c.stream));
    CK(upload(c.cw, hcw.data(), sizeof(float) * N, c.stream));
    CK(upload(c.ch, hch.data(), sizeof(float) * N, c.stream));
    CK(upload(c.offx, hox.data(), sizeof(float) * N, c.stream));
    CK(upload(c.offy, hoy.data(), sizeof(float) * N, c.stream));
    CK(upload(c.ratio, hr.data(), sizeof(float) * N, c.stream));
    // Nesterov::new: prev coords = DB coordinates, prev grads = 0 (src/nesterov.rs:15-24)
    CK(upload(c.prev_x, d->x, sizeof(float) * N, c.stream));
    CK(upload(c.prev_y, d->y, sizeof(float) * N, c.stream));
    for (float *a : {c.prev_gx, c.prev_gy, c.wlgx, c.wlgy})
        CK(cudaMemsetAsync(a, 0, sizeof(float) * ((size_t)N + 4), c.stream));
    CK(cudaMemsetAsync(c.dgp, 0, sizeof(float2) * ((size_t)NM + 4), c.stream));
    CK(cudaMemsetAsync(c.pos, 0, sizeof(int32_t) * ((size_t)NM + 4), c.stream));
    CK(upload(c.slot_cell, hslot_cell.data(), sizeof(int32_t) * P, c.stream));
    CK(upload(c.slot_off, hslot_off.data(), sizeof(float2) * P, c.stream));
    CK(cudaMemsetAsync(c.slot_grad, 0, sizeof(float2) * (P ? P : 1), c.stream));
    CK(upload(c.net_ptr, hnet_ptr.data(), sizeof(int32_t) * (E + 1), c.stream));
    CK(upload(c.cell_slot_ptr, hcell_ptr.data(), sizeof(int32_t) * (NM + 1), c.stream));
    CK(upload(c.cell_slots, hcell_slots.data(), sizeof(int32_t) * hcell_slots.size(), c.stream));
    CK(cudaMemsetAsync(c.dmap, 0, sizeof(unsigned long long) * mn, c.stream));
    for (float **a : maps) CK(cudaMemsetAsync(*a, 0, sizeof(float) * mn, c.stream));
    // scheduler / optimiser state (src/scheduler.rs:52-66, src/nesterov.rs:15-24)
    DevState h;
    memset(&h, 0, sizeof h);
    h.gamma = 4.0f * (c.bin_w + c.bin_h);
    h.base_gamma = h.gamma;
    h.dw = 8e-5f;
    h.alpha = 1.0f;
    h.beta = 0.0f;
    h.expire_waits = c.expire_waits;
    *c.h_st = h;
    CK(cudaMemcpyAsync(c.st, c.h_st, sizeof(DevState), cudaMemcpyHostToDevice, c.stream));
    launch_pack_xy(c);
    launch_scatter_order(c, c.stream);
    c.sort_age = 0;
    // fixed-cell initial density (src/epotential.rs:127-140)
    launch_initial_density(c, nullptr, nullptr, nullptr, nullptr);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c.stream));
    c.map_dirty = false;
    return ERP_OK;
}

extern "C" erp_status erp_create(const erp_design *design, const erp_params *params, erp_ctx **out) {
    HostRange range_("erp_create");
    g_create_err.clear();
    if (!out) {
        g_create_err = "out is NULL";
        return ERP_EINVAL;
    }
    *out = nullptr;
    erp_ctx *ctx = new (std::nothrow) erp_ctx();  // value-initialised: all pointers null
    if (!ctx) return ERP_ENOMEM;
    erp_status s = create_impl(design, params, ctx->c);
    if (s != ERP_OK) {
        g_create_err = ctx->c.err;
        free_ctx(ctx->c);
        delete ctx;
        return s;
    }
    *out = ctx;
    return ERP_OK;
}

extern "C" void erp_destroy(erp_ctx *ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->c.device);
    if (ctx->c.stream) cudaStreamSynchronize(ctx->c.stream);
    free_ctx(ctx->c);
    delete ctx;
}

// ---------------------------------------------------------------------------
#define CTX_CHECK()                        \
    if (!ctx) return ERP_EINVAL;           \
    Ctx &c = ctx->c;                       \
    c.err.clear();                         \
    if (cudaSetDevice(c.device) != cudaSuccess) { c.err = "cudaSetDevice failed"; return ERP_ECUDA; }

// The status bits of the host copy of a context's state.
static erp_status state_status(Ctx &c) {
    if (c.h_st->status & kStatusWaitTimeout) {
        c.err = "a bulk copy into shared memory did not complete within the wait limit";
        return ERP_ETIMEDOUT;
    }
    if (c.h_st->status & 1) {
        c.err = "non-finite HPWL, overflow or step length";
        return ERP_ENAN;
    }
    return ERP_OK;
}

static erp_status pull_state(Ctx &c) {
    CK(cudaMemcpyAsync(c.h_st, c.st, sizeof(DevState), cudaMemcpyDeviceToHost, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    return state_status(c);
}

extern "C" erp_status erp_wirelength(erp_ctx *ctx, float gamma, float *hpwl) {
    CTX_CHECK();
    if (!(gamma > 0)) { c.err = "gamma must be positive"; return ERP_EINVAL; }
    launch_wirelength(c, gamma);
    launch_wl_gather(c);
    CK(cudaGetLastError());
    if (hpwl) {
        erp_status s = pull_state(c);
        *hpwl = c.h_st->hpwl_f;
        return s;
    }
    return ERP_OK;
}

static void enqueue_potential(Ctx &c, bool stage, bool want_psi) {
    if (stage || c.map_dirty) cudaMemsetAsync(c.dmap, 0, sizeof(unsigned long long) * (size_t)c.m * c.n, c.stream);
    launch_density_scatter(c);
    launch_spectral(c, /*zero_map=*/!stage, /*store_rho=*/stage, want_psi);
    launch_force(c, 0);
    c.map_dirty = stage;
}

extern "C" erp_status erp_potential(erp_ctx *ctx, int32_t iteration, float *energy, float *overflow) {
    CTX_CHECK();
    (void)iteration;  // selects the reference's density variant; one fixed-point rule here
    enqueue_potential(c, true, energy != nullptr);
    if (energy) {
        launch_energy(c);
        c.psi_valid = true;
    }
    CK(cudaGetLastError());
    if (energy || overflow) {
        erp_status s = pull_state(c);
        if (energy) *energy = (float)c.h_st->energy;
        if (overflow) *overflow = c.h_st->overflow_f;
        return s;
    }
    return ERP_OK;
}

extern "C" erp_status erp_nesterov(erp_ctx *ctx, int32_t iteration) {
    CTX_CHECK();
    if (iteration < 0) { c.err = "iteration must be >= 0"; return ERP_EINVAL; }
    launch_nesterov(c, iteration);
    CK(cudaGetLastError());
    return ERP_OK;
}

extern "C" erp_status erp_scheduler_update(erp_ctx *ctx, float hpwl, float overflow) {
    CTX_CHECK();
    launch_scheduler(c, 1, hpwl, overflow);
    CK(cudaGetLastError());
    return ERP_OK;
}

extern "C" erp_status erp_should_stop(erp_ctx *ctx, int32_t *stop) {
    CTX_CHECK();
    if (!stop) return ERP_EINVAL;
    erp_status s = pull_state(c);
    const float cur = c.h_st->hpwl_cur, prev = c.h_st->hpwl_prev;
    *stop = (prev != 0.0f && cur != 0.0f && prev > cur * 1.5f) ? 1 : 0;   // src/scheduler.rs:75-81
    return s;
}

namespace erp {
// Placement::step order (src/placement.rs:180-228)
void enqueue_step_kernels(Ctx &c) {
    launch_wirelength(c, -1.0f);
    launch_wl_gather(c);
    launch_density_scatter(c);
    launch_spectral(c, /*zero_map=*/true, /*store_rho=*/false, /*want_psi=*/false);
    launch_force(c, 1);
    launch_nesterov(c, -1);
    launch_scheduler(c, 0, 0.f, 0.f);
}
}  // namespace erp

static int count_kernel_nodes(cudaGraph_t g) {
    size_t nn = 0;
    cudaGraphGetNodes(g, nullptr, &nn);
    std::vector<cudaGraphNode_t> nodes(nn);
    if (nn) cudaGraphGetNodes(g, nodes.data(), &nn);
    int k = 0;
    for (auto nd : nodes) {
        cudaGraphNodeType t;
        if (cudaGraphNodeGetType(nd, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) k++;
    }
    return k;
}

static erp_status ensure_graph(Ctx &c) {
    if (c.graph_ready) return ERP_OK;
    cudaGraph_t g;
    CK(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal));
    enqueue_step_kernels(c);
    cudaError_t e = cudaStreamEndCapture(c.stream, &g);
    if (e != cudaSuccess) {
        c.err = std::string("graph capture: ") + cudaGetErrorString(e);
        cudaGetLastError();
        return ERP_ECUDA;
    }
    c.graph_kernels = count_kernel_nodes(g);
    e = cudaGraphInstantiate(&c.graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        c.err = std::string("graph instantiate: ") + cudaGetErrorString(e);
        return ERP_ECUDA;
    }
    c.graph_ready = true;
    return ERP_OK;
}

// The scatter order follows the cells every kSortEvery steps (a stale order is
// still correct, only slower).
static void refresh_scatter_order(Ctx &c, int steps, cudaStream_t s) {
    c.sort_age += steps;
    if (c.sort_age >= kSortEvery) {
        launch_scatter_order(c, s);
        c.sort_age = 0;
    }
}

static erp_status enqueue_step(Ctx &c) {
    erp_status s = ensure_graph(c);
    if (s != ERP_OK) return s;
    refresh_scatter_order(c, 1, c.stream);
    if (c.map_dirty) {
        CK(cudaMemsetAsync(c.dmap, 0, sizeof(unsigned long long) * (size_t)c.m * c.n, c.stream));
        c.map_dirty = false;
    }
    CK(cudaGraphLaunch(c.graph, c.stream));
    return ERP_OK;
}

extern "C" erp_status erp_step(erp_ctx *ctx, erp_step_stats *stats) {
    HostRange range_("erp_step");
    CTX_CHECK();
    erp_status s = enqueue_step(c);
    if (s != ERP_OK) return s;
    if (stats) {
        s = pull_state(c);
        *stats = c.h_st->last;
        return s;
    }
    return ERP_OK;
}

// The device address of a registered (pinned, device-mapped) host buffer, or
// nullptr for any other memory.
// p[0, n) as device-mapped host memory (registered or cudaHostAlloc'd), or
// nullptr.  Both the first and the last element must be mapped, contiguously,
// so a registration shorter than the array falls back to copies instead of the
// device running past it.  (A range that starts and ends in two different
// registrations with unregistered memory between them is not detected: the
// caller's contract is one registration per array.)
static float *mapped_host(float *p, int n) {
    if (n <= 0) return nullptr;
    cudaPointerAttributes a, b;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess || cudaPointerGetAttributes(&b, p + (n - 1)) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type != cudaMemoryTypeHost || b.type != cudaMemoryTypeHost || !a.devicePointer) return nullptr;
    float *d = static_cast<float *>(a.devicePointer);
    return b.devicePointer == static_cast<void *>(d + (n - 1)) ? d : nullptr;
}

extern "C" erp_status erp_step_host(erp_ctx *ctx, float *x, float *y, erp_step_stats *stats) {
    CTX_CHECK();
    if (!x || !y) return ERP_EINVAL;
    // Registered host buffers are read and written by the device itself (one pass
    // each way, no staging); other host memory goes through copies.
    float *dx = mapped_host(x, c.N), *dy = mapped_host(y, c.N);
    const bool direct = dx && dy;
    if (direct) {
        launch_xy_from_host(c, dx, dy);
    } else {
        CK(cudaMemcpyAsync(c.x, x, sizeof(float) * c.N, cudaMemcpyHostToDevice, c.stream));
        CK(cudaMemcpyAsync(c.y, y, sizeof(float) * c.N, cudaMemcpyHostToDevice, c.stream));
        launch_pack_xy(c);
    }
    erp_status s = enqueue_step(c);
    if (s != ERP_OK) return s;
    if (direct) {
        launch_xy_to_host(c, dx, dy);
    } else {
        CK(cudaMemcpyAsync(x, c.x, sizeof(float) * c.N, cudaMemcpyDeviceToHost, c.stream));
        CK(cudaMemcpyAsync(y, c.y, sizeof(float) * c.N, cudaMemcpyDeviceToHost, c.stream));
    }
    CK(cudaGetLastError());
    s = pull_state(c);
    if (stats) *stats = c.h_st->last;
    return s;
}

extern "C" erp_status erp_run(erp_ctx *ctx, int32_t max_iterations, float stop_overflow,
                              int32_t *iterations_run, erp_step_stats *last) {
    HostRange range_("erp_run");
    CTX_CHECK();
    if (max_iterations < 0) return ERP_EINVAL;
    erp_status s = pull_state(c);
    if (s != ERP_OK) return s;
    const int start = c.h_st->iteration;
    // arm the retire flag
    const float so = stop_overflow > 0 ? stop_overflow : 0.0f;
    CK(cudaMemcpyAsync(&c.st->stop_overflow, &so, sizeof(float), cudaMemcpyHostToDevice, c.stream));
    CK(cudaMemsetAsync(&c.st->done, 0, sizeof(int32_t), c.stream));
    const int chunk = 16;
    int launched = 0;
    cudaEvent_t ev[2];
    CK(cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming));
    int32_t *h_done = nullptr;
    CK(cudaMallocHost((void **)&h_done, 2 * sizeof(int32_t)));
    h_done[0] = h_done[1] = 0;
    int pending = -1;  // buffer index with an outstanding check
    bool stop = false;
    while (!stop && launched < max_iterations) {
        const int k = std::min(chunk, max_iterations - launched);
        for (int i = 0; i < k && s == ERP_OK; ++i) s = enqueue_step(c);
        if (s != ERP_OK) break;
        launched += k;
        const int b = (launched / chunk) & 1;
        CK(cudaMemcpyAsync(&h_done[b], &c.st->done, sizeof(int32_t), cudaMemcpyDeviceToHost, c.stream));
        CK(cudaEventRecord(ev[b], c.stream));
        if (pending >= 0) {
            CK(cudaEventSynchronize(ev[pending]));
            if (h_done[pending]) stop = true;
        }
        pending = b;
    }
    CK(cudaStreamSynchronize(c.stream));
    cudaEventDestroy(ev[0]);
    cudaEventDestroy(ev[1]);
    cudaFreeHost(h_done);
    const float zero = 0.0f;
    CK(cudaMemcpyAsync(&c.st->stop_overflow, &zero, sizeof(float), cudaMemcpyHostToDevice, c.stream));
    CK(cudaMemsetAsync(&c.st->done, 0, sizeof(int32_t), c.stream));
    erp_status s2 = pull_state(c);
    if (iterations_run) *iterations_run = c.h_st->iteration - start;
    if (last) *last = c.h_st->last;
    return s != ERP_OK ? s : s2;
}

extern "C" erp_status erp_get_scalars(erp_ctx *ctx, erp_scalars *o) {
    CTX_CHECK();
    if (!o) return ERP_EINVAL;
    erp_status s = pull_state(c);
    const DevState &h = *c.h_st;
    memset(o, 0, sizeof *o);
    o->iteration = h.iteration;
    o->gamma = h.gamma; o->base_gamma = h.base_gamma; o->density_weight = h.dw;
    o->alpha = h.alpha; o->beta = h.beta;
    o->hpwl_initial = h.hpwl_init; o->hpwl_current = h.hpwl_cur; o->hpwl_previous = h.hpwl_prev;
    o->overflow_current = h.ovf_cur; o->overflow_previous = h.ovf_prev;
    o->hpwl_last = h.hpwl; o->overflow_last = h.overflow; o->energy_last = h.energy;
    o->fixed_shift = c.shift; o->fixed_shift_init = c.shift0;
    o->num_bins_x = c.m; o->num_bins_y = c.n;
    o->bin_w = c.bin_w; o->bin_h = c.bin_h; o->target_density = c.target_density;
    o->graph_kernels = c.graph_kernels;
    return s;
}

extern "C" erp_status erp_set_scalars(erp_ctx *ctx, int32_t iteration, float gamma, float dw,
                                      float alpha, float beta) {
    CTX_CHECK();
    erp_status s = pull_state(c);
    if (s != ERP_OK) return s;
    c.h_st->iteration = iteration;
    c.h_st->gamma = gamma;
    c.h_st->dw = dw;
    c.h_st->alpha = alpha;
    c.h_st->beta = beta;
    CK(cudaMemcpyAsync(c.st, c.h_st, sizeof(DevState), cudaMemcpyHostToDevice, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    return ERP_OK;
}

extern "C" erp_status erp_get_positions(erp_ctx *ctx, float *x, float *y) {
    CTX_CHECK();
    if (!x || !y) return ERP_EINVAL;
    CK(cudaMemcpyAsync(x, c.x, sizeof(float) * c.N, cudaMemcpyDeviceToHost, c.stream));
    CK(cudaMemcpyAsync(y, c.y, sizeof(float) * c.N, cudaMemcpyDeviceToHost, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    return ERP_OK;
}

extern "C" erp_status erp_set_positions(erp_ctx *ctx, const float *x, const float *y) {
    CTX_CHECK();
    if (!x || !y) return ERP_EINVAL;
    CK(cudaMemcpyAsync(c.x, x, sizeof(float) * c.N, cudaMemcpyHostToDevice, c.stream));
    CK(cudaMemcpyAsync(c.y, y, sizeof(float) * c.N, cudaMemcpyHostToDevice, c.stream));
    launch_pack_xy(c);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c.stream));
    return ERP_OK;
}

extern "C" erp_status erp_set_nesterov_history(erp_ctx *ctx, const float *px, const float *py,
                                               const float *pgx, const float *pgy) {
    CTX_CHECK();
    if (!px || !py || !pgx || !pgy) return ERP_EINVAL;
    CK(cudaMemcpyAsync(c.prev_x, px, sizeof(float) * c.N, cudaMemcpyHostToDevice, c.stream));
    CK(cudaMemcpyAsync(c.prev_y, py, sizeof(float) * c.N, cudaMemcpyHostToDevice, c.stream));
    CK(cudaMemcpyAsync(c.prev_gx, pgx, sizeof(float) * c.N, cudaMemcpyHostToDevice, c.stream));
    CK(cudaMemcpyAsync(c.prev_gy, pgy, sizeof(float) * c.N, cudaMemcpyHostToDevice, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    return ERP_OK;
}

extern "C" erp_status erp_get_array(erp_ctx *ctx, erp_array which, void *dst, size_t bytes) {
    CTX_CHECK();
    if (!dst) return ERP_EINVAL;
    const size_t mn = (size_t)c.m * c.n;
    const void *src = nullptr;
    size_t need = 0;
    switch (which) {
    case ERP_ARR_WL_GRAD_X: src = c.wlgx; need = sizeof(float) * c.N; break;
    case ERP_ARR_WL_GRAD_Y: src = c.wlgy; need = sizeof(float) * c.N; break;
    case ERP_ARR_DENS_GRAD_X:
    case ERP_ARR_DENS_GRAD_Y: {   // kept in scatter order on the device: back to cell order
        need = sizeof(float) * c.N;
        if (bytes < need) { c.err = "destination too small"; return ERP_EINVAL; }
        std::vector<float2> g(c.NM ? c.NM : 1);
        std::vector<int32_t> at(c.NM ? c.NM : 1);
        CK(cudaMemcpyAsync(g.data(), c.dgp, sizeof(float2) * c.NM, cudaMemcpyDeviceToHost, c.stream));
        CK(cudaMemcpyAsync(at.data(), c.pos, sizeof(int32_t) * c.NM, cudaMemcpyDeviceToHost, c.stream));
        CK(cudaStreamSynchronize(c.stream));
        float *o = (float *)dst;
        for (int i = 0; i < c.N; ++i) {
            const float2 v = i < c.NM ? g[at[i]] : make_float2(0.0f, 0.0f);
            o[i] = which == ERP_ARR_DENS_GRAD_X ? v.x : v.y;
        }
        return ERP_OK;
    }
    case ERP_ARR_DENSITY_I64: src = c.dmap; need = sizeof(int64_t) * mn; break;
    case ERP_ARR_DENSITY: src = c.rho; need = sizeof(float) * mn; break;
    case ERP_ARR_INITIAL: src = c.initial; need = sizeof(float) * mn; break;
    case ERP_ARR_FIELD_X: src = c.fx; need = sizeof(float) * mn; break;
    case ERP_ARR_FIELD_Y: src = c.fy; need = sizeof(float) * mn; break;
    case ERP_ARR_POTENTIAL: src = c.psi; need = sizeof(float) * mn; break;
    case ERP_ARR_PREV_X: src = c.prev_x; need = sizeof(float) * c.N; break;
    case ERP_ARR_PREV_Y: src = c.prev_y; need = sizeof(float) * c.N; break;
    case ERP_ARR_PREV_GX: src = c.prev_gx; need = sizeof(float) * c.N; break;
    case ERP_ARR_PREV_GY: src = c.prev_gy; need = sizeof(float) * c.N; break;
    case ERP_ARR_PIN_GRAD_X:
    case ERP_ARR_PIN_GRAD_Y: {
        need = sizeof(float) * c.P;
        if (bytes < need) { c.err = "destination too small"; return ERP_EINVAL; }
        std::vector<float2> tmp(c.P ? c.P : 1);
        CK(cudaMemcpyAsync(tmp.data(), c.slot_grad, sizeof(float2) * c.P, cudaMemcpyDeviceToHost, c.stream));
        CK(cudaStreamSynchronize(c.stream));
        float *o = (float *)dst;
        for (int p = 0; p < c.P; ++p) {
            const float2 v = tmp[c.h_slot_of_pin[p]];
            o[p] = which == ERP_ARR_PIN_GRAD_X ? v.x : v.y;
        }
        return ERP_OK;
    }
    case ERP_ARR_NET_HPWL: {
        need = sizeof(float) * c.E;
        if (bytes < need) { c.err = "destination too small"; return ERP_EINVAL; }
        std::vector<float> tmp(c.E ? c.E : 1);
        CK(cudaMemcpyAsync(tmp.data(), c.net_hpwl, sizeof(float) * c.E, cudaMemcpyDeviceToHost, c.stream));
        CK(cudaStreamSynchronize(c.stream));
        float *o = (float *)dst;
        for (int ie = 0; ie < c.E; ++ie) o[c.h_net_of_internal[ie]] = tmp[ie];
        return ERP_OK;
    }
    default: c.err = "unknown array"; return ERP_EINVAL;
    }
    if (bytes < need) { c.err = "destination too small"; return ERP_EINVAL; }
    CK(cudaMemcpyAsync(dst, src, need, cudaMemcpyDeviceToHost, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    return ERP_OK;
}

extern "C" erp_status erp_synchronize(erp_ctx *ctx) {
    CTX_CHECK();
    CK(cudaStreamSynchronize(c.stream));
    return ERP_OK;
}

// reps < 0: -reps whole steps launched eagerly in graph order with an event
// between the stages and no flush (warm caches, as inside the step graph).
static erp_status profile_warm(Ctx &c, int reps, float *ms_out) {
    cudaEvent_t ev[ERP_NUM_STAGES + 1];
    for (auto &e : ev) CK(cudaEventCreate(&e));
    if (c.map_dirty) {
        CK(cudaMemsetAsync(c.dmap, 0, sizeof(unsigned long long) * (size_t)c.m * c.n, c.stream));
        c.map_dirty = false;
    }
    double tot[ERP_NUM_STAGES] = {0};
    erp_status rc = ERP_OK;
    for (int r = 0; r <= reps && rc == ERP_OK; ++r) {   // r == 0: untimed warm-up
        cudaEventRecord(ev[0], c.stream);
        launch_wirelength(c, -1.0f);
        cudaEventRecord(ev[1], c.stream);
        launch_wl_gather(c);
        cudaEventRecord(ev[2], c.stream);
        launch_density_scatter(c);
        cudaEventRecord(ev[3], c.stream);
        launch_spectral(c, /*zero_map=*/true, false, false);
        cudaEventRecord(ev[4], c.stream);
        launch_force(c, 1);
        cudaEventRecord(ev[5], c.stream);
        launch_nesterov(c, -1);
        cudaEventRecord(ev[6], c.stream);
        launch_scheduler(c, 0, 0.f, 0.f);
        cudaEventRecord(ev[7], c.stream);
        const cudaError_t err = cudaEventSynchronize(ev[7]);
        if (err != cudaSuccess) {
            c.err = cudaGetErrorString(err);
            rc = ERP_ECUDA;
            break;
        }
        for (int k = 0; k < ERP_NUM_STAGES && r > 0; ++k) {
            float ms = 0;
            cudaEventElapsedTime(&ms, ev[k], ev[k + 1]);
            tot[k] += ms;
        }
    }
    for (int k = 0; k < ERP_NUM_STAGES; ++k) ms_out[k] = (float)(tot[k] / reps);
    for (auto &e : ev) cudaEventDestroy(e);
    return rc;
}

extern "C" erp_status erp_profile_stages(erp_ctx *ctx, int32_t reps, float *ms_out) {
    CTX_CHECK();
    if (reps == 0 || !ms_out) return ERP_EINVAL;
    if (reps < 0) return profile_warm(c, -reps, ms_out);
    const size_t flush_bytes = 256u << 20;
    void *flush = nullptr;
    CK(cudaMalloc(&flush, flush_bytes));
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    const size_t mn = (size_t)c.m * c.n;
    erp_status rc = ERP_OK;
    for (int stage = 0; stage < ERP_NUM_STAGES && rc == ERP_OK; ++stage) {
        double total = 0;
        for (int r = 0; r <= reps; ++r) {   // r == 0: untimed warm-up
            cudaMemsetAsync(flush, r & 0xff, flush_bytes, c.stream);
            cudaEventRecord(e0, c.stream);
            switch (stage) {
            case ERP_STAGE_WIRELENGTH: launch_wirelength(c, -1.0f); break;
            case ERP_STAGE_WL_GATHER: launch_wl_gather(c); break;
            case ERP_STAGE_DENSITY:
                cudaMemsetAsync(c.dmap, 0, sizeof(unsigned long long) * mn, c.stream);
                launch_density_scatter(c);
                break;
            case ERP_STAGE_SPECTRAL: launch_spectral(c, true, false, false); break;
            case ERP_STAGE_FORCE: launch_force(c, 1); break;
            case ERP_STAGE_NESTEROV: launch_nesterov(c, -1); break;
            default: launch_scheduler(c, 0, 0.f, 0.f); break;
            }
            cudaEventRecord(e1, c.stream);
            cudaError_t err = cudaEventSynchronize(e1);
            if (err != cudaSuccess) {
                c.err = cudaGetErrorString(err);
                rc = ERP_ECUDA;
                break;
            }
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            if (r > 0) total += ms;
        }
        ms_out[stage] = (float)(total / reps);
    }
    c.map_dirty = true;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(flush);
    if (rc == ERP_OK) {
        cudaError_t err = cudaGetLastError();
        if (err != cudaSuccess) { c.err = cudaGetErrorString(err); rc = ERP_ECUDA; }
    }
    return rc;
}

// ---------------------------------------------------------------------------
// headless snapshots (src/drawing.rs:7-60, src/epotential.rs:199-223)
extern "C" erp_status erp_snapshot_size(erp_ctx *ctx, int32_t *width, int32_t *height) {
    CTX_CHECK();
    if (!width || !height) return ERP_EINVAL;
    const double w = ceil((double)c.die_w), h = ceil((double)c.die_h);
    if (!(w >= 1.0) || !(h >= 1.0) || w * h > (double)(1u << 30)) {
        c.err = "die too large for a one-pixel-per-unit image";
        return ERP_EINVAL;
    }
    *width = (int32_t)w;
    *height = (int32_t)h;
    return ERP_OK;
}

extern "C" erp_status erp_snapshot_placement(erp_ctx *ctx, uint8_t *rgb, size_t bytes) {
    int32_t W = 0, H = 0;
    erp_status st = erp_snapshot_size(ctx, &W, &H);
    if (st != ERP_OK) return st;
    Ctx &c = ctx->c;
    const size_t npix = (size_t)W * H;
    if (!rgb || bytes < 3 * npix) { c.err = "destination smaller than width * height * 3"; return ERP_EINVAL; }
    int *d_top = nullptr;
    unsigned char *d_rgb = nullptr;
    CK(cudaMallocAsync((void **)&d_top, sizeof(int) * npix, c.stream));
    CK(cudaMallocAsync((void **)&d_rgb, 3 * npix, c.stream));
    cudaError_t e = launch_snapshot_placement(c, W, H, d_rgb, d_top);
    if (e == cudaSuccess) e = cudaMemcpyAsync(rgb, d_rgb, 3 * npix, cudaMemcpyDeviceToHost, c.stream);
    cudaFreeAsync(d_top, c.stream);
    cudaFreeAsync(d_rgb, c.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
    if (e != cudaSuccess) { c.err = cudaGetErrorString(e); return ERP_ECUDA; }
    return ERP_OK;
}

extern "C" erp_status erp_snapshot_density(erp_ctx *ctx, uint8_t *rgb, size_t bytes) {
    CTX_CHECK();
    const size_t mn = (size_t)c.m * c.n;
    if (!rgb || bytes < 3 * mn) { c.err = "destination smaller than m * n * 3"; return ERP_EINVAL; }
    // the density map of the current positions (as erp_potential stores it)
    enqueue_potential(c, true, false);
    unsigned char *d_rgb = nullptr;
    unsigned *d_mm = nullptr;
    CK(cudaMallocAsync((void **)&d_rgb, 3 * mn, c.stream));
    CK(cudaMallocAsync((void **)&d_mm, 2 * sizeof(unsigned), c.stream));
    cudaError_t e = launch_snapshot_density(c, c.rho, d_rgb, d_mm);
    if (e == cudaSuccess) e = cudaMemcpyAsync(rgb, d_rgb, 3 * mn, cudaMemcpyDeviceToHost, c.stream);
    cudaFreeAsync(d_rgb, c.stream);
    cudaFreeAsync(d_mm, c.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
    if (e != cudaSuccess) { c.err = cudaGetErrorString(e); return ERP_ECUDA; }
    return ERP_OK;
}

// ---------------------------------------------------------------------------
// checkpoint / resume: the state that carries from one Placement::step to the
// next -- positions, Nesterov history (src/nesterov.rs:6-13) and every scalar
// of the scheduler and optimiser (DevState) -- in a versioned host buffer.
namespace {
struct CkptHeader {
    char magic[8];        // "ERPCKPT\0"
    uint32_t version;     // 1
    uint32_t state_bytes; // sizeof(DevState)
    int32_t N, NM, P, E, m, n;
};
constexpr int kCkptArrays = 6;   // x, y, prev_x, prev_y, prev_gx, prev_gy
size_t ckpt_bytes(const Ctx &c) {
    return sizeof(CkptHeader) + sizeof(DevState) + (size_t)kCkptArrays * sizeof(float) * (size_t)c.N;
}
}  // namespace

extern "C" erp_status erp_checkpoint_size(erp_ctx *ctx, size_t *bytes) {
    CTX_CHECK();
    if (!bytes) return ERP_EINVAL;
    *bytes = ckpt_bytes(c);
    return ERP_OK;
}

extern "C" erp_status erp_checkpoint(erp_ctx *ctx, void *buf, size_t bytes) {
    CTX_CHECK();
    if (!buf || bytes < ckpt_bytes(c)) { c.err = "buffer smaller than erp_checkpoint_size"; return ERP_EINVAL; }
    CkptHeader hd;
    memset(&hd, 0, sizeof hd);
    memcpy(hd.magic, "ERPCKPT", 8);
    hd.version = 1;
    hd.state_bytes = (uint32_t)sizeof(DevState);
    hd.N = c.N; hd.NM = c.NM; hd.P = c.P; hd.E = c.E; hd.m = c.m; hd.n = c.n;
    char *o = (char *)buf;
    memcpy(o, &hd, sizeof hd);
    o += sizeof hd;
    CK(cudaMemcpyAsync(o, c.st, sizeof(DevState), cudaMemcpyDeviceToHost, c.stream));
    o += sizeof(DevState);
    const float *arr[kCkptArrays] = {c.x, c.y, c.prev_x, c.prev_y, c.prev_gx, c.prev_gy};
    for (const float *a : arr) {
        CK(cudaMemcpyAsync(o, a, sizeof(float) * c.N, cudaMemcpyDeviceToHost, c.stream));
        o += sizeof(float) * c.N;
    }
    CK(cudaStreamSynchronize(c.stream));
    return ERP_OK;
}

extern "C" erp_status erp_restore(erp_ctx *ctx, const void *buf, size_t bytes) {
    CTX_CHECK();
    if (!buf || bytes < sizeof(CkptHeader)) { c.err = "not a checkpoint"; return ERP_EINVAL; }
    CkptHeader hd;
    memcpy(&hd, buf, sizeof hd);
    if (memcmp(hd.magic, "ERPCKPT", 8) != 0 || hd.version != 1 || hd.state_bytes != sizeof(DevState)) {
        c.err = "not a checkpoint of this library version";
        return ERP_EINVAL;
    }
    if (hd.N != c.N || hd.NM != c.NM || hd.P != c.P || hd.E != c.E || hd.m != c.m || hd.n != c.n) {
        c.err = "checkpoint of a different design or bin grid";
        return ERP_EINVAL;
    }
    if (bytes < ckpt_bytes(c)) { c.err = "truncated checkpoint"; return ERP_EINVAL; }
    const char *i = (const char *)buf + sizeof hd;
    memcpy(c.h_st, i, sizeof(DevState));
    // between steps every reduction's arrival counter is zero; a damaged buffer
    // must not leave the last-block finalizes of the next step unreachable
    memset(c.h_st->ctr, 0, sizeof c.h_st->ctr);
    c.h_st->expire_waits = c.expire_waits;   // the restoring context's own wait rule
    CK(cudaMemcpyAsync(c.st, c.h_st, sizeof(DevState), cudaMemcpyHostToDevice, c.stream));
    i += sizeof(DevState);
    float *arr[kCkptArrays] = {c.x, c.y, c.prev_x, c.prev_y, c.prev_gx, c.prev_gy};
    for (float *a : arr) {
        CK(cudaMemcpyAsync(a, i, sizeof(float) * c.N, cudaMemcpyHostToDevice, c.stream));
        i += sizeof(float) * c.N;
    }
    launch_pack_xy(c);
    c.map_dirty = true;   // the next step starts from a cleared map
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c.stream));
    return ERP_OK;
}

// ---------------------------------------------------------------------------
// batched instances: one graph, one branch per instance
struct erp_batch {
    std::vector<erp_ctx *> ctx;
    cudaStream_t master = nullptr;
    int scatter_cells = 0;                 // autotuned cells per scatter block (0: the alone rule)
    std::vector<std::pair<int, float>> tuning;   // (candidate, ms of all instances' scatters together)
    int spectral_seqs = 0;                 // autotuned sequences per block of the warp-form spectral passes
    bool packed = true;                    // small FP32 instances in packed launches (else a branch each)
    int packed_instances = 0;              // how many of them (at creation)
    void *pack_dev = nullptr;              // argument tables of the packed launches
    size_t pack_cap = 0;
    std::vector<std::pair<int, float>> spec_tuning;   // (candidate, ms of all instances' spectral passes)
    cudaGraphExec_t graph = nullptr;
    bool graph_ready = false;
    cudaGraphExec_t sort_graph = nullptr;  // the active instances' scatter-order refreshes, a branch each
    bool sort_ready = false;
    int graph_kernels = 0;
    DevState **d_states = nullptr;   // device array of the instances' state pointers
    int32_t *d_done = nullptr;
    int32_t *h_done = nullptr;       // pinned
    int device = 0;
    std::string err;
};

static erp_status batch_tune_scatter(erp_batch *b);
static erp_status batch_tune_spectral(erp_batch *b);
static bool packable(const Ctx &c);
// Packed launches pay once several instances share them: one tiny instance
// alone ran 47.9 us per iteration in a branch against 53.5 packed, eight 73.6
// against 63.6, sixty-four 710 against 151.
constexpr int kPackMin = 4;

static erp_status batch_fail(erp_batch *b, erp_status s, const std::string &msg) {
    b->err = msg;
    return s;
}

extern "C" erp_status erp_batch_create(const erp_design *designs, const erp_params *params,
                                       int32_t count, erp_batch **out) {
    HostRange range_("erp_batch_create");
    g_create_err.clear();
    if (!out || !designs || count < 1) {
        g_create_err = "invalid batch arguments";
        return ERP_EINVAL;
    }
    *out = nullptr;
    erp_batch *b = new (std::nothrow) erp_batch();
    if (!b) return ERP_ENOMEM;
    erp_status s = ERP_OK;
    // Instances are independent: their host-side set-up (validation, net
    // classes, pin renumbering, uploads) runs on several host threads.
    std::vector<erp_ctx *> made(count, nullptr);
    std::vector<erp_status> st(count, ERP_OK);
    std::vector<std::string> msg(count);
    std::atomic<int> next(0);
    // largest designs first (pins + cells: the host preparation's work), so that
    // no big one starts last and leaves the other threads idle
    std::vector<int> order(count);
    for (int i = 0; i < count; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        return (int64_t)designs[a].num_pins + designs[a].num_nodes > (int64_t)designs[b].num_pins + designs[b].num_nodes;
    });
    auto worker = [&]() {
        for (int k = next++; k < count; k = next++) {
            const int i = order[k];
            erp_params p;
            memset(&p, 0, sizeof p);
            if (params) p = params[i];
            p.stream = nullptr;   // every instance gets its own stream (its graph branch)
            st[i] = erp_create(designs + i, &p, &made[i]);
            if (st[i] != ERP_OK) msg[i] = g_create_err;
        }
    };
    unsigned nt = std::thread::hardware_concurrency();
    nt = std::max(1u, std::min(nt ? nt : 1u, std::min(16u, (unsigned)count)));
    std::vector<std::thread> pool;
    for (unsigned t = 1; t < nt; ++t) pool.emplace_back(worker);
    worker();
    for (auto &t : pool) t.join();
    for (int i = 0; i < count; ++i) {
        if (made[i]) b->ctx.push_back(made[i]);
        if (st[i] != ERP_OK && s == ERP_OK) {
            s = st[i];
            g_create_err = "instance " + std::to_string(i) + ": " + msg[i];
        }
    }
    if (s == ERP_OK) {
        b->device = b->ctx[0]->c.device;
        for (auto *c : b->ctx)
            if (c->c.device != b->device) {
                s = ERP_EINVAL;
                g_create_err = "all instances of a batch must use the same device";
            }
    }
    if (s == ERP_OK) {
        cudaSetDevice(b->device);
        std::vector<DevState *> sts;
        for (auto *c : b->ctx) sts.push_back(c->c.st);
        bool ok = cudaStreamCreateWithFlags(&b->master, cudaStreamNonBlocking) == cudaSuccess &&
                  cudaMalloc(&b->d_states, sizeof(DevState *) * count) == cudaSuccess &&
                  cudaMalloc(&b->d_done, sizeof(int32_t) * count * 2) == cudaSuccess &&
                  cudaMallocHost(&b->h_done, sizeof(int32_t) * count * 2) == cudaSuccess &&
                  cudaMemcpy(b->d_states, sts.data(), sizeof(DevState *) * count, cudaMemcpyHostToDevice) == cudaSuccess;
        if (!ok) {
            s = ERP_ENOMEM;
            g_create_err = "batch allocation failed";
        }
    }
    if (s == ERP_OK) {
        s = batch_tune_scatter(b);
        if (s == ERP_OK) s = batch_tune_spectral(b);
        if (s != ERP_OK) g_create_err = b->err;
    }
    if (s == ERP_OK) {
        const char *form = getenv("ERP_BATCH_FORM");
        b->packed = !(form && strcmp(form, "branches") == 0);
        b->packed_instances = 0;
        if (b->packed)
            for (auto *x : b->ctx) b->packed_instances += packable(x->c) ? 1 : 0;
        if (b->packed_instances < kPackMin) b->packed_instances = 0;
    }
    if (s != ERP_OK) {
        erp_batch_destroy(b);
        return s;
    }
    *out = b;
    return ERP_OK;
}

extern "C" erp_status erp_batch_tuning(const erp_batch *b, int32_t *chosen, int32_t *cells, float *ms, int32_t cap,
                                       int32_t *count) {
    if (!b || cap < 0 || (cap > 0 && (!cells || !ms))) return ERP_EINVAL;
    if (chosen) *chosen = b->scatter_cells;
    const int k = std::min<int>(cap, (int)b->tuning.size());
    for (int i = 0; i < k; ++i) {
        cells[i] = b->tuning[i].first;
        ms[i] = b->tuning[i].second;
    }
    if (count) *count = (int32_t)b->tuning.size();
    return ERP_OK;
}

// Autotuner of the scatter's block shape for a batch.  Run alone a context
// spreads its cells over many small blocks; with every instance of a batch on the
// GPU at once, fewer fuller blocks (fewer windows to clear and flush) measured
// faster.  Each candidate is timed on a graph of all instances' scatters running
// together; the scatter only adds into the int64 map, which is cleared again
// afterwards, so no placement state changes, and the block shape decides no bit
// of the map.  It runs once, at creation (a second calibration after 128
// iterations, with the cells spread, chose the same shape on the 64-design mix
// and only cost its time).  ERP_BATCH_SCATTER_CELLS=<n> fixes the choice instead.
static erp_status batch_tune_scatter(erp_batch *b) {
    const int cand[] = {0, 512, 1024, 2048};
    if (const char *env = getenv("ERP_BATCH_SCATTER_CELLS")) {
        const int v = atoi(env);
        b->scatter_cells = v < 0 ? 0 : std::min(v, 2048);
        for (auto *x : b->ctx) x->c.scatter_cells = b->scatter_cells;
        return ERP_OK;
    }
    cudaEvent_t fork, e0, e1;
    if (cudaEventCreateWithFlags(&fork, cudaEventDisableTiming) != cudaSuccess) return ERP_ECUDA;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    std::vector<cudaEvent_t> joins(b->ctx.size());
    for (auto &e : joins) cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    float best = 0.0f;
    int best_c = 0;
    erp_status rc = ERP_OK;
    b->tuning.clear();
    for (int c : cand) {
        for (auto *x : b->ctx) x->c.scatter_cells = c;
        cudaGraph_t g;
        cudaGraphExec_t ge = nullptr;
        cudaError_t e = cudaStreamBeginCapture(b->master, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            cudaEventRecord(fork, b->master);
            for (size_t i = 0; i < b->ctx.size(); ++i) {
                Ctx &x = b->ctx[i]->c;
                cudaStreamWaitEvent(x.stream, fork, 0);
                cudaMemsetAsync(x.dmap, 0, sizeof(unsigned long long) * (size_t)x.m * x.n, x.stream);
                launch_density_scatter(x);
                cudaEventRecord(joins[i], x.stream);
                cudaStreamWaitEvent(b->master, joins[i], 0);
            }
            e = cudaStreamEndCapture(b->master, &g);
        }
        if (e == cudaSuccess) {
            e = cudaGraphInstantiate(&ge, g, 0);
            cudaGraphDestroy(g);
        }
        float ms = 0.0f;
        if (e == cudaSuccess) {
            cudaGraphLaunch(ge, b->master);   // warm-up
            cudaEventRecord(e0, b->master);
            for (int r = 0; r < 3; ++r) cudaGraphLaunch(ge, b->master);
            cudaEventRecord(e1, b->master);
            e = cudaEventSynchronize(e1);
            if (e == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
            cudaGraphExecDestroy(ge);
        }
        if (e != cudaSuccess) {
            cudaGetLastError();
            b->err = std::string("scatter autotune: ") + cudaGetErrorString(e);
            rc = ERP_ECUDA;
            break;
        }
        b->tuning.emplace_back(c, ms / 3.0f);
        if (b->tuning.size() == 1 || ms < best) best = ms;
    }
    // The calibration runs the scatters alone, where more, smaller blocks look
    // better than they are inside the step graph, which runs the other passes of
    // every instance beside them (whole runs of the 64-design mix: 2048 cells per
    // block 512k jobs/h, 1024 494k, 512 467k, the alone rule 431k).  So among the
    // candidates within 10 % of the fastest the one with the fewest blocks wins.
    for (const auto &t : b->tuning) {
        const int c = t.first;
        const bool fewer = c == 0 ? false : (best_c == 0 || c > best_c);
        if (t.second * 3.0f <= 1.10f * best && fewer) best_c = c;
    }
    if (best_c == 0)
        for (const auto &t : b->tuning)
            if (t.second * 3.0f <= best) best_c = t.first;
    b->scatter_cells = rc == ERP_OK ? best_c : 0;
    for (auto *x : b->ctx) {   // the maps are cleared again: the calibration leaves no trace
        x->c.scatter_cells = b->scatter_cells;
        cudaMemsetAsync(x->c.dmap, 0, sizeof(unsigned long long) * (size_t)x->c.m * x->c.n, b->master);
    }
    if (cudaStreamSynchronize(b->master) != cudaSuccess && rc == ERP_OK) rc = ERP_ECUDA;
    cudaEventDestroy(fork);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    for (auto &e : joins) cudaEventDestroy(e);
    return rc;
}

// Autotuner of the spectral passes' tile shape for a batch: the sequences (rows
// or columns) per block of the warp-form passes, which serve the sides 64..256
// that most instances of a mix have.  Alone, four per block measured fastest
// at every side; with every instance's passes on the GPU at once the best shape
// can differ, as for the scatter.  Each candidate is timed on a graph of all FP32
// instances' three passes running together, and the fastest is kept.  The
// passes read the (cleared) map and the fixed-cell map and write only the
// intermediates, the fields and the step's overflow, which the first step
// recomputes; the shape decides no bit of the results (a block's rows are
// transformed the same way whichever block holds them).  Instances on the
// tensor-core solve, or with no side in 64..256, keep their shape.
static erp_status batch_tune_spectral(erp_batch *b) {
    const int cand[] = {0, kSeqCandidates[0], kSeqCandidates[1]};
    std::vector<Ctx *> xs;
    for (auto *x : b->ctx) {
        Ctx &c = x->c;
        const bool warp_m = c.m >= 64 && c.m <= 256, warp_n = c.n >= 64 && c.n <= 256;
        if (!c.gemm && (warp_m || warp_n)) xs.push_back(&c);
    }
    b->spec_tuning.clear();
    b->spectral_seqs = 0;
    if (const char *env = getenv("ERP_BATCH_SPECTRAL_SEQS")) {
        const int v = atoi(env);
        b->spectral_seqs = (v == kSeqCandidates[0] || v == kSeqCandidates[1]) ? v : 0;
        for (Ctx *c : xs) c->spectral_seqs = b->spectral_seqs;
        return ERP_OK;
    }
    if (xs.empty()) return ERP_OK;
    cudaEvent_t fork, e0, e1;
    if (cudaEventCreateWithFlags(&fork, cudaEventDisableTiming) != cudaSuccess) return ERP_ECUDA;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    std::vector<cudaEvent_t> joins(xs.size());
    for (auto &e : joins) cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    erp_status rc = ERP_OK;
    float best = 0.0f;
    int best_c = 0;
    for (int cnd : cand) {
        for (Ctx *c : xs) c->spectral_seqs = cnd;
        cudaGraph_t g;
        cudaGraphExec_t ge = nullptr;
        cudaError_t e = cudaStreamBeginCapture(b->master, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            cudaEventRecord(fork, b->master);
            for (size_t i = 0; i < xs.size(); ++i) {
                Ctx &x = *xs[i];
                cudaStreamWaitEvent(x.stream, fork, 0);
                launch_spectral(x, /*zero_map=*/true, /*store_rho=*/false, /*want_psi=*/false);
                cudaEventRecord(joins[i], x.stream);
                cudaStreamWaitEvent(b->master, joins[i], 0);
            }
            e = cudaStreamEndCapture(b->master, &g);
        }
        if (e == cudaSuccess) {
            e = cudaGraphInstantiate(&ge, g, 0);
            cudaGraphDestroy(g);
        }
        float ms = 0.0f;
        if (e == cudaSuccess) {
            cudaGraphLaunch(ge, b->master);   // warm-up
            cudaEventRecord(e0, b->master);
            for (int r = 0; r < 3; ++r) cudaGraphLaunch(ge, b->master);
            cudaEventRecord(e1, b->master);
            e = cudaEventSynchronize(e1);
            if (e == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
            cudaGraphExecDestroy(ge);
        }
        if (e != cudaSuccess) {
            cudaGetLastError();
            b->err = std::string("spectral autotune: ") + cudaGetErrorString(e);
            rc = ERP_ECUDA;
            break;
        }
        b->spec_tuning.emplace_back(cnd, ms / 3.0f);
        if (b->spec_tuning.size() == 1 || ms / 3.0f < best) {
            best = ms / 3.0f;
            best_c = cnd;
        }
    }
    b->spectral_seqs = rc == ERP_OK ? best_c : 0;
    for (Ctx *c : xs) c->spectral_seqs = b->spectral_seqs;
    if (cudaStreamSynchronize(b->master) != cudaSuccess && rc == ERP_OK) rc = ERP_ECUDA;
    cudaEventDestroy(fork);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    for (auto &e : joins) cudaEventDestroy(e);
    return rc;
}

extern "C" erp_status erp_batch_packed(const erp_batch *b, int32_t *packed_instances) {
    if (!b || !packed_instances) return ERP_EINVAL;
    *packed_instances = b->packed_instances;
    return ERP_OK;
}

extern "C" erp_status erp_batch_spectral_tuning(const erp_batch *b, int32_t *chosen, int32_t *seqs, float *ms,
                                                int32_t cap, int32_t *count) {
    if (!b || cap < 0 || (cap > 0 && (!seqs || !ms))) return ERP_EINVAL;
    if (chosen) *chosen = b->spectral_seqs;
    const int k = std::min<int>(cap, (int)b->spec_tuning.size());
    for (int i = 0; i < k; ++i) {
        seqs[i] = b->spec_tuning[i].first;
        ms[i] = b->spec_tuning[i].second;
    }
    if (count) *count = (int32_t)b->spec_tuning.size();
    return ERP_OK;
}

// Whether an instance's step runs in the batch's packed launches: the FP32
// solve in its warp forms (bins 64..256 on both axes), with movable cells and
// nets, and at most 100,000 movable cells (ERP_BATCH_PACK_MAX_CELLS sets the
// cap).  Larger grids, whose kernels are long enough for their launches not to
// matter, and the tensor-core solve keep a graph branch each; so do the larger
// instances, which then run beside the packed chain instead of holding up each
// of its stages (whole runs of the 64-design mix: no cap 501k jobs/h, caps of
// 100k / 50k / 25k / 12k cells 570k / 567k / 556k / 531k, a branch for every
// instance 507k).
static bool packable(const Ctx &c) {
    static const long long max_cells = [] {
        const char *v = getenv("ERP_BATCH_PACK_MAX_CELLS");
        return v ? atoll(v) : 100000LL;
    }();
    return !c.gemm && c.m >= 64 && c.m <= 256 && c.n >= 64 && c.n <= 256 && c.NM > 0 && c.E > 0 &&
           (long long)c.NM <= max_cells;
}

// The packed launches of one step over xs, in stage order, and their argument
// tables (to be uploaded before the launches run).
static void pack_plan(const std::vector<Ctx *> &xs, PackedArena &ar, std::vector<PackedLaunch> &ls) {
    for (PackKind k : {PK_WA, PK_GATHER, PK_SCATTER}) packed_place_stage(k, xs, ar, ls);
    std::vector<SpectralJob> jobs;
    for (Ctx *c : xs) jobs.push_back(SpectralJob{plan_of(*c), spectral_args(*c, true, false, false)});
    for (PackKind k : {PK_ROWS_DCT_W, PK_COLS_W, PK_ROWS_INV_W}) packed_spectral_stage(k, jobs, ar, ls);
    for (PackKind k : {PK_FORCE, PK_GRAD, PK_UPDATE, PK_SCHED}) packed_place_stage(k, xs, ar, ls);
}

static void pack_launch(const std::vector<PackedLaunch> &ls, const void *dev_arena, cudaStream_t s) {
    const unsigned char *dev = static_cast<const unsigned char *>(dev_arena);
    for (const PackedLaunch &l : ls)
        if (!packed_place_launch(l, dev, s)) packed_spectral_launch(l, dev, s);
}

// The packed launches of one step over xs, with their argument tables uploaded
// to the batch's device buffer in the master stream's order: the graph launches
// already queued read the old tables, the ones after this call the new ones, and
// the host does not wait for the queued work.
static erp_status batch_pack_plan(erp_batch *b, const std::vector<Ctx *> &xs, std::vector<PackedLaunch> &ls) {
    PackedArena ar;
    pack_plan(xs, ar, ls);
    if (ar.host.size() > b->pack_cap) {
        if (b->pack_dev) cudaFreeAsync(b->pack_dev, b->master);
        b->pack_dev = nullptr;
        b->pack_cap = 0;
        if (cudaMallocAsync(&b->pack_dev, ar.host.size(), b->master) != cudaSuccess)
            return batch_fail(b, ERP_ENOMEM, "packed argument tables: allocation failed");
        b->pack_cap = ar.host.size();
    }
    if (!ar.host.empty() && cudaMemcpyAsync(b->pack_dev, ar.host.data(), ar.host.size(), cudaMemcpyHostToDevice,
                                            b->master) != cudaSuccess)
        return batch_fail(b, ERP_ECUDA, "packed argument tables: upload failed");
    return ERP_OK;
}

// (Re)capture the batch graph over the instances whose active flag is set:
// the packable ones as one chain of packed launches (one per stage and kernel
// variant), every other one as a branch of its own kernels.
static erp_status batch_graph(erp_batch *b, const std::vector<char> &active) {
    if (b->graph_ready) {
        cudaGraphExecDestroy(b->graph);
        b->graph_ready = false;
    }
    if (b->sort_ready) {
        cudaGraphExecDestroy(b->sort_graph);
        b->sort_ready = false;
    }
    std::vector<Ctx *> xs;
    std::vector<char> branch(b->ctx.size(), 0);
    for (size_t i = 0; i < b->ctx.size(); ++i) {
        if (!active[i]) continue;
        Ctx &c = b->ctx[i]->c;
        if (b->packed && packable(c)) xs.push_back(&c);
        else branch[i] = 1;
    }
    if (xs.size() < (size_t)kPackMin) {   // too few to pay for the table lookups: branches
        for (size_t i = 0; i < b->ctx.size(); ++i)
            if (active[i]) branch[i] = 1;
        xs.clear();
    }
    std::vector<PackedLaunch> ls;
    if (!xs.empty()) {
        erp_status ps = batch_pack_plan(b, xs, ls);
        if (ps != ERP_OK) return ps;
    }
    cudaEvent_t fork;
    if (cudaEventCreateWithFlags(&fork, cudaEventDisableTiming) != cudaSuccess)
        return batch_fail(b, ERP_ECUDA, "cudaEventCreate failed");
    std::vector<cudaEvent_t> joins(b->ctx.size());
    for (auto &e : joins) cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    cudaGraph_t g;
    cudaError_t e = cudaStreamBeginCapture(b->master, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        cudaEventRecord(fork, b->master);
        for (size_t i = 0; i < b->ctx.size(); ++i) {
            if (!branch[i]) continue;
            Ctx &c = b->ctx[i]->c;
            cudaStreamWaitEvent(c.stream, fork, 0);
            enqueue_step_kernels(c);
            cudaEventRecord(joins[i], c.stream);
        }
        pack_launch(ls, b->pack_dev, b->master);
        for (size_t i = 0; i < b->ctx.size(); ++i)
            if (branch[i]) cudaStreamWaitEvent(b->master, joins[i], 0);
        e = cudaStreamEndCapture(b->master, &g);
    }
    if (e == cudaSuccess) {
        b->graph_kernels = count_kernel_nodes(g);
        e = cudaGraphInstantiate(&b->graph, g, 0);
        cudaGraphDestroy(g);
    }
    if (e == cudaSuccess) b->graph_ready = true;
    // The scatter-order refreshes of the same instances, each on its own stream:
    // four operations per instance that would otherwise run one after another on
    // the master stream before every chunk of steps.
    if (e == cudaSuccess) e = cudaStreamBeginCapture(b->master, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        cudaEventRecord(fork, b->master);
        for (size_t i = 0; i < b->ctx.size(); ++i) {
            if (!active[i]) continue;
            Ctx &c = b->ctx[i]->c;
            cudaStreamWaitEvent(c.stream, fork, 0);
            launch_scatter_order(c, c.stream);
            cudaEventRecord(joins[i], c.stream);
            cudaStreamWaitEvent(b->master, joins[i], 0);
        }
        e = cudaStreamEndCapture(b->master, &g);
        if (e == cudaSuccess) {
            e = cudaGraphInstantiate(&b->sort_graph, g, 0);
            cudaGraphDestroy(g);
        }
    }
    if (e == cudaSuccess) b->sort_ready = true;
    cudaEventDestroy(fork);
    for (auto &j : joins) cudaEventDestroy(j);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return batch_fail(b, ERP_ECUDA, std::string("batch graph: ") + cudaGetErrorString(e));
    }
    return ERP_OK;
}

// Every instance's state to its host copy: all copies issued, then one wait per
// stream.  Status bits are left to state_status.
static erp_status pull_states(erp_batch *b) {
    for (auto *x : b->ctx)
        if (cudaMemcpyAsync(x->c.h_st, x->c.st, sizeof(DevState), cudaMemcpyDeviceToHost, x->c.stream) !=
            cudaSuccess)
            return batch_fail(b, ERP_ECUDA, "reading instance state failed");
    for (auto *x : b->ctx)
        if (cudaStreamSynchronize(x->c.stream) != cudaSuccess)
            return batch_fail(b, ERP_ECUDA, "reading instance state failed");
    return ERP_OK;
}

extern "C" erp_status erp_batch_run(erp_batch *b, int32_t max_iterations, float stop_overflow,
                                    int32_t *iterations, erp_step_stats *last) {
    HostRange range_("erp_batch_run");
    if (!b || max_iterations < 0) return ERP_EINVAL;
    b->err.clear();
    if (cudaSetDevice(b->device) != cudaSuccess) return batch_fail(b, ERP_ECUDA, "cudaSetDevice failed");
    const int K = (int)b->ctx.size();
    std::vector<int> start(K);
    // every instance's state copied at once, then one wait per stream (not a
    // wait per copy: four per instance and run, 256 on 64 designs)
    erp_status ps = pull_states(b);
    if (ps != ERP_OK) return ps;
    for (int i = 0; i < K; ++i) {
        Ctx &c = b->ctx[i]->c;
        erp_status si = state_status(c);
        if (si != ERP_OK) return batch_fail(b, si, "instance " + std::to_string(i) + ": " + c.err);
        start[i] = c.h_st->iteration;
        // arm: retire at overflow or after max_iterations more steps
        c.h_st->stop_overflow = stop_overflow > 0 ? stop_overflow : 0.0f;
        c.h_st->stop_iter = start[i] + max_iterations;
        c.h_st->done = max_iterations == 0 ? 1 : 0;
        if (c.map_dirty) {
            cudaMemsetAsync(c.dmap, 0, sizeof(unsigned long long) * (size_t)c.m * c.n, c.stream);
            c.map_dirty = false;
        }
        if (cudaMemcpyAsync(c.st, c.h_st, sizeof(DevState), cudaMemcpyHostToDevice, c.stream) != cudaSuccess)
            return batch_fail(b, ERP_ECUDA, "arming instance failed");
    }
    for (int i = 0; i < K; ++i)
        if (cudaStreamSynchronize(b->ctx[i]->c.stream) != cudaSuccess)
            return batch_fail(b, ERP_ECUDA, "arming instance failed");
    // Launch the graph in chunks; the retire flags of chunk k are read while
    // chunk k+1 runs (double-buffered), and when instances have retired the
    // graph is captured again over the remaining ones.
    std::vector<char> active(K, max_iterations > 0 ? 1 : 0);
    int n_active = max_iterations > 0 ? K : 0;
    erp_status s = n_active ? batch_graph(b, active) : ERP_OK;
    if (s != ERP_OK) return s;
    const int chunk = 16;
    int launched = 0;
    cudaEvent_t ev[2];
    cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming);
    cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming);
    int pending = -1;
    erp_status rs = ERP_OK;
    while (n_active > 0 && launched < max_iterations) {
        const int k = std::min(chunk, max_iterations - launched);
        // every active instance's scatter order when one of them is due (an early
        // refresh changes no result, only which block adds a contribution)
        bool due = false;
        for (int i = 0; i < K; ++i) {
            if (!active[i]) continue;
            Ctx &c = b->ctx[i]->c;
            c.sort_age += k;
            due = due || c.sort_age >= kSortEvery;
        }
        if (due) {
            if (cudaGraphLaunch(b->sort_graph, b->master) != cudaSuccess) {
                rs = batch_fail(b, ERP_ECUDA, "scatter-order graph launch failed");
                break;
            }
            for (int i = 0; i < K; ++i)
                if (active[i]) b->ctx[i]->c.sort_age = 0;
        }
        for (int i = 0; i < k && rs == ERP_OK; ++i)
            if (cudaGraphLaunch(b->graph, b->master) != cudaSuccess)
                rs = batch_fail(b, ERP_ECUDA, "batch graph launch failed");
        if (rs != ERP_OK) break;
        launched += k;
        const int buf = (launched / chunk) & 1;
        launch_gather_done(b->d_states, K, b->d_done + buf * K, b->master);
        cudaMemcpyAsync(b->h_done + buf * K, b->d_done + buf * K, sizeof(int32_t) * K, cudaMemcpyDeviceToHost,
                        b->master);
        cudaEventRecord(ev[buf], b->master);
        if (pending >= 0) {
            if (cudaEventSynchronize(ev[pending]) != cudaSuccess) {
                rs = batch_fail(b, ERP_ECUDA, std::string("batch run: ") + cudaGetErrorString(cudaGetLastError()));
                break;
            }
            int now = 0;
            for (int i = 0; i < K; ++i) now += active[i] && !b->h_done[pending * K + i];
            if (now < n_active) {   // some retired: drop their branches
                for (int i = 0; i < K; ++i)
                    if (b->h_done[pending * K + i]) active[i] = 0;
                n_active = now;
                // captured while the chunk in flight runs on: its graphs are freed when
                // it completes, and the new tables reach the device in stream order
                if (n_active > 0) {
                    rs = batch_graph(b, active);
                    if (rs != ERP_OK) break;
                }
            }
        }
        pending = buf;
    }
    cudaStreamSynchronize(b->master);
    cudaEventDestroy(ev[0]);
    cudaEventDestroy(ev[1]);
    if (rs != ERP_OK) return rs;
    erp_status rc = pull_states(b);
    if (rc != ERP_OK) return rc;
    for (int i = 0; i < K; ++i) {
        Ctx &c = b->ctx[i]->c;
        erp_status si = state_status(c);
        if (iterations) iterations[i] = c.h_st->iteration - start[i];
        if (last) last[i] = c.h_st->last;
        // disarm
        c.h_st->stop_overflow = 0.0f;
        c.h_st->stop_iter = 0;
        c.h_st->done = 0;
        cudaMemcpyAsync(c.st, c.h_st, sizeof(DevState), cudaMemcpyHostToDevice, c.stream);
        if (si != ERP_OK && rc == ERP_OK) {
            rc = si;
            b->err = "instance " + std::to_string(i) + ": " + c.err;
        }
    }
    for (auto *x : b->ctx) cudaStreamSynchronize(x->c.stream);
    return rc;
}

extern "C" erp_ctx *erp_batch_context(erp_batch *b, int32_t i) {
    if (!b || i < 0 || i >= (int)b->ctx.size()) return nullptr;
    return b->ctx[i];
}

extern "C" int32_t erp_batch_size(const erp_batch *b) { return b ? (int32_t)b->ctx.size() : 0; }

extern "C" const char *erp_batch_last_error(const erp_batch *b) {
    return b ? b->err.c_str() : g_create_err.c_str();
}

extern "C" void erp_batch_destroy(erp_batch *b) {
    if (!b) return;
    cudaSetDevice(b->device);
    if (b->master) cudaStreamSynchronize(b->master);
    if (b->graph_ready) cudaGraphExecDestroy(b->graph);
    if (b->sort_ready) cudaGraphExecDestroy(b->sort_graph);
    for (auto *c : b->ctx) erp_destroy(c);
    if (b->master) cudaStreamDestroy(b->master);
    if (b->d_states) cudaFree(b->d_states);
    if (b->d_done) cudaFree(b->d_done);
    if (b->h_done) cudaFreeHost(b->h_done);
    if (b->pack_dev) cudaFree(b->pack_dev);
    delete b;
}

// ---------------------------------------------------------------------------
// serving: continuous batching
extern "C" erp_status erp_estimate_footprint(const erp_design *d, const erp_params *pp, int64_t *bytes) {
    if (!d || !bytes) return ERP_EINVAL;
    int m = pp && pp->num_bins_x ? pp->num_bins_x : 512, n = pp && pp->num_bins_y ? pp->num_bins_y : 512;
    const int64_t N = d->num_nodes, NM = d->num_movable, P = d->num_pins, E = d->num_nets;
    const int64_t mn = (int64_t)m * n;
    int64_t movable_pins = 0;
    if (d->inst_pin_ptr) movable_pins = d->inst_pin_ptr[NM];
    auto al = [](int64_t v) { return (v + 511) & ~int64_t(511); };   // allocation granularity
    int64_t b = 16 * al(4 * (N + 4));
    b += al(4 * P) + 2 * al(8 * P) + al(4 * (E + 1)) + al(4 * E) + al(4 * (NM + 1)) + al(4 * movable_pins);
    b += al(8 * mn) + 9 * al(4 * mn) + al(8 * (int64_t)kMaxPartials) + al(sizeof(DevState));
    b += 5 * al(4 * (int64_t)NM) + al(16 * (int64_t)NM) + 2 * al(4 * (int64_t)scatter_tiles(m, n));   // scatter order
    b += al(4 * (NM + 4)) + al(8 * (NM + 4));   // its inverse, the density gradient in that order
    b += al(8 * (m / 2)) + al(8 * (n / 2)) + al(8 * m) + al(8 * n) + al(4 * m) + al(4 * n);
    if (pp && pp->precision != ERP_PREC_FP32) {   // tensor-core plan: 4 transforms per axis + 7 map buffers
        const int64_t es = pp->precision == ERP_PREC_TF32_GEMM ? 4 : 4;   // fp32, or bf16 hi + lo
        b += es * (2 * (int64_t)m * m + 2 * (int64_t)n * n + (int64_t)m * m + (int64_t)n * n) + es * 7 * mn;
    }
    *bytes = b;
    return ERP_OK;
}

namespace {
struct OwnedDesign {
    std::vector<float> x, y, w, h, npins, pox, poy;
    std::vector<int32_t> pin_inst, net_ptr, net_pins, inst_ptr, inst_pins;
    erp_design d;
    explicit OwnedDesign(const erp_design &s) {
        d = s;
        const size_t N = s.num_nodes, P = s.num_pins, E = s.num_nets;
        auto cpf = [](std::vector<float> &v, const float *p, size_t k) { v.assign(p, p + (p ? k : 0)); };
        auto cpi = [](std::vector<int32_t> &v, const int32_t *p, size_t k) { v.assign(p, p + (p ? k : 0)); };
        cpf(x, s.x, N); cpf(y, s.y, N); cpf(w, s.w, N); cpf(h, s.h, N); cpf(npins, s.num_pins_f, N);
        cpf(pox, s.pin_ox, P); cpf(poy, s.pin_oy, P);
        cpi(pin_inst, s.pin_inst, P);
        cpi(net_ptr, s.net_ptr, E + 1);
        cpi(net_pins, s.net_pins, s.net_ptr ? (size_t)s.net_ptr[E] : 0);
        cpi(inst_ptr, s.inst_pin_ptr, N + 1);
        cpi(inst_pins, s.inst_pins, s.inst_pin_ptr ? (size_t)s.inst_pin_ptr[N] : 0);
        d.x = x.data(); d.y = y.data(); d.w = w.data(); d.h = h.data(); d.num_pins_f = npins.data();
        d.pin_ox = pox.data(); d.pin_oy = poy.data(); d.pin_inst = pin_inst.data();
        d.net_ptr = net_ptr.data(); d.net_pins = net_pins.data();
        d.inst_pin_ptr = inst_ptr.data(); d.inst_pins = inst_pins.data();
    }
};
struct Job {
    int64_t id = 0;
    std::unique_ptr<OwnedDesign> des;
    erp_params prm;
    double submit = 0, admit = 0;
    int64_t footprint = 0;
    erp_ctx *ctx = nullptr;
    int start_iter = 0;
    erp_status prep = ERP_OK;   // outcome of the admission worker's set-up
    int form = -1;              // how its last round ran: -1 none yet, 0 its own branch, 1 packed
    cudaEvent_t ev = nullptr;   // marks its own stream's work when it moves into the packed chain
    bool cancel = false;        // cancelled while its admission worker set it up
    Job() = default;
    Job(const Job &) = delete;
    Job &operator=(const Job &) = delete;
    ~Job() {
        if (ev) cudaEventDestroy(ev);
    }
};
}  // namespace

struct erp_server {
    erp_server_params p;
    std::vector<std::unique_ptr<Job>> queue;   // FIFO (front = index qhead)
    size_t qhead = 0;
    std::vector<std::unique_ptr<Job>> active;
    std::vector<erp_job_result> finished;
    std::vector<std::pair<int64_t, std::pair<std::vector<float>, std::vector<float>>>> pos;
    int64_t used = 0;
    cudaStream_t master = nullptr;
    std::vector<cudaEvent_t> job_ev;   // one per slot
    cudaEvent_t round_ev[2] = {nullptr, nullptr};
    bool round_pending[2] = {false, false};
    std::vector<int64_t> round_ids[2];
    uint64_t round_seq[2] = {0, 0};
    uint64_t rounds_launched = 0;
    std::vector<std::pair<uint64_t, std::unique_ptr<Job>>> grave;   // (last round that references it, job)
    int round = 0;
    // Packed rounds (ERP_SERVER_FORM=packed): the active jobs that batches would
    // pack run each round as one graph of packed launches (one per stage and
    // kernel variant), built for the set of jobs it covers and rebuilt when that
    // set changes.  One slot per round parity: round r reuses the slot of round
    // r-2, which has completed.
    struct PackedSlot {
        std::vector<int64_t> ids;          // the jobs the graph was built for
        cudaGraphExec_t exec = nullptr;
        void *dev = nullptr;               // argument tables
        size_t cap = 0;
        unsigned char *staging = nullptr;  // pinned copy of the tables for the upload
        size_t staging_cap = 0;
    };
    bool packed = true;
    PackedSlot pk[2];
    cudaStream_t pstream = nullptr;
    cudaEvent_t pk_ev[2] = {nullptr, nullptr};
    cudaEvent_t pk_tail = nullptr;     // the packed stream's work before this round's chain
    DevState **d_states = nullptr;       // [2][max_active]
    int32_t *d_done = nullptr, *h_done = nullptr;
    std::chrono::steady_clock::time_point t0;
    std::string err;
    // Admission workers: a job admitted by the pump (slot and budget reserved)
    // is set up on a worker thread -- host preparation, uploads on the job's own
    // stream, graph capture -- and handed back through `ready`; retired
    // contexts are destroyed there as well, so the pump thread only launches,
    // retires and admits.
    std::vector<std::unique_ptr<Job>> preparing;   // owned here while a worker sets it up
    std::mutex mu;
    std::condition_variable cv, ready_cv;
    std::deque<Job *> todo;                        // guarded by mu
    std::deque<erp_ctx *> to_destroy;              // guarded by mu
    std::vector<Job *> ready;                      // guarded by mu
    std::vector<std::thread> workers;
    bool stop = false;                             // guarded by mu
    double now() const {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
};

static void server_worker(erp_server *sv) {
    cudaSetDevice(sv->p.device);
    for (;;) {
        Job *j = nullptr;
        erp_ctx *dead = nullptr;
        {
            std::unique_lock<std::mutex> lk(sv->mu);
            sv->cv.wait(lk, [&] { return sv->stop || !sv->todo.empty() || !sv->to_destroy.empty(); });
            if (!sv->to_destroy.empty()) {
                dead = sv->to_destroy.front();
                sv->to_destroy.pop_front();
            } else if (!sv->todo.empty()) {
                j = sv->todo.front();
                sv->todo.pop_front();
            } else {
                return;   // stop, nothing left
            }
        }
        if (dead) {
            erp_destroy(dead);
            continue;
        }
        erp_status s = erp_create(&j->des->d, &j->prm, &j->ctx);
        if (s == ERP_OK) {
            Ctx &c = j->ctx->c;
            // jobs that share the GPU take the batch's scatter shape: fewer, fuller
            // blocks (the shape the batch calibration keeps on the 64-design mix)
            if (sv->p.max_active > 1) c.scatter_cells = 2048;
            c.h_st->stop_overflow = sv->p.stop_overflow > 0 ? sv->p.stop_overflow : 0.0f;
            c.h_st->stop_iter = sv->p.max_iterations;
            c.h_st->done = 0;
            if (cudaMemcpyAsync(c.st, c.h_st, sizeof(DevState), cudaMemcpyHostToDevice, c.stream) != cudaSuccess)
                s = ERP_ECUDA;
            if (s == ERP_OK) s = ensure_graph(c);
        } else {
            j->ctx = nullptr;
        }
        j->prep = s;
        j->des.reset();   // the context holds its own copy
        {
            std::lock_guard<std::mutex> lk(sv->mu);
            sv->ready.push_back(j);
        }
        sv->ready_cv.notify_one();
    }
}

extern "C" erp_status erp_server_create(const erp_server_params *p, erp_server **out) {
    g_create_err.clear();
    if (!p || !out || p->max_active < 1 || p->hbm_budget_bytes <= 0 || p->max_iterations < 1 || p->chunk < 1) {
        g_create_err = "invalid server parameters";
        return ERP_EINVAL;
    }
    erp_status s = check_device(p->device, g_create_err);
    if (s != ERP_OK) return s;
    erp_server *sv = new (std::nothrow) erp_server();
    if (!sv) return ERP_ENOMEM;
    sv->p = *p;
    sv->t0 = std::chrono::steady_clock::now();
    const int K = p->max_active;
    bool ok = cudaStreamCreateWithFlags(&sv->master, cudaStreamNonBlocking) == cudaSuccess &&
              cudaMalloc(&sv->d_states, sizeof(DevState *) * 2 * K) == cudaSuccess &&
              cudaMalloc(&sv->d_done, sizeof(int32_t) * 2 * K) == cudaSuccess &&
              cudaMallocHost(&sv->h_done, sizeof(int32_t) * 2 * K) == cudaSuccess &&
              cudaEventCreateWithFlags(&sv->round_ev[0], cudaEventDisableTiming) == cudaSuccess &&
              cudaEventCreateWithFlags(&sv->round_ev[1], cudaEventDisableTiming) == cudaSuccess &&
              cudaStreamCreateWithFlags(&sv->pstream, cudaStreamNonBlocking) == cudaSuccess &&
              cudaEventCreateWithFlags(&sv->pk_ev[0], cudaEventDisableTiming) == cudaSuccess &&
              cudaEventCreateWithFlags(&sv->pk_ev[1], cudaEventDisableTiming) == cudaSuccess &&
              cudaEventCreateWithFlags(&sv->pk_tail, cudaEventDisableTiming) == cudaSuccess;
    {   // packed rounds are opt-in: on the 2,000-job stream they took p50 latency from 0.33
        // to 0.26 s but p99 from 0.63 to 0.79 s (a round's stages wait for its largest job)
        const char *form = getenv("ERP_SERVER_FORM");
        sv->packed = K > 1 && form && strcmp(form, "packed") == 0;
    }
    sv->job_ev.resize(K, nullptr);
    for (int i = 0; ok && i < K; ++i)
        ok = cudaEventCreateWithFlags(&sv->job_ev[i], cudaEventDisableTiming) == cudaSuccess;
    if (!ok) {
        erp_server_destroy(sv);
        g_create_err = "server allocation failed";
        return ERP_ENOMEM;
    }
    const unsigned hw = std::thread::hardware_concurrency();
    const int nw = std::max(1, std::min({4, K, (int)(hw ? hw / 2 : 1)}));
    try {
        for (int i = 0; i < nw; ++i) sv->workers.emplace_back(server_worker, sv);
    } catch (...) {
        erp_server_destroy(sv);
        g_create_err = "cannot start admission workers";
        return ERP_ENOMEM;
    }
    *out = sv;
    return ERP_OK;
}

extern "C" erp_status erp_server_submit(erp_server *sv, int64_t job_id, const erp_design *d,
                                        const erp_params *prm) {
    if (!sv || !d) return ERP_EINVAL;
    auto j = std::make_unique<Job>();
    j->id = job_id;
    j->des = std::make_unique<OwnedDesign>(*d);
    memset(&j->prm, 0, sizeof j->prm);
    if (prm) j->prm = *prm;
    j->prm.stream = nullptr;
    j->prm.device = sv->p.device;
    erp_estimate_footprint(&j->des->d, &j->prm, &j->footprint);
    j->submit = sv->now();
    sv->queue.push_back(std::move(j));
    return ERP_OK;
}

// Record a finished job's result (stats, optionally positions); the context
// itself is destroyed later by server_bury.
static void server_record(erp_server *sv, Job &j, erp_status st) {
    erp_job_result r;
    memset(&r, 0, sizeof r);
    r.job_id = j.id;
    r.status = st;
    r.submit_s = j.submit;
    r.admit_s = j.admit;
    r.footprint_bytes = j.footprint;
    if (j.ctx) {
        Ctx &c = j.ctx->c;
        erp_status ps = pull_state(c);
        if (st == ERP_OK) r.status = ps;
        r.iterations = c.h_st->iteration - j.start_iter;
        r.last = c.h_st->last;
        if (sv->p.keep_positions) {
            std::vector<float> x(c.N), y(c.N);
            cudaMemcpyAsync(x.data(), c.x, sizeof(float) * c.N, cudaMemcpyDeviceToHost, c.stream);
            cudaMemcpyAsync(y.data(), c.y, sizeof(float) * c.N, cudaMemcpyDeviceToHost, c.stream);
            cudaStreamSynchronize(c.stream);
            sv->pos.emplace_back(j.id, std::make_pair(std::move(x), std::move(y)));
        }
    }
    r.finish_s = sv->now();
    sv->finished.push_back(r);
}

// The packed graph of one round over xs (the slot's, rebuilt if the set of jobs
// changed): argument tables staged in pinned memory and copied on the packed
// stream, then one step of packed launches captured from that stream.
static erp_status server_pack_slot(erp_server *sv, int buf, const std::vector<Ctx *> &xs,
                                   const std::vector<int64_t> &ids) {
    erp_server::PackedSlot &sl = sv->pk[buf];
    if (sl.exec && sl.ids == ids) return ERP_OK;
    PackedArena ar;
    std::vector<PackedLaunch> ls;
    pack_plan(xs, ar, ls);
    const size_t bytes = ar.host.size();
    if (bytes > sl.cap) {
        if (sl.dev) cudaFree(sl.dev);
        sl.dev = nullptr;
        sl.cap = 0;
        if (cudaMalloc(&sl.dev, bytes) != cudaSuccess) {
            sv->err = "packed argument tables: allocation failed";
            return ERP_ENOMEM;
        }
        sl.cap = bytes;
    }
    if (bytes > sl.staging_cap) {
        if (sl.staging) cudaFreeHost(sl.staging);
        sl.staging = nullptr;
        sl.staging_cap = 0;
        if (cudaMallocHost((void **)&sl.staging, bytes) != cudaSuccess) {
            sv->err = "packed argument tables: allocation failed";
            return ERP_ENOMEM;
        }
        sl.staging_cap = bytes;
    }
    if (bytes) {
        memcpy(sl.staging, ar.host.data(), bytes);
        if (cudaMemcpyAsync(sl.dev, sl.staging, bytes, cudaMemcpyHostToDevice, sv->pstream) != cudaSuccess) {
            sv->err = "packed argument tables: upload failed";
            return ERP_ECUDA;
        }
    }
    if (sl.exec) {
        cudaGraphExecDestroy(sl.exec);
        sl.exec = nullptr;
    }
    sl.ids.clear();
    cudaGraph_t g;
    cudaError_t e = cudaStreamBeginCapture(sv->pstream, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        pack_launch(ls, sl.dev, sv->pstream);
        e = cudaStreamEndCapture(sv->pstream, &g);
    }
    if (e == cudaSuccess) {
        e = cudaGraphInstantiate(&sl.exec, g, 0);
        cudaGraphDestroy(g);
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        sv->err = std::string("packed round graph: ") + cudaGetErrorString(e);
        return ERP_ECUDA;
    }
    sl.ids = ids;
    return ERP_OK;
}

// One scheduling round.  The active jobs that batches would pack (four or more)
// run `chunk` launches of one packed graph on the packed stream; every other
// job launches its own captured step graph `chunk` times on its own stream (so
// admissions and retirements never touch the other jobs' work).  Then the
// round's retire flags are gathered behind an event.  A pump launches round r first and only then reads the flags of round
// r-1, so the GPU always has queued work while the host retires and admits.
// A job retired from round r-1's flags still ran round r (its kernels return
// at entry once retired) and round r's flag gather reads its state, so its
// context is destroyed only after round r has completed (the graveyard).
static erp_status server_launch_round(erp_server *sv, int buf) {
    const int K = (int)sv->active.size();
    std::vector<DevState *> sts(K);
    sv->round_ids[buf].clear();
    // the jobs a batch would pack run as one chain of packed launches
    std::vector<Ctx *> xs;
    std::vector<int64_t> ids;
    std::vector<char> in_pack(K, 0);
    if (sv->packed) {
        for (int i = 0; i < K; ++i)
            if (packable(sv->active[i]->ctx->c)) {
                xs.push_back(&sv->active[i]->ctx->c);
                ids.push_back(sv->active[i]->id);
                in_pack[i] = 1;
            }
        if ((int)xs.size() < kPackMin) {
            xs.clear();
            ids.clear();
            std::fill(in_pack.begin(), in_pack.end(), 0);
        }
    }
    // A job that changes form between rounds (packed <-> its own branch) has its
    // previous round's work on the other stream: the new one waits for it.  A
    // job's first round waits for its own stream too, where its admission worker
    // queued the copy that arms its scalars (stop rules, done flag).
    cudaEventRecord(sv->pk_tail, sv->pstream);
    if (!xs.empty()) {
        for (int i = 0; i < K; ++i) {
            if (!in_pack[i]) continue;
            Job &j = *sv->active[i];
            if (j.form != 1) {
                if (!j.ev && cudaEventCreateWithFlags(&j.ev, cudaEventDisableTiming) != cudaSuccess) {
                    sv->err = "cudaEventCreate failed";
                    return ERP_ECUDA;
                }
                cudaEventRecord(j.ev, j.ctx->c.stream);
                cudaStreamWaitEvent(sv->pstream, j.ev, 0);
            }
            j.form = 1;
        }
        for (Ctx *c : xs) refresh_scatter_order(*c, sv->p.chunk, sv->pstream);
        erp_status s = server_pack_slot(sv, buf, xs, ids);
        if (s != ERP_OK) return s;
        for (int k = 0; k < sv->p.chunk; ++k)
            if (cudaGraphLaunch(sv->pk[buf].exec, sv->pstream) != cudaSuccess) {
                sv->err = "packed round graph launch failed";
                return ERP_ECUDA;
            }
        cudaEventRecord(sv->pk_ev[buf], sv->pstream);
        cudaStreamWaitEvent(sv->master, sv->pk_ev[buf], 0);
    }
    for (int i = 0; i < K; ++i) {
        Ctx &c = sv->active[i]->ctx->c;
        if (in_pack[i]) {
            sts[i] = c.st;
            sv->round_ids[buf].push_back(sv->active[i]->id);
            continue;
        }
        if (sv->active[i]->form == 1) cudaStreamWaitEvent(c.stream, sv->pk_tail, 0);
        sv->active[i]->form = 0;
        erp_status s = ensure_graph(c);
        if (s != ERP_OK) {
            sv->err = c.err;
            return s;
        }
        refresh_scatter_order(c, sv->p.chunk, c.stream);
        for (int k = 0; k < sv->p.chunk; ++k)
            if (cudaGraphLaunch(c.graph, c.stream) != cudaSuccess) {
                sv->err = "job graph launch failed";
                return ERP_ECUDA;
            }
        cudaEventRecord(sv->job_ev[i], c.stream);
        cudaStreamWaitEvent(sv->master, sv->job_ev[i], 0);
        sts[i] = c.st;
        sv->round_ids[buf].push_back(sv->active[i]->id);
    }
    const int off = buf * sv->p.max_active;
    cudaMemcpyAsync(sv->d_states + off, sts.data(), sizeof(DevState *) * K, cudaMemcpyHostToDevice, sv->master);
    launch_gather_done(sv->d_states + off, K, sv->d_done + off, sv->master);
    cudaMemcpyAsync(sv->h_done + off, sv->d_done + off, sizeof(int32_t) * K, cudaMemcpyDeviceToHost, sv->master);
    cudaEventRecord(sv->round_ev[buf], sv->master);
    sv->round_pending[buf] = true;
    sv->round_seq[buf] = ++sv->rounds_launched;
    return ERP_OK;
}

static void server_bury(erp_server *sv, uint64_t completed_round) {
    std::vector<std::pair<uint64_t, std::unique_ptr<Job>>> keep;
    int n = 0;
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        for (auto &g : sv->grave) {
            if (g.first <= completed_round) {
                sv->to_destroy.push_back(g.second->ctx);   // freed on a worker (stream-ordered)
                g.second->ctx = nullptr;
                sv->used -= g.second->footprint;
                ++n;
            } else {
                keep.push_back(std::move(g));
            }
        }
    }
    sv->grave.swap(keep);
    if (n) sv->cv.notify_all();
}

extern "C" erp_status erp_server_pump(erp_server *sv, int32_t *active_out, int32_t *queued_out) {
    HostRange range_("erp_server_pump");
    if (!sv) return ERP_EINVAL;
    sv->err.clear();
    if (cudaSetDevice(sv->p.device) != cudaSuccess) return ERP_ECUDA;
    const int cur = sv->round, prev = sv->round ^ 1;
    // 1. launch this round for the active jobs
    const bool launched = !sv->active.empty();
    if (launched) {
        erp_status s = server_launch_round(sv, cur);
        if (s != ERP_OK) return s;
    }
    // 2. read the previous round's flags; retire (record results) the done jobs
    if (sv->round_pending[prev]) {
        if (cudaEventSynchronize(sv->round_ev[prev]) != cudaSuccess) {
            sv->err = std::string("server round: ") + cudaGetErrorString(cudaGetLastError());
            return ERP_ECUDA;
        }
        sv->round_pending[prev] = false;
        server_bury(sv, sv->round_seq[prev]);   // contexts retired before round prev
        const auto &ids = sv->round_ids[prev];
        std::vector<int64_t> done;
        for (size_t i = 0; i < ids.size(); ++i)
            if (sv->h_done[prev * sv->p.max_active + i]) done.push_back(ids[i]);
        if (!done.empty()) {
            std::vector<std::unique_ptr<Job>> keep;
            const uint64_t last_ref = launched ? sv->round_seq[cur] : sv->round_seq[prev];
            for (auto &j : sv->active) {
                if (std::find(done.begin(), done.end(), j->id) != done.end()) {
                    server_record(sv, *j, ERP_OK);
                    sv->grave.emplace_back(last_ref, std::move(j));
                } else {
                    keep.push_back(std::move(j));
                }
            }
            sv->active.swap(keep);
        }
    }
    if (!launched && !sv->round_pending[cur] && !sv->round_pending[prev])
        server_bury(sv, sv->rounds_launched);   // idle: everything launched has completed
    // 3. jobs the admission workers have finished setting up join the next round
    //    (when nothing runs, wait briefly for one instead of spinning)
    std::vector<Job *> got;
    {
        std::unique_lock<std::mutex> lk(sv->mu);
        if (sv->ready.empty() && sv->active.empty() && !sv->preparing.empty() && !sv->round_pending[0] &&
            !sv->round_pending[1])
            sv->ready_cv.wait_for(lk, std::chrono::milliseconds(2), [&] { return !sv->ready.empty(); });
        got.swap(sv->ready);
    }
    for (Job *jr : got) {
        auto it = std::find_if(sv->preparing.begin(), sv->preparing.end(),
                               [&](const std::unique_ptr<Job> &p) { return p.get() == jr; });
        std::unique_ptr<Job> jp = std::move(*it);
        sv->preparing.erase(it);
        if (jp->prep != ERP_OK || jp->cancel) {
            server_record(sv, *jp, jp->prep != ERP_OK ? jp->prep : ERP_ECANCELED);
            if (jp->ctx) {
                std::lock_guard<std::mutex> lk(sv->mu);
                sv->to_destroy.push_back(jp->ctx);
                jp->ctx = nullptr;
            }
            sv->cv.notify_one();
            sv->used -= jp->footprint;
            continue;
        }
        jp->start_iter = 0;
        sv->active.push_back(std::move(jp));
    }
    // 4. admission: FIFO while the job fits the budget and a slot is free; the
    //    set-up itself runs on a worker
    int admitted = 0;
    while (sv->qhead < sv->queue.size() && (int)(sv->active.size() + sv->preparing.size()) < sv->p.max_active) {
        Job &j = *sv->queue[sv->qhead];
        if (j.footprint > sv->p.hbm_budget_bytes) {   // can never fit
            std::unique_ptr<Job> jp = std::move(sv->queue[sv->qhead++]);
            server_record(sv, *jp, ERP_ENOMEM);
            continue;
        }
        if (sv->used + j.footprint > sv->p.hbm_budget_bytes) break;
        std::unique_ptr<Job> jp = std::move(sv->queue[sv->qhead++]);
        jp->admit = sv->now();
        sv->used += jp->footprint;
        {
            std::lock_guard<std::mutex> lk(sv->mu);
            sv->todo.push_back(jp.get());
        }
        sv->preparing.push_back(std::move(jp));
        ++admitted;
    }
    if (admitted) sv->cv.notify_all();
    if (sv->qhead > 1024 && sv->qhead * 2 > sv->queue.size()) {   // compact the FIFO
        sv->queue.erase(sv->queue.begin(), sv->queue.begin() + sv->qhead);
        sv->qhead = 0;
    }
    if (launched) sv->round ^= 1;
    if (active_out) *active_out = (int32_t)(sv->active.size() + sv->preparing.size());
    if (queued_out) *queued_out = (int32_t)(sv->queue.size() - sv->qhead);
    return ERP_OK;
}

extern "C" erp_status erp_server_cancel(erp_server *sv, int64_t job_id) {
    if (!sv) return ERP_EINVAL;
    sv->err.clear();
    if (cudaSetDevice(sv->p.device) != cudaSuccess) return ERP_ECUDA;
    for (size_t k = sv->qhead; k < sv->queue.size(); ++k)   // queued: its budget was never taken
        if (sv->queue[k]->id == job_id) {
            std::unique_ptr<Job> jp = std::move(sv->queue[k]);
            sv->queue.erase(sv->queue.begin() + (std::ptrdiff_t)k);
            server_record(sv, *jp, ERP_ECANCELED);
            return ERP_OK;
        }
    for (size_t k = 0; k < sv->active.size(); ++k)   // running: retired like a finished job
        if (sv->active[k]->id == job_id) {
            std::unique_ptr<Job> jp = std::move(sv->active[k]);
            sv->active.erase(sv->active.begin() + (std::ptrdiff_t)k);
            if (jp->form == 1) {   // its state is read on its own stream, after the packed work queued
                cudaEventRecord(sv->pk_tail, sv->pstream);
                cudaStreamWaitEvent(jp->ctx->c.stream, sv->pk_tail, 0);
            }
            server_record(sv, *jp, ERP_ECANCELED);
            // the rounds launched so far may still run its kernels: its context goes
            // (and its budget returns) once the last of them has completed
            sv->grave.emplace_back(sv->rounds_launched, std::move(jp));
            return ERP_OK;
        }
    for (auto &jp : sv->preparing)   // being set up: retired when its worker is done
        if (jp->id == job_id) {
            jp->cancel = true;
            return ERP_OK;
        }
    sv->err = "no queued or running job with id " + std::to_string(job_id);
    return ERP_EINVAL;
}

extern "C" erp_status erp_server_poll(erp_server *sv, erp_job_result *out, int32_t cap, int32_t *count) {
    if (!sv || !count || (cap > 0 && !out)) return ERP_EINVAL;
    const int k = std::min<int>(cap, (int)sv->finished.size());
    for (int i = 0; i < k; ++i) out[i] = sv->finished[i];
    sv->finished.erase(sv->finished.begin(), sv->finished.begin() + k);
    *count = k;
    return ERP_OK;
}

extern "C" erp_status erp_server_positions(erp_server *sv, int64_t job_id, float *x, float *y) {
    if (!sv || !x || !y) return ERP_EINVAL;
    for (auto &e : sv->pos)
        if (e.first == job_id) {
            std::copy(e.second.first.begin(), e.second.first.end(), x);
            std::copy(e.second.second.begin(), e.second.second.end(), y);
            return ERP_OK;
        }
    sv->err = "no kept positions for this job";
    return ERP_EINVAL;
}

extern "C" double erp_server_now(const erp_server *sv) { return sv ? sv->now() : 0.0; }

extern "C" const char *erp_server_last_error(const erp_server *sv) { return sv ? sv->err.c_str() : g_create_err.c_str(); }

extern "C" void erp_server_destroy(erp_server *sv) {
    if (!sv) return;
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        sv->todo.clear();   // not started: nothing to undo
        sv->stop = true;
    }
    sv->cv.notify_all();
    for (auto &t : sv->workers) t.join();   // a worker finishes its pending destroys first
    cudaSetDevice(sv->p.device);
    if (sv->master) cudaStreamSynchronize(sv->master);
    if (sv->pstream) cudaStreamSynchronize(sv->pstream);
    for (auto &sl : sv->pk) {
        if (sl.exec) cudaGraphExecDestroy(sl.exec);
        if (sl.dev) cudaFree(sl.dev);
        if (sl.staging) cudaFreeHost(sl.staging);
    }
    for (auto e : sv->pk_ev)
        if (e) cudaEventDestroy(e);
    if (sv->pk_tail) cudaEventDestroy(sv->pk_tail);
    if (sv->pstream) cudaStreamDestroy(sv->pstream);
    for (auto &j : sv->active)
        if (j->ctx) erp_destroy(j->ctx);
    for (auto &j : sv->preparing)
        if (j->ctx) erp_destroy(j->ctx);
    for (auto &g : sv->grave)
        if (g.second->ctx) erp_destroy(g.second->ctx);
    for (auto *c : sv->to_destroy) erp_destroy(c);
    for (auto e : sv->job_ev)
        if (e) cudaEventDestroy(e);
    for (auto e : sv->round_ev)
        if (e) cudaEventDestroy(e);
    if (sv->master) cudaStreamDestroy(sv->master);
    if (sv->d_states) cudaFree(sv->d_states);
    if (sv->d_done) cudaFree(sv->d_done);
    if (sv->h_done) cudaFreeHost(sv->h_done);
    delete sv;
}

// ---------------------------------------------------------------------------
// standalone spectral solve
extern "C" erp_status erp_spectral_create(int32_t m, int32_t n, float bin_w, float bin_h,
                                          int32_t precision, void *stream, erp_spectral **out) {
    g_create_err.clear();
    if (!out || !pow2_ok(m) || !pow2_ok(n) || !(bin_w > 0) || !(bin_h > 0)) {
        g_create_err = "invalid spectral solve parameters";
        return ERP_EINVAL;
    }
    if (precision != ERP_PREC_FP32 && precision != ERP_PREC_TF32_GEMM && precision != ERP_PREC_BF16X3_GEMM) {
        g_create_err = "unsupported precision";
        return ERP_ENOTSUP;
    }
    if (precision != ERP_PREC_FP32 && (m % 128 || n % 128)) {
        g_create_err = "the tensor-core solve needs bin counts that are multiples of 128";
        return ERP_EINVAL;
    }
    int dev = 0;
    cudaGetDevice(&dev);
    erp_status s = check_device(dev, g_create_err);
    if (s != ERP_OK) return s;
    if (precision != ERP_PREC_FP32) {
        erp_spectral *sg = new erp_spectral();
        sg->gemm = dctgemm_create(m, n, bin_w, bin_h, precision == ERP_PREC_TF32_GEMM ? 0 : 1,
                                  (cudaStream_t)stream, g_create_err);
        if (!sg->gemm) {
            delete sg;
            return ERP_ECUDA;
        }
        *out = sg;
        return ERP_OK;
    }
    if (spectral_prepare() != cudaSuccess) { g_create_err = "cudaFuncSetAttribute failed"; return ERP_ECUDA; }
    erp_spectral *sp = new erp_spectral();
    SpectralPlan &p = sp->p;
    memset(&p, 0, sizeof p);
    p.m = m; p.n = n; p.logm = ilog2(m); p.logn = ilog2(n);
    p.bin_w = bin_w; p.bin_h = bin_h;
    p.stream = (cudaStream_t)stream;
    const size_t mn = (size_t)m * n;
    bool ok = cudaMalloc(&p.t1, sizeof(float) * mn) == cudaSuccess &&
              cudaMalloc(&p.tx, sizeof(float) * mn) == cudaSuccess &&
              cudaMalloc(&p.ty, sizeof(float) * mn) == cudaSuccess &&
              cudaMalloc(&p.tp, sizeof(float) * mn) == cudaSuccess &&
              cudaMalloc(&sp->st, sizeof(DevState)) == cudaSuccess;
    if (!ok) {
        cudaFree(p.t1); cudaFree(p.tx); cudaFree(p.ty); cudaFree(p.tp); cudaFree(sp->st);
        delete sp;
        g_create_err = "device allocation failed";
        return ERP_ENOMEM;
    }
    cudaMemsetAsync(sp->st, 0, sizeof(DevState), p.stream);
    spectral_tables(m, n, bin_w, bin_h, &p.tw_m, &p.tw_n, &p.ek_m, &p.ek_n, &p.wu, &p.wv, p.stream);
    p.st = sp->st;
    if (cudaGetLastError() != cudaSuccess) {
        g_create_err = "spectral table set-up failed";
        erp_spectral_destroy(sp);
        return ERP_ECUDA;
    }
    *out = sp;
    return ERP_OK;
}

extern "C" erp_status erp_spectral_solve(erp_spectral *sp, const float *rho, float *fx, float *fy,
                                         float *psi) {
    if (!sp || !rho || !fx || !fy) return ERP_EINVAL;
    if (sp->gemm) {
        const cudaError_t eg = dctgemm_solve(*sp->gemm, rho, fx, fy, psi, nullptr);
        if (eg == cudaErrorTimeout) {
            sp->err = "a bounded wait of the tensor-core solve ran out";
            return ERP_ETIMEDOUT;
        }
        if (eg != cudaSuccess) {
            sp->err = cudaGetErrorString(eg);
            return ERP_ECUDA;
        }
        return ERP_OK;
    }
    SpectralArgs a;
    a.rho_in = rho;
    a.fx = fx;
    a.fy = fy;
    a.psi = psi;
    a.st = sp->st;
    launch_spectral_plan(sp->p, a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        sp->err = cudaGetErrorString(e);
        return ERP_ECUDA;
    }
    return ERP_OK;
}

extern "C" void erp_spectral_destroy(erp_spectral *sp) {
    if (!sp) return;
    if (sp->gemm) dctgemm_destroy(sp->gemm);
    SpectralPlan &p = sp->p;
    void *ptrs[] = {p.t1, p.tx, p.ty, p.tp, p.tw_m, p.tw_n, p.ek_m, p.ek_n, p.wu, p.wv, sp->st};
    for (void *q : ptrs)
        if (q) cudaFree(q);
    delete sp;
}
