// Per-cell / per-net kernels of one Placement::step (src/placement.rs:180-228):
// WA wirelength (src/hpwl.rs), density scatter into an int64 fixed-point map
// (src/density.rs), electric-force gather (src/eforce.rs), the Nesterov update
// (src/nesterov.rs) and the scheduler (src/scheduler.rs).
//
// This translation unit is compiled with -fmad=false: every float expression
// keeps the reference's operation order (no a*b+c contraction), so the density
// contributions -- and hence the integer density map -- are bit-identical to a
// CPU replay of the same rule.
#include <math.h>

#include <algorithm>
#include <climits>
#include <cmath>

#include <atomic>

#include "erp_internal.cuh"
#include "binrange.h"
#include "fixedpoint.h"
#include "reduce.cuh"

namespace erp {

// ============================ wirelength ============================
// One group of W lanes per net (nets sorted by degree class, and by degree
// within a class); lane l holds pins l, l + W, ..., l + (P-1) W in registers, so
// positions are gathered and the four max-shifted exponentials
// (src/hpwl.rs:285-299) evaluated once per pin and reused for the gradient (the
// reference recomputes them, src/hpwl.rs:314-333).  Nets of up to 8 pins take
// one thread each (W = 1: no shuffles, the per-net coefficients computed once);
// nets with more than W*P pins fall back to a loop that recomputes, like the
// reference.  The weighted sums and the gradient use fused multiply-adds and
// the four coefficient pairs one reciprocal each (src/hpwl.rs:304-312 divides
// twice): ulp-level differences, inside the FP32 tolerance of the gradient.
struct WaArgs {
    const int32_t *net_ptr;
    const int32_t *slot_cell;
    const float2 *slot_off;
    const float2 *xy;
    float2 *slot_grad;
    float *net_hpwl;
    float inv_gamma, def_min_x, def_min_y;
};

template <int W, int P>
__device__ __forceinline__ float wa_class(const WaArgs &a, int net_begin, int net_count, int general,
                                          int cblock, int cgrid) {
    const int gl = threadIdx.x & (W - 1);
    constexpr int GPB = kThreads / W;
    const float inv_gamma = a.inv_gamma;
    float hp_acc = 0.0f;
    for (int base = cblock * GPB; base < net_count; base += cgrid * GPB) {
        const int gid = base + (int)threadIdx.x / W;
        const bool active = gid < net_count;
        const int e = net_begin + gid;
        const int s0 = active ? a.net_ptr[e] : 0;
        const int deg = active ? a.net_ptr[e + 1] - s0 : 0;
        const bool in_regs = deg <= W * P;   // group-uniform
        float px[P], py[P];
        float mnx = INFINITY, mxx = -INFINITY, mny = INFINITY, mxy = -INFINITY;
#pragma unroll
        for (int q = 0; q < P; ++q) {
            const int k = gl + q * W;
            px[q] = 0.f;
            py[q] = 0.f;
            if (in_regs && k < deg) {
                const int c = a.slot_cell[s0 + k];
                const float2 o = a.slot_off[s0 + k];
                const float2 p = a.xy[c];
                px[q] = p.x + o.x;                          // src/hpwl.rs:107
                py[q] = p.y + o.y;
                mnx = fminf(mnx, px[q]); mxx = fmaxf(mxx, px[q]);
                mny = fminf(mny, py[q]); mxy = fmaxf(mxy, py[q]);
            }
        }
        if (!in_regs) {
            for (int k = gl; k < deg; k += W) {
                const int c = a.slot_cell[s0 + k];
                const float2 o = a.slot_off[s0 + k];
                const float2 p = a.xy[c];
                const float qx = p.x + o.x, qy = p.y + o.y;
                mnx = fminf(mnx, qx); mxx = fmaxf(mxx, qx);
                mny = fminf(mny, qy); mxy = fmaxf(mxy, qy);
            }
        }
#pragma unroll
        for (int o = W / 2; o > 0; o >>= 1) {
            mnx = fminf(mnx, __shfl_xor_sync(0xffffffffu, mnx, o));
            mxx = fmaxf(mxx, __shfl_xor_sync(0xffffffffu, mxx, o));
            mny = fminf(mny, __shfl_xor_sync(0xffffffffu, mny, o));
            mxy = fmaxf(mxy, __shfl_xor_sync(0xffffffffu, mxy, o));
        }
        if (general) {  // src/hpwl.rs:255-258 initial values
            mnx = fminf(a.def_min_x, mnx); mxx = fmaxf(0.0f, mxx);
            mny = fminf(a.def_min_y, mny); mxy = fmaxf(0.0f, mxy);
        }
        float ex[P], enx[P], ey[P], eny[P];
        float s_xe = 0.f, s_xen = 0.f, s_e = 0.f, s_en = 0.f;
        float s_ye = 0.f, s_yen = 0.f, s_f = 0.f, s_fn = 0.f;
#pragma unroll
        for (int q = 0; q < P; ++q) {
            ex[q] = enx[q] = ey[q] = eny[q] = 0.f;
            if (in_regs && gl + q * W < deg) {
                ex[q] = expf((px[q] - mxx) * inv_gamma);
                enx[q] = expf((mnx - px[q]) * inv_gamma);
                ey[q] = expf((py[q] - mxy) * inv_gamma);
                eny[q] = expf((mny - py[q]) * inv_gamma);
                s_xe = __fmaf_rn(px[q], ex[q], s_xe); s_xen = __fmaf_rn(px[q], enx[q], s_xen);
                s_e += ex[q]; s_en += enx[q];
                s_ye = __fmaf_rn(py[q], ey[q], s_ye); s_yen = __fmaf_rn(py[q], eny[q], s_yen);
                s_f += ey[q]; s_fn += eny[q];
            }
        }
        if (!in_regs) {
            for (int k = gl; k < deg; k += W) {
                const int c = a.slot_cell[s0 + k];
                const float2 o = a.slot_off[s0 + k];
                const float2 p = a.xy[c];
                const float qx = p.x + o.x, qy = p.y + o.y;
                const float e1 = expf((qx - mxx) * inv_gamma), e2 = expf((mnx - qx) * inv_gamma);
                const float e3 = expf((qy - mxy) * inv_gamma), e4 = expf((mny - qy) * inv_gamma);
                s_xe = __fmaf_rn(qx, e1, s_xe); s_xen = __fmaf_rn(qx, e2, s_xen); s_e += e1; s_en += e2;
                s_ye = __fmaf_rn(qy, e3, s_ye); s_yen = __fmaf_rn(qy, e4, s_yen); s_f += e3; s_fn += e4;
            }
        }
#pragma unroll
        for (int o = W / 2; o > 0; o >>= 1) {
            s_xe += __shfl_xor_sync(0xffffffffu, s_xe, o);
            s_xen += __shfl_xor_sync(0xffffffffu, s_xen, o);
            s_e += __shfl_xor_sync(0xffffffffu, s_e, o);
            s_en += __shfl_xor_sync(0xffffffffu, s_en, o);
            s_ye += __shfl_xor_sync(0xffffffffu, s_ye, o);
            s_yen += __shfl_xor_sync(0xffffffffu, s_yen, o);
            s_f += __shfl_xor_sync(0xffffffffu, s_f, o);
            s_fn += __shfl_xor_sync(0xffffffffu, s_fn, o);
        }
        // src/hpwl.rs:304-312: b = +-1/(gamma s), a = (1 - b s_w) / s
        const float r_e = __frcp_rn(s_e), r_en = __frcp_rn(s_en), r_f = __frcp_rn(s_f), r_fn = __frcp_rn(s_fn);
        const float b_x = inv_gamma * r_e, a_x = __fmaf_rn(-b_x, s_xe, 1.0f) * r_e;
        const float b_nx = -inv_gamma * r_en, a_nx = __fmaf_rn(-b_nx, s_xen, 1.0f) * r_en;
        const float b_y = inv_gamma * r_f, a_y = __fmaf_rn(-b_y, s_ye, 1.0f) * r_f;
        const float b_ny = -inv_gamma * r_fn, a_ny = __fmaf_rn(-b_ny, s_yen, 1.0f) * r_fn;
        auto grad = [&](float qx, float qy, float e1, float e2, float e3, float e4) {
            return make_float2(__fmaf_rn(__fmaf_rn(b_x, qx, a_x), e1, -(__fmaf_rn(b_nx, qx, a_nx) * e2)),
                               __fmaf_rn(__fmaf_rn(b_y, qy, a_y), e3, -(__fmaf_rn(b_ny, qy, a_ny) * e4)));
        };
#pragma unroll
        for (int q = 0; q < P; ++q) {
            const int k = gl + q * W;
            if (in_regs && k < deg) a.slot_grad[s0 + k] = grad(px[q], py[q], ex[q], enx[q], ey[q], eny[q]);
        }
        if (!in_regs) {
            for (int k = gl; k < deg; k += W) {
                const int c = a.slot_cell[s0 + k];
                const float2 o = a.slot_off[s0 + k];
                const float2 p = a.xy[c];
                const float qx = p.x + o.x, qy = p.y + o.y;
                const float e1 = expf((qx - mxx) * inv_gamma), e2 = expf((mnx - qx) * inv_gamma);
                const float e3 = expf((qy - mxy) * inv_gamma), e4 = expf((mny - qy) * inv_gamma);
                a.slot_grad[s0 + k] = grad(qx, qy, e1, e2, e3, e4);
            }
        }
        if (active && gl == 0) {
            const float hp = (mxx - mnx) + (mxy - mny);   // src/hpwl.rs:302
            a.net_hpwl[e] = hp;
            hp_acc += hp;
        }
    }
    return hp_acc;
}

// One thread per net of exact degree D, pins stored pin-major (pin q of the
// class's net g at slot0 + q * count + g): the slot reads and gradient writes of
// a warp are coalesced and no net_ptr is read.  Same arithmetic as wa_class.
template <int D>
__device__ __forceinline__ float wa_exact(const WaArgs &a, int net_begin, int net_count, int slot0,
                                          int general, int cblock, int cgrid) {
    const float inv_gamma = a.inv_gamma;
    float hp_acc = 0.0f;
    for (int g = cblock * kThreads + (int)threadIdx.x; g < net_count; g += cgrid * kThreads) {
        float px[D], py[D];
        float mnx = INFINITY, mxx = -INFINITY, mny = INFINITY, mxy = -INFINITY;
#pragma unroll
        for (int q = 0; q < D; ++q) {
            const int sl = slot0 + q * net_count + g;
            const int c = a.slot_cell[sl];
            const float2 o = a.slot_off[sl];
            const float2 p = a.xy[c];
            px[q] = p.x + o.x;                              // src/hpwl.rs:107
            py[q] = p.y + o.y;
            mnx = fminf(mnx, px[q]); mxx = fmaxf(mxx, px[q]);
            mny = fminf(mny, py[q]); mxy = fmaxf(mxy, py[q]);
        }
        if (general) {  // src/hpwl.rs:255-258 initial values
            mnx = fminf(a.def_min_x, mnx); mxx = fmaxf(0.0f, mxx);
            mny = fminf(a.def_min_y, mny); mxy = fmaxf(0.0f, mxy);
        }
        float ex[D], enx[D], ey[D], eny[D];
        float s_xe = 0.f, s_xen = 0.f, s_e = 0.f, s_en = 0.f;
        float s_ye = 0.f, s_yen = 0.f, s_f = 0.f, s_fn = 0.f;
        // Two pins bounded by themselves (no initial min / max): each pin is the
        // maximum or the minimum, so of the eight exponentials six are exp(0) = 1
        // and the other two are exp((min - max) / gamma), the very expressions the
        // general form evaluates for those pins.
        float e2x = 0.f, e2y = 0.f;
        if (D == 2 && !general) {
            e2x = expf((mnx - mxx) * inv_gamma);
            e2y = expf((mny - mxy) * inv_gamma);
        }
#pragma unroll
        for (int q = 0; q < D; ++q) {
            if (D == 2 && !general) {
                ex[q] = px[q] == mxx ? 1.0f : e2x;
                enx[q] = px[q] == mnx ? 1.0f : e2x;
                ey[q] = py[q] == mxy ? 1.0f : e2y;
                eny[q] = py[q] == mny ? 1.0f : e2y;
            } else {
                ex[q] = expf((px[q] - mxx) * inv_gamma);
                enx[q] = expf((mnx - px[q]) * inv_gamma);
                ey[q] = expf((py[q] - mxy) * inv_gamma);
                eny[q] = expf((mny - py[q]) * inv_gamma);
            }
            s_xe = __fmaf_rn(px[q], ex[q], s_xe); s_xen = __fmaf_rn(px[q], enx[q], s_xen);
            s_e += ex[q]; s_en += enx[q];
            s_ye = __fmaf_rn(py[q], ey[q], s_ye); s_yen = __fmaf_rn(py[q], eny[q], s_yen);
            s_f += ey[q]; s_fn += eny[q];
        }
        // src/hpwl.rs:304-312: b = +-1/(gamma s), a = (1 - b s_w) / s
        const float r_e = __frcp_rn(s_e), r_en = __frcp_rn(s_en), r_f = __frcp_rn(s_f), r_fn = __frcp_rn(s_fn);
        const float b_x = inv_gamma * r_e, a_x = __fmaf_rn(-b_x, s_xe, 1.0f) * r_e;
        const float b_nx = -inv_gamma * r_en, a_nx = __fmaf_rn(-b_nx, s_xen, 1.0f) * r_en;
        const float b_y = inv_gamma * r_f, a_y = __fmaf_rn(-b_y, s_ye, 1.0f) * r_f;
        const float b_ny = -inv_gamma * r_fn, a_ny = __fmaf_rn(-b_ny, s_yen, 1.0f) * r_fn;
#pragma unroll
        for (int q = 0; q < D; ++q)
            a.slot_grad[slot0 + q * net_count + g] =
                make_float2(__fmaf_rn(__fmaf_rn(b_x, px[q], a_x), ex[q], -(__fmaf_rn(b_nx, px[q], a_nx) * enx[q])),
                            __fmaf_rn(__fmaf_rn(b_y, py[q], a_y), ey[q], -(__fmaf_rn(b_ny, py[q], a_ny) * eny[q])));
        const float hp = (mxx - mnx) + (mxy - mny);   // src/hpwl.rs:302
        a.net_hpwl[net_begin + g] = hp;
        hp_acc += hp;
    }
    return hp_acc;
}

// All degree classes in one launch: blocks [cls_block[k], cls_block[k+1]) serve
// class k.  The block partials of the HPWL total are summed in double-float by
// the last block to finish (fixed order, src/hpwl.rs:341-342).
struct WaClasses {
    int begin[kNumClasses], count[kNumClasses], general[kNumClasses], slot0[kNumClasses];
    int block0[kNumClasses + 1];
};

struct WaP {
    WaArgs a;
    WaClasses cl;
    float gamma_arg;
    double * partials;
    DevState * st;
};
__device__ __forceinline__ void wa_body(const WaP &p, int bid, int nblk) {
    WaArgs a = p.a;
    const WaClasses &cl = p.cl;
    float gamma_arg = p.gamma_arg;
    double *__restrict__ partials = p.partials;
    DevState * st = p.st;
    __shared__ double shr[kThreads / 32];
    if (st->done) return;
    const float gamma = gamma_arg > 0.f ? gamma_arg : st->gamma;
    a.inv_gamma = 1.0f / gamma;                        // src/hpwl.rs:166
    // the large-degree classes (longest blocks) take the first block indices, so
    // they are dispatched first and the short blocks fill in behind them
    const int vb = (int)nblk - 1 - (int)bid;
    int k = 0;
    while (k + 1 < kNumClasses && vb >= cl.block0[k + 1]) ++k;
    const int cb = vb - cl.block0[k], cg = cl.block0[k + 1] - cl.block0[k];
    float hp;
#define ERP_WA_EXACT(K, D) \
    case K: hp = wa_exact<D>(a, cl.begin[K], cl.count[K], cl.slot0[K], cl.general[K], cb, cg); break;
    switch (k) {
    ERP_WA_EXACT(0, 2)
    ERP_WA_EXACT(1, 2)
    ERP_WA_EXACT(2, 3)
    ERP_WA_EXACT(3, 4)
    ERP_WA_EXACT(4, 5)
    ERP_WA_EXACT(5, 6)
    ERP_WA_EXACT(6, 7)
    ERP_WA_EXACT(7, 8)
    case 8: hp = wa_class<2, 8>(a, cl.begin[8], cl.count[8], cl.general[8], cb, cg); break;
    case 9: hp = wa_class<4, 8>(a, cl.begin[9], cl.count[9], cl.general[9], cb, cg); break;
    default: hp = wa_class<32, 4>(a, cl.begin[10], cl.count[10], cl.general[10], cb, cg); break;
    }
#undef ERP_WA_EXACT
    const Df vals[1] = {block_sum(hp, shr)};
    if (arrive_last(partials, bid, 1, vals, &st->ctr[CTR_HPWL], nblk)) {
        const double tot = sum_partials(partials, nblk, 1, 0, shr);
        if (threadIdx.x == 0) {
            st->hpwl = tot;
            st->hpwl_f = (float)tot;
            st->ctr[CTR_HPWL] = 0;
        }
    }
}
__global__ void __launch_bounds__(kThreads, 4) k_wa(const __grid_constant__ WaP p) { wa_body(p, blockIdx.x, gridDim.x); }


__global__ void k_wl_zero(DevState *st) {
    if (threadIdx.x == 0 && !st->done) {
        st->hpwl = 0.0;
        st->hpwl_f = 0.0f;
    }
}

// compute_gradients (src/hpwl.rs:113-135): instance gradient = sum of its pin
// gradients in macro_2_pins order; movable instances only.  The slot indices of
// up to four pins are loaded, then their gradients, then summed in list order:
// two memory round trips per four pins instead of two per pin.
struct GatherP {
    int NM;
    const int32_t * ptr;
    const int32_t * slots;
    const float2 * g;
    float * gx;
    float * gy;
    const DevState * st;
};
__device__ __forceinline__ void wl_gather_body(const GatherP &p, int bid, int nblk) {
    int NM = p.NM;
    const int32_t *__restrict__ ptr = p.ptr;
    const int32_t *__restrict__ slots = p.slots;
    const float2 *__restrict__ g = p.g;
    float *__restrict__ gx = p.gx;
    float *__restrict__ gy = p.gy;
    const DevState *__restrict__ st = p.st;
    if (st->done) return;
    for (int i = bid * blockDim.x + threadIdx.x; i < NM; i += nblk * blockDim.x) {
        float sx = 0.0f, sy = 0.0f;
        const int e = ptr[i + 1];
        for (int k0 = ptr[i]; k0 < e; k0 += 4) {
            int sl[4];
            float2 v[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) sl[u] = k0 + u < e ? slots[k0 + u] : -1;
#pragma unroll
            for (int u = 0; u < 4; ++u) v[u] = sl[u] >= 0 ? g[sl[u]] : make_float2(0.0f, 0.0f);
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (k0 + u < e) {
                    sx += v[u].x;
                    sy += v[u].y;
                }
        }
        gx[i] = sx;
        gy[i] = sy;
    }
}
__global__ void __launch_bounds__(kThreads) k_wl_gather(const __grid_constant__ GatherP p) { wl_gather_body(p, blockIdx.x, gridDim.x); }


// ============================ density ============================
// Bin coordinate limited to [-1, nbins] before the float->int conversion: the
// clamped ranges below are unchanged for every such value, and no conversion
// or +1 can overflow for huge or non-finite inputs.
__device__ __forceinline__ float clamp_bin(float v, int nbins) {
    return fminf(fmaxf(v, -1.0f), (float)nbins);
}

// triangle_density_function with the max(0) clamp (src/density.rs:7-13), xl = 0
__device__ __forceinline__ float tri_clamped(float x, float s, int k, float bs) {
    const float bin_xl = 0.0f + (float)k * bs;
    const float v = fminf(x + s, bin_xl + bs) - fmaxf(x, bin_xl);
    return v > 0.0f ? v : 0.0f;
}

// compute_density_overflow_map_sequential's bin range and per-(cell, bin)
// contribution (src/density.rs:195-229), accumulated as rint(v * 2^S) into an
// int64 map.  Integer sums are order independent, so the privatisation below
// changes no bit of the result:
//  * each block owns a kWin x kWin bin window in shared memory anchored at its
//    first cell; contributions inside it are accumulated there and flushed with
//    one global atomic per touched bin, the rest go to global memory directly;
//  * a contribution c in [0, 2^63) is kept in the window as three 21-bit pieces
//    in three 32-bit planes (32-bit shared atomics are native; 64-bit ones are
//    several times slower and degrade under contention).  A bin receives at
//    most one contribution per cell and a block owns at most kMaxCellsPerBlock
//    = 2^11 cells, so each plane's sum stays below 2^32 and the flush
//    recombines the exact 64-bit total;
//  * contributions outside the window go to a per-block table of kTable bins
//    (the slot a bin hashes to, claimed by the first bin that reaches it; a
//    bin whose slot is taken goes to global memory), so bins that many of the
//    block's cells share -- late in a diverging run cells pile up along the die
//    edge -- cost one global atomic per block.
// Early on all cells sit within a few bins of the die centre, where this turns
// millions of contended global atomics into a few per block.
//
// Cells are taken in the scatter order (perm, refreshed every few steps by
// launch_scatter_order): movable cells counting-sorted by a kSortTile-bin square
// tile of their position, so a block's cells share a tile and its window sits
// on that tile with kSortPad bins of slack on each side.  Positions come from
// the packed xy array; the stretched offsets, sizes and ratios were gathered
// into the scatter order when it was computed (they never change).  Any
// permutation gives the same integer sums: the order only decides how many
// contributions find the window.
constexpr int kWin = 64;
constexpr int kSortTile = 48, kSortPad = 8;
static_assert(kSortTile + 2 * kSortPad == kWin, "the window covers a tile and its pads");
constexpr int kTableLog = 9, kTable = 1 << kTableLog;   // out-of-window bin table (open, no probing)
constexpr unsigned kEmpty = 0xffffffffu;                 // bin indices are < 4096 * 4096
constexpr int kMaxCellsPerBlock = 2048;
// Warp-aggregated scatter for warps whose cells all fall within kAggSide x kAggSide
// bins.  Measured on the 1M-cell step (rate over 50 steps at iterations 5, 30,
// 100, 300, 500, 800): 3 x 3 boxes 4,715 / 4,634 / 4,654 / 4,448 / 4,416 / 4,520
// iterations/s, per-lane adds only 4,717 / 4,621 / 4,650 / 4,452 / 4,409 / 4,506,
// 5 x 5 boxes 4,596 / 4,547 / 4,653 / 4,443 / 4,406 / 4,518: a box takes one warp
// reduction per bin and plane, which only pays where the warp's cells pile up.
constexpr int kAggSide = 3;
constexpr unsigned long long kPiece = (1ull << 21) - 1;
// Adds the integer s0 + s1 2^21 + s2 2^42 to bin (bx, by): into the block's
// window plane by plane, else into its bin table, else into global memory.
// (s0, s1, s2) are the 21-bit pieces of one contribution c = rint((px * py) *
// 2^S), or their sums over a warp's lanes (each below 2^26).  Every plane's
// total over a block stays below 2^32: a bin receives at most one contribution
// per cell, and a block owns at most kMaxCellsPerBlock = 2^11 cells.
template <int PLANES>
__device__ __forceinline__ void scatter_add(int bx, int by, unsigned s0, unsigned s1, unsigned s2, int wox,
                                            int woy, int n, unsigned *win, unsigned *tkey, unsigned *tplane,
                                            unsigned long long *__restrict__ map) {
    const unsigned wx = (unsigned)(bx - wox), wy = (unsigned)(by - woy);
    if (wx < (unsigned)kWin && wy < (unsigned)kWin) {
        unsigned *w = win + wx * kWin + wy;
        if (s0) atomicAdd(w, s0);
        if (s1) atomicAdd(w + kWin * kWin, s1);
        if (PLANES == 3 && s2) atomicAdd(w + 2 * kWin * kWin, s2);
        return;
    }
    // outside the window: the block's bin table, else global memory
    const unsigned bin = (unsigned)bx * (unsigned)n + (unsigned)by;
    const unsigned slot = (bin * 2654435761u) >> (32 - kTableLog);
    unsigned k = tkey[slot];
    if (k == kEmpty) {
        k = atomicCAS(tkey + slot, kEmpty, bin);
        if (k == kEmpty) k = bin;
    }
    if (k == bin) {
        unsigned *t = tplane + slot;
        if (s0) atomicAdd(t, s0);
        if (s1) atomicAdd(t + kTable, s1);
        if (PLANES == 3 && s2) atomicAdd(t + 2 * kTable, s2);
    } else {
        atomicAdd(map + bin, (unsigned long long)s0 + ((unsigned long long)s1 << 21) +
                                 (PLANES == 3 ? (unsigned long long)s2 << 42 : 0ull));
    }
}

template <int PLANES>
__device__ __forceinline__ void scatter_add(int bx, int by, unsigned long long c, int wox, int woy, int n,
                                            unsigned *win, unsigned *tkey, unsigned *tplane,
                                            unsigned long long *__restrict__ map) {
    scatter_add<PLANES>(bx, by, (unsigned)(c & kPiece), (unsigned)((c >> 21) & kPiece),
                        PLANES == 3 ? (unsigned)(c >> 42) : 0u, wox, woy, n, win, tkey, tplane, map);
}

struct ScatterP {
    int NM;
    const int32_t * perm;
    const float2 * xy;
    const float4 * soff;
    const float * sratio;
    const int32_t * skey;
    int nty;
    int m;
    int n;
    float bw;
    float bh;
    float inv_bw;
    float inv_bh;
    float scale;
    unsigned long long * map;
    const DevState * st;
};
template <int PLANES>
__device__ __forceinline__ void density_scatter_body(const ScatterP &p, int bid, int nblk) {
    int NM = p.NM;
    const int32_t *__restrict__ perm = p.perm;
    const float2 *__restrict__ xy = p.xy;
    const float4 *__restrict__ soff = p.soff;
    const float *__restrict__ sratio = p.sratio;
    const int32_t *__restrict__ skey = p.skey;
    int nty = p.nty;
    int m = p.m;
    int n = p.n;
    float bw = p.bw;
    float bh = p.bh;
    float inv_bw = p.inv_bw;
    float inv_bh = p.inv_bh;
    float scale = p.scale;
    unsigned long long *__restrict__ map = p.map;
    const DevState *__restrict__ st = p.st;
    extern __shared__ unsigned dsm[];
    unsigned *win = dsm;                                  // window planes: bits 0-20, 21-41 (, 42-62)
    unsigned *tkey = dsm + PLANES * kWin * kWin;          // bin table: keys (bin index or kEmpty)
    unsigned *tplane = tkey + kTable;                     // bin table: planes
    {   // shared memory only: overlaps the previous kernel's tail
        uint4 *w4 = reinterpret_cast<uint4 *>(dsm);
        for (int k = threadIdx.x; k < PLANES * kWin * kWin / 4; k += blockDim.x) w4[k] = make_uint4(0u, 0u, 0u, 0u);
        for (int k = threadIdx.x; k < kTable; k += blockDim.x) tkey[k] = kEmpty;
        for (int k = threadIdx.x; k < PLANES * kTable; k += blockDim.x) tplane[k] = 0u;
    }
    if (st->done) return;
    const int per = ((NM + nblk - 1) / nblk + 31) & ~31;   // <= kMaxCellsPerBlock (launcher)
    const int c0 = bid * per, c1 = min(c0 + per, NM);
    int wox = 0, woy = 0;   // window origin: the sort tile of the block's first cell, less the pad
    if (c0 < NM) {
        const int k0 = skey[c0];
        wox = (k0 / nty) * kSortTile - kSortPad;
        woy = (k0 % nty) * kSortTile - kSortPad;
    }
    wox = max(0, min(wox, m - kWin));
    woy = max(0, min(woy, n - kWin));
    __syncthreads();
    for (int base = c0; base < c1; base += blockDim.x) {
        const int p = base + threadIdx.x;
        int bxl = 0, byl = 0, nx = 0, ny = 0;
        float xi = 0.f, yi = 0.f, sxi = 0.f, syi = 0.f, r = 0.f;
        if (p < c1) {
            const float2 q = xy[perm[p]];
            const float4 o = soff[p];   // offx, offy, cw, ch of cell perm[p]
            xi = q.x + o.x;
            yi = q.y + o.y;
            sxi = o.z;
            syi = o.w;
            r = sratio[p];
            int xl = (int)floorf(clamp_bin((xi - 0.0f) * inv_bw, m));
            int xh = (int)ceilf(clamp_bin((xi - 0.0f + sxi) * inv_bw, m)) + 1;
            int yl = (int)floorf(clamp_bin((yi - 0.0f) * inv_bh, n));
            int yh = (int)ceilf(clamp_bin((yi - 0.0f + syi) * inv_bh, n)) + 1;
            xl = max(xl, 0); xh = min(xh, m - 1);
            yl = max(yl, 0); yh = min(yh, n - 1);
            bxl = xl; byl = yl;
            nx = max(xh - xl, 0);
            ny = max(yh - yl, 0);
        }
        // the bins the warp's cells reach together (their full ranges)
        const unsigned full = 0xffffffffu;
        const bool any = nx > 0 && ny > 0;
        const int ax = __reduce_min_sync(full, any ? bxl : INT_MAX);
        const int ay = __reduce_min_sync(full, any ? byl : INT_MAX);
        const int ex = __reduce_max_sync(full, any ? bxl + nx : INT_MIN);
        const int ey = __reduce_max_sync(full, any ? byl + ny : INT_MIN);
        if (ax != INT_MAX && ex - ax <= kAggSide && ey - ay <= kAggSide) {
            // Warp-aggregated atomics.  The warp's cells crowd into at most
            // kAggSide x kAggSide bins (early in the run most cells sit within a
            // few bins of the die centre).  Bin by bin, every lane forms its
            // contribution -- zero outside its own range -- the warp sums the
            // 21-bit pieces, and one lane adds the sums: one atomic per bin and
            // plane instead of up to 32 contending ones.  Integer sums, so the
            // bits are those of the lanes' own adds.
            const int lane = threadIdx.x & 31;
            float pyk[kAggSide];
#pragma unroll
            for (int k = 0; k < kAggSide; ++k) {
                const int by = ay + k;
                pyk[k] = (by >= byl && by < byl + ny) ? tri_clamped(yi, syi, by, bh) : 0.0f;
            }
            for (int bx = ax; bx < ex; ++bx) {
                const float px = (bx >= bxl && bx < bxl + nx) ? r * tri_clamped(xi, sxi, bx, bw) : 0.0f;
#pragma unroll
                for (int k = 0; k < kAggSide; ++k) {
                    if (ay + k < ey) {   // warp-uniform
                        const unsigned long long c = (unsigned long long)fxp_rint_u64((px * pyk[k]) * scale);
                        const unsigned s0 = __reduce_add_sync(full, (unsigned)(c & kPiece));
                        const unsigned s1 = __reduce_add_sync(full, (unsigned)((c >> 21) & kPiece));
                        const unsigned s2 = PLANES == 3 ? __reduce_add_sync(full, (unsigned)(c >> 42)) : 0u;
                        if (lane == 0 && (s0 | s1 | s2))
                            scatter_add<PLANES>(bx, ay + k, s0, s1, s2, wox, woy, n, win, tkey, tplane, map);
                    }
                }
            }
        } else {
            // spread cells: each lane its own bin columns and rows
            for (int dx = 0; dx < nx; ++dx) {
                const int bx = bxl + dx;
                const float px = r * tri_clamped(xi, sxi, bx, bw);
                if (px == 0.0f) continue;   // every contribution of this bin column is 0
                for (int dy = 0; dy < ny; ++dy) {
                    const int by = byl + dy;
                    const float py = tri_clamped(yi, syi, by, bh);
                    const unsigned long long c = (unsigned long long)fxp_rint_u64((px * py) * scale);
                    if (c) scatter_add<PLANES>(bx, by, c, wox, woy, n, win, tkey, tplane, map);
                }
            }
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < kWin * kWin; k += blockDim.x) {
        unsigned long long v = (unsigned long long)win[k] + ((unsigned long long)win[k + kWin * kWin] << 21);
        if (PLANES == 3) v += (unsigned long long)win[k + 2 * kWin * kWin] << 42;
        const int bx = wox + k / kWin, by = woy + k % kWin;
        if (v && bx < m && by < n) atomicAdd(map + (size_t)bx * n + by, v);
    }
    for (int k = threadIdx.x; k < kTable; k += blockDim.x) {
        const unsigned bin = tkey[k];
        if (bin == kEmpty) continue;
        unsigned long long v = (unsigned long long)tplane[k] + ((unsigned long long)tplane[k + kTable] << 21);
        if (PLANES == 3) v += (unsigned long long)tplane[k + 2 * kTable] << 42;
        if (v) atomicAdd(map + bin, v);
    }
}
template <int PLANES>
__global__ void __launch_bounds__(kThreads) k_density_scatter(const __grid_constant__ ScatterP p) { density_scatter_body<PLANES>(p, blockIdx.x, gridDim.x); }


size_t density_scatter_smem(int planes) { return sizeof(unsigned) * (planes * kWin * kWin + (planes + 1) * kTable); }

// Scatter order: counting sort of the movable cells by sort tile.  Ranks within
// a tile follow atomic order (any order is valid, see k_density_scatter).
__global__ void __launch_bounds__(kThreads) k_sort_count(int NM, const float2 *__restrict__ xy,
                                                         const float *__restrict__ offx,
                                                         const float *__restrict__ offy, float inv_bw,
                                                         float inv_bh, int m, int n, int nty, int ntiles,
                                                         int32_t *__restrict__ key, int32_t *__restrict__ rank,
                                                         int32_t *__restrict__ hist) {
    extern __shared__ int32_t tcount[];   // per tile: the block's count, then its base in the tile
    constexpr int PER = 4;
    for (int k = threadIdx.x; k < ntiles; k += blockDim.x) tcount[k] = 0;
    __syncthreads();
    int kk[PER], rr[PER];
    const int base = blockIdx.x * blockDim.x * PER;
#pragma unroll
    for (int t = 0; t < PER; ++t) {
        const int i = base + t * blockDim.x + threadIdx.x;
        kk[t] = -1;
        rr[t] = 0;
        if (i < NM) {
            const float2 q = xy[i];
            int bx = (int)floorf(clamp_bin((q.x + offx[i]) * inv_bw, m));
            int by = (int)floorf(clamp_bin((q.y + offy[i]) * inv_bh, n));
            bx = max(0, min(bx, m - 1));
            by = max(0, min(by, n - 1));
            kk[t] = (bx / kSortTile) * nty + by / kSortTile;
            rr[t] = atomicAdd(tcount + kk[t], 1);
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < ntiles; k += blockDim.x) {
        const int v = tcount[k];
        if (v) tcount[k] = atomicAdd(hist + k, v);
    }
    __syncthreads();
#pragma unroll
    for (int t = 0; t < PER; ++t) {
        const int i = base + t * blockDim.x + threadIdx.x;
        if (kk[t] >= 0) {
            key[i] = kk[t];
            rank[i] = tcount[kk[t]] + rr[t];
        }
    }
}

// exclusive prefix sum of the tile counts (one block)
__global__ void __launch_bounds__(1024) k_sort_scan(int ntiles, const int32_t *__restrict__ hist,
                                                    int32_t *__restrict__ start) {
    __shared__ int32_t part[1024];
    const int per = (ntiles + blockDim.x - 1) / blockDim.x;
    const int b = threadIdx.x * per, e = min(b + per, ntiles);
    int32_t sum = 0;
    for (int k = b; k < e; ++k) sum += hist[k];
    part[threadIdx.x] = sum;
    __syncthreads();
    for (int off = 1; off < (int)blockDim.x; off <<= 1) {
        const int32_t v = (int)threadIdx.x >= off ? part[threadIdx.x - off] : 0;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    int32_t run = threadIdx.x ? part[threadIdx.x - 1] : 0;
    for (int k = b; k < e; ++k) {
        start[k] = run;
        run += hist[k];
    }
}

__global__ void __launch_bounds__(kThreads) k_sort_place(int NM, const int32_t *__restrict__ key,
                                                         const int32_t *__restrict__ rank,
                                                         const int32_t *__restrict__ start,
                                                         const float *__restrict__ offx,
                                                         const float *__restrict__ offy,
                                                         const float *__restrict__ cw, const float *__restrict__ ch,
                                                         const float *__restrict__ ratio, int32_t *__restrict__ perm,
                                                         int32_t *__restrict__ pos, float4 *__restrict__ soff,
                                                         float *__restrict__ sratio, int32_t *__restrict__ skey) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NM; i += gridDim.x * blockDim.x) {
        const int k = key[i];
        const int p = start[k] + rank[i];
        perm[p] = i;
        pos[i] = p;
        soff[p] = make_float4(offx[i], offy[i], cw[i], ch[i]);
        sratio[p] = ratio[i];
        skey[p] = k;
    }
}

int scatter_tiles(int m, int n) { return ((m + kSortTile - 1) / kSortTile) * ((n + kSortTile - 1) / kSortTile); }

static cudaError_t packed_prepare();
cudaError_t place_prepare() {
    cudaError_t e = cudaFuncSetAttribute(k_density_scatter<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)density_scatter_smem(2));
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(k_density_scatter<3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)density_scatter_smem(3));
    if (e != cudaSuccess) return e;
    return packed_prepare();
}

// compute_density_overflow (src/density.rs:16-23): overlap through bin centres
__device__ __forceinline__ float overlap_center(float x, float s, float c, float bs) {
    const float two = 1.0f + 1.0f;
    const float v = fminf(x + s, c + bs / two) - fmaxf(x, c - bs / two);
    return v > 0.0f ? v : 0.0f;
}

// compute_exact_density_overflow_map_parallel (src/density.rs:26-99) for the
// fixed cells, one block per cell, contributions rint(px*py * 2^S0).
__global__ void k_initial_density(int first, int count, const float *__restrict__ x,
                                  const float *__restrict__ y, const float *__restrict__ w,
                                  const float *__restrict__ h, const float *__restrict__ bcx,
                                  const float *__restrict__ bcy, int m, int n, float bw, float bh,
                                  float inv_bw, float inv_bh, float scale,
                                  unsigned long long *__restrict__ acc) {
    for (int ci = blockIdx.x; ci < count; ci += gridDim.x) {
        const int i = first + ci;
        const float xi = x[i], yi = y[i], sxi = w[i], syi = h[i];
        int xl = (int)floorf(clamp_bin((xi - 0.0f) * inv_bw, m));
        int xh = (int)ceilf(clamp_bin((xi - 0.0f + sxi) * inv_bw, m)) + 1;
        int yl = (int)floorf(clamp_bin((yi - 0.0f) * inv_bh, n));
        int yh = (int)ceilf(clamp_bin((yi - 0.0f + syi) * inv_bh, n)) + 1;
        xl = max(xl, 0); xh = min(xh, m - 1);
        yl = max(yl, 0); yh = min(yh, n - 1);
        const int nx = max(xh - xl, 0), ny = max(yh - yl, 0);
        for (int k = threadIdx.x; k < nx * ny; k += blockDim.x) {
            const int bx = xl + k / ny, by = yl + k % ny;
            const float px = overlap_center(xi, sxi, bcx[bx], bw);
            const float py = overlap_center(yi, syi, bcy[by], bh);
            const unsigned long long c = (unsigned long long)fxp_rint_u64((px * py) * scale);   // px, py >= 0
            if (c) atomicAdd(acc + (size_t)bx * n + by, c);
        }
    }
}

__global__ void k_initial_finalize(size_t mn, unsigned long long *__restrict__ acc, float inv,
                                   float td, float *__restrict__ initial) {
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < mn; k += (size_t)gridDim.x * blockDim.x) {
        const float v = fxp_u64_to_float(acc[k]) * inv;
        initial[k] = v * td;                                   // src/epotential.rs:138-140
        acc[k] = 0ull;
    }
}

// ============================ electric force ============================
// triangle_density_function without the clamp (src/eforce.rs:6-13)
__device__ __forceinline__ float tri_raw(float x, float s, int k, float bs) {
    const float bin_xl = 0.0f + (float)k * bs;
    return fminf(x + s, bin_xl + bs) - fmaxf(x, bin_xl);
}

// compute_electric_force (src/eforce.rs:15-91)
struct ForceP {
    int NM;
    const int32_t * perm;
    const float2 * xy;
    const float4 * soff;
    const float * sratio;
    const float * offx;
    const float * offy;
    const float * cw;
    const float * ch;
    const float * ratio;
    int m;
    int n;
    float bw;
    float bh;
    float inv_bw;
    float inv_bh;
    const float * fx;
    const float * fy;
    float2 * dgp;
    const int32_t * pos;
    int rescale;
    const float * wlgx;
    const float * wlgy;
    double * partials;
    DevState * st;
};
__device__ __forceinline__ void force_body(const ForceP &p, int bid, int nblk) {
    int NM = p.NM;
    const int32_t *__restrict__ perm = p.perm;
    const float2 *__restrict__ xy = p.xy;
    const float4 *__restrict__ soff = p.soff;
    const float *__restrict__ sratio = p.sratio;
    const float *__restrict__ offx = p.offx;
    const float *__restrict__ offy = p.offy;
    const float *__restrict__ cw = p.cw;
    const float *__restrict__ ch = p.ch;
    const float *__restrict__ ratio = p.ratio;
    int m = p.m;
    int n = p.n;
    float bw = p.bw;
    float bh = p.bh;
    float inv_bw = p.inv_bw;
    float inv_bh = p.inv_bh;
    const float *__restrict__ fx = p.fx;
    const float *__restrict__ fy = p.fy;
    float2 *__restrict__ dgp = p.dgp;
    const int32_t *__restrict__ pos = p.pos;
    int rescale = p.rescale;
    const float *__restrict__ wlgx = p.wlgx;
    const float *__restrict__ wlgy = p.wlgy;
    double *__restrict__ partials = p.partials;
    DevState * st = p.st;
    __shared__ double shr[kThreads / 32];
    if (st->done) return;
    // the field gathered over cell i's bins (src/eforce.rs)
    auto force = [&](float nx, float ny, float sx, float sy, float r) -> float2 {
        const int xl = force_bin_lo((nx - 0.0f) * inv_bw, m);
        const int xh = force_bin_hi((nx + sx - 0.0f) * inv_bw, m);
        const int yl = force_bin_lo((ny - 0.0f) * inv_bh, n);
        const int yh = force_bin_hi((ny + sy - 0.0f) * inv_bh, n);
        float gx = 0.0f, gy = 0.0f;
        for (int k = xl; k < xh; ++k) {
            const float px = tri_raw(nx, sx, k, bw);
            const float *rx = fx + (size_t)k * n, *ry = fy + (size_t)k * n;
            for (int hh = yl; hh < yh; ++hh) {
                const float py = tri_raw(ny, sy, hh, bh);
                const float area = px * py;
                gx += area * __ldg(rx + hh);
                gy += area * __ldg(ry + hh);
            }
        }
        return make_float2(-gx * r, -gy * r);
    };
    // Inside the step graph (rescale = 1) the iteration-0 density-weight rescale
    // (src/nesterov.rs:47-55) rides on this pass: the WA gradient is complete and
    // the density gradient is produced here, so no extra launch per step.  That
    // pass runs in cell order, so its sums have a fixed grouping; every
    // other pass takes the cells in the scatter order, where a block's cells
    // share a tile and so share field lines.  The gradient is stored in scatter
    // order, dgp[p], coalesced; the Nesterov pass reads it back through pos.
    // (Stored at the cell's own index, two scattered 4-byte stores per cell
    // once the cells have spread and the scatter order no longer follows the
    // cell numbering: 30.4 us at iteration 300 against 25.9 us this way.)
    if (rescale && st->iteration == 0) {   // grid-uniform
        Df sa = df_zero(), sb = df_zero();
        for (int i = bid * blockDim.x + threadIdx.x; i < NM; i += nblk * blockDim.x) {
            const float2 q = xy[i];
            const float2 g = force(q.x + offx[i], q.y + offy[i], cw[i], ch[i], ratio[i]);
            dgp[pos[i]] = g;
            sa = df_add(df_add(sa, fabsf(wlgx[i])), fabsf(wlgy[i]));
            sb = df_add(df_add(sb, fabsf(g.x)), fabsf(g.y));
        }
        Df vals[2];
        vals[0] = block_sum(sa, shr);
        vals[1] = block_sum(sb, shr);
        if (arrive_last(partials, bid, 2, vals, &st->ctr[CTR_ABS], nblk)) {
            const double num = sum_partials(partials, nblk, 2, 0, shr);
            const double den = sum_partials(partials, nblk, 2, 1, shr);
            if (threadIdx.x == 0) {
                st->abs_wl = num;
                st->abs_dens = den;
                st->dw = (float)((double)st->dw * (num / den));
                st->ctr[CTR_ABS] = 0;
            }
        }
        return;
    }
    for (int p = bid * blockDim.x + threadIdx.x; p < NM; p += nblk * blockDim.x) {
        const int i = perm[p];
        const float2 q = xy[i];
        const float4 o = soff[p];   // offx, offy, cw, ch of cell i
        dgp[p] = force(q.x + o.x, q.y + o.y, o.z, o.w, sratio[p]);
    }
}
__global__ void __launch_bounds__(kThreads) k_force(const __grid_constant__ ForceP p) { force_body(p, blockIdx.x, gridDim.x); }


// energy = sum psi * rho (src/epotential.rs:344-346), double-float sums
__global__ void k_energy(size_t mn, const float *__restrict__ psi, const float *__restrict__ rho,
                         double *__restrict__ partials, DevState *st) {
    __shared__ double shr[kThreads / 32];
    Df v = df_zero();
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < mn; k += (size_t)gridDim.x * blockDim.x)
        v = df_add(v, psi[k] * rho[k]);
    const Df vals[1] = {block_sum(v, shr)};
    if (arrive_last(partials, blockIdx.x, 1, vals, &st->ctr[CTR_ENERGY], gridDim.x)) {
        const double tot = sum_partials(partials, gridDim.x, 1, 0, shr);
        if (threadIdx.x == 0) {
            st->energy = tot;
            st->ctr[CTR_ENERGY] = 0;
        }
    }
}

// ============================ Nesterov ============================
// Iteration 0 only: density_weight *= sum|grad WL| / sum|grad D| (src/nesterov.rs:47-55)
__global__ void __launch_bounds__(kThreads) k_dw_rescale(int NM, int iter_arg,
                                                         const float *__restrict__ wlgx,
                                                         const float *__restrict__ wlgy,
                                                         const float2 *__restrict__ dgp,
                                                         const int32_t *__restrict__ pos,
                                                         double *__restrict__ partials,
                                                         DevState *st) {
    __shared__ double shr[kThreads / 32];
    if (st->done) return;
    const int it = iter_arg >= 0 ? iter_arg : st->iteration;
    if (it != 0) return;
    Df a = df_zero(), b = df_zero();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NM; i += gridDim.x * blockDim.x) {
        a = df_add(df_add(a, fabsf(wlgx[i])), fabsf(wlgy[i]));
        const float2 g = dgp[pos[i]];
        b = df_add(df_add(b, fabsf(g.x)), fabsf(g.y));
    }
    Df vals[2];
    vals[0] = block_sum(a, shr);
    vals[1] = block_sum(b, shr);
    if (arrive_last(partials, blockIdx.x, 2, vals, &st->ctr[CTR_ABS], gridDim.x)) {
        const double num = sum_partials(partials, gridDim.x, 2, 0, shr);
        const double den = sum_partials(partials, gridDim.x, 2, 1, shr);
        if (threadIdx.x == 0) {
            st->abs_wl = num;
            st->abs_dens = den;
            st->dw = (float)((double)st->dw * (num / den));
            st->ctr[CTR_ABS] = 0;
        }
    }
}

// Preconditioned combined gradient and Lipschitz sums (src/nesterov.rs:74-95);
// the gradient replaces prev_g (the reference copies it there after the update,
// src/nesterov.rs:143-144, and nothing reads prev_g in between).  The last block
// applies update_momentum (src/nesterov.rs:148-158) and the adaptive step
// length (src/nesterov.rs:98-100).
//
// Both Nesterov kernels move four cells per thread with 128-bit loads and
// stores (the per-cell arrays are 256-byte aligned; a scalar tail covers
// NM % 4).  Each thread's Lipschitz partial over its four cells is FP32 (the
// products are FP32 in the reference) and the block sums are double-float.
struct Cell4 {
    float v[4];
};
__device__ __forceinline__ Cell4 ld4(const float *p, int i4) {
    const float4 t = __ldg(reinterpret_cast<const float4 *>(p) + i4);
    return Cell4{{t.x, t.y, t.z, t.w}};
}
// plain (coherent) load for arrays the same kernel also writes
__device__ __forceinline__ Cell4 ld4w(const float *p, int i4) {
    const float4 t = reinterpret_cast<const float4 *>(p)[i4];
    return Cell4{{t.x, t.y, t.z, t.w}};
}
__device__ __forceinline__ void st4(float *p, int i4, const Cell4 &c) {
    reinterpret_cast<float4 *>(p)[i4] = make_float4(c.v[0], c.v[1], c.v[2], c.v[3]);
}

__device__ __forceinline__ void nesterov_grad_cell(float wlx, float wly, float dgx_, float dgy_, float w,
                                                   float h, float np, float x, float y, float px, float py,
                                                   float &pgx, float &pgy, float dw, float &numf,
                                                   float &denf) {
    const float one = 1.0f;
    const float area = w * h;
    const float inv_pre = one / fminf(np + dw * area, one);
    const float gx = (wlx + dw * dgx_) * inv_pre;
    const float gy = (wly + dw * dgy_) * inv_pre;
    const float dx = x - px, dy = y - py;
    const float ddx = gx - pgx, ddy = gy - pgy;
    pgx = gx;
    pgy = gy;
    numf += dx * dx + dy * dy;
    denf += ddx * ddx + ddy * ddy;
}

struct GradP {
    int NM;
    int iter_arg;
    const float * wlgx;
    const float * wlgy;
    const float2 * dgp;
    const int32_t * pos;
    const float * w;
    const float * h;
    const float * npins;
    const float * x;
    const float * y;
    const float * px;
    const float * py;
    float * pgx;
    float * pgy;
    double * partials;
    DevState * st;
};
__device__ __forceinline__ void nesterov_grad_body(const GradP &p, int bid, int nblk) {
    int NM = p.NM;
    int iter_arg = p.iter_arg;
    const float *__restrict__ wlgx = p.wlgx;
    const float *__restrict__ wlgy = p.wlgy;
    const float2 *__restrict__ dgp = p.dgp;
    const int32_t *__restrict__ pos = p.pos;
    const float *__restrict__ w = p.w;
    const float *__restrict__ h = p.h;
    const float *__restrict__ npins = p.npins;
    const float *__restrict__ x = p.x;
    const float *__restrict__ y = p.y;
    const float *__restrict__ px = p.px;
    const float *__restrict__ py = p.py;
    float *__restrict__ pgx = p.pgx;
    float *__restrict__ pgy = p.pgy;
    double *__restrict__ partials = p.partials;
    DevState * st = p.st;
    __shared__ double shr[kThreads / 32];
    if (st->done) return;
    const float dw = st->dw;
    float numf = 0.0f, denf = 0.0f;
    const int n4 = NM >> 2;
    for (int i4 = bid * blockDim.x + threadIdx.x; i4 < n4; i4 += nblk * blockDim.x) {
        const Cell4 a = ld4(wlgx, i4), b = ld4(wlgy, i4);
        const int4 at = reinterpret_cast<const int4 *>(pos)[i4];
        const float2 g0 = dgp[at.x], g1 = dgp[at.y], g2 = dgp[at.z], g3 = dgp[at.w];
        const Cell4 c = {{g0.x, g1.x, g2.x, g3.x}}, d = {{g0.y, g1.y, g2.y, g3.y}};
        const Cell4 ww = ld4(w, i4), hh = ld4(h, i4), np = ld4(npins, i4);
        const Cell4 xx = ld4(x, i4), yy = ld4(y, i4), qx = ld4(px, i4), qy = ld4(py, i4);
        Cell4 gx = ld4w(pgx, i4), gy = ld4w(pgy, i4);
#pragma unroll
        for (int k = 0; k < 4; ++k)
            nesterov_grad_cell(a.v[k], b.v[k], c.v[k], d.v[k], ww.v[k], hh.v[k], np.v[k], xx.v[k], yy.v[k],
                               qx.v[k], qy.v[k], gx.v[k], gy.v[k], dw, numf, denf);
        st4(pgx, i4, gx);
        st4(pgy, i4, gy);
    }
    if (bid == 0 && threadIdx.x < (NM & 3)) {   // tail cells
        const int i = (n4 << 2) + threadIdx.x;
        float gx = pgx[i], gy = pgy[i];
        const float2 g = dgp[pos[i]];
        nesterov_grad_cell(wlgx[i], wlgy[i], g.x, g.y, w[i], h[i], npins[i], x[i], y[i], px[i],
                           py[i], gx, gy, dw, numf, denf);
        pgx[i] = gx;
        pgy[i] = gy;
    }
    Df vals[2];
    vals[0] = block_sum(numf, shr);
    vals[1] = block_sum(denf, shr);
    if (arrive_last(partials, bid, 2, vals, &st->ctr[CTR_LIP], nblk)) {
        const double tn = sum_partials(partials, nblk, 2, 0, shr);
        const double td = sum_partials(partials, nblk, 2, 1, shr);
        if (threadIdx.x == 0) {
            const int it = iter_arg >= 0 ? iter_arg : st->iteration;
            const float one = 1.0f, two = one + one, four = two + two;
            const float a_prev = st->alpha;
            const float na = (one + sqrtf(four * a_prev * a_prev + one)) / two;
            st->beta = (a_prev - one) / na;
            st->alpha = na;
            if (it > 0 && td > 0.0) st->alpha = (float)sqrt(tn / td);
            st->lip_num = tn;
            st->lip_den = td;
            st->ctr[CTR_LIP] = 0;
        }
    }
}
__global__ void __launch_bounds__(kThreads) k_nesterov_grad(const __grid_constant__ GradP p) { nesterov_grad_body(p, blockIdx.x, gridDim.x); }


// Lookahead + gradient step + clamp + history (src/nesterov.rs:111-145).
__device__ __forceinline__ void nesterov_update_cell(float &x, float &y, float &px, float &py, float gx,
                                                     float gy, float w, float h, float die_w, float die_h,
                                                     float alpha, float beta) {
    const float one = 1.0f;
    const float xo = x, yo = y;
    const float xh = xo + beta * (xo - px);
    const float yh = yo + beta * (yo - py);
    const float hx = die_w - w - one, hy = die_h - h - one;
    float nx = xh - alpha * gx, ny = yh - alpha * gy;
    nx = nx < 0.0f ? 0.0f : (nx > hx ? hx : nx);
    ny = ny < 0.0f ? 0.0f : (ny > hy ? hy : ny);
    px = xo;
    py = yo;
    x = nx;
    y = ny;
}

struct UpdateP {
    int NM;
    const float * w;
    const float * h;
    float die_w;
    float die_h;
    float * x;
    float * y;
    float * px;
    float * py;
    const float * gx;
    const float * gy;
    float2 * xy;
    const DevState * st;
};
__device__ __forceinline__ void nesterov_update_body(const UpdateP &p, int bid, int nblk) {
    int NM = p.NM;
    const float *__restrict__ w = p.w;
    const float *__restrict__ h = p.h;
    float die_w = p.die_w;
    float die_h = p.die_h;
    float *__restrict__ x = p.x;
    float *__restrict__ y = p.y;
    float *__restrict__ px = p.px;
    float *__restrict__ py = p.py;
    const float *__restrict__ gx = p.gx;
    const float *__restrict__ gy = p.gy;
    float2 *__restrict__ xy = p.xy;
    const DevState *__restrict__ st = p.st;
    if (st->done) return;
    const float alpha = st->alpha, beta = st->beta;
    const int n4 = NM >> 2;
    for (int i4 = bid * blockDim.x + threadIdx.x; i4 < n4; i4 += nblk * blockDim.x) {
        Cell4 xx = ld4w(x, i4), yy = ld4w(y, i4), qx = ld4w(px, i4), qy = ld4w(py, i4);
        const Cell4 a = ld4(gx, i4), b = ld4(gy, i4), ww = ld4(w, i4), hh = ld4(h, i4);
#pragma unroll
        for (int k = 0; k < 4; ++k)
            nesterov_update_cell(xx.v[k], yy.v[k], qx.v[k], qy.v[k], a.v[k], b.v[k], ww.v[k], hh.v[k], die_w,
                                 die_h, alpha, beta);
        st4(x, i4, xx);
        st4(y, i4, yy);
        st4(px, i4, qx);
        st4(py, i4, qy);
        float4 *xy4 = reinterpret_cast<float4 *>(xy) + 2 * i4;
        xy4[0] = make_float4(xx.v[0], yy.v[0], xx.v[1], yy.v[1]);
        xy4[1] = make_float4(xx.v[2], yy.v[2], xx.v[3], yy.v[3]);
    }
    if (bid == 0 && threadIdx.x < (NM & 3)) {
        const int i = (n4 << 2) + threadIdx.x;
        float xi = x[i], yi = y[i], pxi = px[i], pyi = py[i];
        nesterov_update_cell(xi, yi, pxi, pyi, gx[i], gy[i], w[i], h[i], die_w, die_h, alpha, beta);
        x[i] = xi;
        y[i] = yi;
        px[i] = pxi;
        py[i] = pyi;
        xy[i] = make_float2(xi, yi);
    }
}
__global__ void __launch_bounds__(kThreads) k_nesterov_update(const __grid_constant__ UpdateP p) { nesterov_update_body(p, blockIdx.x, gridDim.x); }


// xy = (x, y) for every instance, after positions were written from the host.
__global__ void k_pack_xy(int N, const float *__restrict__ x, const float *__restrict__ y,
                          float2 *__restrict__ xy) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
        xy[i] = make_float2(x[i], y[i]);
}

// The host's coordinates read and written by the device directly (registered,
// device-mapped host memory; over NVLink-C2C on a Grace host): one pass fills
// x, y and the interleaved xy, one pass writes the step's result back.
__global__ void k_xy_from_host(int N, const float *__restrict__ hx, const float *__restrict__ hy,
                               float *__restrict__ x, float *__restrict__ y, float2 *__restrict__ xy) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        const float a = hx[i], b = hy[i];
        x[i] = a;
        y[i] = b;
        xy[i] = make_float2(a, b);
    }
}

__global__ void k_xy_to_host(int N, const float2 *__restrict__ xy, float *__restrict__ hx, float *__restrict__ hy) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        const float2 v = xy[i];
        hx[i] = v.x;
        hy[i] = v.y;
    }
}

// ============================ scheduler ============================
struct SchedLogs {
    double ln_shrink, ln_grow, ln_ten;   // ln 0.9999, ln 1.05, ln 10
};

// Scheduler::update + should_stop (src/scheduler.rs:68-130) in FP64, plus the
// step record, the non-finite check and the retire-at-overflow flag.
struct SchedP {
    int use_args;
    float hpwl_arg;
    float ovf_arg;
    SchedLogs lg;
    DevState * st;
};
__device__ __forceinline__ void scheduler_body(const SchedP &p, int bid, int nblk) {
    int use_args = p.use_args;
    float hpwl_arg = p.hpwl_arg;
    float ovf_arg = p.ovf_arg;
    SchedLogs lg = p.lg;
    DevState * st = p.st;
    if (bid != 0) return;
    if (st->done) return;   // warp-uniform
    const float hpwl = use_args ? hpwl_arg : st->hpwl_f;
    const float ovf = use_args ? ovf_arg : st->overflow_f;
    // The density-weight power (lane 0) and the gamma coefficient (lane 1) are
    // independent FP64 powers of constant bases, b^e = exp(e ln b) with ln b
    // computed on the host: one convergent exp call evaluates both.  (FP64 runs
    // at a small fraction of the FP32 rate here; pow's own logarithm was most of
    // this one-warp kernel's time.)
    const int lane = threadIdx.x & 31;
    const int it1 = st->iteration + 1;
    const float ref0 = st->hpwl_init_set ? st->hpwl_init : hpwl;
    const float delta0 = hpwl - st->hpwl_cur;   // hpwl_cur - hpwl_prev after the update below
    // exponents: (ovf - 0.1) * 20 / 9 - 1 (lane 1), iteration, or -delta / ref,
    // each as num / den in the same operation order, so one convergent division
    double lnb, num, den;
    if (lane == 1) {
        lnb = lg.ln_ten;
        num = ((double)ovf - 0.1) * 20.0;
        den = 9.0;
    } else if (delta0 < 0.0f) {
        lnb = lg.ln_shrink;
        num = (double)it1;
        den = 1.0;
    } else {
        lnb = lg.ln_grow;
        num = -(double)delta0;
        den = (double)ref0;
    }
    double ex = num / den;
    if (lane == 1) ex -= 1.0;
    double pw = exp(ex * lnb);
    if (lane == 1) pw = pw < 0.05 ? 0.05 : (pw > 10.0 ? 10.0 : pw);
    else if (delta0 < 0.0f) pw = pw < 0.98 ? 0.98 : pw;
    else pw = pw < 0.95 ? 0.95 : (pw > 1.05 ? 1.05 : pw);
    const double coef_l1 = __shfl_sync(0xffffffffu, pw, 1);
    if (lane != 0) return;
    erp_step_stats rec;
    rec.iteration = st->iteration;
    rec.hpwl = hpwl;
    rec.overflow = ovf;
    rec.density_weight = st->dw;
    rec.gamma = st->gamma;
    st->iteration += 1;
    if (!st->hpwl_init_set) { st->hpwl_init = hpwl; st->hpwl_init_set = 1; }
    st->hpwl_prev = st->hpwl_cur;
    st->hpwl_cur = hpwl;
    if (!st->ovf_init_set) { st->ovf_init = ovf; st->ovf_init_set = 1; }
    st->ovf_prev = st->ovf_cur;
    st->ovf_cur = ovf;
    const double power = pw;   // the rule above, on hpwl_init / hpwl_cur - hpwl_prev / iteration as updated here
    st->dw = (float)((double)st->dw * (1.05 * power));
    st->gamma = (float)((double)st->base_gamma * coef_l1);
    const float cur = st->hpwl_cur, prev = st->hpwl_prev;
    rec.should_stop = (prev != 0.0f && cur != 0.0f && prev > cur * 1.5f) ? 1 : 0;
    rec.alpha = st->alpha;
    rec.beta = st->beta;
    st->last = rec;
    st->last_iter = rec.iteration;
    if (!isfinite(hpwl) || !isfinite(ovf) || !isfinite(st->alpha)) {
        st->status |= 1;
        st->done = 1;
    }
    if (st->stop_overflow > 0.0f && ovf <= st->stop_overflow) st->done = 1;
    if (st->stop_iter > 0 && st->iteration >= st->stop_iter) st->done = 1;
}
__global__ void k_scheduler(const __grid_constant__ SchedP p) { scheduler_body(p, blockIdx.x, gridDim.x); }


__global__ void k_gather_done(DevState *const *states, int count, int32_t *out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x)
        out[i] = states[i]->done;
}

void launch_gather_done(DevState *const *states, int count, int32_t *out, cudaStream_t s) {
    k_gather_done<<<(count + 255) / 256, 256, 0, s>>>(states, count, out);
}

// ============================ launchers ============================
static int grid_for(int work, int cap = 152 * 8) {
    int g = (work + kThreads - 1) / kThreads;
    return g < 1 ? 1 : (g > cap ? cap : g);
}

static int wa_params(Ctx &c, float gamma_arg, WaP &p) {
    WaArgs a;
    a.net_ptr = c.net_ptr;
    a.slot_cell = c.slot_cell;
    a.slot_off = c.slot_off;
    a.xy = c.xy;
    a.slot_grad = c.slot_grad;
    a.net_hpwl = c.net_hpwl;
    a.inv_gamma = 0.f;
    a.def_min_x = c.die_w + 1.0f;
    a.def_min_y = c.die_h + 1.0f;
    WaClasses cl;
    // at most 256 blocks per class: grid-stride loops over several nets per
    // thread measured fastest on the 1M-cell workload (256: 93 us, 1024: 107 us,
    // one net per thread: 121 us); fewer if the block partials of the HPWL sum
    // would not fit, then every class's grid shrinks in proportion
    long long need[kNumClasses], total = 0;
    for (int k = 0; k < kNumClasses; ++k) {
        const int gpb = kThreads / c.cls[k].width;
        need[k] = std::min<long long>((c.cls[k].count + gpb - 1) / gpb, 256);
        total += need[k];
    }
    int blocks = 0;
    for (int k = 0; k < kNumClasses; ++k) {
        const NetClass &nc = c.cls[k];
        cl.begin[k] = nc.begin;
        cl.count[k] = nc.count;
        cl.general[k] = nc.general;
        cl.slot0[k] = nc.slot0;
        cl.block0[k] = blocks;
        long long g = need[k];
        if (total > c.max_partials && g > 0) {
            g = need[k] * (c.max_partials - kNumClasses) / total;
            if (g < 1) g = 1;
        }
        blocks += (int)g;
    }
    cl.block0[kNumClasses] = blocks;
    p = WaP{a, cl, gamma_arg, c.partials, c.st};
    return blocks;
}

void launch_wirelength(Ctx &c, float gamma_arg) {
    WaP p;
    const int blocks = wa_params(c, gamma_arg, p);
    if (blocks == 0) {   // no nets: the total is zero
        k_wl_zero<<<1, 32, 0, c.stream>>>(c.st);
        return;
    }
    k_wa<<<blocks, kThreads, 0, c.stream>>>(p);
}

static int gather_params(Ctx &c, GatherP &p) {
    p = GatherP{c.NM, c.cell_slot_ptr, c.cell_slots, c.slot_grad, c.wlgx, c.wlgy, c.st};
    return grid_for(c.NM);
}

void launch_wl_gather(Ctx &c) {
    GatherP p;
    const int g = gather_params(c, p);
    k_wl_gather<<<g, kThreads, 0, c.stream>>>(p);
}

// Blocks of the scatter.  Alone, a context spreads its cells over up to 608
// blocks (four per SM); a batch autotunes the cells per block, since with many
// instances on the GPU at once fewer, fuller blocks flush fewer windows (see
// erp_batch_create).  Never more than kMaxCellsPerBlock cells per block (the
// window's 21-bit pieces rely on it); the grid decides no bit of the map.
static int scatter_params(Ctx &c, ScatterP &p) {
    const int floor_g = (c.NM + kMaxCellsPerBlock - 1) / kMaxCellsPerBlock;
    const int g = c.scatter_cells > 0 ? std::max((c.NM + c.scatter_cells - 1) / c.scatter_cells, std::max(floor_g, 1))
                                      : std::max(grid_for(c.NM, 152 * 4), floor_g);
    const int nty = (c.n + kSortTile - 1) / kSortTile;
    p = ScatterP{c.NM, c.perm, c.xy, c.soff, c.sratio, c.skey, nty, c.m, c.n, c.bin_w, c.bin_h, c.inv_bw, c.inv_bh,
                 c.fixed_scale, c.dmap, c.st};
    return g;
}

void launch_density_scatter(Ctx &c) {
    ScatterP p;
    const int g = scatter_params(c, p);
    auto kern = c.scatter_planes == 2 ? k_density_scatter<2> : k_density_scatter<3>;
    kern<<<g, kThreads, density_scatter_smem(c.scatter_planes), c.stream>>>(p);
}

void launch_scatter_order(Ctx &c, cudaStream_t s) {
    if (c.NM <= 0) return;
    const int nty = (c.n + kSortTile - 1) / kSortTile;
    const int ntiles = scatter_tiles(c.m, c.n);
    cudaMemsetAsync(c.sort_hist, 0, sizeof(int32_t) * ntiles, s);
    k_sort_count<<<(c.NM + 4 * kThreads - 1) / (4 * kThreads), kThreads, sizeof(int32_t) * ntiles, s>>>(
        c.NM, c.xy, c.offx, c.offy, c.inv_bw, c.inv_bh, c.m, c.n, nty, ntiles, c.sort_key, c.sort_rank,
        c.sort_hist);
    k_sort_scan<<<1, 1024, 0, s>>>(ntiles, c.sort_hist, c.sort_start);
    k_sort_place<<<grid_for(c.NM), kThreads, 0, s>>>(c.NM, c.sort_key, c.sort_rank, c.sort_start, c.offx, c.offy,
                                                     c.cw, c.ch, c.ratio, c.perm, c.pos, c.soff, c.sratio,
                                                     c.skey);
}

void launch_initial_density(Ctx &c, const float *, const float *, const float *, const float *) {
    const int count = c.N - c.NM;
    const size_t mn = (size_t)c.m * c.n;
    if (count > 0) {
        // bin centres (src/placement.rs:81-94)
        float *hcx = new float[c.m], *hcy = new float[c.n];
        for (int i = 0; i < c.m; ++i) {
            float l = 0.0f + (float)i * c.bin_w, hh = fminf(l + c.bin_w, c.die_w);
            hcx[i] = (l + hh) / 2.0f;
        }
        for (int i = 0; i < c.n; ++i) {
            float l = 0.0f + (float)i * c.bin_h, hh = fminf(l + c.bin_h, c.die_h);
            hcy[i] = (l + hh) / 2.0f;
        }
        float *dcx, *dcy;
        ctx_alloc((void **)&dcx, sizeof(float) * c.m, c.stream);
        ctx_alloc((void **)&dcy, sizeof(float) * c.n, c.stream);
        cudaMemcpyAsync(dcx, hcx, sizeof(float) * c.m, cudaMemcpyHostToDevice, c.stream);
        cudaMemcpyAsync(dcy, hcy, sizeof(float) * c.n, cudaMemcpyHostToDevice, c.stream);
        k_initial_density<<<count < 4096 ? count : 4096, kThreads, 0, c.stream>>>(
            c.NM, count, c.x, c.y, c.w, c.h, dcx, dcy, c.m, c.n, c.bin_w, c.bin_h, c.inv_bw, c.inv_bh,
            ldexpf(1.0f, c.shift0), c.dmap);
        cudaStreamSynchronize(c.stream);
        cudaFreeAsync(dcx, c.stream);
        cudaFreeAsync(dcy, c.stream);
        delete[] hcx;
        delete[] hcy;
    }
    k_initial_finalize<<<grid_for((int)(mn > (1u << 30) ? (1u << 30) : mn)), kThreads, 0, c.stream>>>(
        mn, c.dmap, ldexpf(1.0f, -c.shift0), c.target_density, c.initial);
}

// Blocks of the streaming kernels that fit on the GPU at once: their grids stop
// there (grid-stride loops), so no partial last wave runs alone.
// (written by every context set-up, possibly on several host threads at once:
// atomics, though every writer stores the same counts)
static std::atomic<int> g_res_force{0}, g_res_grad{0}, g_res_update{0};
static int fit(int need, const std::atomic<int> &resident_a) {
    const int resident = resident_a.load(std::memory_order_relaxed);
    return resident > 0 && need > resident ? resident : need;
}

static int force_params(Ctx &c, int rescale, ForceP &p) {
    p = ForceP{c.NM, c.perm, c.xy, c.soff, c.sratio, c.offx, c.offy, c.cw, c.ch, c.ratio, c.m, c.n, c.bin_w,
               c.bin_h, c.inv_bw, c.inv_bh, c.fx, c.fy, c.dgp, c.pos, rescale, c.wlgx, c.wlgy, c.partials, c.st};
    return fit(grid_for(c.NM, 152 * 16), g_res_force);
}

void launch_force(Ctx &c, int rescale) {
    ForceP p;
    const int g = force_params(c, rescale, p);
    k_force<<<g, kThreads, 0, c.stream>>>(p);
}

void launch_energy(Ctx &c) {
    const size_t mn = (size_t)c.m * c.n;
    k_energy<<<grid_for((int)(mn > (1u << 30) ? (1u << 30) : mn)), kThreads, 0, c.stream>>>(
        mn, c.psi, c.rho, c.partials, c.st);
}

static int grad_params(Ctx &c, int iter_arg, GradP &p) {
    p = GradP{c.NM, iter_arg, c.wlgx, c.wlgy, c.dgp, c.pos, c.w, c.h, c.npins, c.x, c.y, c.prev_x, c.prev_y,
              c.prev_gx, c.prev_gy, c.partials, c.st};
    return fit(grid_for((c.NM + 3) / 4), g_res_grad);
}

static int update_params(Ctx &c, UpdateP &p) {
    p = UpdateP{c.NM, c.w, c.h, c.die_w, c.die_h, c.x, c.y, c.prev_x, c.prev_y, c.prev_gx, c.prev_gy, c.xy, c.st};
    return fit(grid_for((c.NM + 3) / 4), g_res_update);
}

void launch_nesterov(Ctx &c, int iter_arg) {
    if (iter_arg >= 0) {   // stage entry point; in the step graph k_force does the rescale
        const int g = grid_for(c.NM);
        k_dw_rescale<<<g, kThreads, 0, c.stream>>>(c.NM, iter_arg, c.wlgx, c.wlgy, c.dgp, c.pos,
                                                   c.partials, c.st);
    }
    GradP pg;
    UpdateP pu;
    const int gg = grad_params(c, iter_arg, pg), gu = update_params(c, pu);
    k_nesterov_grad<<<gg, kThreads, 0, c.stream>>>(pg);
    k_nesterov_update<<<gu, kThreads, 0, c.stream>>>(pu);
}

cudaError_t place_occupancy() {
    int dev = 0, sms = 0, a = 0, b = 0, d = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_force, kThreads, 0);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_nesterov_grad, kThreads, 0);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&d, k_nesterov_update, kThreads, 0);
    if (e != cudaSuccess) return e;
    g_res_force.store(a * sms, std::memory_order_relaxed);
    g_res_grad.store(b * sms, std::memory_order_relaxed);
    g_res_update.store(d * sms, std::memory_order_relaxed);
    return cudaSuccess;
}

void launch_pack_xy(Ctx &c) {
    if (c.N > 0) k_pack_xy<<<grid_for(c.N), kThreads, 0, c.stream>>>(c.N, c.x, c.y, c.xy);
}

// Four cells per thread with 16-byte accesses when both host buffers allow it:
// fewer, larger requests across the host link.
__global__ void k_xy_from_host4(int N, const float4 *__restrict__ hx, const float4 *__restrict__ hy,
                                float4 *__restrict__ x, float4 *__restrict__ y, float4 *__restrict__ xy) {
    const int n4 = N >> 2;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += gridDim.x * blockDim.x) {
        const float4 a = hx[i], b = hy[i];
        x[i] = a;
        y[i] = b;
        xy[2 * i] = make_float4(a.x, b.x, a.y, b.y);
        xy[2 * i + 1] = make_float4(a.z, b.z, a.w, b.w);
    }
}

__global__ void k_xy_to_host4(int N, const float4 *__restrict__ xy, float4 *__restrict__ hx, float4 *__restrict__ hy) {
    const int n4 = N >> 2;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += gridDim.x * blockDim.x) {
        const float4 p = xy[2 * i], q = xy[2 * i + 1];
        hx[i] = make_float4(p.x, p.z, q.x, q.z);
        hy[i] = make_float4(p.y, p.w, q.y, q.w);
    }
}

static bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

void launch_xy_from_host(Ctx &c, const float *hx, const float *hy) {
    if (c.N <= 0) return;
    const int n4 = c.N >> 2;
    if (n4 > 0 && aligned16(hx) && aligned16(hy)) {   // device arrays are 256-byte aligned
        k_xy_from_host4<<<grid_for(n4), kThreads, 0, c.stream>>>(c.N, reinterpret_cast<const float4 *>(hx),
                                                                 reinterpret_cast<const float4 *>(hy),
                                                                 reinterpret_cast<float4 *>(c.x),
                                                                 reinterpret_cast<float4 *>(c.y),
                                                                 reinterpret_cast<float4 *>(c.xy));
        const int t = n4 << 2;   // the tail
        if (t < c.N) k_xy_from_host<<<1, 32, 0, c.stream>>>(c.N - t, hx + t, hy + t, c.x + t, c.y + t, c.xy + t);
        return;
    }
    k_xy_from_host<<<grid_for(c.N), kThreads, 0, c.stream>>>(c.N, hx, hy, c.x, c.y, c.xy);
}

void launch_xy_to_host(Ctx &c, float *hx, float *hy) {
    if (c.N <= 0) return;
    const int n4 = c.N >> 2;
    if (n4 > 0 && aligned16(hx) && aligned16(hy)) {
        k_xy_to_host4<<<grid_for(n4), kThreads, 0, c.stream>>>(c.N, reinterpret_cast<const float4 *>(c.xy),
                                                               reinterpret_cast<float4 *>(hx),
                                                               reinterpret_cast<float4 *>(hy));
        const int t = n4 << 2;
        if (t < c.N) k_xy_to_host<<<1, 32, 0, c.stream>>>(c.N - t, c.xy + t, hx + t, hy + t);
        return;
    }
    k_xy_to_host<<<grid_for(c.N), kThreads, 0, c.stream>>>(c.N, c.xy, hx, hy);
}

// update_density_weight's bases 0.9999 and 1.05, update_gamma's 10
// (src/scheduler.rs:92-130)
static SchedP sched_params(Ctx &c, int use_args, float hpwl, float overflow) {
    static const SchedLogs lg = {std::log(0.9999), std::log(1.05), std::log(10.0)};
    return SchedP{use_args, hpwl, overflow, lg, c.st};
}

void launch_scheduler(Ctx &c, int use_args, float hpwl, float overflow) {
    k_scheduler<<<1, 32, 0, c.stream>>>(sched_params(c, use_args, hpwl, overflow));
}

// ---- packed launches (batches) ----
template <typename P, typename F>
static void plan_stage(PackKind k, int variant, const std::vector<Ctx *> &xs, PackedArena &ar,
                       std::vector<PackedLaunch> &out, int threads, size_t smem, F params) {
    std::vector<P> tab;
    std::vector<int32_t> block0(1, 0);
    for (Ctx *c : xs) {
        P p;
        const int g = params(*c, p);
        if (g <= 0) continue;
        tab.push_back(p);
        block0.push_back(block0.back() + g);
    }
    if (tab.empty()) return;
    PackedLaunch l;
    l.kind = k;
    l.variant = variant;
    l.tab = ar.put(tab.data(), sizeof(P) * tab.size());
    l.block0 = ar.put(block0.data(), sizeof(int32_t) * block0.size());
    l.n = (int)tab.size();
    l.blocks = block0.back();
    l.threads = threads;
    l.smem = smem;
    out.push_back(l);
}

void packed_place_stage(PackKind k, const std::vector<Ctx *> &xs, PackedArena &ar, std::vector<PackedLaunch> &out) {
    switch (k) {
    case PK_WA:
        plan_stage<WaP>(k, 0, xs, ar, out, kThreads, 0, [](Ctx &c, WaP &p) { return wa_params(c, -1.0f, p); });
        break;
    case PK_GATHER:
        plan_stage<GatherP>(k, 0, xs, ar, out, kThreads, 0, [](Ctx &c, GatherP &p) { return gather_params(c, p); });
        break;
    case PK_SCATTER:
        for (int planes = 2; planes <= 3; ++planes) {
            std::vector<Ctx *> sub;
            for (Ctx *c : xs)
                if (c->scatter_planes == planes) sub.push_back(c);
            plan_stage<ScatterP>(k, planes, sub, ar, out, kThreads, density_scatter_smem(planes),
                                 [](Ctx &c, ScatterP &p) { return scatter_params(c, p); });
        }
        break;
    case PK_FORCE:
        plan_stage<ForceP>(k, 0, xs, ar, out, kThreads, 0, [](Ctx &c, ForceP &p) { return force_params(c, 1, p); });
        break;
    case PK_GRAD:
        plan_stage<GradP>(k, 0, xs, ar, out, kThreads, 0, [](Ctx &c, GradP &p) { return grad_params(c, -1, p); });
        break;
    case PK_UPDATE:
        plan_stage<UpdateP>(k, 0, xs, ar, out, kThreads, 0, [](Ctx &c, UpdateP &p) { return update_params(c, p); });
        break;
    case PK_SCHED:
        plan_stage<SchedP>(k, 0, xs, ar, out, 32, 0, [](Ctx &c, SchedP &p) {
            p = sched_params(c, 0, 0.f, 0.f);
            return 1;
        });
        break;
    default:
        break;
    }
}

static cudaError_t packed_prepare() {
    cudaError_t e = cudaFuncSetAttribute(k_packed<ScatterP, density_scatter_body<2>, kThreads, 4>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)density_scatter_smem(2));
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(k_packed<ScatterP, density_scatter_body<3>, kThreads, 4>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)density_scatter_smem(3));
}

bool packed_place_launch(const PackedLaunch &l, const unsigned char *dev, cudaStream_t s) {
    switch (l.kind) {
    case PK_WA:
        k_packed<WaP, wa_body, kThreads, 4><<<l.blocks, l.threads, 0, s>>>(packed_args<WaP>(l, dev));
        return true;
    case PK_GATHER:
        k_packed<GatherP, wl_gather_body, kThreads, 4><<<l.blocks, l.threads, 0, s>>>(packed_args<GatherP>(l, dev));
        return true;
    case PK_SCATTER:
        if (l.variant == 2)
            k_packed<ScatterP, density_scatter_body<2>, kThreads, 4><<<l.blocks, l.threads, l.smem, s>>>(
                packed_args<ScatterP>(l, dev));
        else
            k_packed<ScatterP, density_scatter_body<3>, kThreads, 4><<<l.blocks, l.threads, l.smem, s>>>(
                packed_args<ScatterP>(l, dev));
        return true;
    case PK_FORCE:
        k_packed<ForceP, force_body, kThreads, 4><<<l.blocks, l.threads, 0, s>>>(packed_args<ForceP>(l, dev));
        return true;
    case PK_GRAD:
        k_packed<GradP, nesterov_grad_body, kThreads, 3><<<l.blocks, l.threads, 0, s>>>(packed_args<GradP>(l, dev));
        return true;
    case PK_UPDATE:
        k_packed<UpdateP, nesterov_update_body, kThreads, 4><<<l.blocks, l.threads, 0, s>>>(
            packed_args<UpdateP>(l, dev));
        return true;
    case PK_SCHED:
        k_packed<SchedP, scheduler_body, 32, 1><<<l.blocks, l.threads, 0, s>>>(packed_args<SchedP>(l, dev));
        return true;
    default:
        return false;
    }
}

}  // namespace erp
