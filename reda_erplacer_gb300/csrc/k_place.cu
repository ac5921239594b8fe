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

#include "erp_internal.cuh"
#include "reduce.cuh"

namespace erp {

// ============================ wirelength ============================
// One group of W lanes per net (nets sorted by degree class).  Lane l holds pin
// l for W >= degree; the >32-pin class loops over pins (LOOP) and recomputes
// the exponentials in the gradient pass as the reference does
// (src/hpwl.rs:314-333).  Max-shifted exponentials as in src/hpwl.rs:285-299.
template <int W, bool LOOP>
__global__ void __launch_bounds__(kThreads) k_wa(
    int net_begin, int net_count, int general, const int32_t *__restrict__ net_ptr,
    const int32_t *__restrict__ slot_cell, const float2 *__restrict__ slot_off,
    const float *__restrict__ x, const float *__restrict__ y, float2 *__restrict__ slot_grad,
    float *__restrict__ net_hpwl, const DevState *__restrict__ st, float gamma_arg,
    float def_min_x, float def_min_y, double *__restrict__ partials, int part_off) {
    __shared__ double shr[kThreads / 32];
    if (st->done) return;
    const float gamma = gamma_arg > 0.f ? gamma_arg : st->gamma;
    const float inv_gamma = 1.0f / gamma;               // src/hpwl.rs:166
    const int gl = threadIdx.x & (W - 1);
    constexpr int GPB = kThreads / W;
    float hp_acc = 0.0f;
    for (int base = blockIdx.x * GPB; base < net_count; base += gridDim.x * GPB) {
        const int gid = base + (int)threadIdx.x / W;
        const bool active = gid < net_count;
        const int e = net_begin + gid;
        const int s0 = active ? net_ptr[e] : 0;
        const int deg = active ? net_ptr[e + 1] - s0 : 0;
        float mnx = INFINITY, mxx = -INFINITY, mny = INFINITY, mxy = -INFINITY;
        float px = 0.f, py = 0.f;
        const bool has = !LOOP && gl < deg;
        if (!LOOP) {
            if (has) {
                const int c = slot_cell[s0 + gl];
                const float2 o = slot_off[s0 + gl];
                px = x[c] + o.x;                         // src/hpwl.rs:107
                py = y[c] + o.y;
                mnx = mxx = px;
                mny = mxy = py;
            }
        } else {
            for (int k = gl; k < deg; k += W) {
                const int c = slot_cell[s0 + k];
                const float2 o = slot_off[s0 + k];
                const float qx = x[c] + o.x, qy = y[c] + o.y;
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
            mnx = fminf(def_min_x, mnx); mxx = fmaxf(0.0f, mxx);
            mny = fminf(def_min_y, mny); mxy = fmaxf(0.0f, mxy);
        }
        float ex = 0.f, enx = 0.f, ey = 0.f, eny = 0.f;
        float s_xe = 0.f, s_xen = 0.f, s_e = 0.f, s_en = 0.f;
        float s_ye = 0.f, s_yen = 0.f, s_f = 0.f, s_fn = 0.f;
        if (!LOOP) {
            if (has) {
                ex = expf((px - mxx) * inv_gamma);
                enx = expf((mnx - px) * inv_gamma);
                ey = expf((py - mxy) * inv_gamma);
                eny = expf((mny - py) * inv_gamma);
                s_xe = px * ex; s_xen = px * enx; s_e = ex; s_en = enx;
                s_ye = py * ey; s_yen = py * eny; s_f = ey; s_fn = eny;
            }
        } else {
            for (int k = gl; k < deg; k += W) {
                const int c = slot_cell[s0 + k];
                const float2 o = slot_off[s0 + k];
                const float qx = x[c] + o.x, qy = y[c] + o.y;
                const float a = expf((qx - mxx) * inv_gamma), b = expf((mnx - qx) * inv_gamma);
                const float cc = expf((qy - mxy) * inv_gamma), d = expf((mny - qy) * inv_gamma);
                s_xe += qx * a; s_xen += qx * b; s_e += a; s_en += b;
                s_ye += qy * cc; s_yen += qy * d; s_f += cc; s_fn += d;
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
        // src/hpwl.rs:304-312
        const float one = 1.0f;
        const float b_x = inv_gamma / s_e, a_x = (one - b_x * s_xe) / s_e;
        const float b_nx = -inv_gamma / s_en, a_nx = (one - b_nx * s_xen) / s_en;
        const float b_y = inv_gamma / s_f, a_y = (one - b_y * s_ye) / s_f;
        const float b_ny = -inv_gamma / s_fn, a_ny = (one - b_ny * s_yen) / s_fn;
        if (!LOOP) {
            if (has)
                slot_grad[s0 + gl] = make_float2((a_x + b_x * px) * ex - (a_nx + b_nx * px) * enx,
                                                 (a_y + b_y * py) * ey - (a_ny + b_ny * py) * eny);
        } else {
            for (int k = gl; k < deg; k += W) {
                const int c = slot_cell[s0 + k];
                const float2 o = slot_off[s0 + k];
                const float qx = x[c] + o.x, qy = y[c] + o.y;
                const float a = expf((qx - mxx) * inv_gamma), b = expf((mnx - qx) * inv_gamma);
                const float cc = expf((qy - mxy) * inv_gamma), d = expf((mny - qy) * inv_gamma);
                slot_grad[s0 + k] = make_float2((a_x + b_x * qx) * a - (a_nx + b_nx * qx) * b,
                                                (a_y + b_y * qy) * cc - (a_ny + b_ny * qy) * d);
            }
        }
        if (active && gl == 0) {
            const float hp = (mxx - mnx) + (mxy - mny);   // src/hpwl.rs:302
            net_hpwl[e] = hp;
            hp_acc += hp;
        }
    }
    const double b = block_sum((double)hp_acc, shr);
    if (threadIdx.x == 0) partials[part_off + blockIdx.x] = b;
}

// Sum of all per-block HPWL partials (fixed order) -> DevState.hpwl.
__global__ void k_wl_finalize(const double *__restrict__ partials, int count, DevState *st) {
    __shared__ double shr[kThreads / 32];
    if (st->done) return;
    double v = 0.0;
    for (int k = threadIdx.x; k < count; k += blockDim.x) v += partials[k];
    v = block_sum(v, shr);
    if (threadIdx.x == 0) {
        st->hpwl = v;
        st->hpwl_f = (float)v;
    }
}

// compute_gradients (src/hpwl.rs:113-135): instance gradient = sum of its pin
// gradients in macro_2_pins order; movable instances only.
__global__ void __launch_bounds__(kThreads) k_wl_gather(int NM, const int32_t *__restrict__ ptr,
                                                        const int32_t *__restrict__ slots,
                                                        const float2 *__restrict__ g,
                                                        float *__restrict__ gx, float *__restrict__ gy,
                                                        const DevState *__restrict__ st) {
    if (st->done) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NM; i += gridDim.x * blockDim.x) {
        float sx = 0.0f, sy = 0.0f;
        for (int k = ptr[i], e = ptr[i + 1]; k < e; ++k) {
            const float2 v = g[slots[k]];
            sx += v.x;
            sy += v.y;
        }
        gx[i] = sx;
        gy[i] = sy;
    }
}

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
//  * lanes of a warp walk their contributions in lock-step; lanes that hit the
//    same bin combine their integers first (one atomic per distinct bin per
//    warp step);
//  * each block owns a kWin x kWin bin window in shared memory anchored at its
//    first cell; contributions inside it are accumulated there and flushed with
//    one global atomic per touched bin, the rest go to global memory directly.
// Early on all cells sit within a few bins of the die centre, where this turns
// millions of contended global atomics into a few per block.
constexpr int kWin = 64;
__global__ void __launch_bounds__(kThreads) k_density_scatter(
    int NM, const float *__restrict__ x, const float *__restrict__ y,
    const float *__restrict__ offx, const float *__restrict__ offy, const float *__restrict__ cw,
    const float *__restrict__ ch, const float *__restrict__ ratio, int m, int n, float bw,
    float bh, float inv_bw, float inv_bh, float scale, unsigned long long *__restrict__ map,
    const DevState *__restrict__ st) {
    __shared__ long long sh[kThreads];
    __shared__ unsigned long long win[kWin * kWin];
    __shared__ int s_org[2];
    if (st->done) return;
    const int lane = threadIdx.x & 31;
    const int wbase = threadIdx.x & ~31;
    const int per = ((NM + gridDim.x - 1) / gridDim.x + 31) & ~31;
    const int c0 = blockIdx.x * per, c1 = min(c0 + per, NM);
    if (threadIdx.x == 0) {
        int ox = 0, oy = 0;
        if (c0 < NM) {
            ox = (int)floorf(clamp_bin((x[c0] + offx[c0]) * inv_bw, m)) - kWin / 2;
            oy = (int)floorf(clamp_bin((y[c0] + offy[c0]) * inv_bh, n)) - kWin / 2;
        }
        s_org[0] = max(0, min(ox, m - kWin));
        s_org[1] = max(0, min(oy, n - kWin));
    }
    for (int k = threadIdx.x; k < kWin * kWin; k += blockDim.x) win[k] = 0ull;
    __syncthreads();
    const int wox = s_org[0], woy = s_org[1];
    for (int base = c0; base < c1; base += blockDim.x) {
        const int i = base + threadIdx.x;
        int bxl = 0, byl = 0, nx = 0, ny = 0;
        float xi = 0.f, yi = 0.f, sxi = 0.f, syi = 0.f, r = 0.f;
        if (i < c1) {
            xi = x[i] + offx[i];
            yi = y[i] + offy[i];
            sxi = cw[i];
            syi = ch[i];
            r = ratio[i];
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
        const int cnt = nx * ny;
        const int maxcnt = __reduce_max_sync(0xffffffffu, (unsigned)cnt);
        for (int k = 0; k < maxcnt; ++k) {
            long long c = 0;
            int key = -1;
            if (k < cnt) {
                const int dx = k / ny, dy = k - dx * ny;
                const int bx = bxl + dx, by = byl + dy;
                const float px = r * tri_clamped(xi, sxi, bx, bw);
                const float py = tri_clamped(yi, syi, by, bh);
                c = __float2ll_rn((px * py) * scale);
                key = bx * n + by;
            }
            const unsigned peers = __match_any_sync(0xffffffffu, key);
            sh[threadIdx.x] = c;
            __syncwarp();
            if (key >= 0 && lane == __ffs(peers) - 1) {
                long long s = 0;
                for (unsigned p = peers; p; p &= p - 1) s += sh[wbase + __ffs(p) - 1];
                if (s) {
                    const int bx = key / n, by = key - bx * n;
                    const int wx = bx - wox, wy = by - woy;
                    if (wx >= 0 && wx < kWin && wy >= 0 && wy < kWin)
                        atomicAdd(win + wx * kWin + wy, (unsigned long long)s);
                    else
                        atomicAdd(map + key, (unsigned long long)s);
                }
            }
            __syncwarp();
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < kWin * kWin; k += blockDim.x) {
        const unsigned long long v = win[k];
        const int bx = wox + k / kWin, by = woy + k % kWin;
        if (v && bx < m && by < n) atomicAdd(map + (size_t)bx * n + by, v);
    }
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
            const long long c = __float2ll_rn((px * py) * scale);
            if (c) atomicAdd(acc + (size_t)bx * n + by, (unsigned long long)c);
        }
    }
}

__global__ void k_initial_finalize(size_t mn, unsigned long long *__restrict__ acc, float inv,
                                   float td, float *__restrict__ initial) {
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < mn; k += (size_t)gridDim.x * blockDim.x) {
        const float v = __ll2float_rn((long long)acc[k]) * inv;
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

// Rust `f.to_isize().unwrap_or(0)`: truncation; NaN / out of range -> 0
__device__ __forceinline__ long long to_isize0(float v) {
    if (!(v == v) || v >= 9.2e18f || v <= -9.2e18f) return 0;
    return (long long)v;
}

// compute_electric_force (src/eforce.rs:15-91)
__global__ void __launch_bounds__(kThreads) k_force(
    int NM, const float *__restrict__ x, const float *__restrict__ y,
    const float *__restrict__ offx, const float *__restrict__ offy, const float *__restrict__ cw,
    const float *__restrict__ ch, const float *__restrict__ ratio, int m, int n, float bw,
    float bh, float inv_bw, float inv_bh, const float *__restrict__ fx,
    const float *__restrict__ fy, float *__restrict__ gx_out, float *__restrict__ gy_out,
    const DevState *__restrict__ st) {
    if (st->done) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NM; i += gridDim.x * blockDim.x) {
        const float sx = cw[i], sy = ch[i];
        const float nx = x[i] + offx[i], ny = y[i] + offy[i], r = ratio[i];
        long long xl = to_isize0((nx - 0.0f) * inv_bw);
        if (xl < 0) xl = 0;
        long long xh = to_isize0((nx + sx - 0.0f) * inv_bw) + 1;
        if (xh < 0 || xh > m) xh = m;     // a negative end wraps to usize::MAX, then min
        long long yl = to_isize0((ny - 0.0f) * inv_bh);
        if (yl < 0) yl = 0;
        long long yh = to_isize0((ny + sy - 0.0f) * inv_bh) + 1;
        if (yh < 0 || yh > n) yh = n;
        float gx = 0.0f, gy = 0.0f;
        for (int k = (int)xl; k < (int)xh; ++k) {
            const float px = tri_raw(nx, sx, k, bw);
            const float *rx = fx + (size_t)k * n, *ry = fy + (size_t)k * n;
            for (int hh = (int)yl; hh < (int)yh; ++hh) {
                const float py = tri_raw(ny, sy, hh, bh);
                const float area = px * py;
                gx += area * __ldg(rx + hh);
                gy += area * __ldg(ry + hh);
            }
        }
        gx_out[i] = -gx * r;
        gy_out[i] = -gy * r;
    }
}

// energy = sum psi * rho (src/epotential.rs:344-346), FP64
__global__ void k_energy(size_t mn, const float *__restrict__ psi, const float *__restrict__ rho,
                         double *__restrict__ partials, DevState *st) {
    __shared__ double shr[kThreads / 32];
    double v = 0.0;
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < mn; k += (size_t)gridDim.x * blockDim.x)
        v += (double)(psi[k] * rho[k]);
    const double b = block_sum(v, shr);
    double vals[1] = {b};
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
                                                         const float *__restrict__ dgx,
                                                         const float *__restrict__ dgy,
                                                         double *__restrict__ partials,
                                                         DevState *st) {
    __shared__ double shr[kThreads / 32];
    if (st->done) return;
    const int it = iter_arg >= 0 ? iter_arg : st->iteration;
    if (it != 0) return;
    double a = 0.0, b = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NM; i += gridDim.x * blockDim.x) {
        a += (double)fabsf(wlgx[i]) + (double)fabsf(wlgy[i]);
        b += (double)fabsf(dgx[i]) + (double)fabsf(dgy[i]);
    }
    double vals[2];
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
__global__ void __launch_bounds__(kThreads) k_nesterov_grad(
    int NM, int iter_arg, const float *__restrict__ wlgx, const float *__restrict__ wlgy,
    const float *__restrict__ dgx, const float *__restrict__ dgy, const float *__restrict__ w,
    const float *__restrict__ h, const float *__restrict__ npins, const float *__restrict__ x,
    const float *__restrict__ y, const float *__restrict__ px, const float *__restrict__ py,
    float *__restrict__ pgx, float *__restrict__ pgy, double *__restrict__ partials, DevState *st) {
    __shared__ double shr[kThreads / 32];
    if (st->done) return;
    const float dw = st->dw;
    const float one = 1.0f;
    double num = 0.0, den = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NM; i += gridDim.x * blockDim.x) {
        const float area = w[i] * h[i];
        const float inv_pre = one / fminf(npins[i] + dw * area, one);
        const float gx = (wlgx[i] + dw * dgx[i]) * inv_pre;
        const float gy = (wlgy[i] + dw * dgy[i]) * inv_pre;
        const float dx = x[i] - px[i], dy = y[i] - py[i];
        const float ddx = gx - pgx[i], ddy = gy - pgy[i];
        pgx[i] = gx;
        pgy[i] = gy;
        num += (double)(dx * dx) + (double)(dy * dy);
        den += (double)(ddx * ddx) + (double)(ddy * ddy);
    }
    double vals[2];
    vals[0] = block_sum(num, shr);
    vals[1] = block_sum(den, shr);
    if (arrive_last(partials, blockIdx.x, 2, vals, &st->ctr[CTR_LIP], gridDim.x)) {
        const double tn = sum_partials(partials, gridDim.x, 2, 0, shr);
        const double td = sum_partials(partials, gridDim.x, 2, 1, shr);
        if (threadIdx.x == 0) {
            const int it = iter_arg >= 0 ? iter_arg : st->iteration;
            const float two = one + one, four = two + two;
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

// Lookahead + gradient step + clamp + history (src/nesterov.rs:111-145).
__global__ void __launch_bounds__(kThreads) k_nesterov_update(
    int NM, const float *__restrict__ w, const float *__restrict__ h, float die_w, float die_h,
    float *__restrict__ x, float *__restrict__ y, float *__restrict__ px, float *__restrict__ py,
    const float *__restrict__ gx, const float *__restrict__ gy, const DevState *__restrict__ st) {
    if (st->done) return;
    const float alpha = st->alpha, beta = st->beta, one = 1.0f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NM; i += gridDim.x * blockDim.x) {
        const float xo = x[i], yo = y[i];
        const float xh = xo + beta * (xo - px[i]);
        const float yh = yo + beta * (yo - py[i]);
        const float hx = die_w - w[i] - one, hy = die_h - h[i] - one;
        float nx = xh - alpha * gx[i], ny = yh - alpha * gy[i];
        nx = nx < 0.0f ? 0.0f : (nx > hx ? hx : nx);
        ny = ny < 0.0f ? 0.0f : (ny > hy ? hy : ny);
        px[i] = xo;
        py[i] = yo;
        x[i] = nx;
        y[i] = ny;
    }
}

// ============================ scheduler ============================
// Scheduler::update + should_stop (src/scheduler.rs:68-130) in FP64, plus the
// step record, the non-finite check and the retire-at-overflow flag.
__global__ void k_scheduler(int use_args, float hpwl_arg, float ovf_arg, DevState *st) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    if (st->done) return;
    const float hpwl = use_args ? hpwl_arg : st->hpwl_f;
    const float ovf = use_args ? ovf_arg : st->overflow_f;
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
    const float ref = st->hpwl_init;
    const float delta = st->hpwl_cur - st->hpwl_prev;
    double power;
    if (delta < 0.0f) {
        power = pow(0.9999, (double)st->iteration);
        if (power < 0.98) power = 0.98;
    } else {
        power = pow(1.05, -(double)delta / (double)ref);
        power = power < 0.95 ? 0.95 : (power > 1.05 ? 1.05 : power);
    }
    st->dw = (float)((double)st->dw * (1.05 * power));
    double coef = pow(10.0, ((double)st->ovf_cur - 0.1) * 20.0 / 9.0 - 1.0);
    coef = coef < 0.05 ? 0.05 : (coef > 10.0 ? 10.0 : coef);
    st->gamma = (float)((double)st->base_gamma * coef);
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
}

// ============================ launchers ============================
static int grid_for(int work, int cap = 152 * 8) {
    int g = (work + kThreads - 1) / kThreads;
    return g < 1 ? 1 : (g > cap ? cap : g);
}

void launch_wirelength(Ctx &c, float gamma_arg) {
    int off = 0;
    const float def_min_x = c.die_w + 1.0f, def_min_y = c.die_h + 1.0f;
    for (int k = 0; k < kNumClasses; ++k) {
        const NetClass &nc = c.cls[k];
        if (nc.count == 0) continue;
        const int groups_per_block = kThreads / nc.width;
        int grid = (nc.count + groups_per_block - 1) / groups_per_block;
        if (grid > 1024) grid = 1024;
#define ERP_WA(WW, LL)                                                                                      \
    k_wa<WW, LL><<<grid, kThreads, 0, c.stream>>>(nc.begin, nc.count, nc.general, c.net_ptr, c.slot_cell,   \
                                                  c.slot_off, c.x, c.y, c.slot_grad, c.net_hpwl, c.st,      \
                                                  gamma_arg, def_min_x, def_min_y, c.partials, off)
        switch (k) {
        case 0: ERP_WA(2, false); break;
        case 1: ERP_WA(4, false); break;
        case 2: ERP_WA(8, false); break;
        case 3: ERP_WA(16, false); break;
        case 4: ERP_WA(32, false); break;
        default: ERP_WA(32, true); break;
        }
#undef ERP_WA
        off += grid;
    }
    k_wl_finalize<<<1, kThreads, 0, c.stream>>>(c.partials, off, c.st);
}

void launch_wl_gather(Ctx &c) {
    k_wl_gather<<<grid_for(c.NM), kThreads, 0, c.stream>>>(c.NM, c.cell_slot_ptr, c.cell_slots,
                                                           c.slot_grad, c.wlgx, c.wlgy, c.st);
}

void launch_density_scatter(Ctx &c) {
    k_density_scatter<<<grid_for(c.NM, 152 * 4), kThreads, 0, c.stream>>>(
        c.NM, c.x, c.y, c.offx, c.offy, c.cw, c.ch, c.ratio, c.m, c.n, c.bin_w, c.bin_h, c.inv_bw,
        c.inv_bh, c.fixed_scale, c.dmap, c.st);
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
        cudaMalloc(&dcx, sizeof(float) * c.m);
        cudaMalloc(&dcy, sizeof(float) * c.n);
        cudaMemcpyAsync(dcx, hcx, sizeof(float) * c.m, cudaMemcpyHostToDevice, c.stream);
        cudaMemcpyAsync(dcy, hcy, sizeof(float) * c.n, cudaMemcpyHostToDevice, c.stream);
        k_initial_density<<<count < 4096 ? count : 4096, kThreads, 0, c.stream>>>(
            c.NM, count, c.x, c.y, c.w, c.h, dcx, dcy, c.m, c.n, c.bin_w, c.bin_h, c.inv_bw, c.inv_bh,
            ldexpf(1.0f, c.shift0), c.dmap);
        cudaStreamSynchronize(c.stream);
        cudaFree(dcx);
        cudaFree(dcy);
        delete[] hcx;
        delete[] hcy;
    }
    k_initial_finalize<<<grid_for((int)(mn > (1u << 30) ? (1u << 30) : mn)), kThreads, 0, c.stream>>>(
        mn, c.dmap, ldexpf(1.0f, -c.shift0), c.target_density, c.initial);
}

void launch_force(Ctx &c) {
    k_force<<<grid_for(c.NM, 152 * 16), kThreads, 0, c.stream>>>(
        c.NM, c.x, c.y, c.offx, c.offy, c.cw, c.ch, c.ratio, c.m, c.n, c.bin_w, c.bin_h, c.inv_bw,
        c.inv_bh, c.fx, c.fy, c.dgx, c.dgy, c.st);
}

void launch_energy(Ctx &c) {
    const size_t mn = (size_t)c.m * c.n;
    k_energy<<<grid_for((int)(mn > (1u << 30) ? (1u << 30) : mn)), kThreads, 0, c.stream>>>(
        mn, c.psi, c.rho, c.partials, c.st);
}

void launch_nesterov(Ctx &c, int iter_arg) {
    const int g = grid_for(c.NM);
    k_dw_rescale<<<g, kThreads, 0, c.stream>>>(c.NM, iter_arg, c.wlgx, c.wlgy, c.dgx, c.dgy,
                                               c.partials, c.st);
    k_nesterov_grad<<<g, kThreads, 0, c.stream>>>(c.NM, iter_arg, c.wlgx, c.wlgy, c.dgx, c.dgy, c.w,
                                                  c.h, c.npins, c.x, c.y, c.prev_x, c.prev_y,
                                                  c.prev_gx, c.prev_gy, c.partials, c.st);
    k_nesterov_update<<<g, kThreads, 0, c.stream>>>(c.NM, c.w, c.h, c.die_w, c.die_h, c.x, c.y,
                                                    c.prev_x, c.prev_y, c.prev_gx, c.prev_gy, c.st);
}

void launch_scheduler(Ctx &c, int use_args, float hpwl, float overflow) {
    k_scheduler<<<1, 32, 0, c.stream>>>(use_args, hpwl, overflow, c.st);
}

}  // namespace erp
