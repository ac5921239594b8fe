// Spectral Poisson solve of compute_potential (src/epotential.rs:284-343) as
// three shared-memory FFT passes over the bin grid (row index = x bin, m rows;
// column index = y bin, n columns; src/epotential.rs:237-238):
//
//   R1  rows, length n:    t1 = DCT-II_n(rho)                 (rho fused from the
//                          int64 density map + fixed-cell map, with the overflow sum)
//   C1  columns, length m: A  = (4/(mn)) DCT-II_m(t1); then per column the
//                          weighted spectra A*wu/2k^2, A*wv/2k^2 (and A/k^2) go
//                          through IDXST_m / IDCT_m (/ IDCT_m)       -> tx, ty (tp)
//   R2  rows, length n:    field_x = IDCT_n(tx), field_y = IDXST_n(ty), psi = IDCT_n(tp)
//
// The per-axis transforms are the closed forms of the reference pipelines
// (dct2_fft2 / idxst_idct / idct_idxst / idct2, src/dct2d.rs, src/idct2.rs,
// src/idct_idxst.rs, src/idxst_idct.rs, checked separable by impulse probing):
//   DCT-II  y[k] = sum_i x[i] cos(pi k (2i+1) / 2N)                 (x 2/N per axis)
//   IDCT    y[i] = sum_u c_u X[u] cos(pi u (2i+1) / 2N),  c = (1, 2, 2, ...)
//   IDXST   y[i] = sum_u c_u X[u] sin(pi u (2i+1) / 2N) = (-1)^i IDCT(X')[i],
//           X'[0] = 0, X'[u] = X[N-u]
// Each is computed with Makhoul's length-N complex FFT; two real rows (or
// columns) share one complex FFT (real + imaginary part), since the forward
// input is real and the inverse spectra are Hermitian.  The FFT is an in-place
// radix-2 decimation-in-frequency pass in shared memory (natural order in,
// bit-reversed order out), twiddles from FP64-computed tables.
#include "erp_internal.cuh"
#include "bulk_copy.cuh"
#include "fixedpoint.h"
#include "reduce.cuh"

namespace erp {

__device__ __forceinline__ int brev(int k, int logN) { return (int)(__brev((unsigned)k) >> (32 - logN)); }

// In-place radix-2 DIF over nseq sequences of length N (buf[q*N + i]).
template <bool INV>
__device__ __forceinline__ void fft_dif(float2 *buf, int nseq, int N, int logN, const float2 *tw) {
    const int half = N >> 1;
    const int nbf = nseq * half;
    for (int s = 0; s < logN; ++s) {
        const int lh = logN - 1 - s;
        const int h = 1 << lh;
        for (int b = threadIdx.x; b < nbf; b += blockDim.x) {
            const int q = b >> (logN - 1);
            const int r = b & (half - 1);
            const int j = r & (h - 1);
            const int i0 = (q << logN) + ((r >> lh) << (lh + 1)) + j;
            const int i1 = i0 + h;
            const float2 a = buf[i0], c = buf[i1];
            float2 w = tw[j << s];
            if (INV) w.y = -w.y;
            const float dx = a.x - c.x, dy = a.y - c.y;
            buf[i0] = make_float2(a.x + c.x, a.y + c.y);
            buf[i1] = make_float2(dx * w.x - dy * w.y, dx * w.y + dy * w.x);
        }
        __syncthreads();
    }
}

__device__ __forceinline__ int makhoul_pos(int i, int N) { return (i & 1) ? (N - 1 - (i >> 1)) : (i >> 1); }

// IDCT spectrum Vi[u] = e^{i pi u / 2N} (X[u] - i X[N-u]); e = ek[u] = (cos, -sin)
__device__ __forceinline__ float2 idct_spec(float xu, float xnu, float2 e) {
    const float c = e.x, s = -e.y;
    return make_float2(c * xu + s * xnu, s * xu - c * xnu);
}

// ---------------- R1: rows forward DCT-II ----------------
// PAIRS row pairs per block.  Input either the density map (int64 fixed point +
// fixed-cell map, converted exactly as the oracle replays it) or rho directly.
template <int PAIRS>
__global__ void __launch_bounds__(kThreads) k_rows_dct(
    int m, int n, int logn, const float2 *__restrict__ tw_g, const float2 *__restrict__ ek_n,
    const float *__restrict__ rho_in, unsigned long long *__restrict__ dmap,
    const float *__restrict__ initial, float fixed_inv, float coef, float inv_area, int zero_map,
    float *__restrict__ rho_out, float *__restrict__ t1, double *__restrict__ partials,
    DevState *__restrict__ st, double movable_area) {
    if (st && st->done) return;
    extern __shared__ __align__(16) float2 sm[];
    float2 *tw = sm;
    float2 *buf = sm + (n >> 1);
    __shared__ double shr[kThreads / 32];
    for (int k = threadIdx.x; k < (n >> 1); k += blockDim.x) tw[k] = tw_g[k];
    const int row0 = blockIdx.x * 2 * PAIRS;
    Df ovf = df_zero();
    for (int idx = threadIdx.x; idx < PAIRS * n; idx += blockDim.x) {
        const int p = idx >> logn, i = idx & (n - 1);
        float v[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int r = row0 + 2 * p + h;
            const size_t k = (size_t)r * n + i;
            if (rho_in) {
                v[h] = rho_in[k];
            } else {
                const unsigned long long q = dmap[k];
                if (zero_map) dmap[k] = 0ull;
                // d = (float)sum * 2^-S + initial  (src/density.rs:231-236, fixed point)
                const float d = __fadd_rn(__fmul_rn(fxp_u64_to_float(q), fixed_inv), initial[k]);
                const float o = __fsub_rn(d, coef);
                ovf = df_add(ovf, o > 0.0f ? o : 0.0f);    // src/epotential.rs:274-276
                v[h] = __fmul_rn(d, inv_area);               // src/epotential.rs:284-285
                if (rho_out) rho_out[k] = v[h];
            }
        }
        buf[(p << logn) + makhoul_pos(i, n)] = make_float2(v[0], v[1]);
    }
    __syncthreads();
    fft_dif<false>(buf, PAIRS, n, logn, tw);
    for (int idx = threadIdx.x; idx < PAIRS * n; idx += blockDim.x) {
        const int p = idx >> logn, k = idx & (n - 1);
        const int kk = (n - k) & (n - 1);
        const float2 A = buf[(p << logn) + brev(k, logn)];
        float2 B = buf[(p << logn) + brev(kk, logn)];
        B.y = -B.y;
        const float2 e = ek_n[k];
        const float sx = A.x + B.x, sy = A.y + B.y, dx = A.x - B.x, dy = A.y - B.y;
        const int r = row0 + 2 * p;
        t1[(size_t)r * n + k] = 0.5f * (e.x * sx - e.y * sy);
        t1[(size_t)(r + 1) * n + k] = 0.5f * (e.x * dy + e.y * dx);
    }
    if (!rho_in && partials) {
        const Df vals[1] = {block_sum(ovf, shr)};
        if (arrive_last(partials, blockIdx.x, 1, vals, &st->ctr[CTR_OVF], gridDim.x)) {
            const double tot = sum_partials(partials, gridDim.x, 1, 0, shr);
            if (threadIdx.x == 0) {
                st->overflow = tot;
                st->overflow_f = (float)(tot / movable_area);
                st->ctr[CTR_OVF] = 0;
            }
        }
    }
}

// weights of src/frequencies.rs:4-72 evaluated exactly as the oracle does
__device__ __forceinline__ float inv_k2(int u, int j, const float *wu, const float *wv) {
    if (u == 0 && j == 0) return 0.0f;
    const float s = __fadd_rn(__fmul_rn(wu[u], wu[u]), __fmul_rn(wv[j], wv[j]));
    return __fdiv_rn(1.0f, s);
}

// ---------------- C1: columns DCT-II, weights, inverse along m ----------------
template <int CP>
__global__ void __launch_bounds__(kThreads) k_cols(
    int m, int n, int logm, const float2 *__restrict__ tw_g, const float2 *__restrict__ ek_m,
    const float *__restrict__ wu, const float *__restrict__ wv, const float *__restrict__ t1,
    float *__restrict__ tx, float *__restrict__ ty, float *__restrict__ tp, float scale4,
    const DevState *__restrict__ st) {
    if (st && st->done) return;
    constexpr int CB = 2 * CP;
    extern __shared__ __align__(16) float2 sm[];
    float2 *tw = sm;
    float2 *buf = sm + (m >> 1);
    float *A = reinterpret_cast<float *>(buf + CP * m);
    const int j0 = blockIdx.x * CB;
    for (int k = threadIdx.x; k < (m >> 1); k += blockDim.x) tw[k] = tw_g[k];
    float *bf = reinterpret_cast<float *>(buf);
    for (int idx = threadIdx.x; idx < m * CB; idx += blockDim.x) {
        const int i = idx / CB, c = idx - i * CB;
        const float v = t1[(size_t)i * n + j0 + c];
        bf[2 * (((c >> 1) << logm) + makhoul_pos(i, m)) + (c & 1)] = v;
    }
    __syncthreads();
    fft_dif<false>(buf, CP, m, logm, tw);
    for (int idx = threadIdx.x; idx < CP * m; idx += blockDim.x) {
        const int p = idx >> logm, u = idx & (m - 1);
        const int uu = (m - u) & (m - 1);
        const float2 Az = buf[(p << logm) + brev(u, logm)];
        float2 Bz = buf[(p << logm) + brev(uu, logm)];
        Bz.y = -Bz.y;
        const float2 e = ek_m[u];
        const float sx = Az.x + Bz.x, sy = Az.y + Bz.y, dx = Az.x - Bz.x, dy = Az.y - Bz.y;
        A[(2 * p) * m + u] = scale4 * (0.5f * (e.x * sx - e.y * sy));
        A[(2 * p + 1) * m + u] = scale4 * (0.5f * (e.x * dy + e.y * dx));
    }
    __syncthreads();
    const int nkinds = tp ? 3 : 2;
    for (int kind = 0; kind < nkinds; ++kind) {
        // kind 0: field_x  IDXST_m of A*wu_half; kind 1: field_y IDCT_m of A*wv_half;
        // kind 2: potential IDCT_m of A*inv
        const bool sine = kind == 0;
        for (int idx = threadIdx.x; idx < CP * ((m >> 1) + 1); idx += blockDim.x) {
            const int p = idx / ((m >> 1) + 1), u = idx - p * ((m >> 1) + 1);
            const int un = (m - u) & (m - 1);   // partner index (u = 0 pairs with "m", i.e. zero)
            float2 z_u = make_float2(0.f, 0.f), z_n = make_float2(0.f, 0.f);
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int c = 2 * p + h, j = j0 + c;
                const float a_u = A[c * m + u], a_n = A[c * m + un];
                float wgt_u, wgt_n;
                const float iu = inv_k2(u, j, wu, wv), in_ = inv_k2(un, j, wu, wv);
                if (kind == 0) {
                    wgt_u = __fmul_rn(__fmul_rn(wu[u], iu), 0.5f);
                    wgt_n = __fmul_rn(__fmul_rn(wu[un], in_), 0.5f);
                } else if (kind == 1) {
                    wgt_u = __fmul_rn(__fmul_rn(wv[j], iu), 0.5f);
                    wgt_n = __fmul_rn(__fmul_rn(wv[j], in_), 0.5f);
                } else {
                    wgt_u = iu;
                    wgt_n = in_;
                }
                const float xu = __fmul_rn(a_u, wgt_u);
                const float xn = (u == 0) ? 0.0f : __fmul_rn(a_n, wgt_n);   // X[m] := 0
                float2 vu, vn;
                if (!sine) {
                    vu = idct_spec(xu, xn, ek_m[u]);
                    vn = idct_spec(xn, xu, ek_m[un]);
                } else {
                    vu = (u == 0) ? make_float2(0.f, 0.f) : idct_spec(xn, xu, ek_m[u]);
                    vn = idct_spec(xu, xn, ek_m[un]);
                }
                if (h == 0) {
                    z_u.x += vu.x; z_u.y += vu.y; z_n.x += vn.x; z_n.y += vn.y;
                } else {  // + i * V_b
                    z_u.x -= vu.y; z_u.y += vu.x; z_n.x -= vn.y; z_n.y += vn.x;
                }
            }
            buf[(p << logm) + u] = z_u;
            if (u != 0 && u != (m >> 1)) buf[(p << logm) + un] = z_n;
        }
        __syncthreads();
        fft_dif<true>(buf, CP, m, logm, tw);
        float *out = kind == 0 ? tx : (kind == 1 ? ty : tp);
        for (int idx = threadIdx.x; idx < m * CB; idx += blockDim.x) {
            const int i = idx / CB, c = idx - i * CB;
            const int t = i >> 1, src = (i & 1) ? (m - 1 - t) : t;
            const float2 w = buf[((c >> 1) << logm) + brev(src, logm)];
            float v = (c & 1) ? w.y : w.x;
            if (sine && (i & 1)) v = -v;
            out[(size_t)i * n + j0 + c] = v;
        }
        __syncthreads();
    }
}

// ---------------- R2: rows inverse along n ----------------
template <int PAIRS>
__global__ void __launch_bounds__(kThreads) k_rows_inv(
    int m, int n, int logn, const float2 *__restrict__ tw_g, const float2 *__restrict__ ek_n,
    const float *__restrict__ tx, const float *__restrict__ ty, const float *__restrict__ tp,
    float *__restrict__ fx, float *__restrict__ fy, float *__restrict__ psi,
    const DevState *__restrict__ st) {
    if (st && st->done) return;
    extern __shared__ __align__(16) float2 sm[];
    float2 *tw = sm;
    float2 *buf = sm + (n >> 1);
    for (int k = threadIdx.x; k < (n >> 1); k += blockDim.x) tw[k] = tw_g[k];
    const int row0 = blockIdx.x * 2 * PAIRS;
    const int nkinds = tp ? 3 : 2;
    for (int kind = 0; kind < nkinds; ++kind) {
        // kind 0: field_x = IDCT_n(tx); kind 1: field_y = IDXST_n(ty); kind 2: psi = IDCT_n(tp)
        const float *in = kind == 0 ? tx : (kind == 1 ? ty : tp);
        float *out = kind == 0 ? fx : (kind == 1 ? fy : psi);
        const bool sine = kind == 1;
        for (int idx = threadIdx.x; idx < PAIRS * n; idx += blockDim.x) {
            const int p = idx >> logn, i = idx & (n - 1);
            const int r = row0 + 2 * p;
            buf[idx] = make_float2(in[(size_t)r * n + i], in[(size_t)(r + 1) * n + i]);
        }
        __syncthreads();
        for (int idx = threadIdx.x; idx < PAIRS * ((n >> 1) + 1); idx += blockDim.x) {
            const int p = idx / ((n >> 1) + 1), u = idx - p * ((n >> 1) + 1);
            const int un = (n - u) & (n - 1);
            const float2 xu2 = buf[(p << logn) + u];
            const float2 xn2 = (u == 0) ? make_float2(0.f, 0.f) : buf[(p << logn) + un];
            float2 z_u = make_float2(0.f, 0.f), z_n = make_float2(0.f, 0.f);
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const float xu = h ? xu2.y : xu2.x, xn = h ? xn2.y : xn2.x;
                float2 vu, vn;
                if (!sine) {
                    vu = idct_spec(xu, xn, ek_n[u]);
                    vn = idct_spec(xn, xu, ek_n[un]);
                } else {
                    vu = (u == 0) ? make_float2(0.f, 0.f) : idct_spec(xn, xu, ek_n[u]);
                    vn = idct_spec(xu, xn, ek_n[un]);
                }
                if (h == 0) {
                    z_u.x += vu.x; z_u.y += vu.y; z_n.x += vn.x; z_n.y += vn.y;
                } else {
                    z_u.x -= vu.y; z_u.y += vu.x; z_n.x -= vn.y; z_n.y += vn.x;
                }
            }
            buf[(p << logn) + u] = z_u;
            if (u != 0 && u != (n >> 1)) buf[(p << logn) + un] = z_n;
        }
        __syncthreads();
        fft_dif<true>(buf, PAIRS, n, logn, tw);
        for (int idx = threadIdx.x; idx < PAIRS * n; idx += blockDim.x) {
            const int p = idx >> logn, i = idx & (n - 1);
            const int t = i >> 1, src = (i & 1) ? (n - 1 - t) : t;
            const float2 w = buf[(p << logn) + brev(src, logn)];
            float va = w.x, vb = w.y;
            if (sine && (i & 1)) { va = -va; vb = -vb; }
            const int r = row0 + 2 * p;
            out[(size_t)r * n + i] = va;
            out[(size_t)(r + 1) * n + i] = vb;
        }
        __syncthreads();
    }
}

// ===================================================================
// Warp-level four-step FFT for N = 32 * E points (E = 1..32), one warp per
// complex sequence: lane l holds r[k] = z[l + 32k].
//   1. E-point DIF FFT in registers over k        (twiddles W_E = W_N^32)
//   2. twiddle W_N^(l*q)
//   3. 32-point DIF across lanes with xor shuffles (twiddles W_32 = W_N^E)
// after which lane l, register j holds Z[brev_E(j) + E * brev_5(l)].  The
// result is staged in shared memory in natural order under an XOR swizzle
// (index f -> f ^ ((f >> 5) & 31)) that keeps both the scattered store and the
// row-order reads at two wavefronts per 64-bit warp access.
// ===================================================================
__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ int swz(int f) { return f ^ ((f >> 5) & 31); }

template <int E>
__host__ __device__ constexpr int brev_c(int v) {
    int r = 0;
    for (int b = 1; b < E; b <<= 1) r = (r << 1) | ((v & b) ? 1 : 0);
    return r;
}

// tw holds W_{S N}^k (k < S N / 2); the N-point transform uses W_N^i = tw[S i].
template <int E, bool INV, int S = 1>
__device__ __forceinline__ void warp_fft(float2 (&r)[E], const float2 *__restrict__ tw, int lane) {
    constexpr int N = 32 * E;
    // 1. registers
#pragma unroll
    for (int h = E / 2; h >= 1; h >>= 1) {
#pragma unroll
        for (int i0 = 0; i0 < E; ++i0) {
            if (i0 & h) continue;
            const int i1 = i0 + h, j = i0 & (h - 1);
            float2 w = tw[S * 32 * j * (E / (2 * h))];
            if (INV) w.y = -w.y;
            const float2 u = r[i0], v = r[i1];
            r[i0] = make_float2(u.x + v.x, u.y + v.y);
            r[i1] = cmulf(make_float2(u.x - v.x, u.y - v.y), w);
        }
    }
    // 2. twiddles
#pragma unroll
    for (int j = 0; j < E; ++j) {
        const int q = brev_c<E>(j);
        if (q == 0) continue;
        const int idx = lane * q;
        float2 w = idx < N / 2 ? tw[S * idx] : tw[S * (idx - N / 2)];
        if (idx >= N / 2) { w.x = -w.x; w.y = -w.y; }
        if (INV) w.y = -w.y;
        r[j] = cmulf(r[j], w);
    }
    // 3. across lanes
#pragma unroll
    for (int s = 0; s < 5; ++s) {
        const int h = 16 >> s;
        const bool upper = (lane & h) != 0;
        float2 w = tw[S * E * ((lane & (h - 1)) * (16 / h))];
        if (INV) w.y = -w.y;
#pragma unroll
        for (int j = 0; j < E; ++j) {
            const float2 v = r[j];
            const float2 p = make_float2(__shfl_xor_sync(0xffffffffu, v.x, h),
                                         __shfl_xor_sync(0xffffffffu, v.y, h));
            r[j] = upper ? cmulf(make_float2(p.x - v.x, p.y - v.y), w) : make_float2(v.x + p.x, v.y + p.y);
        }
    }
}

// stage the FFT result in natural (swizzled) order
template <int E>
__device__ __forceinline__ void warp_fft_store(const float2 (&r)[E], float2 *buf, int lane) {
    const int pl = (int)(__brev((unsigned)lane) >> 27);
#pragma unroll
    for (int j = 0; j < E; ++j) buf[swz(brev_c<E>(j) + E * pl)] = r[j];
}

// Block-cooperative staging of the per-axis tables in shared memory: the
// half-size FFT's twiddles e^{-2 pi i k / H} = tw_N[2k] (k < H/2), the N-point
// twiddles tw_N (k < N/2) and the DCT post-twiddles ek (k < N), N = 2H.
struct AxisTables {
    float2 *twh, *tw, *ek;
};
template <int NW, int H>
__device__ __forceinline__ AxisTables load_tables(float2 *base, const float2 *__restrict__ tw_g,
                                                  const float2 *__restrict__ ek_g) {
    AxisTables t;
    t.twh = base;
    t.tw = base + H / 2;
    t.ek = base + H / 2 + H;
    for (int k = threadIdx.x; k < H / 2; k += NW * 32) t.twh[k] = tw_g[2 * k];
    for (int k = threadIdx.x; k < H; k += NW * 32) t.tw[k] = tw_g[k];
    for (int k = threadIdx.x; k < 2 * H; k += NW * 32) t.ek[k] = ek_g[k];
    return t;
}
template <int H>
constexpr int tables_f2() { return H / 2 + H + 2 * H; }

// Real DCT-II of the N = 2H values staged at their Makhoul positions in xm
// (v[p] at xm[p]): one H-point complex FFT over z[j] = v[2j] + i v[2j+1], then
// V[k] = E[k] + W_N^k O[k] and y[k] = Re(e^{-i pi k / 2N} V[k]).  Calls emit(k, y)
// for every k in [0, N), each exactly once across the warp.
template <int E, typename Emit>
__device__ __forceinline__ void warp_dct2_real(const float *xm, float2 *zb, const float2 *twh,
                                               const float2 *tw_n, const float2 *ek, int lane, Emit emit) {
    constexpr int H = 32 * E, N = 2 * H;
    float2 r[E];
    const float2 *xm2 = reinterpret_cast<const float2 *>(xm);
#pragma unroll
    for (int k = 0; k < E; ++k) r[k] = xm2[lane + 32 * k];
    warp_fft<E, false>(r, twh, lane);
    warp_fft_store<E>(r, zb, lane);
    __syncwarp();
#pragma unroll 4
    for (int k = lane; k <= H; k += 32) {
        const float2 zk = zb[swz(k & (H - 1))];
        float2 zc = zb[swz((H - k) & (H - 1))];
        zc.y = -zc.y;
        const float2 ev = make_float2(0.5f * (zk.x + zc.x), 0.5f * (zk.y + zc.y));
        const float2 od = make_float2(0.5f * (zk.y - zc.y), -0.5f * (zk.x - zc.x));
        const float2 w = k < H ? tw_n[k] : make_float2(-1.0f, 0.0f);
        const float2 v = make_float2(ev.x + (w.x * od.x - w.y * od.y), ev.y + (w.x * od.y + w.y * od.x));
        const float2 e = ek[k];
        emit(k, e.x * v.x - e.y * v.y);
        if (k > 0 && k < H) {
            const float2 e2 = ek[N - k];
            emit(N - k, e2.x * v.x + e2.y * v.y);
        }
    }
}

// Inverse along one axis of N = 2H real values, IDCT (sine = false) or IDXST
// (sine = true): x(u) returns X[u] for u in [0, N) (the caller's weighted
// input); the Hermitian spectrum Vi is folded into one H-point complex IFFT
// (Fe = Vi[k] + Vi[k+H], Fo = (Vi[k] - Vi[k+H]) e^{+2 pi i k / N}), whose real
// and imaginary parts are w[2j] and w[2j+1].  Calls emit(i, out_i) for every
// output index i in [0, N), each exactly once across the warp.
template <int E, typename XFn, typename Emit>
__device__ __forceinline__ void warp_inv_real(XFn x, bool sine, float2 *zb, const float2 *twh,
                                              const float2 *tw_n, const float2 *ek, int lane, Emit emit) {
    constexpr int H = 32 * E, N = 2 * H;
    float2 r[E];
#pragma unroll 4
    for (int t = 0; t < E; ++t) {
        const int k = lane + 32 * t;
        float2 v[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int u = k + h * H;
            const int un = N - u;   // in (0, N]; X[N] := 0
            const float xu = x(u);
            const float xn = (un == N) ? 0.0f : x(un);
            if (!sine) v[h] = idct_spec(xu, xn, ek[u]);
            else v[h] = (u == 0) ? make_float2(0.f, 0.f) : idct_spec(xn, xu, ek[u]);
        }
        const float2 fe = make_float2(v[0].x + v[1].x, v[0].y + v[1].y);
        const float2 d = make_float2(v[0].x - v[1].x, v[0].y - v[1].y);
        const float2 w = tw_n[k];   // e^{-2 pi i k / N}; Fo = d * conj(w)
        const float2 fo = make_float2(d.x * w.x + d.y * w.y, d.y * w.x - d.x * w.y);
        r[t] = make_float2(fe.x - fo.y, fe.y + fo.x);
    }
    warp_fft<E, true>(r, twh, lane);
    warp_fft_store<E>(r, zb, lane);
    __syncwarp();
#pragma unroll 8
    for (int i = lane; i < N; i += 32) {
        const int p = (i & 1) ? (N - 1 - (i >> 1)) : (i >> 1);
        const float2 z = zb[swz(p >> 1)];
        float val = (p & 1) ? z.y : z.x;
        if (sine && (i & 1)) val = -val;
        emit(i, val);
    }
}

// R1 (warp form): rows forward DCT-II, one warp per row.  From the fixed-point
// map, lane 0 of each warp first issues two bulk copies (the row's int64 sums
// into the warp's work area, the row of the initial map into its stage area)
// on the warp's mbarrier, so the whole row arrives at copy bandwidth while the
// block loads the axis tables; the lanes then convert from shared memory and
// zero the row with 16-byte stores.
struct RowsDctWP {
    int m;
    const float2 * tw_n;
    const float2 * ek_n;
    const float * rho_in;
    unsigned long long * dmap;
    const float * initial;
    float fixed_inv;
    float coef;
    float inv_area;
    int zero_map;
    float * rho_out;
    float * t1;
    double * partials;
    DevState * st;
    double movable_area;
};
template <int E, int NW>
__device__ __forceinline__ void rows_dct_w_body(const RowsDctWP &p, int bid, int nblk) {
    int m = p.m;
    const float2 *__restrict__ tw_n = p.tw_n;
    const float2 *__restrict__ ek_n = p.ek_n;
    const float *__restrict__ rho_in = p.rho_in;
    unsigned long long *__restrict__ dmap = p.dmap;
    const float *__restrict__ initial = p.initial;
    float fixed_inv = p.fixed_inv;
    float coef = p.coef;
    float inv_area = p.inv_area;
    int zero_map = p.zero_map;
    float *__restrict__ rho_out = p.rho_out;
    float *__restrict__ t1 = p.t1;
    double *__restrict__ partials = p.partials;
    DevState *__restrict__ st = p.st;
    double movable_area = p.movable_area;
    constexpr int H = 32 * E, N = 2 * H;
    if (st && st->done) return;
    extern __shared__ __align__(16) float2 sm[];
    __shared__ __align__(8) uint64_t bar[NW];
    __shared__ double shr[NW];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int row = bid * NW + warp;
    float2 *wbase = sm + tables_f2<H>() + warp * 3 * H;   // [2H float2 work | N float stage]
    float *xm = reinterpret_cast<float *>(wbase);
    float2 *zb = wbase + H;
    float *ini_s = reinterpret_cast<float *>(wbase + 2 * H);
    const bool from_map = rho_in == nullptr;
    if (from_map && lane == 0) {
        mbar_init(&bar[warp], 1);
        mbar_expect_tx(&bar[warp], 12u * N);
        bulk_load(wbase, dmap + (size_t)row * N, 8u * N, &bar[warp]);
        bulk_load(ini_s, initial + (size_t)row * N, 4u * N, &bar[warp]);
    }
    __syncwarp();
    const AxisTables tb = load_tables<NW, H>(sm, tw_n, ek_n);
    Df ovf = df_zero();
    if (from_map) {
        if (!mbar_wait(&bar[warp], 0, (st && st->expire_waits) ? 0u : kWaitTries)) {
            if (lane == 0 && st) {
                atomicOr(&st->status, kStatusWaitTimeout);
                st->done = 1;
            }
            mbar_wait(&bar[warp], 0);   // the copy must land before the area is reused
        }
        const unsigned long long *q_s = reinterpret_cast<const unsigned long long *>(wbase);
        float v[2 * E];
        Df ov4[4] = {df_zero(), df_zero(), df_zero(), df_zero()};   // four independent chains
#pragma unroll
        for (int t = 0; t < 2 * E; ++t) {
            const int i = lane + 32 * t;
            // d = (float)sum * 2^-S + initial  (src/density.rs:231-236, fixed point)
            const float d = __fadd_rn(__fmul_rn(fxp_u64_to_float(q_s[i]), fixed_inv), ini_s[i]);
            const float o = __fsub_rn(d, coef);
            ov4[t & 3] = df_add(ov4[t & 3], o > 0.0f ? o : 0.0f);   // src/epotential.rs:274-276
            v[t] = __fmul_rn(d, inv_area);                    // src/epotential.rs:284-285
        }
        ovf = df_add(df_add(ov4[0], ov4[1]), df_add(ov4[2], ov4[3]));
        if (zero_map) {
            ulonglong2 *zr = reinterpret_cast<ulonglong2 *>(dmap + (size_t)row * N);
#pragma unroll
            for (int k = 0; k < N / 64; ++k) zr[lane + 32 * k] = make_ulonglong2(0ull, 0ull);
        }
        if (rho_out) {
#pragma unroll
            for (int t = 0; t < 2 * E; ++t) rho_out[(size_t)row * N + lane + 32 * t] = v[t];
        }
        __syncwarp();   // every lane has read the staged row before xm overwrites it
#pragma unroll
        for (int t = 0; t < 2 * E; ++t) xm[makhoul_pos(lane + 32 * t, N)] = v[t];
    } else {
#pragma unroll 8
        for (int t = 0; t < 2 * E; ++t) {
            const int i = lane + 32 * t;
            xm[makhoul_pos(i, N)] = rho_in[(size_t)row * N + i];
        }
    }
    __syncthreads();   // twiddles + staged rows
    float *out = t1 + (size_t)row * N;
    warp_dct2_real<E>(xm, zb, tb.twh, tb.tw, tb.ek, lane, [&](int k, float y) { out[k] = y; });
    if (from_map && partials) {
        const Df vals[1] = {block_sum(ovf, shr)};
        if (arrive_last(partials, bid, 1, vals, &st->ctr[CTR_OVF], nblk)) {
            const double tot = sum_partials(partials, nblk, 1, 0, shr);
            if (threadIdx.x == 0) {
                st->overflow = tot;
                st->overflow_f = (float)(tot / movable_area);
                st->ctr[CTR_OVF] = 0;
            }
        }
    }
}
template <int E, int NW>
__global__ void __launch_bounds__(NW * 32) k_rows_dct_w(const __grid_constant__ RowsDctWP p) { rows_dct_w_body<E, NW>(p, blockIdx.x, gridDim.x); }


// C1 (warp form): NW columns per block, one warp per column.  Coalesced tile
// load, forward DCT-II along x, A and the column's 1/(wu^2+wv^2) kept in shared
// memory (one division per bin), then for each output kind the weighted inverse
// along x and a coalesced tile store.
struct ColsWP {
    int n;
    const float2 * tw_m;
    const float2 * ek_m;
    const float * wu_g;
    const float * wv;
    const float * t1;
    float * tx;
    float * ty;
    float * tp;
    float scale4;
    const DevState * st;
};
template <int E, int NW>
__device__ __forceinline__ void cols_w_body(const ColsWP &p, int bid, int nblk) {
    int n = p.n;
    const float2 *__restrict__ tw_m = p.tw_m;
    const float2 *__restrict__ ek_m = p.ek_m;
    const float *__restrict__ wu_g = p.wu_g;
    const float *__restrict__ wv = p.wv;
    const float *__restrict__ t1 = p.t1;
    float *__restrict__ tx = p.tx;
    float *__restrict__ ty = p.ty;
    float *__restrict__ tp = p.tp;
    float scale4 = p.scale4;
    const DevState *__restrict__ st = p.st;
    constexpr int H = 32 * E, M = 2 * H;
    constexpr int S = NW + 1;   // tile row stride (odd: conflict-free row-wise access)
    if (st && st->done) return;
    extern __shared__ __align__(16) float2 sm[];
    const AxisTables tb = load_tables<NW, H>(sm, tw_m, ek_m);
    const float2 *twh = tb.twh;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float *ab = reinterpret_cast<float *>(sm + tables_f2<H>() + warp * 3 * H);   // Makhoul staging, then A
    float *ib = ab + M;                                                          // 1/(wu^2 + wv^2)
    float2 *zb = reinterpret_cast<float2 *>(ib + M);                             // FFT staging
    float *wu = reinterpret_cast<float *>(sm + tables_f2<H>() + NW * 3 * H);
    float *tile = wu + M;
    const int j0 = bid * NW;
    for (int k = threadIdx.x; k < M; k += NW * 32) wu[k] = wu_g[k];
    for (int idx = threadIdx.x; idx < M * NW; idx += NW * 32) {
        const int i = idx / NW, c = idx - i * NW;
        tile[i * S + c] = t1[(size_t)i * n + j0 + c];
    }
    __syncthreads();
    const int j = j0 + warp;
    for (int i = lane; i < M; i += 32) ab[makhoul_pos(i, M)] = tile[i * S + warp];
    __syncwarp();
    // forward: results into registers first, then into ab (its Makhoul staging is
    // consumed by the FFT's register load before the post-processing writes)
    {
        float2 r[E];
        const float2 *ab2 = reinterpret_cast<const float2 *>(ab);
#pragma unroll
        for (int k = 0; k < E; ++k) r[k] = ab2[lane + 32 * k];
        warp_fft<E, false>(r, twh, lane);
        warp_fft_store<E>(r, zb, lane);
        __syncwarp();
#pragma unroll 4
        for (int k = lane; k <= H; k += 32) {
            const float2 zk = zb[swz(k & (H - 1))];
            float2 zc = zb[swz((H - k) & (H - 1))];
            zc.y = -zc.y;
            const float2 ev = make_float2(0.5f * (zk.x + zc.x), 0.5f * (zk.y + zc.y));
            const float2 od = make_float2(0.5f * (zk.y - zc.y), -0.5f * (zk.x - zc.x));
            const float2 w = k < H ? tb.tw[k] : make_float2(-1.0f, 0.0f);
            const float2 v = make_float2(ev.x + (w.x * od.x - w.y * od.y), ev.y + (w.x * od.y + w.y * od.x));
            const float2 e = tb.ek[k];
            ab[k] = scale4 * (e.x * v.x - e.y * v.y);
            ib[k] = inv_k2(k, j, wu, wv);
            if (k > 0 && k < H) {
                const float2 e2 = tb.ek[M - k];
                ab[M - k] = scale4 * (e2.x * v.x + e2.y * v.y);
                ib[M - k] = inv_k2(M - k, j, wu, wv);
            }
        }
        __syncwarp();
    }
    const float wvj = wv[j];
    const int nkinds = tp ? 3 : 2;
#pragma unroll 1
    for (int kind = 0; kind < nkinds; ++kind) {
        // kind 0: field_x  IDXST_x of A * wu / 2k^2   (src/idxst_idct.rs, src/frequencies.rs:52-58)
        // kind 1: field_y  IDCT_x  of A * wv / 2k^2   (src/idct_idxst.rs, src/frequencies.rs:60-66)
        // kind 2: potential IDCT_x of A / k^2          (src/idct2.rs)
        auto xfn = [&](int u) -> float {
            const float iv = ib[u];
            float wgt;
            if (kind == 0) wgt = __fmul_rn(__fmul_rn(wu[u], iv), 0.5f);
            else if (kind == 1) wgt = __fmul_rn(__fmul_rn(wvj, iv), 0.5f);
            else wgt = iv;
            return __fmul_rn(ab[u], wgt);
        };
        warp_inv_real<E>(xfn, kind == 0, zb, twh, tb.tw, tb.ek, lane,
                         [&](int i, float v) { tile[i * S + warp] = v; });
        __syncthreads();
        float *out = kind == 0 ? tx : (kind == 1 ? ty : tp);
        for (int idx = threadIdx.x; idx < M * NW; idx += NW * 32) {
            const int i = idx / NW, c = idx - i * NW;
            out[(size_t)i * n + j0 + c] = tile[i * S + c];
        }
        __syncthreads();
    }
}
template <int E, int NW>
__global__ void __launch_bounds__(NW * 32) k_cols_w(const __grid_constant__ ColsWP p) { cols_w_body<E, NW>(p, blockIdx.x, gridDim.x); }


// R2 (warp form): rows inverse along y, one warp per (row, output kind).
struct RowsInvWP {
    int m;
    int nkinds;
    const float2 * tw_n;
    const float2 * ek_n;
    const float * tx;
    const float * ty;
    const float * tp;
    float * fx;
    float * fy;
    float * psi;
    const DevState * st;
};
template <int E, int NW>
__device__ __forceinline__ void rows_inv_w_body(const RowsInvWP &p, int bid, int nblk) {
    int m = p.m;
    int nkinds = p.nkinds;
    const float2 *__restrict__ tw_n = p.tw_n;
    const float2 *__restrict__ ek_n = p.ek_n;
    const float *__restrict__ tx = p.tx;
    const float *__restrict__ ty = p.ty;
    const float *__restrict__ tp = p.tp;
    float *__restrict__ fx = p.fx;
    float *__restrict__ fy = p.fy;
    float *__restrict__ psi = p.psi;
    const DevState *__restrict__ st = p.st;
    constexpr int H = 32 * E, N = 2 * H;
    if (st && st->done) return;
    extern __shared__ __align__(16) float2 sm[];
    const AxisTables tb = load_tables<NW, H>(sm, tw_n, ek_n);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float *xb = reinterpret_cast<float *>(sm + tables_f2<H>() + warp * 2 * H);
    float2 *zb = sm + tables_f2<H>() + warp * 2 * H + H;
    __syncthreads();
    const int task = bid * NW + warp;
    const int row = task / nkinds, kind = task - row * nkinds;
    // kind 0: field_x = IDCT_y(tx); kind 1: field_y = IDXST_y(ty); kind 2: psi = IDCT_y(tp)
    const float *in = (kind == 0 ? tx : (kind == 1 ? ty : tp)) + (size_t)row * N;
    float *out = (kind == 0 ? fx : (kind == 1 ? fy : psi)) + (size_t)row * N;
#pragma unroll 8
    for (int t = 0; t < 2 * E; ++t) xb[lane + 32 * t] = in[lane + 32 * t];
    __syncwarp();
    warp_inv_real<E>([&](int u) { return xb[u]; }, kind == 1, zb, tb.twh, tb.tw, tb.ek, lane,
                     [&](int i, float v) { out[i] = v; });
}
template <int E, int NW>
__global__ void __launch_bounds__(NW * 32) k_rows_inv_w(const __grid_constant__ RowsInvWP p) { rows_inv_w_body<E, NW>(p, blockIdx.x, gridDim.x); }


// ===================================================================
// Group transforms: kQ = 4 warps per sequence (sides 512..2048).  At a 1024^2
// grid there are only 1024 rows or columns, about seven per SM, so one warp
// per sequence leaves the SMs latency bound; splitting each sequence over four
// warps gives four times the warps, each with a quarter of the serial work.
//
// H-point FFT, H = M kQ, M = 32 E, by decimation in frequency: input index
// n = n2 + M q, output index k = k1 + kQ k2 (q, k1 < kQ; n2, k2 < M):
//   a_k1[n2]        = W_H^(n2 k1) sum_q W_kQ^(q k1) z[n2 + M q]   (any thread)
//   Z[k1 + kQ k2]   = sum_n2 W_M^(n2 k2) a_k1[n2]                 (warp k1)
// The first stage reads and writes consecutive elements across lanes; the only
// strided access, the final scatter to natural order, goes through the XOR
// swizzle xsw (two wavefronts per 64-bit warp access for E = 2, 4, 8).  The
// group synchronises with a named barrier of its 128 threads (ids 1..).
// ===================================================================
constexpr int kQ = 4;

__device__ __forceinline__ void group_bar(int id) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(kQ * 32) : "memory");
}

__device__ __forceinline__ int xsw(int f) { return f ^ ((f >> 5) & 15); }

// W_H^idx, 0 <= idx < H, from the half table tw (k < H/2)
template <int H>
__device__ __forceinline__ float2 tw_full(const float2 *tw, int idx) {
    float2 w = idx < H / 2 ? tw[idx] : tw[idx - H / 2];
    if (idx >= H / 2) { w.x = -w.x; w.y = -w.y; }
    return w;
}

// zin(n) gives z[n] (n < H); on exit xs[xsw(k)] = Z[k] for every k < H,
// visible to the whole group.  ys, xs: H float2 each; twh: W_H^k, k < H/2.
template <int E, bool INV, typename ZIn>
__device__ __forceinline__ void group_fft(ZIn zin, const float2 *twh, float2 *ys, float2 *xs, int q, int lane,
                                          int gt, int bar) {
    constexpr int M = 32 * E, H = M * kQ;
#pragma unroll
    for (int n2 = gt; n2 < M; n2 += 32 * kQ) {
        const float2 a0 = zin(n2), a1 = zin(n2 + M), a2 = zin(n2 + 2 * M), a3 = zin(n2 + 3 * M);
        const float2 s0 = make_float2(a0.x + a2.x, a0.y + a2.y), s1 = make_float2(a0.x - a2.x, a0.y - a2.y);
        const float2 s2 = make_float2(a1.x + a3.x, a1.y + a3.y), s3 = make_float2(a1.x - a3.x, a1.y - a3.y);
        float2 x1, x3;
        if (!INV) {   // W_4 = -i
            x1 = make_float2(s1.x + s3.y, s1.y - s3.x);
            x3 = make_float2(s1.x - s3.y, s1.y + s3.x);
        } else {      // W_4 = +i
            x1 = make_float2(s1.x - s3.y, s1.y + s3.x);
            x3 = make_float2(s1.x + s3.y, s1.y - s3.x);
        }
        float2 w1 = tw_full<H>(twh, n2), w2 = tw_full<H>(twh, 2 * n2), w3 = tw_full<H>(twh, 3 * n2);
        if (INV) { w1.y = -w1.y; w2.y = -w2.y; w3.y = -w3.y; }
        ys[n2] = make_float2(s0.x + s2.x, s0.y + s2.y);
        ys[M + n2] = cmulf(x1, w1);
        ys[2 * M + n2] = cmulf(make_float2(s0.x - s2.x, s0.y - s2.y), w2);
        ys[3 * M + n2] = cmulf(x3, w3);
    }
    group_bar(bar);
    float2 r[E];
#pragma unroll
    for (int j = 0; j < E; ++j) r[j] = ys[q * M + lane + 32 * j];
    warp_fft<E, INV, kQ>(r, twh, lane);
    const int pl = (int)(__brev((unsigned)lane) >> 27);
#pragma unroll
    for (int j = 0; j < E; ++j) xs[xsw(q + kQ * (brev_c<E>(j) + E * pl))] = r[j];
    group_bar(bar);
}

// DCT-II post-processing (as warp_dct2_real) from the group FFT of the
// Makhoul-ordered row: emit(k, y[k]) for every k < N across the group.
template <int H, typename Emit>
__device__ __forceinline__ void group_dct2_post(const float2 *xs, const float2 *tw_n, const float2 *ek, int gt,
                                                Emit emit) {
    constexpr int N = 2 * H;
#pragma unroll 2
    for (int k = gt; k <= H; k += 32 * kQ) {
        const float2 zk = xs[xsw(k & (H - 1))];
        float2 zc = xs[xsw((H - k) & (H - 1))];
        zc.y = -zc.y;
        const float2 ev = make_float2(0.5f * (zk.x + zc.x), 0.5f * (zk.y + zc.y));
        const float2 od = make_float2(0.5f * (zk.y - zc.y), -0.5f * (zk.x - zc.x));
        const float2 w = k < H ? tw_n[k] : make_float2(-1.0f, 0.0f);
        const float2 v = make_float2(ev.x + (w.x * od.x - w.y * od.y), ev.y + (w.x * od.y + w.y * od.x));
        const float2 e = ek[k];
        emit(k, e.x * v.x - e.y * v.y);
        if (k > 0 && k < H) {
            const float2 e2 = ek[N - k];
            emit(N - k, e2.x * v.x + e2.y * v.y);
        }
    }
}

// Inverse along one axis (as warp_inv_real) by a group: x(u) gives X[u]; the
// folded Hermitian spectrum is formed inside the group FFT's first stage.
template <int E, typename XFn, typename Emit>
__device__ __forceinline__ void group_inv_real(XFn x, bool sine, float2 *ys, float2 *xs, const float2 *twh,
                                               const float2 *tw_n, const float2 *ek, int q, int lane, int gt,
                                               int bar, Emit emit) {
    constexpr int H = 32 * E * kQ, N = 2 * H;
    auto zin = [&](int k) -> float2 {
        float2 v[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int u = k + h * H;
            const int un = N - u;   // in (0, N]; X[N] := 0
            const float xu = x(u);
            const float xn = (un == N) ? 0.0f : x(un);
            if (!sine) v[h] = idct_spec(xu, xn, ek[u]);
            else v[h] = (u == 0) ? make_float2(0.f, 0.f) : idct_spec(xn, xu, ek[u]);
        }
        const float2 fe = make_float2(v[0].x + v[1].x, v[0].y + v[1].y);
        const float2 d = make_float2(v[0].x - v[1].x, v[0].y - v[1].y);
        const float2 w = tw_n[k];   // e^{-2 pi i k / N}; Fo = d * conj(w)
        const float2 fo = make_float2(d.x * w.x + d.y * w.y, d.y * w.x - d.x * w.y);
        return make_float2(fe.x - fo.y, fe.y + fo.x);
    };
    group_fft<E, true>(zin, twh, ys, xs, q, lane, gt, bar);
#pragma unroll 4
    for (int i = gt; i < N; i += 32 * kQ) {
        const int p = (i & 1) ? (N - 1 - (i >> 1)) : (i >> 1);
        const float2 z = xs[xsw(p >> 1)];
        float val = (p & 1) ? z.y : z.x;
        if (sine && (i & 1)) val = -val;
        emit(i, val);
    }
}

// R1 (group form): rows forward DCT-II, one group of four warps per row, G rows
// per block.  Per group: [0, 2H) the row's int64 sums (bulk copy), later the
// Makhoul staging xm in [0, H) and xs in [H, 2H); [2H, 3H) the row of the
// initial map (bulk copy); [3H, 4H) ys.
template <int E, int G>
__global__ void __launch_bounds__(G * kQ * 32) k_rows_dct_g(
    int m, const float2 *__restrict__ tw_n, const float2 *__restrict__ ek_n,
    const float *__restrict__ rho_in, unsigned long long *__restrict__ dmap,
    const float *__restrict__ initial, float fixed_inv, float coef, float inv_area, int zero_map,
    float *__restrict__ rho_out, float *__restrict__ t1, double *__restrict__ partials,
    DevState *__restrict__ st, double movable_area) {
    constexpr int H = 32 * E * kQ, N = 2 * H, PT = N / (32 * kQ);   // values per thread
    if (st && st->done) return;
    extern __shared__ __align__(16) float2 sm[];
    __shared__ __align__(8) uint64_t bar[G];
    __shared__ double shr[G * kQ];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int grp = warp / kQ, q = warp % kQ, gt = q * 32 + lane, gbar = 1 + grp;
    const int row = blockIdx.x * G + grp;
    float2 *gbase = sm + tables_f2<H>() + grp * 4 * H;
    float *xm = reinterpret_cast<float *>(gbase);
    float2 *xs = gbase + H;
    float *ini_s = reinterpret_cast<float *>(gbase + 2 * H);
    float2 *ys = gbase + 3 * H;
    const bool from_map = rho_in == nullptr;
    if (from_map && gt == 0) {
        mbar_init(&bar[grp], 1);
        mbar_expect_tx(&bar[grp], 12u * N);
        bulk_load(gbase, dmap + (size_t)row * N, 8u * N, &bar[grp]);
        bulk_load(ini_s, initial + (size_t)row * N, 4u * N, &bar[grp]);
    }
    const AxisTables tb = load_tables<G * kQ, H>(sm, tw_n, ek_n);
    __syncthreads();   // tables; the group's barrier initialisation
    Df ovf = df_zero();
    float v[PT];
    if (from_map) {
        if (!mbar_wait(&bar[grp], 0, (st && st->expire_waits) ? 0u : kWaitTries)) {
            if (gt == 0 && st) {
                atomicOr(&st->status, kStatusWaitTimeout);
                st->done = 1;
            }
            mbar_wait(&bar[grp], 0);   // the copy must land before the area is reused
        }
        const unsigned long long *q_s = reinterpret_cast<const unsigned long long *>(gbase);
        Df ov2[2] = {df_zero(), df_zero()};
#pragma unroll
        for (int t = 0; t < PT; ++t) {
            const int i = gt + 32 * kQ * t;
            // d = (float)sum * 2^-S + initial  (src/density.rs:231-236, fixed point)
            const float d = __fadd_rn(__fmul_rn(fxp_u64_to_float(q_s[i]), fixed_inv), ini_s[i]);
            const float o = __fsub_rn(d, coef);
            ov2[t & 1] = df_add(ov2[t & 1], o > 0.0f ? o : 0.0f);   // src/epotential.rs:274-276
            v[t] = __fmul_rn(d, inv_area);                   // src/epotential.rs:284-285
        }
        ovf = df_add(ov2[0], ov2[1]);
        if (zero_map) {
            ulonglong2 *zr = reinterpret_cast<ulonglong2 *>(dmap + (size_t)row * N);
#pragma unroll
            for (int k = 0; k < N / (64 * kQ); ++k) zr[gt + 32 * kQ * k] = make_ulonglong2(0ull, 0ull);
        }
        if (rho_out) {
#pragma unroll
            for (int t = 0; t < PT; ++t) rho_out[(size_t)row * N + gt + 32 * kQ * t] = v[t];
        }
    } else {
#pragma unroll
        for (int t = 0; t < PT; ++t) v[t] = rho_in[(size_t)row * N + gt + 32 * kQ * t];
    }
    group_bar(gbar);   // the staged row is consumed: xm may overwrite it
#pragma unroll
    for (int t = 0; t < PT; ++t) {
        const int i = gt + 32 * kQ * t;
        xm[makhoul_pos(i, N)] = v[t];
    }
    group_bar(gbar);
    const float2 *xm2 = reinterpret_cast<const float2 *>(xm);
    group_fft<E, false>([&](int i) { return xm2[i]; }, tb.twh, ys, xs, q, lane, gt, gbar);
    float *out = t1 + (size_t)row * N;
    group_dct2_post<H>(xs, tb.tw, tb.ek, gt, [&](int k, float y) { out[k] = y; });
    if (from_map && partials) {
        const Df vals[1] = {block_sum(ovf, shr)};
        if (arrive_last(partials, blockIdx.x, 1, vals, &st->ctr[CTR_OVF], gridDim.x)) {
            const double tot = sum_partials(partials, gridDim.x, 1, 0, shr);
            if (threadIdx.x == 0) {
                st->overflow = tot;
                st->overflow_f = (float)(tot / movable_area);
                st->ctr[CTR_OVF] = 0;
            }
        }
    }
}

// C1 (group form): G columns per block, one group per column.  Coalesced tile
// load, forward DCT-II along x into A (shared), 1/(wu^2+wv^2) per bin, then for
// each output kind the weighted inverse along x and a coalesced tile store.
// Per group: ab [0, H) (Makhoul staging, then A, as floats), ib [H, 2H) (floats),
// ys [2H, 3H), xs [3H, 4H).
template <int E, int G>
__global__ void __launch_bounds__(G * kQ * 32) k_cols_g(
    int n, const float2 *__restrict__ tw_m, const float2 *__restrict__ ek_m,
    const float *__restrict__ wu_g, const float *__restrict__ wv, const float *__restrict__ t1,
    float *__restrict__ tx, float *__restrict__ ty, float *__restrict__ tp, float scale4,
    const DevState *__restrict__ st) {
    constexpr int H = 32 * E * kQ, M = 2 * H, S = G + 1;   // tile row stride (odd)
    if (st && st->done) return;
    extern __shared__ __align__(16) float2 sm[];
    const AxisTables tb = load_tables<G * kQ, H>(sm, tw_m, ek_m);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int grp = warp / kQ, q = warp % kQ, gt = q * 32 + lane, gbar = 1 + grp;
    float2 *gbase = sm + tables_f2<H>() + grp * 4 * H;
    float *ab = reinterpret_cast<float *>(gbase);
    float *ib = reinterpret_cast<float *>(gbase + H);
    float2 *ys = gbase + 2 * H, *xs = gbase + 3 * H;
    float *wu = reinterpret_cast<float *>(sm + tables_f2<H>() + G * 4 * H);
    float *tile = wu + M;
    const int j0 = blockIdx.x * G;
    for (int k = threadIdx.x; k < M; k += blockDim.x) wu[k] = wu_g[k];
    for (int idx = threadIdx.x; idx < M * G; idx += blockDim.x) {
        const int i = idx / G, c = idx - i * G;
        tile[i * S + c] = t1[(size_t)i * n + j0 + c];
    }
    __syncthreads();
    const int j = j0 + grp;
    for (int i = gt; i < M; i += 32 * kQ) ab[makhoul_pos(i, M)] = tile[i * S + grp];
    group_bar(gbar);
    {
        const float2 *ab2 = reinterpret_cast<const float2 *>(ab);
        group_fft<E, false>([&](int i) { return ab2[i]; }, tb.twh, ys, xs, q, lane, gt, gbar);   // ab's staging is consumed
        group_dct2_post<H>(xs, tb.tw, tb.ek, gt, [&](int k, float y) {
            ab[k] = scale4 * y;
            ib[k] = inv_k2(k, j, wu, wv);
        });
        group_bar(gbar);
    }
    const float wvj = wv[j];
    const int nkinds = tp ? 3 : 2;
#pragma unroll 1
    for (int kind = 0; kind < nkinds; ++kind) {
        // kind 0: field_x  IDXST_x of A * wu / 2k^2   (src/idxst_idct.rs, src/frequencies.rs:52-58)
        // kind 1: field_y  IDCT_x  of A * wv / 2k^2   (src/idct_idxst.rs, src/frequencies.rs:60-66)
        // kind 2: potential IDCT_x of A / k^2          (src/idct2.rs)
        auto xfn = [&](int u) -> float {
            const float iv = ib[u];
            float wgt;
            if (kind == 0) wgt = __fmul_rn(__fmul_rn(wu[u], iv), 0.5f);
            else if (kind == 1) wgt = __fmul_rn(__fmul_rn(wvj, iv), 0.5f);
            else wgt = iv;
            return __fmul_rn(ab[u], wgt);
        };
        group_inv_real<E>(xfn, kind == 0, ys, xs, tb.twh, tb.tw, tb.ek, q, lane, gt, gbar,
                          [&](int i, float v) { tile[i * S + grp] = v; });
        __syncthreads();
        float *out = kind == 0 ? tx : (kind == 1 ? ty : tp);
        for (int idx = threadIdx.x; idx < M * G; idx += blockDim.x) {
            const int i = idx / G, c = idx - i * G;
            out[(size_t)i * n + j0 + c] = tile[i * S + c];
        }
        __syncthreads();
    }
}

// R2 (group form): rows inverse along y, one group per (row, output kind), G
// tasks per block.  Per group: xb [0, H) (the input row as floats; later xs),
// ys [H, 2H).
template <int E, int G>
__global__ void __launch_bounds__(G * kQ * 32) k_rows_inv_g(
    int m, int nkinds, const float2 *__restrict__ tw_n, const float2 *__restrict__ ek_n,
    const float *__restrict__ tx, const float *__restrict__ ty, const float *__restrict__ tp,
    float *__restrict__ fx, float *__restrict__ fy, float *__restrict__ psi,
    const DevState *__restrict__ st) {
    constexpr int H = 32 * E * kQ, N = 2 * H;
    if (st && st->done) return;
    extern __shared__ __align__(16) float2 sm[];
    const AxisTables tb = load_tables<G * kQ, H>(sm, tw_n, ek_n);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int grp = warp / kQ, q = warp % kQ, gt = q * 32 + lane, gbar = 1 + grp;
    float2 *gbase = sm + tables_f2<H>() + grp * 2 * H;
    float *xb = reinterpret_cast<float *>(gbase);
    float2 *xs = gbase, *ys = gbase + H;   // xs reuses xb once the spectrum is folded
    const int task = blockIdx.x * G + grp;
    const int row = task / nkinds, kind = task - row * nkinds;
    // kind 0: field_x = IDCT_y(tx); kind 1: field_y = IDXST_y(ty); kind 2: psi = IDCT_y(tp)
    const float *in = (kind == 0 ? tx : (kind == 1 ? ty : tp)) + (size_t)row * N;
    float *out = (kind == 0 ? fx : (kind == 1 ? fy : psi)) + (size_t)row * N;
#pragma unroll
    for (int t = 0; t < N / (32 * kQ); ++t) xb[gt + 32 * kQ * t] = in[gt + 32 * kQ * t];
    __syncthreads();   // tables and the staged rows
    group_inv_real<E>([&](int u) { return xb[u]; }, kind == 1, ys, xs, tb.twh, tb.tw, tb.ek, q, lane, gt,
                      gbar, [&](int i, float v) { out[i] = v; });
}

// The density map as rho for the tensor-core solve: the conversion of R1 (same
// float rules, so rho is bit-identical to what the FFT path transforms), the
// double-float overflow sum with the last-block finalize, and the map zeroing.
__global__ void __launch_bounds__(kThreads) k_map_rho(size_t mn, unsigned long long *__restrict__ dmap,
                                                      const float *__restrict__ initial, float fixed_inv, float coef,
                                                      float inv_area, int zero_map, float *__restrict__ rho,
                                                      double *__restrict__ partials, DevState *__restrict__ st,
                                                      double movable_area) {
    __shared__ double shr[kThreads / 32];
    if (st->done) return;
    Df ovf = df_zero();
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < mn; idx += (size_t)gridDim.x * blockDim.x) {
        const unsigned long long q = dmap[idx];
        if (zero_map) dmap[idx] = 0ull;
        // d = (float)sum * 2^-S + initial  (src/density.rs:231-236, fixed point)
        const float d = __fadd_rn(__fmul_rn(fxp_u64_to_float(q), fixed_inv), initial[idx]);
        const float o = __fsub_rn(d, coef);
        ovf = df_add(ovf, o > 0.0f ? o : 0.0f);  // src/epotential.rs:274-276
        rho[idx] = __fmul_rn(d, inv_area);         // src/epotential.rs:284-285
    }
    const Df vals[1] = {block_sum(ovf, shr)};
    if (arrive_last(partials, blockIdx.x, 1, vals, &st->ctr[CTR_OVF], gridDim.x)) {
        const double tot = sum_partials(partials, gridDim.x, 1, 0, shr);
        if (threadIdx.x == 0) {
            st->overflow = tot;
            st->overflow_f = (float)(tot / movable_area);
            st->ctr[CTR_OVF] = 0;
        }
    }
}

void launch_map_rho(const SpectralArgs &a, size_t mn, float *rho, cudaStream_t s) {
    size_t g = (mn + kThreads - 1) / kThreads;
    if (g > 152 * 8) g = 152 * 8;
    k_map_rho<<<(int)g, kThreads, 0, s>>>(mn, a.dmap, a.initial, a.fixed_inv, a.coef, a.inv_bin_area,
                                          a.zero_map ? 1 : 0, rho, a.partials, a.st, a.movable_area);
}

int ilog2(int v) {
    int l = 0;
    while ((1 << l) < v) ++l;
    return l;
}

static size_t rows_smem(int n, int pairs) { return sizeof(float2) * ((size_t)(n >> 1) + (size_t)pairs * n); }
static size_t cols_smem(int m, int cp) {
    return sizeof(float2) * ((size_t)(m >> 1) + (size_t)cp * m) + sizeof(float) * (size_t)(2 * cp) * m;
}

constexpr int kRowPairs = 2;

static int col_pairs(int m) { return m <= 2048 ? 4 : 2; }

// Host-computed tables (FP64 angles rounded to FP32) uploaded to the given
// arrays; pageable copies, so the host buffers can go as soon as the calls return.
void spectral_tables_fill(int m, int n, float bin_w, float bin_h, float2 *tw_m, float2 *tw_n, float2 *ek_m,
                          float2 *ek_n, float *wu, float *wv, cudaStream_t s) {
    auto tw = [](int N) {
        std::vector<float2> h(N / 2);
        for (int k = 0; k < N / 2; ++k) {
            double a = -2.0 * 3.14159265358979323846 * (double)k / (double)N;
            h[k] = make_float2((float)cos(a), (float)sin(a));
        }
        return h;
    };
    auto ek = [](int N) {
        std::vector<float2> h(N);
        for (int k = 0; k < N; ++k) {
            double a = 3.14159265358979323846 * (double)k / (2.0 * N);
            h[k] = make_float2((float)cos(a), (float)-sin(a));
        }
        return h;
    };
    const std::vector<float2> h_twm = tw(m), h_twn = tw(n), h_ekm = ek(m), h_ekn = ek(n);
    std::vector<float> h_wu(m), h_wv(n);
    const float tpm = (float)(2.0 * 3.14159265358979323846) / (float)m;
    for (int i = 0; i < m; ++i) h_wu[i] = (float)i * tpm;
    const float wv_div = bin_w / bin_h;
    const float tpn = (float)(2.0 * 3.14159265358979323846) / (float)n;
    for (int j = 0; j < n; ++j) h_wv[j] = ((float)j * tpn) * wv_div;
    cudaMemcpyAsync(tw_m, h_twm.data(), sizeof(float2) * (m / 2), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(tw_n, h_twn.data(), sizeof(float2) * (n / 2), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(ek_m, h_ekm.data(), sizeof(float2) * m, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(ek_n, h_ekn.data(), sizeof(float2) * n, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(wu, h_wu.data(), sizeof(float) * m, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(wv, h_wv.data(), sizeof(float) * n, cudaMemcpyHostToDevice, s);
}

void spectral_tables(int m, int n, float bin_w, float bin_h, float2 **tw_m, float2 **tw_n,
                     float2 **ek_m, float2 **ek_n, float **wu, float **wv, cudaStream_t s) {
    ctx_alloc((void **)tw_m, sizeof(float2) * (m / 2), s);
    ctx_alloc((void **)tw_n, sizeof(float2) * (n / 2), s);
    ctx_alloc((void **)ek_m, sizeof(float2) * m, s);
    ctx_alloc((void **)ek_n, sizeof(float2) * n, s);
    ctx_alloc((void **)wu, sizeof(float) * m, s);
    ctx_alloc((void **)wv, sizeof(float) * n, s);
    spectral_tables_fill(m, n, bin_w, bin_h, *tw_m, *tw_n, *ek_m, *ek_n, *wu, *wv, s);
    cudaStreamSynchronize(s);
}

constexpr int kRowWarps = 4;   // rows per block, warp kernels
constexpr int kColWarps = 4;   // columns per block, warp kernels

// warp kernels cover N = 64 * E, E = 1..32 (sides 64..2048); NW sequences per
// block (kRowWarps / kColWarps unless a batch's autotuner chose otherwise)
template <int E, int NW = kRowWarps>
static size_t rows_w_smem() { return sizeof(float2) * (size_t)(tables_f2<32 * E>() + NW * 64 * E); }
template <int E, int NW = kRowWarps>
static size_t rows_dct_w_smem() { return sizeof(float2) * (size_t)(tables_f2<32 * E>() + NW * 96 * E); }
template <int E, int NW = kColWarps>
static size_t cols_w_smem() {
    return sizeof(float2) * (size_t)(tables_f2<32 * E>() + NW * 96 * E) + sizeof(float) * (size_t)(64 * E) * (NW + 2);
}

template <int E, int RW = kRowWarps, int CW = kColWarps>
static cudaError_t prepare_w() {
    cudaError_t e = cudaFuncSetAttribute(k_rows_dct_w<E, RW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rows_dct_w_smem<E, RW>());
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_rows_inv_w<E, RW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rows_w_smem<E, RW>());
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_cols_w<E, CW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cols_w_smem<E, CW>());
    return e;
}
// The sequences-per-block alternatives a batch's autotuner can choose for the
// sides it times (64..256, where the warp kernels run): SpectralPlan::seqs.

// group kernels: sides 512..2048 (E = side / 256), G sequences per block
constexpr int kRowGroups = 2, kColGroups = 4, kInvGroups = 4;
static bool group_side(int v) { return v >= 512 && v <= 2048; }
template <int E>
static size_t rows_dct_g_smem() { return sizeof(float2) * (size_t)(tables_f2<128 * E>() + kRowGroups * 4 * 128 * E); }
template <int E>
static size_t cols_g_smem() {
    return sizeof(float2) * (size_t)(tables_f2<128 * E>() + kColGroups * 4 * 128 * E) +
           sizeof(float) * (size_t)(256 * E) * (kColGroups + 2);
}
template <int E>
static size_t rows_inv_g_smem() { return sizeof(float2) * (size_t)(tables_f2<128 * E>() + kInvGroups * 2 * 128 * E); }
template <int E>
static cudaError_t prepare_g() {
    cudaError_t e = cudaFuncSetAttribute(k_rows_dct_g<E, kRowGroups>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)rows_dct_g_smem<E>());
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_cols_g<E, kColGroups>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)cols_g_smem<E>());
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_rows_inv_g<E, kInvGroups>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)rows_inv_g_smem<E>());
    return e;
}
template <int E>
static void rows_dct_g(const SpectralPlan &p, const SpectralArgs &a, bool from_map) {
    k_rows_dct_g<E, kRowGroups><<<p.m / kRowGroups, kRowGroups * kQ * 32, rows_dct_g_smem<E>(), p.stream>>>(
        p.m, p.tw_n, p.ek_n, a.rho_in, a.dmap, a.initial, a.fixed_inv, a.coef, a.inv_bin_area,
        a.zero_map ? 1 : 0, a.rho_out, p.t1, from_map ? a.partials : nullptr, a.st, a.movable_area);
}
template <int E>
static void cols_g(const SpectralPlan &p, const SpectralArgs &a, float scale4, float *tp) {
    k_cols_g<E, kColGroups><<<p.n / kColGroups, kColGroups * kQ * 32, cols_g_smem<E>(), p.stream>>>(
        p.n, p.tw_m, p.ek_m, p.wu, p.wv, p.t1, p.tx, p.ty, tp, scale4, a.st);
}
template <int E>
static void rows_inv_g(const SpectralPlan &p, const SpectralArgs &a, float *tp) {
    const int nk = tp ? 3 : 2;
    k_rows_inv_g<E, kInvGroups><<<p.m * nk / kInvGroups, kInvGroups * kQ * 32, rows_inv_g_smem<E>(), p.stream>>>(
        p.m, nk, p.tw_n, p.ek_n, p.tx, p.ty, tp, a.fx, a.fy, a.psi, a.st);
}
#define ERP_DISPATCH_G(side, FN, ...)           \
    switch (side) {                             \
    case 512: FN<2>(__VA_ARGS__); break;        \
    case 1024: FN<4>(__VA_ARGS__); break;       \
    default: FN<8>(__VA_ARGS__); break;         \
    }

// Opt the spectral kernels into large dynamic shared memory on the current device.
cudaError_t spectral_prepare() {
    cudaError_t e = cudaFuncSetAttribute(k_rows_dct<kRowPairs>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_rows_inv<kRowPairs>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_cols<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_cols<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
    if (e == cudaSuccess) e = prepare_w<1>();
    if (e == cudaSuccess) e = prepare_w<2>();
    if (e == cudaSuccess) e = prepare_w<4>();
    if (e == cudaSuccess) e = prepare_w<8>();
    if (e == cudaSuccess) e = prepare_w<16>();
    if (e == cudaSuccess) e = prepare_w<32>();
    if (e == cudaSuccess) e = prepare_w<1, kSeqCandidates[0], kSeqCandidates[0]>();
    if (e == cudaSuccess) e = prepare_w<2, kSeqCandidates[0], kSeqCandidates[0]>();
    if (e == cudaSuccess) e = prepare_w<4, kSeqCandidates[0], kSeqCandidates[0]>();
    if (e == cudaSuccess) e = prepare_w<1, kSeqCandidates[1], kSeqCandidates[1]>();
    if (e == cudaSuccess) e = prepare_w<2, kSeqCandidates[1], kSeqCandidates[1]>();
    if (e == cudaSuccess) e = prepare_w<4, kSeqCandidates[1], kSeqCandidates[1]>();
    if (e == cudaSuccess) e = prepare_g<2>();
    if (e == cudaSuccess) e = prepare_g<4>();
    if (e == cudaSuccess) e = prepare_g<8>();
    return e;
}

size_t spectral_smem_bytes(int m, int n) {
    size_t a = rows_smem(n, kRowPairs), b = cols_smem(m, col_pairs(m));
    return a > b ? a : b;
}

static bool warp_side(int v) { return v >= 64 && v <= 2048; }


template <int E, int NW>
static void rows_dct_w_nw(const SpectralPlan &p, const SpectralArgs &a, bool from_map) {
    k_rows_dct_w<E, NW><<<p.m / NW, NW * 32, rows_dct_w_smem<E, NW>(), p.stream>>>(RowsDctWP{
        p.m, p.tw_n, p.ek_n, a.rho_in, a.dmap, a.initial, a.fixed_inv, a.coef, a.inv_bin_area,
        a.zero_map ? 1 : 0, a.rho_out, p.t1, from_map ? a.partials : nullptr, a.st, a.movable_area});
}
template <int E, int NW>
static void cols_w_nw(const SpectralPlan &p, const SpectralArgs &a, float scale4, float *tp) {
    k_cols_w<E, NW><<<p.n / NW, NW * 32, cols_w_smem<E, NW>(), p.stream>>>(ColsWP{
        p.n, p.tw_m, p.ek_m, p.wu, p.wv, p.t1, p.tx, p.ty, tp, scale4, a.st});
}
template <int E, int NW>
static void rows_inv_w_nw(const SpectralPlan &p, const SpectralArgs &a, float *tp) {
    const int nk = tp ? 3 : 2;
    k_rows_inv_w<E, NW><<<p.m * nk / NW, NW * 32, rows_w_smem<E, NW>(), p.stream>>>(RowsInvWP{
        p.m, nk, p.tw_n, p.ek_n, p.tx, p.ty, tp, a.fx, a.fy, a.psi, a.st});
}
// the plan's sequences per block: an autotuned alternative (sides 64..256) or
// the fixed shape
template <int E>
static void rows_dct_w(const SpectralPlan &p, const SpectralArgs &a, bool from_map) {
    if constexpr (E <= 4) {
        if (p.seqs == kSeqCandidates[0]) return rows_dct_w_nw<E, kSeqCandidates[0]>(p, a, from_map);
        if (p.seqs == kSeqCandidates[1]) return rows_dct_w_nw<E, kSeqCandidates[1]>(p, a, from_map);
    }
    rows_dct_w_nw<E, kRowWarps>(p, a, from_map);
}
template <int E>
static void cols_w(const SpectralPlan &p, const SpectralArgs &a, float scale4, float *tp) {
    if constexpr (E <= 4) {
        if (p.seqs == kSeqCandidates[0]) return cols_w_nw<E, kSeqCandidates[0]>(p, a, scale4, tp);
        if (p.seqs == kSeqCandidates[1]) return cols_w_nw<E, kSeqCandidates[1]>(p, a, scale4, tp);
    }
    cols_w_nw<E, kColWarps>(p, a, scale4, tp);
}
template <int E>
static void rows_inv_w(const SpectralPlan &p, const SpectralArgs &a, float *tp) {
    if constexpr (E <= 4) {
        if (p.seqs == kSeqCandidates[0]) return rows_inv_w_nw<E, kSeqCandidates[0]>(p, a, tp);
        if (p.seqs == kSeqCandidates[1]) return rows_inv_w_nw<E, kSeqCandidates[1]>(p, a, tp);
    }
    rows_inv_w_nw<E, kRowWarps>(p, a, tp);
}

#define ERP_DISPATCH_E(side, FN, ...)           \
    switch (side) {                             \
    case 64: FN<1>(__VA_ARGS__); break;         \
    case 128: FN<2>(__VA_ARGS__); break;        \
    case 256: FN<4>(__VA_ARGS__); break;        \
    case 512: FN<8>(__VA_ARGS__); break;        \
    case 1024: FN<16>(__VA_ARGS__); break;      \
    default: FN<32>(__VA_ARGS__); break;        \
    }

void launch_spectral_plan(const SpectralPlan &p, const SpectralArgs &a) {
    const int m = p.m, n = p.n;
    const bool from_map = a.rho_in == nullptr;
    const int rb = m / (2 * kRowPairs);
    if (group_side(n)) {
        ERP_DISPATCH_G(n, rows_dct_g, p, a, from_map);
    } else if (warp_side(n)) {
        ERP_DISPATCH_E(n, rows_dct_w, p, a, from_map);
    } else {
        k_rows_dct<kRowPairs><<<rb, kThreads, rows_smem(n, kRowPairs), p.stream>>>(
            m, n, p.logn, p.tw_n, p.ek_n, a.rho_in, a.dmap, a.initial, a.fixed_inv, a.coef,
            a.inv_bin_area, a.zero_map ? 1 : 0, a.rho_out, p.t1, from_map ? a.partials : nullptr, a.st,
            a.movable_area);
    }
    const float scale4 = 4.0f / (float)((double)m * (double)n);
    float *tp = a.psi ? p.tp : nullptr;
    if (group_side(m)) {
        ERP_DISPATCH_G(m, cols_g, p, a, scale4, tp);
    } else if (warp_side(m)) {
        ERP_DISPATCH_E(m, cols_w, p, a, scale4, tp);
    } else if (col_pairs(m) == 4) {
        k_cols<4><<<n / 8, kThreads, cols_smem(m, 4), p.stream>>>(m, n, p.logm, p.tw_m, p.ek_m, p.wu,
                                                                  p.wv, p.t1, p.tx, p.ty, tp, scale4,
                                                                  a.st);
    } else {
        k_cols<2><<<n / 4, kThreads, cols_smem(m, 2), p.stream>>>(m, n, p.logm, p.tw_m, p.ek_m, p.wu,
                                                                  p.wv, p.t1, p.tx, p.ty, tp, scale4,
                                                                  a.st);
    }
    if (group_side(n)) {
        ERP_DISPATCH_G(n, rows_inv_g, p, a, tp);
    } else if (warp_side(n)) {
        ERP_DISPATCH_E(n, rows_inv_w, p, a, tp);
    } else {
        k_rows_inv<kRowPairs><<<rb, kThreads, rows_smem(n, kRowPairs), p.stream>>>(
            m, n, p.logn, p.tw_n, p.ek_n, p.tx, p.ty, tp, a.fx, a.fy, a.psi, a.st);
    }
}

// ---- packed launches of the warp-form passes (batches) ----
// Sides 64..256: each pass of many solves in one launch per (E, NW) in use.
static int packed_nw(const SpectralPlan &p, int E, int fixed) {
    return (E <= 4 && (p.seqs == kSeqCandidates[0] || p.seqs == kSeqCandidates[1])) ? p.seqs : fixed;
}

template <typename P>
static void plan_spectral(PackKind k, int variant, const std::vector<const SpectralJob *> &js, PackedArena &ar,
                          std::vector<PackedLaunch> &out, size_t smem, int threads,
                          P (*params)(const SpectralJob &, int &grid)) {
    std::vector<P> tab;
    std::vector<int32_t> block0(1, 0);
    for (const SpectralJob *j : js) {
        int g = 0;
        tab.push_back(params(*j, g));
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

template <int E, int NW>
static RowsDctWP rows_dct_w_params(const SpectralJob &j, int &grid) {
    const SpectralPlan &p = j.p;
    const SpectralArgs &a = j.a;
    grid = p.m / NW;
    return RowsDctWP{p.m, p.tw_n, p.ek_n, a.rho_in, a.dmap, a.initial, a.fixed_inv, a.coef, a.inv_bin_area,
                     a.zero_map ? 1 : 0, a.rho_out, p.t1, a.rho_in == nullptr ? a.partials : nullptr, a.st,
                     a.movable_area};
}
template <int E, int NW>
static ColsWP cols_w_params(const SpectralJob &j, int &grid) {
    const SpectralPlan &p = j.p;
    const SpectralArgs &a = j.a;
    grid = p.n / NW;
    return ColsWP{p.n, p.tw_m, p.ek_m, p.wu, p.wv, p.t1, p.tx, p.ty, a.psi ? p.tp : nullptr,
                  4.0f / (float)((double)p.m * (double)p.n), a.st};
}
template <int E, int NW>
static RowsInvWP rows_inv_w_params(const SpectralJob &j, int &grid) {
    const SpectralPlan &p = j.p;
    const SpectralArgs &a = j.a;
    const int nk = a.psi ? 3 : 2;
    grid = p.m * nk / NW;
    return RowsInvWP{p.m, nk, p.tw_n, p.ek_n, p.tx, p.ty, a.psi ? p.tp : nullptr, a.fx, a.fy, a.psi, a.st};
}

template <int E, int NW>
static void plan_spectral_en(PackKind k, const std::vector<const SpectralJob *> &js, PackedArena &ar,
                             std::vector<PackedLaunch> &out) {
    const int variant = E * 16 + NW;
    if (k == PK_ROWS_DCT_W)
        plan_spectral<RowsDctWP>(k, variant, js, ar, out, rows_dct_w_smem<E, NW>(), NW * 32, rows_dct_w_params<E, NW>);
    else if (k == PK_COLS_W)
        plan_spectral<ColsWP>(k, variant, js, ar, out, cols_w_smem<E, NW>(), NW * 32, cols_w_params<E, NW>);
    else
        plan_spectral<RowsInvWP>(k, variant, js, ar, out, rows_w_smem<E, NW>(), NW * 32, rows_inv_w_params<E, NW>);
}

template <int E>
static void plan_spectral_e(PackKind k, int NW, const std::vector<const SpectralJob *> &js, PackedArena &ar,
                            std::vector<PackedLaunch> &out) {
    switch (NW) {
    case kSeqCandidates[0]: plan_spectral_en<E, kSeqCandidates[0]>(k, js, ar, out); break;
    case kSeqCandidates[1]: plan_spectral_en<E, kSeqCandidates[1]>(k, js, ar, out); break;
    default: plan_spectral_en<E, kRowWarps>(k, js, ar, out); break;
    }
}

void packed_spectral_stage(PackKind k, const std::vector<SpectralJob> &v, PackedArena &ar,
                           std::vector<PackedLaunch> &out) {
    static_assert(kRowWarps == kColWarps, "one fixed shape for rows and columns");
    for (int E : {1, 2, 4}) {
        for (int NW : {kSeqCandidates[0], kRowWarps, kSeqCandidates[1]}) {
            std::vector<const SpectralJob *> js;
            for (const SpectralJob &j : v) {
                const int side = k == PK_COLS_W ? j.p.m : j.p.n;
                if (side != 64 * E) continue;
                if (packed_nw(j.p, E, kRowWarps) != NW) continue;
                js.push_back(&j);
            }
            if (js.empty()) continue;
            if (E == 1) plan_spectral_e<1>(k, NW, js, ar, out);
            else if (E == 2) plan_spectral_e<2>(k, NW, js, ar, out);
            else plan_spectral_e<4>(k, NW, js, ar, out);
        }
    }
}

template <int E, int NW>
static void packed_spectral_launch_en(const PackedLaunch &l, const unsigned char *dev, cudaStream_t s) {
    if (l.kind == PK_ROWS_DCT_W)
        k_packed<RowsDctWP, rows_dct_w_body<E, NW>, NW * 32, 1><<<l.blocks, NW * 32, l.smem, s>>>(
            packed_args<RowsDctWP>(l, dev));
    else if (l.kind == PK_COLS_W)
        k_packed<ColsWP, cols_w_body<E, NW>, NW * 32, 1><<<l.blocks, NW * 32, l.smem, s>>>(packed_args<ColsWP>(l, dev));
    else
        k_packed<RowsInvWP, rows_inv_w_body<E, NW>, NW * 32, 1><<<l.blocks, NW * 32, l.smem, s>>>(
            packed_args<RowsInvWP>(l, dev));
}

template <int E>
static void packed_spectral_launch_e(const PackedLaunch &l, int NW, const unsigned char *dev, cudaStream_t s) {
    switch (NW) {
    case kSeqCandidates[0]: packed_spectral_launch_en<E, kSeqCandidates[0]>(l, dev, s); break;
    case kSeqCandidates[1]: packed_spectral_launch_en<E, kSeqCandidates[1]>(l, dev, s); break;
    default: packed_spectral_launch_en<E, kRowWarps>(l, dev, s); break;
    }
}

bool packed_spectral_launch(const PackedLaunch &l, const unsigned char *dev, cudaStream_t s) {
    if (l.kind != PK_ROWS_DCT_W && l.kind != PK_COLS_W && l.kind != PK_ROWS_INV_W) return false;
    const int E = l.variant / 16, NW = l.variant % 16;
    if (E == 1) packed_spectral_launch_e<1>(l, NW, dev, s);
    else if (E == 2) packed_spectral_launch_e<2>(l, NW, dev, s);
    else packed_spectral_launch_e<4>(l, NW, dev, s);
    return true;
}

}  // namespace erp
