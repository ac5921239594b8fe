/*
 * spectral_impl.h — TEST INFRASTRUCTURE (oracle).  Restatement of the
 * reference's FFT-based spectral transforms, instantiated twice by
 * erp_oracle.c with REAL = float (SFX f32) and REAL = double (SFX f64).
 *
 *   make_expk            src/utils.rs:232-249
 *   rfft_2d              src/dct2d.rs:281-339
 *   dct2d_preprocess     src/dct2d.rs:47-81
 *   dct2d_postprocess    src/dct2d.rs:98-254
 *   dct2_fft2_forward    src/dct2d.rs:256-279
 *   irfft_2d             src/irfft2d.rs:7-83
 *   idct2 pre/post       src/idct2.rs:9-166
 *   idct_idxst pre/post  src/idct_idxst.rs:9-161
 *   idxst_idct pre/post  src/idxst_idct.rs:9-180
 *   frequency matrices   src/frequencies.rs:4-72
 *
 * The complex FFT under rfft_2d / irfft_2d is rustfft 6.4.1 in the reference
 * (Cargo.toml:27, not vendored).  Any exact DFT matches it up to rounding; this
 * file uses an unnormalised iterative radix-2 FFT whose twiddles are computed
 * in FP64 and rounded to REAL, as rustfft computes its twiddles.  Power-of-two
 * lengths only (every configuration here uses power-of-two bin grids).
 */

#define CAT_(a, b) a##b
#define CAT(a, b) CAT_(a, b)
#define CX CAT(cx_, SFX)
#define FN(name) CAT(name##_, SFX)

typedef struct { REAL re, im; } CX;

static inline CX FN(cmul)(CX a, CX b) {
    CX r; r.re = a.re * b.re - a.im * b.im; r.im = a.re * b.im + a.im * b.re; return r;
}
static inline CX FN(cconj)(CX a) { a.im = -a.im; return a; }
static inline CX FN(cnew)(REAL re, REAL im) { CX r; r.re = re; r.im = im; return r; }

/* twiddle table tw[k] = exp(-2*pi*i*k/n), k < n/2 */
static CX *FN(make_twiddles)(int n) {
    CX *tw = (CX *)malloc(sizeof(CX) * (size_t)(n / 2 > 0 ? n / 2 : 1));
    for (int k = 0; k < n / 2; ++k) {
        double ang = -2.0 * M_PI * (double)k / (double)n;
        tw[k].re = (REAL)cos(ang);
        tw[k].im = (REAL)sin(ang);
    }
    return tw;
}

/* unnormalised in-place radix-2 DIT FFT; inverse uses conj twiddles */
static void FN(fft)(CX *a, int n, int inverse, const CX *tw) {
    for (int i = 1, j = 0; i < n; ++i) {
        int bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) { CX t = a[i]; a[i] = a[j]; a[j] = t; }
    }
    for (int len = 2; len <= n; len <<= 1) {
        int half = len >> 1, step = n / len;
        for (int j = 0; j < half; ++j) {
            CX w = tw[j * step];
            if (inverse) w.im = -w.im;
            for (int i = 0; i < n; i += len) {
                CX u = a[i + j], v = FN(cmul)(a[i + j + half], w);
                a[i + j].re = u.re + v.re; a[i + j].im = u.im + v.im;
                a[i + j + half].re = u.re - v.re; a[i + j + half].im = u.im - v.im;
            }
        }
    }
}

/* make_expk (src/utils.rs:232-249): exp(-i*pi*k/(2n)).  The reference uses the
 * f32 constant for pi and evaluates in T; the FP64 instantiation uses the exact
 * pi so that it serves as an accurate FP64 solve. */
static void FN(make_expk)(int n, CX *out) {
    REAL two_n = (REAL)(2 * n);
    REAL pi = (REAL)PI_VALUE;
    for (int k = 0; k < n; ++k) {
        REAL pik = (REAL)k * pi / two_n;
        out[k].re = COS(pik);
        out[k].im = -SIN(pik);
    }
}

/* rfft_2d (src/dct2d.rs:281-339): row FFTs of the complex input (length n),
 * keep n/2+1, then column FFTs (length m). */
static void FN(rfft_2d)(const CX *input, CX *output, int m, int n) {
    int nf = n / 2 + 1;
    CX *twn = FN(make_twiddles)(n), *twm = FN(make_twiddles)(m);
#pragma omp parallel
    {
        CX *buf = (CX *)malloc(sizeof(CX) * (size_t)(n > m ? n : m));
#pragma omp for schedule(static)
        for (int i = 0; i < m; ++i) {
            memcpy(buf, input + (size_t)i * n, sizeof(CX) * (size_t)n);
            FN(fft)(buf, n, 0, twn);
            memcpy(output + (size_t)i * nf, buf, sizeof(CX) * (size_t)nf);
        }
#pragma omp for schedule(static)
        for (int j = 0; j < nf; ++j) {
            for (int i = 0; i < m; ++i) buf[i] = output[(size_t)i * nf + j];
            FN(fft)(buf, m, 0, twm);
            for (int i = 0; i < m; ++i) output[(size_t)i * nf + j] = buf[i];
        }
        free(buf);
    }
    free(twn); free(twm);
}

/* irfft_2d (src/irfft2d.rs:7-83): column inverse FFTs / m (in place), then
 * row inverse FFTs with Hermitian rebuild and real Nyquist, / n. */
static void FN(irfft_2d)(CX *input, REAL *output, int m, int n) {
    int nf = n / 2 + 1;
    REAL norm_m = (REAL)m, norm_n = (REAL)n;
    CX *twn = FN(make_twiddles)(n), *twm = FN(make_twiddles)(m);
#pragma omp parallel
    {
        CX *buf = (CX *)malloc(sizeof(CX) * (size_t)(n > m ? n : m));
#pragma omp for schedule(static)
        for (int j = 0; j < nf; ++j) {
            for (int i = 0; i < m; ++i) buf[i] = input[(size_t)i * nf + j];
            FN(fft)(buf, m, 1, twm);
            for (int i = 0; i < m; ++i) {
                input[(size_t)i * nf + j].re = buf[i].re / norm_m;
                input[(size_t)i * nf + j].im = buf[i].im / norm_m;
            }
        }
#pragma omp for schedule(static)
        for (int i = 0; i < m; ++i) {
            for (int j = 0; j < nf; ++j) buf[j] = input[(size_t)i * nf + j];
            for (int j = 1; j < nf - 1; ++j) buf[n - j] = FN(cconj)(buf[j]);
            if (n % 2 == 0 && nf > 1) buf[n / 2].im = (REAL)0;
            FN(fft)(buf, n, 1, twn);
            for (int j = 0; j < n; ++j) output[(size_t)i * n + j] = buf[j].re / norm_n;
        }
        free(buf);
    }
    free(twn); free(twm);
}

/* dct2d_preprocess (src/dct2d.rs:47-81): even/odd reorder along both axes,
 * written with row stride n/2 into a buffer of 2*m*(n/2+1) entries. */
static void FN(dct2d_preprocess)(const REAL *x, CX *y, int m, int n) {
    int half_n = n / 2;
    for (int hid = 0; hid < m; ++hid) {
        int dst_row = (hid & 1) == 0 ? hid : 2 * m - (hid + 1);
        size_t dst = (size_t)dst_row * half_n, src = (size_t)hid * n;
        for (int i = 0; i < half_n; ++i) y[dst + i] = FN(cnew)(x[src + (i << 1)], (REAL)0);
        for (int i = 0; i < half_n; ++i)
            y[dst + (n - i - 1)] = FN(cnew)(x[src + (i << 1) + 1], (REAL)0);
    }
}

static inline REAL FN(real_mul)(CX a, CX b) { return a.re * b.re - a.im * b.im; }
static inline REAL FN(imag_mul)(CX a, CX b) { return a.re * b.im + a.im * b.re; }

/* dct2d_postprocess (src/dct2d.rs:98-254) */
static void FN(dct2d_postprocess)(const CX *v, REAL *y, int m, int n, const CX *expk_m,
                                   const CX *expk_n) {
    REAL mn = (REAL)((size_t)m * n);
    int half_m = m / 2, half_n = n / 2;
    REAL four_over_mn = (REAL)4 / mn, two_over_mn = (REAL)2 / mn;
    int vs = half_n + 1;
    CX ekm = expk_m[half_m], ekn = expk_n[half_n];
    y[0] = v[0].re * four_over_mn;
    y[half_n] = FN(real_mul)(ekn, v[half_n]) * four_over_mn;
    size_t row_halfm = (size_t)half_m * n;
    y[row_halfm] = ekm.re * v[(size_t)half_m * vs].re * four_over_mn;
    y[row_halfm + half_n] = ekm.re * FN(real_mul)(ekn, v[(size_t)half_m * vs + half_n]) * four_over_mn;
    for (int wid = 1; wid < half_n; ++wid) {
        CX tmp = v[wid], e = expk_n[wid];
        y[wid] = FN(real_mul)(e, tmp) * four_over_mn;
        y[n - wid] = -FN(imag_mul)(e, tmp) * four_over_mn;
        tmp = v[(size_t)half_m * vs + wid];
        y[row_halfm + wid] = ekm.re * FN(real_mul)(e, tmp) * four_over_mn;
        y[row_halfm + (n - wid)] = -(ekm.re * FN(imag_mul)(e, tmp) * four_over_mn);
    }
    for (int hid = 1; hid < half_m; ++hid) {
        size_t row_up = (size_t)hid * n, row_down = (size_t)(m - hid) * n;
        size_t k = (size_t)hid * vs, km = (size_t)(m - hid) * vs;
        CX t1 = v[k], t2 = v[km], e = expk_m[hid];
        REAL sum_re = t1.re + t2.re, diff_im = t2.im - t1.im;
        REAL up = e.re * sum_re + e.im * diff_im;
        REAL down = -(e.im * sum_re) + e.re * diff_im;
        y[row_up] = up * two_over_mn;
        y[row_down] = down * two_over_mn;
        CX v1 = v[k + half_n], v2 = v[km + half_n];
        CX a = FN(cnew)(v1.re + v2.re, v1.im + v2.im), b = FN(cnew)(v1.re - v2.re, v1.im - v2.im);
        CX upc = FN(cnew)(e.re * a.re - e.im * b.im, e.re * a.im + e.im * b.re);
        CX dnc = FN(cnew)(-(e.im * a.re) - e.re * b.im, -(e.im * a.im) + e.re * b.re);
        y[row_up + half_n] = FN(real_mul)(ekn, upc) * two_over_mn;
        y[row_down + half_n] = FN(real_mul)(ekn, dnc) * two_over_mn;
    }
    for (int hid = 1; hid < half_m; ++hid) {
        size_t row_up = (size_t)hid * n, row_down = (size_t)(m - hid) * n;
        REAL er = expk_m[hid].re, ei = expk_m[hid].im;
        size_t vu = (size_t)hid * vs, vd = (size_t)(m - hid) * vs;
        for (int wid = 1; wid < half_n; ++wid) {
            CX a = v[vu + wid], b = v[vd + wid];
            REAL s_re = a.re + b.re, s_im = a.im + b.im, d_re = a.re - b.re, d_im = a.im - b.im;
            REAL up_re = er * s_re - ei * d_im, up_im = er * s_im + ei * d_re;
            REAL dn_re = -ei * s_re - er * d_im, dn_im = -ei * s_im + er * d_re;
            REAL sr = expk_n[wid].re * two_over_mn, si = expk_n[wid].im * two_over_mn;
            REAL r_up = sr * up_re - si * up_im, i_up = sr * up_im + si * up_re;
            REAL r_dn = sr * dn_re - si * dn_im, i_dn = sr * dn_im + si * dn_re;
            int dst = n - wid;
            y[row_up + wid] = r_up;
            y[row_down + wid] = r_dn;
            y[row_up + dst] = -i_up;
            y[row_down + dst] = -i_dn;
        }
    }
}

/* dct2_fft2_forward (src/dct2d.rs:256-279) */
static void FN(dct2_fft2_forward)(const REAL *x, const CX *expk_m, const CX *expk_n, REAL *out,
                                   int m, int n) {
    int hn = n / 2 + 1;
    CX *pre = (CX *)calloc((size_t)2 * m * hn, sizeof(CX));
    CX *fft = (CX *)calloc((size_t)m * hn, sizeof(CX));
    FN(dct2d_preprocess)(x, pre, m, n);
    FN(rfft_2d)(pre, fft, m, n);
    FN(dct2d_postprocess)(fft, out, m, n, expk_m, expk_n);
    free(pre); free(fft);
}

#define IDX(h, w, nn) ((size_t)(h) * (size_t)(nn) + (size_t)(w))

/* idct2_fft2_preprocess (src/idct2.rs:9-119) */
static void FN(idct2_preprocess)(const REAL *in, CX *out, int m, int n, const CX *em, const CX *en) {
    int half_m = m / 2, half_n = n / 2, nf = half_n + 1;
    REAL two = (REAL)1 + (REAL)1;
    for (int hid = 0; hid < half_m; ++hid)
        for (int wid = 0; wid < half_n; ++wid) {
            int cond = ((hid != 0) << 1) | (wid != 0);
            if (cond == 0) {
                out[0] = FN(cnew)(in[0], (REAL)0);
                REAL v = in[half_n];
                out[half_n] = FN(cconj)(FN(cmul)(en[half_n], FN(cnew)(v, v)));
                v = in[IDX(half_m, 0, n)];
                out[IDX(half_m, 0, nf)] = FN(cconj)(FN(cmul)(em[half_m], FN(cnew)(v, v)));
                v = in[IDX(half_m, half_n, n)];
                out[IDX(half_m, half_n, nf)] =
                    FN(cconj)(FN(cmul)(FN(cmul)(em[half_m], en[half_n]), FN(cnew)((REAL)0, two * v)));
            } else if (cond == 1) {
                REAL a = in[wid], b = in[n - wid];
                out[wid] = FN(cconj)(FN(cmul)(en[wid], FN(cnew)(a, b)));
                a = in[IDX(half_m, wid, n)]; b = in[IDX(half_m, n - wid, n)];
                REAL sum = a + b, diff = a - b;
                out[IDX(half_m, wid, nf)] =
                    FN(cconj)(FN(cmul)(FN(cmul)(em[half_m], en[wid]), FN(cnew)(diff, sum)));
            } else if (cond == 2) {
                REAL a = in[IDX(hid, 0, n)], b = in[IDX(m - hid, 0, n)];
                out[IDX(hid, 0, nf)] = FN(cconj)(FN(cmul)(em[hid], FN(cnew)(a, b)));
                out[IDX(m - hid, 0, nf)] = FN(cconj)(FN(cmul)(em[m - hid], FN(cnew)(b, a)));
                a = in[IDX(hid, half_n, n)]; b = in[IDX(m - hid, half_n, n)];
                REAL sum = a + b, diff = a - b;
                CX w = en[half_n];
                out[IDX(hid, half_n, nf)] =
                    FN(cconj)(FN(cmul)(FN(cmul)(em[hid], w), FN(cnew)(diff, sum)));
                out[IDX(m - hid, half_n, nf)] =
                    FN(cconj)(FN(cmul)(FN(cmul)(em[m - hid], w), FN(cnew)(-diff, sum)));
            } else {
                REAL a = in[IDX(hid, wid, n)], b = in[IDX(hid, n - wid, n)];
                REAL c = in[IDX(m - hid, wid, n)], d = in[IDX(m - hid, n - wid, n)];
                REAL s1 = a + d, s2 = b + c, d1 = a - d, d2 = c - b;
                CX w = FN(cmul)(em[hid], en[wid]), ws = FN(cmul)(em[m - hid], en[wid]);
                out[IDX(hid, wid, nf)] = FN(cconj)(FN(cmul)(w, FN(cnew)(d1, s2)));
                out[IDX(m - hid, wid, nf)] = FN(cconj)(FN(cmul)(ws, FN(cnew)(d2, s1)));
            }
        }
}

/* Shared inverse post-reorder: idct2 (src/idct2.rs:121-142), idct_idxst
 * (src/idct_idxst.rs:102-135) and idxst_idct (src/idxst_idct.rs:116-154)
 * differ only in the sign per quadrant. */
static void FN(inverse_postprocess)(const REAL *x, REAL *y, int m, int n, int variant) {
    REAL mn = (REAL)((size_t)m * n);
    for (int hid = 0; hid < m; ++hid)
        for (int wid = 0; wid < n; ++wid) {
            int cond = ((hid < m / 2) << 1) | (wid < n / 2);
            size_t idx;
            REAL sign = (REAL)1;
            switch (cond) {
            case 0: idx = IDX(((m - hid) << 1) - 1, ((n - wid) << 1) - 1, n); break;
            case 1: idx = IDX(((m - hid) << 1) - 1, wid << 1, n); break;
            case 2: idx = IDX(hid << 1, ((n - wid) << 1) - 1, n); break;
            default: idx = IDX(hid << 1, wid << 1, n); break;
            }
            if (variant == 1 && (cond == 0 || cond == 2)) sign = (REAL)-1; /* idct_idxst */
            if (variant == 2 && (cond == 0 || cond == 1)) sign = (REAL)-1; /* idxst_idct */
            if (variant == 0) y[idx] = x[IDX(hid, wid, n)] * mn;
            else if (variant == 1) y[idx] = sign * x[IDX(hid, wid, n)] * mn;
            else y[idx] = (sign < 0 ? -x[IDX(hid, wid, n)] : x[IDX(hid, wid, n)]) * mn;
        }
}

/* idct_idxst_preprocess (src/idct_idxst.rs:9-100) */
static void FN(idct_idxst_preprocess)(const REAL *in, CX *out, int m, int n, const CX *em,
                                       const CX *en) {
    int half_m = m / 2, half_n = n / 2, nf = half_n + 1;
    CX zero = FN(cnew)((REAL)0, (REAL)0);
    for (int hid = 0; hid < half_m; ++hid)
        for (int wid = 0; wid < half_n; ++wid) {
            int cond = ((hid != 0) << 1) | (wid != 0);
            if (cond == 0) {
                out[0] = zero;
                REAL t1 = in[half_n];
                out[half_n] = FN(cconj)(FN(cmul)(en[half_n], FN(cnew)(t1, t1)));
                out[IDX(half_m, 0, nf)] = zero;
                t1 = in[IDX(half_m, half_n, n)];
                out[IDX(half_m, half_n, nf)] = FN(cconj)(FN(cmul)(
                    FN(cmul)(em[half_m], en[half_n]), FN(cnew)((REAL)0, (REAL)2.0 * t1)));
            } else if (cond == 1) {
                out[wid] = FN(cconj)(FN(cmul)(en[wid], FN(cnew)(in[n - wid], in[wid])));
                REAL t1 = in[IDX(half_m, n - wid, n)], t2 = in[IDX(half_m, wid, n)];
                out[IDX(half_m, wid, nf)] = FN(cconj)(
                    FN(cmul)(FN(cmul)(em[half_m], en[wid]), FN(cnew)(t1 - t2, t1 + t2)));
            } else if (cond == 2) {
                out[IDX(hid, 0, nf)] = zero;
                out[IDX(m - hid, 0, nf)] = zero;
                REAL t1 = in[IDX(hid, half_n, n)], t3 = in[IDX(m - hid, half_n, n)];
                out[IDX(hid, half_n, nf)] = FN(cconj)(
                    FN(cmul)(FN(cmul)(em[hid], en[half_n]), FN(cnew)(t1 - t3, t3 + t1)));
                out[IDX(m - hid, half_n, nf)] = FN(cconj)(
                    FN(cmul)(FN(cmul)(em[m - hid], en[half_n]), FN(cnew)(t3 - t1, t1 + t3)));
            } else {
                REAL t1 = in[IDX(hid, n - wid, n)], t2 = in[IDX(hid, wid, n)];
                REAL t3 = in[IDX(m - hid, n - wid, n)], t4 = in[IDX(m - hid, wid, n)];
                out[IDX(hid, wid, nf)] = FN(cconj)(
                    FN(cmul)(FN(cmul)(em[hid], en[wid]), FN(cnew)(t1 - t4, t3 + t2)));
                out[IDX(m - hid, wid, nf)] = FN(cconj)(
                    FN(cmul)(FN(cmul)(em[m - hid], en[wid]), FN(cnew)(t3 - t2, t1 + t4)));
            }
        }
}

/* idxst_idct_preprocess (src/idxst_idct.rs:9-114) */
static void FN(idxst_idct_preprocess)(const REAL *in, CX *out, int m, int n, const CX *em,
                                       const CX *en) {
    int half_m = m / 2, half_n = n / 2, nf = half_n + 1;
    REAL two = (REAL)1 + (REAL)1;
    CX zero = FN(cnew)((REAL)0, (REAL)0);
    for (int hid = 0; hid < half_m; ++hid)
        for (int wid = 0; wid < half_n; ++wid) {
            int cond = ((hid != 0) << 1) | (wid != 0);
            if (cond == 0) {
                out[0] = zero;
                out[half_n] = zero;
                REAL a = in[IDX(half_m, 0, n)];
                out[IDX(half_m, 0, nf)] = FN(cconj)(FN(cmul)(em[half_m], FN(cnew)(a, a)));
                REAL b = in[IDX(half_m, half_n, n)];
                out[IDX(half_m, half_n, nf)] = FN(cconj)(
                    FN(cmul)(FN(cmul)(em[half_m], en[half_n]), FN(cnew)((REAL)0, two * b)));
            } else if (cond == 1) {
                out[wid] = zero;
                REAL a = in[IDX(half_m, wid, n)], b = in[IDX(half_m, n - wid, n)];
                REAL sum = a + b, diff = a - b;
                out[IDX(half_m, wid, nf)] = FN(cconj)(
                    FN(cmul)(FN(cmul)(em[half_m], en[wid]), FN(cnew)(diff, sum)));
            } else if (cond == 2) {
                REAL a = in[IDX(m - hid, 0, n)], b = in[IDX(hid, 0, n)];
                out[IDX(hid, 0, nf)] = FN(cconj)(FN(cmul)(em[hid], FN(cnew)(a, b)));
                out[IDX(m - hid, 0, nf)] = FN(cconj)(FN(cmul)(em[m - hid], FN(cnew)(b, a)));
                a = in[IDX(m - hid, half_n, n)]; b = in[IDX(hid, half_n, n)];
                REAL sum = a + b, diff = a - b;
                CX e1 = FN(cmul)(em[hid], en[half_n]), e2 = FN(cmul)(em[m - hid], en[half_n]);
                out[IDX(hid, half_n, nf)] = FN(cconj)(FN(cmul)(e1, FN(cnew)(diff, sum)));
                out[IDX(m - hid, half_n, nf)] = FN(cconj)(FN(cmul)(e2, FN(cnew)(-diff, sum)));
            } else {
                REAL a = in[IDX(m - hid, wid, n)], b = in[IDX(m - hid, n - wid, n)];
                REAL c = in[IDX(hid, wid, n)], d = in[IDX(hid, n - wid, n)];
                REAL s1 = c + b, d1 = a - d, s2 = a + d, d2 = c - b;
                CX e1 = FN(cmul)(em[hid], en[wid]), e2 = FN(cmul)(em[m - hid], en[wid]);
                out[IDX(hid, wid, nf)] = FN(cconj)(FN(cmul)(e1, FN(cnew)(d1, s1)));
                out[IDX(m - hid, wid, nf)] = FN(cconj)(FN(cmul)(e2, FN(cnew)(d2, s2)));
            }
        }
}

/* variant 0: idct2_fft2_forward (src/idct2.rs:144-166)
 * variant 1: idct_idxst_forward (src/idct_idxst.rs:137-161)
 * variant 2: idxst_idct_forward (src/idxst_idct.rs:156-180) */
static void FN(inverse_forward)(const REAL *x, const CX *em, const CX *en, REAL *out, int m, int n,
                                int variant) {
    int nf = n / 2 + 1;
    CX *buf = (CX *)calloc((size_t)m * nf, sizeof(CX));
    REAL *fft_out = (REAL *)calloc((size_t)m * n, sizeof(REAL));
    if (variant == 0) FN(idct2_preprocess)(x, buf, m, n, em, en);
    else if (variant == 1) FN(idct_idxst_preprocess)(x, buf, m, n, em, en);
    else FN(idxst_idct_preprocess)(x, buf, m, n, em, en);
    FN(irfft_2d)(buf, fft_out, m, n);
    FN(inverse_postprocess)(fft_out, out, m, n, variant);
    free(buf); free(fft_out);
}

/* compute_frequency_matrices (src/frequencies.rs:4-72) */
static void FN(frequency_matrices)(int m, int n, REAL bin_w, REAL bin_h, REAL *wu_half,
                                   REAL *wv_half, REAL *inv) {
    REAL *wu = (REAL *)malloc(sizeof(REAL) * (size_t)m), *wv = (REAL *)malloc(sizeof(REAL) * (size_t)n);
    REAL tpm = (REAL)(2.0 * M_PI) / (REAL)m;
    for (int i = 0; i < m; ++i) wu[i] = (REAL)i * tpm;
    REAL wv_div = bin_w / bin_h;
    REAL tpn = (REAL)(2.0 * M_PI) / (REAL)n;
    for (int j = 0; j < n; ++j) wv[j] = (REAL)j * tpn * wv_div;
    for (int i = 0; i < m; ++i)
        for (int j = 0; j < n; ++j) {
            size_t k = IDX(i, j, n);
            REAL s = wu[i] * wu[i] + wv[j] * wv[j];
            if (k == 0) s = (REAL)1;
            inv[k] = (REAL)1 / s;
        }
    inv[0] = (REAL)0;
    REAL half = (REAL)0.5;
    for (int i = 0; i < m; ++i)
        for (int j = 0; j < n; ++j) {
            size_t k = IDX(i, j, n);
            wu_half[k] = wu[i] * inv[k] * half;
            wv_half[k] = wv[j] * inv[k] * half;
        }
    free(wu); free(wv);
}

/* The spectral part of compute_potential (src/epotential.rs:287-343). */
static void FN(poisson)(const REAL *rho, int m, int n, REAL bin_w, REAL bin_h, const CX *em,
                        const CX *en, REAL *auv, REAL *fx, REAL *fy, REAL *pot) {
    size_t mn = (size_t)m * n;
    REAL *wu = (REAL *)malloc(sizeof(REAL) * mn), *wv = (REAL *)malloc(sizeof(REAL) * mn);
    REAL *inv = (REAL *)malloc(sizeof(REAL) * mn), *tmp = (REAL *)malloc(sizeof(REAL) * mn);
    FN(frequency_matrices)(m, n, bin_w, bin_h, wu, wv, inv);
    FN(dct2_fft2_forward)(rho, em, en, auv, m, n);
    for (size_t k = 0; k < mn; ++k) tmp[k] = auv[k] * wu[k];
    FN(inverse_forward)(tmp, em, en, fx, m, n, 2);
    for (size_t k = 0; k < mn; ++k) tmp[k] = auv[k] * wv[k];
    FN(inverse_forward)(tmp, em, en, fy, m, n, 1);
    for (size_t k = 0; k < mn; ++k) tmp[k] = auv[k] * inv[k];
    FN(inverse_forward)(tmp, em, en, pot, m, n, 0);
    free(wu); free(wv); free(inv); free(tmp);
}

#undef IDX
#undef CX
#undef FN
#undef CAT
#undef CAT_
