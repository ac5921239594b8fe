// Double-float sums: a value carried as an unevaluated pair hi + lo of FP32
// numbers, renormalised after every addition with Knuth's TwoSum and Dekker's
// FastTwoSum error-free transformations (about 44 significant bits).  The
// reductions of the placement step use them in place of FP64, which issues at
// a small fraction of the FP32 rate on GB300.
//
// The header compiles for the device and for the host (with floating-point
// contraction off and no reassociation, as the build uses), so that a host
// program can check the arithmetic.
#pragma once

#if defined(__CUDACC__)
#define ERP_DF_FN __host__ __device__ __forceinline__
#else
#define ERP_DF_FN static inline
#endif

namespace erp {

struct Df {
    float hi, lo;
};

// round-to-nearest FP32 add / subtract, never fused or reassociated
ERP_DF_FN float df_fadd(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}

ERP_DF_FN float df_fsub(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fsub_rn(a, b);
#else
    return a - b;
#endif
}

ERP_DF_FN Df df_zero() { return Df{0.0f, 0.0f}; }

// s + e == a + b exactly (round to nearest, no overflow)
ERP_DF_FN void two_sum(float a, float b, float &s, float &e) {
    s = df_fadd(a, b);
    const float bv = df_fsub(s, a);
    const float av = df_fsub(s, bv);
    e = df_fadd(df_fsub(a, av), df_fsub(b, bv));
}

// hi + lo == s + e, |lo| <= ulp(hi) / 2, for |s| >= |e|
ERP_DF_FN Df fast_two_sum(float s, float e) {
    const float hi = df_fadd(s, e);
    return Df{hi, df_fsub(e, df_fsub(hi, s))};
}

ERP_DF_FN Df df_add(Df a, Df b) {
    float s, e;
    two_sum(a.hi, b.hi, s, e);
    return fast_two_sum(s, df_fadd(e, df_fadd(a.lo, b.lo)));
}

ERP_DF_FN Df df_add(Df a, float b) {
    float s, e;
    two_sum(a.hi, b, s, e);
    return fast_two_sum(s, df_fadd(e, a.lo));
}

ERP_DF_FN double df_value(Df a) { return (double)a.hi + (double)a.lo; }

}  // namespace erp

#undef ERP_DF_FN
