// The bin range of compute_electric_force (src/eforce.rs:48-69) in 32-bit
// arithmetic.  The reference takes `f.to_isize().unwrap_or(0)` of the scaled
// cell edges (truncation toward zero; NaN and values outside isize give 0),
// raises the lower end to 0, and adds 1 to the upper end, whose negative
// values wrap to usize::MAX, before cutting it to the bin count nb.
//
// Only the position of the truncated value against 0 and nb matters, so no
// 64-bit conversion is needed (those issue on the FP64 pipe, a small fraction
// of the FP32 rate on GB300).  The lower end is also cut to nb: the upper end
// never exceeds nb, so a lower end beyond it gives the same empty range, and a
// loop index can never wrap.
//
// The header compiles for the device and for the host, so that a host program
// can check both ends against the 64-bit rule.
#pragma once

#if defined(__CUDACC__)
#define ERP_BR_FN __host__ __device__ __forceinline__
#else
#define ERP_BR_FN static inline
#endif

namespace erp {

// the reference's `to_isize()` range: values it maps to 0
ERP_BR_FN bool br_outside_isize(float v) { return !(v == v) || v >= 9.2e18f || v <= -9.2e18f; }

// max(to_isize0(v), 0), cut to nb
ERP_BR_FN int force_bin_lo(float v, int nb) {
    if (br_outside_isize(v) || v < 1.0f) return 0;   // trunc(v) <= 0
    if (v >= (float)nb) return nb;                   // trunc(v) >= nb: empty range
    return (int)v;
}

// to_isize0(v) + 1, then (< 0 or > nb) -> nb
ERP_BR_FN int force_bin_hi(float v, int nb) {
    if (br_outside_isize(v)) return 1 > nb ? nb : 1;
    if (v <= -2.0f) return nb;                       // trunc(v) + 1 <= -1: wraps, then cut
    if (v >= (float)nb) return nb;                   // trunc(v) + 1 > nb
    return (int)v + 1;                               // trunc(v) in [-1, nb - 1]
}

}  // namespace erp

#undef ERP_BR_FN
