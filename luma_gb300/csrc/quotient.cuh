// Correctly rounded FP64 division from a reciprocal, for code that divides
// many values by the same divisor or keeps a division off a critical path:
// quotient(a, b, RN(1/b)) returns the same bits as a / b.  Checked bit for
// bit against CUDA's division in tests/test_gpu_quotient.py.
#pragma once

namespace luma {

__device__ __forceinline__ int exponent_of(double v) { return (int)((__double_as_longlong(v) >> 52) & 0x7ff) - 1023; }

// RN(a / b) from y = RN(1 / b) with multiplications and FMAs only.
// q0 = RN(a y) lies within 1.5 ulp of a / b; one correction
// q1 = RN(q0 + RN(a - b q0) y) brings it within one ulp (the remainder and
// the reciprocal's error enter only at about 2^-52 ulp), and a second
// correction with the exact FMA remainder a - b q1 rounds to the correctly
// rounded quotient by Markstein's theorem (P. Markstein, "Computation of
// elementary functions on the IBM RISC System/6000 processor", IBM J. Res.
// Dev. 34(1):111-119, 1990: a faithful quotient plus the remainder times
// the correctly rounded reciprocal, rounded once).  Zeros, non-finite
// values and magnitudes beyond 2^+-400 (where a remainder could leave the
// normal range) take the division itself.  Five dependent FP64 operations
// instead of a division's longer sequence on the solve's critical path.
__device__ __forceinline__ double quotient(double a, double b, double y) {
    const int ea = exponent_of(a), eb = exponent_of(b);
    if (ea < -400 || ea > 400 || eb < -400 || eb > 400) return a / b;
    const double q0 = __dmul_rn(a, y);
    const double q1 = __fma_rn(__fma_rn(-q0, b, a), y, q0);
    return __fma_rn(__fma_rn(-q1, b, a), y, q1);
}

}  // namespace luma
