// turb_div.cuh -- correctly rounded FP64 division by a grid spacing whose
// reciprocal is known.
//
// Method: with y = RN(1/h) and its correction yl = RN((1 - y h)/h) (both made
// once per spacing; 1 - y h is exact in one fused multiply-add), the
// quotient q = RN(a y + RN(a yl)) carries a relative error of about 2^-105
// before its final rounding, so it lies within one ulp of a/h.  Then the
// remainder r = a - h q is exact in one fused multiply-add and RN(q + r y)
// is RN(a/h) (P. Markstein, "Computation of elementary functions on the IBM
// RISC System/6000 processor", IBM J. Res. Dev. 34(1), 1990; Muller et al.,
// Handbook of Floating-Point Arithmetic, on division with an FMA; the
// two-term reciprocal follows Brisebarre, Muller and Raina, "Accelerating
// correctly rounded floating-point division when the divisor is known in
// advance", IEEE Trans. Computers 53(8), 2004).  One multiply and three
// fused multiply-adds.  A zero numerator returns itself (+-0 / h = +-0,
// h > 0); numerators with a binary exponent outside [-900, 900] (no
// underflow of a yl or of the remainder, no overflow), infinities and NaNs
// take the IEEE division.  Both tests read the exponent bits with integer
// instructions.  The equality with __ddiv_rn is checked on the GPU by
// turb_selftest_division.
#pragma once

__device__ __forceinline__ double div_by_spacing(double a, double h, double y, double yl)
{
    unsigned long long bits = (unsigned long long)__double_as_longlong(a);
    unsigned e = (unsigned)(bits >> 52) & 0x7FFu;
    if ((bits << 1) == 0ull) return a;
    if (e < 123u || e > 1923u) return __ddiv_rn(a, h);
    double q = __fma_rn(a, y, __dmul_rn(a, yl));
    double r = __fma_rn(-q, h, a);
    return __fma_rn(r, y, q);
}

// the correction term of the reciprocal of h (host or device)
__host__ __device__ inline double recip_low(double h, double y)
{
    return fma(-y, h, 1.0) / h;
}
