// turb_div.cuh -- correctly rounded FP64 division by a grid spacing whose
// reciprocal is known.
//
// Method (P. Markstein, "Computation of elementary functions on the IBM
// RISC System/6000 processor", IBM J. Res. Dev. 34(1), 1990; also in Muller
// et al., Handbook of Floating-Point Arithmetic, on division with an FMA):
// with y = RN(1/h) and q within one ulp of a/h, the remainder r = a - h*q is
// exact in one fused multiply-add and RN(q + r*y) is RN(a/h).  q0 = RN(a*y)
// can be up to ~2 ulps away, so one correction brings it within an ulp and a
// second one rounds correctly.  y comes from an IEEE division on the host.
// A zero numerator returns itself (+-0 / h = +-0, h > 0); numerators with a
// binary exponent outside [-900, 900] (no underflow of the remainder, no
// overflow), infinities and NaNs take the IEEE division.  Both tests read the
// exponent bits with integer instructions, so the FP64 pipe only sees the one
// multiply and four fused multiply-adds.  The equality with __ddiv_rn is
// checked on the GPU by turb_selftest_division.
#pragma once

__device__ __forceinline__ double div_by_spacing(double a, double h, double y)
{
    unsigned long long bits = (unsigned long long)__double_as_longlong(a);
    unsigned e = (unsigned)(bits >> 52) & 0x7FFu;
    if ((bits << 1) == 0ull) return a;
    if (e < 123u || e > 1923u) return __ddiv_rn(a, h);
    double q = __dmul_rn(a, y);
    double r = __fma_rn(-q, h, a);
    q = __fma_rn(r, y, q);
    r = __fma_rn(-q, h, a);
    return __fma_rn(r, y, q);
}
