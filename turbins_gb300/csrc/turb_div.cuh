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
// turb_selftest_division, that of div_by_spacing_2t (below) on flagged
// spacings by turb_selftest_division_pairs.
#pragma once

#include <cmath>

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

// The two-term quotient alone, q = RN(a y + RN(a yl)), for spacings that pass
// div_two_term_exact below: one multiply and one fused multiply-add.  Zero
// numerators and the exponent range as in div_by_spacing.
__device__ __forceinline__ double div_by_spacing_2t(double a, double h, double y, double yl)
{
    unsigned long long bits = (unsigned long long)__double_as_longlong(a);
    unsigned e = (unsigned)(bits >> 52) & 0x7FFu;
    if ((bits << 1) == 0ull) return a;
    if (e < 123u || e > 1923u) return __ddiv_rn(a, h);
    return __fma_rn(a, y, __dmul_rn(a, yl));
}

// Whether the two-term quotient q = RN(a y + RN(a yl)) equals RN(a/h) for
// every numerator a (with y = RN(1/h), yl = recip_low(h, y)).  Scale h and a
// to h = H 2^-52, a = A 2^-52 with 53-bit integers H, A.  Before its rounding
// q differs from a/h by less than 3 2^-107 (the rounding of a yl and of yl
// itself), so it rounds as a/h unless a/h lies that close to a midpoint
// N 2^-c between doubles (N odd; c = 53 for a/h in [1, 2), c = 54 in
// [1/2, 1)), i.e. unless 2^c A - H N = k with |k| <= 1 (c = 53) or |k| <= 3
// (c = 54); k = 0 is impossible (2^c would divide H N, so H, as N is odd,
// while 0 < H < 2^53).  For a given H each k admits at most two N in range,
// from the congruence H N = -k (mod 2^c), so the check tries the form on
// those few A and on nothing else.  The two-term algorithm is Brisebarre,
// Muller and Raina's (IEEE Trans. Computers 53(8), 2004); this check is
// derived from the bound above and was confirmed by exhaustive search at
// reduced precision.  About 99 % of random spacings pass.  Host only.
inline bool div_two_term_exact(double h, double y, double yl)
{
    int e = 0;
    if (!(h > 0.0) || !std::isfinite(h) || y != 1.0 / h || yl != recip_low(h, y)) return false;
    const double m = std::frexp(h, &e);   // h = m 2^e, m in [1/2, 1)
    if (e < -200 || e > 200) return false;
    const unsigned long long H = (unsigned long long)std::ldexp(m, 53);   // [2^52, 2^53)
    int v = 0;
    while (!((H >> v) & 1ull)) v++;
    if (v >= 2) return true;              // 2^v divides k: no |k| <= 3 is possible
    const unsigned long long Ho = H >> v;
    unsigned long long inv = Ho;          // Ho^-1 modulo 2^64 (Newton's iteration)
    for (int it = 0; it < 6; it++) inv *= 2ull - Ho * inv;
    for (int c = 53; c <= 54; c++) {
        const int kmax = c == 53 ? 1 : 3;
        for (int k = -kmax; k <= kmax; k++) {
            if (k == 0 || (k & ((1 << v) - 1))) continue;
            const int cc = c - v;
            const unsigned long long step = 1ull << cc;
            const long long kk = k / (1 << v);
            const unsigned long long n0 = ((unsigned long long)(-kk) * inv) & (step - 1);
            for (unsigned long long N = n0; N < (1ull << 54); N += step) {
                if (N <= (1ull << 53) || !(N & 1ull)) continue;
                const __int128 num = (__int128)H * (__int128)N + k;
                if (num & (((__int128)1 << c) - 1)) continue;
                const unsigned long long A = (unsigned long long)(num >> c);
                if (A < (1ull << 52) || A >= (1ull << 53) || (A >= H) != (c == 53)) continue;
                const double a = std::ldexp((double)A, e - 53);   // a / h = A / H
                if (fma(a, y, a * yl) != a / h) return false;
            }
        }
    }
    return true;
}
