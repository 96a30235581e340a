// Table-driven natural logarithm and exponential for the transport loops.
//
// GB300 issues two FP64 FMAs per clock per SM, and the library logarithm is
// one of the largest FP64 consumers of a substep (table brackets, the GS
// angle inversion, the hazard depth).  This follows the table-driven method
// of P. T. P. Tang, "Table-driven implementation of the logarithm function in
// IEEE floating-point arithmetic", ACM TOMS 16(4), 1990:
//   x = 2^e m with m in [1, 2),  F = 1 + j/256 the table point nearest m,
//   f = m - F (exact: both in [1, 2], |f| <= 2^-9),  r = f * (1/F),
//   log x = e ln2 + log F + log1p(r),
// log1p(r) by its Taylor series through r^6 (|r| <= 2^-9, so the first
// omitted term is below 2^-62 absolutely and 2^-54 relative to r).  The
// table (RREA_ARENA_LOG_TABLE_ROWS rows of {1/F, log F high, log F low},
// filled on the host in extended precision) opens the arena.  The result is
// within two ulps of the correctly rounded logarithm for every normal
// positive x; zero, negative, subnormal, infinite and NaN inputs go to the
// CUDA log.  The coefficients are the exact rationals of the series; ln 2
// is split into its double rounding and the rounding of the remainder.
#pragma once

#include "../rrea_arena.h"

#include <stdint.h>

namespace rrea_dev {

constexpr double kLn2Hi = 6.93147180559945286227e-01;   // RN(ln 2)
constexpr double kLn2Lo = 2.31904681384629955842e-17;   // RN(ln 2 - kLn2Hi)

__device__ __forceinline__ double flog(const double* __restrict__ arena, double x)
{
#ifdef RREA_CUDA_LIBM
    // parity-study build: CUDA's logarithm everywhere
    (void)arena;
    return log(x);
#endif
    long long const bits = __double_as_longlong(x);
    // normal, positive and finite: sign clear, biased exponent in [1, 2046]
    if (bits < 0x0010000000000000LL || bits >= 0x7ff0000000000000LL) return log(x);
    int const e = static_cast<int>(bits >> 52) - 1023;
    long long const mant = bits & 0x000fffffffffffffLL;
    int const j = static_cast<int>((mant + (1LL << 43)) >> 44);  // nearest of the 257 points, 0..256
    double const m = __longlong_as_double(mant | 0x3ff0000000000000LL);
    double const f = m - (1.0 + static_cast<double>(j) * 0.00390625);
    const double* t = arena + RREA_ARENA_LOG_TABLE + 3 * j;
    double const r = f * __ldg(t);
    double const q = fma(r, fma(r, fma(r, fma(r, -1.0 / 6.0, 1.0 / 5.0), -0.25), 1.0 / 3.0), -0.5);
    double const p = fma(r * r, q, r);
    double const de = static_cast<double>(e);
    double const hi = fma(de, kLn2Hi, __ldg(t + 1));
    double const lo = fma(de, kLn2Lo, __ldg(t + 2)) + p;
    return hi + lo;
}

// Table-driven exponential after P. T. P. Tang, "Table-driven implementation
// of the exponential function in IEEE floating-point arithmetic", ACM TOMS
// 15(2), 1989: k = rint(x 128/ln2), x = k ln2/128 + r with |r| <= ln2/256
// (r from the split of ln2/128, two FMAs), exp x = 2^(k div 128) *
// 2^((k mod 128)/128) * exp(r), expm1(r) by its Taylor series through r^5
// (first omitted term below 2^-62).  2^(j/128) comes from the table as two
// doubles.  Within two ulps of the correctly rounded exponential for
// |x| < 700; larger, infinite and NaN arguments go to the CUDA exp.
constexpr double kInvLn2x128 = 1.84664965233787316142e+02;  // RN(128 / ln 2)
constexpr double kLn2by128Hi = 5.41521234812457272982e-03;  // RN(ln 2 / 128)
constexpr double kLn2by128Lo = 1.81175532331742157843e-19;  // RN(ln 2 / 128 - kLn2by128Hi)

__device__ __forceinline__ double fexp(const double* __restrict__ arena, double x)
{
#ifdef RREA_CUDA_LIBM
    // parity-study build: CUDA's exponential everywhere
    (void)arena;
    return exp(x);
#endif
    if (!(fabs(x) < 700.0)) return exp(x);
    double const kf = rint(x * kInvLn2x128);
    int const k = static_cast<int>(kf);
    double r = fma(-kf, kLn2by128Hi, x);
    r = fma(-kf, kLn2by128Lo, r);
    double const q = fma(r, fma(r, fma(r, 1.0 / 120.0, 1.0 / 24.0), 1.0 / 6.0), 0.5);
    double const p = fma(r * r, q, r);  // expm1(r)
    const double* t = arena + RREA_ARENA_EXP_TABLE + 2 * (k & 127);
    double const th = __ldg(t);
    double const v = th + fma(th, p, __ldg(t + 1));
    // 2^(k >> 7): |k| < 129,300, so the exponent stays in the normal range
    return v * __longlong_as_double(static_cast<long long>((k >> 7) + 1023) << 52);
}

}  // namespace rrea_dev
