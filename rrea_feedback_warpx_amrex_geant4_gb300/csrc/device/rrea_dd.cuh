// Double-double arithmetic (an unevaluated sum hi + lo of two doubles,
// about 106 significant bits) for the few reference primitives that compute
// in long double on the host.  The error-free transformations are the
// published ones: TwoSum (Knuth, TAOCP vol. 2, 4.2.2), FastTwoSum (Dekker
// 1971) and TwoProduct through one fused multiply-add; the compound
// operations follow the "accurate" double-double algorithms of Hida, Li and
// Bailey (QD library paper, 2001).  dd_log is written from the series
//   log(m) = 2 atanh(s) = 2 (s + s^3/3 + s^5/5 + ...),  s = (m-1)/(m+1),
// after the exact reduction x = 2^e m with m in [sqrt(1/2), sqrt(2)).
#pragma once

#include <math.h>

namespace rrea_dev {

struct dd {
    double hi, lo;
};

__device__ __forceinline__ dd dd_from(double a) { return dd{a, 0.0}; }

__device__ __forceinline__ dd two_sum(double a, double b)
{
    double const s = a + b;
    double const bb = s - a;
    double const e = (a - (s - bb)) + (b - bb);
    return dd{s, e};
}
__device__ __forceinline__ dd fast_two_sum(double a, double b)
{
    double const s = a + b;
    return dd{s, b - (s - a)};
}
__device__ __forceinline__ dd two_prod(double a, double b)
{
    double const p = a * b;
    return dd{p, fma(a, b, -p)};
}
__device__ __forceinline__ dd dd_add(dd a, dd b)
{
    dd s = two_sum(a.hi, b.hi);
    dd const t = two_sum(a.lo, b.lo);
    s.lo += t.hi;
    s = fast_two_sum(s.hi, s.lo);
    s.lo += t.lo;
    return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ dd dd_neg(dd a) { return dd{-a.hi, -a.lo}; }
__device__ __forceinline__ dd dd_sub(dd a, dd b) { return dd_add(a, dd_neg(b)); }
__device__ __forceinline__ dd dd_mul(dd a, dd b)
{
    dd p = two_prod(a.hi, b.hi);
    p.lo += a.hi * b.lo + a.lo * b.hi;
    return fast_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ dd dd_mul_d(dd a, double b)
{
    dd p = two_prod(a.hi, b);
    p.lo += a.lo * b;
    return fast_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ dd dd_div(dd a, dd b)
{
    double const q1 = a.hi / b.hi;
    dd r = dd_sub(a, dd_mul_d(b, q1));
    double const q2 = r.hi / b.hi;
    r = dd_sub(r, dd_mul_d(b, q2));
    double const q3 = r.hi / b.hi;
    dd const q = fast_two_sum(q1, q2);
    return dd_add(q, dd_from(q3));
}
__device__ __forceinline__ dd dd_sqrt(dd a)
{
    if (!(a.hi > 0.0)) return dd_from(0.0);
    double const x = sqrt(a.hi);
    dd const r = dd_sub(a, two_prod(x, x));
    return fast_two_sum(x, r.hi / (2.0 * x));
}
__device__ __forceinline__ bool dd_lt(dd a, dd b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ bool dd_gt(dd a, dd b) { return dd_lt(b, a); }

// 1/(2n+1) as double-double, n = 0..22 (exact rationals rounded to
// nearest, hi then remainder).
static __constant__ double kDdInvOdd[23][2] = {
    {0x1.0000000000000p+0, 0x0.0p+0},
    {0x1.5555555555555p-2, 0x1.5555555555555p-56},
    {0x1.999999999999ap-3, -0x1.999999999999ap-57},
    {0x1.2492492492492p-3, 0x1.2492492492492p-57},
    {0x1.c71c71c71c71cp-4, 0x1.c71c71c71c71cp-58},
    {0x1.745d1745d1746p-4, -0x1.745d1745d1746p-59},
    {0x1.3b13b13b13b14p-4, -0x1.3b13b13b13b14p-58},
    {0x1.1111111111111p-4, 0x1.1111111111111p-60},
    {0x1.e1e1e1e1e1e1ep-5, 0x1.e1e1e1e1e1e1ep-61},
    {0x1.af286bca1af28p-5, 0x1.af286bca1af28p-59},
    {0x1.8618618618618p-5, 0x1.8618618618618p-59},
    {0x1.642c8590b2164p-5, 0x1.642c8590b2164p-60},
    {0x1.47ae147ae147bp-5, -0x1.eb851eb851eb8p-61},
    {0x1.2f684bda12f68p-5, 0x1.2f684bda12f68p-59},
    {0x1.1a7b9611a7b96p-5, 0x1.1a7b9611a7b96p-61},
    {0x1.0842108421084p-5, 0x1.0842108421084p-60},
    {0x1.f07c1f07c1f08p-6, -0x1.f07c1f07c1f08p-61},
    {0x1.d41d41d41d41dp-6, 0x1.0750750750750p-60},
    {0x1.bacf914c1bad0p-6, -0x1.bacf914c1bad0p-60},
    {0x1.a41a41a41a41ap-6, 0x1.0690690690690p-60},
    {0x1.8f9c18f9c18fap-6, -0x1.f3831f3831f38p-61},
    {0x1.7d05f417d05f4p-6, 0x1.7d05f417d05f4p-62},
    {0x1.6c16c16c16c17p-6, -0x1.f49f49f49f49fp-61},
};
// log(2) to double-double precision.
constexpr double kDdLn2Hi = 0x1.62e42fefa39efp-1;
constexpr double kDdLn2Lo = 0x1.abc9e3b39803fp-56;

// Natural log of a positive finite double-double.  |s| <= 0.1716 after the
// reduction, so 23 series terms bring the truncation below 2^-110.
__device__ __forceinline__ dd dd_log(dd x)
{
    int e = 0;
    double m = frexp(x.hi, &e);  // x.hi = m 2^e, m in [0.5, 1)
    if (m < 0.70710678118654752440) {
        e -= 1;
    }
    dd const xm{ldexp(x.hi, -e), ldexp(x.lo, -e)};
    dd const s = dd_div(dd_sub(xm, dd_from(1.0)), dd_add(xm, dd_from(1.0)));
    dd const s2 = dd_mul(s, s);
    dd acc{kDdInvOdd[22][0], kDdInvOdd[22][1]};
    for (int n = 21; n >= 0; --n) {
        acc = dd_add(dd_mul(acc, s2), dd{kDdInvOdd[n][0], kDdInvOdd[n][1]});
    }
    dd const lm = dd_mul_d(dd_mul(s, acc), 2.0);
    dd const le = dd_add(two_prod(static_cast<double>(e), kDdLn2Hi), dd_from(static_cast<double>(e) * kDdLn2Lo));
    return dd_add(le, lm);
}

}  // namespace rrea_dev
