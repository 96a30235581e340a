// Device-side primitives of the RREA kinetic step: counter RNG, constants,
// error reporting, and the table queries over the schema-6 arena.
//
// Each function restates the reference primitive cited beside it; the
// arithmetic is kept operation-for-operation so that, compiled without FMA
// contraction, results agree with the reference to the last ulp except where
// the device libm (log/exp/sin/cos/atan2/hypot) rounds differently from the
// host libm.
#pragma once

#include "../rrea_arena.h"
#include "../../../include/rrea_gpu.h"
#include "rrea_fastmath.cuh"

#include <stdint.h>

namespace rrea_dev {

constexpr double kMeC2 = 510998.95000;   // I/RreaConstants.H:9
constexpr double kInvMeC2 = 1.0 / kMeC2;  // k / mc^2 as a product: within an ulp of the quotient
constexpr double kC = 299792458.0;       // I/RreaConstants.H:10
constexpr double kTwoPi = 6.283185307179586476925286766559;
constexpr double kEps = 2.220446049250313080847263336181640625e-16;
constexpr double kDblMin = 2.2250738585072013830902327173324040642192159804623318306e-308;
constexpr double kGl2Node = 0.577350269189625764509148780501957;  // I/RreaGaussLegendre8.H:22

// IEEE classification and comparisons with zero from the bit pattern.  On
// GB300 every FP64 compare (DSETP, isfinite, isnan) takes a slot of the
// narrow FP64 pipe, as much as an FMA; these integer forms give the same
// answer for every input, NaN and signed zero included, on the integer pipe.
__device__ __forceinline__ unsigned long long dbits(double x)
{
    return static_cast<unsigned long long>(__double_as_longlong(x));
}
__device__ __forceinline__ bool finite_bits(double x) { return (__double2hiint(x) & 0x7ff00000) != 0x7ff00000; }
__device__ __forceinline__ bool nan_bits(double x) { return (dbits(x) << 1) > 0xffe0000000000000ull; }
__device__ __forceinline__ bool gt0(double x) { return dbits(x) - 1ull < 0x7ff0000000000000ull; }
__device__ __forceinline__ bool ge0(double x)
{
    unsigned long long const b = dbits(x);
    return b <= 0x7ff0000000000000ull || b == 0x8000000000000000ull;
}
__device__ __forceinline__ bool lt0(double x) { return dbits(x) - 0x8000000000000001ull < 0x7ff0000000000000ull; }
__device__ __forceinline__ bool le0(double x)
{
    unsigned long long const b = dbits(x);
    return b - 0x8000000000000000ull <= 0x7ff0000000000000ull || b == 0ull;
}
__device__ __forceinline__ bool eq0(double x) { return (dbits(x) << 1) == 0ull; }
__device__ __forceinline__ bool ne0(double x) { return (dbits(x) << 1) != 0ull; }
// fmax(x, 0.0) and fmin(x, 0.0) (a NaN operand gives the zero, as fmax and
// fmin return the other operand) with the comparison on the integer pipe.
__device__ __forceinline__ double max0(double x) { return gt0(x) ? x : 0.0; }
__device__ __forceinline__ double min0(double x) { return lt0(x) ? x : 0.0; }

// Division by a divisor that is reused: one IEEE reciprocal y = RN(1/b),
// then one product per quotient, q = RN(a*y), within 1.5 ulp of RN(a/b)
// (finite operands away from overflow and underflow).  On GB300's narrow
// FP64 pipe one DMUL per quotient instead of a division sequence is a
// measured 5 % of the electron kernel; the residual-corrected form
// (Markstein) would restore RN(a/b) at two more FP64 instructions.
struct Divisor {
    double b, y;
};
__host__ __device__ __forceinline__ Divisor make_divisor(double b) { return Divisor{b, 1.0 / b}; }
__device__ __forceinline__ double quot(double a, Divisor const& d) { return a * d.y; }

// Cylindrical radius of a point, sqrt(x^2 + y^2) with one fused rounding of
// the sum: within 1.5 ulp of the reference's std::hypot for every coordinate
// of the domain (|x|, |y| far inside [1e-150, 1e150], where hypot's
// overflow/underflow scaling is never needed) at a third of its FP64 cost.
__device__ __forceinline__ double rz_radius(double x, double y) { return sqrt(fma(x, x, y * y)); }

// Everything a kernel needs that does not change within a step.
struct StepConstants {
    rrea_gpu_config cfg;
    RreaArenaIndex tix;
    double dr, dz;
    Divisor div_dr, div_dz;
    double hm_threshold_eV;
    double photon_cutoff_eV;
    double density_ratio;
    uint64_t step_key;
    double dt_s;
    int32_t hm_enabled;
    int32_t pad;
};

// Per-thread error latch.  Device code never traps: a failing guard records
// its status here and the particle loop unwinds; the kernel then publishes
// the first failure to the global status word.
struct Err {
    int code = 0;
    __device__ __forceinline__ void set(int c)
    {
        if (code == 0) code = c;
    }
};

// ------------------------------------------------------------------ RNG
// O/RreaRng.cpp:9-44 (counter_splitmix64_v1)
__device__ __forceinline__ uint64_t splitmix64(uint64_t v)
{
    v += 0x9e3779b97f4a7c15ULL;
    v = (v ^ (v >> 30)) * 0xbf58476d1ce4e5b9ULL;
    v = (v ^ (v >> 27)) * 0x94d049bb133111ebULL;
    return v ^ (v >> 31);
}

// The seed/particle/step words are fixed for a particle-step: fold them once.
struct RngStream {
    uint64_t folded;  // splitmix(seed) ^ splitmix(pid+c1) ^ splitmix(step+c2)
    __device__ __forceinline__ void init(uint64_t seed, uint64_t pid, uint64_t step)
    {
        folded = splitmix64(seed) ^ splitmix64(pid + 0x100000001b3ULL) ^ splitmix64(step + 0x9e3779b97f4a7c15ULL);
    }
    __device__ __forceinline__ uint64_t counter(uint64_t idx, uint64_t ch) const
    {
        uint64_t s = folded;
        s ^= splitmix64(idx + 0xbf58476d1ce4e5b9ULL);
        s ^= splitmix64(ch + 0x94d049bb133111ebULL);
        return splitmix64(s);
    }
    __device__ __forceinline__ double uniform(uint64_t idx, uint64_t ch) const
    {
        return (__ull2double_rn(counter(idx, ch) >> 12) + 0.5) * 0x1.0p-52;
    }
};

// O/RreaRng.H:17-97
enum : uint64_t {
    kChHardMollerEnergy = 22, kChHardMollerAzimuth = 23,
    kChBremsEnergy = 42, kChBremsAngle = 43, kChBremsAzimuth = 44,
    kChElectronGsAngle = 89, kChElectronGsAzimuth = 90, kChElectronGsFewCount = 91,
    kChElectronGsFewScatter = 92, kChElectronGsFewAzimuth = 93,
    kChElectronCompetingOpticalDepth = 107, kChElectronCompetingChannel = 108,
    kChElectronContinuationOpticalDepth = 124, kChElectronContinuationChannel = 125,
    kChPositronBhabhaEnergy = 74, kChPositronBremsEnergy = 76, kChPositronBremsAngle = 77,
    kChPositronBremsAzimuth = 78, kChPositronAnnihilationPolar = 80, kChPositronAnnihilationAzimuth = 81,
    kChPositronGsAngle = 94, kChPositronGsAzimuth = 95, kChPositronGsFewCount = 96, kChPositronGsFewScatter = 97,
    kChPositronGsFewAzimuth = 98,
    kChPositronCompetingOpticalDepth = 109, kChPositronCompetingChannel = 110,
    kChPositronContinuationOpticalDepth = 126, kChPositronContinuationChannel = 127,
    kChPositronBhabhaAzimuth = 130,
};

// O/RreaParticleInteraction.H:642-710
constexpr uint64_t kSegmentCap = uint64_t{1} << 14;
constexpr uint64_t kLineageCap = uint64_t{1} << 14;  // kRreaTransientLineageCapacity
constexpr uint64_t kEventCap = uint64_t{1} << 13;
__device__ __forceinline__ bool live_hazard_index(uint64_t species, uint64_t segment, uint64_t ordinal,
                                                  uint64_t& out)
{
    if (segment >= kSegmentCap) return false;
    if (ordinal == 0U) {
        out = segment;
        return true;
    }
    if (ordinal >= kEventCap) return false;
    out = (uint64_t{0} << 51) | (species << 49) | (uint64_t{1} << 35) | (segment << 21) | (ordinal << 8);
    return true;
}

// ------------------------------------------------------------------ tables
// Every table grid searched here (energies, path lengths, CDF nodes) holds
// non-negative finite doubles, and so does every query.  For such values the
// IEEE-754 order equals the order of the bit patterns read as signed 64-bit
// integers (after mapping -0.0 to +0.0), so the searches compare integers:
// the same result as comparing doubles, issued on the integer pipe instead
// of GB300's narrow FP64 pipe.
__device__ __forceinline__ long long order_key(double v)
{
    long long const b = __double_as_longlong(v);
    return b == static_cast<long long>(0x8000000000000000ULL) ? 0LL : b;
}

// First index i in [0, n) with x[i] >= q (std::lower_bound), n if none.
__device__ __forceinline__ int lower_bound(const double* __restrict__ x, int n, double q)
{
    long long const qk = order_key(q);
    const long long* __restrict__ xk = reinterpret_cast<const long long*>(x);
    int lo = 0, count = n;
    while (count > 0) {
        int const step = count >> 1;
        int const mid = lo + step;
        if (__ldg(xk + mid) < qk) {
            lo = mid + 1;
            count -= step + 1;
        } else {
            count = step;
        }
    }
    return lo;
}

// Bracket of one query on a hot-table grid, shared by every table that uses
// the same grid (RreaInteractionTable::Interpolate's lower_bound and
// node-exact tests, S/RreaInteractionTables.cpp:1598-1609).
struct Bracket {
    int kind;   // 0 front, 1 back, 2 exact node hi, 3 interior (lo = hi-1)
    int hi;
    double q;
    double t;   // log-space fraction, computed on first use (kind == 3)
    bool have_t;
};

__device__ __forceinline__ bool bracket_hot(const double* __restrict__ arena, RreaTable1DIndex const& h,
                                            double q, Bracket& b, Err& err)
{
    const double* x = arena + h.x;
    int const n = h.n;
    b.q = q;
    b.have_t = false;
    b.t = 0.0;
    if (!finite_bits(q) || q < __ldg(x) || q > __ldg(x + n - 1)) {
        err.set(RREA_GPU_ERR_RANGE);
        return false;
    }
    int const up = lower_bound(x, n, q);
    if (up == 0) { b.kind = 0; b.hi = 0; return true; }
    if (up == n) { b.kind = 1; b.hi = n - 1; return true; }
    b.hi = up;
    if (__ldg(x + up) == q) { b.kind = 2; return true; }
    b.kind = 3;
    return true;
}

// The interpolation fraction of an interior bracket: linear in x for linear
// tables, in log x otherwise (S/RreaInteractionTables.cpp:1610-1616).
__device__ __forceinline__ double bracket_t(const double* __restrict__ arena, RreaTable1DIndex const& h, Bracket& b)
{
    if (!b.have_t) {
        int const up = b.hi;
        // the node spacing's reciprocal is stored (rrea_arena.h)
        if (h.mode == RREA_INTERP_LINEAR) {
            b.t = (b.q - __ldg(arena + h.x + up - 1)) * __ldg(arena + h.ix + up);
        } else {
            b.t = (flog(arena, b.q) - __ldg(arena + h.lx + up - 1)) * __ldg(arena + h.ilx + up);
        }
        b.have_t = true;
    }
    return b.t;
}

// Value of one hot table at a prepared bracket
// (S/RreaInteractionTables.cpp:1599-1629).
__device__ __forceinline__ double eval_hot(const double* __restrict__ arena, RreaTable1DIndex const& h,
                                           Bracket& b, Err& err)
{
    const double* y = arena + h.y;
    if (b.kind == 0) return __ldg(y);
    if (b.kind == 1) return __ldg(y + h.n - 1);
    if (b.kind == 2) return __ldg(y + b.hi);
    bracket_t(arena, h, b);
    double const ylo = __ldg(y + b.hi - 1), yhi = __ldg(y + b.hi);
    if (h.mode == RREA_INTERP_LINEAR) return ylo + b.t * (yhi - ylo);
    bool const pos = gt0(ylo) && gt0(yhi);
    if (h.mode == RREA_INTERP_LOGX_LINEAR || (h.mode == RREA_INTERP_LOGLOG_ZERO_THRESHOLD && !pos)) {
        return ylo + b.t * (yhi - ylo);
    }
    if (!pos) {
        err.set(RREA_GPU_ERR_INVALID_STATE);
        return 0.0;
    }
    const double* ly = arena + h.ly;
    double const llo = __ldg(ly + b.hi - 1), lhi = __ldg(ly + b.hi);
    return fexp(arena, llo + b.t * (lhi - llo));
}

__device__ __forceinline__ double interpolate(const double* __restrict__ arena, RreaTable1DIndex const& h, double q,
                                              Err& err)
{
    Bracket b;
    if (!bracket_hot(arena, h, q, b, err)) return 0.0;
    return eval_hot(arena, h, b, err);
}

// Whether a hot table is strictly positive at a prepared bracket, without
// evaluating its exponential: an interior bracket with two positive nodes is
// exp(finite) > 0 in the log-log modes (node logs are O(10), far from
// underflow); every other case evaluates the value exactly as eval_hot does.
__device__ __forceinline__ bool positive_hot(const double* __restrict__ arena, RreaTable1DIndex const& h,
                                             Bracket& b, Err& err)
{
    if (b.kind == 3 && h.mode != RREA_INTERP_LINEAR && h.mode != RREA_INTERP_LOGX_LINEAR) {
        const double* y = arena + h.y;
        if (__ldg(y + b.hi - 1) > 0.0 && __ldg(y + b.hi) > 0.0) return true;
    }
    return eval_hot(arena, h, b, err) > 0.0;
}

// S/RreaInteractionTables.cpp:624-648 (interp_semilogx_strict).  `lq`, when
// not NaN, is log(q) already computed by the caller for the same q.
// `ilx` holds the reciprocal log spacings of the grid.
__device__ __forceinline__ double semilogx(const double* __restrict__ x, const double* __restrict__ lx,
                                           const double* __restrict__ ilx, const double* __restrict__ y, int n,
                                           double q, Err& err, double lq = __builtin_nan(""))
{
    if (!finite_bits(q) || q < __ldg(x) || q > __ldg(x + n - 1)) {
        err.set(RREA_GPU_ERR_RANGE);
        return 0.0;
    }
    if (q == __ldg(x)) return __ldg(y);
    if (q == __ldg(x + n - 1)) return __ldg(y + n - 1);
    int const hi = lower_bound(x, n, q);
    if (__ldg(x + hi) == q) return __ldg(y + hi);
    int const lo = hi - 1;
    double const lqq = nan_bits(lq) ? log(q) : lq;
    double const t = (lqq - __ldg(lx + lo)) * __ldg(ilx + hi);
    return __ldg(y + lo) + t * (__ldg(y + hi) - __ldg(y + lo));
}

// S/RreaInteractionTables.cpp:110-119
__device__ __forceinline__ double mfp_from_inverse(double inv, Err& err)
{
    if (!finite_bits(inv) || lt0(inv)) {
        err.set(RREA_GPU_ERR_INVALID_STATE);
        return 1.0e99;
    }
    return gt0(inv) ? 1.0 / inv : 1.0e99;
}

// The rate 1/MFP of an inverse-MFP table value as the reference forms it,
// 1 / mfp_from_inverse(inv): 1e-99 for a zero value (the 1e99 m MFP), and
// for a normal positive value 1 / (1 / inv), which is inv to within an ulp;
// returning inv saves two FP64 division sequences per rate.
__device__ __forceinline__ double rate_from_inverse(double inv, Err& err)
{
    if (!finite_bits(inv) || lt0(inv)) {
        err.set(RREA_GPU_ERR_INVALID_STATE);
        return 1.0e-99;
    }
    if (eq0(inv)) return 1.0e-99;
    if (inv < kDblMin) return 1.0 / (1.0 / inv);  // subnormal: 1/inv may overflow
    return inv;
}

// O/RreaMaterialPath.H:213-222
__device__ __forceinline__ double frozen_rate(double v, Err& err)
{
    if (!finite_bits(v) || lt0(v)) {
        err.set(RREA_GPU_ERR_INVALID_STATE);
        return 0.0;
    }
    return v;
}

__device__ __forceinline__ bool charged_in_range(RreaArenaIndex const& ix, double e)
{
    return finite_bits(e) && e >= ix.charged_min_eV && e <= ix.charged_max_eV;
}

// Conditional inverse-CDF sampling: S/RreaInteractionTables.cpp:995-1069;
// `moller` selects the Moller variant (:2584-2653) that log-interpolates
// between groups without the positivity test.
__device__ __forceinline__ double sample_conditional(const double* __restrict__ arena, RreaCondCdfIndex const& ci,
                                                     double e, double cdf_u, bool moller, Err& err)
{
    const double* prim = arena + ci.primary;
    const double* lprim = arena + ci.lprimary;
    const double* start = arena + ci.start;
    const double* u = arena + ci.u;
    const double* v = arena + ci.v;
    cdf_u = max0(fmin(1.0, cdf_u));
    int const ng = ci.ng;
    if (!finite_bits(e) || e < __ldg(prim) || e > __ldg(prim + ng - 1)) {
        err.set(RREA_GPU_ERR_RANGE);
        return 0.0;
    }
    auto sample_group = [&](int g) {
        int const b = static_cast<int>(__ldg(start + g));
        int const en = static_cast<int>(__ldg(start + g + 1));
        int const up = b + lower_bound(u + b, en - b, cdf_u);
        if (up == b) return __ldg(v + b);
        if (up == en) return __ldg(v + en - 1);
        int const lo = up - 1;
        double const denom = __ldg(u + up) - __ldg(u + lo);
        double const t = gt0(denom) ? (cdf_u - __ldg(u + lo)) / denom : 0.0;
        return __ldg(v + lo) + t * (__ldg(v + up) - __ldg(v + lo));
    };
    int const up = lower_bound(prim, ng, e);
    if (up == 0) return sample_group(0);
    if (up == ng) return sample_group(ng - 1);
    if (__ldg(prim + up) == e) return sample_group(up);
    int const lo = up - 1;
    double const y0 = sample_group(lo);
    double const y1 = sample_group(up);
    double const t = (log(e) - __ldg(lprim + lo)) / (__ldg(lprim + up) - __ldg(lprim + lo));
    if (moller || (gt0(y0) && gt0(y1))) {
        return exp(log(y0) + t * (log(y1) - log(y0)));
    }
    return y0 + t * (y1 - y0);
}

// S/RreaInteractionTables.cpp:1071-1110.  The group means are per-group
// constants; the loader accumulates them once in the reference's order and
// stores them (and their logs) in the arena.
__device__ __forceinline__ double group_mean(const double* __restrict__ arena, RreaCondCdfIndex const& ci, int g)
{
    return __ldg(arena + ci.mean + g);
}

__device__ __forceinline__ double mean_conditional(const double* __restrict__ arena, RreaCondCdfIndex const& ci,
                                                   double e, Err& err)
{
    const double* prim = arena + ci.primary;
    const double* lprim = arena + ci.lprimary;
    int const ng = ci.ng;
    if (e < __ldg(prim) || e > __ldg(prim + ng - 1)) {
        err.set(RREA_GPU_ERR_RANGE);
        return 0.0;
    }
    int const up = lower_bound(prim, ng, e);
    if (up == 0) return group_mean(arena, ci, 0);
    if (up == ng) return group_mean(arena, ci, ng - 1);
    if (__ldg(prim + up) == e) return group_mean(arena, ci, up);
    int const lo = up - 1;
    double const y0 = group_mean(arena, ci, lo), y1 = group_mean(arena, ci, up);
    double const t = (log(e) - __ldg(lprim + lo)) / (__ldg(lprim + up) - __ldg(lprim + lo));
    if (gt0(y0) && gt0(y1)) {
        double const l0 = __ldg(arena + ci.lmean + lo), l1 = __ldg(arena + ci.lmean + up);
        return exp(l0 + t * (l1 - l0));
    }
    return y0 + t * (y1 - y0);
}

// S/RreaInteractionTables.cpp:807-827
// `ilg` holds the reciprocal log spacings of the grid.
__device__ __forceinline__ void log_bracket(const double* __restrict__ g, const double* __restrict__ lg,
                                            const double* __restrict__ ilg, int n, double q, int& i, double& frac,
                                            Err& err, double lq = __builtin_nan(""))
{
    int const last = n - 1;
    if (!finite_bits(q) || q < __ldg(g) || q > __ldg(g + last)) {
        err.set(RREA_GPU_ERR_RANGE);
        i = 0;
        frac = 0.0;
        return;
    }
    if (q == __ldg(g)) { i = 0; frac = 0.0; return; }
    if (q == __ldg(g + last)) { i = last - 1; frac = 1.0; return; }
    int lo = 0, hi = last;
    long long const qk = order_key(q);
    const long long* __restrict__ gk = reinterpret_cast<const long long*>(g);
    while (hi - lo > 1) {
        int const m = (lo + hi) / 2;
        if (__ldg(gk + m) <= qk) lo = m; else hi = m;
    }
    i = lo;
    double const llo = __ldg(lg + lo), lhi = __ldg(lg + hi);
    if (lhi == llo) {
        frac = (q == __ldg(g + lo)) ? 0.0 : 1.0;
        return;
    }
    frac = ((nan_bits(lq) ? log(q) : lq) - llo) * __ldg(ilg + hi);
}

// S/RreaInteractionTables.cpp:831-891 (node logs read precomputed)
__device__ __forceinline__ double sample_gs_angle(const double* __restrict__ arena, RreaAngleIndex const& a,
                                                  double e, double n, double u, Err& err,
                                                  double le = __builtin_nan(""))
{
    int const np = a.np, nu = a.nu;
    int ie = 0, ip = 0;
    double te = 0.0, tn = 0.0;
    log_bracket(arena + a.e, arena + a.le, arena + a.ile, a.ne, e, ie, te, err, le);
    log_bracket(arena + a.p, arena + a.lp, arena + a.ilp, a.np, n, ip, tn, err, flog(arena, n));
    if (err.code) return 1.0;
    const double* lomc = arena + a.lomc;
    const double* cu = arena + a.u;
    const double* lur = arena + a.lur;
    const double* ilur = arena + a.ilur;
    const double* icu = arena + a.iu;
    // x / lur[k] and x / u[k] as products with the stored reciprocals; a
    // zero node (reciprocal stored as 0) keeps the reference's division
    auto by_lur = [&](double x, int k) {
        double const r = __ldg(ilur + k);
        return ne0(r) ? x * r : x / __ldg(lur + k);
    };
    auto by_u = [&](double x, int k) {
        double const r = __ldg(icu + k);
        return ne0(r) ? x * r : x / __ldg(cu + k);
    };
    size_t const b00 = (static_cast<size_t>(ie) * np + ip) * nu;
    size_t const b10 = (static_cast<size_t>(ie + 1) * np + ip) * nu;
    size_t const b01 = (static_cast<size_t>(ie) * np + ip + 1) * nu;
    size_t const b11 = (static_cast<size_t>(ie + 1) * np + ip + 1) * nu;
    double const w00 = (1 - te) * (1 - tn), w10 = te * (1 - tn), w01 = (1 - te) * tn, w11 = te * tn;
    auto omc_at = [&](int iu) {
        double const lxx = w00 * __ldg(lomc + b00 + iu) + w10 * __ldg(lomc + b10 + iu)
            + w01 * __ldg(lomc + b01 + iu) + w11 * __ldg(lomc + b11 + iu);
        double const cos_node = 1.0 - fexp(arena, lxx);
        return fmax(1.0 - cos_node, kDblMin);
    };
    int const first = 1, last = nu - 2;
    double one_minus_cos;
    if (last <= first) {
        one_minus_cos = omc_at(first);
    } else if (u <= __ldg(cu + first)) {
        double const d1 = omc_at(first), d2 = omc_at(first + 1);
        double const u1 = __ldg(cu + first);
        double const slope = by_lur(flog(arena, d2 / d1), first);
        double const ueff = fmax(u, u1 * 1.0e-6);
        one_minus_cos = d1 * fexp(arena, slope * flog(arena, by_u(ueff, first)));
    } else if (u >= __ldg(cu + last)) {
        one_minus_cos = omc_at(last);
    } else {
        int lo = first, hi = last;
        long long const uk = order_key(u);
        const long long* __restrict__ cuk = reinterpret_cast<const long long*>(cu);
        while (hi - lo > 1) {
            int const m = (lo + hi) / 2;
            if (__ldg(cuk + m) <= uk) lo = m; else hi = m;
        }
        double const d0 = omc_at(lo), d1 = omc_at(hi);
        // hi == lo + 1 here, so the denominator is the precomputed node ratio log.
        double const fu = by_lur(flog(arena, by_u(u, lo)), lo);
        one_minus_cos = d0 * fexp(arena, fu * flog(arena, d1 / d0));
    }
    double const c = 1.0 - fmin(2.0, one_minus_cos);
    return fmin(1.0, fmax(-1.0, c));
}

}  // namespace rrea_dev
