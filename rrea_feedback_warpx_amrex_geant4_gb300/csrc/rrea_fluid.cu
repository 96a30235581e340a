// Low-energy carrier fluid on the device: the three carrier densities of
// LowEnergyFluidState (S/LowEnergyFluidState.cpp,
// S/LowEnergyFluidFaceTransport.cpp) on the cell grid, and its coupling into
// the Maxwell substeps of RreaAmrexAdvance::AdvanceOneStep
// (S/RreaAmrexAdvance.cpp:593-838).
//
// Every kernel is a coalesced sweep over cells or faces (i fastest); the
// whole state of a 512 x 4096 grid is ~0.5 GB, so each sweep is bound by HBM
// bandwidth.  Reductions (maxima, minima, flags, sums) pre-reduce across the
// warp and post one atomic per warp into a small word/sum block that the
// host reads once per call (once per coupled step, plus the stiffness probe
// that sizes the substeps).  This file is compiled without FMA contraction
// so that every product and sum rounds as in the reference's host build.
#include "rrea_kernels.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

namespace rrea_dev {
namespace fluid {

constexpr double kQe = 1.602176634e-19;      // I/RreaConstants.H:6
constexpr double kEps0 = 8.8541878128e-12;   // I/RreaConstants.H:7
constexpr double kPi = 3.141592653589793238462643383279502884;
constexpr double kNL = 2.6868e25;            // I/RreaConstants.H:16
constexpr double kVacuum = 1.0e-30;          // carrier_transport_vacuum_density_m3 (I/LowEnergyFluidState.H)
constexpr double kEps = 2.220446049250313e-16;
constexpr double kDblMin = 2.2250738585072014e-308;

using u64 = unsigned long long;

// Bit pattern of a nonnegative value as an ordered unsigned key: adding
// +0.0 turns a -0.0 (from max(-0.0, 0.0)) into +0.0, whose key is 0.
__device__ __forceinline__ u64 bits(double x) { return static_cast<u64>(__double_as_longlong(x + 0.0)); }
// total order of doubles as unsigned keys (negatives flipped)
__device__ __forceinline__ u64 ordered(double x)
{
    u64 const b = static_cast<u64>(__double_as_longlong(x));
    return (b >> 63) ? ~b : (b | 0x8000000000000000ULL);
}

inline u64 host_ordered(double x)
{
    u64 b;
    std::memcpy(&b, &x, sizeof(b));
    return (b >> 63) ? ~b : (b | 0x8000000000000000ULL);
}

__device__ __forceinline__ u64 warp_max(u64 v)
{
    for (int o = 16; o > 0; o >>= 1) {
        u64 const w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w > v ? w : v;
    }
    return v;
}
__device__ __forceinline__ u64 warp_min(u64 v)
{
    for (int o = 16; o > 0; o >>= 1) {
        u64 const w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w < v ? w : v;
    }
    return v;
}
__device__ __forceinline__ double warp_sum(double v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ bool lane0() { return (threadIdx.x & 31) == 0; }
// One atomic per warp; every lane of the warp must call these (the kernels
// below run whole warps through their grid-stride loops and reduce after).
__device__ __forceinline__ void post_max(u64* w, u64 v)
{
    v = warp_max(v);
    if (lane0() && v) atomicMax(w, v);
}
__device__ __forceinline__ void post_min(u64* w, u64 v)
{
    v = warp_min(v);
    if (lane0()) atomicMin(w, v);
}
__device__ __forceinline__ void post_sum(double* s, double v)
{
    v = warp_sum(v);
    if (lane0() && v != 0.0) atomicAdd(s, v);
}

// rz_shell_volume (I/RreaConstants.H:37-44)
__device__ __forceinline__ double shell_volume(double r_in, double r_out, double dz)
{
    double const a = r_in > 0.0 ? r_in : 0.0;
    double const b = r_out > 0.0 ? r_out : 0.0;
    return kPi * (b * b - a * a) * dz;
}

// MobilityLaw::At (I/LowEnergyFluidState.H:30-41)
struct Law {
    int reduced;
    double absolute, reduced_mobility, floor;
    __device__ double at(double chi) const { return reduced ? reduced_mobility / fmax(chi, floor) : absolute; }
};

// checked_density_ratio (I/LowEnergyFluidState.H:49-64)
__device__ __forceinline__ double checked_ratio(const double* chi, int64_t k, double scalar)
{
    double const v = chi ? chi[k] : scalar;
    if (!isfinite(v) || v <= 0.0) return scalar > 0.0 ? scalar : 1.0;
    return v;
}

// amrex::max / amrex::min as the reference uses them on finite values
__device__ __forceinline__ double dmax(double a, double b) { return a < b ? b : a; }
__device__ __forceinline__ double dmin(double a, double b) { return b < a ? b : a; }

// exact_pair_loss (S/LowEnergyFluidState.cpp:41-64)
__device__ double pair_loss(double a, double b, double alpha, double dt)
{
    double const small = dmin(a, b);
    double const large = dmax(a, b);
    if (!(small > 0.0) || !(alpha > 0.0) || !(dt > 0.0)) return 0.0;
    double const delta = large - small;
    double remaining;
    if (delta <= 1.0e-12 * dmax(large, 1.0)) {
        remaining = small / (1.0 + alpha * small * dt);
    } else {
        double const ratio = (small / large) * exp(-alpha * delta * dt);
        remaining = ratio >= 1.0 ? small : delta * ratio / (1.0 - ratio);
    }
    return small - dmin(dmax(remaining, 0.0), small);
}

struct Grid {
    int nr, nz;
    double r_lo, z_lo, dr, dz;
    int periodic_z;
    __device__ int64_t cell(int i, int j) const
    {
        if (periodic_z) j = ((j % nz) + nz) % nz;
        return static_cast<int64_t>(i) + static_cast<int64_t>(nr) * j;
    }
};

struct ReactParams {
    int64_t n;
    double dt;
    double nu_const, decay_const, factor_const;
    double a_ei, a_ii, det, det_fraction;
    double max_rate_det;   // max(detachment, 0) for the stiffness bound
    double a_ei_raw, a_ii_raw;
    int table, clear;
};

// UpdateFromIonizationSource (S/LowEnergyFluidState.cpp:105-308) per cell,
// with the MaxReactionFrequency bound (:310-343) of the state it starts from.
__global__ void react_kernel(ReactParams p, double* __restrict__ ne, double* __restrict__ np, double* __restrict__ nn,
                             double* __restrict__ se, double* __restrict__ sp, double* __restrict__ sn,
                             double* __restrict__ rho, const double* __restrict__ nu_cell, u64* words, int w_rate,
                             int w_residual, int w_nan)
{
    u64 worst = 0, rate_max = 0;
    int nan = 0;
    int64_t const stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    int64_t const first = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    for (int64_t k = first; k < p.n; k += stride) {
        double nu = p.nu_const, decay = p.decay_const, factor = p.factor_const;
        if (p.table) {
            nu = nu_cell[k];
            double const x = nu * p.dt;
            decay = exp(-x);
            factor = nu > 0.0 ? -expm1(-x) / nu : p.dt;
        }
        double const e0 = dmax(ne[k], 0.0);
        double const p0 = dmax(np[k], 0.0);
        double const m0 = dmax(nn[k], 0.0);
        if (w_rate >= 0) {
            double const att = p.table ? nu_cell[k] : p.nu_const;
            double const r = att + p.max_rate_det + p.a_ei_raw * (e0 + p0) + p.a_ii_raw * (p0 + m0);
            u64 const b = bits(fabs(r));
            rate_max = b > rate_max ? b : rate_max;
        }
        double const s_low = dmax(se[k], 0.0);
        double const d_pos = dmax(sp[k], 0.0) * p.dt;
        double const d_neg = dmax(sn[k], 0.0) * p.dt;
        double const d_low = s_low * p.dt;
        rho[k] += kQe * (d_pos - d_neg - d_low);
        double const expected = kQe * (p0 + d_pos - m0 - d_neg - e0 - d_low);
        double const e1 = nu > 0.0 ? e0 * decay + s_low * factor : e0 + d_low;
        double const attached = dmax(e0 + d_low - e1, 0.0);
        double e = dmax(e1, 0.0);
        double q = p0 + d_pos;
        double m = m0 + d_neg + attached;
        if (p.det_fraction > 0.0) {
            double const freed = m * p.det_fraction;
            m -= freed;
            e += freed;
        }
        double const l_ei = pair_loss(e, q, p.a_ei, p.dt);
        e = dmax(e - l_ei, 0.0);
        q = dmax(q - l_ei, 0.0);
        double const l_ii = pair_loss(q, m, p.a_ii, p.dt);
        q = dmax(q - l_ii, 0.0);
        m = dmax(m - l_ii, 0.0);
        ne[k] = e;
        np[k] = q;
        nn[k] = m;
        if (p.clear) {
            se[k] = 0.0;
            sp[k] = 0.0;
            sn[k] = 0.0;
        }
        double const actual = kQe * (q - m - e);
        double const scale = dmax(fabs(expected) + kQe * (fabs(q) + fabs(m) + fabs(e)), kDblMin);
        double const r = fabs(actual - expected) / scale;
        if (isnan(r)) nan = 1;
        else if (bits(r) > worst) worst = bits(r);
    }
    post_max(words + w_residual, worst);
    if (w_rate >= 0) post_max(words + w_rate, rate_max);
    if (__any_sync(0xffffffffu, nan) && lane0()) atomicOr(words + w_nan, 1ULL);
}

// MaxReactionFrequency alone (S/LowEnergyFluidState.cpp:310-343)
__global__ void max_rate_kernel(ReactParams p, const double* __restrict__ ne, const double* __restrict__ np,
                                const double* __restrict__ nn, const double* __restrict__ nu_cell, u64* word)
{
    u64 m = 0;
    int64_t const stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t k = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; k < p.n; k += stride) {
        double const att = p.table ? nu_cell[k] : p.nu_const;
        double const r = att + p.max_rate_det + p.a_ei_raw * (dmax(ne[k], 0.0) + dmax(np[k], 0.0))
            + p.a_ii_raw * (dmax(np[k], 0.0) + dmax(nn[k], 0.0));
        u64 const b = bits(fabs(r));
        m = b > m ? b : m;
    }
    post_max(word, m);
}

// ComputeConductivity (S/LowEnergyFluidState.cpp:345-421)
__global__ void conductivity_kernel(int64_t n, int electrons, int ions, Law pos, Law neg, Law ele, double scalar_chi,
                                    const double* __restrict__ chi, const double* __restrict__ mu_cell,
                                    const double* __restrict__ ne, const double* __restrict__ np,
                                    const double* __restrict__ nn, double* __restrict__ sigma, double* __restrict__ tau)
{
    int64_t const stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t k = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; k < n; k += stride) {
        double const d = checked_ratio(chi, k, scalar_chi);
        double v = 0.0;
        if (electrons) v += (mu_cell ? mu_cell[k] : ele.at(d)) * dmax(ne[k], 0.0);
        if (ions) v += pos.at(d) * dmax(np[k], 0.0) + neg.at(d) * dmax(nn[k], 0.0);
        v *= kQe;
        double const s = dmax(v, 0.0);
        sigma[k] = s;
        tau[k] = s > 0.0 ? kEps0 / s : 1.0e300;
    }
}

// ComputeFluidChargeDensity (S/LowEnergyFluidState.cpp:423-455)
__global__ void charge_kernel(int64_t n, const double* __restrict__ ne, const double* __restrict__ np,
                              const double* __restrict__ nn, double* __restrict__ rho)
{
    int64_t const stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t k = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; k < n; k += stride) {
        double const p = dmax(np[k], 0.0), m = dmax(nn[k], 0.0), e = dmax(ne[k], 0.0);
        double net = p - m - e;
        if (fabs(net) <= 64.0 * kEps * (p + m + e)) net = 0.0;
        rho[k] = kQe * net;
    }
}

// RreaEventAccumulator::NormalizeAndSync for the three fluid sources
// (S/RreaEventAccumulator.cpp:280-331): count / (V dt)
__global__ void normalize_sources_kernel(Grid g, double dt, const double* __restrict__ cells,
                                         double* __restrict__ se, double* __restrict__ sp, double* __restrict__ sn)
{
    int64_t const n = static_cast<int64_t>(g.nr) * g.nz;
    int64_t const stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t k = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; k < n; k += stride) {
        int const i = static_cast<int>(k % g.nr);
        double const r_in = g.r_lo + static_cast<double>(i) * g.dr;
        double const denom = shell_volume(r_in, r_in + g.dr, g.dz) * dt;
        se[k] = denom > 0.0 ? cells[k] / denom : 0.0;
        sp[k] = denom > 0.0 ? cells[n + k] / denom : 0.0;
        sn[k] = denom > 0.0 ? cells[2 * n + k] / denom : 0.0;
    }
}

// The closure table on the device: 11 columns of `n` nodes.
struct Closure {
    int n;
    const double *en, *log_en, *k0, *log_k0, *nu2, *nu3, *log_nu3, *dl, *log_dl, *dt, *log_dt;
};

// LowEnergyElectronClosure::Evaluate (S/RreaInteractionTables.cpp:3406-3478);
// status 0 in range, 1 held below, 2 above range, 3 invalid.
__device__ void closure_eval(Closure const& t, double en, int& status, double out[5])
{
    out[0] = out[1] = out[2] = out[3] = out[4] = 0.0;
    if (t.n == 0 || !isfinite(en) || en < 0.0) {
        status = 3;
        return;
    }
    int node = t.n;
    if (en <= t.en[0]) {
        status = en < t.en[0] ? 1 : 0;
        node = 0;
    } else if (en >= t.en[t.n - 1]) {
        status = en > t.en[t.n - 1] ? 2 : 0;
        node = t.n - 1;
    }
    if (node < t.n) {
        out[0] = t.k0[node];
        out[1] = t.nu2[node];
        out[2] = t.nu3[node];
        out[3] = t.dl[node];
        out[4] = t.dt[node];
        return;
    }
    status = 0;
    int lo = 0, hi = t.n;   // first node above en (upper_bound)
    while (lo < hi) {
        int const mid = (lo + hi) >> 1;
        if (t.en[mid] <= en) lo = mid + 1;
        else hi = mid;
    }
    hi = lo;
    lo = hi - 1;
    if (en == t.en[lo]) {
        out[0] = t.k0[lo];
        out[1] = t.nu2[lo];
        out[2] = t.nu3[lo];
        out[3] = t.dl[lo];
        out[4] = t.dt[lo];
        return;
    }
    double const f = (log(en) - t.log_en[lo]) / (t.log_en[hi] - t.log_en[lo]);
    out[0] = exp(t.log_k0[lo] + f * (t.log_k0[hi] - t.log_k0[lo]));
    double const a = t.nu2[lo], b = t.nu2[hi];
    out[1] = a > 0.0 && b > 0.0 ? exp(log(a) + f * log(b / a)) : a + f * (b - a);
    out[2] = exp(t.log_nu3[lo] + f * (t.log_nu3[hi] - t.log_nu3[lo]));
    out[3] = exp(t.log_dl[lo] + f * (t.log_dl[hi] - t.log_dl[lo]));
    out[4] = exp(t.log_dt[lo] + f * (t.log_dt[hi] - t.log_dt[lo]));
}

// BuildElectronClosureCellFields (S/LowEnergyFluidFaceTransport.cpp:1034-1243)
__global__ void closure_kernel(Closure t, Grid g, double scalar_chi, const double* __restrict__ chi,
                               const double* __restrict__ er, const double* __restrict__ ez,
                               const double* __restrict__ ne, const double* __restrict__ src, double* __restrict__ mu,
                               double* __restrict__ nu, double* __restrict__ d3, u64* words, double* sums, int w_held,
                               int w_above, int w_invalid, int w_min_en, int w_max_en, int s_count, int s_held_count,
                               int s_source)
{
    int64_t const n = static_cast<int64_t>(g.nr) * g.nz;
    u64 held = 0, above = 0, invalid = 0, min_en = ~0ULL, max_en = 0;
    double count = 0.0, held_count = 0.0, source = 0.0;
    int64_t const stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t k = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; k < n; k += stride) {
        if (mu) mu[k] = 0.0;
        if (nu) nu[k] = 0.0;
        if (d3) {
            d3[k] = 0.0;
            d3[n + k] = 0.0;
            d3[2 * n + k] = 0.0;
        }
        double const x = chi ? chi[k] : scalar_chi;
        double const e_mag = hypot(er[k], ez[k]);
        double const ev = ne ? ne[k] : 0.0;
        double const sv = src ? src[k] : 0.0;
        if (!isfinite(x) || !(x > 0.0) || !isfinite(e_mag) || !isfinite(ev) || !isfinite(sv)) {
            ++invalid;
            continue;
        }
        double const en = e_mag * 1.0e21 / (x * kNL);
        int status = 3;
        double co[5];
        closure_eval(t, en, status, co);
        if (status == 1) ++held;
        if (status == 2) ++above;
        if (status == 3) {
            ++invalid;
            continue;
        }
        min_en = bits(en) < min_en ? bits(en) : min_en;
        max_en = bits(en) > max_en ? bits(en) : max_en;
        int const i = static_cast<int>(k % g.nr);
        double const r_in = g.r_lo + static_cast<double>(i) * g.dr;
        double const volume = shell_volume(r_in, r_in + g.dr, g.dz);
        double const c = dmax(ev, 0.0) * volume;
        count += c;
        source += dmax(sv, 0.0) * volume;
        if (status == 1) held_count += c;
        if (mu) mu[k] = co[0] / x;
        if (nu) nu[k] = co[1] * x + co[2] * x * x;
        if (d3) {
            double const dl = co[3] / x, dt = co[4] / x;
            double br = 0.0, bz = 0.0;
            if (e_mag > 0.0) {
                br = er[k] / e_mag;
                bz = ez[k] / e_mag;
            }
            double const an = dl - dt;
            d3[k] = dt + an * br * br;
            d3[n + k] = an * br * bz;
            d3[2 * n + k] = dt + an * bz * bz;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        held += __shfl_xor_sync(0xffffffffu, held, o);
        above += __shfl_xor_sync(0xffffffffu, above, o);
        invalid += __shfl_xor_sync(0xffffffffu, invalid, o);
    }
    if (lane0()) {
        if (held) atomicAdd(words + w_held, held);
        if (above) atomicAdd(words + w_above, above);
        if (invalid) atomicAdd(words + w_invalid, invalid);
    }
    post_min(words + w_min_en, min_en);
    post_max(words + w_max_en, max_en);
    post_sum(sums + s_count, count);
    post_sum(sums + s_held_count, held_count);
    post_sum(sums + s_source, source);
}

// The tensor check and largest eigenvalue of BuildExplicitFaceTransport
// (S/LowEnergyFluidFaceTransport.cpp:240-294)
__global__ void tensor_check_kernel(int64_t n, const double* __restrict__ d3, u64* words, int w_eig, int w_bad)
{
    u64 eig = 0;
    int bad = 0;
    int64_t const stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t k = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; k < n; k += stride) {
        double const rr = d3[k], rz = d3[n + k], zz = d3[2 * n + k];
        double const det = rr * zz - rz * rz;
        double const det_scale = dmax(dmax(fabs(rr * zz), fabs(rz * rz)), 1.0);
        if (!isfinite(rr) || !isfinite(rz) || !isfinite(zz) || rr < 0.0 || zz < 0.0
            || det < -(512.0 * kEps * det_scale)) {
            bad = 1;
            continue;
        }
        double const e = 0.5 * (rr + zz + hypot(rr - zz, 2.0 * rz));
        eig = bits(e) > eig ? bits(e) : eig;
    }
    post_max(words + w_eig, eig);
    if (__any_sync(0xffffffffu, bad) && lane0()) atomicOr(words + w_bad, 1ULL);
}

struct TransportParams {
    Grid g;
    int enabled[3];
    int from_field;
    Law law[3];
    double scalar_chi;
    double dt;
    double limiter_cfl;
};

// The frozen carrier density of one cell as the flux law reads it: vacuum
// below 1e-30 m^-3.
__device__ __forceinline__ double carrier(const double* __restrict__ old3, int64_t nc, int s, int64_t k)
{
    double const v = dmax(old3[s * nc + k], 0.0);
    return v > kVacuum ? v : 0.0;
}

// BuildExplicitFaceTransport (S/LowEnergyFluidFaceTransport.cpp:200-565):
// one thread per face, radial faces first; the three carriers' number fluxes
// and the face conductivity.  The periodic duplicate of the axial face
// j = nz is computed as face j = 0 (OverrideSync).
__global__ void face_flux_kernel(TransportParams p, const double* __restrict__ old3, const double* __restrict__ chi,
                                 const double* __restrict__ mu_cell, const double* __restrict__ d3,
                                 const double* __restrict__ efr, const double* __restrict__ efr_add,
                                 const double* __restrict__ efz, const double* __restrict__ efz_add,
                                 double* __restrict__ fr, double* __restrict__ fz, u64* words, int w_sigma)
{
    Grid const& g = p.g;
    int const nr = g.nr, nz = g.nz;
    int64_t const nc = static_cast<int64_t>(nr) * nz;
    int64_t const nfr = static_cast<int64_t>(nr + 1) * nz;
    int64_t const nfz = static_cast<int64_t>(nr) * (nz + 1);
    bool const per = g.periodic_z != 0;
    u64 sig_max = 0;
    auto mobility = [&](int s, int64_t k) {
        if (s == 2 && p.from_field) return dmax(mu_cell[k], 0.0);
        return p.law[s].at(checked_ratio(chi, k, p.scalar_chi));
    };
    auto tensor = [&](int i, int j, int comp) { return d3[comp * nc + g.cell(i, j)]; };
    auto cd = [&](int i, int j) { return carrier(old3, nc, 2, g.cell(i, j)); };
    int64_t const stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; t < nfr + nfz; t += stride) {
        int const dir = t < nfr ? 0 : 1;
        int i, j;
        int64_t f;
        double e_face;
        if (dir == 0) {
            f = t;
            i = static_cast<int>(t % (nr + 1));
            j = static_cast<int>(t / (nr + 1));
            e_face = efr_add ? efr[f] + efr_add[f] : efr[f];
        } else {
            f = t - nfr;
            i = static_cast<int>(f % nr);
            j = static_cast<int>(f / nr);
            int64_t const fe = (per && j == nz) ? static_cast<int64_t>(i) : f;
            e_face = efz_add ? efz[fe] + efz_add[fe] : efz[fe];
            if (per && j == nz) j = 0;
        }
        double flux[3] = {0.0, 0.0, 0.0};
        double sigma = 0.0;
        for (int s = 0; s < 3; ++s) {
            if (!p.enabled[s]) continue;
            bool has_lo = true, has_hi = true;
            double n_lo = 0.0, n_hi = 0.0, mu_lo = 0.0, mu_hi = 0.0;
            if (dir == 0) {
                if (i <= 0) {
                    has_lo = has_hi = false;
                } else if (i > nr - 1) {
                    has_hi = false;
                    int64_t const k = g.cell(i - 1, j);
                    n_lo = carrier(old3, nc, s, k);
                    mu_lo = mobility(s, k);
                } else {
                    int64_t const kl = g.cell(i - 1, j), kh = g.cell(i, j);
                    n_lo = carrier(old3, nc, s, kl);
                    n_hi = carrier(old3, nc, s, kh);
                    mu_lo = mobility(s, kl);
                    mu_hi = mobility(s, kh);
                }
            } else if (!per && j <= 0) {
                has_lo = false;
                int64_t const k = g.cell(i, 0);
                n_hi = carrier(old3, nc, s, k);
                mu_hi = mobility(s, k);
            } else if (!per && j > nz - 1) {
                has_hi = false;
                int64_t const k = g.cell(i, nz - 1);
                n_lo = carrier(old3, nc, s, k);
                mu_lo = mobility(s, k);
            } else {
                int64_t const kl = g.cell(i, j - 1), kh = g.cell(i, j);
                n_lo = carrier(old3, nc, s, kl);
                n_hi = carrier(old3, nc, s, kh);
                mu_lo = mobility(s, kl);
                mu_hi = mobility(s, kh);
            }
            if (!has_lo && !has_hi) continue;
            double const mu_face = has_lo && has_hi ? 0.5 * (mu_lo + mu_hi) : (has_lo ? mu_lo : mu_hi);
            double const velocity = (s == 0 ? 1.0 : -1.0) * mu_face * e_face;
            double donor = 0.0;
            if (velocity > 0.0 && has_lo) donor = n_lo;
            else if (velocity < 0.0 && has_hi) donor = n_hi;
            else if (velocity == 0.0 && has_lo && has_hi) donor = 0.5 * (n_lo + n_hi);
            double number_flux = velocity * donor;
            if (s == 2 && p.from_field) {
                double diffusive = 0.0;
                if (dir == 0) {
                    if (i > 0 && i <= nr - 1) {
                        double const d_rr = 0.5 * (tensor(i - 1, j, 0) + tensor(i, j, 0));
                        double const d_rz = 0.5 * (tensor(i - 1, j, 1) + tensor(i, j, 1));
                        double const grad_r = (n_hi - n_lo) / g.dr;
                        auto axial = [&](int ii, int jj) {
                            if (!per && jj <= 0) return (cd(ii, jj + 1) - cd(ii, jj)) / g.dz;
                            if (!per && jj >= nz - 1) return (cd(ii, jj) - cd(ii, jj - 1)) / g.dz;
                            return (cd(ii, jj + 1) - cd(ii, jj - 1)) / (2.0 * g.dz);
                        };
                        double const grad_z = 0.5 * (axial(i - 1, j) + axial(i, j));
                        diffusive = -(d_rr * grad_r + d_rz * grad_z);
                    } else if (i > nr - 1) {
                        diffusive = 2.0 * tensor(i - 1, j, 0) * n_lo / g.dr;
                    }
                } else {
                    if ((!per && j > 0 && j <= nz - 1) || per) {
                        double const d_rz = 0.5 * (tensor(i, j - 1, 1) + tensor(i, j, 1));
                        double const d_zz = 0.5 * (tensor(i, j - 1, 2) + tensor(i, j, 2));
                        auto radial = [&](int ii, int jj) {
                            if (nr - 1 == 0) return 0.0;
                            if (ii <= 0) return (cd(ii + 1, jj) - cd(ii, jj)) / g.dr;
                            if (ii >= nr - 1) return (cd(ii, jj) - cd(ii - 1, jj)) / g.dr;
                            return (cd(ii + 1, jj) - cd(ii - 1, jj)) / (2.0 * g.dr);
                        };
                        double const grad_r = 0.5 * (radial(i, j - 1) + radial(i, j));
                        double const grad_z = (n_hi - n_lo) / g.dz;
                        diffusive = -(d_rz * grad_r + d_zz * grad_z);
                    } else if (j <= 0) {
                        diffusive = -2.0 * tensor(i, 0, 2) * n_hi / g.dz;
                    } else {
                        diffusive = 2.0 * tensor(i, nz - 1, 2) * n_lo / g.dz;
                    }
                }
                if ((diffusive > 0.0 && (!has_lo || n_lo <= 0.0)) || (diffusive < 0.0 && (!has_hi || n_hi <= 0.0))) {
                    diffusive = 0.0;
                }
                number_flux += diffusive;
            }
            flux[s] = number_flux;
            sigma += kQe * mu_face * donor;
        }
        if (fr) {
            if (dir == 0) {
                fr[f] = flux[0];
                fr[nfr + f] = flux[1];
                fr[2 * nfr + f] = flux[2];
            } else {
                fz[f] = flux[0];
                fz[nfz + f] = flux[1];
                fz[2 * nfz + f] = flux[2];
            }
        }
        sig_max = bits(sigma) > sig_max ? bits(sigma) : sig_max;
    }
    post_max(words + w_sigma, sig_max);
}

struct Metric {
    double volume, shell, a_lo, a_hi;
};
__device__ __forceinline__ Metric metric(Grid const& g, int i)
{
    double const r_lo = g.r_lo + static_cast<double>(i) * g.dr;
    double const r_hi = r_lo + g.dr;
    return Metric{shell_volume(r_lo, r_lo + g.dr, g.dz), kPi * dmax(r_hi * r_hi - r_lo * r_lo, 0.0),
                  2.0 * kPi * r_lo * g.dz, 2.0 * kPi * r_hi * g.dz};
}

__device__ __forceinline__ double outgoing(const double* fr, const double* fz, int64_t nfr, int64_t nfz, int nr, int s,
                                           int i, int j, Metric const& m)
{
    double const f_rlo = fr[s * nfr + i + static_cast<int64_t>(nr + 1) * j];
    double const f_rhi = fr[s * nfr + i + 1 + static_cast<int64_t>(nr + 1) * j];
    double const f_zlo = fz[s * nfz + i + static_cast<int64_t>(nr) * j];
    double const f_zhi = fz[s * nfz + i + static_cast<int64_t>(nr) * (j + 1)];
    double o = dmax(f_rhi, 0.0) * m.a_hi + dmax(-f_rlo, 0.0) * m.a_lo;
    o += (dmax(f_zhi, 0.0) + dmax(-f_zlo, 0.0)) * m.shell;
    return o;
}

// The positivity limiter of ApplyExplicitCarrierTransport
// (S/LowEnergyFluidFaceTransport.cpp:588-688): one scale per donor cell and
// carrier.
__global__ void limiter_kernel(TransportParams p, const double* __restrict__ old3, const double* __restrict__ fr,
                               const double* __restrict__ fz, double* __restrict__ scale3, u64* words, double* sums,
                               int w_unlimited, int w_min_scale, int s_before, int s_removed, int s_enumber,
                               int s_elimited)
{
    Grid const& g = p.g;
    int64_t const nc = static_cast<int64_t>(g.nr) * g.nz;
    int64_t const nfr = static_cast<int64_t>(g.nr + 1) * g.nz;
    int64_t const nfz = static_cast<int64_t>(g.nr) * (g.nz + 1);
    u64 unlimited = 0, min_scale = bits(1.0);
    double before = 0.0, removed = 0.0, e_number = 0.0, e_limited = 0.0;
    int64_t const stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t k = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; k < nc; k += stride) {
        int const i = static_cast<int>(k % g.nr);
        int const j = static_cast<int>(k / g.nr);
        Metric const m = metric(g, i);
        for (int s = 0; s < 3; ++s) {
            if (!p.enabled[s]) {
                scale3[s * nc + k] = 1.0;
                continue;
            }
            double const density = dmax(old3[s * nc + k], 0.0);
            double const out = outgoing(fr, fz, nfr, nfz, g.nr, s, i, j, m);
            double const rate = density > 0.0 ? out / (density * dmax(m.volume, 1.0e-300)) : (out > 0.0 ? 1.0e300 : 0.0);
            unlimited = bits(rate) > unlimited ? bits(rate) : unlimited;
            double limiter = 1.0;
            if (out > 0.0) limiter = density > 0.0 ? dmin(1.0, p.limiter_cfl * density * m.volume / (p.dt * out)) : 0.0;
            scale3[s * nc + k] = limiter;
            min_scale = bits(limiter) < min_scale ? bits(limiter) : min_scale;
            before += out;
            removed += (1.0 - limiter) * out;
            if (s == 2) {
                double const en = density * m.volume;
                e_number += en;
                if (limiter < 1.0) e_limited += en;
            }
        }
    }
    post_max(words + w_unlimited, unlimited);
    post_min(words + w_min_scale, min_scale);
    post_sum(sums + s_before, before);
    post_sum(sums + s_removed, removed);
    post_sum(sums + s_enumber, e_number);
    post_sum(sums + s_elimited, e_limited);
}

// Scales every face flux by its donor's limiter (:690-740) and, when asked,
// writes the total face current of AssembleTotalFaceCurrent
// (S/RreaAmrexAdvance.cpp:840-871): qe (G+ - G- - Ge) plus the kinetic
// net-chord current.
__global__ void scale_faces_kernel(TransportParams p, const double* __restrict__ scale3, double* __restrict__ fr,
                                   double* __restrict__ fz, const double* __restrict__ jr_kin,
                                   const double* __restrict__ jz_kin, double* __restrict__ jr, double* __restrict__ jz)
{
    Grid const& g = p.g;
    int const nr = g.nr, nz = g.nz;
    int64_t const nc = static_cast<int64_t>(nr) * nz;
    int64_t const nfr = static_cast<int64_t>(nr + 1) * nz;
    int64_t const nfz = static_cast<int64_t>(nr) * (nz + 1);
    bool const per = g.periodic_z != 0;
    int64_t const stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; t < nfr + nfz; t += stride) {
        double v[3];
        if (t < nfr) {
            int const i = static_cast<int>(t % (nr + 1));
            int const j = static_cast<int>(t / (nr + 1));
            for (int s = 0; s < 3; ++s) {
                double x = fr[s * nfr + t];
                if (x != 0.0) {
                    int const di = x > 0.0 ? i - 1 : i;
                    x = (di >= 0 && di <= nr - 1) ? x * scale3[s * nc + g.cell(di, j)] : 0.0;
                    fr[s * nfr + t] = x;
                }
                v[s] = x;
            }
            if (jr) {
                double c = 0.0;
                c += kQe * v[0];
                c += -kQe * v[1];
                c += -kQe * v[2];
                jr[t] = c + jr_kin[t];
            }
        } else {
            int64_t const f = t - nfr;
            int const i = static_cast<int>(f % nr);
            int const j = static_cast<int>(f / nr);
            for (int s = 0; s < 3; ++s) {
                double x = fz[s * nfz + f];
                if (x != 0.0) {
                    int const dj = x > 0.0 ? j - 1 : j;
                    bool const inside = per || (dj >= 0 && dj <= nz - 1);
                    x = inside ? x * scale3[s * nc + g.cell(i, dj)] : 0.0;
                    fz[s * nfz + f] = x;
                }
                v[s] = x;
            }
            if (jz) {
                double c = 0.0;
                c += kQe * v[0];
                c += -kQe * v[1];
                c += -kQe * v[2];
                jz[f] = c + jz_kin[f];
            }
        }
    }
}

// The realized outgoing CFL, drift speed, conservative update, density
// checks and carrier centres of ApplyExplicitCarrierTransport
// (:742-953, CollectCarrierDriftCenterDiagnostics :956-1032).  Writes the new
// densities into new3 (disabled carriers copied through).
__global__ void update_kernel(TransportParams p, const double* __restrict__ old3, const double* __restrict__ fr,
                              const double* __restrict__ fz, double* __restrict__ new3, double* __restrict__ rho,
                              const double* __restrict__ chi, u64* words, double* sums, int w_rate, int w_speed,
                              int w_min_density, int w_nonfinite, int s_center)
{
    Grid const& g = p.g;
    int const nr = g.nr;
    int64_t const nc = static_cast<int64_t>(nr) * g.nz;
    int64_t const nfr = static_cast<int64_t>(nr + 1) * g.nz;
    int64_t const nfz = static_cast<int64_t>(nr) * (g.nz + 1);
    u64 rate_max = 0, speed_max = 0, min_density = ordered(0.0);
    int nonfinite = 0;
    double cs[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    int64_t const stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t k = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; k < nc; k += stride) {
        int const i = static_cast<int>(k % nr);
        int const j = static_cast<int>(k / nr);
        Metric const m = metric(g, i);
        int64_t const frl = i + static_cast<int64_t>(nr + 1) * j;
        int64_t const fzl = i + static_cast<int64_t>(nr) * j;
        double fl_r[3], fh_r[3], fl_z[3], fh_z[3];
        for (int s = 0; s < 3; ++s) {
            fl_r[s] = fr[s * nfr + frl];
            fh_r[s] = fr[s * nfr + frl + 1];
            fl_z[s] = fz[s * nfz + fzl];
            fh_z[s] = fz[s * nfz + fzl + nr];
        }
        for (int s = 0; s < 3; ++s) {
            double const o = old3[s * nc + k];
            double v = o;
            if (p.enabled[s]) {
                double const density = dmax(o, 0.0);
                double out = dmax(fh_r[s], 0.0) * m.a_hi + dmax(-fl_r[s], 0.0) * m.a_lo;
                out += (dmax(fh_z[s], 0.0) + dmax(-fl_z[s], 0.0)) * m.shell;
                if (density > 0.0) {
                    double const r = out / (density * dmax(m.volume, 1.0e-300));
                    rate_max = bits(r) > rate_max ? bits(r) : rate_max;
                    double const sp[4] = {-fl_r[s], fh_r[s], -fl_z[s], fh_z[s]};
                    for (double x : sp) {
                        double const sv = dmax(x, 0.0) / density;
                        speed_max = bits(sv) > speed_max ? bits(sv) : speed_max;
                    }
                }
                bool const moves = (s < 2) ? p.enabled[0] : p.enabled[2];
                if (moves) {
                    double const r_delta = fh_r[s] * m.a_hi - fl_r[s] * m.a_lo;
                    double const z_delta = (fh_z[s] - fl_z[s]) * m.shell;
                    v = o - p.dt * (r_delta + z_delta) / dmax(m.volume, 1.0e-300);
                }
            }
            new3[s * nc + k] = v;
            if (!isfinite(v)) nonfinite = 1;
            else if (ordered(v) < min_density) min_density = ordered(v);
        }
        double const cr_lo = kQe * (fl_r[0] - fl_r[1] - fl_r[2]);
        double const cr_hi = kQe * (fh_r[0] - fh_r[1] - fh_r[2]);
        double const cz_lo = kQe * (fl_z[0] - fl_z[1] - fl_z[2]);
        double const cz_hi = kQe * (fh_z[0] - fh_z[1] - fh_z[2]);
        double delta = cr_hi * m.a_hi - cr_lo * m.a_lo;
        delta += (cz_hi - cz_lo) * m.shell;
        rho[k] -= p.dt * delta / dmax(m.volume, 1.0e-300);
        // carrier centres of the new state
        double const pc = dmax(new3[k], 0.0) * m.volume;
        double const qc = dmax(new3[nc + k], 0.0) * m.volume;
        double const rc = g.r_lo + (static_cast<double>(i) + 0.5) * g.dr;
        double const zc = g.z_lo + (static_cast<double>(j) + 0.5) * g.dz;
        double const d = chi ? dmax(chi[k], 1.0e-300) : p.scalar_chi;
        cs[0] += pc;
        cs[1] += qc;
        cs[2] += pc * rc;
        cs[3] += pc * zc;
        cs[4] += qc * rc;
        cs[5] += qc * zc;
        cs[6] += pc * d;
        cs[7] += pc * p.law[0].at(d);
    }
    post_max(words + w_rate, rate_max);
    post_max(words + w_speed, speed_max);
    post_min(words + w_min_density, min_density);
    if (__any_sync(0xffffffffu, nonfinite) && lane0()) atomicOr(words + w_nonfinite, 1ULL);
    if (s_center >= 0) {
        for (int c = 0; c < 8; ++c) post_sum(sums + s_center + c, cs[c]);
    }
}

// The fluid and event-source totals of the reduced diagnostics
// (O/RreaCouplingDiagnostics.cpp:318-333, 469-471, 730-736): plain sums of
// the cell values (MultiFab::sum), RZ volume integrals (volume_integral_rz,
// :89-106), maxima and minima, and the step's sources normalised as
// NormalizeAndSync leaves them (rates by V dt, the ionization count and the
// energy loss by V).  out (sums): 0..2 sum ne, np, nn; 3..5 their volume
// integrals; 6 volume integral of rho; 7 sum rho; 8..10 sum of the three
// source rates; 11 ionization count density sum; 12 energy-loss density sum.
// words: max ne, max sigma, min tau (ordered keys).
__global__ void reductions_kernel(Grid g, double dt, const double* __restrict__ ne, const double* __restrict__ np,
                                  const double* __restrict__ nn, const double* __restrict__ rho,
                                  const double* __restrict__ sigma, const double* __restrict__ tau,
                                  const double* __restrict__ cells, double* sums, u64* words)
{
    int64_t const n = static_cast<int64_t>(g.nr) * g.nz;
    double acc[13];
    for (double& a : acc) a = 0.0;
    u64 max_ne = ordered(-1.0e308), max_sigma = ordered(-1.0e308), min_tau = ordered(1.0e308);
    int64_t const stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t k = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; k < n; k += stride) {
        int const i = static_cast<int>(k % g.nr);
        double const r_in = g.r_lo + static_cast<double>(i) * g.dr;
        double const v = shell_volume(r_in, r_in + g.dr, g.dz);
        acc[0] += ne[k];
        acc[1] += np[k];
        acc[2] += nn[k];
        acc[3] += ne[k] * v;
        acc[4] += np[k] * v;
        acc[5] += nn[k] * v;
        acc[6] += rho[k] * v;
        acc[7] += rho[k];
        if (cells) {
            double const vd = v * dt;
            acc[8] += vd > 0.0 ? cells[k] / vd : 0.0;
            acc[9] += vd > 0.0 ? cells[n + k] / vd : 0.0;
            acc[10] += vd > 0.0 ? cells[2 * n + k] / vd : 0.0;
            acc[11] += v > 0.0 ? cells[3 * n + k] / v : 0.0;
            acc[12] += v > 0.0 ? cells[4 * n + k] / v : 0.0;
        }
        max_ne = ordered(ne[k]) > max_ne ? ordered(ne[k]) : max_ne;
        max_sigma = ordered(sigma[k]) > max_sigma ? ordered(sigma[k]) : max_sigma;
        min_tau = ordered(tau[k]) < min_tau ? ordered(tau[k]) : min_tau;
    }
    for (int c = 0; c < 13; ++c) post_sum(sums + c, acc[c]);
    max_ne = warp_max(max_ne);
    max_sigma = warp_max(max_sigma);
    if (lane0()) {
        atomicMax(words, max_ne);
        atomicMax(words + 1, max_sigma);
    }
    post_min(words + 2, min_tau);
}

}  // namespace fluid
}  // namespace rrea_dev

// ===========================================================================
// Host side: the fluid state of one context and its operations.
// ===========================================================================
namespace rrea_launch {

namespace {

using rrea_dev::fluid::u64;

// words of the reduction block
enum Word {
    kWSigma, kWEig, kWTensorBad, kWUnlimited, kWMinScale, kWRate, kWSpeed, kWMinDensity, kWNonfinite, kWResidual,
    kWResidualNan, kWReaction, kWHeld, kWAbove, kWInvalid, kWMinEn, kWMaxEn, kWords
};
enum Sum { kSBefore, kSRemoved, kSENumber, kSELimited, kSCenter, kSCount = kSCenter + 8, kSHeldCount, kSSource, kSums };

double from_bits(u64 b)
{
    double d;
    std::memcpy(&d, &b, sizeof(d));
    return d;
}
u64 to_bits(double d)
{
    u64 b;
    std::memcpy(&b, &d, sizeof(b));
    return b;
}
double from_ordered(u64 k)
{
    return from_bits((k >> 63) ? (k & 0x7FFFFFFFFFFFFFFFULL) : ~k);
}

}  // namespace

struct FluidState {
    FluidGrid grid{};
    rrea_gpu_fluid_config cfg{};
    int64_t n = 0, nfr = 0, nfz = 0;
    double* block = nullptr;   // one allocation for every field below
    double *ne = nullptr, *np = nullptr, *nn = nullptr;   // views into cur3
    double *cur3 = nullptr, *next3 = nullptr;             // carriers (pos, neg, e) x n, double-buffered
    double *rho = nullptr, *se = nullptr, *sp = nullptr, *sn = nullptr, *sigma = nullptr, *tau = nullptr;
    double *chi = nullptr, *mu = nullptr, *nu = nullptr, *d3 = nullptr;
    double *fr = nullptr, *fz = nullptr, *scale3 = nullptr, *jr = nullptr, *jz = nullptr;
    double* sums = nullptr;
    u64* words = nullptr;
    bool chi_bound = false;
    double* closure = nullptr;   // 11 columns
    int closure_n = 0;
    int blocks = 1;
    std::string error;

    void bind_views()
    {
        np = cur3;
        nn = cur3 + n;
        ne = cur3 + 2 * n;
    }
};

namespace {

rrea_dev::fluid::Grid dev_grid(FluidGrid const& g)
{
    return rrea_dev::fluid::Grid{g.nr, g.nz, g.r_lo, g.z_lo, g.dr, g.dz, g.periodic_z};
}

rrea_dev::fluid::Law ion_law(rrea_gpu_fluid_config const& c, bool positive)
{
    return rrea_dev::fluid::Law{c.ion_mobility_model == RREA_GPU_MOBILITY_REDUCED_STP,
                                positive ? c.positive_ion_mobility_m2_per_vs : c.negative_ion_mobility_m2_per_vs,
                                positive ? c.positive_ion_reduced_mobility_stp_m2_per_vs
                                         : c.negative_ion_reduced_mobility_stp_m2_per_vs,
                                c.ion_mobility_density_ratio_floor};
}
rrea_dev::fluid::Law electron_law(rrea_gpu_fluid_config const& c)
{
    return rrea_dev::fluid::Law{0, c.electron_mobility_m2_per_vs, 0.0, c.ion_mobility_density_ratio_floor};
}

bool mobility_table(rrea_gpu_fluid_config const& c)
{
    return c.electron_drift_enable && c.electron_mobility_model == RREA_GPU_MOBILITY_EN_TABLE_FLUX;
}
bool attachment_table(rrea_gpu_fluid_config const& c) { return c.attachment_model == RREA_GPU_ATTACHMENT_EN_TABLE; }

rrea_dev::fluid::Closure dev_closure(FluidState const& s)
{
    int const m = s.closure_n;
    double const* b = s.closure;
    return rrea_dev::fluid::Closure{m,          b,          b + m,      b + 2 * m, b + 3 * m, b + 4 * m,
                                    b + 5 * m,  b + 6 * m,  b + 7 * m,  b + 8 * m, b + 9 * m, b + 10 * m};
}

cudaError_t reset_reductions(FluidState& s, cudaStream_t stream)
{
    u64 init[kWords];
    for (auto& w : init) w = 0;
    init[kWMinScale] = to_bits(1.0);
    init[kWMinDensity] = ~0ULL;
    init[kWMinEn] = ~0ULL;
    cudaError_t e = cudaMemcpyAsync(s.words, init, sizeof(init), cudaMemcpyHostToDevice, stream);
    if (e != cudaSuccess) return e;
    return cudaMemsetAsync(s.sums, 0, sizeof(double) * kSums, stream);
}

struct Readback {
    u64 w[kWords];
    double s[kSums];
};

cudaError_t read_reductions(FluidState& s, Readback& r, cudaStream_t stream)
{
    cudaError_t e = cudaMemcpyAsync(r.w, s.words, sizeof(r.w), cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(r.s, s.sums, sizeof(r.s), cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    return e;
}

rrea_dev::fluid::ReactParams react_params(FluidState const& s, double dt, bool clear)
{
    rrea_gpu_fluid_config const& c = s.cfg;
    rrea_dev::fluid::ReactParams p{};
    p.n = s.n;
    p.dt = dt;
    p.nu_const = std::max(c.attachment_frequency_s, 0.0);
    p.decay_const = std::exp(-p.nu_const * dt);
    p.factor_const = p.nu_const > 0.0 ? (1.0 - p.decay_const) / p.nu_const : dt;
    p.a_ei = c.electron_ion_recombination_coefficient_m3_per_s;
    p.a_ii = c.ion_ion_recombination_coefficient_m3_per_s;
    p.det = std::max(c.detachment_frequency_s, 0.0);
    p.det_fraction = p.det > 0.0 ? -std::expm1(-p.det * dt) : 0.0;
    p.max_rate_det = p.det;
    p.a_ei_raw = c.electron_ion_recombination_coefficient_m3_per_s;
    p.a_ii_raw = c.ion_ion_recombination_coefficient_m3_per_s;
    p.table = attachment_table(c) ? 1 : 0;
    p.clear = clear ? 1 : 0;
    return p;
}

rrea_dev::fluid::TransportParams transport_params(FluidState const& s, double dt)
{
    rrea_gpu_fluid_config const& c = s.cfg;
    rrea_dev::fluid::TransportParams p{};
    p.g = dev_grid(s.grid);
    p.enabled[0] = p.enabled[1] = c.ion_drift_enable ? 1 : 0;
    p.enabled[2] = c.electron_drift_enable ? 1 : 0;
    p.from_field = mobility_table(c) ? 1 : 0;
    p.law[0] = ion_law(c, true);
    p.law[1] = ion_law(c, false);
    p.law[2] = electron_law(c);
    p.scalar_chi = c.transport_density_ratio;
    p.dt = dt;
    p.limiter_cfl = c.ion_drift_cfl * (1.0 - 512.0 * 2.220446049250313e-16);
    return p;
}

}  // namespace

void fluid_free(FluidState* s)
{
    if (!s) return;
    if (s->block) cudaFree(s->block);
    if (s->closure) cudaFree(s->closure);
    delete s;
}

cudaError_t fluid_create(FluidGrid const& g, int blocks, FluidState*& out)
{
    auto* s = new FluidState();
    s->grid = g;
    s->n = static_cast<int64_t>(g.nr) * g.nz;
    s->nfr = static_cast<int64_t>(g.nr + 1) * g.nz;
    s->nfz = static_cast<int64_t>(g.nr) * (g.nz + 1);
    s->blocks = blocks;
    // carriers x2 (double buffer), rho, 3 sources, sigma, tau, chi, mu, nu, d3 x3,
    // faces x3 each direction, scale x3, current jr/jz, sums, words
    int64_t const n = s->n;
    int64_t const total = 6 * n + 10 * n + 3 * n + 3 * s->nfr + 3 * s->nfz + 3 * n + s->nfr + s->nfz + kSums + kWords;
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&s->block), sizeof(double) * static_cast<size_t>(total));
    if (e != cudaSuccess) {
        delete s;
        return e;
    }
    double* p = s->block;
    auto take = [&](int64_t count) {
        double* q = p;
        p += count;
        return q;
    };
    s->cur3 = take(3 * n);
    s->next3 = take(3 * n);
    s->rho = take(n);
    s->se = take(n);
    s->sp = take(n);
    s->sn = take(n);
    s->sigma = take(n);
    s->tau = take(n);
    s->chi = take(n);
    s->mu = take(n);
    s->nu = take(n);
    take(n);   // spare
    s->d3 = take(3 * n);
    s->fr = take(3 * s->nfr);
    s->fz = take(3 * s->nfz);
    s->scale3 = take(3 * n);
    s->jr = take(s->nfr);
    s->jz = take(s->nfz);
    s->sums = take(kSums);
    s->words = reinterpret_cast<u64*>(take(kWords));
    e = cudaMemset(s->block, 0, sizeof(double) * static_cast<size_t>(total));
    if (e != cudaSuccess) {
        fluid_free(s);
        return e;
    }
    s->bind_views();
    out = s;
    return cudaSuccess;
}

void fluid_set_config(FluidState& s, rrea_gpu_fluid_config const& c) { s.cfg = c; }
rrea_gpu_fluid_config const& fluid_config(FluidState const& s) { return s.cfg; }
std::string const& fluid_error(FluidState const& s) { return s.error; }

cudaError_t fluid_load_closure(FluidState& s, std::vector<double> const& columns, int nodes)
{
    if (s.closure) cudaFree(s.closure);
    s.closure = nullptr;
    s.closure_n = 0;
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&s.closure), sizeof(double) * columns.size());
    if (e != cudaSuccess) return e;
    e = cudaMemcpy(s.closure, columns.data(), sizeof(double) * columns.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) s.closure_n = nodes;
    return e;
}
bool fluid_has_closure(FluidState const& s) { return s.closure_n > 0; }

// field: 0 ne, 1 np, 2 nn, 3 rho, 4 sigma, 5 tau, 6 se, 7 sp, 8 sn, 9 chi, 10 mu, 11 nu, 12 d3 (3n),
// 13/14 the face-current buffers (radial/axial)
double* fluid_field(FluidState& s, int field)
{
    switch (field) {
    case 0: return s.ne;
    case 1: return s.np;
    case 2: return s.nn;
    case 3: return s.rho;
    case 4: return s.sigma;
    case 5: return s.tau;
    case 6: return s.se;
    case 7: return s.sp;
    case 8: return s.sn;
    case 9: return s.chi;
    case 10: return s.mu;
    case 11: return s.nu;
    case 12: return s.d3;
    case 13: return s.jr;
    case 14: return s.jz;
    default: return nullptr;
    }
}
void fluid_bind_chi(FluidState& s, bool bound) { s.chi_bound = bound; }
int64_t fluid_cells(FluidState const& s) { return s.n; }

cudaError_t fluid_take_sources(FluidState& s, const double* cells5, double dt, cudaStream_t stream)
{
    note_launch();
    rrea_dev::fluid::normalize_sources_kernel<<<s.blocks, 256, 0, stream>>>(dev_grid(s.grid), dt, cells5, s.se, s.sp,
                                                                            s.sn);
    return cudaGetLastError();
}

namespace {

void launch_react(FluidState& s, double dt, bool clear, cudaStream_t stream)
{
    note_launch();
    rrea_dev::fluid::react_kernel<<<s.blocks, 256, 0, stream>>>(react_params(s, dt, clear), s.ne, s.np, s.nn, s.se,
                                                                s.sp, s.sn, s.rho, s.nu, s.words, kWReaction,
                                                                kWResidual, kWResidualNan);
}

void launch_conductivity(FluidState& s, cudaStream_t stream)
{
    rrea_gpu_fluid_config const& c = s.cfg;
    note_launch();
    rrea_dev::fluid::conductivity_kernel<<<s.blocks, 256, 0, stream>>>(
        s.n, c.electron_drift_enable ? 1 : 0, c.ion_drift_enable ? 1 : 0, ion_law(c, true), ion_law(c, false),
        electron_law(c), c.transport_density_ratio, s.chi_bound ? s.chi : nullptr, mobility_table(c) ? s.mu : nullptr,
        s.ne, s.np, s.nn, s.sigma, s.tau);
}

void launch_closure(FluidState& s, const double* er, const double* ez, cudaStream_t stream)
{
    rrea_gpu_fluid_config const& c = s.cfg;
    note_launch();
    rrea_dev::fluid::closure_kernel<<<s.blocks, 256, 0, stream>>>(
        dev_closure(s), dev_grid(s.grid), c.transport_density_ratio, s.chi_bound ? s.chi : nullptr, er, ez, s.ne, s.se,
        mobility_table(c) ? s.mu : nullptr, attachment_table(c) ? s.nu : nullptr, mobility_table(c) ? s.d3 : nullptr,
        s.words, s.sums, kWHeld, kWAbove, kWInvalid, kWMinEn, kWMaxEn, kSCount, kSHeldCount, kSSource);
}

// Build (tensor check, face fluxes) + limiter + scaled faces (+ total
// current) + update; the carriers swap buffers.
void launch_transport(FluidState& s, double dt, const double* efr, const double* efr_add, const double* efz,
                      const double* efz_add, const double* jr_kin, const double* jz_kin, bool centres,
                      cudaStream_t stream)
{
    auto const p = transport_params(s, dt);
    bool const table = mobility_table(s.cfg);
    int const face_blocks = s.blocks;
    if (table) {
        note_launch();
        rrea_dev::fluid::tensor_check_kernel<<<s.blocks, 256, 0, stream>>>(s.n, s.d3, s.words, kWEig, kWTensorBad);
    }
    note_launch();
    rrea_dev::fluid::face_flux_kernel<<<face_blocks, 256, 0, stream>>>(
        p, s.cur3, s.chi_bound ? s.chi : nullptr, table ? s.mu : nullptr, table ? s.d3 : nullptr, efr, efr_add, efz,
        efz_add, s.fr, s.fz, s.words, kWSigma);
    note_launch();
    rrea_dev::fluid::limiter_kernel<<<s.blocks, 256, 0, stream>>>(p, s.cur3, s.fr, s.fz, s.scale3, s.words, s.sums,
                                                                  kWUnlimited, kWMinScale, kSBefore, kSRemoved,
                                                                  kSENumber, kSELimited);
    note_launch();
    rrea_dev::fluid::scale_faces_kernel<<<face_blocks, 256, 0, stream>>>(p, s.scale3, s.fr, s.fz, jr_kin, jz_kin,
                                                                         jr_kin ? s.jr : nullptr,
                                                                         jz_kin ? s.jz : nullptr);
    note_launch();
    rrea_dev::fluid::update_kernel<<<s.blocks, 256, 0, stream>>>(p, s.cur3, s.fr, s.fz, s.next3, s.rho,
                                                                 s.chi_bound ? s.chi : nullptr, s.words, s.sums, kWRate,
                                                                 kWSpeed, kWMinDensity, kWNonfinite,
                                                                 centres ? kSCenter : -1);
    std::swap(s.cur3, s.next3);
    s.bind_views();
}

bool fail(FluidState& s, std::string const& m)
{
    s.error = m;
    return false;
}

}  // namespace

bool fluid_validate(FluidState& s, bool require_cfl)
{
    rrea_gpu_fluid_config const& c = s.cfg;
    auto positive = [](double v) { return std::isfinite(v) && v > 0.0; };
    if (c.attachment_model != RREA_GPU_ATTACHMENT_CONSTANT && c.attachment_model != RREA_GPU_ATTACHMENT_EN_TABLE) {
        return fail(s, "fluid attachment model must be constant or en_table_attachment_v1");
    }
    for (double a : {c.electron_ion_recombination_coefficient_m3_per_s, c.ion_ion_recombination_coefficient_m3_per_s}) {
        if (!std::isfinite(a) || a < 0.0) return fail(s, "fluid recombination coefficients must be finite and non-negative");
    }
    if (c.ion_drift_enable) {
        if (c.ion_mobility_model != RREA_GPU_MOBILITY_ABSOLUTE && c.ion_mobility_model != RREA_GPU_MOBILITY_REDUCED_STP) {
            return fail(s, "enabled ion carrier has invalid mobility model");
        }
        bool const red = c.ion_mobility_model == RREA_GPU_MOBILITY_REDUCED_STP;
        if (!positive(red ? c.positive_ion_reduced_mobility_stp_m2_per_vs : c.positive_ion_mobility_m2_per_vs)
            || !positive(red ? c.negative_ion_reduced_mobility_stp_m2_per_vs : c.negative_ion_mobility_m2_per_vs)) {
            return fail(s, "enabled ion carrier requires a positive finite mobility");
        }
        if (red && (!positive(c.ion_mobility_density_ratio_floor) || !positive(c.transport_density_ratio))) {
            return fail(s, "density-scaled carrier mobility requires positive density ratios");
        }
    }
    if (c.electron_drift_enable) {
        if (c.electron_mobility_model != RREA_GPU_MOBILITY_ABSOLUTE
            && c.electron_mobility_model != RREA_GPU_MOBILITY_EN_TABLE_FLUX) {
            return fail(s, "enabled low-energy-electron carrier has invalid mobility model");
        }
        if (c.electron_mobility_model == RREA_GPU_MOBILITY_ABSOLUTE && !positive(c.electron_mobility_m2_per_vs)) {
            return fail(s, "enabled low-energy-electron carrier requires a positive finite mobility");
        }
    }
    if (require_cfl && (c.ion_drift_enable || c.electron_drift_enable)
        && (!std::isfinite(c.ion_drift_cfl) || c.ion_drift_cfl <= 0.0 || c.ion_drift_cfl > 1.0)) {
        return fail(s, "rrea.ion_drift_cfl must be finite and in (0, 1]");
    }
    return true;
}

// Chemistry over dt; returns false (with the error) on a residual above 512 eps.
cudaError_t fluid_react(FluidState& s, double dt, bool clear, double& residual, bool& ok, cudaStream_t stream)
{
    cudaError_t e = reset_reductions(s, stream);
    if (e != cudaSuccess) return e;
    launch_react(s, dt, clear, stream);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    Readback r;
    if ((e = read_reductions(s, r, stream)) != cudaSuccess) return e;
    residual = r.w[kWResidualNan] ? std::nan("") : from_bits(r.w[kWResidual]);
    ok = std::isfinite(residual) && residual <= 512.0 * 2.220446049250313e-16;
    if (!ok) fail(s, "low-energy attachment/recombination violated local charge conservation");
    return cudaSuccess;
}

cudaError_t fluid_max_reaction_frequency(FluidState& s, double& out, cudaStream_t stream)
{
    cudaError_t e = reset_reductions(s, stream);
    if (e != cudaSuccess) return e;
    note_launch();
    rrea_dev::fluid::max_rate_kernel<<<s.blocks, 256, 0, stream>>>(react_params(s, 0.0, false), s.ne, s.np, s.nn,
                                                                   s.nu, s.words + kWReaction);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    Readback r;
    if ((e = read_reductions(s, r, stream)) != cudaSuccess) return e;
    out = from_bits(r.w[kWReaction]);
    return cudaSuccess;
}

cudaError_t fluid_conductivity(FluidState& s, cudaStream_t stream)
{
    launch_conductivity(s, stream);
    return cudaGetLastError();
}

cudaError_t fluid_charge_density(FluidState& s, cudaStream_t stream)
{
    note_launch();
    rrea_dev::fluid::charge_kernel<<<s.blocks, 256, 0, stream>>>(s.n, s.ne, s.np, s.nn, s.rho);
    return cudaGetLastError();
}

cudaError_t fluid_closure(FluidState& s, const double* er_cell, const double* ez_cell, double diag8[8], bool& ok,
                          cudaStream_t stream)
{
    cudaError_t e = reset_reductions(s, stream);
    if (e != cudaSuccess) return e;
    launch_closure(s, er_cell, ez_cell, stream);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    Readback r;
    if ((e = read_reductions(s, r, stream)) != cudaSuccess) return e;
    double const v[8] = {r.w[kWMinEn] == ~0ULL ? std::numeric_limits<double>::max() : from_bits(r.w[kWMinEn]),
                         from_bits(r.w[kWMaxEn]),
                         static_cast<double>(r.w[kWHeld]),
                         static_cast<double>(r.w[kWAbove]),
                         static_cast<double>(r.w[kWInvalid]),
                         r.s[kSCount],
                         r.s[kSHeldCount],
                         r.s[kSSource]};
    std::memcpy(diag8, v, sizeof(v));
    ok = true;
    return cudaSuccess;
}

namespace {

// Post-transport checks of ApplyExplicitCarrierTransport and Build, from a
// readback; dt is the transport interval.
bool transport_checks(FluidState& s, Readback const& r, double dt)
{
    rrea_gpu_fluid_config const& c = s.cfg;
    if (r.w[kWTensorBad]) return fail(s, "en_table_flux_v1 diffusion tensor is not finite symmetric positive-semidefinite");
    double const inv2 = 1.0 / (s.grid.dr * s.grid.dr) + 1.0 / (s.grid.dz * s.grid.dz);
    double const diffusion = 2.0 * dt * from_bits(r.w[kWEig]) * inv2;
    if (!std::isfinite(diffusion) || diffusion >= 1.0) {
        return fail(s, "explicit electron diffusion violates its stability bound");
    }
    double const roundoff = 512.0 * 2.220446049250313e-16;
    if (dt * from_bits(r.w[kWRate]) > c.ion_drift_cfl + roundoff * std::max(1.0, c.ion_drift_cfl)) {
        return fail(s, "limited full-step carrier drift violates outgoing CFL");
    }
    if (r.w[kWNonfinite]) return fail(s, "explicit carrier transport produced a non-finite density");
    if (from_ordered(r.w[kWMinDensity]) < 0.0) {
        return fail(s, "explicit carrier transport produced negative density despite CFL gate");
    }
    return true;
}

}  // namespace

cudaError_t fluid_transport(FluidState& s, double dt, const double* efr, const double* efr_add, const double* efz,
                            const double* efz_add, double diag14[14], bool& ok, cudaStream_t stream)
{
    cudaError_t e = reset_reductions(s, stream);
    if (e != cudaSuccess) return e;
    launch_transport(s, dt, efr, efr_add, efz, efz_add, nullptr, nullptr, true, stream);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    Readback r;
    if ((e = read_reductions(s, r, stream)) != cudaSuccess) return e;
    ok = transport_checks(s, r, dt);
    double const inv2 = 1.0 / (s.grid.dr * s.grid.dr) + 1.0 / (s.grid.dz * s.grid.dz);
    double const rate = from_bits(r.w[kWRate]);
    double const* cs = r.s + kSCenter;
    double v[14] = {from_bits(r.w[kWSigma]),
                    mobility_table(s.cfg) ? 2.0 * dt * from_bits(r.w[kWEig]) * inv2 : 0.0,
                    dt * from_bits(r.w[kWUnlimited]),
                    from_bits(r.w[kWMinScale]),
                    r.s[kSBefore] > 0.0 ? std::clamp(r.s[kSRemoved] / r.s[kSBefore], 0.0, 1.0) : 0.0,
                    r.s[kSENumber] > 0.0 ? std::clamp(r.s[kSELimited] / r.s[kSENumber], 0.0, 1.0) : 0.0,
                    dt * rate,
                    from_bits(r.w[kWSpeed]),
                    rate > 0.0 ? s.cfg.ion_drift_cfl / rate : 1.0e300,
                    cs[0] > 0.0 ? cs[2] / cs[0] : 0.0,
                    cs[0] > 0.0 ? cs[3] / cs[0] : 0.0,
                    cs[1] > 0.0 ? cs[4] / cs[1] : 0.0,
                    cs[1] > 0.0 ? cs[5] / cs[1] : 0.0,
                    cs[0] > 0.0 ? cs[6] / cs[0] : 1.0};
    std::memcpy(diag14, v, sizeof(v));
    return cudaSuccess;
}

const double* fluid_flux(FluidState const& s, int dir) { return dir == 0 ? s.fr : s.fz; }

cudaError_t fluid_reductions(FluidState& s, const double* cells5, double dt, double out16[16], cudaStream_t stream)
{
    cudaError_t e = reset_reductions(s, stream);
    if (e != cudaSuccess) return e;
    u64 init[3] = {rrea_dev::fluid::host_ordered(-1.0e308), rrea_dev::fluid::host_ordered(-1.0e308),
                   rrea_dev::fluid::host_ordered(1.0e308)};
    if ((e = cudaMemcpyAsync(s.words, init, sizeof(init), cudaMemcpyHostToDevice, stream)) != cudaSuccess) return e;
    note_launch();
    rrea_dev::fluid::reductions_kernel<<<s.blocks, 256, 0, stream>>>(dev_grid(s.grid), dt, s.ne, s.np, s.nn, s.rho,
                                                                     s.sigma, s.tau, cells5, s.sums, s.words);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    Readback r;
    if ((e = read_reductions(s, r, stream)) != cudaSuccess) return e;
    for (int c = 0; c < 13; ++c) out16[c] = r.s[c];
    out16[13] = from_ordered(r.w[0]);
    out16[14] = from_ordered(r.w[1]);
    out16[15] = from_ordered(r.w[2]);
    return cudaSuccess;
}

cudaError_t fluid_coupled_step(FluidState& s, CoupledField const& f, double dt, double diag8[8], bool& ok,
                               cudaStream_t stream)
{
    ok = false;
    rrea_gpu_fluid_config const& c = s.cfg;
    bool const tables = mobility_table(c) || attachment_table(c);
    double const eps0 = 8.8541878128e-12;
    cudaError_t e = reset_reductions(s, stream);
    if (e != cudaSuccess) return e;
    // closure fields at the step start, conductivity, and the stiffness probe
    if (tables) launch_closure(s, f.cell_er, f.cell_ez, stream);
    launch_conductivity(s, stream);
    auto const probe = transport_params(s, dt * 1.0e-6);
    bool const table = mobility_table(c);
    if (table) {
        note_launch();
        rrea_dev::fluid::tensor_check_kernel<<<s.blocks, 256, 0, stream>>>(s.n, s.d3, s.words, kWEig, kWTensorBad);
    }
    note_launch();
    rrea_dev::fluid::face_flux_kernel<<<s.blocks, 256, 0, stream>>>(
        probe, s.cur3, s.chi_bound ? s.chi : nullptr, table ? s.mu : nullptr, table ? s.d3 : nullptr, f.er, f.amb_er,
        f.ez, f.amb_ez, nullptr, nullptr, s.words, kWSigma);
    note_launch();
    rrea_dev::fluid::max_rate_kernel<<<s.blocks, 256, 0, stream>>>(react_params(s, 0.0, false), s.ne, s.np, s.nn,
                                                                   s.nu, s.words + kWReaction);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    Readback r;
    if ((e = read_reductions(s, r, stream)) != cudaSuccess) return e;
    if (tables && (r.w[kWAbove] > 0 || r.w[kWInvalid] > 0)) return fail(s, "electron closure range violation"), cudaSuccess;
    if (r.w[kWTensorBad]) {
        return fail(s, "en_table_flux_v1 diffusion tensor is not finite symmetric positive-semidefinite"), cudaSuccess;
    }
    double const inv2 = 1.0 / (s.grid.dr * s.grid.dr) + 1.0 / (s.grid.dz * s.grid.dz);
    double const probe_diffusion = table ? 2.0 * (dt * 1.0e-6) * from_bits(r.w[kWEig]) * inv2 : 0.0;
    double const full_conduction = dt * from_bits(r.w[kWSigma]) / eps0;
    double const full_diffusion = probe_diffusion / 1.0e-6;
    double const full_reaction = dt * from_bits(r.w[kWReaction]);
    if (!std::isfinite(full_conduction) || !std::isfinite(full_diffusion) || !std::isfinite(full_reaction)) {
        return fail(s, "fluid/Maxwell coupling stiffness is non-finite"), cudaSuccess;
    }
    double const required = std::max({full_conduction / c.material_conduction_target,
                                      full_diffusion / c.material_diffusion_target,
                                      full_reaction / c.material_reaction_target});
    if (required > c.material_max_substeps) {
        return fail(s, "fluid/Maxwell coupling exceeds configured maximum substeps"), cudaSuccess;
    }
    int const substeps = std::max(c.material_min_substeps, static_cast<int>(std::ceil(required)));
    double const dts = dt / static_cast<double>(substeps);
    double const restagger = 0.5 * (dt - dts);
    // the substeps: every guard accumulates on the device and is checked
    // once, after the step
    if ((e = reset_reductions(s, stream)) != cudaSuccess) return e;
    if ((e = maxwell_advance_b(f.nr, f.nz, f.dr, f.dz, restagger, f.er, f.ez, f.bt, stream)) != cudaSuccess) return e;
    for (int k = 0; k < substeps; ++k) {
        launch_react(s, 0.5 * dts, false, stream);
        launch_transport(s, dts, f.er, f.amb_er, f.ez, f.amb_ez, f.jr_kin, f.jz_kin, false, stream);
        if ((e = maxwell_advance_b(f.nr, f.nz, f.dr, f.dz, dts, f.er, f.ez, f.bt, stream)) != cudaSuccess) return e;
        if ((e = maxwell_silver_mueller(f.nr, f.nz, f.er, f.ez, f.bt, stream)) != cudaSuccess) return e;
        if ((e = maxwell_advance_e(f.nr, f.nz, f.dr, f.dz, dts, f.bt, s.jr, s.jz, f.er, f.ez, stream)) != cudaSuccess) {
            return e;
        }
        if ((e = field_prep(f.nr, f.nz, f.er, f.ez, f.amb_er, f.amb_ez, f.cell_er, f.cell_ez, stream)) != cudaSuccess) {
            return e;
        }
        if (tables) launch_closure(s, f.cell_er, f.cell_ez, stream);
        launch_react(s, 0.5 * dts, false, stream);
    }
    if ((e = maxwell_advance_b(f.nr, f.nz, f.dr, f.dz, -restagger, f.er, f.ez, f.bt, stream)) != cudaSuccess) return e;
    if ((e = maxwell_silver_mueller(f.nr, f.nz, f.er, f.ez, f.bt, stream)) != cudaSuccess) return e;
    launch_conductivity(s, stream);
    if ((e = cudaMemsetAsync(s.se, 0, sizeof(double) * 3 * static_cast<size_t>(s.n), stream)) != cudaSuccess) return e;
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = read_reductions(s, r, stream)) != cudaSuccess) return e;
    double const residual = r.w[kWResidualNan] ? std::nan("") : from_bits(r.w[kWResidual]);
    double const v[8] = {static_cast<double>(substeps),
                         full_conduction,
                         full_diffusion,
                         full_reaction,
                         dts * from_bits(r.w[kWReaction]),
                         dts * from_bits(r.w[kWSigma]) / eps0,
                         table ? 2.0 * dts * from_bits(r.w[kWEig]) * inv2 : 0.0,
                         residual};
    std::memcpy(diag8, v, sizeof(v));
    if (tables && (r.w[kWAbove] > 0 || r.w[kWInvalid] > 0)) return fail(s, "electron closure range violation"), cudaSuccess;
    if (v[4] > c.material_reaction_guard) return fail(s, "reaction substep out of configured range"), cudaSuccess;
    if (!std::isfinite(residual) || residual > 512.0 * 2.220446049250313e-16) {
        return fail(s, "low-energy attachment/recombination violated local charge conservation"), cudaSuccess;
    }
    if (v[5] > c.material_conduction_guard) {
        return fail(s, "explicit conduction substep out of configured range"), cudaSuccess;
    }
    if (v[6] > c.material_diffusion_guard) return fail(s, "explicit diffusion substep out of configured range"), cudaSuccess;
    ok = transport_checks(s, r, dts);
    return cudaSuccess;
}

}  // namespace rrea_launch
