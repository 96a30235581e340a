// One photon through one outer step on one GPU thread: the reference's
// photon loop (O/RreaPhotonTransport.cpp:9-461) with the final states of
// O/RreaPhotonFinalStates.H:56-365 and the at-rest annihilation of
// TransportStep::spawn_positron_annihilation (O/RreaTransportStep.H:563-702).
//
// A photon flies the straight chord from its captured start (prev_*) to the
// pusher's end point (r, theta, z); an interaction inside the chord ends it
// (photoelectric, pair) or turns it (Compton) to continue the remainder of
// the chord along the new direction.  Side effects go to the same sinks as
// the electron phase: ordered secondary append buffer and the five FP64
// cell-source grids.
#pragma once

#include "rrea_dd.cuh"
#include "rrea_sinks.cuh"

namespace rrea_dev {

// O/RreaRng.H channel ids of the photon phase.
enum : uint64_t {
    kChPhotonOpticalDepth = 51, kChPhotonChannel = 52, kChComptonMu = 53, kChComptonAccept = 54,
    kChPhotoelectricShell = 55, kChPairPolar = 57, kChComptonAzimuth = 58, kChPairAzimuth = 59,
    kChPhotoelectronCos = 60, kChPhotoelectronAzimuth = 65, kChPairInvariant = 66,
    kChAnnihilationEnergy = 80, kChAnnihilationAzimuth = 81,
    kChPhotonContinuationOpticalDepth = 128, kChPhotonContinuationChannel = 129,
};

// I/RreaUniformStream.H:21-53: a splitmix64 stream seeded from the bit
// patterns of two uniforms, for rejection loops that need more draws than
// the counter RNG's fixed channels.
struct UniformStream {
    uint64_t state;
    __device__ __forceinline__ UniformStream(double u1, double u2)
    {
        uint64_t const h2 = splitmix64(static_cast<uint64_t>(__double_as_longlong(u2)));
        state = splitmix64(static_cast<uint64_t>(__double_as_longlong(u1))) ^ ((h2 << 32) | (h2 >> 32));
    }
    __device__ __forceinline__ double next()
    {
        state += 0x9e3779b97f4a7c15ULL;
        uint64_t z = state;
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
        z = z ^ (z >> 31);
        return __ull2double_rn(z >> 11) * 0x1.0p-53;
    }
};

// S/RreaInteractionTables.cpp:40-61
__device__ __forceinline__ double clamp_unit(double v)
{
    if (!finite_bits(v)) return 0.5;
    return max0(fmin(1.0, v));
}
__device__ __forceinline__ double wrap_unit(double v)
{
    if (!finite_bits(v)) return 0.0;
    v = v - floor(v);
    if (lt0(v)) v += 1.0;
    return v;
}

// Photon coefficients at one energy: Compton, photoelectric, pair (nuclear),
// pair (triplet) inverse lengths at STP (S/RreaInteractionTables.cpp:
// 2272-2296).  The four tables share one energy grid in the schema-6 bundle,
// so a single bracket serves all four.
struct PhotonRates {
    double compton, pe, nuclear, triplet;
    __device__ __forceinline__ double total() const { return compton + pe + nuclear + triplet; }
};
__device__ __forceinline__ bool photon_rates(StepConstants const& C, const double* __restrict__ arena, double e,
                                             PhotonRates& r, Err& err)
{
    RreaArenaIndex const& ix = C.tix;
    if (!(e >= ix.photon_min_eV && e <= ix.photon_max_eV)) {
        err.set(RREA_GPU_ERR_RANGE);
        return false;
    }
    if (ix.photon_grid_shared) {
        Bracket b;
        if (!bracket_hot(arena, ix.hot[RREA_T_PH_COMPTON], e, b, err)) return false;
        r.compton = eval_hot(arena, ix.hot[RREA_T_PH_COMPTON], b, err);
        r.pe = eval_hot(arena, ix.hot[RREA_T_PH_PHOTOELECTRIC], b, err);
        r.nuclear = eval_hot(arena, ix.hot[RREA_T_PH_PAIR_NUCLEAR], b, err);
        r.triplet = eval_hot(arena, ix.hot[RREA_T_PH_PAIR_TRIPLET], b, err);
    } else {
        r.compton = interpolate(arena, ix.hot[RREA_T_PH_COMPTON], e, err);
        r.pe = interpolate(arena, ix.hot[RREA_T_PH_PHOTOELECTRIC], e, err);
        r.nuclear = interpolate(arena, ix.hot[RREA_T_PH_PAIR_NUCLEAR], e, err);
        r.triplet = interpolate(arena, ix.hot[RREA_T_PH_PAIR_TRIPLET], e, err);
    }
    return err.code == 0;
}

// SamplePhotonChannel, S/RreaInteractionTables.cpp:2778-2804, on rates
// already evaluated at the same energy: 0 Compton, 1 photoelectric,
// 2 pair (nuclear), 3 pair (triplet).
__device__ __forceinline__ int sample_photon_channel(PhotonRates const& r, double u, Err& err)
{
    u = max0(fmin(1.0, u));
    double const total = r.total();
    if (!(gt0(total)) || !finite_bits(total)) {
        err.set(RREA_GPU_ERR_INVALID_STATE);
        return 0;
    }
    double const target = u * total;
    if (target < r.compton) return 0;
    if (target < r.compton + r.pe) return 1;
    if (target < r.compton + r.pe + r.nuclear) return 2;
    return 3;
}

// SampleComptonKleinNishinaFinalState, S/RreaInteractionTables.cpp:2806-2871
// (Butcher-Messel rejection; the first proposal uses the two counter draws,
// later ones the seeded uniform stream).
struct ComptonState {
    double recoil, scattered, cos_theta;
};
__device__ __forceinline__ ComptonState sample_klein_nishina(double e, double draw_mu, double draw_accept)
{
    draw_mu = max0(fmin(1.0, draw_mu));
    draw_accept = max0(fmin(1.0, draw_accept));
    UniformStream stream(draw_mu, draw_accept);
    double const alpha = e / kMeC2;
    double const eps0 = 1.0 / (1.0 + 2.0 * alpha);
    double const eps0sq = eps0 * eps0;
    double const a1 = -log(eps0);
    double const a2 = 0.5 * (1.0 - eps0sq);
    double epsilon = eps0, onecost = 0.0;
    for (int iter = 0; iter < 128; ++iter) {
        double const u1 = iter == 0 ? draw_mu : stream.next();
        double const u2 = iter == 0 ? draw_accept : stream.next();
        double epsilonsq;
        if (a1 > (a1 + a2) * u1) {
            epsilon = exp(-a1 * u2);
            epsilonsq = epsilon * epsilon;
        } else {
            epsilonsq = eps0sq + (1.0 - eps0sq) * u2;
            epsilon = sqrt(epsilonsq);
        }
        onecost = (1.0 - epsilon) / (epsilon * alpha);
        double const sint2 = onecost * (2.0 - onecost);
        double const greject = 1.0 - epsilon * sint2 / (1.0 + epsilonsq);
        if (greject >= stream.next()) break;
    }
    ComptonState st;
    st.scattered = max0(epsilon * e);
    st.recoil = max0(e - st.scattered);
    st.cos_theta = fmax(-1.0, fmin(1.0, 1.0 - onecost));
    return st;
}

// SamplePhotoelectricFinalState, S/RreaInteractionTables.cpp:2878-2941:
// subshell row by inverse CDF within the primary-energy group at or below
// the photon energy (a node-exact energy selects its own group, which puts
// a duplicated edge energy on the low side).
__device__ __forceinline__ void sample_photoelectric(StepConstants const& C, const double* __restrict__ arena, double e,
                                                     double u, double& electron, double& binding, Err& err)
{
    RreaPhotoelectricIndex const& pi = C.tix.pe;
    const double* prim = arena + pi.primary;
    const double* start = arena + pi.start;
    const double* cu = arena + pi.u;
    const double* bind = arena + pi.binding;
    electron = 0.0;
    binding = 0.0;
    if (!(e >= __ldg(prim) && e <= __ldg(prim + pi.ng - 1))) {
        err.set(RREA_GPU_ERR_RANGE);
        return;
    }
    u = max0(fmin(1.0, u));
    int const up = lower_bound(prim, pi.ng, e);
    int g;
    if (up == 0) g = 0;
    else if (up == pi.ng) g = pi.ng - 1;
    else if (__ldg(prim + up) == e) g = up;
    else g = up - 1;
    int const b = static_cast<int>(__ldg(start + g)), en = static_cast<int>(__ldg(start + g + 1));
    int const row = b + lower_bound(cu + b, en - b, u);
    int const r = row == en ? en - 1 : row;
    double const bnd = __ldg(bind + r);
    if (bnd > e) {
        err.set(RREA_GPU_ERR_INVALID_STATE);
        return;
    }
    binding = bnd;
    electron = max0(e - bnd);
}

// SamplePhotoelectronCosTheta, S/RreaInteractionTables.cpp:2949-3044:
// Sauter-Gavrila angle by bisection of the closed-form CDF in t = 1 - beta
// cos(theta).  The reference evaluates in long double; its primitive
//   P(x) = -c/(3x^3) - (2+bc)/(2x^2) - (2b-1)/x - b log x
// cancels heavily at low energy (the density is O(gamma-1) while the terms
// are O(1)), which costs plain FP64 up to 1e-11 in cos(theta).  Here the
// bisection runs on doubles and each comparison P(mid) < target is decided
// in FP64 when the FP64 value clears a rigorous error bound, and in
// double-double otherwise (Ziv's strategy), so every decision is the exact
// one; the answer is then within one bisection ulp of the exact root.
__device__ __forceinline__ dd sg_prim_dd(dd b, dd c, dd twopbc, dd twobm1, double x)
{
    dd const X = dd_from(x);
    dd const x2 = two_prod(x, x);
    dd const x3 = dd_mul_d(x2, x);
    dd const t1 = dd_neg(dd_div(c, dd_mul_d(x3, 3.0)));
    dd const t2 = dd_neg(dd_div(twopbc, dd_mul_d(x2, 2.0)));
    dd const t3 = dd_neg(dd_div(twobm1, X));
    dd const t4 = dd_neg(dd_mul(b, dd_log(X)));
    return dd_add(dd_add(dd_add(t1, t2), t3), t4);
}
static __device__ __noinline__ double sample_photoelectron_cos(double k, double draw)
{
    double const u = clamp_unit(draw);
    if (le0(u)) return -1.0;
    if (u >= 1.0) return 1.0;
    dd const gamma = dd_add(dd_from(1.0), dd_div(dd_from(k), dd_from(kMeC2)));
    dd const inv_g2 = dd_div(dd_from(1.0), dd_mul(gamma, gamma));
    dd const one_m = dd_sub(dd_from(1.0), inv_g2);
    dd const beta = gt0(one_m.hi) ? dd_sqrt(one_m) : dd_from(0.0);
    if (beta.hi < 1.0e-4) {
        // non-relativistic limit: CDF (2 + m(3 - m^2))/4 in m = cos(theta)
        double lo = -1.0, hi = 1.0;
        for (int it = 0; it < 96; ++it) {
            double const mid = 0.5 * (lo + hi);
            if (mid == lo || mid == hi) break;
            double const cdf = (2.0 + mid * (3.0 - mid * mid)) / 4.0;
            if (cdf < u) lo = mid; else hi = mid;
        }
        return 0.5 * (lo + hi);
    }
    dd const b = dd_mul_d(dd_mul(dd_mul(gamma, dd_sub(gamma, dd_from(1.0))), dd_sub(gamma, dd_from(2.0))), 0.5);
    dd const c = dd_neg(inv_g2);
    dd const twopbc = dd_add(dd_from(2.0), dd_mul(b, c));
    dd const twobm1 = dd_sub(dd_mul_d(b, 2.0), dd_from(1.0));
    dd const one_p_beta = dd_add(dd_from(1.0), beta);
    dd const t_lo = dd_div(inv_g2, one_p_beta);
    dd const t_hi = one_p_beta;
    // the end points as doubles (the bisection variable)
    dd const f_lo = sg_prim_dd(b, c, twopbc, twobm1, t_lo.hi);
    dd const f_hi = sg_prim_dd(b, c, twopbc, twobm1, t_hi.hi);
    dd const total = dd_sub(f_hi, f_lo);
    if (!(gt0(total.hi)) || !finite_bits(total.hi)) return __longlong_as_double(0x7ff8000000000000LL);
    dd const target = dd_add(dd_mul(two_sum(1.0, -u), f_hi), dd_mul_d(f_lo, u));
    double const bd = b.hi, cd = c.hi, pbd = twopbc.hi, bm1d = twobm1.hi, tgt = target.hi;
    double lo = t_lo.hi, hi = t_hi.hi;
    for (int it = 0; it < 128; ++it) {
        double const mid = 0.5 * (lo + hi);
        if (mid == lo || mid == hi) break;
        // FP64 value with a bound on its error: every term carries at most a
        // few roundings (and the libm log one ulp), so 32 eps of the summed
        // magnitudes covers them with margin.
        double const m2 = mid * mid;
        double const t1 = -cd / (3.0 * m2 * mid);
        double const t2 = -pbd / (2.0 * m2);
        double const t3 = -bm1d / mid;
        double const t4 = -bd * log(mid);
        double const p = ((t1 + t2) + t3) + t4;
        double const bound = 32.0 * kEps * (fabs(t1) + fabs(t2) + fabs(t3) + fabs(t4) + fabs(tgt));
        bool below;
        if (p - tgt < -bound) below = true;
        else if (p - tgt > bound) below = false;
        else below = dd_lt(sg_prim_dd(b, c, twopbc, twobm1, mid), target);
        if (below) lo = mid; else hi = mid;
    }
    double const tt = 0.5 * (lo + hi);
    dd const cosv = dd_div(dd_sub(dd_from(1.0), dd_from(tt)), beta);
    return fmax(-1.0, fmin(1.0, cosv.hi));
}

// SamplePairFinalState, S/RreaInteractionTables.cpp:3053-3127, with
// BuildRreaPairEmpiricalFinalState (:1384-1525): replay one training record
// of the correlated pair bank, block chosen by log-energy interpolation, the
// record rotated about the photon axis and its energies closed against the
// available kinetic energy.
struct PairState {
    bool valid, recoil;
    double e_electron, e_positron, e_recoil, local;
    double edir[3], pdir[3], rdir[3];
};
__device__ __forceinline__ void normalize_local(double& x, double& y, double& z)
{
    double const n = sqrt(x * x + y * y + z * z);
    if (le0(n) || !finite_bits(n)) {
        x = 0.0; y = 0.0; z = 1.0;
        return;
    }
    x /= n; y /= n; z /= n;
}
__device__ __forceinline__ double* pair_largest(PairState& st)
{
    double* l = &st.e_electron;
    if (st.e_positron > *l) l = &st.e_positron;
    if (st.e_recoil > *l) l = &st.e_recoil;
    return l;
}
// Photon energy-flow ledger checks of the commit (O/RreaSecondaryCommit.cpp:55-160):
// every Compton, photoelectric and pair record must carry a finite,
// non-negative payload whose parts add up to the incident photon energy
// within 64 eps of it, and whose split into charged (kinetic + created rest
// mass) and local (recoil, binding, sub-cutoff) flows
// (RreaComptonPhotonEnergyFlow, RreaPhotoelectricPhotonEnergyFlow,
// RreaPairPhotonEnergyFlow, O/RreaParticleInteraction.H:1015-1090) matches
// the split recomputed from the recorded energies.  A mismatch fails the
// step closed, as the reference's transaction validation does.
__device__ __forceinline__ bool photon_flow_matches(double actual, double expected, double scale)
{
    return finite_bits(actual) && ge0(actual) && fabs(actual - expected) <= 64.0 * kEps * fmax(scale, 1.0);
}

__device__ __forceinline__ bool photon_payload_ok(double w, double inc)
{
    return finite_bits(w) && finite_bits(inc) && gt0(w) && gt0(inc);
}

// Compton: recoil electron + scattered photon = incident.
__device__ __forceinline__ bool compton_flow_valid(double w, double inc, double recoil, double scattered)
{
    return photon_payload_ok(w, inc) && finite_bits(recoil) && ge0(recoil) && finite_bits(scattered)
        && ge0(scattered) && photon_flow_matches(recoil + scattered, inc, inc);
}

// Photoelectric: photoelectron + binding = incident.
__device__ __forceinline__ bool photoelectric_flow_valid(double w, double inc, double electron, double binding)
{
    return photon_payload_ok(w, inc) && finite_bits(electron) && ge0(electron) && finite_bits(binding)
        && ge0(binding) && photon_flow_matches(electron + binding, inc, inc);
}

// Pair: the local flow the final state booked equals the incident energy
// left after the two rest masses and the kinetic energies (the triplet
// recoil's included), floored at zero.
__device__ __forceinline__ bool pair_flow_valid(double w, double inc, double electron, double positron,
                                                double recoil, bool has_recoil, double local)
{
    if (!(photon_payload_ok(w, inc) && finite_bits(electron) && finite_bits(positron) && finite_bits(recoil)
          && ge0(electron) && ge0(positron) && ge0(recoil))) {
        return false;
    }
    double const expected = fmax(inc - 2.0 * kMeC2 - electron - positron - (has_recoil ? recoil : 0.0), 0.0);
    return photon_flow_matches(fmax(local, 0.0), expected, inc);
}

// Closure of the PairNuclear / PairTriplet group (O/RreaPhotonFinalStates.H:278-364):
// a sub-cutoff positron annihilates at rest into two m_e c^2 photons beside a
// positive ion, inside the same group.
__device__ __forceinline__ bool pair_closure_valid(PairState const& ps, double w, double e_photon, double cutoff,
                                                   double photon_cut, double w_air)
{
    GroupClosure gc;
    gc.begin(0.0, 0.0, w, e_photon, 0.0, false);
    if (ps.e_electron >= cutoff) {
        gc.secondary(-1.0, kMeC2, w, ps.e_electron);
    } else {
        gc.low_energy_electron(w);
        gc.local(w, ps.e_electron, w_air, cutoff);
    }
    if (ps.e_positron >= cutoff) {
        gc.secondary(1.0, kMeC2, w, ps.e_positron);
    } else {
        double local = 0.0;
        for (int q = 0; q < 2; ++q) {
            if (kMeC2 >= photon_cut) gc.secondary(0.0, 0.0, w, kMeC2);
            else local += kMeC2;
        }
        if (gt0(ps.e_positron)) gc.local(w, ps.e_positron, w_air, cutoff);
        gc.local(w, local, w_air, cutoff);
        gc.positive_ion(w);
    }
    if (ps.recoil) {
        if (ps.e_recoil >= cutoff) gc.secondary(-1.0, kMeC2, w, ps.e_recoil);
        gc.ionization(w, ps.e_recoil, cutoff);
        if (ps.e_recoil < cutoff) gc.local(w, ps.e_recoil, w_air, cutoff);
    }
    if (gt0(ps.local)) gc.local(w, ps.local, w_air, cutoff);
    return gc.valid(cutoff);
}

__device__ __forceinline__ void sample_pair(StepConstants const& C, const double* __restrict__ arena, double e,
                                            int channel, double d_inv, double d_polar, double d_azim, PairState& st,
                                            Err& err)
{
    st.valid = false;
    st.recoil = false;
    st.e_electron = st.e_positron = st.e_recoil = st.local = 0.0;
    for (int c = 0; c < 3; ++c) { st.edir[c] = st.pdir[c] = st.rdir[c] = c == 2 ? 1.0 : 0.0; }
    bool const triplet = channel == 3;
    double const threshold = triplet ? 4.0 * kMeC2 : 2.0 * kMeC2;
    if (!(finite_bits(e) && e > threshold)) return;
    RreaPairBankIndex const& pb = C.tix.pair[triplet ? 1 : 0];
    const double* prim = arena + pb.primary;
    const double* start = arena + pb.start;
    int sel = 0;
    if (e >= __ldg(prim + pb.nb - 1)) {
        sel = pb.nb - 1;
    } else if (e > __ldg(prim)) {
        int const hi = lower_bound(prim, pb.nb, e);
        if (__ldg(prim + hi) == e) {
            sel = hi;
        } else {
            int const lo = hi - 1;
            double const t = (log(e) - log(__ldg(prim + lo))) / (log(__ldg(prim + hi)) - log(__ldg(prim + lo)));
            sel = clamp_unit(d_polar) < t ? hi : lo;
        }
    }
    int64_t const b0 = static_cast<int64_t>(__ldg(start + sel));
    int64_t const size = static_cast<int64_t>(__ldg(start + sel + 1)) - b0;
    int64_t idx = static_cast<int64_t>(clamp_unit(d_inv) * static_cast<double>(size));
    if (idx > size - 1) idx = size - 1;
    const double* rec = arena + pb.records + (b0 + idx) * RREA_PAIR_RECORD_DOUBLES;
    int const count = static_cast<int>(__ldg(rec));
    int es = -1, ps = -1, rs = -1;
    for (int slot = 0; slot < count && slot < 3; ++slot) {
        int const pdg = static_cast<int>(__ldg(rec + 1 + slot));
        if (pdg == -11) ps = slot;
        else if (pdg == 11) {
            if (es < 0) es = slot; else rs = slot;
        }
    }
    if (es < 0 || ps < 0 || (triplet && rs < 0)) {
        err.set(RREA_GPU_ERR_INVALID_STATE);
        return;
    }
    double const avail = e - 2.0 * kMeC2;
    double const rot = kTwoPi * clamp_unit(d_azim);
    double sr, cr;
    sincos(rot, &sr, &cr);
    auto rotated = [&](int slot, double* d) {
        double const px = __ldg(rec + 7 + 3 * slot), py = __ldg(rec + 8 + 3 * slot), pz = __ldg(rec + 9 + 3 * slot);
        d[0] = cr * px - sr * py;
        d[1] = sr * px + cr * py;
        d[2] = pz;
        normalize_local(d[0], d[1], d[2]);
    };
    st.valid = true;
    st.e_electron = avail * __ldg(rec + 4 + es);
    st.e_positron = avail * __ldg(rec + 4 + ps);
    rotated(es, st.edir);
    rotated(ps, st.pdir);
    if (triplet) {
        st.recoil = true;
        st.e_recoil = avail * __ldg(rec + 4 + rs);
        rotated(rs, st.rdir);
    }
    double const tol = 64.0 * kEps * fmax(1.0, avail);
    double expl = st.e_electron + st.e_positron + st.e_recoil;
    if (!finite_bits(expl) || lt0(st.e_electron) || lt0(st.e_positron) || lt0(st.e_recoil)) {
        err.set(RREA_GPU_ERR_INVALID_STATE);
        return;
    }
    if (expl > avail) {
        if (expl - avail > tol) {
            err.set(RREA_GPU_ERR_INVALID_STATE);
            return;
        }
        double const scale = avail / expl;
        st.e_electron *= scale; st.e_positron *= scale; st.e_recoil *= scale;
        expl = st.e_electron + st.e_positron + st.e_recoil;
    }
    st.local = avail - expl;
    if (lt0(st.local)) {
        double const corr = -st.local;
        double* l = pair_largest(st);
        if (corr > tol || *l < corr) {
            err.set(RREA_GPU_ERR_INVALID_STATE);
            return;
        }
        *l -= corr;
        st.local = 0.0;
    }
    double accounted = st.e_electron + st.e_positron + st.e_recoil + st.local;
    double const resid = avail - accounted;
    if (fabs(resid) > tol) {
        err.set(RREA_GPU_ERR_INVALID_STATE);
        return;
    }
    if (ge0(resid)) {
        st.local += resid;
    } else if (st.local >= -resid) {
        st.local += resid;
    } else {
        double* l = pair_largest(st);
        if (*l < -resid) {
            err.set(RREA_GPU_ERR_INVALID_STATE);
            return;
        }
        *l -= -resid;
    }
    accounted = st.e_electron + st.e_positron + st.e_recoil + st.local;
    if (lt0(st.e_electron) || lt0(st.e_positron) || lt0(st.e_recoil) || lt0(st.local)
        || fabs(avail - accounted) > tol) {
        err.set(RREA_GPU_ERR_INVALID_STATE);
    }
}

// O/RreaChargedInterleave.H:498-517: a direction given in the local frame
// (transverse basis, axis) of `a` rotated into the lab frame.
__device__ __forceinline__ void rotate_to_axis(double ax, double ay, double az, double lx, double ly, double lz,
                                               double& ox, double& oy, double& oz)
{
    normalize(ax, ay, az);
    normalize(lx, ly, lz);
    double dx = ax, dy = ay, dz = az;
    normalize(dx, dy, dz);
    double rx = 0.0, ry = 0.0, rz = 1.0;
    if (fabs(dz) > 0.9) { rx = 1.0; rz = 0.0; }
    double b1x = ry * dz - rz * dy, b1y = rz * dx - rx * dz, b1z = rx * dy - ry * dx;
    normalize(b1x, b1y, b1z);
    double b2x = dy * b1z - dz * b1y, b2y = dz * b1x - dx * b1z, b2z = dx * b1y - dy * b1x;
    normalize(b2x, b2y, b2z);
    ox = lx * b1x + ly * b2x + lz * ax;
    oy = lx * b1y + ly * b2y + lz * ay;
    oz = lx * b1z + ly * b2z + lz * az;
    normalize(ox, oy, oz);
}

// Photon tile: (r, theta, z) is the pusher's end point, prev_* the start;
// (ux, uy, uz) is the photon momentum in eV.  Returns the disposition
// (0 survive, 1 escape, 2 absorbed, -1 error) and the hazard draws made.
template <int NP>
__device__ __forceinline__ int transport_photon(StepConstants const& C, ElectronArgs const& A, int64_t ip,
                                                uint64_t& events_out, uint32_t& lineage, Err& err)
{
    const double* __restrict__ arena = A.arena;
    rrea_gpu_config const& cfg = C.cfg;
    Geom const g{cfg.r_lo, cfg.r_hi, cfg.z_lo, cfg.z_hi, cfg.periodic_z != 0};
    double const cutoff = cfg.low_energy_cutoff_eV;
    double const photon_cut = C.photon_cutoff_eV;
    double const rho = C.density_ratio;
    double const w_air = C.tix.w_air_eV_per_pair;
    double const dt_s = C.dt_s;

    uint64_t const key = static_cast<uint64_t>(llabs(A.id[ip])) ^ (static_cast<uint64_t>(A.cpu ? A.cpu[ip] : 0) << 40);
    double const weight = A.w[ip];
    double ux = A.ux[ip], uy = A.uy[ip], uz = A.uz[ip];
    double energy = sqrt(ux * ux + uy * uy + uz * uz);
    double dx = ux, dy = uy, dz = uz;
    normalize(dx, dy, dz);
    double const pr0 = A.prev_r[ip], pz0 = A.prev_z[ip];
    if (pr0 > cfg.r_hi + 1.0e-9 * cfg.r_hi || pz0 < cfg.z_lo - 1.0e-9 || pz0 > cfg.z_hi + 1.0e-9 * cfg.z_hi) {
        err.set(RREA_GPU_ERR_GEOMETRY);
        return -1;
    }
    RngStream rng;
    rng.init(cfg.rng_seed, key, C.step_key);
    double const pth0 = A.prev_theta[ip];
    double r1, th1, z1;
    if (A.straight_push) {
        // WarpX's photon push (x += c dt u/|u|) on the Cartesian image of the
        // RZ start point; the tile arrays alias prev_* in this mode.
        double const f = gt0(energy) ? kC * dt_s / energy : 0.0;
        double s0, c0;
        sincos(pth0, &s0, &c0);
        double const x1 = pr0 * c0 + ux * f, y1 = pr0 * s0 + uy * f;
        z1 = pz0 + uz * f;
        r1 = rz_radius(x1, y1);
        th1 = atan2(y1, x1);
    } else {
        r1 = A.r[ip];
        th1 = A.theta[ip];
        z1 = A.z[ip];
    }
    Path<NP> path;
    clip_rz(pr0, pth0, pz0, r1, th1, z1, g, path, err);
    if (err.code) return -1;

    int process = 0;
    auto deposit_local_at = [&](double r, double z, double w, double e) {
        // O/RreaTransportStep.H:530-561
        if (le0(w) || le0(e)) return;
        double const pw = w * e / fmax(w_air, 1.0);
        if (le0(pw)) return;
        deposit_source(C, A.cells, 0, r, z, pw, 0.0, w_air);
    };
    auto add_secondary = [&](int species, double x, double y, double z, double sx, double sy, double sz, double e,
                             double birth) {
        append_secondary(A, ip, key, weight, lineage, species, process, x, y, z, sx, sy, sz, e, birth, err, 2);
    };

    uint64_t ordinal = 0;
    double elapsed_start = 0.0;
    for (;;) {
        if (ordinal >= kEventCap) {
            err.set(RREA_GPU_ERR_RNG_OVERFLOW);
            return -1;
        }
        bool esc, esc_inv;
        clipped_escape_policy(path, g, rz_radius(path.ex, path.ey), path.ez, esc, esc_inv);
        double const ds = path.in_length;
        Intervals<NP> iv;
        build_intervals(path, g, A.prof, rho, iv, err);
        double const chord_dpath = density_path(iv, path, path.in_begin, path.in_end);
        if (le0(weight) || energy < photon_cut) {
            double x, y, z;
            point_at_full(path, g, path.in_begin, x, y, z);
            process = 12;
            deposit_local_at(rz_radius(x, y), z, max0(weight), energy);
            A.id[ip] = -A.id[ip];
            return 2;
        }
        auto commit_no_event = [&]() {
            double x, y, z;
            point_at_full(path, g, path.in_end, x, y, z);
            A.r[ip] = rz_radius(x, y);
            A.theta[ip] = atan2(y, x);
            A.z[ip] = wrap_z(g, z);
            if (!esc) return 0;
            if (esc_inv) A.id[ip] = -A.id[ip];
            return 1;
        };
        if (le0(ds)) return commit_no_event();
        PhotonRates rates;
        if (!photon_rates(C, arena, energy, rates, err)) return -1;
        double const mfp = mfp_from_inverse(rates.total(), err);
        double const tau = chord_dpath / mfp;
        uint64_t idx;
        if (!live_hazard_index(2, 0, ordinal, idx)) {
            err.set(RREA_GPU_ERR_RNG_OVERFLOW);
            return -1;
        }
        ++events_out;
        double const u_int =
            rng.uniform(idx, ordinal == 0 ? kChPhotonOpticalDepth : kChPhotonContinuationOpticalDepth);
        Selection const sel = select_hazard(arena, tau, 0.0, 0.0, 1, u_int, 0.0);
        if (!sel.valid) {
            err.set(RREA_GPU_ERR_INVALID_STATE);
            return -1;
        }
        if (!sel.event) return commit_no_event();
        double const f = fraction_at_density_path(iv, path, path.in_begin, path.in_end, sel.sampled * mfp, err);
        if (!(finite_bits(f) && f >= path.in_begin && f <= path.in_end && path.in_end > path.in_begin)) {
            err.set(RREA_GPU_ERR_INVALID_STATE);
            return -1;
        }
        double const dist = path.full * (f - path.in_begin);
        double px, py, pz;
        point_at_full(path, g, f, px, py, pz);
        double const remaining = max0(path.full - dist);
        double const birth = fmin(1.0, elapsed_start + dist / fmax(kC * dt_s, kDblMin));
        double const pr = rz_radius(px, py);
        int const channel = sample_photon_channel(
            rates, rng.uniform(idx, ordinal == 0 ? kChPhotonChannel : kChPhotonContinuationChannel), err);
        if (err.code) return -1;
        if (channel == 0) {
            // RreaApplyComptonFinalState, O/RreaPhotonFinalStates.H:56-147
            process = 5;
            double const inc = energy;
            ComptonState const cs =
                sample_klein_nishina(inc, rng.uniform(idx, kChComptonMu), rng.uniform(idx, kChComptonAccept));
            double sx, sy, sz;
            cone_direction(dx, dy, dz, cs.cos_theta, rng.uniform(idx, kChComptonAzimuth), sx, sy, sz);
            double rx = inc * dx - cs.scattered * sx, ry = inc * dy - cs.scattered * sy,
                   rz = inc * dz - cs.scattered * sz;
            normalize(rx, ry, rz);
            if (cs.recoil >= cutoff) {
                add_secondary(0, px, py, pz, rx, ry, rz, cs.recoil, birth);
                deposit_source(C, A.cells, 0, pr, pz, weight, cs.recoil, cs.recoil);
            } else {
                deposit_source(C, A.cells, 0, pr, pz, weight, cs.recoil, 0.0);
                deposit_local_at(pr, pz, weight, cs.recoil);
            }
            if (!compton_flow_valid(weight, inc, cs.recoil, cs.scattered)) {
                err.set(RREA_GPU_ERR_INVALID_STATE);
                return -1;
            }
            energy = cs.scattered;
            {
                // closure of the Compton group (O/RreaPhotonFinalStates.H:92-142)
                bool const survives = energy >= photon_cut;
                GroupClosure gc;
                gc.begin(0.0, 0.0, weight, inc, survives ? energy : 0.0, survives);
                if (cs.recoil >= cutoff) gc.secondary(-1.0, kMeC2, weight, cs.recoil);
                gc.ionization(weight, cs.recoil, cutoff);
                if (cs.recoil < cutoff) gc.local(weight, cs.recoil, w_air, cutoff);
                if (!survives) gc.local(weight, energy, w_air, cutoff);
                if (!gc.valid(cutoff)) {
                    err.set(RREA_GPU_ERR_INVALID_STATE);
                    return -1;
                }
            }
            if (energy < photon_cut) {
                deposit_local_at(pr, pz, weight, energy);
                A.id[ip] = -A.id[ip];
                return 2;
            }
            dx = sx; dy = sy; dz = sz;
            A.ux[ip] = energy * dx;
            A.uy[ip] = energy * dy;
            A.uz[ip] = energy * dz;
            double const xt = px + dx * remaining, yt = py + dy * remaining, zt = pz + dz * remaining;
            Path<NP> next;
            clip_xyz(px, py, pz, xt, yt, zt, g, next, err);
            if (err.code) return -1;
            double nx, ny, nz;
            point_at_full(next, g, next.in_end, nx, ny, nz);
            A.r[ip] = rz_radius(nx, ny);
            A.theta[ip] = atan2(ny, nx);
            A.z[ip] = wrap_z(g, nz);
            if (!(gt0(remaining))) return 0;
            path = next;
            elapsed_start = birth;
            ++ordinal;
            continue;
        }
        if (channel == 1) {
            // RreaApplyPhotoelectricFinalState, O/RreaPhotonFinalStates.H:160-224
            process = 6;
            double pe_e, bind;
            sample_photoelectric(C, arena, energy, rng.uniform(idx, kChPhotoelectricShell), pe_e, bind, err);
            if (err.code) return -1;
            double const ee = fmin(pe_e, energy);
            if (ee >= cutoff) {
                if (!charged_in_range(C.tix, ee)) {
                    err.set(RREA_GPU_ERR_RANGE);
                    return -1;
                }
                double const cth = sample_photoelectron_cos(ee, rng.uniform(idx, kChPhotoelectronCos));
                if (!finite_bits(cth)) {
                    err.set(RREA_GPU_ERR_INVALID_STATE);
                    return -1;
                }
                double ex, ey, ez;
                cone_direction(dx, dy, dz, cth, rng.uniform(idx, kChPhotoelectronAzimuth), ex, ey, ez);
                add_secondary(0, px, py, pz, ex, ey, ez, ee, birth);
                deposit_source(C, A.cells, 0, pr, pz, weight, ee, ee);
            } else {
                deposit_source(C, A.cells, 0, pr, pz, weight, ee, 0.0);
                deposit_local_at(pr, pz, weight, ee);
            }
            if (gt0(bind)) deposit_local_at(pr, pz, weight, bind);
            if (!photoelectric_flow_valid(weight, energy, ee, fmax(bind, 0.0))) {
                err.set(RREA_GPU_ERR_INVALID_STATE);
                return -1;
            }
            {
                // closure of the Photoelectric group (O/RreaPhotonFinalStates.H:181-223)
                GroupClosure gc;
                gc.begin(0.0, 0.0, weight, energy, 0.0, false);
                if (ee >= cutoff) gc.secondary(-1.0, kMeC2, weight, ee);
                gc.ionization(weight, ee, cutoff);
                if (ee < cutoff) gc.local(weight, ee, w_air, cutoff);
                if (gt0(bind)) gc.local(weight, bind, w_air, cutoff);
                if (!gc.valid(cutoff)) {
                    err.set(RREA_GPU_ERR_INVALID_STATE);
                    return -1;
                }
            }
            A.id[ip] = -A.id[ip];
            return 2;
        }
        // RreaApplyPairFinalState, O/RreaPhotonFinalStates.H:239-365
        bool const triplet = channel == 3;
        process = triplet ? 8 : 7;
        PairState ps;
        sample_pair(C, arena, energy, channel, rng.uniform(idx, kChPairInvariant), rng.uniform(idx, kChPairPolar),
                    rng.uniform(idx, kChPairAzimuth), ps, err);
        if (err.code) return -1;
        if (!ps.valid) {
            err.set(RREA_GPU_ERR_INVALID_STATE);
            return -1;
        }
        double edx, edy, edz, pdx, pdy, pdz;
        rotate_to_axis(dx, dy, dz, ps.edir[0], ps.edir[1], ps.edir[2], edx, edy, edz);
        rotate_to_axis(dx, dy, dz, ps.pdir[0], ps.pdir[1], ps.pdir[2], pdx, pdy, pdz);
        if (ps.e_electron >= cutoff) {
            add_secondary(0, px, py, pz, edx, edy, edz, ps.e_electron, birth);
        } else {
            deposit_source(C, A.cells, 1, pr, pz, weight, 0.0, 0.0);
            deposit_local_at(pr, pz, weight, ps.e_electron);
        }
        if (ps.e_positron >= cutoff) {
            add_secondary(1, px, py, pz, pdx, pdy, pdz, ps.e_positron, birth);
        } else {
            // spawn_positron_annihilation at rest: two back-to-back photons
            // of m_e c^2 about a direction drawn around the positron's
            double ax = pdx, ay = pdy, az = pdz;
            normalize(ax, ay, az);
            double const d_e = rng.uniform(idx, kChAnnihilationEnergy);
            double const d_a = rng.uniform(idx, kChAnnihilationAzimuth);
            double const cos1 = 2.0 * clamp_unit(d_e) - 1.0;
            double const azim = wrap_unit(d_a);
            double g1x, g1y, g1z;
            cone_direction(ax, ay, az, cos1, azim, g1x, g1y, g1z);
            double const e1 = kMeC2, e2 = kMeC2;
            double local = 0.0;
            if (e1 >= photon_cut) add_secondary(2, px, py, pz, g1x, g1y, g1z, e1, birth);
            else local += e1;
            if (e2 >= photon_cut) add_secondary(2, px, py, pz, -g1x, -g1y, -g1z, e2, birth);
            else local += e2;
            if (gt0(ps.e_positron)) deposit_local_at(pr, pz, weight, ps.e_positron);
            if (gt0(local)) deposit_local_at(pr, pz, weight, local);
            deposit_source(C, A.cells, 2, pr, pz, weight, 0.0, 0.0);
        }
        if (ps.recoil) {
            double rdx, rdy, rdz;
            rotate_to_axis(dx, dy, dz, ps.rdir[0], ps.rdir[1], ps.rdir[2], rdx, rdy, rdz);
            if (ps.e_recoil >= cutoff) add_secondary(0, px, py, pz, rdx, rdy, rdz, ps.e_recoil, birth);
            deposit_source(C, A.cells, 0, pr, pz, weight, ps.e_recoil, 0.0);
            if (ps.e_recoil < cutoff) deposit_local_at(pr, pz, weight, ps.e_recoil);
        }
        if (gt0(ps.local)) deposit_local_at(pr, pz, weight, ps.local);
        if (!pair_flow_valid(weight, energy, ps.e_electron, ps.e_positron, ps.e_recoil, ps.recoil, ps.local)
            || !pair_closure_valid(ps, weight, energy, cutoff, photon_cut, w_air)) {
            err.set(RREA_GPU_ERR_INVALID_STATE);
            return -1;
        }
        A.id[ip] = -A.id[ip];
        return 2;
    }
}

}  // namespace rrea_dev
