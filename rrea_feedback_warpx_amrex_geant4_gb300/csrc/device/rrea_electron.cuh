// One electron through one outer step on one GPU thread: the body of the
// reference's electron loop (O/RreaElectronTransport.cpp:59-889, with the
// shared prologue/escape/writeback of O/RreaTransportStep.H:720-905 and the
// substep/event interleave of O/RreaChargedInterleave.H:546-732).
//
// The reference threads a transaction log through lambdas; here every side
// effect goes straight to its device sink:
//   * secondaries  -> append buffer with (parent index, lineage) keys, ordered
//                     after the kernel into the reference's chunk order;
//   * cell sources -> FP64 atomics into the five cell-source grids with the
//                     order-1 CIC stencil of S/RreaEventAccumulator.cpp:386-502;
//   * tallies      -> not kept (diagnostic ledger only).
#pragma once

#include "rrea_sinks.cuh"

namespace rrea_dev {

// Per-step constants of the charged phases.  Internal to each translation
// unit that includes this header (each sets its own copy before launching).
static __constant__ StepConstants c_step;



// The electron coefficient tables (collision, soft radiative, hard-Moller
// and tracked-brems rates) share one bit-identical 2856-row energy grid in
// the schema-6 bundle (the loader refuses to run the device path otherwise).
// One bracket per distinct query energy therefore serves every table, and
// each table value is interpolated on first use only.  The hazard refreeze
// and the drag segment that follows it query the same frozen energy, so the
// drag reuses the refreeze's bracket instead of searching again.
// The positron tables likewise share one grid among themselves; the cache is
// used with the base table RREA_T_E_COLLISION or RREA_T_P_COLLISION.
struct RateCache {
    long long key = -1;  // bit pattern of the bracketed energy; -1 = none
    Bracket b;
    double v[6];
    unsigned have = 0;  // bit i: v[i] valid (0 collision, 1 soft, 2 hard, 3 brems, 5 annihilation)
};

__device__ __forceinline__ bool rate_bracket(StepConstants const& C, const double* __restrict__ arena, RateCache& rc,
                                             double e, Err& err, int base = RREA_T_E_COLLISION)
{
    long long const key = __double_as_longlong(e);
    if (rc.key == key) return true;
    rc.key = -1;
    rc.have = 0;
    if (!bracket_hot(arena, C.tix.hot[base], e, rc.b, err)) return false;
    rc.key = key;
    return true;
}

__device__ __forceinline__ double rate_value(StepConstants const& C, const double* __restrict__ arena, RateCache& rc,
                                             double e, int which, Err& err, int base = RREA_T_E_COLLISION)
{
    if (!rate_bracket(C, arena, rc, e, err, base)) return 0.0;
    unsigned const bit = 1u << which;
    if (!(rc.have & bit)) {
        rc.v[which] = eval_hot(arena, C.tix.hot[base + which], rc.b, err);
        rc.have |= bit;
    }
    return rc.v[which];
}

__device__ __forceinline__ bool rate_positive(StepConstants const& C, const double* __restrict__ arena, RateCache& rc,
                                              double e, int which, Err& err, int base = RREA_T_E_COLLISION)
{
    if (!rate_bracket(C, arena, rc, e, err, base)) return false;
    unsigned const bit = 1u << which;
    if (rc.have & bit) return gt0(rc.v[which]);
    return positive_hot(arena, C.tix.hot[base + which], rc.b, err);
}

enum { kRateCollision = 0, kRateSoft = 1, kRateMoller = 2, kRateBhabha = 2, kRateBrems = 3, kRateAnnihilation = 5 };

// Competing STP rates, O/RreaChargedFinalStates.H:107-152 with the accessors
// ElectronHardMollerMeanFreePath / ElectronBremsstrahlungMeanFreePath
// (S/RreaInteractionTables.cpp:2394-2412, 2666-2676).
__device__ __forceinline__ void competing_rates(StepConstants const& C, const double* __restrict__ arena,
                                                RateCache& rc, double e, double& s0, double& s1, Err& err)
{
    double const thr = C.hm_threshold_eV;
    bool const m_open = C.hm_enabled && gt0(thr) && e > 2.0 * thr;
    bool const b_open = finite_bits(e) && finite_bits(C.photon_cutoff_eV) && e > C.photon_cutoff_eV;
    s0 = 0.0;
    s1 = 0.0;
    if (m_open) {
        double const inv = rate_value(C, arena, rc, e, kRateMoller, err);
        s0 = (gt0(thr) && e <= 2.0 * thr) ? 1.0e-99 : rate_from_inverse(inv * 1.0, err);
    }
    if (b_open) {
        s1 = rate_from_inverse(rate_value(C, arena, rc, e, kRateBrems, err) * 1.0, err);
    }
    s0 = frozen_rate(s0, err);
    s1 = frozen_rate(s1, err);
}

// Positron competing STP rates, O/RreaChargedFinalStates.H:121-140 with the
// accessors PositronHardBhabhaMeanFreePath, PositronBremsstrahlungMeanFreePath
// and PositronAnnihilationMeanFreePath (S/RreaInteractionTables.cpp:3141-3206):
// Bhabha opens above the production threshold, brems above the photon cut,
// annihilation at every energy.
__device__ __forceinline__ void competing_rates_positron(StepConstants const& C, const double* __restrict__ arena,
                                                         RateCache& rc, double e, double& s0, double& s1, double& s2,
                                                         Err& err)
{
    double const thr = C.hm_threshold_eV;
    s0 = 0.0;
    s1 = 0.0;
    if (!(gt0(thr) && e <= thr)) {
        s0 = rate_from_inverse(rate_value(C, arena, rc, e, kRateBhabha, err, RREA_T_P_COLLISION) * 1.0, err);
    }
    if (e > C.photon_cutoff_eV) {
        s1 = rate_from_inverse(rate_value(C, arena, rc, e, kRateBrems, err, RREA_T_P_COLLISION) * 1.0, err);
    }
    s2 = rate_from_inverse(rate_value(C, arena, rc, e, kRateAnnihilation, err, RREA_T_P_COLLISION) * 1.0, err);
    s0 = frozen_rate(s0, err);
    s1 = frozen_rate(s1, err);
    s2 = frozen_rate(s2, err);
}

// S/RreaInteractionTables.cpp:2414-2440
__device__ __forceinline__ double hard_moller_energy_loss(StepConstants const& C, const double* __restrict__ arena,
                                                          double e, double dr, Err& err)
{
    RreaTable1DIndex const& h = C.tix.hot[RREA_T_E_HARD_MOLLER];
    double const inv = interpolate(arena, h, e, err);
    if (!(gt0(inv))) return 0.0;
    double const mean =
        semilogx(arena + h.x, arena + h.lx, arena + h.ilx, arena + C.tix.hard_moller_mean_secondary, h.n, e, err);
    if (!(gt0(mean))) return 0.0;
    return mean * inv * dr;
}

// electron_ensemble_mean_drag_ev_per_m (O/RreaTransportStep.H:226-247): the
// realized continuous loss plus the mean losses of the discrete hard-Moller
// and tracked-brems channels.
__device__ __forceinline__ double ensemble_mean_drag(StepConstants const& C, const double* __restrict__ arena,
                                                     double e, double rho, Err& err)
{
    if (!(e > 0.0) || !(rho > 0.0)) return 0.0;
    RateCache rc;
    double const col = rate_value(C, arena, rc, e, kRateCollision, err);
    double const soft = rate_value(C, arena, rc, e, kRateSoft, err);
    double const hard = C.hm_enabled ? hard_moller_energy_loss(C, arena, e, rho, err) : 0.0;
    double tracked = 0.0;
    double const inv = rate_value(C, arena, rc, e, kRateBrems, err) * rho;
    if (gt0(inv)) tracked = inv * mean_conditional(arena, C.tix.cdf[RREA_C_BREMS_E], e, err);
    return (col * rho + soft * rho) + hard + tracked;
}

// defer_cd_electron_plane_crossings (O/RreaTransportStep.H:249-332) for one
// continuous segment [b, eff] of an electron's chord, with the crossing rule
// of RreaForEachNonperiodicPlaneCrossing (I/RreaPlaneFlux.H:79-118: upward
// z0 < plane <= z1, downward z1 < plane <= z0) and the accumulation of
// RreaPlaneFluxAccumulator::AddCrossing (:193-283) as device atomics.  The
// energy at a crossing is the segment's start energy less the fixed-energy
// stopping over the density path to the crossing, capped by the segment's
// drag; a crossing is a local runaway when its energy is at or above the
// cutoff and |E| there beats the ensemble mean drag.  Rare (planes only),
// so out of line with its arguments by value; returns a status code.
template <int NP>
__device__ __noinline__ int plane_crossings(StepConstants const& C, ElectronArgs const& A, FieldView const fv,
                                            Path<NP> const path, Geom const g, Intervals<NP> const iv, double b,
                                            double eff, double weight, double k_before, double fixed_stp,
                                            double drag)
{
    double x0, y0, z0, x1, y1, z1;
    point_at_full(path, g, b, x0, y0, z0);
    point_at_full(path, g, eff, x1, y1, z1);
    if (!isfinite(z0) || !isfinite(z1)) return RREA_GPU_ERR_GEOMETRY;
    if (z1 == z0) return 0;
    int const n = A.n_planes;
    const double* __restrict__ pz = A.plane_z;
    double const lo = fmin(z0, z1), hi = fmax(z0, z1);
    // [upper_bound(lo), upper_bound(hi)): the planes in (lo, hi]
    int first = 0, last = 0;
    {
        int a = 0, c = n;
        while (a < c) {
            int const m = (a + c) >> 1;
            if (__ldg(pz + m) <= lo) a = m + 1;
            else c = m;
        }
        first = a;
        c = n;
        while (a < c) {
            int const m = (a + c) >> 1;
            if (__ldg(pz + m) <= hi) a = m + 1;
            else c = m;
        }
        last = a;
    }
    double const inverse_span = 1.0 / (z1 - z0);
    int const d = z1 > z0 ? 0 : 1;
    double const cut = C.cfg.low_energy_cutoff_eV;
    for (int i = first; i < last; ++i) {
        double const fraction = b + (__ldg(pz + i) - z0) * inverse_span * (eff - b);
        double x, y, z;
        point_at_full(path, g, fraction, x, y, z);
        double const r = hypot(x, y);
        double const raw = fixed_stp * density_path(iv, path, b, fraction);
        double const kc = fmax(0.0, k_before - fmin(drag, raw));
        bool local = false;
        if (kc >= cut) {
            Err err;
            double const rho = positive_or(density_ratio_at_z(A.prof, C.cfg.density_ratio, z, err), 1.0);
            double fer, fez, fbt;
            gather(fv, r, z, fer, fez, fbt);
            double const mean_drag = ensemble_mean_drag(C, A.arena, kc, rho, err);
            if (err.code) return err.code;
            double const magnitude = hypot(fer, fez);
            local = isfinite(magnitude) && isfinite(mean_drag) && mean_drag >= 0.0 && magnitude > mean_drag;
        }
        if (!isfinite(weight) || !(weight >= 0.0) || !isfinite(r) || !(r >= 0.0)) return RREA_GPU_ERR_INVALID_STATE;
        double* const bin = A.plane_bins + kPlaneValues * i;
        atomicAdd(bin + d, weight);
        if (local) {
            atomicAdd(bin + 2 + d, weight);
            atomicAdd(bin + 6 + d, weight * r);
            atomicAdd(bin + 8 + d, weight * r * r);
        }
        if (kc >= 1.0e6) atomicAdd(bin + 4 + d, weight);
    }
    return 0;
}

// S/RreaInteractionTables.cpp:2477-2493
__device__ __forceinline__ double elastic_inverse_stp(StepConstants const& C, const double* __restrict__ arena,
                                                      double e, Err& err,
                                                      double le = __builtin_nan(""), int species = 0)
{
    RreaElasticIndex const& el = C.tix.elastic[species];
    double const mfp = semilogx(arena + el.x, arena + el.lx, arena + el.ilx, arena + el.mfp, el.n, e, err, le) / 1.0;
    return frozen_rate(gt0(mfp) ? 1.0 / mfp : 0.0, err);
}

// S/RreaInteractionTables.cpp:2504-2560
__device__ __forceinline__ double sample_gs_cos(StepConstants const& C, const double* __restrict__ arena, double e,
                                                double n, double u, Err& err, double le, int species = 0)
{
    RreaArenaIndex const& ix = C.tix;
    if (!charged_in_range(ix, e)) {
        err.set(RREA_GPU_ERR_RANGE);
        return 1.0;
    }
    if (!finite_bits(u) || lt0(u) || u > 1.0) {
        err.set(RREA_GPU_ERR_INVALID_STATE);
        return 1.0;
    }
    bool const use_gs = e <= ix.gs_wentzel_transition_eV;
    RreaAngleIndex const& a = use_gs ? ix.gs[species] : ix.wentzel[species];
    if (e < __ldg(arena + a.e) || e > __ldg(arena + a.e + a.ne - 1)) {
        err.set(RREA_GPU_ERR_RANGE);
        return 1.0;
    }
    if (!finite_bits(n) || n < ix.gs_few_collision_threshold) {
        err.set(RREA_GPU_ERR_INVALID_STATE);
        return 1.0;
    }
    if (n >= ix.gs_isotropic_above_n) return 2.0 * u - 1.0;
    return sample_gs_angle(arena, a, e, n, u, err, le);
}
__device__ __forceinline__ double sample_single_elastic_cos(StepConstants const& C, const double* __restrict__ arena,
                                                            double e, double cdf_u, Err& err, double le,
                                                            int species = 0)
{
    if (!charged_in_range(C.tix, e)) {
        err.set(RREA_GPU_ERR_RANGE);
        return 1.0;
    }
    RreaElasticIndex const& el = C.tix.elastic[species];
    double const eta = semilogx(arena + el.x, arena + el.lx, arena + el.ilx, arena + el.eta, el.n, e, err, le);
    double const u = fmin(max0(cdf_u), 1.0 - 1.0e-15);
    return 1.0 - 2.0 * eta * u / (1.0 + eta - u);
}
// S/RreaInteractionTables.cpp:2714-2760
__device__ __forceinline__ double tsai_g2(double x)
{
    if (x < 1.0e-3) {
        return x * x * (0.5 + x * (-1.0 / 3.0 + x * (1.0 / 8.0 + x * (-1.0 / 30.0 + x * (1.0 / 144.0)))));
    }
    return -expm1(-x) - x * exp(-x);
}
__device__ __forceinline__ double sample_brems_cos(StepConstants const& C, double e, double cdf_u, Err& err)
{
    if (!charged_in_range(C.tix, e)) {
        err.set(RREA_GPU_ERR_RANGE);
        return 1.0;
    }
    cdf_u = max0(fmin(1.0, cdf_u));
    if (eq0(cdf_u)) return 1.0;
    if (cdf_u == 1.0) return -1.0;
    double constexpr a = 0.625;
    double const umax = 2.0 * (1.0 + e / kMeC2);
    double const target = cdf_u * (0.25 * tsai_g2(a * umax) + 0.75 * tsai_g2(3.0 * a * umax));
    double lo = 0.0, hi = umax;
    for (int it = 0; it < 60; ++it) {
        double const mid = 0.5 * (lo + hi);
        double const m = 0.25 * tsai_g2(a * mid) + 0.75 * tsai_g2(3.0 * a * mid);
        if (m < target) lo = mid; else hi = mid;
    }
    double const f = 0.5 * (lo + hi) / umax;
    return 1.0 - 2.0 * f * f;
}

// Interaction site of one discrete event (RreaInteractionSite,
// O/RreaParticleInteraction.H:943-949).
struct Site {
    double x, y, z, r, birth;
};

// RreaApplyHardMollerFinalState, O/RreaChargedFinalStates.H:164-225
__device__ __forceinline__ void moller_final_state(StepConstants const& C, ElectronArgs const& A, RngStream const& rng,
                                                uint64_t rng_index, int64_t ip, uint64_t key, double weight,
                                                Site const& site, double& k, double& dx, double& dy, double& dz,
                                                uint32_t& lineage, Err& err)
{
    double const kb = k;
    if (!charged_in_range(C.tix, kb)) {
        err.set(RREA_GPU_ERR_RANGE);
        return;
    }
    double sec = sample_conditional(A.arena, C.tix.cdf[RREA_C_MOLLER], kb,
                                    rng.uniform(rng_index, kChHardMollerEnergy), true, err);
    sec = fmax(C.hm_threshold_eV, fmin(sec, 0.5 * kb));
    double pdx, pdy, pdz, sdx, sdy, sdz;
    moller_lab_directions(dx, dy, dz, kb, sec, rng.uniform(rng_index, kChHardMollerAzimuth), pdx, pdy, pdz, sdx, sdy,
                          sdz);
    k = max0(kb - sec);
    dx = pdx; dy = pdy; dz = pdz;
    append_secondary(A, ip, key, weight, lineage, 0, 2, site.x, site.y, site.z, sdx, sdy, sdz, sec, site.birth, err);
    deposit_source(C, A.cells, 0, site.r, site.z, weight, sec, sec);
    // closure of the HardMoller group (O/RreaChargedFinalStates.H:211-224)
    double const cut = C.cfg.low_energy_cutoff_eV;
    GroupClosure gc;
    gc.begin(-1.0, kMeC2, weight, kb, k, true);
    gc.secondary(-1.0, kMeC2, weight, sec);
    gc.ionization(weight, sec, cut);
    if (!gc.valid(cut)) err.set(RREA_GPU_ERR_INVALID_STATE);
}

// RreaApplyBremsFinalState, O/RreaChargedFinalStates.H:329-394; POS selects
// the positron photon-energy CDF and RNG channels.
template <bool POS = false>
__device__ __forceinline__ void brems_final_state(StepConstants const& C, ElectronArgs const& A, RngStream const& rng,
                                               uint64_t rng_index, int64_t ip, uint64_t key, double weight,
                                               Site const& site, double& k, double& dx, double& dy, double& dz,
                                               uint32_t& lineage, Err& err)
{
    double const kb = k;
    if (!charged_in_range(C.tix, kb)) {
        err.set(RREA_GPU_ERR_RANGE);
        return;
    }
    double const sampled = sample_conditional(A.arena, C.tix.cdf[POS ? RREA_C_BREMS_P : RREA_C_BREMS_E], kb,
                                              rng.uniform(rng_index, POS ? kChPositronBremsEnergy : kChBremsEnergy),
                                              false, err);
    double const eg = fmin(max0(sampled), max0(kb));
    double const after = max0(fmax(kb, 0.0) - eg);
    bool const tracked = finite_bits(C.photon_cutoff_eV) && ge0(C.photon_cutoff_eV) && eg >= C.photon_cutoff_eV;
    double const ct = sample_brems_cos(C, kb, rng.uniform(rng_index, POS ? kChPositronBremsAngle : kChBremsAngle), err);
    double gx, gy, gz;
    cone_direction(dx, dy, dz, ct, rng.uniform(rng_index, POS ? kChPositronBremsAzimuth : kChBremsAzimuth), gx, gy,
                   gz);
    photon_recoil(kb, eg, gx, gy, gz, dx, dy, dz);
    k = after;
    if (tracked) {
        append_secondary(A, ip, key, weight, lineage, 2, 4, site.x, site.y, site.z, gx, gy, gz, eg, site.birth, err,
                         POS ? 1 : 0);
    } else if (gt0(eg)) {
        // deposit_local_energy_as_ion_pairs, O/RreaTransportStep.H:530-561
        double const w_air = C.tix.w_air_eV_per_pair;
        double const pw = weight * eg / fmax(w_air, 1.0);
        if (gt0(weight) && gt0(pw)) deposit_source(C, A.cells, 0, site.r, site.z, pw, 0.0, w_air);
    }
    // closure of the Bremsstrahlung group (O/RreaChargedFinalStates.H:377-393)
    double const cut = C.cfg.low_energy_cutoff_eV;
    GroupClosure gc;
    gc.begin(POS ? 1.0 : -1.0, kMeC2, weight, kb, after, true);
    if (tracked) gc.secondary(0.0, 0.0, weight, eg);
    else if (gt0(eg)) gc.local(weight, eg, C.tix.w_air_eV_per_pair, cut);
    if (!gc.valid(cut)) err.set(RREA_GPU_ERR_INVALID_STATE);
}

// The out-of-line helpers below take every argument by value and return
// their results by value: a reference or pointer to a caller variable would
// pin that variable to the thread's stack for the whole transport loop.

struct Dir3 {
    double x, y, z;
    int err;
};

// RreaApplyBhabhaFinalState, O/RreaChargedFinalStates.H:238-288: a
// secondary below the production threshold discards this event only.
__device__ __forceinline__ void bhabha_final_state(StepConstants const& C, ElectronArgs const& A, RngStream const& rng,
                                                   uint64_t rng_index, int64_t ip, uint64_t key, double weight,
                                                   Site const& site, double& k, double& dx, double& dy, double& dz,
                                                   uint32_t& lineage, Err& err)
{
    double const kb = k;
    if (!charged_in_range(C.tix, kb)) {
        err.set(RREA_GPU_ERR_RANGE);
        return;
    }
    double const sec = fmin(sample_conditional(A.arena, C.tix.cdf[RREA_C_BHABHA], kb,
                                               rng.uniform(rng_index, kChPositronBhabhaEnergy), false, err),
                            max0(kb));
    double const thr = C.hm_threshold_eV;
    if (!(gt0(sec)) || (gt0(thr) && sec < thr)) return;
    double pdx, pdy, pdz, sdx, sdy, sdz;
    moller_lab_directions(dx, dy, dz, kb, sec, rng.uniform(rng_index, kChPositronBhabhaAzimuth), pdx, pdy, pdz, sdx,
                          sdy, sdz);
    k = max0(kb - sec);
    dx = pdx; dy = pdy; dz = pdz;
    append_secondary(A, ip, key, weight, lineage, 0, 3, site.x, site.y, site.z, sdx, sdy, sdz, sec, site.birth, err, 1);
    deposit_source(C, A.cells, 2, site.r, site.z, weight, 0.0, sec);
    // closure of the HardBhabha group (O/RreaChargedFinalStates.H:281-294)
    double const cut = C.cfg.low_energy_cutoff_eV;
    GroupClosure gc;
    gc.begin(1.0, kMeC2, weight, kb, k, true);
    gc.secondary(-1.0, kMeC2, weight, sec);
    gc.positive_ion(weight);
    if (!gc.valid(cut)) err.set(RREA_GPU_ERR_INVALID_STATE);
}

// sample_annihilation_photon_energy_fraction (S/RreaInteractionTables.cpp:63-108):
// Heitler two-photon spectrum by 64-step bisection of its primitive.
__device__ __forceinline__ double annihilation_fraction(double gamma, double draw)
{
    if (gamma <= 1.0 + 1.0e-12) return 0.5;
    double const bcm = sqrt(max0((gamma - 1.0) / (gamma + 1.0)));
    double const emin = 0.5 * (1.0 - bcm), emax = 0.5 * (1.0 + bcm);
    double const u = finite_bits(draw) ? max0(fmin(1.0, draw)) : 0.5;
    double const gp1 = gamma + 1.0;
    double const a = 1.0 + 2.0 * gamma / (gp1 * gp1);
    double const c = gp1 * gp1;
    double const flo = a * log(emin) - emin + 1.0 / (c * emin);
    double const fhi = a * log(emax) - emax + 1.0 / (c * emax);
    double const span = fhi - flo;
    if (!(gt0(span))) return 0.5;
    double const target = flo + u * span;
    double lo = emin, hi = emax;
    for (int it = 0; it < 64; ++it) {
        double const mid = 0.5 * (lo + hi);
        if (a * log(mid) - mid + 1.0 / (c * mid) < target) lo = mid; else hi = mid;
    }
    return fmax(emin, fmin(emax, 0.5 * (lo + hi)));
}

// TransportStep::spawn_positron_annihilation (O/RreaTransportStep.H:563-702)
// with SamplePositronAnnihilationFinalState (S/RreaInteractionTables.cpp:
// 3208-3253): two photons, momentum-balanced in flight, back to back at rest;
// a below-cutoff positron first thermalizes its kinetic energy as ion pairs.
// Returns the parent's lineage count after the appended photons.  Taken out
// of line with every argument by value (it runs at most once per positron).
static __device__ __noinline__ uint32_t spawn_annihilation(ElectronArgs A, RngStream rng, uint64_t idx, int64_t ip,
                                                    uint64_t key, double weight, uint32_t lineage, double x, double y,
                                                    double z, double r, double ax, double ay, double az, double k,
                                                    bool at_rest, double birth)
{
    StepConstants const& C = c_step;
    Err err;
    if (le0(weight)) return lineage;
    normalize(ax, ay, az);
    double const ka = at_rest ? 0.0 : max0(k);
    if (!(eq0(ka)) && !charged_in_range(C.tix, ka)) {
        record_failure(A, RREA_GPU_ERR_RANGE, ip);
        return lineage;
    }
    double const d_e = rng.uniform(idx, kChPositronAnnihilationPolar);
    double const d_a = rng.uniform(idx, kChPositronAnnihilationAzimuth);
    double const gamma = 1.0 + ka / kMeC2;
    double const total = 2.0 * kMeC2 + ka;
    double e1 = 0.0, e2 = 0.0, cos1 = 1.0, azim = 0.0;
    bool rest = false;
    if (gamma <= 1.0 + 1.0e-10) {
        e1 = kMeC2;
        e2 = kMeC2;
        cos1 = 2.0 * (finite_bits(d_e) ? max0(fmin(1.0, d_e)) : 0.5) - 1.0;
        azim = finite_bits(d_a) ? d_a - floor(d_a) : 0.0;
        if (lt0(azim)) azim += 1.0;
        rest = true;
    } else {
        double const beta = sqrt(max0(1.0 - 1.0 / (gamma * gamma)));
        double const eps = annihilation_fraction(gamma, d_e);
        e1 = eps * total;
        e2 = max0(total - e1);
        double const denom = eps * gamma * beta;
        if (gt0(e1) && gt0(e2) && gt0(denom)) {
            cos1 = fmax(-1.0, fmin(1.0, (eps * (gamma + 1.0) - 1.0) / denom));
            azim = finite_bits(d_a) ? d_a - floor(d_a) : 0.0;
            if (lt0(azim)) azim += 1.0;
        }
    }
    double g1x, g1y, g1z;
    cone_direction(ax, ay, az, cos1, azim, g1x, g1y, g1z);
    e1 = max0(e1);
    e2 = max0(e2);
    double g2x = -g1x, g2y = -g1y, g2z = -g1z;
    if (!rest && gt0(e2)) {
        double const p = sqrt(max0(ka * (ka + 2.0 * kMeC2)));
        g2x = (p * ax - e1 * g1x) / e2;
        g2y = (p * ay - e1 * g1y) / e2;
        g2z = (p * az - e1 * g1z) / e2;
        normalize(g2x, g2y, g2z);
    }
    double local = 0.0;
    double const cut = C.photon_cutoff_eV;
    double const w_air = C.tix.w_air_eV_per_pair;
    if (e1 >= cut) append_secondary(A, ip, key, weight, lineage, 2, 9, x, y, z, g1x, g1y, g1z, e1, birth, err, 1);
    else local += e1;
    if (e2 >= cut) append_secondary(A, ip, key, weight, lineage, 2, 9, x, y, z, g2x, g2y, g2z, e2, birth, err, 1);
    else local += e2;
    if (at_rest && gt0(k)) {
        double const pw = weight * k / fmax(w_air, 1.0);
        if (gt0(pw)) deposit_source(C, A.cells, 0, r, z, pw, 0.0, w_air);
    }
    if (gt0(local)) {
        double const pw = weight * local / fmax(w_air, 1.0);
        if (gt0(pw)) deposit_source(C, A.cells, 0, r, z, pw, 0.0, w_air);
    }
    deposit_source(C, A.cells, 2, r, z, weight, 0.0, 0.0);
    {
        // closure of the PositronAnnihilation group (O/RreaPositronTransport.cpp:136-162, 710-735)
        double const ecut = C.cfg.low_energy_cutoff_eV;
        GroupClosure gc;
        gc.begin(1.0, kMeC2, weight, max0(k), 0.0, false);
        if (e1 >= cut) gc.secondary(0.0, 0.0, weight, e1);
        if (e2 >= cut) gc.secondary(0.0, 0.0, weight, e2);
        if (at_rest && gt0(k)) gc.local(weight, k, w_air, ecut);
        gc.local(weight, local, w_air, ecut);
        gc.positive_ion(weight);
        if (!gc.valid(ecut)) err.set(RREA_GPU_ERR_INVALID_STATE);
    }
    if (err.code) record_failure(A, err.code, ip);
    return lineage;
}

// Few-collision branch of apply_gs_elastic_scatter (O/RreaTransportStep.H:397-416):
// a Poisson number of single screened-Rutherford deflections.  Rare for
// tracked electrons (n >= 10 elastic collisions per substep at MeV energies),
// so it is kept out of line.
static __device__ __noinline__ Dir3 gs_few_collisions(const double* __restrict__ arena, RngStream rng, uint64_t sub,
                                               double gs_n, double k, double lk, double dx, double dy, double dz,
                                               int species)
{
    uint64_t const ch_count = species ? kChPositronGsFewCount : kChElectronGsFewCount;
    uint64_t const ch_scatter = species ? kChPositronGsFewScatter : kChElectronGsFewScatter;
    uint64_t const ch_azimuth = species ? kChPositronGsFewAzimuth : kChElectronGsFewAzimuth;
    StepConstants const& C = c_step;
    Err err;
    double const few = C.tix.gs_few_collision_threshold;
    int const cap = static_cast<int>(ceil(3.0 * few));
    if (cap >= 255) return Dir3{dx, dy, dz, RREA_GPU_ERR_INVALID_STATE};
    int const cnt = poisson_capped(gs_n, rng.uniform((sub << 8) | 0, ch_count), cap);
    for (int q = 0; q < cnt; ++q) {
        uint64_t const inner = static_cast<uint64_t>(q + 1);
        double const ct =
            sample_single_elastic_cos(C, arena, k, rng.uniform((sub << 8) | inner, ch_scatter), err, lk, species);
        double nx, ny, nz;
        cone_direction(dx, dy, dz, ct, rng.uniform((sub << 8) | inner, ch_azimuth), nx, ny, nz);
        dx = nx; dy = ny; dz = nz;
    }
    return Dir3{dx, dy, dz, err.code};
}

// The 56-step bisection of RreaLimitContinuousSegmentAtCutoff
// (O/RreaParticleInteraction.H:245-263), run only when the drag reaches the
// cutoff inside the segment.  Returns NaN when a loss is not finite.
template <int NP>
__device__ __noinline__ double cutoff_bisection(Intervals<NP> iv, Path<NP> path, double b, double e, double total,
                                                double to_cut)
{
    double lo = b, hi = e;
    for (int it = 0; it < 56; ++it) {
        double const mid = 0.5 * (lo + hi);
        double const l = total * density_path(iv, path, b, mid);
        if (!finite_bits(l) || lt0(l)) return __longlong_as_double(0x7ff8000000000000LL);
        if (l < to_cut) lo = mid; else hi = mid;
    }
    return 0.5 * (lo + hi);
}

// One charged particle through one outer step.  POS = false is the electron
// loop (O/RreaElectronTransport.cpp); POS = true the positron loop
// (O/RreaPositronTransport.cpp:9-878), which shares the substep and event
// engine and differs in charge, channels (Bhabha, brems, annihilation), drag
// tables, GS tables and RNG channels, and ends below the cutoff in at-rest
// annihilation instead of demotion.  Returns the disposition (0 survive,
// 1 escape, 2 demotion / annihilation, 3 zero weight, -1 error).
template <int NP, bool POS = false>
__device__ __forceinline__ int transport_charged(StepConstants const& C, ElectronArgs const& A, int64_t ip,
                                                 uint64_t& subcycles_out, uint64_t& events_out,
                                                 uint32_t& lineage, IonPairCache& ion_pairs, Err& err)
{
    constexpr double q = POS ? 1.0 : -1.0;
    constexpr int species = POS ? 1 : 0;
    constexpr int rate_base = POS ? RREA_T_P_COLLISION : RREA_T_E_COLLISION;
    const double* __restrict__ arena = A.arena;
    rrea_gpu_config const& cfg = C.cfg;
    Geom const g{cfg.r_lo, cfg.r_hi, cfg.z_lo, cfg.z_hi, cfg.periodic_z != 0};
    double const cutoff = cfg.low_energy_cutoff_eV;
    double const rho = C.density_ratio;
    double const w_air = C.tix.w_air_eV_per_pair;
    // ion pairs per eV of drag loss, a product per substep instead of a division
    double const inv_pair_energy = 1.0 / fmax(w_air, 1.0);
    double const hm_thr = C.hm_threshold_eV;
    double const dt_s = C.dt_s;

    // ---- prologue, O/RreaTransportStep.H:730-819
    int32_t const cpu = A.cpu ? A.cpu[ip] : 0;
    uint64_t const key = static_cast<uint64_t>(llabs(A.id[ip])) ^ (static_cast<uint64_t>(cpu) << 40);
    FieldView const fv = A.fv.for_instance(cpu);
    double const weight = A.w[ip];
    if (le0(weight)) {
        A.id[ip] = -A.id[ip];
        return 3;
    }
    double const prev_r = A.prev_r[ip];
    if (prev_r > cfg.r_hi + 1.0e-9 * cfg.r_hi) {
        err.set(RREA_GPU_ERR_GEOMETRY);
        return -1;
    }
    RngStream rng;
    rng.init(cfg.rng_seed, key, C.step_key);
    double dx = A.prev_ux[ip], dy = A.prev_uy[ip], dz = A.prev_uz[ip];
    double k = kinetic_from_proper_velocity(dx, dy, dz);
    normalize(dx, dy, dz);
    double const seed_th = A.prev_theta[ip];
    double sth, cth;
    sincos(seed_th, &sth, &cth);
    double run_x = prev_r * cth;
    double run_y = prev_r * sth;
    double run_z = A.prev_z[ip];
    double const r_particle = prev_r, z_particle = run_z;
    double const x_particle = run_x, y_particle = run_y;

    auto build_chord = [&](double req_dt, Path<NP>& path) -> bool {
        // O/RreaParticleInteraction.H:110-161
        if (!finite_bits(req_dt) || !(ge0(req_dt))) return false;
        double const speed = charged_speed(k);
        double const dn = sqrt(dx * dx + dy * dy + dz * dz);
        if (!finite_bits(speed) || !finite_bits(dn) || !(gt0(dn))) return false;
        double const sc = speed * req_dt / dn;
        double const exx = run_x + sc * dx, eyy = run_y + sc * dy, ezz = run_z + sc * dz;
        clip_xyz(run_x, run_y, run_z, exx, eyy, ezz, g, path, err);
        return finite_bits(path.full) && eq0(path.in_begin);
    };
    auto deposit_local = [&](double r, double z, double e) {
        // O/RreaTransportStep.H:530-561
        if (le0(weight) || le0(e)) return;
        double const pw = weight * e / fmax(w_air, 1.0);
        if (le0(pw)) return;
        deposit_source(C, A.cells, 0, r, z, pw, 0.0, w_air);
    };
    auto finish = [&](int disp) { return disp; };

    Path<NP> path;
    bool const driver_valid = build_chord(dt_s, path);
    if (err.code) return finish(-1);
    bool esc, esc_inv;
    clipped_escape_policy(path, g, rz_radius(path.ex, path.ey), path.ez, esc, esc_inv);
    double const ds = driver_valid ? path.in_length : 0.0;
    Intervals<NP> iv;
    build_intervals(path, g, A.prof, rho, iv, err);
    double const driver_span = fmax(path.in_end, 1.0e-6);
    FieldRange const dfw = path_field_work(fv, g, path, q, 0.0, 1.0, err);
    double const field_work = dfw.work / driver_span;
    double const chord_dpath = density_path(iv, path, path.in_begin, path.in_end);
    double transported_dpath = 0.0, transported_len = 0.0;
    double particle_density =
        gt0(ds) ? chord_dpath / ds : positive_or(density_ratio_at_z(A.prof, C.cfg.density_ratio, z_particle, err), rho);

    // net chord from the captured start (AccumulateChargedSegment), signed
    // with the species charge; deposited by the current pass after the kernel
    auto put_segment = [&](double r1, double z1) {
        if (!A.segments) return;
        SegmentRec& s = A.segments[ip];
        s.a[0] = r_particle;
        s.a[1] = z_particle;
        s.a[2] = r1;
        s.a[3] = z1;
        s.a[4] = q * weight;
        s.faces = 0u;
        s.kind = 1;
    };
    auto commit_escape = [&]() {
        // O/RreaTransportStep.H:829-863: the escape deposit closes on the
        // exact face crossing of the final microchord
        double const u = proper_velocity_from_kinetic(k);
        A.ux[ip] = u * dx;
        A.uy[ip] = u * dy;
        A.uz[ip] = u * dz;
        double sr, sz, cr, cz;
        uint32_t faces;
        if (!charged_crossing(path, g, sr, sz, cr, cz, faces)) {
            // O/RreaTransportLog.H:581-584
            err.set(RREA_GPU_ERR_GEOMETRY);
            return finish(-1);
        }
        if (A.segments) {
            SegmentRec& s = A.segments[ip];
            s.a[0] = r_particle;
            s.a[1] = z_particle;
            s.a[2] = sr;
            s.a[3] = sz;
            s.a[4] = cr;
            s.a[5] = cz;
            s.a[6] = q * weight;
            s.faces = faces;
            s.kind = 2;
        }
        if (esc_inv) A.id[ip] = -A.id[ip];
        return finish(1);
    };
    auto demote = [&](double r, double z) {
        // O/RreaElectronTransport.cpp:151-174, 856-879
        put_segment(r, z);
        deposit_source(C, A.cells, 1, r, z, weight, 0.0, 0.0);
        deposit_local(r, z, k);
        A.id[ip] = -A.id[ip];
        return finish(2);
    };
    auto annihilate = [&](double x, double y, double z, double r, uint64_t idx, double birth) {
        // at-rest annihilation, O/RreaPositronTransport.cpp:131-160, 793-845
        put_segment(r, z);
        lineage = spawn_annihilation(A, rng, idx, ip, key, weight, lineage, x, y, z, r, dx, dy, dz, k, true, birth);
        A.id[ip] = -A.id[ip];
        return finish(2);
    };

    bool const below = k < cutoff;
    if (esc && below) return commit_escape();
    if (!esc && below) {
        if constexpr (POS) return annihilate(x_particle, y_particle, z_particle, r_particle, 0, 1.0);
        else return demote(r_particle, z_particle);
    }
    if (le0(ds)) {
        if (esc) return commit_escape();
        return finish(0);
    }
    if (iv.n == 0) {
        err.set(RREA_GPU_ERR_INVALID_STATE);
        return finish(-1);
    }

    // ---- substep count, O/RreaElectronTransport.cpp:187-279
    uint64_t subcycles;
    RateCache rc;
    {
        double s0, s1, s2 = 0.0;
        if constexpr (POS) competing_rates_positron(C, arena, rc, k, s0, s1, s2, err);
        else competing_rates(C, arena, rc, k, s0, s1, err);
        double const driver_dpath = chord_dpath / driver_span;
        double const target = cfg.max_optical_depth_per_substep;
        uint64_t const cap = cfg.max_subcycles;
        double max_tau, total_stp;
        if constexpr (POS) {
            // O/RreaPositronTransport.cpp:168-185: the summed rate times the path
            total_stp = (s0 + s1) + s2;
            max_tau = total_stp * driver_dpath;
        } else {
            max_tau = (s0 * driver_dpath) + (s1 * driver_dpath);
            total_stp = s0 + s1;
        }
        uint64_t const req = static_cast<uint64_t>(fmax(1.0, ceil(max_tau / target)));
        bool viol = req > cap;
        uint64_t sub = req < cap ? req : cap;
        // selected_material_subcycles, O/RreaTransportStep.H:148-184
        for (int guard = 0; guard < 64; ++guard) {
            double const maximum = total_stp * max_uniform_slice(iv, path, sub);
            double const tol = 64.0 * kEps * fmax(1.0, target);
            if (maximum <= target + tol) break;
            if (sub >= cap) {
                viol = true;
                break;
            }
            double const est = ceil(static_cast<double>(sub) * (maximum / target));
            uint64_t next = sub + 1U;
            if (est >= static_cast<double>(cap)) next = cap;
            else if (est > static_cast<double>(next)) next = static_cast<uint64_t>(est);
            sub = next < cap ? next : cap;
        }
        double const gs_n = elastic_inverse_stp(C, arena, k, err, __builtin_nan(""), species) * driver_dpath;
        double const ke = fmax(k, cutoff);
        double drag_est = 0.0;
        if constexpr (POS) {
            // collision stopping only (O/RreaPositronTransport.cpp:195-201)
            drag_est = rate_value(C, arena, rc, ke, kRateCollision, err, rate_base) * 1.0 * driver_dpath;
        } else if (gt0(ke)) {
            double const col = rate_value(C, arena, rc, ke, kRateCollision, err);
            double const soft = rate_value(C, arena, rc, ke, kRateSoft, err);
            drag_est = (col * 1.0 + soft * 1.0) * driver_dpath;
        }
        double const impulse = fmax(cfg.max_field_impulse_fraction * k, fmax(cfg.field_impulse_floor_eV, 1.0));
        uint64_t const gsd = static_cast<uint64_t>(
            fmax(1.0, ceil(fmin(gs_n, cfg.gs_total_collision_cap) / fmax(cfg.max_gs_collisions_per_substep, 1.0))));
        uint64_t const imd = static_cast<uint64_t>(fmax(1.0, ceil((fabs(field_work) + drag_est) / impulse)));
        uint64_t m = sub;
        if (gsd > m) m = gsd;
        if (imd > m) m = imd;
        subcycles = m < cap ? m : cap;
        if (cfg.strict_transport_guards && viol) err.set(RREA_GPU_ERR_GUARD);
        if (err.code) return finish(-1);
    }
    subcycles_out = subcycles;

    bool exited = false;
    uint64_t completed = 0;
    bool terminated_mid = false;
    bool annihilated = false;
    double mid_r = r_particle, mid_z = z_particle;
    double mid_x = x_particle, mid_y = y_particle, mid_elapsed = 1.0;
    double const sub_dt = dt_s / static_cast<double>(subcycles);
    FieldRange sub_field{0, 0, 0, 0, 0, 0, 0, 0};
    double sub_dt_eff = 0.0;
    uint64_t events = 0;

    auto mark_stopped = [&](double f) {
        if (path.exits && f >= path.in_end) {
            exited = true;
            return;
        }
        double x, y, z;
        point_at_full(path, g, f, x, y, z);
        if (!cartesian_half_open(g, x, y, z)) {
            exited = true;
            return;
        }
        mid_z = z;
        mid_r = rz_radius(x, y);
        if constexpr (POS) {
            // stop point and elapsed fraction for the at-rest annihilation
            mid_x = x;
            mid_y = y;
            double const within = fmin(1.0, max0(f));
            mid_elapsed = fmin(1.0, (static_cast<double>(completed) + within) / static_cast<double>(subcycles));
        }
        terminated_mid = true;
    };
    // O/RreaElectronTransport.cpp:294-400 with RreaPlanContinuousDragSegment
    // (O/RreaChargedInterleave.H:239-292) and the cutoff limiter
    // (O/RreaParticleInteraction.H:203-265).  Returns true when the drag
    // reached the cutoff; `end_out` is the effective end fraction.
    auto continuous = [&](double b, double e, double stop_e, double& end_out) -> bool {
        end_out = b;
        if (!(e > b) || !(gt0(k)) || stop_e < cutoff) return false;
        // The plan's hard-transfer loss feeds only the reference's scalar
        // tally, and its table queries cannot fail at an energy the
        // collision table just accepted, so it is not evaluated here.
        double const sc = frozen_rate(rate_value(C, arena, rc, stop_e, kRateCollision, err, rate_base) * 1.0, err);
        double const ss = frozen_rate(rate_value(C, arena, rc, stop_e, kRateSoft, err, rate_base) * 1.0, err);
        if (err.code) return false;
        double const total = sc + ss;
        // limiter
        double eff = b;
        bool reaches = false;
        bool valid = false;
        if (finite_bits(b) && finite_bits(e) && finite_bits(k) && finite_bits(cutoff) && e >= b && k >= cutoff && ge0(cutoff)) {
            double const to_cut = k - cutoff;
            double const req = total * density_path(iv, path, b, e);
            if (finite_bits(req) && ge0(req)) {
                valid = true;
                if (req < to_cut) {
                    eff = e;
                } else {
                    reaches = true;
                    if (ne0(to_cut)) {
                        eff = cutoff_bisection<NP>(iv, path, b, e, total, to_cut);
                        valid = !nan_bits(eff);
                        if (!valid) {
                            eff = b;
                            reaches = false;
                        }
                    }
                }
            }
        }
        if (!valid) {
            err.set(RREA_GPU_ERR_INVALID_STATE);
            return false;
        }
        double const path_m = density_path(iv, path, b, eff);
        double const raw_col = sc * path_m;
        double const raw_soft = ss * path_m;
        double const avail = max0(k - cutoff);
        double const drag = reaches ? avail : fmin(raw_col + raw_soft, avail);
        double const col = fmin(raw_col, drag);
        // ion pairs, O/RreaChargedInterleave.H:157-196
        if (gt0(col) && gt0(raw_col)) {
#pragma unroll
            for (int i = 0; i < NP; ++i) {
                if (i >= iv.n) break;
                double const bb = fmax(b, iv.begin[i]), ee = fmin(eff, iv.end[i]);
                if (!(ee > bb)) continue;
                double const raw = path.full * (ee - bb) * iv.density[i] * sc;
                // with one interval raw is raw_col (the same products), and
                // col * raw / raw_col is col to within an ulp
                double const loss = NP == 1 ? col : col * raw / raw_col;
                double const pw = weight * loss * inv_pair_energy;
                if (!(gt0(pw))) continue;
                double x, y, z;
                point_at_full(path, g, 0.5 * (bb + ee), x, y, z);
                // deposit_source(kind 0, sec POS ? 0 : cutoff/2, loss w_air) through the cache
                ion_pairs.add(C, A.cells, rz_radius(x, y), z, pw);
            }
        }
        if constexpr (!POS) {
            if (A.n_planes > 0) {
                if (int const code = plane_crossings<NP>(C, A, fv, path, g, iv, b, eff, weight, k, total, drag)) {
                    err.set(code);
                }
            }
        }
        k = max0(k - drag);
        if (reaches) k = cutoff;
        end_out = eff;
        return reaches;
    };
    auto channel_open = [&](int ch, double e) -> bool {
        // O/RreaChargedFinalStates.H:56-96
        if (!charged_in_range(C.tix, e)) {
            err.set(RREA_GPU_ERR_RANGE);
            return false;
        }
        if constexpr (POS) {
            if (!rate_bracket(C, arena, rc, e, err, rate_base)) return false;
            if (ch == 0) {
                return !(gt0(hm_thr) && e <= hm_thr) && rate_positive(C, arena, rc, e, kRateBhabha, err, rate_base);
            }
            if (ch == 1) return e > C.photon_cutoff_eV && rate_positive(C, arena, rc, e, kRateBrems, err, rate_base);
            if (ch == 2) return rate_positive(C, arena, rc, e, kRateAnnihilation, err, rate_base);
            return false;
        }
        if (!rate_bracket(C, arena, rc, e, err)) return false;
        if (ch == 0) {
            return C.hm_enabled && (gt0(hm_thr) && e > 2.0 * hm_thr)
                && rate_positive(C, arena, rc, e, kRateMoller, err);
        }
        if (ch == 1) {
            return (finite_bits(e) && finite_bits(C.photon_cutoff_eV) && e > C.photon_cutoff_eV)
                && rate_positive(C, arena, rc, e, kRateBrems, err);
        }
        return false;
    };

    // ---- substep interleave, O/RreaChargedInterleave.H:693-732
    for (uint64_t sub = 0; sub < subcycles; ++sub) {
        if (k < cutoff) break;
        double sb, se;
        {
            Path<NP> np;
            if (!build_chord(sub_dt, np)) break;
            path = np;
            if (!(gt0(path.full)) || !(gt0(path.in_length))) {
                exited = path.exits;
                break;
            }
            build_intervals(path, g, A.prof, rho, iv, err);
            if (iv.n == 0) {
                err.set(RREA_GPU_ERR_INVALID_STATE);
                break;
            }
#pragma unroll
            for (int i = 0; i < NP; ++i) {
                if (i >= iv.n) break;
                transported_dpath += iv.length[i] * iv.density[i];
                transported_len += iv.length[i];
            }
            sb = path.in_begin;
            se = path.in_end;
            sub_field = path_field_work(fv, g, path, q, sb, se, err);
            sub_dt_eff = sub_dt * (se - sb);
            half_kick(sub_field, 0.5 * sub_dt_eff, q, k, dx, dy, dz);
            if (k < cutoff) {
                mark_stopped(sb);
                break;
            }
        }
        // ---- event interleave, O/RreaChargedInterleave.H:546-664
        {
            double rem = sb;
            uint64_t ordinal = 0;
            while (rem < se && k >= cutoff) {
                if (err.code) break;
                if (ordinal >= kEventCap) {
                    err.set(RREA_GPU_ERR_RNG_OVERFLOW);
                    break;
                }
                double const frozen = k;
                double s0, s1, s2 = 0.0;
                if constexpr (POS) competing_rates_positron(C, arena, rc, frozen, s0, s1, s2, err);
                else competing_rates(C, arena, rc, frozen, s0, s1, err);
                double const seg_dp = density_path(iv, path, rem, se);
                double const t0 = s0 * seg_dp, t1 = s1 * seg_dp, t2 = s2 * seg_dp;
                uint64_t rng_index;
                if (!live_hazard_index(species, sub, ordinal, rng_index)) {
                    err.set(RREA_GPU_ERR_RNG_OVERFLOW);
                    break;
                }
                ++events;
                uint64_t const ch_depth = POS ? (ordinal == 0 ? kChPositronCompetingOpticalDepth
                                                              : kChPositronContinuationOpticalDepth)
                                              : (ordinal == 0 ? kChElectronCompetingOpticalDepth
                                                              : kChElectronContinuationOpticalDepth);
                uint64_t const ch_channel = POS ? (ordinal == 0 ? kChPositronCompetingChannel
                                                                : kChPositronContinuationChannel)
                                                : (ordinal == 0 ? kChElectronCompetingChannel
                                                                : kChElectronContinuationChannel);
                double const u1 = rng.uniform(rng_index, ch_depth);
                double const u2 = rng.uniform(rng_index, ch_channel);
                Selection const selv = select_hazard(arena, t0, t1, t2, POS ? 3 : 2, u1, u2);
                if (!selv.valid) {
                    err.set(RREA_GPU_ERR_INVALID_STATE);
                    break;
                }
                if (!selv.event) {
                    double eff;
                    if (continuous(rem, se, frozen, eff)) mark_stopped(eff);
                    break;
                }
                double const ev = fraction_at_density_path(iv, path, rem, se,
                                                           selv.sampled / (POS ? (s0 + s1) + s2 : s0 + s1), err);
                if (!(finite_bits(rem) && finite_bits(ev) && finite_bits(se) && se > rem && !(ev < rem) && !(ev > se))) {
                    err.set(RREA_GPU_ERR_INVALID_STATE);
                    break;
                }
                double ex, ey, ez;
                point_at_full(path, g, ev, ex, ey, ez);
                double const er = rz_radius(ex, ey);
                {
                    double eff;
                    if (continuous(rem, ev, frozen, eff)) {
                        mark_stopped(eff);
                        break;
                    }
                }
                bool const open_ev = k >= cutoff && channel_open(selv.channel, k);
                if (!open_ev) {
                    bool const open_fr = frozen >= cutoff && channel_open(selv.channel, frozen);
                    if (!open_fr) {
                        err.set(RREA_GPU_ERR_INVALID_STATE);
                        break;
                    }
                    rem = ev;
                    ++ordinal;
                    continue;
                }
                double const within = fmin(1.0, max0(ev));
                double const birth = fmin(1.0, (static_cast<double>(completed) + within) / static_cast<double>(subcycles));
                Site const site{ex, ey, ez, er, birth};
                if constexpr (POS) {
                    if (selv.channel == 0) {
                        bhabha_final_state(C, A, rng, rng_index, ip, key, weight, site, k, dx, dy, dz, lineage, err);
                    } else if (selv.channel == 1) {
                        brems_final_state<true>(C, A, rng, rng_index, ip, key, weight, site, k, dx, dy, dz, lineage,
                                                err);
                    } else {
                        // in-flight annihilation, O/RreaPositronTransport.cpp:700-727
                        put_segment(er, ez);
                        lineage = spawn_annihilation(A, rng, rng_index, ip, key, weight, lineage, ex, ey, ez, er, dx,
                                                     dy, dz, k, false, birth);
                        annihilated = true;
                        break;
                    }
                } else {
                    if (selv.channel == 0) {
                        moller_final_state(C, A, rng, rng_index, ip, key, weight, site, k, dx, dy, dz, lineage, err);
                    } else if (selv.channel == 1) {
                        brems_final_state(C, A, rng, rng_index, ip, key, weight, site, k, dx, dy, dz, lineage, err);
                    }
                }
                if (err.code) break;
                if (k <= cutoff) {
                    mark_stopped(ev);
                    break;
                }
                rem = ev;
                ++ordinal;
            }
        }
        if (err.code) break;
        if (terminated_mid || annihilated) break;
        // ---- finish_interleaved_substep, O/RreaElectronTransport.cpp:502-524
        if (k >= cutoff) {
            // apply_gs_elastic_scatter, O/RreaTransportStep.H:371-423
            // log(k) is shared by the elastic-MFP and angle-table brackets.
            double const lk = (gt0(k)) ? flog(arena, k) : __longlong_as_double(0x7ff8000000000000LL);
            double const gs_n = elastic_inverse_stp(C, arena, k, err, lk, species) * density_path(iv, path, sb, se);
            if (gt0(gs_n)) {
                double const few = C.tix.gs_few_collision_threshold;
                if (gs_n < few) {
                    Dir3 const d3 = gs_few_collisions(arena, rng, sub, gs_n, k, lk, dx, dy, dz, species);
                    dx = d3.x; dy = d3.y; dz = d3.z;
                    if (d3.err) err.set(d3.err);
                    if (err.code) break;
                } else {
                    double const ct = sample_gs_cos(C, arena, k, gs_n,
                                                    rng.uniform(sub << 8, POS ? kChPositronGsAngle : kChElectronGsAngle),
                                                    err, lk, species);
                    double nx, ny, nz;
                    cone_direction(dx, dy, dz, ct, rng.uniform(sub << 8, POS ? kChPositronGsAzimuth : kChElectronGsAzimuth),
                                   nx, ny, nz);
                    dx = nx; dy = ny; dz = nz;
                }
            }
        }
        half_kick(sub_field, 0.5 * sub_dt_eff, q, k, dx, dy, dz);
        if (k < cutoff) {
            mark_stopped(se);
            break;
        }
        {
            // RreaAdvanceRunningChargedPosition, O/RreaParticleInteraction.H:368-392
            double x, y, z;
            point_at_full(path, g, se, x, y, z);
            double const wz = wrap_z(g, z);
            if (!cartesian_half_open(g, x, y, wz)) {
                exited = true;
                break;
            }
            run_x = x;
            run_y = y;
            run_z = wz;
        }
        if (path.exits) {
            exited = true;
            break;
        }
        completed = sub + 1U;
    }
    events_out = events;
    if (err.code) return finish(-1);
    if (exited) clipped_escape_policy(path, g, rz_radius(path.ex, path.ey), path.ez, esc, esc_inv);
    if constexpr (POS) {
        // O/RreaPositronTransport.cpp:764-870
        if (annihilated) {
            A.id[ip] = -A.id[ip];
            return finish(2);
        }
        if (exited) return commit_escape();
        if (terminated_mid) return annihilate(mid_x, mid_y, mid_z, mid_r, subcycles, mid_elapsed);
        if (k < cutoff) return annihilate(run_x, run_y, run_z, rz_radius(run_x, run_y), subcycles, 1.0);
        double const um = proper_velocity_from_kinetic(k);
        A.ux[ip] = um * dx;
        A.uy[ip] = um * dy;
        A.uz[ip] = um * dz;
        A.r[ip] = rz_radius(run_x, run_y);
        A.theta[ip] = atan2(run_y, run_x);
        A.z[ip] = run_z;
        put_segment(A.r[ip], run_z);
        return finish(0);
    }
    if (gt0(transported_len)) particle_density = transported_dpath / transported_len;
    double const end_r = rz_radius(run_x, run_y);
    double fer, fez, fbt;
    gather(fv, end_r, run_z, fer, fez, fbt);
    // electron_ensemble_mean_drag_ev_per_m, O/RreaTransportStep.H:226-247
    double threshold = 0.0;
    {
        double const ke = fmax(k, cutoff);
        // The drag threshold only decides the gate when k <= the hard-Moller
        // threshold; above it only its range check can matter, and that is
        // kept.
        if (!charged_in_range(C.tix, ke)) err.set(RREA_GPU_ERR_RANGE);
        if (gt0(ke) && gt0(particle_density) && k <= hm_thr) {
            double const col = rate_value(C, arena, rc, ke, kRateCollision, err);
            double const soft = rate_value(C, arena, rc, ke, kRateSoft, err);
            double const hard = C.hm_enabled ? hard_moller_energy_loss(C, arena, ke, particle_density, err) : 0.0;
            double tracked = 0.0;
            double const inv = rate_value(C, arena, rc, ke, kRateBrems, err) * particle_density;
            if (gt0(inv)) tracked = inv * mean_conditional(arena, C.tix.cdf[RREA_C_BREMS_E], ke, err);
            threshold = (col * particle_density + soft * particle_density) + hard + tracked;
        }
    }
    if (err.code) return finish(-1);
    bool const below_cut = k < cutoff;
    bool const nonrunaway = gt0(hm_thr) && k <= hm_thr && rz_radius(fer, fez) <= threshold;
    if (exited) return commit_escape();
    if (terminated_mid) return demote(mid_r, mid_z);
    if (below_cut || nonrunaway) return demote(end_r, run_z);
    // CommitSurvivorChargedWriteback, O/RreaTransportStep.H:874-905
    double const um = proper_velocity_from_kinetic(k);
    A.ux[ip] = um * dx;
    A.uy[ip] = um * dy;
    A.uz[ip] = um * dz;
    A.r[ip] = end_r;
    A.theta[ip] = atan2(run_y, run_x);
    A.z[ip] = run_z;
    put_segment(end_r, run_z);
    return finish(0);
}

}  // namespace rrea_dev
