// Newborn residual advance on the GPU (O/RreaNewbornAdvance.cpp:20-996):
// every secondary born at elapsed fraction b < 1 is flown through the rest
// (1 - b) dt of its step with the live loops' modules.  The differences from
// the live loops are only the residual dt, the newborn elapsed clock, the
// substep drivers (GS batching and impulse/drag, no optical-depth cap), the
// packed transient RNG index on the ROOT particle's stream, the Newborn* RNG
// channels, and the final-point and ion-pair fallbacks at the half-open
// domain faces.
//
// One FIFO item per thread.  Children go through the transport sinks of
// ElectronArgs: the item's FIFO position plays the parent index and the
// per-item child counter the lineage, so the ordering pass that orders the
// live phases' secondaries also orders each generation of children into
// FIFO order.  Roots and lineages of the children are assigned by the host
// FIFO driver.
#pragma once

#include "rrea_electron.cuh"
#include "rrea_photon.cuh"

namespace rrea_dev {

// RreaTryPackTransientRngIndex (O/RreaParticleInteraction.H:661-690)
__device__ __forceinline__ bool pack_transient(bool newborn, uint64_t species, uint64_t lineage, uint64_t segment,
                                               uint64_t ordinal, uint64_t inner, uint64_t& out)
{
    if (species >= 3U || lineage >= (uint64_t{1} << 14) || segment >= (uint64_t{1} << 14)
        || ordinal >= (uint64_t{1} << 13) || inner >= (uint64_t{1} << 8)) {
        return false;
    }
    out = (static_cast<uint64_t>(newborn) << 51) | (species << 49) | (lineage << 35) | (segment << 21) | (ordinal << 8)
        | inner;
    return true;
}

enum : uint64_t {
    kChNewbornElectronGsAngle = 112, kChNewbornElectronGsAzimuth = 113, kChNewbornElectronGsFewCount = 114,
    kChNewbornElectronGsFewScatter = 115, kChNewbornElectronGsFewAzimuth = 116,
    kChNewbornPositronGsAngle = 117, kChNewbornPositronGsAzimuth = 118, kChNewbornPositronGsFewCount = 119,
    kChNewbornPositronGsFewScatter = 120, kChNewbornPositronGsFewAzimuth = 121,
    kChNewbornCompetingOpticalDepth = 122, kChNewbornCompetingChannel = 123,
};

__device__ __forceinline__ bool in_half_open(Geom const& g, double x, double y, double z)
{
    return cartesian_half_open(g, x, y, z);
}

// TransportStep::NewbornFinalPoint (O/RreaNewbornAdvance.cpp:20-48)
template <int NP>
__device__ __forceinline__ bool newborn_final_point(Path<NP> const& path, Geom const& g, double fraction, double& x,
                                                    double& y, double& z)
{
    double const span = fraction - path.in_begin;
    double pullback = 1.0e-9;
    for (int attempt = 0; attempt < 5; ++attempt) {
        double const trial =
            attempt == 0 ? fraction : fmax(path.in_begin, fraction - pullback * fmax(span, 1.0e-12));
        point_at_full(path, g, trial, x, y, z);  // z wrapped into a periodic domain
        if (in_half_open(g, x, y, z)) return true;
        if (attempt > 0) pullback *= 100.0;
    }
    return false;
}

// RreaEvaluateElectronStatePolicy at a point: below the cutoff, or a
// low-energy non-runaway whose field does not beat the ensemble mean drag
// (O/RreaParticleInteraction.H:1279-1317; O/RreaTransportStep.H:226-247).
__device__ __forceinline__ bool newborn_electron_demotes(StepConstants const& C, ElectronArgs const& A,
                                                         FieldView const& fv, RateCache& rc, double x, double y,
                                                         double z, double e, Err& err)
{
    double const cut = C.cfg.low_energy_cutoff_eV;
    double const thr = C.hm_threshold_eV;
    double fer, fez, fbt;
    gather(fv, rz_radius(x, y), z, fer, fez, fbt);
    double const rho = positive_or(density_ratio_at_z(A.prof, C.cfg.density_ratio, z, err), 1.0);
    double const ke = fmax(e, cut);
    if (!charged_in_range(C.tix, ke)) err.set(RREA_GPU_ERR_RANGE);
    double drag = 0.0;
    // the drag only decides the gate at or below the hard-Moller threshold
    if (gt0(ke) && gt0(rho) && e <= thr) {
        double const col = rate_value(C, A.arena, rc, ke, kRateCollision, err);
        double const soft = rate_value(C, A.arena, rc, ke, kRateSoft, err);
        double const hard = C.hm_enabled ? hard_moller_energy_loss(C, A.arena, ke, rho, err) : 0.0;
        double tracked = 0.0;
        double const inv = rate_value(C, A.arena, rc, ke, kRateBrems, err) * rho;
        if (gt0(inv)) tracked = inv * mean_conditional(A.arena, C.tix.cdf[RREA_C_BREMS_E], ke, err);
        drag = (col * rho + soft * rho) + hard + tracked;
    }
    return e < cut || (gt0(thr) && e <= thr && rz_radius(fer, fez) <= drag);
}

// TransportStep::AdvanceChargedNewborn (O/RreaNewbornAdvance.cpp:50-777).
// Returns 1 when the newborn survives the residual (p updated, birth 1),
// 0 when it ended, -1 on error.
template <int NP, bool POS>
__device__ int advance_charged_newborn(StepConstants const& C, ElectronArgs const& A, int64_t item,
                                       rrea_gpu_secondary& p, uint32_t& lineage, IonPairCache& ion_pairs, Err& err)
{
    const double* __restrict__ arena = A.arena;
    rrea_gpu_config const& cfg = C.cfg;
    Geom const g{cfg.r_lo, cfg.r_hi, cfg.z_lo, cfg.z_hi, cfg.periodic_z != 0};
    constexpr double q = POS ? 1.0 : -1.0;
    constexpr int species = POS ? 1 : 0;
    constexpr int rate_base = POS ? RREA_T_P_COLLISION : RREA_T_E_COLLISION;
    double const cut = cfg.low_energy_cutoff_eV;
    double const thr = C.hm_threshold_eV;
    double const rho = C.density_ratio;
    double const w_air = C.tix.w_air_eV_per_pair;
    double const w = p.weight;
    uint64_t const key = p.root_key;
    // an ensemble instance is the root particle's cpu ordinal (key bits 40+)
    FieldView const fv = A.fv.for_instance(static_cast<int64_t>(key >> 40));
    uint64_t const root_sp = static_cast<uint64_t>(p.root_species);
    uint64_t const nb_lineage = p.lineage;
    double const birth = p.birth_fraction;
    double const birth_r = rz_radius(p.x, p.y), birth_z = p.z;
    double const residual = fmin(1.0, max0(1.0 - birth));
    double k = p.energy_eV;
    RngStream rng;
    rng.init(cfg.rng_seed, key, C.step_key);
    RateCache rc;
    if (!in_half_open(g, p.x, p.y, p.z)) {
        err.set(RREA_GPU_ERR_GEOMETRY);
        return -1;
    }
    double dx = p.dir_x, dy = p.dir_y, dz = p.dir_z;
    normalize(dx, dy, dz);
    auto pack = [&](uint64_t segment, uint64_t ordinal, uint64_t inner) -> uint64_t {
        uint64_t v = 0;
        if (!pack_transient(true, root_sp, nb_lineage, segment, ordinal, inner, v)) err.set(RREA_GPU_ERR_RNG_OVERFLOW);
        return v;
    };
    auto deposit_local = [&](double r, double z, double e) {
        if (le0(w) || le0(e)) return;
        double const pw = w * e / fmax(w_air, 1.0);
        if (le0(pw)) return;
        deposit_source(C, A.cells, 0, r, z, pw, 0.0, w_air);
    };
    auto put_segment = [&](double r1, double z1) {
        if (!A.segments) return;
        SegmentRec& s = A.segments[item];
        s.a[0] = birth_r; s.a[1] = birth_z; s.a[2] = r1; s.a[3] = z1; s.a[4] = q * w;
        s.faces = 0u;
        s.kind = 1;
    };
    auto put_escape = [&](Path<NP> const& path) -> bool {
        double sr, sz, cr, cz;
        uint32_t faces;
        if (!charged_crossing(path, g, sr, sz, cr, cz, faces)) {
            err.set(RREA_GPU_ERR_GEOMETRY);
            return false;
        }
        if (A.segments) {
            SegmentRec& s = A.segments[item];
            s.a[0] = birth_r; s.a[1] = birth_z; s.a[2] = sr; s.a[3] = sz; s.a[4] = cr; s.a[5] = cz; s.a[6] = q * w;
            s.faces = faces;
            s.kind = 2;
        }
        return true;
    };
    auto annihilate = [&](double x, double y, double z, double r, bool at_rest, uint64_t idx, double b) {
        lineage = spawn_annihilation(A, rng, idx, item, key, w, lineage, x, y, z, r, dx, dy, dz, k, at_rest, b);
    };

    // birth state policy (:99-138): no net chord for a birth demotion
    bool const demote_at_birth =
        POS ? k < cut : newborn_electron_demotes(C, A, fv, rc, p.x, p.y, p.z, k, err);
    if (err.code) return -1;
    if (demote_at_birth) {
        double const rb = rz_radius(p.x, p.y);
        if constexpr (POS) {
            uint64_t const idx = pack(0, 0, 0);
            if (err.code) return -1;
            annihilate(p.x, p.y, p.z, rb, true, idx, birth);
        } else {
            deposit_source(C, A.cells, 1, rb, p.z, w, 0.0, 0.0);
            deposit_local(rb, p.z, k);
        }
        return 0;
    }
    if (!(gt0(residual))) return 1;
    double const u = proper_velocity_from_kinetic(k);
    double const gam = sqrt(1.0 + u * u / (kC * kC));
    double const residual_dt = C.dt_s * residual;
    double const chord = (u / gam) * residual_dt;
    if (!(gt0(chord))) return k >= cut ? 1 : 0;
    double const ex0 = p.x + chord * dx, ey0 = p.y + chord * dy, ez0 = p.z + chord * dz;
    Path<NP> path;
    clip_xyz(p.x, p.y, p.z, ex0, ey0, ez0, g, path, err);
    if (err.code) return -1;
    if (!(gt0(path.full)) || !(gt0(path.in_length))) {
        if (path.exits) return put_escape(path) ? 0 : -1;
        return 1;
    }
    Intervals<NP> iv;
    build_intervals(path, g, A.prof, rho, iv, err);
    if (iv.n == 0) {
        err.set(RREA_GPU_ERR_INVALID_STATE);
        return -1;
    }
    double const driver_dpath = density_path(iv, path, path.in_begin, path.in_end);
    double const gs_total = elastic_inverse_stp(C, arena, k, err, __builtin_nan(""), species) * driver_dpath;
    double drag_est;
    if constexpr (POS) {
        drag_est = rate_value(C, arena, rc, k, kRateCollision, err, rate_base) * 1.0 * driver_dpath;
    } else {
        drag_est = (gt0(k) ? rate_value(C, arena, rc, k, kRateCollision, err) * 1.0
                                  + rate_value(C, arena, rc, k, kRateSoft, err) * 1.0
                            : 0.0)
            * driver_dpath;
    }
    double const work = path_field_work(fv, g, path, q, 0.0, 1.0, err).work;
    double const impulse = fmax(cfg.max_field_impulse_fraction * k, fmax(cfg.field_impulse_floor_eV, 1.0));
    double const span = fmax(path.in_end, 1.0e-6);
    uint64_t const gsd = static_cast<uint64_t>(
        fmax(1.0, ceil(fmin(gs_total / span, cfg.gs_total_collision_cap) / fmax(cfg.max_gs_collisions_per_substep, 1.0))));
    uint64_t const imd = static_cast<uint64_t>(fmax(1.0, ceil(((fabs(work) + drag_est) / span) / impulse)));
    uint64_t substeps = gsd > imd ? gsd : imd;
    if (substeps > cfg.max_subcycles) substeps = cfg.max_subcycles;
    if (substeps >= (uint64_t{1} << 14)) err.set(RREA_GPU_ERR_RNG_OVERFLOW);
    if (err.code) return -1;

    double run_x = p.x, run_y = p.y, run_z = p.z;
    double const sub_dt = residual_dt / static_cast<double>(substeps);
    double final_fraction = 0.0;
    bool terminal_interaction = false, terminal_at_point = false, exited = false;
    uint64_t completed = 0;
    FieldRange sub_field{0, 0, 0, 0, 0, 0, 0, 0};
    double sub_dt_eff = 0.0;
    auto elapsed_at = [&](double f) {
        double const within = fmin(1.0, max0(f));
        double const consumed = (static_cast<double>(completed) + within) / static_cast<double>(substeps);
        return fmin(1.0, birth + residual * consumed);
    };
    auto require_certified = [&]() {
        if (!charged_in_range(C.tix, k)) err.set(RREA_GPU_ERR_RANGE);
    };
    // apply_newborn_drag (:260-360)
    auto continuous = [&](double b, double e, double stop_e, double& end_out) -> bool {
        end_out = b;
        if (!(e > b) || !(gt0(k)) || stop_e < cut) return false;
        double const sc = frozen_rate(rate_value(C, arena, rc, stop_e, kRateCollision, err, rate_base) * 1.0, err);
        double const ss = frozen_rate(rate_value(C, arena, rc, stop_e, kRateSoft, err, rate_base) * 1.0, err);
        if (err.code) return false;
        double const total = sc + ss;
        double eff = b;
        bool reaches = false, valid = false;
        if (finite_bits(b) && finite_bits(e) && finite_bits(k) && finite_bits(cut) && e >= b && k >= cut && ge0(cut)) {
            double const to_cut = k - cut;
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
        double const avail = max0(k - cut);
        double const drag = reaches ? avail : fmin(raw_col + raw_soft, avail);
        double const col = fmin(raw_col, drag);
        for (int t = 0; col > 0.0 && gt0(raw_col) && t < iv.n; ++t) {
            double const bb = fmax(b, iv.begin[t]), ee = fmin(eff, iv.end[t]);
            if (ee > bb) {
                double const raw = path.full * (ee - bb) * iv.density[t] * sc;
                double const loss = col * raw / raw_col;
                double const pw = w * loss / fmax(w_air, 1.0);
                if (gt0(pw)) {
                    double x, y, z;
                    point_at_full(path, g, 0.5 * (bb + ee), x, y, z);
                    double sr = rz_radius(x, y), sz = z;
                    // a source that rounds off the half-open domain falls back to the birth point
                    if (!(finite_bits(sr) && finite_bits(sz) && sr >= g.rlo && sr < g.rhi && sz >= g.zlo && sz < g.zhi)) {
                        sr = rz_radius(p.x, p.y);
                        sz = p.z;
                    }
                    // deposit_source(kind 0, sec POS ? 0 : cut/2, loss w_air) through the cache
                    ion_pairs.add(C, A.cells, sr, sz, pw);
                }
            }
        }
        if constexpr (!POS) {
            if (A.n_planes > 0) {
                if (int const code = plane_crossings<NP>(C, A, fv, path, g, iv, b, eff, w, k, total, drag)) {
                    err.set(code);
                }
            }
        }
        k = max0(k - drag);
        if (reaches) k = cut;
        end_out = eff;
        return reaches;
    };
    auto channel_open = [&](int ch, double e) -> bool {
        if (!charged_in_range(C.tix, e)) {
            err.set(RREA_GPU_ERR_RANGE);
            return false;
        }
        if (!rate_bracket(C, arena, rc, e, err, rate_base)) return false;
        if constexpr (POS) {
            if (ch == 0) return !(gt0(thr) && e <= thr) && rate_positive(C, arena, rc, e, kRateBhabha, err, rate_base);
            if (ch == 1) return e > C.photon_cutoff_eV && rate_positive(C, arena, rc, e, kRateBrems, err, rate_base);
            if (ch == 2) return rate_positive(C, arena, rc, e, kRateAnnihilation, err, rate_base);
            return false;
        } else {
            if (ch == 0) {
                return C.hm_enabled && (gt0(thr) && e > 2.0 * thr) && rate_positive(C, arena, rc, e, kRateMoller, err);
            }
            if (ch == 1) {
                return (finite_bits(e) && finite_bits(C.photon_cutoff_eV) && e > C.photon_cutoff_eV)
                    && rate_positive(C, arena, rc, e, kRateBrems, err);
            }
            return false;
        }
    };

    for (uint64_t sub = 0; sub < substeps; ++sub) {
        if (k < cut) break;
        double sb, se;
        {
            // RreaBuildRunningChargedChord with the residual dt as the step bound
            double const speed = charged_speed(k);
            double const dn = sqrt(dx * dx + dy * dy + dz * dz);
            if (!finite_bits(sub_dt) || !(ge0(sub_dt)) || !finite_bits(speed) || !finite_bits(dn) || !(gt0(dn))) break;
            double const sc = speed * sub_dt / dn;
            double const exx = run_x + sc * dx, eyy = run_y + sc * dy, ezz = run_z + sc * dz;
            Path<NP> np;
            clip_xyz(run_x, run_y, run_z, exx, eyy, ezz, g, np, err);
            if (err.code) break;
            if (!(finite_bits(np.full) && eq0(np.in_begin))) break;
            path = np;
            if (!(gt0(path.full)) || !(gt0(path.in_length))) {
                exited = path.exits;
                final_fraction = 0.0;
                break;
            }
            build_intervals(path, g, A.prof, rho, iv, err);
            if (iv.n == 0) {
                err.set(RREA_GPU_ERR_INVALID_STATE);
                break;
            }
            sb = path.in_begin;
            se = path.in_end;
            final_fraction = se;
            sub_field = path_field_work(fv, g, path, q, sb, se, err);
            sub_dt_eff = sub_dt * (se - sb);
            half_kick(sub_field, 0.5 * sub_dt_eff, q, k, dx, dy, dz);
            if (k < cut) {
                final_fraction = sb;
                terminal_at_point = true;
                break;
            }
            require_certified();
            if (err.code) break;
        }
        {
            double rem = sb;
            uint64_t ordinal = 0;
            while (rem < se && k >= cut) {
                if (err.code) break;
                if (ordinal >= kEventCap) {
                    err.set(RREA_GPU_ERR_RNG_OVERFLOW);
                    break;
                }
                double const frozen = k;
                double s0, s1, s2 = 0.0;
                if constexpr (POS) competing_rates_positron(C, arena, rc, frozen, s0, s1, s2, err);
                else competing_rates(C, arena, rc, frozen, s0, s1, err);
                double const total_stp = (s0 + s1) + s2;
                double const seg_dp = density_path(iv, path, rem, se);
                uint64_t const idx = pack(sub, ordinal, 0);
                if (err.code) break;
                double const u1 = rng.uniform(idx, kChNewbornCompetingOpticalDepth);
                double const u2 = rng.uniform(idx, kChNewbornCompetingChannel);
                Selection const selv = select_hazard(arena, s0 * seg_dp, s1 * seg_dp, s2 * seg_dp, POS ? 3 : 2, u1, u2);
                if (!selv.valid) {
                    err.set(RREA_GPU_ERR_INVALID_STATE);
                    break;
                }
                if (!selv.event) {
                    double eff;
                    if (continuous(rem, se, frozen, eff)) {
                        final_fraction = eff;
                        terminal_at_point = true;
                    }
                    break;
                }
                double const ev = fraction_at_density_path(iv, path, rem, se, selv.sampled / total_stp, err);
                if (!(finite_bits(rem) && finite_bits(ev) && finite_bits(se) && se > rem && !(ev < rem) && !(ev > se))) {
                    err.set(RREA_GPU_ERR_INVALID_STATE);
                    break;
                }
                double ex, ey, ez;
                point_at_full(path, g, ev, ex, ey, ez);
                double const er = rz_radius(ex, ey);
                double const ev_elapsed = elapsed_at(ev);
                {
                    double eff;
                    if (continuous(rem, ev, frozen, eff)) {
                        final_fraction = eff;
                        terminal_at_point = true;
                        break;
                    }
                }
                bool const open_ev = k >= cut && channel_open(selv.channel, k);
                if (!open_ev) {
                    bool const open_fr = frozen >= cut && channel_open(selv.channel, frozen);
                    if (!open_fr) {
                        err.set(RREA_GPU_ERR_INVALID_STATE);
                        break;
                    }
                    rem = ev;
                    ++ordinal;
                    continue;
                }
                Site const site{ex, ey, ez, er, ev_elapsed};
                if constexpr (POS) {
                    if (selv.channel == 0) {
                        bhabha_final_state(C, A, rng, idx, item, key, w, site, k, dx, dy, dz, lineage, err);
                    } else if (selv.channel == 1) {
                        brems_final_state<true>(C, A, rng, idx, item, key, w, site, k, dx, dy, dz, lineage, err);
                    } else {
                        annihilate(ex, ey, ez, er, false, idx, ev_elapsed);
                        put_segment(er, ez);
                        terminal_interaction = true;
                        final_fraction = ev;
                        break;
                    }
                } else {
                    if (selv.channel == 0) {
                        moller_final_state(C, A, rng, idx, item, key, w, site, k, dx, dy, dz, lineage, err);
                    } else if (selv.channel == 1) {
                        brems_final_state(C, A, rng, idx, item, key, w, site, k, dx, dy, dz, lineage, err);
                    }
                }
                if (err.code) break;
                if (k <= cut) {
                    final_fraction = ev;
                    terminal_at_point = true;
                    break;
                }
                rem = ev;
                ++ordinal;
            }
        }
        if (err.code || terminal_interaction || terminal_at_point) break;
        if (k >= cut) {
            double const lk = (gt0(k)) ? flog(arena, k) : __longlong_as_double(0x7ff8000000000000LL);
            double const gs_n = elastic_inverse_stp(C, arena, k, err, lk, species) * density_path(iv, path, sb, se);
            if (gt0(gs_n)) {
                double const few = C.tix.gs_few_collision_threshold;
                if (gs_n < few) {
                    int const cap = static_cast<int>(ceil(3.0 * few));
                    if (cap >= 255) {
                        err.set(RREA_GPU_ERR_INVALID_STATE);
                        break;
                    }
                    uint64_t const i0 = pack(sub, 0, 0);
                    int const cnt = poisson_capped(
                        gs_n, rng.uniform(i0, POS ? kChNewbornPositronGsFewCount : kChNewbornElectronGsFewCount), cap);
                    for (int qq = 0; qq < cnt; ++qq) {
                        uint64_t const ii = pack(sub, 0, static_cast<uint64_t>(qq + 1));
                        double const ct = sample_single_elastic_cos(
                            C, arena, k,
                            rng.uniform(ii, POS ? kChNewbornPositronGsFewScatter : kChNewbornElectronGsFewScatter), err,
                            lk, species);
                        double nx, ny, nz;
                        cone_direction(dx, dy, dz, ct,
                                       rng.uniform(ii, POS ? kChNewbornPositronGsFewAzimuth
                                                           : kChNewbornElectronGsFewAzimuth),
                                       nx, ny, nz);
                        dx = nx; dy = ny; dz = nz;
                    }
                } else {
                    uint64_t const i0 = pack(sub, 0, 0);
                    double const ct = sample_gs_cos(
                        C, arena, k, gs_n, rng.uniform(i0, POS ? kChNewbornPositronGsAngle : kChNewbornElectronGsAngle),
                        err, lk, species);
                    double nx, ny, nz;
                    cone_direction(dx, dy, dz, ct,
                                   rng.uniform(i0, POS ? kChNewbornPositronGsAzimuth : kChNewbornElectronGsAzimuth), nx,
                                   ny, nz);
                    dx = nx; dy = ny; dz = nz;
                }
            }
        }
        if (err.code) break;
        half_kick(sub_field, 0.5 * sub_dt_eff, q, k, dx, dy, dz);
        if (k < cut) {
            final_fraction = se;
            terminal_at_point = true;
            break;
        }
        require_certified();
        if (err.code) break;
        {
            double x, y, z;
            point_at_full(path, g, se, x, y, z);
            if (!in_half_open(g, x, y, z)) {
                exited = true;
                break;
            }
            run_x = x;
            run_y = y;
            run_z = z;
        }
        if (path.exits) {
            exited = true;
            break;
        }
        completed = sub + 1U;
    }
    if (err.code) return -1;
    if (terminal_interaction) return 0;
    double fx, fy, fz;
    if (!newborn_final_point(path, g, final_fraction, fx, fy, fz)) {
        err.set(RREA_GPU_ERR_GEOMETRY);
        return -1;
    }
    double const final_r = rz_radius(fx, fy);
    double const final_elapsed = elapsed_at(final_fraction);
    bool const demote = POS ? k < cut : newborn_electron_demotes(C, A, fv, rc, fx, fy, fz, k, err);
    if (err.code) return -1;
    if (terminal_at_point || demote) {
        if constexpr (POS) {
            uint64_t const seg = substeps < (uint64_t{1} << 14) - 1U ? substeps : (uint64_t{1} << 14) - 1U;
            uint64_t const idx = pack(seg, 0, 0);
            if (err.code) return -1;
            annihilate(fx, fy, fz, final_r, true, idx, final_elapsed);
        } else {
            deposit_source(C, A.cells, 1, final_r, fz, w, 0.0, 0.0);
            deposit_local(final_r, fz, k);
        }
        put_segment(final_r, fz);
        return 0;
    }
    if (exited) return put_escape(path) ? 0 : -1;
    p.x = fx;
    p.y = fy;
    p.z = fz;
    p.dir_x = dx;
    p.dir_y = dy;
    p.dir_z = dz;
    p.energy_eV = k;
    p.birth_fraction = 1.0;
    put_segment(final_r, fz);
    return 1;
}

// TransportStep::AdvancePhotonNewborn (O/RreaNewbornAdvance.cpp:779-996)
template <int NP>
__device__ int advance_photon_newborn(StepConstants const& C, ElectronArgs const& A, int64_t item,
                                      rrea_gpu_secondary& p, uint32_t& lineage, Err& err)
{
    const double* __restrict__ arena = A.arena;
    rrea_gpu_config const& cfg = C.cfg;
    Geom const g{cfg.r_lo, cfg.r_hi, cfg.z_lo, cfg.z_hi, cfg.periodic_z != 0};
    double const cut = cfg.low_energy_cutoff_eV;
    double const photon_cut = C.photon_cutoff_eV;
    double const rho = C.density_ratio;
    double const w_air = C.tix.w_air_eV_per_pair;
    double const w = p.weight;
    uint64_t const key = p.root_key;
    double const residual = fmin(1.0, max0(1.0 - p.birth_fraction));
    if (!(gt0(residual))) return p.energy_eV >= photon_cut ? 1 : 0;
    if (!in_half_open(g, p.x, p.y, p.z)) {
        err.set(RREA_GPU_ERR_GEOMETRY);
        return -1;
    }
    RngStream rng;
    rng.init(cfg.rng_seed, key, C.step_key);
    double dx = p.dir_x, dy = p.dir_y, dz = p.dir_z;
    normalize(dx, dy, dz);
    double energy = p.energy_eV;
    auto deposit_local = [&](double r, double z, double e) {
        if (le0(w) || le0(e)) return;
        double const pw = w * e / fmax(w_air, 1.0);
        if (le0(pw)) return;
        deposit_source(C, A.cells, 0, r, z, pw, 0.0, w_air);
    };
    auto child = [&](int sp, int process, double x, double y, double z, double sx, double sy, double sz, double e,
                     double b) {
        append_secondary(A, item, key, w, lineage, sp, process, x, y, z, sx, sy, sz, e, b, err, p.root_species);
    };
    if (energy < photon_cut) {
        deposit_local(rz_radius(p.x, p.y), p.z, energy);
        return 0;
    }
    double const chord = kC * C.dt_s * residual;
    double const ex0 = p.x + chord * dx, ey0 = p.y + chord * dy, ez0 = p.z + chord * dz;
    Path<NP> path;
    clip_xyz(p.x, p.y, p.z, ex0, ey0, ez0, g, path, err);
    if (err.code) return -1;
    if (!(gt0(path.full)) || !(gt0(path.in_length))) return path.exits ? 0 : 1;
    double elapsed_start = p.birth_fraction;
    for (uint64_t ordinal = 0;; ++ordinal) {
        uint64_t idx;
        if (!pack_transient(true, static_cast<uint64_t>(p.root_species), p.lineage, 0, ordinal, 0, idx)) {
            err.set(RREA_GPU_ERR_RNG_OVERFLOW);
            return -1;
        }
        Intervals<NP> iv;
        build_intervals(path, g, A.prof, rho, iv, err);
        PhotonRates rates;
        if (!photon_rates(C, arena, energy, rates, err)) return -1;
        double const mfp = mfp_from_inverse(rates.total(), err);
        double const tau = density_path(iv, path, path.in_begin, path.in_end) / mfp;
        Selection const sel =
            select_hazard(arena, tau, 0.0, 0.0, 1, rng.uniform(idx, kChNewbornCompetingOpticalDepth), 0.0);
        if (!sel.valid) {
            err.set(RREA_GPU_ERR_INVALID_STATE);
            return -1;
        }
        if (!sel.event) {
            double fx, fy, fz;
            if (!newborn_final_point(path, g, path.in_end, fx, fy, fz)) {
                err.set(RREA_GPU_ERR_GEOMETRY);
                return -1;
            }
            if (path.exits) return 0;
            p.x = fx; p.y = fy; p.z = fz;
            p.dir_x = dx; p.dir_y = dy; p.dir_z = dz;
            p.energy_eV = energy;
            p.birth_fraction = 1.0;
            return 1;
        }
        double const f = fraction_at_density_path(iv, path, path.in_begin, path.in_end, sel.sampled * mfp, err);
        if (!(finite_bits(f) && f >= path.in_begin && f <= path.in_end && path.in_end > path.in_begin)) {
            err.set(RREA_GPU_ERR_INVALID_STATE);
            return -1;
        }
        double const dist = path.full * (f - path.in_begin);
        double const remaining = max0(path.full - dist);
        double px, py, pz;
        point_at_full(path, g, f, px, py, pz);
        double const pr = rz_radius(px, py);
        double const b = fmin(1.0, elapsed_start + dist / fmax(kC * C.dt_s, kDblMin));
        int const channel = sample_photon_channel(rates, rng.uniform(idx, kChNewbornCompetingChannel), err);
        if (err.code) return -1;
        if (channel == 0) {
            double const inc = energy;
            ComptonState const cs =
                sample_klein_nishina(inc, rng.uniform(idx, kChComptonMu), rng.uniform(idx, kChComptonAccept));
            double sx, sy, sz;
            cone_direction(dx, dy, dz, cs.cos_theta, rng.uniform(idx, kChComptonAzimuth), sx, sy, sz);
            double rx = inc * dx - cs.scattered * sx, ry = inc * dy - cs.scattered * sy, rz = inc * dz - cs.scattered * sz;
            normalize(rx, ry, rz);
            if (cs.recoil >= cut) {
                child(0, 5, px, py, pz, rx, ry, rz, cs.recoil, b);
                deposit_source(C, A.cells, 0, pr, pz, w, cs.recoil, cs.recoil);
            } else {
                deposit_source(C, A.cells, 0, pr, pz, w, cs.recoil, 0.0);
                deposit_local(pr, pz, cs.recoil);
            }
            if (!compton_flow_valid(w, inc, cs.recoil, cs.scattered)) {
                err.set(RREA_GPU_ERR_INVALID_STATE);
                return -1;
            }
            energy = cs.scattered;
            {
                // closure of the Compton group
                bool const survives = energy >= photon_cut;
                GroupClosure gc;
                gc.begin(0.0, 0.0, w, inc, survives ? energy : 0.0, survives);
                if (cs.recoil >= cut) gc.secondary(-1.0, kMeC2, w, cs.recoil);
                gc.ionization(w, cs.recoil, cut);
                if (cs.recoil < cut) gc.local(w, cs.recoil, w_air, cut);
                if (!survives) gc.local(w, energy, w_air, cut);
                if (!gc.valid(cut)) {
                    err.set(RREA_GPU_ERR_INVALID_STATE);
                    return -1;
                }
            }
            if (energy < photon_cut) {
                deposit_local(pr, pz, energy);
                return 0;
            }
            dx = sx; dy = sy; dz = sz;
            if (!(gt0(remaining))) {
                p.x = px; p.y = py; p.z = pz;
                p.dir_x = dx; p.dir_y = dy; p.dir_z = dz;
                p.energy_eV = energy;
                p.birth_fraction = 1.0;
                return 1;
            }
            double const tx = px + remaining * dx, ty = py + remaining * dy, tz = pz + remaining * dz;
            clip_xyz(px, py, pz, tx, ty, tz, g, path, err);
            if (err.code) return -1;
            elapsed_start = b;
            continue;
        }
        if (channel == 1) {
            double pe_e, bind;
            sample_photoelectric(C, arena, energy, rng.uniform(idx, kChPhotoelectricShell), pe_e, bind, err);
            if (err.code) return -1;
            double const ee = fmin(pe_e, energy);
            if (ee >= cut) {
                if (!charged_in_range(C.tix, ee)) {
                    err.set(RREA_GPU_ERR_RANGE);
                    return -1;
                }
                double const cth = sample_photoelectron_cos(ee, rng.uniform(idx, kChPhotoelectronCos));
                double sx, sy, sz;
                cone_direction(dx, dy, dz, cth, rng.uniform(idx, kChPhotoelectronAzimuth), sx, sy, sz);
                child(0, 6, px, py, pz, sx, sy, sz, ee, b);
                deposit_source(C, A.cells, 0, pr, pz, w, ee, ee);
            } else {
                deposit_source(C, A.cells, 0, pr, pz, w, ee, 0.0);
                deposit_local(pr, pz, ee);
            }
            if (gt0(bind)) deposit_local(pr, pz, bind);
            if (!photoelectric_flow_valid(w, energy, ee, fmax(bind, 0.0))) {
                err.set(RREA_GPU_ERR_INVALID_STATE);
                return -1;
            }
            GroupClosure gc;  // closure of the Photoelectric group
            gc.begin(0.0, 0.0, w, energy, 0.0, false);
            if (ee >= cut) gc.secondary(-1.0, kMeC2, w, ee);
            gc.ionization(w, ee, cut);
            if (ee < cut) gc.local(w, ee, w_air, cut);
            if (gt0(bind)) gc.local(w, bind, w_air, cut);
            if (!gc.valid(cut)) {
                err.set(RREA_GPU_ERR_INVALID_STATE);
                return -1;
            }
            return 0;
        }
        bool const triplet = channel == 3;
        int const proc = triplet ? 8 : 7;
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
        if (ps.e_electron >= cut) {
            child(0, proc, px, py, pz, edx, edy, edz, ps.e_electron, b);
        } else {
            deposit_source(C, A.cells, 1, pr, pz, w, 0.0, 0.0);
            deposit_local(pr, pz, ps.e_electron);
        }
        if (ps.e_positron >= cut) {
            child(1, proc, px, py, pz, pdx, pdy, pdz, ps.e_positron, b);
        } else {
            lineage = spawn_annihilation(A, rng, idx, item, key, w, lineage, px, py, pz, pr, pdx, pdy, pdz,
                                         ps.e_positron, true, b);
        }
        if (ps.recoil) {
            double rdx, rdy, rdz;
            rotate_to_axis(dx, dy, dz, ps.rdir[0], ps.rdir[1], ps.rdir[2], rdx, rdy, rdz);
            if (ps.e_recoil >= cut) child(0, proc, px, py, pz, rdx, rdy, rdz, ps.e_recoil, b);
            deposit_source(C, A.cells, 0, pr, pz, w, ps.e_recoil, 0.0);
            if (ps.e_recoil < cut) deposit_local(pr, pz, ps.e_recoil);
        }
        if (gt0(ps.local)) deposit_local(pr, pz, ps.local);
        if (!pair_flow_valid(w, energy, ps.e_electron, ps.e_positron, ps.e_recoil, ps.recoil, ps.local)
            || !pair_closure_valid(ps, w, energy, cut, photon_cut, w_air)) {
            err.set(RREA_GPU_ERR_INVALID_STATE);
            return -1;
        }
        return 0;
    }
}

}  // namespace rrea_dev
