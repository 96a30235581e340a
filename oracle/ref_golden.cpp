// Golden-vector generator built from the REFERENCE's own sources (compiled
// in place under the reference checkout against oracle/ref_shim) by
// oracle/Makefile.ref into oracle/_ref/ref_golden.  It evaluates the
// reference's primitives on seeded inputs and writes inputs and outputs as
// .npy fixtures under tests/golden/.  Those fixtures pin the oracle
// restatement (oracle/oracle_core.cpp) and the device kernels to the
// reference's arithmetic.  Test infrastructure only.
#include "RreaChargedInterleave.H"
#include "interleave_scenarios.hpp"
#include "RreaParticleInteraction.H"
#include "RreaRng.H"
#include "rrea/RreaAltitudeProfile.H"
#include "rrea/RreaCicConservingResample.H"
#include "rrea/RreaInteractionTables.H"
#include "rrea/RreaConstants.H"
#include "rrea/RreaMaxwellTMRZ.H"
#include "rrea/RreaPlaneFlux.H"
#include "rrea/RreaSeedSchedule.H"
#include "rrea/RreaSegmentDepositionRZ.H"
#include "rrea/RreaTransportPath.H"

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <limits>
#include <stdexcept>
#include <string>
#include <vector>

namespace {

std::string g_outdir;

struct Gen {
    uint64_t s;
    explicit Gen(uint64_t seed) : s(seed) {}
    uint64_t next()
    {
        uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
        return z ^ (z >> 31);
    }
    double uni() { return (static_cast<double>(next() >> 11) + 0.5) * 0x1.0p-53; }
    double logu(double lo, double hi) { return std::exp(std::log(lo) + uni() * (std::log(hi) - std::log(lo))); }
};

void write_npy(std::string const& name, char const* descr, std::size_t rows, std::size_t cols,
               void const* data, std::size_t item)
{
    std::string path = g_outdir + "/" + name + ".npy";
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) throw std::runtime_error("cannot write " + path);
    char header[256];
    int const hl = std::snprintf(header, sizeof(header),
                                 "{'descr': '%s', 'fortran_order': False, 'shape': (%zu, %zu), }", descr, rows, cols);
    std::string h(header, static_cast<std::size_t>(hl));
    std::size_t total = 10 + h.size() + 1;
    std::size_t pad = (64 - total % 64) % 64;
    h.append(pad, ' ');
    h.push_back('\n');
    unsigned char magic[8] = {0x93, 'N', 'U', 'M', 'P', 'Y', 1, 0};
    std::fwrite(magic, 1, 8, f);
    uint16_t const len = static_cast<uint16_t>(h.size());
    std::fwrite(&len, 2, 1, f);
    std::fwrite(h.data(), 1, h.size(), f);
    std::fwrite(data, item, rows * cols, f);
    std::fclose(f);
}
void write_f8(std::string const& name, std::size_t cols, std::vector<double> const& v)
{
    write_npy(name, "<f8", v.size() / cols, cols, v.data(), 8);
}
void write_u8(std::string const& name, std::size_t cols, std::vector<uint64_t> const& v)
{
    write_npy(name, "<u8", v.size() / cols, cols, v.data(), 8);
}

// Energies that exercise node-exact, ulp-adjacent, threshold and random queries.
std::vector<double> charged_energies(Gen& g, rrea::RreaInteractionTables const& t, int n_random)
{
    std::vector<double> e;
    double const special[] = {1.0e3, 1.0e4, 5.0e4, 1.0e5, 7.2e6, 1.0e8, 1.0e10};
    for (double s : special) {
        e.push_back(s);
        if (s > 1.0e3) e.push_back(std::nextafter(s, 0.0));
        if (s < 1.0e10) e.push_back(std::nextafter(s, 1.0e11));
    }
    e.push_back(2.0 * t.HardMollerSecondaryThresholdEv());
    e.push_back(std::nextafter(2.0 * t.HardMollerSecondaryThresholdEv(), 1.0e11));
    for (int i = 0; i < n_random; ++i) e.push_back(g.logu(1.0e3, 1.0e10));
    return e;
}

// The reference's own charged-loop skeletons behind the scenario runner.
struct RefSkeleton {
    template <class... P>
    static void events(double b, double e, double& k, double cut, int channels, uint64_t max_ordinal, P&&... p)
    {
        rrea::warpx::RreaRunChargedEventInterleave(b, e, k, cut, channels, max_ordinal, "scenario",
                                                   std::forward<P>(p)...);
    }
    template <class... P>
    static void substeps(uint64_t n, double& k, double cut, uint64_t& completed, bool& exited, P&&... p)
    {
        rrea::warpx::RreaRunChargedSubstepInterleave(n, k, cut, completed, exited, std::forward<P>(p)...);
    }
};

}  // namespace

int main(int argc, char** argv)
{
    if (argc < 3) {
        std::fprintf(stderr, "usage: ref_golden <transport_physics.json> <outdir>\n");
        return 2;
    }
    g_outdir = argv[2];
    try {
        rrea::RreaInteractionTables tables;
        tables.Load(argv[1]);
        Gen g(20261203ULL);

        // ---- RNG: O/RreaRng.cpp
        {
            std::vector<uint64_t> rows;
            for (int i = 0; i < 2048; ++i) {
                rrea::warpx::RreaRngKey k{g.next(), g.next() >> (i % 40), g.next() % 100000, g.next() >> 12,
                                          g.next() % 140};
                rows.insert(rows.end(), {k.seed, k.particle_id, k.step, k.interaction_index, k.channel_id,
                                         rrea::warpx::RreaRng::Counter(k)});
                double const u = rrea::warpx::RreaRng::Uniform01(k);
                uint64_t ub;
                std::memcpy(&ub, &u, 8);
                rows.push_back(ub);
            }
            write_u8("ref_rng", 7, rows);
        }

        // ---- hot 1-D tables: RreaInteractionTable::Interpolate via ProbeTableValue
        {
            char const* names[15] = {
                "electron_collision_stopping_air", "electron_soft_radiative_stopping_air",
                "electron_hard_moller_inverse_length_air", "electron_tracked_brems_inverse_length_air",
                "electron_elastic_transport_inverse_length_air", "positron_collision_stopping_air",
                "positron_soft_radiative_stopping_air", "positron_hard_bhabha_inverse_length_air",
                "positron_tracked_brems_inverse_length_air", "positron_elastic_transport_inverse_length_air",
                "positron_annihilation_inverse_length_air", "photon_compton_inverse_length_air",
                "photon_photoelectric_inverse_length_air", "photon_pair_nuclear_inverse_length_air",
                "photon_pair_triplet_inverse_length_air"};
            std::vector<double> rows;
            for (int t = 0; t < 15; ++t) {
                bool const photon = t >= 11;
                double const lo = photon ? 1.0e3 : 1.0e3, hi = photon ? 1.0e11 : 1.0e10;
                std::vector<double> es;
                if (photon) {
                    for (int i = 0; i < 400; ++i) es.push_back(g.logu(lo, hi));
                    double const edges[] = {1.0e3, 1.0e11, 1022000.0, 1021997.9, 2043995.8};
                    for (double x : edges) es.push_back(x);
                } else {
                    es = charged_energies(g, tables, 400);
                }
                for (double e : es) {
                    if (e < lo || e > hi) continue;
                    rows.insert(rows.end(), {static_cast<double>(t), e, tables.ProbeTableValue(names[t], e)});
                }
            }
            write_f8("ref_interp", 3, rows);
        }

        // ---- electron accessors used by the transport loop
        {
            std::vector<double> rows;
            for (double e : charged_energies(g, tables, 1500)) {
                double const dr = (g.uni() < 0.5) ? 1.0 : 0.5 + 1.5 * g.uni();
                rows.insert(rows.end(),
                            {e, dr, tables.ElectronCollisionLoss(e, dr), tables.ElectronSoftRadiativeDrag(e, dr),
                             tables.ElectronHardMollerMeanFreePath(e, dr),
                             tables.ElectronBremsstrahlungMeanFreePath(e, dr),
                             tables.ElectronHardMollerEnergyLoss(e, dr), tables.ElectronTrackedBremsEnergyLoss(e, dr),
                             tables.ElasticMeanFreePath(false, e, dr), tables.ScreeningEta(false, e),
                             tables.ElasticMeanFreePath(true, e, dr), tables.ScreeningEta(true, e)});
            }
            write_f8("ref_electron_accessors", 12, rows);
        }

        // ---- samplers
        {
            std::vector<double> gs;
            for (int i = 0; i < 3000; ++i) {
                int const sp = i % 2;
                double const e = (i % 7 == 0) ? g.logu(5.0e7, 1.0e10) : g.logu(1.0e3, 1.0e10);
                double const n = (i % 11 == 0) ? g.logu(1.0e5, 1.0e7) : g.logu(10.0, 1.0e5);
                double const u = (i % 13 == 0) ? g.uni() * 1.0e-4 : g.uni();
                gs.insert(gs.end(), {static_cast<double>(sp), e, n, u,
                                     tables.SampleGsCosTheta(sp == 1, e, n, u)});
            }
            write_f8("ref_gs_angle", 5, gs);

            std::vector<double> single;
            for (int i = 0; i < 1000; ++i) {
                int const sp = i % 2;
                double const e = g.logu(1.0e3, 1.0e10), u = g.uni();
                single.insert(single.end(), {static_cast<double>(sp), e, u,
                                             tables.SampleSingleElasticCosTheta(sp == 1, e, u)});
            }
            write_f8("ref_single_elastic", 4, single);

            std::vector<double> moller, brems, tsai;
            for (int i = 0; i < 3000; ++i) {
                double const em = (i % 17 == 0) ? std::nextafter(1.0e5, 1.0e11) : g.logu(1.000001e5, 1.0e10);
                double const u = (i % 19 == 0) ? (i % 38 == 0 ? 0.0 : 1.0) : g.uni();
                moller.insert(moller.end(), {em, u, tables.SampleMollerSecondaryEnergy(em, u)});
                double const eb = g.logu(5.0001e4, 1.0e10);
                brems.insert(brems.end(), {eb, u, tables.SampleBremsstrahlungPhotonEnergy(eb, u)});
                double const et = g.logu(1.0e3, 1.0e10);
                tsai.insert(tsai.end(), {et, u, tables.SampleBremsstrahlungCosTheta(et, u)});
            }
            write_f8("ref_moller_energy", 3, moller);
            write_f8("ref_brems_energy", 3, brems);
            write_f8("ref_brems_angle", 3, tsai);
        }

        // ---- kinematics: O/RreaChargedInterleave.H, I/RreaLorentzPush.H
        {
            using namespace rrea::warpx;
            std::vector<double> kick;
            for (int i = 0; i < 2000; ++i) {
                RreaPathFieldSubRange f;
                f.work_eV = (g.uni() - 0.5) * 2.0e5;
                f.avg_ex_v_per_m = (g.uni() - 0.5) * 1.0e6;
                f.avg_ey_v_per_m = (g.uni() - 0.5) * 1.0e6;
                f.avg_ez_v_per_m = (g.uni() - 0.5) * 1.0e6;
                double const bs = (i % 3 == 0) ? 0.0 : 1.0e-3;
                f.avg_bx_t = (g.uni() - 0.5) * bs;
                f.avg_by_t = (g.uni() - 0.5) * bs;
                f.avg_bz_t = (g.uni() - 0.5) * bs;
                double const half_dt = g.logu(1.0e-13, 1.0e-9);
                double const q = (i % 2) ? 1.0 : -1.0;
                double k = g.logu(1.0e3, 1.0e9);
                double dx = g.uni() - 0.5, dy = g.uni() - 0.5, dz = g.uni() - 0.5;
                RreaNormalizeDirection(dx, dy, dz);
                std::vector<double> in = {f.work_eV, f.avg_ex_v_per_m, f.avg_ey_v_per_m, f.avg_ez_v_per_m,
                                          f.avg_bx_t, f.avg_by_t, f.avg_bz_t, half_dt, q, k, dx, dy, dz};
                (void)RreaApplyChargedFieldHalfKick(f, half_dt, q, k, dx, dy, dz);
                kick.insert(kick.end(), in.begin(), in.end());
                kick.insert(kick.end(), {k, dx, dy, dz});
            }
            write_f8("ref_half_kick", 17, kick);

            std::vector<double> cone, mol, rec, poi;
            for (int i = 0; i < 2000; ++i) {
                double ax = g.uni() - 0.5, ay = g.uni() - 0.5, az = (i % 5 == 0) ? 0.95 : g.uni() - 0.5;
                double const ct = 2.0 * g.uni() - 1.0, uphi = g.uni();
                double ox, oy, oz;
                RreaSampleConeDirection(ax, ay, az, ct, uphi, ox, oy, oz);
                cone.insert(cone.end(), {ax, ay, az, ct, uphi, ox, oy, oz});

                double const kp = g.logu(1.0e5, 1.0e9), ks = kp * 0.5 * g.uni(), ua = g.uni();
                double p1, p2, p3, s1, s2, s3;
                RreaSampleMollerLabDirections(ax, ay, az, kp, ks, ua, p1, p2, p3, s1, s2, s3);
                mol.insert(mol.end(), {ax, ay, az, kp, ks, ua, p1, p2, p3, s1, s2, s3});

                double cx = ax, cy = ay, cz = az;
                RreaNormalizeDirection(cx, cy, cz);
                double const k0 = g.logu(5.0e4, 1.0e9), eg = k0 * g.uni();
                double gx = g.uni() - 0.5, gy = g.uni() - 0.5, gz = g.uni() - 0.5;
                std::vector<double> in = {k0, eg, gx, gy, gz, cx, cy, cz};
                RreaApplyPhotonRecoilToChargedDirection(k0, eg, gx, gy, gz, cx, cy, cz);
                rec.insert(rec.end(), in.begin(), in.end());
                rec.insert(rec.end(), {cx, cy, cz});

                double const mean = 10.0 * g.uni(), up = g.uni();
                poi.insert(poi.end(), {mean, up, static_cast<double>(RreaPoissonSampleCapped(mean, up, 30))});
            }
            write_f8("ref_cone", 8, cone);
            write_f8("ref_moller_dirs", 12, mol);
            write_f8("ref_photon_recoil", 11, rec);
            write_f8("ref_poisson", 3, poi);

            std::vector<double> haz;
            for (int i = 0; i < 2000; ++i) {
                std::array<double, 3> taus = {g.uni() * 0.05, (i % 4 == 0) ? 0.0 : g.uni() * 0.05,
                                              (i % 3 == 0) ? g.uni() * 0.01 : 0.0};
                int const cnt = 2 + (i % 2);
                double const u1 = (i % 50 == 0) ? 0.999999 : g.uni(), u2 = (i % 37 == 0) ? 1.0 : g.uni();
                auto const s = RreaSelectCompetingHazard(taus, cnt, u1, u2);
                haz.insert(haz.end(), {taus[0], taus[1], taus[2], static_cast<double>(cnt), u1, u2,
                                       static_cast<double>(s.valid), static_cast<double>(s.event),
                                       static_cast<double>(s.channel), s.sampled_optical_depth,
                                       s.total_optical_depth});
            }
            write_f8("ref_hazard", 11, haz);

            std::vector<double> drag;
            for (int i = 0; i < 2000; ++i) {
                double const b = 0.3 * g.uni(), e = b + (1.0 - b) * g.uni();
                double const cut = 1.0e4, k = cut + g.logu(1.0, 1.0e7);
                double const stop = (i % 9 == 0) ? 0.5 * cut : k;
                double const col = g.logu(1.0e2, 1.0e6), soft = (i % 2) ? 0.0 : g.logu(1.0, 1.0e4),
                             hard = g.logu(1.0, 1.0e3);
                double const len = g.logu(1.0e-3, 100.0), rho = 0.5 + g.uni();
                auto plan = RreaPlanContinuousDragSegment(
                    b, e, k, stop, cut, [&](double bb, double ee) { return len * (ee - bb) * rho; },
                    [&] { return RreaFrozenStoppingPowers{col, soft, hard}; });
                drag.insert(drag.end(), {b, e, k, stop, cut, col, soft, hard, len, rho, plan.effective_end_fraction,
                                         static_cast<double>(plan.applied), static_cast<double>(plan.limit_valid),
                                         static_cast<double>(plan.reaches_cutoff), plan.drag_loss_eV,
                                         plan.collision_loss_eV, plan.soft_radiative_loss_eV,
                                         plan.hard_transfer_loss_eV, plan.raw_collision_loss_eV});
            }
            write_f8("ref_drag_plan", 19, drag);

            std::vector<double> chord;
            for (int i = 0; i < 3000; ++i) {
                double const rhi = 50.0, zlo = 0.0, zhi = 500.0;
                double r = (i % 6 == 0) ? 0.0 : rhi * g.uni();
                if (i % 10 == 1) r = rhi * (1.0 - 1.0e-7 * g.uni());
                double const th = 2.0 * 3.141592653589793 * g.uni() - 3.141592653589793;
                double z = zlo + (zhi - zlo) * g.uni();
                if (i % 10 == 2) z = zhi - 0.05 * g.uni();
                if (i % 10 == 3) z = zlo + 0.05 * g.uni();
                RreaRunningChargedState st;
                st.x_m = r * std::cos(th);
                st.y_m = r * std::sin(th);
                st.z_m = z;
                st.dir_x = g.uni() - 0.5;
                st.dir_y = g.uni() - 0.5;
                st.dir_z = g.uni() - 0.5;
                st.kinetic_energy_eV = g.logu(1.0e3, 1.0e10);
                double const dt = (i % 4 == 0) ? 5.0e-10 : g.logu(1.0e-12, 1.0e-6);
                bool const periodic = (i % 8 == 7);
                auto const ch = RreaBuildRunningChargedChord(st, dt, 5.0e-10, 0.0, rhi, zlo, zhi, periodic);
                auto const& p = ch.path;
                double const np = static_cast<double>(p.in_domain_pieces.size());
                double const p0b = np > 0 ? p.in_domain_pieces[0].begin_fraction : -1.0;
                double const p0e = np > 0 ? p.in_domain_pieces[0].end_fraction : -1.0;
                double const p0s = np > 0 ? p.in_domain_pieces[0].wrapped_z_shift_m : 0.0;
                double const plb = np > 0 ? p.in_domain_pieces.back().begin_fraction : -1.0;
                double const pls = np > 0 ? p.in_domain_pieces.back().wrapped_z_shift_m : 0.0;
                chord.insert(chord.end(),
                             {st.x_m, st.y_m, st.z_m, st.dir_x, st.dir_y, st.dir_z, st.kinetic_energy_eV, dt,
                              static_cast<double>(periodic), static_cast<double>(ch.valid), p.start_x_m, p.start_y_m,
                              p.start_z_m, p.end_x_m, p.end_y_m, p.end_z_m, p.full_length_m,
                              p.in_domain_end_fraction, p.in_domain_length_m, static_cast<double>(p.exits_domain), np,
                              p0b, p0e, p0s, plb, pls});
            }
            write_f8("ref_chord", 26, chord);
        }
        // ---- positron accessors and samplers: S/RreaInteractionTables.cpp:2325-2353,
        //      3129-3206, 2562-2575
        {
            std::vector<double> acc, bha, pbr;
            for (double e : charged_energies(g, tables, 1500)) {
                double const dr = (g.uni() < 0.5) ? 1.0 : 0.5 + 1.5 * g.uni();
                acc.insert(acc.end(), {e, dr, tables.PositronCollisionLoss(e, dr), tables.PositronSoftRadiativeDrag(e, dr),
                                       tables.PositronHardBhabhaMeanFreePath(e, dr),
                                       tables.PositronBremsstrahlungMeanFreePath(e, dr),
                                       tables.PositronAnnihilationMeanFreePath(e, dr)});
                // the conditional CDFs start near the 50 keV production
                // threshold; queries below a CDF's first group abort there
                // (the shim turns that into an exception) and are skipped
                double const u = g.uni();
                double const v = (g.uni() < 0.05) ? 0.0 : g.uni();
                try {
                    double const b = tables.SamplePositronBhabhaSecondaryEnergy(e, u);
                    bha.insert(bha.end(), {e, u, b});
                } catch (std::exception const&) {
                }
                try {
                    double const b = tables.SamplePositronBremsstrahlungPhotonEnergy(e, v);
                    pbr.insert(pbr.end(), {e, v, b});
                } catch (std::exception const&) {
                }
            }
            write_f8("ref_positron_accessors", 7, acc);
            write_f8("ref_bhabha_energy", 3, bha);
            write_f8("ref_positron_brems_energy", 3, pbr);
        }

        // ---- net-chord current: I/RreaSegmentDepositionRZ.H on the coupling's padded grid
        //      (8 x 12 physical cells of 0.75 m x 1.25 m, two pad cells; O/RreaWarpXCoupling.cpp:417-444)
        {
            rrea::SegmentGridRZ grid;
            int const pnr = 8, pnz = 12, pad = 2;
            grid.nr = pnr + pad;
            grid.nz = pnz + 2 * pad;
            grid.dr = 0.75;
            grid.dz = 1.25;
            grid.r_lo = 0.0;
            grid.z_lo = -pad * grid.dz;
            grid.resize();
            double const dt = 3.7e-10;
            double const rhi = pnr * grid.dr, zhi = pnz * grid.dz;
            std::vector<double> segs;  // kind, a0..a6, faces
            for (int i = 0; i < 400; ++i) {
                double const q = (g.uni() < 0.5 ? -1.0 : 1.0) * (0.5 + 1.5 * g.uni());
                double const r0 = (i % 17 == 0) ? 0.2 * grid.dr * g.uni() : rhi * g.uni() * 0.999;
                double const z0 = zhi * g.uni() * 0.999;
                double const len = 2.0 * grid.dr * g.uni();
                double const th = 6.283185307179586 * g.uni();
                double r1 = std::abs(r0 + len * std::cos(th));
                double z1 = z0 + len * std::sin(th);
                r1 = std::min(r1, rhi * 0.999);
                z1 = std::min(std::max(z1, 0.0), zhi * 0.999);
                rrea::DepositSegmentRZ(grid, q, dt, r0, z0, r1, z1);
                segs.insert(segs.end(), {0.0, r0, z0, r1, z1, q, 0.0, 0.0, 0.0});
            }
            for (int i = 0; i < 150; ++i) {
                double const q = (g.uni() < 0.5 ? -1.0 : 1.0) * (0.5 + 1.5 * g.uni());
                int const face = i % 3;  // 0 r_hi, 1 z_lo, 2 z_hi
                double cr, cz;
                std::uint32_t bits;
                if (face == 0) { cr = rhi; cz = zhi * (0.05 + 0.9 * g.uni()); bits = rrea::kEscapeFaceRHi; }
                else if (face == 1) { cr = rhi * 0.95 * g.uni(); cz = 0.0; bits = rrea::kEscapeFaceZLo; }
                else { cr = rhi * 0.95 * g.uni(); cz = zhi; bits = rrea::kEscapeFaceZHi; }
                double const fr0 = std::min(std::abs(cr - (face == 0 ? 0.4 : 0.3 * (g.uni() - 0.5))), rhi * 0.999);
                double const fz0 = std::min(std::max(cz + (face == 1 ? 0.4 : face == 2 ? -0.4 : 0.3 * (g.uni() - 0.5)),
                                                     0.0), zhi * 0.999);
                double const sr0 = std::min(std::abs(fr0 - 0.8 * (g.uni() - 0.5)), rhi * 0.999);
                double const sz0 = std::min(std::max(fz0 - 0.8 * (g.uni() - 0.5), 0.0), zhi * 0.999);
                auto const res = rrea::DepositEscapingSegmentRZ(grid, q, dt, sr0, sz0, fr0, fz0, cr, cz, pnr, pad, pnz,
                                                                bits);
                if (!res.valid) continue;
                segs.insert(segs.end(), {1.0, sr0, sz0, fr0, fz0, cr, cz, q, static_cast<double>(bits)});
            }
            std::vector<double> jr_phys, jz_phys;
            rrea::ConvertPaddedIndexCurrentToPhysicalRZ(pnr, pnz, grid.dr, grid.dz, pad, rrea::qe, grid.jr, grid.jz,
                                                        jr_phys, jz_phys);
            write_f8("ref_netchord_segments", 9, segs);
            write_f8("ref_netchord_rho", 1, grid.rho);
            write_f8("ref_netchord_jr", 1, grid.jr);
            write_f8("ref_netchord_jz", 1, grid.jz);
            write_f8("ref_netchord_jr_phys", 1, jr_phys);
            write_f8("ref_netchord_jz_phys", 1, jz_phys);
        }

        // ---- Maxwell TM-RZ leapfrog with a fixed face current (I/RreaMaxwellTMRZ.H:147-228),
        //      composed as S/RreaAmrexAdvance.cpp:690-780 with no fluid: restagger B by
        //      (dt - dt_sub)/2, `sub` x (B, Silver-Mueller, E), restagger back, Silver-Mueller
        {
            rrea::MaxwellTMRZ f;
            f.nr = 12;
            f.nz = 20;
            f.dr = 0.75;
            f.dz = 1.25;
            f.z_lo = 0.0;
            f.resize();
            for (auto& v : f.er) v = 1.0e4 * (2.0 * g.uni() - 1.0);
            for (auto& v : f.ez) v = 1.0e4 * (2.0 * g.uni() - 1.0);
            for (auto& v : f.btheta) v = 3.0e-5 * (2.0 * g.uni() - 1.0);
            for (int j = 0; j <= f.nz; ++j) f.Bt(0, j) = 0.0;
            for (int j = 0; j < f.nz; ++j) f.Er(0, j) = 0.0;
            std::vector<double> jr(f.er.size()), jz(f.ez.size());
            for (auto& v : jr) v = 2.0e-3 * (2.0 * g.uni() - 1.0);
            for (auto& v : jz) v = 2.0e-3 * (2.0 * g.uni() - 1.0);
            std::vector<double> init;
            init.insert(init.end(), f.er.begin(), f.er.end());
            init.insert(init.end(), f.ez.begin(), f.ez.end());
            init.insert(init.end(), f.btheta.begin(), f.btheta.end());
            init.insert(init.end(), jr.begin(), jr.end());
            init.insert(init.end(), jz.begin(), jz.end());
            double const dt = 0.9 / (rrea::kMaxwellC * std::sqrt(1.0 / (f.dr * f.dr) + 1.0 / (f.dz * f.dz)));
            int const sub = 3;
            double const dts = dt / sub;
            double const restagger = 0.5 * (dt - dts);
            std::vector<double> out;
            for (int step = 0; step < 4; ++step) {
                rrea::MaxwellAdvanceB(f, restagger);
                for (int k = 0; k < sub; ++k) {
                    rrea::MaxwellAdvanceB(f, dts);
                    rrea::MaxwellSilverMueller(f);
                    rrea::MaxwellAdvanceE(f, dts, nullptr, nullptr, &jr, &jz, nullptr, nullptr);
                }
                rrea::MaxwellAdvanceB(f, -restagger);
                rrea::MaxwellSilverMueller(f);
            }
            out.insert(out.end(), f.er.begin(), f.er.end());
            out.insert(out.end(), f.ez.begin(), f.ez.end());
            out.insert(out.end(), f.btheta.begin(), f.btheta.end());
            write_f8("ref_maxwell_init", 1, init);
            write_f8("ref_maxwell_out", 1, out);
            write_f8("ref_maxwell_dt", 1, std::vector<double>{dt});
        }

        // ---- photon samplers: S/RreaInteractionTables.cpp:2778-3253
        {
            std::vector<double> chan, kn, pe, pec, pair, ann;
            for (int i = 0; i < 3000; ++i) {
                double const e = (i % 10 == 0) ? g.logu(1.0e3, 2.0e4) : g.logu(1.0e3, 1.0e11);
                double const u = g.uni();
                chan.insert(chan.end(), {e, u, static_cast<double>(static_cast<int>(tables.SamplePhotonChannel(e, u)))});
                double const ek = g.logu(5.0e4, 1.0e9), u1 = g.uni(), u2 = g.uni();
                auto const c = tables.SampleComptonKleinNishinaFinalState(ek, u1, u2);
                kn.insert(kn.end(), {ek, u1, u2, c.recoil_electron_energy_eV, c.scattered_photon_energy_eV, c.cos_theta});
                double const ep = (i % 7 == 0) ? g.logu(1.0e3, 5.0e3) : g.logu(1.0e3, 1.0e11);
                auto const p = tables.SamplePhotoelectricFinalState(ep, u);
                pe.insert(pe.end(), {ep, u, p.photoelectron_energy_eV, p.binding_energy_eV});
                double const kk = (i % 13 == 0) ? g.logu(1.0e3, 1.2e3) : g.logu(1.0e3, 1.0e10);
                double const up = (i % 29 == 0) ? 0.0 : g.uni();
                pec.insert(pec.end(), {kk, up, tables.SamplePhotoelectronCosTheta(kk, up)});
                double const eg = (i % 9 == 0) ? g.logu(1.0e6, 3.0e6) : g.logu(2.1e6, 1.0e11);
                int const ch = (i % 2 == 0) ? 2 : 3;
                double const d1 = g.uni(), d2 = g.uni(), d3 = g.uni();
                auto const pr = tables.SamplePairFinalState(eg, static_cast<rrea::RreaPhotonChannel>(ch), d1, d2, d3,
                                                            0.5, 0.5);
                pair.insert(pair.end(), {eg, static_cast<double>(ch), d1, d2, d3, static_cast<double>(pr.valid),
                                         pr.electron_energy_eV, pr.positron_energy_eV, pr.recoil_electron_energy_eV,
                                         pr.local_deposit_energy_eV, pr.electron_dir_x, pr.electron_dir_y,
                                         pr.electron_dir_z, pr.positron_dir_x, pr.positron_dir_y, pr.positron_dir_z,
                                         pr.recoil_dir_x, pr.recoil_dir_y, pr.recoil_dir_z});
                double const ka = (i % 5 == 0) ? 0.0 : g.logu(1.0e3, 1.0e9);
                double const a1 = g.uni(), a2 = g.uni() * 3.0 - 1.0;
                auto const an = tables.SamplePositronAnnihilationFinalState(ka, a1, a2);
                ann.insert(ann.end(), {ka, a1, a2, an.photon1_energy_eV, an.photon2_energy_eV, an.photon1_cos_theta,
                                       an.photon1_azimuth_u, static_cast<double>(an.valid),
                                       static_cast<double>(an.at_rest)});
            }
            write_f8("ref_photon_channel", 3, chan);
            write_f8("ref_klein_nishina", 6, kn);
            write_f8("ref_photoelectric", 4, pe);
            write_f8("ref_photoelectron_cos", 3, pec);
            write_f8("ref_pair", 19, pair);
            write_f8("ref_annihilation", 9, ann);
        }
        // ---- altitude density profile: S/RreaAltitudeProfile.cpp (LoadCsv and
        // Interpolate), on a synthetic exponential atmosphere written as CSV
        // with the NRLMSISE column names and units (km, g/cm^3)
        {
            std::string const csv = g_outdir + "/ref_altitude_profile_input.csv";
            {
                std::ofstream f(csv);
                f << "model,altitude_km_MSL,mass_density_g_cm3\n";
                char line[128];
                for (int i = 0; i <= 160; ++i) {
                    double const km = 6.0 + 0.05 * i;
                    std::snprintf(line, sizeof line, "synthetic,%.17g,%.17g\n", km, 1.225e-3 * std::exp(-km / 7.2));
                    f << line;
                }
            }
            rrea::RreaAltitudeProfile prof;
            prof.LoadCsv(csv, "altitude_km_MSL", "mass_density_g_cm3", 1000.0, 1000.0, true);
            std::remove(csv.c_str());
            std::vector<double> nodes, rows;
            for (int i = 0; i <= 160; ++i) {
                double const a = (6.0 + 0.05 * i) * 1000.0;
                nodes.insert(nodes.end(), {a, prof.Interpolate(a)});
            }
            for (int i = 0; i < 4096; ++i) {
                double a = 6000.0 + 8000.0 * g.uni();
                if (i < 161) a = (6.0 + 0.05 * i) * 1000.0;                       // every node
                else if (i < 321) a = (6.0 + 0.05 * (i - 161) + 0.025) * 1000.0;  // every midpoint
                if (i == 321) a = prof.MinAltitudeM();
                if (i == 322) a = prof.MaxAltitudeM();
                rows.insert(rows.end(), {a, prof.Interpolate(a)});
            }
            write_f8("ref_altitude_profile_nodes", 2, nodes);
            write_f8("ref_altitude_profile", 2, rows);
        }
        // ---- seed schedule: S/RreaSeedSchedule.cpp (Load, ValidateProduction)
        // and I/RreaSeedSchedule.H (momentum normalisation, injection window)
        // on a synthetic CSV kept beside the fixtures
        {
            std::string const csv = g_outdir + "/ref_seed_schedule_input.csv";
            {
                std::ofstream f(csv);
                f << "case_id, macro_index,species_id,time_s,x_m,y_m,z_m,r_m,kinetic_energy_eV,ux,uy,uz,"
                     "weight_real_electrons\n";
                char line[1024];
                for (int i = 0; i < 240; ++i) {
                    char const* cid = (i % 11 == 5) ? "X9" : (i % 37 == 7 ? "BAD" : "C2");
                    bool const quoted = (i % 13 == 3);
                    double const rr = 1000.0 * std::sqrt(g.uni()), ph = 6.283185307179586 * g.uni();
                    double const x = rr * std::cos(ph), y = rr * std::sin(ph), z = 8000.0 * g.uni();
                    double r = std::hypot(x, y);
                    if (std::string(cid) == "BAD") r *= 1.001;  // inconsistent radius
                    // E^-1.5 on 1-100 MeV
                    double const u0 = g.uni();
                    double const k = 1.0e6 / std::pow(1.0 - u0 * (1.0 - std::pow(100.0, -0.5)), 2.0);
                    double const ct = std::sqrt(g.uni()), st = std::sqrt(1.0 - ct * ct), az = 6.283185307179586 * g.uni();
                    double dx = st * std::cos(az), dy = st * std::sin(az), dz = -ct;
                    if (i % 5 == 2) {  // a proper velocity instead of a direction hint
                        double const um = rrea::RreaElectronProperVelocityFromKineticEv(k);
                        dx *= um; dy *= um; dz *= um;
                    } else if (i % 7 == 4) {  // a hint of another magnitude
                        dx *= 3.5; dy *= 3.5; dz *= 3.5;
                    }
                    double const t = (i % 17 == 0) ? 1.0e-6 : 2.0e-6 * g.uni();
                    char macro[32] = "";
                    if (i % 6 != 1) std::snprintf(macro, sizeof macro, "%d", 10000 + 3 * ((i * 7919) % 240));
                    char spec[8] = "";
                    if (i % 4 == 1) std::snprintf(spec, sizeof spec, "2");
                    else if (i % 4 == 2) std::snprintf(spec, sizeof spec, "1");
                    std::snprintf(line, sizeof line, "%s%s%s, %s ,%s,%.17g,%.17g,%.17g,%.17g,%.17g,%.17g,%.17g,%.17g,%.17g,%.17g\n",
                                  quoted ? "\"" : "", cid, quoted ? "\"" : "", macro, spec, t, x, y, z, r, k, dx, dy,
                                  dz, 1.0e3 + 1.0e5 * g.uni());
                    f << line;
                    if (i % 50 == 9) f << "   \n";  // blank lines are skipped
                }
            }
            std::vector<double> rows, windows, checks;
            rrea::RreaSeedSchedule all;
            all.Load(csv, "");
            checks.push_back(static_cast<double>(all.Size()));
            rrea::RreaSeedSchedule sched;
            sched.Load(csv, "C2");
            double const win[3][2] = {{0.0, 5.0e-7}, {1.0e-6, 1.0005e-6}, {1.5e-6, 2.5e-6}};
            for (std::size_t i = 0; i < sched.Size(); ++i) {
                auto const& e = sched.Event(i);
                auto const m = rrea::RreaNormalizeSeedMomentum(e.ux, e.uy, e.uz, e.kinetic_energy_eV);
                rows.insert(rows.end(), {static_cast<double>(e.macro_index), static_cast<double>(e.species_id),
                                         e.time_s, e.x_m, e.y_m, e.z_m, e.r_m, e.kinetic_energy_eV, e.ux, e.uy, e.uz,
                                         e.weight_real_electrons, m.ux, m.uy, m.uz});
                for (auto const& w : win) {
                    auto const c = rrea::RreaSeedEventWindowClass(e.time_s, w[0], w[1]);
                    windows.push_back(c == rrea::RreaSeedWindowClass::SkipStale ? -1.0
                                      : c == rrea::RreaSeedWindowClass::Inject ? 0.0 : 1.0);
                }
            }
            auto validates = [&](rrea::RreaSeedSchedule const& s) {
                try {
                    s.ValidateProduction(1.0e4, 1.0e9, 0.0, 1000.0, 0.0, 8000.0);
                    return 1.0;
                } catch (std::exception const&) {
                    return 0.0;
                }
            };
            checks.push_back(validates(sched));
            rrea::RreaSeedSchedule bad;
            bad.Load(csv, "BAD");
            checks.push_back(static_cast<double>(bad.Size()));
            checks.push_back(validates(bad));
            write_f8("ref_seed_schedule_events", 15, rows);
            write_f8("ref_seed_schedule_windows", 3, windows);
            write_f8("ref_seed_schedule_checks", 1, checks);
        }
        // ---- CIC-conserving thinning: I/RreaCicConservingResample.H
        // (RreaThinCicWeights, RreaCicResampleRemovalCapacity) on seeded
        // support groups, with the counter draw u_k = (mix(key + k) >> 11 + 0.5) 2^-53
        {
            std::vector<double> parts, groups;
            for (int gi = 0; gi < 400; ++gi) {
                int const n = 2 + static_cast<int>(g.next() % 11);
                std::vector<rrea::RreaCicResampleParticle> ps(static_cast<std::size_t>(n));
                for (int i = 0; i < n; ++i) {
                    auto& q = ps[static_cast<std::size_t>(i)];
                    uint64_t const kind = g.next() % 16;
                    q.fraction_r = g.uni();
                    q.fraction_z = g.uni();
                    if (kind == 0 && i > 0) {  // same support point as the previous particle
                        q.fraction_r = ps[static_cast<std::size_t>(i - 1)].fraction_r;
                        q.fraction_z = ps[static_cast<std::size_t>(i - 1)].fraction_z;
                    } else if (kind == 1) {
                        q.fraction_r = (g.next() & 1) ? 1.0 : 0.0;
                    } else if (kind == 2) {
                        q.fraction_z = (g.next() & 1) ? 1.0 : 0.0;
                    }
                    q.weight = (kind == 3) ? 0.0 : 0.1 + 9.9 * g.uni();
                }
                std::size_t const capacity = rrea::RreaCicResampleRemovalCapacity(ps);
                std::size_t const max_removals = (gi % 3 == 0) ? static_cast<std::size_t>(n)
                                                                 : static_cast<std::size_t>(g.next() % (n + 1));
                uint64_t const key = g.next();
                std::vector<rrea::RreaCicResampleParticle> out = ps;
                auto const res = rrea::RreaThinCicWeights(out, max_removals, [&](std::size_t k) {
                    return (static_cast<double>(rrea::RreaCicMix64(key + k) >> 11) + 0.5) * 0x1.0p-53;
                });
                for (int i = 0; i < n; ++i) {
                    auto const& a = ps[static_cast<std::size_t>(i)];
                    parts.insert(parts.end(), {static_cast<double>(gi), a.fraction_r, a.fraction_z, a.weight,
                                               out[static_cast<std::size_t>(i)].weight});
                }
                uint64_t const key_hi = key >> 32, key_lo = key & 0xffffffffULL;
                groups.insert(groups.end(), {static_cast<double>(n), static_cast<double>(max_removals),
                                             static_cast<double>(key_hi), static_cast<double>(key_lo),
                                             static_cast<double>(res.removed), static_cast<double>(res.draws),
                                             res.valid ? 1.0 : 0.0, static_cast<double>(capacity)});
            }
            write_f8("ref_cic_thin_particles", 5, parts);
            write_f8("ref_cic_thin_groups", 8, groups);
        }
        // ---- particle charge: DepositChargeCIC (I/RreaSegmentDepositionRZ.H:68-92), the
        //      cell-centred CIC with the axis fold and edge clamps, on a 12 x 20 grid
        {
            rrea::SegmentGridRZ grid;
            grid.nr = 12;
            grid.nz = 20;
            grid.dr = 0.5;
            grid.dz = 2.5;
            grid.r_lo = 0.0;
            grid.z_lo = 10.0;
            grid.resize();
            std::vector<double> parts;
            for (int i = 0; i < 3000; ++i) {
                double const r = (i % 7 == 0) ? 0.6 * grid.dr * g.uni() : 1.02 * grid.nr * grid.dr * g.uni();
                double const z = grid.z_lo + (1.04 * g.uni() - 0.02) * grid.nz * grid.dz;
                double const qw = (g.uni() < 0.3 ? 1.0 : -1.0) * (0.25 + 4.0 * g.uni());
                rrea::DepositChargeCIC(grid, qw, r, z);
                parts.insert(parts.end(), {r, z, qw});
            }
            write_f8("ref_cic_charge_particles", 3, parts);
            write_f8("ref_cic_charge_rho", 1, grid.rho);
            write_f8("ref_cic_charge_grid", 6, {static_cast<double>(grid.nr), static_cast<double>(grid.nz), grid.dr,
                                                 grid.dz, grid.r_lo, grid.z_lo});
        }

        // ---- plane-crossing diagnostic (I/RreaPlaneFlux.H): the crossing
        //      enumeration of RreaForEachNonperiodicPlaneCrossing over seeded
        //      segments (ends on planes, reversals, zero length, a non-finite
        //      end) and RreaPlaneFluxAccumulator::AddCrossing / Flatten over a
        //      crossing batch that ends with invalid crossings
        {
            Gen g(20261204ULL);   // its own stream: the vectors after this block keep theirs
            std::vector<amrex::Real> const planes{-3.0, 0.0, 1.5, 2.0, 4.25, 10.0, 10.5, 30.0};
            std::vector<double> segs, rows;
            for (int i = 0; i < 600; ++i) {
                double z0 = -8.0 + 44.0 * g.uni();
                double z1 = z0 + (g.uni() < 0.5 ? -1.0 : 1.0) * 25.0 * g.uni() * g.uni();
                uint64_t const kind = g.next() % 10;
                if (kind == 0) z0 = planes[g.next() % planes.size()];
                if (kind == 1) z1 = planes[g.next() % planes.size()];
                if (kind == 2) z1 = z0;
                if (kind == 3 && i % 7 == 0) z1 = std::numeric_limits<double>::infinity();
                int count = 0;
                bool const ok = rrea::RreaForEachNonperiodicPlaneCrossing(
                    z0, z1, planes, [&](std::size_t p, amrex::Real, amrex::Real f, int d) {
                        rows.insert(rows.end(), {static_cast<double>(i), static_cast<double>(p), f,
                                                 static_cast<double>(d)});
                        ++count;
                    });
                segs.insert(segs.end(), {z0, z1, ok ? static_cast<double>(count) : -1.0});
            }
            write_f8("ref_plane_segments", 3, segs);
            write_f8("ref_plane_crossings", 4, rows);
            write_f8("ref_plane_planes", 1, std::vector<double>(planes.begin(), planes.end()));
            rrea::RreaPlaneFluxAccumulator acc(planes.size());
            std::vector<double> batch, status;
            for (int i = 0; i < 400; ++i) {
                double const p = static_cast<double>(g.next() % planes.size());
                double const d = (g.next() & 1) ? 1.0 : -1.0;
                double w = 0.1 + 5.0 * g.uni();
                double r = 40.0 * g.uni();
                if (i == 397) w = -1.0;                   // invalid weight
                if (i == 398) r = std::nan("");           // invalid radius
                double const local = (g.next() % 3 == 0) ? 1.0 : 0.0;
                double const mev = (g.next() % 2 == 0) ? 1.0 : 0.0;
                batch.insert(batch.end(), {p, d, w, r, local, mev});
                bool const ok = acc.AddCrossing(static_cast<std::size_t>(p), static_cast<int>(d), w, r, local != 0.0,
                                                mev != 0.0);
                status.push_back(ok ? 1.0 : 0.0);
            }
            write_f8("ref_plane_batch", 6, batch);
            write_f8("ref_plane_batch_ok", 1, status);
            auto const flat = acc.Flatten();
            write_f8("ref_plane_flux", 10, std::vector<double>(flat.begin(), flat.end()));
        }

        // ---- adaptive_resample_v1 global thinning on one rank: the plan of
        //      O/RreaCouplingPopulation.cpp:175-640 (records, sort, support capacity,
        //      greedy requests) around the reference's own RreaPlanGlobalCicThinning,
        //      RreaCicResampleRemovalCapacity and RreaAdaptiveResampleCicUniform
        for (int pc_case = 0; pc_case < 2; ++pc_case) {
            int const nr = 10, nz = 12;
            double const dr = 1.0, dz = 2.0, r_lo = 0.0, z_lo = 0.0;
            bool const positron = pc_case == 1;
            int const n_live = pc_case == 0 ? 4000 : 3200;
            int const n_cand = pc_case == 0 ? 800 : 800;
            long const target = pc_case == 0 ? 1500 : 3000;
            std::uint64_t const seed = 77, salt = pc_case == 0 ? 0 : 12345;
            std::uint64_t const step = 9 + pc_case;
            std::vector<double> live, cand;  // the inputs as the device receives them
            struct Rec {
                int sr, sz, phase;
                bool candidate;
                std::uint64_t high, low;
                double fr, fz, w;
                int member;
            };
            std::vector<Rec> recs;
            auto record = [&](double r, double z, double ux, double uy, double uz, double th, double w, bool c,
                              std::uint64_t high, std::uint64_t low, int member) {
                double const rc = (r - r_lo) / dr + 0.0 - 0.5;
                double const zc = (z - z_lo) / dz + 0.0 - 0.5;
                double const i0 = std::floor(rc), j0 = std::floor(zc);
                double const co = std::cos(th), si = std::sin(th);
                double const ur = ux * co + uy * si, ut = -ux * si + uy * co;
                double const mag = std::sqrt(ux * ux + uy * uy + uz * uz);
                int ex = mag > 0.0 && std::isfinite(mag) ? std::ilogb(mag) : -1024;
                ex = std::max(-1024, std::min(1023, ex));
                recs.push_back(Rec{static_cast<int>(i0), static_cast<int>(j0),
                                   (ex + 1024) * 8 + (ur >= 0.0 ? 1 : 0) + (ut >= 0.0 ? 2 : 0) + (uz >= 0.0 ? 4 : 0),
                                   c, high, low, rc - i0, zc - j0, w, member});
            };
            for (int i = 0; i < n_live; ++i) {
                // clustered: a third of the particles in three cells
                double const r = (i % 3 == 0) ? (0.5 + (i % 9) / 3) * dr + 0.4 * g.uni() : nr * dr * g.uni();
                double const z = (i % 3 == 0) ? 5.0 * dz + 0.7 * dz * g.uni() : nz * dz * g.uni();
                double const th = 6.283185307179586 * g.uni() - 3.141592653589793;
                double const k = g.logu(1.0e4, 1.0e8);
                double const u = rrea::RreaElectronProperVelocityFromKineticEv(k);
                double const mu = 2.0 * g.uni() - 1.0, ph = 6.283185307179586 * g.uni();
                double const sn = std::sqrt(1.0 - mu * mu);
                double const ux = u * sn * std::cos(ph), uy = u * sn * std::sin(ph), uz = u * mu;
                double const w = 0.5 + 1.5 * g.uni();
                std::int64_t const id = 1 + i;
                std::int32_t const cpu = i % 5;
                live.insert(live.end(), {r, z, th, ux, uy, uz, w, static_cast<double>(id), static_cast<double>(cpu)});
                record(r, z, ux, uy, uz, th, w, false, 0,
                       (static_cast<std::uint64_t>(id) << 24) | static_cast<std::uint32_t>(cpu), i);
            }
            for (int i = 0; i < n_cand; ++i) {
                double const rr = (i % 2 == 0) ? (0.6 + (i % 6) / 2) * dr + 0.3 * g.uni() : nr * dr * g.uni();
                double const th = 6.283185307179586 * g.uni() - 3.141592653589793;
                double const x = rr * std::cos(th), y = rr * std::sin(th);
                double const z = (i % 2 == 0) ? 5.0 * dz + 0.9 * dz * g.uni() : nz * dz * g.uni();
                double const k = g.logu(1.0e4, 3.0e7);
                double const mu = 2.0 * g.uni() - 1.0, ph = 6.283185307179586 * g.uni();
                double const sn = std::sqrt(1.0 - mu * mu);
                double const dx = sn * std::cos(ph), dy = sn * std::sin(ph), dzr = mu;
                double const w = 0.5 + 1.5 * g.uni();
                std::uint64_t const root = g.next() >> 8;
                std::uint64_t const lineage = static_cast<std::uint64_t>(i % 37);
                int const root_species = i % 3;
                cand.insert(cand.end(), {x, y, z, dx, dy, dzr, k, w, static_cast<double>(root >> 32),
                                         static_cast<double>(root & 0xffffffffULL), static_cast<double>(lineage),
                                         static_cast<double>(root_species)});
                double const u = rrea::RreaElectronProperVelocityFromKineticEv(k);
                record(std::hypot(x, y), z, u * dx, u * dy, u * dzr, std::atan2(y, x), w, true, root,
                       (lineage << 2) | static_cast<std::uint64_t>(root_species), n_live + i);
            }
            std::sort(recs.begin(), recs.end(), [](Rec const& a, Rec const& b) {
                if (a.sr != b.sr) return a.sr < b.sr;
                if (a.sz != b.sz) return a.sz < b.sz;
                if (a.phase != b.phase) return a.phase < b.phase;
                if (a.candidate != b.candidate) return a.candidate < b.candidate;
                if (a.high != b.high) return a.high < b.high;
                return a.low < b.low;
            });
            std::uint64_t const stream_key = positron ? 0x706f736974726f6eULL : 0x656c656374726f6eULL;
            auto const rng_species = positron ? rrea::warpx::RreaAdaptiveResampleSpecies::Positron
                                              : rrea::warpx::RreaAdaptiveResampleSpecies::Electron;
            std::vector<std::pair<std::size_t, std::size_t>> supports;
            std::vector<std::size_t> caps;
            std::size_t total_cap = 0;
            for (std::size_t b = 0; b < recs.size();) {
                std::size_t e = b + 1;
                while (e < recs.size() && recs[e].sr == recs[b].sr && recs[e].sz == recs[b].sz) ++e;
                std::vector<rrea::RreaCicResampleParticle> sup;
                for (std::size_t i = b; i < e; ++i) sup.push_back({recs[i].fr, recs[i].fz, recs[i].w});
                std::size_t const cap = rrea::RreaCicResampleRemovalCapacity(sup);
                supports.push_back({b, e});
                caps.push_back(cap);
                total_cap += cap;
                b = e;
            }
            long const members = static_cast<long>(recs.size());
            long const nominal = members > target + target / 4
                ? std::min<long>(members - target, static_cast<long>(total_cap)) : 0;
            std::vector<double> new_w(recs.size());
            for (auto const& r : recs) new_w[static_cast<std::size_t>(r.member)] = r.w;
            long remaining = nominal, removed = 0;
            for (std::size_t sidx = 0; sidx < supports.size(); ++sidx) {
                long const request = std::min<long>(remaining, static_cast<long>(caps[sidx]));
                remaining -= request;
                if (request == 0) continue;
                std::vector<rrea::RreaGlobalCicParticle> sup;
                for (std::size_t i = supports[sidx].first; i < supports[sidx].second; ++i) {
                    rrea::RreaGlobalCicParticle q;
                    q.support_r = recs[i].sr;
                    q.support_z = recs[i].sz;
                    q.phase = recs[i].phase;
                    q.source_rank = 0;
                    q.stable_id = recs[i].low;
                    q.fraction_r = recs[i].fr;
                    q.fraction_z = recs[i].fz;
                    q.weight = recs[i].w;
                    q.candidate = recs[i].candidate;
                    q.stable_id_high = recs[i].high;
                    sup.push_back(q);
                }
                auto const plan = rrea::RreaPlanGlobalCicThinning<double>(
                    sup, sup.size() - static_cast<std::size_t>(request), 1, stream_key,
                    [&](std::uint64_t group_id, std::size_t reduction) {
                        return rrea::warpx::RreaAdaptiveResampleCicUniform(seed, group_id ^ salt, step, reduction,
                                                                           rng_species);
                    });
                if (!plan.valid()) throw std::runtime_error("population golden: support plan rejected");
                removed += static_cast<long>(plan.removed);
                for (auto const& u : plan.updates) {
                    for (std::size_t i = supports[sidx].first; i < supports[sidx].second; ++i) {
                        if (recs[i].candidate == u.candidate && recs[i].low == u.stable_id &&
                            recs[i].high == u.stable_id_high) {
                            new_w[static_cast<std::size_t>(recs[i].member)] = u.stored_weight;
                        }
                    }
                }
            }
            std::string const tag = pc_case == 0 ? "ref_population_electron" : "ref_population_positron";
            write_f8(tag + "_live", 9, live);
            write_f8(tag + "_candidates", 12, cand);
            write_f8(tag + "_weights", 1, new_w);
            write_f8(tag + "_plan", 8, {static_cast<double>(members), static_cast<double>(n_live),
                                        static_cast<double>(n_cand), static_cast<double>(supports.size()),
                                        static_cast<double>(total_cap), static_cast<double>(nominal),
                                        static_cast<double>(removed), static_cast<double>(target)});
            write_f8(tag + "_setup", 10, {static_cast<double>(nr), static_cast<double>(nz), dr, dz, r_lo, z_lo,
                                          static_cast<double>(seed), static_cast<double>(salt),
                                          static_cast<double>(step), positron ? 1.0 : 0.0});
        }

        // ---- charged-loop skeletons: O/RreaChargedInterleave.H:546-732 driven by
        // scripted policies (oracle/interleave_scenarios.hpp)
        {
            namespace is = interleave_scenarios;
            std::vector<double> ev, sub;
            for (uint64_t seed = 0; seed < 400; ++seed) {
                is::Trace const t = is::run_event_scenario<RefSkeleton>(is::event_scenario(seed));
                for (std::size_t i = 0; i < t.rec.size(); i += 4) {
                    ev.insert(ev.end(), {static_cast<double>(seed), t.rec[i], t.rec[i + 1], t.rec[i + 2], t.rec[i + 3]});
                }
            }
            for (uint64_t seed = 0; seed < 300; ++seed) {
                is::Trace const t = is::run_substep_scenario<RefSkeleton>(is::substep_scenario(seed));
                for (std::size_t i = 0; i < t.rec.size(); i += 4) {
                    sub.insert(sub.end(), {static_cast<double>(seed), t.rec[i], t.rec[i + 1], t.rec[i + 2], t.rec[i + 3]});
                }
            }
            write_f8("ref_interleave_events", 5, ev);
            write_f8("ref_interleave_substeps", 5, sub);
        }
        std::printf("golden fixtures written to %s\n", g_outdir.c_str());
    } catch (std::exception const& e) {
        std::fprintf(stderr, "ref_golden failed: %s\n", e.what());
        return 1;
    }
    return 0;
}
