// Carrier-fluid golden-vector generator built from the REFERENCE's own fluid
// sources (S/LowEnergyFluidState.cpp, S/LowEnergyFluidFaceTransport.cpp and
// the closure loader in S/RreaInteractionTables.cpp), compiled in place
// against the single-box AMReX stand-in in oracle/ref_shim by
// oracle/Makefile.ref into oracle/_ref/ref_golden_fluid.  It drives the
// reference's LowEnergyFluidState on seeded cell states and writes inputs and
// outputs as .npy fixtures under tests/golden/ (ref_fluid_*).  Those fixtures
// pin the oracle's fluid restatement (oracle/fluid.cpp) and the device
// kernels.  Test infrastructure only.
//
// Layouts: cell fields nr*nz with index i + nr*j; radial-face fields
// (nr+1)*nz, index i + (nr+1)*j; axial-face fields nr*(nz+1), index
// i + nr*j; species-major for the three carriers (positive ion, negative
// ion, electron).
#include "rrea/LowEnergyFluidState.H"
#include "rrea/RreaConstants.H"
#include "rrea/RreaInteractionTables.H"

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <memory>
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

void write_f8(std::string const& name, std::size_t cols, std::vector<double> const& v)
{
    std::string path = g_outdir + "/" + name + ".npy";
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) throw std::runtime_error("cannot write " + path);
    char header[256];
    int const hl = std::snprintf(header, sizeof(header), "{'descr': '<f8', 'fortran_order': False, 'shape': (%zu, %zu), }",
                                 v.size() / cols, cols);
    std::string h(header, static_cast<std::size_t>(hl));
    std::size_t const total = 10 + h.size() + 1;
    h.append((64 - total % 64) % 64, ' ');
    h.push_back('\n');
    unsigned char magic[8] = {0x93, 'N', 'U', 'M', 'P', 'Y', 1, 0};
    std::fwrite(magic, 1, 8, f);
    uint16_t const len = static_cast<uint16_t>(h.size());
    std::fwrite(&len, 2, 1, f);
    std::fwrite(h.data(), 1, h.size(), f);
    std::fwrite(v.data(), 8, v.size(), f);
    std::fclose(f);
}

struct Grid {
    int nr, nz;
    double r_lo, z_lo, dr, dz;
    bool periodic_z;
    amrex::Box cells() const { return amrex::Box(amrex::IntVect(0, 0), amrex::IntVect(nr - 1, nz - 1)); }
    amrex::BoxArray ba() const { return amrex::BoxArray(cells()); }
    amrex::Geometry geom() const
    {
        return amrex::Geometry(cells(), r_lo, z_lo, r_lo + nr * dr, z_lo + nz * dz, periodic_z);
    }
};

// Cell field <-> flat vector over the valid cells.
void put_cells(amrex::MultiFab& mf, Grid const& g, std::vector<double> const& v, int comp = 0)
{
    for (int j = 0; j < g.nz; ++j)
        for (int i = 0; i < g.nr; ++i) mf.at(i, j, comp) = v[static_cast<std::size_t>(i + g.nr * j)];
}
std::vector<double> get_cells(amrex::MultiFab const& mf, Grid const& g, int comp = 0)
{
    std::vector<double> v(static_cast<std::size_t>(g.nr) * g.nz);
    for (int j = 0; j < g.nz; ++j)
        for (int i = 0; i < g.nr; ++i) v[static_cast<std::size_t>(i + g.nr * j)] = mf.at(i, j, comp);
    return v;
}
std::vector<double> get_faces(amrex::MultiFab const& mf, int ni, int nj, int comp)
{
    std::vector<double> v(static_cast<std::size_t>(ni) * nj);
    for (int j = 0; j < nj; ++j)
        for (int i = 0; i < ni; ++i) v[static_cast<std::size_t>(i + ni * j)] = mf.at(i, j, comp);
    return v;
}
void append(std::vector<double>& out, std::vector<double> const& v) { out.insert(out.end(), v.begin(), v.end()); }

// Carrier densities spanning vacuum, exact zeros, negatives (clamped by the
// reference) and 1e2..1e15 m^-3.
double density(Gen& g)
{
    double const u = g.uni();
    if (u < 0.06) return 0.0;
    if (u < 0.09) return -g.logu(1.0, 1.0e6);
    if (u < 0.12) return g.logu(1.0e-34, 1.0e-29);
    return g.logu(1.0e2, 1.0e15);
}
double rate(Gen& g)
{
    double const u = g.uni();
    if (u < 0.15) return 0.0;
    if (u < 0.2) return -g.logu(1.0e8, 1.0e12);
    return g.logu(1.0e8, 1.0e22);
}

rrea::LowEnergyFluidConfig base_config()
{
    rrea::LowEnergyFluidConfig c;
    c.electron_ion_recombination_coefficient_m3_per_s = 2.0e-13;
    c.ion_ion_recombination_coefficient_m3_per_s = 2.0e-12;
    c.detachment_frequency_s = 3.0e4;
    return c;
}

// ---- chemistry: UpdateFromIonizationSource + MaxReactionFrequency +
// ComputeFluidChargeDensity (S/LowEnergyFluidState.cpp:97-320, :389-420)
void reaction_cases(Gen& g, rrea::LowEnergyElectronClosure const&)
{
    Grid const grid{7, 9, 0.0, 0.0, 1.5, 2.0, false};
    std::vector<double> setup, inputs, outputs;
    int const n = grid.nr * grid.nz;
    for (int c = 0; c < 8; ++c) {
        rrea::LowEnergyFluidConfig cfg = base_config();
        double const dt = (c % 4 == 0) ? 2.5e-10 : (c % 4 == 1 ? 1.0e-8 : (c % 4 == 2 ? 1.0e-6 : 3.0e-12));
        bool const table = c >= 4;
        if (c == 1) cfg.detachment_frequency_s = 0.0;
        if (c == 2) cfg.attachment_frequency_s = 0.0;
        if (c == 3) {
            cfg.electron_ion_recombination_coefficient_m3_per_s = 0.0;
            cfg.ion_ion_recombination_coefficient_m3_per_s = 0.0;
        }
        if (c == 6) cfg.detachment_frequency_s = 2.0e9;
        if (table) cfg.attachment_model = "en_table_attachment_v1";
        rrea::LowEnergyFluidState fluid(grid.ba(), amrex::DistributionMapping{}, 1);
        std::vector<double> ne(n), np(n), nn(n), se(n), sp(n), sn(n), rho(n), nu(n);
        for (int k = 0; k < n; ++k) {
            ne[k] = density(g);
            np[k] = density(g);
            nn[k] = density(g);
            if (k % 11 == 3) np[k] = std::max(ne[k], 0.0);   // equal pair: the small-delta branch
            if (k % 13 == 5) nn[k] = std::max(np[k], 0.0);
            se[k] = rate(g);
            sp[k] = rate(g);
            sn[k] = rate(g);
            rho[k] = (g.uni() - 0.5) * 1.0e-4;
            double const u = g.uni();
            nu[k] = u < 0.1 ? 0.0 : g.logu(1.0e3, 1.0e10);
        }
        put_cells(fluid.LowElectronDensity(), grid, ne);
        put_cells(fluid.PositiveIonDensity(), grid, np);
        put_cells(fluid.NegativeIonDensity(), grid, nn);
        put_cells(fluid.LowElectronSourceRate(), grid, se);
        put_cells(fluid.PositiveIonSourceRate(), grid, sp);
        put_cells(fluid.DirectNegativeIonSourceRate(), grid, sn);
        put_cells(fluid.FluidChargeDensity(), grid, rho);
        amrex::MultiFab nu_cell(grid.ba(), amrex::DistributionMapping{}, 1, 1);
        put_cells(nu_cell, grid, nu);
        double const max_rate = fluid.MaxReactionFrequency(cfg, table ? &nu_cell : nullptr);
        bool const clear = (c % 2) == 0;
        fluid.UpdateFromIonizationSource(dt, cfg, nullptr, table ? &nu_cell : nullptr, clear);
        double const residual = fluid.LastReactionChargeConservationResidual();
        std::vector<double> const rho_after = get_cells(fluid.FluidChargeDensity(), grid);
        fluid.ComputeFluidChargeDensity();
        setup.insert(setup.end(), {static_cast<double>(grid.nr), static_cast<double>(grid.nz), dt,
                                   cfg.attachment_frequency_s, cfg.electron_ion_recombination_coefficient_m3_per_s,
                                   cfg.ion_ion_recombination_coefficient_m3_per_s, cfg.detachment_frequency_s,
                                   table ? 1.0 : 0.0, clear ? 1.0 : 0.0, max_rate, residual});
        for (auto const* v : {&ne, &np, &nn, &se, &sp, &sn, &rho, &nu}) append(inputs, *v);
        append(outputs, get_cells(fluid.LowElectronDensity(), grid));
        append(outputs, get_cells(fluid.PositiveIonDensity(), grid));
        append(outputs, get_cells(fluid.NegativeIonDensity(), grid));
        append(outputs, rho_after);
        append(outputs, get_cells(fluid.LowElectronSourceRate(), grid));
        append(outputs, get_cells(fluid.PositiveIonSourceRate(), grid));
        append(outputs, get_cells(fluid.DirectNegativeIonSourceRate(), grid));
        append(outputs, get_cells(fluid.FluidChargeDensity(), grid));   // ComputeFluidChargeDensity
    }
    write_f8("ref_fluid_reaction_setup", 11, setup);
    write_f8("ref_fluid_reaction_in", static_cast<std::size_t>(n), inputs);
    write_f8("ref_fluid_reaction_out", static_cast<std::size_t>(n), outputs);
}

// ---- quasi-neutral charge reconstruction: ComputeFluidChargeDensity's
// 64-eps neutrality rule (S/LowEnergyFluidState.cpp:389-420)
void neutral_cases(Gen& g)
{
    Grid const grid{6, 5, 0.0, 0.0, 1.0, 1.0, false};
    int const n = grid.nr * grid.nz;
    std::vector<double> in, out;
    rrea::LowEnergyFluidState fluid(grid.ba(), amrex::DistributionMapping{}, 1);
    std::vector<double> ne(n), np(n), nn(n);
    for (int k = 0; k < n; ++k) {
        ne[k] = g.logu(1.0e6, 1.0e14);
        nn[k] = g.logu(1.0e6, 1.0e14);
        np[k] = ne[k] + nn[k];
        if (k % 3 == 1) np[k] = std::nextafter(np[k], 1.0e300);
        if (k % 3 == 2) np[k] *= 1.0 + 1.0e-13 * (1 + k % 7);
        if (k % 10 == 9) ne[k] = -1.0;
    }
    put_cells(fluid.LowElectronDensity(), grid, ne);
    put_cells(fluid.PositiveIonDensity(), grid, np);
    put_cells(fluid.NegativeIonDensity(), grid, nn);
    fluid.ComputeFluidChargeDensity();
    for (auto const* v : {&ne, &np, &nn}) append(in, *v);
    append(out, get_cells(fluid.FluidChargeDensity(), grid));
    write_f8("ref_fluid_neutral_in", static_cast<std::size_t>(n), in);
    write_f8("ref_fluid_neutral_out", static_cast<std::size_t>(n), out);
}

// ---- closure cell fields: BuildElectronClosureCellFields
// (S/LowEnergyFluidFaceTransport.cpp:1022-1240) on the dry-air v3 table
void closure_cases(Gen& g, rrea::LowEnergyElectronClosure const& closure)
{
    Grid const grid{9, 12, 0.0, 100.0, 2.0, 3.0, false};
    int const n = grid.nr * grid.nz;
    amrex::MultiFab er(grid.ba(), amrex::DistributionMapping{}, 1, 1), ez(grid.ba(), amrex::DistributionMapping{}, 1, 1);
    amrex::MultiFab den(grid.ba(), amrex::DistributionMapping{}, 1, 1), ne(grid.ba(), amrex::DistributionMapping{}, 1, 1);
    amrex::MultiFab src(grid.ba(), amrex::DistributionMapping{}, 1, 1);
    amrex::MultiFab mu(grid.ba(), amrex::DistributionMapping{}, 1, 1), nu(grid.ba(), amrex::DistributionMapping{}, 1, 1);
    amrex::MultiFab dt(grid.ba(), amrex::DistributionMapping{}, 3, 1);
    std::vector<double> ver(n), vez(n), vden(n), vne(n), vsrc(n);
    for (int k = 0; k < n; ++k) {
        vden[k] = g.logu(0.2, 1.1);
        double const u = g.uni();
        // |E| / (chi N0) * 1e21 in Td: below range, in range, above range
        double const en = u < 0.1 ? 0.0 : (u < 0.2 ? g.logu(1.0e-9, 1.0e-6) : (u < 0.93 ? g.logu(1.0e-6, 100.0)
                                                                                           : g.logu(100.0, 300.0)));
        double const e_mag = en * vden[k] * rrea::n_loschmidt_m3 * 1.0e-21;
        double const ang = 6.283185307179586 * g.uni();
        ver[k] = e_mag * std::cos(ang);
        vez[k] = e_mag * std::sin(ang);
        if (k % 17 == 4) ver[k] = 0.0;
        vne[k] = g.uni() < 0.2 ? 0.0 : g.logu(1.0, 1.0e14);
        vsrc[k] = g.uni() < 0.3 ? 0.0 : g.logu(1.0e10, 1.0e20);
    }
    put_cells(er, grid, ver);
    put_cells(ez, grid, vez);
    put_cells(den, grid, vden);
    put_cells(ne, grid, vne);
    put_cells(src, grid, vsrc);
    rrea::LowEnergyClosureFieldDiagnostics d;
    rrea::BuildElectronClosureCellFields(grid.geom(), er, ez, &den, 1.0, closure, &ne, &src, &mu, &nu, &dt, d);
    std::vector<double> in, out;
    for (auto const* v : {&ver, &vez, &vden, &vne, &vsrc}) append(in, *v);
    append(out, get_cells(mu, grid));
    append(out, get_cells(nu, grid));
    for (int c = 0; c < 3; ++c) append(out, get_cells(dt, grid, c));
    write_f8("ref_fluid_closure_in", static_cast<std::size_t>(n), in);
    write_f8("ref_fluid_closure_out", static_cast<std::size_t>(n), out);
    write_f8("ref_fluid_closure_diag", 14,
             {static_cast<double>(grid.nr), static_cast<double>(grid.nz), grid.r_lo, grid.z_lo, grid.dr, grid.dz,
              d.min_en_td, d.max_en_td, static_cast<double>(d.held_below_cells),
              static_cast<double>(d.above_range_cells), static_cast<double>(d.invalid_cells),
              d.electron_count, d.held_below_electron_count, d.electron_source_rate_per_s});
}

// ---- explicit carrier transport: Prepare/Build/ApplyExplicitCarrierTransport
// and ComputeConductivity (S/LowEnergyFluidFaceTransport.cpp:153-953,
// S/LowEnergyFluidState.cpp:322-387)
struct TransportCase {
    Grid grid;
    bool ions;
    bool reduced_ions;
    bool table_electrons;
    bool density_field;
    double e_scale;
    double dt;
};

void transport_cases(Gen& g, rrea::LowEnergyElectronClosure const& closure)
{
    TransportCase const cases[] = {
        {{8, 10, 0.0, 0.0, 2.0, 3.0, false}, true, false, false, false, 4.0e5, 2.0e-9},
        {{8, 10, 0.0, 0.0, 2.0, 3.0, false}, true, false, false, false, 4.0e5, 5.0e-8},   // limiter active
        {{6, 12, 0.0, -10.0, 1.0, 2.0, true}, true, true, false, true, 3.0e5, 3.0e-8},
        {{7, 9, 0.0, 5.0, 2.0, 2.5, false}, false, false, true, true, 2.0e5, 2.0e-9},
        {{7, 9, 0.0, 5.0, 2.0, 2.5, true}, true, false, true, true, 2.0e5, 4.0e-9},
        {{5, 6, 0.0, 0.0, 1.0, 1.0, false}, true, true, true, false, 1.0e6, 1.0e-10},
    };
    std::vector<double> setup, inputs, outputs;
    for (TransportCase const& tc : cases) {
        Grid const& grid = tc.grid;
        int const nr = grid.nr, nz = grid.nz, n = nr * nz;
        rrea::LowEnergyFluidConfig cfg;
        cfg.ion_drift_enable = tc.ions;
        cfg.electron_drift_enable = true;
        cfg.positive_ion_mobility_m2_per_vs = 2.2e-4;
        cfg.negative_ion_mobility_m2_per_vs = 1.9e-4;
        cfg.electron_mobility_m2_per_vs = 0.06;
        cfg.ion_drift_cfl = 0.45;
        cfg.transport_density_ratio = 0.93;
        if (tc.reduced_ions) {
            cfg.ion_mobility_model = "reduced_stp_density_scaled";
            cfg.positive_ion_reduced_mobility_stp_m2_per_vs = 2.0e-4;
            cfg.negative_ion_reduced_mobility_stp_m2_per_vs = 1.8e-4;
            cfg.ion_mobility_density_ratio_floor = 0.5;
        }
        if (tc.table_electrons) cfg.electron_mobility_model = "en_table_flux_v1";
        amrex::DistributionMapping const dm;
        rrea::LowEnergyFluidState fluid(grid.ba(), dm, 1);
        std::vector<double> ne(n), np(n), nn(n), rho(n), den(n, cfg.transport_density_ratio);
        for (int k = 0; k < n; ++k) {
            // a negative stored density fails the reference's post-transport
            // check; transport inputs are nonnegative
            ne[k] = std::max(density(g), 0.0);
            np[k] = std::max(density(g), 0.0);
            nn[k] = std::max(density(g), 0.0);
            rho[k] = (g.uni() - 0.5) * 1.0e-5;
            if (tc.density_field) den[k] = g.logu(0.3, 1.2);
        }
        put_cells(fluid.LowElectronDensity(), grid, ne);
        put_cells(fluid.PositiveIonDensity(), grid, np);
        put_cells(fluid.NegativeIonDensity(), grid, nn);
        put_cells(fluid.FluidChargeDensity(), grid, rho);
        amrex::MultiFab den_mf(grid.ba(), dm, 1, 1);
        put_cells(den_mf, grid, den);
        amrex::MultiFab const* den_ptr = tc.density_field ? &den_mf : nullptr;
        // face fields
        amrex::BoxArray const bar = amrex::convert(grid.ba(), amrex::IntVect(1, 0));
        amrex::BoxArray const baz = amrex::convert(grid.ba(), amrex::IntVect(0, 1));
        amrex::MultiFab efr(bar, dm, 1, 0), efz(baz, dm, 1, 0), fr(bar, dm, 3, 0), fz(baz, dm, 3, 0);
        std::vector<double> ver(static_cast<std::size_t>(nr + 1) * nz), vez(static_cast<std::size_t>(nr) * (nz + 1));
        for (int j = 0; j < nz; ++j)
            for (int i = 0; i <= nr; ++i) {
                double const u = g.uni();
                double const v = u < 0.08 ? 0.0 : tc.e_scale * (2.0 * g.uni() - 1.0);
                ver[static_cast<std::size_t>(i + (nr + 1) * j)] = v;
                efr.at(i, j) = v;
            }
        for (int j = 0; j <= nz; ++j)
            for (int i = 0; i < nr; ++i) {
                double const u = g.uni();
                double v = u < 0.08 ? 0.0 : tc.e_scale * (2.0 * g.uni() - 1.0);
                if (grid.periodic_z && j == nz) v = vez[static_cast<std::size_t>(i)];
                vez[static_cast<std::size_t>(i + nr * j)] = v;
                efz.at(i, j) = v;
            }
        // closure cell fields (en_table_flux_v1): mobility and the field-aligned
        // tensor from the dry-air table at the cell-averaged field
        amrex::MultiFab mu(grid.ba(), dm, 1, 1), dtens(grid.ba(), dm, 3, 1);
        std::vector<double> vmu(n, 0.0), vd(3 * static_cast<std::size_t>(n), 0.0);
        if (tc.table_electrons) {
            amrex::MultiFab er_c(grid.ba(), dm, 1, 1), ez_c(grid.ba(), dm, 1, 1), dmf(grid.ba(), dm, 1, 1);
            for (int j = 0; j < nz; ++j)
                for (int i = 0; i < nr; ++i) {
                    er_c.at(i, j) = 0.5 * (efr.at(i, j) + efr.at(i + 1, j));
                    ez_c.at(i, j) = 0.5 * (efz.at(i, j) + efz.at(i, j + 1));
                    dmf.at(i, j) = den[static_cast<std::size_t>(i + nr * j)];
                }
            rrea::LowEnergyClosureFieldDiagnostics d;
            rrea::BuildElectronClosureCellFields(grid.geom(), er_c, ez_c, &dmf, cfg.transport_density_ratio, closure,
                                                 nullptr, nullptr, &mu, nullptr, &dtens, d);
            vmu = get_cells(mu, grid);
            for (int c = 0; c < 3; ++c) {
                auto const v = get_cells(dtens, grid, c);
                std::copy(v.begin(), v.end(), vd.begin() + static_cast<std::ptrdiff_t>(c) * n);
            }
        }
        amrex::MultiFab const* mu_ptr = tc.table_electrons ? &mu : nullptr;
        amrex::MultiFab const* d_ptr = tc.table_electrons ? &dtens : nullptr;

        fluid.ComputeConductivity(cfg, den_ptr, mu_ptr);
        std::vector<double> const sigma = get_cells(fluid.Conductivity(), grid);
        std::vector<double> const tau = get_cells(fluid.MaxwellTime(), grid);
        fluid.PrepareExplicitCarrierTransport(grid.geom(), cfg, den_ptr);
        auto const fd = fluid.BuildExplicitFaceTransport(tc.dt, grid.geom(), {&efr, &efz}, cfg, {&fr, &fz}, mu_ptr, d_ptr);
        std::vector<double> raw;
        for (int s = 0; s < 3; ++s) append(raw, get_faces(fr, nr + 1, nz, s));
        for (int s = 0; s < 3; ++s) append(raw, get_faces(fz, nr, nz + 1, s));
        fluid.ApplyExplicitCarrierTransport(tc.dt, grid.geom(), {&fr, &fz}, cfg, den_ptr, true);
        auto const& cd = fluid.LastCarrierDriftDiagnostics();

        setup.insert(setup.end(),
                     {static_cast<double>(nr), static_cast<double>(nz), grid.r_lo, grid.z_lo, grid.dr, grid.dz,
                      grid.periodic_z ? 1.0 : 0.0, tc.ions ? 1.0 : 0.0, tc.reduced_ions ? 1.0 : 0.0,
                      tc.table_electrons ? 1.0 : 0.0, tc.density_field ? 1.0 : 0.0, tc.dt,
                      cfg.positive_ion_mobility_m2_per_vs, cfg.negative_ion_mobility_m2_per_vs,
                      cfg.electron_mobility_m2_per_vs, cfg.positive_ion_reduced_mobility_stp_m2_per_vs,
                      cfg.negative_ion_reduced_mobility_stp_m2_per_vs, cfg.ion_mobility_density_ratio_floor,
                      cfg.ion_drift_cfl, cfg.transport_density_ratio,
                      // diagnostics
                      fd.max_face_conductivity_siemens_per_m, fd.max_explicit_diffusion_number,
                      cd.unlimited_max_outgoing_cfl, cd.min_outflow_scale, cd.limited_outflow_fraction,
                      cd.limited_electron_number_fraction, cd.max_outgoing_cfl, cd.max_drift_speed_m_per_s,
                      cd.cfl_dt_s, cd.positive_ion_center_r_m, cd.positive_ion_center_z_m,
                      cd.negative_ion_center_r_m, cd.negative_ion_center_z_m,
                      cd.density_ratio_at_positive_ion_center, cd.mu_pos_at_positive_ion_center_m2_per_vs});
        std::vector<double> in;
        for (auto const* v : {&ne, &np, &nn, &rho, &den, &vmu}) append(in, *v);
        append(in, vd);
        append(in, ver);
        append(in, vez);
        write_f8("ref_fluid_transport_in_" + std::to_string(setup.size() / 35 - 1), 1, in);
        std::vector<double> out;
        append(out, sigma);
        append(out, tau);
        append(out, raw);
        for (int s = 0; s < 3; ++s) append(out, get_faces(fr, nr + 1, nz, s));
        for (int s = 0; s < 3; ++s) append(out, get_faces(fz, nr, nz + 1, s));
        append(out, get_cells(fluid.PositiveIonDensity(), grid));
        append(out, get_cells(fluid.NegativeIonDensity(), grid));
        append(out, get_cells(fluid.LowElectronDensity(), grid));
        append(out, get_cells(fluid.FluidChargeDensity(), grid));
        write_f8("ref_fluid_transport_out_" + std::to_string(setup.size() / 35 - 1), 1, out);
        (void)inputs;
        (void)outputs;
    }
    write_f8("ref_fluid_transport_setup", 35, setup);
}

}  // namespace

int main(int argc, char** argv)
{
    if (argc < 3) {
        std::fprintf(stderr, "usage: ref_golden_fluid <closure.csv> <outdir>\n");
        return 2;
    }
    g_outdir = argv[2];
    try {
        auto const closure = rrea::LowEnergyElectronClosure::Load(argv[1]);
        Gen g(20261204ULL);
        reaction_cases(g, closure);
        neutral_cases(g);
        closure_cases(g, closure);
        transport_cases(g, closure);
        std::printf("fluid golden fixtures written to %s\n", g_outdir.c_str());
    } catch (std::exception const& e) {
        std::fprintf(stderr, "ref_golden_fluid failed: %s\n", e.what());
        return 1;
    }
    return 0;
}
