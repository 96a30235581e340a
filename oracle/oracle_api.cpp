// ORACLE — test infrastructure only.  C entry points of the CPU restatement
// for ctypes (oracle/oracle.py).  Never linked into the shipped library.
#include "oracle_core.hpp"
#include "interleave.hpp"
#include "interleave_scenarios.hpp"
#include "fluid.hpp"

#include <cmath>
#include <cstring>
#include <memory>
#include <string>

namespace {

std::unique_ptr<rrea_host::TableSet> g_tables;
oracle::StepOutputs g_out;
oracle::CellSources g_cells;
std::string g_error;
std::unique_ptr<rrea_host::ClosureTable> g_closure;

int guard(std::exception const& e)
{
    g_error = e.what();
    if (auto const* oe = dynamic_cast<oracle::OracleError const*>(&e)) {
        return oe->code;
    }
    return RREA_GPU_ERR_TABLES;
}

}  // namespace

namespace {
// The oracle's restated skeletons behind the scenario runner.
struct OracleSkeleton {
    template <class... P>
    static void events(double b, double e, double& k, double cut, int channels, uint64_t max_ordinal, P&&... p)
    {
        oracle::RunChargedEventInterleave(b, e, k, cut, channels, max_ordinal, "scenario", std::forward<P>(p)...);
    }
    template <class... P>
    static void substeps(uint64_t n, double& k, double cut, uint64_t& completed, bool& exited, P&&... p)
    {
        oracle::RunChargedSubstepInterleave(n, k, cut, completed, exited, std::forward<P>(p)...);
    }
};
}  // namespace

extern "C" {

int oracle_load_tables(char const* path)
{
    try {
        auto t = std::make_unique<rrea_host::TableSet>();
        t->Load(path);
        g_tables = std::move(t);
        return 0;
    } catch (std::exception const& e) {
        return guard(e);
    }
}

void oracle_last_error(char* buf, size_t size)
{
    if (size == 0) return;
    std::strncpy(buf, g_error.c_str(), size - 1);
    buf[size - 1] = '\0';
}

int oracle_primitive(int which, double const* in, int64_t n, double* out)
{
    if (!g_tables) return RREA_GPU_ERR_NOT_READY;
    try {
        return oracle::RunPrimitive(*g_tables, which, in, n, out);
    } catch (std::exception const& e) {
        return guard(e);
    }
}

void oracle_rng(uint64_t const* keys, int64_t n, uint64_t* counter, double* uniform)
{
    for (int64_t i = 0; i < n; ++i) {
        uint64_t const* k = keys + 5 * i;
        counter[i] = oracle::rng_counter(k[0], k[1], k[2], k[3], k[4]);
        uniform[i] = oracle::rng_uniform(k[0], k[1], k[2], k[3], k[4]);
    }
}

// Arena export so tests can compare the host loader against the device copy.
// Binds the altitude density profile (n == 0 unbinds it).
int oracle_set_density_profile(double const* altitude_m, double const* density_kg_m3, int64_t n,
                               double altitude_msl_at_z0_m, double reference_density_kg_m3)
{
    try {
        oracle::DensityProfile p;
        if (n > 0) {
            p.altitude_m.assign(altitude_m, altitude_m + n);
            p.density_kg_m3.assign(density_kg_m3, density_kg_m3 + n);
        }
        p.altitude_msl_at_z0_m = altitude_msl_at_z0_m;
        p.reference_density_kg_m3 = reference_density_kg_m3;
        oracle::SetDensityProfile(std::move(p));
        return 0;
    } catch (std::exception const& e) {
        return guard(e);
    }
}

// out[i] = the bound profile's density at altitude_m[i] (mode 0) or the
// transport density ratio at axial position z = altitude_m[i] (mode 1).
int oracle_density_query(int mode, double const* in, int64_t n, double uniform_ratio, double* out)
{
    try {
        for (int64_t i = 0; i < n; ++i) {
            out[i] = mode == 0 ? oracle::BoundDensityProfile().interpolate(in[i])
                               : oracle::DensityRatioAtZ(uniform_ratio, in[i]);
        }
        return 0;
    } catch (std::exception const& e) {
        return guard(e);
    }
}

int64_t oracle_arena_size() { return g_tables ? static_cast<int64_t>(g_tables->arena().size()) : 0; }

int charged_step(bool positron, rrea_gpu_config const* cfg, double const* er, double const* ez, double const* bt,
                 double const* amb_er, double const* amb_ez, int32_t step, double dt_s, rrea_gpu_tile const* tile);

int oracle_electron_step(rrea_gpu_config const* cfg, double const* er, double const* ez, double const* bt,
                         double const* amb_er, double const* amb_ez, int32_t step, double dt_s,
                         rrea_gpu_tile const* tile)
{
    return charged_step(false, cfg, er, ez, bt, amb_er, amb_ez, step, dt_s, tile);
}

int oracle_positron_step(rrea_gpu_config const* cfg, double const* er, double const* ez, double const* bt,
                         double const* amb_er, double const* amb_ez, int32_t step, double dt_s,
                         rrea_gpu_tile const* tile)
{
    return charged_step(true, cfg, er, ez, bt, amb_er, amb_ez, step, dt_s, tile);
}

int charged_step(bool positron, rrea_gpu_config const* cfg, double const* er, double const* ez, double const* bt,
                 double const* amb_er, double const* amb_ez, int32_t step, double dt_s, rrea_gpu_tile const* tile)
{
    if (!g_tables) return RREA_GPU_ERR_NOT_READY;
    try {
        oracle::FieldGrid fg;
        fg.nr = cfg->nr;
        fg.nz = cfg->nz;
        fg.dr = (cfg->r_hi - cfg->r_lo) / cfg->nr;
        fg.dz = (cfg->z_hi - cfg->z_lo) / cfg->nz;
        fg.z_lo = cfg->z_lo;
        std::size_t const ner = static_cast<std::size_t>(cfg->nr + 1) * cfg->nz;
        std::size_t const nez = static_cast<std::size_t>(cfg->nr) * (cfg->nz + 1);
        std::size_t const nbt = static_cast<std::size_t>(cfg->nr + 1) * (cfg->nz + 1);
        fg.er.assign(er, er + ner);
        fg.ez.assign(ez, ez + nez);
        fg.bt.assign(bt, bt + nbt);
        fg.amb_er.assign(amb_er, amb_er + ner);
        fg.amb_ez.assign(amb_ez, amb_ez + nez);
        oracle::ChargedTile t;
        t.n = tile->n;
        t.r = tile->r; t.z = tile->z; t.theta = tile->theta;
        t.ux = tile->ux; t.uy = tile->uy; t.uz = tile->uz; t.w = tile->w;
        t.prev_r = tile->prev_r; t.prev_z = tile->prev_z; t.prev_theta = tile->prev_theta;
        t.prev_ux = tile->prev_ux; t.prev_uy = tile->prev_uy; t.prev_uz = tile->prev_uz;
        t.id = tile->id;
        t.cpu = tile->cpu;
        g_out.clear();
        if (positron) {
            oracle::ApplyPositronTransport(*g_tables, *cfg, fg, step, dt_s, t, g_out);
        } else {
            oracle::ApplyElectronTransport(*g_tables, *cfg, fg, step, dt_s, t, g_out);
        }
        g_cells.nr = cfg->nr;
        g_cells.nz = cfg->nz;
        for (auto& f : g_cells.f) f.assign(static_cast<std::size_t>(cfg->nr) * cfg->nz, 0.0);
        oracle::DepositSources(*cfg, g_out.sources, cfg->low_energy_cutoff_eV, g_cells);
        return 0;
    } catch (std::exception const& e) {
        return guard(e);
    }
}

int oracle_photon_step(rrea_gpu_config const* cfg, int32_t step, double dt_s, rrea_gpu_tile const* tile)
{
    if (!g_tables) return RREA_GPU_ERR_NOT_READY;
    try {
        oracle::ChargedTile t;
        t.n = tile->n;
        t.r = tile->r; t.z = tile->z; t.theta = tile->theta;
        t.ux = tile->ux; t.uy = tile->uy; t.uz = tile->uz; t.w = tile->w;
        t.prev_r = tile->prev_r; t.prev_z = tile->prev_z; t.prev_theta = tile->prev_theta;
        t.prev_ux = tile->prev_ux; t.prev_uy = tile->prev_uy; t.prev_uz = tile->prev_uz;
        t.id = tile->id;
        t.cpu = tile->cpu;
        g_out.clear();
        oracle::ApplyPhotonTransport(*g_tables, *cfg, step, dt_s, t, g_out);
        g_cells.nr = cfg->nr;
        g_cells.nz = cfg->nz;
        for (auto& f : g_cells.f) f.assign(static_cast<std::size_t>(cfg->nr) * cfg->nz, 0.0);
        oracle::DepositSources(*cfg, g_out.sources, cfg->low_energy_cutoff_eV, g_cells);
        return 0;
    } catch (std::exception const& e) {
        return guard(e);
    }
}

// Net-chord current of `n` segment rows (kind, a0..a6, faces) on the padded
// grid of `cfg` (O/RreaWarpXCoupling.cpp:417-544): padded index-space rho,
// Jr, Jz and the physical current densities.
int oracle_deposit_segments(rrea_gpu_config const* cfg, double dt_s, double const* rows, int64_t n, double* rho,
                            double* jr, double* jz, double* jr_phys, double* jz_phys)
{
    try {
        if (cfg->periodic_z) {
            throw oracle::OracleError(RREA_GPU_ERR_ARGUMENT, "net-chord current needs a non-periodic z domain");
        }
        oracle::NetChordGrid g;
        g.Reset(*cfg);
        std::vector<oracle::Segment> segs(static_cast<std::size_t>(n));
        for (int64_t i = 0; i < n; ++i) {
            double const* r = rows + 9 * i;
            oracle::Segment& s = segs[static_cast<std::size_t>(i)];
            s.kind = static_cast<int>(r[0]);
            for (int c = 0; c < 7; ++c) s.a[c] = r[1 + c];
            s.channel = 0;
            s.faces = static_cast<uint32_t>(r[8]);
            s.parent_index = i;
        }
        oracle::DepositNetChords(g, dt_s, segs);
        std::vector<double> jrp, jzp;
        oracle::ConvertNetChordCurrent(g, jrp, jzp);
        std::copy(g.rho.begin(), g.rho.end(), rho);
        std::copy(g.jr.begin(), g.jr.end(), jr);
        std::copy(g.jz.begin(), g.jz.end(), jz);
        std::copy(jrp.begin(), jrp.end(), jr_phys);
        std::copy(jzp.begin(), jzp.end(), jz_phys);
        return 0;
    } catch (std::exception const& e) {
        return guard(e);
    }
}

// Maxwell field step in place on (er, ez, bt) with face current (jr, jz).
int oracle_advance_maxwell(int nr, int nz, double dr, double dz, double dt_s, int substeps, double* er, double* ez,
                           double* bt, double const* jr, double const* jz)
{
    try {
        oracle::MaxwellField f;
        f.nr = nr;
        f.nz = nz;
        f.dr = dr;
        f.dz = dz;
        std::size_t const ner = static_cast<std::size_t>(nr + 1) * nz;
        std::size_t const nez = static_cast<std::size_t>(nr) * (nz + 1);
        std::size_t const nbt = static_cast<std::size_t>(nr + 1) * (nz + 1);
        f.er.assign(er, er + ner);
        f.ez.assign(ez, ez + nez);
        f.bt.assign(bt, bt + nbt);
        std::vector<double> const vjr(jr, jr + ner), vjz(jz, jz + nez);
        oracle::AdvanceMaxwell(f, dt_s, substeps, vjr, vjz);
        std::copy(f.er.begin(), f.er.end(), er);
        std::copy(f.ez.begin(), f.ez.end(), ez);
        std::copy(f.bt.begin(), f.bt.end(), bt);
        return 0;
    } catch (std::exception const& e) {
        return guard(e);
    }
}

namespace {
std::vector<oracle::Secondary> g_survivors;
}

// DrainAndCommitSecondaries over `n` initial secondaries (rrea_gpu_secondary
// records in the phases' order): survivors are kept for oracle_survivors, the
// newborns' sources, segments and cell grids replace the step outputs.
int oracle_drain(rrea_gpu_config const* cfg, double const* er, double const* ez, double const* bt,
                 double const* amb_er, double const* amb_ez, int32_t step, double dt_s,
                 rrea_gpu_secondary const* initial, int64_t n, int64_t* n_survivors)
{
    if (!g_tables) return RREA_GPU_ERR_NOT_READY;
    try {
        oracle::FieldGrid fg;
        fg.nr = cfg->nr;
        fg.nz = cfg->nz;
        fg.dr = (cfg->r_hi - cfg->r_lo) / cfg->nr;
        fg.dz = (cfg->z_hi - cfg->z_lo) / cfg->nz;
        fg.z_lo = cfg->z_lo;
        std::size_t const ner = static_cast<std::size_t>(cfg->nr + 1) * cfg->nz;
        std::size_t const nez = static_cast<std::size_t>(cfg->nr) * (cfg->nz + 1);
        std::size_t const nbt = static_cast<std::size_t>(cfg->nr + 1) * (cfg->nz + 1);
        fg.er.assign(er, er + ner);
        fg.ez.assign(ez, ez + nez);
        fg.bt.assign(bt, bt + nbt);
        fg.amb_er.assign(amb_er, amb_er + ner);
        fg.amb_ez.assign(amb_ez, amb_ez + nez);
        std::vector<oracle::Secondary> init(static_cast<std::size_t>(n));
        for (int64_t i = 0; i < n; ++i) {
            rrea_gpu_secondary const& r = initial[i];
            oracle::Secondary& s = init[static_cast<std::size_t>(i)];
            s.species = r.species;
            s.process = r.process;
            s.root_species = r.root_species;
            s.parent_index = r.parent_index;
            s.root_key = r.root_key;
            s.lineage = r.lineage;
            s.x = r.x; s.y = r.y; s.z = r.z;
            s.dx = r.dir_x; s.dy = r.dir_y; s.dz = r.dir_z;
            s.w = r.weight;
            s.energy = r.energy_eV;
            s.birth = r.birth_fraction;
        }
        g_out.clear();
        oracle::DrainSecondaries(*g_tables, *cfg, fg, step, dt_s, init, g_survivors, g_out);
        g_cells.nr = cfg->nr;
        g_cells.nz = cfg->nz;
        for (auto& f : g_cells.f) f.assign(static_cast<std::size_t>(cfg->nr) * cfg->nz, 0.0);
        oracle::DepositSources(*cfg, g_out.sources, cfg->low_energy_cutoff_eV, g_cells);
        *n_survivors = static_cast<int64_t>(g_survivors.size());
        return 0;
    } catch (std::exception const& e) {
        return guard(e);
    }
}

void oracle_survivors(rrea_gpu_secondary* out)
{
    for (std::size_t i = 0; i < g_survivors.size(); ++i) {
        auto const& s = g_survivors[i];
        rrea_gpu_secondary& o = out[i];
        o.species = s.species;
        o.process = s.process;
        o.root_species = s.root_species;
        o.pad = 0;
        o.parent_index = s.parent_index;
        o.root_key = s.root_key;
        o.lineage = s.lineage;
        o.x = s.x; o.y = s.y; o.z = s.z;
        o.dir_x = s.dx; o.dir_y = s.dy; o.dir_z = s.dz;
        o.weight = s.w;
        o.energy_eV = s.energy;
        o.birth_fraction = s.birth;
    }
}


// Trace of scripted scenario `seed` through the oracle's event (kind 0) or
// substep (kind 1) skeleton: records of {code, a, b, c}; *n receives the
// record count (the trace is truncated to `cap` records).
void oracle_interleave_trace(int kind, uint64_t seed, double* out, int64_t cap, int64_t* n)
{
    namespace is = interleave_scenarios;
    is::Trace const t = kind == 0 ? is::run_event_scenario<OracleSkeleton>(is::event_scenario(seed))
                                  : is::run_substep_scenario<OracleSkeleton>(is::substep_scenario(seed));
    int64_t const records = static_cast<int64_t>(t.rec.size() / 4);
    *n = records;
    for (int64_t i = 0; i < records && i < cap; ++i) {
        for (int j = 0; j < 4; ++j) out[4 * i + j] = t.rec[static_cast<std::size_t>(4 * i + j)];
    }
}

// The photon energy-flow check on n rows of {kind, w, incident, x1, x2, x3,
// has_recoil, local}; ok[i] = 1 where the row passes.
void oracle_photon_flow(double const* rows, int64_t n, int32_t* ok)
{
    for (int64_t i = 0; i < n; ++i) {
        double const* r = rows + 8 * i;
        ok[i] = oracle::PhotonFlowValid(static_cast<int>(r[0]), r[1], r[2], r[3], r[4], r[5], r[6] != 0.0, r[7]) ? 1 : 0;
    }
}

// Elastic angle draws by branch (GS, Wentzel-VI, isotropic, single
// scatter) since the last reset; reset != 0 clears them after reading.
void oracle_elastic_branches(uint64_t* out4, int reset)
{
    for (int k = 0; k < 4; ++k) {
        out4[k] = reset ? oracle::g_elastic_branch[k].exchange(0) : oracle::g_elastic_branch[k].load();
    }
}

void oracle_counts(int64_t* n_sec, int64_t* n_src, int64_t* n_seg)
{
    *n_sec = static_cast<int64_t>(g_out.secondaries.size());
    *n_src = static_cast<int64_t>(g_out.sources.size());
    *n_seg = static_cast<int64_t>(g_out.segments.size());
}

// Secondaries in the rrea_gpu_secondary layout.
void oracle_secondaries(rrea_gpu_secondary* out)
{
    for (std::size_t i = 0; i < g_out.secondaries.size(); ++i) {
        auto const& s = g_out.secondaries[i];
        rrea_gpu_secondary& o = out[i];
        o.species = s.species;
        o.process = s.process;
        o.root_species = s.root_species;
        o.pad = 0;
        o.parent_index = s.parent_index;
        o.root_key = s.root_key;
        o.lineage = s.lineage;
        o.x = s.x; o.y = s.y; o.z = s.z;
        o.dir_x = s.dx; o.dir_y = s.dy; o.dir_z = s.dz;
        o.weight = s.w;
        o.energy_eV = s.energy;
        o.birth_fraction = s.birth;
    }
}

// Sources as rows (kind, r, z, w, secondary_energy, energy_loss, parent).
void oracle_sources(double* out)
{
    for (std::size_t i = 0; i < g_out.sources.size(); ++i) {
        auto const& s = g_out.sources[i];
        double* o = out + 7 * i;
        o[0] = s.kind; o[1] = s.r; o[2] = s.z; o[3] = s.w; o[4] = s.secondary_energy; o[5] = s.energy_loss;
        o[6] = static_cast<double>(s.parent_index);
    }
}

// Segments as rows (kind, a0..a6, channel, faces, parent).
void oracle_segments(double* out)
{
    for (std::size_t i = 0; i < g_out.segments.size(); ++i) {
        auto const& s = g_out.segments[i];
        double* o = out + 11 * i;
        o[0] = s.kind;
        for (int c = 0; c < 7; ++c) o[1 + c] = s.a[c];
        o[8] = static_cast<double>(s.channel);
        o[9] = s.faces;
        o[10] = static_cast<double>(s.parent_index);
    }
}

void oracle_diagnostics(uint64_t* subcycles, uint64_t* events, int32_t* disposition)
{
    for (std::size_t i = 0; i < g_out.subcycles.size(); ++i) {
        subcycles[i] = g_out.subcycles[i];
        events[i] = g_out.events[i];
        disposition[i] = g_out.disposition[i];
    }
}

int oracle_set_planes(double const* z, int64_t n)
{
    std::vector<double> planes(z, z + n);
    for (int64_t i = 0; i < n; ++i) {
        if (!std::isfinite(z[i]) || (i > 0 && !(z[i] > z[i - 1]))) return RREA_GPU_ERR_ARGUMENT;
    }
    oracle::SetPlanes(std::move(planes));
    return 0;
}

// The last step's (or drain's) plane crossings accumulated from zero, 10 per plane.
int oracle_plane_flux(double* out)
{
    std::vector<double> bins(oracle::Planes().size() * 10U, 0.0);
    if (!oracle::AccumulatePlaneCrossings(g_out.crossings, bins)) return RREA_GPU_ERR_INVALID_STATE;
    std::memcpy(out, bins.data(), bins.size() * sizeof(double));
    return 0;
}

// Crossing enumeration of segments (z0, z1) over the given planes: per
// segment up to `cap` (plane, fraction, direction) triples; counts[i] the
// number (-1 on invalid geometry).
void oracle_plane_enumerate(double const* segs, int64_t n, double const* planes, int64_t n_planes, int64_t cap,
                            double* out, int64_t* counts)
{
    std::vector<double> pl(planes, planes + n_planes);
    for (int64_t i = 0; i < n; ++i) {
        int64_t c = 0;
        bool const ok = oracle::ForEachPlaneCrossing(segs[2 * i], segs[2 * i + 1], pl,
                                                     [&](std::size_t p, double f, int d) {
                                                         if (c < cap) {
                                                             out[(i * cap + c) * 3 + 0] = static_cast<double>(p);
                                                             out[(i * cap + c) * 3 + 1] = f;
                                                             out[(i * cap + c) * 3 + 2] = d;
                                                         }
                                                         ++c;
                                                     });
        counts[i] = ok ? c : -1;
    }
}

// Crossings (plane, direction, weight, r, local, mev) added one by one as
// RreaPlaneFluxAccumulator::AddCrossing adds them: an invalid one changes
// nothing and gets ok = 0.  out: n_planes x 10 values.
void oracle_plane_accumulate(double const* rows, int64_t n, int64_t n_planes, double* out, int32_t* ok)
{
    std::vector<double> bins(static_cast<std::size_t>(n_planes) * 10U, 0.0);
    for (int64_t i = 0; i < n; ++i) {
        double const* r = rows + 6 * i;
        std::vector<oracle::PlaneCrossing> one{oracle::PlaneCrossing{static_cast<int>(r[0]), static_cast<int>(r[1]),
                                                                     r[2], r[3], r[4] != 0.0, r[5] != 0.0}};
        std::vector<double> trial = bins;
        ok[i] = oracle::AccumulatePlaneCrossings(one, trial) ? 1 : 0;
        if (ok[i]) bins.swap(trial);
    }
    std::memcpy(out, bins.data(), bins.size() * sizeof(double));
}

void oracle_cell_sources(double* out5)
{
    std::size_t const n = static_cast<std::size_t>(g_cells.nr) * g_cells.nz;
    for (int f = 0; f < 5; ++f) {
        for (std::size_t i = 0; i < n; ++i) out5[f * n + i] = g_cells.f[f].empty() ? 0.0 : g_cells.f[f][i];
    }
}

// ---- carrier fluid (oracle/fluid.cpp)
int oracle_fluid_react(rrea_gpu_fluid_config const* cfg, int64_t n, double dt, double* ne, double* np, double* nn,
                       double* se, double* sp, double* sn, double* rho, double const* nu, int clear, double* residual)
{
    try {
        *residual = oracle_fluid::react(*cfg, static_cast<std::size_t>(n), dt, ne, np, nn, se, sp, sn, rho, nu, clear != 0);
        return 0;
    } catch (std::exception const& e) {
        return guard(e);
    }
}

int oracle_fluid_max_reaction_frequency(rrea_gpu_fluid_config const* cfg, int64_t n, double const* ne,
                                        double const* np, double const* nn, double const* nu, double* out)
{
    try {
        *out = oracle_fluid::max_reaction_frequency(*cfg, static_cast<std::size_t>(n), ne, np, nn, nu);
        return 0;
    } catch (std::exception const& e) {
        return guard(e);
    }
}

int oracle_fluid_conductivity(rrea_gpu_fluid_config const* cfg, int64_t n, double const* ne, double const* np,
                              double const* nn, double const* chi, double const* mu, double* sigma, double* tau)
{
    try {
        oracle_fluid::conductivity(*cfg, static_cast<std::size_t>(n), ne, np, nn, chi, mu, sigma, tau);
        return 0;
    } catch (std::exception const& e) {
        return guard(e);
    }
}

void oracle_fluid_charge_density(int64_t n, double const* ne, double const* np, double const* nn, double* rho)
{
    oracle_fluid::charge_density(static_cast<std::size_t>(n), ne, np, nn, rho);
}

int oracle_fluid_load_closure(char const* path)
{
    try {
        g_closure = std::make_unique<rrea_host::ClosureTable>(rrea_host::load_closure_table(path));
        return 0;
    } catch (std::exception const& e) {
        g_error = e.what();
        return RREA_GPU_ERR_TABLES;
    }
}

int oracle_fluid_closure_fields(int nr, int nz, double r_lo, double z_lo, double dr, double dz, double scalar_chi,
                                double const* er, double const* ez, double const* chi, double const* ne,
                                double const* src, double* mu, double* nu, double* diff3, double* diag8)
{
    try {
        if (!g_closure) oracle::fail(RREA_GPU_ERR_NOT_READY, "no closure table loaded");
        oracle_fluid::ClosureDiag d;
        oracle_fluid::closure_fields(*g_closure, oracle_fluid::Grid{nr, nz, r_lo, z_lo, dr, dz, false}, scalar_chi, er,
                                     ez, chi, ne, src, mu, nu, diff3, d);
        double const v[8] = {d.min_en, d.max_en, d.held_below, d.above_range, d.invalid, d.electron_count,
                             d.held_below_count, d.source_rate};
        std::memcpy(diag8, v, sizeof(v));
        return 0;
    } catch (std::exception const& e) {
        return guard(e);
    }
}

int oracle_fluid_transport(rrea_gpu_fluid_config const* cfg, int nr, int nz, double r_lo, double z_lo, double dr,
                           double dz, int periodic_z, double dt, double* n_pos, double* n_neg, double* n_e, double* rho,
                           double const* chi, double const* mu, double const* diff3, double const* efr,
                           double const* efz, double* flux_r, double* flux_z, double* raw_r, double* raw_z,
                           double* diag14)
{
    try {
        oracle_fluid::TransportDiag d;
        double* const dens[3] = {n_pos, n_neg, n_e};
        oracle_fluid::transport(*cfg, oracle_fluid::Grid{nr, nz, r_lo, z_lo, dr, dz, periodic_z != 0}, dt, dens, rho,
                                chi, mu, diff3, efr, efz, flux_r, flux_z, raw_r, raw_z, d);
        double const v[14] = {d.max_face_conductivity, d.max_diffusion_number, d.unlimited_max_outgoing_cfl,
                              d.min_outflow_scale, d.limited_outflow_fraction, d.limited_electron_number_fraction,
                              d.max_outgoing_cfl, d.max_drift_speed, d.cfl_dt, d.pos_center_r, d.pos_center_z,
                              d.neg_center_r, d.neg_center_z, d.density_ratio_at_pos_center};
        std::memcpy(diag14, v, sizeof(v));
        return 0;
    } catch (std::exception const& e) {
        return guard(e);
    }
}

int oracle_fluid_coupled_step(rrea_gpu_fluid_config const* cfg, int nr, int nz, double z_lo, double dr, double dz,
                              double dt, double* er, double* ez, double* bt, double const* amb_er, double const* amb_ez,
                              double const* jr_kin, double const* jz_kin, double* ne, double* np, double* nn, double* rho,
                              double* se, double* sp, double* sn, double const* chi, double* mu, double* nu,
                              double* diff3, double* sigma, double* diag8)
{
    try {
        std::size_t const n = static_cast<std::size_t>(nr) * nz;
        std::size_t const nfr = static_cast<std::size_t>(nr + 1) * nz, nfz = static_cast<std::size_t>(nr) * (nz + 1);
        oracle::MaxwellField f;
        f.nr = nr;
        f.nz = nz;
        f.dr = dr;
        f.dz = dz;
        f.er.assign(er, er + nfr);
        f.ez.assign(ez, ez + nfz);
        f.bt.assign(bt, bt + static_cast<std::size_t>(nr + 1) * (nz + 1));
        oracle_fluid::State st;
        st.ne.assign(ne, ne + n);
        st.np.assign(np, np + n);
        st.nn.assign(nn, nn + n);
        st.rho.assign(rho, rho + n);
        st.se.assign(se, se + n);
        st.sp.assign(sp, sp + n);
        st.sn.assign(sn, sn + n);
        oracle_fluid::CoupledDiag d;
        oracle_fluid::coupled_step(*cfg, g_closure.get(), oracle_fluid::Grid{nr, nz, 0.0, z_lo, dr, dz, false}, dt, f,
                                   std::vector<double>(amb_er, amb_er + nfr), std::vector<double>(amb_ez, amb_ez + nfz),
                                   std::vector<double>(jr_kin, jr_kin + nfr), std::vector<double>(jz_kin, jz_kin + nfz),
                                   st, chi, d);
        std::copy(f.er.begin(), f.er.end(), er);
        std::copy(f.ez.begin(), f.ez.end(), ez);
        std::copy(f.bt.begin(), f.bt.end(), bt);
        for (auto [dst, src] : {std::pair{ne, &st.ne}, {np, &st.np}, {nn, &st.nn}, {rho, &st.rho}, {se, &st.se},
                                {sp, &st.sp}, {sn, &st.sn}, {sigma, &st.sigma}}) {
            std::copy(src->begin(), src->end(), dst);
        }
        if (mu && !st.mu.empty()) std::copy(st.mu.begin(), st.mu.end(), mu);
        if (nu && !st.nu.empty()) std::copy(st.nu.begin(), st.nu.end(), nu);
        if (diff3 && !st.diff3.empty()) std::copy(st.diff3.begin(), st.diff3.end(), diff3);
        double const v[8] = {static_cast<double>(d.substeps), d.full_conduction, d.full_diffusion, d.full_reaction,
                             d.max_reaction_number, d.max_dt_sigma, d.max_diffusion_number, d.max_residual};
        std::memcpy(diag8, v, sizeof(v));
        return 0;
    } catch (std::exception const& e) {
        return guard(e);
    }
}

}  // extern "C"
