#include "table_set.hpp"

#include "json_lite.hpp"
#include "rreatbl.hpp"

#include <algorithm>
#include <cmath>
#include <fstream>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include <cstdint>

namespace rrea_host {

namespace {

std::string read_text(std::string const& path)
{
    std::ifstream in(path, std::ios::binary);
    if (!in) {
        throw std::runtime_error("cannot open " + path);
    }
    std::ostringstream s;
    s << in.rdbuf();
    return s.str();
}

std::string dir_of(std::string const& path)
{
    std::size_t const slash = path.find_last_of('/');
    return slash == std::string::npos ? std::string(".") : path.substr(0, slash);
}

struct Table1D {
    std::string interpolation;
    std::vector<double> x, y;
};

struct CondGroups {
    std::vector<double> primary;
    std::vector<std::vector<double>> u, v;
};

struct Angle {
    std::vector<double> e, p, u, omc;
};

// Conditional CDF rows grouped by consecutive primary energy
// (RreaInteractionTables.cpp:576-616) with the monotonicity contract of
// ValidateRreaConditionalCdfGroups (:1527-1578).
CondGroups group_conditional(std::vector<double> const& primaries,
                             std::vector<double> const& cdfs,
                             std::vector<double> const& values,
                             std::string const& label)
{
    CondGroups g;
    for (std::size_t i = 0; i < primaries.size(); ++i) {
        double const p = primaries[i];
        if (!(p > 0.0) || !(cdfs[i] >= 0.0 && cdfs[i] <= 1.0) || !(values[i] >= 0.0)) {
            throw std::runtime_error("conditional CDF row invalid: " + label);
        }
        if (g.primary.empty() || g.primary.back() != p) {
            if (!g.primary.empty() && p <= g.primary.back()) {
                throw std::runtime_error("conditional CDF groups not increasing: " + label);
            }
            g.primary.push_back(p);
            g.u.emplace_back();
            g.v.emplace_back();
        }
        if (!g.u.back().empty() && cdfs[i] <= g.u.back().back()) {
            throw std::runtime_error("conditional CDF u not increasing: " + label);
        }
        g.u.back().push_back(cdfs[i]);
        g.v.back().push_back(values[i]);
    }
    if (g.primary.size() < 2) {
        throw std::runtime_error("conditional CDF needs >= 2 groups: " + label);
    }
    for (std::size_t k = 0; k < g.primary.size(); ++k) {
        if (g.u[k].size() < 2 || g.u[k].front() != 0.0 || g.u[k].back() != 1.0) {
            throw std::runtime_error("conditional CDF group endpoints must be 0 and 1: " + label);
        }
        for (std::size_t n = 1; n < g.v[k].size(); ++n) {
            if (g.v[k][n] < g.v[k][n - 1]) {
                throw std::runtime_error("conditional CDF values not monotone: " + label);
            }
        }
    }
    return g;
}

// (energy, path) grouping of a GS/Wentzel inverse-CDF table
// (RreaInteractionTables.cpp:687-772).
Angle load_angle(std::string const& path)
{
    auto const c = ReadRreaTableContainer(path);
    auto const energies = c.column("primary_energy_eV");
    auto const paths = c.column("path_over_elastic_mfp");
    auto const us = c.column("cdf");
    auto const xs = c.column("one_minus_cos_theta");
    std::map<double, std::map<double, std::vector<std::pair<double, double>>>> by_ep;
    for (std::size_t i = 0; i < energies.size(); ++i) {
        by_ep[energies[i]][paths[i]].emplace_back(us[i], xs[i]);
    }
    Angle a;
    for (auto const& ep : by_ep) a.e.push_back(ep.first);
    for (auto const& pp : by_ep.begin()->second) a.p.push_back(pp.first);
    for (auto const& up : by_ep.begin()->second.begin()->second) a.u.push_back(up.first);
    std::size_t const ne = a.e.size(), np = a.p.size(), nu = a.u.size();
    if (ne < 2 || np < 2 || nu < 2) {
        throw std::runtime_error("angle table too small: " + path);
    }
    a.omc.assign(ne * np * nu, 1.0);
    for (std::size_t ie = 0; ie < ne; ++ie) {
        auto const& pm = by_ep.at(a.e[ie]);
        if (pm.size() != np) throw std::runtime_error("angle path count varies: " + path);
        for (std::size_t ip = 0; ip < np; ++ip) {
            auto const& v = pm.at(a.p[ip]);
            if (v.size() != nu) throw std::runtime_error("angle u count varies: " + path);
            for (std::size_t iu = 0; iu < nu; ++iu) {
                if (v[iu].first != a.u[iu]) throw std::runtime_error("angle u grid differs: " + path);
                double const x = v[iu].second;
                if (!(x > 0.0) || x > 2.0) throw std::runtime_error("angle omc out of (0,2]: " + path);
                if (iu > 0 && x > v[iu - 1].second) throw std::runtime_error("angle omc not monotone: " + path);
                a.omc[(ie * np + ip) * nu + iu] = x;
            }
        }
    }
    return a;
}

}  // namespace

int64_t TableSet::push(std::vector<double> const& values)
{
    int64_t const off = static_cast<int64_t>(m_arena.size());
    m_arena.insert(m_arena.end(), values.begin(), values.end());
    // Keep every array 32-byte aligned in the arena.
    while (m_arena.size() % 4 != 0) {
        m_arena.push_back(0.0);
    }
    return off;
}

int64_t TableSet::push_logs(std::vector<double> const& values, bool zero_for_nonpositive)
{
    std::vector<double> logs(values.size());
    for (std::size_t i = 0; i < values.size(); ++i) {
        logs[i] = (values[i] > 0.0 || !zero_for_nonpositive) ? std::log(values[i]) : 0.0;
    }
    return push(logs);
}

int64_t TableSet::push_inverse_spacing(int64_t off, int n)
{
    std::vector<double> inv(static_cast<std::size_t>(n), 0.0);
    for (int i = 1; i < n; ++i) {
        double const d = m_arena[static_cast<std::size_t>(off + i)] - m_arena[static_cast<std::size_t>(off + i - 1)];
        inv[static_cast<std::size_t>(i)] = d != 0.0 ? 1.0 / d : 0.0;
    }
    return push(inv);
}

int64_t TableSet::push_reciprocals(std::vector<double> const& values)
{
    std::vector<double> inv(values.size(), 0.0);
    for (std::size_t i = 0; i < values.size(); ++i) inv[i] = values[i] != 0.0 ? 1.0 / values[i] : 0.0;
    return push(inv);
}

void TableSet::Load(std::string const& config_path)
{
    m_loaded = false;
    m_arena.clear();
    m_index = RreaArenaIndex{};
    {
        // Table of the device logarithm, first in the arena (rrea_arena.h):
        // 1/F and log F split into two doubles, from long double arithmetic.
        std::vector<double> t(3 * RREA_ARENA_LOG_TABLE_ROWS);
        for (int j = 0; j < RREA_ARENA_LOG_TABLE_ROWS; ++j) {
            long double const F = 1.0L + static_cast<long double>(j) / 256.0L;
            long double const L = std::log(F);
            double const hi = static_cast<double>(L);
            t[3 * j] = static_cast<double>(1.0L / F);
            t[3 * j + 1] = hi;
            t[3 * j + 2] = static_cast<double>(L - static_cast<long double>(hi));
        }
        // F = 2: exactly the ln 2 split of the device code, so log(x) for x
        // just below 1 cancels e ln2 + log F exactly
        t[3 * 256 + 1] = 6.93147180559945286227e-01;
        t[3 * 256 + 2] = 2.31904681384629955842e-17;
        if (push(t) != RREA_ARENA_LOG_TABLE) throw std::logic_error("log table must open the arena");
        std::vector<double> x(2 * RREA_ARENA_EXP_TABLE_ROWS);
        for (int j = 0; j < RREA_ARENA_EXP_TABLE_ROWS; ++j) {
            long double const T = std::exp2(static_cast<long double>(j) / 128.0L);
            double const hi = static_cast<double>(T);
            x[2 * j] = hi;
            x[2 * j + 1] = static_cast<double>(T - static_cast<long double>(hi));
        }
        if (push(x) != RREA_ARENA_EXP_TABLE) throw std::logic_error("exp table must follow the log table");
    }
    std::string const dir = dir_of(config_path);
    JsonValue const cfg = ParseJson(read_text(config_path));
    if (cfg.str("schema_version") != "6") {
        throw std::runtime_error("only production schema 6 is supported");
    }
    JsonValue const& scattering = cfg.at("elastic_scattering_model");
    double const transition = scattering.num_or("transition_energy_eV", -1.0);
    double const few = scattering.num_or("few_collision_threshold_n", -1.0);
    double const iso = scattering.num_or("isotropic_above_path_n", -1.0);
    if (!(transition > 0.0) || !(few > 0.0) || !(iso > few)) {
        throw std::runtime_error("invalid elastic_scattering_model thresholds");
    }
    if (cfg.str_or("transport_model", "") != "rrea_mc_pic_v6_geant4_10_7_4p04") {
        throw std::runtime_error("unexpected transport_model");
    }

    static char const* const hot_names[RREA_T_COUNT] = {
        "electron_collision_stopping_air",
        "electron_soft_radiative_stopping_air",
        "electron_hard_moller_inverse_length_air",
        "electron_tracked_brems_inverse_length_air",
        "electron_elastic_transport_inverse_length_air",
        "positron_collision_stopping_air",
        "positron_soft_radiative_stopping_air",
        "positron_hard_bhabha_inverse_length_air",
        "positron_tracked_brems_inverse_length_air",
        "positron_elastic_transport_inverse_length_air",
        "positron_annihilation_inverse_length_air",
        "photon_compton_inverse_length_air",
        "photon_photoelectric_inverse_length_air",
        "photon_pair_nuclear_inverse_length_air",
        "photon_pair_triplet_inverse_length_air",
    };
    static char const* const cdf_names[RREA_C_COUNT] = {
        "electron_moller_secondary_cdf_air",
        "positron_hard_bhabha_secondary_cdf_air",
        "brems_photon_energy_cdf_air",
        "positron_brems_photon_energy_cdf_air",
    };

    std::vector<double> pe_primary, pe_prob_sum;
    std::vector<std::vector<double>> pe_rows_u, pe_rows_b;
    std::map<std::string, Table1D> tables;
    std::map<std::string, CondGroups> cdfs;
    std::map<std::string, Angle> angles;
    std::map<std::string, std::vector<std::vector<double>>> elastic;  // x, mfp, eta, transport

    JsonValue const& list = cfg.at("tables");
    for (auto const& obj : list.items) {
        std::string const name = obj.str("name");
        std::string const kind = obj.str_or("table_kind", "");
        std::string const path = dir + "/" + obj.str("path");
        if (kind == "gs_angle_cdf_2d" || kind == "wentzel_vi_angle_cdf_2d") {
            angles[name] = load_angle(path);
            continue;
        }
        if (name == "electron_elastic_mfp_air" || name == "positron_elastic_mfp_air") {
            auto const c = ReadRreaTableContainer(path);
            std::vector<std::vector<double>> cols = {
                c.column("primary_energy_eV"), c.column("elastic_mfp_m_stp"),
                c.column("screening_eta"), c.column("transport_mfp_m_stp")};
            for (std::size_t i = 0; i < cols[0].size(); ++i) {
                if (!(cols[0][i] > 0.0) || !(cols[1][i] > 0.0) || !(cols[2][i] > 0.0)
                    || (i > 0 && !(cols[0][i] > cols[0][i - 1]))) {
                    throw std::runtime_error("elastic parameter table invalid: " + name);
                }
            }
            elastic[name] = std::move(cols);
            continue;
        }
        if (kind == "conditional_cdf") {
            std::string value_column = obj.str_or("value_column", "");
            if (value_column.empty()) value_column = obj.str("primary_value_column");
            auto const c = ReadRreaTableContainer(path);
            cdfs[name] = group_conditional(c.column("primary_energy_eV"), c.column("cdf_u"),
                                           c.column(value_column), name);
            continue;
        }
        if (kind == "photoelectric_subshell_cdf") {
            // S/RreaInteractionTables.cpp:893-987
            auto const c = ReadRreaTableContainer(path);
            auto const prim = c.column("primary_energy_eV");
            auto const cdf = c.column("cdf_u");
            auto const prob = c.column("subshell_probability");
            auto const bind = c.column("binding_energy_eV");
            auto const relax = c.column("relaxation_energy_eV");
            pe_primary.clear();
            pe_rows_u.clear();
            pe_rows_b.clear();
            for (std::size_t i = 0; i < prim.size(); ++i) {
                if (!(prim[i] > 0.0) || bind[i] < 0.0 || relax[i] < 0.0
                    || relax[i] > bind[i] * (1.0 + 1.0e-9) || bind[i] > prim[i] || cdf[i] < 0.0 || cdf[i] > 1.0
                    || prob[i] < 0.0) {
                    throw std::runtime_error("invalid photoelectric subshell row");
                }
                bool const reset = !pe_primary.empty() && pe_primary.back() == prim[i] && !pe_rows_u.back().empty()
                    && cdf[i] <= pe_rows_u.back().back();
                if (pe_primary.empty() || pe_primary.back() != prim[i] || reset) {
                    if (!pe_primary.empty() && prim[i] < pe_primary.back()) {
                        throw std::runtime_error("photoelectric groups must be nondecreasing");
                    }
                    pe_primary.push_back(prim[i]);
                    pe_rows_u.emplace_back();
                    pe_rows_b.emplace_back();
                    pe_prob_sum.push_back(0.0);
                }
                if (!pe_rows_u.back().empty() && cdf[i] <= pe_rows_u.back().back()) {
                    throw std::runtime_error("photoelectric CDF not increasing within a group");
                }
                pe_rows_u.back().push_back(cdf[i]);
                pe_rows_b.back().push_back(bind[i]);
                pe_prob_sum.back() += prob[i];
            }
            for (std::size_t g = 0; g < pe_primary.size(); ++g) {
                if (std::abs(pe_rows_u[g].back() - 1.0) > 1.0e-12 || std::abs(pe_prob_sum[g] - 1.0) > 1.0e-10) {
                    throw std::runtime_error("photoelectric subshell group does not close at 1");
                }
            }
            continue;
        }
        std::string x_column = obj.str_or("x_column", "energy_eV");
        std::string value_column = obj.str_or("value_column", "");
        if (value_column.empty()) value_column = obj.str("primary_value_column");
        std::string interpolation = obj.str_or("interpolation", "loglog_linear");
        if (obj.str_or("extrapolation", "forbidden") != "forbidden") {
            throw std::runtime_error("table extrapolation must be forbidden: " + name);
        }
        bool const allow_dup = obj.bool_or("allow_duplicate_x", false);
        auto const c = ReadRreaTableContainer(path);
        Table1D t;
        t.interpolation = interpolation;
        t.x = c.column(x_column);
        t.y = c.column(value_column);
        if (t.x.size() != t.y.size() || t.x.size() < 2) {
            throw std::runtime_error("table column sizes invalid: " + name);
        }
        for (std::size_t i = 0; i < t.x.size(); ++i) {
            if (!(t.x[i] > 0.0) || t.y[i] < 0.0
                || (interpolation == "loglog_linear" && !(t.y[i] > 0.0))) {
                throw std::runtime_error("table values invalid: " + name);
            }
            if (i > 0 && (t.x[i] < t.x[i - 1] || (!allow_dup && t.x[i] == t.x[i - 1]))) {
                throw std::runtime_error("table energy grid not increasing: " + name);
            }
        }
        tables[name] = std::move(t);
    }

    auto const charged = cfg.at("charged_energy_range_eV");
    auto const photon = cfg.at("photon_energy_range_eV");
    m_index.charged_min_eV = charged.items.at(0).num();
    m_index.charged_max_eV = charged.items.at(1).num();
    m_index.photon_min_eV = photon.items.at(0).num();
    m_index.photon_max_eV = photon.items.at(1).num();
    m_index.hard_moller_threshold_eV = cfg.num_or("hard_moller_secondary_threshold_eV", 0.0);
    m_index.brems_absolute_cutoff_eV = cfg.num_or("brems_absolute_cutoff_eV", 0.0);
    m_index.reference_density_kg_m3 = cfg.num_or("reference_density_kg_m3", -1.0);
    m_index.gs_few_collision_threshold = few;
    m_index.gs_isotropic_above_n = iso;
    m_index.gs_wentzel_transition_eV = transition;
    m_index.w_air_eV_per_pair = 33.97;  // ICRU Report 31 W value for air
    if (!(m_index.hard_moller_threshold_eV > 0.0) || !(m_index.brems_absolute_cutoff_eV > 0.0)
        || !(m_index.reference_density_kg_m3 > 0.0)) {
        throw std::runtime_error("schema-6 thresholds or reference density invalid");
    }

    // Hot 1-D tables.  Tables sharing a bit-identical energy grid share one
    // arena copy of it (and of its logs).
    std::vector<std::pair<std::vector<double> const*, std::pair<int64_t, int64_t>>> grids;
    for (int t = 0; t < RREA_T_COUNT; ++t) {
        auto const it = tables.find(hot_names[t]);
        if (it == tables.end()) {
            throw std::runtime_error(std::string("missing required table ") + hot_names[t]);
        }
        Table1D const& tab = it->second;
        RreaTable1DIndex& h = m_index.hot[t];
        h.n = static_cast<int32_t>(tab.x.size());
        if (tab.interpolation == "loglog_linear") h.mode = RREA_INTERP_LOGLOG;
        else if (tab.interpolation == "loglog_positive_with_zero_threshold") h.mode = RREA_INTERP_LOGLOG_ZERO_THRESHOLD;
        else if (tab.interpolation == "logx_linear") h.mode = RREA_INTERP_LOGX_LINEAR;
        else if (tab.interpolation == "linear") h.mode = RREA_INTERP_LINEAR;
        else throw std::runtime_error("unsupported interpolation " + tab.interpolation);
        bool reused = false;
        for (auto const& g : grids) {
            if (*g.first == tab.x) {
                h.x = g.second.first;
                h.lx = g.second.second;
                reused = true;
                break;
            }
        }
        if (!reused) {
            h.x = push(tab.x);
            h.lx = push_logs(tab.x, false);
            grids.push_back({&tab.x, {h.x, h.lx}});
        }
        h.ix = push_inverse_spacing(h.x, h.n);
        h.ilx = push_inverse_spacing(h.lx, h.n);
        h.y = push(tab.y);
        h.ly = push_logs(tab.y, true);
    }
    auto shared = [&](int first, int last) {
        bool const linear = m_index.hot[first].mode == RREA_INTERP_LINEAR;
        for (int t = first + 1; t <= last; ++t) {
            if (m_index.hot[t].x != m_index.hot[first].x) return 0;
            if ((m_index.hot[t].mode == RREA_INTERP_LINEAR) != linear) return 0;
        }
        return 1;
    };
    m_index.electron_grid_shared = shared(RREA_T_E_COLLISION, RREA_T_E_ELASTIC_TRANSPORT);
    m_index.positron_grid_shared = shared(RREA_T_P_COLLISION, RREA_T_P_ANNIHILATION);
    m_index.photon_grid_shared = shared(RREA_T_PH_COMPTON, RREA_T_PH_PAIR_TRIPLET);
    // Certified-range coverage (RreaInteractionTables.cpp:1979-2017).
    for (int t = 0; t < RREA_T_COUNT; ++t) {
        RreaTable1DIndex const& h = m_index.hot[t];
        double const lo = (t >= RREA_T_PH_COMPTON) ? m_index.photon_min_eV : m_index.charged_min_eV;
        double const hi = (t >= RREA_T_PH_COMPTON) ? m_index.photon_max_eV : m_index.charged_max_eV;
        if (m_arena[h.x] != lo || m_arena[h.x + h.n - 1] != hi) {
            throw std::runtime_error(std::string("table does not cover certified range: ") + hot_names[t]);
        }
    }

    for (int c = 0; c < RREA_C_COUNT; ++c) {
        auto const it = cdfs.find(cdf_names[c]);
        if (it == cdfs.end()) {
            throw std::runtime_error(std::string("missing conditional CDF ") + cdf_names[c]);
        }
        CondGroups const& g = it->second;
        RreaCondCdfIndex& ci = m_index.cdf[c];
        ci.ng = static_cast<int32_t>(g.primary.size());
        ci.primary = push(g.primary);
        ci.lprimary = push_logs(g.primary, false);
        std::vector<double> start(g.primary.size() + 1, 0.0), u, v;
        for (std::size_t k = 0; k < g.primary.size(); ++k) {
            start[k] = static_cast<double>(u.size());
            u.insert(u.end(), g.u[k].begin(), g.u[k].end());
            v.insert(v.end(), g.v[k].begin(), g.v[k].end());
        }
        start.back() = static_cast<double>(u.size());
        ci.total = static_cast<int32_t>(u.size());
        ci.start = push(start);
        ci.u = push(u);
        ci.v = push(v);
        // Per-group mean of the inverse CDF, trapezoid over the u nodes in the
        // reference's accumulation order (RreaInteractionTables.cpp:1075-1085).
        std::vector<double> mean(g.primary.size(), 0.0);
        for (std::size_t k = 0; k < g.primary.size(); ++k) {
            std::vector<double> const& gu = g.u[k];
            std::vector<double> const& gv = g.v[k];
            double m = gu.front() * gv.front();
            for (std::size_t i = 1; i < gu.size(); ++i) {
                m += 0.5 * (gv[i - 1] + gv[i]) * (gu[i] - gu[i - 1]);
            }
            m += (1.0 - gu.back()) * gv.back();
            mean[k] = m;
        }
        ci.mean = push(mean);
        ci.lmean = push_logs(mean, true);
    }

    for (int s = 0; s < 2; ++s) {
        auto const it = elastic.find(s == 0 ? "electron_elastic_mfp_air" : "positron_elastic_mfp_air");
        if (it == elastic.end()) throw std::runtime_error("missing elastic parameter table");
        auto const& cols = it->second;
        if (cols[0].front() != 1.0e3 || cols[0].back() != 1.0e10) {
            throw std::runtime_error("elastic parameter table must cover 1 keV - 10 GeV");
        }
        RreaElasticIndex& e = m_index.elastic[s];
        e.n = static_cast<int32_t>(cols[0].size());
        e.x = push(cols[0]);
        e.lx = push_logs(cols[0], false);
        e.mfp = push(cols[1]);
        e.eta = push(cols[2]);
        e.ilx = push_inverse_spacing(e.lx, e.n);
    }

    auto put_angle = [&](RreaAngleIndex& ai, char const* name, double lo, double hi) {
        auto const it = angles.find(name);
        if (it == angles.end()) throw std::runtime_error(std::string("missing angle table ") + name);
        Angle const& a = it->second;
        if (a.e.front() != lo || a.e.back() != hi || a.p.front() > few || a.p.back() < iso) {
            throw std::runtime_error(std::string("angle table coverage invalid: ") + name);
        }
        ai.ne = static_cast<int32_t>(a.e.size());
        ai.np = static_cast<int32_t>(a.p.size());
        ai.nu = static_cast<int32_t>(a.u.size());
        ai.e = push(a.e);
        ai.le = push_logs(a.e, false);
        ai.p = push(a.p);
        ai.lp = push_logs(a.p, false);
        ai.u = push(a.u);
        std::vector<double> lur(a.u.size(), 0.0);
        for (std::size_t i = 0; i + 1 < a.u.size(); ++i) {
            lur[i] = (a.u[i] > 0.0) ? std::log(a.u[i + 1] / a.u[i]) : 0.0;
        }
        ai.lur = push(lur);
        ai.omc = push(a.omc);
        ai.lomc = push_logs(a.omc, false);
        ai.ile = push_inverse_spacing(ai.le, ai.ne);
        ai.ilp = push_inverse_spacing(ai.lp, ai.np);
        ai.ilur = push_reciprocals(lur);
        ai.iu = push_reciprocals(a.u);
    };
    put_angle(m_index.gs[0], "electron_gs_angle_cdf_air", m_index.charged_min_eV, transition);
    put_angle(m_index.gs[1], "positron_gs_angle_cdf_air", m_index.charged_min_eV, transition);
    put_angle(m_index.wentzel[0], "electron_wentzel_vi_angle_cdf_air", transition, m_index.charged_max_eV);
    put_angle(m_index.wentzel[1], "positron_wentzel_vi_angle_cdf_air", transition, m_index.charged_max_eV);

    // Mean hard-Moller delta-ray energy per event on the rate grid: midpoint
    // quadrature of the secondary sampler over 4096 uniform nodes, only where
    // the rate is positive (RreaInteractionTables.cpp:2146-2179).
    {
        RreaTable1DIndex const& rate = m_index.hot[RREA_T_E_HARD_MOLLER];
        RreaCondCdfIndex const& mc = m_index.cdf[RREA_C_MOLLER];
        std::vector<double> mean(static_cast<std::size_t>(rate.n), 0.0);
        int const samples = 4096;
        for (int i = 0; i < rate.n; ++i) {
            double const e = m_arena[rate.x + i];
            if (!(m_arena[rate.y + i] > 0.0)) {
                continue;
            }
            if (e < m_arena[mc.primary] || e > m_arena[mc.primary + mc.ng - 1]) {
                throw std::runtime_error("hard-Moller rate positive outside the Moller CDF range");
            }
            double acc = 0.0;
            for (int s = 0; s < samples; ++s) {
                acc += HostSampleConditional(*this, RREA_C_MOLLER, e,
                                             (static_cast<double>(s) + 0.5) / samples, true);
            }
            mean[static_cast<std::size_t>(i)] = acc / static_cast<double>(samples);
        }
        m_index.hard_moller_mean_secondary = push(mean);
    }
    // Photoelectric subshell CDF.
    {
        if (pe_primary.size() < 2 || pe_primary.front() != m_index.photon_min_eV
            || pe_primary.back() != m_index.photon_max_eV) {
            throw std::runtime_error("photoelectric subshell CDF must cover the photon range");
        }
        RreaPhotoelectricIndex& pi = m_index.pe;
        pi.ng = static_cast<int32_t>(pe_primary.size());
        pi.primary = push(pe_primary);
        std::vector<double> start(pe_primary.size() + 1), u, b;
        for (std::size_t g = 0; g < pe_primary.size(); ++g) {
            start[g] = static_cast<double>(u.size());
            u.insert(u.end(), pe_rows_u[g].begin(), pe_rows_u[g].end());
            b.insert(b.end(), pe_rows_b[g].begin(), pe_rows_b[g].end());
        }
        start.back() = static_cast<double>(u.size());
        pi.total = static_cast<int32_t>(u.size());
        pi.start = push(start);
        pi.u = push(u);
        pi.binding = push(b);
    }
    LoadPairBank(dir + "/final_state/pair_final_state_samples_air.bin.rtb",
                 dir + "/final_state/pair_final_state_samples_air.index.json");
    m_index.total_doubles = static_cast<int64_t>(m_arena.size());
    m_loaded = true;
}

// Training split of the correlated pair bank with its record contract
// (S/RreaInteractionTables.cpp:1123-1370).
void TableSet::LoadPairBank(std::string const& bin_path, std::string const& index_path)
{
    auto const bank = ReadRreaTableContainer(bin_path);
    if (bank.header.str_or("kind", "") != "records" || bank.header.str_or("record_bytes", "") != "144") {
        throw std::runtime_error("pair final-state container is not a 144-byte record set");
    }
    auto const target_z = bank.column("target_Z");
    auto const channel_code = bank.column("channel_code");
    auto const lepton_count = bank.column("lepton_count");
    auto const flags = bank.column("flags");
    auto const primary = bank.column("primary_energy_eV");
    auto const recoil = bank.column("local_recoil_fraction");
    std::vector<double> pdg[3], reserved[3], frac[3], dxs[3], dys[3], dzs[3];
    for (int slot = 0; slot < 3; ++slot) {
        std::string const p = "p" + std::to_string(slot) + "_";
        pdg[slot] = bank.column(p + "pdg");
        reserved[slot] = bank.column(p + "reserved");
        frac[slot] = bank.column(p + "kinetic_fraction");
        dxs[slot] = bank.column(p + "dir_x");
        dys[slot] = bank.column(p + "dir_y");
        dzs[slot] = bank.column(p + "dir_z");
    }
    std::size_t const rows = bank.rows();
    JsonValue const index = ParseJson(read_text(index_path));
    if (JsonValue const* failures = index.find("failures")) {
        if (!failures->items.empty()) throw std::runtime_error("pair index reports producer failures");
    }
    struct Block {
        int channel;
        double energy;
        std::size_t offset, count;
    };
    std::vector<Block> blocks;
    std::vector<std::pair<std::size_t, std::size_t>> ranges;
    for (auto const& b : index.at("blocks").items) {
        std::string const split = b.str("split");
        std::string const ch = b.str("channel");
        int const channel = ch == "nuclear" ? 0 : (ch == "triplet" ? 1 : -1);
        if (channel < 0) throw std::runtime_error("unknown pair channel " + ch);
        double const energy = b.at("primary_energy_eV").num();
        std::size_t const byte_offset = static_cast<std::size_t>(b.at("byte_offset").num());
        std::size_t const offset = static_cast<std::size_t>(b.at("record_offset").num());
        std::size_t const count = static_cast<std::size_t>(b.at("count").num());
        if (!(energy > 0.0) || offset > rows || count > rows - offset || byte_offset != 64 + offset * 144) {
            throw std::runtime_error("pair index block has invalid offset/count");
        }
        if (count > 0) ranges.emplace_back(offset, offset + count);
        if (split != "training") {
            if (split != "holdout") throw std::runtime_error("pair split must be training or holdout");
            continue;
        }
        if (count == 0) continue;
        if (count < 4096) throw std::runtime_error("pair training block has fewer than 4096 records");
        blocks.push_back(Block{channel, energy, offset, count});
    }
    std::sort(ranges.begin(), ranges.end());
    std::size_t next = 0;
    for (auto const& r : ranges) {
        if (r.first != next) throw std::runtime_error("pair index blocks overlap or leave a gap");
        next = r.second;
    }
    if (next != rows) throw std::runtime_error("pair index does not cover the bank");
    std::stable_sort(blocks.begin(), blocks.end(), [](Block const& a, Block const& b) {
        return a.channel != b.channel ? a.channel < b.channel : a.energy < b.energy;
    });
    double const closure_tol = 64.0 * 2.220446049250313080847263336181640625e-16;
    for (int channel = 0; channel < 2; ++channel) {
        std::vector<double> energies, starts, recs;
        double last = 0.0;
        for (Block const& b : blocks) {
            if (b.channel != channel) continue;
            if (!(b.energy > last)) throw std::runtime_error("pair training energies not increasing");
            last = b.energy;
            energies.push_back(b.energy);
            starts.push_back(static_cast<double>(recs.size() / RREA_PAIR_RECORD_DOUBLES));
            int const expect = channel == 1 ? 3 : 2;
            for (std::size_t i = 0; i < b.count; ++i) {
                std::size_t const row = b.offset + i;
                int const z = static_cast<int>(std::llround(target_z[row]));
                auto const code = static_cast<uint32_t>(std::llround(channel_code[row]));
                int const count = static_cast<int>(std::llround(lepton_count[row]));
                auto const fl = static_cast<uint32_t>(std::llround(flags[row]));
                int const rec_channel = code == 1u ? 0 : (code == 2u ? 1 : -1);
                if ((z != 6 && z != 7 && z != 8 && z != 18) || (fl & 1u) == 0u || (fl & ~3u) != 0u
                    || rec_channel != channel || count != expect
                    || std::abs(primary[row] - b.energy) > 1.0e-12 * b.energy || recoil[row] < 0.0
                    || recoil[row] > 1.0) {
                    throw std::runtime_error("pair final-state record metadata is invalid");
                }
                double fsum = recoil[row];
                int ne = 0, np = 0;
                for (int slot = 0; slot < 3; ++slot) {
                    if (std::llround(reserved[slot][row]) != 0) throw std::runtime_error("pair reserved word set");
                    if (slot < expect) {
                        double const n = std::sqrt(dxs[slot][row] * dxs[slot][row] + dys[slot][row] * dys[slot][row]
                                                   + dzs[slot][row] * dzs[slot][row]);
                        if (frac[slot][row] < 0.0 || std::abs(n - 1.0) > 1.0e-8) {
                            throw std::runtime_error("pair particle record invalid");
                        }
                        fsum += frac[slot][row];
                        long const pd = std::llround(pdg[slot][row]);
                        ne += pd == 11 ? 1 : 0;
                        np += pd == -11 ? 1 : 0;
                    } else if (std::llround(pdg[slot][row]) != 0 || frac[slot][row] != 0.0 || dxs[slot][row] != 0.0
                               || dys[slot][row] != 0.0 || dzs[slot][row] != 0.0) {
                        throw std::runtime_error("pair unused slot not zero");
                    }
                }
                if (ne != expect - 1 || np != 1 || std::abs(fsum - 1.0) > closure_tol) {
                    throw std::runtime_error("pair record topology/closure invalid");
                }
                recs.push_back(static_cast<double>(count));
                for (int slot = 0; slot < 3; ++slot) recs.push_back(static_cast<double>(std::llround(pdg[slot][row])));
                for (int slot = 0; slot < 3; ++slot) recs.push_back(frac[slot][row]);
                for (int slot = 0; slot < 3; ++slot) {
                    recs.push_back(dxs[slot][row]);
                    recs.push_back(dys[slot][row]);
                    recs.push_back(dzs[slot][row]);
                }
            }
        }
        if (energies.size() < 2 || last < 1.0e11) throw std::runtime_error("pair training blocks do not cover 100 GeV");
        starts.push_back(static_cast<double>(recs.size() / RREA_PAIR_RECORD_DOUBLES));
        RreaPairBankIndex& pb = m_index.pair[channel];
        pb.nb = static_cast<int32_t>(energies.size());
        pb.primary = push(energies);
        pb.lprimary = push_logs(energies, false);
        pb.start = push(starts);
        pb.records = push(recs);
    }
}

// Conditional inverse-CDF sampling (RreaInteractionTables.cpp:995-1069 and the
// Moller variant :2584-2653, which always log-interpolates between groups).
double HostSampleConditional(TableSet const& tables, int which, double primary_eV,
                             double cdf_u, bool moller_always_log)
{
    RreaCondCdfIndex const& ci = tables.index().cdf[which];
    double const* prim = tables.at(ci.primary);
    double const* start = tables.at(ci.start);
    double const* u = tables.at(ci.u);
    double const* v = tables.at(ci.v);
    cdf_u = std::max(0.0, std::min(1.0, cdf_u));
    auto sample_group = [&](int g) {
        int const b = static_cast<int>(start[g]);
        int const e = static_cast<int>(start[g + 1]);
        double const* ub = u + b;
        double const* up = std::lower_bound(ub, u + e, cdf_u);
        if (up == ub) return v[b];
        if (up == u + e) return v[e - 1];
        int const hi = static_cast<int>(up - u);
        int const lo = hi - 1;
        double const denom = u[hi] - u[lo];
        double const t = denom > 0.0 ? (cdf_u - u[lo]) / denom : 0.0;
        return v[lo] + t * (v[hi] - v[lo]);
    };
    if (!std::isfinite(primary_eV) || primary_eV < prim[0] || primary_eV > prim[ci.ng - 1]) {
        throw std::runtime_error("conditional CDF primary energy outside range");
    }
    if (!moller_always_log) {
        if (primary_eV == prim[0]) return sample_group(0);
        if (primary_eV == prim[ci.ng - 1]) return sample_group(ci.ng - 1);
    }
    double const* up = std::lower_bound(prim, prim + ci.ng, primary_eV);
    if (up == prim) return sample_group(0);
    if (up == prim + ci.ng) return sample_group(ci.ng - 1);
    int const hi = static_cast<int>(up - prim);
    int const lo = hi - 1;
    if (prim[hi] == primary_eV) return sample_group(hi);
    double const y0 = sample_group(lo);
    double const y1 = sample_group(hi);
    double const t = (std::log(primary_eV) - std::log(prim[lo]))
        / (std::log(prim[hi]) - std::log(prim[lo]));
    if (moller_always_log || (y0 > 0.0 && y1 > 0.0)) {
        return std::exp(std::log(y0) + t * (std::log(y1) - std::log(y0)));
    }
    return y0 + t * (y1 - y0);
}

}  // namespace rrea_host
