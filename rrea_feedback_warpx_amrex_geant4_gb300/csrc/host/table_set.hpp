// Host loader for the schema-6 transport table bundle.  Reads
// transport_physics.json and its RREATBL containers, validates the contracts
// the transport relies on, and packs every table into one FP64 arena laid out
// by RreaArenaIndex (rrea_arena.h) for a single upload to HBM.
//
// Follows RreaInteractionTables::Load (native_amrex_rrea/src/
// RreaInteractionTables.cpp:1659-2230): table classification by name and
// table_kind, conditional-CDF grouping (:559-619), elastic MFP (:650-685),
// GS/Wentzel 2-D angle tables (:687-772), and the load-time hard-Moller mean
// secondary quadrature (:2142-2179).
#pragma once

#include "../rrea_arena.h"

#include <string>
#include <vector>

namespace rrea_host {

struct PhotoelectricRow {
    double cdf_u;
    double binding_eV;
    double relaxation_eV;
};

class TableSet {
public:
    // Throws std::runtime_error on any contract violation.
    void Load(std::string const& transport_physics_json);

    bool loaded() const { return m_loaded; }
    RreaArenaIndex const& index() const { return m_index; }
    std::vector<double> const& arena() const { return m_arena; }
    double const* at(int64_t offset) const { return m_arena.data() + offset; }

private:
    void LoadPairBank(std::string const& bin_path, std::string const& index_path);
    int64_t push(std::vector<double> const& values);
    int64_t push_logs(std::vector<double> const& values, bool zero_for_nonpositive);
    // 1 / (a[i] - a[i-1]) for the arena array at `off` of `n` doubles (0 at i = 0
    // and where two nodes coincide)
    int64_t push_inverse_spacing(int64_t off, int n);
    // 1 / v[i] (0 where v[i] = 0)
    int64_t push_reciprocals(std::vector<double> const& values);

    bool m_loaded = false;
    std::vector<double> m_arena;
    RreaArenaIndex m_index{};
};

// Host restatement of the reference's Moller secondary sampler, used at load
// to tabulate the mean delta-ray energy (RreaInteractionTables.cpp:2584-2653).
double HostSampleConditional(TableSet const& tables, int which, double primary_eV,
                             double cdf_u, bool moller_always_log);

}  // namespace rrea_host
