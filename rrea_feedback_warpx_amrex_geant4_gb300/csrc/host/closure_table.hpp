// Low-energy electron closure table: the measured dry-air E/N bundle behind
// the en_table_flux_v1 / en_table_attachment_v1 fluid models
// (LowEnergyElectronClosure, I/RreaInteractionTables.H:494-566).  The loader
// applies the reference's validation (S/RreaInteractionTables.cpp:3267-3404);
// the log columns are taken on the host so the interpolation nodes are the
// same doubles on every consumer.
#pragma once

#include <stdexcept>
#include <string>
#include <vector>

namespace rrea_host {

struct ClosureTableError : std::runtime_error {
    explicit ClosureTableError(std::string const& m) : std::runtime_error(m) {}
};

struct ClosureTable {
    std::vector<double> en_td, log_en_td;
    std::vector<double> k0, log_k0;    // reduced flux mobility at Loschmidt [m^2/V/s]
    std::vector<double> nu2;           // two-body attachment frequency at Loschmidt [1/s], may be 0
    std::vector<double> nu3, log_nu3;  // three-body attachment frequency at Loschmidt [1/s]
    std::vector<double> dl, log_dl;    // longitudinal diffusion at Loschmidt [m^2/s]
    std::vector<double> dt, log_dt;    // transverse diffusion at Loschmidt [m^2/s]
    std::size_t size() const { return en_td.size(); }
};

// Parses and validates one schema-3 closure CSV; throws ClosureTableError.
ClosureTable load_closure_table(std::string const& path);

// Range status of one evaluation (RreaClosureRangeStatus).
enum ClosureStatus { kClosureInRange = 0, kClosureHeldBelow = 1, kClosureAboveRange = 2, kClosureInvalid = 3 };

}  // namespace rrea_host
