// Seed schedule input adapter: the CSV event list the overlay injects as
// native seed electrons and positrons (RreaSeedSchedule, I/RreaSeedSchedule.H
// and S/RreaSeedSchedule.cpp; injection rule of
// RreaWarpXCoupling::InjectScheduledSeeds, O/RreaCouplingSources.cpp:96-215).
#pragma once

#include "../../../include/rrea_gpu.h"

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

namespace rrea_host {

// Seed species ids of the optional species_id column (I/RreaSeedSchedule.H:94-97).
constexpr int kSeedElectron = 1;
constexpr int kSeedPositron = 2;

// Below this magnitude the (ux, uy, uz) triple is a direction hint rescaled
// from the kinetic energy; at or above it, already the proper velocity in
// m/s (I/RreaSeedSchedule.H:16-27).
constexpr double kSeedDirectionHintMaxMPerS = 1.0e6;

struct SeedScheduleError : std::runtime_error {
    int code;
    SeedScheduleError(int c, std::string const& m) : std::runtime_error(m), code(c) {}
};

// RreaElectronProperVelocityFromKineticEv (I/RreaSeedSchedule.H:31-43).
double electron_proper_velocity(double kinetic_energy_eV);

// RreaNormalizeSeedMomentum (I/RreaSeedSchedule.H:55-71): a direction hint
// is rescaled to the proper velocity of the kinetic energy; a proper
// velocity (or a degenerate hint) passes through.
void normalize_seed_momentum(double ux, double uy, double uz, double kinetic_energy_eV, double out[3]);

// RreaSeedEventWindowClass (I/RreaSeedSchedule.H:76-91): -1 stale (before the
// window), 0 inject, 1 beyond the window [begin, end).
int seed_window_class(double time_s, double begin_s, double end_s);

class SeedSchedule {
public:
    // RreaSeedSchedule::Load (S/RreaSeedSchedule.cpp:75-144): rows of the
    // given case (all rows when case_id is empty), macro_index defaulting to
    // the CSV line number, species_id to electron; sorted by (time_s,
    // macro_index).  Throws SeedScheduleError.
    void load(std::string const& path, std::string const& case_id);
    // RreaSeedSchedule::ValidateProduction (S/RreaSeedSchedule.cpp:146-244).
    void validate(double e_min_eV, double e_max_eV, double r_min_m, double r_max_m, double z_min_m,
                  double z_max_m) const;

    std::vector<rrea_gpu_seed_event> const& events() const { return m_events; }
    // The injection cursor (the coupling's m_next_seed_event).
    int64_t cursor = 0;

private:
    std::vector<rrea_gpu_seed_event> m_events;
};

}  // namespace rrea_host
