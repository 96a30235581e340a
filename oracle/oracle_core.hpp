// ORACLE — test infrastructure only.  A scalar CPU restatement of the
// reference's per-timestep kinetic step (RREA overlay,
// native_amrex_rrea/warpx_overlay/Source/Rrea/ and native_amrex_rrea/src/),
// used by tests/, __graft_entry__.smoke() and bench.py's CPU baseline to
// check the GPU path.  The shipped GPU path never calls into this directory.
//
// Every function cites the reference file:line it restates.  Shorthand:
//   O/ = native_amrex_rrea/warpx_overlay/Source/Rrea/
//   S/ = native_amrex_rrea/src/
//   I/ = native_amrex_rrea/include/rrea/
#pragma once

#include <atomic>
#include "../rrea_feedback_warpx_amrex_geant4_gb300/csrc/host/table_set.hpp"
#include "../include/rrea_gpu.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <limits>
#include <stdexcept>
#include <string>
#include <vector>

namespace oracle {

constexpr double kMeC2 = 510998.95000;          // I/RreaConstants.H:9
constexpr double kC = 299792458.0;              // I/RreaConstants.H:10
constexpr double kTwoPi = 6.283185307179586476925286766559;
constexpr double kEps = std::numeric_limits<double>::epsilon();

struct OracleError : std::runtime_error {
    int code;
    OracleError(int c, std::string const& m) : std::runtime_error(m), code(c) {}
};

[[noreturn]] inline void fail(int code, std::string const& msg) { throw OracleError(code, msg); }

// ---------------------------------------------------------------- RNG
// O/RreaRng.cpp:9-44
inline uint64_t splitmix64(uint64_t v)
{
    v += 0x9e3779b97f4a7c15ULL;
    v = (v ^ (v >> 30U)) * 0xbf58476d1ce4e5b9ULL;
    v = (v ^ (v >> 27U)) * 0x94d049bb133111ebULL;
    return v ^ (v >> 31U);
}
inline uint64_t rng_counter(uint64_t seed, uint64_t pid, uint64_t step, uint64_t idx, uint64_t ch)
{
    uint64_t s = splitmix64(seed);
    s ^= splitmix64(pid + 0x100000001b3ULL);
    s ^= splitmix64(step + 0x9e3779b97f4a7c15ULL);
    s ^= splitmix64(idx + 0xbf58476d1ce4e5b9ULL);
    s ^= splitmix64(ch + 0x94d049bb133111ebULL);
    return splitmix64(s);
}
inline double rng_uniform(uint64_t seed, uint64_t pid, uint64_t step, uint64_t idx, uint64_t ch)
{
    return (static_cast<double>(rng_counter(seed, pid, step, idx, ch) >> 12U) + 0.5) * 0x1.0p-52;
}

// O/RreaRng.H:17-97 channel ids used by the transport phases.
enum Channel : uint64_t {
    kHardMollerEnergy = 22, kHardMollerAzimuth = 23,
    kBremsEnergy = 42, kBremsAngle = 43, kBremsAzimuth = 44,
    kElectronGsAngle = 89, kElectronGsAzimuth = 90, kElectronGsFewCount = 91,
    kElectronGsFewScatter = 92, kElectronGsFewAzimuth = 93,
    kElectronCompetingOpticalDepth = 107, kElectronCompetingChannel = 108,
    kElectronContinuationOpticalDepth = 124, kElectronContinuationChannel = 125,
    kPositronBhabhaEnergy = 74, kPositronBremsEnergy = 76, kPositronBremsAngle = 77, kPositronBremsAzimuth = 78,
    kAnnihilationPolar = 80, kAnnihilationAzimuth = 81,
    kPositronGsAngle = 94, kPositronGsAzimuth = 95, kPositronGsFewCount = 96, kPositronGsFewScatter = 97,
    kPositronGsFewAzimuth = 98,
    kPositronCompetingOpticalDepth = 109, kPositronCompetingChannel = 110,
    kPositronContinuationOpticalDepth = 126, kPositronContinuationChannel = 127,
    kPositronBhabhaAzimuth = 130,
    kNewbornElectronGsAngle = 112, kNewbornElectronGsAzimuth = 113, kNewbornElectronGsFewCount = 114,
    kNewbornElectronGsFewScatter = 115, kNewbornElectronGsFewAzimuth = 116,
    kNewbornPositronGsAngle = 117, kNewbornPositronGsAzimuth = 118, kNewbornPositronGsFewCount = 119,
    kNewbornPositronGsFewScatter = 120, kNewbornPositronGsFewAzimuth = 121,
    kNewbornCompetingOpticalDepth = 122, kNewbornCompetingChannel = 123,
};

// O/RreaParticleInteraction.H:642-710
constexpr uint64_t kLineageCap = uint64_t{1} << 14;
constexpr uint64_t kSegmentCap = uint64_t{1} << 14;
constexpr uint64_t kEventCap = uint64_t{1} << 13;
constexpr uint64_t kInnerCap = uint64_t{1} << 8;
inline bool try_pack_transient(bool newborn, uint64_t species, uint64_t lineage, uint64_t segment,
                               uint64_t ordinal, uint64_t inner, uint64_t& out)
{
    if (species >= 3U || lineage >= kLineageCap || segment >= kSegmentCap || ordinal >= kEventCap
        || inner >= kInnerCap) {
        return false;
    }
    out = (static_cast<uint64_t>(newborn) << 51) | (species << 49) | (lineage << 35) | (segment << 21)
        | (ordinal << 8) | inner;
    return true;
}
inline bool try_live_hazard_index(uint64_t species, uint64_t segment, uint64_t ordinal, uint64_t& out)
{
    if (species >= 3U) return false;
    if (ordinal == 0U) {
        if (segment >= kSegmentCap) return false;
        out = segment;
        return true;
    }
    return try_pack_transient(false, species, 1U, segment, ordinal, 0U, out);
}

// ---------------------------------------------------------------- output records
struct Secondary {
    int species;  // 0 e-, 1 e+, 2 photon  (O/RreaParticleInteraction.H:28-32)
    int process;  // RreaSecondaryProcess ordinal
    double x, y, z, dx, dy, dz, w, energy, birth;
    uint64_t root_key, lineage;
    int root_species;
    int64_t parent_index;
};

struct Source {
    int kind;  // 0 ionization event, 1 low-energy electron, 2 positive ion only
    double r, z, w, secondary_energy, energy_loss;
    int64_t parent_index;
};

struct Segment {
    int kind;  // 0 net chord, 1 escape
    double a[7];
    uint64_t channel;
    uint32_t faces;
    int64_t parent_index;
};

// One deferred plane crossing (RreaPlaneFluxCrossing, I/RreaPlaneFlux.H:48-55).
struct PlaneCrossing {
    int plane;
    int direction;  // +1 up, -1 down
    double weight, r;
    bool local_runaway, at_least_one_mev;
};

struct StepOutputs {
    std::vector<Secondary> secondaries;
    std::vector<Source> sources;
    std::vector<Segment> segments;
    std::vector<PlaneCrossing> crossings;
    // per-particle diagnostics for parity: substeps used, events drawn
    std::vector<uint64_t> subcycles;
    std::vector<uint64_t> events;
    std::vector<int32_t> disposition;  // 0 survive, 1 escape, 2 demote, 3 skip (w<=0), -1 invalid input
    void clear()
    {
        secondaries.clear();
        sources.clear();
        segments.clear();
        crossings.clear();
        subcycles.clear();
        events.clear();
        disposition.clear();
    }
};

// Charged tile view (O/RreaTransportStep.H:454-468): current state written
// back, prev_* read as the authoritative pre-push state.
struct ChargedTile {
    int64_t n = 0;
    double* r = nullptr;
    double* z = nullptr;
    double* theta = nullptr;
    double* ux = nullptr;
    double* uy = nullptr;
    double* uz = nullptr;
    double const* w = nullptr;
    double const* prev_r = nullptr;
    double const* prev_z = nullptr;
    double const* prev_theta = nullptr;
    double const* prev_ux = nullptr;
    double const* prev_uy = nullptr;
    double const* prev_uz = nullptr;
    int64_t* id = nullptr;  // > 0 valid; the step negates invalidated ids
    int32_t const* cpu = nullptr;
};

struct FieldGrid {
    int nr = 0, nz = 0;
    double dr = 0.0, dz = 0.0, z_lo = 0.0;
    std::vector<double> er, ez, bt, amb_er, amb_ez;
};

struct CellSources {
    int nr = 0, nz = 0;
    std::vector<double> f[5];  // low e-, positive ion, direct negative ion, ionization count, energy loss
};

// Runs the electron phase of one step (O/RreaElectronTransport.cpp:9-902)
// over one tile.  Throws OracleError on any fail-closed guard.
void ApplyElectronTransport(rrea_host::TableSet const& tables, rrea_gpu_config const& cfg,
                            FieldGrid const& field, int step, double dt_s, ChargedTile& tile,
                            StepOutputs& out);

// Positron phase of one step (O/RreaPositronTransport.cpp:9-878) over one
// tile.  Dispositions: 0 survive, 1 escape, 2 annihilated, 3 zero weight.
void ApplyPositronTransport(rrea_host::TableSet const& tables, rrea_gpu_config const& cfg,
                            FieldGrid const& field, int step, double dt_s, ChargedTile& tile,
                            StepOutputs& out);

// DrainAndCommitSecondaries (O/RreaSecondaryCommit.cpp:9-638): the step's
// secondaries (`initial`, in the phases' group order: electron, photon,
// positron) are advanced FIFO through the rest of the step by
// AdvanceChargedNewborn / AdvancePhotonNewborn (O/RreaNewbornAdvance.cpp);
// children join the FIFO with lineages allocated per root.  `survivors` gets
// the final survivors in FIFO order (birth fraction 1); `out` gets the
// newborns' sources and charged segments.
void DrainSecondaries(rrea_host::TableSet const& tables, rrea_gpu_config const& cfg, FieldGrid const& field,
                      int step, double dt_s, std::vector<Secondary> const& initial, std::vector<Secondary>& survivors,
                      StepOutputs& out);

// Photon phase of one step (O/RreaPhotonTransport.cpp:9-461) over one tile:
// prev_* is the captured start, (r, theta, z) the straight-push endpoint.
void ApplyPhotonTransport(rrea_host::TableSet const& tables, rrea_gpu_config const& cfg, int step, double dt_s,
                          ChargedTile& tile, StepOutputs& out);

// Padded net-chord grid of the coupling (O/RreaWarpXCoupling.cpp:417-444):
// nr + 2 cells in r, nz + 4 in z (two pad cells below and above).
struct NetChordGrid {
    int nr = 0, nz = 0;          // padded sizes
    int phys_nr = 0, phys_z_begin = 0, phys_nz = 0;
    double dr = 0.0, dz = 0.0, r_lo = 0.0, z_lo = 0.0;
    std::vector<double> rho, jr, jz;  // rho nr*nz; jr (nr+1)*nz; jz nr*(nz+1)
    void Reset(rrea_gpu_config const& cfg);
};

// Replays the step's charged segments into the grid: DepositSegmentRZ for a
// net chord and DepositEscapingSegmentRZ for an escape
// (I/RreaSegmentDepositionRZ.H:96-397).  Throws on an escape whose boundary
// cloud cannot be closed.
void DepositNetChords(NetChordGrid& g, double dt_s, std::vector<Segment> const& segments);

// ConvertPaddedIndexCurrentToPhysicalRZ (I/RreaSegmentDepositionRZ.H:399-458)
// with the coupling's charge per index flux (the elementary charge).
void ConvertNetChordCurrent(NetChordGrid const& g, std::vector<double>& jr_phys, std::vector<double>& jz_phys);

// Maxwell TM-RZ field on the replicated vectors (I/RreaMaxwellTMRZ.H:61-85):
// er (nr+1)*nz, ez nr*(nz+1), bt (nr+1)*(nz+1).
struct MaxwellField {
    int nr = 0, nz = 0;
    double dr = 0.0, dz = 0.0;
    std::vector<double> er, ez, bt;
};

// One outer field step with the face current (jr, jz) held over `substeps`
// equal material substeps: the Maxwell part of RreaAmrexAdvance::AdvanceOneStep
// (S/RreaAmrexAdvance.cpp:593-800) with no fluid current or conductivity.
// Throws on a CFL violation.
void AdvanceMaxwell(MaxwellField& f, double dt_s, int substeps, std::vector<double> const& jr,
                    std::vector<double> const& jz);
// Its three leapfrog pieces (I/RreaMaxwellTMRZ.H:143-214): B at the interior
// corners, first-order Silver-Mueller on the open faces, E with the face
// current and no conductivity.
void MaxwellAdvanceB(MaxwellField& f, double dt);
void MaxwellSilverMueller(MaxwellField& f);
void MaxwellAdvanceE(MaxwellField& f, double dt, std::vector<double> const& jr, std::vector<double> const& jz);

// Transport density ratio at an axial position, TransportDensityRatioAtZ
// (O/RreaWarpXCoupling.cpp:79-95): the configured uniform ratio, or, with an
// altitude profile bound (rrea.air_density_model=altitude_profile), the
// profile density at altitude_msl_at_z0 + z over the tables' reference
// density.  The profile interpolates linearly between strictly increasing
// altitude nodes and fails outside them (S/RreaAltitudeProfile.cpp:125-147).
struct DensityProfile {
    std::vector<double> altitude_m, density_kg_m3;
    double altitude_msl_at_z0_m = 0.0;
    double reference_density_kg_m3 = 0.0;
    bool enabled() const { return !altitude_m.empty(); }
    double interpolate(double altitude_m) const;
};
// Binds (or, with no nodes, unbinds) the profile; validates it as
// RreaAltitudeProfile::LoadCsv does (S/RreaAltitudeProfile.cpp:97-117).
void SetDensityProfile(DensityProfile p);
DensityProfile const& BoundDensityProfile();
double DensityRatioAtZ(double uniform_ratio, double z_m);
// The step's fallback ratio: the ratio at the domain's axial centre, else
// the configured ratio, else 1 (O/RreaParticleInteraction.cpp:27-35).
double StepDensityRatio(rrea_gpu_config const& cfg);

// Elastic angle draws by branch since the last reset: GS inverse CDF
// (E <= the Wentzel transition), Wentzel-VI inverse CDF, the isotropic branch
// (n >= isotropic_above_path_n) and single screened-Rutherford scatters.
extern std::atomic<uint64_t> g_elastic_branch[4];

// Photon energy-flow ledger check of one interaction (oracle_core.cpp).
bool PhotonFlowValid(int kind, double w, double inc, double x1, double x2, double x3, bool has_recoil, double local);

// Primitive-level evaluation for fixture comparisons (ids listed in oracle_core.cpp).
int RunPrimitive(rrea_host::TableSet const& tables, int which, double const* in, int64_t n, double* out);

// The plane-crossing diagnostic's planes (empty: off); strictly increasing.
void SetPlanes(std::vector<double> planes);
std::vector<double> const& Planes();

// RreaForEachNonperiodicPlaneCrossing (I/RreaPlaneFlux.H:79-118): calls
// cb(plane index, segment fraction, direction) for every plane in (z0, z1]
// (upward) or (z1, z0] (downward), in crossing order; false on a non-finite
// end or planes that are not strictly increasing.
template <class F>
bool ForEachPlaneCrossing(double z0, double z1, std::vector<double> const& planes, F&& cb)
{
    if (!std::isfinite(z0) || !std::isfinite(z1)) return false;
    for (std::size_t i = 0; i < planes.size(); ++i) {
        if (!std::isfinite(planes[i]) || (i > 0 && !(planes[i] > planes[i - 1]))) return false;
    }
    if (z1 == z0) return true;
    double const inverse_span = 1.0 / (z1 - z0);
    std::size_t const first =
        static_cast<std::size_t>(std::upper_bound(planes.begin(), planes.end(), std::min(z0, z1)) - planes.begin());
    std::size_t const last =
        static_cast<std::size_t>(std::upper_bound(planes.begin(), planes.end(), std::max(z0, z1)) - planes.begin());
    if (z1 > z0) {
        for (std::size_t i = first; i < last; ++i) cb(i, (planes[i] - z0) * inverse_span, 1);
    } else {
        for (std::size_t j = last; j > first; --j) cb(j - 1, (planes[j - 1] - z0) * inverse_span, -1);
    }
    return true;
}

// RreaPlaneFluxAccumulator::AddCrossing (I/RreaPlaneFlux.H:193-283) over the
// crossings in order, into 10 values per plane in Flatten's order; false
// (bins unchanged from the failing crossing on) on an invalid crossing.
bool AccumulatePlaneCrossings(std::vector<PlaneCrossing> const& crossings, std::vector<double>& bins);

// O/RreaCouplingSources.cpp:435-512 + S/RreaEventAccumulator.cpp:386-502
void DepositSources(rrea_gpu_config const& cfg, std::vector<Source> const& sources,
                    double low_energy_cutoff_eV, CellSources& cells);

}  // namespace oracle
