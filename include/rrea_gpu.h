/*
 * rrea_gpu.h — C-ABI of the GB300 kinetic step for the RREA overlay.
 *
 * This library replaces the per-timestep e-/e+/photon transport that the
 * reference runs inside
 *   void rrea::warpx::RreaParticleInteraction::Apply(WarpX&, RreaWarpXCoupling&,
 *        rrea::RreaInteractionTables const&, int step, amrex::Real time_s,
 *        amrex::Real dt_s)
 * (native_amrex_rrea/warpx_overlay/Source/Rrea/RreaParticleInteraction.H:1609-1623,
 *  body in RreaParticleInteraction.cpp:12-62).  The overlay keeps that C++
 * signature; its body gathers the species tiles, calls rrea_gpu_apply_electrons(),
 * rrea_gpu_apply_photons() and rrea_gpu_apply_positrons() (the reference's
 * phase order), and
 * raises amrex::Abort on a non-OK status, which preserves the fail-closed
 * contract of the reference (every guard aborts the whole step before any
 * side effect is committed).
 *
 * Plain pointers and sizes only; no C++ or torch types cross this boundary.
 * Every entry point returns an rrea_gpu_status; none aborts or traps.
 */
#ifndef RREA_GPU_H
#define RREA_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    RREA_GPU_OK = 0,
    RREA_GPU_ERR_ARGUMENT = 1,        /* bad pointer, size or configuration */
    RREA_GPU_ERR_TABLES = 2,          /* table bundle missing or violates its contract */
    RREA_GPU_ERR_CUDA = 3,            /* a CUDA runtime call failed */
    RREA_GPU_ERR_RANGE = 4,           /* a table query left its certified range */
    RREA_GPU_ERR_GEOMETRY = 5,        /* a particle state outside the domain or non-finite */
    RREA_GPU_ERR_RNG_OVERFLOW = 6,    /* packed RNG index / event ordinal overflow */
    RREA_GPU_ERR_GUARD = 7,           /* strict optical-depth subcycle guard */
    RREA_GPU_ERR_CAPACITY = 8,        /* an output buffer is too small for this step */
    RREA_GPU_ERR_INVALID_STATE = 9,   /* non-finite rate, invalid hazard selection */
    RREA_GPU_ERR_NOT_READY = 10       /* tables, field or particles not uploaded */
} rrea_gpu_status;

/* Species ordinals, as RreaSecondarySpecies
 * (RreaParticleInteraction.H:28-32). */
enum { RREA_SPECIES_ELECTRON = 0, RREA_SPECIES_POSITRON = 1, RREA_SPECIES_PHOTON = 2 };

/*
 * Per-run transport configuration.  Field meanings follow
 * RreaParticleInteractionConfig (RreaParticleInteraction.H:1576-1596) and the
 * coupling accessors LowEnergyCutoffEv / PhotonCutoffEv / RngSeed
 * (RreaWarpXCoupling.H:240-250).  rrea_gpu_default_config() fills the
 * reference defaults.
 */
typedef struct {
    /* geometry: RZ domain [r_lo, r_hi) x [z_lo, z_hi), cells nr x nz */
    double r_lo, r_hi, z_lo, z_hi;
    int32_t nr, nz;
    int32_t periodic_z;
    int32_t strict_transport_guards;
    /* material: uniform density ratio rho/rho_table (rho_table = 1.20479 kg/m^3) */
    double density_ratio;
    /* cuts; photon_cutoff_eV is forced to the tables' brems cutoff */
    double low_energy_cutoff_eV;
    double photon_cutoff_eV;
    /* substep controls */
    double max_optical_depth_per_substep;
    uint64_t max_subcycles;
    double max_gs_collisions_per_substep;
    double gs_total_collision_cap;
    double max_field_impulse_fraction;
    double field_impulse_floor_eV;
    uint64_t rng_seed;
    int32_t debug_disable_hard_moller;
    int32_t reserved0;
} rrea_gpu_config;

typedef struct rrea_gpu_ctx rrea_gpu_ctx;

/* Reference defaults (RreaParticleInteraction.H:1576-1596; tracking cut 1 keV). */
void rrea_gpu_default_config(rrea_gpu_config* cfg);

/* Creates a context on the current CUDA device.  Allocates device scratch
 * sized for `capacity` particles per species. */
rrea_gpu_status rrea_gpu_create(const rrea_gpu_config* cfg, int64_t capacity, rrea_gpu_ctx** out);
rrea_gpu_status rrea_gpu_destroy(rrea_gpu_ctx* ctx);

/* Loads transport_physics.json and its RREATBL containers
 * (replaces RreaInteractionTables::Load, S/RreaInteractionTables.cpp:1659). */
rrea_gpu_status rrea_gpu_load_tables(rrea_gpu_ctx* ctx, const char* transport_physics_json);

/* Binds an altitude density profile to the transport
 * (rrea.air_density_model=altitude_profile; replaces the profile half of
 * RreaWarpXCoupling::TransportDensityRatioAtZ, O/RreaWarpXCoupling.cpp:79-95,
 * and RreaAltitudeProfile, S/RreaAltitudeProfile.cpp:37-147).  The density
 * ratio at axial position z is Interpolate(altitude_msl_at_z0_m + z) /
 * reference_density_kg_m3, linear between the n nodes; every material
 * interval takes it at its piece midpoint (O/RreaMaterialPath.H:60-114).
 * Altitudes strictly increasing, densities strictly positive and finite,
 * n >= 2, reference density positive (RREA_GPU_ERR_ARGUMENT otherwise); the
 * domain's axial centre, where each step takes its fallback ratio
 * (O/RreaParticleInteraction.cpp:27-35), must lie inside the profile
 * (RREA_GPU_ERR_RANGE).  A transport query outside the profile fails the
 * step with RREA_GPU_ERR_RANGE, as the reference throws.  n == 0 restores the
 * configured uniform ratio.  Host pointers, copied. */
rrea_gpu_status rrea_gpu_set_density_profile(rrea_gpu_ctx* ctx, const double* altitude_m,
                                             const double* density_kg_m3, int64_t n,
                                             double altitude_msl_at_z0_m,
                                             double reference_density_kg_m3);

/*
 * Plane-crossing diagnostic (rrea.cd_plane_z_m; RreaPlaneFluxState and
 * RreaPlaneFluxAccumulator, I/RreaPlaneFlux.H; the crossings of
 * defer_cd_electron_plane_crossings, O/RreaTransportStep.H:249-332, taken
 * by the electron phase and the electrons' newborn legs).  Every electron
 * continuous-loss segment adds its weight to each plane it crosses
 * (upward z0 < plane <= z1, downward z1 < plane <= z0), per direction, in
 * three selections: all tracked, local runaway (|E| at the crossing above
 * the ensemble mean drag at the crossing energy), and >= 1 MeV; the local
 * runaways also add w r and w r^2.  The accumulators are cumulative on the
 * device (atomics), 10 per plane in RreaPlaneFluxAccumulator::Flatten's
 * order: all up/down, local-runaway up/down, >= 1 MeV up/down, w r up/down,
 * w r^2 up/down.
 *
 * set_planes: n_planes strictly increasing finite z (0 turns it off; not in
 * ensemble mode); the accumulators start at zero.  plane_flux copies them
 * out (10 n_planes doubles).  restore_plane_flux sets them (RestoreFlat:
 * finite and nonnegative), NULL zeroes them.
 */
rrea_gpu_status rrea_gpu_set_planes(rrea_gpu_ctx* ctx, const double* plane_z, int32_t n_planes);
rrea_gpu_status rrea_gpu_plane_flux(rrea_gpu_ctx* ctx, double* values);
rrea_gpu_status rrea_gpu_restore_plane_flux(rrea_gpu_ctx* ctx, const double* values);

/* Sets the Maxwell (scattered) field and the static ambient field on the
 * replicated TM-RZ vectors (I/RreaMaxwellTMRZ.H:61-85): er (nr+1)*nz,
 * ez nr*(nz+1), btheta (nr+1)*(nz+1); amb_er/amb_ez as er/ez.  Host pointers. */
rrea_gpu_status rrea_gpu_set_field(rrea_gpu_ctx* ctx, const double* er, const double* ez,
                                   const double* btheta, const double* amb_er,
                                   const double* amb_ez);

/*
 * One species tile in host memory, as the overlay's WarpX tile holds it
 * (PIdx r, z, theta, ux, uy, uz, w and the runtime rrea_prev_* components,
 * RreaWarpXCoupling.cpp:111-149).  id > 0 marks a valid particle; the step
 * negates the id of every particle it removes.
 */
typedef struct {
    int64_t n;
    double* r;
    double* z;
    double* theta;
    double* ux;
    double* uy;
    double* uz;
    double* w;
    double* prev_r;
    double* prev_z;
    double* prev_theta;
    double* prev_ux;
    double* prev_uy;
    double* prev_uz;
    int64_t* id;
    int32_t* cpu;
} rrea_gpu_tile;

/* One secondary produced by the step (RreaSecondaryParticle,
 * RreaParticleInteraction.H:612-635), in the reference's deterministic
 * order (parent index, then creation order within the parent). */
typedef struct {
    int32_t species;
    int32_t process;
    int32_t root_species;
    int32_t pad;
    int64_t parent_index;
    uint64_t root_key;
    uint64_t lineage;
    double x, y, z, dir_x, dir_y, dir_z, weight, energy_eV, birth_fraction;
} rrea_gpu_secondary;

/*
 * Drop-in for the electron phase of RreaParticleInteraction::Apply
 * (TransportStep::ApplyElectronTransport, RreaElectronTransport.cpp:9-902):
 * copies the tile to HBM, transports every valid electron through one outer
 * step dt on the GPU, copies the tile back, and returns the secondaries in
 * deterministic order.  `secondaries` may be NULL to only count them.
 */
rrea_gpu_status rrea_gpu_apply_electrons(rrea_gpu_ctx* ctx, rrea_gpu_tile* tile, int32_t step,
                                         double time_s, double dt_s,
                                         rrea_gpu_secondary* secondaries,
                                         int64_t secondary_capacity, int64_t* n_secondaries);

/* Cell-source grids (S/RreaEventAccumulator.cpp:129-164 field ids 0..4:
 * low-energy electrons, positive ions, direct negative ions, ionization
 * count, energy loss), each nr*nz, i + nr*j.  Accumulated since the last
 * rrea_gpu_reset_sources(). */
rrea_gpu_status rrea_gpu_download_sources(rrea_gpu_ctx* ctx, double* out5);
rrea_gpu_status rrea_gpu_reset_sources(rrea_gpu_ctx* ctx);

/*
 * Net-chord current of the charged phases (RREA J deposition,
 * RreaWarpXCoupling.cpp:417-544 with RreaSegmentDepositionRZ.H): each
 * transported electron or positron deposits its committed chord (captured
 * start -> end point, stop point or annihilation point), and each escape its
 * chord to the exact face crossing plus the boundary-cloud closure, as
 * charge-conserving (Umeda zigzag) index-space fluxes on the coupling's padded
 * grid (nr + 2 cells in r; nz + 4 in z, two pad cells below and above).  The
 * grid accumulates over the phases run since the last reset; the reference
 * resets it once per step (ResetNetChordStep).  Only for a non-periodic z
 * domain (the reference refuses periodic z here); otherwise these calls return
 * RREA_GPU_ERR_ARGUMENT.
 *   download_current:        physical face current densities [A/m^2],
 *                            Jr (nr+1)*nz and Jz nr*(nz+1), index i + stride*j
 *                            (ConvertPaddedIndexCurrentToPhysicalRZ).
 *   download_current_index:  the padded grids themselves: rho (nr+2)*(nz+4),
 *                            Jr (nr+3)*(nz+4), Jz (nr+2)*(nz+5), in units of
 *                            weight * index / s (for continuity checks).
 */
rrea_gpu_status rrea_gpu_reset_current(rrea_gpu_ctx* ctx);
rrea_gpu_status rrea_gpu_download_current(rrea_gpu_ctx* ctx, double* jr, double* jz);
rrea_gpu_status rrea_gpu_download_current_index(rrea_gpu_ctx* ctx, double* rho, double* jr, double* jz);

/*
 * Field update kept on the device (RreaAmrexAdvance::AdvanceOneStep's Maxwell
 * part, S/RreaAmrexAdvance.cpp:593-800, with the leapfrog of
 * RreaMaxwellTMRZ.H:147-228): the accumulated net-chord current is converted
 * to physical Jr/Jz and drives `substeps` equal leapfrog substeps of the
 * scattered TM field (B restaggered by (dt - dt_sub)/2 before and after,
 * first-order Silver-Mueller on the open faces).  The kinetic current alone:
 * with the carrier fluid, rrea_gpu_advance_field_coupled runs the step with
 * the fluid's current and conductivity instead.  The cell fields the transport gathers are refreshed afterwards.  Refuses a
 * step violating c dt sqrt(dr^-2 + dz^-2) < 1, and periodic z.
 */
rrea_gpu_status rrea_gpu_advance_field(rrea_gpu_ctx* ctx, double dt_s, int32_t substeps);
/* Copies the scattered field vectors (layouts as rrea_gpu_set_field). */
rrea_gpu_status rrea_gpu_download_field(rrea_gpu_ctx* ctx, double* er, double* ez, double* btheta);

/*
 * The field update of a sharded run, in two halves around the caller's
 * allreduce of the face current (the only exchange of the path;
 * RreaWarpXCoupling.cpp:715-717, RreaAmrexAdvance.cpp:870-871).
 * current_device converts the step's net-chord current to the physical
 * face currents and returns their device vectors on the context's device
 * (Jr: (nr+1)*nz doubles, Jz: nr*(nz+1), layouts as download_current); the
 * caller sums them across ranks in place.  advance_field_from_current then
 * runs the Maxwell update of advance_field on those vectors as they stand.
 * advance_field is current_device followed by advance_field_from_current.
 */
rrea_gpu_status rrea_gpu_current_device(rrea_gpu_ctx* ctx, double** d_jr, double** d_jz);
rrea_gpu_status rrea_gpu_advance_field_from_current(rrea_gpu_ctx* ctx, double dt_s, int32_t substeps);

/*
 * Population ceiling (RreaWarpXCoupling::EnforcePopulationCeiling,
 * RreaCouplingPopulation.cpp:100-146).  count_live counts the valid
 * (id > 0) particles of the context's resident tile of `species`.
 * population_projection is RreaStrictPopulationProjection
 * (RreaParticleInteraction.H:1257-1275): survivors = current - removals,
 * projected = survivors + insertions (saturating at UINT64_MAX on overflow);
 * RREA_GPU_OK when projected <= ceiling (< ceiling with reject_equality),
 * RREA_GPU_ERR_CAPACITY otherwise or when removals > current, where the
 * reference aborts.  A ceiling of 0 means "no ceiling" in the reference and
 * is the caller's to skip.  No context is needed for the projection.
 */
rrea_gpu_status rrea_gpu_count_live(rrea_gpu_ctx* ctx, int32_t species, int64_t* live);

/*
 * Charge of the resident charged particles on the cell-centred grid
 * (RreaWarpXCoupling::DepositParticleChargeToRreaGrid,
 * O/RreaWarpXCoupling.cpp:376-389, in the cell-centred CIC convention of
 * DepositChargeCIC, I/RreaSegmentDepositionRZ.H:68-92): every valid electron
 * deposits -w and every valid positron +w with bilinear weights from the
 * four nearest cell centres, the support folded evenly at the axis and
 * clamped at r_hi and both z edges.  rho receives nr*nz values (index
 * i + nr*j) in elementary charges per cell; the charge density in C/m^3 is
 * rho * 1.602176634e-19 / (pi (r_{i+1}^2 - r_i^2) dz).  WarpX's own
 * DepositCharge is in the absent WarpX sources: this is the reference's
 * header convention.  Host pointer. */
rrea_gpu_status rrea_gpu_deposit_charge_resident(rrea_gpu_ctx* ctx, double* rho);

/*
 * Census of a resident species tile: the particle reductions of the
 * overlay's reduced diagnostics (species_weight_statistics and
 * electron_species_weight_above_energy, O/RreaCouplingDiagnostics.cpp:122-194,
 * behind the N_kinetic_e_real, N_kinetic_e_ge_1MeV_real, N_photon_real and
 * N_positron_real columns of rrea_reduced.csv) plus a weighted energy
 * spectrum, reduced on the device.  Over the valid (id > 0) particles, with
 * K = RreaKineticEnergyEvFromProperVelocity(u) for e-/e+
 * (O/RreaParticleInteraction.H:1494-1505) and K = |u| for photons, out gets
 *   [0] count  [1] largest weight  [2] sum w  [3] sum w^2  [4] sum w K [eV]
 *   [5] weight with K < edges[0]  [6] weight with K >= edges[n_edges - 1]
 *   [7 .. 7 + n_thresholds)              weight with K >= thresholds_eV[t]
 *   [7 + n_thresholds .. + n_edges - 1)  weight with edges[b] <= K < edges[b+1]
 * K is evaluated with round-to-nearest operations in this formula's order,
 * so bin and threshold membership are exact; the sums are FP64 atomics.
 * 2 <= n_edges <= 1025 (strictly increasing), 0 <= n_thresholds <= 16; host
 * pointers. */
rrea_gpu_status rrea_gpu_census_resident(rrea_gpu_ctx* ctx, int32_t species, const double* edges_eV, int32_t n_edges,
                                         const double* thresholds_eV, int32_t n_thresholds, double* out);
rrea_gpu_status rrea_gpu_population_projection(uint64_t current, uint64_t removals, uint64_t insertions,
                                               uint64_t ceiling, int32_t reject_equality, uint64_t* projected);

/* Commits the survivors of the last resident drain (rrea_gpu_drain_resident)
 * into the resident species tiles: the particle-creation half of
 * DrainAndCommitSecondaries (RreaWarpXCoupling::CommitLocalParticleBatch,
 * O/RreaCouplingSources.cpp:240-330, with the captured pre-push state of
 * append_rrea_previous_position_attributes, :28-100).  Each record becomes a
 * particle at (hypot(x, y), z, atan2(y, x)) with, for e-/e+, the proper
 * velocity of its kinetic energy along its direction and, for photons, the
 * momentum E along it; records with weight <= 0 (and photons with E <= 0)
 * are dropped as there.  Particles are appended in FIFO order with ids
 * continuing after the largest id staged for the species (AMReX's NextID is
 * in the absent AMReX sources: this is the library's rule).  committed[3]
 * (may be null) receives the counts per species (RREA_SPECIES_* order).
 * RREA_GPU_ERR_CAPACITY, with no tile changed, when a tile would exceed the
 * context capacity. */
rrea_gpu_status rrea_gpu_commit_survivors_resident(rrea_gpu_ctx* ctx, int64_t* committed);

/* Removes the invalid particles (id <= 0: escaped, demoted, annihilated)
 * from a resident species tile, keeping the order of the valid ones, as
 * WarpX's removal of invalid particles does between steps.  n_live (may be
 * null) receives the new tile size. */
rrea_gpu_status rrea_gpu_compact_resident(rrea_gpu_ctx* ctx, int32_t species, int64_t* n_live);

/* Charge-exact stochastic thinning of order-1 CIC support groups, the
 * per-support primitive of the population control's adaptive_resample_v1
 * (RreaThinCicWeights and RreaCicResampleRemovalCapacity,
 * I/RreaCicConservingResample.H:46-351).  Group g is rows
 * [offsets[g], offsets[g+1]) (at most 64) of fraction_r, fraction_z (the
 * order-1 CIC fractions in [0, 1]) and weight (updated in place: removed
 * particles get weight 0; the four cell charges are kept to round-off and
 * each weight keeps its expectation).  At most max_removals[g] particles
 * are removed, with uniforms u_k = (mix64(keys[g] + k) >> 11 + 1/2) 2^-53
 * (mix64 = RreaCicMix64).  Per group: removed, draws, valid (0 where the
 * reference's primitive reports an invalid plan, weights then partly
 * updated as there) and the removal capacity (live particles minus the rank
 * of their CIC columns).  The global planning of the transaction (which
 * supports thin and by how much) is not part of this call.  Host pointers;
 * groups of more than 64 particles give RREA_GPU_ERR_ARGUMENT. */
rrea_gpu_status rrea_gpu_thin_cic_groups(rrea_gpu_ctx* ctx, const double* fraction_r, const double* fraction_z,
                                        double* weight, const int64_t* offsets, int64_t n_groups,
                                        const int64_t* max_removals, const uint64_t* keys, int64_t* removed,
                                        int64_t* draws, int32_t* valid, int64_t* capacity);

/*
 * Adaptive population control (rrea.population_ceiling_policy =
 * adaptive_resample_v1) of the resident electron or positron population.
 *
 * population_thin_resident is the global thinning plan of
 * RreaWarpXCoupling::PreflightAndApplySecondaryPopulationControl
 * (O/RreaCouplingPopulation.cpp:175-640) on one rank: when the live
 * particles of `species` plus its staged candidates exceed 1.25 x target,
 * min(members - target, removal capacity) particles leave by charge-exact
 * thinning of their order-1 CIC supports (RreaPlanGlobalCicThinning,
 * I/RreaCicConservingResample.H:489-640), support by support in sorted
 * order, with the species' RreaAdaptiveResampleCicUniform stream
 * (rng_seed, group id ^ salt, step).  A live particle thinned to weight 0 is
 * invalidated (negated id: rrea_gpu_compact_resident removes it); a
 * candidate keeps its record with its new weight (weight 0: dropped at the
 * commit).  The candidates are the last resident drain's survivors when
 * `candidates` is NULL (call between rrea_gpu_drain_resident and
 * rrea_gpu_commit_survivors_resident), else the n_candidates host records,
 * whose weights are updated in place.  stats (may be NULL) receives 8
 * values: members, live members, candidate members, supports, removal
 * capacity, geometric floor, nominal request, removed.  Nothing is applied
 * when a support's plan is rejected or the plans remove less than the
 * nominal request (RREA_GPU_ERR_INVALID_STATE, where the reference aborts),
 * or when a particle lies beyond 32767 cells of the grid
 * (RREA_GPU_ERR_GEOMETRY).  Live stable ids are the packed id/cpu word
 * (id << 24 | cpu): AMReX's own packing is in the absent AMReX sources.
 *
 * population_split_resident is the split refill of
 * AdaptiveResampleOneSpecies (:686-767): when 0 < live < target/2 and the
 * floor is positive, every valid particle with weight >= 2 x floor halves
 * its weight and an identical clone (captured state = own state, cpu word
 * kept) joins the tile end in tile order with the next species ids
 * (RreaAdaptiveResampleSplitOutcome, O/RreaRng.H:163-175).  added (may be
 * NULL) receives the clone count; RREA_GPU_ERR_CAPACITY, with nothing
 * changed, when the clones do not fit.
 */
rrea_gpu_status rrea_gpu_population_thin_resident(rrea_gpu_ctx* ctx, int32_t species, int64_t target, int32_t step,
                                                 uint64_t salt, rrea_gpu_secondary* candidates, int64_t n_candidates,
                                                 int64_t* stats);
rrea_gpu_status rrea_gpu_population_split_resident(rrea_gpu_ctx* ctx, int32_t species, int64_t target,
                                                  double split_min_weight, int64_t* added);

/*
 * Weight-doubling merge above the cap, for a resident species tile.  NO
 * COUNTERPART IN THE REFERENCE: above its cap the overlay either aborts
 * (strict_abort_v1, O/RreaCouplingPopulation.cpp:100-146) or thins
 * (adaptive_resample_v1, above); the scale-up and profiled-atmosphere
 * cases ask for a merge that doubles weights instead, validated
 * statistically.
 *
 * When the tile holds more than `target` valid particles, they are grouped
 * by (cell-centred grid cell of the position, the quarter octave of |u|^2,
 * the sign of u_z) and, inside a group, consecutive particles in tile order
 * pair up.  R = min(live - target, pairs) pairs merge, spread evenly over
 * the pairs in group order (pair j when floor((j+1) R / P) > floor(j R / P)).
 * A merging pair (a, b) keeps a with probability w_a / (w_a + w_b), else b,
 * with a counter-hash uniform of (rng_seed, species, step, the two stream
 * keys |id| ^ cpu << 40); the kept particle carries w_a + w_b and the other
 * is invalidated (negated id: rrea_gpu_compact_resident removes it).  Every
 * weighted sum keeps its expectation, each cell's weight is kept exactly
 * (up to the rounding of w_a + w_b), and the same call gives the same result
 * on the same tile.  stats (may be NULL) receives 5 values: live particles,
 * groups, pairs, requested merges, merged pairs.  Not in ensemble mode.
 */
rrea_gpu_status rrea_gpu_population_merge_resident(rrea_gpu_ctx* ctx, int32_t species, int64_t target, int32_t step,
                                                  int64_t* stats);

/* Number of particles (valid or not) in a resident species tile.  NO COUNTERPART IN THE
 * REFERENCE (WarpX containers know their own size). */
rrea_gpu_status rrea_gpu_resident_count(rrea_gpu_ctx* ctx, int32_t species, int64_t* n);

/*
 * Transient FIFO of DrainAndCommitSecondaries (RreaSecondaryCommit.cpp:9-638,
 * residual advance RreaNewbornAdvance.cpp:20-996).  Every pending secondary
 * born at elapsed fraction b < 1 is flown through the remaining (1 - b) dt of
 * the step on its root particle's RNG streams (Newborn* channels 112-123);
 * its children join the FIFO behind every queued item (a breadth-first walk)
 * with a lineage from the per-root counter; the survivors come back in FIFO
 * order with birth_fraction 1, ready for the overlay's AddNParticles.  The
 * residual flights deposit into the context's cell sources and net-chord
 * current.  Birth payloads are checked first (RREA_GPU_ERR_ARGUMENT: unknown
 * species, non-finite fields, weight <= 0, birth outside [0, 1], lineage at
 * the 2^14 capacity) and survivors last (RREA_GPU_ERR_INVALID_STATE), where
 * the reference aborts the transaction.
 *   drain_secondaries: host records in (the Apply secondaries of every phase,
 *                      in phase order), host survivors out.  Discards the
 *                      resident queue.
 *   drain_resident:    drains the queue that the rrea_gpu_step_*_resident
 *                      calls filled since the last drain; survivors stay in
 *                      HBM until fetch_survivors.
 *   pending_secondaries: size of the resident queue; discard != 0 empties it.
 *   last_drain_stats:  FIFO items advanced and survivors of the last drain.
 */
/*
 * The whole of RreaParticleInteraction::Apply in one call
 * (O/RreaParticleInteraction.cpp:12-62: the electron, photon and positron
 * phases, then DrainAndCommitSecondaries, O/RreaSecondaryCommit.cpp:9-638,
 * up to the survivors' AddNParticles): each host tile goes up, its phase
 * runs as rrea_gpu_apply_* does, the phases' secondaries queue on the device
 * in phase order and the transient FIFO drains them there (as
 * rrea_gpu_drain_secondaries would over the concatenated secondaries), then
 * the tiles come back and the survivors land in `survivors` in FIFO order.
 * A NULL tile skips its species.  The caller's tiles and survivor buffer
 * change only when every phase and the drain succeeded (fail closed); a
 * survivor count above survivor_capacity is RREA_GPU_ERR_CAPACITY with
 * *n_survivors set.  Results equal the per-phase calls followed by
 * drain_secondaries; no secondary crosses to the host.
 */
rrea_gpu_status rrea_gpu_apply_step(rrea_gpu_ctx* ctx, rrea_gpu_tile* electrons, rrea_gpu_tile* photons,
                                    rrea_gpu_tile* positrons, int32_t step, double time_s, double dt_s,
                                    rrea_gpu_secondary* survivors, int64_t survivor_capacity, int64_t* n_survivors);
rrea_gpu_status rrea_gpu_drain_secondaries(rrea_gpu_ctx* ctx, const rrea_gpu_secondary* pending,
                                           int64_t n_pending, int32_t step, double dt_s,
                                           rrea_gpu_secondary* survivors, int64_t survivor_capacity,
                                           int64_t* n_survivors);
rrea_gpu_status rrea_gpu_drain_resident(rrea_gpu_ctx* ctx, int32_t step, double dt_s, int64_t* n_survivors);
rrea_gpu_status rrea_gpu_fetch_survivors(rrea_gpu_ctx* ctx, rrea_gpu_secondary* survivors, int64_t capacity,
                                         int64_t* n_survivors);
rrea_gpu_status rrea_gpu_pending_secondaries(rrea_gpu_ctx* ctx, int64_t* n_pending, int32_t discard);
rrea_gpu_status rrea_gpu_last_drain_stats(rrea_gpu_ctx* ctx, int64_t* fifo_items, int64_t* survivors);

/* Per-particle diagnostics of the last electron step: substeps used,
 * hazard draws made and terminal disposition (0 survive, 1 escape,
 * 2 demotion, 3 zero-weight skip, -1 not transported). */
rrea_gpu_status rrea_gpu_download_diagnostics(rrea_gpu_ctx* ctx, int64_t n, uint64_t* subcycles,
                                              uint64_t* events, int32_t* disposition);

/* Accuracy check of the device's table-driven logarithm (which = 0) and
 * exponential (which = 1): for the n host values x, writes the table-driven
 * result and the CUDA function's, both computed on the device.  Needs loaded
 * tables (the math tables open the arena).  NO COUNTERPART IN THE REFERENCE. */
rrea_gpu_status rrea_gpu_selftest_math(rrea_gpu_ctx* ctx, int32_t which, const double* x, int64_t n, double* fast,
                                       double* libm);

/* Kernels this library has launched in this process (all contexts), for
 * launch accounting around a timed region.  NO COUNTERPART IN THE REFERENCE. */
rrea_gpu_status rrea_gpu_kernel_launches(uint64_t* count);

/* Copies the last error message (NUL-terminated, truncated to size). */
void rrea_gpu_last_error(const rrea_gpu_ctx* ctx, char* buf, size_t size);

/*
 * Resident engine mode: the electron tile stays in HBM across steps.  In this
 * mode the captured pre-push state (rrea_prev_*) IS the current state, which
 * is what CaptureRreaPositionsBeforePush (RreaWarpXCoupling.cpp:151-208)
 * establishes before WarpX's own charged push, whose kick the transport step
 * discards (RreaTransportStep.H:705-820).
 *   stage:  host tile -> HBM (prev_* are ignored)
 *   step:   one outer step on the resident tile, no host copies; its ordered
 *           secondaries join the resident drain queue
 *   fetch:  HBM -> host tile (r, z, theta, ux, uy, uz, w, id, cpu; tile->n must equal
 *           rrea_gpu_resident_count, which committed survivors and compaction change)
 */
rrea_gpu_status rrea_gpu_stage_electrons(rrea_gpu_ctx* ctx, const rrea_gpu_tile* tile);
rrea_gpu_status rrea_gpu_step_electrons_resident(rrea_gpu_ctx* ctx, int32_t step, double dt_s,
                                                 int64_t* n_secondaries);
rrea_gpu_status rrea_gpu_fetch_electrons(rrea_gpu_ctx* ctx, rrea_gpu_tile* tile);

/*
 * Drop-in for the positron phase of RreaParticleInteraction::Apply
 * (TransportStep::ApplyPositronTransport, RreaPositronTransport.cpp:9-878):
 * the electron engine with charge +1, the Bhabha / brems / in-flight
 * annihilation channels (RreaChargedFinalStates.H:226-394,
 * RreaTransportStep.H:563-702) and at-rest annihilation below the cutoff.
 * Tile, secondaries and diagnostics as for electrons; disposition 2 means
 * annihilated; secondaries carry root_species = RREA_SPECIES_POSITRON.
 */
rrea_gpu_status rrea_gpu_apply_positrons(rrea_gpu_ctx* ctx, rrea_gpu_tile* tile, int32_t step,
                                         double time_s, double dt_s,
                                         rrea_gpu_secondary* secondaries,
                                         int64_t secondary_capacity, int64_t* n_secondaries);

/* Resident positron mode: as the resident electron mode, on the context's
 * positron tile. */
rrea_gpu_status rrea_gpu_stage_positrons(rrea_gpu_ctx* ctx, const rrea_gpu_tile* tile);
rrea_gpu_status rrea_gpu_step_positrons_resident(rrea_gpu_ctx* ctx, int32_t step, double dt_s,
                                                 int64_t* n_secondaries);
rrea_gpu_status rrea_gpu_fetch_positrons(rrea_gpu_ctx* ctx, rrea_gpu_tile* tile);

/*
 * Drop-in for the photon phase of RreaParticleInteraction::Apply
 * (TransportStep::ApplyPhotonTransport, RreaPhotonTransport.cpp:9-461, final
 * states RreaPhotonFinalStates.H:56-365).  The tile's (r, theta, z) is the
 * end point of WarpX's straight photon push and prev_* its captured start;
 * (ux, uy, uz) is the photon momentum in eV.  Each photon flies its chord,
 * interacts at most once per chord (Compton continues along the new
 * direction for the rest of the chord), and the absorbed or escaped ones
 * get a negated id.  Secondaries come back in deterministic order with
 * root_species = RREA_SPECIES_PHOTON.  Diagnostics: subcycles 0, events =
 * hazard draws, disposition 0 survive, 1 escape, 2 absorbed.
 */
rrea_gpu_status rrea_gpu_apply_photons(rrea_gpu_ctx* ctx, rrea_gpu_tile* tile, int32_t step,
                                       double time_s, double dt_s,
                                       rrea_gpu_secondary* secondaries,
                                       int64_t secondary_capacity, int64_t* n_secondaries);

/*
 * Resident photon mode: the context keeps one resident tile per species, so
 * the photon tile stays in HBM next to the electron tile.  The staged photon
 * tile holds photons at their start point.
 * The step pushes each photon straight by c*dt along its momentum (the
 * WarpX photon pusher, x += c dt u/|u| in Cartesian coordinates) and then
 * runs the photon phase on that chord, all on the device.  stage/fetch move
 * the tile as for electrons.
 */
rrea_gpu_status rrea_gpu_stage_photons(rrea_gpu_ctx* ctx, const rrea_gpu_tile* tile);
rrea_gpu_status rrea_gpu_step_photons_resident(rrea_gpu_ctx* ctx, int32_t step, double dt_s,
                                               int64_t* n_secondaries);
rrea_gpu_status rrea_gpu_fetch_photons(rrea_gpu_ctx* ctx, rrea_gpu_tile* tile);

/* Launch shape of the transport kernels: threads per block (32..128, a
 * multiple of 32) and resident 128-thread blocks per SM (1 to 64; the
 * electron kernel variant follows the residency: 2, 4, 8, 12 or 16 blocks
 * with 255, 128, 64, 40 or 32 registers per thread; default 16, the full
 * 64 warps per SM; the positron kernel has the 2, 4, 8 and 16 variants).
 * A charged tile too small to fill that residency in one wave runs the
 * variant with the most registers that still holds it (results do not
 * depend on the variant).  The grid is one resident wave with a grid-stride
 * loop.  `diagnostics` enables the per-particle diagnostic arrays. */
rrea_gpu_status rrea_gpu_set_launch(rrea_gpu_ctx* ctx, int32_t threads_per_block, int32_t blocks_per_sm,
                                    int32_t diagnostics);
/* Scheduling order of the resident charged phases: 1 (default) visits a
 * tile of 65,536 or more particles lowest |u| first, by a counting sort of
 * the tile each step; 0 visits it in tile order.  Results never depend on
 * it (every result is indexed by the particle's tile slot). */
rrea_gpu_status rrea_gpu_set_schedule(rrea_gpu_ctx* ctx, int32_t cost_order);

/* Counts and device time of the last step: particles transported (valid on
 * entry), secondaries produced, and the transport kernel's duration measured
 * with CUDA events on the context stream. */
rrea_gpu_status rrea_gpu_last_step_stats(rrea_gpu_ctx* ctx, int64_t* transported, int64_t* secondaries,
                                         double* kernel_ms);

/* The context's CUDA stream (a cudaStream_t), for timing with events. */
rrea_gpu_status rrea_gpu_stream(rrea_gpu_ctx* ctx, void** stream);

/*
 * Allocation-free secondary ordering.  NO COUNTERPART IN THE REFERENCE: the
 * reference orders secondaries on the host inside its transport step; this
 * entry point exists for device-side integrations.
 *
 * Puts `n_secondaries` records from d_unordered into d_ordered in the
 * deterministic order of rrea_gpu_apply_electrons / rrea_gpu_apply_photons
 * (parent index, then lineage): record s goes to
 * (sum of d_counts[0 .. s.parent_index-1]) + s.lineage.
 *
 * Who needs it: a caller that owns every device buffer through its own
 * arena or fixed memory budget (for example a PIC code whose particle and
 * field arena already holds the GPU's memory) and therefore must not have a
 * library call cudaMalloc or cudaFree in the middle of its step - those
 * calls would bypass the arena's accounting, and cudaFree synchronizes the
 * whole device.  This function calls no allocating routine: its scratch
 * (per-parent offsets, scan block sums, an error word; about 2 MiB) is a
 * fixed device array inside this library, sized for at most
 * RREA_GPU_NOALLOC_MAX_PARENTS parents per call.
 *
 * Arguments (all device pointers in the current device's memory):
 *   d_counts      n_parents uint32 counts: records per parent
 *   d_unordered   n_secondaries records; each (parent_index, lineage) pair
 *                 must appear once, with lineage < d_counts[parent_index]
 *   d_ordered     n_secondaries records of output; must not overlap
 *                 d_unordered; needs no initialisation
 *   stream        a cudaStream_t, or NULL for the legacy default stream
 *   message       optional host buffer for an error description
 * Nothing the caller passes needs to start at zero; the internal error word
 * is cleared by each call before use.
 *
 * Returns RREA_GPU_ERR_CAPACITY (with a message) when n_parents exceeds
 * RREA_GPU_NOALLOC_MAX_PARENTS, RREA_GPU_ERR_ARGUMENT for negative sizes,
 * null or overlapping buffers, and RREA_GPU_ERR_INVALID_STATE when the
 * records are inconsistent with the counts, including two records with the
 * same (parent_index, lineage) pair (such records are skipped, no
 * out-of-range write happens; the output's content is then unspecified).
 * The call blocks until the pass on `stream` has finished.
 *
 * Every call looks up the scratch array's device address for the current
 * device and context (cudaGetSymbolAddress, a host-side lookup), so the
 * address stays right after cudaDeviceReset or under another context.  The
 * first call on a device may load this library's device code there; if
 * stream capture is used anywhere in the process, make one call before
 * capture starts.  All calls on one device share the one scratch array,
 * which keeps the last call's contents: calls that overlap in time (from two
 * host threads, or on two streams) race on it and must be serialised by the
 * caller.
 */
#define RREA_GPU_NOALLOC_MAX_PARENTS (1 << 18)
rrea_gpu_status rrea_gpu_order_secondaries_noalloc(const uint32_t* d_counts, int64_t n_parents,
                                                   const rrea_gpu_secondary* d_unordered,
                                                   int64_t n_secondaries, rrea_gpu_secondary* d_ordered,
                                                   void* stream, char* message, size_t message_size);

/*
 * Seed schedule input adapter (RreaSeedSchedule, I/RreaSeedSchedule.H and
 * S/RreaSeedSchedule.cpp): the CSV event list the overlay injects as native
 * seeds.  Columns case_id, time_s, x_m, y_m, z_m, r_m, kinetic_energy_eV,
 * ux, uy, uz, weight_real_electrons (required) and macro_index, species_id
 * (optional: the CSV line number, electron).  Host-only calls except the
 * injection; no GPU is needed to load, list or validate a schedule.
 *   load:     the rows of case_id (all rows when empty or null), sorted by
 *             (time_s, macro_index) (S/RreaSeedSchedule.cpp:75-144);
 *             RREA_GPU_ERR_ARGUMENT on a missing file or column, a duplicate
 *             column or a non-numeric cell (message via
 *             rrea_gpu_seed_schedule_last_error).
 *   validate: RreaSeedSchedule::ValidateProduction (:146-244) against the
 *             certified charged energy range and the half-open RZ domain.
 *   events:   copies the sorted events out (capacity >= size).
 *   inject:   RreaWarpXCoupling::InjectScheduledSeeds
 *             (O/RreaCouplingSources.cpp:96-215) on the resident tiles: events
 *             from the schedule's cursor with time in [time_s, time_s + dt_s)
 *             are appended to the resident electron or positron tile, earlier
 *             (stale) events are skipped, the cursor advances past both; the
 *             momentum is RreaNormalizeSeedMomentum (I/RreaSeedSchedule.H:55-71),
 *             the weight weight_real_electrons, the captured state the
 *             particle's own, ids continue the species' counter.
 *             injected[2] (may be null): electrons, positrons added.
 *             RREA_GPU_ERR_CAPACITY, with nothing appended, past the capacity.
 */
typedef struct rrea_gpu_seed_schedule rrea_gpu_seed_schedule;
typedef struct {
    int32_t macro_index;
    int32_t species_id;   /* 1 electron, 2 positron */
    double time_s;
    double x_m, y_m, z_m, r_m;
    double kinetic_energy_eV;
    double ux, uy, uz;    /* direction hint (|u| < 1e6) or proper velocity (m/s) */
    double weight;        /* weight_real_electrons */
} rrea_gpu_seed_event;

rrea_gpu_status rrea_gpu_seed_schedule_load(const char* path, const char* case_id, rrea_gpu_seed_schedule** out);
rrea_gpu_status rrea_gpu_seed_schedule_free(rrea_gpu_seed_schedule* schedule);
rrea_gpu_status rrea_gpu_seed_schedule_size(const rrea_gpu_seed_schedule* schedule, int64_t* n);
rrea_gpu_status rrea_gpu_seed_schedule_events(const rrea_gpu_seed_schedule* schedule, rrea_gpu_seed_event* out,
                                              int64_t capacity, int64_t* n);
rrea_gpu_status rrea_gpu_seed_schedule_validate(const rrea_gpu_seed_schedule* schedule, double electron_min_energy_eV,
                                                double electron_max_energy_eV, double radial_min_m,
                                                double radial_max_m, double axial_min_m, double axial_max_m);
/* The message of the last failed seed-schedule call on this thread. */
void rrea_gpu_seed_schedule_last_error(char* buf, size_t size);
rrea_gpu_status rrea_gpu_inject_seeds_resident(rrea_gpu_ctx* ctx, rrea_gpu_seed_schedule* schedule, double time_s,
                                               double dt_s, int64_t* injected);

/*
 * ---- Low-energy carrier fluid -------------------------------------------
 * The three carrier densities of LowEnergyFluidState (S/LowEnergyFluidState.cpp,
 * S/LowEnergyFluidFaceTransport.cpp) held on the context's cell grid
 * (nr x nz, index i + nr*j), with their ionization source rates, the
 * conservative fluid charge, the diagnostic conductivity, and the
 * caller-evaluated closure fields.  Carrier ordinals: 0 positive ion,
 * 1 negative ion, 2 low-energy electron (the face-flux component order).
 */
enum {
    RREA_GPU_MOBILITY_ABSOLUTE = 0,       /* "absolute" */
    RREA_GPU_MOBILITY_EN_TABLE_FLUX = 1,  /* electrons: "en_table_flux_v1" */
    RREA_GPU_MOBILITY_REDUCED_STP = 2     /* ions: "reduced_stp_density_scaled" */
};
enum { RREA_GPU_ATTACHMENT_CONSTANT = 0, RREA_GPU_ATTACHMENT_EN_TABLE = 1 /* "en_table_attachment_v1" */ };

/* LowEnergyFluidConfig (I/LowEnergyFluidState.H:80-124) and the material
 * substep controls of RreaAmrexAdvanceConfig (I/RreaAmrexAdvance.H:51-58).
 * rrea_gpu_default_fluid_config() fills the reference defaults. */
typedef struct {
    double electron_mobility_m2_per_vs;                  /* 0.1 */
    double positive_ion_mobility_m2_per_vs;              /* 2e-4 */
    double negative_ion_mobility_m2_per_vs;              /* 2e-4 */
    double positive_ion_reduced_mobility_stp_m2_per_vs;  /* 0 */
    double negative_ion_reduced_mobility_stp_m2_per_vs;  /* 0 */
    double ion_mobility_density_ratio_floor;             /* 0 */
    double ion_drift_cfl;                                /* 0.5 */
    double transport_density_ratio;                      /* 1: Loschmidt-relative, where no ratio field is bound */
    double attachment_frequency_s;                       /* 2e6 */
    double electron_ion_recombination_coefficient_m3_per_s; /* 0 */
    double ion_ion_recombination_coefficient_m3_per_s;      /* 0 */
    double detachment_frequency_s;                          /* 0 */
    int32_t ion_drift_enable;                            /* 0 */
    int32_t electron_drift_enable;                       /* 1 */
    int32_t electron_mobility_model;                     /* RREA_GPU_MOBILITY_ABSOLUTE */
    int32_t ion_mobility_model;                          /* RREA_GPU_MOBILITY_ABSOLUTE */
    int32_t attachment_model;                            /* RREA_GPU_ATTACHMENT_CONSTANT */
    int32_t material_min_substeps;                       /* 2 */
    int32_t material_max_substeps;                       /* 64 */
    int32_t reserved0;
    double material_conduction_target;                   /* 0.08 */
    double material_conduction_guard;                    /* 0.1 */
    double material_diffusion_target;                    /* 0.8 */
    double material_diffusion_guard;                     /* 1.0 */
    double material_reaction_target;                     /* 0.08 */
    double material_reaction_guard;                      /* 0.1 */
} rrea_gpu_fluid_config;

void rrea_gpu_default_fluid_config(rrea_gpu_fluid_config* cfg);

/* Allocates the fluid state on the context's grid, all zero, and binds the
 * configuration (validated as ValidateCarrierTransportConfig,
 * S/LowEnergyFluidFaceTransport.cpp:87-163, plus the model names and
 * nonnegative finite recombination coefficients).  Calling it again rebinds
 * the configuration and keeps the state. */
rrea_gpu_status rrea_gpu_fluid_configure(rrea_gpu_ctx* ctx, const rrea_gpu_fluid_config* cfg);

/* Loads the dry-air electron closure table (LowEnergyElectronClosure::Load,
 * S/RreaInteractionTables.cpp:3267-3404: exact schema-3 header, strictly
 * increasing E/N nodes, positive coefficients, the derivation identities
 * within 1e-9) onto the device. */
rrea_gpu_status rrea_gpu_fluid_load_closure(rrea_gpu_ctx* ctx, const char* csv_path);

/* Host <-> device copies of the state (each pointer may be NULL to skip it).
 * set_state writes the carrier densities and the conservative charge;
 * get_state also reads the conductivity and the Maxwell time. */
rrea_gpu_status rrea_gpu_fluid_set_state(rrea_gpu_ctx* ctx, const double* n_pos, const double* n_neg,
                                         const double* n_e, const double* rho_fluid);
rrea_gpu_status rrea_gpu_fluid_get_state(rrea_gpu_ctx* ctx, double* n_pos, double* n_neg, double* n_e,
                                         double* rho_fluid, double* sigma, double* tau_m);
/* Source rates [m^-3 s^-1]: low-energy electrons, positive ions, direct
 * negative ions. */
rrea_gpu_status rrea_gpu_fluid_set_source_rates(rrea_gpu_ctx* ctx, const double* s_e, const double* s_pos,
                                                const double* s_neg);
rrea_gpu_status rrea_gpu_fluid_get_source_rates(rrea_gpu_ctx* ctx, double* s_e, double* s_pos, double* s_neg);
/* The Loschmidt-relative density ratio of every cell (the mobility and
 * closure density; NULL unbinds it and the scalar transport ratio applies). */
rrea_gpu_status rrea_gpu_fluid_set_density_ratio(rrea_gpu_ctx* ctx, const double* chi);
/* Caller-evaluated closure fields: electron mobility, attachment frequency
 * and the RZ diffusion tensor (3 x nr*nz: Drr, Drz, Dzz); NULL skips one. */
rrea_gpu_status rrea_gpu_fluid_set_closure_fields(rrea_gpu_ctx* ctx, const double* mu_e, const double* nu_att,
                                                  const double* diffusion3);
rrea_gpu_status rrea_gpu_fluid_get_closure_fields(rrea_gpu_ctx* ctx, double* mu_e, double* nu_att,
                                                  double* diffusion3);

/* The kinetic cell sources 0..2 accumulated since rrea_gpu_reset_sources,
 * normalised by cell volume and dt (RreaEventAccumulator::NormalizeAndSync,
 * S/RreaEventAccumulator.cpp:280-331) and copied into the fluid source rates
 * (O/RreaWarpXCoupling.cpp:689-706). */
rrea_gpu_status rrea_gpu_fluid_take_sources(rrea_gpu_ctx* ctx, double dt_s);

/* Local chemistry over dt (UpdateFromIonizationSource,
 * S/LowEnergyFluidState.cpp:105-308): exact attachment with the constant or
 * table frequency, detachment, electron-ion then ion-ion pair loss, the
 * conservative charge advanced by the source charge.  Fails closed with
 * RREA_GPU_ERR_INVALID_STATE when the normalised charge residual exceeds
 * 512 eps (or is not finite); *residual (may be NULL) receives it. */
rrea_gpu_status rrea_gpu_fluid_react(rrea_gpu_ctx* ctx, double dt_s, int32_t clear_sources, double* residual);
/* MaxReactionFrequency (S/LowEnergyFluidState.cpp:310-343). */
rrea_gpu_status rrea_gpu_fluid_max_reaction_frequency(rrea_gpu_ctx* ctx, double* out);
/* ComputeConductivity and ComputeFluidChargeDensity
 * (S/LowEnergyFluidState.cpp:345-455). */
rrea_gpu_status rrea_gpu_fluid_conductivity(rrea_gpu_ctx* ctx);
rrea_gpu_status rrea_gpu_fluid_charge_density(rrea_gpu_ctx* ctx);

/* BuildElectronClosureCellFields (S/LowEnergyFluidFaceTransport.cpp:1034-1243)
 * from cell fields er_cell/ez_cell (nr*nz; NULL for both: the cell averages
 * of the context's total field), writing the mobility, attachment and
 * diffusion fields.  diag (may be NULL) receives 8 doubles: min E/N, max
 * E/N [Td], held-below, above-range and invalid cell counts, electron count,
 * held-below electron count, electron source rate [1/s]. */
rrea_gpu_status rrea_gpu_fluid_evaluate_closure(rrea_gpu_ctx* ctx, const double* er_cell, const double* ez_cell,
                                                double* diag);

/* One explicit carrier-transport update over dt with the face field
 * efr ((nr+1)*nz) / efz (nr*(nz+1)) from the host (both NULL: the context's
 * total Yee field, scattered plus ambient): PrepareExplicitCarrierTransport,
 * BuildExplicitFaceTransport and ApplyExplicitCarrierTransport
 * (S/LowEnergyFluidFaceTransport.cpp:165-954).  flux_r (3*(nr+1)*nz) and
 * flux_z (3*nr*(nz+1)), species-major, receive the limited number fluxes
 * (may be NULL).  diag (may be NULL) receives 14 doubles: max face
 * conductivity, max explicit diffusion number, unlimited max outgoing CFL,
 * min outflow scale, limited outflow fraction, limited electron-number
 * fraction, max outgoing CFL, max drift speed, CFL dt, positive-ion centre
 * r and z, negative-ion centre r and z, mobility-weighted density ratio at
 * the positive-ion centre.  Fails closed (RREA_GPU_ERR_INVALID_STATE) on a
 * non-PSD tensor, a diffusion number >= 1, an outgoing CFL above
 * ion_drift_cfl, or a negative or non-finite density. */
rrea_gpu_status rrea_gpu_fluid_transport(rrea_gpu_ctx* ctx, double dt_s, const double* efr, const double* efz,
                                         double* flux_r, double* flux_z, double* diag);

/*
 * The coupled fluid + Maxwell step of one outer dt (RreaAmrexAdvance::
 * AdvanceOneStep, S/RreaAmrexAdvance.cpp:593-838): closure fields at the
 * step start (table models), the stiffness probe choosing the shared
 * material substeps, then per substep a half reaction, transport with the
 * limited face flux, the total face current (fluid + the step's kinetic
 * net-chord current), B / Silver-Mueller / E, the closure fields on the new
 * field, and the second half reaction; the B restagger, the final
 * conductivity, and the source rates cleared.  diag (may be NULL) receives
 * 8 doubles: substeps, full conduction, diffusion and reaction numbers of
 * the probe, max reaction number, max dt sigma_face / eps0, max diffusion
 * number, max reaction charge residual.  Guards fail closed
 * (RREA_GPU_ERR_INVALID_STATE) at the end of the step.  Requires a
 * non-periodic z and the Yee CFL, like rrea_gpu_advance_field.
 */
rrea_gpu_status rrea_gpu_advance_field_coupled(rrea_gpu_ctx* ctx, double dt_s, double* diag);
/* The fluid and event-source totals of the reduced diagnostics
 * (O/RreaCouplingDiagnostics.cpp:318-333, 469-471, 730-736) from the fluid
 * state and the cell sources accumulated since rrea_gpu_reset_sources,
 * normalised as NormalizeAndSync leaves them for a step of dt_s.  out16:
 * total_ne_low, total_n_pos, total_n_neg (plain cell sums), N_low_e_real,
 * N_pos_real, N_neg_real, rho_fluid_C (RZ volume integrals),
 * total_rho_fluid, total_S_low_electron, total_S_positive_ion,
 * total_S_direct_negative_ion, ionization_event_count,
 * total_energy_loss_ev_m3 (cell sums), max_ne_low, max_sigma, min_tau_m. */
rrea_gpu_status rrea_gpu_fluid_reductions(rrea_gpu_ctx* ctx, double dt_s, double* out16);
/* The two halves of the coupled step of a sharded run, as
 * rrea_gpu_current_device / rrea_gpu_advance_field_from_current are for the
 * kinetic-only update: the caller sums the kinetic face current
 * (rrea_gpu_current_device) and the five cell-source grids
 * (rrea_gpu_sources_device: 5 x nr*nz device doubles, field-major) across
 * ranks in place, calls rrea_gpu_fluid_take_sources, then
 * rrea_gpu_advance_field_coupled_from_current, which runs the coupled step
 * on the current vectors as they stand; the fluid and the field are
 * replicated, so every rank computes the same update.
 * rrea_gpu_advance_field_coupled is rrea_gpu_current_device followed by
 * rrea_gpu_advance_field_coupled_from_current. */
rrea_gpu_status rrea_gpu_sources_device(rrea_gpu_ctx* ctx, double** cells5);
rrea_gpu_status rrea_gpu_advance_field_coupled_from_current(rrea_gpu_ctx* ctx, double dt_s, double* diag);

/*
 * ---- Batched ensemble --------------------------------------------------
 * Many independent uniform-field avalanche instances advanced by one launch
 * sequence per step (the batched-ensemble pattern; the overlay itself runs
 * one instance per process).  A particle's cpu ordinal is its instance k:
 * its RNG key |id| ^ k << 40 gives every instance its own streams, ids are
 * counted per instance and species, and a committed secondary takes its
 * root's instance.  Each instance therefore evolves exactly as the same
 * particles on their own context with cpu = k.  No feedback: the instances
 * keep their uniform ambient fields and deposit neither current nor cell
 * sources.
 *
 * configure: once, before staging; ambient_ez[k] is instance k's uniform E_z.
 * partition: stable partition of a species tile by instance (the order
 *   inside an instance is kept), so each instance is one slice; counts
 *   (n_instances) receives the slice sizes.  Valid until the tile next
 *   gains or loses slots (commit, compaction, staging).
 * retire: invalidates every particle of an instance (the end of its run).
 * census / population_thin: rrea_gpu_census_resident and
 *   rrea_gpu_population_thin_resident (without staged candidates) on one
 *   instance's slice of the last partition.
 * population_thin_all: the population control of every instance in one
 *   pass, no partition needed: instance k, due when its valid particles
 *   exceed 1.25 targets[k] (host, n_instances; 0 = no control), is thinned
 *   exactly as population_thin(species, k, targets[k], step, salt) would
 *   thin its slice.  removed_per_instance (host, n_instances) receives the
 *   removals; stats the totals in population_thin's layout.  A rejected or
 *   short plan of any instance applies nothing.
 */
rrea_gpu_status rrea_gpu_ensemble_configure(rrea_gpu_ctx* ctx, int32_t n_instances, const double* ambient_ez);
rrea_gpu_status rrea_gpu_ensemble_partition(rrea_gpu_ctx* ctx, int32_t species, int64_t* counts);
rrea_gpu_status rrea_gpu_ensemble_retire(rrea_gpu_ctx* ctx, int32_t instance);
rrea_gpu_status rrea_gpu_ensemble_census(rrea_gpu_ctx* ctx, int32_t species, int32_t instance, const double* edges_eV,
                                         int32_t n_edges, const double* thresholds_eV, int32_t n_thresholds,
                                         double* out);
rrea_gpu_status rrea_gpu_ensemble_population_thin(rrea_gpu_ctx* ctx, int32_t species, int32_t instance,
                                                  int64_t target, int32_t step, uint64_t salt, int64_t* stats);
rrea_gpu_status rrea_gpu_ensemble_population_thin_all(rrea_gpu_ctx* ctx, int32_t species, const int64_t* targets,
                                                      int32_t step, uint64_t salt, int64_t* removed_per_instance,
                                                      int64_t* stats);

/*
 * ---- Pathwise adjoint of the charged push --------------------------------
 * Gradients of a smoothed runaway count and of the net charge crossing a
 * plane (the time integral of J_z through it) with respect to an axial
 * field profile E_z(z) on n_nodes equally spaced nodes over [z_lo, z_hi]
 * (linear between nodes, clamped outside): the differentiation pattern
 * built on the kinetic step (the overlay has no such mode).  The
 * differentiated model is the continuous part of the charged substep (the
 * chord of length v(K) dt/substeps, the two-point Gauss-Legendre field work,
 * the half kicks of O/RreaChargedInterleave.H:100-138 without B, the
 * tables' collision plus soft radiative drag of :218-292) with the discrete
 * outcomes frozen: one rotation per particle and substep drawn from the
 * counter RNG stands in for the elastic deflection, a particle whose drag
 * reaches the cutoff stops at the same substep, and nothing else branches.
 *   loss = sum_i w_i [ sig((K_i(T) - k_threshold) / k_width)
 *          - plane_weight (sig((z_i(T) - z_plane) / z_width) - sig((z_i(0) - z_plane) / z_width)) ]
 * The forward pass checkpoints every `checkpoint_every` steps; the reverse
 * pass recomputes each segment from its checkpoint and runs the
 * hand-written adjoint back through it.
 *
 * stage: the seeds (host arrays: z, direction xyz (3n, normalised here),
 *   kinetic energy, weight, id); needs the tables loaded.
 * forward: the loss for the node values at e_nodes_device (DEVICE pointer,
 *   n_nodes doubles); records where every particle ended (stopped in the
 *   drag, or below the cutoff after a kick).
 * forward_frozen: the same with every particle ending exactly where the
 *   last forward ended it, whatever the new nodes: the frozen-topology loss
 *   that backward differentiates (finite differences compare against it).
 * backward: d loss / d E_k into grad_device (DEVICE pointer) for the nodes
 *   of the last forward (run after it, with the same nodes).
 * final_state: z, dx, dy, dz, K, alive (6 x n host doubles) of the forward.
 */
typedef struct {
    double z_lo, z_hi;          /* node span [m] (default 0..500) */
    int32_t n_nodes;            /* 256 */
    int32_t steps;              /* 2000 */
    int32_t substeps;           /* 4 */
    int32_t checkpoint_every;   /* 32 */
    double dt_s;                /* 5e-10 */
    double density_ratio;       /* stopping-power density ratio, 1 */
    double cutoff_eV;           /* 1e4 */
    double scatter_rms_rad;     /* 0.02 */
    double k_threshold_eV;      /* 1e6 */
    double k_width_eV;          /* 5e4 */
    double z_plane_m;           /* 400 */
    double z_width_m;           /* 1 */
    double plane_weight;        /* 1 */
    uint64_t rng_seed;          /* 1 */
} rrea_gpu_adjoint_config;

void rrea_gpu_default_adjoint_config(rrea_gpu_adjoint_config* cfg);
rrea_gpu_status rrea_gpu_adjoint_stage(rrea_gpu_ctx* ctx, const rrea_gpu_adjoint_config* cfg, int64_t n,
                                       const double* z, const double* dir3, const double* kinetic_eV,
                                       const double* weight, const uint64_t* id);
rrea_gpu_status rrea_gpu_adjoint_forward(rrea_gpu_ctx* ctx, const double* e_nodes_device, double* loss);
rrea_gpu_status rrea_gpu_adjoint_forward_frozen(rrea_gpu_ctx* ctx, const double* e_nodes_device, double* loss);
rrea_gpu_status rrea_gpu_adjoint_backward(rrea_gpu_ctx* ctx, const double* e_nodes_device, double* grad_device);
rrea_gpu_status rrea_gpu_adjoint_final_state(rrea_gpu_ctx* ctx, double* state6);

#ifdef __cplusplus
}
#endif

#endif /* RREA_GPU_H */
