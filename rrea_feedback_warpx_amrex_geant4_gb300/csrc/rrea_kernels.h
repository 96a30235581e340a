// Host-visible launchers of the device kernels (rrea_kernels.cu).
#pragma once

#include "device/rrea_device_common.cuh"

#include <cuda_runtime.h>

#include <string>
#include <vector>

namespace rrea_dev {
struct ElectronArgs;
struct SegmentRec;
struct NetGrid;

// Device columns of one species tile: r, z, theta, ux, uy, uz, w and the
// captured prev_r, prev_z, prev_theta, prev_ux, prev_uy, prev_uz; id; cpu.
constexpr int kTileColumns = 13;
struct TileColumns {
    double* d[kTileColumns];
    int64_t* id;
    int32_t* cpu;
};
}

namespace rrea_launch {

// Every kernel launch of the library is noted here (a process-wide atomic
// counter), so the count rrea_gpu_kernel_launches reports is exact.
void note_launch();
unsigned long long launches_noted();

cudaError_t set_step_constants(rrea_dev::StepConstants const& c, cudaStream_t stream);
cudaError_t field_prep(int nr, int nz, const double* er, const double* ez, const double* amb_er, const double* amb_ez,
                       double* cell_er, double* cell_ez, cudaStream_t stream);
cudaError_t electron_step(rrea_dev::ElectronArgs const& args, int blocks, int threads, int min_blocks, bool periodic,
                          cudaStream_t stream);
// Positron phase (rrea_positron_kernels.cu): its own constant bank, set
// once per phase before its launches; min_blocks picks the register variant
// as for electrons (2, 4, 8 or 16 resident 128-thread blocks per SM).
cudaError_t positron_constants(rrea_dev::StepConstants const& sc, cudaStream_t stream);
cudaError_t positron_step(rrea_dev::ElectronArgs const& args, int blocks, int threads, int min_blocks, bool periodic,
                          cudaStream_t stream);
// Photon phase (rrea_photon_kernels.cu): its own constant bank, set once
// per phase before its launches.
cudaError_t photon_constants(rrea_dev::StepConstants const& sc, cudaStream_t stream);
cudaError_t photon_step(rrea_dev::ElectronArgs const& args, int blocks, int threads, bool periodic, cudaStream_t stream);
// Net-chord current (rrea_deposit.cu): replay the segment records of one
// charged phase into the padded grid; convert the grid to physical J.
cudaError_t netchord_deposit(rrea_dev::SegmentRec const* seg, int64_t n, rrea_dev::NetGrid const& g, double dt,
                             int* status, long long* fail_index, int blocks, cudaStream_t stream);
cudaError_t netchord_convert(rrea_dev::NetGrid const& g, double* jr_phys, double* jz_phys, cudaStream_t stream);
// Cell-centred CIC charge q * w of a tile's valid particles (rrea_deposit.cu).
cudaError_t particle_charge(const double* r, const double* z, const double* w, const int64_t* id, int64_t n, double q,
                            int nr, int nz, double r_lo, double z_lo, double dr, double dz, double* rho, int blocks,
                            cudaStream_t stream);
// Maxwell TM-RZ step with a fixed face current (rrea_field.cu).
cudaError_t maxwell_step(int nr, int nz, double dr, double dz, double dt, int substeps, double* er, double* ez,
                         double* bt, const double* jr, const double* jz, cudaStream_t stream);
// Transient FIFO of the secondaries (rrea_newborn.cu): its own constant
// bank, payload checks (mode 0 birth payloads, 1 final survivors), the
// residual advance of one chunk of FIFO items, survivor compaction, and the
// adoption of the chunk's ordered children into the FIFO tail.
cudaError_t newborn_constants(rrea_dev::StepConstants const& sc, cudaStream_t stream);
cudaError_t validate_fifo(const rrea_gpu_secondary* items, int64_t n, int mode, unsigned long long* invalid,
                          long long* first, cudaStream_t stream);
// The positron and photon kernels run on side[0] and side[1] (joined back
// into `stream`) when the side streams and events are given.
cudaError_t newborn_step(rrea_dev::ElectronArgs const& args, rrea_gpu_secondary* items, int64_t n, uint32_t* alive,
                         int max_blocks, bool periodic, cudaStream_t stream, cudaStream_t const side[2],
                         cudaEvent_t fork, cudaEvent_t const join[2]);
cudaError_t gather_roots(const rrea_gpu_secondary* items, int64_t n, unsigned long long* out, cudaStream_t stream);
cudaError_t compact_survivors(const rrea_gpu_secondary* items, const uint32_t* alive, const int64_t* offsets,
                              int64_t n, rrea_gpu_secondary* out, cudaStream_t stream);
cudaError_t adopt_children(const rrea_gpu_secondary* ordered, int64_t n, const rrea_gpu_secondary* items,
                           const uint64_t* lineage, rrea_gpu_secondary* out, cudaStream_t stream);
cudaError_t eval_math(const double* arena, int which, const double* x, int64_t n, double* fast, double* libm,
                      cudaStream_t stream);
cudaError_t count_live(const int64_t* id, int64_t n, unsigned long long* out, int blocks, cudaStream_t stream);
int64_t scan_scratch_elems(int64_t n);
// Exclusive scan of per-parent counts into offsets (block_scratch holds
// scan_scratch_elems(n) elements); the first half of order_secondaries.
cudaError_t exclusive_scan_counts(const uint32_t* counts, int64_t n, int64_t* offsets, int64_t* block_scratch,
                                  cudaStream_t stream);
cudaError_t order_secondaries(const uint32_t* counts, int64_t n, int64_t* offsets, int64_t* block_scratch,
                              const rrea_gpu_secondary* unordered, int64_t count, rrea_gpu_secondary* ordered,
                              cudaStream_t stream);

// Resident commit of the drain survivors of one species (rrea_commit.cu):
// commit_rank flags the records the species accepts and scans them
// (offsets[n-1] + flags[n-1] accepted); commit_scatter writes them to tile
// rows base + rank with ids first_id + rank.
cudaError_t commit_rank(const rrea_gpu_secondary* surv, int64_t n, int species, uint32_t* flags, int64_t* offsets,
                        int64_t* scan_scratch, cudaStream_t stream);
cudaError_t commit_scatter(const rrea_gpu_secondary* surv, int64_t n, int species, const int64_t* offsets,
                           rrea_dev::TileColumns const& tile, int64_t base, int64_t first_id, const int64_t* ids,
                           cudaStream_t stream);
// Stable compaction of the valid (id > 0) rows of src into dst; offsets[n-1]
// + flags[n-1] is the new row count.
cudaError_t compact_tile(rrea_dev::TileColumns const& src, int64_t n, uint32_t* flags, int64_t* offsets,
                         int64_t* scan_scratch, rrea_dev::TileColumns const& dst, cudaStream_t stream);

// Charge-exact thinning of CIC support groups (rrea_resample.cu): group g is
// rows [offsets[g], offsets[g+1]) of fr, fz, w (w updated in place).
cudaError_t cic_thin(const double* fr, const double* fz, double* w, const int64_t* offsets, int64_t n_groups,
                     const int64_t* max_removals, const uint64_t* keys, int64_t* removed, int64_t* draws,
                     int32_t* valid, int64_t* capacity, cudaStream_t stream);

// Scheduling order of a charged tile (lowest |u| first, ended particles
// last) into order[0, n); scratch holds cost_order_scratch_elems() words.
int cost_order_scratch_elems();
cudaError_t cost_order(const double* ux, const double* uy, const double* uz, const int64_t* id, int64_t n,
                       uint32_t* scratch, uint32_t* order, int blocks, cudaStream_t stream);

// Census of a species tile (rrea_census.cu): over the valid rows, the
// weight sums (w, w^2, w K), under/overflow weight, weight at or above each
// threshold and the weighted spectrum over [edges[0], edges[n_edges-1]) are
// added into out (5 + n_thresholds + n_edges - 1 doubles), the particle count
// into *count and the largest weight's bit pattern into *max_bits (all
// zeroed by the caller).  n_edges <= 1025, n_thresholds <= 16.
cudaError_t census(const double* ux, const double* uy, const double* uz, const double* w, const int64_t* id, int64_t n,
                   bool photon, const double* edges, int n_edges, const double* thresholds, int n_thresholds,
                   double* out, unsigned long long* count, unsigned long long* max_bits, int blocks,
                   cudaStream_t stream);

// Adaptive population control of one charged species (rrea_population.cu):
// the live tile rows and the staged candidates of the transaction.
struct PopulationInput {
    const double *r, *z, *theta, *ux, *uy, *uz;
    double* w;
    int64_t* id;
    const int32_t* cpu;
    int64_t n_tile;
    rrea_gpu_secondary* cand;
    int64_t n_cand;
    int species;
    int periodic_z;
    double r_lo, z_lo, z_hi, dr, dz;
    int64_t target;
    uint64_t rng_seed, salt;
    int64_t step;
    // ensemble (population_thin_instances): a plan per instance, the
    // instance being a live row's cpu ordinal, with targets[k] (host memory)
    // per instance
    const int64_t* targets;
    int32_t n_inst;
};
// members, live and candidate members, supports, removal capacity and the
// geometric floor, the nominal request, particles removed; status is an
// rrea_gpu_status (0: plan applied or nothing due)
struct PopulationStats {
    int64_t members, live, candidates, supports, capacity, floor, requested, removed;
    int status;
};
struct PopulationWork;
void population_work_free(PopulationWork* work);
// Weight-doubling merge of a resident tile above `target` live particles
// (rrea_population.cu): pairs inside (cell, |u| octave, u_z sign) groups,
// R = min(live - target, pairs) of them merged, evenly spread.
struct MergeInput {
    const double *r, *z, *ux, *uy, *uz;
    double* w;
    int64_t* id;
    const int32_t* cpu;
    int64_t n_tile;
    int species;
    int64_t nr, nz;
    double r_lo, z_lo, dr, dz;
    int64_t target;
    uint64_t rng_seed;
    int64_t step;
};
struct MergeStats {
    int64_t live, groups, pairs, requested, merged;
    int status;
};
cudaError_t population_merge(MergeInput const& in, PopulationWork*& work, MergeStats& stats, cudaStream_t stream);
// Global CIC thinning plan and its application (nothing is applied unless
// status is 0).
cudaError_t population_thin(PopulationInput const& in, PopulationWork*& work, PopulationStats& stats, int blocks,
                            cudaStream_t stream);
// The per-instance plans of an ensemble in one pass (in.n_inst > 0); the
// stats are totals and removed_per_instance (host, n_inst) the removals.
cudaError_t population_thin_instances(PopulationInput const& in, PopulationWork*& work, PopulationStats& stats,
                                      int64_t* removed_per_instance, cudaStream_t stream);
// Split refill of the tile's first n rows: weight halved for every valid
// particle at or above twice min_w, clones appended at rows n.. with ids
// from first_id in tile order; *added < 0 when the clones exceed `room`
// (nothing changed).
cudaError_t population_split(rrea_dev::TileColumns const& t, int64_t n, double min_w, PopulationWork*& work,
                             int64_t first_id, int64_t room, int64_t* added, cudaStream_t stream);

// Maxwell leapfrog pieces (I/RreaMaxwellTMRZ.H:143-214) for the coupled step.
cudaError_t maxwell_advance_b(int nr, int nz, double dr, double dz, double dt, const double* er, const double* ez,
                              double* bt, cudaStream_t stream);
cudaError_t maxwell_silver_mueller(int nr, int nz, const double* er, const double* ez, double* bt, cudaStream_t stream);
cudaError_t maxwell_advance_e(int nr, int nz, double dr, double dz, double dt, const double* bt, const double* jr,
                              const double* jz, double* er, double* ez, cudaStream_t stream);

// Low-energy carrier fluid (rrea_fluid.cu).  A failed fail-closed check
// returns cudaSuccess with ok = false and the message in fluid_error().
struct FluidGrid {
    int nr, nz;
    double r_lo, z_lo, dr, dz;
    int periodic_z;
};
struct FluidState;
// The device field of the coupled step: scattered er/ez/bt, ambient faces,
// the cell averages the closure and the gather read, the kinetic current.
struct CoupledField {
    int nr, nz;
    double dr, dz;
    double *er, *ez, *bt;
    const double *amb_er, *amb_ez;
    double *cell_er, *cell_ez;
    const double *jr_kin, *jz_kin;
};
cudaError_t fluid_create(FluidGrid const& g, int blocks, FluidState*& out);
void fluid_free(FluidState* s);
void fluid_set_config(FluidState& s, rrea_gpu_fluid_config const& c);
rrea_gpu_fluid_config const& fluid_config(FluidState const& s);
std::string const& fluid_error(FluidState const& s);
bool fluid_validate(FluidState& s, bool require_cfl);
cudaError_t fluid_load_closure(FluidState& s, std::vector<double> const& columns, int nodes);
bool fluid_has_closure(FluidState const& s);
// 0 ne, 1 np, 2 nn, 3 rho, 4 sigma, 5 tau, 6 se, 7 sp, 8 sn, 9 chi, 10 mu, 11 nu, 12 diffusion (3n),
// 13/14 the face-current buffers (radial/axial)
double* fluid_field(FluidState& s, int field);
void fluid_bind_chi(FluidState& s, bool bound);
int64_t fluid_cells(FluidState const& s);
const double* fluid_flux(FluidState const& s, int dir);
// The reduced diagnostics' fluid and source totals (16 doubles; layout at
// rrea_gpu_fluid_reductions); cells5 may be null.
cudaError_t fluid_reductions(FluidState& s, const double* cells5, double dt, double out16[16], cudaStream_t stream);
cudaError_t fluid_take_sources(FluidState& s, const double* cells5, double dt, cudaStream_t stream);
cudaError_t fluid_react(FluidState& s, double dt, bool clear, double& residual, bool& ok, cudaStream_t stream);
cudaError_t fluid_max_reaction_frequency(FluidState& s, double& out, cudaStream_t stream);
cudaError_t fluid_conductivity(FluidState& s, cudaStream_t stream);
cudaError_t fluid_charge_density(FluidState& s, cudaStream_t stream);
cudaError_t fluid_closure(FluidState& s, const double* er_cell, const double* ez_cell, double diag8[8], bool& ok,
                          cudaStream_t stream);
cudaError_t fluid_transport(FluidState& s, double dt, const double* efr, const double* efr_add, const double* efz,
                            const double* efz_add, double diag14[14], bool& ok, cudaStream_t stream);
cudaError_t fluid_coupled_step(FluidState& s, CoupledField const& f, double dt, double diag8[8], bool& ok,
                               cudaStream_t stream);

// Batched ensemble (rrea_ensemble.cu): per-instance survivor ids, the stable
// partition of a tile by instance, the retirement of an instance.
struct EnsembleWork;
void ensemble_work_free(EnsembleWork* w);
cudaError_t ensemble_survivor_ids(const rrea_gpu_secondary* surv, int64_t n, int species, uint32_t n_inst,
                                  int64_t* next_id, EnsembleWork*& w, const int64_t** ids, cudaStream_t stream);
cudaError_t ensemble_partition(rrea_dev::TileColumns const& src, int64_t n, uint32_t n_inst,
                               rrea_dev::TileColumns const& dst, EnsembleWork*& w, int64_t* counts_host,
                               cudaStream_t stream);
cudaError_t ensemble_retire(int64_t* id, const int32_t* cpu, int64_t n, int32_t inst, cudaStream_t stream);

// Pathwise adjoint of the charged push (rrea_adjoint.cu).
struct AdjointSetup {
    int64_t n;
    int n_nodes;
    double z0, dz_node;
    int steps, substeps, ckpt_every;
    double dt, rho, cutoff, scatter_rms;
    double k_th, tau_k, z_p, tau_z, lambda;
    uint64_t seed;
    RreaTable1DIndex col, soft;
};
struct AdjointState;
void adjoint_free(AdjointState* s);
int adjoint_max_nodes();
// seeds6: z, dx, dy, dz, K, alive (6 x n, host); w (n); id (n)
cudaError_t adjoint_stage(AdjointSetup const& in, const double* seeds6, const double* w, const uint64_t* id,
                          int blocks, AdjointState*& out);
// replay = false records every particle's end; replay = true ends every
// particle where the last recording forward ended it (frozen topology)
cudaError_t adjoint_forward(AdjointState& s, const double* arena, const double* e_nodes, bool replay, double& loss,
                            cudaStream_t stream);
bool adjoint_recorded(AdjointState const& s);
cudaError_t adjoint_backward(AdjointState& s, const double* arena, const double* e_nodes, double* grad,
                             cudaStream_t stream);
cudaError_t adjoint_final_state(AdjointState const& s, double* host6);

}  // namespace rrea_launch
