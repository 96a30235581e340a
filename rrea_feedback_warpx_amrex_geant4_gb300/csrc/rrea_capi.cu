// C-ABI of the GB300 kinetic step (include/rrea_gpu.h).  Host C++ around the
// kernels in rrea_kernels.cu, rrea_photon_kernels.cu and rrea_newborn.cu:
// owns the device arena, field vectors, one resident tile per species and
// every per-step buffer.  The buffers of a species phase are allocated at
// create/load time, so a phase allocates nothing; only the secondary FIFO
// of the drain grows on demand.
#include "../../include/rrea_gpu.h"

#include "device/rrea_electron_args.cuh"
#include "device/rrea_resample.cuh"
#include "host/closure_table.hpp"
#include "host/seed_schedule.hpp"
#include "host/table_set.hpp"
#include "rrea_kernels.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace {

constexpr int kTileDoubles = 13;
// resident charged tiles at least this large are scheduled by momentum
constexpr int64_t kScheduleMinParticles = 1 << 16;
constexpr int kSpecies = 3;
// Chunks of a drop-in phase call whose upload overlaps the compute of the
// chunks before it, and the tile size from which that pays.
constexpr int kPhaseChunks = 4;
#ifndef RREA_PIPELINE_MIN_PARTICLES
#define RREA_PIPELINE_MIN_PARTICLES (1LL << 18)
#endif
constexpr int64_t kPipelineMinParticles = RREA_PIPELINE_MIN_PARTICLES;

// Device SoA of one species: r, z, theta, ux, uy, uz, w, prev_r, prev_z,
// prev_theta, prev_ux, prev_uy, prev_uz, then id and cpu.
struct SpeciesTile {
    double* d[kTileDoubles] = {};
    int64_t* id = nullptr;
    int32_t* cpu = nullptr;
    int64_t n = 0;
};

thread_local std::string g_seed_error;

rrea_gpu_status seed_fail(int code, std::string const& msg)
{
    g_seed_error = msg;
    return static_cast<rrea_gpu_status>(code);
}

// Dense slots for the transient roots (the RNG key and species of the live
// particle whose streams a FIFO item draws from): an open-addressing table
// filled once per drain from the initial items; children inherit their
// item's slot, so no lookup happens after the start.
// The table lives in the context across drains; an epoch stamp marks the
// entries of the current drain, so starting a drain clears nothing.
class RootSlots {
public:
    void reset(size_t expected)
    {
        size_t cap = 16;
        while (cap < 2 * expected) cap <<= 1;
        if (cap > entries_.size()) {
            entries_.assign(cap, Entry{});
            epoch_ = 0;
        }
        mask_ = entries_.size() - 1;
        ++epoch_;
    }
    // slot of (key, species); `fresh` is the slot a new root receives
    uint32_t find_or_insert(uint64_t key, int32_t species, uint32_t fresh, bool& inserted)
    {
        uint64_t h = key ^ (static_cast<uint64_t>(static_cast<uint32_t>(species)) << 61);
        h ^= h >> 33;
        h *= 0xff51afd7ed558ccdULL;
        h ^= h >> 33;
        for (size_t i = static_cast<size_t>(h) & mask_;; i = (i + 1) & mask_) {
            Entry& e = entries_[i];
            if (e.stamp != epoch_) {
                e = Entry{key, epoch_, species, fresh};
                inserted = true;
                return fresh;
            }
            if (e.key == key && e.species == species) {
                inserted = false;
                return e.slot;
            }
        }
    }

private:
    // one 24-byte entry per bucket: a probe touches one cache line
    struct Entry {
        uint64_t key = 0;
        uint64_t stamp = 0;  // epoch of the drain that filled it; older = empty
        int32_t species = 0;
        uint32_t slot = 0;
    };
    std::vector<Entry> entries_;
    uint64_t epoch_ = 0;
    size_t mask_ = 0;
};

}  // namespace

struct rrea_gpu_seed_schedule {
    rrea_host::SeedSchedule s;
};

struct rrea_gpu_ctx {
    rrea_gpu_config cfg{};
    int64_t capacity = 0;
    int device = 0;
    cudaStream_t stream = nullptr;
    // side streams and events that let the drain's species kernels overlap
    cudaStream_t side[2] = {nullptr, nullptr};
    cudaEvent_t fork_ev = nullptr;
    cudaEvent_t roots_ev = nullptr;  // the initial FIFO items' roots have reached the host
    // rrea_gpu_apply_step: host tiles of later phases uploaded on side[0]
    // behind a chunked electron tile's uploads, while its kernels run
    rrea_gpu_tile const* prefetch[kSpecies] = {nullptr, nullptr, nullptr};
    bool prefetched[kSpecies] = {false, false, false};
    cudaEvent_t prefetch_ev = nullptr;
    cudaEvent_t join_ev[2] = {nullptr, nullptr};
    int num_sms = 0;

    rrea_host::TableSet tables;
    bool tables_loaded = false;
    double* d_arena = nullptr;

    double* d_er = nullptr;
    double* d_ez = nullptr;
    double* d_bt = nullptr;
    double* d_amb_er = nullptr;
    double* d_amb_ez = nullptr;
    double* d_cell_er = nullptr;
    double* d_cell_ez = nullptr;
    bool field_set = false;
    bool has_b = false;

    // altitude density profile: n altitudes then n densities on the device
    double* d_profile = nullptr;
    int profile_n = 0;
    double profile_alt0 = 0.0, profile_ref = 0.0;
    double profile_step_ratio = 1.0;  // the ratio at the domain's axial centre

    // plane-crossing diagnostic: plane z, then kPlaneValues accumulators per plane
    double* d_planes = nullptr;
    int32_t n_planes = 0;

    // one resident SoA tile per species (RREA_SPECIES_ELECTRON/POSITRON/PHOTON)
    SpeciesTile tiles[kSpecies];

    rrea_gpu_secondary* d_sec_unordered = nullptr;
    rrea_gpu_secondary* d_sec_ordered = nullptr;
    int64_t sec_capacity = 0;
    unsigned long long* d_sec_count = nullptr;
    uint32_t* d_sec_per_parent = nullptr;
    int64_t* d_offsets = nullptr;
    int64_t* d_scan_scratch = nullptr;
    double* d_cells = nullptr;
    // net-chord current (non-periodic z only): one record per tile slot and
    // the padded index-space grid plus the physical face currents
    rrea_dev::SegmentRec* d_seg = nullptr;
    rrea_dev::NetGrid net{};
    bool netchord = false;
    double* d_jr_phys = nullptr;
    double* d_jz_phys = nullptr;
    uint64_t* d_diag_sub = nullptr;
    uint64_t* d_diag_ev = nullptr;
    int32_t* d_diag_disp = nullptr;
    int* d_status = nullptr;
    long long* d_fail_index = nullptr;
    unsigned long long* d_transported = nullptr;
    unsigned long long* d_work = nullptr;  // dynamic scheduling counters of the phase kernels, one per chunk
    // a drop-in phase call uploads its host tile in chunks on side[0] while
    // the kernels of earlier chunks run on `stream` and side[1]
    cudaEvent_t chunk_up[kPhaseChunks] = {};
    cudaEvent_t chunk_done[kPhaseChunks] = {};
    // transient FIFO of DrainAndCommitSecondaries: the resident phases queue
    // their ordered secondaries in d_fifo[0, fifo_pending); a drain advances
    // the FIFO chunk by chunk and leaves the survivors in d_surv[0, n_surv)
    rrea_gpu_secondary* d_fifo = nullptr;
    int64_t fifo_cap = 0;
    int64_t fifo_pending = 0;
    rrea_gpu_secondary* d_surv = nullptr;
    int64_t surv_cap = 0;
    int64_t n_surv = 0;
    // resident commit: the next id per species and the rank scratch of the
    // survivor list; the spare tile the compaction writes into
    int64_t next_id[kSpecies] = {1, 1, 1};
    uint32_t* d_commit_flags = nullptr;
    int64_t* d_commit_offsets = nullptr;
    int64_t* d_commit_scan = nullptr;
    int64_t commit_cap = 0;
    SpeciesTile spare;
    bool spare_ready = false;
    uint32_t* d_alive = nullptr;
    uint32_t* d_cost_scratch = nullptr;  // histogram and cursors of the scheduling order, one per chunk
    double* d_census = nullptr;          // census sums, edges and thresholds (first census call)
    double* d_rho_cells = nullptr;       // particle charge grid nr*nz (first deposit call)
    rrea_launch::PopulationWork* pop_work = nullptr;  // population-control plan scratch (first use)
    rrea_gpu_secondary* d_pc_cand = nullptr;          // host candidates of a population-control call
    rrea_launch::FluidState* fluid = nullptr;         // low-energy carrier fluid (rrea_gpu_fluid_configure)
    // batched ensemble (rrea_gpu_ensemble_configure): per-instance uniform
    // fields, per-instance next ids, and the slices of the last partition
    int32_t n_instances = 0;
    double* d_inst_cells = nullptr;                   // cell Er (n x nr*nz) then cell Ez (n x nr*nz)
    int64_t* d_inst_next_id = nullptr;                // n x 3
    rrea_launch::EnsembleWork* ens_work = nullptr;
    rrea_launch::AdjointState* adjoint = nullptr;      // rrea_gpu_adjoint_stage
    std::vector<int64_t> inst_offsets[kSpecies];      // n + 1 slice bounds per species
    bool part_valid[kSpecies] = {false, false, false};
    int64_t pc_cand_cap = 0;
    uint64_t* d_child_lineage = nullptr;
    unsigned long long* d_invalid = nullptr;
    // roots of the initial FIFO items (16 B each) on the device and in pinned
    // host memory, grown with the FIFO
    unsigned long long* d_roots = nullptr;
    unsigned long long* h_roots = nullptr;
    int64_t roots_cap = 0;
    RootSlots root_slots;
    int64_t last_drain_items = 0;
    cudaEvent_t ev_start = nullptr;
    cudaEvent_t ev_stop = nullptr;
    float last_kernel_ms = 0.0f;
    int64_t last_transported = 0;
    int64_t last_secondaries = 0;
    int launch_threads = 128;
    int launch_blocks_per_sm = 16;
    int launch_min_blocks = 16;
    bool diagnostics = true;
    bool schedule_order = true;   // visit large charged tiles lowest |u| first (rrea_gpu_set_schedule)

    std::string last_error;
};

namespace {

rrea_gpu_status fail(rrea_gpu_ctx* ctx, rrea_gpu_status code, std::string const& msg)
{
    if (ctx) ctx->last_error = msg;
    return code;
}

rrea_gpu_status cuda_fail(rrea_gpu_ctx* ctx, cudaError_t e, char const* where)
{
    return fail(ctx, RREA_GPU_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define RREA_CUDA(ctx, call)                                  \
    do {                                                      \
        cudaError_t const _e = (call);                        \
        if (_e != cudaSuccess) return cuda_fail(ctx, _e, #call); \
    } while (0)

template <class T>
cudaError_t dalloc(T** p, size_t count)
{
    return cudaMalloc(reinterpret_cast<void**>(p), count * sizeof(T) > 0 ? count * sizeof(T) : sizeof(T));
}

void dfree(void* p)
{
    if (p) cudaFree(p);
}

bool config_valid(rrea_gpu_config const& c, std::string& why)
{
    if (!(std::isfinite(c.r_lo) && std::isfinite(c.r_hi) && std::isfinite(c.z_lo) && std::isfinite(c.z_hi))
        || !(c.r_lo >= 0.0) || !(c.r_hi > c.r_lo) || !(c.z_hi > c.z_lo)) {
        why = "invalid RZ domain";
        return false;
    }
    if (c.r_lo != 0.0) {
        why = "the RZ domain must start on the axis (r_lo = 0)";
        return false;
    }
    if (c.nr < 1 || c.nz < 1) {
        why = "field grid must have at least one cell per direction";
        return false;
    }
    if (!(c.max_optical_depth_per_substep > 0.0) || !std::isfinite(c.max_optical_depth_per_substep)
        || c.max_subcycles == 0 || c.max_subcycles >= (uint64_t{1} << 14)) {
        why = "invalid subcycle controls (max_subcycles must be in [1, 16383])";
        return false;
    }
    if (!(c.low_energy_cutoff_eV > 0.0) || !std::isfinite(c.low_energy_cutoff_eV)) {
        why = "low_energy_cutoff_eV must be finite and positive";
        return false;
    }
    if (!(c.max_gs_collisions_per_substep > 0.0) || !(c.gs_total_collision_cap > 0.0)
        || !(c.max_field_impulse_fraction > 0.0) || !(c.field_impulse_floor_eV >= 0.0)) {
        why = "invalid substep driver controls";
        return false;
    }
    return true;
}

}  // namespace

extern "C" {

void rrea_gpu_default_config(rrea_gpu_config* cfg)
{
    if (!cfg) return;
    std::memset(cfg, 0, sizeof(*cfg));
    cfg->r_lo = 0.0;
    cfg->r_hi = 50.0;
    cfg->z_lo = 0.0;
    cfg->z_hi = 500.0;
    cfg->nr = 32;
    cfg->nz = 256;
    cfg->periodic_z = 0;
    cfg->strict_transport_guards = 1;
    cfg->density_ratio = 1.0;
    cfg->low_energy_cutoff_eV = 1.0e3;
    cfg->photon_cutoff_eV = 5.0e4;
    cfg->max_optical_depth_per_substep = 0.05;
    cfg->max_subcycles = 256;
    cfg->max_gs_collisions_per_substep = 32.0;
    cfg->gs_total_collision_cap = 1024.0;
    cfg->max_field_impulse_fraction = 0.1;
    cfg->field_impulse_floor_eV = 1.0e4;
    cfg->rng_seed = 0;
    cfg->debug_disable_hard_moller = 0;
}

rrea_gpu_status rrea_gpu_create(const rrea_gpu_config* cfg, int64_t capacity, rrea_gpu_ctx** out)
{
    if (!cfg || !out || capacity < 1) return RREA_GPU_ERR_ARGUMENT;
    *out = nullptr;
    std::string why;
    if (!config_valid(*cfg, why)) return RREA_GPU_ERR_ARGUMENT;
    rrea_gpu_ctx* ctx = new (std::nothrow) rrea_gpu_ctx();
    if (!ctx) return RREA_GPU_ERR_CAPACITY;
    ctx->cfg = *cfg;
    ctx->capacity = capacity;
    auto bail = [&](rrea_gpu_status s) {
        rrea_gpu_destroy(ctx);
        return s;
    };
    if (cudaGetDevice(&ctx->device) != cudaSuccess) return bail(RREA_GPU_ERR_CUDA);
    if (cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, ctx->device) != cudaSuccess) {
        return bail(RREA_GPU_ERR_CUDA);
    }
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) return bail(RREA_GPU_ERR_CUDA);
    for (int k = 0; k < 2; ++k) {
        if (cudaStreamCreateWithFlags(&ctx->side[k], cudaStreamNonBlocking) != cudaSuccess
            || cudaEventCreateWithFlags(&ctx->join_ev[k], cudaEventDisableTiming) != cudaSuccess) {
            return bail(RREA_GPU_ERR_CUDA);
        }
    }
    if (cudaEventCreateWithFlags(&ctx->fork_ev, cudaEventDisableTiming) != cudaSuccess) return bail(RREA_GPU_ERR_CUDA);
    if (cudaEventCreateWithFlags(&ctx->roots_ev, cudaEventDisableTiming) != cudaSuccess) return bail(RREA_GPU_ERR_CUDA);
    if (cudaEventCreateWithFlags(&ctx->prefetch_ev, cudaEventDisableTiming) != cudaSuccess) {
        return bail(RREA_GPU_ERR_CUDA);
    }
    for (int k = 0; k < kPhaseChunks; ++k) {
        if (cudaEventCreateWithFlags(&ctx->chunk_up[k], cudaEventDisableTiming) != cudaSuccess
            || cudaEventCreateWithFlags(&ctx->chunk_done[k], cudaEventDisableTiming) != cudaSuccess) {
            return bail(RREA_GPU_ERR_CUDA);
        }
    }
    size_t const n = static_cast<size_t>(capacity);
    size_t const ner = static_cast<size_t>(cfg->nr + 1) * cfg->nz;
    size_t const nez = static_cast<size_t>(cfg->nr) * (cfg->nz + 1);
    size_t const nbt = static_cast<size_t>(cfg->nr + 1) * (cfg->nz + 1);
    size_t const ncell = static_cast<size_t>(cfg->nr) * cfg->nz;
    bool ok = dalloc(&ctx->d_er, ner) == cudaSuccess && dalloc(&ctx->d_ez, nez) == cudaSuccess
        && dalloc(&ctx->d_bt, nbt) == cudaSuccess && dalloc(&ctx->d_amb_er, ner) == cudaSuccess
        && dalloc(&ctx->d_amb_ez, nez) == cudaSuccess && dalloc(&ctx->d_cell_er, ncell) == cudaSuccess
        && dalloc(&ctx->d_cell_ez, ncell) == cudaSuccess && dalloc(&ctx->d_cells, 5 * ncell) == cudaSuccess;
    for (int sp = 0; ok && sp < kSpecies; ++sp) {
        SpeciesTile& st = ctx->tiles[sp];
        for (int f = 0; ok && f < kTileDoubles; ++f) ok = dalloc(&st.d[f], n) == cudaSuccess;
        ok = ok && dalloc(&st.id, n) == cudaSuccess && dalloc(&st.cpu, n) == cudaSuccess;
    }
    ctx->netchord = cfg->periodic_z == 0;
    {
        // O/RreaWarpXCoupling.cpp:417-444: two pad cells beyond r_hi, below z_lo and above z_hi
        int constexpr pad = 2;
        rrea_dev::NetGrid& g = ctx->net;
        g.phys_nr = cfg->nr;
        g.phys_nz = cfg->nz;
        g.phys_z_begin = pad;
        g.nr = cfg->nr + pad;
        g.nz = cfg->nz + 2 * pad;
        g.dr = (cfg->r_hi - cfg->r_lo) / cfg->nr;
        g.dz = (cfg->z_hi - cfg->z_lo) / cfg->nz;
        g.r_lo = cfg->r_lo;
        g.z_lo = cfg->z_lo - pad * g.dz;
        if (ctx->netchord) {
            ok = ok && dalloc(&ctx->d_seg, n) == cudaSuccess
                && dalloc(&g.rho, static_cast<size_t>(g.nr) * g.nz) == cudaSuccess
                && dalloc(&g.jr, static_cast<size_t>(g.nr + 1) * g.nz) == cudaSuccess
                && dalloc(&g.jz, static_cast<size_t>(g.nr) * (g.nz + 1)) == cudaSuccess
                && dalloc(&ctx->d_jr_phys, static_cast<size_t>(cfg->nr + 1) * cfg->nz) == cudaSuccess
                && dalloc(&ctx->d_jz_phys, static_cast<size_t>(cfg->nr) * (cfg->nz + 1)) == cudaSuccess;
        }
    }
    ctx->sec_capacity = 2 * capacity + 4096;
    size_t const nsec = static_cast<size_t>(ctx->sec_capacity);
    ok = ok && dalloc(&ctx->d_sec_unordered, nsec) == cudaSuccess && dalloc(&ctx->d_sec_ordered, nsec) == cudaSuccess
        && dalloc(&ctx->d_sec_count, 1) == cudaSuccess && dalloc(&ctx->d_sec_per_parent, n) == cudaSuccess
        && dalloc(&ctx->d_offsets, n) == cudaSuccess
        && dalloc(&ctx->d_scan_scratch, static_cast<size_t>(rrea_launch::scan_scratch_elems(capacity))) == cudaSuccess
        && dalloc(&ctx->d_diag_sub, n) == cudaSuccess && dalloc(&ctx->d_diag_ev, n) == cudaSuccess
        && dalloc(&ctx->d_diag_disp, n) == cudaSuccess && dalloc(&ctx->d_status, 1) == cudaSuccess
        && dalloc(&ctx->d_fail_index, 1) == cudaSuccess && dalloc(&ctx->d_transported, 1) == cudaSuccess
        && dalloc(&ctx->d_alive, n) == cudaSuccess && dalloc(&ctx->d_child_lineage, nsec) == cudaSuccess
        && dalloc(&ctx->d_cost_scratch,
                  static_cast<size_t>(kPhaseChunks) * rrea_launch::cost_order_scratch_elems()) == cudaSuccess
        && dalloc(&ctx->d_invalid, 1) == cudaSuccess && dalloc(&ctx->d_work, kPhaseChunks) == cudaSuccess
        && cudaEventCreate(&ctx->ev_start) == cudaSuccess && cudaEventCreate(&ctx->ev_stop) == cudaSuccess;
    if (!ok) return bail(RREA_GPU_ERR_CUDA);
    if (cudaMemsetAsync(ctx->d_cells, 0, 5 * ncell * sizeof(double), ctx->stream) != cudaSuccess) {
        return bail(RREA_GPU_ERR_CUDA);
    }
    if (ctx->netchord && rrea_gpu_reset_current(ctx) != RREA_GPU_OK) return bail(RREA_GPU_ERR_CUDA);
    *out = ctx;
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_destroy(rrea_gpu_ctx* ctx)
{
    if (!ctx) return RREA_GPU_OK;
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    dfree(ctx->d_arena);
    rrea_launch::fluid_free(ctx->fluid);
    dfree(ctx->d_inst_cells);
    dfree(ctx->d_inst_next_id);
    rrea_launch::ensemble_work_free(ctx->ens_work);
    rrea_launch::adjoint_free(ctx->adjoint);
    dfree(ctx->d_er);
    dfree(ctx->d_ez);
    dfree(ctx->d_bt);
    dfree(ctx->d_amb_er);
    dfree(ctx->d_amb_ez);
    dfree(ctx->d_cell_er);
    dfree(ctx->d_cell_ez);
    for (auto& st : ctx->tiles) {
        for (auto* p : st.d) dfree(p);
        dfree(st.id);
        dfree(st.cpu);
    }
    dfree(ctx->d_profile);
    dfree(ctx->d_planes);
    dfree(ctx->d_sec_unordered);
    dfree(ctx->d_sec_ordered);
    dfree(ctx->d_sec_count);
    dfree(ctx->d_sec_per_parent);
    dfree(ctx->d_offsets);
    dfree(ctx->d_scan_scratch);
    dfree(ctx->d_cells);
    dfree(ctx->d_seg);
    dfree(ctx->net.rho);
    dfree(ctx->net.jr);
    dfree(ctx->net.jz);
    dfree(ctx->d_jr_phys);
    dfree(ctx->d_jz_phys);
    dfree(ctx->d_diag_sub);
    dfree(ctx->d_diag_ev);
    dfree(ctx->d_diag_disp);
    dfree(ctx->d_status);
    dfree(ctx->d_fail_index);
    dfree(ctx->d_transported);
    dfree(ctx->d_fifo);
    dfree(ctx->d_surv);
    dfree(ctx->d_commit_flags);
    dfree(ctx->d_commit_offsets);
    dfree(ctx->d_commit_scan);
    if (ctx->spare_ready) {
        for (int f = 0; f < kTileDoubles; ++f) dfree(ctx->spare.d[f]);
        dfree(ctx->spare.id);
        dfree(ctx->spare.cpu);
    }
    dfree(ctx->d_alive);
    dfree(ctx->d_cost_scratch);
    dfree(ctx->d_census);
    dfree(ctx->d_rho_cells);
    rrea_launch::population_work_free(ctx->pop_work);
    dfree(ctx->d_pc_cand);
    dfree(ctx->d_child_lineage);
    dfree(ctx->d_invalid);
    dfree(ctx->d_roots);
    if (ctx->h_roots) cudaFreeHost(ctx->h_roots);
    dfree(ctx->d_work);
    if (ctx->ev_start) cudaEventDestroy(ctx->ev_start);
    if (ctx->ev_stop) cudaEventDestroy(ctx->ev_stop);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    for (int k = 0; k < 2; ++k) {
        if (ctx->side[k]) {
            cudaStreamSynchronize(ctx->side[k]);
            cudaStreamDestroy(ctx->side[k]);
        }
        if (ctx->join_ev[k]) cudaEventDestroy(ctx->join_ev[k]);
    }
    if (ctx->fork_ev) cudaEventDestroy(ctx->fork_ev);
    if (ctx->roots_ev) cudaEventDestroy(ctx->roots_ev);
    if (ctx->prefetch_ev) cudaEventDestroy(ctx->prefetch_ev);
    for (int k = 0; k < kPhaseChunks; ++k) {
        if (ctx->chunk_up[k]) cudaEventDestroy(ctx->chunk_up[k]);
        if (ctx->chunk_done[k]) cudaEventDestroy(ctx->chunk_done[k]);
    }
    delete ctx;
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_load_tables(rrea_gpu_ctx* ctx, const char* path)
{
    if (!ctx || !path) return RREA_GPU_ERR_ARGUMENT;
    try {
        ctx->tables.Load(path);
    } catch (std::exception const& e) {
        ctx->tables_loaded = false;
        return fail(ctx, RREA_GPU_ERR_TABLES, e.what());
    }
    // The photon cutoff is the bundle's brems cutoff; a differing configured
    // value is refused (RreaCouplingConfig.cpp:1334-1342).
    double const brems_cut = ctx->tables.index().brems_absolute_cutoff_eV;
    if (std::isfinite(ctx->cfg.photon_cutoff_eV) && ctx->cfg.photon_cutoff_eV != brems_cut) {
        return fail(ctx, RREA_GPU_ERR_ARGUMENT, "photon_cutoff_eV does not match the tables' brems_absolute_cutoff_eV");
    }
    ctx->cfg.photon_cutoff_eV = brems_cut;
    double const hm = ctx->tables.index().hard_moller_threshold_eV;
    if (!(hm > ctx->cfg.low_energy_cutoff_eV)) {
        return fail(ctx, RREA_GPU_ERR_ARGUMENT, "hard-Moller threshold must exceed the tracking cutoff");
    }
    if (ctx->cfg.low_energy_cutoff_eV < ctx->tables.index().charged_min_eV) {
        return fail(ctx, RREA_GPU_ERR_ARGUMENT, "tracking cutoff below the certified charged range");
    }
    // The charged kernels bracket each energy once per species and evaluate
    // every coefficient table at that bracket.
    if (!ctx->tables.index().electron_grid_shared || !ctx->tables.index().positron_grid_shared) {
        return fail(ctx, RREA_GPU_ERR_TABLES,
                    "the electron (positron) coefficient tables must share one energy grid");
    }
    auto const& arena = ctx->tables.arena();
    dfree(ctx->d_arena);
    ctx->d_arena = nullptr;
    RREA_CUDA(ctx, dalloc(&ctx->d_arena, arena.size()));
    RREA_CUDA(ctx, cudaMemcpyAsync(ctx->d_arena, arena.data(), arena.size() * sizeof(double), cudaMemcpyHostToDevice,
                                   ctx->stream));
    RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->tables_loaded = true;
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_set_field(rrea_gpu_ctx* ctx, const double* er, const double* ez, const double* bt,
                                   const double* amb_er, const double* amb_ez)
{
    if (!ctx || !er || !ez || !bt || !amb_er || !amb_ez) return RREA_GPU_ERR_ARGUMENT;
    rrea_gpu_config const& c = ctx->cfg;
    size_t const ner = static_cast<size_t>(c.nr + 1) * c.nz;
    size_t const nez = static_cast<size_t>(c.nr) * (c.nz + 1);
    size_t const nbt = static_cast<size_t>(c.nr + 1) * (c.nz + 1);
    bool any_b = false;
    for (size_t i = 0; i < nbt; ++i) {
        if (bt[i] != 0.0) {
            any_b = true;
            break;
        }
    }
    RREA_CUDA(ctx, cudaMemcpyAsync(ctx->d_er, er, ner * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    RREA_CUDA(ctx, cudaMemcpyAsync(ctx->d_ez, ez, nez * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    RREA_CUDA(ctx, cudaMemcpyAsync(ctx->d_bt, bt, nbt * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    RREA_CUDA(ctx, cudaMemcpyAsync(ctx->d_amb_er, amb_er, ner * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    RREA_CUDA(ctx, cudaMemcpyAsync(ctx->d_amb_ez, amb_ez, nez * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    RREA_CUDA(ctx, rrea_launch::field_prep(c.nr, c.nz, ctx->d_er, ctx->d_ez, ctx->d_amb_er, ctx->d_amb_ez,
                                           ctx->d_cell_er, ctx->d_cell_ez, ctx->stream));
    RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->has_b = any_b;
    ctx->field_set = true;
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_set_density_profile(rrea_gpu_ctx* ctx, const double* altitude_m, const double* density_kg_m3,
                                             int64_t n, double altitude_msl_at_z0_m, double reference_density_kg_m3)
{
    if (!ctx) return RREA_GPU_ERR_ARGUMENT;
    if (n == 0) {
        ctx->profile_n = 0;
        return RREA_GPU_OK;
    }
    // RreaAltitudeProfile::LoadCsv (S/RreaAltitudeProfile.cpp:97-117) and the
    // reference density the ratio is taken against (O/RreaWarpXCoupling.cpp:88-93)
    if (!altitude_m || !density_kg_m3 || n < 2 || n > (int64_t{1} << 24)) {
        return fail(ctx, RREA_GPU_ERR_ARGUMENT, "altitude profile needs at least two rows");
    }
    for (int64_t i = 0; i < n; ++i) {
        if (!std::isfinite(altitude_m[i]) || !std::isfinite(density_kg_m3[i])) {
            return fail(ctx, RREA_GPU_ERR_ARGUMENT, "altitude profile values must be finite");
        }
        if (i > 0 && !(altitude_m[i] > altitude_m[i - 1])) {
            return fail(ctx, RREA_GPU_ERR_ARGUMENT, "altitude profile altitudes must be strictly increasing");
        }
        if (!(density_kg_m3[i] > 0.0)) {
            return fail(ctx, RREA_GPU_ERR_ARGUMENT, "altitude profile requires strictly positive densities");
        }
    }
    if (!(reference_density_kg_m3 > 0.0) || !std::isfinite(reference_density_kg_m3) ||
        !std::isfinite(altitude_msl_at_z0_m)) {
        return fail(ctx, RREA_GPU_ERR_ARGUMENT, "altitude profile needs a positive reference density and a finite datum");
    }
    // every step asks for the ratio at the domain's axial centre
    // (O/RreaParticleInteraction.cpp:27-35): it must lie inside the profile
    double const a = altitude_msl_at_z0_m + 0.5 * (ctx->cfg.z_lo + ctx->cfg.z_hi);
    if (!(a >= altitude_m[0] && a <= altitude_m[n - 1])) {
        return fail(ctx, RREA_GPU_ERR_RANGE, "the domain's axial centre lies outside the altitude profile");
    }
    int64_t const up = std::upper_bound(altitude_m, altitude_m + n, a) - altitude_m;
    double v;
    if (up == 0) {
        v = density_kg_m3[0];
    } else if (up == n) {
        v = density_kg_m3[n - 1];
    } else {
        double const span = altitude_m[up] - altitude_m[up - 1];
        double const t = span > 0.0 ? (a - altitude_m[up - 1]) / span : 0.0;
        v = (1.0 - t) * density_kg_m3[up - 1] + t * density_kg_m3[up];
    }
    double* d = nullptr;
    if (cudaMalloc(&d, static_cast<size_t>(2 * n) * sizeof(double)) != cudaSuccess) {
        cudaGetLastError();
        return fail(ctx, RREA_GPU_ERR_CUDA, "altitude profile allocation failed");
    }
    RREA_CUDA(ctx, cudaMemcpyAsync(d, altitude_m, static_cast<size_t>(n) * sizeof(double), cudaMemcpyHostToDevice,
                                   ctx->stream));
    RREA_CUDA(ctx, cudaMemcpyAsync(d + n, density_kg_m3, static_cast<size_t>(n) * sizeof(double),
                                   cudaMemcpyHostToDevice, ctx->stream));
    RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    dfree(ctx->d_profile);
    ctx->d_profile = d;
    ctx->profile_n = static_cast<int>(n);
    ctx->profile_alt0 = altitude_msl_at_z0_m;
    ctx->profile_ref = reference_density_kg_m3;
    ctx->profile_step_ratio = v / reference_density_kg_m3;
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_set_planes(rrea_gpu_ctx* ctx, const double* plane_z, int32_t n_planes)
{
    if (!ctx || n_planes < 0 || (n_planes > 0 && !plane_z)) return RREA_GPU_ERR_ARGUMENT;
    if (n_planes > 0 && ctx->n_instances > 0) {
        return fail(ctx, RREA_GPU_ERR_ARGUMENT, "the plane diagnostic is not available in ensemble mode");
    }
    // RreaPlaneLocationsAreStrictlyIncreasingFinite (I/RreaPlaneFlux.H:62-77)
    for (int32_t i = 0; i < n_planes; ++i) {
        if (!std::isfinite(plane_z[i]) || (i > 0 && !(plane_z[i] > plane_z[i - 1]))) {
            return fail(ctx, RREA_GPU_ERR_ARGUMENT, "plane z must be finite and strictly increasing");
        }
    }
    double* d = nullptr;
    if (n_planes > 0) {
        size_t const words = static_cast<size_t>(n_planes) * (1 + rrea_dev::kPlaneValues);
        if (cudaMalloc(&d, words * sizeof(double)) != cudaSuccess) {
            cudaGetLastError();
            return fail(ctx, RREA_GPU_ERR_CUDA, "plane diagnostic allocation failed");
        }
        RREA_CUDA(ctx, cudaMemcpyAsync(d, plane_z, static_cast<size_t>(n_planes) * sizeof(double),
                                       cudaMemcpyHostToDevice, ctx->stream));
        RREA_CUDA(ctx, cudaMemsetAsync(d + n_planes, 0, (words - n_planes) * sizeof(double), ctx->stream));
        RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    dfree(ctx->d_planes);
    ctx->d_planes = d;
    ctx->n_planes = n_planes;
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_plane_flux(rrea_gpu_ctx* ctx, double* values)
{
    if (!ctx || (ctx->n_planes > 0 && !values)) return RREA_GPU_ERR_ARGUMENT;
    if (ctx->n_planes == 0) return RREA_GPU_OK;
    size_t const n = static_cast<size_t>(ctx->n_planes) * rrea_dev::kPlaneValues;
    RREA_CUDA(ctx, cudaMemcpyAsync(values, ctx->d_planes + ctx->n_planes, n * sizeof(double), cudaMemcpyDeviceToHost,
                                   ctx->stream));
    RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_restore_plane_flux(rrea_gpu_ctx* ctx, const double* values)
{
    if (!ctx) return RREA_GPU_ERR_ARGUMENT;
    if (ctx->n_planes == 0) return RREA_GPU_OK;
    size_t const n = static_cast<size_t>(ctx->n_planes) * rrea_dev::kPlaneValues;
    double* const bins = ctx->d_planes + ctx->n_planes;
    if (!values) {
        RREA_CUDA(ctx, cudaMemsetAsync(bins, 0, n * sizeof(double), ctx->stream));
    } else {
        // RreaPlaneFluxAccumulator::RestoreFlat (I/RreaPlaneFlux.H:178-202)
        for (size_t i = 0; i < n; ++i) {
            if (!std::isfinite(values[i]) || values[i] < 0.0) {
                return fail(ctx, RREA_GPU_ERR_ARGUMENT, "plane accumulators must be finite and nonnegative");
            }
        }
        RREA_CUDA(ctx, cudaMemcpyAsync(bins, values, n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    }
    RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RREA_GPU_OK;
}

}  // extern "C"

namespace {

// The pointer and size checks of a host tile, before any copy.
rrea_gpu_status check_tile(rrea_gpu_ctx* ctx, rrea_gpu_tile const* t)
{
    if (t->n > ctx->capacity) return fail(ctx, RREA_GPU_ERR_CAPACITY, "tile larger than the context capacity");
    double* const host[kTileDoubles] = {t->r, t->z, t->theta, t->ux, t->uy, t->uz, t->w,
                                        t->prev_r, t->prev_z, t->prev_theta, t->prev_ux, t->prev_uy, t->prev_uz};
    for (int f = 0; f < kTileDoubles; ++f) {
        if (!host[f]) return fail(ctx, RREA_GPU_ERR_ARGUMENT, "null tile component");
    }
    if (!t->id) return fail(ctx, RREA_GPU_ERR_ARGUMENT, "null tile id");
    return RREA_GPU_OK;
}

rrea_gpu_status stage_tile(rrea_gpu_ctx* ctx, int species, rrea_gpu_tile const* t)
{
    SpeciesTile& st = ctx->tiles[species];
    if (t->n > ctx->capacity) return fail(ctx, RREA_GPU_ERR_CAPACITY, "tile larger than the context capacity");
    double* const host[kTileDoubles] = {t->r, t->z, t->theta, t->ux, t->uy, t->uz, t->w,
                                        t->prev_r, t->prev_z, t->prev_theta, t->prev_ux, t->prev_uy, t->prev_uz};
    size_t const bytes = static_cast<size_t>(t->n) * sizeof(double);
    for (int f = 0; f < kTileDoubles; ++f) {
        if (!host[f]) return fail(ctx, RREA_GPU_ERR_ARGUMENT, "null tile component");
        if (t->n) RREA_CUDA(ctx, cudaMemcpyAsync(st.d[f], host[f], bytes, cudaMemcpyHostToDevice, ctx->stream));
    }
    if (!t->id) return fail(ctx, RREA_GPU_ERR_ARGUMENT, "null tile id");
    if (t->n) {
        RREA_CUDA(ctx, cudaMemcpyAsync(st.id, t->id, static_cast<size_t>(t->n) * sizeof(int64_t),
                                       cudaMemcpyHostToDevice, ctx->stream));
        if (t->cpu) {
            RREA_CUDA(ctx, cudaMemcpyAsync(st.cpu, t->cpu, static_cast<size_t>(t->n) * sizeof(int32_t),
                                           cudaMemcpyHostToDevice, ctx->stream));
        } else {
            RREA_CUDA(ctx, cudaMemsetAsync(st.cpu, 0, static_cast<size_t>(t->n) * sizeof(int32_t), ctx->stream));
        }
    }
    st.n = t->n;
    return RREA_GPU_OK;
}

// Per-step constants of every transport kernel.
rrea_dev::StepConstants step_constants(rrea_gpu_ctx const* ctx, int32_t step, double dt_s)
{
    rrea_gpu_config const& c = ctx->cfg;
    rrea_dev::StepConstants sc{};
    sc.cfg = c;
    sc.tix = ctx->tables.index();
    sc.dr = (c.r_hi - c.r_lo) / c.nr;
    sc.dz = (c.z_hi - c.z_lo) / c.nz;
    sc.div_dr = rrea_dev::make_divisor(sc.dr);
    sc.div_dz = rrea_dev::make_divisor(sc.dz);
    sc.hm_threshold_eV = sc.tix.hard_moller_threshold_eV;
    sc.photon_cutoff_eV = c.photon_cutoff_eV;
    // RreaParticleInteraction.cpp:33-35 with a uniform density ratio
    // O/RreaParticleInteraction.cpp:27-35: the ratio at the domain's axial
    // centre, else the configured ratio, else 1
    double const configured = c.density_ratio > 0.0 ? c.density_ratio : 1.0;
    sc.density_ratio = ctx->profile_n > 0 ? (ctx->profile_step_ratio > 0.0 ? ctx->profile_step_ratio : configured)
                                          : configured;
    sc.step_key = static_cast<uint64_t>(step > 0 ? step : 0);
    sc.dt_s = dt_s;
    sc.hm_enabled = c.debug_disable_hard_moller ? 0 : 1;
    return sc;
}

// The sinks, tables and field view every transport kernel shares.
rrea_dev::ElectronArgs sink_args(rrea_gpu_ctx* ctx, rrea_dev::StepConstants const& sc)
{
    rrea_gpu_config const& c = ctx->cfg;
    rrea_dev::ElectronArgs a{};
    a.sec = ctx->d_sec_unordered;
    a.sec_count = ctx->d_sec_count;
    a.sec_capacity = ctx->sec_capacity;
    a.sec_per_parent = ctx->d_sec_per_parent;
    a.cells = ctx->d_cells;
    a.prof.n = ctx->profile_n;
    a.prof.alt = ctx->profile_n ? ctx->d_profile : nullptr;
    a.prof.val = ctx->profile_n ? ctx->d_profile + ctx->profile_n : nullptr;
    a.prof.alt0 = ctx->profile_alt0;
    a.prof.ref = ctx->profile_ref;
    a.diag_subcycles = ctx->diagnostics ? ctx->d_diag_sub : nullptr;
    a.diag_events = ctx->diagnostics ? ctx->d_diag_ev : nullptr;
    a.diag_disposition = ctx->diagnostics ? ctx->d_diag_disp : nullptr;
    a.status = ctx->d_status;
    a.fail_index = ctx->d_fail_index;
    a.transported = ctx->d_transported;
    a.arena = ctx->d_arena;
    a.fv.cell_er = ctx->d_cell_er;
    a.fv.cell_ez = ctx->d_cell_ez;
    a.fv.bt = ctx->d_bt;
    a.fv.nr = c.nr;
    a.fv.nz = c.nz;
    a.fv.dr = sc.dr;
    a.fv.dz = sc.dz;
    a.fv.div_dr = sc.div_dr;
    a.fv.div_dz = sc.div_dz;
    a.fv.r_lo = c.r_lo;
    a.fv.z_lo = c.z_lo;
    a.fv.periodic = c.periodic_z != 0;
    a.fv.has_b = ctx->has_b;
    a.fv.inst_cells = 0;
    a.fv.inst_bt = 0;
    if (ctx->n_instances > 0) {
        // ensemble: instance k's uniform field; no feedback, so no cell
        // sources and no B
        size_t const cells = static_cast<size_t>(c.nr) * c.nz;
        a.cells = nullptr;
        a.fv.cell_er = ctx->d_inst_cells;
        a.fv.cell_ez = ctx->d_inst_cells + cells * ctx->n_instances;
        a.fv.inst_cells = static_cast<int64_t>(cells);
        a.fv.has_b = false;
    }
    // the instances of an ensemble would share the planes' accumulators
    if (ctx->n_planes > 0 && ctx->n_instances == 0) {
        a.n_planes = ctx->n_planes;
        a.plane_z = ctx->d_planes;
        a.plane_bins = ctx->d_planes + ctx->n_planes;
    }
    return a;
}

// Uploads tile elements [off, off + len) of every column on `s`.
rrea_gpu_status upload_range(rrea_gpu_ctx* ctx, SpeciesTile& st, rrea_gpu_tile const* t, int64_t off, int64_t len,
                             cudaStream_t s)
{
    if (len <= 0) return RREA_GPU_OK;
    double* const host[kTileDoubles] = {t->r, t->z, t->theta, t->ux, t->uy, t->uz, t->w,
                                        t->prev_r, t->prev_z, t->prev_theta, t->prev_ux, t->prev_uy, t->prev_uz};
    size_t const bytes = static_cast<size_t>(len) * sizeof(double);
    for (int f = 0; f < kTileDoubles; ++f) {
        RREA_CUDA(ctx, cudaMemcpyAsync(st.d[f] + off, host[f] + off, bytes, cudaMemcpyHostToDevice, s));
    }
    RREA_CUDA(ctx, cudaMemcpyAsync(st.id + off, t->id + off, static_cast<size_t>(len) * sizeof(int64_t),
                                   cudaMemcpyHostToDevice, s));
    if (t->cpu) {
        RREA_CUDA(ctx, cudaMemcpyAsync(st.cpu + off, t->cpu + off, static_cast<size_t>(len) * sizeof(int32_t),
                                       cudaMemcpyHostToDevice, s));
    } else {
        RREA_CUDA(ctx, cudaMemsetAsync(st.cpu + off, 0, static_cast<size_t>(len) * sizeof(int32_t), s));
    }
    return RREA_GPU_OK;
}

// Launches one species phase (electron, positron or photon) on the device
// tile.  `aliased` runs the resident engine mode: the captured pre-push
// state is the current state (for photons the kernel then performs the
// straight push itself).  With a host tile (the drop-in calls) the upload
// is part of the launch: a large tile goes up in kPhaseChunks chunks on a
// side stream, and the kernel of each chunk starts as soon as its chunk has
// landed, on alternating streams so a chunk's tail overlaps the next one.
rrea_gpu_status launch_phase(rrea_gpu_ctx* ctx, int species, int32_t step, double dt_s, bool aliased,
                             rrea_gpu_tile const* host = nullptr)
{
    if (!ctx->tables_loaded || !ctx->field_set) {
        return fail(ctx, RREA_GPU_ERR_NOT_READY, "tables and field must be set before a step");
    }
    if (!(dt_s > 0.0) || !std::isfinite(dt_s)) return fail(ctx, RREA_GPU_ERR_ARGUMENT, "dt must be finite and positive");
    rrea_gpu_config const& c = ctx->cfg;
    rrea_dev::StepConstants const sc = step_constants(ctx, step, dt_s);
    RREA_CUDA(ctx, rrea_launch::set_step_constants(sc, ctx->stream));
    if (species == RREA_SPECIES_PHOTON) RREA_CUDA(ctx, rrea_launch::photon_constants(sc, ctx->stream));
    if (species == RREA_SPECIES_POSITRON) RREA_CUDA(ctx, rrea_launch::positron_constants(sc, ctx->stream));
    RREA_CUDA(ctx, cudaMemsetAsync(ctx->d_sec_count, 0, sizeof(unsigned long long), ctx->stream));
    RREA_CUDA(ctx, cudaMemsetAsync(ctx->d_status, 0, sizeof(int), ctx->stream));
    RREA_CUDA(ctx, cudaMemsetAsync(ctx->d_transported, 0, sizeof(unsigned long long), ctx->stream));

    rrea_dev::ElectronArgs a = sink_args(ctx, sc);
    SpeciesTile& st = ctx->tiles[species];
    if (host) st.n = host->n;
    a.n = st.n;
    double** t = st.d;
    a.r = t[0]; a.z = t[1]; a.theta = t[2]; a.ux = t[3]; a.uy = t[4]; a.uz = t[5]; a.w = t[6];
    if (aliased) {
        a.prev_r = t[0]; a.prev_z = t[1]; a.prev_theta = t[2]; a.prev_ux = t[3]; a.prev_uy = t[4]; a.prev_uz = t[5];
    } else {
        a.prev_r = t[7]; a.prev_z = t[8]; a.prev_theta = t[9]; a.prev_ux = t[10]; a.prev_uy = t[11]; a.prev_uz = t[12];
    }
    a.id = st.id;
    a.cpu = st.cpu;
    a.straight_push = (species == RREA_SPECIES_PHOTON && aliased) ? 1 : 0;
    a.segments = (species != RREA_SPECIES_PHOTON && ctx->netchord) ? ctx->d_seg : nullptr;
    // The charged kernels are long against their upload, so chunking hides
    // the upload for the price of three extra kernel tails; the photon
    // kernel is short and loses more to the tails than it gains.
    int const chunks =
        (host && species != RREA_SPECIES_PHOTON && a.n >= kPipelineMinParticles) ? kPhaseChunks : 1;
    // Register variant of the charged kernels: the configured residency, or,
    // for a tile too small to fill it, the variant with the most registers
    // per thread that still holds the whole tile in one resident wave (a
    // positron tile of 131 k particles fills 27 of 64 warps per SM: the
    // 64-register variant instead of the 32-register one).  Every variant runs
    // the same arithmetic; only spills and occupancy differ.
    int min_blocks = ctx->launch_min_blocks;
    if (chunks == 1) {
        int64_t const warps_per_sm = ((a.n + 31) / 32 + ctx->num_sms - 1) / ctx->num_sms;
        int const fit = warps_per_sm <= 8 ? 2 : warps_per_sm <= 16 ? 4 : warps_per_sm <= 32 ? 8 : 16;
        if (fit < min_blocks) min_blocks = fit;
    }
#ifndef RREA_STATIC_SCHEDULE
    RREA_CUDA(ctx, cudaMemsetAsync(ctx->d_work, 0, sizeof(unsigned long long) * chunks, ctx->stream));
#endif
    RREA_CUDA(ctx, cudaEventRecord(ctx->ev_start, ctx->stream));
    if (host && chunks == 1) {
        if (ctx->prefetched[species]) {
            // already uploaded behind the electron tile (rrea_gpu_apply_step)
            ctx->prefetched[species] = false;
            RREA_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ctx->prefetch_ev, 0));
        } else {
            rrea_gpu_status const s = upload_range(ctx, st, host, 0, a.n, ctx->stream);
            if (s != RREA_GPU_OK) return s;
        }
    }
#ifndef RREA_STATIC_SCHEDULE
    // a charged tile on the device in one piece is visited in its
    // scheduling order (lowest |u| first): warps then hold particles of
    // similar substep counts
    if (chunks == 1 && species != RREA_SPECIES_PHOTON && ctx->schedule_order && a.n >= kScheduleMinParticles) {
        RREA_CUDA(ctx, rrea_launch::cost_order(a.ux, a.uy, a.uz, a.id, a.n, ctx->d_cost_scratch, ctx->d_alive,
                                               ctx->num_sms * 4, ctx->stream));
        a.order = ctx->d_alive;
    }
#endif
    if (chunks > 1) {
        RREA_CUDA(ctx, cudaStreamWaitEvent(ctx->side[0], ctx->ev_start, 0));
        RREA_CUDA(ctx, cudaStreamWaitEvent(ctx->side[1], ctx->ev_start, 0));
    }
    for (int k = 0; k < chunks && a.n > 0; ++k) {
        int64_t const off = a.n * k / chunks;
        int64_t const len = a.n * (k + 1) / chunks - off;
        cudaStream_t const cs = (k % 2 == 0) ? ctx->stream : ctx->side[1];
        if (chunks > 1) {
            rrea_gpu_status const s = upload_range(ctx, st, host, off, len, ctx->side[0]);
            if (s != RREA_GPU_OK) return s;
            RREA_CUDA(ctx, cudaEventRecord(ctx->chunk_up[k], ctx->side[0]));
            RREA_CUDA(ctx, cudaStreamWaitEvent(cs, ctx->chunk_up[k], 0));
        }
        rrea_dev::ElectronArgs b = a;
        b.n = len;
        b.index_base = off;
        b.r += off; b.z += off; b.theta += off; b.ux += off; b.uy += off; b.uz += off; b.w += off;
        b.prev_r += off; b.prev_z += off; b.prev_theta += off; b.prev_ux += off; b.prev_uy += off; b.prev_uz += off;
        b.id += off;
        b.cpu += off;
        b.sec_per_parent += off;
        if (b.segments) b.segments += off;
        if (b.diag_subcycles) b.diag_subcycles += off;
        if (b.diag_events) b.diag_events += off;
        if (b.diag_disposition) b.diag_disposition += off;
#ifndef RREA_STATIC_SCHEDULE
        b.work = ctx->d_work + k;
        // a chunk of a drop-in tile is visited in its own scheduling order
        // (chunk-local indices at d_alive + off), built once the chunk has landed
        if (chunks > 1 && species != RREA_SPECIES_PHOTON && ctx->schedule_order && len >= kScheduleMinParticles) {
            RREA_CUDA(ctx, rrea_launch::cost_order(b.ux, b.uy, b.uz, b.id, len,
                                                   ctx->d_cost_scratch + k * rrea_launch::cost_order_scratch_elems(),
                                                   ctx->d_alive + off, ctx->num_sms * 4, cs));
            b.order = ctx->d_alive + off;
        }
#endif
        int64_t const want = (len + ctx->launch_threads - 1) / ctx->launch_threads;
        int64_t const cap = static_cast<int64_t>(ctx->num_sms) * ctx->launch_blocks_per_sm * (128 / ctx->launch_threads);
        int const blocks = static_cast<int>(want < cap ? want : cap);
        if (species == RREA_SPECIES_PHOTON) {
            RREA_CUDA(ctx, rrea_launch::photon_step(b, blocks > 0 ? blocks : 1, ctx->launch_threads, c.periodic_z != 0,
                                                    cs));
        } else if (species == RREA_SPECIES_POSITRON) {
            RREA_CUDA(ctx, rrea_launch::positron_step(b, blocks > 0 ? blocks : 1, ctx->launch_threads, min_blocks,
                                                      c.periodic_z != 0, cs));
        } else {
            RREA_CUDA(ctx, rrea_launch::electron_step(b, blocks > 0 ? blocks : 1, ctx->launch_threads, min_blocks,
                                                      c.periodic_z != 0, cs));
        }
        if (chunks > 1) RREA_CUDA(ctx, cudaEventRecord(ctx->chunk_done[k], cs));
    }
    if (chunks > 1) {
        // later phases' tiles go up behind this tile's chunks, under its kernels
        bool any = false;
        for (int sp = 0; sp < kSpecies; ++sp) {
            rrea_gpu_tile const* t = ctx->prefetch[sp];
            if (!t || sp == species) continue;
            ctx->prefetch[sp] = nullptr;
            rrea_gpu_status const s = upload_range(ctx, ctx->tiles[sp], t, 0, t->n, ctx->side[0]);
            if (s != RREA_GPU_OK) return s;
            ctx->prefetched[sp] = true;
            any = true;
        }
        if (any) RREA_CUDA(ctx, cudaEventRecord(ctx->prefetch_ev, ctx->side[0]));
        RREA_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ctx->chunk_done[chunks - 1], 0));
        RREA_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ctx->chunk_done[chunks - 2], 0));
    }
    RREA_CUDA(ctx, cudaEventRecord(ctx->ev_stop, ctx->stream));
    if (a.n > 0) {
        if (a.segments) {
            RREA_CUDA(ctx, rrea_launch::netchord_deposit(a.segments, a.n, ctx->net, dt_s, ctx->d_status,
                                                         ctx->d_fail_index, ctx->num_sms * 8, ctx->stream));
        }
    }
    unsigned long long count = 0;
    unsigned long long transported = 0;
    int status = 0;
    long long fail_index = -1;
    RREA_CUDA(ctx, cudaMemcpyAsync(&count, ctx->d_sec_count, sizeof(count), cudaMemcpyDeviceToHost, ctx->stream));
    RREA_CUDA(ctx, cudaMemcpyAsync(&status, ctx->d_status, sizeof(status), cudaMemcpyDeviceToHost, ctx->stream));
    RREA_CUDA(ctx, cudaMemcpyAsync(&fail_index, ctx->d_fail_index, sizeof(fail_index), cudaMemcpyDeviceToHost,
                                   ctx->stream));
    RREA_CUDA(ctx, cudaMemcpyAsync(&transported, ctx->d_transported, sizeof(transported), cudaMemcpyDeviceToHost,
                                   ctx->stream));
    RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->last_transported = static_cast<int64_t>(transported);
    ctx->last_kernel_ms = 0.0f;
    if (a.n > 0) RREA_CUDA(ctx, cudaEventElapsedTime(&ctx->last_kernel_ms, ctx->ev_start, ctx->ev_stop));
    if (status != 0) {
        return fail(ctx, static_cast<rrea_gpu_status>(status),
                    std::string(species == RREA_SPECIES_PHOTON ? "photon"
                                : species == RREA_SPECIES_POSITRON ? "positron" : "electron")
                        + " transport guard failed (status " + std::to_string(status) + ") at particle "
                        + std::to_string(fail_index));
    }
    if (count > static_cast<unsigned long long>(ctx->sec_capacity)) {
        return fail(ctx, RREA_GPU_ERR_CAPACITY, "secondary buffer overflow");
    }
    ctx->last_secondaries = static_cast<int64_t>(count);
    RREA_CUDA(ctx, rrea_launch::order_secondaries(ctx->d_sec_per_parent, a.n, ctx->d_offsets, ctx->d_scan_scratch,
                                                  ctx->d_sec_unordered, ctx->last_secondaries, ctx->d_sec_ordered,
                                                  ctx->stream));
    return RREA_GPU_OK;
}

rrea_gpu_status unstage_tile(rrea_gpu_ctx* ctx, int species, rrea_gpu_tile* t)
{
    SpeciesTile& st = ctx->tiles[species];
    double* const host[6] = {t->r, t->z, t->theta, t->ux, t->uy, t->uz};
    size_t const bytes = static_cast<size_t>(t->n) * sizeof(double);
    if (t->n) {
        for (int f = 0; f < 6; ++f) {
            RREA_CUDA(ctx, cudaMemcpyAsync(host[f], st.d[f], bytes, cudaMemcpyDeviceToHost, ctx->stream));
        }
        RREA_CUDA(ctx, cudaMemcpyAsync(t->id, st.id, static_cast<size_t>(t->n) * sizeof(int64_t),
                                       cudaMemcpyDeviceToHost, ctx->stream));
    }
    return RREA_GPU_OK;
}

rrea_gpu_status apply_phase(rrea_gpu_ctx* ctx, int species, rrea_gpu_tile* tile, int32_t step, double dt_s,
                            rrea_gpu_secondary* secondaries, int64_t secondary_capacity, int64_t* n_secondaries)
{
    if (!ctx || !tile || tile->n < 0) return RREA_GPU_ERR_ARGUMENT;
    rrea_gpu_status s = check_tile(ctx, tile);
    if (s != RREA_GPU_OK) return s;
    s = launch_phase(ctx, species, step, dt_s, /*aliased=*/false, tile);
    if (s != RREA_GPU_OK) return s;
    if (n_secondaries) *n_secondaries = ctx->last_secondaries;
    if (secondaries && ctx->last_secondaries > secondary_capacity) {
        return fail(ctx, RREA_GPU_ERR_CAPACITY, "caller secondary buffer too small");
    }
    s = unstage_tile(ctx, species, tile);
    if (s != RREA_GPU_OK) return s;
    if (secondaries && ctx->last_secondaries > 0) {
        RREA_CUDA(ctx, cudaMemcpyAsync(secondaries, ctx->d_sec_ordered,
                                       static_cast<size_t>(ctx->last_secondaries) * sizeof(rrea_gpu_secondary),
                                       cudaMemcpyDeviceToHost, ctx->stream));
    }
    RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RREA_GPU_OK;
}

rrea_gpu_status stage_species(rrea_gpu_ctx* ctx, int species, const rrea_gpu_tile* tile)
{
    if (!ctx || !tile || tile->n < 0) return RREA_GPU_ERR_ARGUMENT;
    rrea_gpu_status const s = stage_tile(ctx, species, tile);
    if (s != RREA_GPU_OK) return s;
    // ids committed later continue after the largest staged id
    int64_t top = 0;
    for (int64_t i = 0; i < tile->n; ++i) {
        int64_t const a = tile->id[i] < 0 ? -tile->id[i] : tile->id[i];
        top = a > top ? a : top;
    }
    ctx->next_id[species] = top + 1;
    ctx->part_valid[species] = false;
    if (ctx->n_instances > 0) {
        // per-instance counters continue after each instance's largest id
        std::vector<int64_t> next(static_cast<size_t>(ctx->n_instances), 1);
        for (int64_t i = 0; i < tile->n; ++i) {
            int32_t const k = tile->cpu ? tile->cpu[i] : 0;
            if (k < 0 || k >= ctx->n_instances) {
                return fail(ctx, RREA_GPU_ERR_ARGUMENT, "an ensemble particle's cpu ordinal is not an instance");
            }
            int64_t const a = tile->id[i] < 0 ? -tile->id[i] : tile->id[i];
            next[static_cast<size_t>(k)] = std::max(next[static_cast<size_t>(k)], a + 1);
        }
        for (int32_t k = 0; k < ctx->n_instances; ++k) {
            RREA_CUDA(ctx, cudaMemcpyAsync(ctx->d_inst_next_id + 3 * static_cast<int64_t>(k) + species,
                                           &next[static_cast<size_t>(k)], sizeof(int64_t), cudaMemcpyHostToDevice,
                                           ctx->stream));
        }
    }
    RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RREA_GPU_OK;
}

rrea_dev::TileColumns columns(SpeciesTile const& st)
{
    rrea_dev::TileColumns t{};
    for (int f = 0; f < kTileDoubles; ++f) t.d[f] = st.d[f];
    t.id = st.id;
    t.cpu = st.cpu;
    return t;
}

rrea_gpu_status fetch_species(rrea_gpu_ctx* ctx, int species, rrea_gpu_tile* tile)
{
    if (!ctx || !tile || tile->n != ctx->tiles[species].n) return RREA_GPU_ERR_ARGUMENT;
    rrea_gpu_status const s = unstage_tile(ctx, species, tile);
    if (s != RREA_GPU_OK) return s;
    // a resident tile also gains particles (committed survivors): their
    // weights and cpu words come back too
    SpeciesTile const& st = ctx->tiles[species];
    if (tile->n && tile->w) {
        RREA_CUDA(ctx, cudaMemcpyAsync(tile->w, st.d[6], static_cast<size_t>(tile->n) * sizeof(double),
                                       cudaMemcpyDeviceToHost, ctx->stream));
    }
    if (tile->n && tile->cpu) {
        RREA_CUDA(ctx, cudaMemcpyAsync(tile->cpu, st.cpu, static_cast<size_t>(tile->n) * sizeof(int32_t),
                                       cudaMemcpyDeviceToHost, ctx->stream));
    }
    RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RREA_GPU_OK;
}

// Makes `buf` hold at least `need` records with the `keep` records that
// started at `from` moved to its front.  Reallocates (synchronizing the
// stream) only when the buffer is too small or the records must move.
rrea_gpu_status grow_records(rrea_gpu_ctx* ctx, rrea_gpu_secondary*& buf, int64_t& cap, int64_t need, int64_t from,
                             int64_t keep)
{
    if (need <= cap && from == 0) return RREA_GPU_OK;
    int64_t const target = need > cap ? std::max<int64_t>(need, std::max<int64_t>(2 * cap, 4096)) : cap;
    rrea_gpu_secondary* nb = nullptr;
    RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    RREA_CUDA(ctx, dalloc(&nb, static_cast<size_t>(target)));
    if (keep > 0) {
        RREA_CUDA(ctx, cudaMemcpyAsync(nb, buf + from, static_cast<size_t>(keep) * sizeof(rrea_gpu_secondary),
                                       cudaMemcpyDeviceToDevice, ctx->stream));
        RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    dfree(buf);
    buf = nb;
    cap = target;
    return RREA_GPU_OK;
}

// Appends the last phase's ordered secondaries to the pending FIFO.
rrea_gpu_status queue_secondaries(rrea_gpu_ctx* ctx)
{
    int64_t const n = ctx->last_secondaries;
    if (n <= 0) return RREA_GPU_OK;
    rrea_gpu_status const s =
        grow_records(ctx, ctx->d_fifo, ctx->fifo_cap, ctx->fifo_pending + n, 0, ctx->fifo_pending);
    if (s != RREA_GPU_OK) return s;
    RREA_CUDA(ctx, cudaMemcpyAsync(ctx->d_fifo + ctx->fifo_pending, ctx->d_sec_ordered,
                                   static_cast<size_t>(n) * sizeof(rrea_gpu_secondary), cudaMemcpyDeviceToDevice,
                                   ctx->stream));
    ctx->fifo_pending += n;
    return RREA_GPU_OK;
}

rrea_gpu_status step_resident(rrea_gpu_ctx* ctx, int species, int32_t step, double dt_s, int64_t* n_secondaries)
{
    if (!ctx) return RREA_GPU_ERR_ARGUMENT;
    rrea_gpu_status s = launch_phase(ctx, species, step, dt_s, /*aliased=*/true);
    if (s != RREA_GPU_OK) return s;
    if (n_secondaries) *n_secondaries = ctx->last_secondaries;
    s = queue_secondaries(ctx);
    if (s != RREA_GPU_OK) return s;
    RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RREA_GPU_OK;
}

// DrainAndCommitSecondaries' transient FIFO (O/RreaSecondaryCommit.cpp:331-474)
// over d_fifo[0, n_initial).  The FIFO is a breadth-first walk: the children
// of a chunk are appended behind every item already queued, so advancing it
// chunk by chunk (at most `capacity` items, one thread each) and merging each
// chunk's children in item order reproduces the reference's batch-of-1024
// order exactly.  Lineages of the children come from one counter per root
// (RNG key, root species), seeded by the initial items and kept here on the
// host: a child's root is its item's root, so only the per-item child counts
// cross to the host.
rrea_gpu_status drain_fifo(rrea_gpu_ctx* ctx, int32_t step, double dt_s, int64_t n_initial)
{
    if (!ctx->tables_loaded || !ctx->field_set) {
        return fail(ctx, RREA_GPU_ERR_NOT_READY, "tables and field must be set before a drain");
    }
    if (!(dt_s > 0.0) || !std::isfinite(dt_s)) return fail(ctx, RREA_GPU_ERR_ARGUMENT, "dt must be finite and positive");
    rrea_gpu_config const& c = ctx->cfg;
    rrea_dev::StepConstants const sc = step_constants(ctx, step, dt_s);
    ctx->n_surv = 0;
    ctx->last_drain_items = 0;
    RREA_CUDA(ctx, rrea_launch::newborn_constants(sc, ctx->stream));
    auto check_payloads = [&](rrea_gpu_secondary const* items, int64_t n, int mode) -> rrea_gpu_status {
        unsigned long long invalid = 0;
        long long first = INT64_MAX;
        RREA_CUDA(ctx, cudaMemsetAsync(ctx->d_invalid, 0, sizeof(unsigned long long), ctx->stream));
        RREA_CUDA(ctx, cudaMemcpyAsync(ctx->d_fail_index, &first, sizeof(first), cudaMemcpyHostToDevice, ctx->stream));
        RREA_CUDA(ctx, rrea_launch::validate_fifo(items, n, mode, ctx->d_invalid, ctx->d_fail_index, ctx->stream));
        RREA_CUDA(ctx, cudaMemcpyAsync(&invalid, ctx->d_invalid, sizeof(invalid), cudaMemcpyDeviceToHost, ctx->stream));
        RREA_CUDA(ctx, cudaMemcpyAsync(&first, ctx->d_fail_index, sizeof(first), cudaMemcpyDeviceToHost, ctx->stream));
        RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        if (invalid == 0) return RREA_GPU_OK;
        return fail(ctx, mode == 0 ? RREA_GPU_ERR_ARGUMENT : RREA_GPU_ERR_INVALID_STATE,
                    std::string(mode == 0 ? "transient FIFO received an invalid birth payload"
                                          : "transient work graph contains invalid final survivors")
                        + " (" + std::to_string(invalid) + " records, first at " + std::to_string(first) + ")");
    };
    rrea_gpu_status s = check_payloads(ctx->d_fifo, n_initial, 0);
    if (s != RREA_GPU_OK) return s;

    // slot[k] is the root slot of FIFO item root_base + k (FIFO indices
    // count every item merged since the drain began); next[s] is the next
    // free lineage of slot s
    std::vector<uint32_t> slot(static_cast<size_t>(n_initial));
    std::vector<uint64_t> next;
    if (n_initial > ctx->roots_cap) {
        RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        int64_t const cap = std::max<int64_t>(n_initial, 2 * ctx->roots_cap);
        dfree(ctx->d_roots);
        if (ctx->h_roots) cudaFreeHost(ctx->h_roots);
        ctx->d_roots = nullptr;
        ctx->h_roots = nullptr;
        ctx->roots_cap = 0;
        RREA_CUDA(ctx, dalloc(&ctx->d_roots, static_cast<size_t>(2 * cap)));
        RREA_CUDA(ctx, cudaMallocHost(reinterpret_cast<void**>(&ctx->h_roots),
                                      static_cast<size_t>(2 * cap) * sizeof(unsigned long long)));
        ctx->roots_cap = cap;
    }
    if (n_initial > 0) {
        RREA_CUDA(ctx, rrea_launch::gather_roots(ctx->d_fifo, n_initial, ctx->d_roots, ctx->stream));
        RREA_CUDA(ctx, cudaMemcpyAsync(ctx->h_roots, ctx->d_roots,
                                       static_cast<size_t>(2 * n_initial) * sizeof(unsigned long long),
                                       cudaMemcpyDeviceToHost, ctx->stream));
        RREA_CUDA(ctx, cudaEventRecord(ctx->roots_ev, ctx->stream));
    }
    // The root table is built on the host while the first chunk's newborn
    // kernels run: only the lineages of that chunk's children need it.
    bool roots_built = false;
    auto build_roots = [&]() -> rrea_gpu_status {
        roots_built = true;
        if (n_initial <= 0) return RREA_GPU_OK;
        RREA_CUDA(ctx, cudaEventSynchronize(ctx->roots_ev));
        unsigned long long const* roots = ctx->h_roots;
        RootSlots& table = ctx->root_slots;
        table.reset(static_cast<size_t>(n_initial));
        for (int64_t i = 0; i < n_initial; ++i) {
            uint64_t const key = roots[2 * i];
            int32_t const species = static_cast<int32_t>(roots[2 * i + 1] >> 32);
            uint64_t const lin = roots[2 * i + 1] & 0xffffffffULL;
            // the records of one parent are adjacent: reuse the previous slot
            uint32_t s;
            if (i > 0 && roots[2 * i] == roots[2 * i - 2] && (roots[2 * i + 1] >> 32) == (roots[2 * i - 1] >> 32)) {
                s = slot[static_cast<size_t>(i - 1)];
            } else {
                bool inserted = false;
                s = table.find_or_insert(key, species, static_cast<uint32_t>(next.size()), inserted);
                if (inserted) next.push_back(0);
            }
            slot[static_cast<size_t>(i)] = s;
            next[s] = std::max<uint64_t>(next[s], lin + 1U);
        }
        return RREA_GPU_OK;
    };
    std::vector<uint32_t> counts;
    std::vector<uint64_t> lineage;
    int64_t cursor = 0, tail = n_initial;
    size_t root_base = 0;
    while (cursor < tail) {
        int64_t const chunk = std::min<int64_t>(tail - cursor, ctx->capacity);
        RREA_CUDA(ctx, cudaMemsetAsync(ctx->d_sec_count, 0, sizeof(unsigned long long), ctx->stream));
        RREA_CUDA(ctx, cudaMemsetAsync(ctx->d_status, 0, sizeof(int), ctx->stream));
        rrea_dev::ElectronArgs a = sink_args(ctx, sc);
        a.diag_subcycles = nullptr;
        a.diag_events = nullptr;
        a.diag_disposition = nullptr;
        a.segments = ctx->netchord ? ctx->d_seg : nullptr;
        rrea_gpu_secondary* const items = ctx->d_fifo + cursor;
        RREA_CUDA(ctx, rrea_launch::newborn_step(a, items, chunk, ctx->d_alive, ctx->num_sms * 8, c.periodic_z != 0,
                                                 ctx->stream, ctx->side, ctx->fork_ev, ctx->join_ev));
        if (a.segments) {
            RREA_CUDA(ctx, rrea_launch::netchord_deposit(a.segments, chunk, ctx->net, dt_s, ctx->d_status,
                                                         ctx->d_fail_index, ctx->num_sms * 8, ctx->stream));
        }
        unsigned long long count = 0;
        int status = 0;
        long long fail_index = -1;
        int64_t last_offset = 0;
        uint32_t last_alive = 0;
        RREA_CUDA(ctx, rrea_launch::exclusive_scan_counts(ctx->d_alive, chunk, ctx->d_offsets, ctx->d_scan_scratch,
                                                          ctx->stream));
        RREA_CUDA(ctx, cudaMemcpyAsync(&count, ctx->d_sec_count, sizeof(count), cudaMemcpyDeviceToHost, ctx->stream));
        RREA_CUDA(ctx, cudaMemcpyAsync(&status, ctx->d_status, sizeof(status), cudaMemcpyDeviceToHost, ctx->stream));
        RREA_CUDA(ctx, cudaMemcpyAsync(&fail_index, ctx->d_fail_index, sizeof(fail_index), cudaMemcpyDeviceToHost,
                                       ctx->stream));
        RREA_CUDA(ctx, cudaMemcpyAsync(&last_offset, ctx->d_offsets + (chunk - 1), sizeof(last_offset),
                                       cudaMemcpyDeviceToHost, ctx->stream));
        RREA_CUDA(ctx, cudaMemcpyAsync(&last_alive, ctx->d_alive + (chunk - 1), sizeof(last_alive),
                                       cudaMemcpyDeviceToHost, ctx->stream));
        counts.resize(static_cast<size_t>(chunk));
        RREA_CUDA(ctx, cudaMemcpyAsync(counts.data(), ctx->d_sec_per_parent, static_cast<size_t>(chunk) * sizeof(uint32_t),
                                       cudaMemcpyDeviceToHost, ctx->stream));
        if (!roots_built) {
            s = build_roots();
            if (s != RREA_GPU_OK) return s;
        }
        RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        if (status != 0) {
            return fail(ctx, static_cast<rrea_gpu_status>(status),
                        "newborn transport guard failed (status " + std::to_string(status) + ") at FIFO item "
                            + std::to_string(cursor + fail_index));
        }
        if (count > static_cast<unsigned long long>(ctx->sec_capacity)) {
            return fail(ctx, RREA_GPU_ERR_CAPACITY, "newborn child buffer overflow");
        }
        // survivors of the chunk, in FIFO order
        int64_t const survivors = last_offset + static_cast<int64_t>(last_alive);
        s = grow_records(ctx, ctx->d_surv, ctx->surv_cap, ctx->n_surv + survivors, 0, ctx->n_surv);
        if (s != RREA_GPU_OK) return s;
        RREA_CUDA(ctx, rrea_launch::compact_survivors(items, ctx->d_alive, ctx->d_offsets, chunk,
                                                      ctx->d_surv + ctx->n_surv, ctx->stream));
        ctx->n_surv += survivors;
        // children: lineage per root in merge order, then appended behind the tail
        int64_t const n_children = static_cast<int64_t>(count);
        if (n_children > 0) {
            lineage.resize(static_cast<size_t>(n_children));
            size_t j = 0;
            for (int64_t i = 0; i < chunk; ++i) {
                uint32_t const ci = counts[static_cast<size_t>(i)];
                if (ci == 0) continue;
                uint32_t const s = slot[static_cast<size_t>(ctx->last_drain_items) - root_base + static_cast<size_t>(i)];
                uint64_t& nx = next[s];
                for (uint32_t t = 0; t < ci; ++t) {
                    if (nx >= rrea_dev::kLineageCap || j >= lineage.size()) {
                        return fail(ctx, RREA_GPU_ERR_RNG_OVERFLOW, "transient FIFO lineage overflow");
                    }
                    lineage[j++] = nx++;
                    slot.push_back(s);
                }
            }
            if (j != lineage.size()) return fail(ctx, RREA_GPU_ERR_INVALID_STATE, "newborn child count mismatch");
            RREA_CUDA(ctx, rrea_launch::order_secondaries(ctx->d_sec_per_parent, chunk, ctx->d_offsets,
                                                          ctx->d_scan_scratch, ctx->d_sec_unordered, n_children,
                                                          ctx->d_sec_ordered, ctx->stream));
            RREA_CUDA(ctx, cudaMemcpyAsync(ctx->d_child_lineage, lineage.data(),
                                           static_cast<size_t>(n_children) * sizeof(uint64_t), cudaMemcpyHostToDevice,
                                           ctx->stream));
            // make room behind the tail; items before the cursor are no longer needed
            if (tail + n_children > ctx->fifo_cap) {
                s = grow_records(ctx, ctx->d_fifo, ctx->fifo_cap, tail - cursor + n_children, cursor, tail - cursor);
                if (s != RREA_GPU_OK) return s;
                tail -= cursor;
                cursor = 0;
            }
            RREA_CUDA(ctx, rrea_launch::adopt_children(ctx->d_sec_ordered, n_children, ctx->d_fifo + cursor,
                                                       ctx->d_child_lineage, ctx->d_fifo + tail, ctx->stream));
            tail += n_children;
        }
        ctx->last_drain_items += chunk;
        cursor += chunk;
        // slots of merged items are no longer needed
        size_t const done = static_cast<size_t>(ctx->last_drain_items) - root_base;
        if (done > (1u << 20) && done * 2 > slot.size()) {
            slot.erase(slot.begin(), slot.begin() + static_cast<std::ptrdiff_t>(done));
            root_base += done;
        }
    }
    return check_payloads(ctx->d_surv, ctx->n_surv, 1);
}

}  // namespace

extern "C" {

rrea_gpu_status rrea_gpu_apply_electrons(rrea_gpu_ctx* ctx, rrea_gpu_tile* tile, int32_t step, double time_s,
                                         double dt_s, rrea_gpu_secondary* secondaries, int64_t secondary_capacity,
                                         int64_t* n_secondaries)
{
    (void)time_s;
    return apply_phase(ctx, RREA_SPECIES_ELECTRON, tile, step, dt_s, secondaries, secondary_capacity, n_secondaries);
}

rrea_gpu_status rrea_gpu_apply_positrons(rrea_gpu_ctx* ctx, rrea_gpu_tile* tile, int32_t step, double time_s,
                                         double dt_s, rrea_gpu_secondary* secondaries, int64_t secondary_capacity,
                                         int64_t* n_secondaries)
{
    (void)time_s;
    return apply_phase(ctx, RREA_SPECIES_POSITRON, tile, step, dt_s, secondaries, secondary_capacity, n_secondaries);
}

rrea_gpu_status rrea_gpu_apply_photons(rrea_gpu_ctx* ctx, rrea_gpu_tile* tile, int32_t step, double time_s,
                                       double dt_s, rrea_gpu_secondary* secondaries, int64_t secondary_capacity,
                                       int64_t* n_secondaries)
{
    (void)time_s;
    return apply_phase(ctx, RREA_SPECIES_PHOTON, tile, step, dt_s, secondaries, secondary_capacity, n_secondaries);
}

rrea_gpu_status rrea_gpu_download_sources(rrea_gpu_ctx* ctx, double* out5)
{
    if (!ctx || !out5) return RREA_GPU_ERR_ARGUMENT;
    size_t const n = static_cast<size_t>(ctx->cfg.nr) * ctx->cfg.nz * 5;
    RREA_CUDA(ctx, cudaMemcpyAsync(out5, ctx->d_cells, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_reset_sources(rrea_gpu_ctx* ctx)
{
    if (!ctx) return RREA_GPU_ERR_ARGUMENT;
    size_t const n = static_cast<size_t>(ctx->cfg.nr) * ctx->cfg.nz * 5;
    RREA_CUDA(ctx, cudaMemsetAsync(ctx->d_cells, 0, n * sizeof(double), ctx->stream));
    RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_reset_current(rrea_gpu_ctx* ctx)
{
    if (!ctx) return RREA_GPU_ERR_ARGUMENT;
    if (!ctx->netchord) return fail(ctx, RREA_GPU_ERR_ARGUMENT, "net-chord current needs a non-periodic z domain");
    rrea_dev::NetGrid const& g = ctx->net;
    RREA_CUDA(ctx, cudaMemsetAsync(g.rho, 0, static_cast<size_t>(g.nr) * g.nz * sizeof(double), ctx->stream));
    RREA_CUDA(ctx, cudaMemsetAsync(g.jr, 0, static_cast<size_t>(g.nr + 1) * g.nz * sizeof(double), ctx->stream));
    RREA_CUDA(ctx, cudaMemsetAsync(g.jz, 0, static_cast<size_t>(g.nr) * (g.nz + 1) * sizeof(double), ctx->stream));
    RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_download_current(rrea_gpu_ctx* ctx, double* jr, double* jz)
{
    if (!ctx || !jr || !jz) return RREA_GPU_ERR_ARGUMENT;
    if (!ctx->netchord) return fail(ctx, RREA_GPU_ERR_ARGUMENT, "net-chord current needs a non-periodic z domain");
    rrea_gpu_config const& c = ctx->cfg;
    RREA_CUDA(ctx, rrea_launch::netchord_convert(ctx->net, ctx->d_jr_phys, ctx->d_jz_phys, ctx->stream));
    RREA_CUDA(ctx, cudaMemcpyAsync(jr, ctx->d_jr_phys, static_cast<size_t>(c.nr + 1) * c.nz * sizeof(double),
                                   cudaMemcpyDeviceToHost, ctx->stream));
    RREA_CUDA(ctx, cudaMemcpyAsync(jz, ctx->d_jz_phys, static_cast<size_t>(c.nr) * (c.nz + 1) * sizeof(double),
                                   cudaMemcpyDeviceToHost, ctx->stream));
    RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_download_current_index(rrea_gpu_ctx* ctx, double* rho, double* jr, double* jz)
{
    if (!ctx || !rho || !jr || !jz) return RREA_GPU_ERR_ARGUMENT;
    if (!ctx->netchord) return fail(ctx, RREA_GPU_ERR_ARGUMENT, "net-chord current needs a non-periodic z domain");
    rrea_dev::NetGrid const& g = ctx->net;
    RREA_CUDA(ctx, cudaMemcpyAsync(rho, g.rho, static_cast<size_t>(g.nr) * g.nz * sizeof(double),
                                   cudaMemcpyDeviceToHost, ctx->stream));
    RREA_CUDA(ctx, cudaMemcpyAsync(jr, g.jr, static_cast<size_t>(g.nr + 1) * g.nz * sizeof(double),
                                   cudaMemcpyDeviceToHost, ctx->stream));
    RREA_CUDA(ctx, cudaMemcpyAsync(jz, g.jz, static_cast<size_t>(g.nr) * (g.nz + 1) * sizeof(double),
                                   cudaMemcpyDeviceToHost, ctx->stream));
    RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_current_device(rrea_gpu_ctx* ctx, double** d_jr, double** d_jz)
{
    if (!ctx) return RREA_GPU_ERR_ARGUMENT;
    if (!ctx->netchord) return fail(ctx, RREA_GPU_ERR_ARGUMENT, "the net-chord current needs a non-periodic z domain");
    RREA_CUDA(ctx, rrea_launch::netchord_convert(ctx->net, ctx->d_jr_phys, ctx->d_jz_phys, ctx->stream));
    RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (d_jr) *d_jr = ctx->d_jr_phys;
    if (d_jz) *d_jz = ctx->d_jz_phys;
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_advance_field(rrea_gpu_ctx* ctx, double dt_s, int32_t substeps)
{
    rrea_gpu_status const s = rrea_gpu_current_device(ctx, nullptr, nullptr);
    if (s != RREA_GPU_OK) return s;
    return rrea_gpu_advance_field_from_current(ctx, dt_s, substeps);
}

rrea_gpu_status rrea_gpu_advance_field_from_current(rrea_gpu_ctx* ctx, double dt_s, int32_t substeps)
{
    if (!ctx || !(dt_s > 0.0) || !std::isfinite(dt_s) || substeps < 1) return RREA_GPU_ERR_ARGUMENT;
    if (!ctx->field_set) return fail(ctx, RREA_GPU_ERR_NOT_READY, "the field must be set before it is advanced");
    if (!ctx->netchord) return fail(ctx, RREA_GPU_ERR_ARGUMENT, "the field update needs a non-periodic z domain");
    rrea_gpu_config const& c = ctx->cfg;
    rrea_dev::NetGrid const& g = ctx->net;
    double const cfl = 299792458.0 * dt_s * std::sqrt(1.0 / (g.dr * g.dr) + 1.0 / (g.dz * g.dz));
    if (!std::isfinite(cfl) || !(cfl < 1.0)) {
        return fail(ctx, RREA_GPU_ERR_ARGUMENT, "Maxwell TM violates the Yee CFL condition c dt sqrt(dr^-2+dz^-2) < 1");
    }
    RREA_CUDA(ctx, rrea_launch::maxwell_step(c.nr, c.nz, g.dr, g.dz, dt_s, substeps, ctx->d_er, ctx->d_ez, ctx->d_bt,
                                             ctx->d_jr_phys, ctx->d_jz_phys, ctx->stream));
    RREA_CUDA(ctx, rrea_launch::field_prep(c.nr, c.nz, ctx->d_er, ctx->d_ez, ctx->d_amb_er, ctx->d_amb_ez,
                                           ctx->d_cell_er, ctx->d_cell_ez, ctx->stream));
    RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->has_b = true;
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_download_field(rrea_gpu_ctx* ctx, double* er, double* ez, double* bt)
{
    if (!ctx || !er || !ez || !bt) return RREA_GPU_ERR_ARGUMENT;
    if (!ctx->field_set) return fail(ctx, RREA_GPU_ERR_NOT_READY, "no field has been set");
    rrea_gpu_config const& c = ctx->cfg;
    size_t const ner = static_cast<size_t>(c.nr + 1) * c.nz;
    size_t const nez = static_cast<size_t>(c.nr) * (c.nz + 1);
    size_t const nbt = static_cast<size_t>(c.nr + 1) * (c.nz + 1);
    RREA_CUDA(ctx, cudaMemcpyAsync(er, ctx->d_er, ner * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    RREA_CUDA(ctx, cudaMemcpyAsync(ez, ctx->d_ez, nez * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    RREA_CUDA(ctx, cudaMemcpyAsync(bt, ctx->d_bt, nbt * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_drain_secondaries(rrea_gpu_ctx* ctx, const rrea_gpu_secondary* pending, int64_t n_pending,
                                           int32_t step, double dt_s, rrea_gpu_secondary* survivors,
                                           int64_t survivor_capacity, int64_t* n_survivors)
{
    if (!ctx || n_pending < 0 || (n_pending > 0 && !pending) || survivor_capacity < 0) return RREA_GPU_ERR_ARGUMENT;
    ctx->fifo_pending = 0;
    rrea_gpu_status s = grow_records(ctx, ctx->d_fifo, ctx->fifo_cap, n_pending, 0, 0);
    if (s != RREA_GPU_OK) return s;
    if (n_pending > 0) {
        RREA_CUDA(ctx, cudaMemcpyAsync(ctx->d_fifo, pending, static_cast<size_t>(n_pending) * sizeof(rrea_gpu_secondary),
                                       cudaMemcpyHostToDevice, ctx->stream));
    }
    s = drain_fifo(ctx, step, dt_s, n_pending);
    if (s != RREA_GPU_OK) return s;
    if (n_survivors) *n_survivors = ctx->n_surv;
    if (survivors && ctx->n_surv > survivor_capacity) {
        return fail(ctx, RREA_GPU_ERR_CAPACITY, "caller survivor buffer too small");
    }
    if (survivors && ctx->n_surv > 0) {
        RREA_CUDA(ctx, cudaMemcpyAsync(survivors, ctx->d_surv, static_cast<size_t>(ctx->n_surv) * sizeof(rrea_gpu_secondary),
                                       cudaMemcpyDeviceToHost, ctx->stream));
    }
    RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_apply_step(rrea_gpu_ctx* ctx, rrea_gpu_tile* electrons, rrea_gpu_tile* photons,
                                    rrea_gpu_tile* positrons, int32_t step, double time_s, double dt_s,
                                    rrea_gpu_secondary* survivors, int64_t survivor_capacity, int64_t* n_survivors)
{
    (void)time_s;
    if (!ctx || survivor_capacity < 0 || (survivor_capacity > 0 && !survivors)) return RREA_GPU_ERR_ARGUMENT;
    // Apply's phase order (O/RreaParticleInteraction.cpp:12-62)
    struct Phase {
        int species;
        rrea_gpu_tile* tile;
    } const phases[3] = {{RREA_SPECIES_ELECTRON, electrons}, {RREA_SPECIES_PHOTON, photons},
                         {RREA_SPECIES_POSITRON, positrons}};
    for (Phase const& ph : phases) {
        if (!ph.tile) continue;
        if (ph.tile->n < 0) return RREA_GPU_ERR_ARGUMENT;
        rrea_gpu_status const s = check_tile(ctx, ph.tile);
        if (s != RREA_GPU_OK) return s;
    }
    // the phases' secondaries queue on the device in phase order, and the
    // transient FIFO drains them there: no secondary crosses to the host
    ctx->fifo_pending = 0;
    // photon and positron tiles that go up in one piece are uploaded under a
    // chunked electron phase's kernels
    if (electrons && electrons->n >= kPipelineMinParticles) {
        for (Phase const& ph : phases) {
            if (ph.tile && ph.species != RREA_SPECIES_ELECTRON && ph.tile->n > 0
                && (ph.species == RREA_SPECIES_PHOTON || ph.tile->n < kPipelineMinParticles)) {
                ctx->prefetch[ph.species] = ph.tile;
            }
        }
    }
    auto clear_prefetch = [&]() {
        for (int sp = 0; sp < kSpecies; ++sp) {
            ctx->prefetch[sp] = nullptr;
            ctx->prefetched[sp] = false;
        }
    };
    for (Phase const& ph : phases) {
        if (!ph.tile) continue;
        rrea_gpu_status s = launch_phase(ctx, ph.species, step, dt_s, /*aliased=*/false, ph.tile);
        if (s == RREA_GPU_OK) s = queue_secondaries(ctx);
        if (s != RREA_GPU_OK) {
            ctx->fifo_pending = 0;
            clear_prefetch();
            cudaStreamSynchronize(ctx->side[0]);
            return s;
        }
    }
    clear_prefetch();
    int64_t const n = ctx->fifo_pending;
    ctx->fifo_pending = 0;
    rrea_gpu_status s = drain_fifo(ctx, step, dt_s, n);
    if (s != RREA_GPU_OK) return s;
    if (n_survivors) *n_survivors = ctx->n_surv;
    if (ctx->n_surv > survivor_capacity) return fail(ctx, RREA_GPU_ERR_CAPACITY, "caller survivor buffer too small");
    // every guard passed: only now do the caller's tiles change
    for (Phase const& ph : phases) {
        if (!ph.tile) continue;
        s = unstage_tile(ctx, ph.species, ph.tile);
        if (s != RREA_GPU_OK) return s;
    }
    if (ctx->n_surv > 0) {
        RREA_CUDA(ctx, cudaMemcpyAsync(survivors, ctx->d_surv, static_cast<size_t>(ctx->n_surv) * sizeof(rrea_gpu_secondary),
                                       cudaMemcpyDeviceToHost, ctx->stream));
    }
    RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_drain_resident(rrea_gpu_ctx* ctx, int32_t step, double dt_s, int64_t* n_survivors)
{
    if (!ctx) return RREA_GPU_ERR_ARGUMENT;
    int64_t const n = ctx->fifo_pending;
    // the queued records are consumed whether or not the drain succeeds
    ctx->fifo_pending = 0;
    rrea_gpu_status const s = drain_fifo(ctx, step, dt_s, n);
    if (s != RREA_GPU_OK) return s;
    if (n_survivors) *n_survivors = ctx->n_surv;
    RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_fetch_survivors(rrea_gpu_ctx* ctx, rrea_gpu_secondary* survivors, int64_t capacity,
                                         int64_t* n_survivors)
{
    if (!ctx || capacity < 0 || (capacity > 0 && !survivors)) return RREA_GPU_ERR_ARGUMENT;
    if (n_survivors) *n_survivors = ctx->n_surv;
    if (ctx->n_surv > capacity) return fail(ctx, RREA_GPU_ERR_CAPACITY, "caller survivor buffer too small");
    if (ctx->n_surv > 0) {
        RREA_CUDA(ctx, cudaMemcpyAsync(survivors, ctx->d_surv, static_cast<size_t>(ctx->n_surv) * sizeof(rrea_gpu_secondary),
                                       cudaMemcpyDeviceToHost, ctx->stream));
    }
    RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_commit_survivors_resident(rrea_gpu_ctx* ctx, int64_t* committed)
{
    if (!ctx) return RREA_GPU_ERR_ARGUMENT;
    int64_t added[kSpecies] = {0, 0, 0};
    int64_t const n = ctx->n_surv;
    if (n > 0) {
        if (n > ctx->commit_cap) {
            dfree(ctx->d_commit_flags);
            dfree(ctx->d_commit_offsets);
            dfree(ctx->d_commit_scan);
            ctx->d_commit_flags = nullptr;
            ctx->d_commit_offsets = nullptr;
            ctx->d_commit_scan = nullptr;
            ctx->commit_cap = 0;
            int64_t const cap = n + n / 2 + 1024;
            if (dalloc(&ctx->d_commit_flags, static_cast<size_t>(cap)) != cudaSuccess
                || dalloc(&ctx->d_commit_offsets, static_cast<size_t>(cap)) != cudaSuccess
                || dalloc(&ctx->d_commit_scan, static_cast<size_t>(rrea_launch::scan_scratch_elems(cap))) != cudaSuccess) {
                cudaGetLastError();
                return fail(ctx, RREA_GPU_ERR_CUDA, "commit scratch allocation failed");
            }
            ctx->commit_cap = cap;
        }
        // all three species are ranked before any tile changes, so a full
        // tile leaves every tile as it was
        for (int species = 0; species < kSpecies; ++species) {
            RREA_CUDA(ctx, rrea_launch::commit_rank(ctx->d_surv, n, species, ctx->d_commit_flags,
                                                    ctx->d_commit_offsets, ctx->d_commit_scan, ctx->stream));
            int64_t last_off = 0;
            uint32_t last_flag = 0;
            RREA_CUDA(ctx, cudaMemcpyAsync(&last_off, ctx->d_commit_offsets + n - 1, sizeof(last_off),
                                           cudaMemcpyDeviceToHost, ctx->stream));
            RREA_CUDA(ctx, cudaMemcpyAsync(&last_flag, ctx->d_commit_flags + n - 1, sizeof(last_flag),
                                           cudaMemcpyDeviceToHost, ctx->stream));
            RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
            added[species] = last_off + last_flag;
            if (ctx->tiles[species].n + added[species] > ctx->capacity) {
                return fail(ctx, RREA_GPU_ERR_CAPACITY, "committed survivors exceed the resident tile capacity");
            }
        }
        for (int species = 0; species < kSpecies; ++species) {
            if (added[species] == 0) continue;
            SpeciesTile& st = ctx->tiles[species];
            RREA_CUDA(ctx, rrea_launch::commit_rank(ctx->d_surv, n, species, ctx->d_commit_flags,
                                                    ctx->d_commit_offsets, ctx->d_commit_scan, ctx->stream));
            const int64_t* ids = nullptr;
            if (ctx->n_instances > 0) {
                RREA_CUDA(ctx, rrea_launch::ensemble_survivor_ids(ctx->d_surv, n, species,
                                                                  static_cast<uint32_t>(ctx->n_instances),
                                                                  ctx->d_inst_next_id, ctx->ens_work, &ids,
                                                                  ctx->stream));
            }
            RREA_CUDA(ctx, rrea_launch::commit_scatter(ctx->d_surv, n, species, ctx->d_commit_offsets, columns(st),
                                                       st.n, ctx->next_id[species], ids, ctx->stream));
            ctx->part_valid[species] = false;
            st.n += added[species];
            ctx->next_id[species] += added[species];
        }
        RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        ctx->n_surv = 0;
    }
    if (committed) {
        for (int species = 0; species < kSpecies; ++species) committed[species] = added[species];
    }
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_compact_resident(rrea_gpu_ctx* ctx, int32_t species, int64_t* n_live)
{
    if (!ctx || species < 0 || species >= kSpecies) return RREA_GPU_ERR_ARGUMENT;
    SpeciesTile& st = ctx->tiles[species];
    int64_t const n = st.n;
    if (n > 0) {
        if (!ctx->spare_ready) {
            size_t const cap = static_cast<size_t>(ctx->capacity);
            bool ok = true;
            for (int f = 0; f < kTileDoubles; ++f) ok = ok && dalloc(&ctx->spare.d[f], cap) == cudaSuccess;
            ok = ok && dalloc(&ctx->spare.id, cap) == cudaSuccess && dalloc(&ctx->spare.cpu, cap) == cudaSuccess;
            if (!ok) {
                cudaGetLastError();
                for (int f = 0; f < kTileDoubles; ++f) {
                    dfree(ctx->spare.d[f]);
                    ctx->spare.d[f] = nullptr;
                }
                dfree(ctx->spare.id);
                dfree(ctx->spare.cpu);
                ctx->spare.id = nullptr;
                ctx->spare.cpu = nullptr;
                return fail(ctx, RREA_GPU_ERR_CUDA, "compaction tile allocation failed");
            }
            ctx->spare_ready = true;
        }
        RREA_CUDA(ctx, rrea_launch::compact_tile(columns(st), n, ctx->d_sec_per_parent, ctx->d_offsets,
                                                 ctx->d_scan_scratch, columns(ctx->spare), ctx->stream));
        int64_t last_off = 0;
        uint32_t last_flag = 0;
        RREA_CUDA(ctx, cudaMemcpyAsync(&last_off, ctx->d_offsets + n - 1, sizeof(last_off), cudaMemcpyDeviceToHost,
                                       ctx->stream));
        RREA_CUDA(ctx, cudaMemcpyAsync(&last_flag, ctx->d_sec_per_parent + n - 1, sizeof(last_flag),
                                       cudaMemcpyDeviceToHost, ctx->stream));
        RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        for (int f = 0; f < kTileDoubles; ++f) std::swap(st.d[f], ctx->spare.d[f]);
        std::swap(st.id, ctx->spare.id);
        std::swap(st.cpu, ctx->spare.cpu);
        st.n = last_off + last_flag;
        ctx->part_valid[species] = false;
    }
    if (n_live) *n_live = st.n;
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_seed_schedule_load(const char* path, const char* case_id, rrea_gpu_seed_schedule** out)
{
    if (!path || !out) return seed_fail(RREA_GPU_ERR_ARGUMENT, "null path or output");
    *out = nullptr;
    auto* s = new (std::nothrow) rrea_gpu_seed_schedule();
    if (!s) return seed_fail(RREA_GPU_ERR_ARGUMENT, "out of host memory");
    try {
        s->s.load(path, case_id ? case_id : "");
    } catch (rrea_host::SeedScheduleError const& e) {
        delete s;
        return seed_fail(e.code, e.what());
    } catch (std::exception const& e) {
        delete s;
        return seed_fail(RREA_GPU_ERR_ARGUMENT, e.what());
    }
    *out = s;
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_seed_schedule_free(rrea_gpu_seed_schedule* schedule)
{
    delete schedule;
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_seed_schedule_size(const rrea_gpu_seed_schedule* schedule, int64_t* n)
{
    if (!schedule || !n) return RREA_GPU_ERR_ARGUMENT;
    *n = static_cast<int64_t>(schedule->s.events().size());
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_seed_schedule_events(const rrea_gpu_seed_schedule* schedule, rrea_gpu_seed_event* out,
                                              int64_t capacity, int64_t* n)
{
    if (!schedule || capacity < 0) return RREA_GPU_ERR_ARGUMENT;
    std::vector<rrea_gpu_seed_event> const& ev = schedule->s.events();
    if (n) *n = static_cast<int64_t>(ev.size());
    if (static_cast<int64_t>(ev.size()) > capacity) return seed_fail(RREA_GPU_ERR_CAPACITY, "event buffer too small");
    if (!ev.empty()) {
        if (!out) return RREA_GPU_ERR_ARGUMENT;
        std::memcpy(out, ev.data(), ev.size() * sizeof(rrea_gpu_seed_event));
    }
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_seed_schedule_validate(const rrea_gpu_seed_schedule* schedule, double e_min, double e_max,
                                                double r_min, double r_max, double z_min, double z_max)
{
    if (!schedule) return RREA_GPU_ERR_ARGUMENT;
    try {
        schedule->s.validate(e_min, e_max, r_min, r_max, z_min, z_max);
    } catch (rrea_host::SeedScheduleError const& e) {
        return seed_fail(e.code, e.what());
    }
    return RREA_GPU_OK;
}

void rrea_gpu_seed_schedule_last_error(char* buf, size_t size)
{
    if (!buf || size == 0) return;
    std::strncpy(buf, g_seed_error.c_str(), size - 1);
    buf[size - 1] = '\0';
}

rrea_gpu_status rrea_gpu_inject_seeds_resident(rrea_gpu_ctx* ctx, rrea_gpu_seed_schedule* schedule, double time_s,
                                               double dt_s, int64_t* injected)
{
    if (!ctx || !schedule) return RREA_GPU_ERR_ARGUMENT;
    if (injected) injected[0] = injected[1] = 0;
    rrea_host::SeedSchedule& sched = schedule->s;
    std::vector<rrea_gpu_seed_event> const& events = sched.events();
    if (!(dt_s > 0.0) || events.empty()) return RREA_GPU_OK;
    // O/RreaCouplingSources.cpp:124-151: stale events are skipped, the window's
    // events injected, the first later event stops the walk
    double const end = time_s + dt_s;
    std::vector<rrea_gpu_seed_event const*> pick[2];
    int64_t c = sched.cursor;
    for (; c < static_cast<int64_t>(events.size()); ++c) {
        rrea_gpu_seed_event const& e = events[static_cast<size_t>(c)];
        int const cls = rrea_host::seed_window_class(e.time_s, time_s, end);
        if (cls < 0) continue;
        if (cls > 0) break;
        pick[e.species_id == rrea_host::kSeedPositron ? 1 : 0].push_back(&e);
    }
    int const tile_of[2] = {RREA_SPECIES_ELECTRON, RREA_SPECIES_POSITRON};
    for (int k = 0; k < 2; ++k) {
        if (ctx->tiles[tile_of[k]].n + static_cast<int64_t>(pick[k].size()) > ctx->capacity) {
            return fail(ctx, RREA_GPU_ERR_CAPACITY, "injected seeds exceed the resident tile capacity");
        }
    }
    for (int k = 0; k < 2; ++k) {
        size_t const m = pick[k].size();
        if (m == 0) continue;
        SpeciesTile& st = ctx->tiles[tile_of[k]];
        // columns as append_rrea_previous_position_attributes builds them
        // (O/RreaCouplingSources.cpp:28-100): captured state = own state
        std::vector<double> col(static_cast<size_t>(kTileDoubles) * m);
        std::vector<int64_t> ids(m);
        for (size_t i = 0; i < m; ++i) {
            rrea_gpu_seed_event const& e = *pick[k][i];
            double u[3];
            rrea_host::normalize_seed_momentum(e.ux, e.uy, e.uz, e.kinetic_energy_eV, u);
            double const r = std::hypot(e.x_m, e.y_m), th = std::atan2(e.y_m, e.x_m);
            double const v[kTileDoubles] = {r, e.z_m, th, u[0], u[1], u[2], e.weight, r, e.z_m, th, u[0], u[1], u[2]};
            for (int f = 0; f < kTileDoubles; ++f) col[static_cast<size_t>(f) * m + i] = v[f];
            ids[i] = ctx->next_id[tile_of[k]] + static_cast<int64_t>(i);
        }
        for (int f = 0; f < kTileDoubles; ++f) {
            RREA_CUDA(ctx, cudaMemcpyAsync(st.d[f] + st.n, col.data() + static_cast<size_t>(f) * m,
                                           m * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
        }
        RREA_CUDA(ctx, cudaMemcpyAsync(st.id + st.n, ids.data(), m * sizeof(int64_t), cudaMemcpyHostToDevice,
                                       ctx->stream));
        RREA_CUDA(ctx, cudaMemsetAsync(st.cpu + st.n, 0, m * sizeof(int32_t), ctx->stream));
        RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        st.n += static_cast<int64_t>(m);
        ctx->next_id[tile_of[k]] += static_cast<int64_t>(m);
        if (injected) injected[k] = static_cast<int64_t>(m);
    }
    sched.cursor = c;
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_thin_cic_groups(rrea_gpu_ctx* ctx, const double* fraction_r, const double* fraction_z,
                                        double* weight, const int64_t* offsets, int64_t n_groups,
                                        const int64_t* max_removals, const uint64_t* keys, int64_t* removed,
                                        int64_t* draws, int32_t* valid, int64_t* capacity)
{
    if (!ctx || n_groups < 0 || (n_groups > 0 && (!fraction_r || !fraction_z || !weight || !offsets ||
                                                  !max_removals || !keys || !removed || !draws || !valid ||
                                                  !capacity))) {
        return RREA_GPU_ERR_ARGUMENT;
    }
    if (n_groups == 0) return RREA_GPU_OK;
    if (offsets[0] != 0) return fail(ctx, RREA_GPU_ERR_ARGUMENT, "group offsets must start at 0");
    for (int64_t g = 0; g < n_groups; ++g) {
        int64_t const size = offsets[g + 1] - offsets[g];
        if (size < 0 || size > rrea_dev::kCicMaxGroup) {
            return fail(ctx, RREA_GPU_ERR_ARGUMENT, "a CIC group holds 0 to 64 particles");
        }
    }
    int64_t const n = offsets[n_groups];
    size_t const bn = static_cast<size_t>(n) * sizeof(double), bg = static_cast<size_t>(n_groups);
    double *d_fr = nullptr, *d_fz = nullptr, *d_w = nullptr;
    int64_t *d_off = nullptr, *d_max = nullptr, *d_rem = nullptr, *d_draw = nullptr, *d_cap = nullptr;
    uint64_t* d_key = nullptr;
    int32_t* d_valid = nullptr;
    bool ok = dalloc(&d_fr, static_cast<size_t>(n) + 1) == cudaSuccess &&
              dalloc(&d_fz, static_cast<size_t>(n) + 1) == cudaSuccess &&
              dalloc(&d_w, static_cast<size_t>(n) + 1) == cudaSuccess && dalloc(&d_off, bg + 1) == cudaSuccess &&
              dalloc(&d_max, bg) == cudaSuccess && dalloc(&d_key, bg) == cudaSuccess &&
              dalloc(&d_rem, bg) == cudaSuccess && dalloc(&d_draw, bg) == cudaSuccess &&
              dalloc(&d_valid, bg) == cudaSuccess && dalloc(&d_cap, bg) == cudaSuccess;
    auto release = [&]() {
        dfree(d_fr); dfree(d_fz); dfree(d_w); dfree(d_off); dfree(d_max); dfree(d_key);
        dfree(d_rem); dfree(d_draw); dfree(d_valid); dfree(d_cap);
    };
    if (!ok) {
        cudaGetLastError();
        release();
        return fail(ctx, RREA_GPU_ERR_CUDA, "thinning scratch allocation failed");
    }
    cudaError_t e = cudaSuccess;
    auto up = [&](void* d, const void* h, size_t bytes) {
        if (e == cudaSuccess && bytes) e = cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, ctx->stream);
    };
    auto down = [&](void* h, const void* d, size_t bytes) {
        if (e == cudaSuccess && bytes) e = cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, ctx->stream);
    };
    up(d_fr, fraction_r, bn);
    up(d_fz, fraction_z, bn);
    up(d_w, weight, bn);
    up(d_off, offsets, (bg + 1) * sizeof(int64_t));
    up(d_max, max_removals, bg * sizeof(int64_t));
    up(d_key, keys, bg * sizeof(uint64_t));
    if (e == cudaSuccess) {
        e = rrea_launch::cic_thin(d_fr, d_fz, d_w, d_off, n_groups, d_max, d_key, d_rem, d_draw, d_valid, d_cap,
                                  ctx->stream);
    }
    down(weight, d_w, bn);
    down(removed, d_rem, bg * sizeof(int64_t));
    down(draws, d_draw, bg * sizeof(int64_t));
    down(valid, d_valid, bg * sizeof(int32_t));
    down(capacity, d_cap, bg * sizeof(int64_t));
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    release();
    if (e != cudaSuccess) return fail(ctx, RREA_GPU_ERR_CUDA, std::string("thinning: ") + cudaGetErrorString(e));
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_resident_count(rrea_gpu_ctx* ctx, int32_t species, int64_t* n)
{
    if (!ctx || !n || species < 0 || species >= kSpecies) return RREA_GPU_ERR_ARGUMENT;
    *n = ctx->tiles[species].n;
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_pending_secondaries(rrea_gpu_ctx* ctx, int64_t* n_pending, int32_t discard)
{
    if (!ctx) return RREA_GPU_ERR_ARGUMENT;
    if (n_pending) *n_pending = ctx->fifo_pending;
    if (discard) ctx->fifo_pending = 0;
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_last_drain_stats(rrea_gpu_ctx* ctx, int64_t* fifo_items, int64_t* survivors)
{
    if (!ctx) return RREA_GPU_ERR_ARGUMENT;
    if (fifo_items) *fifo_items = ctx->last_drain_items;
    if (survivors) *survivors = ctx->n_surv;
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_selftest_math(rrea_gpu_ctx* ctx, int32_t which, const double* x, int64_t n, double* fast,
                                      double* libm)
{
    if (!ctx || n < 0 || (n > 0 && (!x || !fast || !libm)) || which < 0 || which > 1) return RREA_GPU_ERR_ARGUMENT;
    if (!ctx->tables_loaded) return fail(ctx, RREA_GPU_ERR_NOT_READY, "the math tables are part of the loaded arena");
    if (n == 0) return RREA_GPU_OK;
    double* d = nullptr;
    RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    RREA_CUDA(ctx, dalloc(&d, static_cast<size_t>(3 * n)));
    size_t const bytes = static_cast<size_t>(n) * sizeof(double);
    cudaError_t e = cudaMemcpyAsync(d, x, bytes, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = rrea_launch::eval_math(ctx->d_arena, which, d, n, d + n, d + 2 * n, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(fast, d + n, bytes, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(libm, d + 2 * n, bytes, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    dfree(d);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "selftest_math");
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_kernel_launches(uint64_t* count)
{
    if (!count) return RREA_GPU_ERR_ARGUMENT;
    *count = rrea_launch::launches_noted();
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_census_resident(rrea_gpu_ctx* ctx, int32_t species, const double* edges_eV, int32_t n_edges,
                                         const double* thresholds_eV, int32_t n_thresholds, double* out)
{
    constexpr int kMaxEdges = 1025, kMaxThresholds = 16;
    constexpr int kSums = 5 + kMaxThresholds + kMaxEdges - 1;
    if (!ctx || !out || species < 0 || species >= kSpecies) return RREA_GPU_ERR_ARGUMENT;
    if (n_edges < 2 || n_edges > kMaxEdges || !edges_eV || n_thresholds < 0 || n_thresholds > kMaxThresholds
        || (n_thresholds > 0 && !thresholds_eV)) {
        return fail(ctx, RREA_GPU_ERR_ARGUMENT, "census needs 2..1025 edges and at most 16 thresholds");
    }
    for (int k = 0; k < n_edges; ++k) {
        if (!std::isfinite(edges_eV[k]) || (k > 0 && !(edges_eV[k] > edges_eV[k - 1]))) {
            return fail(ctx, RREA_GPU_ERR_ARGUMENT, "census edges must be finite and strictly increasing");
        }
    }
    for (int k = 0; k < n_thresholds; ++k) {
        if (std::isnan(thresholds_eV[k])) return fail(ctx, RREA_GPU_ERR_ARGUMENT, "census threshold is NaN");
    }
    // sums | edges | thresholds | count and max-weight words
    size_t const words = kSums + kMaxEdges + kMaxThresholds + 2;
    if (!ctx->d_census) RREA_CUDA(ctx, dalloc(&ctx->d_census, words));
    double* const sums = ctx->d_census;
    double* const edges = sums + kSums;
    double* const thr = edges + kMaxEdges;
    auto* const words64 = reinterpret_cast<unsigned long long*>(thr + kMaxThresholds);
    int const n_sums = 5 + n_thresholds + n_edges - 1;
    RREA_CUDA(ctx, cudaMemsetAsync(sums, 0, sizeof(double) * n_sums, ctx->stream));
    RREA_CUDA(ctx, cudaMemsetAsync(words64, 0, 2 * sizeof(unsigned long long), ctx->stream));
    RREA_CUDA(ctx, cudaMemcpyAsync(edges, edges_eV, sizeof(double) * n_edges, cudaMemcpyHostToDevice, ctx->stream));
    if (n_thresholds > 0) {
        RREA_CUDA(ctx, cudaMemcpyAsync(thr, thresholds_eV, sizeof(double) * n_thresholds, cudaMemcpyHostToDevice,
                                       ctx->stream));
    }
    SpeciesTile const& st = ctx->tiles[species];
    RREA_CUDA(ctx, rrea_launch::census(st.d[3], st.d[4], st.d[5], st.d[6], st.id, st.n, species == RREA_SPECIES_PHOTON,
                                       edges, n_edges, thr, n_thresholds, sums, words64, words64 + 1,
                                       ctx->num_sms * 8, ctx->stream));
    unsigned long long w64[2] = {0, 0};
    RREA_CUDA(ctx, cudaMemcpyAsync(out + 2, sums, sizeof(double) * n_sums, cudaMemcpyDeviceToHost, ctx->stream));
    RREA_CUDA(ctx, cudaMemcpyAsync(w64, words64, sizeof(w64), cudaMemcpyDeviceToHost, ctx->stream));
    RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    double max_w = 0.0;
    std::memcpy(&max_w, &w64[1], sizeof(max_w));
    out[0] = static_cast<double>(w64[0]);
    out[1] = w64[0] ? max_w : 0.0;
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_deposit_charge_resident(rrea_gpu_ctx* ctx, double* rho)
{
    if (!ctx || !rho) return RREA_GPU_ERR_ARGUMENT;
    rrea_gpu_config const& c = ctx->cfg;
    size_t const cells = static_cast<size_t>(c.nr) * c.nz;
    if (!ctx->d_rho_cells) RREA_CUDA(ctx, dalloc(&ctx->d_rho_cells, cells));
    RREA_CUDA(ctx, cudaMemsetAsync(ctx->d_rho_cells, 0, cells * sizeof(double), ctx->stream));
    double const dr = (c.r_hi - c.r_lo) / c.nr, dz = (c.z_hi - c.z_lo) / c.nz;
    int const species[2] = {RREA_SPECIES_ELECTRON, RREA_SPECIES_POSITRON};
    double const charge[2] = {-1.0, 1.0};
    for (int k = 0; k < 2; ++k) {
        SpeciesTile const& st = ctx->tiles[species[k]];
        RREA_CUDA(ctx, rrea_launch::particle_charge(st.d[0], st.d[1], st.d[6], st.id, st.n, charge[k], c.nr, c.nz,
                                                    c.r_lo, c.z_lo, dr, dz, ctx->d_rho_cells, ctx->num_sms * 8,
                                                    ctx->stream));
    }
    RREA_CUDA(ctx, cudaMemcpyAsync(rho, ctx->d_rho_cells, cells * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_population_thin_resident(rrea_gpu_ctx* ctx, int32_t species, int64_t target, int32_t step,
                                                 uint64_t salt, rrea_gpu_secondary* candidates, int64_t n_candidates,
                                                 int64_t* stats)
{
    if (!ctx || (species != RREA_SPECIES_ELECTRON && species != RREA_SPECIES_POSITRON) || target < 0 ||
        n_candidates < 0 || (n_candidates > 0 && !candidates)) {
        return fail(ctx, RREA_GPU_ERR_ARGUMENT, "population control takes e- or e+, a target >= 0 and a candidate array");
    }
    rrea_gpu_config const& c = ctx->cfg;
    rrea_gpu_secondary* d_cand = ctx->d_surv;
    int64_t n_cand = ctx->n_surv;
    if (candidates) {
        if (n_candidates > ctx->pc_cand_cap) {
            dfree(ctx->d_pc_cand);
            ctx->d_pc_cand = nullptr;
            ctx->pc_cand_cap = 0;
            RREA_CUDA(ctx, dalloc(&ctx->d_pc_cand, static_cast<size_t>(n_candidates)));
            ctx->pc_cand_cap = n_candidates;
        }
        d_cand = ctx->d_pc_cand;
        n_cand = n_candidates;
        if (n_cand > 0) {
            RREA_CUDA(ctx, cudaMemcpyAsync(d_cand, candidates, static_cast<size_t>(n_cand) * sizeof(rrea_gpu_secondary),
                                           cudaMemcpyHostToDevice, ctx->stream));
        }
    }
    SpeciesTile& st = ctx->tiles[species];
    rrea_launch::PopulationInput in{};
    in.r = st.d[0]; in.z = st.d[1]; in.theta = st.d[2]; in.ux = st.d[3]; in.uy = st.d[4]; in.uz = st.d[5];
    in.w = st.d[6];
    in.id = st.id;
    in.cpu = st.cpu;
    in.n_tile = st.n;
    in.cand = d_cand;
    in.n_cand = n_cand;
    in.species = species;
    in.periodic_z = c.periodic_z;
    in.r_lo = c.r_lo;
    in.z_lo = c.z_lo;
    in.z_hi = c.z_hi;
    in.dr = (c.r_hi - c.r_lo) / c.nr;
    in.dz = (c.z_hi - c.z_lo) / c.nz;
    in.target = target;
    in.rng_seed = c.rng_seed;
    in.salt = salt;
    in.step = step;
    rrea_launch::PopulationStats ps{};
    RREA_CUDA(ctx, rrea_launch::population_thin(in, ctx->pop_work, ps, ctx->num_sms * 8, ctx->stream));
    if (stats) {
        int64_t const v[8] = {ps.members, ps.live, ps.candidates, ps.supports, ps.capacity, ps.floor, ps.requested,
                              ps.removed};
        for (int k = 0; k < 8; ++k) stats[k] = v[k];
    }
    if (ps.status != 0) {
        return fail(ctx, static_cast<rrea_gpu_status>(ps.status),
                    ps.status == RREA_GPU_ERR_GEOMETRY
                        ? "population control found a particle outside the supported grid"
                        : "population control plan rejected (invalid support plan or insufficient progress); "
                          "nothing was applied");
    }
    if (candidates && n_cand > 0) {
        RREA_CUDA(ctx, cudaMemcpyAsync(candidates, d_cand, static_cast<size_t>(n_cand) * sizeof(rrea_gpu_secondary),
                                       cudaMemcpyDeviceToHost, ctx->stream));
    }
    RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_population_split_resident(rrea_gpu_ctx* ctx, int32_t species, int64_t target,
                                                  double split_min_weight, int64_t* added)
{
    if (!ctx || (species != RREA_SPECIES_ELECTRON && species != RREA_SPECIES_POSITRON) || target < 0 ||
        !std::isfinite(split_min_weight)) {
        return fail(ctx, RREA_GPU_ERR_ARGUMENT, "split refill takes e- or e+, a target >= 0 and a finite floor");
    }
    if (added) *added = 0;
    int64_t live = 0;
    rrea_gpu_status const s = rrea_gpu_count_live(ctx, species, &live);
    if (s != RREA_GPU_OK) return s;
    // RreaAdaptiveResampleAction (O/RreaRng.H:139-153): split strictly below half the target
    if (!(live > 0 && live < target / 2 && split_min_weight > 0.0)) return RREA_GPU_OK;
    if (ctx->n_instances > 0) return fail(ctx, RREA_GPU_ERR_ARGUMENT, "the split refill has no ensemble form");
    SpeciesTile& st = ctx->tiles[species];
    int64_t n_added = 0;
    RREA_CUDA(ctx, rrea_launch::population_split(columns(st), st.n, split_min_weight, ctx->pop_work,
                                                 ctx->next_id[species], ctx->capacity - st.n, &n_added, ctx->stream));
    if (n_added < 0) return fail(ctx, RREA_GPU_ERR_CAPACITY, "split clones exceed the resident tile capacity");
    RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    st.n += n_added;
    ctx->next_id[species] += n_added;
    if (added) *added = n_added;
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_population_merge_resident(rrea_gpu_ctx* ctx, int32_t species, int64_t target, int32_t step,
                                                  int64_t* stats)
{
    if (!ctx || species < 0 || species >= kSpecies || target < 0) {
        return fail(ctx, RREA_GPU_ERR_ARGUMENT, "merge takes a species and a target >= 0");
    }
    if (ctx->n_instances > 0) return fail(ctx, RREA_GPU_ERR_ARGUMENT, "the merge has no ensemble form");
    rrea_gpu_config const& c = ctx->cfg;
    SpeciesTile& st = ctx->tiles[species];
    rrea_launch::MergeInput in{};
    in.r = st.d[0];
    in.z = st.d[1];
    in.ux = st.d[3];
    in.uy = st.d[4];
    in.uz = st.d[5];
    in.w = st.d[6];
    in.id = st.id;
    in.cpu = st.cpu;
    in.n_tile = st.n;
    in.species = species;
    in.nr = c.nr;
    in.nz = c.nz;
    in.r_lo = c.r_lo;
    in.z_lo = c.z_lo;
    in.dr = (c.r_hi - c.r_lo) / c.nr;
    in.dz = (c.z_hi - c.z_lo) / c.nz;
    in.target = target;
    in.rng_seed = c.rng_seed;
    in.step = step;
    rrea_launch::MergeStats ms{};
    RREA_CUDA(ctx, rrea_launch::population_merge(in, ctx->pop_work, ms, ctx->stream));
    if (ms.status != 0) return fail(ctx, static_cast<rrea_gpu_status>(ms.status), "merge plan exceeds its index range");
    if (stats) {
        int64_t const v[5] = {ms.live, ms.groups, ms.pairs, ms.requested, ms.merged};
        std::copy(v, v + 5, stats);
    }
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_count_live(rrea_gpu_ctx* ctx, int32_t species, int64_t* live)
{
    if (!ctx || !live || species < 0 || species >= kSpecies) return RREA_GPU_ERR_ARGUMENT;
    SpeciesTile const& st = ctx->tiles[species];
    RREA_CUDA(ctx, cudaMemsetAsync(ctx->d_transported, 0, sizeof(unsigned long long), ctx->stream));
    RREA_CUDA(ctx, rrea_launch::count_live(st.id, st.n, ctx->d_transported, ctx->num_sms * 4, ctx->stream));
    unsigned long long count = 0;
    RREA_CUDA(ctx, cudaMemcpyAsync(&count, ctx->d_transported, sizeof(count), cudaMemcpyDeviceToHost, ctx->stream));
    RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    *live = static_cast<int64_t>(count);
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_population_projection(uint64_t current, uint64_t removals, uint64_t insertions,
                                               uint64_t ceiling, int32_t reject_equality, uint64_t* projected)
{
    // RreaStrictPopulationProjection (O/RreaParticleInteraction.H:1257-1275)
    uint64_t p = 0;
    bool fits;
    if (removals > current) {
        fits = false;
    } else {
        uint64_t const survivors = current - removals;
        if (insertions > UINT64_MAX - survivors) {
            p = UINT64_MAX;
            fits = false;
        } else {
            p = survivors + insertions;
            fits = reject_equality ? p < ceiling : p <= ceiling;
        }
    }
    if (projected) *projected = p;
    return fits ? RREA_GPU_OK : RREA_GPU_ERR_CAPACITY;
}

rrea_gpu_status rrea_gpu_download_diagnostics(rrea_gpu_ctx* ctx, int64_t n, uint64_t* subcycles, uint64_t* events,
                                              int32_t* disposition)
{
    if (!ctx || n < 0 || n > ctx->capacity) return RREA_GPU_ERR_ARGUMENT;
    if (!ctx->diagnostics) return fail(ctx, RREA_GPU_ERR_NOT_READY, "diagnostics are disabled");
    if (n == 0) return RREA_GPU_OK;
    if (subcycles) {
        RREA_CUDA(ctx, cudaMemcpyAsync(subcycles, ctx->d_diag_sub, n * sizeof(uint64_t), cudaMemcpyDeviceToHost,
                                       ctx->stream));
    }
    if (events) {
        RREA_CUDA(ctx, cudaMemcpyAsync(events, ctx->d_diag_ev, n * sizeof(uint64_t), cudaMemcpyDeviceToHost,
                                       ctx->stream));
    }
    if (disposition) {
        RREA_CUDA(ctx, cudaMemcpyAsync(disposition, ctx->d_diag_disp, n * sizeof(int32_t), cudaMemcpyDeviceToHost,
                                       ctx->stream));
    }
    RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RREA_GPU_OK;
}

void rrea_gpu_last_error(const rrea_gpu_ctx* ctx, char* buf, size_t size)
{
    if (!buf || size == 0) return;
    std::string const& m = ctx ? ctx->last_error : std::string("no context");
    std::strncpy(buf, m.c_str(), size - 1);
    buf[size - 1] = '\0';
}

// ---- resident engine mode (inputs already in HBM) --------------------------

rrea_gpu_status rrea_gpu_stage_electrons(rrea_gpu_ctx* ctx, const rrea_gpu_tile* tile)
{
    return stage_species(ctx, RREA_SPECIES_ELECTRON, tile);
}

rrea_gpu_status rrea_gpu_step_electrons_resident(rrea_gpu_ctx* ctx, int32_t step, double dt_s, int64_t* n_secondaries)
{
    return step_resident(ctx, RREA_SPECIES_ELECTRON, step, dt_s, n_secondaries);
}

rrea_gpu_status rrea_gpu_fetch_electrons(rrea_gpu_ctx* ctx, rrea_gpu_tile* tile)
{
    return fetch_species(ctx, RREA_SPECIES_ELECTRON, tile);
}

rrea_gpu_status rrea_gpu_stage_positrons(rrea_gpu_ctx* ctx, const rrea_gpu_tile* tile)
{
    return stage_species(ctx, RREA_SPECIES_POSITRON, tile);
}

rrea_gpu_status rrea_gpu_step_positrons_resident(rrea_gpu_ctx* ctx, int32_t step, double dt_s, int64_t* n_secondaries)
{
    return step_resident(ctx, RREA_SPECIES_POSITRON, step, dt_s, n_secondaries);
}

rrea_gpu_status rrea_gpu_fetch_positrons(rrea_gpu_ctx* ctx, rrea_gpu_tile* tile)
{
    return fetch_species(ctx, RREA_SPECIES_POSITRON, tile);
}

rrea_gpu_status rrea_gpu_stage_photons(rrea_gpu_ctx* ctx, const rrea_gpu_tile* tile)
{
    return stage_species(ctx, RREA_SPECIES_PHOTON, tile);
}

rrea_gpu_status rrea_gpu_step_photons_resident(rrea_gpu_ctx* ctx, int32_t step, double dt_s, int64_t* n_secondaries)
{
    return step_resident(ctx, RREA_SPECIES_PHOTON, step, dt_s, n_secondaries);
}

rrea_gpu_status rrea_gpu_fetch_photons(rrea_gpu_ctx* ctx, rrea_gpu_tile* tile)
{
    return fetch_species(ctx, RREA_SPECIES_PHOTON, tile);
}

rrea_gpu_status rrea_gpu_set_launch(rrea_gpu_ctx* ctx, int32_t threads_per_block, int32_t blocks_per_sm,
                                    int32_t diagnostics)
{
    if (!ctx || threads_per_block < 32 || threads_per_block > 128 || (threads_per_block % 32) != 0 || blocks_per_sm < 1
        || blocks_per_sm > 64) {
        return RREA_GPU_ERR_ARGUMENT;
    }
    ctx->launch_threads = threads_per_block;
    ctx->launch_blocks_per_sm = blocks_per_sm;
    ctx->diagnostics = diagnostics != 0;
    // Register budget of the electron kernel follows the requested
    // residency (16 resident 128-thread blocks: 32 registers).
    int const resident = blocks_per_sm * threads_per_block / 128;
    ctx->launch_min_blocks = resident >= 16 ? 16 : resident >= 12 ? 12 : resident >= 8 ? 8 : resident >= 4 ? 4 : 2;
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_set_schedule(rrea_gpu_ctx* ctx, int32_t cost_order)
{
    if (!ctx) return RREA_GPU_ERR_ARGUMENT;
    ctx->schedule_order = cost_order != 0;
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_last_step_stats(rrea_gpu_ctx* ctx, int64_t* transported, int64_t* secondaries,
                                         double* kernel_ms)
{
    if (!ctx) return RREA_GPU_ERR_ARGUMENT;
    if (transported) *transported = ctx->last_transported;
    if (secondaries) *secondaries = ctx->last_secondaries;
    if (kernel_ms) *kernel_ms = static_cast<double>(ctx->last_kernel_ms);
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_stream(rrea_gpu_ctx* ctx, void** stream)
{
    if (!ctx || !stream) return RREA_GPU_ERR_ARGUMENT;
    *stream = ctx->stream;
    return RREA_GPU_OK;
}

}  // extern "C"

// ===========================================================================
// Low-energy carrier fluid (rrea_fluid.cu)
// ===========================================================================
namespace {

rrea_gpu_status fluid_ready(rrea_gpu_ctx* ctx)
{
    if (!ctx) return RREA_GPU_ERR_ARGUMENT;
    if (!ctx->fluid) return fail(ctx, RREA_GPU_ERR_NOT_READY, "the carrier fluid is not configured");
    return RREA_GPU_OK;
}

rrea_gpu_status fluid_checked(rrea_gpu_ctx* ctx, bool ok)
{
    return ok ? RREA_GPU_OK : fail(ctx, RREA_GPU_ERR_INVALID_STATE, rrea_launch::fluid_error(*ctx->fluid));
}

rrea_gpu_status fluid_copy(rrea_gpu_ctx* ctx, int field, const double* host, int64_t count)
{
    if (!host) return RREA_GPU_OK;
    RREA_CUDA(ctx, cudaMemcpyAsync(rrea_launch::fluid_field(*ctx->fluid, field), host, sizeof(double) * count,
                                   cudaMemcpyHostToDevice, ctx->stream));
    return RREA_GPU_OK;
}

rrea_gpu_status fluid_fetch(rrea_gpu_ctx* ctx, int field, double* host, int64_t count)
{
    if (!host) return RREA_GPU_OK;
    RREA_CUDA(ctx, cudaMemcpyAsync(host, rrea_launch::fluid_field(*ctx->fluid, field), sizeof(double) * count,
                                   cudaMemcpyDeviceToHost, ctx->stream));
    return RREA_GPU_OK;
}

}  // namespace

extern "C" {

void rrea_gpu_default_fluid_config(rrea_gpu_fluid_config* c)
{
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    // LowEnergyFluidConfig (I/LowEnergyFluidState.H:80-124)
    c->electron_mobility_m2_per_vs = 0.1;
    c->positive_ion_mobility_m2_per_vs = 2.0e-4;
    c->negative_ion_mobility_m2_per_vs = 2.0e-4;
    c->ion_drift_cfl = 0.5;
    c->transport_density_ratio = 1.0;
    c->attachment_frequency_s = 2.0e6;
    c->electron_drift_enable = 1;
    // RreaAmrexAdvanceConfig (I/RreaAmrexAdvance.H:51-58)
    c->material_min_substeps = 2;
    c->material_max_substeps = 64;
    c->material_conduction_target = 0.08;
    c->material_conduction_guard = 0.1;
    c->material_diffusion_target = 0.8;
    c->material_diffusion_guard = 1.0;
    c->material_reaction_target = 0.08;
    c->material_reaction_guard = 0.1;
}

rrea_gpu_status rrea_gpu_fluid_configure(rrea_gpu_ctx* ctx, const rrea_gpu_fluid_config* cfg)
{
    if (!ctx || !cfg) return RREA_GPU_ERR_ARGUMENT;
    if (!(cfg->material_min_substeps >= 1) || !(cfg->material_max_substeps >= cfg->material_min_substeps)
        || !(cfg->material_conduction_target > 0.0) || !(cfg->material_diffusion_target > 0.0)
        || !(cfg->material_reaction_target > 0.0)) {
        return fail(ctx, RREA_GPU_ERR_ARGUMENT, "invalid material substep controls");
    }
    if (!ctx->fluid) {
        rrea_gpu_config const& c = ctx->cfg;
        rrea_launch::FluidGrid const g{c.nr, c.nz, c.r_lo, c.z_lo, (c.r_hi - c.r_lo) / c.nr, (c.z_hi - c.z_lo) / c.nz,
                                       c.periodic_z};
        RREA_CUDA(ctx, rrea_launch::fluid_create(g, std::max(1, ctx->num_sms * 4), ctx->fluid));
    }
    rrea_gpu_fluid_config const previous = rrea_launch::fluid_config(*ctx->fluid);
    rrea_launch::fluid_set_config(*ctx->fluid, *cfg);
    if (!rrea_launch::fluid_validate(*ctx->fluid, true)) {
        std::string const why = rrea_launch::fluid_error(*ctx->fluid);
        rrea_launch::fluid_set_config(*ctx->fluid, previous);
        return fail(ctx, RREA_GPU_ERR_ARGUMENT, why);
    }
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_fluid_load_closure(rrea_gpu_ctx* ctx, const char* csv_path)
{
    if (rrea_gpu_status const s = fluid_ready(ctx)) return s;
    if (!csv_path) return fail(ctx, RREA_GPU_ERR_ARGUMENT, "no closure table path");
    try {
        rrea_host::ClosureTable const t = rrea_host::load_closure_table(csv_path);
        std::vector<double> cols;
        for (auto const* v : {&t.en_td, &t.log_en_td, &t.k0, &t.log_k0, &t.nu2, &t.nu3, &t.log_nu3, &t.dl, &t.log_dl,
                              &t.dt, &t.log_dt}) {
            cols.insert(cols.end(), v->begin(), v->end());
        }
        RREA_CUDA(ctx, rrea_launch::fluid_load_closure(*ctx->fluid, cols, static_cast<int>(t.size())));
    } catch (std::exception const& e) {
        return fail(ctx, RREA_GPU_ERR_TABLES, e.what());
    }
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_fluid_set_state(rrea_gpu_ctx* ctx, const double* n_pos, const double* n_neg, const double* n_e,
                                         const double* rho_fluid)
{
    if (rrea_gpu_status const s = fluid_ready(ctx)) return s;
    int64_t const n = rrea_launch::fluid_cells(*ctx->fluid);
    for (auto [f, p] : {std::pair{1, n_pos}, {2, n_neg}, {0, n_e}, {3, rho_fluid}}) {
        if (rrea_gpu_status const s = fluid_copy(ctx, f, p, n)) return s;
    }
    RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_fluid_get_state(rrea_gpu_ctx* ctx, double* n_pos, double* n_neg, double* n_e,
                                         double* rho_fluid, double* sigma, double* tau_m)
{
    if (rrea_gpu_status const s = fluid_ready(ctx)) return s;
    int64_t const n = rrea_launch::fluid_cells(*ctx->fluid);
    for (auto [f, p] : {std::pair{1, n_pos}, {2, n_neg}, {0, n_e}, {3, rho_fluid}, {4, sigma}, {5, tau_m}}) {
        if (rrea_gpu_status const s = fluid_fetch(ctx, f, p, n)) return s;
    }
    RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_fluid_set_source_rates(rrea_gpu_ctx* ctx, const double* s_e, const double* s_pos,
                                                const double* s_neg)
{
    if (rrea_gpu_status const s = fluid_ready(ctx)) return s;
    int64_t const n = rrea_launch::fluid_cells(*ctx->fluid);
    for (auto [f, p] : {std::pair{6, s_e}, {7, s_pos}, {8, s_neg}}) {
        if (rrea_gpu_status const s = fluid_copy(ctx, f, p, n)) return s;
    }
    RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_fluid_get_source_rates(rrea_gpu_ctx* ctx, double* s_e, double* s_pos, double* s_neg)
{
    if (rrea_gpu_status const s = fluid_ready(ctx)) return s;
    int64_t const n = rrea_launch::fluid_cells(*ctx->fluid);
    for (auto [f, p] : {std::pair{6, s_e}, {7, s_pos}, {8, s_neg}}) {
        if (rrea_gpu_status const s = fluid_fetch(ctx, f, p, n)) return s;
    }
    RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_fluid_set_density_ratio(rrea_gpu_ctx* ctx, const double* chi)
{
    if (rrea_gpu_status const s = fluid_ready(ctx)) return s;
    int64_t const n = rrea_launch::fluid_cells(*ctx->fluid);
    if (chi) {
        for (int64_t k = 0; k < n; ++k) {
            if (!std::isfinite(chi[k]) || !(chi[k] > 0.0)) {
                return fail(ctx, RREA_GPU_ERR_ARGUMENT, "density ratios must be finite and positive");
            }
        }
        if (rrea_gpu_status const s = fluid_copy(ctx, 9, chi, n)) return s;
        RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    rrea_launch::fluid_bind_chi(*ctx->fluid, chi != nullptr);
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_fluid_set_closure_fields(rrea_gpu_ctx* ctx, const double* mu_e, const double* nu_att,
                                                  const double* diffusion3)
{
    if (rrea_gpu_status const s = fluid_ready(ctx)) return s;
    int64_t const n = rrea_launch::fluid_cells(*ctx->fluid);
    for (auto [f, p, c] : {std::tuple{10, mu_e, n}, {11, nu_att, n}, {12, diffusion3, 3 * n}}) {
        if (rrea_gpu_status const s = fluid_copy(ctx, f, p, c)) return s;
    }
    RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_fluid_get_closure_fields(rrea_gpu_ctx* ctx, double* mu_e, double* nu_att, double* diffusion3)
{
    if (rrea_gpu_status const s = fluid_ready(ctx)) return s;
    int64_t const n = rrea_launch::fluid_cells(*ctx->fluid);
    for (auto [f, p, c] : {std::tuple{10, mu_e, n}, {11, nu_att, n}, {12, diffusion3, 3 * n}}) {
        if (rrea_gpu_status const s = fluid_fetch(ctx, f, p, c)) return s;
    }
    RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_fluid_take_sources(rrea_gpu_ctx* ctx, double dt_s)
{
    if (rrea_gpu_status const s = fluid_ready(ctx)) return s;
    if (!(dt_s > 0.0) || !std::isfinite(dt_s)) return fail(ctx, RREA_GPU_ERR_ARGUMENT, "source normalisation needs dt > 0");
    RREA_CUDA(ctx, rrea_launch::fluid_take_sources(*ctx->fluid, ctx->d_cells, dt_s, ctx->stream));
    RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_fluid_react(rrea_gpu_ctx* ctx, double dt_s, int32_t clear_sources, double* residual)
{
    if (rrea_gpu_status const s = fluid_ready(ctx)) return s;
    if (!std::isfinite(dt_s) || dt_s < 0.0) return fail(ctx, RREA_GPU_ERR_ARGUMENT, "the fluid needs dt >= 0");
    if (!rrea_launch::fluid_validate(*ctx->fluid, false)) return fluid_checked(ctx, false);
    double r = 0.0;
    bool ok = false;
    RREA_CUDA(ctx, rrea_launch::fluid_react(*ctx->fluid, dt_s, clear_sources != 0, r, ok, ctx->stream));
    if (residual) *residual = r;
    return fluid_checked(ctx, ok);
}

rrea_gpu_status rrea_gpu_fluid_max_reaction_frequency(rrea_gpu_ctx* ctx, double* out)
{
    if (rrea_gpu_status const s = fluid_ready(ctx)) return s;
    if (!out) return RREA_GPU_ERR_ARGUMENT;
    RREA_CUDA(ctx, rrea_launch::fluid_max_reaction_frequency(*ctx->fluid, *out, ctx->stream));
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_fluid_conductivity(rrea_gpu_ctx* ctx)
{
    if (rrea_gpu_status const s = fluid_ready(ctx)) return s;
    RREA_CUDA(ctx, rrea_launch::fluid_conductivity(*ctx->fluid, ctx->stream));
    RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_fluid_charge_density(rrea_gpu_ctx* ctx)
{
    if (rrea_gpu_status const s = fluid_ready(ctx)) return s;
    RREA_CUDA(ctx, rrea_launch::fluid_charge_density(*ctx->fluid, ctx->stream));
    RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_fluid_evaluate_closure(rrea_gpu_ctx* ctx, const double* er_cell, const double* ez_cell,
                                                double* diag)
{
    if (rrea_gpu_status const s = fluid_ready(ctx)) return s;
    if (!rrea_launch::fluid_has_closure(*ctx->fluid)) return fail(ctx, RREA_GPU_ERR_NOT_READY, "no closure table loaded");
    if ((er_cell == nullptr) != (ez_cell == nullptr)) return fail(ctx, RREA_GPU_ERR_ARGUMENT, "give both cell fields or neither");
    int64_t const n = rrea_launch::fluid_cells(*ctx->fluid);
    const double* er = ctx->d_cell_er;
    const double* ez = ctx->d_cell_ez;
    if (er_cell) {
        // the face-current buffers hold the host cell fields for this call
        double* scratch_r = rrea_launch::fluid_field(*ctx->fluid, 13);
        double* scratch_z = rrea_launch::fluid_field(*ctx->fluid, 14);
        RREA_CUDA(ctx, cudaMemcpyAsync(scratch_r, er_cell, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
        RREA_CUDA(ctx, cudaMemcpyAsync(scratch_z, ez_cell, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
        er = scratch_r;
        ez = scratch_z;
    } else if (!ctx->field_set) {
        return fail(ctx, RREA_GPU_ERR_NOT_READY, "no field has been set");
    }
    double d[8];
    bool ok = false;
    RREA_CUDA(ctx, rrea_launch::fluid_closure(*ctx->fluid, er, ez, d, ok, ctx->stream));
    if (diag) std::memcpy(diag, d, sizeof(d));
    return fluid_checked(ctx, ok);
}

rrea_gpu_status rrea_gpu_fluid_transport(rrea_gpu_ctx* ctx, double dt_s, const double* efr, const double* efz,
                                         double* flux_r, double* flux_z, double* diag)
{
    if (rrea_gpu_status const s = fluid_ready(ctx)) return s;
    if (!std::isfinite(dt_s) || dt_s <= 0.0) {
        return fail(ctx, RREA_GPU_ERR_ARGUMENT, "explicit carrier transport requires finite, positive dt");
    }
    if ((efr == nullptr) != (efz == nullptr)) return fail(ctx, RREA_GPU_ERR_ARGUMENT, "give both face fields or neither");
    if (!rrea_launch::fluid_validate(*ctx->fluid, true)) return fluid_checked(ctx, false);
    rrea_gpu_config const& c = ctx->cfg;
    int64_t const nfr = static_cast<int64_t>(c.nr + 1) * c.nz, nfz = static_cast<int64_t>(c.nr) * (c.nz + 1);
    const double *er = ctx->d_er, *ez = ctx->d_ez, *er_add = ctx->d_amb_er, *ez_add = ctx->d_amb_ez;
    if (efr) {
        double* scratch_r = rrea_launch::fluid_field(*ctx->fluid, 13);
        double* scratch_z = rrea_launch::fluid_field(*ctx->fluid, 14);
        RREA_CUDA(ctx, cudaMemcpyAsync(scratch_r, efr, sizeof(double) * nfr, cudaMemcpyHostToDevice, ctx->stream));
        RREA_CUDA(ctx, cudaMemcpyAsync(scratch_z, efz, sizeof(double) * nfz, cudaMemcpyHostToDevice, ctx->stream));
        er = scratch_r;
        ez = scratch_z;
        er_add = ez_add = nullptr;
    } else if (!ctx->field_set) {
        return fail(ctx, RREA_GPU_ERR_NOT_READY, "no field has been set");
    }
    double d[14];
    bool ok = false;
    RREA_CUDA(ctx, rrea_launch::fluid_transport(*ctx->fluid, dt_s, er, er_add, ez, ez_add, d, ok, ctx->stream));
    if (flux_r) {
        RREA_CUDA(ctx, cudaMemcpyAsync(flux_r, rrea_launch::fluid_flux(*ctx->fluid, 0), sizeof(double) * 3 * nfr,
                                       cudaMemcpyDeviceToHost, ctx->stream));
    }
    if (flux_z) {
        RREA_CUDA(ctx, cudaMemcpyAsync(flux_z, rrea_launch::fluid_flux(*ctx->fluid, 1), sizeof(double) * 3 * nfz,
                                       cudaMemcpyDeviceToHost, ctx->stream));
    }
    RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (diag) std::memcpy(diag, d, sizeof(d));
    return fluid_checked(ctx, ok);
}

rrea_gpu_status rrea_gpu_fluid_reductions(rrea_gpu_ctx* ctx, double dt_s, double* out16)
{
    if (rrea_gpu_status const s = fluid_ready(ctx)) return s;
    if (!out16 || !(dt_s > 0.0) || !std::isfinite(dt_s)) return RREA_GPU_ERR_ARGUMENT;
    double v[16];
    RREA_CUDA(ctx, rrea_launch::fluid_reductions(*ctx->fluid, ctx->d_cells, dt_s, v, ctx->stream));
    std::memcpy(out16, v, sizeof(v));
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_advance_field_coupled(rrea_gpu_ctx* ctx, double dt_s, double* diag)
{
    if (rrea_gpu_status const s = fluid_ready(ctx)) return s;
    double* jr = nullptr;
    double* jz = nullptr;
    if (rrea_gpu_status const s = rrea_gpu_current_device(ctx, &jr, &jz)) return s;
    return rrea_gpu_advance_field_coupled_from_current(ctx, dt_s, diag);
}

rrea_gpu_status rrea_gpu_sources_device(rrea_gpu_ctx* ctx, double** cells5)
{
    if (!ctx || !cells5) return RREA_GPU_ERR_ARGUMENT;
    *cells5 = ctx->d_cells;
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_advance_field_coupled_from_current(rrea_gpu_ctx* ctx, double dt_s, double* diag)
{
    if (rrea_gpu_status const s = fluid_ready(ctx)) return s;
    if (!ctx->field_set) return fail(ctx, RREA_GPU_ERR_NOT_READY, "no field has been set");
    rrea_gpu_config const& c = ctx->cfg;
    if (c.periodic_z || !ctx->netchord) {
        return fail(ctx, RREA_GPU_ERR_ARGUMENT, "the coupled field step needs a non-periodic z");
    }
    double const dr = (c.r_hi - c.r_lo) / c.nr, dz = (c.z_hi - c.z_lo) / c.nz;
    if (!std::isfinite(dt_s) || !(dt_s > 0.0)) return fail(ctx, RREA_GPU_ERR_ARGUMENT, "the field step needs dt > 0");
    double const cfl = 299792458.0 * dt_s * std::sqrt(1.0 / (dr * dr) + 1.0 / (dz * dz));
    if (!std::isfinite(cfl) || !(cfl < 1.0)) {
        return fail(ctx, RREA_GPU_ERR_ARGUMENT, "Maxwell TM violates the two-dimensional Yee CFL condition");
    }
    if (!rrea_launch::fluid_validate(*ctx->fluid, true)) return fluid_checked(ctx, false);
    rrea_gpu_fluid_config const& fc = rrea_launch::fluid_config(*ctx->fluid);
    bool const tables = (fc.electron_drift_enable && fc.electron_mobility_model == RREA_GPU_MOBILITY_EN_TABLE_FLUX)
        || fc.attachment_model == RREA_GPU_ATTACHMENT_EN_TABLE;
    if (tables && !rrea_launch::fluid_has_closure(*ctx->fluid)) {
        return fail(ctx, RREA_GPU_ERR_NOT_READY, "en_table fluid models require a loaded electron closure");
    }
    // the step's kinetic face current as rrea_gpu_current_device left it
    // (summed across ranks by the caller of a sharded step)
    rrea_launch::CoupledField const f{c.nr,          c.nz,          dr,           dz,
                                      ctx->d_er,     ctx->d_ez,     ctx->d_bt,    ctx->d_amb_er,
                                      ctx->d_amb_ez, ctx->d_cell_er, ctx->d_cell_ez, ctx->d_jr_phys,
                                      ctx->d_jz_phys};
    double d[8];
    bool ok = false;
    RREA_CUDA(ctx, rrea_launch::fluid_coupled_step(*ctx->fluid, f, dt_s, d, ok, ctx->stream));
    RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->has_b = true;
    if (diag) std::memcpy(diag, d, sizeof(d));
    return fluid_checked(ctx, ok);
}

}  // extern "C"

// ===========================================================================
// Batched ensemble (rrea_ensemble.cu)
// ===========================================================================
extern "C" {

rrea_gpu_status rrea_gpu_ensemble_configure(rrea_gpu_ctx* ctx, int32_t n_instances, const double* ambient_ez)
{
    if (!ctx || n_instances < 1 || n_instances > (1 << 16) || !ambient_ez) {
        return fail(ctx, RREA_GPU_ERR_ARGUMENT, "an ensemble needs 1..65536 instances and their fields");
    }
    if (ctx->n_instances > 0) return fail(ctx, RREA_GPU_ERR_ARGUMENT, "the ensemble is already configured");
    for (int32_t k = 0; k < n_instances; ++k) {
        if (!std::isfinite(ambient_ez[k])) return fail(ctx, RREA_GPU_ERR_ARGUMENT, "instance fields must be finite");
    }
    rrea_gpu_config const& c = ctx->cfg;
    size_t const cells = static_cast<size_t>(c.nr) * c.nz;
    std::vector<double> host(2 * cells * static_cast<size_t>(n_instances), 0.0);
    // a uniform ambient E_z: every cell average is the value itself
    for (int32_t k = 0; k < n_instances; ++k) {
        std::fill(host.begin() + static_cast<std::ptrdiff_t>(cells * (n_instances + k)),
                  host.begin() + static_cast<std::ptrdiff_t>(cells * (n_instances + k + 1)), ambient_ez[k]);
    }
    RREA_CUDA(ctx, dalloc(&ctx->d_inst_cells, host.size()));
    RREA_CUDA(ctx, dalloc(&ctx->d_inst_next_id, 3 * static_cast<size_t>(n_instances)));
    RREA_CUDA(ctx, cudaMemcpy(ctx->d_inst_cells, host.data(), host.size() * sizeof(double), cudaMemcpyHostToDevice));
    std::vector<int64_t> ones(3 * static_cast<size_t>(n_instances), 1);
    RREA_CUDA(ctx, cudaMemcpy(ctx->d_inst_next_id, ones.data(), ones.size() * sizeof(int64_t), cudaMemcpyHostToDevice));
    ctx->n_instances = n_instances;
    ctx->netchord = false;   // no feedback: neither current nor cell sources
    ctx->field_set = true;
    for (auto& v : ctx->part_valid) v = false;
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_ensemble_partition(rrea_gpu_ctx* ctx, int32_t species, int64_t* counts)
{
    if (!ctx || species < 0 || species >= kSpecies) return RREA_GPU_ERR_ARGUMENT;
    if (ctx->n_instances < 1) return fail(ctx, RREA_GPU_ERR_NOT_READY, "no ensemble is configured");
    if (!ctx->spare_ready) {
        // the compaction's spare tile receives the partitioned copy
        int64_t live = 0;
        rrea_gpu_status const s = rrea_gpu_compact_resident(ctx, species, &live);
        if (s != RREA_GPU_OK) return s;
        if (!ctx->spare_ready) {
            size_t const cap = static_cast<size_t>(ctx->capacity);
            bool ok = true;
            for (int f = 0; f < kTileDoubles; ++f) ok = ok && dalloc(&ctx->spare.d[f], cap) == cudaSuccess;
            ok = ok && dalloc(&ctx->spare.id, cap) == cudaSuccess && dalloc(&ctx->spare.cpu, cap) == cudaSuccess;
            if (!ok) return fail(ctx, RREA_GPU_ERR_CUDA, "partition tile allocation failed");
            ctx->spare_ready = true;
        }
    }
    SpeciesTile& st = ctx->tiles[species];
    std::vector<int64_t> n_k(static_cast<size_t>(ctx->n_instances), 0);
    RREA_CUDA(ctx, rrea_launch::ensemble_partition(columns(st), st.n, static_cast<uint32_t>(ctx->n_instances),
                                                   columns(ctx->spare), ctx->ens_work, n_k.data(), ctx->stream));
    int64_t total = 0;
    for (int64_t v : n_k) total += v;
    if (total != st.n) return fail(ctx, RREA_GPU_ERR_INVALID_STATE, "a particle's cpu ordinal is not an instance");
    if (st.n > 0) {
        for (int f = 0; f < kTileDoubles; ++f) std::swap(st.d[f], ctx->spare.d[f]);
        std::swap(st.id, ctx->spare.id);
        std::swap(st.cpu, ctx->spare.cpu);
    }
    auto& off = ctx->inst_offsets[species];
    off.assign(static_cast<size_t>(ctx->n_instances) + 1, 0);
    for (int32_t k = 0; k < ctx->n_instances; ++k) off[k + 1] = off[k] + n_k[static_cast<size_t>(k)];
    ctx->part_valid[species] = true;
    if (counts) std::copy(n_k.begin(), n_k.end(), counts);
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_ensemble_retire(rrea_gpu_ctx* ctx, int32_t instance)
{
    if (!ctx || instance < 0 || instance >= ctx->n_instances) return RREA_GPU_ERR_ARGUMENT;
    for (int species = 0; species < kSpecies; ++species) {
        SpeciesTile& st = ctx->tiles[species];
        RREA_CUDA(ctx, rrea_launch::ensemble_retire(st.id, st.cpu, st.n, instance, ctx->stream));
    }
    RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RREA_GPU_OK;
}

namespace {

rrea_gpu_status instance_slice(rrea_gpu_ctx* ctx, int32_t species, int32_t instance, int64_t& begin, int64_t& n)
{
    if (!ctx || species < 0 || species >= kSpecies || instance < 0 || instance >= ctx->n_instances) {
        return RREA_GPU_ERR_ARGUMENT;
    }
    if (!ctx->part_valid[species]) {
        return fail(ctx, RREA_GPU_ERR_NOT_READY, "the tile changed since its last ensemble partition");
    }
    begin = ctx->inst_offsets[species][static_cast<size_t>(instance)];
    n = ctx->inst_offsets[species][static_cast<size_t>(instance) + 1] - begin;
    return RREA_GPU_OK;
}

}  // namespace

rrea_gpu_status rrea_gpu_ensemble_census(rrea_gpu_ctx* ctx, int32_t species, int32_t instance, const double* edges_eV,
                                         int32_t n_edges, const double* thresholds_eV, int32_t n_thresholds,
                                         double* out)
{
    int64_t begin = 0, n = 0;
    if (rrea_gpu_status const s = instance_slice(ctx, species, instance, begin, n)) return s;
    // the census of the instance's slice is the census of a tile that holds it alone
    SpeciesTile& st = ctx->tiles[species];
    SpeciesTile const whole = st;
    for (int f = 0; f < kTileDoubles; ++f) st.d[f] += begin;
    st.id += begin;
    st.cpu += begin;
    st.n = n;
    rrea_gpu_status const s =
        rrea_gpu_census_resident(ctx, species, edges_eV, n_edges, thresholds_eV, n_thresholds, out);
    st = whole;
    return s;
}

rrea_gpu_status rrea_gpu_ensemble_population_thin(rrea_gpu_ctx* ctx, int32_t species, int32_t instance,
                                                  int64_t target, int32_t step, uint64_t salt, int64_t* stats)
{
    int64_t begin = 0, n = 0;
    if (rrea_gpu_status const s = instance_slice(ctx, species, instance, begin, n)) return s;
    SpeciesTile& st = ctx->tiles[species];
    SpeciesTile const whole = st;
    int64_t const n_surv = ctx->n_surv;
    for (int f = 0; f < kTileDoubles; ++f) st.d[f] += begin;
    st.id += begin;
    st.cpu += begin;
    st.n = n;
    ctx->n_surv = 0;   // the instance's live particles alone, no staged candidates
    rrea_gpu_status const s = rrea_gpu_population_thin_resident(ctx, species, target, step, salt, nullptr, 0, stats);
    st = whole;
    ctx->n_surv = n_surv;
    return s;
}

rrea_gpu_status rrea_gpu_ensemble_population_thin_all(rrea_gpu_ctx* ctx, int32_t species, const int64_t* targets,
                                                      int32_t step, uint64_t salt, int64_t* removed_per_instance,
                                                      int64_t* stats)
{
    if (!ctx || (species != RREA_SPECIES_ELECTRON && species != RREA_SPECIES_POSITRON) || !targets ||
        !removed_per_instance) {
        return RREA_GPU_ERR_ARGUMENT;
    }
    if (ctx->n_instances <= 0) return fail(ctx, RREA_GPU_ERR_NOT_READY, "no ensemble is configured");
    for (int32_t k = 0; k < ctx->n_instances; ++k) {
        if (targets[k] < 0) return fail(ctx, RREA_GPU_ERR_ARGUMENT, "population targets must be >= 0");
    }
    rrea_gpu_config const& c = ctx->cfg;
    SpeciesTile& st = ctx->tiles[species];
    rrea_launch::PopulationInput in{};
    in.r = st.d[0]; in.z = st.d[1]; in.theta = st.d[2]; in.ux = st.d[3]; in.uy = st.d[4]; in.uz = st.d[5];
    in.w = st.d[6];
    in.id = st.id;
    in.cpu = st.cpu;
    in.n_tile = st.n;
    in.species = species;
    in.periodic_z = c.periodic_z;
    in.r_lo = c.r_lo;
    in.z_lo = c.z_lo;
    in.z_hi = c.z_hi;
    in.dr = (c.r_hi - c.r_lo) / c.nr;
    in.dz = (c.z_hi - c.z_lo) / c.nz;
    in.rng_seed = c.rng_seed;
    in.salt = salt;
    in.step = step;
    in.targets = targets;
    in.n_inst = ctx->n_instances;
    rrea_launch::PopulationStats ps{};
    RREA_CUDA(ctx, rrea_launch::population_thin_instances(in, ctx->pop_work, ps, removed_per_instance, ctx->stream));
    if (stats) {
        int64_t const v[8] = {ps.members, ps.live, ps.candidates, ps.supports, ps.capacity, ps.floor, ps.requested,
                              ps.removed};
        for (int k = 0; k < 8; ++k) stats[k] = v[k];
    }
    if (ps.status != 0) {
        return fail(ctx, static_cast<rrea_gpu_status>(ps.status),
                    ps.status == RREA_GPU_ERR_GEOMETRY
                        ? "population control found a particle outside the supported grid"
                        : "population control plan rejected (invalid support plan or insufficient progress); "
                          "nothing was applied");
    }
    RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RREA_GPU_OK;
}

}  // extern "C"

// ===========================================================================
// Pathwise adjoint of the charged push (rrea_adjoint.cu)
// ===========================================================================
extern "C" {

void rrea_gpu_default_adjoint_config(rrea_gpu_adjoint_config* c)
{
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    c->z_lo = 0.0;
    c->z_hi = 500.0;
    c->n_nodes = 256;
    c->steps = 2000;
    c->substeps = 4;
    c->checkpoint_every = 32;
    c->dt_s = 5.0e-10;
    c->density_ratio = 1.0;
    c->cutoff_eV = 1.0e4;
    c->scatter_rms_rad = 0.02;
    c->k_threshold_eV = 1.0e6;
    c->k_width_eV = 5.0e4;
    c->z_plane_m = 400.0;
    c->z_width_m = 1.0;
    c->plane_weight = 1.0;
    c->rng_seed = 1;
}

rrea_gpu_status rrea_gpu_adjoint_stage(rrea_gpu_ctx* ctx, const rrea_gpu_adjoint_config* cfg, int64_t n,
                                       const double* z, const double* dir3, const double* kinetic_eV,
                                       const double* weight, const uint64_t* id)
{
    if (!ctx || !cfg || n < 0 || (n > 0 && (!z || !dir3 || !kinetic_eV || !weight || !id))) {
        return RREA_GPU_ERR_ARGUMENT;
    }
    if (!ctx->tables_loaded) return fail(ctx, RREA_GPU_ERR_NOT_READY, "the adjoint reads the loaded stopping powers");
    if (cfg->n_nodes < 2 || cfg->n_nodes > rrea_launch::adjoint_max_nodes() || !(cfg->z_hi > cfg->z_lo)
        || cfg->steps < 1 || cfg->substeps < 1 || cfg->checkpoint_every < 1 || !(cfg->dt_s > 0.0)
        || !(cfg->density_ratio > 0.0) || !(cfg->cutoff_eV > 0.0) || !(cfg->k_width_eV > 0.0)
        || !(cfg->z_width_m > 0.0) || !(cfg->scatter_rms_rad >= 0.0)) {
        return fail(ctx, RREA_GPU_ERR_ARGUMENT, "invalid adjoint configuration");
    }
    std::vector<double> seeds(6 * static_cast<size_t>(n));
    for (int64_t i = 0; i < n; ++i) {
        double const dx = dir3[3 * i], dy = dir3[3 * i + 1], dz = dir3[3 * i + 2];
        double const norm = std::sqrt(dx * dx + dy * dy + dz * dz);
        if (!(norm > 0.0) || !std::isfinite(norm) || !std::isfinite(z[i]) || !(kinetic_eV[i] > cfg->cutoff_eV)) {
            return fail(ctx, RREA_GPU_ERR_ARGUMENT, "adjoint seeds need finite states above the cutoff");
        }
        seeds[static_cast<size_t>(i)] = z[i];
        seeds[static_cast<size_t>(n + i)] = dx / norm;
        seeds[static_cast<size_t>(2 * n + i)] = dy / norm;
        seeds[static_cast<size_t>(3 * n + i)] = dz / norm;
        seeds[static_cast<size_t>(4 * n + i)] = kinetic_eV[i];
        seeds[static_cast<size_t>(5 * n + i)] = 1.0;
    }
    RreaArenaIndex const& ix = ctx->tables.index();
    for (int t : {RREA_T_E_COLLISION, RREA_T_E_SOFT_RAD}) {
        if (ix.hot[t].mode != RREA_INTERP_LOGLOG && ix.hot[t].mode != RREA_INTERP_LOGLOG_ZERO_THRESHOLD) {
            return fail(ctx, RREA_GPU_ERR_TABLES, "the adjoint's stopping powers must be log-log tables");
        }
    }
    rrea_launch::AdjointSetup in{};
    in.n = n;
    in.n_nodes = cfg->n_nodes;
    in.z0 = cfg->z_lo;
    in.dz_node = (cfg->z_hi - cfg->z_lo) / (cfg->n_nodes - 1);
    in.steps = cfg->steps;
    in.substeps = cfg->substeps;
    in.ckpt_every = cfg->checkpoint_every;
    in.dt = cfg->dt_s;
    in.rho = cfg->density_ratio;
    in.cutoff = cfg->cutoff_eV;
    in.scatter_rms = cfg->scatter_rms_rad;
    in.k_th = cfg->k_threshold_eV;
    in.tau_k = cfg->k_width_eV;
    in.z_p = cfg->z_plane_m;
    in.tau_z = cfg->z_width_m;
    in.lambda = cfg->plane_weight;
    in.seed = cfg->rng_seed;
    in.col = ix.hot[RREA_T_E_COLLISION];
    in.soft = ix.hot[RREA_T_E_SOFT_RAD];
    RREA_CUDA(ctx, rrea_launch::adjoint_stage(in, seeds.data(), weight, id, ctx->num_sms * 4, ctx->adjoint));
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_adjoint_forward(rrea_gpu_ctx* ctx, const double* e_nodes_device, double* loss)
{
    if (!ctx || !e_nodes_device || !loss) return RREA_GPU_ERR_ARGUMENT;
    if (!ctx->adjoint) return fail(ctx, RREA_GPU_ERR_NOT_READY, "no adjoint problem is staged");
    RREA_CUDA(ctx, rrea_launch::adjoint_forward(*ctx->adjoint, ctx->d_arena, e_nodes_device, false, *loss,
                                                ctx->stream));
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_adjoint_forward_frozen(rrea_gpu_ctx* ctx, const double* e_nodes_device, double* loss)
{
    if (!ctx || !e_nodes_device || !loss) return RREA_GPU_ERR_ARGUMENT;
    if (!ctx->adjoint || !rrea_launch::adjoint_recorded(*ctx->adjoint)) {
        return fail(ctx, RREA_GPU_ERR_NOT_READY, "no recording adjoint forward has run");
    }
    RREA_CUDA(ctx, rrea_launch::adjoint_forward(*ctx->adjoint, ctx->d_arena, e_nodes_device, true, *loss,
                                                ctx->stream));
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_adjoint_backward(rrea_gpu_ctx* ctx, const double* e_nodes_device, double* grad_device)
{
    if (!ctx || !e_nodes_device || !grad_device) return RREA_GPU_ERR_ARGUMENT;
    if (!ctx->adjoint || !rrea_launch::adjoint_recorded(*ctx->adjoint)) {
        return fail(ctx, RREA_GPU_ERR_NOT_READY, "the reverse pass follows a recording forward");
    }
    RREA_CUDA(ctx, rrea_launch::adjoint_backward(*ctx->adjoint, ctx->d_arena, e_nodes_device, grad_device,
                                                 ctx->stream));
    RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RREA_GPU_OK;
}

rrea_gpu_status rrea_gpu_adjoint_final_state(rrea_gpu_ctx* ctx, double* state6)
{
    if (!ctx || !state6) return RREA_GPU_ERR_ARGUMENT;
    if (!ctx->adjoint) return fail(ctx, RREA_GPU_ERR_NOT_READY, "no adjoint problem is staged");
    RREA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    RREA_CUDA(ctx, rrea_launch::adjoint_final_state(*ctx->adjoint, state6));
    return RREA_GPU_OK;
}

}  // extern "C"
