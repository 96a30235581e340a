// Arguments of the species transport kernels (electron and photon phases):
// the species tile (SoA in HBM), the per-step output sinks and the field
// view (unused by the photon phase).  Shared by the kernel
// translation unit and the host-side launcher.
#pragma once

#include "rrea_device_path.cuh"

namespace rrea_dev {

// One charged particle's net-chord record for the current deposition
// (TransportSideEffects::AccumulateChargedSegment / AccumulateChargedEscape,
// O/RreaTransportLog.H:556-599).  kind 0: nothing to deposit; 1: segment
// (a0..a4 = r0, z0, r1, z1, signed weight); 2: escape (a0..a6 = trajectory
// start r, z, final microchord start r, z, crossing r, z, signed weight).
struct SegmentRec {
    double a[7];
    int32_t kind;
    uint32_t faces;
};

// The coupling's padded net-chord grid (O/RreaWarpXCoupling.cpp:417-444):
// rho nr*nz, jr (nr+1)*nz, jz nr*(nz+1), index-space fluxes.
struct NetGrid {
    int nr, nz;                           // padded cells
    int phys_nr, phys_z_begin, phys_nz;   // physical block inside the padding
    double dr, dz, r_lo, z_lo;            // z_lo of the padded grid
    double* rho;
    double* jr;
    double* jz;
};

struct ElectronArgs {
    int64_t n;
    // The current and prev_* arrays may alias (resident engine mode, where
    // the captured pre-push state IS the current state): no __restrict__.
    double* r;
    double* z;
    double* theta;
    double* ux;
    double* uy;
    double* uz;
    const double* __restrict__ w;
    const double* prev_r;
    const double* prev_z;
    const double* prev_theta;
    const double* prev_ux;
    const double* prev_uy;
    const double* prev_uz;
    int64_t* __restrict__ id;
    const int32_t* __restrict__ cpu;
    // secondaries (unordered append) and per-parent counts for the ordering pass
    rrea_gpu_secondary* __restrict__ sec;
    unsigned long long* __restrict__ sec_count;
    int64_t sec_capacity;
    uint32_t* __restrict__ sec_per_parent;
    // cell sources: 5 grids of nr*nz
    double* __restrict__ cells;
    // altitude density profile (prof.n == 0: uniform density ratio)
    DensityProfile prof;
    // optional per-particle diagnostics (may be null)
    uint64_t* __restrict__ diag_subcycles;
    uint64_t* __restrict__ diag_events;
    int32_t* __restrict__ diag_disposition;
    // status: first failing code and particle
    int* __restrict__ status;
    long long* __restrict__ fail_index;
    // particles transported this step (id > 0 on entry)
    unsigned long long* __restrict__ transported;
    const double* __restrict__ arena;
    FieldView fv;
    // photon phase only: 1 = push each photon straight by c*dt from its
    // current state before transporting the chord (resident mode)
    int32_t straight_push;
    // charged phases: one net-chord record per tile slot (may be null)
    SegmentRec* __restrict__ segments;
    // dynamic scheduling: warps take the next 32 particles from this counter
    // (zeroed before the launch); null = static grid-stride assignment
    unsigned long long* __restrict__ work;
    // tile index of element 0 of every per-particle array above: a launch
    // over one chunk of a tile passes offset arrays and the chunk's start,
    // so parent indices and failure indices stay tile indices
    int64_t index_base;
    // optional scheduling order of the tile indices (null: the end of the
    // tile first); it changes which thread visits a particle, never a result
    const uint32_t* __restrict__ order;
    // plane-crossing diagnostic of the electrons' continuous segments:
    // n_planes strictly increasing plane z and kPlaneValues accumulators per
    // plane (n_planes = 0: off)
    int32_t n_planes;
    const double* __restrict__ plane_z;
    double* __restrict__ plane_bins;
};

// Accumulators per plane, in the reference's flattened order
// (RreaPlaneFluxAccumulator::Flatten, I/RreaPlaneFlux.H:161-176): up and down
// weight of all tracked, local-runaway and >= 1 MeV crossings, then the
// local-runaway crossings' up and down sums of w r and of w r^2.
constexpr int kPlaneValues = 10;

// Visits every particle index of [0, n) once.  With a work counter each warp
// claims the next 32 indices when it is done with its previous ones, so a
// slow particle does not hold up the ones a static assignment would have
// queued behind it on the same thread.  The claims run from the end of the
// tile: committed survivors, appended there, are mostly slow low-energy
// particles, and starting with them keeps them out of the launch's tail.
template <class F>
__device__ __forceinline__ void for_each_particle(int64_t n, unsigned long long* work, F&& f,
                                                  const uint32_t* __restrict__ order = nullptr)
{
    if (work) {
        int const lane = threadIdx.x & 31;
        for (;;) {
            unsigned long long base = 0;
            if (lane == 0) base = atomicAdd(work, 32ULL);
            base = __shfl_sync(0xffffffffu, base, 0);
            if (base >= static_cast<unsigned long long>(n)) break;
            int64_t const k = static_cast<int64_t>(base) + lane;
            if (k < n) f(order ? static_cast<int64_t>(__ldg(order + k)) : n - 1 - k);
        }
    } else {
        for (int64_t ip = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; ip < n;
             ip += static_cast<int64_t>(gridDim.x) * blockDim.x) {
            f(ip);
        }
    }
}

}  // namespace rrea_dev
