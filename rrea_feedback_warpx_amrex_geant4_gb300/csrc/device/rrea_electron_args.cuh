// Arguments of the species transport kernels (electron and photon phases):
// the species tile (SoA in HBM), the per-step output sinks and the field
// view (unused by the photon phase).  Shared by the kernel
// translation unit and the host-side launcher.
#pragma once

#include "rrea_device_path.cuh"

namespace rrea_dev {

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
};

}  // namespace rrea_dev
