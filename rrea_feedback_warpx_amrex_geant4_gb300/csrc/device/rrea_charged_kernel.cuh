// The charged transport kernels (electron and positron phases): one thread
// per particle through one full outer step, the grid-stride (or work-counter)
// body shared by both.  Included by the translation units that instantiate
// them (rrea_kernels.cu: electrons, rrea_positron_kernels.cu: positrons);
// each of them has its own copy of the step constants c_step.
#pragma once

#include "rrea_electron.cuh"

namespace rrea_dev {

// MinBlocks trades registers for resident warps: 2 -> up to 255 registers
// (8 warps/SM), 4 -> 128 (16), 8 -> 64 (32), 12 -> 40 (48), 16 -> 32 (64).
// The transport loop is latency-bound (instruction fetch and dependent
// FP64 chains), so full residency wins despite the spills it forces.
// NP is the chord piece capacity: 1 for absorbing z faces, 4 for periodic z.
// Grid-stride body shared by the electron and positron kernels.
template <int NP, bool POS>
__device__ __forceinline__ void charged_step_body(ElectronArgs const& A)
{
    StepConstants const& C = c_step;
    // one ion-pair slot per thread (the kernels launch at most 128 threads per block)
    __shared__ IonPairSlot ion_slots[128];
    IonPairSlot* const my_slot = ion_slots + threadIdx.x;
    unsigned int moved = 0;
    for_each_particle(A.n, A.work, [&](int64_t ip) {
        if (!(A.id[ip] > 0)) {
            if (A.segments) A.segments[ip].kind = 0;
            if (A.sec_per_parent) A.sec_per_parent[ip] = 0;
            if (A.diag_disposition) A.diag_disposition[ip] = -1;
            if (A.diag_subcycles) A.diag_subcycles[ip] = 0;
            if (A.diag_events) A.diag_events[ip] = 0;
            return;
        }
        Err err;
        uint64_t sub = 0, ev = 0;
        uint32_t lineage = 0;
        ++moved;
        if (A.segments) A.segments[ip].kind = 0;
        IonPairCache ion_pairs;
        ion_pairs.init(my_slot, POS ? 0.0 : 0.5 * C.cfg.low_energy_cutoff_eV, C.tix.w_air_eV_per_pair);
        int const disp = transport_charged<NP, POS>(C, A, ip, sub, ev, lineage, ion_pairs, err);
        ion_pairs.flush(C, A.cells);
        // Every record this particle appended carries a lineage below this
        // count, so the ordering scan/scatter stays in bounds on every path.
        if (A.sec_per_parent) A.sec_per_parent[ip] = lineage;
        if (err.code) record_failure(A, err.code, ip);
        if (A.diag_disposition) A.diag_disposition[ip] = disp;
        if (A.diag_subcycles) A.diag_subcycles[ip] = sub;
        if (A.diag_events) A.diag_events[ip] = ev;
    }, A.order);
    // warp-aggregated count of transported particles
    unsigned int const warp_total = __reduce_add_sync(0xffffffffu, moved);
    if ((threadIdx.x & 31) == 0 && warp_total) atomicAdd(A.transported, static_cast<unsigned long long>(warp_total));
}

template <int MinBlocks, int NP>
__global__ void __launch_bounds__(128, MinBlocks) electron_step_kernel(const __grid_constant__ ElectronArgs A)
{
    charged_step_body<NP, false>(A);
}

template <int MinBlocks, int NP>
__global__ void __launch_bounds__(128, MinBlocks) positron_step_kernel(const __grid_constant__ ElectronArgs A)
{
    charged_step_body<NP, true>(A);
}

}  // namespace rrea_dev
