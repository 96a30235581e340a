// Photon phase kernel of the GB300 kinetic step: one thread per photon, one
// full outer step (chord flight, at most one interaction per chord, Compton
// continuation), secondaries appended for the shared ordering pass.
#include "rrea_kernels.h"

#include "device/rrea_photon.cuh"

#include <cuda_runtime.h>

namespace rrea_dev {

__constant__ StepConstants c_step_photon;

template <int NP>
__global__ void __launch_bounds__(128, 2) photon_step_kernel(const __grid_constant__ ElectronArgs A)
{
    StepConstants const& C = c_step_photon;
    unsigned int moved = 0;
    for_each_particle(A.n, A.work, [&](int64_t ip) {
        if (!(A.id[ip] > 0)) {
            if (A.sec_per_parent) A.sec_per_parent[ip] = 0;
            if (A.diag_disposition) A.diag_disposition[ip] = -1;
            if (A.diag_subcycles) A.diag_subcycles[ip] = 0;
            if (A.diag_events) A.diag_events[ip] = 0;
            return;
        }
        Err err;
        uint64_t ev = 0;
        uint32_t lineage = 0;
        ++moved;
        int const disp = transport_photon<NP>(C, A, ip, ev, lineage, err);
        // every appended record of this photon has a lineage below this count
        if (A.sec_per_parent) A.sec_per_parent[ip] = lineage;
        if (err.code) record_failure(A, err.code, ip);
        if (A.diag_disposition) A.diag_disposition[ip] = disp;
        if (A.diag_subcycles) A.diag_subcycles[ip] = 0;
        if (A.diag_events) A.diag_events[ip] = ev;
    });
    unsigned int const warp_total = __reduce_add_sync(0xffffffffu, moved);
    if ((threadIdx.x & 31) == 0 && warp_total) atomicAdd(A.transported, static_cast<unsigned long long>(warp_total));
}

}  // namespace rrea_dev

namespace rrea_launch {

cudaError_t photon_constants(rrea_dev::StepConstants const& sc, cudaStream_t stream)
{
    return cudaMemcpyToSymbolAsync(rrea_dev::c_step_photon, &sc, sizeof(sc), 0, cudaMemcpyHostToDevice, stream);
}

cudaError_t photon_step(rrea_dev::ElectronArgs const& args, int blocks, int threads, bool periodic, cudaStream_t stream)
{
    rrea_launch::note_launch();
    if (periodic) {
        rrea_dev::photon_step_kernel<RREA_ARENA_MAX_PIECES><<<blocks, threads, 0, stream>>>(args);
    } else {
        rrea_dev::photon_step_kernel<1><<<blocks, threads, 0, stream>>>(args);
    }
    return cudaGetLastError();
}

}  // namespace rrea_launch
