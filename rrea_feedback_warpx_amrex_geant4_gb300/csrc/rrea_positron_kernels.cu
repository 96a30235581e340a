// Positron phase kernel of the GB300 kinetic step: one thread per positron,
// one full outer step (the charged body shared with the electron phase, with
// Bhabha, positron brems and annihilation in place of Moller and electron
// brems).  A translation unit of its own, so its register variants compile
// beside the electron kernel's.
#include "rrea_kernels.h"

#include "device/rrea_charged_kernel.cuh"

#include <cuda_runtime.h>

namespace rrea_launch {

cudaError_t positron_constants(rrea_dev::StepConstants const& sc, cudaStream_t stream)
{
    return cudaMemcpyToSymbolAsync(rrea_dev::c_step, &sc, sizeof(sc), 0, cudaMemcpyHostToDevice, stream);
}

cudaError_t positron_step(rrea_dev::ElectronArgs const& args, int blocks, int threads, int min_blocks, bool periodic,
                          cudaStream_t stream)
{
    note_launch();
    if (periodic) {
        rrea_dev::positron_step_kernel<16, RREA_ARENA_MAX_PIECES><<<blocks, threads, 0, stream>>>(args);
        return cudaGetLastError();
    }
    switch (min_blocks) {
    case 2: rrea_dev::positron_step_kernel<2, 1><<<blocks, threads, 0, stream>>>(args); break;
    case 4: rrea_dev::positron_step_kernel<4, 1><<<blocks, threads, 0, stream>>>(args); break;
    case 8: rrea_dev::positron_step_kernel<8, 1><<<blocks, threads, 0, stream>>>(args); break;
    default: rrea_dev::positron_step_kernel<16, 1><<<blocks, threads, 0, stream>>>(args); break;
    }
    return cudaGetLastError();
}

}  // namespace rrea_launch
