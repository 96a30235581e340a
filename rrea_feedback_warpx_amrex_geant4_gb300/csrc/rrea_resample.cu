// One thread per CIC support group: the thinning primitive of
// device/rrea_resample.cuh over groups laid out back to back.
#include "rrea_kernels.h"

#include "device/rrea_resample.cuh"

#include <cuda_runtime.h>

namespace rrea_dev {
namespace {

__global__ void cic_thin_kernel(const double* __restrict__ fr, const double* __restrict__ fz, double* __restrict__ w,
                                const int64_t* __restrict__ offsets, int64_t n_groups,
                                const int64_t* __restrict__ max_removals, const uint64_t* __restrict__ keys,
                                int64_t* __restrict__ removed, int64_t* __restrict__ draws,
                                int32_t* __restrict__ valid, int64_t* __restrict__ capacity)
{
    for (int64_t gi = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; gi < n_groups;
         gi += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        int64_t const b = offsets[gi];
        int const n = static_cast<int>(offsets[gi + 1] - b);
        int live = 0;
        for (int i = 0; i < n; ++i) live += w[b + i] > 0.0 ? 1 : 0;
        int const rank = cic_constraint_rank(fr + b, fz + b, w + b, n);
        capacity[gi] = live > rank ? live - rank : 0;
        CicThinResult const r = cic_thin(fr + b, fz + b, w + b, n, max_removals[gi], keys[gi]);
        removed[gi] = r.removed;
        draws[gi] = r.draws;
        valid[gi] = r.valid ? 1 : 0;
    }
}

}  // namespace
}  // namespace rrea_dev

namespace rrea_launch {

cudaError_t cic_thin(const double* fr, const double* fz, double* w, const int64_t* offsets, int64_t n_groups,
                     const int64_t* max_removals, const uint64_t* keys, int64_t* removed, int64_t* draws,
                     int32_t* valid, int64_t* capacity, cudaStream_t stream)
{
    if (n_groups <= 0) return cudaSuccess;
    note_launch();
    int const threads = 64;
    int64_t const blocks = (n_groups + threads - 1) / threads;
    rrea_dev::cic_thin_kernel<<<static_cast<unsigned>(blocks < 65535 ? blocks : 65535), threads, 0, stream>>>(
        fr, fz, w, offsets, n_groups, max_removals, keys, removed, draws, valid, capacity);
    return cudaGetLastError();
}

}  // namespace rrea_launch
