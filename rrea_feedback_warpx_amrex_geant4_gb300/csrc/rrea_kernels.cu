// Kernels of the GB300 kinetic step and their launchers.
//
//   field_prep_kernel     cell-centred total field (Maxwell + ambient face
//                         averages), once per step
//   electron_step_kernel  one thread per electron, full outer step (the
//                         positron kernel lives in rrea_positron_kernels.cu)
//   scan / scatter        orders the appended secondaries into the reference's
//                         deterministic order (parent index, then lineage)
#include "rrea_kernels.h"

#include <atomic>

#include "device/rrea_charged_kernel.cuh"

#include <cuda_runtime.h>

namespace rrea_dev {

__global__ void field_prep_kernel(int nr, int nz, const double* __restrict__ er, const double* __restrict__ ez,
                                  const double* __restrict__ amb_er, const double* __restrict__ amb_ez,
                                  double* __restrict__ cell_er, double* __restrict__ cell_ez)
{
    int64_t const total = static_cast<int64_t>(nr) * nz;
    for (int64_t c = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; c < total;
         c += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        int const i = static_cast<int>(c % nr);
        int const j = static_cast<int>(c / nr);
        // S/RreaAmrexAdvance.cpp:556-565: 0.5*((m+a)_lo + (m+a)_hi)
        size_t const rlo = static_cast<size_t>(i) + static_cast<size_t>(nr + 1) * j;
        double const elo = er[rlo] + amb_er[rlo];
        double const ehi = er[rlo + 1] + amb_er[rlo + 1];
        cell_er[c] = 0.5 * (elo + ehi);
        size_t const zlo = static_cast<size_t>(i) + static_cast<size_t>(nr) * j;
        size_t const zhi = static_cast<size_t>(i) + static_cast<size_t>(nr) * (j + 1);
        double const zl = ez[zlo] + amb_ez[zlo];
        double const zh = ez[zhi] + amb_ez[zhi];
        cell_ez[c] = 0.5 * (zl + zh);
    }
}

// The table-driven log (which 0) or exp (which 1) next to the CUDA
// function, for the accuracy test.
__global__ void eval_math_kernel(const double* __restrict__ arena, int which, const double* __restrict__ x,
                                 int64_t n, double* __restrict__ fast, double* __restrict__ libm)
{
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        fast[i] = which == 0 ? flog(arena, x[i]) : fexp(arena, x[i]);
        libm[i] = which == 0 ? log(x[i]) : exp(x[i]);
    }
}

// Live (id > 0) particles of a tile, warp-aggregated.
__global__ void count_live_kernel(const int64_t* __restrict__ id, int64_t n, unsigned long long* __restrict__ out)
{
    unsigned int live = 0;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        live += id[i] > 0 ? 1u : 0u;
    }
    unsigned int const warp_total = __reduce_add_sync(0xffffffffu, live);
    if ((threadIdx.x & 31) == 0 && warp_total) atomicAdd(out, static_cast<unsigned long long>(warp_total));
}

// Exclusive scan of per-parent secondary counts (uint32 -> int64 offsets),
// three passes: block sums, scan of block sums, block-local scan + offset.
constexpr int kScanBlock = 1024;

__device__ __forceinline__ int64_t block_exclusive_scan(int64_t v, int64_t& total)
{
    __shared__ int64_t warp_sums[32];
    int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int64_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int64_t const y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int64_t s = lane < (blockDim.x >> 5) ? warp_sums[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int64_t const y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        warp_sums[lane] = s;
    }
    __syncthreads();
    int64_t const prefix = (warp > 0 ? warp_sums[warp - 1] : 0) + x - v;
    total = warp_sums[(blockDim.x >> 5) - 1];
    __syncthreads();
    return prefix;
}

__global__ void __launch_bounds__(kScanBlock) scan_block_sums(const uint32_t* __restrict__ counts, int64_t n,
                                                              int64_t* __restrict__ block_sums)
{
    int64_t const i = blockIdx.x * static_cast<int64_t>(kScanBlock) + threadIdx.x;
    int64_t const v = i < n ? counts[i] : 0;
    int64_t total;
    (void)block_exclusive_scan(v, total);
    if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanBlock) scan_block_offsets(int64_t* __restrict__ block_sums, int64_t nblocks)
{
    // single block; loops for more than kScanBlock blocks
    int64_t carry = 0;
    for (int64_t base = 0; base < nblocks; base += kScanBlock) {
        int64_t const i = base + threadIdx.x;
        int64_t const v = i < nblocks ? block_sums[i] : 0;
        int64_t total;
        int64_t const p = block_exclusive_scan(v, total);
        if (i < nblocks) block_sums[i] = carry + p;
        carry += total;
    }
}

__global__ void __launch_bounds__(kScanBlock) scan_apply(const uint32_t* __restrict__ counts, int64_t n,
                                                         const int64_t* __restrict__ block_offsets,
                                                         int64_t* __restrict__ offsets)
{
    int64_t const i = blockIdx.x * static_cast<int64_t>(kScanBlock) + threadIdx.x;
    int64_t const v = i < n ? counts[i] : 0;
    int64_t total;
    int64_t const p = block_exclusive_scan(v, total);
    if (i < n) offsets[i] = block_offsets[blockIdx.x] + p;
}

__global__ void scatter_secondaries(const rrea_gpu_secondary* __restrict__ in, int64_t count,
                                    const int64_t* __restrict__ offsets, rrea_gpu_secondary* __restrict__ out)
{
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < count;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        rrea_gpu_secondary const s = in[i];
        out[offsets[s.parent_index] + static_cast<int64_t>(s.lineage)] = s;
    }
}

}  // namespace rrea_dev

namespace rrea_launch {

namespace {
std::atomic<unsigned long long> g_launches{0};
}

void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
unsigned long long launches_noted() { return g_launches.load(std::memory_order_relaxed); }


cudaError_t set_step_constants(rrea_dev::StepConstants const& c, cudaStream_t stream)
{
    return cudaMemcpyToSymbolAsync(rrea_dev::c_step, &c, sizeof(c), 0, cudaMemcpyHostToDevice, stream);
}

cudaError_t field_prep(int nr, int nz, const double* er, const double* ez, const double* amb_er, const double* amb_ez,
                       double* cell_er, double* cell_ez, cudaStream_t stream)
{
    int64_t const total = static_cast<int64_t>(nr) * nz;
    int const threads = 256;
    int const blocks = static_cast<int>((total + threads - 1) / threads);
    note_launch();
    rrea_dev::field_prep_kernel<<<blocks > 0 ? blocks : 1, threads, 0, stream>>>(nr, nz, er, ez, amb_er, amb_ez,
                                                                                  cell_er, cell_ez);
    return cudaGetLastError();
}

cudaError_t electron_step(rrea_dev::ElectronArgs const& args, int blocks, int threads, int min_blocks, bool periodic,
                          cudaStream_t stream)
{
    note_launch();
    if (periodic) {
        rrea_dev::electron_step_kernel<16, RREA_ARENA_MAX_PIECES><<<blocks, threads, 0, stream>>>(args);
        return cudaGetLastError();
    }
    switch (min_blocks) {
    case 4: rrea_dev::electron_step_kernel<4, 1><<<blocks, threads, 0, stream>>>(args); break;
    case 8: rrea_dev::electron_step_kernel<8, 1><<<blocks, threads, 0, stream>>>(args); break;
    case 12: rrea_dev::electron_step_kernel<12, 1><<<blocks, threads, 0, stream>>>(args); break;
    case 16: rrea_dev::electron_step_kernel<16, 1><<<blocks, threads, 0, stream>>>(args); break;
    default: rrea_dev::electron_step_kernel<2, 1><<<blocks, threads, 0, stream>>>(args); break;
    }
    return cudaGetLastError();
}

cudaError_t eval_math(const double* arena, int which, const double* x, int64_t n, double* fast, double* libm,
                      cudaStream_t stream)
{
    if (n <= 0) return cudaSuccess;
    note_launch();
    int64_t const b = (n + 255) / 256;
    rrea_dev::eval_math_kernel<<<static_cast<unsigned>(b < 4096 ? b : 4096), 256, 0, stream>>>(arena, which, x, n,
                                                                                                fast, libm);
    return cudaGetLastError();
}

cudaError_t count_live(const int64_t* id, int64_t n, unsigned long long* out, int blocks, cudaStream_t stream)
{
    if (n <= 0) return cudaSuccess;
    note_launch();
    rrea_dev::count_live_kernel<<<blocks, 256, 0, stream>>>(id, n, out);
    return cudaGetLastError();
}

int64_t scan_scratch_elems(int64_t n) { return (n + rrea_dev::kScanBlock - 1) / rrea_dev::kScanBlock + 1; }

cudaError_t exclusive_scan_counts(const uint32_t* counts, int64_t n, int64_t* offsets, int64_t* block_scratch,
                                  cudaStream_t stream)
{
    if (n <= 0) return cudaSuccess;
    for (int k = 0; k < 3; ++k) note_launch();
    int64_t const nblocks = (n + rrea_dev::kScanBlock - 1) / rrea_dev::kScanBlock;
    rrea_dev::scan_block_sums<<<static_cast<unsigned>(nblocks), rrea_dev::kScanBlock, 0, stream>>>(counts, n,
                                                                                                  block_scratch);
    rrea_dev::scan_block_offsets<<<1, rrea_dev::kScanBlock, 0, stream>>>(block_scratch, nblocks);
    rrea_dev::scan_apply<<<static_cast<unsigned>(nblocks), rrea_dev::kScanBlock, 0, stream>>>(counts, n, block_scratch,
                                                                                             offsets);
    return cudaGetLastError();
}

cudaError_t order_secondaries(const uint32_t* counts, int64_t n, int64_t* offsets, int64_t* block_scratch,
                              const rrea_gpu_secondary* unordered, int64_t count, rrea_gpu_secondary* ordered,
                              cudaStream_t stream)
{
    if (n <= 0) return cudaSuccess;
    cudaError_t const e = exclusive_scan_counts(counts, n, offsets, block_scratch, stream);
    if (e != cudaSuccess) return e;
    if (count > 0) {
        note_launch();
        int const threads = 256;
        int64_t const blocks = (count + threads - 1) / threads;
        rrea_dev::scatter_secondaries<<<static_cast<unsigned>(blocks < 65535 ? blocks : 65535), threads, 0, stream>>>(
            unordered, count, offsets, ordered);
    }
    return cudaGetLastError();
}

}  // namespace rrea_launch
