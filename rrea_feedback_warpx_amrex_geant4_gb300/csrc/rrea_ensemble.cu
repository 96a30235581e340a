// Batched ensemble of independent avalanche instances in one set of species
// tiles.  An instance is a particle's cpu ordinal (the high field of its RNG
// key |id| ^ cpu << 40), so every instance draws from its own streams; ids
// are counted per instance and species, and a committed secondary takes its
// root's instance (key bits 40 and up).  With these two rules each
// instance's particles, ids, streams and results are exactly those of the
// same instance run alone with cpu = k: one launch sequence advances every
// instance instead of one sequence per instance.
//
// Kernels here: the per-instance ids of the survivor commit (a stable radix
// sort by instance, ranks within each instance's run), the stable partition
// of a tile by instance (so an instance is one contiguous slice for its
// census, retirement and population control), and the retirement of an
// instance.
#include "rrea_kernels.h"

#include <cub/device/device_radix_sort.cuh>
#include <cuda_runtime.h>

namespace rrea_dev {
namespace {

__device__ __forceinline__ bool accepts(rrea_gpu_secondary const& s, int species)
{
    return s.species == species && s.weight > 0.0 && (species != RREA_SPECIES_PHOTON || s.energy_eV > 0.0);
}

// Key of every survivor: its instance when it is committed into `species`,
// else the sentinel n_inst (sorted last).
__global__ void survivor_keys_kernel(const rrea_gpu_secondary* __restrict__ surv, int64_t n, int species,
                                     uint32_t n_inst, uint32_t* __restrict__ keys, uint32_t* __restrict__ vals)
{
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        rrea_gpu_secondary const s = surv[i];
        uint32_t const inst = static_cast<uint32_t>(s.root_key >> 40);
        keys[i] = accepts(s, species) && inst < n_inst ? inst : n_inst;
        vals[i] = static_cast<uint32_t>(i);
    }
}

// First and one-past-last sorted position of every instance's run.
__global__ void run_bounds_kernel(const uint32_t* __restrict__ keys, int64_t n, uint32_t n_inst,
                                  int64_t* __restrict__ begin, int64_t* __restrict__ end)
{
    for (int64_t p = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; p < n;
         p += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        uint32_t const k = keys[p];
        if (k >= n_inst) continue;
        if (p == 0 || keys[p - 1] != k) begin[k] = p;
        if (p == n - 1 || keys[p + 1] != k) end[k] = p + 1;
    }
}

// ids of the committed survivors: the instance's next id plus the rank in
// its run (FIFO order within the instance, the sort being stable).
__global__ void survivor_ids_kernel(const uint32_t* __restrict__ keys, const uint32_t* __restrict__ vals, int64_t n,
                                    uint32_t n_inst, const int64_t* __restrict__ begin,
                                    const int64_t* __restrict__ next_id, int species, int64_t* __restrict__ ids)
{
    for (int64_t p = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; p < n;
         p += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        uint32_t const k = keys[p];
        if (k >= n_inst) continue;
        ids[vals[p]] = next_id[3 * static_cast<int64_t>(k) + species] + (p - begin[k]);
    }
}

__global__ void advance_next_id_kernel(const int64_t* __restrict__ begin, const int64_t* __restrict__ end,
                                       uint32_t n_inst, int species, int64_t* __restrict__ next_id)
{
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n_inst; k += gridDim.x * blockDim.x) {
        next_id[3 * static_cast<int64_t>(k) + species] += end[k] - begin[k];
    }
}

__global__ void tile_keys_kernel(const int32_t* __restrict__ cpu, int64_t n, uint32_t* __restrict__ keys,
                                 uint32_t* __restrict__ vals, unsigned long long* __restrict__ counts, uint32_t n_inst)
{
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        uint32_t const k = static_cast<uint32_t>(cpu[i]);
        keys[i] = k;
        vals[i] = static_cast<uint32_t>(i);
        if (k < n_inst) atomicAdd(counts + k, 1ULL);
    }
}

__global__ void gather_tile_kernel(TileColumns src, const uint32_t* __restrict__ perm, int64_t n, TileColumns dst)
{
    for (int64_t p = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; p < n;
         p += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        int64_t const i = perm[p];
#pragma unroll
        for (int f = 0; f < kTileColumns; ++f) dst.d[f][p] = src.d[f][i];
        dst.id[p] = src.id[i];
        dst.cpu[p] = src.cpu[i];
    }
}

__global__ void retire_kernel(int64_t* __restrict__ id, const int32_t* __restrict__ cpu, int64_t n, int32_t inst)
{
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        if (cpu[i] == inst && id[i] > 0) id[i] = -id[i];
    }
}

int grid_of(int64_t n)
{
    int64_t const b = (n + 255) / 256;
    return static_cast<int>(b < 1 ? 1 : (b > 4096 ? 4096 : b));
}

int key_bits(uint32_t n_inst)
{
    int b = 1;
    while ((1u << b) <= n_inst && b < 31) ++b;
    return b;
}

}  // namespace
}  // namespace rrea_dev

namespace rrea_launch {

struct EnsembleWork {
    int64_t cap = 0;
    uint32_t *keys_in = nullptr, *keys_out = nullptr, *vals_in = nullptr, *vals_out = nullptr;
    void* cub_temp = nullptr;
    size_t cub_bytes = 0;
    int64_t* ids = nullptr;
    int64_t *begin = nullptr, *end = nullptr;   // n_inst each
    unsigned long long* counts = nullptr;       // n_inst
    uint32_t n_inst = 0;
};

void ensemble_work_free(EnsembleWork* w)
{
    if (!w) return;
    for (void* p : {static_cast<void*>(w->keys_in), static_cast<void*>(w->keys_out), static_cast<void*>(w->vals_in),
                    static_cast<void*>(w->vals_out), w->cub_temp, static_cast<void*>(w->ids),
                    static_cast<void*>(w->begin), static_cast<void*>(w->end), static_cast<void*>(w->counts)}) {
        if (p) cudaFree(p);
    }
    delete w;
}

namespace {

cudaError_t reserve(EnsembleWork*& w, int64_t n, uint32_t n_inst)
{
    if (!w) w = new EnsembleWork();
    cudaError_t e = cudaSuccess;
    if (w->n_inst < n_inst) {
        for (void* p : {static_cast<void*>(w->begin), static_cast<void*>(w->end), static_cast<void*>(w->counts)}) {
            if (p) cudaFree(p);
        }
        if ((e = cudaMalloc(&w->begin, sizeof(int64_t) * n_inst)) != cudaSuccess) return e;
        if ((e = cudaMalloc(&w->end, sizeof(int64_t) * n_inst)) != cudaSuccess) return e;
        if ((e = cudaMalloc(&w->counts, sizeof(unsigned long long) * n_inst)) != cudaSuccess) return e;
        w->n_inst = n_inst;
    }
    if (w->cap < n) {
        int64_t const cap = n + n / 4 + 1024;
        for (void* p : {static_cast<void*>(w->keys_in), static_cast<void*>(w->keys_out), static_cast<void*>(w->vals_in),
                        static_cast<void*>(w->vals_out), static_cast<void*>(w->ids), w->cub_temp}) {
            if (p) cudaFree(p);
        }
        w->cub_temp = nullptr;
        if ((e = cudaMalloc(&w->keys_in, sizeof(uint32_t) * cap)) != cudaSuccess) return e;
        if ((e = cudaMalloc(&w->keys_out, sizeof(uint32_t) * cap)) != cudaSuccess) return e;
        if ((e = cudaMalloc(&w->vals_in, sizeof(uint32_t) * cap)) != cudaSuccess) return e;
        if ((e = cudaMalloc(&w->vals_out, sizeof(uint32_t) * cap)) != cudaSuccess) return e;
        if ((e = cudaMalloc(&w->ids, sizeof(int64_t) * cap)) != cudaSuccess) return e;
        size_t bytes = 0;
        e = cub::DeviceRadixSort::SortPairs(nullptr, bytes, w->keys_in, w->keys_out, w->vals_in, w->vals_out,
                                            static_cast<int>(cap), 0, 32);
        if (e != cudaSuccess) return e;
        if ((e = cudaMalloc(&w->cub_temp, bytes)) != cudaSuccess) return e;
        w->cub_bytes = bytes;
        w->cap = cap;
    }
    return cudaSuccess;
}

cudaError_t sort_by_key(EnsembleWork& w, int64_t n, uint32_t n_inst, cudaStream_t stream)
{
    size_t bytes = w.cub_bytes;
    return cub::DeviceRadixSort::SortPairs(w.cub_temp, bytes, w.keys_in, w.keys_out, w.vals_in, w.vals_out,
                                           static_cast<int>(n), 0, rrea_dev::key_bits(n_inst), stream);
}

}  // namespace

cudaError_t ensemble_survivor_ids(const rrea_gpu_secondary* surv, int64_t n, int species, uint32_t n_inst,
                                  int64_t* next_id, EnsembleWork*& w, const int64_t** ids, cudaStream_t stream)
{
    cudaError_t e = reserve(w, n, n_inst);
    if (e != cudaSuccess) return e;
    *ids = w->ids;
    if (n == 0) return cudaSuccess;
    if ((e = cudaMemsetAsync(w->begin, 0, sizeof(int64_t) * n_inst, stream)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(w->end, 0, sizeof(int64_t) * n_inst, stream)) != cudaSuccess) return e;
    int const g = rrea_dev::grid_of(n);
    note_launch();
    rrea_dev::survivor_keys_kernel<<<g, 256, 0, stream>>>(surv, n, species, n_inst, w->keys_in, w->vals_in);
    if ((e = sort_by_key(*w, n, n_inst, stream)) != cudaSuccess) return e;
    note_launch();
    rrea_dev::run_bounds_kernel<<<g, 256, 0, stream>>>(w->keys_out, n, n_inst, w->begin, w->end);
    note_launch();
    rrea_dev::survivor_ids_kernel<<<g, 256, 0, stream>>>(w->keys_out, w->vals_out, n, n_inst, w->begin, next_id,
                                                          species, w->ids);
    note_launch();
    rrea_dev::advance_next_id_kernel<<<rrea_dev::grid_of(n_inst), 256, 0, stream>>>(w->begin, w->end, n_inst, species,
                                                                                   next_id);
    return cudaGetLastError();
}

cudaError_t ensemble_partition(rrea_dev::TileColumns const& src, int64_t n, uint32_t n_inst,
                               rrea_dev::TileColumns const& dst, EnsembleWork*& w, int64_t* counts_host,
                               cudaStream_t stream)
{
    cudaError_t e = reserve(w, n, n_inst);
    if (e != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(w->counts, 0, sizeof(unsigned long long) * n_inst, stream)) != cudaSuccess) return e;
    if (n > 0) {
        int const g = rrea_dev::grid_of(n);
        note_launch();
        rrea_dev::tile_keys_kernel<<<g, 256, 0, stream>>>(src.cpu, n, w->keys_in, w->vals_in, w->counts, n_inst);
        if ((e = sort_by_key(*w, n, n_inst, stream)) != cudaSuccess) return e;
        note_launch();
        rrea_dev::gather_tile_kernel<<<g, 256, 0, stream>>>(src, w->vals_out, n, dst);
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    static_assert(sizeof(unsigned long long) == sizeof(int64_t), "count width");
    e = cudaMemcpyAsync(counts_host, w->counts, sizeof(int64_t) * n_inst, cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    return e;
}

cudaError_t ensemble_retire(int64_t* id, const int32_t* cpu, int64_t n, int32_t inst, cudaStream_t stream)
{
    if (n == 0) return cudaSuccess;
    note_launch();
    rrea_dev::retire_kernel<<<rrea_dev::grid_of(n), 256, 0, stream>>>(id, cpu, n, inst);
    return cudaGetLastError();
}

}  // namespace rrea_launch
