// rrea_gpu_order_secondaries_noalloc: the deterministic secondary-ordering
// pass (exclusive scan of per-parent counts, then scatter to
// offset[parent] + lineage) on caller-owned device buffers, with its
// scratch in a file-scope device array instead of allocated memory.
//
// Scratch layout (int64 words, one array per device, loaded with this
// library's device image):
//   [0, kMaxParents)                      per-parent offsets
//   [kMaxParents, kMaxParents + kBlocks)  scan block sums
//   [kMaxParents + kBlocks]               consistency error word
// Offsets and block sums are written before they are read on every call,
// so neither needs to start at zero.  The error word must be zero when the
// scatter starts; each call clears it itself before launching.
//
// The scatter claims each output slot with a compare-and-swap on the
// record's parent_index word, after a first pass has set that word to -1 in
// every output slot (the output is the caller's buffer and needs no
// initialisation).  A second record aimed at a claimed slot is a duplicated
// (parent_index, lineage) pair: it is reported, never written.  With the
// counts summing to n_secondaries, every record landing inside the output
// and no slot claimed twice, every output slot is written exactly once.
#include "../../include/rrea_gpu.h"

#include "rrea_kernels.h"

#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>

namespace {

constexpr int64_t kMaxParents = RREA_GPU_NOALLOC_MAX_PARENTS;
constexpr int64_t kScanBlock = 1024;
constexpr int64_t kBlocks = (kMaxParents + kScanBlock - 1) / kScanBlock + 1;
constexpr int64_t kScratchWords = kMaxParents + kBlocks + 8;

static __device__ __align__(256) int64_t g_order_scratch[kScratchWords];

// Marks every output slot unclaimed (parent_index = -1).
__global__ void unclaim_slots_kernel(rrea_gpu_secondary* __restrict__ out, int64_t count)
{
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < count;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        out[i].parent_index = -1;
    }
}

// Scatter with the checks the internal pass does not need (its inputs are
// produced by the transport kernel): every record must name a parent in
// [0, n), carry a lineage below that parent's count, and land inside
// [0, count); the counts must sum to count.  A violating record is skipped
// and the error word records the first violation kind.
__global__ void scatter_checked_kernel(const rrea_gpu_secondary* __restrict__ in, int64_t count,
                                       const uint32_t* __restrict__ counts, int64_t n,
                                       const int64_t* __restrict__ offsets, rrea_gpu_secondary* __restrict__ out,
                                       unsigned long long* __restrict__ err)
{
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        int64_t const total = n > 0 ? offsets[n - 1] + static_cast<int64_t>(counts[n - 1]) : 0;
        if (total != count) atomicCAS(err, 0ULL, 1ULL);
    }
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < count;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        rrea_gpu_secondary const s = in[i];
        int64_t const p = s.parent_index;
        if (p < 0 || p >= n) {
            atomicCAS(err, 0ULL, 2ULL);
            continue;
        }
        if (s.lineage >= static_cast<uint64_t>(counts[p])) {
            atomicCAS(err, 0ULL, 3ULL);
            continue;
        }
        int64_t const dst = offsets[p] + static_cast<int64_t>(s.lineage);
        if (dst < 0 || dst >= count) {
            atomicCAS(err, 0ULL, 4ULL);
            continue;
        }
        auto* const claim = reinterpret_cast<unsigned long long*>(&out[dst].parent_index);
        if (atomicCAS(claim, ~0ULL, static_cast<unsigned long long>(p)) != ~0ULL) {
            atomicCAS(err, 0ULL, 5ULL);
            continue;
        }
        out[dst] = s;
    }
}

rrea_gpu_status report(char* message, size_t size, rrea_gpu_status s, char const* text)
{
    if (message && size > 0) {
        std::strncpy(message, text, size - 1);
        message[size - 1] = '\0';
    }
    return s;
}

}  // namespace

extern "C" rrea_gpu_status rrea_gpu_order_secondaries_noalloc(const uint32_t* d_counts, int64_t n_parents,
                                                              const rrea_gpu_secondary* d_unordered,
                                                              int64_t n_secondaries, rrea_gpu_secondary* d_ordered,
                                                              void* stream, char* message, size_t message_size)
{
    char text[256];
    if (message && message_size > 0) message[0] = '\0';
    if (n_parents < 0 || n_secondaries < 0) {
        return report(message, message_size, RREA_GPU_ERR_ARGUMENT, "negative size");
    }
    if (n_parents > kMaxParents) {
        std::snprintf(text, sizeof(text),
                      "n_parents = %lld exceeds the fixed scratch of this entry point (at most %lld parents "
                      "per call); split the tile or use rrea_gpu_apply_electrons",
                      static_cast<long long>(n_parents), static_cast<long long>(kMaxParents));
        return report(message, message_size, RREA_GPU_ERR_CAPACITY, text);
    }
    if ((n_parents > 0 && !d_counts) || (n_secondaries > 0 && (!d_unordered || !d_ordered))) {
        return report(message, message_size, RREA_GPU_ERR_ARGUMENT, "null device buffer");
    }
    if (n_secondaries > 0) {
        auto const a = reinterpret_cast<uintptr_t>(d_unordered);
        auto const b = reinterpret_cast<uintptr_t>(d_ordered);
        uintptr_t const bytes = static_cast<uintptr_t>(n_secondaries) * sizeof(rrea_gpu_secondary);
        if (a < b + bytes && b < a + bytes) {
            return report(message, message_size, RREA_GPU_ERR_ARGUMENT, "input and output secondaries overlap");
        }
    }
    if (n_parents == 0 && n_secondaries > 0) {
        return report(message, message_size, RREA_GPU_ERR_INVALID_STATE, "secondaries without parents");
    }
    if (n_parents == 0) return RREA_GPU_OK;

    // The array's device address is looked up on every call, with the
    // caller's device and context current: a cached address would go stale
    // after cudaDeviceReset or under another context on the same device.
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_order_scratch);
    if (e != cudaSuccess || !p) {
        std::snprintf(text, sizeof(text), "cudaGetSymbolAddress: %s",
                      e != cudaSuccess ? cudaGetErrorString(e) : "null address");
        return report(message, message_size, RREA_GPU_ERR_CUDA, text);
    }
    int64_t* const scratch = static_cast<int64_t*>(p);
    int64_t* const offsets = scratch;
    int64_t* const block_sums = scratch + kMaxParents;
    auto* const err_word = reinterpret_cast<unsigned long long*>(scratch + kMaxParents + kBlocks);
    cudaStream_t const s = static_cast<cudaStream_t>(stream);

    e = cudaMemsetAsync(err_word, 0, sizeof(unsigned long long), s);
    if (e == cudaSuccess) e = rrea_launch::exclusive_scan_counts(d_counts, n_parents, offsets, block_sums, s);
    int const threads = 256;
    int64_t blocks = (n_secondaries + threads - 1) / threads;
    if (blocks < 1) blocks = 1;
    if (blocks > 65535) blocks = 65535;
    if (e == cudaSuccess && n_secondaries > 0) {
        rrea_launch::note_launch();
        unclaim_slots_kernel<<<static_cast<unsigned>(blocks), threads, 0, s>>>(d_ordered, n_secondaries);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        rrea_launch::note_launch();
        scatter_checked_kernel<<<static_cast<unsigned>(blocks), threads, 0, s>>>(
            d_unordered, n_secondaries, d_counts, n_parents, offsets, d_ordered, err_word);
        e = cudaGetLastError();
    }
    unsigned long long flag = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&flag, err_word, sizeof(flag), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        std::snprintf(text, sizeof(text), "CUDA: %s", cudaGetErrorString(e));
        return report(message, message_size, RREA_GPU_ERR_CUDA, text);
    }
    if (flag != 0) {
        static char const* const why[] = {
            "", "per-parent counts do not sum to n_secondaries", "a record's parent_index is outside [0, n_parents)",
            "a record's lineage is not below its parent's count", "a record's destination is outside the output",
            "two records share one (parent_index, lineage) pair"};
        std::snprintf(text, sizeof(text), "inconsistent input: %s (offending records were skipped)",
                      why[flag < 6 ? flag : 0]);
        return report(message, message_size, RREA_GPU_ERR_INVALID_STATE, text);
    }
    return RREA_GPU_OK;
}
