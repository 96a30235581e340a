// Transient FIFO kernels of DrainAndCommitSecondaries
// (O/RreaSecondaryCommit.cpp:9-638): one generation chunk of FIFO items is
// advanced through its residual dt by one kernel per species, the survivors
// are compacted in FIFO order, and the ordered children are adopted into
// the FIFO tail with their root, parent index and lineage.
#include "rrea_kernels.h"

#include "device/rrea_newborn.cuh"

namespace rrea_dev {
namespace {

// Resident blocks of 128 threads per SM the newborn kernels are compiled
// for.  A drain holds few items, each a long dependent chain, so the goal is
// one wave with the fewest spills, not full residency (4 blocks, 128
// registers, measured within noise of 8 blocks, 64 registers, on the bench
// step).
#ifndef RREA_NEWBORN_MIN_BLOCKS
#define RREA_NEWBORN_MIN_BLOCKS 4
#endif

// SPECIES 1 positron, 2 photon, 0 every other species id (the reference
// advances anything that is not a photon or a positron as an electron).
template <int NP, int SPECIES>
__global__ void __launch_bounds__(128, RREA_NEWBORN_MIN_BLOCKS) newborn_kernel(const __grid_constant__ ElectronArgs A, rrea_gpu_secondary* __restrict__ items,
                                                      int64_t n, uint32_t* __restrict__ alive)
{
    StepConstants const& C = c_step;
    __shared__ IonPairSlot ion_slots[128];  // one per thread; launched with 128 threads
    for (int64_t ip = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; ip < n;
         ip += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        int const raw = items[ip].species;
        int const sp = raw == 1 ? 1 : (raw == 2 ? 2 : 0);
        if (sp != SPECIES) continue;
        rrea_gpu_secondary p = items[ip];
        if (A.segments) A.segments[ip].kind = 0;
        Err err;
        uint32_t lineage = 0;
        int res = 1;
        double const e = p.energy_eV;
        bool const certified = SPECIES == 2
            ? (isfinite(e) && e >= C.tix.photon_min_eV && e <= C.tix.photon_max_eV)
            : charged_in_range(C.tix, e);
        if (!certified) {
            err.set(RREA_GPU_ERR_RANGE);
        } else if (p.birth_fraction < 1.0) {
            if constexpr (SPECIES == 2) {
                res = advance_photon_newborn<NP>(C, A, ip, p, lineage, err);
            } else {
                IonPairCache ion_pairs;
                ion_pairs.init(ion_slots + threadIdx.x, SPECIES == 1 ? 0.0 : 0.5 * C.cfg.low_energy_cutoff_eV,
                               C.tix.w_air_eV_per_pair);
                res = advance_charged_newborn<NP, SPECIES == 1>(C, A, ip, p, lineage, ion_pairs, err);
                ion_pairs.flush(C, A.cells);
            }
        }
        // every child carries a local index below this count
        A.sec_per_parent[ip] = lineage;
        if (err.code) {
            record_failure(A, err.code, ip);
            res = 0;
        }
        alive[ip] = res == 1 ? 1u : 0u;
        if (res == 1) {
            p.birth_fraction = 1.0;
            items[ip] = p;
        }
    }
}

__global__ void compact_survivors_kernel(const rrea_gpu_secondary* __restrict__ items, const uint32_t* __restrict__ alive,
                                         const int64_t* __restrict__ offsets, int64_t n, rrea_gpu_secondary* __restrict__ out)
{
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        if (alive[i]) out[offsets[i]] = items[i];
    }
}

// The FIFO merge of one chunk's children: root key and species and the
// original parent index come from the item that spawned the child, the
// lineage from the per-root counter kept by the host.
__global__ void adopt_children_kernel(const rrea_gpu_secondary* __restrict__ ordered, int64_t n,
                                      const rrea_gpu_secondary* __restrict__ items, const uint64_t* __restrict__ lineage,
                                      rrea_gpu_secondary* __restrict__ out)
{
    for (int64_t j = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; j < n;
         j += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        rrea_gpu_secondary c = ordered[j];
        rrea_gpu_secondary const& parent = items[c.parent_index];
        c.root_key = parent.root_key;
        c.root_species = parent.root_species;
        c.parent_index = parent.parent_index;
        c.lineage = lineage[j];
        out[j] = c;
    }
}

// Payload checks of the FIFO: mode 0 the birth payloads entering it
// (O/RreaSecondaryCommit.cpp:337-373), mode 1 the final survivors at their
// transported endpoint (:480-515).  Counts the failures and keeps the
// lowest failing index.
__global__ void validate_fifo_kernel(const rrea_gpu_secondary* __restrict__ items, int64_t n, int mode,
                                     unsigned long long* __restrict__ invalid, long long* __restrict__ first)
{
    StepConstants const& C = c_step;
    rrea_gpu_config const& cfg = C.cfg;
    Geom const g{cfg.r_lo, cfg.r_hi, cfg.z_lo, cfg.z_hi, cfg.periodic_z != 0};
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        rrea_gpu_secondary const& s = items[i];
        bool const photon = s.species == 2;
        bool const known = s.species >= 0 && s.species <= 2;
        bool const finite = isfinite(s.x) && isfinite(s.y) && isfinite(s.z) && isfinite(s.dir_x) && isfinite(s.dir_y)
            && isfinite(s.dir_z) && isfinite(s.weight) && isfinite(s.energy_eV);
        bool ok;
        if (mode == 0) {
            ok = known && s.root_species >= 0 && s.root_species <= 2 && finite && isfinite(s.birth_fraction)
                && s.weight > 0.0 && (photon ? s.energy_eV > 0.0 : s.energy_eV >= 0.0) && !(s.birth_fraction < 0.0)
                && !(s.birth_fraction > 1.0) && s.lineage < kLineageCap;
        } else {
            bool const certified = photon ? (s.energy_eV >= C.tix.photon_min_eV && s.energy_eV <= C.tix.photon_max_eV)
                                          : charged_in_range(C.tix, s.energy_eV);
            ok = known && finite && s.weight > 0.0
                && (photon ? s.energy_eV > 0.0 : s.energy_eV >= cfg.low_energy_cutoff_eV) && certified
                && cartesian_half_open(g, s.x, s.y, s.z);
        }
        if (!ok) {
            atomicAdd(invalid, 1ULL);
            atomicMin(first, static_cast<long long>(i));
        }
    }
}

// The roots and lineages of the initial FIFO items, 16 B per item
// (root key; root species << 32 | lineage), for the host's lineage counters.
__global__ void gather_roots_kernel(const rrea_gpu_secondary* __restrict__ items, int64_t n,
                                    unsigned long long* __restrict__ out)
{
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        out[2 * i] = items[i].root_key;
        out[2 * i + 1] = (static_cast<unsigned long long>(static_cast<uint32_t>(items[i].root_species)) << 32)
            | static_cast<uint32_t>(items[i].lineage);
    }
}

int grid_for(int64_t n, int cap)
{
    int64_t const b = (n + 127) / 128;
    return static_cast<int>(b < 1 ? 1 : (b > cap ? cap : b));
}

}  // namespace
}  // namespace rrea_dev

namespace rrea_launch {

cudaError_t newborn_constants(rrea_dev::StepConstants const& sc, cudaStream_t stream)
{
    return cudaMemcpyToSymbolAsync(rrea_dev::c_step, &sc, sizeof(sc), 0, cudaMemcpyHostToDevice, stream);
}

cudaError_t validate_fifo(const rrea_gpu_secondary* items, int64_t n, int mode, unsigned long long* invalid,
                          long long* first, cudaStream_t stream)
{
    if (n <= 0) return cudaSuccess;
    note_launch();
    rrea_dev::validate_fifo_kernel<<<rrea_dev::grid_for(n, 65535), 128, 0, stream>>>(items, n, mode, invalid, first);
    return cudaGetLastError();
}

cudaError_t newborn_step(rrea_dev::ElectronArgs const& args, rrea_gpu_secondary* items, int64_t n, uint32_t* alive,
                         int max_blocks, bool periodic, cudaStream_t stream, cudaStream_t const side[2],
                         cudaEvent_t fork, cudaEvent_t const join[2])
{
    using namespace rrea_dev;
    if (n <= 0) return cudaSuccess;
    int const blocks = grid_for(n, max_blocks);
    for (int k = 0; k < 3; ++k) note_launch();
    // The species kernels touch disjoint items, so the positron and photon
    // ones run beside the electron one; each is a short wave whose length is
    // its longest item, and side by side their latencies overlap.
    cudaStream_t s1 = stream, s2 = stream;
    if (side && fork && join) {
        cudaError_t e = cudaEventRecord(fork, stream);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(side[0], fork, 0);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(side[1], fork, 0);
        if (e != cudaSuccess) return e;
        s1 = side[0];
        s2 = side[1];
    }
    if (periodic) {
        newborn_kernel<4, 0><<<blocks, 128, 0, stream>>>(args, items, n, alive);
        newborn_kernel<4, 1><<<blocks, 128, 0, s1>>>(args, items, n, alive);
        newborn_kernel<4, 2><<<blocks, 128, 0, s2>>>(args, items, n, alive);
    } else {
        newborn_kernel<1, 0><<<blocks, 128, 0, stream>>>(args, items, n, alive);
        newborn_kernel<1, 1><<<blocks, 128, 0, s1>>>(args, items, n, alive);
        newborn_kernel<1, 2><<<blocks, 128, 0, s2>>>(args, items, n, alive);
    }
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && s1 != stream) {
        e = cudaEventRecord(join[0], s1);
        if (e == cudaSuccess) e = cudaEventRecord(join[1], s2);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(stream, join[0], 0);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(stream, join[1], 0);
    }
    return e;
}

cudaError_t gather_roots(const rrea_gpu_secondary* items, int64_t n, unsigned long long* out, cudaStream_t stream)
{
    if (n <= 0) return cudaSuccess;
    note_launch();
    rrea_dev::gather_roots_kernel<<<rrea_dev::grid_for(n, 65535), 128, 0, stream>>>(items, n, out);
    return cudaGetLastError();
}

cudaError_t compact_survivors(const rrea_gpu_secondary* items, const uint32_t* alive, const int64_t* offsets,
                              int64_t n, rrea_gpu_secondary* out, cudaStream_t stream)
{
    if (n <= 0) return cudaSuccess;
    note_launch();
    rrea_dev::compact_survivors_kernel<<<rrea_dev::grid_for(n, 65535), 128, 0, stream>>>(items, alive, offsets, n,
                                                                                          out);
    return cudaGetLastError();
}

cudaError_t adopt_children(const rrea_gpu_secondary* ordered, int64_t n, const rrea_gpu_secondary* items,
                           const uint64_t* lineage, rrea_gpu_secondary* out, cudaStream_t stream)
{
    if (n <= 0) return cudaSuccess;
    note_launch();
    rrea_dev::adopt_children_kernel<<<rrea_dev::grid_for(n, 65535), 128, 0, stream>>>(ordered, n, items, lineage,
                                                                                       out);
    return cudaGetLastError();
}

}  // namespace rrea_launch
