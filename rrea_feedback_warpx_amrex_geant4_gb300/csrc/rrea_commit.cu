// Resident-mode commit of the transient FIFO's survivors into the species
// tiles, and the stable compaction of a tile's invalid particles.
//
// The commit restates the particle-creation half of
// DrainAndCommitSecondaries: RreaWarpXCoupling::CommitLocalParticleBatch
// (O/RreaCouplingSources.cpp:240-330) turns each surviving record into a
// WarpX particle (proper velocity from the kinetic energy along the record's
// direction for e-/e+, photon momentum E along it), and
// append_rrea_previous_position_attributes (:28-100) sets the captured
// pre-push state to the new particle's own state.  Records with weight <= 0,
// and photons with energy <= 0, are dropped as there.  Ids are assigned in
// FIFO order per species from a per-species counter (AMReX's NextID lives in
// the absent AMReX sources; this is the rule the oracle uses too).
//
// The compaction is what WarpX's removal of invalid particles does to the
// tile between steps: valid particles keep their order.
#include "rrea_kernels.h"

#include <cuda_runtime.h>

namespace rrea_dev {
namespace {

constexpr double kCommitMeC2 = 510998.95000;  // I/RreaConstants.H:9
constexpr double kCommitC = 299792458.0;      // I/RreaConstants.H:10

__device__ __forceinline__ bool commit_accepts(rrea_gpu_secondary const& s, int species)
{
    return s.species == species && s.weight > 0.0 && (species != RREA_SPECIES_PHOTON || s.energy_eV > 0.0);
}

__global__ void commit_flags_kernel(const rrea_gpu_secondary* __restrict__ surv, int64_t n, int species,
                                    uint32_t* __restrict__ flags)
{
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        flags[i] = commit_accepts(surv[i], species) ? 1u : 0u;
    }
}

// Appends accepted records of `species` at tile index base + offsets[i],
// with ids first_id + offsets[i] on cpu 0, or (ensemble mode, ids given)
// the per-instance ids on the root's instance.
__global__ void commit_scatter_kernel(const rrea_gpu_secondary* __restrict__ surv, int64_t n, int species,
                                      const int64_t* __restrict__ offsets, TileColumns t, int64_t base,
                                      int64_t first_id, const int64_t* __restrict__ ids)
{
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        rrea_gpu_secondary const s = surv[i];
        if (!commit_accepts(s, species)) continue;
        int64_t const k = base + offsets[i];
        double px = s.dir_x, py = s.dir_y, pz = s.dir_z;
        double const norm = sqrt(px * px + py * py + pz * pz);
        if (species == RREA_SPECIES_PHOTON) {
            // O/RreaCouplingSources.cpp:286-295
            double const scale = norm > 0.0 ? s.energy_eV / norm : s.energy_eV;
            px = s.dir_x * scale;
            py = s.dir_y * scale;
            pz = norm > 0.0 ? s.dir_z * scale : s.energy_eV;
        } else if (s.energy_eV > 0.0) {
            // :296-306 with RreaElectronProperVelocityFromKineticEv (I/RreaSeedSchedule.H:31-43)
            double const gamma = 1.0 + s.energy_eV / kCommitMeC2;
            double const u_mag = kCommitC * sqrt(fmax(__dmul_rn(gamma, gamma) - 1.0, 0.0));
            if (norm > 0.0) {
                px = u_mag * px / norm;
                py = u_mag * py / norm;
                pz = u_mag * pz / norm;
            } else {
                px = 0.0;
                py = 0.0;
                pz = u_mag;
            }
        }
        double const r = hypot(s.x, s.y);
        double const th = atan2(s.y, s.x);
        double const v[kTileColumns] = {r, s.z, th, px, py, pz, s.weight, r, s.z, th, px, py, pz};
#pragma unroll
        for (int f = 0; f < kTileColumns; ++f) t.d[f][k] = v[f];
        t.id[k] = ids ? ids[i] : first_id + offsets[i];
        t.cpu[k] = ids ? static_cast<int32_t>(s.root_key >> 40) : 0;
    }
}

__global__ void valid_flags_kernel(const int64_t* __restrict__ id, int64_t n, uint32_t* __restrict__ flags)
{
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        flags[i] = id[i] > 0 ? 1u : 0u;
    }
}

__global__ void compact_tile_kernel(TileColumns src, int64_t n, const int64_t* __restrict__ offsets, TileColumns dst)
{
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        int64_t const id = src.id[i];
        if (id <= 0) continue;
        int64_t const k = offsets[i];
#pragma unroll
        for (int f = 0; f < kTileColumns; ++f) dst.d[f][k] = src.d[f][i];
        dst.id[k] = id;
        dst.cpu[k] = src.cpu[i];
    }
}

// Scheduling order of a charged tile: particles binned by |u|^2 in
// quarter octaves (the exponent and top two mantissa bits of the double, an
// integer key), lowest momentum first.  Slow low-energy particles (many
// GS-limited substeps) then start first and share warps with particles of
// a similar substep count; ended particles (id <= 0) go last.  The order
// only schedules: every result is indexed by the particle's tile index.
constexpr int kCostBins = 128;

__device__ __forceinline__ int cost_bin(double ux, double uy, double uz, int64_t id)
{
    if (id <= 0) return kCostBins - 1;
    unsigned long long const b = static_cast<unsigned long long>(__double_as_longlong(ux * ux + uy * uy + uz * uz));
    // |u|^2 of 10 keV is 2^51.7 (m/s)^2 and of 20 MeV 2^66.9: bins from 2^48
    int const key = static_cast<int>(b >> 50) - 4 * (1023 + 48);
    return key < 0 ? 0 : (key > kCostBins - 2 ? kCostBins - 2 : key);
}

__global__ void cost_hist_kernel(const double* __restrict__ ux, const double* __restrict__ uy,
                                 const double* __restrict__ uz, const int64_t* __restrict__ id, int64_t n,
                                 uint32_t* __restrict__ hist)
{
    __shared__ uint32_t local[kCostBins];
    for (int i = threadIdx.x; i < kCostBins; i += blockDim.x) local[i] = 0;
    __syncthreads();
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        atomicAdd(&local[cost_bin(ux[i], uy[i], uz[i], id[i])], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kCostBins; i += blockDim.x) {
        if (local[i]) atomicAdd(&hist[i], local[i]);
    }
}

// hist[0, kCostBins) counts, cursor[kCostBins, 2 kCostBins) zeroed slots
__global__ void cost_scatter_kernel(const double* __restrict__ ux, const double* __restrict__ uy,
                                    const double* __restrict__ uz, const int64_t* __restrict__ id, int64_t n,
                                    uint32_t* __restrict__ hist, uint32_t* __restrict__ order)
{
    __shared__ uint32_t start[kCostBins];
    if (threadIdx.x == 0) {
        uint32_t acc = 0;
        for (int i = 0; i < kCostBins; ++i) {
            start[i] = acc;
            acc += hist[i];
        }
    }
    __syncthreads();
    uint32_t* cursor = hist + kCostBins;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        int const bin = cost_bin(ux[i], uy[i], uz[i], id[i]);
        order[start[bin] + atomicAdd(&cursor[bin], 1u)] = static_cast<uint32_t>(i);
    }
}

unsigned grid_for(int64_t n, int threads)
{
    int64_t const b = (n + threads - 1) / threads;
    return static_cast<unsigned>(b < 65535 ? (b > 0 ? b : 1) : 65535);
}

}  // namespace
}  // namespace rrea_dev

namespace rrea_launch {

cudaError_t commit_rank(const rrea_gpu_secondary* surv, int64_t n, int species, uint32_t* flags, int64_t* offsets,
                        int64_t* scan_scratch, cudaStream_t stream)
{
    if (n <= 0) return cudaSuccess;
    note_launch();
    rrea_dev::commit_flags_kernel<<<rrea_dev::grid_for(n, 256), 256, 0, stream>>>(surv, n, species, flags);
    return exclusive_scan_counts(flags, n, offsets, scan_scratch, stream);
}

cudaError_t commit_scatter(const rrea_gpu_secondary* surv, int64_t n, int species, const int64_t* offsets,
                           rrea_dev::TileColumns const& tile, int64_t base, int64_t first_id, const int64_t* ids,
                           cudaStream_t stream)
{
    if (n <= 0) return cudaSuccess;
    note_launch();
    rrea_dev::commit_scatter_kernel<<<rrea_dev::grid_for(n, 128), 128, 0, stream>>>(surv, n, species, offsets, tile,
                                                                                   base, first_id, ids);
    return cudaGetLastError();
}

cudaError_t compact_tile(rrea_dev::TileColumns const& src, int64_t n, uint32_t* flags, int64_t* offsets,
                         int64_t* scan_scratch, rrea_dev::TileColumns const& dst, cudaStream_t stream)
{
    if (n <= 0) return cudaSuccess;
    note_launch();
    rrea_dev::valid_flags_kernel<<<rrea_dev::grid_for(n, 256), 256, 0, stream>>>(src.id, n, flags);
    cudaError_t const e = exclusive_scan_counts(flags, n, offsets, scan_scratch, stream);
    if (e != cudaSuccess) return e;
    note_launch();
    rrea_dev::compact_tile_kernel<<<rrea_dev::grid_for(n, 256), 256, 0, stream>>>(src, n, offsets, dst);
    return cudaGetLastError();
}

int cost_order_scratch_elems() { return 2 * rrea_dev::kCostBins; }

cudaError_t cost_order(const double* ux, const double* uy, const double* uz, const int64_t* id, int64_t n,
                       uint32_t* scratch, uint32_t* order, int blocks, cudaStream_t stream)
{
    if (n <= 0) return cudaSuccess;
    cudaError_t const e = cudaMemsetAsync(scratch, 0, sizeof(uint32_t) * 2 * rrea_dev::kCostBins, stream);
    if (e != cudaSuccess) return e;
    note_launch();
    rrea_dev::cost_hist_kernel<<<blocks, 256, 0, stream>>>(ux, uy, uz, id, n, scratch);
    note_launch();
    rrea_dev::cost_scatter_kernel<<<blocks, 256, 0, stream>>>(ux, uy, uz, id, n, scratch, order);
    return cudaGetLastError();
}

}  // namespace rrea_launch
