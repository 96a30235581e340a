// Adaptive population control (adaptive_resample_v1) of one charged species
// on the device: the global thinning plan of
// RreaWarpXCoupling::PreflightAndApplySecondaryPopulationControl
// (O/RreaCouplingPopulation.cpp:175-640) and the split refill of
// AdaptiveResampleOneSpecies (:686-767), for a single rank.
//
// Thinning, over the live particles of the species and the transaction's
// staged candidates (the drain survivors not yet committed):
//   1. every member becomes a record: its order-1 CIC support (the cell-
//      centred cell below-left of it), the fractions inside it, a phase bin
//      (the exponent of |u| and the signs of u_r, u_theta, u_z), its weight,
//      whether it is a candidate, and its stable identity (live: the packed
//      id/cpu word; candidate: root RNG particle id and lineage/root species);
//   2. the records are sorted by (support_r, support_z, phase, candidate,
//      identity high, identity low): three stable radix passes, least
//      significant key first;
//   3. each support's removal capacity is its live count minus the rank of
//      its CIC columns (RreaCicResampleRemovalCapacity);
//   4. when the members exceed 1.25 x target, the nominal request
//      min(members - target, total capacity) is handed out to the supports
//      in sorted order, each up to its capacity;
//   5. each support with a request thins its records in sorted order with
//      RreaThinCicWeights (RreaPlanGlobalCicThinning,
//      I/RreaCicConservingResample.H:489-640), its uniforms
//      RreaAdaptiveResampleCicUniform(seed, group id ^ salt, step, k) on the
//      species' channel, and its four cell moments are rechecked
//      (RreaRoundAndVerifyCicWeights);
//   6. the new weights go back: a live particle at weight zero is
//      invalidated, a candidate keeps its record with the new weight (zero
//      drops it at the commit).
// One thread per support runs steps 3 and 5; the records, sort, scans and
// scatters are one thread per member.
#include "rrea_kernels.h"

#include "device/rrea_electron_args.cuh"
#include "device/rrea_resample.cuh"

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

namespace rrea_dev {
namespace {

constexpr uint64_t kStreamElectron = 0x656c656374726f6eULL;  // "electron"
constexpr uint64_t kStreamPositron = 0x706f736974726f6eULL;  // "positron"
constexpr uint64_t kChResampleElectron = 131;                // AdaptiveResampleCicElectron, O/RreaRng.H:96
constexpr uint64_t kChResamplePositron = 132;
constexpr int kSupportBias = 32768;

__device__ __forceinline__ uint64_t support_key(int sr, int sz, uint64_t stream_key)
{
    // RreaGlobalCicSupportKey, I/RreaCicConservingResample.H:421-429
    uint64_t const cells = (static_cast<uint64_t>(static_cast<uint32_t>(sr)) << 32) | static_cast<uint32_t>(sz);
    return cic_mix64(cells ^ cic_mix64(stream_key));
}

__global__ void flags_live_kernel(const int64_t* __restrict__ id, int64_t n, uint32_t* __restrict__ flags)
{
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        flags[i] = id[i] > 0 ? 1u : 0u;
    }
}

__global__ void flags_cand_kernel(const rrea_gpu_secondary* __restrict__ c, int64_t n, int species,
                                  uint32_t* __restrict__ flags)
{
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        flags[i] = (c[i].species == species && c[i].weight > 0.0) ? 1u : 0u;
    }
}

__global__ void scatter_members_kernel(const uint32_t* __restrict__ flags, const int64_t* __restrict__ offsets,
                                       int64_t n, int64_t base, int64_t* __restrict__ members)
{
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        if (flags[i]) members[base + offsets[i]] = i;
    }
}

// The record of every member (O/RreaCouplingPopulation.cpp:230-290).
__global__ void records_kernel(rrea_launch::PopulationInput in, const int64_t* __restrict__ members,
                               int64_t n_live, int64_t n_members, uint64_t* __restrict__ k1,
                               uint64_t* __restrict__ k2, uint64_t* __restrict__ k3, uint32_t* __restrict__ perm,
                               double* __restrict__ fr, double* __restrict__ fz, double* __restrict__ w,
                               int* __restrict__ status, uint64_t* __restrict__ k0 = nullptr)
{
    double constexpr me_c2 = 510998.95000;  // I/RreaConstants.H:9
    double constexpr c_light = 299792458.0;  // I/RreaConstants.H:10
    for (int64_t m = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; m < n_members;
         m += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        int64_t const src = members[m];
        double r, z, th, ux, uy, uz, wt;
        uint64_t high, low, inst;
        uint32_t cand;
        if (m < n_live) {
            r = in.r[src];
            z = in.z[src];
            th = in.theta[src];
            ux = in.ux[src];
            uy = in.uy[src];
            uz = in.uz[src];
            wt = in.w[src];
            high = 0;
            // the particle's packed id/cpu word (40-bit id above the 24-bit cpu)
            low = (static_cast<uint64_t>(in.id[src]) << 24) | static_cast<uint32_t>(in.cpu ? in.cpu[src] & 0xffffff : 0);
            inst = in.cpu ? static_cast<uint64_t>(static_cast<uint32_t>(in.cpu[src])) : 0;
            cand = 0;
        } else {
            rrea_gpu_secondary const s = in.cand[src];
            double const gamma = 1.0 + s.energy_eV / me_c2;
            double const u = c_light * sqrt(fmax(__dmul_rn(gamma, gamma) - 1.0, 0.0));
            r = hypot(s.x, s.y);
            z = s.z;
            th = atan2(s.y, s.x);
            ux = u * s.dir_x;
            uy = u * s.dir_y;
            uz = u * s.dir_z;
            wt = s.weight;
            high = s.root_key;
            low = (s.lineage << 2) | static_cast<uint64_t>(static_cast<uint32_t>(s.root_species));
            inst = s.root_key >> 40;
            cand = 1;
        }
        if (in.periodic_z) {
            double const length = in.z_hi - in.z_lo;
            double shifted = fmod(z - in.z_lo, length);
            if (shifted < 0.0) shifted += length;
            z = in.z_lo + shifted;
        }
        double const rc = (r - in.r_lo) / in.dr - 0.5;
        double const zc = (z - in.z_lo) / in.dz - 0.5;
        double const i0 = floor(rc), j0 = floor(zc);
        if (!isfinite(rc) || !isfinite(zc) || !(i0 >= -kSupportBias) || !(i0 < kSupportBias) ||
            !(j0 >= -kSupportBias) || !(j0 < kSupportBias)) {
            atomicCAS(status, 0, RREA_GPU_ERR_GEOMETRY);
            continue;
        }
        // phase bin: exponent of |u| and the signs of u_r, u_theta, u_z
        double s_th, c_th;
        sincos(th, &s_th, &c_th);
        double const ur = __dadd_rn(__dmul_rn(ux, c_th), __dmul_rn(uy, s_th));
        double const ut = __dadd_rn(__dmul_rn(-ux, s_th), __dmul_rn(uy, c_th));
        double const mag = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(ux, ux), __dmul_rn(uy, uy)), __dmul_rn(uz, uz)));
        int ex = (mag > 0.0 && isfinite(mag)) ? ilogb(mag) : -1024;
        ex = max(-1024, min(1023, ex));
        uint32_t const phase = static_cast<uint32_t>((ex + 1024) * 8 + (ur >= 0.0 ? 1 : 0) + (ut >= 0.0 ? 2 : 0) +
                                                     (uz >= 0.0 ? 4 : 0));
        k1[m] = (static_cast<uint64_t>(static_cast<int>(i0) + kSupportBias) << 48) |
                (static_cast<uint64_t>(static_cast<int>(j0) + kSupportBias) << 32) |
                (static_cast<uint64_t>(phase) << 1) | cand;
        k2[m] = high;
        k3[m] = low;
        if (k0) k0[m] = inst;
        perm[m] = static_cast<uint32_t>(m);
        fr[m] = rc - i0;
        fz[m] = zc - j0;
        w[m] = wt;
    }
}

__global__ void gather_u64_kernel(const uint64_t* __restrict__ src, const uint32_t* __restrict__ perm, int64_t n,
                                  uint64_t* __restrict__ dst)
{
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        dst[i] = src[perm[i]];
    }
}

// Sorted copies of the records and the support heads.
__global__ void sorted_kernel(const uint32_t* __restrict__ perm, int64_t n, const uint64_t* __restrict__ k1s,
                              const uint64_t* __restrict__ k2, const uint64_t* __restrict__ k3,
                              const double* __restrict__ fr, const double* __restrict__ fz,
                              const double* __restrict__ w, double* __restrict__ sfr, double* __restrict__ sfz,
                              double* __restrict__ sw, double* __restrict__ sw0, uint64_t* __restrict__ k2s,
                              uint64_t* __restrict__ k3s, uint32_t* __restrict__ heads)
{
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        uint32_t const m = perm[i];
        sfr[i] = fr[m];
        sfz[i] = fz[m];
        sw[i] = w[m];
        sw0[i] = w[m];
        k2s[i] = k2[m];
        k3s[i] = k3[m];
        heads[i] = (i == 0 || (k1s[i] >> 32) != (k1s[i - 1] >> 32)) ? 1u : 0u;
    }
}

__global__ void group_begin_kernel(const uint32_t* __restrict__ heads, const int64_t* __restrict__ offsets,
                                   int64_t n, int64_t* __restrict__ begin)
{
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        if (heads[i]) begin[offsets[i]] = i;
    }
}

// Removal capacity per support: live members minus the rank of their CIC columns.
__global__ void group_capacity_kernel(const int64_t* __restrict__ begin, int64_t groups, int64_t n,
                                      const double* __restrict__ sfr, const double* __restrict__ sfz,
                                      const double* __restrict__ sw, int64_t* __restrict__ capacity)
{
    for (int64_t g = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; g < groups;
         g += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        int64_t const b = begin[g];
        int64_t const e = g + 1 < groups ? begin[g + 1] : n;
        int64_t live = 0;
        for (int64_t i = b; i < e; ++i) live += sw[i] > 0.0 ? 1 : 0;
        int const rank = cic_constraint_rank_any(sfr + b, sfz + b, sw + b, e - b);
        capacity[g] = live > rank ? live - rank : 0;
    }
}

struct ResampleDraw {
    RngStream rng;
    uint64_t channel;
    __device__ double operator()(uint64_t k) const { return rng.uniform(k, channel); }
};

// Thinning of every support with a request (RreaPlanGlobalCicThinning on one
// support, O/RreaCouplingPopulation.cpp:452-478).
__global__ void group_thin_kernel(rrea_launch::PopulationInput in, const int64_t* __restrict__ begin, int64_t groups,
                                  int64_t n, const uint64_t* __restrict__ k1s, const uint64_t* __restrict__ k2s,
                                  const uint64_t* __restrict__ k3s, const double* __restrict__ sfr,
                                  const double* __restrict__ sfz, double* __restrict__ sw,
                                  const double* __restrict__ sw0, const int64_t* __restrict__ capacity,
                                  const int64_t* __restrict__ cap_prefix, int64_t nominal,
                                  unsigned long long* __restrict__ removed, int* __restrict__ status)
{
    uint64_t const stream_key = in.species == RREA_SPECIES_POSITRON ? kStreamPositron : kStreamElectron;
    uint64_t const channel = in.species == RREA_SPECIES_POSITRON ? kChResamplePositron : kChResampleElectron;
    for (int64_t g = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; g < groups;
         g += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        int64_t const left = nominal - cap_prefix[g];
        int64_t const request = left <= 0 ? 0 : (left < capacity[g] ? left : capacity[g]);
        if (request == 0) continue;
        int64_t const b = begin[g];
        int64_t const e = g + 1 < groups ? begin[g + 1] : n;
        uint64_t const key1 = k1s[b];
        int const sr = static_cast<int>(key1 >> 48) - kSupportBias;
        int const sz = static_cast<int>((key1 >> 32) & 0xffffu) - kSupportBias;
        uint64_t const id = cic_mix64(support_key(sr, sz, stream_key) ^ cic_mix64(k2s[b]) ^ cic_mix64(k3s[b]) ^
                                      (key1 & 1u));
        ResampleDraw draw;
        draw.rng.init(in.rng_seed, id ^ in.salt, static_cast<uint64_t>(in.step));
        draw.channel = channel;
        CicThinResult const r = cic_thin_window(sfr + b, sfz + b, sw + b, e - b, request, draw);
        if (!r.valid || r.removed == 0 || !cic_moments_kept(sfr + b, sfz + b, sw0 + b, sw + b, e - b)) {
            atomicCAS(status, 0, RREA_GPU_ERR_INVALID_STATE);
            continue;
        }
        atomicAdd(removed, static_cast<unsigned long long>(r.removed));
    }
}

__global__ void apply_kernel(rrea_launch::PopulationInput in, const uint32_t* __restrict__ perm,
                             const int64_t* __restrict__ members, int64_t n_live, int64_t n,
                             const double* __restrict__ sw)
{
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        uint32_t const m = perm[i];
        int64_t const src = members[m];
        double const wn = sw[i];
        if (static_cast<int64_t>(m) < n_live) {
            in.w[src] = wn;
            if (!(wn > 0.0)) in.id[src] = -in.id[src];
        } else {
            in.cand[src].weight = wn;
        }
    }
}

// Split refill (RreaAdaptiveResampleSplitOutcome, O/RreaRng.H:163-175): a
// valid particle at or above twice the floor halves its weight and an
// identical clone joins the tile end in tile order.
__global__ void split_flags_kernel(const double* __restrict__ w, const int64_t* __restrict__ id, int64_t n,
                                   double min_w, uint32_t* __restrict__ flags)
{
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        flags[i] = (id[i] > 0 && min_w > 0.0 && !(w[i] < 2.0 * min_w)) ? 1u : 0u;
    }
}

__global__ void split_scatter_kernel(TileColumns t, int64_t n, const uint32_t* __restrict__ flags,
                                     const int64_t* __restrict__ offsets, int64_t first_id)
{
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        if (!flags[i]) continue;
        double const half = 0.5 * t.d[6][i];
        t.d[6][i] = half;
        int64_t const k = n + offsets[i];
        double const v[kTileColumns] = {t.d[0][i], t.d[1][i], t.d[2][i], t.d[3][i], t.d[4][i], t.d[5][i], half,
                                        t.d[0][i], t.d[1][i], t.d[2][i], t.d[3][i], t.d[4][i], t.d[5][i]};
#pragma unroll
        for (int f = 0; f < kTileColumns; ++f) t.d[f][k] = v[f];
        t.id[k] = first_id + offsets[i];
        t.cpu[k] = t.cpu[i];
    }
}

// ---- ensemble: the plans of every instance in one pass -----------------
// Valid live rows per instance (the instance is the cpu ordinal); a
// shared-memory histogram per block when the instances fit.
__global__ void instance_members_kernel(const int64_t* __restrict__ id, const int32_t* __restrict__ cpu, int64_t n,
                                        uint32_t n_inst, bool shared_hist,
                                        unsigned long long* __restrict__ counts)
{
    extern __shared__ unsigned long long hist[];
    if (shared_hist) {
        for (uint32_t k = threadIdx.x; k < n_inst; k += blockDim.x) hist[k] = 0;
        __syncthreads();
    }
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        uint32_t const k = static_cast<uint32_t>(cpu[i]);
        if (id[i] <= 0 || k >= n_inst) continue;
        atomicAdd(shared_hist ? hist + k : counts + k, 1ULL);
    }
    if (shared_hist) {
        __syncthreads();
        for (uint32_t k = threadIdx.x; k < n_inst; k += blockDim.x) {
            if (hist[k]) atomicAdd(counts + k, hist[k]);
        }
    }
}

// Members: valid live rows of the instances due for thinning.
__global__ void flags_due_kernel(const int64_t* __restrict__ id, const int32_t* __restrict__ cpu, int64_t n,
                                 const int64_t* __restrict__ due_target, uint32_t n_inst, uint32_t* __restrict__ flags)
{
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        uint32_t const k = static_cast<uint32_t>(cpu[i]);
        flags[i] = (id[i] > 0 && k < n_inst && due_target[k] >= 0) ? 1u : 0u;
    }
}

// Sorted copies of the records and the heads of the (instance, support) groups.
__global__ void heads_instances_kernel(const uint32_t* __restrict__ perm, int64_t n, const uint64_t* __restrict__ k0s,
                                       const uint64_t* __restrict__ k1s, const uint64_t* __restrict__ k2,
                                       const uint64_t* __restrict__ k3, const double* __restrict__ fr,
                                       const double* __restrict__ fz, const double* __restrict__ w,
                                       double* __restrict__ sfr, double* __restrict__ sfz, double* __restrict__ sw,
                                       double* __restrict__ sw0, uint64_t* __restrict__ k2s,
                                       uint64_t* __restrict__ k3s, uint32_t* __restrict__ heads)
{
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        uint32_t const m = perm[i];
        sfr[i] = fr[m];
        sfz[i] = fz[m];
        sw[i] = w[m];
        sw0[i] = w[m];
        k2s[i] = k2[m];
        k3s[i] = k3[m];
        heads[i] = (i == 0 || k0s[i] != k0s[i - 1] || (k1s[i] >> 32) != (k1s[i - 1] >> 32)) ? 1u : 0u;
    }
}

// Each group's instance, the instances' capacity totals and the capacity
// prefix at each instance's first group.
__global__ void group_instances_kernel(const int64_t* __restrict__ begin, int64_t groups,
                                       const uint64_t* __restrict__ k0s, const int64_t* __restrict__ capacity,
                                       const int64_t* __restrict__ cap_prefix, uint32_t* __restrict__ ginst,
                                       unsigned long long* __restrict__ cap_per_inst, int64_t* __restrict__ inst_base)
{
    for (int64_t g = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; g < groups;
         g += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        uint64_t const k = k0s[begin[g]];
        ginst[g] = static_cast<uint32_t>(k);
        atomicAdd(cap_per_inst + k, static_cast<unsigned long long>(capacity[g]));
        if (g == 0 || k0s[begin[g - 1]] != k) inst_base[k] = cap_prefix[g];
    }
}

// The request of each due instance (RreaAdaptiveResampleAction): its
// excess over the target, at most its removal capacity.
__global__ void nominal_kernel(const unsigned long long* __restrict__ members, const unsigned long long* __restrict__ cap,
                               const int64_t* __restrict__ due_target, uint32_t n_inst, int64_t* __restrict__ nominal)
{
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n_inst; k += gridDim.x * blockDim.x) {
        int64_t const n = static_cast<int64_t>(members[k]), t = due_target[k];
        int64_t const c = static_cast<int64_t>(cap[k]);
        nominal[k] = t >= 0 ? (n - t < c ? n - t : c) : 0;
    }
}

// group_thin_kernel with the request taken from the group's instance.
__global__ void group_thin_instances_kernel(rrea_launch::PopulationInput in, const int64_t* __restrict__ begin,
                                            int64_t groups, int64_t n, const uint64_t* __restrict__ k1s,
                                            const uint64_t* __restrict__ k2s, const uint64_t* __restrict__ k3s,
                                            const double* __restrict__ sfr, const double* __restrict__ sfz,
                                            double* __restrict__ sw, const double* __restrict__ sw0,
                                            const int64_t* __restrict__ capacity,
                                            const int64_t* __restrict__ cap_prefix, const uint32_t* __restrict__ ginst,
                                            const int64_t* __restrict__ inst_base, const int64_t* __restrict__ nominal,
                                            unsigned long long* __restrict__ removed_per_inst, int* __restrict__ status)
{
    uint64_t const stream_key = in.species == RREA_SPECIES_POSITRON ? kStreamPositron : kStreamElectron;
    uint64_t const channel = in.species == RREA_SPECIES_POSITRON ? kChResamplePositron : kChResampleElectron;
    for (int64_t g = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; g < groups;
         g += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        uint32_t const k = ginst[g];
        int64_t const left = nominal[k] - (cap_prefix[g] - inst_base[k]);
        int64_t const request = left <= 0 ? 0 : (left < capacity[g] ? left : capacity[g]);
        if (request == 0) continue;
        int64_t const b = begin[g];
        int64_t const e = g + 1 < groups ? begin[g + 1] : n;
        uint64_t const key1 = k1s[b];
        int const sr = static_cast<int>(key1 >> 48) - kSupportBias;
        int const sz = static_cast<int>((key1 >> 32) & 0xffffu) - kSupportBias;
        uint64_t const id = cic_mix64(support_key(sr, sz, stream_key) ^ cic_mix64(k2s[b]) ^ cic_mix64(k3s[b]) ^
                                      (key1 & 1u));
        ResampleDraw draw;
        draw.rng.init(in.rng_seed, id ^ in.salt, static_cast<uint64_t>(in.step));
        draw.channel = channel;
        CicThinResult const r = cic_thin_window(sfr + b, sfz + b, sw + b, e - b, request, draw);
        if (!r.valid || r.removed == 0 || !cic_moments_kept(sfr + b, sfz + b, sw0 + b, sw + b, e - b)) {
            atomicCAS(status, 0, RREA_GPU_ERR_INVALID_STATE);
            continue;
        }
        atomicAdd(removed_per_inst + k, static_cast<unsigned long long>(r.removed));
    }
}

// apply_kernel for the members of instances with a request.
__global__ void apply_instances_kernel(rrea_launch::PopulationInput in, const uint32_t* __restrict__ perm,
                                       const int64_t* __restrict__ members, int64_t n,
                                       const double* __restrict__ sw, const uint64_t* __restrict__ k0s,
                                       const int64_t* __restrict__ nominal)
{
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        if (nominal[k0s[i]] <= 0) continue;
        int64_t const src = members[perm[i]];
        double const wn = sw[i];
        in.w[src] = wn;
        if (!(wn > 0.0)) in.id[src] = -in.id[src];
    }
}

int blocks_for(int64_t n)
{
    int64_t b = (n + 255) / 256;
    return static_cast<int>(b < 1 ? 1 : (b > 65535 ? 65535 : b));
}

// ---------------------------------------------------------------------------
// Weight-doubling merge above the cap (a policy of this library: the
// reference has strict_abort_v1 and adaptive_resample_v1 only).  Live
// particles are grouped by (cell, |u| quarter octave, sign of u_z); inside a
// group, in tile order, consecutive members pair up; an evenly spread subset
// of the pairs merges, each pair into one particle that carries both weights,
// which member survives being drawn with probability proportional to its
// weight.  Any weighted sum of the particles keeps its expectation, and the
// weight of every cell is kept exactly (up to the rounding of w_a + w_b).

// group key: bits 34..57 the cell row z, 14..33 the cell column r, 1..13 the
// |u|^2 quarter octave (its double's exponent and two leading mantissa
// bits), bit 0 the sign of u_z
__global__ void merge_keys_kernel(rrea_launch::MergeInput in, const int64_t* __restrict__ members, int64_t n,
                                  uint64_t* __restrict__ keys, uint32_t* __restrict__ perm)
{
    for (int64_t k = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; k < n;
         k += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        int64_t const i = members[k];
        double const fr = (in.r[i] - in.r_lo) / in.dr;
        double const fz = (in.z[i] - in.z_lo) / in.dz;
        int64_t ir = fr >= 0.0 ? static_cast<int64_t>(fr) : 0;
        int64_t iz = fz >= 0.0 ? static_cast<int64_t>(fz) : 0;
        ir = ir < in.nr ? ir : in.nr - 1;
        iz = iz < in.nz ? iz : in.nz - 1;
        double const ux = in.ux[i], uy = in.uy[i], uz = in.uz[i];
        // |u|^2 rounded product by product and sum by sum (no contraction),
        // so the key is reproducible off the device
        double const u2 = __dadd_rn(__dadd_rn(__dmul_rn(ux, ux), __dmul_rn(uy, uy)), __dmul_rn(uz, uz));
        uint64_t const bin = (static_cast<uint64_t>(__double_as_longlong(u2)) >> 50) & 0x1fffULL;
        keys[k] = (static_cast<uint64_t>(iz) << 34) | (static_cast<uint64_t>(ir) << 14) | (bin << 1)
            | (__double_as_longlong(uz) < 0 ? 1ULL : 0ULL);
        perm[k] = static_cast<uint32_t>(k);
    }
}

__global__ void merge_heads_kernel(const uint64_t* __restrict__ sorted_keys, int64_t n, uint32_t* __restrict__ heads)
{
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        heads[i] = (i == 0 || sorted_keys[i] != sorted_keys[i - 1]) ? 1u : 0u;
    }
}

// a pair starts at every even rank of a group that has a next member
__global__ void merge_pairs_kernel(const uint64_t* __restrict__ sorted_keys, const uint32_t* __restrict__ heads,
                                   const int64_t* __restrict__ group_of, const int64_t* __restrict__ begin, int64_t n,
                                   uint32_t* __restrict__ pair_head)
{
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        int64_t const g = group_of[i] + heads[i] - 1;
        int64_t const rank = i - begin[g];
        pair_head[i] = ((rank & 1) == 0 && i + 1 < n && sorted_keys[i + 1] == sorted_keys[i]) ? 1u : 0u;
    }
}

// The uniform of one pair: counter hashing of (seed, species, step, the two
// particles' stream keys |id| ^ cpu << 40) with splitmix64.
__device__ __forceinline__ double merge_uniform(uint64_t seed, int species, int64_t step, uint64_t ka, uint64_t kb)
{
    uint64_t h = splitmix64(seed ^ 0x6d65726765ULL ^ (static_cast<uint64_t>(species) << 56));
    h = splitmix64(h ^ static_cast<uint64_t>(step));
    h = splitmix64(h ^ ka);
    h = splitmix64(h ^ kb);
    return (static_cast<double>(h >> 11) + 0.5) * 0x1.0p-53;
}

// pair j (in sorted order) merges when floor((j + 1) R / P) > floor(j R / P):
// R of the P pairs, spread evenly over the groups
__global__ void merge_apply_kernel(rrea_launch::MergeInput in, const int64_t* __restrict__ members, const uint32_t* __restrict__ perm,
                                   const uint32_t* __restrict__ pair_head, const int64_t* __restrict__ pair_ordinal,
                                   int64_t n, uint64_t pairs, uint64_t merges, unsigned long long* __restrict__ merged)
{
    unsigned int done = 0;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        if (!pair_head[i]) continue;
        uint64_t const j = static_cast<uint64_t>(pair_ordinal[i]);
        if ((j + 1) * merges / pairs == j * merges / pairs) continue;
        int64_t const a = members[perm[i]], b = members[perm[i + 1]];
        double const wa = in.w[a], wb = in.w[b];
        uint64_t const ka = static_cast<uint64_t>(llabs(in.id[a])) ^ (static_cast<uint64_t>(in.cpu ? in.cpu[a] : 0) << 40);
        uint64_t const kb = static_cast<uint64_t>(llabs(in.id[b])) ^ (static_cast<uint64_t>(in.cpu ? in.cpu[b] : 0) << 40);
        double const u = merge_uniform(in.rng_seed, in.species, in.step, ka, kb);
        double const sum = wa + wb;
        bool const keep_a = u * sum < wa;
        int64_t const keep = keep_a ? a : b, drop = keep_a ? b : a;
        in.w[keep] = sum;
        in.id[drop] = -in.id[drop];
        ++done;
    }
    unsigned int const warp_total = __reduce_add_sync(0xffffffffu, done);
    if ((threadIdx.x & 31) == 0 && warp_total) atomicAdd(merged, static_cast<unsigned long long>(warp_total));
}

}  // namespace
}  // namespace rrea_dev

namespace rrea_launch {

// Device scratch of the plan, grown on demand and kept between calls.
struct PopulationWork {
    int64_t cap = 0;
    uint32_t* flags = nullptr;
    int64_t* offsets = nullptr;
    int64_t* scan_scratch = nullptr;
    int64_t* members = nullptr;
    uint64_t* k1 = nullptr;
    uint64_t* k2 = nullptr;
    uint64_t* k3 = nullptr;
    uint64_t* ka = nullptr;  // key ping-pong
    uint64_t* kb = nullptr;
    uint64_t* k2s = nullptr;
    uint64_t* k3s = nullptr;
    uint32_t* perm_a = nullptr;
    uint32_t* perm_b = nullptr;
    double* fr = nullptr;
    double* fz = nullptr;
    double* w = nullptr;
    double* sfr = nullptr;
    double* sfz = nullptr;
    double* sw = nullptr;
    double* sw0 = nullptr;
    int64_t* begin = nullptr;
    int64_t* capacity = nullptr;
    int64_t* cap_prefix = nullptr;
    void* cub_temp = nullptr;
    size_t cub_bytes = 0;
    int* status = nullptr;
    unsigned long long* removed = nullptr;
    // ensemble plans: instance keys, per-instance words, group instances
    uint64_t* k0 = nullptr;
    int64_t* inst_words = nullptr;
    uint32_t* ginst = nullptr;
    int64_t inst_cap = 0, group_cap = 0;
};

namespace {

void release(PopulationWork& p)
{
    void* ptrs[] = {p.flags, p.offsets, p.scan_scratch, p.members, p.k1, p.k2, p.k3, p.ka, p.kb, p.k2s, p.k3s,
                    p.perm_a, p.perm_b, p.fr, p.fz, p.w, p.sfr, p.sfz, p.sw, p.sw0, p.begin, p.capacity,
                    p.cap_prefix, p.cub_temp, p.status, p.removed, p.k0, p.inst_words, p.ginst};
    for (void* q : ptrs) {
        if (q) cudaFree(q);
    }
    p = PopulationWork{};
}

template <class T>
cudaError_t grab(T** p, int64_t n)
{
    return cudaMalloc(reinterpret_cast<void**>(p), static_cast<size_t>(n > 0 ? n : 1) * sizeof(T));
}

cudaError_t ensure(PopulationWork& p, int64_t n)
{
    if (n <= p.cap && p.status) return cudaSuccess;
    release(p);
    int64_t const cap = std::max<int64_t>(n + n / 4, 1 << 12);
    cudaError_t e = cudaSuccess;
    auto g = [&](auto** q, int64_t count) {
        if (e == cudaSuccess) e = grab(q, count);
    };
    g(&p.flags, cap);
    g(&p.offsets, cap);
    g(&p.scan_scratch, scan_scratch_elems(cap));
    g(&p.members, cap);
    g(&p.k1, cap);
    g(&p.k2, cap);
    g(&p.k3, cap);
    g(&p.k0, cap);
    g(&p.ka, cap);
    g(&p.kb, cap);
    g(&p.k2s, cap);
    g(&p.k3s, cap);
    g(&p.perm_a, cap);
    g(&p.perm_b, cap);
    g(&p.fr, cap);
    g(&p.fz, cap);
    g(&p.w, cap);
    g(&p.sfr, cap);
    g(&p.sfz, cap);
    g(&p.sw, cap);
    g(&p.sw0, cap);
    g(&p.begin, cap);
    g(&p.capacity, cap);
    g(&p.cap_prefix, cap);
    g(&p.status, 1);
    g(&p.removed, 1);
    if (e == cudaSuccess) {
        size_t sort_bytes = 0, scan_bytes = 0;
        e = cub::DeviceRadixSort::SortPairs(nullptr, sort_bytes, p.ka, p.kb, p.perm_a, p.perm_b,
                                            static_cast<int>(std::min<int64_t>(cap, INT32_MAX)));
        if (e == cudaSuccess) {
            e = cub::DeviceScan::ExclusiveSum(nullptr, scan_bytes, p.capacity, p.cap_prefix,
                                              static_cast<int>(std::min<int64_t>(cap, INT32_MAX)));
        }
        p.cub_bytes = std::max(sort_bytes, scan_bytes);
        if (e == cudaSuccess) e = cudaMalloc(&p.cub_temp, p.cub_bytes);
    }
    if (e != cudaSuccess) {
        release(p);
        return e;
    }
    p.cap = cap;
    return cudaSuccess;
}

// stable sort of (key, perm) pairs of n records by key
cudaError_t sort_by(PopulationWork& p, uint64_t const* keys_in_member_order, uint32_t*& perm, uint32_t*& perm_spare,
                    int64_t n, cudaStream_t s, int end_bit = 64)
{
    note_launch();
    rrea_dev::gather_u64_kernel<<<rrea_dev::blocks_for(n), 256, 0, s>>>(keys_in_member_order, perm, n, p.ka);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    size_t bytes = p.cub_bytes;
    e = cub::DeviceRadixSort::SortPairs(p.cub_temp, bytes, p.ka, p.kb, perm, perm_spare, static_cast<int>(n), 0, end_bit,
                                        s);
    std::swap(perm, perm_spare);
    return e;
}

}  // namespace

void population_work_free(PopulationWork* p)
{
    if (!p) return;
    release(*p);
    delete p;
}

cudaError_t population_thin(PopulationInput const& in, PopulationWork*& work, PopulationStats& st, int blocks,
                            cudaStream_t s)
{
    using namespace rrea_dev;
    (void)blocks;
    st = PopulationStats{};
    if (!work) work = new PopulationWork{};
    PopulationWork& p = *work;
    int64_t const n_all = in.n_tile + in.n_cand;
    if (n_all > INT32_MAX) {
        st.status = RREA_GPU_ERR_CAPACITY;
        return cudaSuccess;
    }
    cudaError_t e = ensure(p, n_all);
    if (e != cudaSuccess) return e;
    // members: valid live rows, then the species' candidates
    int64_t counts[2] = {0, 0};
    for (int part = 0; part < 2; ++part) {
        int64_t const n = part == 0 ? in.n_tile : in.n_cand;
        if (n == 0) continue;
        note_launch();
        if (part == 0) flags_live_kernel<<<blocks_for(n), 256, 0, s>>>(in.id, n, p.flags);
        else flags_cand_kernel<<<blocks_for(n), 256, 0, s>>>(in.cand, n, in.species, p.flags);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        if ((e = exclusive_scan_counts(p.flags, n, p.offsets, p.scan_scratch, s)) != cudaSuccess) return e;
        note_launch();
        scatter_members_kernel<<<blocks_for(n), 256, 0, s>>>(p.flags, p.offsets, n, counts[0], p.members);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        int64_t last_off = 0;
        uint32_t last_flag = 0;
        if ((e = cudaMemcpyAsync(&last_off, p.offsets + n - 1, sizeof(last_off), cudaMemcpyDeviceToHost, s)) ||
            (e = cudaMemcpyAsync(&last_flag, p.flags + n - 1, sizeof(last_flag), cudaMemcpyDeviceToHost, s)) ||
            (e = cudaStreamSynchronize(s))) {
            return e;
        }
        counts[part] = last_off + last_flag;
    }
    int64_t const n = counts[0] + counts[1];
    st.live = counts[0];
    st.candidates = counts[1];
    st.members = n;
    // RreaAdaptiveResampleAction: thinning strictly above 1.25 x target
    bool const due = in.target > 0 && n > in.target + in.target / 4;
    if (!due || n == 0) return cudaSuccess;
    if ((e = cudaMemsetAsync(p.status, 0, sizeof(int), s)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(p.removed, 0, sizeof(unsigned long long), s)) != cudaSuccess) return e;
    note_launch();
    records_kernel<<<blocks_for(n), 256, 0, s>>>(in, p.members, counts[0], n, p.k1, p.k2, p.k3, p.perm_a, p.fr, p.fz,
                                                 p.w, p.status);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    // least significant key first: identity low, identity high, then
    // (support, phase, candidate); every pass is stable
    uint32_t* perm = p.perm_a;
    uint32_t* spare = p.perm_b;
    if ((e = sort_by(p, p.k3, perm, spare, n, s)) != cudaSuccess) return e;
    if ((e = sort_by(p, p.k2, perm, spare, n, s)) != cudaSuccess) return e;
    if ((e = sort_by(p, p.k1, perm, spare, n, s)) != cudaSuccess) return e;
    // p.kb now holds k1 in sorted order
    note_launch();
    sorted_kernel<<<blocks_for(n), 256, 0, s>>>(perm, n, p.kb, p.k2, p.k3, p.fr, p.fz, p.w, p.sfr, p.sfz, p.sw,
                                                p.sw0, p.k2s, p.k3s, p.flags);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = exclusive_scan_counts(p.flags, n, p.offsets, p.scan_scratch, s)) != cudaSuccess) return e;
    note_launch();
    group_begin_kernel<<<blocks_for(n), 256, 0, s>>>(p.flags, p.offsets, n, p.begin);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    int64_t last_off = 0;
    uint32_t last_flag = 0;
    int status = 0;
    if ((e = cudaMemcpyAsync(&last_off, p.offsets + n - 1, sizeof(last_off), cudaMemcpyDeviceToHost, s)) ||
        (e = cudaMemcpyAsync(&last_flag, p.flags + n - 1, sizeof(last_flag), cudaMemcpyDeviceToHost, s)) ||
        (e = cudaMemcpyAsync(&status, p.status, sizeof(status), cudaMemcpyDeviceToHost, s)) ||
        (e = cudaStreamSynchronize(s))) {
        return e;
    }
    if (status != 0) {
        st.status = status;
        return cudaSuccess;
    }
    int64_t const groups = last_off + last_flag;
    st.supports = groups;
    note_launch();
    group_capacity_kernel<<<blocks_for(groups), 256, 0, s>>>(p.begin, groups, n, p.sfr, p.sfz, p.sw, p.capacity);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    size_t bytes = p.cub_bytes;
    if ((e = cub::DeviceScan::ExclusiveSum(p.cub_temp, bytes, p.capacity, p.cap_prefix, static_cast<int>(groups), s))) {
        return e;
    }
    int64_t last_cap = 0, last_prefix = 0;
    if ((e = cudaMemcpyAsync(&last_cap, p.capacity + groups - 1, sizeof(last_cap), cudaMemcpyDeviceToHost, s)) ||
        (e = cudaMemcpyAsync(&last_prefix, p.cap_prefix + groups - 1, sizeof(last_prefix), cudaMemcpyDeviceToHost,
                             s)) ||
        (e = cudaStreamSynchronize(s))) {
        return e;
    }
    st.capacity = last_prefix + last_cap;
    st.floor = n - st.capacity;
    int64_t const nominal = std::min<int64_t>(n - in.target, st.capacity);
    st.requested = nominal;
    if (nominal <= 0) return cudaSuccess;
    note_launch();
    group_thin_kernel<<<blocks_for(groups), 64, 0, s>>>(in, p.begin, groups, n, p.kb, p.k2s, p.k3s, p.sfr, p.sfz, p.sw,
                                                        p.sw0, p.capacity, p.cap_prefix, nominal, p.removed, p.status);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    unsigned long long removed = 0;
    if ((e = cudaMemcpyAsync(&removed, p.removed, sizeof(removed), cudaMemcpyDeviceToHost, s)) ||
        (e = cudaMemcpyAsync(&status, p.status, sizeof(status), cudaMemcpyDeviceToHost, s)) ||
        (e = cudaStreamSynchronize(s))) {
        return e;
    }
    st.removed = static_cast<int64_t>(removed);
    if (status != 0 || st.removed < nominal) {
        // an owner rejected its plan, or the plans made insufficient progress:
        // nothing is applied (the reference aborts the transaction)
        st.status = status != 0 ? status : RREA_GPU_ERR_INVALID_STATE;
        return cudaSuccess;
    }
    note_launch();
    apply_kernel<<<blocks_for(n), 256, 0, s>>>(in, perm, p.members, counts[0], n, p.sw);
    return cudaGetLastError();
}

cudaError_t population_thin_instances(PopulationInput const& in, PopulationWork*& work, PopulationStats& st,
                                      int64_t* removed_per_instance, cudaStream_t s)
{
    using namespace rrea_dev;
    st = PopulationStats{};
    uint32_t const n_inst = static_cast<uint32_t>(in.n_inst);
    for (uint32_t k = 0; k < n_inst; ++k) removed_per_instance[k] = 0;
    if (n_inst == 0 || in.n_tile == 0) return cudaSuccess;
    if (!in.cpu || in.n_cand != 0 || in.n_tile > INT32_MAX) {
        st.status = in.n_tile > INT32_MAX ? RREA_GPU_ERR_CAPACITY : RREA_GPU_ERR_ARGUMENT;
        return cudaSuccess;
    }
    if (!work) work = new PopulationWork{};
    PopulationWork& p = *work;
    cudaError_t e = ensure(p, in.n_tile);
    if (e != cudaSuccess) return e;
    // per-instance words: members, due target (-1: not due), capacity,
    // capacity base, request, removals; the group instances
    if (p.inst_cap < static_cast<int64_t>(n_inst) || p.group_cap < p.cap) {
        if (p.inst_words) cudaFree(p.inst_words);
        if (p.ginst) cudaFree(p.ginst);
        p.inst_words = nullptr;
        p.ginst = nullptr;
        p.inst_cap = p.group_cap = 0;
        if ((e = cudaMalloc(&p.inst_words, sizeof(int64_t) * 6 * static_cast<size_t>(n_inst))) != cudaSuccess) return e;
        if ((e = cudaMalloc(&p.ginst, sizeof(uint32_t) * static_cast<size_t>(p.cap))) != cudaSuccess) return e;
        p.inst_cap = n_inst;
        p.group_cap = p.cap;
    }
    auto* const members_k = reinterpret_cast<unsigned long long*>(p.inst_words);
    int64_t* const due_k = p.inst_words + n_inst;
    auto* const cap_k = reinterpret_cast<unsigned long long*>(p.inst_words + 2 * n_inst);
    int64_t* const base_k = p.inst_words + 3 * n_inst;
    int64_t* const nominal_k = p.inst_words + 4 * n_inst;
    auto* const removed_k = reinterpret_cast<unsigned long long*>(p.inst_words + 5 * n_inst);
    if ((e = cudaMemsetAsync(p.inst_words, 0, sizeof(int64_t) * 6 * n_inst, s)) != cudaSuccess) return e;
    bool const shared_hist = n_inst <= 4096;
    note_launch();
    instance_members_kernel<<<blocks_for(in.n_tile), 256, shared_hist ? sizeof(unsigned long long) * n_inst : 0, s>>>(
        in.id, in.cpu, in.n_tile, n_inst, shared_hist, members_k);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    // RreaAdaptiveResampleAction per instance: due strictly above 1.25 x target
    std::vector<int64_t> members(n_inst), due(n_inst, -1);
    if ((e = cudaMemcpyAsync(members.data(), members_k, sizeof(int64_t) * n_inst, cudaMemcpyDeviceToHost, s)) ||
        (e = cudaStreamSynchronize(s))) {
        return e;
    }
    bool any = false;
    for (uint32_t k = 0; k < n_inst; ++k) {
        int64_t const t = in.targets[k];
        st.live += members[k];
        if (t > 0 && members[k] > t + t / 4) {
            due[k] = t;
            any = true;
        }
    }
    if (!any) return cudaSuccess;
    if ((e = cudaMemcpyAsync(due_k, due.data(), sizeof(int64_t) * n_inst, cudaMemcpyHostToDevice, s)) != cudaSuccess) {
        return e;
    }
    note_launch();
    flags_due_kernel<<<blocks_for(in.n_tile), 256, 0, s>>>(in.id, in.cpu, in.n_tile, due_k, n_inst, p.flags);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = exclusive_scan_counts(p.flags, in.n_tile, p.offsets, p.scan_scratch, s)) != cudaSuccess) return e;
    note_launch();
    scatter_members_kernel<<<blocks_for(in.n_tile), 256, 0, s>>>(p.flags, p.offsets, in.n_tile, 0, p.members);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    int64_t last_off = 0;
    uint32_t last_flag = 0;
    if ((e = cudaMemcpyAsync(&last_off, p.offsets + in.n_tile - 1, sizeof(last_off), cudaMemcpyDeviceToHost, s)) ||
        (e = cudaMemcpyAsync(&last_flag, p.flags + in.n_tile - 1, sizeof(last_flag), cudaMemcpyDeviceToHost, s)) ||
        (e = cudaMemsetAsync(p.status, 0, sizeof(int), s)) || (e = cudaStreamSynchronize(s))) {
        return e;
    }
    int64_t const n = last_off + last_flag;
    st.members = n;
    if (n == 0) return cudaSuccess;
    note_launch();
    records_kernel<<<blocks_for(n), 256, 0, s>>>(in, p.members, n, n, p.k1, p.k2, p.k3, p.perm_a, p.fr, p.fz, p.w,
                                                 p.status, p.k0);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    // (instance, support, phase, candidate, identity high, identity low):
    // four stable passes, least significant first; the instance pass sorts
    // only the bits an instance number has
    int inst_bits = 1;
    while (inst_bits < 32 && (1u << inst_bits) < n_inst) ++inst_bits;
    uint32_t* perm = p.perm_a;
    uint32_t* spare = p.perm_b;
    if ((e = sort_by(p, p.k3, perm, spare, n, s)) != cudaSuccess) return e;
    if ((e = sort_by(p, p.k2, perm, spare, n, s)) != cudaSuccess) return e;
    if ((e = sort_by(p, p.k1, perm, spare, n, s)) != cudaSuccess) return e;
    if ((e = sort_by(p, p.k0, perm, spare, n, s, inst_bits)) != cudaSuccess) return e;
    // p.kb holds the sorted instances; the sorted k1 into p.ka
    note_launch();
    gather_u64_kernel<<<blocks_for(n), 256, 0, s>>>(p.k1, perm, n, p.ka);
    note_launch();
    heads_instances_kernel<<<blocks_for(n), 256, 0, s>>>(perm, n, p.kb, p.ka, p.k2, p.k3, p.fr, p.fz, p.w, p.sfr,
                                                         p.sfz, p.sw, p.sw0, p.k2s, p.k3s, p.flags);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = exclusive_scan_counts(p.flags, n, p.offsets, p.scan_scratch, s)) != cudaSuccess) return e;
    note_launch();
    group_begin_kernel<<<blocks_for(n), 256, 0, s>>>(p.flags, p.offsets, n, p.begin);
    int status = 0;
    if ((e = cudaGetLastError()) ||
        (e = cudaMemcpyAsync(&last_off, p.offsets + n - 1, sizeof(last_off), cudaMemcpyDeviceToHost, s)) ||
        (e = cudaMemcpyAsync(&last_flag, p.flags + n - 1, sizeof(last_flag), cudaMemcpyDeviceToHost, s)) ||
        (e = cudaMemcpyAsync(&status, p.status, sizeof(status), cudaMemcpyDeviceToHost, s)) ||
        (e = cudaStreamSynchronize(s))) {
        return e;
    }
    if (status != 0) {
        st.status = status;
        return cudaSuccess;
    }
    int64_t const groups = last_off + last_flag;
    st.supports = groups;
    note_launch();
    group_capacity_kernel<<<blocks_for(groups), 256, 0, s>>>(p.begin, groups, n, p.sfr, p.sfz, p.sw, p.capacity);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    size_t bytes = p.cub_bytes;
    if ((e = cub::DeviceScan::ExclusiveSum(p.cub_temp, bytes, p.capacity, p.cap_prefix, static_cast<int>(groups), s))) {
        return e;
    }
    note_launch();
    group_instances_kernel<<<blocks_for(groups), 256, 0, s>>>(p.begin, groups, p.kb, p.capacity, p.cap_prefix,
                                                              p.ginst, cap_k, base_k);
    note_launch();
    nominal_kernel<<<blocks_for(n_inst), 256, 0, s>>>(members_k, cap_k, due_k, n_inst, nominal_k);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    std::vector<int64_t> cap(n_inst), nominal(n_inst);
    if ((e = cudaMemcpyAsync(cap.data(), cap_k, sizeof(int64_t) * n_inst, cudaMemcpyDeviceToHost, s)) ||
        (e = cudaMemcpyAsync(nominal.data(), nominal_k, sizeof(int64_t) * n_inst, cudaMemcpyDeviceToHost, s)) ||
        (e = cudaStreamSynchronize(s))) {
        return e;
    }
    for (uint32_t k = 0; k < n_inst; ++k) {
        st.capacity += cap[k];
        st.requested += nominal[k] > 0 ? nominal[k] : 0;
    }
    st.floor = n - st.capacity;
    if (st.requested <= 0) return cudaSuccess;
    note_launch();
    group_thin_instances_kernel<<<blocks_for(groups), 64, 0, s>>>(in, p.begin, groups, n, p.ka, p.k2s, p.k3s, p.sfr,
                                                                  p.sfz, p.sw, p.sw0, p.capacity, p.cap_prefix,
                                                                  p.ginst, base_k, nominal_k, removed_k, p.status);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    std::vector<int64_t> removed(n_inst);
    if ((e = cudaMemcpyAsync(removed.data(), removed_k, sizeof(int64_t) * n_inst, cudaMemcpyDeviceToHost, s)) ||
        (e = cudaMemcpyAsync(&status, p.status, sizeof(status), cudaMemcpyDeviceToHost, s)) ||
        (e = cudaStreamSynchronize(s))) {
        return e;
    }
    bool short_plan = false;
    for (uint32_t k = 0; k < n_inst; ++k) {
        st.removed += removed[k];
        short_plan = short_plan || removed[k] < nominal[k];
    }
    if (status != 0 || short_plan) {
        // as population_thin: a rejected or short plan applies nothing
        st.status = status != 0 ? status : RREA_GPU_ERR_INVALID_STATE;
        return cudaSuccess;
    }
    for (uint32_t k = 0; k < n_inst; ++k) removed_per_instance[k] = removed[k];
    note_launch();
    apply_instances_kernel<<<blocks_for(n), 256, 0, s>>>(in, perm, p.members, n, p.sw, p.kb, nominal_k);
    return cudaGetLastError();
}

cudaError_t population_split(rrea_dev::TileColumns const& t, int64_t n, double min_w, PopulationWork*& work,
                             int64_t first_id, int64_t room, int64_t* added, cudaStream_t s)
{
    using namespace rrea_dev;
    *added = 0;
    if (n <= 0) return cudaSuccess;
    if (!work) work = new PopulationWork{};
    cudaError_t e = ensure(*work, n);
    if (e != cudaSuccess) return e;
    PopulationWork& p = *work;
    note_launch();
    split_flags_kernel<<<blocks_for(n), 256, 0, s>>>(t.d[6], t.id, n, min_w, p.flags);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = exclusive_scan_counts(p.flags, n, p.offsets, p.scan_scratch, s)) != cudaSuccess) return e;
    int64_t last_off = 0;
    uint32_t last_flag = 0;
    if ((e = cudaMemcpyAsync(&last_off, p.offsets + n - 1, sizeof(last_off), cudaMemcpyDeviceToHost, s)) ||
        (e = cudaMemcpyAsync(&last_flag, p.flags + n - 1, sizeof(last_flag), cudaMemcpyDeviceToHost, s)) ||
        (e = cudaStreamSynchronize(s))) {
        return e;
    }
    int64_t const clones = last_off + last_flag;
    if (clones > room) {
        *added = -clones;  // the tile cannot take the clones: nothing changed
        return cudaSuccess;
    }
    if (clones == 0) return cudaSuccess;
    note_launch();
    split_scatter_kernel<<<blocks_for(n), 256, 0, s>>>(t, n, p.flags, p.offsets, first_id);
    *added = clones;
    return cudaGetLastError();
}

cudaError_t population_merge(MergeInput const& in, PopulationWork*& work, MergeStats& st, cudaStream_t s)
{
    using namespace rrea_dev;
    st = MergeStats{};
    if (in.n_tile <= 0) return cudaSuccess;
    if (in.n_tile > INT32_MAX) {
        st.status = RREA_GPU_ERR_CAPACITY;
        return cudaSuccess;
    }
    if (!work) work = new PopulationWork{};
    PopulationWork& p = *work;
    cudaError_t e = ensure(p, in.n_tile);
    if (e != cudaSuccess) return e;
    int64_t const nt = in.n_tile;
    note_launch();
    flags_live_kernel<<<blocks_for(nt), 256, 0, s>>>(in.id, nt, p.flags);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = exclusive_scan_counts(p.flags, nt, p.offsets, p.scan_scratch, s)) != cudaSuccess) return e;
    note_launch();
    scatter_members_kernel<<<blocks_for(nt), 256, 0, s>>>(p.flags, p.offsets, nt, 0, p.members);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    int64_t last_off = 0;
    uint32_t last_flag = 0;
    if ((e = cudaMemcpyAsync(&last_off, p.offsets + nt - 1, sizeof(last_off), cudaMemcpyDeviceToHost, s)) ||
        (e = cudaMemcpyAsync(&last_flag, p.flags + nt - 1, sizeof(last_flag), cudaMemcpyDeviceToHost, s)) ||
        (e = cudaStreamSynchronize(s))) {
        return e;
    }
    int64_t const n = last_off + last_flag;
    st.live = n;
    if (n <= in.target || n < 2) return cudaSuccess;
    note_launch();
    merge_keys_kernel<<<blocks_for(n), 256, 0, s>>>(in, p.members, n, p.k1, p.perm_a);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    uint32_t* perm = p.perm_a;
    uint32_t* spare = p.perm_b;
    if ((e = sort_by(p, p.k1, perm, spare, n, s, 58)) != cudaSuccess) return e;
    // p.kb: the keys in sorted order; groups and their first members
    note_launch();
    merge_heads_kernel<<<blocks_for(n), 256, 0, s>>>(p.kb, n, p.flags);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = exclusive_scan_counts(p.flags, n, p.offsets, p.scan_scratch, s)) != cudaSuccess) return e;
    note_launch();
    group_begin_kernel<<<blocks_for(n), 256, 0, s>>>(p.flags, p.offsets, n, p.begin);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    uint32_t* const pair_head = reinterpret_cast<uint32_t*>(p.k2);
    note_launch();
    merge_pairs_kernel<<<blocks_for(n), 256, 0, s>>>(p.kb, p.flags, p.offsets, p.begin, n, pair_head);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = exclusive_scan_counts(pair_head, n, p.cap_prefix, p.scan_scratch, s)) != cudaSuccess) return e;
    int64_t groups_off = 0, pairs_off = 0;
    uint32_t groups_flag = 0, pairs_flag = 0;
    if ((e = cudaMemcpyAsync(&groups_off, p.offsets + n - 1, sizeof(groups_off), cudaMemcpyDeviceToHost, s)) ||
        (e = cudaMemcpyAsync(&groups_flag, p.flags + n - 1, sizeof(groups_flag), cudaMemcpyDeviceToHost, s)) ||
        (e = cudaMemcpyAsync(&pairs_off, p.cap_prefix + n - 1, sizeof(pairs_off), cudaMemcpyDeviceToHost, s)) ||
        (e = cudaMemcpyAsync(&pairs_flag, pair_head + n - 1, sizeof(pairs_flag), cudaMemcpyDeviceToHost, s)) ||
        (e = cudaStreamSynchronize(s))) {
        return e;
    }
    st.groups = groups_off + groups_flag;
    st.pairs = pairs_off + pairs_flag;
    st.requested = std::min<int64_t>(n - in.target, st.pairs);
    if (st.requested <= 0) return cudaSuccess;
    if ((e = cudaMemsetAsync(p.removed, 0, sizeof(unsigned long long), s)) != cudaSuccess) return e;
    note_launch();
    merge_apply_kernel<<<blocks_for(n), 256, 0, s>>>(in, p.members, perm, pair_head, p.cap_prefix, n,
                                                     static_cast<uint64_t>(st.pairs),
                                                     static_cast<uint64_t>(st.requested), p.removed);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    unsigned long long merged = 0;
    if ((e = cudaMemcpyAsync(&merged, p.removed, sizeof(merged), cudaMemcpyDeviceToHost, s)) ||
        (e = cudaStreamSynchronize(s))) {
        return e;
    }
    st.merged = static_cast<int64_t>(merged);
    return cudaSuccess;
}

}  // namespace rrea_launch
