// Census of a resident species tile: the particle reductions behind the
// overlay's reduced diagnostics (species_weight_statistics and
// electron_species_weight_above_energy, O/RreaCouplingDiagnostics.cpp:122-194)
// plus a weighted kinetic-energy spectrum, computed where the tile lives.
//
// Every valid particle (id > 0) contributes its weight w to the count, the
// weight sums (w, w^2, w K), the maximum weight, the weight at or above each
// threshold and one spectrum bin.  K is RreaLiveParticle::KineticEnergyEv
// (RreaKineticEnergyEvFromProperVelocity, O/RreaParticleInteraction.H:1494-1505)
// for e-/e+ and PhotonEnergyEv = |u| (O/RreaParticleSweep.H:56-59) for
// photons, evaluated with explicit round-to-nearest operations (no
// contraction), so a host evaluation of the same formula sees the same K and
// bin and threshold membership are exact.  Bins are [edges[b], edges[b+1]);
// K below edges[0] or at or above the last edge goes to the under- or
// overflow weight.
#include "rrea_kernels.h"

#include <cuda_runtime.h>

namespace rrea_dev {
namespace {

constexpr double kCensusMeC2 = 510998.95000;  // I/RreaConstants.H:9
constexpr double kCensusC = 299792458.0;      // I/RreaConstants.H:10

__device__ __forceinline__ double census_energy(double ux, double uy, double uz, bool photon)
{
    double const u2 = __dadd_rn(__dadd_rn(__dmul_rn(ux, ux), __dmul_rn(uy, uy)), __dmul_rn(uz, uz));
    if (photon) return __dsqrt_rn(u2);
    double const c2 = kCensusC * kCensusC;
    double const gamma = __dsqrt_rn(__dadd_rn(1.0, __ddiv_rn(u2, c2)));
    return __ddiv_rn(__dmul_rn(u2, kCensusMeC2), __dmul_rn(c2, __dadd_rn(gamma, 1.0)));
}

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// out layout (doubles): sum_w, sum_w2, sum_wK, under_w, over_w,
// above[n_thr], hist[n_edges - 1]; count and the max-weight bit pattern in
// their own words.
__global__ void census_kernel(const double* __restrict__ ux, const double* __restrict__ uy,
                              const double* __restrict__ uz, const double* __restrict__ w,
                              const int64_t* __restrict__ id, int64_t n, int photon,
                              const double* __restrict__ edges, int n_edges, const double* __restrict__ thr, int n_thr,
                              double* __restrict__ out, unsigned long long* __restrict__ count,
                              unsigned long long* __restrict__ max_bits)
{
    extern __shared__ double sh[];
    int const n_bins = n_edges - 1;
    int const n_out = 5 + n_thr + n_bins;
    double* const s_out = sh;                  // n_out
    double* const s_edges = sh + n_out;        // n_edges
    __shared__ unsigned long long s_count, s_max;
    for (int k = threadIdx.x; k < n_out; k += blockDim.x) s_out[k] = 0.0;
    for (int k = threadIdx.x; k < n_edges; k += blockDim.x) s_edges[k] = edges[k];
    if (threadIdx.x == 0) {
        s_count = 0;
        s_max = 0;
    }
    __syncthreads();
    double const lo = s_edges[0];
    double const hi = s_edges[n_edges - 1];
    int const lane = threadIdx.x & 31;
    int64_t const stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    // every lane of a warp runs the same number of iterations, so the
    // shuffles below see all 32 lanes
    int64_t const first = blockIdx.x * static_cast<int64_t>(blockDim.x) + (threadIdx.x & ~31);
    for (int64_t base = first; base < n; base += stride) {
        int64_t const i = base + lane;
        bool const valid = i < n && id[i] > 0;
        double wi = 0.0, k = 0.0;
        if (valid) {
            wi = w[i];
            k = census_energy(ux[i], uy[i], uz[i], photon != 0);
        }
        unsigned const ballot = __ballot_sync(0xffffffffu, valid);
        if (ballot == 0u) continue;
        double const sw = warp_sum(wi);
        double const sw2 = warp_sum(wi * wi);
        double const swk = warp_sum(valid ? __dmul_rn(wi, k) : 0.0);
        if (lane == 0) {
            atomicAdd(&s_out[0], sw);
            atomicAdd(&s_out[1], sw2);
            atomicAdd(&s_out[2], swk);
            atomicAdd(&s_count, static_cast<unsigned long long>(__popc(ballot)));
        }
        for (int t = 0; t < n_thr; ++t) {
            double const a = warp_sum(valid && k >= thr[t] ? wi : 0.0);
            if (lane == 0 && a != 0.0) atomicAdd(&s_out[5 + t], a);
        }
        if (valid) {
            if (wi > 0.0) atomicMax(&s_max, static_cast<unsigned long long>(__double_as_longlong(wi)));
            if (!(k >= lo)) {
                atomicAdd(&s_out[3], wi);
            } else if (!(k < hi)) {
                atomicAdd(&s_out[4], wi);
            } else {
                // last edge <= k: edges[b] <= k < edges[b + 1]
                int a = 0, b = n_edges - 1;
                while (b - a > 1) {
                    int const m = (a + b) >> 1;
                    if (s_edges[m] <= k) a = m; else b = m;
                }
                atomicAdd(&s_out[5 + n_thr + a], wi);
            }
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < n_out; k += blockDim.x) {
        if (s_out[k] != 0.0) atomicAdd(&out[k], s_out[k]);
    }
    if (threadIdx.x == 0) {
        if (s_count) atomicAdd(count, s_count);
        if (s_max) atomicMax(max_bits, s_max);
    }
}

}  // namespace
}  // namespace rrea_dev

namespace rrea_launch {

cudaError_t census(const double* ux, const double* uy, const double* uz, const double* w, const int64_t* id, int64_t n,
                   bool photon, const double* edges, int n_edges, const double* thresholds, int n_thresholds,
                   double* out, unsigned long long* count, unsigned long long* max_bits, int blocks,
                   cudaStream_t stream)
{
    if (n <= 0) return cudaSuccess;
    int const threads = 256;
    int64_t want = (n + threads - 1) / threads;
    if (want < blocks) blocks = static_cast<int>(want);
    if (blocks < 1) blocks = 1;
    size_t const shmem = static_cast<size_t>(5 + n_thresholds + (n_edges - 1) + n_edges) * sizeof(double);
    note_launch();
    rrea_dev::census_kernel<<<blocks, threads, shmem, stream>>>(ux, uy, uz, w, id, n, photon ? 1 : 0, edges, n_edges,
                                                               thresholds, n_thresholds, out, count, max_bits);
    return cudaGetLastError();
}

}  // namespace rrea_launch
