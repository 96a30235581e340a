// Net-chord current deposition on the GPU: every charged particle's segment
// record (written by the electron / positron kernels) is replayed into the
// coupling's padded index-space grid with FP64 atomics, then converted to the
// physical face current densities.
//
//   netchord_deposit_kernel  one thread per tile slot: DepositSegmentRZ or
//                            DepositEscapingSegmentRZ
//                            (I/RreaSegmentDepositionRZ.H:96-397)
//   netchord_convert_kernel  ConvertPaddedIndexCurrentToPhysicalRZ
//                            (I/RreaSegmentDepositionRZ.H:399-458)
//
// The padded grid is the coupling's (O/RreaWarpXCoupling.cpp:417-444): two
// pad cells beyond r_hi and two below z_lo and above z_hi.  Every index is
// clamped into the grid as the reference clamps it, so any finite segment
// deposits in bounds; non-finite segments are refused before any write.
//
// The face fluxes and the CIC charge of a segment go through a warp-level
// pre-reduction: the lanes of a warp that reach the same deposit at the same
// time and aim at the same grid entry are grouped (a labeled partition of
// the coalesced lanes, keyed on grid and index), their values summed with a
// shuffle reduction, and one lane issues the single FP64 atomic.  Particles
// of an avalanche crowd a few cells near the axis, where this removes most
// of the atomic traffic to one address.
#include "rrea_kernels.h"

#include "device/rrea_electron_args.cuh"

#include <cooperative_groups.h>
#include <cooperative_groups/reduce.h>
#include <cuda_runtime.h>

namespace rrea_dev {
namespace {

namespace cg = cooperative_groups;

enum : unsigned long long { kGridRho = 1, kGridJr = 2, kGridJz = 3 };

// base[idx] += v, pre-reduced over the lanes that target the same entry.
__device__ __forceinline__ void warp_add(double* base, size_t idx, unsigned long long grid, double v)
{
    cg::coalesced_group const active = cg::coalesced_threads();
    cg::coalesced_group const same = cg::labeled_partition(active, (grid << 56) | static_cast<unsigned long long>(idx));
    double const sum = cg::reduce(same, v, cg::plus<double>());
    if (same.thread_rank() == 0) atomicAdd(base + idx, sum);
}

constexpr int kMaxCutsPerSegment = 1 << 16;

// Cell-boundary crossings of one coordinate along the segment, in
// increasing fraction: t_k = (k - a) / (b - a) for the integers k strictly
// between a and b (the same expression the reference sorts).
struct CrossSeq {
    double a, b, k, k_end, step;
    bool done;
    __device__ void init(double a_, double b_)
    {
        a = a_;
        b = b_;
        done = (a == b);
        if (done) return;
        double const lo = fmin(a, b), hi = fmax(a, b);
        if (b > a) {
            k = ceil(lo);
            k_end = floor(hi);
            step = 1.0;
        } else {
            k = floor(hi);
            k_end = ceil(lo);
            step = -1.0;
        }
        advance_to_interior();
    }
    __device__ double value() const { return (k - a) / (b - a); }
    __device__ bool in_range() const { return step > 0.0 ? k <= k_end : k >= k_end; }
    // skip crossings at t <= 0 (the start itself), stop at t >= 1
    __device__ void advance_to_interior()
    {
        while (!done && in_range() && !(value() > 0.0)) k += step;
        if (!done && (!in_range() || !(value() < 1.0))) done = true;
    }
    __device__ double peek() const { return done ? 2.0 : value(); }
    __device__ void pop()
    {
        k += step;
        advance_to_interior();
    }
};

__device__ __forceinline__ void cic_charge(NetGrid const& g, double q, double r, double z)
{
    double const xr = (r - g.r_lo) / g.dr - 0.5;
    double const xz = (z - g.z_lo) / g.dz - 0.5;
    int const i0 = static_cast<int>(floor(xr));
    int const j0 = static_cast<int>(floor(xz));
    double const fr = xr - i0, fz = xz - j0;
#pragma unroll
    for (int a = 0; a < 2; ++a) {
#pragma unroll
        for (int b = 0; b < 2; ++b) {
            int i = i0 + a, j = j0 + b;
            if (i < 0) i = -1 - i;
            if (i >= g.nr) i = g.nr - 1;
            if (j < 0) j = 0;
            if (j >= g.nz) j = g.nz - 1;
            warp_add(g.rho, static_cast<size_t>(i) + static_cast<size_t>(g.nr) * j, kGridRho,
                     q * (a == 0 ? 1.0 - fr : fr) * (b == 0 ? 1.0 - fz : fz));
        }
    }
}

__device__ __forceinline__ void deposit_piece(NetGrid const& g, double q_over_dt, double xr0, double xz0, double xr1,
                                              double xz1)
{
    double fr_flux = q_over_dt * (xr1 - xr0);
    double const fz_flux = q_over_dt * (xz1 - xz0);
    double const mr = 0.5 * (xr0 + xr1), mz = 0.5 * (xz0 + xz1);
    {
        int const jf = static_cast<int>(floor(mz));
        double const fz = mz - jf;
        int const fi = static_cast<int>(floor(mr)) + 1;
        if (fi <= 0) fr_flux = 0.0;
#pragma unroll
        for (int b = 0; b < 2; ++b) {
            int j = jf + b;
            if (j < 0) j = 0;
            if (j >= g.nz) j = g.nz - 1;
            int i = fi;
            if (i <= 0) continue;
            if (i > g.nr) i = g.nr;
            warp_add(g.jr, static_cast<size_t>(i) + static_cast<size_t>(g.nr + 1) * j, kGridJr,
                     fr_flux * (b == 0 ? 1.0 - fz : fz));
        }
    }
    {
        int const ifc = static_cast<int>(floor(mr));
        double const fr = mr - ifc;
        int const fj = static_cast<int>(floor(mz)) + 1;
#pragma unroll
        for (int a = 0; a < 2; ++a) {
            int i = ifc + a;
            if (i < 0) i = -1 - i;
            if (i >= g.nr) i = g.nr - 1;
            int j = fj;
            if (j < 0) j = 0;
            if (j > g.nz) j = g.nz;
            warp_add(g.jz, static_cast<size_t>(i) + static_cast<size_t>(g.nr) * j, kGridJz,
                     fz_flux * (a == 0 ? 1.0 - fr : fr));
        }
    }
}

// DepositSegmentRZ: pieces between consecutive cell-boundary crossings of
// either coordinate (merged in increasing fraction; a shared crossing gives
// an empty piece, which is skipped as in the reference).
__device__ bool deposit_segment(NetGrid const& g, double q, double dt, double r0, double z0, double r1, double z1)
{
    double const q_over_dt = q / dt;
    double const xr0 = (r0 - g.r_lo) / g.dr - 0.5, xz0 = (z0 - g.z_lo) / g.dz - 0.5;
    double const xr1 = (r1 - g.r_lo) / g.dr - 0.5, xz1 = (z1 - g.z_lo) / g.dz - 0.5;
    CrossSeq cr, cz;
    cr.init(xr0, xr1);
    cz.init(xz0, xz1);
    double s0 = 0.0;
    for (int guard = 0; guard < kMaxCutsPerSegment; ++guard) {
        double const tr = cr.peek(), tz = cz.peek();
        double s1;
        if (tr > 1.0 && tz > 1.0) {
            s1 = 1.0;
        } else if (tr <= tz) {
            s1 = tr;
            cr.pop();
        } else {
            s1 = tz;
            cz.pop();
        }
        if (s1 > s0) {
            deposit_piece(g, q_over_dt, xr0 + s0 * (xr1 - xr0), xz0 + s0 * (xz1 - xz0), xr0 + s1 * (xr1 - xr0),
                          xz0 + s1 * (xz1 - xz0));
        }
        if (s1 == 1.0) return true;
        s0 = s1;
    }
    return false;
}

struct Move {
    size_t from, to, face;
    double charge;
    int radial, orient;
};

// DepositEscapingSegmentRZ: the two chords to the exact face crossing plus
// the outward flux that removes the crossing cloud's remaining physical
// support, shared equally by the active faces of a corner.
__device__ bool deposit_escape(NetGrid const& g, double q, double dt, double sr0, double sz0, double fr0, double fz0,
                               double cr, double cz, uint32_t faces)
{
    uint32_t constexpr known = 1u | 2u | 4u;
    if (!(dt > 0.0) || !isfinite(q) || !isfinite(dt) || !isfinite(sr0) || !isfinite(sz0) || !isfinite(fr0)
        || !isfinite(fz0) || !isfinite(cr) || !isfinite(cz) || g.phys_nr <= 0 || g.phys_nr >= g.nr
        || g.phys_nz <= 0 || g.phys_z_begin <= 0 || g.phys_z_begin + g.phys_nz >= g.nz || faces == 0u
        || (faces & ~known) != 0u || ((faces & 2u) && (faces & 4u))) {
        return false;
    }
    if (faces & 1u) cr = g.r_lo + g.phys_nr * g.dr;
    if (faces & 2u) cz = g.z_lo + g.phys_z_begin * g.dz;
    else if (faces & 4u) cz = g.z_lo + (g.phys_z_begin + g.phys_nz) * g.dz;
    Move moves[8];
    int nm = 0;
    double const xr = (cr - g.r_lo) / g.dr - 0.5;
    double const xz = (cz - g.z_lo) / g.dz - 0.5;
    int const i0 = static_cast<int>(floor(xr));
    int const j0 = static_cast<int>(floor(xz));
    double const fr = xr - i0, fz = xz - j0;
    for (int a = 0; a < 2; ++a) {
        for (int b = 0; b < 2; ++b) {
            int i = i0 + a;
            int const j = j0 + b;
            if (i < 0) i = -1 - i;
            if (i < 0 || i >= g.nr || j < 0 || j >= g.nz) return false;
            bool const physical = i < g.phys_nr && j >= g.phys_z_begin && j < g.phys_z_begin + g.phys_nz;
            if (!physical) continue;
            uint32_t cand[2];
            int nc = 0;
            if ((faces & 1u) && i == g.phys_nr - 1) cand[nc++] = 1u;
            if ((faces & 2u) && j == g.phys_z_begin) cand[nc++] = 2u;
            if ((faces & 4u) && j == g.phys_z_begin + g.phys_nz - 1 && nc < 2) cand[nc++] = 4u;
            if (nc == 0) return false;
            double const share = q * (a == 0 ? 1.0 - fr : fr) * (b == 0 ? 1.0 - fz : fz) / nc;
            size_t const from = static_cast<size_t>(i) + static_cast<size_t>(g.nr) * j;
            for (int c = 0; c < nc && nm < 8; ++c) {
                Move& m = moves[nm++];
                m.from = from;
                m.charge = share;
                if (cand[c] == 1u) {
                    m.to = static_cast<size_t>(i + 1) + static_cast<size_t>(g.nr) * j;
                    m.face = static_cast<size_t>(g.phys_nr) + static_cast<size_t>(g.nr + 1) * j;
                    m.radial = 1;
                    m.orient = 1;
                } else {
                    int const face_j = cand[c] == 2u ? g.phys_z_begin : g.phys_z_begin + g.phys_nz;
                    int const to_j = cand[c] == 2u ? j - 1 : j + 1;
                    m.to = static_cast<size_t>(i) + static_cast<size_t>(g.nr) * to_j;
                    m.face = static_cast<size_t>(i) + static_cast<size_t>(g.nr) * face_j;
                    m.radial = 0;
                    m.orient = cand[c] == 2u ? -1 : 1;
                }
            }
        }
    }
    if (nm == 0) return false;
    cic_charge(g, -q, sr0, sz0);
    cic_charge(g, q, cr, cz);
    if (!deposit_segment(g, q, dt, sr0, sz0, fr0, fz0)) return false;
    if (!deposit_segment(g, q, dt, fr0, fz0, cr, cz)) return false;
    for (int m = 0; m < nm; ++m) {
        double const flux = moves[m].orient * moves[m].charge / dt;
        if (moves[m].radial) atomicAdd(g.jr + moves[m].face, flux);
        else atomicAdd(g.jz + moves[m].face, flux);
        atomicAdd(g.rho + moves[m].from, -moves[m].charge);
        atomicAdd(g.rho + moves[m].to, moves[m].charge);
    }
    return true;
}

__global__ void netchord_deposit_kernel(const SegmentRec* __restrict__ seg, int64_t n, NetGrid g, double dt,
                                        int* __restrict__ status, long long* __restrict__ fail_index)
{
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        SegmentRec const s = seg[i];
        bool ok = true;
        if (s.kind == 1) {
            if (s.a[4] == 0.0) continue;
            ok = isfinite(s.a[0]) && isfinite(s.a[1]) && isfinite(s.a[2]) && isfinite(s.a[3]) && isfinite(s.a[4])
                && deposit_segment(g, s.a[4], dt, s.a[0], s.a[1], s.a[2], s.a[3]);
        } else if (s.kind == 2) {
            if (s.a[6] == 0.0) continue;
            ok = deposit_escape(g, s.a[6], dt, s.a[0], s.a[1], s.a[2], s.a[3], s.a[4], s.a[5], s.faces);
        }
        if (!ok && atomicCAS(status, 0, RREA_GPU_ERR_GEOMETRY) == 0) *fail_index = static_cast<long long>(i);
    }
}

// DepositChargeCIC (I/RreaSegmentDepositionRZ.H:68-92) of every valid
// particle of a tile, charge q * w, onto the cell-centred nr x nz grid: the
// convention of the overlay's DepositParticleChargeToRreaGrid
// (O/RreaWarpXCoupling.cpp:376-389).
__global__ void particle_charge_kernel(const double* __restrict__ r, const double* __restrict__ z,
                                       const double* __restrict__ w, const int64_t* __restrict__ id, int64_t n,
                                       double q, int nr, int nz, double r_lo, double z_lo, double dr, double dz,
                                       double* __restrict__ rho)
{
    for (int64_t p = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; p < n;
         p += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        if (!(id[p] > 0)) continue;
        double const qw = q * w[p];
        double const xr = (r[p] - r_lo) / dr - 0.5;
        double const xz = (z[p] - z_lo) / dz - 0.5;
        int const i0 = static_cast<int>(floor(xr));
        int const j0 = static_cast<int>(floor(xz));
        double const fr = xr - i0, fz = xz - j0;
#pragma unroll
        for (int a = 0; a < 2; ++a) {
#pragma unroll
            for (int b = 0; b < 2; ++b) {
                int i = i0 + a, j = j0 + b;
                if (i < 0) i = -1 - i;
                if (i >= nr) i = nr - 1;
                if (j < 0) j = 0;
                if (j >= nz) j = nz - 1;
                warp_add(rho, static_cast<size_t>(i) + static_cast<size_t>(nr) * j, kGridRho,
                         qw * (a == 0 ? 1.0 - fr : fr) * (b == 0 ? 1.0 - fz : fz));
            }
        }
    }
}

__global__ void netchord_convert_kernel(NetGrid g, double* __restrict__ jr_phys, double* __restrict__ jz_phys)
{
    double constexpr pi = 3.14159265358979323846;
    double constexpr qe = 1.602176634e-19;
    int const nr = g.phys_nr, nz = g.phys_nz, pad = g.phys_z_begin;
    int64_t const n_r = static_cast<int64_t>(nr + 1) * nz;
    int64_t const n_z = static_cast<int64_t>(nr) * (nz + 1);
    for (int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; t < n_r + n_z;
         t += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        if (t < n_r) {
            int const i = static_cast<int>(t % (nr + 1));
            int const jp = static_cast<int>(t / (nr + 1));
            double const flux = g.jr[static_cast<size_t>(i) + static_cast<size_t>(g.nr + 1) * (jp + pad)];
            double const rf = i * g.dr;
            jr_phys[t] = (flux == 0.0 || rf <= 0.0) ? 0.0 : qe * flux / (2.0 * pi * rf * g.dz);
        } else {
            int64_t const u = t - n_r;
            int const i = static_cast<int>(u % nr);
            int const jp = static_cast<int>(u / nr);
            double const flux = g.jz[static_cast<size_t>(i) + static_cast<size_t>(g.nr) * (jp + pad)];
            double const rlo = i * g.dr, rhi = (i + 1) * g.dr;
            jz_phys[u] = flux == 0.0 ? 0.0 : qe * flux / (pi * (rhi * rhi - rlo * rlo));
        }
    }
}

}  // namespace
}  // namespace rrea_dev

namespace rrea_launch {

cudaError_t netchord_deposit(rrea_dev::SegmentRec const* seg, int64_t n, rrea_dev::NetGrid const& g, double dt,
                             int* status, long long* fail_index, int blocks, cudaStream_t stream)
{
    if (n <= 0) return cudaSuccess;
    note_launch();
    rrea_dev::netchord_deposit_kernel<<<blocks, 256, 0, stream>>>(seg, n, g, dt, status, fail_index);
    return cudaGetLastError();
}

cudaError_t particle_charge(const double* r, const double* z, const double* w, const int64_t* id, int64_t n, double q,
                            int nr, int nz, double r_lo, double z_lo, double dr, double dz, double* rho, int blocks,
                            cudaStream_t stream)
{
    if (n <= 0) return cudaSuccess;
    int64_t const want = (n + 255) / 256;
    if (want < blocks) blocks = static_cast<int>(want);
    note_launch();
    rrea_dev::particle_charge_kernel<<<blocks > 0 ? blocks : 1, 256, 0, stream>>>(r, z, w, id, n, q, nr, nz, r_lo, z_lo,
                                                                                  dr, dz, rho);
    return cudaGetLastError();
}

cudaError_t netchord_convert(rrea_dev::NetGrid const& g, double* jr_phys, double* jz_phys, cudaStream_t stream)
{
    int64_t const total = static_cast<int64_t>(g.phys_nr + 1) * g.phys_nz + static_cast<int64_t>(g.phys_nr) * (g.phys_nz + 1);
    int const blocks = static_cast<int>((total + 255) / 256);
    note_launch();
    rrea_dev::netchord_convert_kernel<<<blocks > 0 ? blocks : 1, 256, 0, stream>>>(g, jr_phys, jz_phys);
    return cudaGetLastError();
}

}  // namespace rrea_launch
