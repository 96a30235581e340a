// Maxwell TM-RZ field update on the device (I/RreaMaxwellTMRZ.H:147-228),
// composed as the Maxwell part of RreaAmrexAdvance::AdvanceOneStep
// (S/RreaAmrexAdvance.cpp:690-780): restagger B by (dt - dt_sub)/2, then per
// material substep B, Silver-Mueller, E with the face current, then restagger
// back and Silver-Mueller.  One thread per mesh element; B and E are separate
// launches because each reads the other's neighbours.
#include "rrea_kernels.h"

#include <cuda_runtime.h>

namespace rrea_dev {
namespace {

constexpr double kEps0 = 8.8541878128e-12;
constexpr double kMu0 = 1.25663706212e-6;
constexpr double kCLight = 299792458.0;

__device__ __forceinline__ size_t er_at(int nr, int i, int j)
{
    return static_cast<size_t>(i) + static_cast<size_t>(nr + 1) * j;
}
__device__ __forceinline__ size_t ez_at(int nr, int i, int j)
{
    return static_cast<size_t>(i) + static_cast<size_t>(nr) * j;
}

// dBtheta/dt = dEz/dr - dEr/dz at interior corners
__global__ void advance_b_kernel(int nr, int nz, double dr, double dz, double dt, const double* __restrict__ er,
                                 const double* __restrict__ ez, double* __restrict__ bt)
{
    int64_t const total = static_cast<int64_t>(nr - 1) * (nz - 1);
    for (int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; t < total;
         t += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        int const i = 1 + static_cast<int>(t % (nr - 1));
        int const j = 1 + static_cast<int>(t / (nr - 1));
        bt[er_at(nr, i, j)] += dt * ((ez[ez_at(nr, i, j)] - ez[ez_at(nr, i - 1, j)]) / dr
                                     - (er[er_at(nr, i, j)] - er[er_at(nr, i, j - 1)]) / dz);
    }
}

// Silver-Mueller boundary corners; where the reference's passes overlap the
// later pass wins: axis, then the z rows, then the outer column.
__global__ void silver_mueller_kernel(int nr, int nz, const double* __restrict__ er, const double* __restrict__ ez,
                                      double* __restrict__ bt)
{
    int64_t const total = static_cast<int64_t>(nr + 1) * (nz + 1);
    for (int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; t < total;
         t += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        int const i = static_cast<int>(t % (nr + 1));
        int const j = static_cast<int>(t / (nr + 1));
        size_t const c = er_at(nr, i, j);
        if (i == 0) bt[c] = 0.0;
        else if (j == 0) bt[c] = -er[er_at(nr, i, 0)] / kCLight;
        else if (j == nz) bt[c] = er[er_at(nr, i, nz - 1)] / kCLight;
        else if (i == nr) bt[c] = -ez[ez_at(nr, nr - 1, j)] / kCLight;
    }
}

// Ampere with the face current, no conductivity: Er on radial faces (axis
// face pinned to 0), Ez on axial faces.
__global__ void advance_e_kernel(int nr, int nz, double dr, double dz, double dt, const double* __restrict__ bt,
                                 const double* __restrict__ jr, const double* __restrict__ jz, double* __restrict__ er,
                                 double* __restrict__ ez)
{
    double const c2dt = dt / (kEps0 * kMu0);
    int64_t const n_r = static_cast<int64_t>(nr + 1) * nz;
    int64_t const n_z = static_cast<int64_t>(nr) * (nz + 1);
    for (int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; t < n_r + n_z;
         t += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        if (t < n_r) {
            int const i = static_cast<int>(t % (nr + 1));
            int const j = static_cast<int>(t / (nr + 1));
            size_t const face = er_at(nr, i, j);
            if (i == 0) {
                er[face] = 0.0;
                continue;
            }
            double const a = 0.0 * dt / (2.0 * kEps0);
            double drive = -c2dt * (bt[er_at(nr, i, j + 1)] - bt[er_at(nr, i, j)]) / dz;
            drive -= dt / kEps0 * jr[face];
            er[face] = ((1.0 - a) * er[face] + drive) / (1.0 + a);
        } else {
            int64_t const u = t - n_r;
            int const i = static_cast<int>(u % nr);
            int const j = static_cast<int>(u / nr);
            size_t const face = ez_at(nr, i, j);
            double const a = 0.0 * dt / (2.0 * kEps0);
            double drive = c2dt * ((i + 1) * bt[er_at(nr, i + 1, j)] - i * bt[er_at(nr, i, j)]) / ((i + 0.5) * dr);
            drive -= dt / kEps0 * jz[face];
            ez[face] = ((1.0 - a) * ez[face] + drive) / (1.0 + a);
        }
    }
}

int blocks_for(int64_t n)
{
    int64_t const b = (n + 255) / 256;
    return static_cast<int>(b < 1 ? 1 : (b > 65535 ? 65535 : b));
}

}  // namespace
}  // namespace rrea_dev

namespace rrea_launch {

cudaError_t maxwell_advance_b(int nr, int nz, double dr, double dz, double dt, const double* er, const double* ez,
                              double* bt, cudaStream_t stream)
{
    if (nr > 1 && nz > 1) {
        note_launch();
        rrea_dev::advance_b_kernel<<<rrea_dev::blocks_for(static_cast<int64_t>(nr - 1) * (nz - 1)), 256, 0, stream>>>(
            nr, nz, dr, dz, dt, er, ez, bt);
    }
    return cudaGetLastError();
}

cudaError_t maxwell_silver_mueller(int nr, int nz, const double* er, const double* ez, double* bt, cudaStream_t stream)
{
    note_launch();
    rrea_dev::silver_mueller_kernel<<<rrea_dev::blocks_for(static_cast<int64_t>(nr + 1) * (nz + 1)), 256, 0, stream>>>(
        nr, nz, er, ez, bt);
    return cudaGetLastError();
}

cudaError_t maxwell_advance_e(int nr, int nz, double dr, double dz, double dt, const double* bt, const double* jr,
                              const double* jz, double* er, double* ez, cudaStream_t stream)
{
    note_launch();
    rrea_dev::advance_e_kernel<<<rrea_dev::blocks_for(static_cast<int64_t>(nr + 1) * nz
                                                      + static_cast<int64_t>(nr) * (nz + 1)),
                                 256, 0, stream>>>(nr, nz, dr, dz, dt, bt, jr, jz, er, ez);
    return cudaGetLastError();
}

cudaError_t maxwell_step(int nr, int nz, double dr, double dz, double dt, int substeps, double* er, double* ez,
                         double* bt, const double* jr, const double* jz, cudaStream_t stream)
{
    using namespace rrea_dev;
    double const dts = dt / static_cast<double>(substeps);
    double const restagger = 0.5 * (dt - dts);
    int const nb_b = blocks_for(static_cast<int64_t>(nr - 1) * (nz - 1));
    int const nb_s = blocks_for(static_cast<int64_t>(nr + 1) * (nz + 1));
    int const nb_e = blocks_for(static_cast<int64_t>(nr + 1) * nz + static_cast<int64_t>(nr) * (nz + 1));
    bool const interior = nr > 1 && nz > 1;
    if (interior) {
        note_launch();
        advance_b_kernel<<<nb_b, 256, 0, stream>>>(nr, nz, dr, dz, restagger, er, ez, bt);
    }
    for (int k = 0; k < substeps; ++k) {
        if (interior) {
            note_launch();
            advance_b_kernel<<<nb_b, 256, 0, stream>>>(nr, nz, dr, dz, dts, er, ez, bt);
        }
        note_launch();
        silver_mueller_kernel<<<nb_s, 256, 0, stream>>>(nr, nz, er, ez, bt);
        note_launch();
        advance_e_kernel<<<nb_e, 256, 0, stream>>>(nr, nz, dr, dz, dts, bt, jr, jz, er, ez);
    }
    if (interior) {
        note_launch();
        advance_b_kernel<<<nb_b, 256, 0, stream>>>(nr, nz, dr, dz, -restagger, er, ez, bt);
    }
    note_launch();
    silver_mueller_kernel<<<nb_s, 256, 0, stream>>>(nr, nz, er, ez, bt);
    return cudaGetLastError();
}

}  // namespace rrea_launch
