// Single-box, single-rank stand-in for the part of AMReX that the
// reference's carrier-fluid sources (S/LowEnergyFluidState.cpp,
// S/LowEnergyFluidFaceTransport.cpp) use: IntVect/Box/BoxArray with an index
// type, a Geometry over one RZ domain, Array4 views, a MultiFab holding ONE
// fab (valid box grown by nGrow), an MFIter that visits it once, ParallelFor /
// LoopOnCpu in AMReX's k-j-i loop order, periodic FillBoundary and
// OverrideSync, and no-op rank reductions.  Only used to compile those
// reference sources into the golden-vector generator under oracle/_ref;
// never part of the shipped library.
#pragma once

#ifndef AMREX_SPACEDIM
#define AMREX_SPACEDIM 2
#endif
#ifndef AMREX_GPU_HOST_DEVICE
#define AMREX_GPU_HOST_DEVICE
#define AMREX_GPU_DEVICE
#define AMREX_FORCE_INLINE inline
#endif
#ifndef BL_PROFILE
#define BL_PROFILE(name)
#endif

#include "AMReX.H"
#include "AMReX_Algorithm.H"
#include "AMReX_REAL.H"

#include <array>
#include <cmath>
#include <cstddef>
#include <limits>
#include <stdexcept>
#include <vector>

namespace amrex {

template <class T, std::size_t N>
using GpuArray = std::array<T, N>;
template <class T, std::size_t N>
using Array = std::array<T, N>;

struct IntVect {
    int v[3] = {0, 0, 0};
    IntVect() = default;
    IntVect(int a, int b, int c = 0) : v{a, b, c} {}
    int operator[](int d) const { return v[d]; }
    int& operator[](int d) { return v[d]; }
    bool operator==(IntVect const& o) const { return v[0] == o.v[0] && v[1] == o.v[1] && v[2] == o.v[2]; }
    bool operator!=(IntVect const& o) const { return !(*this == o); }
};

struct IndexType {
    bool node[2] = {false, false};
    bool nodeCentered(int d) const { return node[d]; }
    IntVect toIntVect() const { return IntVect(node[0] ? 1 : 0, node[1] ? 1 : 0); }
    bool operator==(IndexType const& o) const { return node[0] == o.node[0] && node[1] == o.node[1]; }
};

struct Box {
    IntVect lo, hi;
    IndexType type;
    Box() = default;
    Box(IntVect const& l, IntVect const& h) : lo(l), hi(h) {}
    int smallEnd(int d) const { return lo[d]; }
    int bigEnd(int d) const { return hi[d]; }
    IntVect const& smallEnd() const { return lo; }
    IntVect const& bigEnd() const { return hi; }
    IndexType ixType() const { return type; }
    bool operator==(Box const& o) const { return lo == o.lo && hi == o.hi && type == o.type; }
    bool operator!=(Box const& o) const { return !(*this == o); }
};

// A cell-centred box converted to the given staggering: nodal directions
// gain the high face.
inline Box convert(Box const& cell, IntVect const& nodal)
{
    Box b = cell;
    for (int d = 0; d < 2; ++d) {
        b.type.node[d] = nodal[d] != 0;
        if (b.type.node[d]) ++b.hi[d];
    }
    return b;
}

struct BoxArray {
    Box cell_box;   // the one cell-centred box
    IndexType type;
    BoxArray() = default;
    explicit BoxArray(Box const& b) : cell_box(b) {}
    Box box() const
    {
        IntVect n(type.node[0] ? 1 : 0, type.node[1] ? 1 : 0);
        return convert(cell_box, n);
    }
    bool operator==(BoxArray const& o) const { return cell_box == o.cell_box && type == o.type; }
    bool operator!=(BoxArray const& o) const { return !(*this == o); }
};

inline BoxArray convert(BoxArray const& ba, IntVect const& nodal)
{
    BoxArray out = ba;
    out.type.node[0] = nodal[0] != 0;
    out.type.node[1] = nodal[1] != 0;
    return out;
}

struct DistributionMapping {
    bool operator==(DistributionMapping const&) const { return true; }
    bool operator!=(DistributionMapping const&) const { return false; }
};

struct Periodicity {
    bool periodic[2] = {false, false};
    int period[2] = {0, 0};
};

class Geometry {
public:
    Geometry() = default;
    Geometry(Box const& domain, double r_lo, double z_lo, double r_hi, double z_hi, bool periodic_z)
        : m_domain(domain), m_plo{r_lo, z_lo}, m_phi{r_hi, z_hi}, m_periodic{false, periodic_z}
    {
        for (int d = 0; d < 2; ++d) {
            m_dx[d] = (m_phi[d] - m_plo[d]) / static_cast<double>(domain.hi[d] - domain.lo[d] + 1);
        }
    }
    Box const& Domain() const { return m_domain; }
    double ProbLo(int d) const { return m_plo[d]; }
    double ProbHi(int d) const { return m_phi[d]; }
    GpuArray<double, AMREX_SPACEDIM> ProbLoArray() const { return {m_plo[0], m_plo[1]}; }
    double CellSize(int d) const { return m_dx[d]; }
    GpuArray<double, AMREX_SPACEDIM> CellSizeArray() const { return {m_dx[0], m_dx[1]}; }
    bool isPeriodic(int d) const { return m_periodic[d]; }
    Periodicity periodicity() const
    {
        Periodicity p;
        for (int d = 0; d < 2; ++d) {
            p.periodic[d] = m_periodic[d];
            p.period[d] = m_domain.hi[d] - m_domain.lo[d] + 1;
        }
        return p;
    }

private:
    Box m_domain;
    double m_plo[2] = {0.0, 0.0};
    double m_phi[2] = {1.0, 1.0};
    double m_dx[2] = {1.0, 1.0};
    bool m_periodic[2] = {false, false};
};

template <class T>
struct Array4 {
    T* p = nullptr;
    int lo[3] = {0, 0, 0};
    int hi[3] = {0, 0, 0};
    long long jstride = 0, kstride = 0, nstride = 0;
    int ncomp = 0;
    Array4() = default;
    template <class U>
    Array4(Array4<U> const& o)   // Array4<T> -> Array4<T const>
        : p(o.p), lo{o.lo[0], o.lo[1], o.lo[2]}, hi{o.hi[0], o.hi[1], o.hi[2]}, jstride(o.jstride),
          kstride(o.kstride), nstride(o.nstride), ncomp(o.ncomp)
    {
    }
    T& operator()(int i, int j, int k, int n = 0) const
    {
        if (i < lo[0] || i > hi[0] || j < lo[1] || j > hi[1] || k != 0 || n < 0 || n >= ncomp) {
            throw std::runtime_error("Array4 index out of range");
        }
        return p[(i - lo[0]) + jstride * (j - lo[1]) + nstride * n];
    }
};

class MultiFab;

class MFIter {
public:
    explicit MFIter(MultiFab const& mf, bool /*tiling*/ = false);
    bool isValid() const { return !m_done; }
    MFIter& operator++()
    {
        m_done = true;
        return *this;
    }
    Box tilebox() const;
    Box validbox() const;
    Box growntilebox(int n = 1) const;

private:
    MultiFab const* m_mf;
    bool m_done = false;
};

inline bool TilingIfNotGPU() { return false; }

class MultiFab {
public:
    MultiFab() = default;
    MultiFab(BoxArray const& ba, DistributionMapping const&, int ncomp, int ngrow) : m_ba(ba), m_ncomp(ncomp), m_ngrow(ngrow)
    {
        Box const v = ba.box();
        m_glo = IntVect(v.lo[0] - ngrow, v.lo[1] - ngrow);
        m_ghi = IntVect(v.hi[0] + ngrow, v.hi[1] + ngrow);
        m_nx = m_ghi[0] - m_glo[0] + 1;
        m_ny = m_ghi[1] - m_glo[1] + 1;
        m_data.assign(static_cast<std::size_t>(m_nx) * m_ny * ncomp, 0.0);
    }
    BoxArray const& boxArray() const { return m_ba; }
    DistributionMapping DistributionMap() const { return {}; }
    int nComp() const { return m_ncomp; }
    int nGrow() const { return m_ngrow; }
    IndexType ixType() const { return m_ba.type; }
    Box validbox() const { return m_ba.box(); }

    Array4<Real> array(MFIter const&) { return view(); }
    Array4<Real const> array(MFIter const&) const { return cview(); }
    Array4<Real const> const_array(MFIter const&) const { return cview(); }

    void setVal(double v) { std::fill(m_data.begin(), m_data.end(), v); }

    // Fills the ghost cells that are periodic images of valid cells (only z
    // can be periodic in RZ); other ghosts keep their values, as AMReX leaves
    // physical-boundary ghosts alone.
    void FillBoundary(Periodicity const& per)
    {
        if (!per.periodic[1]) return;
        Box const v = validbox();
        int const period = per.period[1];
        auto a = view();
        for (int n = 0; n < m_ncomp; ++n) {
            for (int j = m_glo[1]; j <= m_ghi[1]; ++j) {
                if (j >= v.lo[1] && j <= v.hi[1]) continue;
                int jj = j;
                while (jj < v.lo[1]) jj += period;
                while (jj > v.hi[1]) jj -= period;
                if (jj < v.lo[1] || jj > v.hi[1]) continue;
                for (int i = v.lo[0]; i <= v.hi[0]; ++i) a(i, j, 0, n) = a(i, jj, 0, n);
            }
        }
    }
    // Nodal data on a periodic direction holds the same physical face at both
    // ends of the box; the low copy owns it.
    void OverrideSync(Periodicity const& per)
    {
        if (!(per.periodic[1] && m_ba.type.node[1])) return;
        Box const v = validbox();
        auto a = view();
        for (int n = 0; n < m_ncomp; ++n) {
            for (int i = v.lo[0]; i <= v.hi[0]; ++i) a(i, v.hi[1], 0, n) = a(i, v.lo[1], 0, n);
        }
    }
    void FillBoundaryAndSync(Periodicity const& per)
    {
        OverrideSync(per);
        FillBoundary(per);
    }
    void SumBoundary(Periodicity const&) {}

    double norm0(int comp = 0, int nghost = 0, bool /*local*/ = false) const
    {
        double m = 0.0;
        Box const v = validbox();
        auto a = cview();
        for (int j = v.lo[1] - nghost; j <= v.hi[1] + nghost; ++j) {
            for (int i = v.lo[0] - nghost; i <= v.hi[0] + nghost; ++i) m = std::max(m, std::abs(a(i, j, 0, comp)));
        }
        return m;
    }
    bool contains_nan(int scomp, int ncomp, int ngrow, bool /*local*/ = false) const
    {
        Box const v = validbox();
        auto a = cview();
        for (int n = scomp; n < scomp + ncomp; ++n) {
            for (int j = v.lo[1] - ngrow; j <= v.hi[1] + ngrow; ++j) {
                for (int i = v.lo[0] - ngrow; i <= v.hi[0] + ngrow; ++i) {
                    if (std::isnan(a(i, j, 0, n))) return true;
                }
            }
        }
        return false;
    }
    static void Copy(MultiFab& dst, MultiFab const& src, int scomp, int dcomp, int ncomp, int nghost)
    {
        Box const v = dst.validbox();
        auto d = dst.view();
        auto s = src.cview();
        for (int n = 0; n < ncomp; ++n) {
            for (int j = v.lo[1] - nghost; j <= v.hi[1] + nghost; ++j) {
                for (int i = v.lo[0] - nghost; i <= v.hi[0] + nghost; ++i) d(i, j, 0, dcomp + n) = s(i, j, 0, scomp + n);
            }
        }
    }

    // Host access for the generator: component n at (i, j), ghosts included.
    double& at(int i, int j, int n = 0) { return view()(i, j, 0, n); }
    double at(int i, int j, int n = 0) const { return cview()(i, j, 0, n); }

private:
    Array4<Real> view()
    {
        Array4<Real> a;
        fill(a, m_data.data());
        return a;
    }
    Array4<Real const> cview() const
    {
        Array4<Real const> a;
        fill(a, m_data.data());
        return a;
    }
    template <class A, class P>
    void fill(A& a, P* ptr) const
    {
        a.p = ptr;
        a.lo[0] = m_glo[0];
        a.lo[1] = m_glo[1];
        a.hi[0] = m_ghi[0];
        a.hi[1] = m_ghi[1];
        a.jstride = m_nx;
        a.kstride = static_cast<long long>(m_nx) * m_ny;
        a.nstride = a.kstride;
        a.ncomp = m_ncomp;
    }
    BoxArray m_ba;
    int m_ncomp = 1;
    int m_ngrow = 0;
    IntVect m_glo, m_ghi;
    int m_nx = 0, m_ny = 0;
    std::vector<double> m_data;
};

inline MFIter::MFIter(MultiFab const& mf, bool) : m_mf(&mf) {}
inline Box MFIter::tilebox() const { return m_mf->validbox(); }
inline Box MFIter::validbox() const { return m_mf->validbox(); }
inline Box MFIter::growntilebox(int n) const
{
    Box b = m_mf->validbox();
    for (int d = 0; d < 2; ++d) {
        b.lo[d] -= n;
        b.hi[d] += n;
    }
    return b;
}

template <class F>
void LoopOnCpu(Box const& bx, F&& f)
{
    for (int j = bx.lo[1]; j <= bx.hi[1]; ++j) {
        for (int i = bx.lo[0]; i <= bx.hi[0]; ++i) f(i, j, 0);
    }
}
template <class F>
void ParallelFor(Box const& bx, F&& f)
{
    LoopOnCpu(bx, f);
}

namespace ParallelDescriptor {
inline int MyProc() { return 0; }
inline void ReduceRealMax(double&) {}
inline void ReduceRealMax(double*, int) {}
inline void ReduceRealMin(double&) {}
inline void ReduceRealMin(double*, int) {}
inline void ReduceRealSum(double&) {}
inline void ReduceRealSum(double*, int) {}
inline void ReduceLongSum(Long*, int) {}
inline void ReduceIntMin(int&) {}
template <class T>
inline void Bcast(T*, int, int) {}
}  // namespace ParallelDescriptor

namespace Math {
template <class T>
T abs(T x) { return std::abs(x); }
}  // namespace Math

}  // namespace amrex
