// Device transport geometry and kinematics: chord construction and RZ
// clipping, material path, path field work, half kick, cone sampling and
// the competing-hazard selection.  Register-resident, fixed-capacity
// structures replace the reference's heap vectors; the arithmetic follows the
// cited reference primitives operation for operation.
#pragma once

#include "rrea_device_common.cuh"

namespace rrea_dev {

// I/RreaTransportPath.H:13-73
struct Piece {
    double begin, end, length, shift;
};

// NP is the piece capacity: 1 for an absorbing z domain (a clipped chord
// has exactly one in-domain piece), RREA_ARENA_MAX_PIECES for periodic z.
template <int NP>
struct Path {
    double sx, sy, sz, ex, ey, ez;
    double full, in_begin, in_end, in_length;
    bool exits;
    int npieces;
    Piece pieces[NP];
};

struct Geom {
    double rlo, rhi, zlo, zhi;
    bool periodic;
};

// S/RreaTransportPath.cpp:13-27
__device__ __forceinline__ double wrap_z(Geom const& g, double z)
{
    if (!g.periodic) return z;
    double const len = g.zhi - g.zlo;
    if (!(gt0(len))) return z;
    double w = fmod(z - g.zlo, len);
    if (lt0(w)) w += len;
    return g.zlo + w;
}
// S/RreaTransportPath.cpp:42-52
template <int NP>
__device__ __forceinline__ void point_at_full(Path<NP> const& p, Geom const& g, double f, double& x, double& y, double& z)
{
    f = max0(fmin(1.0, f));
    x = p.sx + f * (p.ex - p.sx);
    y = p.sy + f * (p.ey - p.sy);
    z = wrap_z(g, p.sz + f * (p.ez - p.sz));
}
// S/RreaTransportPath.cpp:54-71
template <int NP>
__device__ __forceinline__ void point_at_piece(Path<NP> const& p, Geom const& g, Piece const& pc, double f, double& x,
                                               double& y, double& z)
{
    f = fmax(pc.begin, fmin(pc.end, f));
    x = p.sx + f * (p.ex - p.sx);
    y = p.sy + f * (p.ey - p.sy);
    z = p.sz + f * (p.ez - p.sz) + pc.shift;
    z = fmax(g.zlo, fmin(g.zhi, z));
}
// S/RreaTransportPath.cpp:29-40
__device__ __forceinline__ bool outside_certified(Geom const& g, double r, double z)
{
    if (!finite_bits(r) || !finite_bits(z)) return true;
    if (r < g.rlo || r >= g.rhi) return true;
    return !g.periodic && (z < g.zlo || z >= g.zhi);
}

// S/RreaTransportPath.cpp:73-295 on Cartesian chord ends (x0, y0, z0) ->
// (x1, y1, z1) with their radii r0, r1.  Periodic seams use double
// arithmetic where the host reference uses long double.
template <int NP>
__device__ __forceinline__ void clip_chord(double x0, double y0, double z0, double r0, double x1, double y1, double z1,
                                           double r1, bool ends_finite, Geom const& g, Path<NP>& p, Err& err)
{
    if (!ends_finite || !finite_bits(r0) || !finite_bits(z0) || !finite_bits(r1) || !finite_bits(z1) || lt0(r0) || lt0(r1)) {
        err.set(RREA_GPU_ERR_GEOMETRY);
        p.npieces = 0;
        p.full = 0.0;
        p.in_begin = p.in_end = p.in_length = 0.0;
        p.exits = false;
        return;
    }
    p.sx = x0;
    p.sy = y0;
    p.sz = z0;
    p.ex = x1;
    p.ey = y1;
    p.ez = z1;
    double const dx = p.ex - p.sx, dy = p.ey - p.sy, dz = p.ez - p.sz;
    p.full = sqrt(dx * dx + dy * dy + dz * dz);
    p.in_begin = 0.0;
    double const scale = fmax(1.0, fmax(g.rhi, fmax(fabs(g.zlo), fabs(g.zhi))));
    double const tol = 64.0 * kEps * scale;
    if (r0 < g.rlo - tol || r0 > g.rhi + tol || z0 < g.zlo - tol || z0 > g.zhi + tol) {
        err.set(RREA_GPU_ERR_GEOMETRY);
    }
    double exit_fraction = 1.0;
    if (!g.periodic) {
        if (gt0(dz)) {
            double const c = (g.zhi - z0) / dz;
            if (ge0(c) && c < exit_fraction) exit_fraction = c;
        } else if (lt0(dz)) {
            double const c = (g.zlo - z0) / dz;
            if (ge0(c) && c < exit_fraction) exit_fraction = c;
        }
    }
    double const a = dx * dx + dy * dy;
    if (gt0(a)) {
        double const b = 2.0 * (p.sx * dx + p.sy * dy);
        for (int cyl = 0; cyl < 2; ++cyl) {
            bool const outer = cyl == 0;
            double const radius = outer ? g.rhi : g.rlo;
            if (!outer && !(gt0(g.rlo))) break;
            double const c = p.sx * p.sx + p.sy * p.sy - radius * radius;
            double const disc = b * b - 4.0 * a * c;
            if (lt0(disc)) continue;
            double const root = sqrt(max0(disc));
            double const inv2a = 0.5 / a;
            double const roots[2] = {(-b - root) * inv2a, (-b + root) * inv2a};
            for (int q = 0; q < 2; ++q) {
                double const cand = roots[q];
                if (le0(cand) || cand > 1.0) continue;
                double const deriv = 2.0 * a * cand + b;
                bool const leaves = outer ? gt0(deriv) : deriv < 0.0;
                if (leaves && ge0(cand) && cand < exit_fraction) exit_fraction = cand;
            }
        }
    }
    p.in_end = max0(fmin(1.0, exit_fraction));
    p.in_length = p.full * (p.in_end - p.in_begin);
    p.exits = p.in_end < 1.0 - 64.0 * kEps;

    if constexpr (NP == 1) {
        // Absorbing z: no seams, so the breakpoints are [in_begin, in_end]
        // (already sorted); deduplication drops the piece when the two are
        // within the tolerance.  Static indices keep the path in registers.
        double const l = p.in_begin, r = p.in_end;
        bool const dup = fabs(l - r) <= 128.0 * kEps * fmax(1.0, fmax(fabs(l), fabs(r)));
        p.npieces = 0;
        if (!dup && r > l) {
            p.pieces[0] = Piece{l, r, p.full * (r - l), 0.0};
            p.npieces = 1;
        }
        return;
    }
    // Breakpoints: [in_begin, seams..., in_end], sorted and deduplicated.
    double bp[NP + 1];
    int nb = 0;
    bp[nb++] = p.in_begin;
    if (g.periodic && fabs(dz) > 0.0 && p.in_end > p.in_begin) {
        double const zend = z0 + dz * p.in_end;
        double const period = g.zhi - g.zlo;
        double const low = fmin(z0, zend), high = fmax(z0, zend);
        double const first = floor((low - g.zlo) / period) + 1.0;
        double const last = ceil((high - g.zlo) / period) - 1.0;
        for (double image = first; image <= last; image += 1.0) {
            double const seam = g.zlo + image * period;
            double const frac = (seam - z0) / dz;
            double const ftol = 128.0 * kEps * fmax(1.0, fabs(frac));
            if (frac > p.in_begin + ftol && frac < p.in_end - ftol) {
                if (nb >= NP) {
                    err.set(RREA_GPU_ERR_CAPACITY);
                    break;
                }
                bp[nb++] = frac;
            }
        }
    }
    bp[nb++] = p.in_end;
    // insertion sort (tiny)
    for (int i = 1; i < nb; ++i) {
        double const v = bp[i];
        int j = i - 1;
        while (j >= 0 && bp[j] > v) {
            bp[j + 1] = bp[j];
            --j;
        }
        bp[j + 1] = v;
    }
    // std::unique with a relative tolerance
    int nu = 0;
    for (int i = 0; i < nb; ++i) {
        if (nu > 0) {
            double const l = bp[nu - 1], r = bp[i];
            if (fabs(l - r) <= 128.0 * kEps * fmax(1.0, fmax(fabs(l), fabs(r)))) continue;
        }
        bp[nu++] = bp[i];
    }
    double const period_m = g.zhi - g.zlo;
    p.npieces = 0;
    for (int i = 1; i < nu; ++i) {
        double const b0 = bp[i - 1], e0 = bp[i];
        if (!(e0 > b0)) continue;
        double shift = 0.0;
        if (g.periodic) {
            double const mid = 0.5 * (b0 + e0);
            double const mid_z = z0 + mid * dz;
            double const image = floor((mid_z - g.zlo) / period_m);
            shift = -image * period_m;
        }
        p.pieces[p.npieces++] = Piece{b0, e0, p.full * (e0 - b0), shift};
    }
}

// ClipRz as the reference calls it, on cylindrical ends (r, theta, z).
template <int NP>
__device__ __forceinline__ void clip_rz(double r0, double th0, double z0, double r1, double th1, double z1,
                                        Geom const& g, Path<NP>& p, Err& err)
{
    bool const finite = finite_bits(th0) && finite_bits(th1);
    double s0 = 0.0, c0 = 1.0, s1 = 0.0, c1 = 1.0;
    if (finite) {
        sincos(th0, &s0, &c0);
        sincos(th1, &s1, &c1);
    }
    clip_chord(r0 * c0, r0 * s0, z0, r0, r1 * c1, r1 * s1, z1, r1, finite, g, p, err);
}

// The chords the transport loops build run between Cartesian points, which
// the reference passes through ClipRz's (r, theta, z) interface as
// (hypot(x, y), atan2(y, x), z) and turns back into r cos(theta),
// r sin(theta).  Clipping the Cartesian ends directly gives the same chord to
// within an ulp of each coordinate and saves an atan2 and a sincos per end.
template <int NP>
__device__ __forceinline__ void clip_xyz(double x0, double y0, double z0, double x1, double y1, double z1, Geom const& g,
                                         Path<NP>& p, Err& err)
{
    bool const finite = finite_bits(x0) && finite_bits(y0) && finite_bits(x1) && finite_bits(y1);
    clip_chord(x0, y0, z0, rz_radius(x0, y0), x1, y1, z1, rz_radius(x1, y1), finite, g, p, err);
}

// ------------------------------------------------------------ kinematics
// I/RreaSeedSchedule.H:31-43
__device__ __forceinline__ double proper_velocity_from_kinetic(double k)
{
    if (le0(k)) return 0.0;
    double const gm = 1.0 + k * kInvMeC2;
    return kC * sqrt(max0(gm * gm - 1.0));
}
// O/RreaParticleInteraction.H:1494-1506
__device__ __forceinline__ double kinetic_from_proper_velocity(double ux, double uy, double uz)
{
    double const u2 = ux * ux + uy * uy + uz * uz;
    double const gm = sqrt(1.0 + u2 / (kC * kC));
    return u2 * kMeC2 / ((kC * kC) * (gm + 1.0));
}
// O/RreaParticleInteraction.H:92-105
__device__ __forceinline__ double charged_speed(double k)
{
    if (!finite_bits(k) || lt0(k)) return __longlong_as_double(0x7ff8000000000000LL);
    double const gm = 1.0 + k * kInvMeC2;
    double const b2 = max0(1.0 - 1.0 / (gm * gm));
    return kC * sqrt(b2);
}
// O/RreaChargedInterleave.H:294-307.  The reference divides by sqrt(n2);
// scaling by rsqrt(n2) (within an ulp of 1/sqrt(n2)) gives the same unit
// vector to within two ulps per component for a third of the FP64
// instructions.  A zero norm falls back to +z as in the reference.
__device__ __forceinline__ void normalize(double& x, double& y, double& z)
{
    double const n2 = x * x + y * y + z * z;
    if (!(gt0(n2))) {
        x = 0.0; y = 0.0; z = 1.0;
        return;
    }
    double const inv = rsqrt(n2);
    x *= inv; y *= inv; z *= inv;
}
// O/RreaChargedInterleave.H:309-364.  The reference normalises five times:
// the axis, a copy of it, the first and second basis vectors and the
// result.  The copy of a unit axis, the cross product of two orthonormal
// vectors and the rotated unit vector are already unit to within a few ulps,
// so only the axis and the first basis vector are normalised here; the
// direction differs from the reference's by ulps (and is renormalised by the
// next half kick).
__device__ __forceinline__ void cone_direction(double ax, double ay, double az, double cos_t, double u_phi,
                                               double& ox, double& oy, double& oz)
{
    normalize(ax, ay, az);
    double const dx = ax, dy = ay, dz = az;
    double rx = 0.0, ry = 0.0, rz = 1.0;
    if (fabs(dz) > 0.9) { rx = 1.0; rz = 0.0; }
    double b1x = ry * dz - rz * dy, b1y = rz * dx - rx * dz, b1z = rx * dy - ry * dx;
    normalize(b1x, b1y, b1z);
    double const b2x = dy * b1z - dz * b1y, b2y = dz * b1x - dx * b1z, b2z = dx * b1y - dy * b1x;
    cos_t = fmin(1.0, fmax(-1.0, cos_t));
    // cos^2 is rounded on its own before the subtraction, as the reference's
    // x86-64 build rounds it: a fused 1 - cos^2 differs by up to an ulp of 1,
    // which a small-angle deflection (cos near 1, the Wentzel-VI energies)
    // amplifies by 1/sin^2 in sin and then in every later direction.
    double const sin_t = sqrt(max0(1.0 - __dmul_rn(cos_t, cos_t)));
    double const phi = kTwoPi * u_phi;
    double sp, cp;
    sincos(phi, &sp, &cp);
    ox = ax * cos_t + sin_t * (cp * b1x + sp * b2x);
    oy = ay * cos_t + sin_t * (cp * b1y + sp * b2y);
    oz = az * cos_t + sin_t * (cp * b1z + sp * b2z);
}
// O/RreaChargedInterleave.H:371-389
__device__ __forceinline__ int poisson_capped(double mean, double u, int kmax)
{
    if (le0(mean)) return 0;
    double p = exp(-mean);
    double cum = p;
    int k = 0;
    while (u > cum && k < kmax) {
        ++k;
        p *= mean / static_cast<double>(k);
        cum += p;
    }
    return k;
}
__device__ __forceinline__ double unit_cycle(double u)
{
    u -= floor(u);
    return lt0(u) ? u + 1.0 : u;
}
// O/RreaChargedInterleave.H:391-463
__device__ __forceinline__ double moller_cos(double kp, double ks_or_scat)
{
    double const v = ks_or_scat * (kp + 2.0 * kMeC2) / (kp * (ks_or_scat + 2.0 * kMeC2));
    return sqrt(fmin(1.0, max0(v)));
}
__device__ __forceinline__ void moller_lab_directions(double px, double py, double pz, double kp, double ks,
                                                      double u_az, double& opx, double& opy, double& opz,
                                                      double& osx, double& osy, double& osz)
{
    normalize(px, py, pz);
    u_az = unit_cycle(u_az);
    double cs;
    {
        double const a = max0(kp), b = max0(ks);
        cs = (le0(a) || le0(b)) ? 1.0 : moller_cos(a, b);
    }
    double cpm;
    {
        double const scat = max0(kp - ks);
        cpm = (le0(kp) || le0(scat)) ? 1.0 : moller_cos(kp, scat);
    }
    cone_direction(px, py, pz, cs, u_az, osx, osy, osz);
    cone_direction(px, py, pz, cpm, unit_cycle(u_az + 0.5), opx, opy, opz);
}
// O/RreaChargedInterleave.H:465-496
__device__ __forceinline__ void photon_recoil(double k0, double eg, double gx, double gy, double gz, double& cx,
                                              double& cy, double& cz)
{
    eg = max0(eg);
    if (le0(k0) || le0(eg)) return;
    normalize(cx, cy, cz);
    normalize(gx, gy, gz);
    double const p0 = sqrt(max0(k0 * (k0 + 2.0 * kMeC2)));
    double const px = p0 * cx - eg * gx, py = p0 * cy - eg * gy, pz = p0 * cz - eg * gz;
    double const n = sqrt(px * px + py * py + pz * pz);
    if (gt0(n)) {
        Divisor const d = make_divisor(n);
        cx = quot(px, d); cy = quot(py, d); cz = quot(pz, d);
        normalize(cx, cy, cz);
    }
}

struct FieldRange {
    double work, ex, ey, ez, bx, by, bz, length;
};

// O/RreaChargedInterleave.H:100-138 with the Boris rotation of
// I/RreaLorentzPush.H:21-46
__device__ __forceinline__ void half_kick(FieldRange const& f, double half_dt, double q, double& k, double& dx,
                                          double& dy, double& dz)
{
    double const umag = proper_velocity_from_kinetic(k);
    double const s = q * (kC * kC / kMeC2) * half_dt;
    double const uxm = umag * dx + s * f.ex;
    double const uym = umag * dy + s * f.ey;
    double const uzm = umag * dz + s * f.ez;
    double const gamma = sqrt(1.0 + (uxm * uxm + uym * uym + uzm * uzm) / (kC * kC));
    Divisor const d2g = make_divisor(2.0 * gamma);
    double const tx = quot(s * f.bx, d2g), ty = quot(s * f.by, d2g), tz = quot(s * f.bz, d2g);
    double const t2 = tx * tx + ty * ty + tz * tz;
    Divisor const d1t = make_divisor(1.0 + t2);
    double const sx = quot(2.0 * tx, d1t), sy = quot(2.0 * ty, d1t), sz = quot(2.0 * tz, d1t);
    double const ppx = uxm + uym * tz - uzm * ty;
    double const ppy = uym + uzm * tx - uxm * tz;
    double const ppz = uzm + uxm * ty - uym * tx;
    double const ux = uxm + ppy * sz - ppz * sy;
    double const uy = uym + ppz * sx - ppx * sz;
    double const uz = uzm + ppx * sy - ppy * sx;
    double const norm = sqrt(ux * ux + uy * uy + uz * uz);
    if (gt0(norm) && finite_bits(norm)) {
        Divisor const dn = make_divisor(norm);
        dx = quot(ux, dn); dy = quot(uy, dn); dz = quot(uz, dn);
    }
    k = max0(k + 0.5 * f.work);
}

// ------------------------------------------------------------ field gather
// Cell-centred total field (Maxwell + ambient face averages, computed once
// per step by a prep kernel exactly as S/RreaAmrexAdvance.cpp:556-565 forms
// them) and the corner Btheta of the replicated Maxwell vectors.
struct FieldView {
    Divisor div_dr, div_dz;
    const double* __restrict__ cell_er;  // nr*nz, i + nr*j
    const double* __restrict__ cell_ez;  // nr*nz
    const double* __restrict__ bt;       // (nr+1)*(nz+1), i + (nr+1)*j
    int nr, nz;
    double dr, dz, r_lo, z_lo;
    bool periodic;
    bool has_b;
    // ensemble mode: instance k's fields follow instance k-1's at these
    // strides (0: one field for every particle)
    int64_t inst_cells, inst_bt;

    // The field of one ensemble instance (the particle's cpu ordinal).
    __device__ __forceinline__ FieldView for_instance(int64_t inst) const
    {
        FieldView v = *this;
        if (inst_cells) {
            v.cell_er += inst * inst_cells;
            v.cell_ez += inst * inst_cells;
            v.bt += inst * inst_bt;
        }
        return v;
    }
};

// S/RreaAmrexAdvance.cpp:532-579 with I/RreaFieldGatherStencil.H:49-133 and
// MaxwellBthetaAt :511-530
__device__ __forceinline__ void gather(FieldView const& fv, double r, double z, double& er, double& ez, double& bth)
{
    double const fx = quot(r - fv.r_lo, fv.div_dr) + 0.0 - 0.5;
    double const fz = quot(z - fv.z_lo, fv.div_dz) + 0.0 - 0.5;
    double const flx = floor(fx), flz = floor(fz);
    int const ir0 = static_cast<int>(flx);
    int const iz0 = static_cast<int>(flz);
    double const tx = fx - static_cast<double>(ir0);
    double const tz = fz - static_cast<double>(iz0);
    int const i0 = max(0, min(fv.nr - 1, ir0));
    int const i1 = max(0, min(fv.nr - 1, ir0 + 1));
    int j0, j1;
    if (fv.periodic) {
        j0 = (iz0 + fv.nz) % fv.nz;
        j1 = (iz0 + 1 + fv.nz) % fv.nz;
    } else {
        j0 = max(0, min(fv.nz - 1, iz0));
        j1 = max(0, min(fv.nz - 1, iz0 + 1));
    }
    size_t const r0 = static_cast<size_t>(fv.nr) * j0, r1 = static_cast<size_t>(fv.nr) * j1;
    double const e00 = __ldg(fv.cell_er + i0 + r0), e01 = __ldg(fv.cell_er + i0 + r1);
    double const e10 = __ldg(fv.cell_er + i1 + r0), e11 = __ldg(fv.cell_er + i1 + r1);
    double const z00 = __ldg(fv.cell_ez + i0 + r0), z01 = __ldg(fv.cell_ez + i0 + r1);
    double const z10 = __ldg(fv.cell_ez + i1 + r0), z11 = __ldg(fv.cell_ez + i1 + r1);
    double const first_center = fv.r_lo + 0.5 * fv.dr;
    double const axis = r >= first_center ? 1.0 : max0((r - fv.r_lo) / (0.5 * fv.dr));
    er = ((1.0 - tx) * ((1.0 - tz) * e00 + tz * e01) + tx * ((1.0 - tz) * e10 + tz * e11)) * axis;
    ez = (1.0 - tx) * ((1.0 - tz) * z00 + tz * z01) + tx * ((1.0 - tz) * z10 + tz * z11);
    if (!fv.has_b || le0(r)) {
        bth = 0.0;
        if (!fv.has_b && gt0(r)) bth = 0.0;
        return;
    }
    double const fr = fmin(max0(quot(r, fv.div_dr)), static_cast<double>(fv.nr));
    double const fzz = fmin(max0(quot(z - fv.z_lo, fv.div_dz)), static_cast<double>(fv.nz));
    int const a0 = min(static_cast<int>(floor(fr)), fv.nr - 1);
    int const b0 = min(static_cast<int>(floor(fzz)), fv.nz - 1);
    double const tr = fr - a0, tzz = fzz - b0;
    size_t const w = static_cast<size_t>(fv.nr + 1);
    bth = (1.0 - tr) * ((1.0 - tzz) * __ldg(fv.bt + a0 + w * b0) + tzz * __ldg(fv.bt + a0 + w * (b0 + 1)))
        + tr * ((1.0 - tzz) * __ldg(fv.bt + a0 + 1 + w * b0) + tzz * __ldg(fv.bt + a0 + 1 + w * (b0 + 1)));
}

// O/RreaPathFieldWork.H:57-150 with the two-node rule of
// I/RreaGaussLegendre8.H:24-60
template <int NP>
__device__ __forceinline__ FieldRange path_field_work(FieldView const& fv, Geom const& g, Path<NP> const& p, double q,
                                                      double begin, double end, Err& err)
{
    FieldRange res{0, 0, 0, 0, 0, 0, 0, 0};
    if (!(gt0(p.full))) return res;
    begin = fmax(p.in_begin, begin);
    end = fmin(p.in_end, end);
    if (!(end > begin)) return res;
    Divisor const dfull = make_divisor(p.full);
    double const pdx = quot(p.ex - p.sx, dfull);
    double const pdy = quot(p.ey - p.sy, dfull);
    double const pdz = quot(p.ez - p.sz, dfull);
#pragma unroll
    for (int ip = 0; ip < NP; ++ip) {
        if (ip >= p.npieces) break;
        Piece const& pc = p.pieces[ip];
        double const pb = fmax(begin, pc.begin);
        double const pe = fmin(end, pc.end);
        if (!(pe > pb)) continue;
        double const mid = 0.5 * (pb + pe);
        double const half = 0.5 * (pe - pb);
        double const off = half * kGl2Node;
        double acc[7];
#pragma unroll
        for (int node = 0; node < 2; ++node) {
            double const f = node == 0 ? mid - off : mid + off;
            double x, y, z;
            point_at_piece(p, g, pc, f, x, y, z);
            // r and the radial unit vector from one rsqrt of r^2 (within two
            // ulps of hypot and of the quotients by it)
            double const r2 = fma(x, x, y * y);
            double r = 0.0, rad = 0.0, rc = 1.0, rs = 0.0;
            if (gt0(r2)) {
                double const inv = rsqrt(r2);
                r = r2 * inv;
                rad = (pdx * x + pdy * y) * inv;
                rc = x * inv;
                rs = y * inv;
            }
            double er, ez, bth;
            gather(fv, r, z, er, ez, bth);
            double const work = q * (er * rad + ez * pdz) * 1.0;
            if (!finite_bits(work) || !finite_bits(er) || !finite_bits(ez) || !finite_bits(bth)) {
                err.set(RREA_GPU_ERR_INVALID_STATE);
            }
            double const v[7] = {work, er * rc, er * rs, ez, -bth * rs, bth * rc, 0.0};
            if (node == 0) {
#pragma unroll
                for (int c = 0; c < 7; ++c) acc[c] = v[c];
            } else {
#pragma unroll
                for (int c = 0; c < 7; ++c) acc[c] = half * (acc[c] + v[c]);
            }
        }
        res.work += p.full * acc[0];
        res.ex += p.full * acc[1];
        res.ey += p.full * acc[2];
        res.ez += p.full * acc[3];
        res.bx += p.full * acc[4];
        res.by += p.full * acc[5];
        res.bz += p.full * acc[6];
        res.length += p.full * (pe - pb);
    }
    if (gt0(res.length)) {
        Divisor const dl = make_divisor(res.length);
        res.ex = quot(res.ex, dl); res.ey = quot(res.ey, dl); res.ez = quot(res.ez, dl);
        res.bx = quot(res.bx, dl); res.by = quot(res.by, dl); res.bz = quot(res.bz, dl);
    }
    return res;
}

// ------------------------------------------------------------ material path
// O/RreaMaterialPath.H:47-199: one interval per in-domain piece, with the
// piece's density ratio taken at its midpoint.
template <int NP>
struct Intervals {
    int n;
    double begin[NP], end[NP], length[NP], density[NP];
};

__device__ __forceinline__ double positive_or(double v, double fb) { return gt0(v) ? v : fb; }

// The altitude density profile bound to the context
// (rrea.air_density_model=altitude_profile); n == 0 is the uniform ratio.
struct DensityProfile {
    const double* alt;  // n strictly increasing altitudes above mean sea level (m)
    const double* val;  // n densities (kg/m^3), strictly positive
    int n;
    double alt0;        // altitude of z = 0 (ProfileAltitudeMslAtZ, O/RreaWarpXCoupling.cpp:67-71)
    double ref;         // the tables' reference density (kg/m^3)
};

// TransportDensityRatioAtZ (O/RreaWarpXCoupling.cpp:79-95) with
// RreaAltitudeProfile::Interpolate (S/RreaAltitudeProfile.cpp:125-147): the
// uniform ratio without a profile; with one, the density interpolated
// linearly at alt0 + z over the reference density.  An altitude outside the
// profile fails the step (the reference throws).  The interpolation is
// evaluated without contraction so it rounds as the reference does.
__device__ __forceinline__ double density_ratio_at_z(DensityProfile const& d, double uniform, double z, Err& err)
{
    if (d.n == 0) return uniform;
    double const a = d.alt0 + z;
    if (!(a >= __ldg(d.alt) && a <= __ldg(d.alt + d.n - 1))) {
        err.set(RREA_GPU_ERR_RANGE);
        return uniform;
    }
    // std::upper_bound: the first node above a
    long long const ak = order_key(a);
    const long long* __restrict__ xk = reinterpret_cast<const long long*>(d.alt);
    int up = 0, count = d.n;
    while (count > 0) {
        int const step = count >> 1;
        if (__ldg(xk + up + step) <= ak) {
            up += step + 1;
            count -= step + 1;
        } else {
            count = step;
        }
    }
    double v;
    if (up == 0) {
        v = __ldg(d.val);
    } else if (up == d.n) {
        v = __ldg(d.val + d.n - 1);
    } else {
        int const lo = up - 1;
        double const span = __ldg(d.alt + up) - __ldg(d.alt + lo);
        double const t = gt0(span) ? (a - __ldg(d.alt + lo)) / span : 0.0;
        v = __dadd_rn(__dmul_rn(1.0 - t, __ldg(d.val + lo)), __dmul_rn(t, __ldg(d.val + up)));
    }
    return v / d.ref;
}

// :60-114
template <int NP>
__device__ __forceinline__ void build_intervals(Path<NP> const& p, double rho, Intervals<NP>& iv)
{
    iv.n = 0;
    if constexpr (NP == 1) {
        Piece const& pc = p.pieces[0];
        if (p.npieces < 1 || !(gt0(pc.length))) return;
        double dl = 0.0;
        if (pc.end > pc.begin && gt0(p.full)) dl = p.full * (pc.end - pc.begin) * positive_or(rho, rho);
        iv.begin[0] = pc.begin;
        iv.end[0] = pc.end;
        iv.length[0] = pc.length;
        iv.density[0] = positive_or(dl / pc.length, rho);
        iv.n = 1;
    } else {
        for (int i = 0; i < p.npieces; ++i) {
            Piece const& pc = p.pieces[i];
            if (!(gt0(pc.length))) continue;
            double dl = 0.0;
            if (pc.end > pc.begin && gt0(p.full)) dl = p.full * (pc.end - pc.begin) * positive_or(rho, rho);
            iv.begin[iv.n] = pc.begin;
            iv.end[iv.n] = pc.end;
            iv.length[iv.n] = pc.length;
            iv.density[iv.n] = positive_or(dl / pc.length, rho);
            ++iv.n;
        }
    }
}
// :60-114 with the density profile: each piece's ratio at its midpoint
// (integrate_density_piece_m's midpoint rule); `rho` is the step's ratio,
// the fallback of a non-positive value.
// Kept out of line: the uniform-density transport never calls it, and its
// code stays out of the transport loop.
template <int NP>
__device__ __noinline__ void build_intervals_profile(Path<NP> const& p, Geom const& g, DensityProfile const& dp,
                                                     double rho, Intervals<NP>& iv, Err& err)
{
    iv.n = 0;
#pragma unroll 1
    for (int i = 0; i < p.npieces; ++i) {
        Piece const& pc = p.pieces[i];
        if (!(gt0(pc.length))) continue;
        double dl = 0.0;
        if (pc.end > pc.begin && gt0(p.full)) {
            double x, y, z;
            point_at_piece(p, g, pc, 0.5 * (pc.begin + pc.end), x, y, z);
            dl = p.full * (pc.end - pc.begin) * positive_or(density_ratio_at_z(dp, rho, z, err), rho);
        }
        iv.begin[iv.n] = pc.begin;
        iv.end[iv.n] = pc.end;
        iv.length[iv.n] = pc.length;
        iv.density[iv.n] = positive_or(dl / pc.length, rho);
        ++iv.n;
    }
}
template <int NP>
__device__ __forceinline__ void build_intervals(Path<NP> const& p, Geom const& g, DensityProfile const& dp,
                                                double rho, Intervals<NP>& iv, Err& err)
{
    if (dp.n == 0) build_intervals(p, rho, iv);
    else build_intervals_profile(p, g, dp, rho, iv, err);
}
// :117-136
template <int NP>
__device__ __forceinline__ double density_path(Intervals<NP> const& iv, Path<NP> const& p, double b, double e)
{
    b = fmax(p.in_begin, b);
    e = fmin(p.in_end, e);
    if (!(e > b)) return 0.0;
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < NP; ++i) {
        if (i >= iv.n) break;
        double const bb = fmax(b, iv.begin[i]), ee = fmin(e, iv.end[i]);
        if (ee > bb) s += p.full * (ee - bb) * iv.density[i];
    }
    return s;
}
// :142-170
template <int NP>
__device__ __forceinline__ double fraction_at_density_path(Intervals<NP> const& iv, Path<NP> const& p, double b, double e,
                                                           double target, Err& err)
{
    b = fmax(p.in_begin, b);
    e = fmin(p.in_end, e);
    if (!finite_bits(target) || lt0(target)) {
        err.set(RREA_GPU_ERR_INVALID_STATE);
        return e;
    }
    double rem = target;
#pragma unroll
    for (int i = 0; i < NP; ++i) {
        if (i >= iv.n) break;
        double const bb = fmax(b, iv.begin[i]), ee = fmin(e, iv.end[i]);
        if (!(ee > bb) || !(gt0(iv.density[i]))) continue;
        double const c = p.full * (ee - bb) * iv.density[i];
        if (rem <= c) return bb + rem / (p.full * iv.density[i]);
        rem -= c;
    }
    return e;
}
// :175-199
template <int NP>
__device__ __forceinline__ double max_uniform_slice(Intervals<NP> const& iv, Path<NP> const& p, uint64_t n)
{
    double const span = p.in_end - p.in_begin;
    double const d = static_cast<double>(n);
    double m = 0.0;
    for (uint64_t i = 0; i < n; ++i) {
        m = fmax(m, density_path(iv, p, p.in_begin + static_cast<double>(i) / d * span,
                                 p.in_begin + static_cast<double>(i + 1U) / d * span));
    }
    return m;
}

// ------------------------------------------------------------ hazards
// O/RreaParticleInteraction.H:1402-1454
struct Selection {
    bool valid, event;
    int channel;
    double sampled, total;
};
__device__ __forceinline__ Selection select_hazard(const double* __restrict__ arena, double t0, double t1, double t2,
                                                  int count, double u1, double u2)
{
    Selection r{false, false, -1, 0.0, 0.0};
    double const taus[3] = {t0, t1, t2};
    if (count < 1 || count > 3 || !finite_bits(u1) || !finite_bits(u2)) return r;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        if (i >= count) break;
        if (!finite_bits(taus[i]) || lt0(taus[i])) return r;
        r.total += taus[i];
    }
    r.valid = finite_bits(r.total);
    if (!r.valid) return r;
    u1 = max0(fmin(1.0, u1));
    r.sampled = -flog(arena, fmax(1.0e-30, 1.0 - u1));
    if (!(r.sampled < r.total)) return r;
    r.event = true;
    u2 = max0(fmin(1.0, u2));
    double const target = u2 * r.total;
    double cum = 0.0;
    int last_open = -1;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        if (i >= count) break;
        if (gt0(taus[i])) last_open = i;
        cum += taus[i];
        if (target < cum) {
            r.channel = i;
            return r;
        }
    }
    r.channel = last_open;
    r.valid = r.channel >= 0;
    r.event = r.valid;
    return r;
}

// ------------------------------------------------------------ terminal helpers
// O/RreaParticleInteraction.H:318-354
__device__ __forceinline__ bool cartesian_half_open(Geom const& g, double x, double y, double z)
{
    if (!finite_bits(x) || !finite_bits(y)) return false;
    double const r = rz_radius(x, y);
    return finite_bits(r) && finite_bits(z) && g.rhi > g.rlo && g.zhi > g.zlo && r >= g.rlo && r < g.rhi && z >= g.zlo
        && z < g.zhi;
}
// RreaChargedBoundaryCrossingForPath (O/RreaParticleInteraction.H:468-540):
// the exact absorbing-face point of the final microchord and the crossed
// faces (bits 1 r_hi, 2 z_lo, 4 z_hi).  Returns false when no face is
// certified.
template <int NP>
__device__ __forceinline__ bool charged_crossing(Path<NP> const& p, Geom const& g, double& sr, double& sz, double& cr,
                                                 double& cz, uint32_t& faces)
{
    double cx, cy;
    point_at_full(p, g, p.in_end, cx, cy, cz);
    cz = wrap_z(g, cz);
    cr = rz_radius(cx, cy);
    sr = rz_radius(p.sx, p.sy);
    sz = wrap_z(g, p.sz);
    double const scale = fmax(1.0, fmax(g.rhi, fmax(fabs(g.zlo), fabs(g.zhi))));
    double const tol = 512.0 * kEps * scale;
    bool const on_r = fabs(cr - g.rhi) <= tol;
    bool const on_zlo = !g.periodic && fabs(cz - g.zlo) <= tol;
    bool const on_zhi = !g.periodic && fabs(cz - g.zhi) <= tol;
    double const dx = p.ex - p.sx, dy = p.ey - p.sy, dz = p.ez - p.sz;
    double const outward = cx * dx + cy * dy;
    faces = 0u;
    if (on_r && outward > -tol * scale) { faces |= 1u; cr = g.rhi; }
    if (on_zlo && lt0(dz)) { faces |= 2u; cz = g.zlo; }
    if (on_zhi && gt0(dz)) { faces |= 4u; cz = g.zhi; }
    if (faces == 0u) {
        if (on_r) { faces |= 1u; cr = g.rhi; }
        if (on_zhi) { faces |= 4u; cz = g.zhi; }
    }
    return faces != 0u && finite_bits(sr) && finite_bits(sz) && finite_bits(cr) && finite_bits(cz);
}

// O/RreaParticleInteraction.H:409-452 (clipped policy: RREA owns every escape)
template <int NP>
__device__ __forceinline__ void clipped_escape_policy(Path<NP> const& p, Geom const& g, double er, double ez,
                                                      bool& escapes, bool& invalidate)
{
    if (!finite_bits(er) || !finite_bits(ez)) {
        escapes = true;
        invalidate = true;
        return;
    }
    double const cz = wrap_z(g, ez);
    bool const outside = outside_certified(g, er, cz);
    escapes = p.exits || outside;
    invalidate = escapes;
}

}  // namespace rrea_dev
