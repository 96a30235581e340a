// ORACLE — test infrastructure only (see oracle_core.hpp).
#include "oracle_core.hpp"
#include "interleave.hpp"

#include <map>

#include <cstring>
#include <functional>
#include <sstream>

namespace oracle {

std::atomic<uint64_t> g_elastic_branch[4] = {};

void interleave_abort(int code, std::string const& message) { fail(code, message); }

// Photon energy-flow ledger checks of DrainAndCommitSecondaries
// (O/RreaSecondaryCommit.cpp:55-160) on one Compton (kind 0), photoelectric
// (kind 1) or pair (kind 2) interaction: a finite, non-negative payload whose
// parts add up to the incident energy, and a booked local flow equal to the
// split RreaComptonPhotonEnergyFlow / RreaPhotoelectricPhotonEnergyFlow /
// RreaPairPhotonEnergyFlow (O/RreaParticleInteraction.H:1015-1090) recomputes
// from the recorded energies, within 64 eps of the incident energy.
//   Compton: x1 = recoil, x2 = scattered; photoelectric: x1 = electron,
//   x2 = binding; pair: x1 = electron, x2 = positron, x3 = recoil.
bool PhotonFlowValid(int kind, double w, double inc, double x1, double x2, double x3, bool has_recoil, double local)
{
    double const eps64 = 64.0 * std::numeric_limits<double>::epsilon();
    auto matches = [&](double actual, double expected) {
        return std::isfinite(actual) && actual >= 0.0 && std::abs(actual - expected) <= eps64 * std::max(inc, 1.0);
    };
    if (!(std::isfinite(w) && std::isfinite(inc) && w > 0.0 && inc > 0.0)) return false;
    if (!(std::isfinite(x1) && std::isfinite(x2) && x1 >= 0.0 && x2 >= 0.0)) return false;
    if (kind == 0 || kind == 1) return matches(x1 + x2, inc);
    if (!(std::isfinite(x3) && x3 >= 0.0)) return false;
    double const expected = std::max(inc - 2.0 * kMeC2 - x1 - x2 - (has_recoil ? x3 : 0.0), 0.0);
    return matches(std::max(local, 0.0), expected);
}

namespace {

using rrea_host::TableSet;

// ======================================================================
// Transport path: I/RreaTransportPath.H:13-73, S/RreaTransportPath.cpp:13-295
// ======================================================================
struct Piece {
    double begin = 0.0, end = 0.0, length = 0.0, shift = 0.0;
};

struct Path {
    double sx = 0, sy = 0, sz = 0, ex = 0, ey = 0, ez = 0;
    double full = 0, in_begin = 0, in_end = 0, in_length = 0;
    bool exits = false, periodic = false;
    double rlo = 0, rhi = 0, zlo = 0, zhi = 0;
    std::vector<Piece> pieces;

    // S/RreaTransportPath.cpp:13-27
    double WrapZ(double z) const
    {
        if (!periodic) return z;
        double const len = zhi - zlo;
        if (!(len > 0.0)) return z;
        double w = std::fmod(z - zlo, len);
        if (w < 0.0) w += len;
        return zlo + w;
    }
    // S/RreaTransportPath.cpp:29-40
    bool OutsideCertified(double r, double z) const
    {
        if (!std::isfinite(r) || !std::isfinite(z)) return true;
        if (r < rlo || r >= rhi) return true;
        return !periodic && (z < zlo || z >= zhi);
    }
    // S/RreaTransportPath.cpp:42-52
    void PointAtFull(double f, double& x, double& y, double& z) const
    {
        f = std::max(0.0, std::min(1.0, f));
        x = sx + f * (ex - sx);
        y = sy + f * (ey - sy);
        z = WrapZ(sz + f * (ez - sz));
    }
    // S/RreaTransportPath.cpp:54-71
    void PointAtPiece(Piece const& p, double f, double& x, double& y, double& z) const
    {
        f = std::max(p.begin, std::min(p.end, f));
        x = sx + f * (ex - sx);
        y = sy + f * (ey - sy);
        z = sz + f * (ez - sz) + p.shift;
        z = std::max(zlo, std::min(zhi, z));
    }
};

// S/RreaTransportPath.cpp:73-295
Path ClipRz(double r0, double th0, double z0, double r1, double th1, double z1, double rlo,
            double rhi, double zlo, double zhi, bool periodic)
{
    auto finite = [](double v) { return std::isfinite(v); };
    if (!finite(r0) || !finite(th0) || !finite(z0) || !finite(r1) || !finite(th1) || !finite(z1)
        || r0 < 0.0 || r1 < 0.0 || rlo < 0.0 || !(rlo < rhi) || !(zlo < zhi)) {
        fail(RREA_GPU_ERR_GEOMETRY, "ClipRzTransportPath received invalid geometry or coordinates");
    }
    Path p;
    p.periodic = periodic;
    p.rlo = rlo;
    p.rhi = rhi;
    p.zlo = zlo;
    p.zhi = zhi;
    p.sx = r0 * std::cos(th0);
    p.sy = r0 * std::sin(th0);
    p.sz = z0;
    p.ex = r1 * std::cos(th1);
    p.ey = r1 * std::sin(th1);
    p.ez = z1;
    double const dx = p.ex - p.sx, dy = p.ey - p.sy, dz = p.ez - p.sz;
    p.full = std::sqrt(dx * dx + dy * dy + dz * dz);
    p.in_begin = 0.0;
    double const scale = std::max(1.0, std::max(rhi, std::max(std::abs(zlo), std::abs(zhi))));
    double const tol = 64.0 * kEps * scale;
    if (r0 < rlo - tol || r0 > rhi + tol || z0 < zlo - tol || z0 > zhi + tol) {
        fail(RREA_GPU_ERR_GEOMETRY, "previous particle position is outside the physical RZ domain");
    }
    double exit_fraction = 1.0;
    auto keep = [&](double c) {
        if (c >= 0.0 && c < exit_fraction) exit_fraction = c;
    };
    if (!periodic) {
        if (dz > 0.0) keep((zhi - z0) / dz);
        else if (dz < 0.0) keep((zlo - z0) / dz);
    }
    double const a = dx * dx + dy * dy;
    if (a > 0.0) {
        double const b = 2.0 * (p.sx * dx + p.sy * dy);
        auto cyl = [&](double radius, bool outer) {
            double const c = p.sx * p.sx + p.sy * p.sy - radius * radius;
            double const disc = b * b - 4.0 * a * c;
            if (disc < 0.0) return;
            double const root = std::sqrt(std::max(disc, 0.0));
            double const inv2a = 0.5 / a;
            double const roots[2] = {(-b - root) * inv2a, (-b + root) * inv2a};
            for (double cand : roots) {
                if (cand <= 0.0 || cand > 1.0) continue;
                double const deriv = 2.0 * a * cand + b;
                bool const leaves = outer ? deriv > 0.0 : deriv < 0.0;
                if (leaves) keep(cand);
            }
        };
        cyl(rhi, true);
        if (rlo > 0.0) cyl(rlo, false);
    }
    p.in_end = std::max(0.0, std::min(1.0, exit_fraction));
    p.in_length = p.full * (p.in_end - p.in_begin);
    p.exits = p.in_end < 1.0 - 64.0 * kEps;

    std::vector<double> bp = {p.in_begin, p.in_end};
    if (periodic && std::abs(dz) > 0.0 && p.in_end > p.in_begin) {
        long double const lz0 = static_cast<long double>(z0);
        long double const lz1 = lz0 + static_cast<long double>(dz) * static_cast<long double>(p.in_end);
        long double const lzlo = static_cast<long double>(zlo);
        long double const period = static_cast<long double>(zhi - zlo);
        long double const low = std::min(lz0, lz1), high = std::max(lz0, lz1);
        long double const first_ld = std::floor((low - lzlo) / period) + 1.0L;
        long double const last_ld = std::ceil((high - lzlo) / period) - 1.0L;
        if (last_ld - first_ld + 1.0L > 1000000.0L) {
            fail(RREA_GPU_ERR_GEOMETRY, "periodic path crosses more than 1,000,000 seams");
        }
        long long const first = static_cast<long long>(first_ld);
        long long const last = static_cast<long long>(last_ld);
        for (long long image = first; image <= last; ++image) {
            long double const seam = lzlo + static_cast<long double>(image) * period;
            double const frac = static_cast<double>((seam - lz0) / static_cast<long double>(dz));
            double const ftol = 128.0 * kEps * std::max(1.0, std::abs(frac));
            if (frac > p.in_begin + ftol && frac < p.in_end - ftol) bp.push_back(frac);
        }
    }
    std::sort(bp.begin(), bp.end());
    bp.erase(std::unique(bp.begin(), bp.end(),
                         [](double l, double r) {
                             return std::abs(l - r)
                                 <= 128.0 * kEps * std::max(1.0, std::max(std::abs(l), std::abs(r)));
                         }),
             bp.end());
    double const period_m = zhi - zlo;
    for (std::size_t i = 1; i < bp.size(); ++i) {
        double const b0 = bp[i - 1], e0 = bp[i];
        if (!(e0 > b0)) continue;
        double const mid = 0.5 * (b0 + e0);
        double const mid_z = z0 + mid * dz;
        double shift = 0.0;
        if (periodic) {
            double const image = std::floor((mid_z - zlo) / period_m);
            shift = -image * period_m;
        }
        p.pieces.push_back(Piece{b0, e0, p.full * (e0 - b0), shift});
    }
    return p;
}

// ======================================================================
// Tables: S/RreaInteractionTables.cpp
// ======================================================================
struct Tables {
    TableSet const& t;
    RreaArenaIndex const& ix;
    explicit Tables(TableSet const& ts) : t(ts), ix(ts.index()) {}

    // RreaInteractionTable::Interpolate, S/RreaInteractionTables.cpp:1580-1630
    double interpolate(int which, double q) const
    {
        RreaTable1DIndex const& h = ix.hot[which];
        double const* x = t.at(h.x);
        double const* y = t.at(h.y);
        double const* lx = t.at(h.lx);
        double const* ly = t.at(h.ly);
        int const n = h.n;
        if (!std::isfinite(q) || q < x[0] || q > x[n - 1]) {
            std::ostringstream m;
            m.precision(17);
            m << "interaction table " << which << " query " << q << " eV outside certified range";
            fail(RREA_GPU_ERR_RANGE, m.str());
        }
        double const* up = std::lower_bound(x, x + n, q);
        if (up == x) return y[0];
        if (up == x + n) return y[n - 1];
        int const hi = static_cast<int>(up - x);
        int const lo = hi - 1;
        if (x[hi] == q) return y[hi];
        if (h.mode == RREA_INTERP_LINEAR) {
            double const tt = (q - x[lo]) / (x[hi] - x[lo]);
            return y[lo] + tt * (y[hi] - y[lo]);
        }
        double const tt = (std::log(q) - lx[lo]) / (lx[hi] - lx[lo]);
        bool const pos = y[lo] > 0.0 && y[hi] > 0.0;
        if (h.mode == RREA_INTERP_LOGX_LINEAR || (h.mode == RREA_INTERP_LOGLOG_ZERO_THRESHOLD && !pos)) {
            return y[lo] + tt * (y[hi] - y[lo]);
        }
        if (!pos) fail(RREA_GPU_ERR_INVALID_STATE, "loglog_linear requires positive bracket");
        return std::exp(ly[lo] + tt * (ly[hi] - ly[lo]));
    }

    // S/RreaInteractionTables.cpp:624-648
    static double semilogx(double const* x, double const* lx, double const* y, int n, double q)
    {
        if (n < 2) return n ? y[0] : 0.0;
        if (!std::isfinite(q) || q < x[0] || q > x[n - 1]) {
            fail(RREA_GPU_ERR_RANGE, "elastic-table query outside its inclusive energy range");
        }
        if (q == x[0]) return y[0];
        if (q == x[n - 1]) return y[n - 1];
        double const* up = std::lower_bound(x, x + n, q);
        int const hi = static_cast<int>(up - x);
        int const lo = hi - 1;
        if (x[hi] == q) return y[hi];
        double const tt = (std::log(q) - lx[lo]) / (lx[hi] - lx[lo]);
        return y[lo] + tt * (y[hi] - y[lo]);
    }

    static double mfp_from_inverse(double inv)
    {
        // S/RreaInteractionTables.cpp:110-119
        if (!std::isfinite(inv) || inv < 0.0) {
            fail(RREA_GPU_ERR_INVALID_STATE, "process inverse length must be finite and nonnegative");
        }
        return inv > 0.0 ? 1.0 / inv : 1.0e99;
    }

    void require_charged(double e) const
    {
        // S/RreaInteractionTables.cpp:2241-2264
        if (!std::isfinite(e) || !(e >= ix.charged_min_eV && e <= ix.charged_max_eV)) {
            std::ostringstream m;
            m.precision(17);
            m << "schema-6 charged sampler energy " << e << " eV outside the certified range";
            fail(RREA_GPU_ERR_RANGE, m.str());
        }
    }

    // :2382-2392, :2655-2664
    double ElectronCollisionLoss(double e, double dr) const { return interpolate(RREA_T_E_COLLISION, e) * dr; }
    double ElectronSoftRadiativeDrag(double e, double dr) const { return interpolate(RREA_T_E_SOFT_RAD, e) * dr; }
    // :2394-2412
    double ElectronHardMollerMeanFreePath(double e, double dr) const
    {
        double const inv = interpolate(RREA_T_E_HARD_MOLLER, e);
        if (ix.hard_moller_threshold_eV > 0.0 && e <= 2.0 * ix.hard_moller_threshold_eV) return 1.0e99;
        return mfp_from_inverse(inv * dr);
    }
    // :3129-3178, 3196-3206
    double PositronCollisionLoss(double e, double dr) const { return interpolate(RREA_T_P_COLLISION, e) * dr; }
    double PositronSoftRadiativeDrag(double e, double dr) const { return interpolate(RREA_T_P_SOFT_RAD, e) * dr; }
    double PositronBremsstrahlungMeanFreePath(double e, double dr) const
    {
        return mfp_from_inverse(interpolate(RREA_T_P_TRACKED_BREMS, e) * dr);
    }
    double PositronHardBhabhaMeanFreePath(double e, double dr) const
    {
        double const inv = interpolate(RREA_T_P_HARD_BHABHA, e);
        if (ix.hard_moller_threshold_eV > 0.0 && e <= ix.hard_moller_threshold_eV) return 1.0e99;
        return mfp_from_inverse(inv * dr);
    }
    double PositronAnnihilationMeanFreePath(double e, double dr) const
    {
        return mfp_from_inverse(interpolate(RREA_T_P_ANNIHILATION, e) * dr);
    }
    // :2325-2353 (the three rates the positron channel gates read)
    void PositronGateRates(double e, double& bhabha_inv, double& brems_inv, double& annihilation_inv) const
    {
        if (!(e >= ix.charged_min_eV && e <= ix.charged_max_eV)) {
            fail(RREA_GPU_ERR_RANGE, "schema-6 positron energy outside the certified range");
        }
        interpolate(RREA_T_P_COLLISION, e);
        interpolate(RREA_T_P_SOFT_RAD, e);
        bhabha_inv = interpolate(RREA_T_P_HARD_BHABHA, e);
        brems_inv = interpolate(RREA_T_P_TRACKED_BREMS, e);
        interpolate(RREA_T_P_ELASTIC_TRANSPORT, e);
        annihilation_inv = interpolate(RREA_T_P_ANNIHILATION, e);
    }
    // :2666-2676
    double ElectronBremsstrahlungMeanFreePath(double e, double dr) const
    {
        return mfp_from_inverse(interpolate(RREA_T_E_TRACKED_BREMS, e) * dr);
    }
    // :2414-2440
    double ElectronHardMollerEnergyLoss(double e, double dr) const
    {
        RreaTable1DIndex const& h = ix.hot[RREA_T_E_HARD_MOLLER];
        double const inv = interpolate(RREA_T_E_HARD_MOLLER, e);
        if (!(inv > 0.0)) return 0.0;
        double const mean = semilogx(t.at(h.x), t.at(h.lx), t.at(ix.hard_moller_mean_secondary), h.n, e);
        if (!(mean > 0.0)) return 0.0;
        return mean * inv * dr;
    }
    // :1071-1110
    double mean_conditional(int which, double e) const
    {
        RreaCondCdfIndex const& ci = ix.cdf[which];
        double const* prim = t.at(ci.primary);
        double const* start = t.at(ci.start);
        double const* u = t.at(ci.u);
        double const* v = t.at(ci.v);
        auto group_mean = [&](int g) {
            int const b = static_cast<int>(start[g]), en = static_cast<int>(start[g + 1]);
            double mean = u[b] * v[b];
            for (int i = b + 1; i < en; ++i) mean += 0.5 * (v[i - 1] + v[i]) * (u[i] - u[i - 1]);
            mean += (1.0 - u[en - 1]) * v[en - 1];
            return mean;
        };
        if (e < prim[0] || e > prim[ci.ng - 1]) {
            fail(RREA_GPU_ERR_RANGE, "conditional-CDF mean query outside its range");
        }
        double const* up = std::lower_bound(prim, prim + ci.ng, e);
        if (up == prim) return group_mean(0);
        if (up == prim + ci.ng) return group_mean(ci.ng - 1);
        int const hi = static_cast<int>(up - prim);
        if (prim[hi] == e) return group_mean(hi);
        int const lo = hi - 1;
        double const y0 = group_mean(lo), y1 = group_mean(hi);
        double const tt = (std::log(e) - std::log(prim[lo])) / (std::log(prim[hi]) - std::log(prim[lo]));
        return y0 > 0.0 && y1 > 0.0 ? std::exp(std::log(y0) + tt * (std::log(y1) - std::log(y0)))
                                    : y0 + tt * (y1 - y0);
    }
    // :2678-2696
    double ElectronTrackedBremsEnergyLoss(double e, double dr) const
    {
        double const inv = interpolate(RREA_T_E_TRACKED_BREMS, e) * dr;
        if (!(inv > 0.0)) return 0.0;
        return inv * mean_conditional(RREA_C_BREMS_E, e);
    }
    // :2298-2324 (only the two rates the channel gates read)
    void ElectronGateRates(double e, double& moller_inv, double& brems_inv) const
    {
        if (!(e >= ix.charged_min_eV && e <= ix.charged_max_eV)) {
            fail(RREA_GPU_ERR_RANGE, "schema-6 electron energy outside the certified range");
        }
        interpolate(RREA_T_E_COLLISION, e);
        interpolate(RREA_T_E_SOFT_RAD, e);
        moller_inv = interpolate(RREA_T_E_HARD_MOLLER, e);
        brems_inv = interpolate(RREA_T_E_TRACKED_BREMS, e);
        interpolate(RREA_T_E_ELASTIC_TRANSPORT, e);
    }
    // :2477-2502
    double ElasticMeanFreePath(int species, double e, double dr) const
    {
        RreaElasticIndex const& el = ix.elastic[species];
        return semilogx(t.at(el.x), t.at(el.lx), t.at(el.mfp), el.n, e) / dr;
    }
    double ScreeningEta(int species, double e) const
    {
        RreaElasticIndex const& el = ix.elastic[species];
        return semilogx(t.at(el.x), t.at(el.lx), t.at(el.eta), el.n, e);
    }
    // :807-827
    static void log_bracket(double const* g, int n, double q, int& i, double& frac)
    {
        int const last = n - 1;
        if (!std::isfinite(q) || q < g[0] || q > g[last]) {
            fail(RREA_GPU_ERR_RANGE, "elastic-angle query outside its tabulated range");
        }
        if (q == g[0]) { i = 0; frac = 0.0; return; }
        if (q == g[last]) { i = last - 1; frac = 1.0; return; }
        int lo = 0, hi = last;
        while (hi - lo > 1) {
            int const m = (lo + hi) / 2;
            if (g[m] <= q) lo = m; else hi = m;
        }
        i = lo;
        double const llo = std::log(g[lo]), lhi = std::log(g[hi]);
        if (lhi == llo) { frac = (q == g[lo]) ? 0.0 : 1.0; return; }
        frac = (std::log(q) - llo) / (lhi - llo);
    }
    // :831-891
    double sample_gs_angle(RreaAngleIndex const& a, double e, double n, double u) const
    {
        int const np = a.np, nu = a.nu;
        int ie = 0, ip = 0;
        double te = 0.0, tn = 0.0;
        log_bracket(t.at(a.e), a.ne, e, ie, te);
        log_bracket(t.at(a.p), a.np, n, ip, tn);
        double const* omc = t.at(a.omc);
        double const* cu = t.at(a.u);
        auto cos_at_node = [&](int iu) {
            auto val = [&](int ei, int pi) { return omc[(static_cast<std::size_t>(ei) * np + pi) * nu + iu]; };
            double const la = std::log(val(ie, ip));
            double const lb = std::log(val(ie + 1, ip));
            double const lc = std::log(val(ie, ip + 1));
            double const ld = std::log(val(ie + 1, ip + 1));
            double const lxx = (1 - te) * (1 - tn) * la + te * (1 - tn) * lb + (1 - te) * tn * lc + te * tn * ld;
            return 1.0 - std::exp(lxx);
        };
        auto omc_at = [&](int iu) { return std::max(1.0 - cos_at_node(iu), std::numeric_limits<double>::min()); };
        int const first = 1, last = nu - 2;
        double one_minus_cos;
        if (last <= first) {
            one_minus_cos = omc_at(first);
        } else if (u <= cu[first]) {
            double const d1 = omc_at(first), d2 = omc_at(first + 1);
            double const u1 = cu[first], u2 = cu[first + 1];
            double const slope = std::log(d2 / d1) / std::log(u2 / u1);
            double const ueff = std::max(u, u1 * 1.0e-6);
            one_minus_cos = d1 * std::exp(slope * std::log(ueff / u1));
        } else if (u >= cu[last]) {
            one_minus_cos = omc_at(last);
        } else {
            int lo = first, hi = last;
            while (hi - lo > 1) {
                int const m = (lo + hi) / 2;
                if (cu[m] <= u) lo = m; else hi = m;
            }
            double const d0 = omc_at(lo), d1 = omc_at(hi);
            double const fu = std::log(u / cu[lo]) / std::log(cu[hi] / cu[lo]);
            one_minus_cos = d0 * std::exp(fu * std::log(d1 / d0));
        }
        double const c = 1.0 - std::min(2.0, one_minus_cos);
        return std::min(1.0, std::max(-1.0, c));
    }
    // :2504-2544
    double SampleGsCosTheta(int species, double e, double n, double u) const
    {
        require_charged(e);
        if (!std::isfinite(u) || u < 0.0 || u > 1.0) fail(RREA_GPU_ERR_INVALID_STATE, "GS cdf query not in [0,1]");
        bool const use_gs = e <= ix.gs_wentzel_transition_eV;
        RreaAngleIndex const& a = use_gs ? ix.gs[species] : ix.wentzel[species];
        double const* eg = t.at(a.e);
        if (e < eg[0] || e > eg[a.ne - 1]) fail(RREA_GPU_ERR_RANGE, "GS energy outside the model branch");
        if (!std::isfinite(n) || n < ix.gs_few_collision_threshold) {
            fail(RREA_GPU_ERR_INVALID_STATE, "GS path n below the multiple-scattering branch");
        }
        if (n >= ix.gs_isotropic_above_n) {
            g_elastic_branch[2].fetch_add(1, std::memory_order_relaxed);
            return 2.0 * u - 1.0;
        }
        g_elastic_branch[use_gs ? 0 : 1].fetch_add(1, std::memory_order_relaxed);
        return sample_gs_angle(a, e, n, u);
    }
    // :2546-2560
    double SampleSingleElasticCosTheta(int species, double e, double cdf_u) const
    {
        require_charged(e);
        g_elastic_branch[3].fetch_add(1, std::memory_order_relaxed);
        double const eta = ScreeningEta(species, e);
        double const u = std::min(std::max(cdf_u, 0.0), 1.0 - 1.0e-15);
        return 1.0 - 2.0 * eta * u / (1.0 + eta - u);
    }
    // :2584-2653
    double SampleMollerSecondaryEnergy(double e, double u) const
    {
        require_charged(e);
        return rrea_host::HostSampleConditional(t, RREA_C_MOLLER, e, u, true);
    }
    // :2698-2712
    double SampleBremsstrahlungPhotonEnergy(double e, double u) const
    {
        require_charged(e);
        return rrea_host::HostSampleConditional(t, RREA_C_BREMS_E, e, u, false);
    }
    // :3180-3194 and :2562-2575 (general sampler, log interpolation between groups)
    double SamplePositronBhabhaSecondaryEnergy(double e, double u) const
    {
        require_charged(e);
        return rrea_host::HostSampleConditional(t, RREA_C_BHABHA, e, u, false);
    }
    double SamplePositronBremsstrahlungPhotonEnergy(double e, double u) const
    {
        require_charged(e);
        return rrea_host::HostSampleConditional(t, RREA_C_BREMS_P, e, u, false);
    }
    // :2714-2760
    double SampleBremsstrahlungCosTheta(double e, double cdf_u) const
    {
        require_charged(e);
        cdf_u = std::max(0.0, std::min(1.0, cdf_u));
        if (cdf_u == 0.0) return 1.0;
        if (cdf_u == 1.0) return -1.0;
        double constexpr a = 0.625;
        auto g2 = [](double x) {
            if (x < 1.0e-3) {
                return x * x * (0.5 + x * (-1.0 / 3.0 + x * (1.0 / 8.0 + x * (-1.0 / 30.0 + x * (1.0 / 144.0)))));
            }
            return -std::expm1(-x) - x * std::exp(-x);
        };
        auto mix = [&](double uu) { return 0.25 * g2(a * uu) + 0.75 * g2(3.0 * a * uu); };
        double const umax = 2.0 * (1.0 + e / kMeC2);
        double const target = cdf_u * mix(umax);
        double lo = 0.0, hi = umax;
        for (int it = 0; it < 60; ++it) {
            double const mid = 0.5 * (lo + hi);
            if (mix(mid) < target) lo = mid; else hi = mid;
        }
        double const f = 0.5 * (lo + hi) / umax;
        return 1.0 - 2.0 * f * f;
    }
};

// ======================================================================
// Kinematics: O/RreaChargedInterleave.H, I/RreaLorentzPush.H,
// I/RreaSeedSchedule.H:31-43, O/RreaParticleInteraction.H:92-105, 1494-1506
// ======================================================================
double proper_velocity_from_kinetic(double k)
{
    if (k <= 0.0) return 0.0;
    double const g = 1.0 + k / kMeC2;
    return kC * std::sqrt(std::max(g * g - 1.0, 0.0));
}
double kinetic_from_proper_velocity(double ux, double uy, double uz)
{
    double const u2 = ux * ux + uy * uy + uz * uz;
    double const g = std::sqrt(1.0 + u2 / (kC * kC));
    return u2 * kMeC2 / ((kC * kC) * (g + 1.0));
}
double charged_speed(double k)
{
    if (!std::isfinite(k) || k < 0.0) return std::numeric_limits<double>::quiet_NaN();
    double const g = 1.0 + k / kMeC2;
    double const b2 = std::max(0.0, 1.0 - 1.0 / (g * g));
    return kC * std::sqrt(b2);
}
void normalize(double& x, double& y, double& z)
{
    double const n = std::sqrt(x * x + y * y + z * z);
    if (n <= 0.0) { x = 0.0; y = 0.0; z = 1.0; return; }
    x /= n; y /= n; z /= n;
}
void transverse_basis(double dx, double dy, double dz, double& b1x, double& b1y, double& b1z, double& b2x,
                      double& b2y, double& b2z)
{
    normalize(dx, dy, dz);
    double rx = 0.0, ry = 0.0, rz = 1.0;
    if (std::abs(dz) > 0.9) { rx = 1.0; rz = 0.0; }
    b1x = ry * dz - rz * dy;
    b1y = rz * dx - rx * dz;
    b1z = rx * dy - ry * dx;
    normalize(b1x, b1y, b1z);
    b2x = dy * b1z - dz * b1y;
    b2y = dz * b1x - dx * b1z;
    b2z = dx * b1y - dy * b1x;
    normalize(b2x, b2y, b2z);
}
void cone_direction(double ax, double ay, double az, double cos_t, double u_phi, double& ox, double& oy,
                    double& oz)
{
    normalize(ax, ay, az);
    double b1x, b1y, b1z, b2x, b2y, b2z;
    transverse_basis(ax, ay, az, b1x, b1y, b1z, b2x, b2y, b2z);
    cos_t = std::min(1.0, std::max(-1.0, cos_t));
    double const sin_t = std::sqrt(std::max(0.0, 1.0 - cos_t * cos_t));
    double const phi = kTwoPi * u_phi;
    double const cp = std::cos(phi), sp = std::sin(phi);
    ox = ax * cos_t + sin_t * (cp * b1x + sp * b2x);
    oy = ay * cos_t + sin_t * (cp * b1y + sp * b2y);
    oz = az * cos_t + sin_t * (cp * b1z + sp * b2z);
    normalize(ox, oy, oz);
}
int poisson_capped(double mean, double u, int kmax)
{
    if (mean <= 0.0) return 0;
    double p = std::exp(-mean);
    double cum = p;
    int k = 0;
    while (u > cum && k < kmax) {
        ++k;
        p *= mean / static_cast<double>(k);
        cum += p;
    }
    return k;
}
double unit_cycle(double u)
{
    u -= std::floor(u);
    return u < 0.0 ? u + 1.0 : u;
}
double moller_secondary_cos(double kp, double ks)
{
    kp = std::max(kp, 0.0);
    ks = std::max(ks, 0.0);
    if (kp <= 0.0 || ks <= 0.0) return 1.0;
    double const v = ks * (kp + 2.0 * kMeC2) / (kp * (ks + 2.0 * kMeC2));
    return std::sqrt(std::min(1.0, std::max(0.0, v)));
}
double moller_primary_cos(double kp, double ks)
{
    double const scat = std::max(0.0, kp - ks);
    if (kp <= 0.0 || scat <= 0.0) return 1.0;
    double const v = scat * (kp + 2.0 * kMeC2) / (kp * (scat + 2.0 * kMeC2));
    return std::sqrt(std::min(1.0, std::max(0.0, v)));
}
void moller_lab_directions(double px, double py, double pz, double kp, double ks, double u_az, double& opx,
                           double& opy, double& opz, double& osx, double& osy, double& osz)
{
    normalize(px, py, pz);
    u_az = unit_cycle(u_az);
    cone_direction(px, py, pz, moller_secondary_cos(kp, ks), u_az, osx, osy, osz);
    cone_direction(px, py, pz, moller_primary_cos(kp, ks), unit_cycle(u_az + 0.5), opx, opy, opz);
}
void photon_recoil(double k0, double eg, double gx, double gy, double gz, double& cx, double& cy, double& cz)
{
    eg = std::max(eg, 0.0);
    if (k0 <= 0.0 || eg <= 0.0) return;
    normalize(cx, cy, cz);
    normalize(gx, gy, gz);
    double const p0 = std::sqrt(std::max(0.0, k0 * (k0 + 2.0 * kMeC2)));
    double const px = p0 * cx - eg * gx, py = p0 * cy - eg * gy, pz = p0 * cz - eg * gz;
    double const n = std::sqrt(px * px + py * py + pz * pz);
    if (n > 0.0) {
        cx = px / n; cy = py / n; cz = pz / n;
        normalize(cx, cy, cz);
    }
}

struct FieldRange {
    double work = 0, ex = 0, ey = 0, ez = 0, bx = 0, by = 0, bz = 0, length = 0;
};

// O/RreaChargedInterleave.H:100-138 + I/RreaLorentzPush.H:21-46
void half_kick(FieldRange const& f, double half_dt, double q, double& k, double& dx, double& dy, double& dz)
{
    double const umag = proper_velocity_from_kinetic(k);
    double const s = q * (kC * kC / kMeC2) * half_dt;
    double const uxm = umag * dx + s * f.ex;
    double const uym = umag * dy + s * f.ey;
    double const uzm = umag * dz + s * f.ez;
    double const gamma = std::sqrt(1.0 + (uxm * uxm + uym * uym + uzm * uzm) / (kC * kC));
    double const tx = s * f.bx / (2.0 * gamma), ty = s * f.by / (2.0 * gamma), tz = s * f.bz / (2.0 * gamma);
    double const t2 = tx * tx + ty * ty + tz * tz;
    double const sx = 2.0 * tx / (1.0 + t2), sy = 2.0 * ty / (1.0 + t2), sz = 2.0 * tz / (1.0 + t2);
    double const ppx = uxm + uym * tz - uzm * ty;
    double const ppy = uym + uzm * tx - uxm * tz;
    double const ppz = uzm + uxm * ty - uym * tx;
    double const ux = uxm + ppy * sz - ppz * sy;
    double const uy = uym + ppz * sx - ppx * sz;
    double const uz = uzm + ppx * sy - ppy * sx;
    double const norm = std::sqrt(ux * ux + uy * uy + uz * uz);
    if (norm > 0.0 && std::isfinite(norm)) {
        dx = ux / norm; dy = uy / norm; dz = uz / norm;
    }
    k = std::max(0.0, k + 0.5 * f.work);
}

// ======================================================================
// Field gather: S/RreaAmrexAdvance.cpp:511-579, I/RreaFieldGatherStencil.H
// ======================================================================
struct Gather {
    FieldGrid const& fg;
    rrea_gpu_config const& cfg;
    double cell_er(int i, int j) const
    {
        std::size_t const lo = static_cast<std::size_t>(i) + static_cast<std::size_t>(fg.nr + 1) * j;
        std::size_t const hi = static_cast<std::size_t>(i + 1) + static_cast<std::size_t>(fg.nr + 1) * j;
        return 0.5 * ((fg.er[lo] + fg.amb_er[lo]) + (fg.er[hi] + fg.amb_er[hi]));
    }
    double cell_ez(int i, int j) const
    {
        std::size_t const lo = static_cast<std::size_t>(i) + static_cast<std::size_t>(fg.nr) * j;
        std::size_t const hi = static_cast<std::size_t>(i) + static_cast<std::size_t>(fg.nr) * (j + 1);
        return 0.5 * ((fg.ez[lo] + fg.amb_ez[lo]) + (fg.ez[hi] + fg.amb_ez[hi]));
    }
    double bt(int i, int j) const
    {
        return fg.bt[static_cast<std::size_t>(i) + static_cast<std::size_t>(fg.nr + 1) * j];
    }
    void at(double r, double z, double& er, double& ez, double& bth) const
    {
        bool const periodic = cfg.periodic_z != 0;
        double const fx = (r - cfg.r_lo) / fg.dr + 0.0 - 0.5;
        double const fz = (z - cfg.z_lo) / fg.dz + 0.0 - 0.5;
        int const ir0 = static_cast<int>(std::floor(fx));
        int const iz0 = static_cast<int>(std::floor(fz));
        double const tx = fx - static_cast<double>(ir0);
        double const tz = fz - static_cast<double>(iz0);
        int const i0 = std::max(0, std::min(fg.nr - 1, ir0));
        int const i1 = std::max(0, std::min(fg.nr - 1, ir0 + 1));
        int j0 = periodic ? iz0 : std::max(0, std::min(fg.nz - 1, iz0));
        int j1 = periodic ? iz0 + 1 : std::max(0, std::min(fg.nz - 1, iz0 + 1));
        if (periodic) {
            j0 = (j0 + fg.nz) % fg.nz;
            j1 = (j1 + fg.nz) % fg.nz;
        }
        auto bil = [&](double f00, double f01, double f10, double f11) {
            return (1.0 - tx) * ((1.0 - tz) * f00 + tz * f01) + tx * ((1.0 - tz) * f10 + tz * f11);
        };
        double const first_center = cfg.r_lo + 0.5 * fg.dr;
        double const axis = r >= first_center ? 1.0 : std::max(0.0, (r - cfg.r_lo) / (0.5 * fg.dr));
        er = bil(cell_er(i0, j0), cell_er(i0, j1), cell_er(i1, j0), cell_er(i1, j1)) * axis;
        ez = bil(cell_ez(i0, j0), cell_ez(i0, j1), cell_ez(i1, j0), cell_ez(i1, j1));
        // MaxwellBthetaAt, S/RreaAmrexAdvance.cpp:511-530
        if (r <= 0.0) {
            bth = 0.0;
        } else {
            double const fr = std::clamp(r / fg.dr, 0.0, static_cast<double>(fg.nr));
            double const fzz = std::clamp((z - fg.z_lo) / fg.dz, 0.0, static_cast<double>(fg.nz));
            int const a0 = std::min(static_cast<int>(std::floor(fr)), fg.nr - 1);
            int const b0 = std::min(static_cast<int>(std::floor(fzz)), fg.nz - 1);
            double const tr = fr - a0, tzz = fzz - b0;
            bth = (1.0 - tr) * ((1.0 - tzz) * bt(a0, b0) + tzz * bt(a0, b0 + 1))
                + tr * ((1.0 - tzz) * bt(a0 + 1, b0) + tzz * bt(a0 + 1, b0 + 1));
        }
    }
};

// O/RreaPathFieldWork.H:57-150 with I/RreaGaussLegendre8.H:24-60
FieldRange path_field_work(Gather const& g, Path const& path, double q, double begin, double end)
{
    FieldRange res;
    if (!(path.full > 0.0)) return res;
    begin = std::max(path.in_begin, begin);
    end = std::min(path.in_end, end);
    if (!(end > begin)) return res;
    double const pdx = (path.ex - path.sx) / path.full;
    double const pdy = (path.ey - path.sy) / path.full;
    double const pdz = (path.ez - path.sz) / path.full;
    static long double const kGl2 = 0.577350269189625764509148780501957L;
    for (Piece const& piece : path.pieces) {
        double const pb = std::max(begin, piece.begin);
        double const pe = std::min(end, piece.end);
        if (!(pe > pb)) continue;
        auto node = [&](double f, std::array<double, 7>& o) {
            double x, y, z;
            path.PointAtPiece(piece, f, x, y, z);
            double const r = std::hypot(x, y);
            double rad = 0.0, rc = 1.0, rs = 0.0;
            if (r > 0.0) {
                rad = (pdx * x + pdy * y) / r;
                rc = x / r;
                rs = y / r;
            }
            double er, ez, bth;
            g.at(r, z, er, ez, bth);
            double const work = q * (er * rad + ez * pdz) * 1.0;
            if (!std::isfinite(work) || !std::isfinite(er) || !std::isfinite(ez) || !std::isfinite(bth)) {
                fail(RREA_GPU_ERR_INVALID_STATE, "substep field-impulse gather is non-finite");
            }
            o = {work, er * rc, er * rs, ez, -bth * rs, bth * rc, 0.0};
        };
        double const mid = 0.5 * (pb + pe);
        double const half = 0.5 * (pe - pb);
        double const off = half * static_cast<double>(kGl2);
        std::array<double, 7> below, above;
        node(mid - off, below);
        node(mid + off, above);
        std::array<double, 7> integ;
        for (int c = 0; c < 7; ++c) integ[c] = half * (below[c] + above[c]);
        res.work += path.full * integ[0];
        res.ex += path.full * integ[1];
        res.ey += path.full * integ[2];
        res.ez += path.full * integ[3];
        res.bx += path.full * integ[4];
        res.by += path.full * integ[5];
        res.bz += path.full * integ[6];
        res.length += path.full * (pe - pb);
    }
    if (res.length > 0.0) {
        res.ex /= res.length; res.ey /= res.length; res.ez /= res.length;
        res.bx /= res.length; res.by /= res.length; res.bz /= res.length;
    }
    return res;
}

// ======================================================================
// Material path: O/RreaMaterialPath.H, with the density ratio of
// TransportDensityRatioAtZ (uniform or altitude profile)
// ======================================================================
struct Interval {
    double begin = 0, end = 0, length = 0, density = 1.0;
};
double positive_or(double v, double fb) { return v > 0.0 ? v : fb; }

}  // namespace

namespace {
DensityProfile g_profile;
}

// RreaAltitudeProfile::Interpolate, S/RreaAltitudeProfile.cpp:125-147
double DensityProfile::interpolate(double altitude) const
{
    if (!enabled()) fail(RREA_GPU_ERR_NOT_READY, "altitude profile was not loaded");
    if (altitude < altitude_m.front() || altitude > altitude_m.back() || std::isnan(altitude)) {
        fail(RREA_GPU_ERR_RANGE, "altitude " + std::to_string(altitude) + " m is outside the profile range");
    }
    auto const upper = std::upper_bound(altitude_m.begin(), altitude_m.end(), altitude);
    if (upper == altitude_m.begin()) return density_kg_m3.front();
    if (upper == altitude_m.end()) return density_kg_m3.back();
    std::size_t const hi = static_cast<std::size_t>(upper - altitude_m.begin());
    std::size_t const lo = hi - 1;
    double const span = altitude_m[hi] - altitude_m[lo];
    double const t = span > 0.0 ? (altitude - altitude_m[lo]) / span : 0.0;
    return (1.0 - t) * density_kg_m3[lo] + t * density_kg_m3[hi];
}

// RreaAltitudeProfile::LoadCsv's checks (S/RreaAltitudeProfile.cpp:97-117,
// density column loaded with require_positive) and the reference density
// the ratio is taken against (O/RreaWarpXCoupling.cpp:88-93).
void SetDensityProfile(DensityProfile p)
{
    if (p.altitude_m.empty() && p.density_kg_m3.empty()) {
        g_profile = DensityProfile{};
        return;
    }
    if (p.altitude_m.size() != p.density_kg_m3.size() || p.altitude_m.size() < 2) {
        fail(RREA_GPU_ERR_ARGUMENT, "altitude profile needs at least two rows");
    }
    for (std::size_t i = 0; i < p.altitude_m.size(); ++i) {
        if (!std::isfinite(p.altitude_m[i]) || !std::isfinite(p.density_kg_m3[i])) {
            fail(RREA_GPU_ERR_ARGUMENT, "altitude profile values must be finite");
        }
        if (i > 0 && p.altitude_m[i] <= p.altitude_m[i - 1]) {
            fail(RREA_GPU_ERR_ARGUMENT, "altitude profile altitudes must be strictly increasing");
        }
        if (!(p.density_kg_m3[i] > 0.0)) {
            fail(RREA_GPU_ERR_ARGUMENT, "altitude profile requires strictly positive densities");
        }
    }
    if (!(p.reference_density_kg_m3 > 0.0) || !std::isfinite(p.reference_density_kg_m3)
        || !std::isfinite(p.altitude_msl_at_z0_m)) {
        fail(RREA_GPU_ERR_ARGUMENT, "altitude profile needs a positive reference density and a finite datum");
    }
    g_profile = std::move(p);
}

DensityProfile const& BoundDensityProfile() { return g_profile; }

// O/RreaWarpXCoupling.cpp:79-95 (ProfileAltitudeMslAtZ, :67-71)
double DensityRatioAtZ(double uniform_ratio, double z_m)
{
    if (!g_profile.enabled()) return uniform_ratio;
    return g_profile.interpolate(g_profile.altitude_msl_at_z0_m + z_m) / g_profile.reference_density_kg_m3;
}

double StepDensityRatio(rrea_gpu_config const& cfg)
{
    return positive_or(DensityRatioAtZ(cfg.density_ratio, 0.5 * (cfg.z_lo + cfg.z_hi)),
                       positive_or(cfg.density_ratio, 1.0));
}

namespace {

// :87-114; `density_ratio` is the ratio without a profile and `fallback`
// the step's ratio
std::vector<Interval> build_intervals(Path const& path, double density_ratio, double fallback)
{
    std::vector<Interval> out;
    for (Piece const& piece : path.pieces) {
        if (!(piece.length > 0.0)) continue;
        // integrate_density_piece_m (:60-85): midpoint rule
        double dl = 0.0;
        {
            double const b = std::max(piece.begin, piece.begin);
            double const e = std::min(piece.end, piece.end);
            if (e > b && path.full > 0.0) {
                double x, y, z;
                path.PointAtPiece(piece, 0.5 * (b + e), x, y, z);
                dl = path.full * (e - b) * positive_or(DensityRatioAtZ(density_ratio, z), fallback);
            }
        }
        Interval iv;
        iv.begin = piece.begin;
        iv.end = piece.end;
        iv.length = piece.length;
        iv.density = positive_or(dl / piece.length, fallback);
        out.push_back(iv);
    }
    return out;
}
// :117-136
double density_path(std::vector<Interval> const& iv, Path const& path, double b, double e)
{
    b = std::max(path.in_begin, b);
    e = std::min(path.in_end, e);
    if (!(e > b)) return 0.0;
    double s = 0.0;
    for (Interval const& i : iv) {
        double const bb = std::max(b, i.begin), ee = std::min(e, i.end);
        if (ee > bb) s += path.full * (ee - bb) * i.density;
    }
    return s;
}
// :142-170
double fraction_at_density_path(std::vector<Interval> const& iv, Path const& path, double b, double e,
                                double target)
{
    b = std::max(path.in_begin, b);
    e = std::min(path.in_end, e);
    if (!std::isfinite(target) || target < 0.0) fail(RREA_GPU_ERR_INVALID_STATE, "sampled density path invalid");
    double rem = target;
    for (Interval const& i : iv) {
        double const bb = std::max(b, i.begin), ee = std::min(e, i.end);
        if (!(ee > bb) || !(i.density > 0.0)) continue;
        double const c = path.full * (ee - bb) * i.density;
        if (rem <= c) return bb + rem / (path.full * i.density);
        rem -= c;
    }
    return e;
}
// :175-199
double max_uniform_slice(std::vector<Interval> const& iv, Path const& path, uint64_t n)
{
    if (n == 0) fail(RREA_GPU_ERR_INVALID_STATE, "zero subcycles");
    double const span = path.in_end - path.in_begin;
    double const d = static_cast<double>(n);
    double m = 0.0;
    for (uint64_t i = 0; i < n; ++i) {
        m = std::max(m, density_path(iv, path, path.in_begin + static_cast<double>(i) / d * span,
                                     path.in_begin + static_cast<double>(i + 1U) / d * span));
    }
    return m;
}
// :213-222
double frozen_rate(double v)
{
    if (!std::isfinite(v) || v < 0.0) fail(RREA_GPU_ERR_INVALID_STATE, "frozen material-path rate invalid");
    return v;
}

// ======================================================================
// Substep sizing: O/RreaTransportStep.H:104-184
// ======================================================================
uint64_t driver_count(double amount, double per)
{
    return static_cast<uint64_t>(std::max(1.0, std::ceil(amount / per)));
}
uint64_t selected_material_subcycles(double max_tau, std::vector<Interval> const& iv, Path const& path,
                                     rrea_gpu_config const& cfg, bool& viol, double total_stp)
{
    double const target = cfg.max_optical_depth_per_substep;
    if (!(target > 0.0) || cfg.max_subcycles == 0) fail(RREA_GPU_ERR_ARGUMENT, "invalid subcycle controls");
    uint64_t const cap = cfg.max_subcycles;
    uint64_t const req = static_cast<uint64_t>(std::max(1.0, std::ceil(max_tau / target)));
    viol = req > cap;
    uint64_t sub = std::min(req, cap);
    for (;;) {
        double const maximum = total_stp * max_uniform_slice(iv, path, sub);
        double const tol = 64.0 * kEps * std::max(1.0, target);
        if (maximum <= target + tol) return sub;
        if (sub >= cap) { viol = true; return sub; }
        long double const est = std::ceil(static_cast<long double>(sub) * static_cast<long double>(maximum / target));
        uint64_t next = sub + 1U;
        if (est >= static_cast<long double>(cap)) next = cap;
        else if (est > static_cast<long double>(next)) next = static_cast<uint64_t>(est);
        sub = std::min(next, cap);
    }
}

// ======================================================================
// Continuous drag: O/RreaParticleInteraction.H:203-265,
// O/RreaChargedInterleave.H:157-292
// ======================================================================
struct Limit {
    double end = 0.0;
    bool reaches = false;
    bool valid = false;
};
template <typename F>
Limit limit_at_cutoff(double b, double e, double k, double cut, F&& loss_to)
{
    Limit r{b, false, false};
    if (!std::isfinite(b) || !std::isfinite(e) || !std::isfinite(k) || !std::isfinite(cut) || !(e >= b)
        || !(k >= cut) || !(cut >= 0.0)) {
        return r;
    }
    if (e == b) {
        r.valid = true;
        r.reaches = k == cut;
        return r;
    }
    double const to_cut = k - cut;
    double const req = loss_to(e);
    if (!std::isfinite(req) || req < 0.0) return r;
    r.valid = true;
    if (req < to_cut) { r.end = e; return r; }
    r.reaches = true;
    if (to_cut == 0.0) return r;
    double lo = b, hi = e;
    for (int it = 0; it < 56; ++it) {
        double const mid = 0.5 * (lo + hi);
        double const l = loss_to(mid);
        if (!std::isfinite(l) || l < 0.0) {
            r.valid = false;
            r.reaches = false;
            r.end = b;
            return r;
        }
        if (l < to_cut) lo = mid; else hi = mid;
    }
    r.end = 0.5 * (lo + hi);
    return r;
}

struct DragPlan {
    double end = 0.0;
    bool applied = false, limit_valid = true, reaches = false;
    double drag = 0, collision = 0, soft = 0, hard = 0, raw_collision = 0, collision_stp = 0;
};

template <typename DP>
DragPlan plan_drag(double b, double e, double k, double stop_e, double cut, DP&& dpath, double stp_col,
                   double stp_soft, double stp_hard)
{
    DragPlan p;
    p.end = b;
    if (!(e > b) || !(k > 0.0) || stop_e < cut) return p;
    p.collision_stp = stp_col;
    double const total = stp_col + stp_soft;
    Limit const lim = limit_at_cutoff(b, e, k, cut, [&](double re) { return total * dpath(b, re); });
    if (!lim.valid) { p.limit_valid = false; return p; }
    p.applied = true;
    p.reaches = lim.reaches;
    p.end = lim.end;
    double const path_m = dpath(b, p.end);
    p.raw_collision = stp_col * path_m;
    double const raw_soft = stp_soft * path_m;
    double const avail = std::max(0.0, k - cut);
    p.drag = lim.reaches ? avail : std::min(p.raw_collision + raw_soft, avail);
    p.collision = std::min(p.raw_collision, p.drag);
    p.soft = std::max(0.0, p.drag - p.collision);
    p.hard = std::min(stp_hard * path_m, avail);
    return p;
}

// ======================================================================
// Competing hazard: O/RreaParticleInteraction.H:1402-1492
// ======================================================================
struct Selection {
    bool valid = false, event = false;
    int channel = -1;
    double sampled = 0.0, total = 0.0;
};
Selection select_hazard(std::array<double, 3> const& taus, int count, double u1, double u2)
{
    Selection r;
    if (count < 1 || count > 3 || !std::isfinite(u1) || !std::isfinite(u2)) return r;
    for (int i = 0; i < count; ++i) {
        double const t = taus[static_cast<std::size_t>(i)];
        if (!std::isfinite(t) || t < 0.0) return r;
        r.total += t;
    }
    r.valid = std::isfinite(r.total);
    if (!r.valid) return r;
    u1 = std::max(0.0, std::min(1.0, u1));
    r.sampled = -std::log(std::max(1.0e-30, 1.0 - u1));
    if (!(r.sampled < r.total)) return r;
    r.event = true;
    u2 = std::max(0.0, std::min(1.0, u2));
    double const target = u2 * r.total;
    double cum = 0.0;
    int last_open = -1;
    for (int i = 0; i < count; ++i) {
        double const t = taus[static_cast<std::size_t>(i)];
        if (t > 0.0) last_open = i;
        cum += t;
        if (target < cum) { r.channel = i; return r; }
    }
    r.channel = last_open;
    r.valid = r.channel >= 0;
    r.event = r.valid;
    return r;
}

// ======================================================================
// Terminal / boundary helpers: O/RreaParticleInteraction.H:267-540
// ======================================================================
bool half_open_rz(double r, double z, double rlo, double rhi, double zlo, double zhi)
{
    return std::isfinite(r) && std::isfinite(z) && rhi > rlo && zhi > zlo && r >= rlo && r < rhi && z >= zlo
        && z < zhi;
}
bool cartesian_half_open(double x, double y, double z, double rlo, double rhi, double zlo, double zhi)
{
    if (!std::isfinite(x) || !std::isfinite(y)) return false;
    return half_open_rz(std::hypot(x, y), z, rlo, rhi, zlo, zhi);
}
bool advance_running(Path const& path, double f, double rlo, double rhi, double zlo, double zhi, double& rx,
                     double& ry, double& rz)
{
    double x, y, z;
    path.PointAtFull(f, x, y, z);
    double const wz = path.WrapZ(z);
    if (!cartesian_half_open(x, y, wz, rlo, rhi, zlo, zhi)) return false;
    rx = x;
    ry = y;
    rz = wz;
    return true;
}
struct EscapePolicy {
    bool escapes = false, invalidate = false;
};
EscapePolicy clipped_escape_policy(Path const& path, double er, double ez)
{
    EscapePolicy p;
    if (!std::isfinite(er) || !std::isfinite(ez)) {
        p.escapes = true;
        p.invalidate = true;
        return p;
    }
    double const cz = path.WrapZ(ez);
    bool const outside = path.OutsideCertified(er, cz);
    bool const strictly = er < path.rlo || er > path.rhi || (!path.periodic && (ez < path.zlo || ez > path.zhi));
    p.escapes = path.exits || outside;
    p.invalidate = p.escapes && !strictly;
    if (p.escapes) p.invalidate = true;  // clipped policy: RREA owns every escape
    return p;
}
struct Crossing {
    bool valid = false;
    double sr = 0, sz = 0, cr = 0, cz = 0;
    uint32_t faces = 0;
};
Crossing boundary_crossing(Path const& path)
{
    Crossing r;
    double cx, cy;
    path.PointAtFull(path.in_end, cx, cy, r.cz);
    r.cz = path.WrapZ(r.cz);
    r.cr = std::hypot(cx, cy);
    r.sr = std::hypot(path.sx, path.sy);
    r.sz = path.WrapZ(path.sz);
    double const scale = std::max(1.0, std::max(path.rhi, std::max(std::abs(path.zlo), std::abs(path.zhi))));
    double const tol = 512.0 * kEps * scale;
    bool const on_r = std::abs(r.cr - path.rhi) <= tol;
    bool const on_zlo = !path.periodic && std::abs(r.cz - path.zlo) <= tol;
    bool const on_zhi = !path.periodic && std::abs(r.cz - path.zhi) <= tol;
    double const dx = path.ex - path.sx, dy = path.ey - path.sy, dz = path.ez - path.sz;
    double const outward = cx * dx + cy * dy;
    // I/RreaSegmentDepositionRZ.H face bits: r_hi = 1, z_lo = 2, z_hi = 4
    if (on_r && outward > -tol * scale) { r.faces |= 1u; r.cr = path.rhi; }
    if (on_zlo && dz < 0.0) { r.faces |= 2u; r.cz = path.zlo; }
    if (on_zhi && dz > 0.0) { r.faces |= 4u; r.cz = path.zhi; }
    if (r.faces == 0u) {
        if (on_r) { r.faces |= 1u; r.cr = path.rhi; }
        if (on_zhi) { r.faces |= 4u; r.cz = path.zhi; }
    }
    r.valid = r.faces != 0u && std::isfinite(r.sr) && std::isfinite(r.sz) && std::isfinite(r.cr)
        && std::isfinite(r.cz);
    return r;
}

// ======================================================================
// Photon samplers: S/RreaInteractionTables.cpp:2272-2296, 2762-3127,
// 1374-1525, 3208-3253, 63-108; I/RreaUniformStream.H:21-53
// ======================================================================
struct UniformStream {
    uint64_t state;
    static uint64_t sm(uint64_t x)
    {
        x += 0x9E3779B97F4A7C15ULL;
        x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
        x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
        return x ^ (x >> 31);
    }
    UniformStream(double u1, double u2)
    {
        uint64_t b1, b2;
        std::memcpy(&b1, &u1, 8);
        std::memcpy(&b2, &u2, 8);
        uint64_t const h2 = sm(b2);
        state = sm(b1) ^ ((h2 << 32) | (h2 >> 32));
    }
    double next()
    {
        state += 0x9E3779B97F4A7C15ULL;
        uint64_t z = state;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
        z = z ^ (z >> 31);
        return static_cast<double>(z >> 11) * (1.0 / 9007199254740992.0);
    }
};

double clamp_unit(double v)
{
    if (!std::isfinite(v)) return 0.5;
    return std::max(0.0, std::min(1.0, v));
}
double wrap_unit(double v)
{
    if (!std::isfinite(v)) return 0.0;
    v = v - std::floor(v);
    if (v < 0.0) v += 1.0;
    return v;
}

struct PhotonRates {
    double compton, pe, nuclear, triplet;
    double total() const { return compton + pe + nuclear + triplet; }
};
PhotonRates photon_rates(Tables const& t, double e, double dr)
{
    if (!(e >= t.ix.photon_min_eV && e <= t.ix.photon_max_eV)) {
        fail(RREA_GPU_ERR_RANGE, "schema-6 photon energy outside the certified range");
    }
    return PhotonRates{t.interpolate(RREA_T_PH_COMPTON, e) * dr, t.interpolate(RREA_T_PH_PHOTOELECTRIC, e) * dr,
                       t.interpolate(RREA_T_PH_PAIR_NUCLEAR, e) * dr, t.interpolate(RREA_T_PH_PAIR_TRIPLET, e) * dr};
}
void require_photon(Tables const& t, double e)
{
    if (!std::isfinite(e) || !(e >= t.ix.photon_min_eV && e <= t.ix.photon_max_eV)) {
        fail(RREA_GPU_ERR_RANGE, "schema-6 photon sampler energy outside the certified range");
    }
}
// :2778-2804; 0 Compton, 1 photoelectric, 2 pair nuclear, 3 pair triplet
int sample_photon_channel(Tables const& t, double e, double u)
{
    require_photon(t, e);
    u = std::max(0.0, std::min(1.0, u));
    PhotonRates const r = photon_rates(t, e, 1.0);
    double const total = r.total();
    if (!(total > 0.0) || !std::isfinite(total)) fail(RREA_GPU_ERR_INVALID_STATE, "photon rates sum to zero");
    double const target = u * total;
    if (target < r.compton) return 0;
    if (target < r.compton + r.pe) return 1;
    if (target < r.compton + r.pe + r.nuclear) return 2;
    return 3;
}
struct ComptonState {
    double recoil, scattered, cos_theta;
};
// :2806-2871
ComptonState sample_klein_nishina(Tables const& t, double e, double draw_mu, double draw_accept)
{
    require_photon(t, e);
    if (e <= 0.0) fail(RREA_GPU_ERR_INVALID_STATE, "Compton sampler requires positive energy");
    draw_mu = std::max(0.0, std::min(1.0, draw_mu));
    draw_accept = std::max(0.0, std::min(1.0, draw_accept));
    UniformStream stream(draw_mu, draw_accept);
    double const alpha = e / kMeC2;
    double const eps0 = 1.0 / (1.0 + 2.0 * alpha);
    double const eps0sq = eps0 * eps0;
    double const a1 = -std::log(eps0);
    double const a2 = 0.5 * (1.0 - eps0sq);
    double epsilon = eps0, onecost = 0.0;
    for (int iter = 0; iter < 128; ++iter) {
        double const u1 = iter == 0 ? draw_mu : stream.next();
        double const u2 = iter == 0 ? draw_accept : stream.next();
        double epsilonsq;
        if (a1 > (a1 + a2) * u1) {
            epsilon = std::exp(-a1 * u2);
            epsilonsq = epsilon * epsilon;
        } else {
            epsilonsq = eps0sq + (1.0 - eps0sq) * u2;
            epsilon = std::sqrt(epsilonsq);
        }
        onecost = (1.0 - epsilon) / (epsilon * alpha);
        double const sint2 = onecost * (2.0 - onecost);
        double const greject = 1.0 - epsilon * sint2 / (1.0 + epsilonsq);
        if (greject >= stream.next()) break;
    }
    double mu = 1.0 - onecost;
    mu = std::max(-1.0, std::min(1.0, mu));
    ComptonState st;
    st.scattered = std::max(0.0, epsilon * e);
    st.recoil = std::max(0.0, e - st.scattered);
    st.cos_theta = mu;
    return st;
}
// :2878-2941 -> (photoelectron energy, binding energy)
void sample_photoelectric(Tables const& t, double e, double u, double& electron, double& binding)
{
    require_photon(t, e);
    RreaPhotoelectricIndex const& pi = t.ix.pe;
    double const* prim = t.t.at(pi.primary);
    double const* start = t.t.at(pi.start);
    double const* cu = t.t.at(pi.u);
    double const* bind = t.t.at(pi.binding);
    if (e < prim[0] || e > prim[pi.ng - 1]) fail(RREA_GPU_ERR_RANGE, "photoelectric primary out of range");
    u = std::max(0.0, std::min(1.0, u));
    double const* up = std::lower_bound(prim, prim + pi.ng, e);
    int g;
    if (up == prim) g = 0;
    else if (up == prim + pi.ng) g = pi.ng - 1;
    else if (*up == e) g = static_cast<int>(up - prim);
    else g = static_cast<int>(up - prim) - 1;
    int const b = static_cast<int>(start[g]), en = static_cast<int>(start[g + 1]);
    double const* row = std::lower_bound(cu + b, cu + en, u);
    int const r = row == cu + en ? en - 1 : static_cast<int>(row - cu);
    if (bind[r] > e) fail(RREA_GPU_ERR_INVALID_STATE, "photoelectric binding exceeds photon energy");
    binding = bind[r];
    electron = std::max(0.0, e - bind[r]);
}
// :2949-3044 (long double as in the reference)
double sample_photoelectron_cos(Tables const& t, double k, double draw)
{
    if (!(k == 0.0)) t.require_charged(k);
    long double const u = static_cast<long double>(clamp_unit(draw));
    if (u <= 0.0L) return -1.0;
    if (u >= 1.0L) return 1.0;
    long double const gamma = 1.0L + static_cast<long double>(k) / static_cast<long double>(kMeC2);
    long double const inv_g2 = 1.0L / (gamma * gamma);
    long double const beta = std::sqrt(std::max(0.0L, 1.0L - inv_g2));
    if (beta < 1.0e-4L) {
        long double lo = -1.0L, hi = 1.0L;
        for (int it = 0; it < 96; ++it) {
            long double const mid = 0.5L * (lo + hi);
            if (mid == lo || mid == hi) break;
            long double const cdf = (2.0L + mid * (3.0L - mid * mid)) / 4.0L;
            if (cdf < u) lo = mid; else hi = mid;
        }
        return static_cast<double>(0.5L * (lo + hi));
    }
    long double const b = 0.5L * gamma * (gamma - 1.0L) * (gamma - 2.0L);
    long double const c = -inv_g2;
    long double const t_lo = inv_g2 / (1.0L + beta);
    long double const t_hi = 1.0L + beta;
    auto prim = [c, b](long double x) {
        return -c / (3.0L * x * x * x) - (2.0L + b * c) / (2.0L * x * x) - (2.0L * b - 1.0L) / x - b * std::log(x);
    };
    long double const f_lo = prim(t_lo), f_hi = prim(t_hi);
    long double const total = f_hi - f_lo;
    if (!(total > 0.0L) || !std::isfinite(total)) fail(RREA_GPU_ERR_INVALID_STATE, "Sauter-Gavrila normalization");
    long double const target = (1.0L - u) * f_hi + u * f_lo;
    long double lo = t_lo, hi = t_hi;
    for (int it = 0; it < 128; ++it) {
        long double const mid = 0.5L * (lo + hi);
        if (mid == lo || mid == hi) break;
        if (prim(mid) < target) lo = mid; else hi = mid;
    }
    long double const tt = 0.5L * (lo + hi);
    return static_cast<double>(std::max(-1.0L, std::min(1.0L, (1.0L - tt) / beta)));
}
struct PairState {
    bool valid = false;
    double e_electron = 0, e_positron = 0, e_recoil = 0, local = 0;
    double edir[3] = {0, 0, 1}, pdir[3] = {0, 0, 1}, rdir[3] = {0, 0, 1};
    bool recoil = false;
};
void normalize_local(double& x, double& y, double& z)
{
    double const n = std::sqrt(x * x + y * y + z * z);
    if (n <= 0.0 || !std::isfinite(n)) { x = 0.0; y = 0.0; z = 1.0; return; }
    x /= n; y /= n; z /= n;
}
// :3053-3127 with BuildRreaPairEmpiricalFinalState :1384-1525; channel 2 nuclear, 3 triplet
PairState sample_pair(Tables const& t, double e, int channel, double d_inv, double d_polar, double d_azim)
{
    require_photon(t, e);
    PairState st;
    bool const triplet = channel == 3;
    double const threshold = triplet ? 4.0 * kMeC2 : 2.0 * kMeC2;
    if (!(std::isfinite(e) && e > threshold)) return st;
    RreaPairBankIndex const& pb = t.ix.pair[triplet ? 1 : 0];
    double const* prim = t.t.at(pb.primary);
    double const* start = t.t.at(pb.start);
    int sel = 0;
    if (e >= prim[pb.nb - 1]) {
        sel = pb.nb - 1;
    } else if (e > prim[0]) {
        double const* up = std::lower_bound(prim, prim + pb.nb, e);
        int const hi = static_cast<int>(up - prim);
        if (prim[hi] == e) {
            sel = hi;
        } else {
            int const lo = hi - 1;
            double const tt = (std::log(e) - std::log(prim[lo])) / (std::log(prim[hi]) - std::log(prim[lo]));
            sel = clamp_unit(d_polar) < tt ? hi : lo;
        }
    }
    std::size_t const b0 = static_cast<std::size_t>(start[sel]);
    std::size_t const size = static_cast<std::size_t>(start[sel + 1]) - b0;
    std::size_t const idx = std::min(size - 1, static_cast<std::size_t>(clamp_unit(d_inv) * static_cast<double>(size)));
    double const* rec = t.t.at(pb.records) + (b0 + idx) * RREA_PAIR_RECORD_DOUBLES;
    int const count = static_cast<int>(rec[0]);
    int es = -1, ps = -1, rs = -1;
    for (int slot = 0; slot < count; ++slot) {
        int const pdg = static_cast<int>(rec[1 + slot]);
        if (pdg == -11) ps = slot;
        else if (pdg == 11) { if (es < 0) es = slot; else rs = slot; }
    }
    if (es < 0 || ps < 0 || (triplet && rs < 0)) fail(RREA_GPU_ERR_INVALID_STATE, "pair record topology");
    double const avail = e - 2.0 * kMeC2;
    double const rot = kTwoPi * clamp_unit(d_azim);
    double const cr = std::cos(rot), sr = std::sin(rot);
    auto rotated = [&](int slot, double* d) {
        double const px = rec[7 + 3 * slot], py = rec[8 + 3 * slot], pz = rec[9 + 3 * slot];
        d[0] = cr * px - sr * py;
        d[1] = sr * px + cr * py;
        d[2] = pz;
        normalize_local(d[0], d[1], d[2]);
    };
    st.valid = true;
    st.e_electron = avail * rec[4 + es];
    st.e_positron = avail * rec[4 + ps];
    rotated(es, st.edir);
    rotated(ps, st.pdir);
    if (triplet) {
        st.recoil = true;
        st.e_recoil = avail * rec[4 + rs];
        rotated(rs, st.rdir);
    }
    double const tol = 64.0 * kEps * std::max(1.0, avail);
    auto sum = [&]() { return st.e_electron + st.e_positron + st.e_recoil; };
    double expl = sum();
    if (!std::isfinite(expl) || st.e_electron < 0.0 || st.e_positron < 0.0 || st.e_recoil < 0.0) {
        fail(RREA_GPU_ERR_INVALID_STATE, "pair record negative energy");
    }
    if (expl > avail) {
        if (expl - avail > tol) fail(RREA_GPU_ERR_INVALID_STATE, "pair record closure");
        double const scale = avail / expl;
        st.e_electron *= scale; st.e_positron *= scale; st.e_recoil *= scale;
        expl = sum();
    }
    st.local = avail - expl;
    auto reduce_largest = [&](double corr) {
        double* es_[3] = {&st.e_electron, &st.e_positron, &st.e_recoil};
        double** largest = std::max_element(es_, es_ + 3, [](double const* a, double const* b) { return *a < *b; });
        if (**largest < corr) fail(RREA_GPU_ERR_INVALID_STATE, "pair closure correction");
        **largest -= corr;
    };
    if (st.local < 0.0) {
        double const corr = -st.local;
        if (corr > tol) fail(RREA_GPU_ERR_INVALID_STATE, "pair negative remainder");
        reduce_largest(corr);
        st.local = 0.0;
    }
    double accounted = sum() + st.local;
    double resid = avail - accounted;
    if (std::abs(resid) > tol) fail(RREA_GPU_ERR_INVALID_STATE, "pair closure residual");
    if (resid >= 0.0) st.local += resid;
    else if (st.local >= -resid) st.local += resid;
    else reduce_largest(-resid);
    accounted = sum() + st.local;
    if (st.e_electron < 0.0 || st.e_positron < 0.0 || st.e_recoil < 0.0 || st.local < 0.0
        || std::abs(avail - accounted) > tol) {
        fail(RREA_GPU_ERR_INVALID_STATE, "pair nonnegative closure");
    }
    return st;
}
// O/RreaChargedInterleave.H:498-517
void rotate_to_axis(double ax, double ay, double az, double lx, double ly, double lz, double& ox, double& oy,
                    double& oz)
{
    normalize(ax, ay, az);
    normalize(lx, ly, lz);
    double b1x, b1y, b1z, b2x, b2y, b2z;
    transverse_basis(ax, ay, az, b1x, b1y, b1z, b2x, b2y, b2z);
    ox = lx * b1x + ly * b2x + lz * ax;
    oy = lx * b1y + ly * b2y + lz * ay;
    oz = lx * b1z + ly * b2z + lz * az;
    normalize(ox, oy, oz);
}
struct AnnihilationState {
    double e1 = 0, e2 = 0, cos1 = 1, azim = 0;
    bool valid = false, at_rest = false;
};
// :63-108
double annihilation_fraction(double gamma, double draw)
{
    if (gamma <= 1.0 + 1.0e-12) return 0.5;
    double const bcm = std::sqrt(std::max(0.0, (gamma - 1.0) / (gamma + 1.0)));
    double const emin = 0.5 * (1.0 - bcm), emax = 0.5 * (1.0 + bcm);
    double const u = clamp_unit(draw);
    double const gp1 = gamma + 1.0;
    double const a = 1.0 + 2.0 * gamma / (gp1 * gp1);
    auto F = [a, gp1](double x) { return a * std::log(x) - x + 1.0 / (gp1 * gp1 * x); };
    double const flo = F(emin), fhi = F(emax);
    double const span = fhi - flo;
    if (!(span > 0.0)) return 0.5;
    double const target = flo + u * span;
    double lo = emin, hi = emax;
    for (int it = 0; it < 64; ++it) {
        double const mid = 0.5 * (lo + hi);
        if (F(mid) < target) lo = mid; else hi = mid;
    }
    return std::max(emin, std::min(emax, 0.5 * (lo + hi)));
}
// :3208-3253
AnnihilationState sample_annihilation(Tables const& t, double k, double d_energy, double d_azim)
{
    if (!(k == 0.0)) t.require_charged(k);
    AnnihilationState st;
    k = std::max(0.0, k);
    double const gamma = 1.0 + k / kMeC2;
    double const total = 2.0 * kMeC2 + k;
    if (gamma <= 1.0 + 1.0e-10) {
        st.e1 = kMeC2;
        st.e2 = kMeC2;
        st.cos1 = 2.0 * clamp_unit(d_energy) - 1.0;
        st.azim = wrap_unit(d_azim);
        st.valid = true;
        st.at_rest = true;
        return st;
    }
    double const beta = std::sqrt(std::max(0.0, 1.0 - 1.0 / (gamma * gamma)));
    double const eps = annihilation_fraction(gamma, d_energy);
    st.e1 = eps * total;
    st.e2 = std::max(0.0, total - st.e1);
    if (st.e1 <= 0.0 || st.e2 <= 0.0) return st;
    double const denom = eps * gamma * beta;
    if (denom <= 0.0) return st;
    st.cos1 = std::max(-1.0, std::min(1.0, (eps * (gamma + 1.0) - 1.0) / denom));
    st.azim = wrap_unit(d_azim);
    st.valid = true;
    st.at_rest = false;
    return st;
}

}  // namespace

// ======================================================================
// Electron phase: O/RreaElectronTransport.cpp:9-902 (+ O/RreaTransportStep.H
// prologue/escape/writeback :720-905)
// ======================================================================
namespace {
std::vector<double> g_planes;
}  // namespace

void SetPlanes(std::vector<double> planes) { g_planes = std::move(planes); }
std::vector<double> const& Planes() { return g_planes; }

bool AccumulatePlaneCrossings(std::vector<PlaneCrossing> const& crossings, std::vector<double>& bins)
{
    for (PlaneCrossing const& c : crossings) {
        std::size_t const base = static_cast<std::size_t>(c.plane) * 10U;
        if (c.plane < 0 || base + 10U > bins.size() || (c.direction != 1 && c.direction != -1)
            || !std::isfinite(c.weight) || !(c.weight >= 0.0) || !std::isfinite(c.r) || !(c.r >= 0.0)) {
            return false;
        }
        std::size_t const d = c.direction > 0 ? 0U : 1U;
        bins[base + d] += c.weight;
        if (c.local_runaway) bins[base + 2U + d] += c.weight;
        if (c.at_least_one_mev) bins[base + 4U + d] += c.weight;
        if (c.local_runaway) {
            bins[base + 6U + d] += c.weight * c.r;
            bins[base + 8U + d] += c.weight * c.r * c.r;
        }
    }
    return true;
}

namespace {

// defer_cd_electron_plane_crossings (O/RreaTransportStep.H:249-332) for one
// electron continuous segment [b, eff].
void defer_plane_crossings(Tables const& tables, rrea_gpu_config const& cfg, Gather const& gather, Path const& path,
                           std::vector<Interval> const& iv, double b, double eff, double weight, double k_before,
                           double stopping_energy, double drag, bool hm_enabled, std::vector<PlaneCrossing>& out)
{
    if (g_planes.empty() || !(eff > b)) return;
    double bx, by, bz, ex, ey, ez;
    path.PointAtFull(b, bx, by, bz);
    path.PointAtFull(eff, ex, ey, ez);
    // electron_realized_continuous_loss_ev_per_m at the frozen energy, STP
    double const fixed_stp = tables.ElectronCollisionLoss(stopping_energy, 1.0)
        + tables.ElectronSoftRadiativeDrag(stopping_energy, 1.0);
    double const cut = cfg.low_energy_cutoff_eV;
    bool const valid = ForEachPlaneCrossing(bz, ez, g_planes, [&](std::size_t i, double sf, int direction) {
        double const f = b + sf * (eff - b);
        double x, y, z;
        path.PointAtFull(f, x, y, z);
        double const r = std::hypot(x, y);
        double const raw = fixed_stp * density_path(iv, path, b, f);
        double const kc = std::max(0.0, k_before - std::min(drag, raw));
        bool local = false;
        if (kc >= cut) {
            double const rho = positive_or(DensityRatioAtZ(cfg.density_ratio, z), 1.0);
            double fer, fez, fbt;
            gather.at(r, z, fer, fez, fbt);
            double mean_drag = 0.0;
            if (kc > 0.0 && rho > 0.0) {
                double const hard = hm_enabled ? tables.ElectronHardMollerEnergyLoss(kc, rho) : 0.0;
                mean_drag = (tables.ElectronCollisionLoss(kc, rho) + tables.ElectronSoftRadiativeDrag(kc, rho)) + hard
                    + tables.ElectronTrackedBremsEnergyLoss(kc, rho);
            }
            double const magnitude = std::hypot(fer, fez);
            local = std::isfinite(magnitude) && std::isfinite(mean_drag) && mean_drag >= 0.0 && magnitude > mean_drag;
        }
        out.push_back(PlaneCrossing{static_cast<int>(i), direction, weight, r, local, kc >= 1.0e6});
    });
    if (!valid) fail(RREA_GPU_ERR_GEOMETRY, "plane crossing enumeration received invalid geometry");
}

}  // namespace

void ApplyElectronTransport(TableSet const& ts, rrea_gpu_config const& cfg, FieldGrid const& field, int step,
                            double dt_s, ChargedTile& tile, StepOutputs& out)
{
    Tables const tables(ts);
    Gather const gather{field, cfg};
    double const rlo = cfg.r_lo, rhi = cfg.r_hi, zlo = cfg.z_lo, zhi = cfg.z_hi;
    bool const periodic = cfg.periodic_z != 0;
    double const cutoff = cfg.low_energy_cutoff_eV;
    double const photon_cut = cfg.photon_cutoff_eV;
    double const hm_thr = ts.index().hard_moller_threshold_eV;
    bool const hm_enabled = cfg.debug_disable_hard_moller == 0;
    // RreaParticleInteraction.cpp:27-35
    double const density_ratio = StepDensityRatio(cfg);
    uint64_t const seed = cfg.rng_seed;
    uint64_t const step_key = static_cast<uint64_t>(std::max(step, 0));
    double const w_air = ts.index().w_air_eV_per_pair;

    out.subcycles.assign(static_cast<std::size_t>(tile.n), 0);
    out.events.assign(static_cast<std::size_t>(tile.n), 0);
    out.disposition.assign(static_cast<std::size_t>(tile.n), -1);
    std::vector<uint64_t>& out_subcycles = out.subcycles;
    std::vector<uint64_t>& out_events = out.events;
    std::vector<int32_t>& out_disposition = out.disposition;

    // OpenMP over 64-particle chunks, schedule(dynamic,1), per-chunk logs
    // merged in chunk order (O/RreaElectronTransport.cpp:42-58, 892-897).
    constexpr int64_t kChunk = 64;
    int64_t const n_chunks = (tile.n + kChunk - 1) / kChunk;
    std::vector<StepOutputs> chunk_out(static_cast<std::size_t>(n_chunks));
    std::vector<int> chunk_err(static_cast<std::size_t>(n_chunks), 0);
    std::vector<std::string> chunk_msg(static_cast<std::size_t>(n_chunks));
#pragma omp parallel for schedule(dynamic, 1) if (n_chunks > 1)
    for (int64_t chunk = 0; chunk < n_chunks; ++chunk) {
      StepOutputs& cout = chunk_out[static_cast<std::size_t>(chunk)];
      try {
      int64_t const ip_end = std::min(tile.n, (chunk + 1) * kChunk);
      for (int64_t ip = chunk * kChunk; ip < ip_end; ++ip) {
        if (!(tile.id[ip] > 0)) continue;
        std::size_t const sp = static_cast<std::size_t>(ip);
        uint64_t lineage = 0;  // TransportSideEffects::spawn_transient_lineage (O/RreaTransportLog.H:179)
        int current_process = 0;
        // ---- BeginRunningChargedParticle (O/RreaTransportStep.H:720-820)
        uint64_t const key = static_cast<uint64_t>(std::llabs(tile.id[ip]))
            ^ (static_cast<uint64_t>(tile.cpu ? tile.cpu[ip] : 0) << 40);
        double const weight = tile.w[ip];
        if (weight <= 0.0) {
            tile.id[ip] = -tile.id[ip];
            out_disposition[sp] = 3;
            continue;
        }
        if (tile.prev_r[ip] > rhi + 1.0e-9 * rhi) {
            fail(RREA_GPU_ERR_GEOMETRY, "RREA electron survived outside the domain");
        }
        double dx = tile.prev_ux[ip], dy = tile.prev_uy[ip], dz = tile.prev_uz[ip];
        double k = kinetic_from_proper_velocity(dx, dy, dz);
        normalize(dx, dy, dz);
        double const seed_r = tile.prev_r[ip], seed_th = tile.prev_theta[ip];
        double run_x = seed_r * std::cos(seed_th);
        double run_y = seed_r * std::sin(seed_th);
        double run_z = tile.prev_z[ip];
        double const r_particle = seed_r, z_particle = run_z;

        auto build_chord = [&](double req_dt, Path& path) -> bool {
            // O/RreaParticleInteraction.H:110-161
            if (!std::isfinite(req_dt) || !std::isfinite(dt_s) || !(req_dt >= 0.0) || !(dt_s > 0.0)) return false;
            double const speed = charged_speed(k);
            double const dn = std::sqrt(dx * dx + dy * dy + dz * dz);
            if (!std::isfinite(speed) || !std::isfinite(dn) || !(dn > 0.0)) return false;
            double const sc = speed * req_dt / dn;
            double const exx = run_x + sc * dx, eyy = run_y + sc * dy, ezz = run_z + sc * dz;
            path = ClipRz(std::hypot(run_x, run_y), std::atan2(run_y, run_x), run_z, std::hypot(exx, eyy),
                          std::atan2(eyy, exx), ezz, rlo, rhi, zlo, zhi, periodic);
            return std::isfinite(path.full) && path.in_begin == 0.0;
        };

        Path driver;
        bool const driver_valid = build_chord(dt_s, driver);
        EscapePolicy escape = clipped_escape_policy(driver, std::hypot(driver.ex, driver.ey), driver.ez);
        double const ds = driver_valid ? driver.in_length : 0.0;
        std::vector<Interval> const driver_iv = build_intervals(driver, density_ratio, density_ratio);
        double const driver_span = std::max(driver.in_end, 1.0e-6);
        double const field_work = path_field_work(gather, driver, -1.0, 0.0, 1.0).work / driver_span;

        double const chord_dpath = density_path(driver_iv, driver, driver.in_begin, driver.in_end);
        double transported_dpath = 0.0, transported_len = 0.0;
        double particle_density =
            ds > 0.0 ? chord_dpath / ds : positive_or(DensityRatioAtZ(cfg.density_ratio, z_particle), density_ratio);
        Path path = driver;
        std::vector<Interval> iv = driver_iv;

        auto push_source = [&](int kind, double r, double z, double w, double sec, double loss) {
            cout.sources.push_back(Source{kind, r, z, w, sec, loss, ip});
        };
        auto push_segment = [&](int kind, std::array<double, 7> const& a, uint64_t ch, uint32_t faces) {
            Segment s;
            s.kind = kind;
            for (int c = 0; c < 7; ++c) s.a[c] = a[c];
            s.channel = ch;
            s.faces = faces;
            s.parent_index = ip;
            cout.segments.push_back(s);
        };
        auto add_secondary = [&](int species, double x, double y, double z, double sx, double sy, double sz,
                                 double e, double birth) {
            Secondary s;
            s.species = species;
            s.process = current_process;
            s.x = x; s.y = y; s.z = z;
            s.dx = sx; s.dy = sy; s.dz = sz;
            s.w = weight;
            s.energy = e;
            s.birth = birth;
            s.root_key = key;
            s.lineage = lineage++;
            s.root_species = 0;
            s.parent_index = ip;
            cout.secondaries.push_back(s);
        };
        // TransportStep::deposit_local_energy_as_ion_pairs (O/RreaTransportStep.H:530-561)
        auto deposit_local = [&](double r, double z, double w, double e) {
            if (w <= 0.0 || e <= 0.0) return;
            double const pw = w * e / std::max(w_air, 1.0);
            if (pw <= 0.0) return;
            push_source(0, r, z, pw, 0.0, w_air);
        };
        // CommitChargedEscape (O/RreaTransportStep.H:829-863)
        auto commit_escape = [&]() {
            double const u = proper_velocity_from_kinetic(k);
            tile.ux[ip] = u * dx;
            tile.uy[ip] = u * dy;
            tile.uz[ip] = u * dz;
            Crossing const c = boundary_crossing(path);
            // TransportSideEffects::AccumulateChargedEscape (O/RreaTransportLog.H:573-584)
            if (!c.valid) fail(RREA_GPU_ERR_GEOMETRY, "charged escape has no certified absorbing-face crossing");
            push_segment(1, {r_particle, z_particle, c.sr, c.sz, c.cr, c.cz, -weight}, 1u, c.faces);
            if (escape.invalidate) tile.id[ip] = -tile.id[ip];
            out_disposition[sp] = 1;
        };
        auto demote = [&](double r, double z) {
            // O/RreaElectronTransport.cpp:151-174 and :856-879
            current_process = 12;  // LowEnergyDemotion
            push_source(1, r, z, weight, 0.0, 0.0);
            deposit_local(r, z, weight, k);
            push_segment(0, {r_particle, z_particle, r, z, -weight, 0.0, 0.0}, 2u, 0u);
            tile.id[ip] = -tile.id[ip];
            out_disposition[sp] = 2;
        };

        // :129-175
        bool const below = k < cutoff;
        int const initial = escape.escapes ? 1 : (below ? 2 : 0);
        if (initial == 1 && below) { commit_escape(); continue; }
        if (initial == 2) { demote(r_particle, z_particle); continue; }
        if (ds <= 0.0) {
            if (escape.escapes) commit_escape();
            else out_disposition[sp] = 0;
            continue;
        }
        if (driver_iv.empty()) fail(RREA_GPU_ERR_INVALID_STATE, "positive length but no material segments");

        // competing STP rates (O/RreaChargedFinalStates.H:107-152)
        auto competing = [&](double e) {
            std::array<double, 3> s{};
            bool const m_open = hm_enabled && hm_thr > 0.0 && e > 2.0 * hm_thr;
            if (m_open) {
                double const mfp = tables.ElectronHardMollerMeanFreePath(e, 1.0);
                s[0] = frozen_rate(mfp > 0.0 ? 1.0 / mfp : 0.0);
            } else {
                s[0] = frozen_rate(0.0);
            }
            bool const b_open = std::isfinite(e) && std::isfinite(photon_cut) && e > photon_cut;
            if (b_open) {
                double const mfp = tables.ElectronBremsstrahlungMeanFreePath(e, 1.0);
                s[1] = frozen_rate(mfp > 0.0 ? 1.0 / mfp : 0.0);
            } else {
                s[1] = frozen_rate(0.0);
            }
            s[2] = 0.0;
            return s;
        };
        // RreaChargedChannelOpenAt (O/RreaChargedFinalStates.H:56-96)
        auto channel_open = [&](int ch, double e) {
            double mi, bi;
            tables.ElectronGateRates(e, mi, bi);
            if (ch == 0) return hm_enabled && (hm_thr > 0.0 && e > 2.0 * hm_thr) && mi > 0.0;
            if (ch == 1) return (std::isfinite(e) && std::isfinite(photon_cut) && e > photon_cut) && bi > 0.0;
            return false;
        };

        std::array<double, 3> const init = competing(k);
        double const driver_dpath = chord_dpath / driver_span;
        bool viol = false;
        uint64_t subcycles = selected_material_subcycles((init[0] * driver_dpath) + (init[1] * driver_dpath),
                                                         driver_iv, driver, cfg, viol, init[0] + init[1]);
        {
            double const gs_n = frozen_rate([&] {
                double const mfp = tables.ElasticMeanFreePath(0, k, 1.0);
                return mfp > 0.0 ? 1.0 / mfp : 0.0;
            }()) * driver_dpath;
            double const ke = std::max(k, cutoff);
            double const drag_est = (ke > 0.0 ? tables.ElectronCollisionLoss(ke, 1.0)
                                                    + tables.ElectronSoftRadiativeDrag(ke, 1.0)
                                              : 0.0)
                * driver_dpath;
            double const impulse = std::max(cfg.max_field_impulse_fraction * k,
                                            std::max(cfg.field_impulse_floor_eV, 1.0));
            uint64_t const gsd = driver_count(std::min(gs_n, cfg.gs_total_collision_cap),
                                              std::max(cfg.max_gs_collisions_per_substep, 1.0));
            uint64_t const imd = driver_count(std::abs(field_work) + drag_est, impulse);
            subcycles = std::min<uint64_t>(std::max({subcycles, gsd, imd}), cfg.max_subcycles);
        }
        if (cfg.strict_transport_guards && viol) {
            fail(RREA_GPU_ERR_GUARD, "strict transport guard: optical-depth subcycle cap exceeded");
        }
        out_subcycles[sp] = subcycles;

        bool exited = false;
        uint64_t completed = 0;
        bool terminated_mid = false;
        double mid_r = r_particle, mid_z = z_particle;
        double const sub_dt = dt_s / static_cast<double>(subcycles);
        FieldRange sub_field;
        double sub_dt_eff = 0.0;
        uint64_t events = 0;

        auto elapsed_at = [&](double f) {
            double const within = std::min(1.0, std::max(0.0, f));
            return std::min(1.0, (static_cast<double>(completed) + within) / static_cast<double>(subcycles));
        };
        auto mark_stopped = [&](double f) {
            if (path.exits && f >= path.in_end) { exited = true; return; }
            double x, y, z;
            path.PointAtFull(f, x, y, z);
            double const r = std::hypot(x, y);
            if (!cartesian_half_open(x, y, z, rlo, rhi, zlo, zhi)) { exited = true; return; }
            mid_z = z;
            mid_r = r;
            terminated_mid = true;
        };
        // apply_electron_continuous_segment (:294-400)
        auto continuous = [&](double b, double e, double stop_e) -> Limit {
            auto dp = [&](double bb, double ee) { return density_path(iv, path, bb, ee); };
            double sc = 0, ss = 0, sh = 0;
            bool const need = (e > b) && (k > 0.0) && !(stop_e < cutoff);
            if (need) {
                sc = frozen_rate(tables.ElectronCollisionLoss(stop_e, 1.0));
                ss = frozen_rate(tables.ElectronSoftRadiativeDrag(stop_e, 1.0));
                sh = (hm_enabled && hm_thr > 0.0 && stop_e > 2.0 * hm_thr)
                    ? frozen_rate(tables.ElectronHardMollerEnergyLoss(stop_e, 1.0))
                    : 0.0;
            }
            DragPlan const plan = plan_drag(b, e, k, stop_e, cutoff, dp, sc, ss, sh);
            if (!plan.limit_valid) fail(RREA_GPU_ERR_INVALID_STATE, "continuous stopping has no monotone cutoff point");
            if (!plan.applied) return Limit{b, false, true};
            // RreaPartitionContinuousIonPairs (O/RreaChargedInterleave.H:157-196)
            if (plan.collision > 0.0 && plan.raw_collision > 0.0) {
                for (Interval const& i : iv) {
                    double const bb = std::max(b, i.begin), ee = std::min(plan.end, i.end);
                    if (!(ee > bb)) continue;
                    double const raw = path.full * (ee - bb) * i.density * plan.collision_stp;
                    double const loss = plan.collision * raw / plan.raw_collision;
                    double const pw = weight * loss / std::max(w_air, 1.0);
                    if (!(pw > 0.0)) continue;
                    double x, y, z;
                    path.PointAtFull(0.5 * (bb + ee), x, y, z);
                    push_source(0, std::hypot(x, y), z, pw, 0.5 * cutoff, w_air);
                }
            }
            defer_plane_crossings(tables, cfg, gather, path, iv, b, plan.end, weight, k, stop_e, plan.drag, hm_enabled,
                                  cout.crossings);
            k = std::max(0.0, k - plan.drag);
            if (plan.reaches) k = cutoff;
            return Limit{plan.end, plan.reaches, true};
        };

        // RreaRunChargedSubstepInterleave (O/RreaChargedInterleave.H:693-732)
        double sb = 0.0, se = 0.0;
        uint64_t cur_sub = 0;
        RunChargedSubstepInterleave(
            subcycles, k, cutoff, completed, exited,
            // build_substep (:535-598): chord, intervals, field sub-range, leading half kick
            [&](uint64_t sub, double& b, double& e) {
                cur_sub = sub;
                Path np;
                if (!build_chord(sub_dt, np)) return false;
                path = np;
                if (!(path.full > 0.0) || !(path.in_length > 0.0)) {
                    exited = path.exits;
                    return false;
                }
                iv = build_intervals(path, density_ratio, density_ratio);
                if (iv.empty()) fail(RREA_GPU_ERR_INVALID_STATE, "microchord with no material intervals");
                for (Interval const& i : iv) {
                    transported_dpath += i.length * i.density;
                    transported_len += i.length;
                }
                sb = path.in_begin;
                se = path.in_end;
                b = sb;
                e = se;
                sub_field = path_field_work(gather, path, -1.0, sb, se);
                sub_dt_eff = sub_dt * (se - sb);
                half_kick(sub_field, 0.5 * sub_dt_eff, -1.0, k, dx, dy, dz);
                if (k < cutoff) {
                    mark_stopped(sb);
                    return false;
                }
                return true;
            },
            // run_events: RreaRunChargedEventInterleave (:546-664)
            [&](uint64_t sub, double b, double e) {
                std::array<double, 3> stp{};
                uint64_t rng_index = 0;
                double ex = 0, ey = 0, ez = 0, er = 0;
                RunChargedEventInterleave(
                    b, e, k, cutoff, 2, kEventCap, "electron",
                    [&](double frozen, double rb, double re) {
                        stp = competing(frozen);
                        double const seg_dp = density_path(iv, path, rb, re);
                        return std::array<double, 3>{stp[0] * seg_dp, stp[1] * seg_dp, 0.0};
                    },
                    [&](uint64_t ordinal) {
                        if (!try_live_hazard_index(0, sub, ordinal, rng_index)) {
                            fail(RREA_GPU_ERR_RNG_OVERFLOW, "electron repeated-hazard RNG index overflow");
                        }
                        ++events;
                        uint64_t const od_ch =
                            ordinal == 0 ? kElectronCompetingOpticalDepth : kElectronContinuationOpticalDepth;
                        uint64_t const cc_ch = ordinal == 0 ? kElectronCompetingChannel : kElectronContinuationChannel;
                        double const u1 = rng_uniform(seed, key, step_key, rng_index, od_ch);
                        double const u2 = rng_uniform(seed, key, step_key, rng_index, cc_ch);
                        return std::pair<double, double>{u1, u2};
                    },
                    [&](double tau, double rb, double re) {
                        return fraction_at_density_path(iv, path, rb, re, tau / (stp[0] + stp[1]));
                    },
                    [&](double rb, double re, double frozen) {
                        Limit const l = continuous(rb, re, frozen);
                        return SegmentLimit{l.reaches, l.end};
                    },
                    [&](double f) { mark_stopped(f); },
                    [&](double f) {
                        path.PointAtFull(f, ex, ey, ez);
                        er = std::hypot(ex, ey);
                    },
                    [&](int ch, double en) { return channel_open(ch, en); },
                    [&](int channel, double ev_frac) {
                        double const birth = elapsed_at(ev_frac);
                        if (channel == 0) {
                            // RreaApplyHardMollerFinalState (O/RreaChargedFinalStates.H:164-225)
                            double const kb = k;
                            double sec = tables.SampleMollerSecondaryEnergy(
                                kb, rng_uniform(seed, key, step_key, rng_index, kHardMollerEnergy));
                            sec = std::max(hm_thr, std::min(sec, 0.5 * kb));
                            double pdx = dx, pdy = dy, pdz = dz, sdx = dx, sdy = dy, sdz = dz;
                            moller_lab_directions(dx, dy, dz, kb, sec,
                                                  rng_uniform(seed, key, step_key, rng_index, kHardMollerAzimuth),
                                                  pdx, pdy, pdz, sdx, sdy, sdz);
                            k = std::max(0.0, kb - sec);
                            dx = pdx; dy = pdy; dz = pdz;
                            current_process = 2;  // HardMoller
                            add_secondary(0, ex, ey, ez, sdx, sdy, sdz, sec, birth);
                            push_source(0, er, ez, weight, sec, sec);
                        } else if (channel == 1) {
                            // RreaApplyBremsFinalState (O/RreaChargedFinalStates.H:329-394)
                            double const kb = k;
                            double const eu = rng_uniform(seed, key, step_key, rng_index, kBremsEnergy);
                            double const sampled = tables.SampleBremsstrahlungPhotonEnergy(kb, eu);
                            // RreaClassifyBremsEnergyDisposition (O/RreaParticleInteraction.H:1552-1574)
                            double const eg = std::min(std::max(sampled, 0.0), std::max(kb, 0.0));
                            double const after = std::max(0.0, std::max(kb, 0.0) - eg);
                            bool const tracked = std::isfinite(photon_cut) && photon_cut >= 0.0 && eg >= photon_cut;
                            double gx = dx, gy = dy, gz = dz;
                            double const ct = tables.SampleBremsstrahlungCosTheta(
                                kb, rng_uniform(seed, key, step_key, rng_index, kBremsAngle));
                            cone_direction(dx, dy, dz, ct, rng_uniform(seed, key, step_key, rng_index, kBremsAzimuth),
                                           gx, gy, gz);
                            photon_recoil(kb, eg, gx, gy, gz, dx, dy, dz);
                            k = after;
                            current_process = 4;  // Bremsstrahlung
                            if (tracked) {
                                add_secondary(2, ex, ey, ez, gx, gy, gz, eg, birth);
                            } else if (eg > 0.0) {
                                deposit_local(er, ez, weight, eg);
                            }
                        }
                        return true;
                    });
            },
            [&] { return terminated_mid; },
            // finish_interleaved_substep (:502-524): elastic scatter, trailing half kick
            [&](uint64_t sub, double, double) {
                if (k >= cutoff) {
                    // apply_gs_elastic_scatter (O/RreaTransportStep.H:371-423)
                    double const mfp = tables.ElasticMeanFreePath(0, k, 1.0);
                    double const gs_n = frozen_rate(mfp > 0.0 ? 1.0 / mfp : 0.0) * density_path(iv, path, sb, se);
                    if (gs_n > 0.0) {
                        auto gkey = [&](uint64_t ch, uint64_t inner) {
                            return rng_uniform(seed, key, step_key, (sub << 8) | inner, ch);
                        };
                        auto deflect = [&](double ct, double uphi) {
                            double nx, ny, nz;
                            cone_direction(dx, dy, dz, ct, uphi, nx, ny, nz);
                            dx = nx; dy = ny; dz = nz;
                        };
                        double const few = ts.index().gs_few_collision_threshold;
                        if (gs_n < few) {
                            int const cap = static_cast<int>(std::ceil(3.0 * few));
                            if (cap >= 255) fail(RREA_GPU_ERR_INVALID_STATE, "GS few-collision cap too large");
                            int const cnt = poisson_capped(gs_n, gkey(kElectronGsFewCount, 0), cap);
                            for (int q = 0; q < cnt; ++q) {
                                double const ct = tables.SampleSingleElasticCosTheta(
                                    0, k, gkey(kElectronGsFewScatter, static_cast<uint64_t>(q + 1)));
                                deflect(ct, gkey(kElectronGsFewAzimuth, static_cast<uint64_t>(q + 1)));
                            }
                        } else {
                            double const ct = tables.SampleGsCosTheta(0, k, gs_n, gkey(kElectronGsAngle, 0));
                            deflect(ct, gkey(kElectronGsAzimuth, 0));
                        }
                    }
                }
                half_kick(sub_field, 0.5 * sub_dt_eff, -1.0, k, dx, dy, dz);
                if (k < cutoff) {
                    mark_stopped(se);
                    return true;
                }
                return false;
            },
            // RreaAdvanceRunningChargedPosition (O/RreaParticleInteraction.H:368-392)
            [&](double e) { return advance_running(path, e, rlo, rhi, zlo, zhi, run_x, run_y, run_z); },
            [&] { return path.exits; });
        (void)cur_sub;
        out_events[sp] = events;
        if (exited) {
            escape = clipped_escape_policy(path, std::hypot(path.ex, path.ey), path.ez);
        }
        if (transported_len > 0.0) particle_density = transported_dpath / transported_len;
        double const end_r = std::hypot(run_x, run_y);
        double fer, fez, fbt;
        gather.at(end_r, run_z, fer, fez, fbt);
        // electron_ensemble_mean_drag_ev_per_m (O/RreaTransportStep.H:226-247)
        double threshold = 0.0;
        {
            double const ke = std::max(k, cutoff);
            if (ke > 0.0 && particle_density > 0.0) {
                double const hard = hm_enabled ? tables.ElectronHardMollerEnergyLoss(ke, particle_density) : 0.0;
                threshold = (tables.ElectronCollisionLoss(ke, particle_density)
                             + tables.ElectronSoftRadiativeDrag(ke, particle_density))
                    + hard + tables.ElectronTrackedBremsEnergyLoss(ke, particle_density);
            }
        }
        // RreaEvaluateElectronStatePolicy (O/RreaParticleInteraction.H:1302-1317)
        bool const below_cut = k < cutoff;
        bool const nonrunaway = hm_thr > 0.0 && k <= hm_thr && std::hypot(fer, fez) <= threshold;
        int disp;
        if (exited) disp = 1;
        else if (terminated_mid) disp = 2;
        else disp = (below_cut || nonrunaway) ? 2 : 0;
        if (disp == 1) { commit_escape(); continue; }
        if (disp == 2) {
            double const dr_ = terminated_mid ? mid_r : end_r;
            double const dz_ = terminated_mid ? mid_z : run_z;
            demote(dr_, dz_);
            continue;
        }
        // CommitSurvivorChargedWriteback (O/RreaTransportStep.H:874-905)
        double const um = proper_velocity_from_kinetic(k);
        tile.ux[ip] = um * dx;
        tile.uy[ip] = um * dy;
        tile.uz[ip] = um * dz;
        tile.r[ip] = end_r;
        tile.theta[ip] = std::atan2(run_y, run_x);
        tile.z[ip] = run_z;
        push_segment(0, {r_particle, z_particle, end_r, run_z, -weight, 0.0, 0.0}, 0u, 0u);
        out_disposition[sp] = 0;
      }
      } catch (OracleError const& e) {
        chunk_err[static_cast<std::size_t>(chunk)] = e.code;
        chunk_msg[static_cast<std::size_t>(chunk)] = e.what();
      }
    }
    for (int64_t chunk = 0; chunk < n_chunks; ++chunk) {
        if (chunk_err[static_cast<std::size_t>(chunk)] != 0) {
            fail(chunk_err[static_cast<std::size_t>(chunk)], chunk_msg[static_cast<std::size_t>(chunk)]);
        }
    }
    for (auto& c : chunk_out) {
        out.secondaries.insert(out.secondaries.end(), c.secondaries.begin(), c.secondaries.end());
        out.sources.insert(out.sources.end(), c.sources.begin(), c.sources.end());
        out.segments.insert(out.segments.end(), c.segments.begin(), c.segments.end());
        out.crossings.insert(out.crossings.end(), c.crossings.begin(), c.crossings.end());
    }
}

// ======================================================================
// Positron phase: O/RreaPositronTransport.cpp:9-878 with the Bhabha and
// brems final states of O/RreaChargedFinalStates.H:226-394 and
// TransportStep::spawn_positron_annihilation (O/RreaTransportStep.H:563-702).
// ======================================================================
namespace {

// spawn_positron_annihilation (O/RreaTransportStep.H:563-702).  `emit` and
// `deposit` are the caller's secondary and ion-pair sinks.
template <typename Emit, typename Deposit, typename Source>
void spawn_annihilation(Tables const& tables, double photon_cut, double x, double y, double z, double r,
                        double zs, double ax, double ay, double az, double w, double k, bool at_rest,
                        double d_energy, double d_azim, double birth, Emit&& emit, Deposit&& deposit,
                        Source&& source)
{
    if (w <= 0.0) return;
    normalize(ax, ay, az);
    double const ka = at_rest ? 0.0 : std::max(k, 0.0);
    AnnihilationState const an = sample_annihilation(tables, ka, d_energy, d_azim);
    double g1x, g1y, g1z;
    cone_direction(ax, ay, az, an.cos1, an.azim, g1x, g1y, g1z);
    double const e1 = std::max(an.e1, 0.0), e2 = std::max(an.e2, 0.0);
    double g2x = -g1x, g2y = -g1y, g2z = -g1z;
    if (!an.at_rest && e2 > 0.0) {
        double const p = std::sqrt(std::max(0.0, ka * (ka + 2.0 * kMeC2)));
        g2x = (p * ax - e1 * g1x) / e2;
        g2y = (p * ay - e1 * g1y) / e2;
        g2z = (p * az - e1 * g1z) / e2;
        normalize(g2x, g2y, g2z);
    }
    double local = 0.0;
    if (e1 >= photon_cut) emit(x, y, z, g1x, g1y, g1z, e1, birth);
    else local += e1;
    if (e2 >= photon_cut) emit(x, y, z, g2x, g2y, g2z, e2, birth);
    else local += e2;
    if (at_rest && k > 0.0) deposit(r, zs, w, k);
    if (local > 0.0) deposit(r, zs, w, local);
    source(r, zs, w);
}

}  // namespace

void ApplyPositronTransport(TableSet const& ts, rrea_gpu_config const& cfg, FieldGrid const& field, int step,
                            double dt_s, ChargedTile& tile, StepOutputs& out)
{
    Tables const tables(ts);
    Gather const gather{field, cfg};
    double const rlo = cfg.r_lo, rhi = cfg.r_hi, zlo = cfg.z_lo, zhi = cfg.z_hi;
    bool const periodic = cfg.periodic_z != 0;
    double const cutoff = cfg.low_energy_cutoff_eV;
    double const photon_cut = cfg.photon_cutoff_eV;
    double const hm_thr = ts.index().hard_moller_threshold_eV;
    double const density_ratio = StepDensityRatio(cfg);
    uint64_t const seed = cfg.rng_seed;
    uint64_t const step_key = static_cast<uint64_t>(std::max(step, 0));
    double const w_air = ts.index().w_air_eV_per_pair;

    out.subcycles.assign(static_cast<std::size_t>(tile.n), 0);
    out.events.assign(static_cast<std::size_t>(tile.n), 0);
    out.disposition.assign(static_cast<std::size_t>(tile.n), -1);

    constexpr int64_t kChunk = 64;
    int64_t const n_chunks = (tile.n + kChunk - 1) / kChunk;
    std::vector<StepOutputs> chunk_out(static_cast<std::size_t>(n_chunks));
    std::vector<int> chunk_err(static_cast<std::size_t>(n_chunks), 0);
    std::vector<std::string> chunk_msg(static_cast<std::size_t>(n_chunks));
#pragma omp parallel for schedule(dynamic, 1) if (n_chunks > 1)
    for (int64_t chunk = 0; chunk < n_chunks; ++chunk) {
      StepOutputs& cout = chunk_out[static_cast<std::size_t>(chunk)];
      try {
      int64_t const ip_end = std::min(tile.n, (chunk + 1) * kChunk);
      for (int64_t ip = chunk * kChunk; ip < ip_end; ++ip) {
        if (!(tile.id[ip] > 0)) continue;
        std::size_t const sp = static_cast<std::size_t>(ip);
        uint64_t lineage = 0;
        int current_process = 0;
        // ---- BeginRunningChargedParticle (O/RreaTransportStep.H:720-820), charge +1
        uint64_t const key = static_cast<uint64_t>(std::llabs(tile.id[ip]))
            ^ (static_cast<uint64_t>(tile.cpu ? tile.cpu[ip] : 0) << 40);
        double const weight = tile.w[ip];
        if (weight <= 0.0) {
            tile.id[ip] = -tile.id[ip];
            out.disposition[sp] = 3;
            continue;
        }
        if (tile.prev_r[ip] > rhi + 1.0e-9 * rhi) {
            fail(RREA_GPU_ERR_GEOMETRY, "RREA positron survived outside the domain");
        }
        double dx = tile.prev_ux[ip], dy = tile.prev_uy[ip], dz = tile.prev_uz[ip];
        double k = kinetic_from_proper_velocity(dx, dy, dz);
        normalize(dx, dy, dz);
        double const seed_r = tile.prev_r[ip], seed_th = tile.prev_theta[ip];
        double run_x = seed_r * std::cos(seed_th);
        double run_y = seed_r * std::sin(seed_th);
        double run_z = tile.prev_z[ip];
        double const x_particle = run_x, y_particle = run_y;
        double const r_particle = seed_r, z_particle = run_z;

        auto build_chord = [&](double req_dt, Path& path) -> bool {
            // O/RreaParticleInteraction.H:110-161
            if (!std::isfinite(req_dt) || !std::isfinite(dt_s) || !(req_dt >= 0.0) || !(dt_s > 0.0)) return false;
            double const speed = charged_speed(k);
            double const dn = std::sqrt(dx * dx + dy * dy + dz * dz);
            if (!std::isfinite(speed) || !std::isfinite(dn) || !(dn > 0.0)) return false;
            double const sc = speed * req_dt / dn;
            double const exx = run_x + sc * dx, eyy = run_y + sc * dy, ezz = run_z + sc * dz;
            path = ClipRz(std::hypot(run_x, run_y), std::atan2(run_y, run_x), run_z, std::hypot(exx, eyy),
                          std::atan2(eyy, exx), ezz, rlo, rhi, zlo, zhi, periodic);
            return std::isfinite(path.full) && path.in_begin == 0.0;
        };

        Path driver;
        bool const driver_valid = build_chord(dt_s, driver);
        EscapePolicy escape = clipped_escape_policy(driver, std::hypot(driver.ex, driver.ey), driver.ez);
        double const ds = driver_valid ? driver.in_length : 0.0;
        std::vector<Interval> const driver_iv = build_intervals(driver, density_ratio, density_ratio);
        double const driver_span = std::max(driver.in_end, 1.0e-6);
        double const field_work = path_field_work(gather, driver, 1.0, 0.0, 1.0).work / driver_span;
        Path path = driver;
        std::vector<Interval> iv = driver_iv;

        auto push_source = [&](int kind, double r, double z, double w, double sec, double loss) {
            cout.sources.push_back(Source{kind, r, z, w, sec, loss, ip});
        };
        auto push_segment = [&](int kind, std::array<double, 7> const& a, uint64_t ch, uint32_t faces) {
            Segment sg;
            sg.kind = kind;
            for (int c = 0; c < 7; ++c) sg.a[c] = a[c];
            sg.channel = ch;
            sg.faces = faces;
            sg.parent_index = ip;
            cout.segments.push_back(sg);
        };
        auto add_secondary = [&](int species, double x, double y, double z, double sx, double sy, double sz,
                                 double e, double birth) {
            Secondary s2;
            s2.species = species;
            s2.process = current_process;
            s2.x = x; s2.y = y; s2.z = z;
            s2.dx = sx; s2.dy = sy; s2.dz = sz;
            s2.w = weight;
            s2.energy = e;
            s2.birth = birth;
            s2.root_key = key;
            s2.lineage = lineage++;
            s2.root_species = 1;
            s2.parent_index = ip;
            cout.secondaries.push_back(s2);
        };
        auto deposit_local = [&](double r, double z, double w, double e) {
            if (w <= 0.0 || e <= 0.0) return;
            double const pw = w * e / std::max(w_air, 1.0);
            if (pw <= 0.0) return;
            push_source(0, r, z, pw, 0.0, w_air);
        };
        auto annihilate = [&](double x, double y, double z, double r, double w, double ke, bool at_rest,
                              uint64_t idx, double birth) {
            current_process = 9;  // PositronAnnihilation
            spawn_annihilation(
                tables, photon_cut, x, y, z, r, z, dx, dy, dz, w, ke, at_rest,
                rng_uniform(seed, key, step_key, idx, kAnnihilationPolar),
                rng_uniform(seed, key, step_key, idx, kAnnihilationAzimuth), birth,
                [&](double px, double py, double pz, double gx, double gy, double gz, double e, double b) {
                    add_secondary(2, px, py, pz, gx, gy, gz, e, b);
                },
                deposit_local, [&](double rr, double zz, double ww) { push_source(2, rr, zz, ww, 0.0, 0.0); });
        };
        // CommitChargedEscape (O/RreaTransportStep.H:829-863), mesh weight +w
        auto commit_escape = [&]() {
            double const u = proper_velocity_from_kinetic(k);
            tile.ux[ip] = u * dx;
            tile.uy[ip] = u * dy;
            tile.uz[ip] = u * dz;
            Crossing const c = boundary_crossing(path);
            // TransportSideEffects::AccumulateChargedEscape (O/RreaTransportLog.H:573-584)
            if (!c.valid) fail(RREA_GPU_ERR_GEOMETRY, "charged escape has no certified absorbing-face crossing");
            push_segment(1, {r_particle, z_particle, c.sr, c.sz, c.cr, c.cz, weight}, 1u, c.faces);
            if (escape.invalidate) tile.id[ip] = -tile.id[ip];
            out.disposition[sp] = 1;
        };

        // :112-160
        bool const below = k < cutoff;
        if (escape.escapes && below) { commit_escape(); continue; }
        if (!escape.escapes && below) {
            annihilate(x_particle, y_particle, z_particle, r_particle, weight, k, true, 0, 1.0);
            push_segment(0, {r_particle, z_particle, r_particle, z_particle, weight, 0.0, 0.0}, 4u, 0u);
            tile.id[ip] = -tile.id[ip];
            out.disposition[sp] = 2;
            continue;
        }
        if (ds <= 0.0) {
            if (escape.escapes) commit_escape();
            else out.disposition[sp] = 0;
            continue;
        }
        if (driver_iv.empty()) fail(RREA_GPU_ERR_INVALID_STATE, "positron path has positive length but no material");

        // RreaChargedCompetingStpRates(is_positron) (O/RreaChargedFinalStates.H:107-152)
        auto competing = [&](double e) {
            std::array<double, 3> s{};
            bool const b_open = !(hm_thr > 0.0 && e <= hm_thr);
            if (b_open) {
                double const mfp = tables.PositronHardBhabhaMeanFreePath(e, 1.0);
                s[0] = frozen_rate(mfp > 0.0 ? 1.0 / mfp : 0.0);
            } else {
                s[0] = frozen_rate(0.0);
            }
            if (e > photon_cut) {
                double const mfp = tables.PositronBremsstrahlungMeanFreePath(e, 1.0);
                s[1] = frozen_rate(mfp > 0.0 ? 1.0 / mfp : 0.0);
            } else {
                s[1] = frozen_rate(0.0);
            }
            double const mfp = tables.PositronAnnihilationMeanFreePath(e, 1.0);
            s[2] = frozen_rate(mfp > 0.0 ? 1.0 / mfp : 0.0);
            return s;
        };
        // RreaChargedChannelOpenAt(is_positron) (O/RreaChargedFinalStates.H:56-81)
        auto channel_open = [&](int ch, double e) {
            double bi, ri, ai;
            tables.PositronGateRates(e, bi, ri, ai);
            if (ch == 0) return !(hm_thr > 0.0 && e <= hm_thr) && bi > 0.0;
            if (ch == 1) return e > photon_cut && ri > 0.0;
            if (ch == 2) return ai > 0.0;
            return false;
        };

        std::array<double, 3> const init = competing(k);
        double const init_total = init[0] + init[1] + init[2];
        double const driver_dpath = density_path(driver_iv, driver, driver.in_begin, driver.in_end) / driver_span;
        bool viol = false;
        uint64_t subcycles =
            selected_material_subcycles(init_total * driver_dpath, driver_iv, driver, cfg, viol, init_total);
        {
            double const gs_n = frozen_rate([&] {
                double const mfp = tables.ElasticMeanFreePath(1, k, 1.0);
                return mfp > 0.0 ? 1.0 / mfp : 0.0;
            }()) * driver_dpath;
            double const drag_est = tables.PositronCollisionLoss(std::max(k, cutoff), 1.0) * driver_dpath;
            double const impulse = std::max(cfg.max_field_impulse_fraction * k,
                                            std::max(cfg.field_impulse_floor_eV, 1.0));
            uint64_t const gsd = driver_count(std::min(gs_n, cfg.gs_total_collision_cap),
                                              std::max(cfg.max_gs_collisions_per_substep, 1.0));
            uint64_t const imd = driver_count(std::abs(field_work) + drag_est, impulse);
            subcycles = std::min<uint64_t>(std::max({subcycles, gsd, imd}), cfg.max_subcycles);
        }
        if (cfg.strict_transport_guards && viol) {
            fail(RREA_GPU_ERR_GUARD, "strict transport guard: optical-depth subcycle cap exceeded");
        }
        out.subcycles[sp] = subcycles;

        bool exited = false;
        bool annihilated = false;
        uint64_t completed = 0;
        bool stopped = false;
        double stop_x = x_particle, stop_y = y_particle, stop_z = z_particle, stop_r = r_particle;
        double stop_elapsed = 1.0;
        double const sub_dt = dt_s / static_cast<double>(subcycles);
        FieldRange sub_field;
        double sub_dt_eff = 0.0;
        uint64_t events = 0;

        auto elapsed_at = [&](double f) {
            double const within = std::min(1.0, std::max(0.0, f));
            return std::min(1.0, (static_cast<double>(completed) + within) / static_cast<double>(subcycles));
        };
        auto mark_stopped = [&](double f) {
            if (path.exits && f >= path.in_end) { exited = true; return; }
            double x, y, z;
            path.PointAtFull(f, x, y, z);
            if (!cartesian_half_open(x, y, z, rlo, rhi, zlo, zhi)) { exited = true; return; }
            stop_x = x;
            stop_y = y;
            stop_z = z;
            stop_r = std::hypot(x, y);
            stop_elapsed = elapsed_at(f);
            stopped = true;
        };
        // apply_positron_continuous_segment (:268-365)
        auto continuous = [&](double b, double e, double stop_e) -> Limit {
            auto dp = [&](double bb, double ee) { return density_path(iv, path, bb, ee); };
            double sc = 0, ss = 0;
            bool const need = (e > b) && (k > 0.0) && !(stop_e < cutoff);
            if (need) {
                sc = frozen_rate(tables.PositronCollisionLoss(stop_e, 1.0));
                ss = frozen_rate(tables.PositronSoftRadiativeDrag(stop_e, 1.0));
            }
            DragPlan const plan = plan_drag(b, e, k, stop_e, cutoff, dp, sc, ss, 0.0);
            if (!plan.limit_valid) fail(RREA_GPU_ERR_INVALID_STATE, "positron stopping has no monotone cutoff point");
            if (!plan.applied) return Limit{b, false, true};
            k = std::max(0.0, k - plan.drag);
            if (plan.reaches) k = cutoff;
            if (plan.collision > 0.0 && plan.raw_collision > 0.0) {
                for (Interval const& i : iv) {
                    double const bb = std::max(b, i.begin), ee = std::min(plan.end, i.end);
                    if (!(ee > bb)) continue;
                    double const raw = path.full * (ee - bb) * i.density * plan.collision_stp;
                    double const loss = plan.collision * raw / plan.raw_collision;
                    double const pw = weight * loss / std::max(w_air, 1.0);
                    if (!(pw > 0.0)) continue;
                    double x, y, z;
                    path.PointAtFull(0.5 * (bb + ee), x, y, z);
                    push_source(0, std::hypot(x, y), z, pw, 0.0, w_air);
                }
            }
            return Limit{plan.end, plan.reaches, true};
        };

        // RreaRunChargedSubstepInterleave (O/RreaChargedInterleave.H:693-732)
        double sb = 0.0, se = 0.0;
        RunChargedSubstepInterleave(
            subcycles, k, cutoff, completed, exited,
            [&](uint64_t, double& b, double& e) {
                Path np;
                if (!build_chord(sub_dt, np)) return false;
                path = np;
                if (!(path.full > 0.0) || !(path.in_length > 0.0)) {
                    exited = path.exits;
                    return false;
                }
                iv = build_intervals(path, density_ratio, density_ratio);
                if (iv.empty()) fail(RREA_GPU_ERR_INVALID_STATE, "positron microchord with no material intervals");
                sb = path.in_begin;
                se = path.in_end;
                b = sb;
                e = se;
                sub_field = path_field_work(gather, path, 1.0, sb, se);
                sub_dt_eff = sub_dt * (se - sb);
                half_kick(sub_field, 0.5 * sub_dt_eff, 1.0, k, dx, dy, dz);
                if (k < cutoff) {
                    mark_stopped(sb);
                    return false;
                }
                return true;
            },
            // RreaRunChargedEventInterleave (:546-664) with three channels
            [&](uint64_t sub, double b, double e) {
                std::array<double, 3> stp{};
                uint64_t rng_index = 0;
                double ex = 0, ey = 0, ez = 0, er = 0;
                RunChargedEventInterleave(
                    b, e, k, cutoff, 3, kEventCap, "positron",
                    [&](double frozen, double rb, double re) {
                        stp = competing(frozen);
                        double const seg_dp = density_path(iv, path, rb, re);
                        return std::array<double, 3>{stp[0] * seg_dp, stp[1] * seg_dp, stp[2] * seg_dp};
                    },
                    [&](uint64_t ordinal) {
                        if (!try_live_hazard_index(1, sub, ordinal, rng_index)) {
                            fail(RREA_GPU_ERR_RNG_OVERFLOW, "positron repeated-hazard RNG index overflow");
                        }
                        ++events;
                        uint64_t const od_ch =
                            ordinal == 0 ? kPositronCompetingOpticalDepth : kPositronContinuationOpticalDepth;
                        uint64_t const cc_ch = ordinal == 0 ? kPositronCompetingChannel : kPositronContinuationChannel;
                        double const u1 = rng_uniform(seed, key, step_key, rng_index, od_ch);
                        double const u2 = rng_uniform(seed, key, step_key, rng_index, cc_ch);
                        return std::pair<double, double>{u1, u2};
                    },
                    [&](double tau, double rb, double re) {
                        return fraction_at_density_path(iv, path, rb, re, tau / (stp[0] + stp[1] + stp[2]));
                    },
                    [&](double rb, double re, double frozen) {
                        Limit const l = continuous(rb, re, frozen);
                        return SegmentLimit{l.reaches, l.end};
                    },
                    [&](double f) { mark_stopped(f); },
                    [&](double f) {
                        path.PointAtFull(f, ex, ey, ez);
                        er = std::hypot(ex, ey);
                    },
                    [&](int ch, double en) { return channel_open(ch, en); },
                    [&](int channel, double ev_frac) {
                        double const birth = elapsed_at(ev_frac);
                        if (channel == 0) {
                            // RreaApplyBhabhaFinalState (O/RreaChargedFinalStates.H:238-288)
                            double const kb = k;
                            double const sec = std::min(
                                tables.SamplePositronBhabhaSecondaryEnergy(
                                    kb, rng_uniform(seed, key, step_key, rng_index, kPositronBhabhaEnergy)),
                                std::max(0.0, kb));
                            if (sec > 0.0 && !(hm_thr > 0.0 && sec < hm_thr)) {
                                double pdx = dx, pdy = dy, pdz = dz, sdx = dx, sdy = dy, sdz = dz;
                                moller_lab_directions(dx, dy, dz, kb, sec,
                                                      rng_uniform(seed, key, step_key, rng_index, kPositronBhabhaAzimuth),
                                                      pdx, pdy, pdz, sdx, sdy, sdz);
                                k = std::max(0.0, kb - sec);
                                dx = pdx; dy = pdy; dz = pdz;
                                current_process = 3;  // HardBhabha
                                add_secondary(0, ex, ey, ez, sdx, sdy, sdz, sec, birth);
                                push_source(2, er, ez, weight, 0.0, sec);
                            }
                        } else if (channel == 1) {
                            // RreaApplyBremsFinalState, positron CDF (O/RreaChargedFinalStates.H:329-394)
                            double const kb = k;
                            double const eu = rng_uniform(seed, key, step_key, rng_index, kPositronBremsEnergy);
                            double const sampled = tables.SamplePositronBremsstrahlungPhotonEnergy(kb, eu);
                            double const eg = std::min(std::max(sampled, 0.0), std::max(kb, 0.0));
                            double const after = std::max(0.0, std::max(kb, 0.0) - eg);
                            bool const tracked = std::isfinite(photon_cut) && photon_cut >= 0.0 && eg >= photon_cut;
                            double gx = dx, gy = dy, gz = dz;
                            double const ct = tables.SampleBremsstrahlungCosTheta(
                                kb, rng_uniform(seed, key, step_key, rng_index, kPositronBremsAngle));
                            cone_direction(dx, dy, dz, ct,
                                           rng_uniform(seed, key, step_key, rng_index, kPositronBremsAzimuth), gx, gy, gz);
                            photon_recoil(kb, eg, gx, gy, gz, dx, dy, dz);
                            k = after;
                            current_process = 4;  // Bremsstrahlung
                            if (tracked) {
                                add_secondary(2, ex, ey, ez, gx, gy, gz, eg, birth);
                            } else if (eg > 0.0) {
                                deposit_local(er, ez, weight, eg);
                            }
                        } else {
                            // in-flight annihilation (:700-727): the parent is consumed
                            annihilate(ex, ey, ez, er, weight, k, false, rng_index, birth);
                            push_segment(0, {r_particle, z_particle, er, ez, weight, 0.0, 0.0}, 4u, 0u);
                            annihilated = true;
                            return false;
                        }
                        return true;
                    });
            },
            [&] { return stopped || annihilated; },
            // finish_interleaved_substep (:478-499)
            [&](uint64_t sub, double, double) {
                if (k >= cutoff) {
                    double const mfp = tables.ElasticMeanFreePath(1, k, 1.0);
                    double const gs_n = frozen_rate(mfp > 0.0 ? 1.0 / mfp : 0.0) * density_path(iv, path, sb, se);
                    if (gs_n > 0.0) {
                        auto gkey = [&](uint64_t ch, uint64_t inner) {
                            return rng_uniform(seed, key, step_key, (sub << 8) | inner, ch);
                        };
                        auto deflect = [&](double ct, double uphi) {
                            double nx, ny, nz;
                            cone_direction(dx, dy, dz, ct, uphi, nx, ny, nz);
                            dx = nx; dy = ny; dz = nz;
                        };
                        double const few = ts.index().gs_few_collision_threshold;
                        if (gs_n < few) {
                            int const cap = static_cast<int>(std::ceil(3.0 * few));
                            if (cap >= 255) fail(RREA_GPU_ERR_INVALID_STATE, "GS few-collision cap too large");
                            int const cnt = poisson_capped(gs_n, gkey(kPositronGsFewCount, 0), cap);
                            for (int q = 0; q < cnt; ++q) {
                                double const ct = tables.SampleSingleElasticCosTheta(
                                    1, k, gkey(kPositronGsFewScatter, static_cast<uint64_t>(q + 1)));
                                deflect(ct, gkey(kPositronGsFewAzimuth, static_cast<uint64_t>(q + 1)));
                            }
                        } else {
                            double const ct = tables.SampleGsCosTheta(1, k, gs_n, gkey(kPositronGsAngle, 0));
                            deflect(ct, gkey(kPositronGsAzimuth, 0));
                        }
                    }
                }
                half_kick(sub_field, 0.5 * sub_dt_eff, 1.0, k, dx, dy, dz);
                if (k < cutoff) {
                    mark_stopped(se);
                    return true;
                }
                return false;
            },
            [&](double e) { return advance_running(path, e, rlo, rhi, zlo, zhi, run_x, run_y, run_z); },
            [&] { return path.exits; });
        out.events[sp] = events;
        if (exited) {
            escape = clipped_escape_policy(path, std::hypot(path.ex, path.ey), path.ez);
        }
        if (annihilated) {
            tile.id[ip] = -tile.id[ip];
            out.disposition[sp] = 2;
            continue;
        }
        // RreaResolveChargedTransportTerminal (O/RreaParticleInteraction.H:292-312)
        int disp;
        if (exited) disp = 1;
        else if (stopped) disp = 2;
        else disp = k < cutoff ? 2 : 0;
        if (disp == 1) { commit_escape(); continue; }
        if (disp == 2) {
            double const ax = stopped ? stop_x : run_x;
            double const ay = stopped ? stop_y : run_y;
            double const az = stopped ? stop_z : run_z;
            double const ar = stopped ? stop_r : std::hypot(run_x, run_y);
            annihilate(ax, ay, az, ar, weight, k, true, subcycles, stopped ? stop_elapsed : 1.0);
            push_segment(0, {r_particle, z_particle, ar, az, weight, 0.0, 0.0}, 4u, 0u);
            tile.id[ip] = -tile.id[ip];
            out.disposition[sp] = 2;
            continue;
        }
        // CommitSurvivorChargedWriteback (O/RreaTransportStep.H:874-905)
        double const end_r = std::hypot(run_x, run_y);
        double const um = proper_velocity_from_kinetic(k);
        tile.ux[ip] = um * dx;
        tile.uy[ip] = um * dy;
        tile.uz[ip] = um * dz;
        tile.r[ip] = end_r;
        tile.theta[ip] = std::atan2(run_y, run_x);
        tile.z[ip] = run_z;
        push_segment(0, {r_particle, z_particle, end_r, run_z, weight, 0.0, 0.0}, 0u, 0u);
        out.disposition[sp] = 0;
      }
      } catch (OracleError const& e) {
        chunk_err[static_cast<std::size_t>(chunk)] = e.code;
        chunk_msg[static_cast<std::size_t>(chunk)] = e.what();
      }
    }
    for (int64_t chunk = 0; chunk < n_chunks; ++chunk) {
        if (chunk_err[static_cast<std::size_t>(chunk)] != 0) {
            fail(chunk_err[static_cast<std::size_t>(chunk)], chunk_msg[static_cast<std::size_t>(chunk)]);
        }
    }
    for (auto& c : chunk_out) {
        out.secondaries.insert(out.secondaries.end(), c.secondaries.begin(), c.secondaries.end());
        out.sources.insert(out.sources.end(), c.sources.begin(), c.sources.end());
        out.segments.insert(out.segments.end(), c.segments.begin(), c.segments.end());
        out.crossings.insert(out.crossings.end(), c.crossings.begin(), c.crossings.end());
    }
}

// ======================================================================
// Newborn FIFO: O/RreaSecondaryCommit.cpp:9-638 and
// O/RreaNewbornAdvance.cpp:20-996
// ======================================================================
namespace {

// Everything one newborn advance produces besides its own survival.
struct NewbornEffects {
    std::vector<Secondary> children;  // root and lineage are assigned at the FIFO merge
    std::vector<Source> sources;
    std::vector<Segment> segments;
    std::vector<PlaneCrossing> crossings;
};

struct NewbornContext {
    Tables const& tables;
    TableSet const& ts;
    rrea_gpu_config const& cfg;
    Gather const& gather;
    int step;
    double dt_s;
};

// RreaNewbornResidualFraction / RreaNewbornElapsedStepFraction (O/RreaParticleInteraction.H:171-197)
double newborn_residual(double birth) { return std::min(1.0, std::max(0.0, 1.0 - birth)); }
double newborn_elapsed(double birth, double residual, uint64_t completed, uint64_t substeps, double f)
{
    double const within = std::min(1.0, std::max(0.0, f));
    double const consumed = (static_cast<double>(completed) + within) / static_cast<double>(substeps);
    return std::min(1.0, birth + residual * consumed);
}

// TransportStep::NewbornFinalPoint (O/RreaNewbornAdvance.cpp:20-48)
bool newborn_final_point(Path const& path, double fraction, rrea_gpu_config const& cfg, double& x, double& y,
                         double& z)
{
    double const span = fraction - path.in_begin;
    double pullback = 1.0e-9;
    for (int attempt = 0; attempt < 5; ++attempt) {
        double const trial =
            attempt == 0 ? fraction : std::max(path.in_begin, fraction - pullback * std::max(span, 1.0e-12));
        path.PointAtFull(trial, x, y, z);
        if (cartesian_half_open(x, y, path.WrapZ(z), cfg.r_lo, cfg.r_hi, cfg.z_lo, cfg.z_hi)) {
            z = path.WrapZ(z);
            return true;
        }
        if (attempt > 0) pullback *= 100.0;
    }
    return false;
}

// RreaEvaluateElectronStatePolicy with electron_ensemble_mean_drag_ev_per_m
// (O/RreaParticleInteraction.H:1279-1317, O/RreaTransportStep.H:226-247)
bool electron_demotes_at(NewbornContext const& c, double x, double y, double z, double e)
{
    double const cut = c.cfg.low_energy_cutoff_eV;
    double const thr = c.ts.index().hard_moller_threshold_eV;
    double fer, fez, fbt;
    c.gather.at(std::hypot(x, y), z, fer, fez, fbt);
    double const rho = positive_or(DensityRatioAtZ(c.cfg.density_ratio, z), 1.0);
    double const ke = std::max(e, cut);
    double drag = 0.0;
    if (ke > 0.0 && rho > 0.0) {
        double const hard = c.cfg.debug_disable_hard_moller == 0 ? c.tables.ElectronHardMollerEnergyLoss(ke, rho) : 0.0;
        drag = (c.tables.ElectronCollisionLoss(ke, rho) + c.tables.ElectronSoftRadiativeDrag(ke, rho)) + hard
            + c.tables.ElectronTrackedBremsEnergyLoss(ke, rho);
    }
    bool const below = e < cut;
    bool const nonrunaway = thr > 0.0 && e <= thr && std::hypot(fer, fez) <= drag;
    return below || nonrunaway;
}

uint64_t pack_newborn(Secondary const& p, uint64_t segment, uint64_t ordinal, uint64_t inner)
{
    uint64_t v = 0;
    if (!try_pack_transient(true, static_cast<uint64_t>(p.root_species), p.lineage, segment, ordinal, inner, v)) {
        fail(RREA_GPU_ERR_RNG_OVERFLOW, "newborn RNG index overflow");
    }
    return v;
}

// TransportStep::AdvanceChargedNewborn (O/RreaNewbornAdvance.cpp:50-777)
bool advance_charged_newborn(NewbornContext const& c, Secondary& p, NewbornEffects& fx)
{
    Tables const& tables = c.tables;
    rrea_gpu_config const& cfg = c.cfg;
    bool const pos = p.species == 1;
    double const q = pos ? 1.0 : -1.0;
    int const sp = pos ? 1 : 0;
    double const rlo = cfg.r_lo, rhi = cfg.r_hi, zlo = cfg.z_lo, zhi = cfg.z_hi;
    bool const periodic = cfg.periodic_z != 0;
    double const cut = cfg.low_energy_cutoff_eV;
    double const photon_cut = cfg.photon_cutoff_eV;
    double const thr = c.ts.index().hard_moller_threshold_eV;
    bool const hm_enabled = cfg.debug_disable_hard_moller == 0;
    double const rho = StepDensityRatio(cfg);
    double const w_air = c.ts.index().w_air_eV_per_pair;
    uint64_t const seed = cfg.rng_seed, key = p.root_key;
    uint64_t const step_key = static_cast<uint64_t>(std::max(c.step, 0));
    double const w = p.w;
    double const birth_r = std::hypot(p.x, p.y), birth_z = p.z;
    double const residual = newborn_residual(p.birth);
    double k = p.energy;
    int current_process = 0;
    if (!cartesian_half_open(p.x, p.y, p.z, rlo, rhi, zlo, zhi)) {
        fail(RREA_GPU_ERR_GEOMETRY, "charged transient born outside the half-open domain");
    }
    double dx = p.dx, dy = p.dy, dz = p.dz;
    normalize(dx, dy, dz);
    auto add_child = [&](int species, double x, double y, double z, double sx, double sy, double sz, double e,
                         double birth) {
        Secondary ch{};
        ch.species = species;
        ch.process = current_process;
        ch.x = x; ch.y = y; ch.z = z;
        ch.dx = sx; ch.dy = sy; ch.dz = sz;
        ch.w = w;
        ch.energy = e;
        ch.birth = birth;
        fx.children.push_back(ch);
    };
    auto push_source = [&](int kind, double r, double z, double ww, double sec, double loss) {
        fx.sources.push_back(Source{kind, r, z, ww, sec, loss, -1});
    };
    auto deposit_local = [&](double r, double z, double ww, double e) {
        if (ww <= 0.0 || e <= 0.0) return;
        double const pw = ww * e / std::max(w_air, 1.0);
        if (pw <= 0.0) return;
        push_source(0, r, z, pw, 0.0, w_air);
    };
    auto push_segment = [&](double r1, double z1) {
        Segment sg{};
        sg.kind = 0;
        sg.a[0] = birth_r; sg.a[1] = birth_z; sg.a[2] = r1; sg.a[3] = z1; sg.a[4] = q * w;
        sg.channel = 8u;
        sg.parent_index = -1;
        fx.segments.push_back(sg);
    };
    auto push_escape = [&](Path const& path) {
        Crossing const cr = boundary_crossing(path);
        if (!cr.valid) fail(RREA_GPU_ERR_GEOMETRY, "charged escape has no certified absorbing-face crossing");
        Segment sg{};
        sg.kind = 1;
        sg.a[0] = birth_r; sg.a[1] = birth_z; sg.a[2] = cr.sr; sg.a[3] = cr.sz; sg.a[4] = cr.cr; sg.a[5] = cr.cz;
        sg.a[6] = q * w;
        sg.channel = 8u | 1u;
        sg.faces = cr.faces;
        sg.parent_index = -1;
        fx.segments.push_back(sg);
    };
    auto annihilate = [&](double x, double y, double z, double r, double ke, bool at_rest, uint64_t idx,
                          double birth) {
        current_process = 9;
        spawn_annihilation(
            tables, photon_cut, x, y, z, r, z, dx, dy, dz, w, ke, at_rest,
            rng_uniform(seed, key, step_key, idx, kAnnihilationPolar),
            rng_uniform(seed, key, step_key, idx, kAnnihilationAzimuth), birth,
            [&](double px, double py, double pz, double gx, double gy, double gz, double e, double b) {
                add_child(2, px, py, pz, gx, gy, gz, e, b);
            },
            deposit_local, [&](double rr, double zz, double ww) { push_source(2, rr, zz, ww, 0.0, 0.0); });
    };
    // birth state policy (:99-138): no net chord for a birth demotion
    bool const demote_at_birth = pos ? k < cut : electron_demotes_at(c, p.x, p.y, p.z, k);
    if (demote_at_birth) {
        double const rb = std::hypot(p.x, p.y);
        if (pos) {
            annihilate(p.x, p.y, p.z, rb, k, true, pack_newborn(p, 0, 0, 0), p.birth);
        } else {
            current_process = 12;
            push_source(1, rb, p.z, w, 0.0, 0.0);
            deposit_local(rb, p.z, w, k);
        }
        return false;
    }
    if (!(residual > 0.0)) return true;
    double const u = proper_velocity_from_kinetic(k);
    double const gam = std::sqrt(1.0 + u * u / (kC * kC));
    double const residual_dt = c.dt_s * residual;
    double const chord = (u / gam) * residual_dt;
    if (!(chord > 0.0)) return k >= cut;
    double const ex = p.x + chord * dx, ey = p.y + chord * dy, ez = p.z + chord * dz;
    Path const driver = ClipRz(std::hypot(p.x, p.y), std::atan2(p.y, p.x), p.z, std::hypot(ex, ey), std::atan2(ey, ex),
                               ez, rlo, rhi, zlo, zhi, periodic);
    if (!(driver.full > 0.0) || !(driver.in_length > 0.0)) {
        if (driver.exits) {
            push_escape(driver);
            return false;
        }
        return true;
    }
    std::vector<Interval> const driver_iv = build_intervals(driver, rho, rho);
    if (driver_iv.empty()) fail(RREA_GPU_ERR_INVALID_STATE, "charged transient path has no material intervals");
    auto require_certified = [&]() {
        if (!std::isfinite(k) || !(k >= c.ts.index().charged_min_eV && k <= c.ts.index().charged_max_eV)) {
            fail(RREA_GPU_ERR_RANGE, "newborn charged energy left the certified range");
        }
    };
    double const driver_dpath = density_path(driver_iv, driver, driver.in_begin, driver.in_end);
    double const gs_total = frozen_rate([&] {
        double const mfp = tables.ElasticMeanFreePath(sp, k, 1.0);
        return mfp > 0.0 ? 1.0 / mfp : 0.0;
    }()) * driver_dpath;
    double drag_est;
    if (pos) {
        drag_est = tables.PositronCollisionLoss(k, 1.0) * driver_dpath;
    } else {
        drag_est = (k > 0.0 ? tables.ElectronCollisionLoss(k, 1.0) + tables.ElectronSoftRadiativeDrag(k, 1.0) : 0.0)
            * driver_dpath;
    }
    double const work = path_field_work(c.gather, driver, q, 0.0, 1.0).work;
    double const impulse = std::max(cfg.max_field_impulse_fraction * k, std::max(cfg.field_impulse_floor_eV, 1.0));
    double const span = std::max(driver.in_end, 1.0e-6);
    uint64_t const substeps = std::min<uint64_t>(
        std::max(driver_count(std::min(gs_total / span, cfg.gs_total_collision_cap),
                              std::max(cfg.max_gs_collisions_per_substep, 1.0)),
                 driver_count((std::abs(work) + drag_est) / span, impulse)),
        cfg.max_subcycles);
    if (substeps >= kSegmentCap) fail(RREA_GPU_ERR_RNG_OVERFLOW, "newborn substep count outside the RNG budget");

    auto competing = [&](double e) {
        std::array<double, 3> st{};
        if (pos) {
            if (!(thr > 0.0 && e <= thr)) {
                double const mfp = tables.PositronHardBhabhaMeanFreePath(e, 1.0);
                st[0] = frozen_rate(mfp > 0.0 ? 1.0 / mfp : 0.0);
            }
            if (e > photon_cut) {
                double const mfp = tables.PositronBremsstrahlungMeanFreePath(e, 1.0);
                st[1] = frozen_rate(mfp > 0.0 ? 1.0 / mfp : 0.0);
            }
            double const mfp = tables.PositronAnnihilationMeanFreePath(e, 1.0);
            st[2] = frozen_rate(mfp > 0.0 ? 1.0 / mfp : 0.0);
        } else {
            if (hm_enabled && thr > 0.0 && e > 2.0 * thr) {
                double const mfp = tables.ElectronHardMollerMeanFreePath(e, 1.0);
                st[0] = frozen_rate(mfp > 0.0 ? 1.0 / mfp : 0.0);
            }
            if (std::isfinite(e) && std::isfinite(photon_cut) && e > photon_cut) {
                double const mfp = tables.ElectronBremsstrahlungMeanFreePath(e, 1.0);
                st[1] = frozen_rate(mfp > 0.0 ? 1.0 / mfp : 0.0);
            }
        }
        return st;
    };
    auto channel_open = [&](int ch, double e) {
        if (pos) {
            double bi, ri, ai;
            tables.PositronGateRates(e, bi, ri, ai);
            if (ch == 0) return !(thr > 0.0 && e <= thr) && bi > 0.0;
            if (ch == 1) return e > photon_cut && ri > 0.0;
            if (ch == 2) return ai > 0.0;
            return false;
        }
        double mi, bi;
        tables.ElectronGateRates(e, mi, bi);
        if (ch == 0) return hm_enabled && (thr > 0.0 && e > 2.0 * thr) && mi > 0.0;
        if (ch == 1) return (std::isfinite(e) && std::isfinite(photon_cut) && e > photon_cut) && bi > 0.0;
        return false;
    };

    double run_x = p.x, run_y = p.y, run_z = p.z;
    double const sub_dt = residual_dt / static_cast<double>(substeps);
    double final_fraction = 0.0;
    bool terminal_interaction = false, terminal_at_point = false, exited = false;
    uint64_t completed = 0;
    Path path = driver;
    std::vector<Interval> iv = driver_iv;
    FieldRange sub_field;
    double sub_dt_eff = 0.0;
    auto elapsed_at = [&](double f) { return newborn_elapsed(p.birth, residual, completed, substeps, f); };
    // apply_newborn_drag (:260-360): the live drag module; an ion-pair source
    // that rounds off the half-open domain falls back to the birth position
    auto continuous = [&](double b, double e, double stop_e) -> Limit {
        auto dp = [&](double bb, double ee) { return density_path(iv, path, bb, ee); };
        double sc = 0, ss = 0;
        bool const need = (e > b) && (k > 0.0) && !(stop_e < cut);
        if (need) {
            sc = frozen_rate(pos ? tables.PositronCollisionLoss(stop_e, 1.0) : tables.ElectronCollisionLoss(stop_e, 1.0));
            ss = frozen_rate(pos ? tables.PositronSoftRadiativeDrag(stop_e, 1.0)
                                 : tables.ElectronSoftRadiativeDrag(stop_e, 1.0));
        }
        DragPlan const plan = plan_drag(b, e, k, stop_e, cut, dp, sc, ss, 0.0);
        if (!plan.limit_valid) fail(RREA_GPU_ERR_INVALID_STATE, "newborn stopping has no monotone cutoff point");
        if (!plan.applied) return Limit{b, false, true};
        if (plan.collision > 0.0 && plan.raw_collision > 0.0) {
            for (Interval const& i : iv) {
                double const bb = std::max(b, i.begin), ee = std::min(plan.end, i.end);
                if (!(ee > bb)) continue;
                double const raw = path.full * (ee - bb) * i.density * plan.collision_stp;
                double const loss = plan.collision * raw / plan.raw_collision;
                double const pw = w * loss / std::max(w_air, 1.0);
                if (!(pw > 0.0)) continue;
                double x, y, z;
                path.PointAtFull(0.5 * (bb + ee), x, y, z);
                double sr = std::hypot(x, y), sz = path.WrapZ(z);
                if (!(std::isfinite(sr) && std::isfinite(sz) && sr >= rlo && sr < rhi && sz >= zlo && sz < zhi)) {
                    sr = std::hypot(p.x, p.y);
                    sz = p.z;
                }
                push_source(0, sr, sz, pw, pos ? 0.0 : 0.5 * cut, w_air);
            }
        }
        if (!pos) {
            defer_plane_crossings(tables, cfg, c.gather, path, iv, b, plan.end, w, k, stop_e, plan.drag, hm_enabled,
                                  fx.crossings);
        }
        k = std::max(0.0, k - plan.drag);
        if (plan.reaches) k = cut;
        return Limit{plan.end, plan.reaches, true};
    };
    auto build_chord = [&](Path& out) -> bool {
        // RreaBuildRunningChargedChord with the residual dt as the step bound
        if (!std::isfinite(sub_dt) || !std::isfinite(residual_dt) || !(sub_dt >= 0.0) || !(residual_dt > 0.0)) {
            return false;
        }
        double const speed = charged_speed(k);
        double const dn = std::sqrt(dx * dx + dy * dy + dz * dz);
        if (!std::isfinite(speed) || !std::isfinite(dn) || !(dn > 0.0)) return false;
        double const sc = speed * sub_dt / dn;
        double const exx = run_x + sc * dx, eyy = run_y + sc * dy, ezz = run_z + sc * dz;
        out = ClipRz(std::hypot(run_x, run_y), std::atan2(run_y, run_x), run_z, std::hypot(exx, eyy),
                     std::atan2(eyy, exx), ezz, rlo, rhi, zlo, zhi, periodic);
        return std::isfinite(out.full) && out.in_begin == 0.0;
    };

    // RreaRunChargedSubstepInterleave (O/RreaChargedInterleave.H:693-732), as
    // the reference's newborn advance runs it (O/RreaNewbornAdvance.cpp:440-640)
    double sb = 0.0, se = 0.0;
    RunChargedSubstepInterleave(
        substeps, k, cut, completed, exited,
        [&](uint64_t, double& b, double& e) {
            Path np;
            if (!build_chord(np)) return false;
            path = np;
            if (!(path.full > 0.0) || !(path.in_length > 0.0)) {
                exited = path.exits;
                final_fraction = 0.0;
                return false;
            }
            iv = build_intervals(path, rho, rho);
            if (iv.empty()) fail(RREA_GPU_ERR_INVALID_STATE, "transient microchord has no material intervals");
            sb = path.in_begin;
            se = path.in_end;
            b = sb;
            e = se;
            final_fraction = se;
            sub_field = path_field_work(c.gather, path, q, sb, se);
            sub_dt_eff = sub_dt * (se - sb);
            half_kick(sub_field, 0.5 * sub_dt_eff, q, k, dx, dy, dz);
            if (k < cut) {
                final_fraction = sb;
                terminal_at_point = true;
                return false;
            }
            require_certified();
            return true;
        },
        [&](uint64_t sub, double b, double e) {
            double ex2 = 0, ey2 = 0, ez2 = 0, er2 = 0, ev_elapsed = 1.0;
            uint64_t idx = 0;
            std::array<double, 3> st{};
            RunChargedEventInterleave(
                b, e, k, cut, pos ? 3 : 2, kEventCap, pos ? "newborn positron" : "newborn electron",
                [&](double frozen, double rb, double re) {
                    st = competing(frozen);
                    double const seg_dp = density_path(iv, path, rb, re);
                    return std::array<double, 3>{st[0] * seg_dp, st[1] * seg_dp, st[2] * seg_dp};
                },
                [&](uint64_t ordinal) {
                    idx = pack_newborn(p, sub, ordinal, 0);
                    double const u1 = rng_uniform(seed, key, step_key, idx, kNewbornCompetingOpticalDepth);
                    double const u2 = rng_uniform(seed, key, step_key, idx, kNewbornCompetingChannel);
                    return std::pair<double, double>{u1, u2};
                },
                [&](double tau, double rb, double re) {
                    return fraction_at_density_path(iv, path, rb, re, tau / (st[0] + st[1] + st[2]));
                },
                [&](double rb, double re, double frozen) {
                    Limit const l = continuous(rb, re, frozen);
                    return SegmentLimit{l.reaches, l.end};
                },
                [&](double f) {
                    final_fraction = f;
                    terminal_at_point = true;
                },
                [&](double f) {
                    path.PointAtFull(f, ex2, ey2, ez2);
                    er2 = std::hypot(ex2, ey2);
                    ez2 = path.WrapZ(ez2);
                    ev_elapsed = elapsed_at(f);
                },
                [&](int ch, double en) { return channel_open(ch, en); },
                [&](int channel, double ev) {
                        auto R = [&](uint64_t ch) { return rng_uniform(seed, key, step_key, idx, ch); };
                        if (channel == 0 && !pos) {
                            double const kb = k;
                            double sec = tables.SampleMollerSecondaryEnergy(kb, R(kHardMollerEnergy));
                            sec = std::max(thr, std::min(sec, 0.5 * kb));
                            double pdx = dx, pdy = dy, pdz = dz, sdx = dx, sdy = dy, sdz = dz;
                            moller_lab_directions(dx, dy, dz, kb, sec, R(kHardMollerAzimuth), pdx, pdy, pdz, sdx, sdy, sdz);
                            k = std::max(0.0, kb - sec);
                            dx = pdx; dy = pdy; dz = pdz;
                            current_process = 2;
                            add_child(0, ex2, ey2, ez2, sdx, sdy, sdz, sec, ev_elapsed);
                            push_source(0, er2, ez2, w, sec, sec);
                        } else if (channel == 0) {
                            double const kb = k;
                            double const sec =
                                std::min(tables.SamplePositronBhabhaSecondaryEnergy(kb, R(kPositronBhabhaEnergy)),
                                         std::max(0.0, kb));
                            if (sec > 0.0 && !(thr > 0.0 && sec < thr)) {
                                double pdx = dx, pdy = dy, pdz = dz, sdx = dx, sdy = dy, sdz = dz;
                                moller_lab_directions(dx, dy, dz, kb, sec, R(kPositronBhabhaAzimuth), pdx, pdy, pdz, sdx,
                                                      sdy, sdz);
                                k = std::max(0.0, kb - sec);
                                dx = pdx; dy = pdy; dz = pdz;
                                current_process = 3;
                                add_child(0, ex2, ey2, ez2, sdx, sdy, sdz, sec, ev_elapsed);
                                push_source(2, er2, ez2, w, 0.0, sec);
                            }
                        } else if (channel == 1) {
                            double const kb = k;
                            double const sampled = pos
                                ? tables.SamplePositronBremsstrahlungPhotonEnergy(kb, R(kPositronBremsEnergy))
                                : tables.SampleBremsstrahlungPhotonEnergy(kb, R(kBremsEnergy));
                            double const eg = std::min(std::max(sampled, 0.0), std::max(kb, 0.0));
                            double const after = std::max(0.0, std::max(kb, 0.0) - eg);
                            bool const tracked = std::isfinite(photon_cut) && photon_cut >= 0.0 && eg >= photon_cut;
                            double gx = dx, gy = dy, gz = dz;
                            double const ct = tables.SampleBremsstrahlungCosTheta(kb, R(pos ? kPositronBremsAngle : kBremsAngle));
                            cone_direction(dx, dy, dz, ct, R(pos ? kPositronBremsAzimuth : kBremsAzimuth), gx, gy, gz);
                            photon_recoil(kb, eg, gx, gy, gz, dx, dy, dz);
                            k = after;
                            current_process = 4;
                            if (tracked) add_child(2, ex2, ey2, ez2, gx, gy, gz, eg, ev_elapsed);
                            else if (eg > 0.0) deposit_local(er2, ez2, w, eg);
                    } else {
                        annihilate(ex2, ey2, ez2, er2, k, false, idx, ev_elapsed);
                        push_segment(er2, ez2);
                        terminal_interaction = true;
                        final_fraction = ev;
                        return false;
                    }
                    return true;
                });
        },
        [&] { return terminal_interaction || terminal_at_point; },
        [&](uint64_t sub, double, double) {
                if (k >= cut) {
                    double const mfp = tables.ElasticMeanFreePath(sp, k, 1.0);
                    double const gs_n = frozen_rate(mfp > 0.0 ? 1.0 / mfp : 0.0) * density_path(iv, path, sb, se);
                    if (gs_n > 0.0) {
                        auto gkey = [&](uint64_t ch, uint64_t inner) {
                            return rng_uniform(seed, key, step_key, pack_newborn(p, sub, 0, inner), ch);
                        };
                        auto deflect = [&](double ct, double uphi) {
                            double nx, ny, nz;
                            cone_direction(dx, dy, dz, ct, uphi, nx, ny, nz);
                            dx = nx; dy = ny; dz = nz;
                        };
                        double const few = c.ts.index().gs_few_collision_threshold;
                        if (gs_n < few) {
                            int const cap = static_cast<int>(std::ceil(3.0 * few));
                            if (cap >= 255) fail(RREA_GPU_ERR_INVALID_STATE, "GS few-collision cap too large");
                            int const cnt =
                                poisson_capped(gs_n, gkey(pos ? kNewbornPositronGsFewCount : kNewbornElectronGsFewCount, 0),
                                               cap);
                            for (int qq = 0; qq < cnt; ++qq) {
                                uint64_t const inner = static_cast<uint64_t>(qq + 1);
                                double const ct = tables.SampleSingleElasticCosTheta(
                                    sp, k, gkey(pos ? kNewbornPositronGsFewScatter : kNewbornElectronGsFewScatter, inner));
                                deflect(ct, gkey(pos ? kNewbornPositronGsFewAzimuth : kNewbornElectronGsFewAzimuth, inner));
                            }
                        } else {
                            double const ct = tables.SampleGsCosTheta(
                                sp, k, gs_n, gkey(pos ? kNewbornPositronGsAngle : kNewbornElectronGsAngle, 0));
                            deflect(ct, gkey(pos ? kNewbornPositronGsAzimuth : kNewbornElectronGsAzimuth, 0));
                        }
                    }
                }
            half_kick(sub_field, 0.5 * sub_dt_eff, q, k, dx, dy, dz);
            if (k < cut) {
                final_fraction = se;
                terminal_at_point = true;
                return true;
            }
            require_certified();
            return false;
        },
        [&](double e) { return advance_running(path, e, rlo, rhi, zlo, zhi, run_x, run_y, run_z); },
        [&] { return path.exits; });
    if (terminal_interaction) return false;
    double fx_, fy_, fz_;
    if (!newborn_final_point(path, final_fraction, cfg, fx_, fy_, fz_)) {
        fail(RREA_GPU_ERR_GEOMETRY, "newborn charged transport could not place its final point");
    }
    double const final_r = std::hypot(fx_, fy_);
    double const final_elapsed = elapsed_at(final_fraction);
    bool const demote = pos ? k < cut : electron_demotes_at(c, fx_, fy_, fz_, k);
    if (terminal_at_point || demote) {
        if (pos) {
            annihilate(fx_, fy_, fz_, final_r, k, true, pack_newborn(p, std::min<uint64_t>(substeps, kSegmentCap - 1), 0, 0),
                       final_elapsed);
        } else {
            current_process = 12;
            push_source(1, final_r, fz_, w, 0.0, 0.0);
            deposit_local(final_r, fz_, w, k);
        }
        push_segment(final_r, fz_);
        return false;
    }
    if (exited) {
        push_escape(path);
        return false;
    }
    p.x = fx_; p.y = fy_; p.z = fz_;
    p.dx = dx; p.dy = dy; p.dz = dz;
    p.energy = k;
    p.birth = 1.0;
    push_segment(final_r, fz_);
    return true;
}

// TransportStep::AdvancePhotonNewborn (O/RreaNewbornAdvance.cpp:779-996)
bool advance_photon_newborn(NewbornContext const& c, Secondary& p, NewbornEffects& fx)
{
    Tables const& tables = c.tables;
    rrea_gpu_config const& cfg = c.cfg;
    double const rlo = cfg.r_lo, rhi = cfg.r_hi, zlo = cfg.z_lo, zhi = cfg.z_hi;
    bool const periodic = cfg.periodic_z != 0;
    double const cut = cfg.low_energy_cutoff_eV;
    double const photon_cut = cfg.photon_cutoff_eV;
    double const rho = StepDensityRatio(cfg);
    double const w_air = c.ts.index().w_air_eV_per_pair;
    uint64_t const seed = cfg.rng_seed, key = p.root_key;
    uint64_t const step_key = static_cast<uint64_t>(std::max(c.step, 0));
    double const w = p.w;
    int current_process = 0;
    double const residual = newborn_residual(p.birth);
    if (!(residual > 0.0)) return p.energy >= photon_cut;
    if (!cartesian_half_open(p.x, p.y, p.z, rlo, rhi, zlo, zhi)) {
        fail(RREA_GPU_ERR_GEOMETRY, "photon transient born outside the half-open domain");
    }
    double dx = p.dx, dy = p.dy, dz = p.dz;
    normalize(dx, dy, dz);
    double energy = p.energy;
    auto add_child = [&](int species, double x, double y, double z, double sx, double sy, double sz, double e,
                         double birth) {
        Secondary ch{};
        ch.species = species;
        ch.process = current_process;
        ch.x = x; ch.y = y; ch.z = z;
        ch.dx = sx; ch.dy = sy; ch.dz = sz;
        ch.w = w;
        ch.energy = e;
        ch.birth = birth;
        fx.children.push_back(ch);
    };
    auto push_source = [&](int kind, double r, double z, double ww, double sec, double loss) {
        fx.sources.push_back(Source{kind, r, z, ww, sec, loss, -1});
    };
    auto deposit_local = [&](double r, double z, double ww, double e) {
        if (ww <= 0.0 || e <= 0.0) return;
        double const pw = ww * e / std::max(w_air, 1.0);
        if (pw <= 0.0) return;
        push_source(0, r, z, pw, 0.0, w_air);
    };
    if (energy < photon_cut) {
        current_process = 12;
        deposit_local(std::hypot(p.x, p.y), p.z, w, energy);
        return false;
    }
    double const chord = kC * c.dt_s * residual;
    double const ex = p.x + chord * dx, ey = p.y + chord * dy, ez = p.z + chord * dz;
    Path path = ClipRz(std::hypot(p.x, p.y), std::atan2(p.y, p.x), p.z, std::hypot(ex, ey), std::atan2(ey, ex), ez, rlo,
                       rhi, zlo, zhi, periodic);
    if (!(path.full > 0.0) || !(path.in_length > 0.0)) return !path.exits;
    double elapsed_start = p.birth;
    uint64_t ordinal = 0;
    for (;;) {
        uint64_t const idx = pack_newborn(p, 0, ordinal, 0);
        std::vector<Interval> const iv = build_intervals(path, rho, rho);
        PhotonRates const rates = photon_rates(tables, energy, 1.0);
        double const mfp = Tables::mfp_from_inverse(rates.total());
        double const tau = density_path(iv, path, path.in_begin, path.in_end) / mfp;
        auto R = [&](uint64_t ch) { return rng_uniform(seed, key, step_key, idx, ch); };
        Selection const sel = select_hazard({tau, 0.0, 0.0}, 1, R(kNewbornCompetingOpticalDepth), 0.0);
        if (!sel.valid) fail(RREA_GPU_ERR_INVALID_STATE, "newborn photon hazard selection invalid");
        if (!sel.event) {
            double fx_, fy_, fz_;
            if (!newborn_final_point(path, path.in_end, cfg, fx_, fy_, fz_)) {
                fail(RREA_GPU_ERR_GEOMETRY, "newborn photon could not place its final point");
            }
            if (path.exits) return false;
            p.x = fx_; p.y = fy_; p.z = fz_;
            p.dx = dx; p.dy = dy; p.dz = dz;
            p.energy = energy;
            p.birth = 1.0;
            return true;
        }
        double const f = fraction_at_density_path(iv, path, path.in_begin, path.in_end, sel.sampled * mfp);
        if (!(std::isfinite(f) && f >= path.in_begin && f <= path.in_end && path.in_end > path.in_begin)) {
            fail(RREA_GPU_ERR_INVALID_STATE, "newborn photon event depth outside its chord");
        }
        double const dist = path.full * (f - path.in_begin);
        double const remaining = std::max(0.0, path.full - dist);
        double px, py, pz;
        path.PointAtFull(f, px, py, pz);
        double const pr = std::hypot(px, py);
        pz = path.WrapZ(pz);
        double const birth =
            std::min(1.0, elapsed_start + dist / std::max(kC * c.dt_s, std::numeric_limits<double>::min()));
        int const channel = sample_photon_channel(tables, energy, R(kNewbornCompetingChannel));
        if (channel == 0) {
            current_process = 5;
            double const inc = energy;
            ComptonState const cs = sample_klein_nishina(tables, inc, R(53), R(54));
            double sx, sy, sz;
            cone_direction(dx, dy, dz, cs.cos_theta, R(58), sx, sy, sz);
            double rx = inc * dx - cs.scattered * sx, ry = inc * dy - cs.scattered * sy, rz = inc * dz - cs.scattered * sz;
            normalize(rx, ry, rz);
            if (cs.recoil >= cut) {
                add_child(0, px, py, pz, rx, ry, rz, cs.recoil, birth);
                push_source(0, pr, pz, w, cs.recoil, cs.recoil);
            } else {
                push_source(0, pr, pz, w, cs.recoil, 0.0);
                deposit_local(pr, pz, w, cs.recoil);
            }
            if (!PhotonFlowValid(0, w, inc, cs.recoil, cs.scattered, 0.0, false, 0.0)) {
                fail(RREA_GPU_ERR_INVALID_STATE, "newborn Compton photon energy flow does not close");
            }
            energy = cs.scattered;
            if (energy < photon_cut) {
                deposit_local(pr, pz, w, energy);
                return false;
            }
            dx = sx; dy = sy; dz = sz;
            if (!(remaining > 0.0)) {
                p.x = px; p.y = py; p.z = pz;
                p.dx = dx; p.dy = dy; p.dz = dz;
                p.energy = energy;
                p.birth = 1.0;
                return true;
            }
            double const tx = px + remaining * dx, ty = py + remaining * dy, tz = pz + remaining * dz;
            path = ClipRz(pr, std::atan2(py, px), pz, std::hypot(tx, ty), std::atan2(ty, tx), tz, rlo, rhi, zlo, zhi,
                          periodic);
            elapsed_start = birth;
            ++ordinal;
            continue;
        }
        if (channel == 1) {
            current_process = 6;
            double pe_e, bind;
            sample_photoelectric(tables, energy, R(55), pe_e, bind);
            double const ee = std::min(pe_e, energy);
            if (ee >= cut) {
                double sx, sy, sz;
                cone_direction(dx, dy, dz, sample_photoelectron_cos(tables, ee, R(60)), R(65), sx, sy, sz);
                add_child(0, px, py, pz, sx, sy, sz, ee, birth);
                push_source(0, pr, pz, w, ee, ee);
            } else {
                push_source(0, pr, pz, w, ee, 0.0);
                deposit_local(pr, pz, w, ee);
            }
            if (bind > 0.0) deposit_local(pr, pz, w, bind);
            if (!PhotonFlowValid(1, w, energy, ee, std::max(bind, 0.0), 0.0, false, 0.0)) {
                fail(RREA_GPU_ERR_INVALID_STATE, "newborn photoelectric photon energy flow does not close");
            }
            return false;
        }
        bool const triplet = channel == 3;
        current_process = triplet ? 8 : 7;
        PairState const ps = sample_pair(tables, energy, channel, R(66), R(57), R(59));
        if (!ps.valid) fail(RREA_GPU_ERR_INVALID_STATE, "pair channel without phase space");
        double edx, edy, edz, pdx, pdy, pdz;
        rotate_to_axis(dx, dy, dz, ps.edir[0], ps.edir[1], ps.edir[2], edx, edy, edz);
        rotate_to_axis(dx, dy, dz, ps.pdir[0], ps.pdir[1], ps.pdir[2], pdx, pdy, pdz);
        if (ps.e_electron >= cut) {
            add_child(0, px, py, pz, edx, edy, edz, ps.e_electron, birth);
        } else {
            push_source(1, pr, pz, w, 0.0, 0.0);
            deposit_local(pr, pz, w, ps.e_electron);
        }
        if (ps.e_positron >= cut) {
            add_child(1, px, py, pz, pdx, pdy, pdz, ps.e_positron, birth);
        } else {
            spawn_annihilation(
                tables, photon_cut, px, py, pz, pr, pz, pdx, pdy, pdz, w, ps.e_positron, true, R(80), R(81), birth,
                [&](double qx, double qy, double qz, double gx, double gy, double gz, double e, double b) {
                    add_child(2, qx, qy, qz, gx, gy, gz, e, b);
                },
                deposit_local, [&](double rr, double zz, double ww) { push_source(2, rr, zz, ww, 0.0, 0.0); });
        }
        if (ps.recoil) {
            double rdx, rdy, rdz;
            rotate_to_axis(dx, dy, dz, ps.rdir[0], ps.rdir[1], ps.rdir[2], rdx, rdy, rdz);
            if (ps.e_recoil >= cut) add_child(0, px, py, pz, rdx, rdy, rdz, ps.e_recoil, birth);
            push_source(0, pr, pz, w, ps.e_recoil, 0.0);
            if (ps.e_recoil < cut) deposit_local(pr, pz, w, ps.e_recoil);
        }
        if (ps.local > 0.0) deposit_local(pr, pz, w, ps.local);
        if (!PhotonFlowValid(2, w, energy, ps.e_electron, ps.e_positron, ps.e_recoil, ps.recoil, ps.local)) {
            fail(RREA_GPU_ERR_INVALID_STATE, "newborn pair photon energy flow does not close");
        }
        return false;
    }
}

}  // namespace

void DrainSecondaries(TableSet const& ts, rrea_gpu_config const& cfg, FieldGrid const& field, int step, double dt_s,
                      std::vector<Secondary> const& initial, std::vector<Secondary>& survivors, StepOutputs& out)
{
    Tables const tables(ts);
    Gather const gather{field, cfg};
    NewbornContext const c{tables, ts, cfg, gather, step, dt_s};
    // birth payloads entering the FIFO (O/RreaSecondaryCommit.cpp:337-373)
    for (Secondary const& s : initial) {
        bool const known = s.species >= 0 && s.species <= 2 && s.root_species >= 0 && s.root_species <= 2;
        bool const finite = std::isfinite(s.x) && std::isfinite(s.y) && std::isfinite(s.z) && std::isfinite(s.dx)
            && std::isfinite(s.dy) && std::isfinite(s.dz) && std::isfinite(s.w) && std::isfinite(s.energy)
            && std::isfinite(s.birth);
        bool const energy_ok = s.species == 2 ? s.energy > 0.0 : s.energy >= 0.0;
        if (!known || !finite || !(s.w > 0.0) || !energy_ok || s.birth < 0.0 || s.birth > 1.0
            || s.lineage >= kLineageCap) {
            fail(RREA_GPU_ERR_ARGUMENT, "transient FIFO received an invalid birth payload");
        }
    }
    std::vector<Secondary> work(initial.begin(), initial.end());
    std::map<std::pair<uint64_t, int>, uint64_t> next_lineage;
    for (Secondary const& s : work) {
        uint64_t& nx = next_lineage[{s.root_key, s.root_species}];
        nx = std::max(nx, s.lineage + 1U);
    }
    survivors.clear();
    constexpr std::size_t kBatch = 1024;
    for (std::size_t cursor = 0; cursor < work.size();) {
        std::size_t const count = std::min(kBatch, work.size() - cursor);
        std::vector<NewbornEffects> fx(count);
        std::vector<char> alive(count, 1);
        std::vector<int> err(count, 0);
        std::vector<std::string> msg(count);
#pragma omp parallel for schedule(dynamic, 1) if (count > 1)
        for (long o = 0; o < static_cast<long>(count); ++o) {
            std::size_t const i = static_cast<std::size_t>(o);
            try {
                Secondary& s = work[cursor + i];
                double const e = s.energy;
                bool const certified = s.species == 2
                    ? (std::isfinite(e) && e >= ts.index().photon_min_eV && e <= ts.index().photon_max_eV)
                    : (std::isfinite(e) && e >= ts.index().charged_min_eV && e <= ts.index().charged_max_eV);
                if (!certified) fail(RREA_GPU_ERR_RANGE, "transient FIFO particle outside its certified energy range");
                if (s.birth < 1.0) {
                    alive[i] = s.species == 2 ? advance_photon_newborn(c, s, fx[i]) : advance_charged_newborn(c, s, fx[i]);
                }
            } catch (OracleError const& e) {
                err[i] = e.code;
                msg[i] = e.what();
            }
        }
        for (std::size_t i = 0; i < count; ++i) {
            if (err[i] != 0) fail(err[i], msg[i]);
        }
        for (std::size_t i = 0; i < count; ++i) {
            Secondary const parent = work[cursor + i];
            for (Secondary ch : fx[i].children) {
                ch.root_key = parent.root_key;
                ch.root_species = parent.root_species;
                ch.parent_index = parent.parent_index;
                uint64_t& nx = next_lineage[{ch.root_key, ch.root_species}];
                if (nx >= kLineageCap) fail(RREA_GPU_ERR_RNG_OVERFLOW, "transient FIFO lineage overflow");
                ch.lineage = nx++;
                work.push_back(ch);
            }
            out.sources.insert(out.sources.end(), fx[i].sources.begin(), fx[i].sources.end());
            out.crossings.insert(out.crossings.end(), fx[i].crossings.begin(), fx[i].crossings.end());
            out.segments.insert(out.segments.end(), fx[i].segments.begin(), fx[i].segments.end());
            if (alive[i]) {
                Secondary s = work[cursor + i];
                s.birth = 1.0;
                survivors.push_back(s);
            }
        }
        cursor += count;
    }
    // final survivors at their transported endpoint (O/RreaSecondaryCommit.cpp:480-515)
    for (Secondary const& s : survivors) {
        bool const finite = std::isfinite(s.x) && std::isfinite(s.y) && std::isfinite(s.z) && std::isfinite(s.dx)
            && std::isfinite(s.dy) && std::isfinite(s.dz) && std::isfinite(s.w) && std::isfinite(s.energy);
        bool const photon = s.species == 2;
        bool const energy_ok = photon ? s.energy > 0.0 : s.energy >= cfg.low_energy_cutoff_eV;
        bool const certified = photon
            ? (s.energy >= ts.index().photon_min_eV && s.energy <= ts.index().photon_max_eV)
            : (s.energy >= ts.index().charged_min_eV && s.energy <= ts.index().charged_max_eV);
        if (!finite || !(s.w > 0.0) || !energy_ok || !certified
            || !cartesian_half_open(s.x, s.y, s.z, cfg.r_lo, cfg.r_hi, cfg.z_lo, cfg.z_hi)) {
            fail(RREA_GPU_ERR_INVALID_STATE, "transient work graph contains invalid final survivors");
        }
    }
}

// ======================================================================
// Photon phase: O/RreaPhotonTransport.cpp:9-461 with the final states of
// O/RreaPhotonFinalStates.H:56-365 and TransportStep::spawn_positron_annihilation
// (O/RreaTransportStep.H:563-702).  The photon tile's current (r, theta, z)
// is WarpX's straight push endpoint; prev_* is the captured start.
// ======================================================================
void ApplyPhotonTransport(TableSet const& ts, rrea_gpu_config const& cfg, int step, double dt_s, ChargedTile& tile,
                          StepOutputs& out)
{
    Tables const tables(ts);
    double const rlo = cfg.r_lo, rhi = cfg.r_hi, zlo = cfg.z_lo, zhi = cfg.z_hi;
    bool const periodic = cfg.periodic_z != 0;
    double const cutoff = cfg.low_energy_cutoff_eV;
    double const photon_cut = cfg.photon_cutoff_eV;
    double const density_ratio = StepDensityRatio(cfg);
    uint64_t const seed = cfg.rng_seed;
    uint64_t const step_key = static_cast<uint64_t>(std::max(step, 0));
    double const w_air = ts.index().w_air_eV_per_pair;

    out.subcycles.assign(static_cast<std::size_t>(tile.n), 0);
    out.events.assign(static_cast<std::size_t>(tile.n), 0);
    out.disposition.assign(static_cast<std::size_t>(tile.n), -1);
    std::vector<uint64_t>& out_events = out.events;
    std::vector<int32_t>& out_disposition = out.disposition;

    constexpr int64_t kChunk = 64;
    int64_t const n_chunks = (tile.n + kChunk - 1) / kChunk;
    std::vector<StepOutputs> chunk_out(static_cast<std::size_t>(n_chunks));
    std::vector<int> chunk_err(static_cast<std::size_t>(n_chunks), 0);
    std::vector<std::string> chunk_msg(static_cast<std::size_t>(n_chunks));
#pragma omp parallel for schedule(dynamic, 1) if (n_chunks > 1)
    for (int64_t chunk = 0; chunk < n_chunks; ++chunk) {
      StepOutputs& cout = chunk_out[static_cast<std::size_t>(chunk)];
      try {
      int64_t const ip_end = std::min(tile.n, (chunk + 1) * kChunk);
      for (int64_t ip = chunk * kChunk; ip < ip_end; ++ip) {
        if (!(tile.id[ip] > 0)) continue;
        std::size_t const sp = static_cast<std::size_t>(ip);
        uint64_t const key = static_cast<uint64_t>(std::llabs(tile.id[ip]))
            ^ (static_cast<uint64_t>(tile.cpu ? tile.cpu[ip] : 0) << 40);
        uint64_t lineage = 0;
        int current_process = 0;
        double const weight = tile.w[ip];
        double energy = std::sqrt(tile.ux[ip] * tile.ux[ip] + tile.uy[ip] * tile.uy[ip] + tile.uz[ip] * tile.uz[ip]);
        double dx = tile.ux[ip], dy = tile.uy[ip], dz = tile.uz[ip];
        normalize(dx, dy, dz);
        if (tile.prev_r[ip] > rhi + 1.0e-9 * rhi || tile.prev_z[ip] < zlo - 1.0e-9
            || tile.prev_z[ip] > zhi + 1.0e-9 * zhi) {
            fail(RREA_GPU_ERR_GEOMETRY, "RREA photon survived outside the domain");
        }
        Path path = ClipRz(tile.prev_r[ip], tile.prev_theta[ip], tile.prev_z[ip], tile.r[ip], tile.theta[ip],
                           tile.z[ip], rlo, rhi, zlo, zhi, periodic);
        uint64_t ordinal = 0;
        double elapsed_start = 0.0;
        auto push_source = [&](int kind, double r, double z, double w, double sec, double loss) {
            cout.sources.push_back(Source{kind, r, z, w, sec, loss, ip});
        };
        auto deposit_local_at = [&](double r, double z, double w, double e) {
            if (w <= 0.0 || e <= 0.0) return;
            double const pw = w * e / std::max(w_air, 1.0);
            if (pw <= 0.0) return;
            push_source(0, r, z, pw, 0.0, w_air);
        };
        auto add_secondary = [&](int species, double x, double y, double z, double sx, double sy, double sz, double e,
                                 double birth) {
            Secondary s2;
            s2.species = species;
            s2.process = current_process;
            s2.x = x; s2.y = y; s2.z = z;
            s2.dx = sx; s2.dy = sy; s2.dz = sz;
            s2.w = weight;
            s2.energy = e;
            s2.birth = birth;
            s2.root_key = key;
            s2.lineage = lineage++;
            s2.root_species = 2;
            s2.parent_index = ip;
            cout.secondaries.push_back(s2);
        };
        int disp = 0;
        for (;;) {
            if (ordinal >= kEventCap) fail(RREA_GPU_ERR_RNG_OVERFLOW, "photon event ordinal overflow");
            EscapePolicy const esc = clipped_escape_policy(path, std::hypot(path.ex, path.ey), path.ez);
            double const ds = path.in_length;
            std::vector<Interval> const iv = build_intervals(path, density_ratio, density_ratio);
            double const chord_dpath = density_path(iv, path, path.in_begin, path.in_end);
            if (weight <= 0.0 || energy < photon_cut) {
                double x, y, z;
                path.PointAtFull(path.in_begin, x, y, z);
                current_process = 12;
                deposit_local_at(std::hypot(x, y), z, std::max(weight, 0.0), energy);
                tile.id[ip] = -tile.id[ip];
                disp = 2;
                break;
            }
            auto commit_no_event = [&]() {
                double x, y, z;
                path.PointAtFull(path.in_end, x, y, z);
                tile.r[ip] = std::hypot(x, y);
                tile.theta[ip] = std::atan2(y, x);
                tile.z[ip] = path.WrapZ(z);
                if (!esc.escapes) return 0;
                if (esc.invalidate) tile.id[ip] = -tile.id[ip];
                return 1;
            };
            if (ds <= 0.0) {
                disp = commit_no_event();
                break;
            }
            PhotonRates const rates = photon_rates(tables, energy, 1.0);
            double const mfp = Tables::mfp_from_inverse(rates.total());
            double const tau = chord_dpath / mfp;
            uint64_t idx;
            if (!try_live_hazard_index(2, 0, ordinal, idx)) fail(RREA_GPU_ERR_RNG_OVERFLOW, "photon RNG index");
            out_events[sp] += 1;
            double const u_int = rng_uniform(seed, key, step_key, idx, ordinal == 0 ? 51 : 128);
            Selection const sel = select_hazard({tau, 0.0, 0.0}, 1, u_int, 0.0);
            if (!sel.valid || !sel.event) {
                if (!sel.valid) fail(RREA_GPU_ERR_INVALID_STATE, "photon hazard selection invalid");
                disp = commit_no_event();
                break;
            }
            double const f = fraction_at_density_path(iv, path, path.in_begin, path.in_end, sel.sampled * mfp);
            if (!(std::isfinite(f) && f >= path.in_begin && f <= path.in_end && path.in_end > path.in_begin)) {
                fail(RREA_GPU_ERR_INVALID_STATE, "photon event depth outside its chord");
            }
            double const dist = path.full * (f - path.in_begin);
            double px, py, pz;
            path.PointAtFull(f, px, py, pz);
            double const remaining = std::max(0.0, path.full - dist);
            double const birth =
                std::min(1.0, elapsed_start + dist / std::max(kC * dt_s, std::numeric_limits<double>::min()));
            double const pr = std::hypot(px, py);
            int const channel = sample_photon_channel(
                tables, energy, rng_uniform(seed, key, step_key, idx, ordinal == 0 ? 52 : 129));
            auto R = [&](uint64_t ch) { return rng_uniform(seed, key, step_key, idx, ch); };
            bool repeat = false;
            Path next;
            if (channel == 0) {
                // RreaApplyComptonFinalState, O/RreaPhotonFinalStates.H:56-147
                current_process = 5;
                double const inc = energy;
                ComptonState const cs = sample_klein_nishina(tables, inc, R(53), R(54));
                double sx, sy, sz;
                cone_direction(dx, dy, dz, cs.cos_theta, R(58), sx, sy, sz);
                double rx = inc * dx - cs.scattered * sx, ry = inc * dy - cs.scattered * sy,
                       rz = inc * dz - cs.scattered * sz;
                normalize(rx, ry, rz);
                if (cs.recoil >= cutoff) {
                    add_secondary(0, px, py, pz, rx, ry, rz, cs.recoil, birth);
                    push_source(0, pr, pz, weight, cs.recoil, cs.recoil);
                } else {
                    push_source(0, pr, pz, weight, cs.recoil, 0.0);
                    deposit_local_at(pr, pz, weight, cs.recoil);
                }
                if (!PhotonFlowValid(0, weight, inc, cs.recoil, cs.scattered, 0.0, false, 0.0)) {
                    fail(RREA_GPU_ERR_INVALID_STATE, "Compton photon energy flow does not close");
                }
                energy = cs.scattered;
                if (energy < photon_cut) {
                    deposit_local_at(pr, pz, weight, energy);
                    tile.id[ip] = -tile.id[ip];
                    disp = 2;
                } else {
                    dx = sx; dy = sy; dz = sz;
                    tile.ux[ip] = energy * dx;
                    tile.uy[ip] = energy * dy;
                    tile.uz[ip] = energy * dz;
                    double const xt = px + dx * remaining, yt = py + dy * remaining, zt = pz + dz * remaining;
                    next = ClipRz(pr, std::atan2(py, px), pz, std::hypot(xt, yt), std::atan2(yt, xt), zt, rlo, rhi, zlo,
                                  zhi, periodic);
                    double nx, ny, nz;
                    next.PointAtFull(next.in_end, nx, ny, nz);
                    tile.r[ip] = std::hypot(nx, ny);
                    tile.theta[ip] = std::atan2(ny, nx);
                    tile.z[ip] = next.WrapZ(nz);
                    repeat = remaining > 0.0;
                    disp = 0;
                }
            } else if (channel == 1) {
                // RreaApplyPhotoelectricFinalState, O/RreaPhotonFinalStates.H:160-224
                current_process = 6;
                double pe_e, bind;
                sample_photoelectric(tables, energy, R(55), pe_e, bind);
                double const ee = std::min(pe_e, energy);
                if (ee >= cutoff) {
                    double ex, ey, ez;
                    cone_direction(dx, dy, dz, sample_photoelectron_cos(tables, ee, R(60)), R(65), ex, ey, ez);
                    add_secondary(0, px, py, pz, ex, ey, ez, ee, birth);
                    push_source(0, pr, pz, weight, ee, ee);
                } else {
                    push_source(0, pr, pz, weight, ee, 0.0);
                    deposit_local_at(pr, pz, weight, ee);
                }
                if (bind > 0.0) deposit_local_at(pr, pz, weight, bind);
                if (!PhotonFlowValid(1, weight, energy, ee, std::max(bind, 0.0), 0.0, false, 0.0)) {
                    fail(RREA_GPU_ERR_INVALID_STATE, "photoelectric photon energy flow does not close");
                }
                tile.id[ip] = -tile.id[ip];
                disp = 2;
            } else {
                // RreaApplyPairFinalState, O/RreaPhotonFinalStates.H:239-365
                bool const triplet = channel == 3;
                current_process = triplet ? 8 : 7;
                PairState const ps = sample_pair(tables, energy, channel, R(66), R(57), R(59));
                if (!ps.valid) fail(RREA_GPU_ERR_INVALID_STATE, "pair channel without phase space");
                double edx, edy, edz, pdx, pdy, pdz;
                rotate_to_axis(dx, dy, dz, ps.edir[0], ps.edir[1], ps.edir[2], edx, edy, edz);
                rotate_to_axis(dx, dy, dz, ps.pdir[0], ps.pdir[1], ps.pdir[2], pdx, pdy, pdz);
                if (ps.e_electron >= cutoff) {
                    add_secondary(0, px, py, pz, edx, edy, edz, ps.e_electron, birth);
                } else {
                    push_source(1, pr, pz, weight, 0.0, 0.0);
                    deposit_local_at(pr, pz, weight, ps.e_electron);
                }
                if (ps.e_positron >= cutoff) {
                    add_secondary(1, px, py, pz, pdx, pdy, pdz, ps.e_positron, birth);
                } else {
                    // spawn_positron_annihilation at rest, O/RreaTransportStep.H:563-702
                    double ax = pdx, ay = pdy, az = pdz;
                    normalize(ax, ay, az);
                    AnnihilationState const an = sample_annihilation(tables, 0.0, R(80), R(81));
                    double g1x, g1y, g1z;
                    cone_direction(ax, ay, az, an.cos1, an.azim, g1x, g1y, g1z);
                    double const e1 = std::max(an.e1, 0.0), e2 = std::max(an.e2, 0.0);
                    double g2x = -g1x, g2y = -g1y, g2z = -g1z;
                    double local = 0.0;
                    // the annihilation photons join the pair's transaction group
                    if (e1 >= photon_cut) add_secondary(2, px, py, pz, g1x, g1y, g1z, e1, birth);
                    else local += e1;
                    if (e2 >= photon_cut) add_secondary(2, px, py, pz, g2x, g2y, g2z, e2, birth);
                    else local += e2;
                    if (ps.e_positron > 0.0) deposit_local_at(pr, pz, weight, ps.e_positron);
                    if (local > 0.0) deposit_local_at(pr, pz, weight, local);
                    push_source(2, pr, pz, weight, 0.0, 0.0);
                }
                if (ps.recoil) {
                    double rdx, rdy, rdz;
                    rotate_to_axis(dx, dy, dz, ps.rdir[0], ps.rdir[1], ps.rdir[2], rdx, rdy, rdz);
                    if (ps.e_recoil >= cutoff) add_secondary(0, px, py, pz, rdx, rdy, rdz, ps.e_recoil, birth);
                    push_source(0, pr, pz, weight, ps.e_recoil, 0.0);
                    if (ps.e_recoil < cutoff) deposit_local_at(pr, pz, weight, ps.e_recoil);
                }
                if (ps.local > 0.0) deposit_local_at(pr, pz, weight, ps.local);
                if (!PhotonFlowValid(2, weight, energy, ps.e_electron, ps.e_positron, ps.e_recoil, ps.recoil, ps.local)) {
                    fail(RREA_GPU_ERR_INVALID_STATE, "pair photon energy flow does not close");
                }
                tile.id[ip] = -tile.id[ip];
                disp = 2;
            }
            if (repeat) {
                path = next;
                elapsed_start = birth;
                ++ordinal;
                continue;
            }
            break;
        }
        out_disposition[sp] = disp;
      }
      } catch (OracleError const& e) {
        chunk_err[static_cast<std::size_t>(chunk)] = e.code;
        chunk_msg[static_cast<std::size_t>(chunk)] = e.what();
      }
    }
    for (int64_t chunk = 0; chunk < n_chunks; ++chunk) {
        if (chunk_err[static_cast<std::size_t>(chunk)] != 0) {
            fail(chunk_err[static_cast<std::size_t>(chunk)], chunk_msg[static_cast<std::size_t>(chunk)]);
        }
    }
    for (auto& c : chunk_out) {
        out.secondaries.insert(out.secondaries.end(), c.secondaries.begin(), c.secondaries.end());
        out.sources.insert(out.sources.end(), c.sources.begin(), c.sources.end());
    }
}

// Primitive-level entry points, one row of inputs per call, matching the
// golden fixtures written by oracle/ref_golden.cpp.
int RunPrimitive(TableSet const& ts, int which, double const* in, int64_t n, double* out)
{
    Tables const t(ts);
    for (int64_t i = 0; i < n; ++i) {
        switch (which) {
        case 1: {  // (table, e) -> value
            double const* a = in + 2 * i;
            out[i] = t.interpolate(static_cast<int>(a[0]), a[1]);
            break;
        }
        case 2: {  // (e, dr) -> 10 accessors
            double const* a = in + 2 * i;
            double* o = out + 10 * i;
            double const e = a[0], dr = a[1];
            o[0] = t.ElectronCollisionLoss(e, dr);
            o[1] = t.ElectronSoftRadiativeDrag(e, dr);
            o[2] = t.ElectronHardMollerMeanFreePath(e, dr);
            o[3] = t.ElectronBremsstrahlungMeanFreePath(e, dr);
            o[4] = t.ElectronHardMollerEnergyLoss(e, dr);
            o[5] = t.ElectronTrackedBremsEnergyLoss(e, dr);
            o[6] = t.ElasticMeanFreePath(0, e, dr);
            o[7] = t.ScreeningEta(0, e);
            o[8] = t.ElasticMeanFreePath(1, e, dr);
            o[9] = t.ScreeningEta(1, e);
            break;
        }
        case 3: {
            double const* a = in + 4 * i;
            out[i] = t.SampleGsCosTheta(static_cast<int>(a[0]), a[1], a[2], a[3]);
            break;
        }
        case 4: {
            double const* a = in + 3 * i;
            out[i] = t.SampleSingleElasticCosTheta(static_cast<int>(a[0]), a[1], a[2]);
            break;
        }
        case 5: out[i] = t.SampleMollerSecondaryEnergy(in[2 * i], in[2 * i + 1]); break;
        case 6: out[i] = t.SampleBremsstrahlungPhotonEnergy(in[2 * i], in[2 * i + 1]); break;
        case 7: out[i] = t.SampleBremsstrahlungCosTheta(in[2 * i], in[2 * i + 1]); break;
        case 8: {
            double const* a = in + 13 * i;
            FieldRange f;
            f.work = a[0]; f.ex = a[1]; f.ey = a[2]; f.ez = a[3]; f.bx = a[4]; f.by = a[5]; f.bz = a[6];
            double k = a[9], dx = a[10], dy = a[11], dz = a[12];
            half_kick(f, a[7], a[8], k, dx, dy, dz);
            double* o = out + 4 * i;
            o[0] = k; o[1] = dx; o[2] = dy; o[3] = dz;
            break;
        }
        case 9: {
            double const* a = in + 5 * i;
            double* o = out + 3 * i;
            cone_direction(a[0], a[1], a[2], a[3], a[4], o[0], o[1], o[2]);
            break;
        }
        case 10: {
            double const* a = in + 6 * i;
            double* o = out + 6 * i;
            moller_lab_directions(a[0], a[1], a[2], a[3], a[4], a[5], o[0], o[1], o[2], o[3], o[4], o[5]);
            break;
        }
        case 11: {
            double const* a = in + 8 * i;
            double* o = out + 3 * i;
            o[0] = a[5]; o[1] = a[6]; o[2] = a[7];
            photon_recoil(a[0], a[1], a[2], a[3], a[4], o[0], o[1], o[2]);
            break;
        }
        case 12: out[i] = poisson_capped(in[2 * i], in[2 * i + 1], 30); break;
        case 13: {
            double const* a = in + 6 * i;
            std::array<double, 3> taus = {a[0], a[1], a[2]};
            Selection const s = select_hazard(taus, static_cast<int>(a[3]), a[4], a[5]);
            double* o = out + 5 * i;
            o[0] = s.valid; o[1] = s.event; o[2] = s.channel; o[3] = s.sampled; o[4] = s.total;
            break;
        }
        case 14: {
            double const* a = in + 10 * i;
            double const len = a[8], rho = a[9];
            DragPlan const p = plan_drag(a[0], a[1], a[2], a[3], a[4],
                                         [&](double bb, double ee) { return len * (ee - bb) * rho; }, a[5], a[6],
                                         a[7]);
            double* o = out + 9 * i;
            o[0] = p.end; o[1] = p.applied; o[2] = p.limit_valid; o[3] = p.reaches; o[4] = p.drag;
            o[5] = p.collision; o[6] = p.soft; o[7] = p.hard; o[8] = p.raw_collision;
            break;
        }
        case 15: {
            double const* a = in + 9 * i;
            double* o = out + 17 * i;
            double const x = a[0], y = a[1], z = a[2], dx = a[3], dy = a[4], dz = a[5], k = a[6], dt = a[7];
            bool const periodic = a[8] != 0.0;
            // RreaBuildRunningChargedChord, O/RreaParticleInteraction.H:110-161
            bool valid = false;
            Path p;
            double const speed = charged_speed(k);
            double const dn = std::sqrt(dx * dx + dy * dy + dz * dz);
            if (std::isfinite(speed) && std::isfinite(dn) && dn > 0.0) {
                double const sc = speed * dt / dn;
                double const ex = x + sc * dx, ey = y + sc * dy, ez = z + sc * dz;
                p = ClipRz(std::hypot(x, y), std::atan2(y, x), z, std::hypot(ex, ey), std::atan2(ey, ex), ez, 0.0,
                           50.0, 0.0, 500.0, periodic);
                valid = std::isfinite(p.full) && p.in_begin == 0.0;
            }
            double const np = static_cast<double>(p.pieces.size());
            o[0] = valid; o[1] = p.sx; o[2] = p.sy; o[3] = p.sz; o[4] = p.ex; o[5] = p.ey; o[6] = p.ez;
            o[7] = p.full; o[8] = p.in_end; o[9] = p.in_length; o[10] = p.exits; o[11] = np;
            o[12] = np > 0 ? p.pieces[0].begin : -1.0;
            o[13] = np > 0 ? p.pieces[0].end : -1.0;
            o[14] = np > 0 ? p.pieces[0].shift : 0.0;
            o[15] = np > 0 ? p.pieces.back().begin : -1.0;
            o[16] = np > 0 ? p.pieces.back().shift : 0.0;
            break;
        }
        case 16: out[i] = sample_photon_channel(t, in[2 * i], in[2 * i + 1]); break;
        case 17: {  // (e, draw_mu, draw_accept) -> recoil, scattered, cos
            double const* a = in + 3 * i;
            ComptonState const c = sample_klein_nishina(t, a[0], a[1], a[2]);
            out[3 * i] = c.recoil; out[3 * i + 1] = c.scattered; out[3 * i + 2] = c.cos_theta;
            break;
        }
        case 18: {  // (e, u) -> electron, binding
            sample_photoelectric(t, in[2 * i], in[2 * i + 1], out[2 * i], out[2 * i + 1]);
            break;
        }
        case 19: out[i] = sample_photoelectron_cos(t, in[2 * i], in[2 * i + 1]); break;
        case 20: {  // (e, channel, inv, polar, azim) -> valid, ee, ep, er, local, 9 dirs
            double const* a = in + 5 * i;
            PairState const p = sample_pair(t, a[0], static_cast<int>(a[1]), a[2], a[3], a[4]);
            double* o = out + 14 * i;
            o[0] = p.valid; o[1] = p.e_electron; o[2] = p.e_positron; o[3] = p.e_recoil; o[4] = p.local;
            for (int c = 0; c < 3; ++c) { o[5 + c] = p.edir[c]; o[8 + c] = p.pdir[c]; o[11 + c] = p.rdir[c]; }
            break;
        }
        case 21: {  // (k, d_energy, d_azim) -> e1, e2, cos1, azim, valid, at_rest
            double const* a = in + 3 * i;
            AnnihilationState const an = sample_annihilation(t, a[0], a[1], a[2]);
            double* o = out + 6 * i;
            o[0] = an.e1; o[1] = an.e2; o[2] = an.cos1; o[3] = an.azim; o[4] = an.valid; o[5] = an.at_rest;
            break;
        }
        case 22: {  // (e, dr) -> positron collision, soft, Bhabha MFP, brems MFP, annihilation MFP
            double const e = in[2 * i], dr = in[2 * i + 1];
            double* o = out + 5 * i;
            o[0] = t.PositronCollisionLoss(e, dr);
            o[1] = t.PositronSoftRadiativeDrag(e, dr);
            o[2] = t.PositronHardBhabhaMeanFreePath(e, dr);
            o[3] = t.PositronBremsstrahlungMeanFreePath(e, dr);
            o[4] = t.PositronAnnihilationMeanFreePath(e, dr);
            break;
        }
        case 23: out[i] = t.SamplePositronBhabhaSecondaryEnergy(in[2 * i], in[2 * i + 1]); break;
        case 24: out[i] = t.SamplePositronBremsstrahlungPhotonEnergy(in[2 * i], in[2 * i + 1]); break;
        default:
            fail(RREA_GPU_ERR_ARGUMENT, "unknown primitive");
        }
    }
    return 0;
}

// ======================================================================
// Net-chord current: I/RreaSegmentDepositionRZ.H:64-458 and the coupling's
// padded grid (O/RreaWarpXCoupling.cpp:417-544)
// ======================================================================
void NetChordGrid::Reset(rrea_gpu_config const& cfg)
{
    int constexpr pad = 2;
    phys_nr = cfg.nr;
    phys_nz = cfg.nz;
    phys_z_begin = pad;
    nr = cfg.nr + pad;
    nz = cfg.nz + 2 * pad;
    dr = (cfg.r_hi - cfg.r_lo) / cfg.nr;
    dz = (cfg.z_hi - cfg.z_lo) / cfg.nz;
    r_lo = cfg.r_lo;
    z_lo = cfg.z_lo - pad * dz;
    rho.assign(static_cast<std::size_t>(nr) * nz, 0.0);
    jr.assign(static_cast<std::size_t>(nr + 1) * nz, 0.0);
    jz.assign(static_cast<std::size_t>(nr) * (nz + 1), 0.0);
}

namespace {

// :67-90
void cic_charge(NetChordGrid& g, double q, double r, double z)
{
    double const xr = (r - g.r_lo) / g.dr - 0.5;
    double const xz = (z - g.z_lo) / g.dz - 0.5;
    int const i0 = static_cast<int>(std::floor(xr));
    int const j0 = static_cast<int>(std::floor(xz));
    double const fr = xr - i0, fz = xz - j0;
    double const wr[2] = {1.0 - fr, fr};
    double const wz[2] = {1.0 - fz, fz};
    for (int a = 0; a < 2; ++a) {
        for (int b = 0; b < 2; ++b) {
            int i = i0 + a, j = j0 + b;
            if (i < 0) i = -1 - i;
            if (i >= g.nr) i = g.nr - 1;
            if (j < 0) j = 0;
            if (j >= g.nz) j = g.nz - 1;
            g.rho[static_cast<std::size_t>(i) + static_cast<std::size_t>(g.nr) * j] += q * wr[a] * wz[b];
        }
    }
}

// :96-150: index-space fluxes of one in-cell piece, midpoint transverse weights
void deposit_piece(NetChordGrid& g, double q_over_dt, double xr0, double xz0, double xr1, double xz1)
{
    double fr_flux = q_over_dt * (xr1 - xr0);
    double const fz_flux = q_over_dt * (xz1 - xz0);
    double const mr = 0.5 * (xr0 + xr1), mz = 0.5 * (xz0 + xz1);
    {
        int const jf = static_cast<int>(std::floor(mz));
        double const fz = mz - jf;
        int const fi = static_cast<int>(std::floor(mr)) + 1;
        if (fi <= 0) fr_flux = 0.0;
        for (int b = 0; b < 2; ++b) {
            int j = jf + b;
            if (j < 0) j = 0;
            if (j >= g.nz) j = g.nz - 1;
            int i = fi;
            if (i <= 0) continue;
            if (i > g.nr) i = g.nr;
            g.jr[static_cast<std::size_t>(i) + static_cast<std::size_t>(g.nr + 1) * j] +=
                fr_flux * (b == 0 ? 1.0 - fz : fz);
        }
    }
    {
        int const ifc = static_cast<int>(std::floor(mr));
        double const fr = mr - ifc;
        int const fj = static_cast<int>(std::floor(mz)) + 1;
        for (int a = 0; a < 2; ++a) {
            int i = ifc + a;
            if (i < 0) i = -1 - i;
            if (i >= g.nr) i = g.nr - 1;
            int j = fj;
            if (j < 0) j = 0;
            if (j > g.nz) j = g.nz;
            g.jz[static_cast<std::size_t>(i) + static_cast<std::size_t>(g.nr) * j] +=
                fz_flux * (a == 0 ? 1.0 - fr : fr);
        }
    }
}

// :152-189: split at CIC cell boundaries in both directions, then deposit
void deposit_segment(NetChordGrid& g, double q, double dt, double r0, double z0, double r1, double z1)
{
    double const q_over_dt = q / dt;
    double const xr0 = (r0 - g.r_lo) / g.dr - 0.5, xz0 = (z0 - g.z_lo) / g.dz - 0.5;
    double const xr1 = (r1 - g.r_lo) / g.dr - 0.5, xz1 = (z1 - g.z_lo) / g.dz - 0.5;
    std::vector<double> cuts{0.0, 1.0};
    auto add = [&cuts](double a, double b) {
        if (a == b) return;
        double const lo = std::min(a, b), hi = std::max(a, b);
        for (double k = std::ceil(lo); k <= std::floor(hi); ++k) {
            double const t = (k - a) / (b - a);
            if (t > 0.0 && t < 1.0) cuts.push_back(t);
        }
    };
    add(xr0, xr1);
    add(xz0, xz1);
    std::sort(cuts.begin(), cuts.end());
    for (std::size_t p = 0; p + 1 < cuts.size(); ++p) {
        double const s0 = cuts[p], s1 = cuts[p + 1];
        if (s1 <= s0) continue;
        deposit_piece(g, q_over_dt, xr0 + s0 * (xr1 - xr0), xz0 + s0 * (xz1 - xz0), xr0 + s1 * (xr1 - xr0),
                      xz0 + s1 * (xz1 - xz0));
    }
}

// :229-397
bool deposit_escape(NetChordGrid& g, double q, double dt, double sr0, double sz0, double fr0, double fz0, double cr,
                    double cz, uint32_t faces)
{
    uint32_t constexpr known = 1u | 2u | 4u;
    if (!(dt > 0.0) || !std::isfinite(q) || !std::isfinite(dt) || !std::isfinite(sr0) || !std::isfinite(sz0)
        || !std::isfinite(fr0) || !std::isfinite(fz0) || !std::isfinite(cr) || !std::isfinite(cz)
        || g.phys_nr <= 0 || g.phys_nr >= g.nr || g.phys_nz <= 0 || g.phys_z_begin <= 0
        || g.phys_z_begin + g.phys_nz >= g.nz || faces == 0u || (faces & ~known) != 0u
        || ((faces & 2u) && (faces & 4u))) {
        return false;
    }
    if (faces & 1u) cr = g.r_lo + g.phys_nr * g.dr;
    if (faces & 2u) cz = g.z_lo + g.phys_z_begin * g.dz;
    else if (faces & 4u) cz = g.z_lo + (g.phys_z_begin + g.phys_nz) * g.dz;
    struct Move {
        std::size_t from, to, face;
        double charge;
        bool radial;
        int orient;
    };
    std::vector<Move> moves;
    double const xr = (cr - g.r_lo) / g.dr - 0.5;
    double const xz = (cz - g.z_lo) / g.dz - 0.5;
    int const i0 = static_cast<int>(std::floor(xr));
    int const j0 = static_cast<int>(std::floor(xz));
    double const fr = xr - i0, fz = xz - j0;
    double const wr[2] = {1.0 - fr, fr};
    double const wz[2] = {1.0 - fz, fz};
    for (int a = 0; a < 2; ++a) {
        for (int b = 0; b < 2; ++b) {
            int i = i0 + a;
            int const j = j0 + b;
            if (i < 0) i = -1 - i;
            if (i < 0 || i >= g.nr || j < 0 || j >= g.nz) return false;
            bool const physical = i < g.phys_nr && j >= g.phys_z_begin && j < g.phys_z_begin + g.phys_nz;
            if (!physical) continue;
            uint32_t cand[3];
            int nc = 0;
            if ((faces & 1u) && i == g.phys_nr - 1) cand[nc++] = 1u;
            if ((faces & 2u) && j == g.phys_z_begin) cand[nc++] = 2u;
            if ((faces & 4u) && j == g.phys_z_begin + g.phys_nz - 1) cand[nc++] = 4u;
            if (nc == 0) return false;
            double const share = q * wr[a] * wz[b] / nc;
            std::size_t const from = static_cast<std::size_t>(i) + static_cast<std::size_t>(g.nr) * j;
            for (int c = 0; c < nc; ++c) {
                if (cand[c] == 1u) {
                    moves.push_back(Move{from, static_cast<std::size_t>(i + 1) + static_cast<std::size_t>(g.nr) * j,
                                         static_cast<std::size_t>(g.phys_nr) + static_cast<std::size_t>(g.nr + 1) * j,
                                         share, true, 1});
                } else {
                    int const face_j = cand[c] == 2u ? g.phys_z_begin : g.phys_z_begin + g.phys_nz;
                    int const to_j = cand[c] == 2u ? j - 1 : j + 1;
                    moves.push_back(Move{from, static_cast<std::size_t>(i) + static_cast<std::size_t>(g.nr) * to_j,
                                         static_cast<std::size_t>(i) + static_cast<std::size_t>(g.nr) * face_j, share,
                                         false, cand[c] == 2u ? -1 : 1});
                }
            }
        }
    }
    if (moves.empty()) return false;
    cic_charge(g, -q, sr0, sz0);
    cic_charge(g, q, cr, cz);
    deposit_segment(g, q, dt, sr0, sz0, fr0, fz0);
    deposit_segment(g, q, dt, fr0, fz0, cr, cz);
    for (Move const& m : moves) {
        double const flux = m.orient * m.charge / dt;
        if (m.radial) g.jr[m.face] += flux;
        else g.jz[m.face] += flux;
        g.rho[m.from] -= m.charge;
        g.rho[m.to] += m.charge;
    }
    return true;
}

}  // namespace

// O/RreaWarpXCoupling.cpp:446-544 (AccumulateChargedSegment / AccumulateChargedEscape)
void DepositNetChords(NetChordGrid& g, double dt_s, std::vector<Segment> const& segments)
{
    for (Segment const& s : segments) {
        if (s.kind == 0) {
            double const q = s.a[4];
            if (q == 0.0) continue;
            deposit_segment(g, q, dt_s, s.a[0], s.a[1], s.a[2], s.a[3]);
        } else {
            double const q = s.a[6];
            if (q == 0.0) continue;
            if (!deposit_escape(g, q, dt_s, s.a[0], s.a[1], s.a[2], s.a[3], s.a[4], s.a[5], s.faces)) {
                fail(RREA_GPU_ERR_GEOMETRY, "charged escape could not close its exact boundary CIC cloud");
            }
        }
    }
}

void ConvertNetChordCurrent(NetChordGrid const& g, std::vector<double>& jr_phys, std::vector<double>& jz_phys)
{
    double constexpr pi = 3.14159265358979323846;
    double constexpr qe = 1.602176634e-19;
    int const nr = g.phys_nr, nz = g.phys_nz, pad = g.phys_z_begin;
    jr_phys.assign(static_cast<std::size_t>(nr + 1) * nz, 0.0);
    jz_phys.assign(static_cast<std::size_t>(nr) * (nz + 1), 0.0);
    for (int j = pad; j < pad + nz; ++j) {
        for (int i = 0; i <= nr; ++i) {
            double const flux = g.jr[static_cast<std::size_t>(i) + static_cast<std::size_t>(g.nr + 1) * j];
            double const rf = i * g.dr;
            if (flux == 0.0 || rf <= 0.0) continue;
            jr_phys[static_cast<std::size_t>(i) + static_cast<std::size_t>(nr + 1) * (j - pad)] +=
                qe * flux / (2.0 * pi * rf * g.dz);
        }
    }
    for (int j = pad; j <= pad + nz; ++j) {
        for (int i = 0; i < nr; ++i) {
            double const flux = g.jz[static_cast<std::size_t>(i) + static_cast<std::size_t>(g.nr) * j];
            if (flux == 0.0) continue;
            double const rlo = i * g.dr, rhi = (i + 1) * g.dr;
            jz_phys[static_cast<std::size_t>(i) + static_cast<std::size_t>(nr) * (j - pad)] +=
                qe * flux / (pi * (rhi * rhi - rlo * rlo));
        }
    }
}

// ======================================================================
// Maxwell TM-RZ: I/RreaMaxwellTMRZ.H:147-228 composed as
// S/RreaAmrexAdvance.cpp:690-780 (no fluid)
// ======================================================================
namespace {

constexpr double kEps0 = 8.8541878128e-12;
constexpr double kMu0 = 1.25663706212e-6;

inline std::size_t er_at(MaxwellField const& f, int i, int j)
{
    return static_cast<std::size_t>(i) + static_cast<std::size_t>(f.nr + 1) * j;
}
inline std::size_t ez_at(MaxwellField const& f, int i, int j)
{
    return static_cast<std::size_t>(i) + static_cast<std::size_t>(f.nr) * j;
}

}  // namespace

// :143-154, dBtheta/dt = dEz/dr - dEr/dz at interior corners
void MaxwellAdvanceB(MaxwellField& f, double dt)
{
    for (int j = 1; j < f.nz; ++j) {
        for (int i = 1; i < f.nr; ++i) {
            f.bt[er_at(f, i, j)] += dt * ((f.ez[ez_at(f, i, j)] - f.ez[ez_at(f, i - 1, j)]) / f.dr
                                         - (f.er[er_at(f, i, j)] - f.er[er_at(f, i, j - 1)]) / f.dz);
        }
    }
}
// :156-175, first-order Silver-Mueller on the outer r and both z faces
void MaxwellSilverMueller(MaxwellField& f)
{
    for (int j = 0; j <= f.nz; ++j) f.bt[er_at(f, f.nr, j)] = -f.ez[ez_at(f, f.nr - 1, j)] / kC;
    for (int i = 1; i <= f.nr; ++i) {
        f.bt[er_at(f, i, 0)] = -f.er[er_at(f, i, 0)] / kC;
        f.bt[er_at(f, i, f.nz)] = f.er[er_at(f, i, f.nz - 1)] / kC;
    }
    for (int j = 0; j <= f.nz; ++j) f.bt[er_at(f, 0, j)] = 0.0;
}
// :177-214 with no conductivity and no ambient term
void MaxwellAdvanceE(MaxwellField& f, double dt, std::vector<double> const& jr, std::vector<double> const& jz)
{
    double const c2dt = dt / (kEps0 * kMu0);
    for (int j = 0; j < f.nz; ++j) {
        for (int i = 1; i <= f.nr; ++i) {
            std::size_t const face = er_at(f, i, j);
            double const a = 0.0 * dt / (2.0 * kEps0);
            double drive = -c2dt * (f.bt[er_at(f, i, j + 1)] - f.bt[er_at(f, i, j)]) / f.dz;
            drive -= dt / kEps0 * jr[face];
            f.er[face] = ((1.0 - a) * f.er[face] + drive) / (1.0 + a);
        }
        f.er[er_at(f, 0, j)] = 0.0;
    }
    for (int j = 0; j <= f.nz; ++j) {
        for (int i = 0; i < f.nr; ++i) {
            std::size_t const face = ez_at(f, i, j);
            double const a = 0.0 * dt / (2.0 * kEps0);
            double drive = c2dt * ((i + 1) * f.bt[er_at(f, i + 1, j)] - i * f.bt[er_at(f, i, j)]) / ((i + 0.5) * f.dr);
            drive -= dt / kEps0 * jz[face];
            f.ez[face] = ((1.0 - a) * f.ez[face] + drive) / (1.0 + a);
        }
    }
}

void AdvanceMaxwell(MaxwellField& f, double dt_s, int substeps, std::vector<double> const& jr,
                    std::vector<double> const& jz)
{
    if (!std::isfinite(dt_s) || dt_s <= 0.0 || substeps < 1) fail(RREA_GPU_ERR_ARGUMENT, "invalid field step");
    double const cfl = kC * dt_s * std::sqrt(1.0 / (f.dr * f.dr) + 1.0 / (f.dz * f.dz));
    if (!std::isfinite(cfl) || !(cfl < 1.0)) fail(RREA_GPU_ERR_ARGUMENT, "Maxwell TM violates the Yee CFL condition");
    double const dts = dt_s / static_cast<double>(substeps);
    double const restagger = 0.5 * (dt_s - dts);
    MaxwellAdvanceB(f, restagger);
    for (int k = 0; k < substeps; ++k) {
        MaxwellAdvanceB(f, dts);
        MaxwellSilverMueller(f);
        MaxwellAdvanceE(f, dts, jr, jz);
    }
    MaxwellAdvanceB(f, -restagger);
    MaxwellSilverMueller(f);
}

// O/RreaCouplingSources.cpp:435-512 + S/RreaEventAccumulator.cpp:129-164, 386-502
void DepositSources(rrea_gpu_config const& cfg, std::vector<Source> const& sources, double cutoff,
                    CellSources& cells)
{
    int const nr = cells.nr, nz = cells.nz;
    for (auto& f : cells.f) {
        if (f.size() != static_cast<std::size_t>(nr) * nz) f.assign(static_cast<std::size_t>(nr) * nz, 0.0);
    }
    double const dr = (cfg.r_hi - cfg.r_lo) / nr, dz = (cfg.z_hi - cfg.z_lo) / nz;
    bool const periodic = cfg.periodic_z != 0;
    auto add = [&](int field, double r, double z, double value) {
        if (!std::isfinite(value) || value == 0.0) return;
        double zz = z;
        if (periodic) {
            double const len = cfg.z_hi - cfg.z_lo;
            double s = std::fmod(zz - cfg.z_lo, len);
            if (s < 0.0) s += len;
            zz = cfg.z_lo + s;
        }
        int const ic = static_cast<int>(std::floor((r - cfg.r_lo) / dr));
        int const jc = static_cast<int>(std::floor((zz - cfg.z_lo) / dz));
        if (ic < 0 || ic >= nr || jc < 0 || jc >= nz) return;
        double const rc = (r - cfg.r_lo) / dr + 0.0 - 0.5;
        int const i0 = static_cast<int>(std::floor(rc));
        double const wr1 = rc - i0, wr0 = 1.0 - wr1;
        double const zc = (zz - cfg.z_lo) / dz + 0.0 - 0.5;
        int const j0 = static_cast<int>(std::floor(zc));
        double const wz1 = zc - j0, wz0 = 1.0 - wz1;
        for (int a = 0; a < 2; ++a) {
            double const wz = a == 0 ? wz0 : wz1;
            if (wz == 0.0) continue;
            int j = j0 + a;
            if (j < 0 || j > nz - 1) {
                if (periodic) { j = ((j % nz) + nz) % nz; } else { continue; }
            }
            for (int b = 0; b < 2; ++b) {
                double const wr = b == 0 ? wr0 : wr1;
                double const v = value * wr * wz;
                if (v == 0.0) continue;
                int i = i0 + b;
                if (i < 0 || i > nr - 1) {
                    if (i == -1 && cfg.r_lo == 0.0) i = 0; else continue;
                }
                if (!std::isfinite(v) || v == 0.0) continue;
                cells.f[field][static_cast<std::size_t>(i) + static_cast<std::size_t>(nr) * j] += v;
            }
        }
    };
    for (Source const& s : sources) {
        if (s.w <= 0.0) continue;
        if (s.kind == 0) {
            // AccumulateIonizationEvent
            add(1, s.r, s.z, s.w);
            if (s.secondary_energy < cutoff) add(0, s.r, s.z, s.w);
            add(3, s.r, s.z, s.w);
            add(4, s.r, s.z, std::max(s.w, 0.0) * std::max(s.energy_loss, 0.0));
        } else if (s.kind == 1) {
            // AccumulateLowEnergyElectron
            add(0, s.r, s.z, s.w);
            add(3, s.r, s.z, s.w);
            add(4, s.r, s.z, std::max(s.w, 0.0) * std::max(std::max(s.energy_loss, 0.0), 0.0));
        } else {
            // AccumulatePositiveIonSourceOnly
            add(1, s.r, s.z, s.w);
            add(3, s.r, s.z, s.w);
            add(4, s.r, s.z, std::max(s.w, 0.0) * std::max(s.energy_loss, 0.0));
        }
    }
}

}  // namespace oracle
