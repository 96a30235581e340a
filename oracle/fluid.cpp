// ORACLE — test infrastructure only.  CPU restatement of the reference's
// low-energy carrier fluid (LowEnergyFluidState: S/LowEnergyFluidState.cpp,
// S/LowEnergyFluidFaceTransport.cpp) on one RZ cell grid, plus the coupled
// fluid/Maxwell step of RreaAmrexAdvance::AdvanceOneStep
// (S/RreaAmrexAdvance.cpp:593-838).  Pinned to the reference's own fluid
// sources by the ref_fluid_* golden vectors (oracle/ref_golden_fluid.cpp).
// Never linked into the shipped library.
//
// Layouts: cells i + nr*j; radial faces i + (nr+1)*j (j < nz); axial faces
// i + nr*j (j <= nz); three carriers species-major (0 positive ion,
// 1 negative ion, 2 electron).  Every expression keeps the reference's
// operand order (this file is built without FMA contraction).
#include "oracle_core.hpp"
#include "fluid.hpp"

#include <algorithm>
#include <cmath>
#include <limits>
#include <string>
#include <vector>

namespace oracle_fluid {

namespace {

constexpr double kQe = 1.602176634e-19;      // I/RreaConstants.H:6
constexpr double kEps0 = 8.8541878128e-12;   // I/RreaConstants.H:7
constexpr double kPi = 3.141592653589793238462643383279502884;
constexpr double kNL = 2.6868e25;            // I/RreaConstants.H:16
constexpr double kVacuum = 1.0e-30;          // carrier_transport_vacuum_density_m3, I/LowEnergyFluidState.H
constexpr double kEps = std::numeric_limits<double>::epsilon();

[[noreturn]] void fail(std::string const& m) { oracle::fail(RREA_GPU_ERR_INVALID_STATE, m); }
[[noreturn]] void bad_arg(std::string const& m) { oracle::fail(RREA_GPU_ERR_ARGUMENT, m); }

// MobilityLaw::At (I/LowEnergyFluidState.H:30-41)
struct Law {
    bool reduced;
    double absolute, reduced_mobility, floor;
    double at(double chi) const { return reduced ? reduced_mobility / std::max(chi, floor) : absolute; }
};
Law ion_law(rrea_gpu_fluid_config const& c, bool positive)
{
    return Law{c.ion_mobility_model == RREA_GPU_MOBILITY_REDUCED_STP,
               positive ? c.positive_ion_mobility_m2_per_vs : c.negative_ion_mobility_m2_per_vs,
               positive ? c.positive_ion_reduced_mobility_stp_m2_per_vs
                        : c.negative_ion_reduced_mobility_stp_m2_per_vs,
               c.ion_mobility_density_ratio_floor};
}
Law electron_law(rrea_gpu_fluid_config const& c)
{
    return Law{false, c.electron_mobility_m2_per_vs, 0.0, c.ion_mobility_density_ratio_floor};
}

// checked_density_ratio (I/LowEnergyFluidState.H:49-64)
double checked_ratio(double const* chi, std::size_t k, double scalar)
{
    double const v = chi ? chi[k] : scalar;
    if (!std::isfinite(v) || v <= 0.0) return scalar > 0.0 ? scalar : 1.0;
    return v;
}

// rz_shell_volume (I/RreaConstants.H:37-44)
double shell_volume(double r_in, double r_out, double dz)
{
    double const a = r_in > 0.0 ? r_in : 0.0;
    double const b = r_out > 0.0 ? r_out : 0.0;
    return kPi * (b * b - a * a) * dz;
}

// exact_pair_loss (S/LowEnergyFluidState.cpp:41-64)
double pair_loss(double a, double b, double alpha, double dt)
{
    double const small = std::min(a, b);
    double const large = std::max(a, b);
    if (!(small > 0.0) || !(alpha > 0.0) || !(dt > 0.0)) return 0.0;
    double const delta = large - small;
    double remaining;
    if (delta <= 1.0e-12 * std::max(large, 1.0)) {
        remaining = small / (1.0 + alpha * small * dt);
    } else {
        double const ratio = (small / large) * std::exp(-alpha * delta * dt);
        remaining = ratio >= 1.0 ? small : delta * ratio / (1.0 - ratio);
    }
    return small - std::min(std::max(remaining, 0.0), small);
}

}  // namespace

// ValidateCarrierTransportConfig (S/LowEnergyFluidFaceTransport.cpp:87-163)
void validate_transport(rrea_gpu_fluid_config const& c, bool require_cfl)
{
    auto positive = [](double v) { return std::isfinite(v) && v > 0.0; };
    if (c.ion_drift_enable) {
        if (c.ion_mobility_model != RREA_GPU_MOBILITY_ABSOLUTE && c.ion_mobility_model != RREA_GPU_MOBILITY_REDUCED_STP) {
            bad_arg("enabled ion carrier has invalid mobility model");
        }
        bool const red = c.ion_mobility_model == RREA_GPU_MOBILITY_REDUCED_STP;
        if (!positive(red ? c.positive_ion_reduced_mobility_stp_m2_per_vs : c.positive_ion_mobility_m2_per_vs)
            || !positive(red ? c.negative_ion_reduced_mobility_stp_m2_per_vs : c.negative_ion_mobility_m2_per_vs)) {
            bad_arg("enabled ion carrier requires a positive finite mobility");
        }
        if (red && (!positive(c.ion_mobility_density_ratio_floor) || !positive(c.transport_density_ratio))) {
            bad_arg("density-scaled carrier mobility requires positive density ratios");
        }
    }
    if (c.electron_drift_enable) {
        if (c.electron_mobility_model != RREA_GPU_MOBILITY_ABSOLUTE
            && c.electron_mobility_model != RREA_GPU_MOBILITY_EN_TABLE_FLUX) {
            bad_arg("enabled low-energy-electron carrier has invalid mobility model");
        }
        if (c.electron_mobility_model == RREA_GPU_MOBILITY_ABSOLUTE && !positive(c.electron_mobility_m2_per_vs)) {
            bad_arg("enabled low-energy-electron carrier requires a positive finite mobility");
        }
    }
    if (!c.ion_drift_enable && !c.electron_drift_enable) return;
    if (require_cfl && (!std::isfinite(c.ion_drift_cfl) || c.ion_drift_cfl <= 0.0 || c.ion_drift_cfl > 1.0)) {
        bad_arg("rrea.ion_drift_cfl must be finite and in (0, 1]");
    }
}

// UpdateFromIonizationSource (S/LowEnergyFluidState.cpp:105-308)
double react(rrea_gpu_fluid_config const& c, std::size_t n, double dt, double* ne, double* np, double* nn,
             double* se, double* sp, double* sn, double* rho, double const* nu_cell, bool clear)
{
    if (!std::isfinite(dt) || dt < 0.0) bad_arg("LowEnergyFluidState requires non-negative dt");
    bool const table = c.attachment_model == RREA_GPU_ATTACHMENT_EN_TABLE;
    if (c.attachment_model != RREA_GPU_ATTACHMENT_CONSTANT && !table) bad_arg("unknown attachment model");
    if (table != (nu_cell != nullptr)) bad_arg("en_table_attachment_v1 requires exactly its attachment field");
    for (double a : {c.electron_ion_recombination_coefficient_m3_per_s, c.ion_ion_recombination_coefficient_m3_per_s}) {
        if (!std::isfinite(a) || a < 0.0) bad_arg("fluid recombination coefficients must be finite and non-negative");
    }
    double const nu_const = std::max(c.attachment_frequency_s, 0.0);
    double const decay_const = std::exp(-nu_const * dt);
    double const factor_const = nu_const > 0.0 ? (1.0 - decay_const) / nu_const : dt;
    double const a_ei = c.electron_ion_recombination_coefficient_m3_per_s;
    double const a_ii = c.ion_ion_recombination_coefficient_m3_per_s;
    double const det = std::max(c.detachment_frequency_s, 0.0);
    double const det_fraction = det > 0.0 ? -std::expm1(-det * dt) : 0.0;
    double worst = 0.0;
    bool nonfinite = false;
    for (std::size_t k = 0; k < n; ++k) {
        double nu = nu_const, decay = decay_const, factor = factor_const;
        if (table) {
            nu = nu_cell[k];
            double const x = nu * dt;
            decay = std::exp(-x);
            factor = nu > 0.0 ? -std::expm1(-x) / nu : dt;
        }
        double const s_low = std::max(se[k], 0.0);
        double const d_pos = std::max(sp[k], 0.0) * dt;
        double const d_neg = std::max(sn[k], 0.0) * dt;
        double const d_low = s_low * dt;
        double const e0 = std::max(ne[k], 0.0);
        double const p0 = std::max(np[k], 0.0);
        double const m0 = std::max(nn[k], 0.0);
        rho[k] += kQe * (d_pos - d_neg - d_low);
        double const expected = kQe * (p0 + d_pos - m0 - d_neg - e0 - d_low);
        double const e1 = nu > 0.0 ? e0 * decay + s_low * factor : e0 + d_low;
        double const attached = std::max(e0 + d_low - e1, 0.0);
        double e = std::max(e1, 0.0);
        double p = p0 + d_pos;
        double m = m0 + d_neg + attached;
        if (det_fraction > 0.0) {
            double const freed = m * det_fraction;
            m -= freed;
            e += freed;
        }
        double const l_ei = pair_loss(e, p, a_ei, dt);
        e = std::max(e - l_ei, 0.0);
        p = std::max(p - l_ei, 0.0);
        double const l_ii = pair_loss(p, m, a_ii, dt);
        p = std::max(p - l_ii, 0.0);
        m = std::max(m - l_ii, 0.0);
        ne[k] = e;
        np[k] = p;
        nn[k] = m;
        if (clear) se[k] = sp[k] = sn[k] = 0.0;
        double const actual = kQe * (p - m - e);
        double const scale =
            std::max(std::abs(expected) + kQe * (std::abs(p) + std::abs(m) + std::abs(e)), std::numeric_limits<double>::min());
        double const r = std::abs(actual - expected) / scale;
        if (std::isnan(r)) nonfinite = true;
        worst = std::max(worst, r);
    }
    double const residual = nonfinite ? std::numeric_limits<double>::quiet_NaN() : worst;
    if (!std::isfinite(residual) || residual > 512.0 * kEps) {
        fail("low-energy attachment/recombination violated local charge conservation");
    }
    return residual;
}

// MaxReactionFrequency (S/LowEnergyFluidState.cpp:310-343)
double max_reaction_frequency(rrea_gpu_fluid_config const& c, std::size_t n, double const* ne, double const* np,
                              double const* nn, double const* nu_cell)
{
    bool const table = c.attachment_model == RREA_GPU_ATTACHMENT_EN_TABLE;
    if (table != (nu_cell != nullptr)) bad_arg("reaction stiffness requires the selected attachment binding");
    double const nu_const = std::max(c.attachment_frequency_s, 0.0);
    double const det = std::max(c.detachment_frequency_s, 0.0);
    double const a_ei = c.electron_ion_recombination_coefficient_m3_per_s;
    double const a_ii = c.ion_ion_recombination_coefficient_m3_per_s;
    double m = 0.0;
    for (std::size_t k = 0; k < n; ++k) {
        double const att = table ? nu_cell[k] : nu_const;
        double const rate = att + det + a_ei * (std::max(ne[k], 0.0) + std::max(np[k], 0.0))
            + a_ii * (std::max(np[k], 0.0) + std::max(nn[k], 0.0));
        m = std::max(m, std::abs(rate));
    }
    return m;
}

// ComputeConductivity (S/LowEnergyFluidState.cpp:345-421)
void conductivity(rrea_gpu_fluid_config const& c, std::size_t n, double const* ne, double const* np, double const* nn,
                  double const* chi, double const* mu_cell, double* sigma, double* tau)
{
    validate_transport(c, false);
    bool const ions = c.ion_drift_enable != 0;
    bool const electrons = c.electron_drift_enable != 0;
    bool const from_field = electrons && c.electron_mobility_model == RREA_GPU_MOBILITY_EN_TABLE_FLUX;
    if (from_field != (mu_cell != nullptr)) bad_arg("en_table_flux_v1 conductivity requires exactly its mobility field");
    Law const pos = ion_law(c, true), neg = ion_law(c, false), ele = electron_law(c);
    for (std::size_t k = 0; k < n; ++k) {
        double const d = checked_ratio(chi, k, c.transport_density_ratio);
        double v = 0.0;
        if (electrons) v += (from_field ? mu_cell[k] : ele.at(d)) * std::max(ne[k], 0.0);
        if (ions) v += pos.at(d) * std::max(np[k], 0.0) + neg.at(d) * std::max(nn[k], 0.0);
        v *= kQe;
        sigma[k] = std::max(v, 0.0);
        tau[k] = sigma[k] > 0.0 ? kEps0 / sigma[k] : 1.0e300;
    }
}

// ComputeFluidChargeDensity (S/LowEnergyFluidState.cpp:423-455)
void charge_density(std::size_t n, double const* ne, double const* np, double const* nn, double* rho)
{
    for (std::size_t k = 0; k < n; ++k) {
        double const p = std::max(np[k], 0.0), m = std::max(nn[k], 0.0), e = std::max(ne[k], 0.0);
        double net = p - m - e;
        if (std::abs(net) <= 64.0 * kEps * (p + m + e)) net = 0.0;
        rho[k] = kQe * net;
    }
}

// LowEnergyElectronClosure::Evaluate (S/RreaInteractionTables.cpp:3406-3478)
Coefficients evaluate(rrea_host::ClosureTable const& t, double en, int& status)
{
    Coefficients out{};
    std::size_t const n = t.size();
    if (n == 0 || !std::isfinite(en) || en < 0.0) {
        status = rrea_host::kClosureInvalid;
        return out;
    }
    std::size_t node = n;
    if (en <= t.en_td.front()) {
        status = en < t.en_td.front() ? rrea_host::kClosureHeldBelow : rrea_host::kClosureInRange;
        node = 0;
    } else if (en >= t.en_td.back()) {
        status = en > t.en_td.back() ? rrea_host::kClosureAboveRange : rrea_host::kClosureInRange;
        node = n - 1;
    }
    if (node < n) {
        out = {t.k0[node], t.nu2[node], t.nu3[node], t.dl[node], t.dt[node]};
        return out;
    }
    status = rrea_host::kClosureInRange;
    std::size_t const hi = static_cast<std::size_t>(std::upper_bound(t.en_td.begin(), t.en_td.end(), en) - t.en_td.begin());
    std::size_t const lo = hi - 1;
    if (en == t.en_td[lo]) {
        out = {t.k0[lo], t.nu2[lo], t.nu3[lo], t.dl[lo], t.dt[lo]};
        return out;
    }
    double const f = (std::log(en) - t.log_en_td[lo]) / (t.log_en_td[hi] - t.log_en_td[lo]);
    out.k0 = std::exp(t.log_k0[lo] + f * (t.log_k0[hi] - t.log_k0[lo]));
    double const a = t.nu2[lo], b = t.nu2[hi];
    out.nu2 = a > 0.0 && b > 0.0 ? std::exp(std::log(a) + f * std::log(b / a)) : a + f * (b - a);
    out.nu3 = std::exp(t.log_nu3[lo] + f * (t.log_nu3[hi] - t.log_nu3[lo]));
    out.dl = std::exp(t.log_dl[lo] + f * (t.log_dl[hi] - t.log_dl[lo]));
    out.dt = std::exp(t.log_dt[lo] + f * (t.log_dt[hi] - t.log_dt[lo]));
    return out;
}

// BuildElectronClosureCellFields (S/LowEnergyFluidFaceTransport.cpp:1034-1243)
void closure_fields(rrea_host::ClosureTable const& t, Grid const& g, double scalar_chi, double const* er,
                    double const* ez, double const* chi, double const* ne, double const* src, double* mu, double* nu,
                    double* diff3, ClosureDiag& d)
{
    std::size_t const n = static_cast<std::size_t>(g.nr) * g.nz;
    if (mu) std::fill(mu, mu + n, 0.0);
    if (nu) std::fill(nu, nu + n, 0.0);
    if (diff3) std::fill(diff3, diff3 + 3 * n, 0.0);
    for (int j = 0; j < g.nz; ++j) {
        for (int i = 0; i < g.nr; ++i) {
            std::size_t const k = static_cast<std::size_t>(i) + static_cast<std::size_t>(g.nr) * j;
            double const x = chi ? chi[k] : scalar_chi;
            double const e_mag = std::hypot(er[k], ez[k]);
            double const ev = ne ? ne[k] : 0.0;
            double const sv = src ? src[k] : 0.0;
            if (!std::isfinite(x) || !(x > 0.0) || !std::isfinite(e_mag) || !std::isfinite(ev) || !std::isfinite(sv)) {
                ++d.invalid;
                continue;
            }
            double const en = e_mag * 1.0e21 / (x * kNL);
            int status = rrea_host::kClosureInvalid;
            Coefficients const co = evaluate(t, en, status);
            if (status == rrea_host::kClosureHeldBelow) ++d.held_below;
            if (status == rrea_host::kClosureAboveRange) ++d.above_range;
            if (status == rrea_host::kClosureInvalid) {
                ++d.invalid;
                continue;
            }
            d.min_en = std::min(d.min_en, en);
            d.max_en = std::max(d.max_en, en);
            double const local_mu = co.k0 / x;
            double const r_in = g.r_lo + static_cast<double>(i) * g.dr;
            double const volume = shell_volume(r_in, r_in + g.dr, g.dz);
            double const count = std::max(ev, 0.0) * volume;
            d.electron_count += count;
            d.source_rate += std::max(sv, 0.0) * volume;
            if (status == rrea_host::kClosureHeldBelow) d.held_below_count += count;
            if (mu) mu[k] = local_mu;
            if (nu) nu[k] = co.nu2 * x + co.nu3 * x * x;
            if (diff3) {
                double const dl = co.dl / x, dt = co.dt / x;
                double br = 0.0, bz = 0.0;
                if (e_mag > 0.0) {
                    br = er[k] / e_mag;
                    bz = ez[k] / e_mag;
                }
                double const an = dl - dt;
                diff3[k] = dt + an * br * br;
                diff3[n + k] = an * br * bz;
                diff3[2 * n + k] = dt + an * bz * bz;
            }
        }
    }
}

// BuildExplicitFaceTransport (S/LowEnergyFluidFaceTransport.cpp:200-565) on the
// frozen state dens: the tensor check and stability bound, then every face's
// drift (+ table diffusion) number flux; fr/fz (3 x faces, zeroed here).
void build_faces(rrea_gpu_fluid_config const& c, Grid const& g, double dt, double const* const dens[3],
                 double const* chi, double const* mu_cell, double const* diff3, double const* efr,
                 double const* efz, double* fr_out, double* fz_out, TransportDiag& out)
{
    int const nr = g.nr, nz = g.nz;
    bool const per = g.periodic_z;
    std::size_t const nc = static_cast<std::size_t>(nr) * nz;
    std::size_t const nfr = static_cast<std::size_t>(nr + 1) * nz;
    std::size_t const nfz = static_cast<std::size_t>(nr) * (nz + 1);
    bool const from_field = c.electron_drift_enable && c.electron_mobility_model == RREA_GPU_MOBILITY_EN_TABLE_FLUX;
    if (!std::isfinite(dt) || dt <= 0.0) bad_arg("explicit carrier face transport requires finite, positive dt");
    if (from_field != (mu_cell != nullptr) || from_field != (diff3 != nullptr)) {
        bad_arg("en_table_flux_v1 face transport requires exactly its mobility and diffusion-tensor fields");
    }
    auto wrap = [&](int j) { return per ? ((j % nz) + nz) % nz : j; };
    auto cell = [&](int i, int j) { return static_cast<std::size_t>(i) + static_cast<std::size_t>(nr) * wrap(j); };
    auto carrier = [&](int s, int i, int j) {
        double const v = std::max(dens[s][cell(i, j)], 0.0);
        return v > kVacuum ? v : 0.0;
    };
    Law const laws[3] = {ion_law(c, true), ion_law(c, false), electron_law(c)};
    auto mobility = [&](int s, int i, int j) {
        if (s == 2 && from_field) return std::max(mu_cell[cell(i, j)], 0.0);
        return laws[s].at(checked_ratio(chi, cell(i, j), c.transport_density_ratio));
    };
    auto tensor = [&](int i, int j, int comp) { return diff3[static_cast<std::size_t>(comp) * nc + cell(i, j)]; };
    bool const enabled[3] = {c.ion_drift_enable != 0, c.ion_drift_enable != 0, c.electron_drift_enable != 0};
    // ---- Build: tensor check and stability bound
    out = TransportDiag{};
    if (from_field) {
        bool invalid = false;
        double max_eig = 0.0;
        for (std::size_t k = 0; k < nc; ++k) {
            double const rr = diff3[k], rz = diff3[nc + k], zz = diff3[2 * nc + k];
            double const det = rr * zz - rz * rz;
            double const det_scale = std::max({std::abs(rr * zz), std::abs(rz * rz), 1.0});
            if (!std::isfinite(rr) || !std::isfinite(rz) || !std::isfinite(zz) || rr < 0.0 || zz < 0.0
                || det < -(512.0 * kEps * det_scale)) {
                invalid = true;
                continue;
            }
            max_eig = std::max(max_eig, 0.5 * (rr + zz + std::hypot(rr - zz, 2.0 * rz)));
        }
        if (invalid) fail("en_table_flux_v1 diffusion tensor is not finite symmetric positive-semidefinite");
        double const inv2 = 1.0 / (g.dr * g.dr) + 1.0 / (g.dz * g.dz);
        out.max_diffusion_number = 2.0 * dt * max_eig * inv2;
        if (!std::isfinite(out.max_diffusion_number) || out.max_diffusion_number >= 1.0) {
            fail("explicit electron diffusion violates its stability bound");
        }
    }
    // ---- Build: face number fluxes
    std::fill(fr_out, fr_out + 3 * nfr, 0.0);
    std::fill(fz_out, fz_out + 3 * nfz, 0.0);
    double* const fr = fr_out;
    double* const fz = fz_out;
    auto face = [&](int dir, int i, int j, double e_face, double* flux3) {
        double sigma = 0.0;
        for (int s = 0; s < 3; ++s) {
            if (!enabled[s]) continue;
            bool has_lo = true, has_hi = true;
            double n_lo = 0.0, n_hi = 0.0, mu_lo = 0.0, mu_hi = 0.0;
            if (dir == 0) {
                if (i <= 0) {
                    has_lo = has_hi = false;
                } else if (i > nr - 1) {
                    has_hi = false;
                    n_lo = carrier(s, i - 1, j);
                    mu_lo = mobility(s, i - 1, j);
                } else {
                    n_lo = carrier(s, i - 1, j);
                    n_hi = carrier(s, i, j);
                    mu_lo = mobility(s, i - 1, j);
                    mu_hi = mobility(s, i, j);
                }
            } else if (!per && j <= 0) {
                has_lo = false;
                n_hi = carrier(s, i, 0);
                mu_hi = mobility(s, i, 0);
            } else if (!per && j > nz - 1) {
                has_hi = false;
                n_lo = carrier(s, i, nz - 1);
                mu_lo = mobility(s, i, nz - 1);
            } else {
                n_lo = carrier(s, i, j - 1);
                n_hi = carrier(s, i, j);
                mu_lo = mobility(s, i, j - 1);
                mu_hi = mobility(s, i, j);
            }
            if (!has_lo && !has_hi) continue;
            double const mu_face = has_lo && has_hi ? 0.5 * (mu_lo + mu_hi) : (has_lo ? mu_lo : mu_hi);
            double const velocity = (s == 0 ? 1.0 : -1.0) * mu_face * e_face;
            double donor = 0.0;
            if (velocity > 0.0 && has_lo) donor = n_lo;
            else if (velocity < 0.0 && has_hi) donor = n_hi;
            else if (velocity == 0.0 && has_lo && has_hi) donor = 0.5 * (n_lo + n_hi);
            double number_flux = velocity * donor;
            if (s == 2 && from_field) {
                double diffusive = 0.0;
                if (dir == 0) {
                    if (i > 0 && i <= nr - 1) {
                        double const d_rr = 0.5 * (tensor(i - 1, j, 0) + tensor(i, j, 0));
                        double const d_rz = 0.5 * (tensor(i - 1, j, 1) + tensor(i, j, 1));
                        double const grad_r = (n_hi - n_lo) / g.dr;
                        auto axial = [&](int ii, int jj) {
                            if (!per && jj <= 0) return (carrier(2, ii, jj + 1) - carrier(2, ii, jj)) / g.dz;
                            if (!per && jj >= nz - 1) return (carrier(2, ii, jj) - carrier(2, ii, jj - 1)) / g.dz;
                            return (carrier(2, ii, jj + 1) - carrier(2, ii, jj - 1)) / (2.0 * g.dz);
                        };
                        double const grad_z = 0.5 * (axial(i - 1, j) + axial(i, j));
                        diffusive = -(d_rr * grad_r + d_rz * grad_z);
                    } else if (i > nr - 1) {
                        diffusive = 2.0 * tensor(i - 1, j, 0) * n_lo / g.dr;
                    }
                } else {
                    if ((!per && j > 0 && j <= nz - 1) || per) {
                        double const d_rz = 0.5 * (tensor(i, j - 1, 1) + tensor(i, j, 1));
                        double const d_zz = 0.5 * (tensor(i, j - 1, 2) + tensor(i, j, 2));
                        auto radial = [&](int ii, int jj) {
                            if (nr - 1 == 0) return 0.0;
                            if (ii <= 0) return (carrier(2, ii + 1, jj) - carrier(2, ii, jj)) / g.dr;
                            if (ii >= nr - 1) return (carrier(2, ii, jj) - carrier(2, ii - 1, jj)) / g.dr;
                            return (carrier(2, ii + 1, jj) - carrier(2, ii - 1, jj)) / (2.0 * g.dr);
                        };
                        double const grad_r = 0.5 * (radial(i, j - 1) + radial(i, j));
                        double const grad_z = (n_hi - n_lo) / g.dz;
                        diffusive = -(d_rz * grad_r + d_zz * grad_z);
                    } else if (j <= 0) {
                        diffusive = -2.0 * tensor(i, 0, 2) * n_hi / g.dz;
                    } else {
                        diffusive = 2.0 * tensor(i, nz - 1, 2) * n_lo / g.dz;
                    }
                }
                if ((diffusive > 0.0 && (!has_lo || n_lo <= 0.0)) || (diffusive < 0.0 && (!has_hi || n_hi <= 0.0))) {
                    diffusive = 0.0;
                }
                number_flux += diffusive;
            }
            flux3[s] = number_flux;
            sigma += kQe * mu_face * donor;
        }
        out.max_face_conductivity = std::max(out.max_face_conductivity, sigma);
    };
    for (int j = 0; j < nz; ++j) {
        for (int i = 0; i <= nr; ++i) {
            std::size_t const f = static_cast<std::size_t>(i) + static_cast<std::size_t>(nr + 1) * j;
            double v[3] = {0.0, 0.0, 0.0};
            face(0, i, j, efr[f], v);
            for (int s = 0; s < 3; ++s) fr[s * nfr + f] = v[s];
        }
    }
    for (int j = 0; j <= nz; ++j) {
        for (int i = 0; i < nr; ++i) {
            std::size_t const f = static_cast<std::size_t>(i) + static_cast<std::size_t>(nr) * j;
            double v[3] = {0.0, 0.0, 0.0};
            face(1, i, j, efz[f], v);
            for (int s = 0; s < 3; ++s) fz[s * nfz + f] = v[s];
        }
    }
    if (per) {   // OverrideSync: the low copy of the periodic face owns it
        for (int s = 0; s < 3; ++s)
            for (int i = 0; i < nr; ++i) fz[s * nfz + i + static_cast<std::size_t>(nr) * nz] = fz[s * nfz + i];
    }
}

// PrepareExplicitCarrierTransport + BuildExplicitFaceTransport +
// ApplyExplicitCarrierTransport (S/LowEnergyFluidFaceTransport.cpp:165-954)
void transport(rrea_gpu_fluid_config const& c, Grid const& g, double dt, double* const dens[3], double* rho,
               double const* chi, double const* mu_cell, double const* diff3, double const* efr, double const* efz,
               double* flux_r, double* flux_z, double* raw_r, double* raw_z, TransportDiag& out)
{
    validate_transport(c, true);
    if (!std::isfinite(dt) || dt <= 0.0) bad_arg("explicit carrier face transport requires finite, positive dt");
    int const nr = g.nr, nz = g.nz;
    bool const per = g.periodic_z;
    std::size_t const nc = static_cast<std::size_t>(nr) * nz;
    std::size_t const nfr = static_cast<std::size_t>(nr + 1) * nz;
    std::size_t const nfz = static_cast<std::size_t>(nr) * (nz + 1);
    bool const from_field = c.electron_drift_enable && c.electron_mobility_model == RREA_GPU_MOBILITY_EN_TABLE_FLUX;
    if (from_field != (mu_cell != nullptr) || from_field != (diff3 != nullptr)) {
        bad_arg("en_table_flux_v1 face transport requires exactly its mobility and diffusion-tensor fields");
    }
    // frozen post-chemistry state (Prepare): a periodic z wraps the rows
    auto wrap = [&](int j) { return per ? ((j % nz) + nz) % nz : j; };
    auto cell = [&](int i, int j) { return static_cast<std::size_t>(i) + static_cast<std::size_t>(nr) * wrap(j); };
    std::vector<double> old[3];
    for (int s = 0; s < 3; ++s) old[s].assign(dens[s], dens[s] + nc);
    auto carrier = [&](int s, int i, int j) {
        double const v = std::max(old[s][cell(i, j)], 0.0);
        return v > kVacuum ? v : 0.0;
    };
    Law const laws[3] = {ion_law(c, true), ion_law(c, false), electron_law(c)};
    auto mobility = [&](int s, int i, int j) {
        if (s == 2 && from_field) return std::max(mu_cell[cell(i, j)], 0.0);
        return laws[s].at(checked_ratio(chi, cell(i, j), c.transport_density_ratio));
    };
    auto tensor = [&](int i, int j, int comp) { return diff3[static_cast<std::size_t>(comp) * nc + cell(i, j)]; };
    bool const enabled[3] = {c.ion_drift_enable != 0, c.ion_drift_enable != 0, c.electron_drift_enable != 0};
    out = TransportDiag{};
    std::vector<double> fr(3 * nfr, 0.0), fz(3 * nfz, 0.0);
    double const* const frozen[3] = {old[0].data(), old[1].data(), old[2].data()};
    build_faces(c, g, dt, frozen, chi, mu_cell, diff3, efr, efz, fr.data(), fz.data(), out);
    if (raw_r) std::copy(fr.begin(), fr.end(), raw_r);
    if (raw_z) std::copy(fz.begin(), fz.end(), raw_z);

    // ---- Apply: positivity limiter per donor cell and carrier
    auto FR = [&](int s, int i, int j) -> double& {
        return fr[static_cast<std::size_t>(s) * nfr + i + static_cast<std::size_t>(nr + 1) * j];
    };
    auto FZ = [&](int s, int i, int j) -> double& {
        return fz[static_cast<std::size_t>(s) * nfz + i + static_cast<std::size_t>(nr) * j];
    };
    struct Metric {
        double volume, shell, a_lo, a_hi;
    };
    auto metric = [&](int i) {
        double const r_lo = g.r_lo + static_cast<double>(i) * g.dr;
        double const r_hi = r_lo + g.dr;
        return Metric{shell_volume(r_lo, r_lo + g.dr, g.dz), kPi * std::max(r_hi * r_hi - r_lo * r_lo, 0.0),
                      2.0 * kPi * r_lo * g.dz, 2.0 * kPi * r_hi * g.dz};
    };
    auto outgoing_of = [&](int s, int i, int j, Metric const& m) {
        double o = std::max(FR(s, i + 1, j), 0.0) * m.a_hi + std::max(-FR(s, i, j), 0.0) * m.a_lo;
        o += (std::max(FZ(s, i, j + 1), 0.0) + std::max(-FZ(s, i, j), 0.0)) * m.shell;
        return o;
    };
    double const roundoff = 512.0 * kEps;
    double const limiter_cfl = c.ion_drift_cfl * (1.0 - roundoff);
    std::vector<double> scale(3 * nc, 1.0);
    double unlimited = 0.0, before = 0.0, removed = 0.0, e_number = 0.0, e_limited = 0.0;
    out.min_outflow_scale = 1.0;
    for (int j = 0; j < nz; ++j) {
        for (int i = 0; i < nr; ++i) {
            Metric const m = metric(i);
            for (int s = 0; s < 3; ++s) {
                if (!enabled[s]) continue;
                double const density = std::max(old[s][cell(i, j)], 0.0);
                double const outgoing = outgoing_of(s, i, j, m);
                double const rate = density > 0.0 ? outgoing / (density * std::max(m.volume, 1.0e-300))
                                                  : (outgoing > 0.0 ? 1.0e300 : 0.0);
                unlimited = std::max(unlimited, rate);
                double limiter = 1.0;
                if (outgoing > 0.0) {
                    limiter = density > 0.0 ? std::min(1.0, limiter_cfl * density * m.volume / (dt * outgoing)) : 0.0;
                }
                scale[static_cast<std::size_t>(s) * nc + cell(i, j)] = limiter;
                out.min_outflow_scale = std::min(out.min_outflow_scale, limiter);
                before += outgoing;
                removed += (1.0 - limiter) * outgoing;
                if (s == 2) {
                    double const en = density * m.volume;
                    e_number += en;
                    if (limiter < 1.0) e_limited += en;
                }
            }
        }
    }
    for (int s = 0; s < 3; ++s) {
        for (int j = 0; j < nz; ++j) {
            for (int i = 0; i <= nr; ++i) {
                double& v = FR(s, i, j);
                if (v == 0.0) continue;
                int const di = v > 0.0 ? i - 1 : i;
                v = (di >= 0 && di <= nr - 1) ? v * scale[static_cast<std::size_t>(s) * nc + cell(di, j)] : 0.0;
            }
        }
        for (int j = 0; j <= nz; ++j) {
            for (int i = 0; i < nr; ++i) {
                double& v = FZ(s, i, j);
                if (v == 0.0) continue;
                int const dj = v > 0.0 ? j - 1 : j;
                bool const inside = per || (dj >= 0 && dj <= nz - 1);
                v = inside ? v * scale[static_cast<std::size_t>(s) * nc + cell(i, dj)] : 0.0;
            }
        }
        if (per) {
            for (int i = 0; i < nr; ++i) FZ(s, i, nz) = FZ(s, i, 0);
        }
    }
    out.unlimited_max_outgoing_cfl = dt * unlimited;
    out.limited_outflow_fraction = before > 0.0 ? std::clamp(removed / before, 0.0, 1.0) : 0.0;
    out.limited_electron_number_fraction = e_number > 0.0 ? std::clamp(e_limited / e_number, 0.0, 1.0) : 0.0;
    // realized outgoing CFL and drift speed
    double max_rate = 0.0, max_speed = 0.0;
    for (int j = 0; j < nz; ++j) {
        for (int i = 0; i < nr; ++i) {
            Metric const m = metric(i);
            for (int s = 0; s < 3; ++s) {
                if (!enabled[s]) continue;
                double const density = std::max(old[s][cell(i, j)], 0.0);
                double const outgoing = outgoing_of(s, i, j, m);
                if (density > 0.0) {
                    max_rate = std::max(max_rate, outgoing / (density * std::max(m.volume, 1.0e-300)));
                    for (double o : {-FR(s, i, j), FR(s, i + 1, j), -FZ(s, i, j), FZ(s, i, j + 1)}) {
                        max_speed = std::max(max_speed, std::max(o, 0.0) / density);
                    }
                }
            }
        }
    }
    out.max_outgoing_cfl = dt * max_rate;
    if (out.max_outgoing_cfl > c.ion_drift_cfl + roundoff * std::max(1.0, c.ion_drift_cfl)) {
        fail("limited full-step carrier drift violates outgoing CFL");
    }
    out.max_drift_speed = max_speed;
    out.cfl_dt = max_rate > 0.0 ? c.ion_drift_cfl / max_rate : 1.0e300;
    // conservative update of the densities and the fluid charge
    bool nonfinite = false;
    double min_density = 0.0;
    for (int j = 0; j < nz; ++j) {
        for (int i = 0; i < nr; ++i) {
            Metric const m = metric(i);
            std::size_t const k = cell(i, j);
            auto updated = [&](int s) {
                double const r_delta = FR(s, i + 1, j) * m.a_hi - FR(s, i, j) * m.a_lo;
                double const z_delta = (FZ(s, i, j + 1) - FZ(s, i, j)) * m.shell;
                return old[s][k] - dt * (r_delta + z_delta) / std::max(m.volume, 1.0e-300);
            };
            if (enabled[0]) {
                dens[0][k] = updated(0);
                dens[1][k] = updated(1);
            }
            if (enabled[2]) dens[2][k] = updated(2);
            auto cur_r = [&](int ii) { return kQe * (FR(0, ii, j) - FR(1, ii, j) - FR(2, ii, j)); };
            auto cur_z = [&](int jj) { return kQe * (FZ(0, i, jj) - FZ(1, i, jj) - FZ(2, i, jj)); };
            double delta = cur_r(i + 1) * m.a_hi - cur_r(i) * m.a_lo;
            delta += (cur_z(j + 1) - cur_z(j)) * m.shell;
            rho[k] -= dt * delta / std::max(m.volume, 1.0e-300);
            for (int s = 0; s < 3; ++s) {
                double const v = dens[s][k];
                if (!std::isfinite(v)) nonfinite = true;
                else min_density = std::min(min_density, v);
            }
        }
    }
    if (nonfinite) fail("explicit carrier transport produced a non-finite density");
    if (min_density < 0.0) fail("explicit carrier transport produced negative density despite CFL gate");
    // carrier centres (CollectCarrierDriftCenterDiagnostics, :956-1032)
    Law const pos = ion_law(c, true);
    double sums[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int j = 0; j < nz; ++j) {
        for (int i = 0; i < nr; ++i) {
            std::size_t const k = cell(i, j);
            double const volume = metric(i).volume;
            double const p = std::max(dens[0][k], 0.0) * volume;
            double const q = std::max(dens[1][k], 0.0) * volume;
            double const rc = g.r_lo + (static_cast<double>(i) + 0.5) * g.dr;
            double const zc = g.z_lo + (static_cast<double>(j) + 0.5) * g.dz;
            sums[0] += p;
            sums[1] += q;
            sums[2] += p * rc;
            sums[3] += p * zc;
            sums[4] += q * rc;
            sums[5] += q * zc;
            double const d = chi ? std::max(chi[k], 1.0e-300) : c.transport_density_ratio;
            sums[6] += p * d;
            sums[7] += p * pos.at(d);
        }
    }
    if (sums[0] > 0.0) {
        out.pos_center_r = sums[2] / sums[0];
        out.pos_center_z = sums[3] / sums[0];
        out.density_ratio_at_pos_center = sums[6] / sums[0];
        out.mu_pos_at_pos_center = sums[7] / sums[0];
    }
    if (sums[1] > 0.0) {
        out.neg_center_r = sums[4] / sums[1];
        out.neg_center_z = sums[5] / sums[1];
    }
    if (flux_r) std::copy(fr.begin(), fr.end(), flux_r);
    if (flux_z) std::copy(fz.begin(), fz.end(), flux_z);
}

}  // namespace oracle_fluid

namespace oracle_fluid {

// RreaAmrexAdvance::AdvanceOneStep (S/RreaAmrexAdvance.cpp:593-838) with the
// fluid: the closure fields at the step start, the stiffness probe, the
// shared material substeps (half reaction, transport, total face current,
// B / Silver-Mueller / E, committed field, closure fields, half reaction),
// the B restagger, the final conductivity and the cleared sources.  The
// material-continuity audit (VerifyMaterialContinuity) is not restated.
void coupled_step(rrea_gpu_fluid_config const& c, rrea_host::ClosureTable const* table, Grid const& g, double dt,
                  oracle::MaxwellField& f, std::vector<double> const& amb_er, std::vector<double> const& amb_ez,
                  std::vector<double> const& jr_kin, std::vector<double> const& jz_kin, State& st, double const* chi,
                  CoupledDiag& diag)
{
    if (!std::isfinite(dt) || dt <= 0.0) bad_arg("RreaAmrexAdvance requires finite, positive dt");
    if (g.periodic_z) bad_arg("the coupled field step needs a non-periodic z");
    double const cfl = 299792458.0 * dt * std::sqrt(1.0 / (f.dr * f.dr) + 1.0 / (f.dz * f.dz));
    if (!std::isfinite(cfl) || !(cfl < 1.0)) bad_arg("Maxwell TM violates the two-dimensional Yee CFL condition");
    bool const mob_table = c.electron_drift_enable && c.electron_mobility_model == RREA_GPU_MOBILITY_EN_TABLE_FLUX;
    bool const att_table = c.attachment_model == RREA_GPU_ATTACHMENT_EN_TABLE;
    if ((mob_table || att_table) && table == nullptr) bad_arg("en_table fluid models require a loaded electron closure");
    int const nr = g.nr, nz = g.nz;
    std::size_t const n = static_cast<std::size_t>(nr) * nz;
    std::size_t const nfr = static_cast<std::size_t>(nr + 1) * nz, nfz = static_cast<std::size_t>(nr) * (nz + 1);
    std::vector<double> sigma(n), tau(n), fr(3 * nfr), fz(3 * nfz);
    // total face field (CommitMaxwellTotalField, :477-505)
    std::vector<double> tr(nfr), tz(nfz);
    auto commit = [&] {
        for (std::size_t k = 0; k < nfr; ++k) tr[k] = f.er[k] + amb_er[k];
        for (std::size_t k = 0; k < nfz; ++k) tz[k] = f.ez[k] + amb_ez[k];
    };
    commit();
    // EvaluateClosureFields (:282-440): cell averages of the committed field
    auto evaluate_closure = [&] {
        std::vector<double> er(n), ez(n);
        for (int j = 0; j < nz; ++j)
            for (int i = 0; i < nr; ++i) {
                std::size_t const k = static_cast<std::size_t>(i) + static_cast<std::size_t>(nr) * j;
                er[k] = 0.5 * (tr[i + static_cast<std::size_t>(nr + 1) * j] + tr[i + 1 + static_cast<std::size_t>(nr + 1) * j]);
                ez[k] = 0.5 * (tz[k] + tz[k + static_cast<std::size_t>(nr)]);
            }
        ClosureDiag d;
        closure_fields(*table, g, c.transport_density_ratio, er.data(), ez.data(), chi, st.ne.data(), st.se.data(),
                       mob_table ? st.mu.data() : nullptr, att_table ? st.nu.data() : nullptr,
                       mob_table ? st.diff3.data() : nullptr, d);
        if (d.above_range > 0 || d.invalid > 0) fail("electron closure range violation");
    };
    if (mob_table) {
        st.mu.resize(n);
        st.diff3.resize(3 * n);
    }
    if (att_table) st.nu.resize(n);
    if (mob_table || att_table) evaluate_closure();
    double const* mu = mob_table ? st.mu.data() : nullptr;
    double const* d3 = mob_table ? st.diff3.data() : nullptr;
    double const* nu = att_table ? st.nu.data() : nullptr;
    // the stiffness probe on a non-mutating transport build
    conductivity(c, n, st.ne.data(), st.np.data(), st.nn.data(), chi, mu, sigma.data(), tau.data());
    TransportDiag probe;
    {
        State scratch = st;
        double* const dens[3] = {scratch.np.data(), scratch.nn.data(), scratch.ne.data()};
        build_faces(c, g, dt * 1.0e-6, dens, chi, mu, d3, tr.data(), tz.data(), fr.data(), fz.data(), probe);
    }
    double const eps0 = 8.8541878128e-12;
    diag.full_conduction = dt * probe.max_face_conductivity / eps0;
    diag.full_diffusion = probe.max_diffusion_number / 1.0e-6;
    diag.full_reaction = dt * max_reaction_frequency(c, n, st.ne.data(), st.np.data(), st.nn.data(), nu);
    if (!std::isfinite(diag.full_conduction) || !std::isfinite(diag.full_diffusion) || !std::isfinite(diag.full_reaction)) {
        fail("fluid/Maxwell coupling stiffness is non-finite");
    }
    double const required = std::max({diag.full_conduction / c.material_conduction_target,
                                      diag.full_diffusion / c.material_diffusion_target,
                                      diag.full_reaction / c.material_reaction_target});
    if (required > c.material_max_substeps) fail("fluid/Maxwell coupling exceeds configured maximum substeps");
    int const substeps = std::max(c.material_min_substeps, static_cast<int>(std::ceil(required)));
    diag.substeps = substeps;
    double const dts = dt / static_cast<double>(substeps);
    double const restagger = 0.5 * (dt - dts);
    oracle::MaxwellAdvanceB(f, restagger);
    auto half_reaction = [&] {
        double const number = dts * max_reaction_frequency(c, n, st.ne.data(), st.np.data(), st.nn.data(), nu);
        diag.max_reaction_number = std::max(diag.max_reaction_number, number);
        if (number > c.material_reaction_guard) fail("reaction substep out of configured range");
        double const r = react(c, n, 0.5 * dts, st.ne.data(), st.np.data(), st.nn.data(), st.se.data(), st.sp.data(),
                               st.sn.data(), st.rho.data(), nu, false);
        diag.max_residual = std::max(diag.max_residual, r);
    };
    std::vector<double> jr(nfr), jz(nfz);
    double const qe = kQe;
    for (int s = 0; s < substeps; ++s) {
        half_reaction();
        conductivity(c, n, st.ne.data(), st.np.data(), st.nn.data(), chi, mu, sigma.data(), tau.data());
        TransportDiag td;
        double* const dens[3] = {st.np.data(), st.nn.data(), st.ne.data()};
        transport(c, g, dts, dens, st.rho.data(), chi, mu, d3, tr.data(), tz.data(), fr.data(), fz.data(), nullptr,
                  nullptr, td);
        double const sig = dts * td.max_face_conductivity / eps0;
        diag.max_dt_sigma = std::max(diag.max_dt_sigma, sig);
        if (sig > c.material_conduction_guard) fail("explicit conduction substep out of configured range");
        diag.max_diffusion_number = std::max(diag.max_diffusion_number, td.max_diffusion_number);
        if (td.max_diffusion_number > c.material_diffusion_guard) fail("explicit diffusion substep out of configured range");
        // AssembleTotalFaceCurrent (:840-871): qe (G+ - G- - Ge) + kinetic
        for (std::size_t k = 0; k < nfr; ++k) {
            double v = 0.0;
            v += qe * fr[k];
            v += -qe * fr[nfr + k];
            v += -qe * fr[2 * nfr + k];
            jr[k] = v + jr_kin[k];
        }
        for (std::size_t k = 0; k < nfz; ++k) {
            double v = 0.0;
            v += qe * fz[k];
            v += -qe * fz[nfz + k];
            v += -qe * fz[2 * nfz + k];
            jz[k] = v + jz_kin[k];
        }
        oracle::MaxwellAdvanceB(f, dts);
        oracle::MaxwellSilverMueller(f);
        oracle::MaxwellAdvanceE(f, dts, jr, jz);
        commit();
        if (mob_table || att_table) evaluate_closure();
        half_reaction();
    }
    oracle::MaxwellAdvanceB(f, -restagger);
    oracle::MaxwellSilverMueller(f);
    conductivity(c, n, st.ne.data(), st.np.data(), st.nn.data(), chi, mu, sigma.data(), tau.data());
    st.sigma = sigma;
    st.tau = tau;
    std::fill(st.se.begin(), st.se.end(), 0.0);
    std::fill(st.sp.begin(), st.sp.end(), 0.0);
    std::fill(st.sn.begin(), st.sn.end(), 0.0);
}

}  // namespace oracle_fluid
