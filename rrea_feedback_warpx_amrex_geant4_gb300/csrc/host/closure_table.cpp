// Closure table loader (see closure_table.hpp).
#include "closure_table.hpp"

#include "csv_text.hpp"

#include <cmath>
#include <fstream>
#include <sstream>

namespace rrea_host {

namespace {

constexpr double kNLoschmidt = 2.6868e25;  // I/RreaConstants.H:16
constexpr double kTownsend = 1.0e-21;      // I/RreaConstants.H:17

[[noreturn]] void fail(std::string const& m) { throw ClosureTableError(m); }

// A whole cell must parse as one number.
double number(std::string const& text, char const* column)
{
    std::istringstream in(text);
    double v = 0.0;
    in >> v;
    if (!in || !in.eof()) fail(std::string("invalid numeric value in closure column ") + column + ": " + text);
    return v;
}

bool close(double got, double want, double floor_scale)
{
    return std::abs(got - want) <= 1.0e-9 * floor_scale;
}

}  // namespace

ClosureTable load_closure_table(std::string const& path)
{
    static char const* const kHeader =
        "en_td,flux_drift_velocity_m_per_s,reduced_flux_mobility_ref_m2_per_v_s,"
        "longitudinal_diffusion_ref_m2_per_s,transverse_diffusion_ref_m2_per_s,eta_over_n2_cm5,"
        "three_body_rate_cm6_per_s,three_body_frequency_ref_s,eta_over_n_cm2,two_body_rate_cm3_per_s,"
        "two_body_frequency_ref_s,relative_uncertainty_mobility,relative_uncertainty_three_body,"
        "relative_uncertainty_two_body,source_row";
    std::ifstream file(path, std::ios::binary);
    if (!file) fail("cannot open closure table: " + path);
    std::stringstream text;
    text << file.rdbuf();
    std::string line;
    // the header is the first line that is neither blank nor a comment
    while (std::getline(text, line)) {
        std::string const t = csv::trim(line);
        if (!t.empty() && t.front() != '#') break;
    }
    if (csv::trim(line) != kHeader) fail("electron closure table header must exactly match schema 3");
    double const n0_cm3 = kNLoschmidt * 1.0e-6;
    ClosureTable t;
    while (std::getline(text, line)) {
        std::string const trimmed = csv::trim(line);
        if (trimmed.empty() || trimmed.front() == '#') continue;
        std::vector<std::string> const c = csv::split_cells(line);
        if (c.size() != 15) fail("electron closure table row must have exactly 15 columns");
        double const en = number(c[0], "en_td");
        double const w = number(c[1], "flux_drift_velocity_m_per_s");
        double const k0 = number(c[2], "reduced_flux_mobility_ref_m2_per_v_s");
        double const dl = number(c[3], "longitudinal_diffusion_ref_m2_per_s");
        double const dt = number(c[4], "transverse_diffusion_ref_m2_per_s");
        double const eta3 = number(c[5], "eta_over_n2_cm5");
        double const k3 = number(c[6], "three_body_rate_cm6_per_s");
        double const nu3 = number(c[7], "three_body_frequency_ref_s");
        double const eta2 = number(c[8], "eta_over_n_cm2");
        double const k2 = number(c[9], "two_body_rate_cm3_per_s");
        double const nu2 = number(c[10], "two_body_frequency_ref_s");
        for (double v : {en, w, k0, dl, dt, eta3, k3, nu3}) {
            if (!std::isfinite(v) || !(v > 0.0)) fail("electron closure table values must be finite and positive: " + line);
        }
        for (double v : {eta2, k2, nu2}) {
            if (!std::isfinite(v) || v < 0.0) {
                fail("electron closure two-body values must be finite and non-negative: " + line);
            }
        }
        if ((eta2 == 0.0) != (k2 == 0.0) || (k2 == 0.0) != (nu2 == 0.0)) {
            fail("electron closure two-body columns must become positive together");
        }
        if (!t.en_td.empty() && !(en > t.en_td.back())) fail("electron closure E/N nodes must be strictly increasing");
        if (c[14].empty()) fail("electron closure table rows must carry a source_row id");
        // the derivation chain: k2 = W eta/N, nu2 = k2 N0, k3 = W eta/N^2,
        // nu3 = k3 N0^2, K0 = W / (E/N N0)
        double const k2_want = (w * 100.0) * eta2;
        double const nu2_want = k2_want * n0_cm3;
        double const k3_want = (w * 100.0) * eta3;
        double const nu3_want = k3_want * n0_cm3 * n0_cm3;
        double const k0_want = w / (en * kTownsend * kNLoschmidt);
        if (!close(k2, k2_want, std::max(k2_want, 1.0e-300)) || !close(nu2, nu2_want, std::max(nu2_want, 1.0e-300))
            || !close(k3, k3_want, k3_want) || !close(nu3, nu3_want, nu3_want) || !close(k0, k0_want, k0_want)) {
            fail("electron closure row fails its derivation identity (two-/three-body rates, frequencies, and K0): "
                 + line);
        }
        t.en_td.push_back(en);
        t.log_en_td.push_back(std::log(en));
        t.k0.push_back(k0);
        t.log_k0.push_back(std::log(k0));
        t.nu2.push_back(nu2);
        t.nu3.push_back(nu3);
        t.log_nu3.push_back(std::log(nu3));
        t.dl.push_back(dl);
        t.log_dl.push_back(std::log(dl));
        t.dt.push_back(dt);
        t.log_dt.push_back(std::log(dt));
    }
    if (t.size() < 2) fail("electron closure table needs at least two E/N nodes");
    return t;
}

}  // namespace rrea_host
