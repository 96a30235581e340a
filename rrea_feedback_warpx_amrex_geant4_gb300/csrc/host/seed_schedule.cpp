// Seed schedule input adapter (see seed_schedule.hpp for the reference
// interfaces each function follows).
#include "seed_schedule.hpp"

#include "csv_text.hpp"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <fstream>
#include <limits>
#include <map>
#include <set>
#include <sstream>

namespace rrea_host {

namespace {

constexpr double kMeC2 = 510998.95000;  // I/RreaConstants.H:9
constexpr double kC = 299792458.0;      // I/RreaConstants.H:10

[[noreturn]] void fail(int code, std::string const& msg) { throw SeedScheduleError(code, msg); }

using csv::split_cells;
using csv::trim;

// A whole cell must parse as one number (S/RreaSeedSchedule.cpp:28-39).
template <typename T>
T number(std::string const& text, char const* column)
{
    std::istringstream in(text);
    T v{};
    in >> v;
    if (!in || !in.eof()) {
        fail(RREA_GPU_ERR_ARGUMENT, std::string("invalid numeric value in seed schedule column ") + column + ": " + text);
    }
    return v;
}

struct Columns {
    std::map<std::string, int> index;
    // a required column must exist; a short row reads as an empty cell
    std::string required(std::vector<std::string> const& row, char const* name) const
    {
        auto const it = index.find(name);
        if (it == index.end()) fail(RREA_GPU_ERR_ARGUMENT, std::string("missing seed schedule column: ") + name);
        return static_cast<std::size_t>(it->second) < row.size() ? row[static_cast<std::size_t>(it->second)]
                                                                 : std::string();
    }
    std::string optional(std::vector<std::string> const& row, char const* name) const
    {
        auto const it = index.find(name);
        if (it == index.end()) return {};
        return static_cast<std::size_t>(it->second) < row.size() ? row[static_cast<std::size_t>(it->second)]
                                                                 : std::string();
    }
};

}  // namespace

double electron_proper_velocity(double k)
{
    if (k <= 0.0) return 0.0;
    double const gamma = 1.0 + k / kMeC2;
    return kC * std::sqrt(std::max(gamma * gamma - 1.0, 0.0));
}

void normalize_seed_momentum(double ux, double uy, double uz, double k, double out[3])
{
    double const norm = std::sqrt(ux * ux + uy * uy + uz * uz);
    if (k > 0.0 && norm > 0.0 && norm < kSeedDirectionHintMaxMPerS) {
        double const u = electron_proper_velocity(k);
        out[0] = u * ux / norm;
        out[1] = u * uy / norm;
        out[2] = u * uz / norm;
        return;
    }
    out[0] = ux;
    out[1] = uy;
    out[2] = uz;
}

int seed_window_class(double t, double begin, double end)
{
    if (t < begin) return -1;
    if (t >= end) return 1;
    return 0;
}

void SeedSchedule::load(std::string const& path, std::string const& case_id)
{
    std::ifstream in(path);
    if (!in) fail(RREA_GPU_ERR_ARGUMENT, "could not open the seed schedule: " + path);
    std::string header;
    if (!std::getline(in, header)) fail(RREA_GPU_ERR_ARGUMENT, "empty seed schedule: " + path);
    Columns cols;
    std::vector<std::string> const names = split_cells(header);
    for (std::size_t i = 0; i < names.size(); ++i) {
        if (!cols.index.emplace(names[i], static_cast<int>(i)).second) {
            fail(RREA_GPU_ERR_ARGUMENT, "duplicate seed schedule column: " + names[i]);
        }
    }
    std::vector<rrea_gpu_seed_event> events;
    std::string line;
    int line_number = 1;
    while (std::getline(in, line)) {
        ++line_number;
        if (trim(line).empty()) continue;
        std::vector<std::string> const row = split_cells(line);
        if (!case_id.empty() && cols.required(row, "case_id") != case_id) continue;
        cols.required(row, "case_id");
        rrea_gpu_seed_event e{};
        std::string const macro = cols.optional(row, "macro_index");
        e.macro_index = macro.empty() ? line_number : number<int>(macro, "macro_index");
        std::string const species = cols.optional(row, "species_id");
        e.species_id = species.empty() ? kSeedElectron : number<int>(species, "species_id");
        e.time_s = number<double>(cols.required(row, "time_s"), "time_s");
        e.x_m = number<double>(cols.required(row, "x_m"), "x_m");
        e.y_m = number<double>(cols.required(row, "y_m"), "y_m");
        e.z_m = number<double>(cols.required(row, "z_m"), "z_m");
        e.r_m = number<double>(cols.required(row, "r_m"), "r_m");
        e.kinetic_energy_eV = number<double>(cols.required(row, "kinetic_energy_eV"), "kinetic_energy_eV");
        e.ux = number<double>(cols.required(row, "ux"), "ux");
        e.uy = number<double>(cols.required(row, "uy"), "uy");
        e.uz = number<double>(cols.required(row, "uz"), "uz");
        e.weight = number<double>(cols.required(row, "weight_real_electrons"), "weight_real_electrons");
        events.push_back(e);
    }
    std::sort(events.begin(), events.end(), [](rrea_gpu_seed_event const& a, rrea_gpu_seed_event const& b) {
        if (a.time_s != b.time_s) return a.time_s < b.time_s;
        return a.macro_index < b.macro_index;
    });
    m_events = std::move(events);
    cursor = 0;
}

void SeedSchedule::validate(double e_min, double e_max, double r_min, double r_max, double z_min, double z_max) const
{
    auto finite = [](double v) { return std::isfinite(v); };
    if (!finite(e_min) || !finite(e_max) || !(e_min > 0.0) || e_max < e_min || !finite(r_min) || !finite(r_max) ||
        !finite(z_min) || !finite(z_max) || !(r_max > r_min) || !(z_max > z_min)) {
        fail(RREA_GPU_ERR_ARGUMENT, "seed validation bounds are not a finite positive energy range and a nonempty domain");
    }
    double const eps = std::numeric_limits<double>::epsilon();
    std::set<int> seen;
    for (rrea_gpu_seed_event const& e : m_events) {
        // The first failing rule names the row; the rules run in the order
        // the overlay's production validation applies them.
        auto reject = [&](char const* rule) {
            fail(RREA_GPU_ERR_ARGUMENT,
                 "seed row with macro_index " + std::to_string(e.macro_index) + " rejected: " + rule);
        };
        bool const position_finite = finite(e.x_m) && finite(e.y_m) && finite(e.r_m) && finite(e.z_m);
        double const radius = std::hypot(e.x_m, e.y_m);
        double const r_tol = 128.0 * eps * std::max({1.0, radius, std::abs(e.r_m)});
        struct Rule {
            bool broken;
            char const* text;
        };
        Rule const identity[] = {
            {e.macro_index < 0, "negative macro_index"},
            {!seen.insert(e.macro_index).second, "macro_index repeats within the case"},
            {e.species_id != kSeedElectron && e.species_id != kSeedPositron, "species_id is neither 1 (e-) nor 2 (e+)"},
            {!finite(e.time_s) || e.time_s < 0.0, "time_s is negative or not finite"},
            {!finite(e.weight) || !(e.weight > 0.0), "weight_real_electrons is not a finite positive number"},
            {!position_finite, "a position column is not finite"},
            {position_finite && std::abs(e.r_m - radius) > r_tol, "r_m does not equal the radius of (x_m, y_m)"},
            {position_finite && (radius < r_min || !(radius < r_max) || e.z_m < z_min || !(e.z_m < z_max)),
             "start point lies outside the RZ domain [r_min, r_max) x [z_min, z_max)"},
            {!finite(e.kinetic_energy_eV) || e.kinetic_energy_eV < e_min || e.kinetic_energy_eV > e_max,
             "kinetic_energy_eV lies outside the tables' charged energy range"},
            {!finite(e.ux) || !finite(e.uy) || !finite(e.uz), "a momentum column is not finite"},
        };
        for (Rule const& rule : identity) {
            if (rule.broken) reject(rule.text);
        }
        double const norm = std::hypot(std::hypot(e.ux, e.uy), e.uz);
        if (!finite(norm) || !(norm > 0.0)) reject("the momentum vector is zero or overflows");
        double k = e.kinetic_energy_eV;
        if (!(norm < kSeedDirectionHintMaxMPerS)) {
            // a proper velocity, not a direction hint: its kinetic energy,
            // written without the cancellation of gamma - 1
            double const q = norm / kC;
            double const gamma = std::hypot(1.0, q);
            k = kMeC2 * q * (q / (gamma + 1.0));
        }
        if (!finite(k) || k < e_min || k > e_max) reject("the energy of the given momentum lies outside the tables' range");
        double const k_tol = 256.0 * eps * std::max({1.0, k, e.kinetic_energy_eV});
        if (std::abs(k - e.kinetic_energy_eV) > k_tol) {
            reject("the energy of the given proper velocity does not match kinetic_energy_eV");
        }
    }
}

}  // namespace rrea_host
