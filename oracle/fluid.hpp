// ORACLE — test infrastructure only.  Declarations of the carrier-fluid
// restatement in oracle/fluid.cpp.
#pragma once

#include "../include/rrea_gpu.h"
#include "../rrea_feedback_warpx_amrex_geant4_gb300/csrc/host/closure_table.hpp"

#include <cstddef>
#include <limits>
#include <vector>

namespace oracle { struct MaxwellField; }

namespace oracle_fluid {

struct Grid {
    int nr, nz;
    double r_lo, z_lo, dr, dz;
    bool periodic_z;
};

struct Coefficients {
    double k0, nu2, nu3, dl, dt;
};

struct ClosureDiag {
    double min_en = std::numeric_limits<double>::max();
    double max_en = 0.0;
    double held_below = 0.0, above_range = 0.0, invalid = 0.0;
    double electron_count = 0.0, held_below_count = 0.0, source_rate = 0.0;
};

struct TransportDiag {
    double max_face_conductivity = 0.0;
    double max_diffusion_number = 0.0;
    double unlimited_max_outgoing_cfl = 0.0;
    double min_outflow_scale = 1.0;
    double limited_outflow_fraction = 0.0;
    double limited_electron_number_fraction = 0.0;
    double max_outgoing_cfl = 0.0;
    double max_drift_speed = 0.0;
    double cfl_dt = 1.0e300;
    double pos_center_r = 0.0, pos_center_z = 0.0;
    double neg_center_r = 0.0, neg_center_z = 0.0;
    double density_ratio_at_pos_center = 1.0;
    double mu_pos_at_pos_center = 0.0;
};

// The fluid state of one grid (cells i + nr*j) with its closure fields.
struct State {
    std::vector<double> ne, np, nn, rho, se, sp, sn;   // densities, charge, source rates
    std::vector<double> mu, nu, diff3;                 // closure fields (table models)
    std::vector<double> sigma, tau;                    // diagnostic conductivity
};

struct CoupledDiag {
    int substeps = 0;
    double full_conduction = 0.0, full_diffusion = 0.0, full_reaction = 0.0;
    double max_reaction_number = 0.0, max_dt_sigma = 0.0, max_diffusion_number = 0.0, max_residual = 0.0;
};

void validate_transport(rrea_gpu_fluid_config const& c, bool require_cfl);
double react(rrea_gpu_fluid_config const& c, std::size_t n, double dt, double* ne, double* np, double* nn, double* se,
             double* sp, double* sn, double* rho, double const* nu_cell, bool clear);
double max_reaction_frequency(rrea_gpu_fluid_config const& c, std::size_t n, double const* ne, double const* np,
                              double const* nn, double const* nu_cell);
void conductivity(rrea_gpu_fluid_config const& c, std::size_t n, double const* ne, double const* np, double const* nn,
                  double const* chi, double const* mu_cell, double* sigma, double* tau);
void charge_density(std::size_t n, double const* ne, double const* np, double const* nn, double* rho);
Coefficients evaluate(rrea_host::ClosureTable const& t, double en, int& status);
void closure_fields(rrea_host::ClosureTable const& t, Grid const& g, double scalar_chi, double const* er,
                    double const* ez, double const* chi, double const* ne, double const* src, double* mu, double* nu,
                    double* diff3, ClosureDiag& d);
void build_faces(rrea_gpu_fluid_config const& c, Grid const& g, double dt, double const* const dens[3],
                 double const* chi, double const* mu_cell, double const* diff3, double const* efr,
                 double const* efz, double* fr_out, double* fz_out, TransportDiag& out);
// dens = {positive ion, negative ion, electron}, updated in place.
void transport(rrea_gpu_fluid_config const& c, Grid const& g, double dt, double* const dens[3], double* rho,
               double const* chi, double const* mu_cell, double const* diff3, double const* efr, double const* efz,
               double* flux_r, double* flux_z, double* raw_r, double* raw_z, TransportDiag& out);

void coupled_step(rrea_gpu_fluid_config const& c, rrea_host::ClosureTable const* table, Grid const& g, double dt,
                  oracle::MaxwellField& f, std::vector<double> const& amb_er, std::vector<double> const& amb_ez,
                  std::vector<double> const& jr_kin, std::vector<double> const& jz_kin, State& st, double const* chi,
                  CoupledDiag& diag);

}  // namespace oracle_fluid
