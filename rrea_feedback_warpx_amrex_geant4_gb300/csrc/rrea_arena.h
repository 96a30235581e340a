// Layout of the schema-6 table arena: one flat FP64 array (uploaded once to
// HBM, read through L2) plus this POD index of element offsets into it.  The
// index is plain data so the same struct is filled by the host loader and
// read by device code from __constant__ memory.
//
// The interpolation denominators (node spacings, the CDF node ratios and
// nodes the GS inversion divides by) are stored as reciprocals, so a query
// multiplies instead of running an FP64 division sequence; the quotient is
// then within 1.5 ulp of the reference's.
//
// Every logarithm the reference takes of a TABLE NODE at query time
// (node energies, node values, GS one-minus-cos nodes, CDF u-node ratios) is
// precomputed here once with the host libm.  The reference computes exactly
// these logs on the host at query time (native_amrex_rrea/src/
// RreaInteractionTables.cpp:1615-1629, 818-819, 844-847, 874, 885), so the
// device reads bit-identical operands and only query-dependent logs are
// evaluated on the GPU.
#pragma once

#include <stdint.h>

#define RREA_ARENA_MAX_PIECES 4

// The arena opens with the table of the table-driven logarithm
// (device/rrea_fastmath.cuh): for j = 0..256, F = 1 + j/256, three doubles
// {RN(1/F), RN(log F), RN(log F - RN(log F))}.
#define RREA_ARENA_LOG_TABLE 0
#define RREA_ARENA_LOG_TABLE_ROWS 257
// Then the table of the table-driven exponential: for j = 0..127, two
// doubles {RN(2^(j/128)), RN(2^(j/128) - RN(2^(j/128)))}, at the next
// 32-byte boundary.
#define RREA_ARENA_EXP_TABLE 772
#define RREA_ARENA_EXP_TABLE_ROWS 128

enum RreaInterpMode {
    RREA_INTERP_LOGLOG = 0,
    RREA_INTERP_LOGLOG_ZERO_THRESHOLD = 1,
    RREA_INTERP_LOGX_LINEAR = 2,
    RREA_INTERP_LINEAR = 3,
};

// Hot 1-D tables, in the reference's RREA_HOT_TABLES order
// (native_amrex_rrea/include/rrea/RreaInteractionTables.H:92-114).
enum RreaHotTable {
    RREA_T_E_COLLISION = 0,
    RREA_T_E_SOFT_RAD = 1,
    RREA_T_E_HARD_MOLLER = 2,
    RREA_T_E_TRACKED_BREMS = 3,
    RREA_T_E_ELASTIC_TRANSPORT = 4,
    RREA_T_P_COLLISION = 5,
    RREA_T_P_SOFT_RAD = 6,
    RREA_T_P_HARD_BHABHA = 7,
    RREA_T_P_TRACKED_BREMS = 8,
    RREA_T_P_ELASTIC_TRANSPORT = 9,
    RREA_T_P_ANNIHILATION = 10,
    RREA_T_PH_COMPTON = 11,
    RREA_T_PH_PHOTOELECTRIC = 12,
    RREA_T_PH_PAIR_NUCLEAR = 13,
    RREA_T_PH_PAIR_TRIPLET = 14,
    RREA_T_COUNT = 15,
};

enum RreaCondCdf {
    RREA_C_MOLLER = 0,
    RREA_C_BHABHA = 1,
    RREA_C_BREMS_E = 2,
    RREA_C_BREMS_P = 3,
    RREA_C_COUNT = 4,
};

typedef struct {
    int32_t n;      // rows
    int32_t mode;   // RreaInterpMode
    int64_t x;      // energy nodes
    int64_t lx;     // log(energy nodes)
    int64_t y;      // values
    int64_t ly;     // log(values), 0 where value <= 0
    int64_t ix;     // 1 / (x[i] - x[i-1]) at i >= 1 (0 at i = 0)
    int64_t ilx;    // 1 / (lx[i] - lx[i-1]) at i >= 1 (0 at i = 0)
} RreaTable1DIndex;

typedef struct {
    int32_t ng;        // primary-energy groups
    int32_t total;     // total nodes over all groups
    int64_t primary;   // ng primary energies
    int64_t lprimary;  // ng log primary energies
    int64_t start;     // ng+1 node offsets (stored as doubles, exact integers)
    int64_t u;         // cdf nodes
    int64_t v;         // sampled values
    int64_t mean;      // ng per-group means (RreaInteractionTables.cpp:1075-1085 quadrature)
    int64_t lmean;     // ng logs of the group means (0 where the mean is not positive)
} RreaCondCdfIndex;

typedef struct {
    int32_t n;
    int32_t pad;
    int64_t x;     // energies
    int64_t lx;    // log energies
    int64_t mfp;   // elastic collision MFP at STP [m]
    int64_t eta;   // screening eta
    int64_t ilx;   // 1 / (lx[i] - lx[i-1]) at i >= 1
} RreaElasticIndex;

typedef struct {
    int32_t ne, np, nu, pad;
    int64_t e, le;      // energy grid and logs
    int64_t p, lp;      // path grid and logs
    int64_t u;          // shared cdf nodes
    int64_t lur;        // log(u[i+1]/u[i]) for i in [0, nu-1)
    int64_t omc;        // one_minus_cos, (ie*np+ip)*nu+iu
    int64_t lomc;       // log(one_minus_cos)
    int64_t ile, ilp;   // 1 / (le[i] - le[i-1]), 1 / (lp[i] - lp[i-1]) at i >= 1
    int64_t ilur;       // 1 / lur[i] (0 where lur[i] = 0)
    int64_t iu;         // 1 / u[i] (0 where u[i] = 0)
} RreaAngleIndex;

// Photoelectric subshell CDF (S/RreaInteractionTables.cpp:893-987): groups
// of (cdf_u, binding energy) rows per primary energy; duplicated edge
// energies appear as two consecutive groups.
typedef struct {
    int32_t ng;
    int32_t total;
    int64_t primary;   // ng
    int64_t start;     // ng+1 row offsets (exact integers)
    int64_t u;         // rows: cumulative subshell probability
    int64_t binding;   // rows: binding energy [eV]
} RreaPhotoelectricIndex;

// Correlated pair final-state bank, training split only
// (S/RreaInteractionTables.cpp:1187-1370): blocks sorted by primary energy,
// each a run of 16-double records
//   [lepton_count, pdg0, pdg1, pdg2, frac0, frac1, frac2,
//    dx0, dy0, dz0, dx1, dy1, dz1, dx2, dy2, dz2].
#define RREA_PAIR_RECORD_DOUBLES 16
typedef struct {
    int32_t nb;
    int32_t pad;
    int64_t primary;   // nb block energies
    int64_t lprimary;  // nb logs
    int64_t start;     // nb+1 record offsets (exact integers)
    int64_t records;   // records * RREA_PAIR_RECORD_DOUBLES
} RreaPairBankIndex;

typedef struct {
    RreaTable1DIndex hot[RREA_T_COUNT];
    RreaCondCdfIndex cdf[RREA_C_COUNT];
    RreaElasticIndex elastic[2];       // 0 electron, 1 positron
    RreaAngleIndex gs[2];              // option4 GS, E <= transition
    RreaAngleIndex wentzel[2];         // WentzelVI, E > transition
    int64_t hard_moller_mean_secondary;  // on the hard-Moller rate grid
    RreaPhotoelectricIndex pe;
    RreaPairBankIndex pair[2];         // 0 nuclear, 1 triplet
    int64_t total_doubles;
    double charged_min_eV, charged_max_eV;
    double photon_min_eV, photon_max_eV;
    double hard_moller_threshold_eV;
    double brems_absolute_cutoff_eV;
    double reference_density_kg_m3;
    double gs_few_collision_threshold;
    double gs_isotropic_above_n;
    double gs_wentzel_transition_eV;
    double w_air_eV_per_pair;
    // 1 when all five electron (six positron, four photon) coefficient tables
    // share one bit-identical energy grid, so one bracket search serves all.
    int32_t electron_grid_shared;
    int32_t positron_grid_shared;
    int32_t photon_grid_shared;
    int32_t pad0;
} RreaArenaIndex;
