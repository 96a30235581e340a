// A C++17 host of the C-ABI, shaped like the overlay's GB300 Apply body:
// the per-species SoA tiles live in host vectors (standing in for WarpX's
// particle tiles), the phases run through rrea_gpu_apply_*, and a non-OK
// status ends the program the way amrex::Abort ends the overlay.  It proves
// that include/rrea_gpu.h compiles as C++ and that the structure layouts the
// C++ compiler assigns are the ones the library and the ctypes binding use.
//
//   overlay_host layout
//       prints "<struct>.<field> <offset>" and "<struct> <size>" lines
//   overlay_host apply <transport_physics.json> <in.bin> <out.bin>
//       in.bin:  rrea_gpu_config (raw bytes), int64 step, double dt_s,
//                int64 n, the 13 FP64 tile columns, int64 ids, int32 cpu
//       out.bin: the tile after the electron phase (13 columns, ids), then
//                int64 count and the ordered secondaries
#include "rrea_gpu.h"

#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

static_assert(sizeof(rrea_gpu_config) == 136, "rrea_gpu_config layout");
static_assert(sizeof(rrea_gpu_secondary) == 112, "rrea_gpu_secondary layout");
static_assert(sizeof(rrea_gpu_tile) == 8 + 15 * sizeof(void*), "rrea_gpu_tile layout");
static_assert(offsetof(rrea_gpu_secondary, parent_index) == 16, "secondary parent_index");
static_assert(offsetof(rrea_gpu_secondary, x) == 40, "secondary payload");

namespace {

#define FIELD(S, F) std::printf("%s.%s %zu\n", #S, #F, offsetof(S, F))

void print_layout()
{
    std::printf("rrea_gpu_config %zu\n", sizeof(rrea_gpu_config));
    FIELD(rrea_gpu_config, r_lo); FIELD(rrea_gpu_config, r_hi); FIELD(rrea_gpu_config, z_lo);
    FIELD(rrea_gpu_config, z_hi); FIELD(rrea_gpu_config, nr); FIELD(rrea_gpu_config, nz);
    FIELD(rrea_gpu_config, periodic_z); FIELD(rrea_gpu_config, strict_transport_guards);
    FIELD(rrea_gpu_config, density_ratio); FIELD(rrea_gpu_config, low_energy_cutoff_eV);
    FIELD(rrea_gpu_config, photon_cutoff_eV); FIELD(rrea_gpu_config, max_optical_depth_per_substep);
    FIELD(rrea_gpu_config, max_subcycles); FIELD(rrea_gpu_config, max_gs_collisions_per_substep);
    FIELD(rrea_gpu_config, gs_total_collision_cap); FIELD(rrea_gpu_config, max_field_impulse_fraction);
    FIELD(rrea_gpu_config, field_impulse_floor_eV); FIELD(rrea_gpu_config, rng_seed);
    FIELD(rrea_gpu_config, debug_disable_hard_moller); FIELD(rrea_gpu_config, reserved0);
    std::printf("rrea_gpu_tile %zu\n", sizeof(rrea_gpu_tile));
    FIELD(rrea_gpu_tile, n); FIELD(rrea_gpu_tile, r); FIELD(rrea_gpu_tile, z); FIELD(rrea_gpu_tile, theta);
    FIELD(rrea_gpu_tile, ux); FIELD(rrea_gpu_tile, uy); FIELD(rrea_gpu_tile, uz); FIELD(rrea_gpu_tile, w);
    FIELD(rrea_gpu_tile, prev_r); FIELD(rrea_gpu_tile, prev_z); FIELD(rrea_gpu_tile, prev_theta);
    FIELD(rrea_gpu_tile, prev_ux); FIELD(rrea_gpu_tile, prev_uy); FIELD(rrea_gpu_tile, prev_uz);
    FIELD(rrea_gpu_tile, id); FIELD(rrea_gpu_tile, cpu);
    std::printf("rrea_gpu_secondary %zu\n", sizeof(rrea_gpu_secondary));
    FIELD(rrea_gpu_secondary, species); FIELD(rrea_gpu_secondary, process); FIELD(rrea_gpu_secondary, root_species);
    FIELD(rrea_gpu_secondary, pad); FIELD(rrea_gpu_secondary, parent_index); FIELD(rrea_gpu_secondary, root_key);
    FIELD(rrea_gpu_secondary, lineage); FIELD(rrea_gpu_secondary, x); FIELD(rrea_gpu_secondary, y);
    FIELD(rrea_gpu_secondary, z); FIELD(rrea_gpu_secondary, dir_x); FIELD(rrea_gpu_secondary, dir_y);
    FIELD(rrea_gpu_secondary, dir_z); FIELD(rrea_gpu_secondary, weight); FIELD(rrea_gpu_secondary, energy_eV);
    FIELD(rrea_gpu_secondary, birth_fraction);
    std::printf("rrea_gpu_seed_event %zu\n", sizeof(rrea_gpu_seed_event));
    FIELD(rrea_gpu_seed_event, macro_index); FIELD(rrea_gpu_seed_event, species_id);
    FIELD(rrea_gpu_seed_event, time_s); FIELD(rrea_gpu_seed_event, x_m); FIELD(rrea_gpu_seed_event, y_m);
    FIELD(rrea_gpu_seed_event, z_m); FIELD(rrea_gpu_seed_event, r_m); FIELD(rrea_gpu_seed_event, kinetic_energy_eV);
    FIELD(rrea_gpu_seed_event, ux); FIELD(rrea_gpu_seed_event, uy); FIELD(rrea_gpu_seed_event, uz);
    FIELD(rrea_gpu_seed_event, weight);
}

// The overlay's species tile: SoA columns as WarpX holds them.
struct HostTile {
    std::vector<double> col[13];
    std::vector<int64_t> id;
    std::vector<int32_t> cpu;

    rrea_gpu_tile view()
    {
        rrea_gpu_tile t{};
        t.n = static_cast<int64_t>(id.size());
        double** dst[13] = {&t.r, &t.z, &t.theta, &t.ux, &t.uy, &t.uz, &t.w,
                            &t.prev_r, &t.prev_z, &t.prev_theta, &t.prev_ux, &t.prev_uy, &t.prev_uz};
        for (int f = 0; f < 13; ++f) *dst[f] = col[f].data();
        t.id = id.data();
        t.cpu = cpu.data();
        return t;
    }
};

[[noreturn]] void abort_step(rrea_gpu_ctx* ctx, rrea_gpu_status s, char const* where)
{
    char msg[1024] = {0};
    rrea_gpu_last_error(ctx, msg, sizeof(msg));
    std::fprintf(stderr, "%s failed with status %d: %s\n", where, static_cast<int>(s), msg);
    std::exit(2);
}

template <class T>
void read_into(std::ifstream& in, T* p, size_t n)
{
    in.read(reinterpret_cast<char*>(p), static_cast<std::streamsize>(n * sizeof(T)));
    if (!in) {
        std::fprintf(stderr, "short input\n");
        std::exit(3);
    }
}

int apply(char const* tables, char const* in_path, char const* out_path)
{
    std::ifstream in(in_path, std::ios::binary);
    rrea_gpu_config cfg;
    int64_t step = 0, n = 0;
    double dt = 0.0;
    read_into(in, &cfg, 1);
    read_into(in, &step, 1);
    read_into(in, &dt, 1);
    read_into(in, &n, 1);
    HostTile tile;
    for (auto& c : tile.col) {
        c.resize(static_cast<size_t>(n));
        read_into(in, c.data(), c.size());
    }
    tile.id.resize(static_cast<size_t>(n));
    tile.cpu.resize(static_cast<size_t>(n));
    read_into(in, tile.id.data(), tile.id.size());
    read_into(in, tile.cpu.data(), tile.cpu.size());

    rrea_gpu_ctx* ctx = nullptr;
    rrea_gpu_status s = rrea_gpu_create(&cfg, n > 0 ? n : 1, &ctx);
    if (s != RREA_GPU_OK) abort_step(nullptr, s, "rrea_gpu_create");
    if ((s = rrea_gpu_load_tables(ctx, tables)) != RREA_GPU_OK) abort_step(ctx, s, "rrea_gpu_load_tables");
    // zero scattered field over a uniform ambient E_z (the first step of a run)
    size_t const ner = static_cast<size_t>(cfg.nr + 1) * cfg.nz, nez = static_cast<size_t>(cfg.nr) * (cfg.nz + 1);
    std::vector<double> er(ner, 0.0), ez(nez, 0.0), bt(static_cast<size_t>(cfg.nr + 1) * (cfg.nz + 1), 0.0);
    std::vector<double> amb_er(ner, 0.0), amb_ez(nez, -5.0e5);
    s = rrea_gpu_set_field(ctx, er.data(), ez.data(), bt.data(), amb_er.data(), amb_ez.data());
    if (s != RREA_GPU_OK) abort_step(ctx, s, "rrea_gpu_set_field");

    std::vector<rrea_gpu_secondary> secondaries(static_cast<size_t>(2 * n + 4096));
    int64_t n_sec = 0;
    rrea_gpu_tile view = tile.view();
    s = rrea_gpu_apply_electrons(ctx, &view, static_cast<int32_t>(step), 0.0, dt, secondaries.data(),
                                 static_cast<int64_t>(secondaries.size()), &n_sec);
    if (s != RREA_GPU_OK) abort_step(ctx, s, "rrea_gpu_apply_electrons");

    std::ofstream out(out_path, std::ios::binary);
    for (auto const& c : tile.col) out.write(reinterpret_cast<char const*>(c.data()), c.size() * sizeof(double));
    out.write(reinterpret_cast<char const*>(tile.id.data()), tile.id.size() * sizeof(int64_t));
    out.write(reinterpret_cast<char const*>(&n_sec), sizeof(n_sec));
    out.write(reinterpret_cast<char const*>(secondaries.data()), n_sec * sizeof(rrea_gpu_secondary));
    rrea_gpu_destroy(ctx);
    return out ? 0 : 4;
}

}  // namespace

int main(int argc, char** argv)
{
    if (argc >= 2 && std::string(argv[1]) == "layout") {
        print_layout();
        return 0;
    }
    if (argc == 5 && std::string(argv[1]) == "apply") return apply(argv[2], argv[3], argv[4]);
    std::fprintf(stderr, "usage: overlay_host layout | apply <tables.json> <in.bin> <out.bin>\n");
    return 1;
}
