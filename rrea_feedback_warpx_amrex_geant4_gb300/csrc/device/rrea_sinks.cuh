// Per-step output sinks shared by the species kernels: the order-1 cell
// deposit into the five FP64 cell-source grids, the secondary append buffer
// and the first-failure status word.
#pragma once

#include "rrea_device_path.cuh"
#include "rrea_electron_args.cuh"

namespace rrea_dev {

// Order-1 cell deposit (S/RreaEventAccumulator.cpp:386-502, field ids of
// :129-164) for the uniform RZ grid with r_lo on the axis.  One source feeds
// up to four fields at the same point, so its stencil (containing cell,
// order-1 weights, axis fold) is built once and applied to each value.
struct CellStencil {
    bool valid;
    int i0, j0;  // lower-left stencil cell before folding
    int i[2], j[2];
    bool use_i[2], use_j[2];
    double wr[2], wz[2];
};

// Cells of the order-1 stencil with lower-left cell (i0, j0): the radial
// fold onto the axis cell and the periodic z wrap, or a dropped row/column.
__device__ __forceinline__ void stencil_cells(StepConstants const& C, int i0, int j0, int i[2], int j[2], bool use_i[2],
                                              bool use_j[2])
{
    rrea_gpu_config const& cfg = C.cfg;
    int const nr = cfg.nr, nz = cfg.nz;
#pragma unroll
    for (int a = 0; a < 2; ++a) {
        int jj = j0 + a;
        use_j[a] = true;
        if (jj < 0 || jj > nz - 1) {
            if (cfg.periodic_z) jj = ((jj % nz) + nz) % nz;
            else use_j[a] = false;
        }
        j[a] = jj;
        int ii = i0 + a;
        use_i[a] = true;
        if (ii < 0 || ii > nr - 1) {
            if (ii == -1 && eq0(cfg.r_lo)) ii = 0;
            else use_i[a] = false;
        }
        i[a] = ii;
    }
}

__device__ __forceinline__ CellStencil make_stencil(StepConstants const& C, double r, double z)
{
    CellStencil st;
    rrea_gpu_config const& cfg = C.cfg;
    int const nr = cfg.nr, nz = cfg.nz;
    double zz = z;
    if (cfg.periodic_z) {
        double const len = cfg.z_hi - cfg.z_lo;
        double s = fmod(zz - cfg.z_lo, len);
        if (lt0(s)) s += len;
        zz = cfg.z_lo + s;
    }
    double const fr = quot(r - cfg.r_lo, C.div_dr);
    double const fz = quot(zz - cfg.z_lo, C.div_dz);
    int const ic = static_cast<int>(floor(fr));
    int const jc = static_cast<int>(floor(fz));
    st.valid = !(ic < 0 || ic >= nr || jc < 0 || jc >= nz);
    if (!st.valid) return st;
    double const rc = fr + 0.0 - 0.5;
    int const i0 = static_cast<int>(floor(rc));
    st.wr[1] = rc - i0;
    st.wr[0] = 1.0 - st.wr[1];
    double const zc = fz + 0.0 - 0.5;
    int const j0 = static_cast<int>(floor(zc));
    st.wz[1] = zc - j0;
    st.wz[0] = 1.0 - st.wz[1];
    st.i0 = i0;
    st.j0 = j0;
    stencil_cells(C, i0, j0, st.i, st.j, st.use_i, st.use_j);
    return st;
}

__device__ __forceinline__ void stencil_add(StepConstants const& C, double* __restrict__ cells, CellStencil const& st,
                                            int field, double value)
{
    if (!st.valid || !finite_bits(value) || eq0(value)) return;
    int const nr = C.cfg.nr;
    double* grid = cells + static_cast<size_t>(field) * nr * C.cfg.nz;
#pragma unroll
    for (int a = 0; a < 2; ++a) {
        double const wz = st.wz[a];
        if (eq0(wz) || !st.use_j[a]) continue;
#pragma unroll
        for (int b = 0; b < 2; ++b) {
            double const v = value * st.wr[b] * wz;
            if (eq0(v) || !st.use_i[b] || !finite_bits(v)) continue;
            atomicAdd(grid + st.i[b] + static_cast<size_t>(nr) * st.j[a], v);
        }
    }
}

// O/RreaCouplingSources.cpp:435-512
__device__ __forceinline__ void deposit_source(StepConstants const& C, double* __restrict__ cells, int kind,
                                               double r, double z, double w, double sec_e, double loss)
{
    if (le0(w) || !cells) return;   // no cell sources in ensemble mode
    CellStencil const st = make_stencil(C, r, z);
    if (!st.valid) return;
    if (kind == 0) {  // AccumulateIonizationEvent
        stencil_add(C, cells, st, 1, w);
        if (sec_e < C.cfg.low_energy_cutoff_eV) stencil_add(C, cells, st, 0, w);
        stencil_add(C, cells, st, 3, w);
        stencil_add(C, cells, st, 4, max0(w) * max0(loss));
    } else if (kind == 1) {  // AccumulateLowEnergyElectron
        stencil_add(C, cells, st, 0, w);
        stencil_add(C, cells, st, 3, w);
        stencil_add(C, cells, st, 4, max0(w) * max0(fmax(loss, 0.0)));
    } else {  // AccumulatePositiveIonSourceOnly
        stencil_add(C, cells, st, 1, w);
        stencil_add(C, cells, st, 3, w);
        stencil_add(C, cells, st, 4, max0(w) * max0(loss));
    }
}

// Per-particle accumulator of the ion-pair sources of the continuous drag
// (AccumulateIonizationEvent with a fixed secondary energy and loss = W_air).
// The substeps of one particle almost always deposit into the same four
// cells, so their order-1 weights are summed per cell and written with one
// atomic per cell and field when the stencil moves or the particle is done,
// instead of sixteen atomics per substep into a few hot cells.  Only the
// order of the additions differs from depositing each source at once (the
// atomics already make that order arbitrary).  The running sums sit in a
// per-thread shared-memory slot: the transport state around them lives in
// local memory that misses L1, and the slot is touched every substep.  The
// stencil is named by its lower-left cell (i0, j0) packed in one word; the
// folded cells and their use flags follow from it (stencil_cells).
struct IonPairSlot {
    long long key;  // (j0 << 32) | (i0 & 0xffffffff); kIonPairEmpty = none
    double acc[4];  // sum of w * wr[b] * wz[a] at acc[2 * a + b]
};
constexpr long long kIonPairEmpty = static_cast<long long>(0x8000000000000000ULL);


struct IonPairCache {
    IonPairSlot* slot;
    double sec_e, loss;

    __device__ __forceinline__ void init(IonPairSlot* s, double sec, double loss_per_pair)
    {
        slot = s;
        slot->key = kIonPairEmpty;
        sec_e = sec;
        loss = loss_per_pair;
    }
    __device__ __forceinline__ void flush(StepConstants const& C, double* __restrict__ cells)
    {
        long long const key = slot->key;
        if (key == kIonPairEmpty) return;
        slot->key = kIonPairEmpty;
        int i[2], j[2];
        bool use_i[2], use_j[2];
        stencil_cells(C, static_cast<int>(static_cast<unsigned int>(key & 0xffffffffLL)), static_cast<int>(key >> 32), i,
                      j, use_i, use_j);
        int const nr = C.cfg.nr;
        size_t const plane = static_cast<size_t>(nr) * C.cfg.nz;
        bool const low = sec_e < C.cfg.low_energy_cutoff_eV;
#pragma unroll
        for (int a = 0; a < 2; ++a) {
            if (!use_j[a]) continue;
#pragma unroll
            for (int b = 0; b < 2; ++b) {
                double const v = slot->acc[2 * a + b];
                if (eq0(v) || !use_i[b] || !finite_bits(v)) continue;
                double* cell = cells + i[b] + static_cast<size_t>(nr) * j[a];
                atomicAdd(cell + plane * 1, v);
                if (low) atomicAdd(cell, v);
                atomicAdd(cell + plane * 3, v);
                double const l = v * max0(loss);
                if (ne0(l) && finite_bits(l)) atomicAdd(cell + plane * 4, l);
            }
        }
    }
    // deposit_source(C, cells, 0, r, z, w, sec_e, loss) for w > 0
    __device__ __forceinline__ void add(StepConstants const& C, double* __restrict__ cells, double r, double z, double w)
    {
        if (!cells) return;
        CellStencil const st = make_stencil(C, r, z);
        if (!st.valid) return;
        long long const key = (static_cast<long long>(st.j0) << 32) | static_cast<unsigned int>(st.i0);
        if (slot->key != key) {
            flush(C, cells);
            slot->key = key;
#pragma unroll
            for (int q = 0; q < 4; ++q) slot->acc[q] = 0.0;
        }
        double const wv = max0(w);
#pragma unroll
        for (int a = 0; a < 2; ++a) {
            double const wz = st.wz[a];
            if (eq0(wz) || !st.use_j[a]) continue;
#pragma unroll
            for (int b = 0; b < 2; ++b) {
                double const v = wv * st.wr[b] * wz;
                if (eq0(v) || !st.use_i[b] || !finite_bits(v)) continue;
                slot->acc[2 * a + b] += v;
            }
        }
    }
};

// Conservation closure of one interaction group,
// RreaValidateSecondaryGroupConservation (O/RreaParticleInteraction.H:1099-1251):
// rest-mass-inclusive energy and charge in (the parent before the event and
// the neutral target electron of every ionization or positive-ion source)
// against out (the surviving parent, the secondaries, the local
// recoil/binding/sub-cutoff energy, the ions and low-energy electrons of the
// sources), within 64 eps of the larger side.  The ion pairs of a local
// deposit (ionization sources below the cutoff) add the same rest energy and
// charge to both sides and only widen the tolerance, as in the reference.
struct GroupClosure {
    double in_e, out_e, in_q, out_q, thru_q;
    bool finite;

    __device__ __forceinline__ void begin(double q_parent, double rest_parent, double w, double e_before, double e_after,
                                          bool survives)
    {
        finite = finite_bits(w) && finite_bits(e_before) && finite_bits(e_after) && gt0(w) && ge0(e_before) && ge0(e_after);
        in_q = q_parent * w;
        out_q = survives ? in_q : 0.0;
        in_e = w * (e_before + rest_parent);
        out_e = survives ? w * (e_after + rest_parent) : 0.0;
        thru_q = fabs(in_q) + fabs(out_q);
    }
    __device__ __forceinline__ void secondary(double q, double rest, double w, double e)
    {
        finite = finite && finite_bits(w) && finite_bits(e) && gt0(w) && ge0(e);
        out_q += q * w;
        thru_q += fabs(q * w);
        out_e += w * (e + rest);
    }
    // AccumulateIonizationEvent with event weight w and secondary energy sec_e
    __device__ __forceinline__ void ionization(double w, double sec_e, double cutoff)
    {
        finite = finite && finite_bits(w) && finite_bits(sec_e) && gt0(w);
        in_e += w * kMeC2;
        out_q += w;
        thru_q += w;
        if (sec_e < cutoff) {
            out_q -= w;
            thru_q += w;
            out_e += w * kMeC2;
        }
    }
    // AccumulatePositiveIonSourceOnly with event weight w
    __device__ __forceinline__ void positive_ion(double w)
    {
        finite = finite && finite_bits(w) && gt0(w);
        in_e += w * kMeC2;
        out_q += w;
        thru_q += w;
    }
    // AccumulateLowEnergyElectron with event weight w
    __device__ __forceinline__ void low_energy_electron(double w)
    {
        finite = finite && finite_bits(w) && gt0(w);
        out_q -= w;
        thru_q += w;
        out_e += w * kMeC2;
    }
    // deposit_local_energy_as_ion_pairs: the local energy and its pairs
    __device__ __forceinline__ void local(double w, double e, double w_air, double cutoff)
    {
        if (le0(w) || le0(e)) return;
        out_e += w * e;
        finite = finite && finite_bits(e);
        double const pw = w * e / fmax(w_air, 1.0);
        if (gt0(pw)) ionization(pw, 0.0, cutoff);
    }
    __device__ __forceinline__ bool valid(double cutoff) const
    {
        if (!(finite && finite_bits(cutoff) && gt0(cutoff) && finite_bits(in_e) && finite_bits(out_e) && finite_bits(in_q)
              && finite_bits(out_q))) {
            return false;
        }
        double const tol_q = 64.0 * kEps * fmax(1.0, thru_q);
        double const tol_e = 64.0 * kEps * fmax(1.0, fmax(fabs(in_e), fabs(out_e)));
        return fabs(out_q - in_q) <= tol_q && fabs(out_e - in_e) <= tol_e;
    }
};

__device__ __forceinline__ void record_failure(ElectronArgs const& A, int code, int64_t ip)
{
    if (atomicCAS(A.status, 0, code) == 0) {
        *A.fail_index = static_cast<long long>(A.index_base + ip);
    }
}

// TransportSideEffects::AddSecondary (O/RreaTransportLog.H:437-447): the
// record carries the parent's RNG key and its per-parent lineage counter.
__device__ __forceinline__ void append_secondary(ElectronArgs const& A, int64_t ip, uint64_t key, double weight,
                                                 uint32_t& lineage, int species, int process, double x, double y,
                                                 double z, double sx, double sy, double sz, double e, double birth,
                                                 Err& err, int root_species = 0)
{
    unsigned long long const slot = atomicAdd(A.sec_count, 1ULL);
    if (slot < static_cast<unsigned long long>(A.sec_capacity)) {
        rrea_gpu_secondary s;
        s.species = species;
        s.process = process;
        s.root_species = root_species;
        s.pad = 0;
        s.parent_index = A.index_base + ip;
        s.root_key = key;
        s.lineage = lineage;
        s.x = x; s.y = y; s.z = z;
        s.dir_x = sx; s.dir_y = sy; s.dir_z = sz;
        s.weight = weight;
        s.energy_eV = e;
        s.birth_fraction = birth;
        A.sec[slot] = s;
    } else {
        err.set(RREA_GPU_ERR_CAPACITY);
    }
    ++lineage;
}

}  // namespace rrea_dev
