// Pathwise adjoint of the charged push with respect to an axial field
// profile E_z(z): the gradient pattern built on the kinetic step.
//
// The differentiated model is the continuous part of the charged substep
// (O/RreaChargedInterleave.H:100-138 and :218-292 with the two-node field
// work of O/RreaPathFieldWork.H:57-150), with every discrete outcome frozen:
//
//   chord     L = v(K) h along d from z (h = dt / substeps), z1 = z + L d_z
//   work      W = q d_z L <E>,  <E> = (E(z + a L d_z) + E(z + b L d_z)) / 2
//             (two-point Gauss-Legendre, a, b = 1/2 -+ 1/(2 sqrt 3))
//   kick      d <- (u(K) d + s <E> z^) / |.|,  K <- K + W / 2,
//             s = q (c^2 / m c^2) h / 2  (the half kick without B)
//   drag      K <- K - rho S(K) L, S the tables' collision plus soft
//             radiative stopping power (log-log, as the transport reads them)
//   kick      as above, with the same <E> and W
//   scatter   d <- R d, R a rotation drawn once from the counter RNG of
//             (seed, particle, step, substep): the frozen elastic deflection
//
// E(z) interpolates the profile nodes linearly (clamped outside).  A
// particle whose drag would take it below the cutoff stops there (a frozen
// topology: it stops at the same substep in the reverse pass).  The loss is
// the smoothed runaway count plus the smoothed net charge crossing the
// plane z_p (the time integral of J_z through the plane, by charge
// conservation):
//   J = sum_i w_i [ sig((K_i(T) - K_th) / tau_K)
//                   - lambda (sig((z_i(T) - z_p) / tau_z) - sig((z_i(0) - z_p) / tau_z)) ]
// with sig the logistic function (the electron charge is -e; lambda counts
// it in elementary charges).
//
// Forward: one thread per particle, the state checkpointed every C steps.
// Reverse: per checkpoint segment, last to first, the forward is recomputed
// from the checkpoint onto a tape of substep inputs (with each substep's
// stopping power, its derivative and the frozen rotation, so the adjoint
// evaluates neither tables nor the RNG again), then the adjoint runs back
// through it; the node gradient is accumulated per block in shared
// memory and added to the output once per block and node.
#include "rrea_kernels.h"

#include <cuda_runtime.h>

namespace rrea_dev {
namespace adj {

constexpr double kGlA = 0.21132486540518711775;   // 1/2 - 1/(2 sqrt 3)
constexpr double kGlB = 0.78867513459481288225;   // 1/2 + 1/(2 sqrt 3)
constexpr int kMaxNodes = 2048;

struct Params {
    int64_t n;
    int n_nodes;
    double z0, dz_node;     // node k at z0 + k dz_node
    int steps, substeps, ckpt_every;
    double h;               // substep duration
    double rho;             // density ratio of the stopping power
    double cutoff;          // eV
    double scatter_rms;     // rad
    double k_th, tau_k, z_p, tau_z, lambda;
    uint64_t seed;
    RreaTable1DIndex col, soft;
    // each particle's end: (global substep << 1) | kind (0 stopped in the
    // drag, 1 below the cutoff after the second kick), -1 for none.  A
    // recording forward writes it; a replaying one (and the reverse pass)
    // ends every particle exactly there, so a perturbed profile keeps the
    // topology of the recorded run.
    int32_t* ends;
    int replay;
};

struct State {
    double z, dx, dy, dz, k;
    int alive;
};

__device__ __forceinline__ double sig(double x) { return 1.0 / (1.0 + exp(-x)); }
__device__ __forceinline__ double dsig(double x)
{
    double const s = sig(x);
    return s * (1.0 - s);
}

// E(z) and dE/dz of the profile; node weights for the reverse pass.
__device__ __forceinline__ double field(Params const& p, const double* __restrict__ e, double z, double& slope, int& k0,
                                       double& f)
{
    double const x = (z - p.z0) / p.dz_node;
    if (!(x > 0.0)) {
        slope = 0.0;
        k0 = 0;
        f = 0.0;
        return e[0];
    }
    if (!(x < static_cast<double>(p.n_nodes - 1))) {
        slope = 0.0;
        k0 = p.n_nodes - 2;
        f = 1.0;
        return e[p.n_nodes - 1];
    }
    k0 = static_cast<int>(floor(x));
    f = x - static_cast<double>(k0);
    slope = (e[k0 + 1] - e[k0]) / p.dz_node;
    return (1.0 - f) * e[k0] + f * e[k0 + 1];
}

// rho S(K) and its K-derivative from the two log-log hot tables.
__device__ __forceinline__ double drag_power(Params const& p, const double* __restrict__ arena, double k, double& dk)
{
    double total = 0.0;
    dk = 0.0;
    for (RreaTable1DIndex const* h : {&p.col, &p.soft}) {
        Err err;
        Bracket b;
        if (!bracket_hot(arena, *h, k, b, err)) continue;
        double const v = eval_hot(arena, *h, b, err);
        total += v;
        if (b.kind != 3) continue;   // constant beyond the grid (a node itself has measure zero)
        // d/dK in the table's mode: log-log between positive nodes, linear
        // in the log-energy fraction otherwise (the zero-threshold rule)
        const double* y = arena + h->y;
        double const ylo = __ldg(y + b.hi - 1), yhi = __ldg(y + b.hi);
        double const ilx = __ldg(arena + h->ilx + b.hi);
        if (h->mode == RREA_INTERP_LOGLOG || (ylo > 0.0 && yhi > 0.0)) {
            const double* ly = arena + h->ly;
            dk += v * (__ldg(ly + b.hi) - __ldg(ly + b.hi - 1)) * ilx / k;
        } else {
            dk += (yhi - ylo) * ilx / k;
        }
    }
    dk *= p.rho;
    return p.rho * total;
}

__device__ __forceinline__ double speed(double k) { double const g = 1.0 + k * kInvMeC2; return kC * sqrt(1.0 - 1.0 / (g * g)); }
__device__ __forceinline__ double dspeed(double k)
{
    double const g = 1.0 + k * kInvMeC2;
    double const beta = sqrt(1.0 - 1.0 / (g * g));
    return kC / (g * g * g * beta) * kInvMeC2;
}
__device__ __forceinline__ double umag(double k) { double const g = 1.0 + k * kInvMeC2; return kC * sqrt(g * g - 1.0); }
__device__ __forceinline__ double dumag(double k)
{
    double const g = 1.0 + k * kInvMeC2;
    return kC * g / sqrt(g * g - 1.0) * kInvMeC2;
}

// The frozen rotation of (particle, step, substep): axis uniform on the
// sphere, angle Gaussian with the configured rms.
__device__ __forceinline__ void rotation(Params const& p, uint64_t id, int step, int sub, double n[3], double& c,
                                         double& s)
{
    uint64_t const key = splitmix64(p.seed ^ splitmix64(id * 0x9e3779b97f4a7c15ULL + 0x5eed))
        ^ (static_cast<uint64_t>(step) << 20) ^ static_cast<uint64_t>(sub);
    auto uni = [&](int k) {
        return (static_cast<double>(splitmix64(key * 4 + k) >> 11) + 0.5) * 0x1.0p-53;
    };
    double const mu = 2.0 * uni(0) - 1.0, phi = 6.283185307179586 * uni(1);
    double const st = sqrt(fmax(0.0, 1.0 - mu * mu));
    n[0] = st * cos(phi);
    n[1] = st * sin(phi);
    n[2] = mu;
    double const g = sqrt(-2.0 * log(uni(2))) * cos(6.283185307179586 * uni(3));
    double const th = p.scatter_rms * g;
    c = cos(th);
    s = sin(th);
}

// Rodrigues: v cos + (n x v) sin + n (n.v) (1 - cos); its transpose is the
// same with -sin.
__device__ __forceinline__ void rotate(double const n[3], double c, double s, double v[3])
{
    double const nv = n[0] * v[0] + n[1] * v[1] + n[2] * v[2];
    double const cx = n[1] * v[2] - n[2] * v[1], cy = n[2] * v[0] - n[0] * v[2], cz = n[0] * v[1] - n[1] * v[0];
    double const r[3] = {v[0] * c + cx * s + n[0] * nv * (1.0 - c), v[1] * c + cy * s + n[1] * nv * (1.0 - c),
                         v[2] * c + cz * s + n[2] * nv * (1.0 - c)};
    v[0] = r[0];
    v[1] = r[1];
    v[2] = r[2];
}

__device__ __forceinline__ int32_t end_code(Params const& p, int step, int sub, int kind)
{
    return ((step * p.substeps + sub) << 1) | kind;
}

// Values of one substep that the reverse pass reads back instead of
// evaluating them again: the stopping power and its K-derivative at K1, and
// the frozen rotation (axis, cos, sin).  kAux columns of n per tape entry.
constexpr int kAux = 7;

// One substep forward; `end` is the particle's end record (see Params).
// With `aux` (column stride n, particle i) the drag and rotation go to the
// tape beside the substep's input state.
__device__ __forceinline__ void substep(Params const& p, const double* __restrict__ e,
                                        const double* __restrict__ arena, uint64_t id, int step, int sub, State& st,
                                        int32_t& end, double* __restrict__ aux = nullptr, int64_t i = 0)
{
    if (!st.alive) return;
    double const q = -1.0;
    double const L = speed(st.k) * p.h;
    double sl;
    int k0;
    double f;
    double const e1 = field(p, e, st.z + kGlA * L * st.dz, sl, k0, f);
    double const e2 = field(p, e, st.z + kGlB * L * st.dz, sl, k0, f);
    double const eavg = 0.5 * (e1 + e2);
    double const w = q * st.dz * L * eavg;
    double const s = q * (kC * kC * kInvMeC2) * 0.5 * p.h;
    // kick 1
    double u = umag(st.k);
    double m[3] = {u * st.dx, u * st.dy, u * st.dz + s * eavg};
    double nm = sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]);
    double d[3] = {m[0] / nm, m[1] / nm, m[2] / nm};
    double k1 = st.k + 0.5 * w;
    double const z1 = st.z + L * st.dz;
    // drag
    double ds;
    double const sp = drag_power(p, arena, k1, ds);
    double const loss = sp * L;
    if (aux) {
        aux[i] = sp;
        aux[p.n + i] = ds;
    }
    bool const stop = p.replay ? end == end_code(p, step, sub, 0) : !(k1 - loss > p.cutoff);
    if (stop) {
        st.z = z1;
        st.k = p.cutoff;
        st.alive = 0;
        if (!p.replay) end = end_code(p, step, sub, 0);
        return;
    }
    double const k2 = k1 - loss;
    // kick 2
    u = umag(k2);
    m[0] = u * d[0];
    m[1] = u * d[1];
    m[2] = u * d[2] + s * eavg;
    nm = sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]);
    d[0] = m[0] / nm;
    d[1] = m[1] / nm;
    d[2] = m[2] / nm;
    double const k3 = k2 + 0.5 * w;
    double n[3], c, sn;
    rotation(p, id, step, sub, n, c, sn);
    if (aux) {
        aux[2 * p.n + i] = n[0];
        aux[3 * p.n + i] = n[1];
        aux[4 * p.n + i] = n[2];
        aux[5 * p.n + i] = c;
        aux[6 * p.n + i] = sn;
    }
    rotate(n, c, sn, d);
    st.z = z1;
    st.k = k3;
    st.dx = d[0];
    st.dy = d[1];
    st.dz = d[2];
    bool const below = p.replay ? end == end_code(p, step, sub, 1) : !(k3 > p.cutoff);
    if (below) {
        st.alive = 0;
        if (!p.replay) end = end_code(p, step, sub, 1);
    }
}

struct Adj {
    double z, dx, dy, dz, k;
};

// One substep backward: `in` is the substep's input state and `aux` its
// tape values (column stride n, particle i); `a` holds the output adjoint
// and becomes the input adjoint; node gradients go to g.
__device__ __forceinline__ void substep_adjoint(Params const& p, const double* __restrict__ e,
                                                const double* __restrict__ aux, int64_t i, int step, int sub,
                                                State const& in, int32_t end, Adj& a, double* g)
{
    if (!in.alive) return;   // frozen: nothing moved
    double const q = -1.0;
    double const v = speed(in.k);
    double const L = v * p.h;
    double sl1, sl2, f1, f2;
    int n1, n2;
    double const za = in.z + kGlA * L * in.dz, zb = in.z + kGlB * L * in.dz;
    double const e1 = field(p, e, za, sl1, n1, f1);
    double const e2 = field(p, e, zb, sl2, n2, f2);
    double const eavg = 0.5 * (e1 + e2);
    double const w = q * in.dz * L * eavg;
    double const s = q * (kC * kC * kInvMeC2) * 0.5 * p.h;
    double const u0 = umag(in.k);
    double const m1[3] = {u0 * in.dx, u0 * in.dy, u0 * in.dz + s * eavg};
    double const nm1 = sqrt(m1[0] * m1[0] + m1[1] * m1[1] + m1[2] * m1[2]);
    double const d1[3] = {m1[0] / nm1, m1[1] / nm1, m1[2] / nm1};
    double const k1 = in.k + 0.5 * w;
    double const sp = aux[i], dsp = aux[p.n + i];
    double const loss = sp * L;
    if (end == end_code(p, step, sub, 0)) {
        // stopped in the drag: z1 = z + L d_z, K the constant cutoff, d as it came
        a = Adj{a.z, a.dx, a.dy, a.dz + a.z * L, a.z * in.dz * p.h * dspeed(in.k)};
        return;
    }
    double ez_bar = 0.0, l_bar = 0.0, w_bar = 0.0;
    double d1_bar[3];
    double const z1_bar = a.z;
    double const k2 = k1 - loss;
    double const u2 = umag(k2);
    double const m2[3] = {u2 * d1[0], u2 * d1[1], u2 * d1[2] + s * eavg};
    double const nm2 = sqrt(m2[0] * m2[0] + m2[1] * m2[1] + m2[2] * m2[2]);
    double const d2[3] = {m2[0] / nm2, m2[1] / nm2, m2[2] / nm2};
    // scatter: d3 = R d2 -> d2_bar = R^T d3_bar
    double const n[3] = {aux[2 * p.n + i], aux[3 * p.n + i], aux[4 * p.n + i]};
    double const c = aux[5 * p.n + i], sn = aux[6 * p.n + i];
    double d2_bar[3] = {a.dx, a.dy, a.dz};
    rotate(n, c, -sn, d2_bar);
    // kick 2: d2 = m2 / |m2|, K3 = K2 + W/2
    double const dd = d2[0] * d2_bar[0] + d2[1] * d2_bar[1] + d2[2] * d2_bar[2];
    double m2_bar[3];
    for (int i = 0; i < 3; ++i) m2_bar[i] = (d2_bar[i] - d2[i] * dd) / nm2;
    double const u2_bar = m2_bar[0] * d1[0] + m2_bar[1] * d1[1] + m2_bar[2] * d1[2];
    for (int i = 0; i < 3; ++i) d1_bar[i] = u2 * m2_bar[i];
    ez_bar += s * m2_bar[2];
    double const k2_bar = a.k + u2_bar * dumag(k2);
    w_bar += 0.5 * a.k;
    // drag: K2 = K1 - rho S(K1) L
    double const k1_bar = k2_bar * (1.0 - dsp * L);
    l_bar -= k2_bar * sp;
    // kick 1: d1 = m1 / |m1|, K1 = K + W/2
    double const dd1 = d1[0] * d1_bar[0] + d1[1] * d1_bar[1] + d1[2] * d1_bar[2];
    double m1_bar[3];
    for (int i = 0; i < 3; ++i) m1_bar[i] = (d1_bar[i] - d1[i] * dd1) / nm1;
    double const u0_bar = m1_bar[0] * in.dx + m1_bar[1] * in.dy + m1_bar[2] * in.dz;
    Adj r{0.0, u0 * m1_bar[0], u0 * m1_bar[1], u0 * m1_bar[2], k1_bar + u0_bar * dumag(in.k)};
    ez_bar += s * m1_bar[2];
    w_bar += 0.5 * k1_bar;
    // W = q dz L <E>
    r.dz += w_bar * q * L * eavg;
    l_bar += w_bar * q * in.dz * eavg;
    ez_bar += w_bar * q * in.dz * L;
    // <E> = (E(za) + E(zb)) / 2
    double const e_bar = 0.5 * ez_bar;
    atomicAdd(g + n1, e_bar * (1.0 - f1));
    atomicAdd(g + n1 + 1, e_bar * f1);
    atomicAdd(g + n2, e_bar * (1.0 - f2));
    atomicAdd(g + n2 + 1, e_bar * f2);
    double const za_bar = e_bar * sl1, zb_bar = e_bar * sl2;
    r.z += za_bar + zb_bar + z1_bar;
    l_bar += (za_bar * kGlA + zb_bar * kGlB) * in.dz + z1_bar * in.dz;
    r.dz += (za_bar * kGlA + zb_bar * kGlB) * L + z1_bar * L;
    // L = v(K) h
    r.k += l_bar * p.h * dspeed(in.k);
    a = r;
}

__device__ __forceinline__ State load(const double* __restrict__ s, int64_t n, int64_t i)
{
    return State{s[i], s[n + i], s[2 * n + i], s[3 * n + i], s[4 * n + i], s[5 * n + i] != 0.0 ? 1 : 0};
}
__device__ __forceinline__ void store(double* __restrict__ s, int64_t n, int64_t i, State const& st)
{
    s[i] = st.z;
    s[n + i] = st.dx;
    s[2 * n + i] = st.dy;
    s[3 * n + i] = st.dz;
    s[4 * n + i] = st.k;
    s[5 * n + i] = st.alive ? 1.0 : 0.0;
}

// Forward over every step: checkpoints ckpt[c] (6 x n each) at the steps
// c * C; final state and the loss.
__global__ void forward_kernel(Params p, const double* __restrict__ e, const double* __restrict__ arena,
                               const double* __restrict__ seeds, const double* __restrict__ w,
                               const uint64_t* __restrict__ id, double* __restrict__ ckpt,
                               double* __restrict__ final_state, double* __restrict__ partials)
{
    double acc = 0.0;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < p.n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        State st = load(seeds, p.n, i);
        double const z_init = st.z;
        int32_t end = p.replay ? p.ends[i] : -1;
        for (int t = 0; t < p.steps; ++t) {
            if (t % p.ckpt_every == 0) store(ckpt + static_cast<int64_t>(t / p.ckpt_every) * 6 * p.n, p.n, i, st);
            for (int q = 0; q < p.substeps; ++q) substep(p, e, arena, id[i], t, q, st, end);
        }
        if (!p.replay) p.ends[i] = end;
        store(final_state, p.n, i, st);
        acc += w[i] * (sig((st.k - p.k_th) / p.tau_k)
                       - p.lambda * (sig((st.z - p.z_p) / p.tau_z) - sig((z_init - p.z_p) / p.tau_z)));
    }
    // the loss is summed in a fixed order (warp tree, the warps of a block
    // in turn, then the blocks in turn by sum_partials_kernel), so the same
    // nodes give the same loss to the bit and finite differences of the loss
    // carry only its rounding
    __shared__ double warp_sums[32];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) warp_sums[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = 0.0;
        for (int k = 0; k < static_cast<int>(blockDim.x >> 5); ++k) b += warp_sums[k];
        partials[blockIdx.x] = b;
    }
}

// The block partials summed in order with Neumaier's compensation, so the
// loss is the correctly rounded sum of the partials to within an ulp or two
// and a difference of two losses carries only their final roundings.
__global__ void sum_partials_kernel(const double* __restrict__ partials, int count, double* loss)
{
    double s = 0.0, c = 0.0;
    for (int k = 0; k < count; ++k) {
        double const x = partials[k];
        double const t = s + x;
        c += fabs(s) >= fabs(x) ? (s - t) + x : (x - t) + s;
        s = t;
    }
    *loss = s + c;
}

// Reverse pass over one checkpoint segment [t0, t1): recompute onto the tape
// (substep inputs, 6 x n per entry), then run the adjoint back through it.
__global__ void reverse_segment_kernel(Params p, const double* __restrict__ e, const double* __restrict__ arena,
                                       const uint64_t* __restrict__ id, const double* __restrict__ ckpt, int t0,
                                       int t1, double* __restrict__ tape, double* __restrict__ aux,
                                       double* __restrict__ adj, double* __restrict__ grad)
{
    extern __shared__ double g[];
    for (int k = threadIdx.x; k < p.n_nodes; k += blockDim.x) g[k] = 0.0;
    __syncthreads();
    int64_t const entries = static_cast<int64_t>(t1 - t0) * p.substeps;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < p.n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        State st = load(ckpt, p.n, i);
        int32_t end = p.ends[i];
        for (int t = t0; t < t1; ++t) {
            for (int q = 0; q < p.substeps; ++q) {
                int64_t const k = static_cast<int64_t>(t - t0) * p.substeps + q;
                store(tape + k * 6 * p.n, p.n, i, st);
                substep(p, e, arena, id[i], t, q, st, end, aux + k * kAux * p.n, i);
            }
        }
        Adj a{adj[i], adj[p.n + i], adj[2 * p.n + i], adj[3 * p.n + i], adj[4 * p.n + i]};
        for (int64_t k = entries - 1; k >= 0; --k) {
            int const t = t0 + static_cast<int>(k / p.substeps), q = static_cast<int>(k % p.substeps);
            State const in = load(tape + k * 6 * p.n, p.n, i);
            substep_adjoint(p, e, aux + k * kAux * p.n, i, t, q, in, end, a, g);
        }
        adj[i] = a.z;
        adj[p.n + i] = a.dx;
        adj[2 * p.n + i] = a.dy;
        adj[3 * p.n + i] = a.dz;
        adj[4 * p.n + i] = a.k;
    }
    __syncthreads();
    for (int k = threadIdx.x; k < p.n_nodes; k += blockDim.x) {
        if (g[k] != 0.0) atomicAdd(grad + k, g[k]);
    }
}

// The loss adjoint at the final state.
__global__ void seed_adjoint_kernel(Params p, const double* __restrict__ final_state, const double* __restrict__ w,
                                    double* __restrict__ adj)
{
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < p.n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        double const z = final_state[i], k = final_state[4 * p.n + i];
        adj[i] = -w[i] * p.lambda * dsig((z - p.z_p) / p.tau_z) / p.tau_z;
        adj[p.n + i] = 0.0;
        adj[2 * p.n + i] = 0.0;
        adj[3 * p.n + i] = 0.0;
        adj[4 * p.n + i] = w[i] * dsig((k - p.k_th) / p.tau_k) / p.tau_k;
    }
}

}  // namespace adj
}  // namespace rrea_dev

namespace rrea_launch {

struct AdjointState {
    rrea_dev::adj::Params p{};
    int64_t cap = 0;
    double* seeds = nullptr;   // 6 x n
    double* w = nullptr;
    uint64_t* id = nullptr;
    double* ckpt = nullptr;    // n_ckpt x 6 x n
    double* final_state = nullptr;
    double* tape = nullptr;    // C x substeps x 6 x n
    double* aux = nullptr;     // C x substeps x kAux x n
    double* adj = nullptr;     // 5 x n
    double* loss = nullptr;
    double* partials = nullptr;   // one loss partial per forward block
    int32_t* ends = nullptr;   // n end records (Params::ends)
    bool recorded = false;     // a recording forward has run
    int blocks = 1;
};

void adjoint_free(AdjointState* s)
{
    if (!s) return;
    for (void* ptr : {static_cast<void*>(s->seeds), static_cast<void*>(s->w), static_cast<void*>(s->id),
                      static_cast<void*>(s->ckpt), static_cast<void*>(s->final_state), static_cast<void*>(s->tape),
                      static_cast<void*>(s->aux),
                      static_cast<void*>(s->adj), static_cast<void*>(s->loss), static_cast<void*>(s->partials),
                      static_cast<void*>(s->ends)}) {
        if (ptr) cudaFree(ptr);
    }
    delete s;
}

cudaError_t adjoint_stage(AdjointSetup const& in, const double* seeds6, const double* w, const uint64_t* id,
                          int blocks, AdjointState*& out)
{
    adjoint_free(out);
    out = nullptr;
    auto* s = new AdjointState();
    rrea_dev::adj::Params& p = s->p;
    p.n = in.n;
    p.n_nodes = in.n_nodes;
    p.z0 = in.z0;
    p.dz_node = in.dz_node;
    p.steps = in.steps;
    p.substeps = in.substeps;
    p.ckpt_every = in.ckpt_every;
    p.h = in.dt / in.substeps;
    p.rho = in.rho;
    p.cutoff = in.cutoff;
    p.scatter_rms = in.scatter_rms;
    p.k_th = in.k_th;
    p.tau_k = in.tau_k;
    p.z_p = in.z_p;
    p.tau_z = in.tau_z;
    p.lambda = in.lambda;
    p.seed = in.seed;
    p.col = in.col;
    p.soft = in.soft;
    s->blocks = blocks;
    int64_t const n = in.n;
    int64_t const n_ckpt = (in.steps + in.ckpt_every - 1) / in.ckpt_every;
    cudaError_t e = cudaSuccess;
    auto alloc = [&](auto** ptr, int64_t count) {
        if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(ptr), sizeof(**ptr) * static_cast<size_t>(count > 0 ? count : 1));
    };
    alloc(&s->seeds, 6 * n);
    alloc(&s->w, n);
    alloc(&s->id, n);
    alloc(&s->ckpt, n_ckpt * 6 * n);
    alloc(&s->final_state, 6 * n);
    alloc(&s->tape, static_cast<int64_t>(in.ckpt_every) * in.substeps * 6 * n);
    alloc(&s->aux, static_cast<int64_t>(in.ckpt_every) * in.substeps * rrea_dev::adj::kAux * n);
    alloc(&s->adj, 5 * n);
    alloc(&s->loss, 1);
    alloc(&s->partials, blocks);
    alloc(&s->ends, n);
    p.ends = s->ends;
    p.replay = 0;
    if (e == cudaSuccess && n > 0) {
        e = cudaMemcpy(s->seeds, seeds6, sizeof(double) * 6 * n, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(s->w, w, sizeof(double) * n, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(s->id, id, sizeof(uint64_t) * n, cudaMemcpyHostToDevice);
    }
    if (e != cudaSuccess) {
        adjoint_free(s);
        return e;
    }
    out = s;
    return cudaSuccess;
}

cudaError_t adjoint_forward(AdjointState& s, const double* arena, const double* e_nodes, bool replay, double& loss,
                            cudaStream_t stream)
{
    cudaError_t e = cudaSuccess;
    rrea_dev::adj::Params p = s.p;
    p.replay = replay ? 1 : 0;
    note_launch();
    rrea_dev::adj::forward_kernel<<<s.blocks, 128, 0, stream>>>(p, e_nodes, arena, s.seeds, s.w, s.id, s.ckpt,
                                                               s.final_state, s.partials);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    note_launch();
    rrea_dev::adj::sum_partials_kernel<<<1, 1, 0, stream>>>(s.partials, s.blocks, s.loss);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if (!replay) s.recorded = true;
    e = cudaMemcpyAsync(&loss, s.loss, sizeof(double), cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    return e;
}

bool adjoint_recorded(AdjointState const& s) { return s.recorded; }

cudaError_t adjoint_backward(AdjointState& s, const double* arena, const double* e_nodes, double* grad,
                             cudaStream_t stream)
{
    rrea_dev::adj::Params p = s.p;
    p.replay = 1;   // the reverse pass follows the recorded ends
    cudaError_t e = cudaMemsetAsync(grad, 0, sizeof(double) * p.n_nodes, stream);
    if (e != cudaSuccess) return e;
    note_launch();
    rrea_dev::adj::seed_adjoint_kernel<<<s.blocks, 256, 0, stream>>>(p, s.final_state, s.w, s.adj);
    int const n_ckpt = (p.steps + p.ckpt_every - 1) / p.ckpt_every;
    size_t const shmem = sizeof(double) * static_cast<size_t>(p.n_nodes);
    for (int c = n_ckpt - 1; c >= 0; --c) {
        int const t0 = c * p.ckpt_every;
        int const t1 = t0 + p.ckpt_every < p.steps ? t0 + p.ckpt_every : p.steps;
        note_launch();
        rrea_dev::adj::reverse_segment_kernel<<<s.blocks, 128, shmem, stream>>>(
            p, e_nodes, arena, s.id, s.ckpt + static_cast<int64_t>(c) * 6 * p.n, t0, t1, s.tape, s.aux, s.adj, grad);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t adjoint_final_state(AdjointState const& s, double* host6)
{
    return cudaMemcpy(host6, s.final_state, sizeof(double) * 6 * static_cast<size_t>(s.p.n), cudaMemcpyDeviceToHost);
}

int adjoint_max_nodes() { return rrea_dev::adj::kMaxNodes; }

}  // namespace rrea_launch
