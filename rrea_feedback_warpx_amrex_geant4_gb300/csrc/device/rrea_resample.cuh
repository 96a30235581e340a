// Charge-exact stochastic thinning of the particles of one order-1 CIC
// support (the per-support primitive of the population control's
// adaptive_resample_v1; RreaThinCicWeights and
// RreaCicResampleRemovalCapacity, I/RreaCicConservingResample.H:46-351).
//
// Every particle of a group deposits w ((1-fr)(1-fz), fr(1-fz), (1-fr)fz,
// fr fz) into the same four cells.  Up to five live particles at a time, a
// direction d in the null space of their four-row CIC matrix moves the
// weights to one of the two non-negative endpoints w + alpha d, chosen with
// the probabilities that make E[alpha] = 0: the four cell charges are kept
// and every weight keeps its expectation, while at least one weight reaches
// zero per draw.
//
// The reference evaluates the linear algebra in long double; here it runs
// in double-double (about 106 bits, above the 64-bit extended format the
// reference's golden vectors come from).  The pivot and sign tolerances
// are the reference's: 512 ulps of that extended format (2^-54).
#pragma once

#include "rrea_dd.cuh"

#include <stdint.h>

namespace rrea_dev {

constexpr int kCicMaxGroup = 64;
constexpr double kCicTolerance = 0x1p-54;  // 512 x 2^-63

struct CicColumn {
    dd v[4];
};

__device__ __forceinline__ CicColumn cic_column(double fr, double fz)
{
    dd const r1 = dd_sub(dd_from(1.0), dd_from(fr));
    dd const z1 = dd_sub(dd_from(1.0), dd_from(fz));
    dd const r = dd_from(fr), z = dd_from(fz);
    return CicColumn{{dd_mul(r1, z1), dd_mul(r, z1), dd_mul(r1, z), dd_mul(r, z)}};
}

__device__ __forceinline__ dd dd_absv(dd a) { return a.hi < 0.0 || (a.hi == 0.0 && a.lo < 0.0) ? dd_neg(a) : a; }
__device__ __forceinline__ bool dd_gt_d(dd a, double b) { return dd_gt(a, dd_from(b)); }
__device__ __forceinline__ bool dd_lt_d(dd a, double b) { return dd_lt(a, dd_from(b)); }
__device__ __forceinline__ bool dd_is_zero(dd a) { return a.hi == 0.0 && a.lo == 0.0; }

// A mixed-sign null vector of the 4 x n matrix of the columns (n <= 5), by
// reduced row echelon elimination with partial pivoting; false when the
// columns are independent or the vector found is numerically one-signed
// (I/RreaCicConservingResample.H:62-160).
__device__ inline bool cic_null_direction(CicColumn const* cols, int n, dd* dir)
{
    dd m[4][5];
    for (int c = 0; c < n; ++c) {
        for (int r = 0; r < 4; ++r) m[r][c] = cols[c].v[r];
    }
    int pivot_col[4] = {-1, -1, -1, -1};
    bool is_pivot[5] = {false, false, false, false, false};
    int rank = 0;
    for (int c = 0; c < n && rank < 4; ++c) {
        int pivot = rank;
        dd best = dd_from(0.0);
        for (int r = rank; r < 4; ++r) {
            dd const a = dd_absv(m[r][c]);
            if (dd_gt(a, best)) {
                best = a;
                pivot = r;
            }
        }
        if (!dd_gt_d(best, kCicTolerance)) continue;
        if (pivot != rank) {
            for (int j = 0; j < 5; ++j) {
                dd const t = m[pivot][j];
                m[pivot][j] = m[rank][j];
                m[rank][j] = t;
            }
        }
        dd const scale = m[rank][c];
        for (int j = 0; j < n; ++j) m[rank][j] = dd_div(m[rank][j], scale);
        for (int r = 0; r < 4; ++r) {
            if (r == rank) continue;
            dd const f = m[r][c];
            if (dd_is_zero(f)) continue;
            for (int j = 0; j < n; ++j) m[r][j] = dd_sub(m[r][j], dd_mul(f, m[rank][j]));
        }
        pivot_col[rank] = c;
        is_pivot[c] = true;
        ++rank;
    }
    if (rank == n) return false;
    int free_col = n;
    for (int c = n - 1; c >= 0; --c) {
        if (!is_pivot[c]) {
            free_col = c;
            break;
        }
    }
    if (free_col == n) return false;
    for (int c = 0; c < n; ++c) dir[c] = dd_from(0.0);
    dir[free_col] = dd_from(1.0);
    for (int rr = rank - 1; rr >= 0; --rr) {
        int const p = pivot_col[rr];
        dd value = dd_from(0.0);
        for (int c = 0; c < n; ++c) {
            if (c != p) value = dd_add(value, dd_mul(m[rr][c], dir[c]));
        }
        dir[p] = dd_neg(value);
    }
    dd max_abs = dd_from(0.0);
    for (int c = 0; c < n; ++c) {
        dd const a = dd_absv(dir[c]);
        if (dd_gt(a, max_abs)) max_abs = a;
    }
    if (!(max_abs.hi > 0.0) || !isfinite(max_abs.hi)) return false;
    bool pos = false, neg = false;
    for (int c = 0; c < n; ++c) {
        dir[c] = dd_div(dir[c], max_abs);
        pos = pos || dd_gt_d(dir[c], kCicTolerance);
        neg = neg || dd_lt_d(dir[c], -kCicTolerance);
    }
    return pos && neg;
}

// Rank of the CIC columns of the live particles (:162-205); the removal
// capacity of a group is its live count minus this rank (:209-224).
__device__ inline int cic_constraint_rank(const double* fr, const double* fz, const double* w, int n)
{
    dd basis[4][4];
    int rank = 0;
    for (int i = 0; i < n && rank < 4; ++i) {
        if (!(w[i] > 0.0)) continue;
        CicColumn col = cic_column(fr[i], fz[i]);
        dd* v = col.v;
        for (int r = 0; r < rank; ++r) {
            int p = 0;
            while (p < 4 && !dd_gt_d(dd_absv(basis[r][p]), kCicTolerance)) ++p;
            if (p == 4) continue;
            dd const f = dd_div(v[p], basis[r][p]);
            for (int j = p; j < 4; ++j) v[j] = dd_sub(v[j], dd_mul(f, basis[r][j]));
        }
        int p = 0;
        while (p < 4 && !dd_gt_d(dd_absv(v[p]), kCicTolerance)) ++p;
        if (p == 4) continue;
        dd const pv = v[p];
        for (int j = 0; j < 4; ++j) basis[rank][j] = j < p ? dd_from(0.0) : dd_div(v[j], pv);
        ++rank;
    }
    return rank;
}

// The group's uniform stream: u_k = (mix64(key + k) >> 11 + 1/2) 2^-53.
__device__ __forceinline__ uint64_t cic_mix64(uint64_t v)
{
    v += 0x9e3779b97f4a7c15ULL;
    v = (v ^ (v >> 30)) * 0xbf58476d1ce4e5b9ULL;
    v = (v ^ (v >> 27)) * 0x94d049bb133111ebULL;
    return v ^ (v >> 31);
}
__device__ __forceinline__ double cic_uniform(uint64_t key, uint64_t k)
{
    return (static_cast<double>(cic_mix64(key + k) >> 11) + 0.5) * 0x1.0p-53;
}

struct CicThinResult {
    int64_t removed, draws;
    bool valid;
};

// RreaThinCicWeights (:226-351) on w[0, n) in place.
__device__ inline CicThinResult cic_thin(const double* fr, const double* fz, double* w, int n, int64_t max_removals,
                                         uint64_t key)
{
    CicThinResult res{0, 0, true};
    uint8_t active[kCicMaxGroup];
    int n_active = 0;
    for (int i = 0; i < n; ++i) {
        if (!isfinite(fr[i]) || !isfinite(fz[i]) || fr[i] < 0.0 || fr[i] > 1.0 || fz[i] < 0.0 || fz[i] > 1.0 ||
            !isfinite(w[i]) || w[i] < 0.0) {
            res.valid = false;
            return res;
        }
        if (w[i] > 0.0) active[n_active++] = static_cast<uint8_t>(i);
    }
    constexpr double kEps = 2.220446049250313080847263336181640625e-16;
    while (res.removed < max_removals && n_active >= 2) {
        int const m = n_active < 5 ? n_active : 5;
        CicColumn cols[5];
        for (int c = 0; c < m; ++c) cols[c] = cic_column(fr[active[c]], fz[active[c]]);
        dd dir[5];
        if (!cic_null_direction(cols, m, dir)) {
            if (n_active > m) res.valid = false;
            return res;
        }
        dd a_plus = dd_from(__longlong_as_double(0x7ff0000000000000LL));
        dd a_minus = a_plus;
        int hit_plus = m, hit_minus = m;
        for (int c = 0; c < m; ++c) {
            dd const wc = dd_from(w[active[c]]);
            if (dd_lt_d(dir[c], 0.0)) {
                dd const b = dd_div(wc, dd_neg(dir[c]));
                if (dd_lt(b, a_plus)) {
                    a_plus = b;
                    hit_plus = c;
                }
            } else if (dd_gt_d(dir[c], 0.0)) {
                dd const b = dd_div(wc, dir[c]);
                if (dd_lt(b, a_minus)) {
                    a_minus = b;
                    hit_minus = c;
                }
            }
        }
        if (!isfinite(a_plus.hi) || !isfinite(a_minus.hi) || a_plus.hi < 0.0 || a_minus.hi < 0.0 ||
            hit_plus == m || hit_minus == m) {
            res.valid = false;
            return res;
        }
        double const u = cic_uniform(key, static_cast<uint64_t>(res.draws));
        if (!(u > 0.0) || !(u < 1.0)) {
            res.valid = false;
            return res;
        }
        ++res.draws;
        dd const p_plus = dd_div(a_minus, dd_add(a_plus, a_minus));
        bool const take_plus = dd_lt(dd_from(u), p_plus);
        dd const alpha = take_plus ? a_plus : dd_neg(a_minus);
        int const zero = take_plus ? hit_plus : hit_minus;
        for (int c = 0; c < m; ++c) {
            double const w0 = w[active[c]];
            dd upd = dd_add(dd_from(w0), dd_mul(alpha, dir[c]));
            if (c == zero) upd = dd_from(0.0);
            double const slack = 512.0 * kEps * static_cast<double>(m) * fmax(1.0, fabs(w0));
            if (dd_lt_d(upd, 0.0) && !dd_gt_d(dd_neg(upd), slack)) upd = dd_from(0.0);
            if (dd_lt_d(upd, 0.0) || !isfinite(upd.hi)) {
                res.valid = false;
                return res;
            }
            w[active[c]] = upd.hi > 0.0 ? upd.hi + upd.lo : 0.0;
        }
        int kept = 0;
        for (int c = 0; c < n_active; ++c) {
            if (w[active[c]] != 0.0) active[kept++] = active[c];
        }
        int const removed_now = n_active - kept;
        n_active = kept;
        if (removed_now == 0) {
            res.valid = false;
            return res;
        }
        res.removed += removed_now;
    }
    return res;
}

// RreaThinCicWeights over a support of any size in global memory, with the
// uniform of draw k from draw(k).  The reference's active list is the live
// particles in index order and a draw only changes its first five entries,
// so the list is kept as a window of those (at most) five followed by the
// untouched particles from `cursor` on: the window is compacted after each
// draw and refilled in index order, which is the reference's erase of the
// zeroed entries, at O(1) per draw instead of O(n).
template <class Draw>
__device__ inline CicThinResult cic_thin_window(const double* fr, const double* fz, double* w, int64_t n,
                                                int64_t max_removals, Draw const& draw)
{
    CicThinResult res{0, 0, true};
    int64_t n_active = 0;
    for (int64_t i = 0; i < n; ++i) {
        if (!isfinite(fr[i]) || !isfinite(fz[i]) || fr[i] < 0.0 || fr[i] > 1.0 || fz[i] < 0.0 || fz[i] > 1.0 ||
            !isfinite(w[i]) || w[i] < 0.0) {
            res.valid = false;
            return res;
        }
        if (w[i] > 0.0) ++n_active;
    }
    int64_t win[5];
    int nw = 0;
    int64_t cursor = 0;
    auto refill = [&]() {
        while (nw < 5 && cursor < n) {
            if (w[cursor] > 0.0) win[nw++] = cursor;
            ++cursor;
        }
    };
    refill();
    constexpr double kEps = 2.220446049250313080847263336181640625e-16;
    while (res.removed < max_removals && n_active >= 2) {
        int const m = nw;  // min(5, n_active): the window is full whenever five are live
        CicColumn cols[5];
        for (int c = 0; c < m; ++c) cols[c] = cic_column(fr[win[c]], fz[win[c]]);
        dd dir[5];
        if (!cic_null_direction(cols, m, dir)) {
            if (n_active > m) res.valid = false;
            return res;
        }
        dd a_plus = dd_from(__longlong_as_double(0x7ff0000000000000LL));
        dd a_minus = a_plus;
        int hit_plus = m, hit_minus = m;
        for (int c = 0; c < m; ++c) {
            dd const wc = dd_from(w[win[c]]);
            if (dd_lt_d(dir[c], 0.0)) {
                dd const b = dd_div(wc, dd_neg(dir[c]));
                if (dd_lt(b, a_plus)) {
                    a_plus = b;
                    hit_plus = c;
                }
            } else if (dd_gt_d(dir[c], 0.0)) {
                dd const b = dd_div(wc, dir[c]);
                if (dd_lt(b, a_minus)) {
                    a_minus = b;
                    hit_minus = c;
                }
            }
        }
        if (!isfinite(a_plus.hi) || !isfinite(a_minus.hi) || a_plus.hi < 0.0 || a_minus.hi < 0.0 ||
            hit_plus == m || hit_minus == m) {
            res.valid = false;
            return res;
        }
        double const u = draw(static_cast<uint64_t>(res.draws));
        if (!(u > 0.0) || !(u < 1.0)) {
            res.valid = false;
            return res;
        }
        ++res.draws;
        dd const p_plus = dd_div(a_minus, dd_add(a_plus, a_minus));
        bool const take_plus = dd_lt(dd_from(u), p_plus);
        dd const alpha = take_plus ? a_plus : dd_neg(a_minus);
        int const zero = take_plus ? hit_plus : hit_minus;
        for (int c = 0; c < m; ++c) {
            double const w0 = w[win[c]];
            dd upd = dd_add(dd_from(w0), dd_mul(alpha, dir[c]));
            if (c == zero) upd = dd_from(0.0);
            double const slack = 512.0 * kEps * static_cast<double>(m) * fmax(1.0, fabs(w0));
            if (dd_lt_d(upd, 0.0) && !dd_gt_d(dd_neg(upd), slack)) upd = dd_from(0.0);
            if (dd_lt_d(upd, 0.0) || !isfinite(upd.hi)) {
                res.valid = false;
                return res;
            }
            w[win[c]] = upd.hi > 0.0 ? upd.hi + upd.lo : 0.0;
        }
        int kept = 0;
        for (int c = 0; c < nw; ++c) {
            if (w[win[c]] != 0.0) win[kept++] = win[c];
        }
        int const removed_now = nw - kept;
        nw = kept;
        if (removed_now == 0) {
            res.valid = false;
            return res;
        }
        n_active -= removed_now;
        res.removed += removed_now;
        refill();
    }
    return res;
}

// Rank of the CIC columns of a support of any size (at most four, found
// among its first independent columns; :162-205).
__device__ inline int cic_constraint_rank_any(const double* fr, const double* fz, const double* w, int64_t n)
{
    dd basis[4][4];
    int rank = 0;
    for (int64_t i = 0; i < n && rank < 4; ++i) {
        if (!(w[i] > 0.0)) continue;
        CicColumn col = cic_column(fr[i], fz[i]);
        dd* v = col.v;
        for (int r = 0; r < rank; ++r) {
            int p = 0;
            while (p < 4 && !dd_gt_d(dd_absv(basis[r][p]), kCicTolerance)) ++p;
            if (p == 4) continue;
            dd const f = dd_div(v[p], basis[r][p]);
            for (int j = p; j < 4; ++j) v[j] = dd_sub(v[j], dd_mul(f, basis[r][j]));
        }
        int p = 0;
        while (p < 4 && !dd_gt_d(dd_absv(v[p]), kCicTolerance)) ++p;
        if (p == 4) continue;
        dd const pv = v[p];
        for (int j = 0; j < 4; ++j) basis[rank][j] = j < p ? dd_from(0.0) : dd_div(v[j], pv);
        ++rank;
    }
    return rank;
}

// RreaRoundAndVerifyCicWeights (:424-468) with FP64 storage: the four cell
// moments of the thinned weights agree with those of the original weights
// within 512 ulps x support size x max(1, |moment|).
__device__ inline bool cic_moments_kept(const double* fr, const double* fz, const double* w0, const double* w1,
                                        int64_t n)
{
    dd before[4] = {dd_from(0.0), dd_from(0.0), dd_from(0.0), dd_from(0.0)};
    dd after[4] = {dd_from(0.0), dd_from(0.0), dd_from(0.0), dd_from(0.0)};
    for (int64_t i = 0; i < n; ++i) {
        CicColumn const c = cic_column(fr[i], fz[i]);
        for (int k = 0; k < 4; ++k) {
            before[k] = dd_add(before[k], dd_mul(dd_from(w0[i]), c.v[k]));
            after[k] = dd_add(after[k], dd_mul(dd_from(w1[i]), c.v[k]));
        }
    }
    constexpr double kEps = 2.220446049250313080847263336181640625e-16;
    for (int k = 0; k < 4; ++k) {
        double const scale = fmax(1.0, fabs(before[k].hi));
        double const tol = 512.0 * kEps * static_cast<double>(n) * scale;
        dd const diff = dd_absv(dd_sub(after[k], before[k]));
        if (dd_gt_d(diff, tol)) return false;
    }
    return true;
}

}  // namespace rrea_dev
