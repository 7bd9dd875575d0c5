// Smoothed-aggregation multigrid for the complex Hermitian connection Laplacian of the field
// solve.
//
// Host set-up (once per field solve, the matrix is fixed across the 50 inverse iterations):
//  * greedy aggregation on the matrix graph: pass 1 makes an aggregate of every node whose
//    neighbours are all free (node + neighbours), pass 2 attaches the rest to a neighbouring
//    aggregate, pass 3 makes singletons of what is left;
//  * tentative prolongation with a parallel-transported near-null vector: smooth vectors of L
//    satisfy x_j ~ -(A_ji / |A_ji|) x_i along an edge, so t is propagated from each root
//    along the aggregation tree and T(i, agg i) = t_i / sqrt|agg|;
//  * the prolongation smoothed by one Jacobi step, P_sa = (I - w_p D^-1 A) T, and Galerkin
//    coarse operators A_{l+1} = P_sa^H A_l P_sa, down to <= kCoarseMax rows, whose dense inverse
//    is applied on the device.
// Device V(1,1) cycle with weighted Jacobi (omega = 0.8, symmetric pre/post smoothing, exact
// coarse solve).  Pre-smoothing, residual and restriction are one operator R per level,
// prolongation and post-smoothing another (P), so a level costs two grid barriers.
#pragma once
#include <algorithm>
#include <cmath>
#include <complex>
#include <memory>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "mtk_ctx.cuh"

namespace mtk {

// Builds CSR rows in parallel: fn(row, add) calls add(col, value) for the entries of `row`
// (duplicates are summed in call order).  Two passes over the rows: the first counts the
// distinct columns of every row, the second writes each row (sorted by column) straight into
// the final arrays.  A row is accumulated in a dense per-thread array of the column count when
// those arrays stay below 256 MB over all threads, otherwise as (column, value) pairs that
// are stably sorted; both sum duplicates in call order, so the arrays are the same either way.
// Every row is formed by one thread in the same order whatever the thread count.
template <typename V, typename RowFn>
void build_rows_parallel(int nrows, int ncols, RowFn fn, std::vector<int>& ptr, std::vector<int>& col,
                         std::vector<V>& val) {
    int nt = 1;
#ifdef _OPENMP
    nt = omp_get_max_threads();
#endif
    const bool dense = (double)ncols * nt * (sizeof(V) + 1) <= 256.0 * 1024 * 1024;
    ptr.assign(nrows + 1, 0);
#pragma omp parallel
    {
        std::vector<int> cols;
        std::vector<char> used(dense ? ncols : 0, 0);
#pragma omp for schedule(static)
        for (int r = 0; r < nrows; r++) {
            cols.clear();
            if (dense) {
                fn(r, [&](int c, V) {
                    if (!used[c]) { used[c] = 1; cols.push_back(c); }
                });
                for (int c : cols) used[c] = 0;
                ptr[r + 1] = (int)cols.size();
            } else {
                fn(r, [&](int c, V) { cols.push_back(c); });
                std::sort(cols.begin(), cols.end());
                ptr[r + 1] = (int)(std::unique(cols.begin(), cols.end()) - cols.begin());
            }
        }
    }
    for (int r = 0; r < nrows; r++) ptr[r + 1] += ptr[r];
    col.resize(ptr[nrows]);
    val.resize(ptr[nrows]);
#pragma omp parallel
    {
        std::vector<int> cols;
        std::vector<V> acc(dense ? ncols : 0, V(0));
        std::vector<char> used(dense ? ncols : 0, 0);
        std::vector<std::pair<int, V>> ent;
#pragma omp for schedule(static)
        for (int r = 0; r < nrows; r++) {
            int q = ptr[r];
            if (dense) {
                cols.clear();
                fn(r, [&](int c, V v) {
                    if (!used[c]) { used[c] = 1; cols.push_back(c); acc[c] = V(0); }
                    acc[c] += v;
                });
                std::sort(cols.begin(), cols.end());
                for (int c : cols) { col[q] = c; val[q] = acc[c]; used[c] = 0; q++; }
            } else {
                ent.clear();
                fn(r, [&](int c, V v) { ent.emplace_back(c, v); });
                std::stable_sort(ent.begin(), ent.end(), [](const auto& x, const auto& y) { return x.first < y.first; });
                q--;
                for (size_t k = 0; k < ent.size(); k++) {
                    if (k == 0 || ent[k].first != ent[k - 1].first) {
                        q++;
                        col[q] = ent[k].first;
                        val[q] = ent[k].second;
                    } else {
                        val[q] += ent[k].second;
                    }
                }
            }
        }
    }
}

// Sums K per-row terms over rows [0, n) in an order that does not depend on the thread count
// or on scheduling: fixed blocks of 4096 rows are summed in parallel, the block sums in order.
// fn(i, acc) adds row i's terms to acc[0..K).
template <int K, typename Fn>
void det_row_sums(int n, Fn fn, double (&out)[K]) {
    constexpr int kRows = 4096;
    const int nb = (n + kRows - 1) / kRows;
    std::vector<double> part((size_t)nb * K, 0.0);
#pragma omp parallel for schedule(static)
    for (int b = 0; b < nb; b++) {
        double acc[K] = {};
        const int e = std::min(n, (b + 1) * kRows);
        for (int i = b * kRows; i < e; i++) fn(i, acc);
        for (int k = 0; k < K; k++) part[(size_t)b * K + k] = acc[k];
    }
    for (int k = 0; k < K; k++) out[k] = 0.0;
    for (int b = 0; b < nb; b++)
        for (int k = 0; k < K; k++) out[k] += part[(size_t)b * K + k];
}

constexpr int kMaxLevels = 8;
constexpr int kCoarseMax = 384;
constexpr double kOmega = 0.8;   // Jacobi weight of the pre- and post-smoothing
constexpr double kAlpha = 1.0;   // coarse-correction scale

// ------------------------------------------------------------------ host hierarchy
struct HostCsr {
    int n = 0;
    std::vector<int> ptr, col;
    std::vector<std::complex<double>> val;
};

struct HostLevel {
    HostCsr A;                                 // operator of this level (level 0: from the ELL)
    std::vector<int> agg;                      // aggregate of each row (-> next level row)
    std::vector<std::complex<double>> T;       // tentative prolongation coefficient per row
    std::vector<int> mptr, mem;                // members of each aggregate
    std::vector<double> dinv;                  // 1 / diag
    double wp = 0;                             // prolongation smoothing weight
};

// The V(1,1) cycle written as three sparse operators per level (x = omega D^-1 r pre-smoothing,
// coarse correction scaled by alpha, post-smoothing), so each level is one SpMV phase:
//   down  r_{l+1} = R r_l,            R = T^H (I - omega A D^-1)
//   up    y_l = S r_l + P y_{l+1},    S = omega D^-1 (2 I - A omega D^-1),
//                                     P = alpha (I - omega D^-1 A) T   (= alpha R^H)
struct HostCycleOps {
    HostCsr R, S, P;
};

struct HostHierarchy {
    std::vector<HostLevel> lv;
    std::vector<HostCycleOps> ops;
    int nc = 0;                                // coarsest size
    std::vector<std::complex<double>> Ainv;    // dense inverse of the coarsest operator
};

inline int aggregate_level(HostLevel& L) {
    const HostCsr& A = L.A;
    const int n = A.n;
    L.agg.assign(n, -1);
    std::vector<int> parent(n, -1);
    int na = 0;
    // pass 1
    for (int i = 0; i < n; i++) {
        if (L.agg[i] >= 0) continue;
        bool free_nbrs = true;
        for (int p = A.ptr[i]; p < A.ptr[i + 1]; p++) {
            int j = A.col[p];
            if (j != i && L.agg[j] >= 0) { free_nbrs = false; break; }
        }
        if (!free_nbrs) continue;
        L.agg[i] = na;
        for (int p = A.ptr[i]; p < A.ptr[i + 1]; p++) {
            int j = A.col[p];
            if (j != i) { L.agg[j] = na; parent[j] = i; }
        }
        na++;
    }
    // pass 2: attach to the strongest aggregated neighbour (|a|^2 = re^2 + im^2, the first
    // largest in row order)
    for (int i = 0; i < n; i++) {
        if (L.agg[i] >= 0) continue;
        int best = -1;
        double bw = -1;
        for (int p = A.ptr[i]; p < A.ptr[i + 1]; p++) {
            int j = A.col[p];
            if (j == i || L.agg[j] < 0) continue;
            double w = std::norm(A.val[p]);
            if (w > bw) { bw = w; best = j; }
        }
        if (best >= 0) { L.agg[i] = L.agg[best]; parent[i] = best; }
    }
    // pass 3: singletons / new aggregates for what is left
    for (int i = 0; i < n; i++)
        if (L.agg[i] < 0) { L.agg[i] = na++; parent[i] = -1; }
    // transported near-null vector along the parent forest: t = 1 at a root, t_v = -(a / |a|) t_parent
    // with a = A(v, parent).  Each value depends on its parent's only, so the forest is resolved
    // in parallel rounds (round r computes the nodes whose parent was resolved before round r):
    // the same values as any sequential order.
    // (every entry of t and of the round arrays is written before it is read: no serial zeroing)
    std::unique_ptr<std::complex<double>[]> t(new std::complex<double>[n]);
    std::vector<int> cnt(na, 0);
    for (int i = 0; i < n; i++) cnt[L.agg[i]]++;
    {
        std::unique_ptr<int[]> rnd_a(new int[n]), rnd_b(new int[n]);   // resolving round (-1: not yet)
        int* rnd = rnd_a.get();
        int* rnd_next = rnd_b.get();
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; i++) {
            rnd[i] = parent[i] < 0 ? 0 : -1;
            if (parent[i] < 0) t[i] = 1.0;
        }
        for (int r = 1;; r++) {
#pragma omp parallel for schedule(static)
            for (int i = 0; i < n; i++) rnd_next[i] = rnd[i];
            int changed = 0;
#pragma omp parallel for schedule(static) reduction(+ : changed)
            for (int v = 0; v < n; v++) {
                if (rnd[v] >= 0) continue;
                const int pv = parent[v];
                if (rnd[pv] < 0) continue;
                std::complex<double> a(0, 0);
                for (int p = A.ptr[v]; p < A.ptr[v + 1]; p++) if (A.col[p] == pv) { a = A.val[p]; break; }
                const double m = std::sqrt(std::norm(a));
                t[v] = m > 0 ? -(a / m) * t[pv] : t[pv];
                rnd_next[v] = r;
                changed++;
            }
            std::swap(rnd, rnd_next);
            if (!changed) break;
        }
    }
    L.T.resize(n);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; i++) L.T[i] = t[i] / std::sqrt((double)cnt[L.agg[i]]);
    L.mptr.assign(na + 1, 0);
    for (int i = 0; i < n; i++) L.mptr[L.agg[i] + 1]++;
    for (int a = 0; a < na; a++) L.mptr[a + 1] += L.mptr[a];
    L.mem.resize(n);
    {
        std::vector<int> fill(L.mptr.begin(), L.mptr.end() - 1);
        for (int i = 0; i < n; i++) L.mem[fill[L.agg[i]]++] = i;
    }
    L.dinv.resize(n);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; i++) {
        double d = 0;
        for (int p = A.ptr[i]; p < A.ptr[i + 1]; p++) if (A.col[p] == i) d = A.val[p].real();
        L.dinv[i] = d > 0 ? 1.0 / d : 1.0;
    }
    return na;
}

// Hermitian positive definite inverse (complex Cholesky), returns false if not HPD.  Column
// updates and the n substitutions run in parallel (each entry is still a sequential sum).
inline bool hpd_inverse(std::vector<std::complex<double>>& A, int n) {
    using cd = std::complex<double>;
    std::vector<cd> L(A);
    for (int j = 0; j < n; j++) {
        double d = L[(size_t)j * n + j].real();
        for (int k = 0; k < j; k++) d -= std::norm(L[(size_t)j * n + k]);
        if (!(d > 0)) return false;
        d = std::sqrt(d);
        L[(size_t)j * n + j] = d;
#pragma omp parallel for schedule(static) if (n - j > 64)
        for (int i = j + 1; i < n; i++) {
            cd s = L[(size_t)i * n + j];
            for (int k = 0; k < j; k++) s -= L[(size_t)i * n + k] * std::conj(L[(size_t)j * n + k]);
            L[(size_t)i * n + j] = s / d;
        }
    }
    std::vector<cd> inv((size_t)n * n, 0.0);
#pragma omp parallel
    {
        std::vector<cd> y(n), xcol(n);
#pragma omp for schedule(static)
        for (int col = 0; col < n; col++) {
            for (int i = 0; i < n; i++) {
                cd s = i == col ? cd(1, 0) : cd(0, 0);
                for (int k = 0; k < i; k++) s -= L[(size_t)i * n + k] * y[k];
                y[i] = s / L[(size_t)i * n + i].real();
            }
            for (int i = n - 1; i >= 0; i--) {
                cd s = y[i];
                for (int k = i + 1; k < n; k++) s -= std::conj(L[(size_t)k * n + i]) * xcol[k];
                xcol[i] = s / L[(size_t)i * n + i].real();
            }
            for (int i = 0; i < n; i++) inv[(size_t)i * n + col] = xcol[i];
        }
    }
    A.swap(inv);
    return true;
}

// Hermitian transpose of an n x m complex CSR.  Threads count the columns of contiguous row
// blocks and offsets are laid out block by block, so every output row lists its entries in
// ascending input row (the serial result, for any thread count).
inline HostCsr hcsr_adjoint(const HostCsr& M, int m) {
    HostCsr Tm;
    Tm.n = m;
    Tm.ptr.assign(m + 1, 0);
    Tm.col.resize(M.col.size());
    Tm.val.resize(M.col.size());
    int nt = 1;
#ifdef _OPENMP
    nt = omp_get_max_threads();
#endif
    std::vector<std::vector<int>> cnt(nt);
#pragma omp parallel num_threads(nt)
    {
        int t = 0;
#ifdef _OPENMP
        t = omp_get_thread_num();
#endif
        const int r0 = (int)((long long)M.n * t / nt), r1 = (int)((long long)M.n * (t + 1) / nt);
        std::vector<int>& c = cnt[t];
        c.assign(m, 0);
        for (int p = M.ptr[r0]; p < M.ptr[r1]; p++) c[M.col[p]]++;
#pragma omp barrier
#pragma omp single
        {
            for (int a = 0; a < m; a++) {
                int s = 0;
                for (int u = 0; u < nt; u++) s += cnt[u][a];
                Tm.ptr[a + 1] = s;
            }
            for (int a = 0; a < m; a++) Tm.ptr[a + 1] += Tm.ptr[a];
            for (int a = 0; a < m; a++) {
                int off = Tm.ptr[a];
                for (int u = 0; u < nt; u++) {
                    const int k = cnt[u][a];
                    cnt[u][a] = off;
                    off += k;
                }
            }
        }
        for (int i = r0; i < r1; i++)
            for (int p = M.ptr[i]; p < M.ptr[i + 1]; p++) {
                const int q = c[M.col[p]]++;
                Tm.col[q] = i;
                Tm.val[q] = std::conj(M.val[p]);
            }
    }
    return Tm;
}

// Builds the smoothed-aggregation hierarchy from the level-0 ELL rows (nbr[3*f+j], val[j*n+f],
// diag d).  Per level: aggregates and T (aggregate_level), the smoothed prolongation
// P_sa = (I - w_p D^-1 A) T with w_p = (4/3) / rho(D^-1 A) (power estimate raised by 5 percent),
// and the Galerkin coarse operator P_sa^H A P_sa.  The cycle operators (V(1,1), Jacobi weight
// kOmega, coarse correction scale kAlpha)
//   R = P_sa^H (I - omega A D^-1),  S = omega D^-1 (2 I - A omega D^-1),
//   P = alpha (I - omega D^-1 A) P_sa = alpha R^H
// are formed for levels >= first_ops (the device applies level 0 from the ELL rows, the
// aggregates, T and w_p).
// Level-0 CSR from the ELL rows: the diagonal and the neighbours, sorted by column.  A boundary
// side (nbr -1) has no entry and lowers the diagonal by 1 (diag is that of a face with three
// neighbours), which gives the reference's #neighbours + 1e-9.
inline HostCsr ell_to_csr(int n, const std::vector<int>& nbr3, const std::vector<std::complex<double>>& vals,
                          double diag) {
    using cd = std::complex<double>;
    HostCsr A0;
    A0.n = n;
    A0.ptr.assign(n + 1, 0);
    for (int f = 0; f < n; f++) {
        int k = 1;
        for (int j = 0; j < 3; j++) k += nbr3[3 * (size_t)f + j] >= 0;
        A0.ptr[f + 1] = A0.ptr[f] + k;
    }
    A0.col.resize(A0.ptr[n]);
    A0.val.resize(A0.ptr[n]);
#pragma omp parallel for schedule(static)
    for (int f = 0; f < n; f++) {
        struct E { int c; cd v; } e[4];
        int k = 1, missing = 0;
        for (int j = 0; j < 3; j++) {
            const int g = nbr3[3 * (size_t)f + j];
            if (g < 0) { missing++; continue; }
            e[k++] = {g, vals[(size_t)j * n + f]};
        }
        e[0] = {f, cd(missing ? diag - (double)missing : diag, 0)};
        std::sort(e, e + k, [](const E& a, const E& b) { return a.c < b.c; });
        for (int q = 0; q < k; q++) { A0.col[A0.ptr[f] + q] = e[q].c; A0.val[A0.ptr[f] + q] = e[q].v; }
    }
    return A0;
}

inline bool build_hierarchy(int n, const std::vector<int>& nbr3, const std::vector<std::complex<double>>& vals,
                            double diag, HostHierarchy& H, int first_ops = 0) {
    using cd = std::complex<double>;
    H.lv.clear();
    H.ops.clear();
    HostCsr cur = ell_to_csr(n, nbr3, vals, diag);
    const double omega = kOmega, alpha = kAlpha;
    while (cur.n > kCoarseMax && (int)H.lv.size() < kMaxLevels - 1) {
        HostLevel L;
        L.A = std::move(cur);
        const int na = aggregate_level(L);
        if (na >= L.A.n) return false;   // no coarsening
        const HostCsr& A = L.A;
        const int ln = A.n;
        double rho = 0;
        {
            std::vector<cd> v(ln), w(ln);
#pragma omp parallel for schedule(static)
            for (int i = 0; i < ln; i++) v[i] = cd((i & 1) ? 1.0 : -1.0 + 0.25 * (double)(((unsigned)i * 7919u) % 5u), 0.1 * (double)(((unsigned)i * 104729u) % 7u));
            for (int it = 0; it < 12; it++) {
                double red[3];   // v^H A v, v^H D v, |w|^2
                det_row_sums<3>(
                    ln,
                    [&](int i, double* acc) {
                        cd av = 0;
                        for (int p = A.ptr[i]; p < A.ptr[i + 1]; p++) av += A.val[p] * v[A.col[p]];
                        w[i] = L.dinv[i] * av;
                        acc[0] += (std::conj(v[i]) * av).real();
                        acc[1] += std::norm(v[i]) / L.dinv[i];
                        acc[2] += std::norm(w[i]);
                    },
                    red);
                rho = red[1] > 0 ? red[0] / red[1] : 0.0;
                const double sc = red[2] > 0 ? 1.0 / std::sqrt(red[2]) : 0.0;
#pragma omp parallel for schedule(static)
                for (int i = 0; i < ln; i++) v[i] = w[i] * sc;
            }
            rho *= 1.05;
        }
        L.wp = rho > 0 ? (4.0 / 3.0) / rho : 0.0;
        const double wp = L.wp;
        HostCsr Psa, AP;
        Psa.n = ln;
        build_rows_parallel<cd>(
            ln, na,
            [&](int i, auto add) {
                add(L.agg[i], L.T[i]);
                for (int p = A.ptr[i]; p < A.ptr[i + 1]; p++) add(L.agg[A.col[p]], -wp * L.dinv[i] * A.val[p] * L.T[A.col[p]]);
            },
            Psa.ptr, Psa.col, Psa.val);
        AP.n = ln;
        build_rows_parallel<cd>(
            ln, na,
            [&](int i, auto add) {
                for (int p = A.ptr[i]; p < A.ptr[i + 1]; p++) {
                    const int k = A.col[p];
                    for (int q = Psa.ptr[k]; q < Psa.ptr[k + 1]; q++) add(Psa.col[q], A.val[p] * Psa.val[q]);
                }
            },
            AP.ptr, AP.col, AP.val);
        const HostCsr Ph = hcsr_adjoint(Psa, na);
        HostCsr next;
        next.n = na;
        build_rows_parallel<cd>(
            na, na,
            [&](int a2, auto add) {
                for (int t = Ph.ptr[a2]; t < Ph.ptr[a2 + 1]; t++) {
                    const int i = Ph.col[t];
                    const cd pv = Ph.val[t];
                    for (int q = AP.ptr[i]; q < AP.ptr[i + 1]; q++) add(AP.col[q], pv * AP.val[q]);
                }
            },
            next.ptr, next.col, next.val);
        for (int a2 = 0; a2 < na; a2++)   // Hermitian diagonal
            for (int p = next.ptr[a2]; p < next.ptr[a2 + 1]; p++)
                if (next.col[p] == a2) next.val[p] = cd(next.val[p].real(), 0.0);
        HostCycleOps O;
        if ((int)H.lv.size() >= first_ops) {
            O.S.n = ln;
            O.S.ptr = A.ptr;
            O.S.col = A.col;
            O.S.val.resize(A.val.size());
#pragma omp parallel for schedule(static)
            for (int i = 0; i < ln; i++)
                for (int p = A.ptr[i]; p < A.ptr[i + 1]; p++) {
                    const int j = A.col[p];
                    cd v = -A.val[p] * (omega * L.dinv[j]);
                    if (j == i) v += 2.0;
                    O.S.val[p] = omega * L.dinv[i] * v;
                }
            O.P.n = ln;
            build_rows_parallel<cd>(
                ln, na,
                [&](int i, auto add) {
                    for (int q = Psa.ptr[i]; q < Psa.ptr[i + 1]; q++) add(Psa.col[q], alpha * Psa.val[q]);
                    for (int q = AP.ptr[i]; q < AP.ptr[i + 1]; q++) add(AP.col[q], -alpha * omega * L.dinv[i] * AP.val[q]);
                },
                O.P.ptr, O.P.col, O.P.val);
            O.R = hcsr_adjoint(O.P, na);
            for (cd& v : O.R.val) v /= alpha;
        }
        H.ops.push_back(std::move(O));
        H.lv.push_back(std::move(L));
        cur = std::move(next);
    }
    if (cur.n > kCoarseMax) return false;
    H.nc = cur.n;
    H.Ainv.assign((size_t)cur.n * cur.n, 0.0);
    for (int i = 0; i < cur.n; i++)
        for (int p = cur.ptr[i]; p < cur.ptr[i + 1]; p++) H.Ainv[(size_t)i * cur.n + cur.col[p]] = cur.val[p];
    for (int i = 0; i < cur.n; i++)   // Hermitian part (round-off of the Galerkin products)
        for (int j = 0; j < i; j++) {
            const cd m = 0.5 * (H.Ainv[(size_t)i * cur.n + j] + std::conj(H.Ainv[(size_t)j * cur.n + i]));
            H.Ainv[(size_t)i * cur.n + j] = m;
            H.Ainv[(size_t)j * cur.n + i] = std::conj(m);
        }
    return hpd_inverse(H.Ainv, cur.n);
}

// ------------------------------------------------------------------ device hierarchy
template <typename T> struct Cv;
template <> struct Cv<float> { using V2 = float2; };
template <> struct Cv<double> { using V2 = double2; };

template <typename T>
struct DevCsr {
    using V2 = typename Cv<T>::V2;
    int n;           // rows
    int group;       // lanes per row (power of two, 1..32)
    const int* ptr;
    const int* col;
    const V2* val;
    // SELL-32 copy (mtk_sell.cuh), used by one-lane-per-row phases when present
    const int* sptr = nullptr;
    const int* scol = nullptr;
    const V2* sval = nullptr;
};

template <typename T>
struct DevLevel {
    using V2 = typename Cv<T>::V2;
    DevCsr<T> R, S, P;
    V2* r;           // right-hand side of this level (level 0: the PCG residual)
    V2* y;           // cycle output of this level (level 0: the PCG z)
};

template <typename T>
struct DevHierarchy {
    using V2 = typename Cv<T>::V2;
    int nlev;                    // levels with smoothing (coarsest excluded)
    DevLevel<T> L[kMaxLevels];
    int nc;
    const V2* Ainv;              // nc x nc dense
    V2* rc;                      // coarsest right-hand side
    V2* yc;                      // coarsest solution
};

// Level 0 applied from the ELL rows of the operator: rows are numbered by aggregate (aggregate a
// owns rows cptr[a] .. cptr[a+1]-1), and chunk w of at most 32 rows, chunk[w] .. chunk[w+1]-1,
// holds whole aggregates, so one warp forms the restriction of a chunk with a segmented sum.
template <typename T>
struct DevLevel0 {
    using V2 = typename Cv<T>::V2;
    int nagg, nchunk;
    const int* agg;      // aggregate (level-1 row) of each row
    const V2* t;         // T(k, agg k): transported near-null coefficient / sqrt|aggregate|
    const int* chunk;    // chunk starts, nchunk + 1 entries
    T dinv;              // 1 / (3 + 1e-9): the uniform ELL diagonal (boundary sides are entries -1)
    T omega, alpha, wp;  // smoothing weight, coarse-correction scale, prolongation smoothing
};

template <typename V2> __device__ __forceinline__ V2 cmulv(V2 a, V2 b) {
    V2 o; o.x = a.x * b.x - a.y * b.y; o.y = a.x * b.y + a.y * b.x; return o;
}
template <typename V2> __device__ __forceinline__ V2 cconjmul(V2 a, V2 b) {   // conj(a) * b
    V2 o; o.x = a.x * b.x + a.y * b.y; o.y = a.x * b.y - a.y * b.x; return o;
}

}  // namespace mtk
