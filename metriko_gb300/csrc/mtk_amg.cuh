// Aggregation multigrid for the complex Hermitian connection Laplacian of the field solve.
//
// Host set-up (once per field solve, the matrix is fixed across the 50 inverse iterations):
//  * greedy aggregation on the matrix graph: pass 1 makes an aggregate of every node whose
//    neighbours are all free (node + neighbours), pass 2 attaches the rest to a neighbouring
//    aggregate, pass 3 makes singletons of what is left;
//  * tentative prolongation with a parallel-transported near-null vector: smooth vectors of L
//    satisfy x_j ~ -(A_ji / |A_ji|) x_i along an edge, so t is propagated from each root
//    along the aggregation tree and T(i, agg i) = t_i / sqrt|agg|;
//  * Galerkin coarse operators A_{l+1} = T^H A_l T, down to <= kCoarseMax rows, whose dense
//    inverse is applied on the device.
// Device V(1,1) cycle with weighted Jacobi (omega = 0.8, symmetric pre/post smoothing, exact
// coarse solve) and the coarse correction scaled by alpha = 1.8 (plain aggregation
// under-corrects; any alpha < 2 keeps the cycle Hermitian positive definite).  Pre-smoothing,
// residual and restriction are fused per aggregate, prolongation and post-smoothing per row,
// so a cycle costs two grid barriers per level.
#pragma once
#include <algorithm>
#include <cmath>
#include <complex>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "mtk_ctx.cuh"

namespace mtk {

// Builds CSR rows in parallel: fn(row, add) calls add(col, value) for the entries of `row`
// (duplicates are summed).  Two passes over the rows: the first counts the distinct columns of
// every row, the second writes each row (sorted by column) straight into the final arrays, so
// there are no per-thread buffers to grow and concatenate.  Every row is formed by one thread
// in the same order whatever the thread count, so the result does not depend on it.
template <typename V, typename RowFn>
void build_rows_parallel(int nrows, int ncols, RowFn fn, std::vector<int>& ptr, std::vector<int>& col,
                         std::vector<V>& val) {
    ptr.assign(nrows + 1, 0);
#pragma omp parallel
    {
        std::vector<char> used(ncols, 0);
        std::vector<int> cols;
#pragma omp for schedule(static)
        for (int r = 0; r < nrows; r++) {
            cols.clear();
            fn(r, [&](int c, V) {
                if (!used[c]) { used[c] = 1; cols.push_back(c); }
            });
            for (int c : cols) used[c] = 0;
            ptr[r + 1] = (int)cols.size();
        }
    }
    for (int r = 0; r < nrows; r++) ptr[r + 1] += ptr[r];
    col.resize(ptr[nrows]);
    val.resize(ptr[nrows]);
#pragma omp parallel
    {
        std::vector<V> acc(ncols, V(0));
        std::vector<char> used(ncols, 0);
        std::vector<int> cols;
#pragma omp for schedule(static)
        for (int r = 0; r < nrows; r++) {
            cols.clear();
            fn(r, [&](int c, V v) {
                if (!used[c]) { used[c] = 1; cols.push_back(c); acc[c] = V(0); }
                acc[c] += v;
            });
            std::sort(cols.begin(), cols.end());
            int q = ptr[r];
            for (int c : cols) { col[q] = c; val[q] = acc[c]; used[c] = 0; q++; }
        }
    }
}

constexpr int kMaxLevels = 8;
constexpr int kCoarseMax = 384;
constexpr double kOmega = 0.8;   // Jacobi weight of the pre- and post-smoothing
constexpr double kAlpha = 1.8;   // coarse-correction scale

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

inline void aggregate_level(HostLevel& L, HostCsr& next) {
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
    // pass 2: attach to the strongest aggregated neighbour
    for (int i = 0; i < n; i++) {
        if (L.agg[i] >= 0) continue;
        int best = -1;
        double bw = -1;
        for (int p = A.ptr[i]; p < A.ptr[i + 1]; p++) {
            int j = A.col[p];
            if (j == i || L.agg[j] < 0) continue;
            double w = std::abs(A.val[p]);
            if (w > bw) { bw = w; best = j; }
        }
        if (best >= 0) { L.agg[i] = L.agg[best]; parent[i] = best; }
    }
    // pass 3: singletons / new aggregates for what is left
    for (int i = 0; i < n; i++)
        if (L.agg[i] < 0) { L.agg[i] = na++; parent[i] = -1; }
    // transported near-null vector along the parent tree (parents precede in pass order)
    std::vector<std::complex<double>> t(n, std::complex<double>(0, 0));
    std::vector<int> order;
    order.reserve(n);
    std::vector<char> done(n, 0);
    std::vector<int> cnt(na, 0);
    for (int i = 0; i < n; i++) cnt[L.agg[i]]++;
    // resolve in dependency order (a parent is a root or attached earlier)
    std::vector<int> stack;
    for (int i = 0; i < n; i++) {
        if (done[i]) continue;
        stack.clear();
        int k = i;
        while (k >= 0 && !done[k]) { stack.push_back(k); k = parent[k]; }
        for (int s = (int)stack.size() - 1; s >= 0; s--) {
            int v = stack[s];
            int pv = parent[v];
            if (pv < 0) {
                t[v] = 1.0;
            } else {
                std::complex<double> a(0, 0);
                for (int p = A.ptr[v]; p < A.ptr[v + 1]; p++) if (A.col[p] == pv) { a = A.val[p]; break; }
                double m = std::abs(a);
                t[v] = m > 0 ? -(a / m) * t[pv] : t[pv];
            }
            done[v] = 1;
        }
    }
    L.T.resize(n);
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
    // Galerkin coarse operator (rows = aggregates)
    next.n = na;
    build_rows_parallel<std::complex<double>>(
        na, na,
        [&](int a, auto add) {
            for (int m = L.mptr[a]; m < L.mptr[a + 1]; m++) {
                const int i = L.mem[m];
                const std::complex<double> ti = std::conj(L.T[i]);
                for (int p = A.ptr[i]; p < A.ptr[i + 1]; p++) {
                    const int j = A.col[p];
                    add(L.agg[j], ti * A.val[p] * L.T[j]);
                }
            }
        },
        next.ptr, next.col, next.val);
    for (int a = 0; a < na; a++)      // Hermitian diagonal
        for (int p = next.ptr[a]; p < next.ptr[a + 1]; p++)
            if (next.col[p] == a) next.val[p] = std::complex<double>(next.val[p].real(), 0.0);
}

// Hermitian positive definite inverse (complex Cholesky), returns false if not HPD.
inline bool hpd_inverse(std::vector<std::complex<double>>& A, int n) {
    using cd = std::complex<double>;
    std::vector<cd> L(A);
    for (int j = 0; j < n; j++) {
        double d = L[(size_t)j * n + j].real();
        for (int k = 0; k < j; k++) d -= std::norm(L[(size_t)j * n + k]);
        if (!(d > 0)) return false;
        d = std::sqrt(d);
        L[(size_t)j * n + j] = d;
        for (int i = j + 1; i < n; i++) {
            cd s = L[(size_t)i * n + j];
            for (int k = 0; k < j; k++) s -= L[(size_t)i * n + k] * std::conj(L[(size_t)j * n + k]);
            L[(size_t)i * n + j] = s / d;
        }
    }
    std::vector<cd> inv((size_t)n * n, 0.0), y(n);
    for (int col = 0; col < n; col++) {
        for (int i = 0; i < n; i++) {
            cd s = i == col ? cd(1, 0) : cd(0, 0);
            for (int k = 0; k < i; k++) s -= L[(size_t)i * n + k] * y[k];
            y[i] = s / L[(size_t)i * n + i].real();
        }
        for (int i = n - 1; i >= 0; i--) {
            cd s = y[i];
            for (int k = i + 1; k < n; k++) s -= std::conj(L[(size_t)k * n + i]) * inv[(size_t)k * n + col];
            inv[(size_t)i * n + col] = s / L[(size_t)i * n + i].real();
        }
    }
    A.swap(inv);
    return true;
}

// Builds the hierarchy from the level-0 ELL rows (nbr[3*f+j], val[j*n+f], diag d).  The cycle
// operators R, S, P are formed for levels >= first_ops (the device applies level 0 directly from
// the ELL rows, the aggregates and T).
inline bool build_hierarchy(int n, const std::vector<int>& nbr3, const std::vector<std::complex<double>>& vals,
                            double diag, HostHierarchy& H, int first_ops = 0) {
    H.lv.clear();
    HostCsr A0;
    A0.n = n;
    A0.ptr.resize(n + 1);
    A0.col.resize(4 * (size_t)n);
    A0.val.resize(4 * (size_t)n);
#pragma omp parallel for schedule(static)
    for (int f = 0; f < n; f++) {
        A0.ptr[f] = 4 * f;
        struct E { int c; std::complex<double> v; } e[4];
        e[0] = {f, std::complex<double>(diag, 0)};
        for (int j = 0; j < 3; j++) e[1 + j] = {nbr3[3 * f + j], vals[(size_t)j * n + f]};
        std::sort(e, e + 4, [](const E& a, const E& b) { return a.c < b.c; });
        for (int k = 0; k < 4; k++) { A0.col[4 * (size_t)f + k] = e[k].c; A0.val[4 * (size_t)f + k] = e[k].v; }
    }
    A0.ptr[n] = 4 * n;
    HostCsr cur = std::move(A0);
    while (cur.n > kCoarseMax && (int)H.lv.size() < kMaxLevels - 1) {
        HostLevel L;
        L.A = std::move(cur);
        HostCsr next;
        aggregate_level(L, next);
        if (next.n >= L.A.n) return false;   // no coarsening
        H.lv.push_back(std::move(L));
        cur = std::move(next);
    }
    if (cur.n > kCoarseMax) return false;
    H.nc = cur.n;
    // cycle operators
    using cd = std::complex<double>;
    const double omega = kOmega, alpha = kAlpha;
    H.ops.resize(H.lv.size());
    for (size_t l = (size_t)std::max(first_ops, 0); l < H.lv.size(); l++) {
        const HostLevel& L = H.lv[l];
        const HostCsr& A = L.A;
        const int n = A.n;
        const int na = (int)L.mptr.size() - 1;
        HostCycleOps& O = H.ops[l];
        // S: same pattern as A
        O.S.n = n;
        O.S.ptr = A.ptr;
        O.S.col = A.col;
        O.S.val.resize(A.val.size());
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; i++)
            for (int p = A.ptr[i]; p < A.ptr[i + 1]; p++) {
                int j = A.col[p];
                cd v = -A.val[p] * (omega * L.dinv[j]);
                if (j == i) v += 2.0;
                O.S.val[p] = omega * L.dinv[i] * v;
            }
        // P: row i -> aggregates of i and of its neighbours
        O.P.n = n;
        build_rows_parallel<cd>(
            n, na,
            [&](int i, auto add) {
                add(L.agg[i], alpha * L.T[i]);
                for (int p = A.ptr[i]; p < A.ptr[i + 1]; p++) {
                    int j = A.col[p];
                    add(L.agg[j], -alpha * omega * L.dinv[i] * A.val[p] * L.T[j]);
                }
            },
            O.P.ptr, O.P.col, O.P.val);
        // R = P^H / alpha
        O.R.n = na;
        O.R.ptr.assign(na + 1, 0);
        for (int b : O.P.col) O.R.ptr[b + 1]++;
        for (int a = 0; a < na; a++) O.R.ptr[a + 1] += O.R.ptr[a];
        O.R.col.resize(O.P.col.size());
        O.R.val.resize(O.P.col.size());
        std::vector<int> fill(O.R.ptr.begin(), O.R.ptr.end() - 1);
        for (int i = 0; i < n; i++)
            for (int p = O.P.ptr[i]; p < O.P.ptr[i + 1]; p++) {
                int a = O.P.col[p];
                int q = fill[a]++;
                O.R.col[q] = i;
                O.R.val[q] = std::conj(O.P.val[p]) / alpha;
            }
    }
    H.Ainv.assign((size_t)cur.n * cur.n, 0.0);
    for (int i = 0; i < cur.n; i++)
        for (int p = cur.ptr[i]; p < cur.ptr[i + 1]; p++) H.Ainv[(size_t)i * cur.n + cur.col[p]] = cur.val[p];
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
    T dinv;              // 1 / diagonal (every row of a closed mesh has three neighbours)
    T omega, alpha;
};

template <typename V2> __device__ __forceinline__ V2 cmulv(V2 a, V2 b) {
    V2 o; o.x = a.x * b.x - a.y * b.y; o.y = a.x * b.y + a.y * b.x; return o;
}
template <typename V2> __device__ __forceinline__ V2 cconjmul(V2 a, V2 b) {   // conj(a) * b
    V2 o; o.x = a.x * b.x + a.y * b.y; o.y = a.x * b.y - a.y * b.x; return o;
}

}  // namespace mtk
