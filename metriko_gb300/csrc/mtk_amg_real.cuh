// Smoothed-aggregation multigrid for the free-variable block of the IGM normal operator.
//
// K_yy = 2 W_y^T S W_y couples the two parametric functions (u, v) of every raw vertex; away
// from seams the 2x2 block between two vertices is a multiple of the identity and the smooth
// (near-null) vectors are the constants of each function.  Across a seam the transition
// rotates (u, v), so aggregation only follows identity-coupled vertex pairs: no aggregate
// straddles a seam rotation, and constants per component stay the right near-null vectors.
// Coarse dofs are (aggregate, component).  The tentative prolongation is smoothed by one
// Jacobi step, coarse operators are Galerkin products with the smoothed prolongation, and the
// V(1,1) cycle is written as R / S / P sparse operators per level:
//   down r_{l+1} = R r_l,  up y_l = S r_l + P y_{l+1}.
#pragma once
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "mtk_amg.cuh"
#include "mtk_ctx.cuh"

namespace mtk {

constexpr int kRMaxLevels = 8;
constexpr int kRCoarseMax = 512;

struct RCsr {
    int n = 0;
    std::vector<int> ptr, col;
    std::vector<double> val;
};

struct RLevel {
    RCsr A;
    std::vector<int> node, comp;   // dof -> node, component
    int nnode = 0;
    std::vector<int> agg;          // dof -> coarse dof
    std::vector<double> T;         // dof -> prolongation weight
    std::vector<double> dinv;
};

struct RCycleOps { RCsr R, S, P; };

struct RHierarchy {
    std::vector<RLevel> lv;
    std::vector<RCycleOps> ops;
    int nc = 0;
    std::vector<double> Ainv;
};

inline double rcsr_at(const RCsr& A, int i, int j) {
    auto b = A.col.begin() + A.ptr[i], e = A.col.begin() + A.ptr[i + 1];
    auto it = std::lower_bound(b, e, j);
    return (it != e && *it == j) ? A.val[A.ptr[i] + (it - A.col.begin() - A.ptr[i])] : 0.0;
}

// Aggregation of one level.  Fills L.agg (dof -> coarse dof), L.T (tentative prolongation
// weight 1/sqrt|aggregate|, so T has orthonormal columns), L.dinv, and the coarse dof ->
// (node, comp) map.  Returns the number of coarse dofs.
inline int raggregate(RLevel& L, std::vector<int>& cnode, std::vector<int>& ccomp, int& cnnode) {
    const RCsr& A = L.A;
    const int n = A.n, nn = L.nnode;
    std::vector<int> nd0(nn, -1), nd1(nn, -1);
#pragma omp parallel for schedule(static)
    for (int d = 0; d < n; d++) (L.comp[d] == 0 ? nd0 : nd1)[L.node[d]] = d;   // (node, comp) -> dof is one to one
    auto paired = [&](int v) { return nd0[v] >= 0 && nd1[v] >= 0; };
    // identity-coupled node neighbours (the 2x2 block between the two nodes is a multiple of I)
    std::vector<int> nptr(nn + 1, 0), nadj;
    {
        auto coupled = [&](int v, int p) {
            const int e = A.col[p], w = L.node[e];
            if (w == v || L.comp[e] != 0 || !paired(w)) return false;
            const double uu = A.val[p];
            const double vv = rcsr_at(A, nd1[v], nd1[w]);
            const double uv = rcsr_at(A, nd0[v], nd1[w]), vu = rcsr_at(A, nd1[v], nd0[w]);
            const double sm = std::fabs(uu) + std::fabs(vv);
            if (sm == 0) return false;
            return !(std::fabs(uv) + std::fabs(vu) > 1e-9 * sm || std::fabs(uu - vv) > 1e-9 * sm);
        };
        // one test per entry of the comp-0 rows (flags), then counts and the list from the flags
        std::vector<unsigned char> flag(A.col.size(), 0);
#pragma omp parallel for schedule(static)
        for (int v = 0; v < nn; v++) {
            int cnt = 0;
            if (paired(v))
                for (int p = A.ptr[nd0[v]]; p < A.ptr[nd0[v] + 1]; p++)
                    if (coupled(v, p)) { flag[p] = 1; cnt++; }
            nptr[v + 1] = cnt;
        }
        for (int v = 0; v < nn; v++) nptr[v + 1] += nptr[v];
        nadj.resize(nptr[nn]);
#pragma omp parallel for schedule(static)
        for (int v = 0; v < nn; v++) {
            if (!paired(v)) continue;
            int q = nptr[v];
            for (int p = A.ptr[nd0[v]]; p < A.ptr[nd0[v] + 1]; p++)
                if (flag[p]) nadj[q++] = L.node[A.col[p]];
        }
    }
    // visiting order: breadth-first over the identity-coupled graph, so that roots are packed
    // next to each other whatever the input numbering (index order on a subdivided mesh puts the
    // coarse vertices first and leaves large remainders for pass 2)
    std::vector<int> order;
    order.reserve(nn);
    {
        std::vector<char> seen(nn, 0);
        for (int s0 = 0; s0 < nn; s0++) {
            if (seen[s0]) continue;
            seen[s0] = 1;
            size_t head = order.size();
            order.push_back(s0);
            while (head < order.size()) {
                const int v = order[head++];
                for (int p = nptr[v]; p < nptr[v + 1]; p++)
                    if (!seen[nadj[p]]) { seen[nadj[p]] = 1; order.push_back(nadj[p]); }
            }
        }
    }
    std::vector<int> nagg(nn, -1);
    int na = 0;
    for (int v : order) {   // pass 1: a free node with free neighbours roots an aggregate
        if (nagg[v] >= 0 || !paired(v)) continue;
        bool ok = true;
        for (int p = nptr[v]; p < nptr[v + 1]; p++) if (nagg[nadj[p]] >= 0) { ok = false; break; }
        if (!ok) continue;
        nagg[v] = na;
        for (int p = nptr[v]; p < nptr[v + 1]; p++) nagg[nadj[p]] = na;
        na++;
    }
    std::vector<int> size(na, 0);
    for (int v = 0; v < nn; v++) if (nagg[v] >= 0) size[nagg[v]]++;
    std::vector<int> attach(nn, -1);
    for (int v : order) {   // pass 2: join the smallest neighbouring pass-1 aggregate
        if (nagg[v] >= 0 || !paired(v)) continue;
        int best = -1;
        for (int p = nptr[v]; p < nptr[v + 1]; p++) {
            const int a2 = nagg[nadj[p]];
            if (a2 >= 0 && (best < 0 || size[a2] < size[best])) best = a2;
        }
        attach[v] = best;
    }
    for (int v = 0; v < nn; v++)
        if (attach[v] >= 0) { nagg[v] = attach[v]; size[attach[v]]++; }
    for (int v : order) {   // pass 3: what is left forms aggregates with its free neighbours
        if (nagg[v] >= 0) continue;
        nagg[v] = na;
        int cnt = 1;
        for (int p = nptr[v]; p < nptr[v + 1]; p++) if (nagg[nadj[p]] < 0) { nagg[nadj[p]] = na; cnt++; }
        size.push_back(cnt);
        na++;
    }
    // coarse dofs: (aggregate, comp) for the comps present, numbered by aggregate
    std::vector<int> cd0(na, -1), cd1(na, -1);
    for (int v = 0; v < nn; v++) {
        const int a2 = nagg[v];
        if (nd0[v] >= 0) cd0[a2] = 0;
        if (nd1[v] >= 0) cd1[a2] = 0;
    }
    cnnode = na;
    cnode.clear();
    ccomp.clear();
    int ncd = 0;
    for (int a2 = 0; a2 < na; a2++) {
        if (cd0[a2] >= 0) { cd0[a2] = ncd++; cnode.push_back(a2); ccomp.push_back(0); }
        if (cd1[a2] >= 0) { cd1[a2] = ncd++; cnode.push_back(a2); ccomp.push_back(1); }
    }
    L.agg.resize(n);
    L.T.resize(n);
    L.dinv.resize(n);
#pragma omp parallel for schedule(static)
    for (int d = 0; d < n; d++) {
        const int a2 = nagg[L.node[d]];
        L.agg[d] = L.comp[d] == 0 ? cd0[a2] : cd1[a2];
        L.T[d] = 1.0 / std::sqrt((double)size[a2]);
        const double dg = rcsr_at(A, d, d);
        L.dinv[d] = dg > 0 ? 1.0 / dg : 1.0;
    }
    return ncd;
}

// Transpose of an n x m CSR.  Threads count the columns of contiguous row blocks, offsets are
// laid out block by block, so every output row lists its entries in ascending input row: the
// same arrays as a serial transpose, for any thread count.
inline RCsr rcsr_transpose(const RCsr& M, int m) {
    RCsr Tm;
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
            for (int a = 0; a < m; a++) {   // cnt becomes the write offset of each block
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
                Tm.val[q] = M.val[p];
            }
    }
    return Tm;
}

// Inverse of an SPD matrix (n x n, row-major) by Cholesky; false if not SPD.  The updates of a
// column and the n substitutions are independent, so both run in parallel (same arithmetic as
// the serial order: every entry is still a sequential sum).
inline bool spd_inverse_dense(std::vector<double>& A, int n) {
    std::vector<double> L(A);
    bool ok = true;
    for (int j = 0; j < n && ok; j++) {
        double d = L[(size_t)j * n + j];
        for (int k = 0; k < j; k++) d -= L[(size_t)j * n + k] * L[(size_t)j * n + k];
        if (!(d > 0)) { ok = false; break; }
        d = std::sqrt(d);
        L[(size_t)j * n + j] = d;
#pragma omp parallel for schedule(static) if (n - j > 64)
        for (int i = j + 1; i < n; i++) {
            double s = L[(size_t)i * n + j];
            for (int k = 0; k < j; k++) s -= L[(size_t)i * n + k] * L[(size_t)j * n + k];
            L[(size_t)i * n + j] = s / d;
        }
    }
    if (!ok) return false;
    std::vector<double> inv((size_t)n * n, 0.0);
#pragma omp parallel
    {
        std::vector<double> y(n), xcol(n);
#pragma omp for schedule(static)
        for (int col = 0; col < n; col++) {
            for (int i = 0; i < n; i++) {
                double s = i == col ? 1.0 : 0.0;
                for (int k = 0; k < i; k++) s -= L[(size_t)i * n + k] * y[k];
                y[i] = s / L[(size_t)i * n + i];
            }
            for (int i = n - 1; i >= 0; i--) {
                double s = y[i];
                for (int k = i + 1; k < n; k++) s -= L[(size_t)k * n + i] * xcol[k];
                xcol[i] = s / L[(size_t)i * n + i];
            }
            for (int i = 0; i < n; i++) inv[(size_t)i * n + col] = xcol[i];
        }
    }
    A.swap(inv);
    return true;
}

// Smoothed-aggregation hierarchy.  Per level: aggregates and T (raggregate), rho = the spectral
// radius of D^-1 A (power estimate), the smoothed prolongator P_sa = (I - w_p D^-1 A) T with
// w_p = (4/3) / rho, and the Galerkin coarse operator P_sa^T A P_sa.  Cycle operators (V(1,1),
// Jacobi weight omega = min(omega_cap, 1.5 / rho), so omega rho <= 1.5 < 2 keeps the smoother
// convergent; coarse correction scaled by alpha):
//   R = P_sa^T (I - omega A D^-1),  S = omega D^-1 (2 I - A omega D^-1),
//   P = alpha (I - omega D^-1 A) P_sa = alpha (P_sa - omega D^-1 (A P_sa)) = alpha R^T.
inline bool build_real_hierarchy(RCsr A0, std::vector<int> node, std::vector<int> comp, int nnode, RHierarchy& H,
                                 double omega_cap = 1.0, double alpha = 1.0) {
    H.lv.clear();
    H.ops.clear();
    RLevel cur;
    cur.A = std::move(A0);
    cur.node = std::move(node);
    cur.comp = std::move(comp);
    cur.nnode = nnode;
    while (cur.A.n > kRCoarseMax && (int)H.lv.size() < kRMaxLevels - 1) {
        std::vector<int> cn, cc;
        int cnn = 0;
        const int na = raggregate(cur, cn, cc, cnn);
        if (na >= cur.A.n * 0.9) return false;   // stalled coarsening
        const RCsr& A = cur.A;
        const int n = A.n;
        // spectral radius of D^-1 A: 12 power steps (Rayleigh quotient in the D inner product) from
        // a fixed oscillating start; the estimate is below rho, so it is raised by 5 percent
        double rho = 0;
        {
            std::vector<double> v(n), w(n);
#pragma omp parallel for schedule(static)
            for (int i = 0; i < n; i++) v[i] = (i & 1) ? 1.0 : -1.0 + 0.25 * (double)(((unsigned)i * 7919u) % 5u);
            for (int it = 0; it < 12; it++) {
                double red[3];   // v^T A v, v^T D v, |w|^2
                det_row_sums<3>(
                    n,
                    [&](int i, double* acc) {
                        double av = 0;
                        for (int p = A.ptr[i]; p < A.ptr[i + 1]; p++) av += A.val[p] * v[A.col[p]];
                        w[i] = cur.dinv[i] * av;
                        acc[0] += v[i] * av;
                        acc[1] += v[i] * v[i] / cur.dinv[i];
                        acc[2] += w[i] * w[i];
                    },
                    red);
                rho = red[1] > 0 ? red[0] / red[1] : 0.0;
                const double sc = red[2] > 0 ? 1.0 / std::sqrt(red[2]) : 0.0;
#pragma omp parallel for schedule(static)
                for (int i = 0; i < n; i++) v[i] = w[i] * sc;
            }
            rho *= 1.05;
        }
        const double wp = rho > 0 ? (4.0 / 3.0) / rho : 0.0;
        const double omega = rho > 0 ? std::min(omega_cap, 1.5 / rho) : omega_cap;
        RCsr Psa, AP;
        Psa.n = n;
        build_rows_parallel<double>(
            n, na,
            [&](int i, auto add) {
                add(cur.agg[i], cur.T[i]);
                for (int p = A.ptr[i]; p < A.ptr[i + 1]; p++)
                    add(cur.agg[A.col[p]], -wp * cur.dinv[i] * A.val[p] * cur.T[A.col[p]]);
            },
            Psa.ptr, Psa.col, Psa.val);
        AP.n = n;
        build_rows_parallel<double>(
            n, na,
            [&](int i, auto add) {
                for (int p = A.ptr[i]; p < A.ptr[i + 1]; p++) {
                    const int k = A.col[p];
                    for (int q = Psa.ptr[k]; q < Psa.ptr[k + 1]; q++) add(Psa.col[q], A.val[p] * Psa.val[q]);
                }
            },
            AP.ptr, AP.col, AP.val);
        const RCsr Pt = rcsr_transpose(Psa, na);
        RLevel nxt;
        nxt.A.n = na;
        build_rows_parallel<double>(
            na, na,
            [&](int a2, auto add) {
                for (int t = Pt.ptr[a2]; t < Pt.ptr[a2 + 1]; t++) {
                    const int i = Pt.col[t];
                    const double pv = Pt.val[t];
                    for (int q = AP.ptr[i]; q < AP.ptr[i + 1]; q++) add(AP.col[q], pv * AP.val[q]);
                }
            },
            nxt.A.ptr, nxt.A.col, nxt.A.val);
        // cycle operators of this level
        RCycleOps O;
        O.S.n = n;
        O.S.ptr = A.ptr;
        O.S.col = A.col;
        O.S.val.resize(A.val.size());
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; i++)
            for (int p = A.ptr[i]; p < A.ptr[i + 1]; p++) {
                const int j = A.col[p];
                double v = -A.val[p] * omega * cur.dinv[j];
                if (j == i) v += 2.0;
                O.S.val[p] = omega * cur.dinv[i] * v;
            }
        // P row i = alpha (Psa row - omega dinv_i AP row): merge of two column-sorted rows
        O.P.n = n;
        O.P.ptr.assign(n + 1, 0);
        auto merge_row = [&](int i, int* oc, double* ov) {
            int a = Psa.ptr[i], ae = Psa.ptr[i + 1], b = AP.ptr[i], be = AP.ptr[i + 1], k = 0;
            const double sb = -alpha * omega * cur.dinv[i];
            while (a < ae || b < be) {
                int c2;
                double v = 0;
                if (b >= be || (a < ae && Psa.col[a] < AP.col[b])) { c2 = Psa.col[a]; v = alpha * Psa.val[a++]; }
                else if (a >= ae || AP.col[b] < Psa.col[a]) { c2 = AP.col[b]; v = sb * AP.val[b++]; }
                else { c2 = Psa.col[a]; v = alpha * Psa.val[a++] + sb * AP.val[b++]; }
                if (oc) { oc[k] = c2; ov[k] = v; }
                k++;
            }
            return k;
        };
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; i++) O.P.ptr[i + 1] = merge_row(i, nullptr, nullptr);
        for (int i = 0; i < n; i++) O.P.ptr[i + 1] += O.P.ptr[i];
        O.P.col.resize(O.P.ptr[n]);
        O.P.val.resize(O.P.ptr[n]);
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; i++) merge_row(i, O.P.col.data() + O.P.ptr[i], O.P.val.data() + O.P.ptr[i]);
        O.R = rcsr_transpose(O.P, na);
        for (double& v : O.R.val) v /= alpha;
        H.ops.push_back(std::move(O));
        H.lv.push_back(std::move(cur));
        cur = std::move(nxt);
        cur.node = std::move(cn);
        cur.comp = std::move(cc);
        cur.nnode = cnn;
    }
    if (cur.A.n > kRCoarseMax) return false;
    H.nc = cur.A.n;
    H.Ainv.assign((size_t)H.nc * H.nc, 0.0);
    for (int i = 0; i < H.nc; i++)
        for (int p = cur.A.ptr[i]; p < cur.A.ptr[i + 1]; p++) H.Ainv[(size_t)i * H.nc + cur.A.col[p]] = cur.A.val[p];
    for (int i = 0; i < H.nc; i++)   // symmetrise the round-off of the Galerkin products
        for (int j = 0; j < i; j++) {
            const double m = 0.5 * (H.Ainv[(size_t)i * H.nc + j] + H.Ainv[(size_t)j * H.nc + i]);
            H.Ainv[(size_t)i * H.nc + j] = m;
            H.Ainv[(size_t)j * H.nc + i] = m;
        }
    return spd_inverse_dense(H.Ainv, H.nc);
}

// ------------------------------------------------------------------ device side
template <typename T>
struct RDevCsr {
    int n, group;
    const int* ptr;
    const int* col;
    const T* val;
    // SELL-32 copy (mtk_sell.cuh), used by the one-lane-per-row phases when present
    const int* sptr = nullptr;
    const int* scol = nullptr;
    const T* sval = nullptr;
};

template <typename T>
struct RDevLevel {
    RDevCsr<T> R, S, P;
    T* r;
    T* y;
};

template <typename T>
struct RDevHierarchy {
    int nlev;
    RDevLevel<T> L[kRMaxLevels];
    int nc;
    const T* Ainv;
    T* rc;
    T* yc;
};

template <typename T>
__device__ __forceinline__ T rcsr_row(const RDevCsr<T>& M, int row, int lane, int g, const T* __restrict__ x) {
    T s = T(0);
    const int e = __ldg(M.ptr + row + 1);
    for (int p = __ldg(M.ptr + row) + lane; p < e; p += 4 * g) {   // four loads in flight per lane
        int c[4];
        T v[4], xv[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const int pu = p + u * g;
            c[u] = pu < e ? __ldg(M.col + pu) : -1;
            v[u] = pu < e ? __ldg(M.val + pu) : T(0);
        }
#pragma unroll
        for (int u = 0; u < 4; u++) xv[u] = c[u] >= 0 ? __ldcg(x + c[u]) : T(0);
#pragma unroll
        for (int u = 0; u < 4; u++)
            if (c[u] >= 0) s += v[u] * xv[u];
    }
    return s;
}

// Row sum of the SELL-32 copy: the lane of `row` within its slice walks the row's entries in
// CSR order, four loads in flight, each load coalesced across the slice's 32 lanes.
template <typename T>
__device__ __forceinline__ T rsell_row(const RDevCsr<T>& M, int row, const T* __restrict__ x) {
    T s = T(0);
    const int sl = row >> 5;
    const int e = __ldg(M.sptr + sl + 1);
    for (int p = __ldg(M.sptr + sl) + (row & 31); p < e; p += 4 * 32) {
        int c[4];
        T v[4], xv[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const int pu = p + u * 32;
            c[u] = pu < e ? __ldg(M.scol + pu) : -1;
            v[u] = pu < e ? __ldg(M.sval + pu) : T(0);
        }
#pragma unroll
        for (int u = 0; u < 4; u++) xv[u] = c[u] >= 0 ? __ldcg(x + c[u]) : T(0);
#pragma unroll
        for (int u = 0; u < 4; u++)
            if (c[u] >= 0) s += v[u] * xv[u];
    }
    return s;
}

template <typename T>
__device__ __forceinline__ T rrow1(const RDevCsr<T>& M, int row, const T* __restrict__ x) {
    return M.sptr ? rsell_row(M, row, x) : rcsr_row(M, row, 0, 1, x);
}

// out[row] = scale * (M x + M2 x2); mask (may be null) zeroes rows where mask != 0.  Rows are
// spread over groups of M.group lanes (1..32) with a warp-uniform loop and fixed-order reduction.
template <typename T>
__device__ void rcsr_phase(const RDevCsr<T>& M, const T* x, const RDevCsr<T>* M2, const T* x2, T* out, T scale,
                           const unsigned char* mask, T* xdot = nullptr, const __half* phi = nullptr, int nphi = 0,
                           const T* yc = nullptr) {
    const int stride = gridDim.x * blockDim.x;
    const int t0 = blockIdx.x * blockDim.x + threadIdx.x;
    const int g = M.group;
    // optional extra term out += sum_k phi[row kp + k] yc[k] (phi row-major FP16, each row padded
    // to kp = nphi rounded up to 8 entries: one 16-byte load per 8 columns; yc replicated)
    const int kp = (nphi + 7) & ~7;
    auto extra = [&](int row) {
        T e = T(0);
        for (int k0 = 0; k0 < nphi; k0 += 8) {
            const uint4 v = __ldg(reinterpret_cast<const uint4*>(phi + (size_t)row * kp + k0));
            const __half2* h2 = reinterpret_cast<const __half2*>(&v);
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const float2 f = __half22float2(h2[q]);
                if (k0 + 2 * q < nphi) e += (T)f.x * yc[k0 + 2 * q];
                if (k0 + 2 * q + 1 < nphi) e += (T)f.y * yc[k0 + 2 * q + 1];
            }
        }
        return e;
    };
    if (g == 1) {
        for (int row = t0; row < M.n; row += stride) {
            T s = rrow1(M, row, x);
            if (M2) s += rrow1(*M2, row, x2);
            const T o = (mask && mask[row]) ? T(0) : (phi ? scale * s + extra(row) : scale * s);
            out[row] = o;
            if (xdot) *xdot += __ldcg(x + row) * o;
        }
        return;
    }
    const int lane = threadIdx.x & 31, gpw = 32 / g, sub = lane / g, sl = lane % g;
    for (int rbase = (t0 >> 5) * gpw; rbase < M.n; rbase += (stride >> 5) * gpw) {   // warp-uniform
        const int row = rbase + sub;
        T s = T(0);
        if (row < M.n) {
            s = rcsr_row(M, row, sl, g, x);
            if (M2) s += rcsr_row(*M2, row, sl, g, x2);
        }
        for (int o = g >> 1; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (sl == 0 && row < M.n) {
            const T o = (mask && mask[row]) ? T(0) : (phi ? scale * s + extra(row) : scale * s);
            out[row] = o;
            if (xdot) *xdot += __ldcg(x + row) * o;
        }
    }
}

// z = out_scale * B r on the hierarchy; level 0 reads H.L[0].r and writes H.L[0].y (masked);
// rz (may be null) accumulates this thread's share of r . z.  With phi (row-major FP16, nphi
// columns, rows padded to a multiple of 8) the level-0 output also gets phi * yc, in the same
// pass.
template <typename T>
__device__ bool rvcycle(const RDevHierarchy<T>& H, T out_scale, const unsigned char* mask0, const GridBarrier& bar,
                        T* rz = nullptr, const __half* phi = nullptr, int nphi = 0, const T* yc = nullptr) {
    const int stride = gridDim.x * blockDim.x;
    const int t0 = blockIdx.x * blockDim.x + threadIdx.x;
    for (int l = 0; l < H.nlev; l++) {
        T* rnext = (l + 1 < H.nlev) ? H.L[l + 1].r : H.rc;
        rcsr_phase<T>(H.L[l].R, H.L[l].r, nullptr, nullptr, rnext, T(1), nullptr);
        if (!grid_sync(bar)) return false;
    }
    {
        const int lane = threadIdx.x & 31;
        for (int a = t0 >> 5; a < H.nc; a += stride >> 5) {
            T s = T(0);
            const T* row = H.Ainv + (size_t)a * H.nc;
            for (int b = lane; b < H.nc; b += 32) s += row[b] * __ldcg(H.rc + b);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if (lane == 0) H.yc[a] = s;
        }
    }
    if (!grid_sync(bar)) return false;
    for (int l = H.nlev - 1; l >= 0; l--) {
        const T* yn = (l + 1 < H.nlev) ? H.L[l + 1].y : H.yc;
        rcsr_phase<T>(H.L[l].S, H.L[l].r, &H.L[l].P, yn, H.L[l].y, l == 0 ? out_scale : T(1), l == 0 ? mask0 : nullptr,
                      l == 0 ? rz : nullptr, l == 0 ? phi : nullptr, nphi, yc);
        if (l > 0 && !grid_sync(bar)) return false;
    }
    return true;
}

}  // namespace mtk
