// Aggregation multigrid for the free-variable block of the IGM normal operator.
//
// K_yy = 2 W_y^T S W_y couples the two parametric functions (u, v) of every raw vertex; away
// from seams the 2x2 block between two vertices is a multiple of the identity and the smooth
// (near-null) vectors are the constants of each function.  Across a seam the transition
// rotates (u, v), so aggregation only follows identity-coupled vertex pairs: no aggregate
// straddles a seam rotation, and constants per component stay the right near-null vectors.
// Coarse dofs are (aggregate, component); the coarse operators are Galerkin products, and the
// V(1,1) cycle is written as R / S / P sparse operators per level exactly as for the field:
//   down r_{l+1} = R r_l,  up y_l = S r_l + P y_{l+1}.
#pragma once
#include <algorithm>
#include <cmath>
#include <vector>

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

// One coarsening step.  Fills L.agg / L.T / L.dinv, returns the coarse operator and the coarse
// dof -> (node, comp) map.
inline void rcoarsen(RLevel& L, RCsr& next, std::vector<int>& cnode, std::vector<int>& ccomp, int& cnnode) {
    const RCsr& A = L.A;
    const int n = A.n, nn = L.nnode;
    // node dof lists
    std::vector<int> nd0(nn, -1), nd1(nn, -1);
    for (int d = 0; d < n; d++) (L.comp[d] == 0 ? nd0 : nd1)[L.node[d]] = d;
    auto paired = [&](int v) { return nd0[v] >= 0 && nd1[v] >= 0; };
    // identity-coupled node neighbours
    std::vector<int> nptr(nn + 1, 0), nadj;
    {
        std::vector<std::vector<int>> tmp(nn);
        for (int v = 0; v < nn; v++) {
            if (!paired(v)) continue;
            int du = nd0[v], dv = nd1[v];
            for (int p = A.ptr[du]; p < A.ptr[du + 1]; p++) {
                int e = A.col[p];
                int w = L.node[e];
                if (w == v || L.comp[e] != 0 || !paired(w)) continue;
                double uu = A.val[p];
                double vv = rcsr_at(A, dv, nd1[w]);
                double uv = rcsr_at(A, du, nd1[w]), vu = rcsr_at(A, dv, nd0[w]);
                double s = std::fabs(uu) + std::fabs(vv);
                if (s == 0) continue;
                if (std::fabs(uv) + std::fabs(vu) > 1e-9 * s || std::fabs(uu - vv) > 1e-9 * s) continue;
                tmp[v].push_back(w);
            }
        }
        for (int v = 0; v < nn; v++) nptr[v + 1] = nptr[v] + (int)tmp[v].size();
        nadj.reserve(nptr[nn]);
        for (int v = 0; v < nn; v++) nadj.insert(nadj.end(), tmp[v].begin(), tmp[v].end());
    }
    std::vector<int> nagg(nn, -1);
    int na = 0;
    for (int v = 0; v < nn; v++) {   // pass 1
        if (nagg[v] >= 0 || !paired(v)) continue;
        bool ok = true;
        for (int p = nptr[v]; p < nptr[v + 1]; p++) if (nagg[nadj[p]] >= 0) { ok = false; break; }
        if (!ok) continue;
        nagg[v] = na;
        for (int p = nptr[v]; p < nptr[v + 1]; p++) nagg[nadj[p]] = na;
        na++;
    }
    for (int v = 0; v < nn; v++) {   // pass 2
        if (nagg[v] >= 0 || !paired(v)) continue;
        for (int p = nptr[v]; p < nptr[v + 1]; p++)
            if (nagg[nadj[p]] >= 0) { nagg[v] = nagg[nadj[p]]; break; }
    }
    for (int v = 0; v < nn; v++) if (nagg[v] < 0) nagg[v] = na++;   // pass 3
    std::vector<int> size(na, 0);
    for (int v = 0; v < nn; v++) size[nagg[v]]++;
    // coarse dofs: (aggregate, comp) for the comps present
    std::vector<int> cd0(na, -1), cd1(na, -1);
    cnnode = na;
    cnode.clear();
    ccomp.clear();
    for (int v = 0; v < nn; v++) {
        int a = nagg[v];
        if (nd0[v] >= 0 && cd0[a] < 0) { cd0[a] = 0; }
        if (nd1[v] >= 0 && cd1[a] < 0) { cd1[a] = 0; }
    }
    int ncd = 0;
    for (int a = 0; a < na; a++) {
        if (cd0[a] >= 0) { cd0[a] = ncd++; cnode.push_back(a); ccomp.push_back(0); }
        if (cd1[a] >= 0) { cd1[a] = ncd++; cnode.push_back(a); ccomp.push_back(1); }
    }
    L.agg.resize(n);
    L.T.resize(n);
    L.dinv.resize(n);
    for (int d = 0; d < n; d++) {
        int a = nagg[L.node[d]];
        L.agg[d] = L.comp[d] == 0 ? cd0[a] : cd1[a];
        L.T[d] = 1.0 / std::sqrt((double)size[a]);
        double dg = rcsr_at(A, d, d);
        L.dinv[d] = dg > 0 ? 1.0 / dg : 1.0;
    }
    // members of each coarse dof, Galerkin product
    std::vector<int> mptr(ncd + 1, 0), mem(n);
    for (int d = 0; d < n; d++) mptr[L.agg[d] + 1]++;
    for (int a = 0; a < ncd; a++) mptr[a + 1] += mptr[a];
    {
        std::vector<int> fill(mptr.begin(), mptr.end() - 1);
        for (int d = 0; d < n; d++) mem[fill[L.agg[d]]++] = d;
    }
    next.n = ncd;
    build_rows_parallel<double>(
        ncd, ncd,
        [&](int a, auto add) {
            for (int m = mptr[a]; m < mptr[a + 1]; m++) {
                const int i = mem[m];
                for (int p = A.ptr[i]; p < A.ptr[i + 1]; p++) add(L.agg[A.col[p]], L.T[i] * A.val[p] * L.T[A.col[p]]);
            }
        },
        next.ptr, next.col, next.val);
}

inline bool spd_inverse_dense(std::vector<double>& A, int n) {
    std::vector<double> L(A);
    for (int j = 0; j < n; j++) {
        double d = L[(size_t)j * n + j];
        for (int k = 0; k < j; k++) d -= L[(size_t)j * n + k] * L[(size_t)j * n + k];
        if (!(d > 0)) return false;
        d = std::sqrt(d);
        L[(size_t)j * n + j] = d;
        for (int i = j + 1; i < n; i++) {
            double s = L[(size_t)i * n + j];
            for (int k = 0; k < j; k++) s -= L[(size_t)i * n + k] * L[(size_t)j * n + k];
            L[(size_t)i * n + j] = s / d;
        }
    }
    std::vector<double> inv((size_t)n * n, 0.0), y(n);
    for (int col = 0; col < n; col++) {
        for (int i = 0; i < n; i++) {
            double s = i == col ? 1.0 : 0.0;
            for (int k = 0; k < i; k++) s -= L[(size_t)i * n + k] * y[k];
            y[i] = s / L[(size_t)i * n + i];
        }
        for (int i = n - 1; i >= 0; i--) {
            double s = y[i];
            for (int k = i + 1; k < n; k++) s -= L[(size_t)k * n + i] * inv[(size_t)k * n + col];
            inv[(size_t)i * n + col] = s / L[(size_t)i * n + i];
        }
    }
    A.swap(inv);
    return true;
}

// A0: the level-0 operator (symmetric positive definite), node/comp of its dofs.
inline bool build_real_hierarchy(RCsr A0, std::vector<int> node, std::vector<int> comp, int nnode, RHierarchy& H,
                                 double omega = 0.8, double alpha = 1.8) {
    H.lv.clear();
    H.ops.clear();
    RLevel cur;
    cur.A = std::move(A0);
    cur.node = std::move(node);
    cur.comp = std::move(comp);
    cur.nnode = nnode;
    while (cur.A.n > kRCoarseMax && (int)H.lv.size() < kRMaxLevels - 1) {
        RCsr next;
        std::vector<int> cn, cc;
        int cnn = 0;
        rcoarsen(cur, next, cn, cc, cnn);
        if (next.n >= cur.A.n * 0.9) return false;   // stalled coarsening
        H.lv.push_back(std::move(cur));
        cur = RLevel();
        cur.A = std::move(next);
        cur.node = std::move(cn);
        cur.comp = std::move(cc);
        cur.nnode = cnn;
    }
    if (cur.A.n > kRCoarseMax) return false;
    H.nc = cur.A.n;
    H.Ainv.assign((size_t)H.nc * H.nc, 0.0);
    for (int i = 0; i < H.nc; i++)
        for (int p = cur.A.ptr[i]; p < cur.A.ptr[i + 1]; p++) H.Ainv[(size_t)i * H.nc + cur.A.col[p]] = cur.A.val[p];
    if (!spd_inverse_dense(H.Ainv, H.nc)) return false;
    H.ops.resize(H.lv.size());
    for (size_t l = 0; l < H.lv.size(); l++) {
        const RLevel& L = H.lv[l];
        const RCsr& A = L.A;
        const int n = A.n;
        const int na = (l + 1 < H.lv.size()) ? H.lv[l + 1].A.n : H.nc;
        RCycleOps& O = H.ops[l];
        O.S.n = n;
        O.S.ptr = A.ptr;
        O.S.col = A.col;
        O.S.val.resize(A.val.size());
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; i++)
            for (int p = A.ptr[i]; p < A.ptr[i + 1]; p++) {
                int j = A.col[p];
                double v = -A.val[p] * omega * L.dinv[j];
                if (j == i) v += 2.0;
                O.S.val[p] = omega * L.dinv[i] * v;
            }
        O.P.n = n;
        build_rows_parallel<double>(
            n, na,
            [&](int i, auto add) {
                add(L.agg[i], alpha * L.T[i]);
                for (int p = A.ptr[i]; p < A.ptr[i + 1]; p++)
                    add(L.agg[A.col[p]], -alpha * omega * L.dinv[i] * A.val[p] * L.T[A.col[p]]);
            },
            O.P.ptr, O.P.col, O.P.val);
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
                O.R.val[q] = O.P.val[p] / alpha;
            }
    }
    return true;
}

// ------------------------------------------------------------------ device side
template <typename T>
struct RDevCsr {
    int n, group;
    const int* ptr;
    const int* col;
    const T* val;
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
    for (int p = M.ptr[row] + lane; p < M.ptr[row + 1]; p += g) s += M.val[p] * __ldcg(x + M.col[p]);
    return s;
}

// out[row] = scale * (M x + M2 x2); mask (may be null) zeroes rows where mask != 0.  Rows are
// spread over groups of M.group lanes (1..32) with a warp-uniform loop and fixed-order reduction.
template <typename T>
__device__ void rcsr_phase(const RDevCsr<T>& M, const T* x, const RDevCsr<T>* M2, const T* x2, T* out, T scale,
                           const unsigned char* mask) {
    const int stride = gridDim.x * blockDim.x;
    const int t0 = blockIdx.x * blockDim.x + threadIdx.x;
    const int g = M.group;
    if (g == 1) {
        for (int row = t0; row < M.n; row += stride) {
            T s = rcsr_row(M, row, 0, 1, x);
            if (M2) s += rcsr_row(*M2, row, 0, 1, x2);
            out[row] = (mask && mask[row]) ? T(0) : scale * s;
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
        if (sl == 0 && row < M.n) out[row] = (mask && mask[row]) ? T(0) : scale * s;
    }
}

// z = out_scale * B r on the hierarchy; level 0 reads H.L[0].r and writes H.L[0].y (masked).
template <typename T>
__device__ bool rvcycle(const RDevHierarchy<T>& H, T out_scale, const unsigned char* mask0, const GridBarrier& bar) {
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
        rcsr_phase<T>(H.L[l].S, H.L[l].r, &H.L[l].P, yn, H.L[l].y, l == 0 ? out_scale : T(1), l == 0 ? mask0 : nullptr);
        if (l > 0 && !grid_sync(bar)) return false;
    }
    return true;
}

}  // namespace mtk
