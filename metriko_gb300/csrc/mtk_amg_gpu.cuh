// Device build of the complex smoothed-aggregation hierarchy of mtk_amg.cuh (the field's
// connection Laplacian).
//
// CDevBuilder produces the same level-0 data (aggregates, T, w_p), inner-level cycle operators
// (R, S, P) and coarse inverse as build_hierarchy(..., first_ops = 1), bit for bit: the
// aggregation (the greedy passes as rounds of a distance-2 independent-set test, the transport
// along the parent forest), the spectral-radius estimate, P_sa, A P_sa, the Galerkin product
// and the cycle operators run on the device with explicit round-to-nearest operations in the
// order of the host's std::complex<double> arithmetic (a * b = (ac - bd, ad + bc), a real factor
// scales both components, sums start from 0 and follow the host's visit order); only the
// coarsest operator comes back to the host, for its dense inverse.
#pragma once
#include <chrono>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "mtk_amg.cuh"
#include "mtk_amg_real_gpu.cuh"

namespace mtk {

struct DevCsrC {
    int n = 0;
    size_t nnz = 0;
    DBuf<int> ptr, col;
    DBuf<double2> val;
};

struct DevCycleOpsC { DevCsrC R, S, P; };

namespace cgpu {

__device__ __forceinline__ double2 cmul_rn(double2 a, double2 b) {
    return make_double2(__dsub_rn(__dmul_rn(a.x, b.x), __dmul_rn(a.y, b.y)),
                        __dadd_rn(__dmul_rn(a.x, b.y), __dmul_rn(a.y, b.x)));
}
__device__ __forceinline__ double2 rscale(double s, double2 a) { return make_double2(__dmul_rn(s, a.x), __dmul_rn(s, a.y)); }
__device__ __forceinline__ double2 cadd_rn(double2 a, double2 b) { return make_double2(__dadd_rn(a.x, b.x), __dadd_rn(a.y, b.y)); }

// P_sa row i: (agg_i, T_i), then (agg_j, ((-wp dinv_i) A_ij) T_j)
struct PsaVisit {
    const int *Ap, *Ac;
    const double2* Av;
    const int* agg;
    const double2* T;
    const double* dinv;
    double wp;
    template <class Add>
    __device__ void operator()(int i, Add& add) const {
        add(agg[i], T[i]);
        const double a0 = __dmul_rn(-wp, dinv[i]);
        for (int p = Ap[i]; p < Ap[i + 1]; p++) {
            const int j = Ac[p];
            add(agg[j], cmul_rn(rscale(a0, Av[p]), T[j]));
        }
    }
};

// (A B) row i
struct ProdVisit {
    const int *Ap, *Ac;
    const double2* Av;
    const int *Bp, *Bc;
    const double2* Bv;
    template <class Add>
    __device__ void operator()(int i, Add& add) const {
        for (int p = Ap[i]; p < Ap[i + 1]; p++) {
            const int k = Ac[p];
            const double2 a = Av[p];
            for (int q = Bp[k]; q < Bp[k + 1]; q++) add(Bc[q], cmul_rn(a, Bv[q]));
        }
    }
};

// P row i: alpha P_sa row, then ((-alpha omega) dinv_i) (A P_sa) row
struct ProlongVisit {
    const int *Pp, *Pc;
    const double2* Pv;
    const int *Bp, *Bc;
    const double2* Bv;
    const double* dinv;
    double alpha, omega;
    template <class Add>
    __device__ void operator()(int i, Add& add) const {
        for (int q = Pp[i]; q < Pp[i + 1]; q++) add(Pc[q], rscale(alpha, Pv[q]));
        const double sb = __dmul_rn(__dmul_rn(-alpha, omega), dinv[i]);
        for (int q = Bp[i]; q < Bp[i + 1]; q++) add(Bc[q], rscale(sb, Bv[q]));
    }
};

constexpr int kCapRow = 64;

struct SortedAcc {
    int cols[kCapRow];
    double2 vals[kCapRow];
    int cnt = 0;
    int* err;
    __device__ void operator()(int c, double2 v) {
        int lo = 0, hi = cnt;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (cols[mid] < c) lo = mid + 1; else hi = mid;
        }
        if (lo < cnt && cols[lo] == c) { vals[lo] = cadd_rn(vals[lo], v); return; }
        if (cnt >= kCapRow) { *err = 1; return; }
        for (int k = cnt; k > lo; k--) { cols[k] = cols[k - 1]; vals[k] = vals[k - 1]; }
        cols[lo] = c;
        vals[lo] = cadd_rn(make_double2(0.0, 0.0), v);
        cnt++;
    }
};

template <class Visit>
__global__ void rows_sorted(int n, Visit visit, int* cnt_out, const int* __restrict__ optr, int* ocol, double2* oval,
                            int* err) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        SortedAcc acc;
        acc.err = err;
        visit(i, acc);
        if (!optr) { cnt_out[i] = acc.cnt; continue; }
        const int o = optr[i];
        for (int k = 0; k < acc.cnt; k++) { ocol[o + k] = acc.cols[k]; oval[o + k] = acc.vals[k]; }
    }
}

constexpr int kHash = 256;
constexpr int kCapGal = 160;

struct HashAcc {
    int hc[kHash];
    double2 hv[kHash];
    int cnt = 0;
    int* err;
    __device__ void init() { for (int s = 0; s < kHash; s++) hc[s] = -1; }
    __device__ void operator()(int c, double2 v) {
        unsigned h = ((unsigned)c * 2654435761u) & (kHash - 1);
        while (hc[h] >= 0 && hc[h] != c) h = (h + 1) & (kHash - 1);
        if (hc[h] == c) { hv[h] = cadd_rn(hv[h], v); return; }
        if (cnt >= kCapGal) { *err = 1; return; }
        hc[h] = c;
        hv[h] = cadd_rn(make_double2(0.0, 0.0), v);
        cnt++;
    }
};

template <class Visit>
__global__ void __launch_bounds__(128) rows_hash(int n, Visit visit, int* cnt_out, const int* __restrict__ optr, int* ocol,
                                                 double2* oval, int* err) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        HashAcc acc;
        acc.err = err;
        acc.init();
        visit(i, acc);
        if (!optr) { cnt_out[i] = acc.cnt; continue; }
        const int o = optr[i];
        int m = 0;
        for (int s = 0; s < kHash; s++)
            if (acc.hc[s] >= 0) {
                int k = m++;
                while (k > 0 && ocol[o + k - 1] > acc.hc[s]) {
                    ocol[o + k] = ocol[o + k - 1];
                    oval[o + k] = oval[o + k - 1];
                    k--;
                }
                ocol[o + k] = acc.hc[s];
                oval[o + k] = acc.hv[s];
            }
    }
}

struct DenseAcc {
    double2* acc;
    unsigned char* mark;
    int cnt = 0;
    __device__ void operator()(int c, double2 v) {
        if (!mark[c]) { mark[c] = 1; acc[c] = cadd_rn(make_double2(0.0, 0.0), v); cnt++; }
        else acc[c] = cadd_rn(acc[c], v);
    }
};

template <class Visit>
__global__ void rows_dense(int n, int ncols, Visit visit, double2* scratch, unsigned char* marks, int* cnt_out,
                           const int* __restrict__ optr, int* ocol, double2* oval) {
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    double2* acc = scratch + (size_t)tid * ncols;
    unsigned char* mark = marks + (size_t)tid * ncols;
    for (int i = tid; i < n; i += gridDim.x * blockDim.x) {
        DenseAcc a{acc, mark, 0};
        visit(i, a);
        if (!optr) {
            cnt_out[i] = a.cnt;
            for (int c = 0; c < ncols; c++) mark[c] = 0;
            continue;
        }
        int o = optr[i];
        for (int c = 0; c < ncols; c++)
            if (mark[c]) { ocol[o] = c; oval[o] = acc[c]; o++; mark[c] = 0; }
    }
}

// adjoint: fill at atomic positions, then per output row (one warp) each entry to its rank;
// values conjugated and divided by div (div != 1)
static __global__ void adjoint_fill(int n, const int* __restrict__ Mp, const int* __restrict__ Mc,
                                    const double2* __restrict__ Mv, int* fill, int* ucol, double2* uval) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        for (int p = Mp[i]; p < Mp[i + 1]; p++) {
            const int pos = atomicAdd(fill + Mc[p], 1);
            ucol[pos] = i;
            uval[pos] = Mv[p];
        }
}
static __global__ void adjoint_rank(int m, const int* __restrict__ tp, const int* __restrict__ ucol,
                                    const double2* __restrict__ uval, int* tcol, double2* tval, double div) {
    const int lane = threadIdx.x & 31;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    for (int a = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; a < m; a += warps) {
        const int b = tp[a], e = tp[a + 1];
        for (int k = b + lane; k < e; k += 32) {
            const int c = ucol[k];
            int r = 0;
            for (int j = b; j < e; j++) r += ucol[j] < c ? 1 : 0;
            double2 v = make_double2(uval[k].x, -uval[k].y);
            if (div != 1.0) v = make_double2(__ddiv_rn(v.x, div), __ddiv_rn(v.y, div));
            tcol[b + r] = c;
            tval[b + r] = v;
        }
    }
}

// Hermitian diagonal of a Galerkin product: imaginary part of diagonal entries set to 0
static __global__ void real_diagonal(int n, const int* __restrict__ Ap, const int* __restrict__ Ac, double2* Av) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        for (int p = Ap[i]; p < Ap[i + 1]; p++)
            if (Ac[p] == i) Av[p].y = 0.0;
}

// S = omega D^-1 (2 I - A omega D^-1) on the pattern of A
static __global__ void smoother_vals(int n, const int* __restrict__ Ap, const int* __restrict__ Ac,
                                     const double2* __restrict__ Av, const double* __restrict__ dinv, double omega,
                                     double2* Sv) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double di = __dmul_rn(omega, dinv[i]);
        for (int p = Ap[i]; p < Ap[i + 1]; p++) {
            const int j = Ac[p];
            double2 v = rscale(__dmul_rn(omega, dinv[j]), make_double2(-Av[p].x, -Av[p].y));
            if (j == i) v.x = __dadd_rn(v.x, 2.0);
            Sv[p] = rscale(di, v);
        }
    }
}

// dinv_i = 1 / Re A_ii (1 where not positive), as aggregate_level (last diagonal entry wins)
static __global__ void diag_inv(int n, const int* __restrict__ Ap, const int* __restrict__ Ac,
                                const double2* __restrict__ Av, double* dinv) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double d = 0;
        for (int p = Ap[i]; p < Ap[i + 1]; p++)
            if (Ac[p] == i) d = Av[p].x;
        dinv[i] = d > 0 ? __ddiv_rn(1.0, d) : 1.0;
    }
}

static __global__ void rho_start(int n, double2* v) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double re = (i & 1) ? 1.0 : __dadd_rn(-1.0, __dmul_rn(0.25, (double)(((unsigned)i * 7919u) % 5u)));
        v[i] = make_double2(re, __dmul_rn(0.1, (double)(((unsigned)i * 104729u) % 7u)));
    }
}
// per row: w = dinv (A v); terms Re(conj(v) A v), |v|^2 / dinv, |w|^2
static __global__ void rho_rows(int n, const int* __restrict__ Ap, const int* __restrict__ Ac,
                                const double2* __restrict__ Av, const double* __restrict__ dinv,
                                const double2* __restrict__ v, double2* w, double* t3) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double2 av = make_double2(0.0, 0.0);
        for (int p = Ap[i]; p < Ap[i + 1]; p++) av = cadd_rn(av, cmul_rn(Av[p], v[Ac[p]]));
        const double2 wi = rscale(dinv[i], av);
        w[i] = wi;
        const double2 vi = v[i];
        t3[3 * (size_t)i] = __dsub_rn(__dmul_rn(vi.x, av.x), __dmul_rn(-vi.y, av.y));
        t3[3 * (size_t)i + 1] = __ddiv_rn(__dadd_rn(__dmul_rn(vi.x, vi.x), __dmul_rn(vi.y, vi.y)), dinv[i]);
        t3[3 * (size_t)i + 2] = __dadd_rn(__dmul_rn(wi.x, wi.x), __dmul_rn(wi.y, wi.y));
    }
}
static __global__ void scale_vec(int n, const double2* __restrict__ w, const double* __restrict__ sc, double2* v) {
    const double s = *sc;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) v[i] = rscale(s, w[i]);
}
static __global__ void to_f32_vals(size_t n, const double2* __restrict__ a, float2* b) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        b[i] = make_float2((float)a[i].x, (float)a[i].y);
}

// ---------------------------------------------------------------- aggregation (aggregate_level)
// Pass 1 of aggregate_level (rows in index order; a row whose neighbours are all free roots an
// aggregate with them) is the lexicographically first distance-2 independent set of the row
// graph.  It is found in rounds: a node whose closed distance-2 neighbourhood holds no root and
// no lower undecided node becomes a root, a node with a root within distance 2 is covered.  Each
// round is two passes (distance 1, then distance 2) reading the previous pass's arrays only.
// state: 0 undecided, 1 root, 2 covered.
static __global__ void mis_near(int n, const int* __restrict__ Ap, const int* __restrict__ Ac,
                                const signed char* __restrict__ state, int* low1, unsigned char* root1) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const signed char si = state[i];
        int lo = si == 0 ? i : 0x7fffffff;
        unsigned char rt = si == 1;
        for (int p = Ap[i]; p < Ap[i + 1]; p++) {
            const int j = Ac[p];
            if (j == i) continue;
            const signed char sj = state[j];
            if (sj == 0 && j < lo) lo = j;
            if (sj == 1) rt = 1;
        }
        low1[i] = lo;
        root1[i] = rt;
    }
}
static __global__ void mis_decide(int n, const int* __restrict__ Ap, const int* __restrict__ Ac,
                                  const int* __restrict__ low1, const unsigned char* __restrict__ root1,
                                  signed char* state, int* undecided) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (state[i] != 0) continue;
        int lo = low1[i];
        unsigned char rt = root1[i];
        for (int p = Ap[i]; p < Ap[i + 1]; p++) {
            const int j = Ac[p];
            if (j == i) continue;
            lo = min(lo, low1[j]);
            rt |= root1[j];
        }
        if (rt) state[i] = 2;
        else if (lo == i) state[i] = 1;
        else *undecided = 1;
    }
}
static __global__ void root_flags(int n, const signed char* __restrict__ state, int* flag) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) flag[i] = state[i] == 1;
}
// pass 1 assignment: a root and its neighbours (a node has at most one root neighbour)
static __global__ void agg_pass1(int n, const int* __restrict__ Ap, const int* __restrict__ Ac,
                                 const signed char* __restrict__ state, const int* __restrict__ rid, int* agg, int* parent) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int a = -1, pa = -1;
        if (state[i] == 1) {
            a = rid[i];
        } else {
            for (int p = Ap[i]; p < Ap[i + 1]; p++) {
                const int j = Ac[p];
                if (j != i && state[j] == 1) { a = rid[j]; pa = j; break; }
            }
        }
        agg[i] = a;
        parent[i] = pa;
    }
}
// pass 2: a node left over attaches to its strongest neighbour among those aggregated at its
// turn in index order (pass-1 nodes, and pass-2 nodes of lower index); *err when there is none
static __global__ void agg_pass2(int n, const int* __restrict__ Ap, const int* __restrict__ Ac,
                                 const double2* __restrict__ Av, const int* __restrict__ agg1, int* parent, int* err) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (agg1[i] >= 0) continue;
        int best = -1;
        double bw = -1.0;
        for (int p = Ap[i]; p < Ap[i + 1]; p++) {
            const int j = Ac[p];
            if (j == i || (agg1[j] < 0 && j > i)) continue;
            const double2 a = Av[p];
            const double w = __dadd_rn(__dmul_rn(a.x, a.x), __dmul_rn(a.y, a.y));
            if (w > bw) { bw = w; best = j; }
        }
        parent[i] = best;
        if (best < 0) *err = 1;
    }
}
// pass-2 aggregates along the parent chains (each step to a lower index or a pass-1 node)
static __global__ void agg_resolve(int n, const int* __restrict__ parent, const int* __restrict__ prev, int* agg,
                                   int* changed) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (prev[i] >= 0) continue;
        const int a = prev[parent[i]];
        if (a >= 0) { agg[i] = a; *changed = 1; }
    }
}
// transported near-null vector, in rounds of the parent forest: t = 1 at a root,
// t_v = -(a / |a|) t_parent with a the first entry of row v in the parent's column
static __global__ void transport_round(int n, int round, const int* __restrict__ Ap, const int* __restrict__ Ac,
                                       const double2* __restrict__ Av, const int* __restrict__ parent, int* stage,
                                       double2* t, int* changed) {
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        if (stage[v] >= 0) continue;
        const int pv = parent[v];
        if (pv < 0) {
            t[v] = make_double2(1.0, 0.0);
            stage[v] = round;
            *changed = 1;
            continue;
        }
        const int sp = stage[pv];
        if (sp < 0 || sp >= round) continue;
        double2 a = make_double2(0.0, 0.0);
        for (int p = Ap[v]; p < Ap[v + 1]; p++)
            if (Ac[p] == pv) { a = Av[p]; break; }
        const double m = __dsqrt_rn(__dadd_rn(__dmul_rn(a.x, a.x), __dmul_rn(a.y, a.y)));
        t[v] = m > 0 ? cmul_rn(make_double2(-__ddiv_rn(a.x, m), -__ddiv_rn(a.y, m)), t[pv]) : t[pv];
        stage[v] = round;
        *changed = 1;
    }
}
static __global__ void agg_count(int n, const int* __restrict__ agg, int* cnt) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) atomicAdd(cnt + agg[i], 1);
}
static __global__ void t_scale(int n, const int* __restrict__ agg, const int* __restrict__ cnt, double2* t) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double s = __dsqrt_rn((double)cnt[agg[i]]);
        t[i] = make_double2(__ddiv_rn(t[i].x, s), __ddiv_rn(t[i].y, s));
    }
}

}  // namespace cgpu

// Host driver of the complex device build.  Outputs: level 0 (host: aggregates, members, T, w_p),
// the cycle operators of levels 1.. on the device, the coarsest inverse (host).
class CDevBuilder {
   public:
    CDevBuilder(mtk_ctx* c, cudaStream_t st) : c_(c), st_(st) {}

    int build(HostCsr A0, HostLevel& L0, std::vector<DevCycleOpsC>& ops, int& nc, std::vector<std::complex<double>>& Ainv,
              bool& ok) {
        using cd = std::complex<double>;
        ok = false;
        ops.clear();
        const char* dbg = getenv("MTK_DEBUG");
        const bool debug = dbg && dbg[0] == '1';
        auto t0 = std::chrono::steady_clock::now();
        auto lap = [&](const char* what, int lvl) {
            if (!debug) return;
            cudaStreamSynchronize(st_);
            const auto t = std::chrono::steady_clock::now();
            fprintf(stderr, "[mg device]     field level %d %-18s %7.1f ms\n", lvl, what,
                    std::chrono::duration<double, std::milli>(t - t0).count());
            t0 = t;
        };
        MTK_TRY(err_.alloc(1));
        MTK_TRY(err_.zero(st_));
        MTK_TRY(tot_.alloc(1));
        DevCsrC dA;
        MTK_TRY(upload(A0, dA));
        int cur_n = A0.n;
        A0 = HostCsr();
        const double omega = kOmega, alpha = kAlpha;
        int levels = 0;
        while (cur_n > kCoarseMax && levels < kMaxLevels - 1) {
            HostLevel L;
            const int ln = cur_n;
            DBuf<double> dinv;
            MTK_TRY(dinv.alloc(ln));
            cgpu::diag_inv<<<grid(ln), kStream, 0, st_>>>(ln, dA.ptr.p, dA.col.p, dA.val.p, dinv.p);
            MTK_TRY(spectral_radius_launch(dA, dinv.p));
            DBuf<int> agg;
            DBuf<double2> T;
            int na = 0;
            bool agg_ok = false;
            MTK_TRY(aggregate_device(dA, agg, T, na, agg_ok));
            if (!agg_ok || na >= ln) return MTK_OK;
            double rho = 0;
            MTK_TRY(spectral_radius_finish(ln, rho));
            L.wp = rho > 0 ? (4.0 / 3.0) / rho : 0.0;
            lap("aggregate + rho", levels);
            const bool dense = na <= rgpu::kDenseCols;
            if (dense) MTK_TRY(dense_scratch(na));
            DevCsrC Psa, AP, Ph, Ac;
            // rows of level 0 are short (the ELL stencil): sorted arrays; deeper levels: a table, or
            // dense scratch rows when the next level is small
            auto rows = [&](int nr, auto visit, int* cnt, const int* optr, int* oc, double2* ov) {
                if (dense)
                    cgpu::rows_dense<<<rgpu::kDenseGrid, kStream, 0, st_>>>(nr, na, visit, dacc_.p, dmark_.p, cnt, optr, oc, ov);
                else if (levels == 0)
                    cgpu::rows_sorted<<<grid(nr), kStream, 0, st_>>>(nr, visit, cnt, optr, oc, ov, err_.p);
                else
                    cgpu::rows_hash<<<grid(nr), 128, 0, st_>>>(nr, visit, cnt, optr, oc, ov, err_.p);
            };
            const cgpu::PsaVisit pv{dA.ptr.p, dA.col.p, dA.val.p, agg.p, T.p, dinv.p, L.wp};
            MTK_TRY(two_pass(ln, Psa, [&](int* cnt, const int* optr, int* oc, double2* ov) { rows(ln, pv, cnt, optr, oc, ov); }));
            const cgpu::ProdVisit ap{dA.ptr.p, dA.col.p, dA.val.p, Psa.ptr.p, Psa.col.p, Psa.val.p};
            MTK_TRY(two_pass(ln, AP, [&](int* cnt, const int* optr, int* oc, double2* ov) { rows(ln, ap, cnt, optr, oc, ov); }));
            MTK_TRY(adjoint(Psa, na, Ph, 1.0));
            const cgpu::ProdVisit gv{Ph.ptr.p, Ph.col.p, Ph.val.p, AP.ptr.p, AP.col.p, AP.val.p};
            MTK_TRY(two_pass(na, Ac, [&](int* cnt, const int* optr, int* oc, double2* ov) {
                if (dense)
                    cgpu::rows_dense<<<rgpu::kDenseGrid, kStream, 0, st_>>>(na, na, gv, dacc_.p, dmark_.p, cnt, optr, oc, ov);
                else
                    cgpu::rows_hash<<<grid(na), 128, 0, st_>>>(na, gv, cnt, optr, oc, ov, err_.p);
            }));
            cgpu::real_diagonal<<<grid(na), kStream, 0, st_>>>(na, Ac.ptr.p, Ac.col.p, Ac.val.p);
            lap("Psa, A Psa, Galerkin", levels);
            DevCycleOpsC O;
            if (levels >= 1) {   // level 0 is applied from the ELL rows
                O.S.n = ln;
                O.S.nnz = dA.nnz;
                MTK_TRY(O.S.ptr.alloc(ln + 1));
                MTK_TRY(O.S.col.alloc(std::max<size_t>(dA.nnz, 1)));
                MTK_TRY(O.S.val.alloc(std::max<size_t>(dA.nnz, 1)));
                MTK_CUDA_TRY(cudaMemcpyAsync(O.S.ptr.p, dA.ptr.p, sizeof(int) * (ln + 1), cudaMemcpyDeviceToDevice, st_));
                MTK_CUDA_TRY(cudaMemcpyAsync(O.S.col.p, dA.col.p, sizeof(int) * dA.nnz, cudaMemcpyDeviceToDevice, st_));
                cgpu::smoother_vals<<<grid(ln), kStream, 0, st_>>>(ln, dA.ptr.p, dA.col.p, dA.val.p, dinv.p, omega, O.S.val.p);
                const cgpu::ProlongVisit pr{Psa.ptr.p, Psa.col.p, Psa.val.p, AP.ptr.p, AP.col.p, AP.val.p, dinv.p, alpha, omega};
                MTK_TRY(two_pass(ln, O.P, [&](int* cnt, const int* optr, int* oc, double2* ov) { rows(ln, pr, cnt, optr, oc, ov); }));
                MTK_TRY(adjoint(O.P, na, O.R, alpha));
                lap("S, P, R", levels);
            }
            MTK_CUDA_TRY(cudaGetLastError());
            int herr = 0;
            MTK_CUDA_TRY(cudaMemcpyAsync(&herr, err_.p, sizeof(int), cudaMemcpyDeviceToHost, st_));
            MTK_CUDA_TRY(cudaStreamSynchronize(st_));
            if (herr) return MTK_OK;
            ops.push_back(std::move(O));
            if (levels == 0) {   // level 0 data for the caller: aggregates, T, members in row order
                L0.agg.resize(ln);
                L0.T.resize(ln);
                MTK_CUDA_TRY(cudaMemcpyAsync(L0.agg.data(), agg.p, sizeof(int) * ln, cudaMemcpyDeviceToHost, st_));
                MTK_CUDA_TRY(cudaMemcpyAsync(reinterpret_cast<double2*>(L0.T.data()), T.p, sizeof(double2) * ln,
                                             cudaMemcpyDeviceToHost, st_));
                MTK_CUDA_TRY(cudaStreamSynchronize(st_));
                L0.mptr.assign(na + 1, 0);
                for (int i = 0; i < ln; i++) L0.mptr[L0.agg[i] + 1]++;
                for (int a = 0; a < na; a++) L0.mptr[a + 1] += L0.mptr[a];
                L0.mem.resize(ln);
                std::vector<int> fill(L0.mptr.begin(), L0.mptr.end() - 1);
                for (int i = 0; i < ln; i++) L0.mem[fill[L0.agg[i]]++] = i;
                L0.wp = L.wp;
                L0.A.n = ln;
            }
            levels++;
            cur_n = na;
            dA = std::move(Ac);
            lap("level data", levels - 1);
        }
        if (cur_n > kCoarseMax) return MTK_OK;
        HostCsr cur;
        MTK_TRY(download(dA, cur));
        nc = cur.n;
        Ainv.assign((size_t)nc * nc, cd(0.0));
        for (int i = 0; i < nc; i++)
            for (int p = cur.ptr[i]; p < cur.ptr[i + 1]; p++) Ainv[(size_t)i * nc + cur.col[p]] = cur.val[p];
        for (int i = 0; i < nc; i++)
            for (int j = 0; j < i; j++) {
                const cd m = 0.5 * (Ainv[(size_t)i * nc + j] + std::conj(Ainv[(size_t)j * nc + i]));
                Ainv[(size_t)i * nc + j] = m;
                Ainv[(size_t)j * nc + i] = std::conj(m);
            }
        ok = levels > 0 && hpd_inverse(Ainv, nc);
        lap("coarse inverse", levels);
        return MTK_OK;
    }

    mtk_ctx* c_;
    cudaStream_t st_;
    DBuf<int> err_, cnt_, ucol_;
    DBuf<long long> bsum_, tot_;
    DBuf<double2> rv_, rw_, uval_, dacc_;
    DBuf<double> rt_, rpart_;
    DBuf<unsigned char> dmark_;
    int dense_cols_ = 0;

    int grid(long long n) const {
        const long long g = (n + kStream - 1) / kStream;
        return (int)std::max(1LL, std::min(g, (long long)c_->num_sms * 16));
    }
    // aggregate_level on the device (the same aggregates and T): the pass-1 roots by rounds of
    // the distance-2 independent-set test, pass 2 and the transport by rounds over the parent
    // forest.  ok = false (the host build takes over) if a row is left without an aggregate.
    int aggregate_device(const DevCsrC& dA, DBuf<int>& agg, DBuf<double2>& T, int& na, bool& ok) {
        ok = false;
        const int n = dA.n;
        const int g = grid(n);
        DBuf<signed char> state;
        DBuf<unsigned char> root1;
        DBuf<int> low1, flag, rid, parent, prev, stage, cnt, word;
        MTK_TRY(state.alloc(n));
        MTK_TRY(root1.alloc(n));
        MTK_TRY(low1.alloc(n));
        MTK_TRY(flag.alloc(n));
        MTK_TRY(rid.alloc(n + 1));
        MTK_TRY(parent.alloc(n));
        MTK_TRY(prev.alloc(n));
        MTK_TRY(stage.alloc(n));
        MTK_TRY(agg.alloc(n));
        MTK_TRY(T.alloc(n));
        MTK_TRY(word.alloc(2));
        MTK_TRY(state.zero(st_));
        int h = 0;
        auto read_word = [&](int& out) -> int {
            MTK_CUDA_TRY(cudaMemcpyAsync(&out, word.p, sizeof(int), cudaMemcpyDeviceToHost, st_));
            MTK_CUDA_TRY(cudaStreamSynchronize(st_));
            return MTK_OK;
        };
        // every loop below settles at least one node per round: n + 1 rounds bound them
        for (int round = 0;; round++) {
            if (round > n) return MTK_OK;
            MTK_CUDA_TRY(cudaMemsetAsync(word.p, 0, sizeof(int), st_));
            cgpu::mis_near<<<g, kStream, 0, st_>>>(n, dA.ptr.p, dA.col.p, state.p, low1.p, root1.p);
            cgpu::mis_decide<<<g, kStream, 0, st_>>>(n, dA.ptr.p, dA.col.p, low1.p, root1.p, state.p, word.p);
            c_->kernels += 2;
            MTK_TRY(read_word(h));
            if (!h) break;
        }
        cgpu::root_flags<<<g, kStream, 0, st_>>>(n, state.p, flag.p);
        size_t total = 0;
        MTK_TRY(scan(n, flag.p, rid.p, total));
        na = (int)total;
        cgpu::agg_pass1<<<g, kStream, 0, st_>>>(n, dA.ptr.p, dA.col.p, state.p, rid.p, agg.p, parent.p);
        MTK_CUDA_TRY(cudaMemsetAsync(word.p, 0, sizeof(int), st_));
        cgpu::agg_pass2<<<g, kStream, 0, st_>>>(n, dA.ptr.p, dA.col.p, dA.val.p, agg.p, parent.p, word.p);
        c_->kernels += 3;
        MTK_TRY(read_word(h));
        if (h) return MTK_OK;
        for (int round = 0;; round++) {
            if (round > n) return MTK_OK;
            MTK_CUDA_TRY(cudaMemcpyAsync(prev.p, agg.p, sizeof(int) * n, cudaMemcpyDeviceToDevice, st_));
            MTK_CUDA_TRY(cudaMemsetAsync(word.p, 0, sizeof(int), st_));
            cgpu::agg_resolve<<<g, kStream, 0, st_>>>(n, parent.p, prev.p, agg.p, word.p);
            c_->kernels++;
            MTK_TRY(read_word(h));
            if (!h) break;
        }
        MTK_CUDA_TRY(cudaMemsetAsync(stage.p, 0xff, sizeof(int) * n, st_));
        for (int round = 0;; round++) {
            if (round > n) return MTK_OK;
            MTK_CUDA_TRY(cudaMemsetAsync(word.p, 0, sizeof(int), st_));
            cgpu::transport_round<<<g, kStream, 0, st_>>>(n, round, dA.ptr.p, dA.col.p, dA.val.p, parent.p, stage.p, T.p,
                                                          word.p);
            c_->kernels++;
            MTK_TRY(read_word(h));
            if (!h) break;
        }
        MTK_TRY(cnt.alloc(std::max(na, 1)));
        MTK_TRY(cnt.zero(st_));
        cgpu::agg_count<<<g, kStream, 0, st_>>>(n, agg.p, cnt.p);
        cgpu::t_scale<<<g, kStream, 0, st_>>>(n, agg.p, cnt.p, T.p);
        c_->kernels += 2;
        MTK_CUDA_TRY(cudaGetLastError());
        ok = true;
        return MTK_OK;
    }
    int dense_scratch(int ncols) {
        if (ncols <= dense_cols_) return MTK_OK;
        const size_t threads = (size_t)rgpu::kDenseGrid * kStream;
        MTK_TRY(dacc_.alloc(threads * ncols));
        MTK_TRY(dmark_.alloc(threads * ncols));
        MTK_TRY(dmark_.zero(st_));
        dense_cols_ = ncols;
        return MTK_OK;
    }
    int upload(const HostCsr& A, DevCsrC& D) {
        D.n = A.n;
        D.nnz = A.col.size();
        MTK_TRY(D.ptr.upload(A.ptr.data(), A.ptr.size(), st_));
        MTK_TRY(D.col.upload(A.col.data(), A.col.size(), st_));
        MTK_TRY(D.val.upload(reinterpret_cast<const double2*>(A.val.data()), A.val.size(), st_));
        return MTK_OK;
    }
    int download(const DevCsrC& D, HostCsr& A) {
        A.n = D.n;
        A.ptr.resize(D.n + 1);
        A.col.resize(D.nnz);
        A.val.resize(D.nnz);
        MTK_CUDA_TRY(cudaMemcpyAsync(A.ptr.data(), D.ptr.p, sizeof(int) * (D.n + 1), cudaMemcpyDeviceToHost, st_));
        if (D.nnz) {
            MTK_CUDA_TRY(cudaMemcpyAsync(A.col.data(), D.col.p, sizeof(int) * D.nnz, cudaMemcpyDeviceToHost, st_));
            MTK_CUDA_TRY(cudaMemcpyAsync(reinterpret_cast<double2*>(A.val.data()), D.val.p, sizeof(double2) * D.nnz,
                                         cudaMemcpyDeviceToHost, st_));
        }
        MTK_CUDA_TRY(cudaStreamSynchronize(st_));
        return MTK_OK;
    }
    int scan(int n, const int* cnt, int* ptr, size_t& total) {
        const int nb = (n + rgpu::kScanBlock - 1) / rgpu::kScanBlock;
        if (bsum_.n < (size_t)std::max(nb, 1)) MTK_TRY(bsum_.alloc(std::max(nb, 1)));
        if (n == 0) {
            MTK_CUDA_TRY(cudaMemsetAsync(ptr, 0, sizeof(int), st_));
            total = 0;
            return MTK_OK;
        }
        rgpu::scan_block_sums<<<nb, 256, 0, st_>>>(n, cnt, bsum_.p);
        rgpu::scan_block_offsets<<<1, 32, 0, st_>>>(nb, bsum_.p, tot_.p);
        rgpu::scan_apply<<<nb, 32, 0, st_>>>(n, cnt, bsum_.p, ptr);
        long long t = 0;
        MTK_CUDA_TRY(cudaMemcpyAsync(&t, tot_.p, sizeof(long long), cudaMemcpyDeviceToHost, st_));
        MTK_CUDA_TRY(cudaStreamSynchronize(st_));
        if (t > 2147483647LL) { mtk_set_last_error("multigrid operator beyond 2^31 entries", __FILE__, __LINE__); return MTK_ERR_BAD_INPUT; }
        total = (size_t)t;
        return MTK_OK;
    }
    template <typename Launch>
    int two_pass(int n, DevCsrC& D, Launch launch) {
        D.n = n;
        if (cnt_.n < (size_t)std::max(n, 1)) MTK_TRY(cnt_.alloc(std::max(n, 1)));
        MTK_TRY(D.ptr.alloc(n + 1));
        launch(cnt_.p, nullptr, nullptr, nullptr);
        MTK_CUDA_TRY(cudaGetLastError());
        MTK_TRY(scan(n, cnt_.p, D.ptr.p, D.nnz));
        MTK_TRY(D.col.alloc(std::max<size_t>(D.nnz, 1)));
        MTK_TRY(D.val.alloc(std::max<size_t>(D.nnz, 1)));
        launch(nullptr, D.ptr.p, D.col.p, D.val.p);
        MTK_CUDA_TRY(cudaGetLastError());
        return MTK_OK;
    }
    int adjoint(const DevCsrC& M, int m, DevCsrC& Tm, double div) {
        Tm.n = m;
        Tm.nnz = M.nnz;
        if (cnt_.n < (size_t)std::max(m, 1)) MTK_TRY(cnt_.alloc(std::max(m, 1)));
        MTK_CUDA_TRY(cudaMemsetAsync(cnt_.p, 0, sizeof(int) * std::max(m, 1), st_));
        rgpu::col_counts<<<grid((long long)M.nnz), kStream, 0, st_>>>((int)M.nnz, M.col.p, cnt_.p);
        MTK_TRY(Tm.ptr.alloc(m + 1));
        size_t tot = 0;
        MTK_TRY(scan(m, cnt_.p, Tm.ptr.p, tot));
        MTK_TRY(Tm.col.alloc(std::max<size_t>(M.nnz, 1)));
        MTK_TRY(Tm.val.alloc(std::max<size_t>(M.nnz, 1)));
        if (ucol_.n < std::max<size_t>(M.nnz, 1)) {
            MTK_TRY(ucol_.alloc(std::max<size_t>(M.nnz, 1)));
            MTK_TRY(uval_.alloc(std::max<size_t>(M.nnz, 1)));
        }
        MTK_CUDA_TRY(cudaMemcpyAsync(cnt_.p, Tm.ptr.p, sizeof(int) * m, cudaMemcpyDeviceToDevice, st_));
        cgpu::adjoint_fill<<<grid(M.n), kStream, 0, st_>>>(M.n, M.ptr.p, M.col.p, M.val.p, cnt_.p, ucol_.p, uval_.p);
        cgpu::adjoint_rank<<<grid(32LL * m), kStream, 0, st_>>>(m, Tm.ptr.p, ucol_.p, uval_.p, Tm.col.p, Tm.val.p, div);
        MTK_CUDA_TRY(cudaGetLastError());
        return MTK_OK;
    }
    int spectral_radius_launch(const DevCsrC& A, const double* dinv) {
        const int n = A.n;
        const int nb = (n + rgpu::kRhoRows - 1) / rgpu::kRhoRows;
        if (rv_.n < (size_t)n) { MTK_TRY(rv_.alloc(n)); MTK_TRY(rw_.alloc(n)); MTK_TRY(rt_.alloc(3 * (size_t)n)); }
        if (rpart_.n < 3 * (size_t)nb + 4) MTK_TRY(rpart_.alloc(3 * (size_t)nb + 4));
        cgpu::rho_start<<<grid(n), kStream, 0, st_>>>(n, rv_.p);
        double* tot = rpart_.p + 3 * (size_t)nb;
        for (int it = 0; it < 12; it++) {
            cgpu::rho_rows<<<grid(n), kStream, 0, st_>>>(n, A.ptr.p, A.col.p, A.val.p, dinv, rv_.p, rw_.p, rt_.p);
            rgpu::rho_block_sums<<<nb, 256, 0, st_>>>(n, rt_.p, rpart_.p);
            rgpu::rho_total<<<1, 32, 0, st_>>>(nb, rpart_.p, tot);
            cgpu::scale_vec<<<grid(n), kStream, 0, st_>>>(n, rw_.p, tot + 3, rv_.p);
        }
        MTK_CUDA_TRY(cudaGetLastError());
        return MTK_OK;
    }
    int spectral_radius_finish(int n, double& rho) {
        const int nb = (n + rgpu::kRhoRows - 1) / rgpu::kRhoRows;
        double red[3] = {0, 0, 0};
        MTK_CUDA_TRY(cudaMemcpyAsync(red, rpart_.p + 3 * (size_t)nb, 3 * sizeof(double), cudaMemcpyDeviceToHost, st_));
        MTK_CUDA_TRY(cudaStreamSynchronize(st_));
        rho = red[1] > 0 ? red[0] / red[1] : 0.0;
        rho *= 1.05;
        return MTK_OK;
    }
};

}  // namespace mtk
