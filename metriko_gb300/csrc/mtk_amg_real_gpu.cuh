// Device build of the smoothed-aggregation hierarchy of mtk_amg_real.cuh.
//
// build_real_hierarchy_dev produces the same per-level cycle operators (R, S, P) and coarse
// inverse as build_real_hierarchy, bit for bit: the aggregation (a sequential breadth-first
// pass) stays on the host, every floating-point product and sum of the spectral-radius estimate,
// the smoothed prolongation, A P_sa, the Galerkin product and the cycle operators runs on the
// device with explicit round-to-nearest operations (no contraction into fused multiply-adds) in
// the order of the host code: entries of a row are summed in the order the host's
// build_rows_parallel visits them (first 0 + v, then + v in call order), rows come out sorted by
// column, transposes keep rows ascending within a column, and the spectral-radius sums run over
// the host's fixed blocks of 4096 rows, block sums in block order.
#pragma once
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "mtk_amg_real.cuh"
#include "mtk_common.cuh"
#include "mtk_ctx.cuh"

namespace mtk {

struct DevCsr64 {
    int n = 0;
    size_t nnz = 0;
    DBuf<int> ptr, col;
    DBuf<double> val;
};

struct DevCycleOps { DevCsr64 R, S, P; };

namespace rgpu {

constexpr int kCapRow = 96;     // distinct columns of a sorted-array row (P_sa, A P_sa)
constexpr int kHash = 256;      // slots of the open-addressing row (power of two)
constexpr int kCapGal = 160;    // distinct columns of an open-addressing row
constexpr int kDenseCols = 2048;   // at most this many columns: dense scratch rows
constexpr int kDenseGrid = 32;     // blocks x kStream threads of the dense-row kernels
constexpr int kRhoRows = 4096;  // row block of the spectral-radius sums (det_row_sums)
constexpr int kScanBlock = 1024;

// ---------------------------------------------------------------- exclusive scan of counts
// out[0] = 0, out[i + 1] = out[i] + cnt[i]; bsum: per-block totals (nb = ceil(n / kScanBlock)).
static __global__ void scan_block_sums(int n, const int* __restrict__ cnt, long long* bsum) {
    __shared__ long long s[32];
    const int b = blockIdx.x;
    long long v = 0;
    for (int i = b * kScanBlock + threadIdx.x; i < min(n, (b + 1) * kScanBlock); i += blockDim.x) v += cnt[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        long long t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += s[w];
        bsum[b] = t;
    }
}

// one thread: exclusive scan of the block totals in place, total in *tot
static __global__ void scan_block_offsets(int nb, long long* bsum, long long* tot) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    long long run = 0;
    for (int b = 0; b < nb; b++) {
        const long long v = bsum[b];
        bsum[b] = run;
        run += v;
    }
    *tot = run;
}

// per block: sequential scan by one warp over kScanBlock counts (32 lanes x 32 values)
static __global__ void scan_apply(int n, const int* __restrict__ cnt, const long long* __restrict__ boff, int* out) {
    if (threadIdx.x >= 32) return;
    const int lane = threadIdx.x;
    const int base = blockIdx.x * kScanBlock + lane * 32;
    int loc[32];
    int s = 0;
#pragma unroll
    for (int k = 0; k < 32; k++) {
        const int i = base + k;
        loc[k] = s;
        s += i < n ? cnt[i] : 0;
    }
    int pre = s;   // inclusive scan of lane totals
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, pre, o);
        if (lane >= o) pre += t;
    }
    const long long off = boff[blockIdx.x] + (pre - s);
#pragma unroll
    for (int k = 0; k < 32; k++) {
        const int i = base + k;
        if (i < n) out[i + 1] = (int)(off + loc[k] + cnt[i]);
    }
    if (blockIdx.x == 0 && lane == 0) out[0] = 0;
}

// ---------------------------------------------------------------- row builders
// A row is visited as a sequence of (column, value) candidates; duplicates are summed in visit
// order starting from 0 (as the host's dense accumulator), and the row is written sorted by
// column.  Three accumulators: a sorted small array (short rows), an open-addressing table
// (long rows, many columns) and a dense scratch row (few columns).

// P_sa row i: (agg_i, T_i), then (agg_j, -wp dinv_i A_ij T_j) over the entries of row i
struct PsaVisit {
    const int *Ap, *Ac;
    const double* Av;
    const int* agg;
    const double *T, *dinv;
    double wp;
    template <class Add>
    __device__ void operator()(int i, Add& add) const {
        add(agg[i], T[i]);
        const double a0 = __dmul_rn(-wp, dinv[i]);
        for (int p = Ap[i]; p < Ap[i + 1]; p++) {
            const int j = Ac[p];
            add(agg[j], __dmul_rn(__dmul_rn(a0, Av[p]), T[j]));
        }
    }
};

// (A B) row i: sum_p A_ip B_row(col_p)
struct ProdVisit {
    const int *Ap, *Ac;
    const double* Av;
    const int *Bp, *Bc;
    const double* Bv;
    template <class Add>
    __device__ void operator()(int i, Add& add) const {
        for (int p = Ap[i]; p < Ap[i + 1]; p++) {
            const int k = Ac[p];
            const double a = Av[p];
            for (int q = Bp[k]; q < Bp[k + 1]; q++) add(Bc[q], __dmul_rn(a, Bv[q]));
        }
    }
};

// Cut-vertex stiffness row c: for the faces around c (in vf order), (b, g_a . g_b) for the
// face's corners b, a the corner of c (the IGM free block's S, as its host assembly).
struct StiffVisit {
    const int *vf_ptr, *vf_face, *cutF;
    const double* grad;
    template <class Add>
    __device__ void operator()(int c, Add& add) const {
        for (int k = vf_ptr[c]; k < vf_ptr[c + 1]; k++) {
            const int f = vf_face[k];
            const int a = cutF[3 * f] == c ? 0 : (cutF[3 * f + 1] == c ? 1 : 2);
            const double ga0 = grad[6 * f + 2 * a], ga1 = grad[6 * f + 2 * a + 1];
            for (int j = 0; j < 3; j++)
                add(cutF[3 * f + j], __dadd_rn(__dmul_rn(ga0, grad[6 * f + 2 * j]), __dmul_rn(ga1, grad[6 * f + 2 * j + 1])));
        }
    }
};

// Row j of 2 W_y^T S W (free columns: K_yy + delta on the diagonal; translation columns: C_yJ):
// for the W^T entries (r = 2c + k, w1) of y_j, the stiffness row of c, the W entries of
// 2 c' + k: (y', 2 w1 s w2) for free y' (translations: the slot -1 - tag).
struct FreeBlockVisit {
    const int *yt_ptr, *yt_row;
    const double* yt_val;
    const int *hs_ptr, *hs_col;
    const double* hs_val;
    const int *w_ptr, *w_tag;
    const double* w_val;
    double delta;
    bool translations;
    template <class Add>
    __device__ void operator()(int j, Add& add) const {
        for (int e = yt_ptr[j]; e < yt_ptr[j + 1]; e++) {
            const int r = yt_row[e], c2 = r >> 1, kk = r & 1;
            const double w2 = __dmul_rn(2.0, yt_val[e]);
            for (int p = hs_ptr[c2]; p < hs_ptr[c2 + 1]; p++) {
                const int r2 = 2 * hs_col[p] + kk;
                const double ws = __dmul_rn(w2, hs_val[p]);
                for (int e2 = w_ptr[r2]; e2 < w_ptr[r2 + 1]; e2++) {
                    const int y2 = w_tag[e2];
                    if (translations ? y2 < 0 : y2 >= 0) add(translations ? -1 - y2 : y2, __dmul_rn(ws, w_val[e2]));
                }
            }
        }
        if (!translations) add(j, delta);
    }
};

// FP32 values of a free block without its diagonal shift delta
static __global__ void free_block_f32(int n, const int* __restrict__ Kp, const int* __restrict__ Kc,
                                      const double* __restrict__ Kv, double delta, float* out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        for (int q = Kp[i]; q < Kp[i + 1]; q++) out[q] = (float)(Kc[q] == i ? __dsub_rn(Kv[q], delta) : Kv[q]);
}

struct SortedAcc {
    int cols[kCapRow];
    double vals[kCapRow];
    int cnt = 0;
    int* err;
    __device__ void operator()(int c, double v) {
        int lo = 0, hi = cnt;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (cols[mid] < c) lo = mid + 1; else hi = mid;
        }
        if (lo < cnt && cols[lo] == c) { vals[lo] = __dadd_rn(vals[lo], v); return; }
        if (cnt >= kCapRow) { *err = 1; return; }
        for (int k = cnt; k > lo; k--) { cols[k] = cols[k - 1]; vals[k] = vals[k - 1]; }
        cols[lo] = c;
        vals[lo] = __dadd_rn(0.0, v);
        cnt++;
    }
};

template <class Visit>
__global__ void rows_sorted(int n, Visit visit, int* cnt_out, const int* __restrict__ optr, int* ocol, double* oval,
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

struct HashAcc {
    int hc[kHash];
    double hv[kHash];
    int cnt = 0;
    int* err;
    __device__ void init() { for (int s = 0; s < kHash; s++) hc[s] = -1; }
    __device__ void operator()(int c, double v) {
        unsigned h = ((unsigned)c * 2654435761u) & (kHash - 1);
        while (hc[h] >= 0 && hc[h] != c) h = (h + 1) & (kHash - 1);
        if (hc[h] == c) { hv[h] = __dadd_rn(hv[h], v); return; }
        if (cnt >= kCapGal) { *err = 1; return; }
        hc[h] = c;
        hv[h] = __dadd_rn(0.0, v);
        cnt++;
    }
};

template <class Visit>
__global__ void __launch_bounds__(128) rows_hash(int n, Visit visit, int* cnt_out, const int* __restrict__ optr, int* ocol,
                                                 double* oval, int* err) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        HashAcc acc;
        acc.err = err;
        acc.init();
        visit(i, acc);
        if (!optr) { cnt_out[i] = acc.cnt; continue; }
        const int o = optr[i];
        int m = 0;   // compact, insertion sort by column
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
    double* acc;
    unsigned char* mark;
    int cnt = 0;
    __device__ void operator()(int c, double v) {
        if (!mark[c]) { mark[c] = 1; acc[c] = __dadd_rn(0.0, v); cnt++; }
        else acc[c] = __dadd_rn(acc[c], v);
    }
};

// ncols small: row i accumulates in scratch row (i mod the scratch rows is not used: one
// scratch row per thread of the grid, rows processed in grid-stride order)
template <class Visit>
__global__ void rows_dense(int n, int ncols, Visit visit, double* scratch, unsigned char* marks, int* cnt_out,
                           const int* __restrict__ optr, int* ocol, double* oval) {
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    double* acc = scratch + (size_t)tid * ncols;
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

// ---------------------------------------------------------------- transpose
static __global__ void col_counts(int nnz, const int* __restrict__ col, int* cnt) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < nnz; p += gridDim.x * blockDim.x) atomicAdd(cnt + col[p], 1);
}
static __global__ void transpose_fill(int n, const int* __restrict__ Mp, const int* __restrict__ Mc, const double* __restrict__ Mv,
                               int* fill, int* tcol, double* tval) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        for (int p = Mp[i]; p < Mp[i + 1]; p++) {
            const int pos = atomicAdd(fill + Mc[p], 1);
            tcol[pos] = i;
            tval[pos] = Mv[p];
        }
}
// One warp per output row: each entry goes to its rank among the row's entries (input rows are
// distinct within an output row), so rows come out ascending (the host transpose's order);
// values / div (div != 1).
static __global__ void transpose_rank(int m, const int* __restrict__ tp, const int* __restrict__ ucol,
                               const double* __restrict__ uval, int* tcol, double* tval, double div) {
    const int lane = threadIdx.x & 31;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    for (int a = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; a < m; a += warps) {
        const int b = tp[a], e = tp[a + 1];
        for (int k = b + lane; k < e; k += 32) {
            const int c = ucol[k];
            int r = 0;
            for (int j = b; j < e; j++) r += ucol[j] < c ? 1 : 0;
            tcol[b + r] = c;
            tval[b + r] = div != 1.0 ? __ddiv_rn(uval[k], div) : uval[k];
        }
    }
}

// ---------------------------------------------------------------- cycle operators
// S = omega D^-1 (2 I - A omega D^-1) on the pattern of A
static __global__ void smoother_vals(int n, const int* __restrict__ Ap, const int* __restrict__ Ac, const double* __restrict__ Av,
                              const double* __restrict__ dinv, double omega, double* Sv) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double di = __dmul_rn(omega, dinv[i]);
        for (int p = Ap[i]; p < Ap[i + 1]; p++) {
            const int j = Ac[p];
            double v = __dmul_rn(__dmul_rn(-Av[p], omega), dinv[j]);
            if (j == i) v = __dadd_rn(v, 2.0);
            Sv[p] = __dmul_rn(di, v);
        }
    }
}

// P row i = alpha P_sa row + (-alpha omega dinv_i) (A P_sa) row, merged by column
static __global__ void prolong_rows(int n, const int* __restrict__ Pp, const int* __restrict__ Pc, const double* __restrict__ Pv,
                             const int* __restrict__ Bp, const int* __restrict__ Bc, const double* __restrict__ Bv,
                             const double* __restrict__ dinv, double alpha, double omega, int* cnt_out,
                             const int* __restrict__ optr, int* ocol, double* oval) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int a = Pp[i];
        const int ae = Pp[i + 1];
        int b = Bp[i];
        const int be = Bp[i + 1];
        int k = 0;
        const double sb = __dmul_rn(__dmul_rn(-alpha, omega), dinv[i]);
        const int o = optr ? optr[i] : 0;
        while (a < ae || b < be) {
            int c2;
            double v;
            if (b >= be || (a < ae && Pc[a] < Bc[b])) { c2 = Pc[a]; v = __dmul_rn(alpha, Pv[a]); a++; }
            else if (a >= ae || Bc[b] < Pc[a]) { c2 = Bc[b]; v = __dmul_rn(sb, Bv[b]); b++; }
            else { c2 = Pc[a]; v = __dadd_rn(__dmul_rn(alpha, Pv[a]), __dmul_rn(sb, Bv[b])); a++; b++; }
            if (optr) { ocol[o + k] = c2; oval[o + k] = v; }
            k++;
        }
        if (!optr) cnt_out[i] = k;
    }
}

// ---------------------------------------------------------------- spectral radius of D^-1 A
static __global__ void rho_start(int n, double* v) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        v[i] = (i & 1) ? 1.0 : __dadd_rn(-1.0, __dmul_rn(0.25, (double)(((unsigned)i * 7919u) % 5u)));
}
// per row: w = dinv (A v); terms v (A v), v v / dinv, w w
static __global__ void rho_rows(int n, const int* __restrict__ Ap, const int* __restrict__ Ac, const double* __restrict__ Av,
                         const double* __restrict__ dinv, const double* __restrict__ v, double* w, double* t3) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double av = 0.0;
        for (int p = Ap[i]; p < Ap[i + 1]; p++) av = __dadd_rn(av, __dmul_rn(Av[p], v[Ac[p]]));
        const double wi = __dmul_rn(dinv[i], av);
        w[i] = wi;
        t3[3 * (size_t)i] = __dmul_rn(v[i], av);
        t3[3 * (size_t)i + 1] = __ddiv_rn(__dmul_rn(v[i], v[i]), dinv[i]);
        t3[3 * (size_t)i + 2] = __dmul_rn(wi, wi);
    }
}
// One CTA per block of kRhoRows rows: the terms are staged through shared memory in chunks and
// summed by one thread in row order (the host's per-block order).
constexpr int kRhoChunk = 1024;
static __global__ void rho_block_sums(int n, const double* __restrict__ t3, double* part) {
    __shared__ double sh[3 * kRhoChunk];
    const int b = blockIdx.x;
    const int r0 = b * kRhoRows, r1 = min(n, r0 + kRhoRows);
    double a0 = 0.0, a1 = 0.0, a2 = 0.0;
    for (int c0 = r0; c0 < r1; c0 += kRhoChunk) {
        const int m = min(kRhoChunk, r1 - c0);
        for (int k = threadIdx.x; k < 3 * m; k += blockDim.x) sh[k] = t3[3 * (size_t)c0 + k];
        __syncthreads();
        if (threadIdx.x == 0)
            for (int k = 0; k < m; k++) {
                a0 = __dadd_rn(a0, sh[3 * k]);
                a1 = __dadd_rn(a1, sh[3 * k + 1]);
                a2 = __dadd_rn(a2, sh[3 * k + 2]);
            }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[3 * (size_t)b] = a0;
        part[3 * (size_t)b + 1] = a1;
        part[3 * (size_t)b + 2] = a2;
    }
}
// one thread: block sums in order into out[0..3), and the normalisation 1 / sqrt(out[2]) in out[3]
static __global__ void rho_total(int nb, const double* __restrict__ part, double* out) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    double o0 = 0.0, o1 = 0.0, o2 = 0.0;
    for (int b = 0; b < nb; b++) {
        o0 = __dadd_rn(o0, part[3 * (size_t)b]);
        o1 = __dadd_rn(o1, part[3 * (size_t)b + 1]);
        o2 = __dadd_rn(o2, part[3 * (size_t)b + 2]);
    }
    out[0] = o0;
    out[1] = o1;
    out[2] = o2;
    out[3] = o2 > 0 ? __ddiv_rn(1.0, __dsqrt_rn(o2)) : 0.0;
}
static __global__ void scale_vec(int n, const double* __restrict__ w, const double* __restrict__ sc, double* v) {
    const double s = *sc;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) v[i] = __dmul_rn(w[i], s);
}

// dinv_i = 1 / A_ii (1 where the diagonal is missing or not positive), as raggregate
static __global__ void diag_inv(int n, const int* __restrict__ Ap, const int* __restrict__ Ac, const double* __restrict__ Av,
                         double* dinv) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int lo = Ap[i], hi = Ap[i + 1];
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (Ac[mid] < i) lo = mid + 1; else hi = mid;
        }
        const double dg = (lo < Ap[i + 1] && Ac[lo] == i) ? Av[lo] : 0.0;
        dinv[i] = dg > 0 ? __ddiv_rn(1.0, dg) : 1.0;
    }
}

static __global__ void to_f32_vals(size_t n, const double* __restrict__ a, float* b) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) b[i] = (float)a[i];
}

}  // namespace rgpu

// Host driver of the device build.
class RDevBuilder {
   public:
    RDevBuilder(mtk_ctx* c, cudaStream_t st) : c_(c), st_(st) {}

    // ok = false (status MTK_OK) where build_real_hierarchy would fail or a row exceeds the
    // kernels' capacity; the caller then builds on the host from A0, node and comp, which are
    // handed back unchanged.
    // dA0 (may be null): the device copy of A0 (moved in), else A0 is uploaded
    int build(RCsr& A0, std::vector<int>& node, std::vector<int>& comp, int nnode, std::vector<DevCycleOps>& ops,
              int& nc, std::vector<double>& Ainv, bool& ok, DevCsr64* dA0 = nullptr, double omega_cap = 1.0,
              double alpha = 1.0) {
        dA0_ = dA0;
        RLevel cur;
        std::swap(cur.A, A0);
        std::swap(cur.node, node);
        std::swap(cur.comp, comp);
        cur.nnode = nnode;
        RLevel* give_back = &cur;   // level 0 returns to the caller
        RLevel lv0;
        const int st = run(cur, lv0, give_back, ops, nc, Ainv, ok, omega_cap, alpha);
        std::swap(give_back->A, A0);
        std::swap(give_back->node, node);
        std::swap(give_back->comp, comp);
        return st;
    }

    // capacity flag and scan total of the row builders (the free-block assembly uses them before
    // build); failed(): a row exceeded its accumulator
    int prepare() {
        MTK_TRY(err_.alloc(1));
        MTK_TRY(err_.zero(st_));
        MTK_TRY(tot_.alloc(1));
        return MTK_OK;
    }
    int failed(bool& f) {
        int h = 0;
        MTK_CUDA_TRY(cudaMemcpyAsync(&h, err_.p, sizeof(int), cudaMemcpyDeviceToHost, st_));
        MTK_CUDA_TRY(cudaStreamSynchronize(st_));
        f = h != 0;
        return MTK_OK;
    }

    int run(RLevel& cur, RLevel& lv0, RLevel*& give_back, std::vector<DevCycleOps>& ops, int& nc,
            std::vector<double>& Ainv, bool& ok, double omega_cap, double alpha) {
        ok = false;
        ops.clear();
        const char* dbg = getenv("MTK_DEBUG");
        const bool debug = dbg && dbg[0] == '1';
        auto t0 = std::chrono::steady_clock::now();
        auto lap = [&](const char* what, int lvl) {   // stage times (MTK_DEBUG=1)
            if (!debug) return;
            cudaStreamSynchronize(st_);
            const auto t = std::chrono::steady_clock::now();
            fprintf(stderr, "[mg device]     level %d %-18s %7.1f ms\n", lvl, what,
                    std::chrono::duration<double, std::milli>(t - t0).count());
            t0 = t;
        };
        MTK_TRY(err_.alloc(1));
        MTK_TRY(err_.zero(st_));
        MTK_TRY(tot_.alloc(1));
        DevCsr64 dA;
        if (dA0_) dA = std::move(*dA0_);
        else MTK_TRY(upload(cur.A, dA));
        int levels = 0;
        lap("upload", 0);
        while (cur.A.n > kRCoarseMax && levels < kRMaxLevels - 1) {
            std::vector<int> cn, cc;
            int cnn = 0;
            const int n = cur.A.n;
            // the spectral radius needs no aggregates: its power steps run on the device while the
            // host aggregates
            DBuf<int> agg;
            DBuf<double> T, dinv;
            MTK_TRY(dinv.alloc(n));
            rgpu::diag_inv<<<grid(n), kStream, 0, st_>>>(n, dA.ptr.p, dA.col.p, dA.val.p, dinv.p);
            MTK_TRY(spectral_radius_launch(dA, dinv.p));
            const int na = raggregate(cur, cn, cc, cnn);
            if (na >= cur.A.n * 0.9) return MTK_OK;
            MTK_TRY(agg.upload(cur.agg.data(), n, st_));
            MTK_TRY(T.upload(cur.T.data(), n, st_));
            double rho = 0;
            MTK_TRY(spectral_radius_finish(n, rho));
            lap("aggregate (host) + rho", levels);
            const double wp = rho > 0 ? (4.0 / 3.0) / rho : 0.0;
            const double omega = rho > 0 ? std::min(omega_cap, 1.5 / rho) : omega_cap;
            DevCsr64 Psa, AP, Pt, Ac;
            const bool dense = na <= rgpu::kDenseCols;
            if (dense) MTK_TRY(dense_scratch(na));
            // P_sa = (I - wp D^-1 A) T
            // rows of level 0 are short (the mesh stencil): sorted arrays; deeper levels: a table,
            // or dense scratch rows when the next level is small
            auto rows = [&](int nr, auto visit, int* cnt, const int* optr, int* oc, double* ov) {
                if (dense)
                    rgpu::rows_dense<<<rgpu::kDenseGrid, kStream, 0, st_>>>(nr, na, visit, dacc_.p, dmark_.p, cnt, optr, oc, ov);
                else if (levels == 0)
                    rgpu::rows_sorted<<<grid(nr), kStream, 0, st_>>>(nr, visit, cnt, optr, oc, ov, err_.p);
                else
                    rgpu::rows_hash<<<grid(nr), 128, 0, st_>>>(nr, visit, cnt, optr, oc, ov, err_.p);
            };
            const rgpu::PsaVisit pv{dA.ptr.p, dA.col.p, dA.val.p, agg.p, T.p, dinv.p, wp};
            MTK_TRY(two_pass(n, Psa, [&](int* cnt, const int* optr, int* oc, double* ov) { rows(n, pv, cnt, optr, oc, ov); }));
            // A P_sa
            const rgpu::ProdVisit ap{dA.ptr.p, dA.col.p, dA.val.p, Psa.ptr.p, Psa.col.p, Psa.val.p};
            MTK_TRY(two_pass(n, AP, [&](int* cnt, const int* optr, int* oc, double* ov) { rows(n, ap, cnt, optr, oc, ov); }));
            lap("Psa, A Psa", levels);
            // P_sa^T (A P_sa)
            MTK_TRY(transpose(Psa, na, Pt, 1.0));
            const rgpu::ProdVisit gv{Pt.ptr.p, Pt.col.p, Pt.val.p, AP.ptr.p, AP.col.p, AP.val.p};
            MTK_TRY(two_pass(na, Ac, [&](int* cnt, const int* optr, int* oc, double* ov) {
                if (dense)
                    rgpu::rows_dense<<<rgpu::kDenseGrid, kStream, 0, st_>>>(na, na, gv, dacc_.p, dmark_.p, cnt, optr, oc, ov);
                else
                    rgpu::rows_hash<<<grid(na), 128, 0, st_>>>(na, gv, cnt, optr, oc, ov, err_.p);
            }));
            lap("Galerkin", levels);
            DevCycleOps O;
            // S on the pattern of A
            O.S.n = n;
            O.S.nnz = dA.nnz;
            MTK_TRY(O.S.ptr.alloc(n + 1));
            MTK_TRY(O.S.col.alloc(dA.nnz));
            MTK_TRY(O.S.val.alloc(dA.nnz));
            MTK_CUDA_TRY(cudaMemcpyAsync(O.S.ptr.p, dA.ptr.p, sizeof(int) * (n + 1), cudaMemcpyDeviceToDevice, st_));
            MTK_CUDA_TRY(cudaMemcpyAsync(O.S.col.p, dA.col.p, sizeof(int) * dA.nnz, cudaMemcpyDeviceToDevice, st_));
            rgpu::smoother_vals<<<grid(n), kStream, 0, st_>>>(n, dA.ptr.p, dA.col.p, dA.val.p, dinv.p, omega, O.S.val.p);
            MTK_TRY(two_pass(n, O.P, [&](int* cnt, const int* optr, int* oc, double* ov) {
                rgpu::prolong_rows<<<grid(n), kStream, 0, st_>>>(n, Psa.ptr.p, Psa.col.p, Psa.val.p, AP.ptr.p, AP.col.p,
                                                                 AP.val.p, dinv.p, alpha, omega, cnt, optr, oc, ov);
            }));
            MTK_TRY(transpose(O.P, na, O.R, alpha));
            MTK_CUDA_TRY(cudaGetLastError());
            lap("S, P, R", levels);
            int herr = 0;
            MTK_CUDA_TRY(cudaMemcpyAsync(&herr, err_.p, sizeof(int), cudaMemcpyDeviceToHost, st_));
            MTK_CUDA_TRY(cudaStreamSynchronize(st_));
            if (herr) return MTK_OK;   // a row beyond the kernels' capacity: host build
            ops.push_back(std::move(O));
            levels++;
            // next level: the host keeps the matrix for its aggregation (or the coarse inverse)
            RLevel nxt;
            MTK_TRY(download(Ac, nxt.A));
            lap("download", levels - 1);
            if (levels == 1) {   // keep level 0 for the caller
                std::swap(lv0.A, cur.A);
                std::swap(lv0.node, cur.node);
                std::swap(lv0.comp, cur.comp);
                give_back = &lv0;
            }
            cur = std::move(nxt);
            cur.node = std::move(cn);
            cur.comp = std::move(cc);
            cur.nnode = cnn;
            dA = std::move(Ac);
        }
        if (cur.A.n > kRCoarseMax) return MTK_OK;
        nc = cur.A.n;
        Ainv.assign((size_t)nc * nc, 0.0);
        for (int i = 0; i < nc; i++)
            for (int p = cur.A.ptr[i]; p < cur.A.ptr[i + 1]; p++) Ainv[(size_t)i * nc + cur.A.col[p]] = cur.A.val[p];
        for (int i = 0; i < nc; i++)
            for (int j = 0; j < i; j++) {
                const double m = 0.5 * (Ainv[(size_t)i * nc + j] + Ainv[(size_t)j * nc + i]);
                Ainv[(size_t)i * nc + j] = m;
                Ainv[(size_t)j * nc + i] = m;
            }
        ok = spd_inverse_dense(Ainv, nc);
        lap("coarse inverse", levels);
        return MTK_OK;
    }

    mtk_ctx* c_;
    cudaStream_t st_;
    DevCsr64* dA0_ = nullptr;
    DBuf<int> err_, cnt_;
    DBuf<long long> bsum_, tot_;
    DBuf<double> rv_, rw_, rt_, rpart_;
    DBuf<double> dacc_, uval_;
    DBuf<int> ucol_;
    DBuf<unsigned char> dmark_;
    int dense_cols_ = 0;

    // scratch rows of the dense accumulator (one per thread of the kDenseGrid x kStream grid);
    // marks start (and are left) zero
    int dense_scratch(int ncols) {
        if (ncols <= dense_cols_) return MTK_OK;
        const size_t threads = (size_t)rgpu::kDenseGrid * kStream;
        MTK_TRY(dacc_.alloc(threads * ncols));
        MTK_TRY(dmark_.alloc(threads * ncols));
        MTK_TRY(dmark_.zero(st_));
        dense_cols_ = ncols;
        return MTK_OK;
    }

    int grid(long long n) const {
        const long long g = (n + kStream - 1) / kStream;
        return (int)std::max(1LL, std::min(g, (long long)c_->num_sms * 16));
    }

    int upload(const RCsr& A, DevCsr64& D) {
        D.n = A.n;
        D.nnz = A.col.size();
        MTK_TRY(D.ptr.upload(A.ptr.data(), A.ptr.size(), st_));
        MTK_TRY(D.col.upload(A.col.data(), A.col.size(), st_));
        MTK_TRY(D.val.upload(A.val.data(), A.val.size(), st_));
        return MTK_OK;
    }
    int download(const DevCsr64& D, RCsr& A) {
        A.n = D.n;
        A.ptr.resize(D.n + 1);
        A.col.resize(D.nnz);
        A.val.resize(D.nnz);
        MTK_CUDA_TRY(cudaMemcpyAsync(A.ptr.data(), D.ptr.p, sizeof(int) * (D.n + 1), cudaMemcpyDeviceToHost, st_));
        if (D.nnz) {
            MTK_CUDA_TRY(cudaMemcpyAsync(A.col.data(), D.col.p, sizeof(int) * D.nnz, cudaMemcpyDeviceToHost, st_));
            MTK_CUDA_TRY(cudaMemcpyAsync(A.val.data(), D.val.p, sizeof(double) * D.nnz, cudaMemcpyDeviceToHost, st_));
        }
        MTK_CUDA_TRY(cudaStreamSynchronize(st_));
        return MTK_OK;
    }

    // counts (cnt) -> ptr (n + 1), returns the total
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

    // rows by a count pass and a fill pass of the same kernel
    template <typename Launch>
    int two_pass(int n, DevCsr64& D, Launch launch) {
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

    int transpose(const DevCsr64& M, int m, DevCsr64& Tm, double div) {
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
        rgpu::transpose_fill<<<grid(M.n), kStream, 0, st_>>>(M.n, M.ptr.p, M.col.p, M.val.p, cnt_.p, ucol_.p, uval_.p);
        rgpu::transpose_rank<<<grid(32LL * m), kStream, 0, st_>>>(m, Tm.ptr.p, ucol_.p, uval_.p, Tm.col.p, Tm.val.p, div);
        MTK_CUDA_TRY(cudaGetLastError());
        return MTK_OK;
    }

    // 12 power steps of D^-1 A from the host's fixed start (queued on the stream), then the
    // Rayleigh quotient of the last step raised by 5 percent
    int spectral_radius_finish(int n, double& rho) {
        const int nb = (n + rgpu::kRhoRows - 1) / rgpu::kRhoRows;
        double red[3] = {0, 0, 0};
        MTK_CUDA_TRY(cudaMemcpyAsync(red, rpart_.p + 3 * (size_t)nb, 3 * sizeof(double), cudaMemcpyDeviceToHost, st_));
        MTK_CUDA_TRY(cudaStreamSynchronize(st_));
        rho = red[1] > 0 ? red[0] / red[1] : 0.0;
        rho *= 1.05;
        return MTK_OK;
    }
    int spectral_radius_launch(const DevCsr64& A, const double* dinv) {
        const int n = A.n;
        const int nb = (n + rgpu::kRhoRows - 1) / rgpu::kRhoRows;
        if (rv_.n < (size_t)n) { MTK_TRY(rv_.alloc(n)); MTK_TRY(rw_.alloc(n)); MTK_TRY(rt_.alloc(3 * (size_t)n)); }
        if (rpart_.n < 3 * (size_t)nb + 4) MTK_TRY(rpart_.alloc(3 * (size_t)nb + 4));
        rgpu::rho_start<<<grid(n), kStream, 0, st_>>>(n, rv_.p);
        double* tot = rpart_.p + 3 * (size_t)nb;
        for (int it = 0; it < 12; it++) {
            rgpu::rho_rows<<<grid(n), kStream, 0, st_>>>(n, A.ptr.p, A.col.p, A.val.p, dinv, rv_.p, rw_.p, rt_.p);
            rgpu::rho_block_sums<<<nb, 256, 0, st_>>>(n, rt_.p, rpart_.p);
            rgpu::rho_total<<<1, 32, 0, st_>>>(nb, rpart_.p, tot);
            rgpu::scale_vec<<<grid(n), kStream, 0, st_>>>(n, rw_.p, tot + 3, rv_.p);
        }
        MTK_CUDA_TRY(cudaGetLastError());
        return MTK_OK;
    }
};

}  // namespace mtk
