// Smoothest N-RoSy field on the device: connection-Laplacian assembly, complex Hermitian
// SpMV, persistent PCG (FP32 or FP64) and the inverse power iteration with FP64 residuals,
// Rayleigh quotient and normalisation.
//
// Replaces (metriko) face_rosy_field.h:17-23 + :72-110 and sparse_linear_solver.h:29-54.
// The reference factorises L once (CHOLMOD simplicial LDL^T or Eigen SparseLU) and runs 50
// triangular-solve pairs; here every inverse-iteration step is a preconditioned CG solve of
// L x = M u to a relative residual `tol`, warm-started from the Galerkin guess
// x0 = u (u^H M u) / (u^H L u), with MIXED precision running the CG in FP32 inside FP64
// iterative refinement.
//
// Layout (n = nF faces, structure of arrays so every per-face load is coalesced):
//   nbr[j*n + f]  int32   neighbour face across halfedge j of f
//   v64[j*n + f]  double2 off-diagonal value L(f, nbr)       v32: float2 copy
//   d64[f], d32[f]        diagonal (#neighbours + 1e-9)     inv32/inv64: Jacobi inverse
// Algorithmic bytes per SpMV row: FP32 3*(8+4) + 4 + 2*8 = 56 B, FP64 3*(16+4) + 8 + 2*16 = 100 B.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "mtk_amg.cuh"
#include "mtk_amg_gpu.cuh"
#include "mtk_ctx.cuh"
#include "mtk_sell.cuh"

namespace mtk {

template <typename T> struct V2of;
template <> struct V2of<float> { using type = float2; };
template <> struct V2of<double> { using type = double2; };

template <typename T>
struct ComplexEll {
    using V2 = typename V2of<T>::type;
    int n;
    const int* nbr;
    const V2* val;
    const T* diag;
    __device__ __forceinline__ V2 row(int i, const V2* __restrict__ x) const {
        V2 xi = __ldcg(x + i);
        T d = diag[i];
        T re = d * xi.x, im = d * xi.y;
#pragma unroll
        for (int j = 0; j < 3; j++) {
            int c = nbr[j * n + i];
            V2 a = val[j * n + i];
            V2 xc = __ldcg(x + c);
            re += a.x * xc.x - a.y * xc.y;
            im += a.x * xc.y + a.y * xc.x;
        }
        V2 o;
        o.x = re;
        o.y = im;
        return o;
    }
};

// ---------------------------------------------------------------------------- assembly
// One thread per face: off-diagonals -(-e^{i theta})^N = -e^{i N (theta + pi)}, diagonal
// #neighbours + 1e-9 (face_rosy_field.h:52-75).  No atomics: every row is written by its owner.
// Every row keeps the uniform diagonal 3 + 1e-9 of a closed mesh; a boundary side (nbr_in -1:
// no neighbour, nothing in L, :64) becomes the entry -1 on the row's own column, so the row
// applies (3 - #boundary sides + 1e-9) to its own value, the reference's diagonal.  The kernels
// and the multigrid passes that factor A = d I + (ELL entries) then need no per-row diagonal.
__global__ void field_assemble(int n, int N, const int* __restrict__ nbr_in, const double* __restrict__ theta,
                               const double* __restrict__ area, int* nbr, double2* v64, float2* v32,
                               double* d64, float* d32, double* inv64, float* inv32, float* area32) {
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < n; f += gridDim.x * blockDim.x) {
        for (int j = 0; j < 3; j++) {
            int g = nbr_in[3 * f + j];
            double2 a;
            if (g < 0) {
                g = f;
                a = make_double2(-1.0, 0.0);
            } else {
                double s, c;
                sincos((double)N * (theta[3 * f + j] + 3.14159265358979323846), &s, &c);
                a = make_double2(-c, -s);
            }
            nbr[j * n + f] = g;
            v64[j * n + f] = a;
            v32[j * n + f] = make_float2((float)a.x, (float)a.y);
        }
        double d = 3.0 + 1e-9;
        d64[f] = d;
        d32[f] = (float)d;
        inv64[f] = 1.0 / d;
        inv32[f] = (float)(1.0 / d);
        area32[f] = (float)area[f];
    }
}

// ---------------------------------------------------------------------------- persistent PCG
// Solves A x = b (Hermitian positive definite) from the given x.  Three bounded grid
// barriers per iteration; all scalars are reduced in a fixed order, so the iterates are
// bit-reproducible for a given grid size.  status: 0 converged, 3 cap, 4 breakdown, 5 timeout.
template <typename T>
__global__ void __launch_bounds__(kBlock, 1) pcg_complex(ComplexEll<T> A, const T* __restrict__ minv,
                                                     const typename V2of<T>::type* __restrict__ b,
                                                     typename V2of<T>::type* x, typename V2of<T>::type* r,
                                                     typename V2of<T>::type* z, typename V2of<T>::type* p,
                                                     typename V2of<T>::type* q, T* partials, GridBarrier bar,
                                                     double tol2, int maxit, int* out) {
    using V2 = typename V2of<T>::type;
    const int n = A.n;
    const int stride = gridDim.x * blockDim.x;
    const int t0 = blockIdx.x * blockDim.x + threadIdx.x;
    T red2[2];
    T red1[1];
    // phase 0: r = b - A x, z = M^-1 r, p = z
    red2[0] = T(0);
    red2[1] = T(0);
    for (int i = t0; i < n; i += stride) {
        V2 ax = A.row(i, x);
        V2 bi = b[i];
        V2 ri;
        ri.x = bi.x - ax.x;
        ri.y = bi.y - ax.y;
        T m = minv[i];
        V2 zi;
        zi.x = m * ri.x;
        zi.y = m * ri.y;
        r[i] = ri;
        z[i] = zi;
        p[i] = zi;
        red2[0] += ri.x * zi.x + ri.y * zi.y;
        red2[1] += ri.x * ri.x + ri.y * ri.y;
    }
    publish_partials<T, 2>(red2, partials);
    int status = 3, it = 0;
    if (!grid_sync(bar)) { status = 5; goto done; }
    gather_partials<T, 2>(partials, red2);
    {
        T rz = red2[0], rr = red2[1];
        for (;;) {
            if ((double)rr <= tol2) { status = 0; break; }
            if (it >= maxit) { status = 3; break; }
            // phase 1: q = A p, <p, q>
            red1[0] = T(0);
            for (int i = t0; i < n; i += stride) {
                V2 qi = A.row(i, p);
                q[i] = qi;
                V2 pi = p[i];
                red1[0] += pi.x * qi.x + pi.y * qi.y;
            }
            publish_partials<T, 1>(red1, partials + 2 * gridDim.x);
            if (!grid_sync(bar)) { status = 5; break; }
            gather_partials<T, 1>(partials + 2 * gridDim.x, red1);
            T pq = red1[0];
            if (!(pq > T(0))) { status = 4; break; }
            T alpha = rz / pq;
            // phase 2: x += a p, r -= a q, z = M^-1 r
            red2[0] = T(0);
            red2[1] = T(0);
            for (int i = t0; i < n; i += stride) {
                V2 pi = p[i], qi = q[i], xi = x[i], ri = r[i];
                xi.x += alpha * pi.x;
                xi.y += alpha * pi.y;
                ri.x -= alpha * qi.x;
                ri.y -= alpha * qi.y;
                T m = minv[i];
                V2 zi;
                zi.x = m * ri.x;
                zi.y = m * ri.y;
                x[i] = xi;
                r[i] = ri;
                z[i] = zi;
                red2[0] += ri.x * zi.x + ri.y * zi.y;
                red2[1] += ri.x * ri.x + ri.y * ri.y;
            }
            publish_partials<T, 2>(red2, partials + 3 * gridDim.x);
            if (!grid_sync(bar)) { status = 5; break; }
            gather_partials<T, 2>(partials + 3 * gridDim.x, red2);
            T rz_new = red2[0];
            rr = red2[1];
            if (rr != rr) { status = 4; break; }
            T beta = rz_new / rz;
            rz = rz_new;
            // phase 3: p = z + b p
            for (int i = t0; i < n; i += stride) {
                V2 zi = z[i], pi = p[i];
                pi.x = zi.x + beta * pi.x;
                pi.y = zi.y + beta * pi.y;
                p[i] = pi;
            }
            it++;
            if (!grid_sync(bar)) { status = 5; break; }
        }
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            out[2] = 0;
            reinterpret_cast<double*>(out + 4)[0] = (double)rr;
        }
    }
done:
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        out[0] = status;
        out[1] = it;
    }
}

// ---------------------------------------------------------------------------- multigrid PCG
// Levels >= 1 are CSR cycle operators (csr_phase); level 0 is applied straight from the ELL rows
// of A, the aggregates and T (DevLevel0), fused with the CG vector updates.

// a x + y for a real scalar a, one rounding per component (owners and neighbours that recompute
// the same value get the same bits)
template <typename V2, typename T> __device__ __forceinline__ V2 axpy2(T a, V2 x, V2 y) {
    V2 o;
    o.x = fmaT<T>(a, x.x, y.x);
    o.y = fmaT<T>(a, x.y, y.y);
    return o;
}

// Accumulates row `row` of M x over the entries lane, lane + g, ... with four loads in flight.
template <typename T>
__device__ __forceinline__ void csr_row_acc(const DevCsr<T>& M, int row, int lane, int g,
                                            const typename V2of<T>::type* __restrict__ x, T& re, T& im) {
    using V2 = typename V2of<T>::type;
    const int e = __ldg(M.ptr + row + 1);
    for (int p = __ldg(M.ptr + row) + lane; p < e; p += 4 * g) {
        int c[4];
        V2 v[4], xv[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const int pu = p + u * g;
            c[u] = pu < e ? __ldg(M.col + pu) : -1;
            v[u] = pu < e ? __ldg(M.val + pu) : V2{};
        }
#pragma unroll
        for (int u = 0; u < 4; u++) xv[u] = c[u] >= 0 ? __ldcg(x + c[u]) : V2{};
#pragma unroll
        for (int u = 0; u < 4; u++)
            if (c[u] >= 0) {
                re += v[u].x * xv[u].x - v[u].y * xv[u].y;
                im += v[u].x * xv[u].y + v[u].y * xv[u].x;
            }
    }
}

// The same row sum from the SELL-32 copy: the row's lane walks its entries in CSR order, 32
// apart in the slice (each load coalesced across the slice's 32 lanes).
template <typename T>
__device__ __forceinline__ void sell_row_acc(const DevCsr<T>& M, int row, const typename V2of<T>::type* __restrict__ x,
                                             T& re, T& im) {
    using V2 = typename V2of<T>::type;
    const int sl = row >> 5;
    const int e = __ldg(M.sptr + sl + 1);
    for (int p = __ldg(M.sptr + sl) + (row & 31); p < e; p += 4 * 32) {
        int c[4];
        V2 v[4], xv[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const int pu = p + u * 32;
            c[u] = pu < e ? __ldg(M.scol + pu) : -1;
            v[u] = pu < e ? __ldg(M.sval + pu) : V2{};
        }
#pragma unroll
        for (int u = 0; u < 4; u++) xv[u] = c[u] >= 0 ? __ldcg(x + c[u]) : V2{};
#pragma unroll
        for (int u = 0; u < 4; u++)
            if (c[u] >= 0) {
                re += v[u].x * xv[u].x - v[u].y * xv[u].y;
                im += v[u].x * xv[u].y + v[u].y * xv[u].x;
            }
    }
}

template <typename T>
__device__ __forceinline__ void row1_acc(const DevCsr<T>& M, int row, const typename V2of<T>::type* __restrict__ x, T& re,
                                         T& im) {
    if (M.sptr) sell_row_acc(M, row, x, re, im);
    else csr_row_acc(M, row, 0, 1, x, re, im);
}

// One CSR phase over all rows: out[row] = M x (+ M2 x2), each row on a group of M.group lanes
// (1, 2, ..., 32; lanes stride the row, then a fixed-order butterfly reduction) across the grid.
template <typename T>
__device__ void csr_phase(const DevCsr<T>& M, const typename V2of<T>::type* x, const DevCsr<T>* M2,
                          const typename V2of<T>::type* x2, typename V2of<T>::type* out) {
    using V2 = typename V2of<T>::type;
    const int stride = gridDim.x * blockDim.x;
    const int t0 = blockIdx.x * blockDim.x + threadIdx.x;
    const int g = M.group;
    if (g == 1) {
        for (int row = t0; row < M.n; row += stride) {
            T re = T(0), im = T(0);
            row1_acc(M, row, x, re, im);
            if (M2) row1_acc(*M2, row, x2, re, im);
            V2 o;
            o.x = re;
            o.y = im;
            out[row] = o;
        }
        return;
    }
    const int lane = threadIdx.x & 31, gpw = 32 / g, sub = lane / g, sl = lane % g;
    for (int rbase = (t0 >> 5) * gpw; rbase < M.n; rbase += (stride >> 5) * gpw) {   // warp-uniform
        const int row = rbase + sub;
        T re = T(0), im = T(0);
        if (row < M.n) {
            csr_row_acc(M, row, sl, g, x, re, im);
            if (M2) csr_row_acc(*M2, row, sl, g, x2, re, im);
        }
        for (int o = g >> 1; o > 0; o >>= 1) {
            re += __shfl_xor_sync(0xffffffffu, re, o);
            im += __shfl_xor_sync(0xffffffffu, im, o);
        }
        if (sl == 0 && row < M.n) {
            V2 v;
            v.x = re;
            v.y = im;
            out[row] = v;
        }
    }
}

// Inner V-cycle over the CSR levels (the first of them is level 1): down r_{l+1} = R r_l,
// coarsest y = A_c^-1 r_c (dense, warp per row), up y_l = S r_l + P y_{l+1}; a grid barrier
// after every phase (2 nlev + 1).
template <typename T>
__device__ bool vcycle_inner(const DevHierarchy<T>& H, const GridBarrier& bar) {
    using V2 = typename V2of<T>::type;
    const int stride = gridDim.x * blockDim.x;
    const int t0 = blockIdx.x * blockDim.x + threadIdx.x;
    for (int l = 0; l < H.nlev; l++) {
        V2* rnext = (l + 1 < H.nlev) ? H.L[l + 1].r : H.rc;
        csr_phase<T>(H.L[l].R, H.L[l].r, nullptr, nullptr, rnext);
        if (!grid_sync(bar)) return false;
    }
    {
        const int lane = threadIdx.x & 31;
        for (int a = t0 >> 5; a < H.nc; a += stride >> 5) {
            T re = T(0), im = T(0);
            const V2* row = H.Ainv + (size_t)a * H.nc;
            for (int b = lane; b < H.nc; b += 32) {
                const V2 m = row[b], rb = __ldcg(H.rc + b);
                re += m.x * rb.x - m.y * rb.y;
                im += m.x * rb.y + m.y * rb.x;
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                re += __shfl_xor_sync(0xffffffffu, re, o);
                im += __shfl_xor_sync(0xffffffffu, im, o);
            }
            if (lane == 0) {
                V2 v;
                v.x = re;
                v.y = im;
                H.yc[a] = v;
            }
        }
    }
    if (!grid_sync(bar)) return false;
    for (int l = H.nlev - 1; l >= 0; l--) {
        const V2* yn = (l + 1 < H.nlev) ? H.L[l + 1].y : H.yc;
        csr_phase<T>(H.L[l].S, H.L[l].r, &H.L[l].P, yn, H.L[l].y);
        if (!grid_sync(bar)) return false;
    }
    return true;
}

// Level-0 phase A: p = z + beta p_old (own row, and recomputed for the three neighbours), q = A p
// with the uniform diagonal dg; writes p to pn and q; returns the partial Re p^H q.
template <typename T>
__device__ __forceinline__ T l0_direction_spmv(const ComplexEll<T>& A, T dg, const typename V2of<T>::type* z,
                                               const typename V2of<T>::type* po, T beta,
                                               typename V2of<T>::type* __restrict__ pn,
                                               typename V2of<T>::type* __restrict__ q) {
    using V2 = typename V2of<T>::type;
    const int n = A.n, stride = gridDim.x * blockDim.x;
    T pq = T(0);
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride) {
        int c[3];
        V2 a[3], zc[3], pc[3];
#pragma unroll
        for (int j = 0; j < 3; j++) {
            c[j] = __ldg(A.nbr + j * n + k);
            a[j] = __ldg(A.val + j * n + k);
        }
        const V2 zk = __ldcg(z + k), pk = __ldcg(po + k);
#pragma unroll
        for (int j = 0; j < 3; j++) {
            zc[j] = __ldcg(z + c[j]);
            pc[j] = __ldcg(po + c[j]);
        }
        const V2 pown = axpy2(beta, pk, zk);
        T re = dg * pown.x, im = dg * pown.y;
#pragma unroll
        for (int j = 0; j < 3; j++) {
            const V2 pj = axpy2(beta, pc[j], zc[j]);
            re += a[j].x * pj.x - a[j].y * pj.y;
            im += a[j].x * pj.y + a[j].y * pj.x;
        }
        V2 qk;
        qk.x = re;
        qk.y = im;
        pn[k] = pown;
        q[k] = qk;
        pq += pown.x * re + pown.y * im;
    }
    return pq;
}

// sum over the three neighbours of A_kj x_j (the ELL off-diagonals of row k)
template <typename T>
__device__ __forceinline__ void ell_offdiag(const ComplexEll<T>& A, int k, const typename V2of<T>::type* x, T& re,
                                            T& im) {
    using V2 = typename V2of<T>::type;
    int c[3];
    V2 a[3], xc[3];
#pragma unroll
    for (int j = 0; j < 3; j++) {
        c[j] = __ldg(A.nbr + j * A.n + k);
        a[j] = __ldg(A.val + j * A.n + k);
    }
#pragma unroll
    for (int j = 0; j < 3; j++) xc[j] = __ldcg(x + c[j]);
    re = T(0);
    im = T(0);
#pragma unroll
    for (int j = 0; j < 3; j++) {
        re += a[j].x * xc[j].x - a[j].y * xc[j].y;
        im += a[j].x * xc[j].y + a[j].y * xc[j].x;
    }
}

// Level-0 phase B: r' = r - alpha q (own row and neighbours), and when `update` x += alpha p and
// rn = r'; s = (I - omega A / d) r' (the pre-smoothed residual, first factor of the restriction).
template <typename T>
__device__ __forceinline__ void l0_update_smooth(const ComplexEll<T>& A, const DevLevel0<T>& L0,
                                                 const typename V2of<T>::type* r, const typename V2of<T>::type* q,
                                                 T alpha, const typename V2of<T>::type* p,
                                                 typename V2of<T>::type* x, typename V2of<T>::type* rn,
                                                 typename V2of<T>::type* __restrict__ sv, bool update) {
    using V2 = typename V2of<T>::type;
    const int n = A.n, stride = gridDim.x * blockDim.x;
    const T od = L0.omega * L0.dinv, keep = T(1) - L0.omega;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride) {
        int c[3];
        V2 a[3], rc[3];
#pragma unroll
        for (int j = 0; j < 3; j++) {
            c[j] = __ldg(A.nbr + j * n + k);
            a[j] = __ldg(A.val + j * n + k);
        }
        V2 rk = __ldcg(r + k);
#pragma unroll
        for (int j = 0; j < 3; j++) rc[j] = __ldcg(r + c[j]);
        if (update) {
            V2 qc[3];
            const V2 qk = __ldcg(q + k);
#pragma unroll
            for (int j = 0; j < 3; j++) qc[j] = __ldcg(q + c[j]);
            rk = axpy2(-alpha, qk, rk);
#pragma unroll
            for (int j = 0; j < 3; j++) rc[j] = axpy2(-alpha, qc[j], rc[j]);
            const V2 pk = __ldcg(p + k), xk = __ldcg(x + k);
            x[k] = axpy2(alpha, pk, xk);
            rn[k] = rk;
        }
        T sr = keep * rk.x, si = keep * rk.y;
#pragma unroll
        for (int j = 0; j < 3; j++) {
            sr -= od * (a[j].x * rc[j].x - a[j].y * rc[j].y);
            si -= od * (a[j].x * rc[j].y + a[j].y * rc[j].x);
        }
        V2 o;
        o.x = sr;
        o.y = si;
        sv[k] = o;
    }
}

// Level-0 phase C: s' = (I - w_p A / d) s and r1[a] = sum over the rows k of aggregate a of
// conj(T_k) s'_k: one warp per chunk, inclusive segmented scan over the lanes of each aggregate
// (fixed order), the last lane of an aggregate writes it.
template <typename T>
__device__ __forceinline__ void l0_restrict(const ComplexEll<T>& A, const DevLevel0<T>& L0,
                                            const typename V2of<T>::type* sv, typename V2of<T>::type* r1) {
    using V2 = typename V2of<T>::type;
    const int lane = threadIdx.x & 31;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    const T opd = L0.wp * L0.dinv, keep = T(1) - L0.wp;
    for (int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < L0.nchunk; w += nwarps) {
        const int beg = __ldg(L0.chunk + w), end = __ldg(L0.chunk + w + 1);
        const bool act = beg + lane < end;
        const int k = act ? beg + lane : beg;   // inactive lanes read a valid row, store nothing
        const int ag = act ? __ldg(L0.agg + k) : -1;
        const V2 tk = __ldg(L0.t + k), sk = __ldcg(sv + k);
        T nr, ni;
        ell_offdiag(A, k, sv, nr, ni);
        const T sr = keep * sk.x - opd * nr, si = keep * sk.y - opd * ni;
        T vx = act ? tk.x * sr + tk.y * si : T(0);   // conj(T_k) * s'
        T vy = act ? tk.x * si - tk.y * sr : T(0);
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const T ux = __shfl_up_sync(0xffffffffu, vx, o), uy = __shfl_up_sync(0xffffffffu, vy, o);
            const int ua = __shfl_up_sync(0xffffffffu, ag, o);
            if (lane >= o && ua == ag) {
                vx += ux;
                vy += uy;
            }
        }
        const int next = __shfl_down_sync(0xffffffffu, ag, 1);
        if (act && (lane == 31 || next != ag)) {
            V2 v;
            v.x = vx;
            v.y = vy;
            r1[ag] = v;
        }
    }
}

// Level-0 phase D: v = P_sa y1 = (I - w_p A / d) u with u_k = T_k y1[agg k].
template <typename T>
__device__ __forceinline__ void l0_prolong(const ComplexEll<T>& A, const DevLevel0<T>& L0,
                                           const typename V2of<T>::type* y1, typename V2of<T>::type* __restrict__ vv) {
    using V2 = typename V2of<T>::type;
    const int n = A.n, stride = gridDim.x * blockDim.x;
    const T opd = L0.wp * L0.dinv, keep = T(1) - L0.wp;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride) {
        int c[3], ac[3];
        V2 a[3], tc[3], yc[3];
#pragma unroll
        for (int j = 0; j < 3; j++) {
            c[j] = __ldg(A.nbr + j * n + k);
            a[j] = __ldg(A.val + j * n + k);
        }
        const int ak = __ldg(L0.agg + k);
        const V2 tk = __ldg(L0.t + k);
#pragma unroll
        for (int j = 0; j < 3; j++) {
            ac[j] = __ldg(L0.agg + c[j]);
            tc[j] = __ldg(L0.t + c[j]);
        }
        const V2 yk = __ldcg(y1 + ak);
#pragma unroll
        for (int j = 0; j < 3; j++) yc[j] = __ldcg(y1 + ac[j]);
        T sx = keep * (tk.x * yk.x - tk.y * yk.y), sy = keep * (tk.x * yk.y + tk.y * yk.x);
#pragma unroll
        for (int j = 0; j < 3; j++) {
            const T ux = tc[j].x * yc[j].x - tc[j].y * yc[j].y, uy = tc[j].x * yc[j].y + tc[j].y * yc[j].x;
            sx -= opd * (a[j].x * ux - a[j].y * uy);
            sy -= opd * (a[j].x * uy + a[j].y * ux);
        }
        V2 o;
        o.x = sx;
        o.y = sy;
        vv[k] = o;
    }
}

// Level-0 phase E: z = S r + alpha (I - omega A / d) v, i.e.
// z_k = omega/d ((2 - omega) r_k - omega/d sum_j A_kj r_j) + alpha ((1 - omega) v_k - omega/d sum_j A_kj v_j)
// over the three neighbours; adds the partials Re r^H z and |r|^2.
template <typename T>
__device__ __forceinline__ void l0_smooth_up(const ComplexEll<T>& A, const DevLevel0<T>& L0,
                                             const typename V2of<T>::type* r, const typename V2of<T>::type* vv,
                                             typename V2of<T>::type* __restrict__ z, T& rz, T& rr) {
    using V2 = typename V2of<T>::type;
    const int n = A.n, stride = gridDim.x * blockDim.x;
    const T om = L0.omega, od = L0.omega * L0.dinv, al = L0.alpha;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride) {
        int c[3];
        V2 a[3], rc[3], vc[3];
#pragma unroll
        for (int j = 0; j < 3; j++) {
            c[j] = __ldg(A.nbr + j * n + k);
            a[j] = __ldg(A.val + j * n + k);
        }
        const V2 rk = __ldcg(r + k), vk = __ldcg(vv + k);
#pragma unroll
        for (int j = 0; j < 3; j++) {
            rc[j] = __ldcg(r + c[j]);
            vc[j] = __ldcg(vv + c[j]);
        }
        T sx = (T(2) - om) * rk.x, sy = (T(2) - om) * rk.y;
        T ux = (T(1) - om) * vk.x, uy = (T(1) - om) * vk.y;
#pragma unroll
        for (int j = 0; j < 3; j++) {
            sx -= od * (a[j].x * rc[j].x - a[j].y * rc[j].y);
            sy -= od * (a[j].x * rc[j].y + a[j].y * rc[j].x);
            ux -= od * (a[j].x * vc[j].x - a[j].y * vc[j].y);
            uy -= od * (a[j].x * vc[j].y + a[j].y * vc[j].x);
        }
        V2 zk;
        zk.x = od * sx + al * ux;
        zk.y = od * sy + al * uy;
        z[k] = zk;
        rz += rk.x * zk.x + rk.y * zk.y;
        rr += rk.x * rk.x + rk.y * rk.y;
    }
}

// PCG with the V-cycle preconditioner (status codes as pcg_complex).  Per iteration: phase A
// (direction + SpMV), B (residual, solution, pre-smoothed residual), C (restriction), the inner
// cycle, D (smoothed prolongation), E (post-smoothing, z and the r^H z, |r|^2 partials):
// 2 nlev_inner + 6 grid barriers.  Residual and direction are double-buffered (r0/r1, p0/p1)
// because neighbours recompute them; sv and vv hold the level-0 intermediates.
template <typename T>
__global__ void __launch_bounds__(kBlock, 1) pcg_complex_mg(ComplexEll<T> A, DevLevel0<T> L0, T dg,
                                                        const DevHierarchy<T>* __restrict__ Hp,
                                                        const typename V2of<T>::type* __restrict__ b,
                                                        typename V2of<T>::type* x, typename V2of<T>::type* r0,
                                                        typename V2of<T>::type* r1, typename V2of<T>::type* z,
                                                        typename V2of<T>::type* p0, typename V2of<T>::type* p1,
                                                        typename V2of<T>::type* q, typename V2of<T>::type* sv,
                                                        typename V2of<T>::type* vv, T* partials, GridBarrier bar,
                                                        double tol2, int maxit, int* out) {
    using V2 = typename V2of<T>::type;
    const DevHierarchy<T>& H = *Hp;
    V2* rl1 = H.nlev > 0 ? H.L[0].r : H.rc;
    const V2* yl1 = H.nlev > 0 ? H.L[0].y : H.yc;
    const int n = A.n;
    const int stride = gridDim.x * blockDim.x;
    const int t0 = blockIdx.x * blockDim.x + threadIdx.x;
    T red2[2];
    T red1[1];
    int status = 3, it = 0;
    T rr = T(0);
    V2* rcur = r0;
    V2* rnext = r1;
    for (int i = t0; i < n; i += stride) {
        V2 ax = A.row(i, x);
        V2 bi = b[i];
        V2 ri;
        ri.x = bi.x - ax.x;
        ri.y = bi.y - ax.y;
        rcur[i] = ri;
    }
    if (!grid_sync(bar)) { status = 5; goto done; }
    l0_update_smooth<T>(A, L0, rcur, nullptr, T(0), nullptr, nullptr, nullptr, sv, false);
    if (!grid_sync(bar)) { status = 5; goto done; }
    l0_restrict<T>(A, L0, sv, rl1);
    if (!grid_sync(bar)) { status = 5; goto done; }
    if (!vcycle_inner(H, bar)) { status = 5; goto done; }
    l0_prolong<T>(A, L0, yl1, vv);
    if (!grid_sync(bar)) { status = 5; goto done; }
    red2[0] = T(0);
    red2[1] = T(0);
    l0_smooth_up<T>(A, L0, rcur, vv, z, red2[0], red2[1]);
    publish_partials<T, 2>(red2, partials);
    if (!grid_sync(bar)) { status = 5; goto done; }
    gather_partials<T, 2>(partials, red2);
    {
        T rz = red2[0];
        rr = red2[1];
        T beta = T(0);
        const V2* pold = z;   // first direction p = z
        V2* pw = p0;
        for (;;) {
            if ((double)rr <= tol2) { status = 0; break; }
            if (it >= maxit) { status = 3; break; }
            red1[0] = l0_direction_spmv<T>(A, dg, z, pold, beta, pw, q);
            publish_partials<T, 1>(red1, partials + 2 * gridDim.x);
            if (!grid_sync(bar)) { status = 5; break; }
            gather_partials<T, 1>(partials + 2 * gridDim.x, red1);
            const T pq = red1[0];
            if (!(pq > T(0))) { status = 4; break; }
            const T alpha = rz / pq;
            l0_update_smooth<T>(A, L0, rcur, q, alpha, pw, x, rnext, sv, true);
            if (!grid_sync(bar)) { status = 5; break; }
            {
                V2* tmp = rcur;
                rcur = rnext;
                rnext = tmp;
            }
            l0_restrict<T>(A, L0, sv, rl1);
            if (!grid_sync(bar)) { status = 5; break; }
            if (!vcycle_inner(H, bar)) { status = 5; break; }
            l0_prolong<T>(A, L0, yl1, vv);
            if (!grid_sync(bar)) { status = 5; break; }
            red2[0] = T(0);
            red2[1] = T(0);
            l0_smooth_up<T>(A, L0, rcur, vv, z, red2[0], red2[1]);
            publish_partials<T, 2>(red2, partials + 3 * gridDim.x);
            if (!grid_sync(bar)) { status = 5; break; }
            gather_partials<T, 2>(partials + 3 * gridDim.x, red2);
            const T rz_new = red2[0];
            rr = red2[1];
            if (rr != rr || !(rz_new > T(0))) { status = 4; break; }
            beta = rz_new / rz;
            rz = rz_new;
            pold = pw;
            pw = (pw == p0) ? p1 : p0;
            it++;
        }
    }
done:
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        out[0] = status;
        out[1] = it;
        reinterpret_cast<double*>(out + 4)[0] = (double)rr;
    }
}

// ---------------------------------------------------------------------------- FP64 vector kernels
// K1: Lu = L u (FP64), b = M u, partials [u^H L u, u^H M u, |b|^2]
__global__ void power_prepare(ComplexEll<double> A, const double* __restrict__ area, const double2* __restrict__ u,
                              double2* b, double2* Lu, double* partials) {
    double red[3] = {0, 0, 0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < A.n; i += gridDim.x * blockDim.x) {
        double2 ui = u[i];
        double2 li = A.row(i, u);
        double a = area[i];
        double2 bi = make_double2(a * ui.x, a * ui.y);
        Lu[i] = li;
        b[i] = bi;
        red[0] += ui.x * li.x + ui.y * li.y;
        red[1] += a * (ui.x * ui.x + ui.y * ui.y);
        red[2] += bi.x * bi.x + bi.y * bi.y;
    }
    publish_partials<double, 3>(red, partials);
}

// Sums K partials per slot (written by a grid of nb blocks) into out[0..K) in fixed order.
__global__ void finalize_partials(const double* partials, int nb, int K, double* out) {
    __shared__ double s[kBlock];
    for (int k = 0; k < K; k++) {
        double x = 0;
        for (int i = threadIdx.x; i < nb; i += blockDim.x) x += partials[k * nb + i];
        s[threadIdx.x] = x;
        __syncthreads();
        for (int w = blockDim.x / 2; w > 0; w >>= 1) {
            if (threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
            __syncthreads();
        }
        if (threadIdx.x == 0) out[k] = s[0];
        __syncthreads();
    }
}

// Subspace warm start.  The inverse iterates on a sphere stay inside a nearly degenerate
// cluster of eigenvectors, so the previous m iterates span the solution well: the start of
// each solve is the Galerkin solution of L x = b on V = [u_k, ..., u_{k-m+1}] (L V is kept
// from power_prepare, so no extra operator applications).  m = 6: at 1.3M faces the field stage
// took 535 / 505 / 502 / 496 ms with m = 12 / 8 / 6 / 4 (2284 / 2235 / 2257 / 2287 PCG passes):
// the Gram row and the start combination cost 4 complex FP64 multiply-adds per vector and row,
// which the GB300's FP64 rate makes the larger term beyond six vectors.
constexpr int kRing = 6;

// partials for j < cnt: [Re, Im] of u^H (L V_j) and of V_j^H b
struct RingPtrs { const double2* V[kRing]; const double2* LV[kRing]; int cnt; };

// One pass over the rows for all C ring vectors (u and b read once); per j the same row order
// and the same fixed-order block and grid reductions as one pass per vector.
template <int C>
__global__ void gram_row(int n, RingPtrs R, const double2* __restrict__ u, const double2* __restrict__ b,
                         double* partials) {
    double red[4 * C];
#pragma unroll
    for (int k = 0; k < 4 * C; k++) red[k] = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double2 ui = u[i], bi = b[i];
#pragma unroll
        for (int j = 0; j < C; j++) {
            const double2 li = R.LV[j][i], vi = R.V[j][i];
            red[4 * j + 0] += ui.x * li.x + ui.y * li.y;   // conj(u) * Lv
            red[4 * j + 1] += ui.x * li.y - ui.y * li.x;
            red[4 * j + 2] += vi.x * bi.x + vi.y * bi.y;   // conj(v) * b
            red[4 * j + 3] += vi.x * bi.y - vi.y * bi.x;
        }
    }
    publish_partials<double, 4 * C>(red, partials);
}

struct StartCoef { double re[kRing], im[kRing]; const double2* V[kRing]; const double2* LV[kRing]; int cnt; };

// x = V y, r = b - (L V) y, r32 = r, partial |r|^2 (C ring vectors, unrolled)
template <int C>
__global__ void combine_start(int n, StartCoef c, const double2* __restrict__ b, double2* x, double2* r, float2* r32,
                              double* partials) {
    double red[1] = {0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double xr = 0, xi = 0, lr = 0, li = 0;
#pragma unroll
        for (int j = 0; j < C; j++) {
            double2 v = c.V[j][i], l = c.LV[j][i];
            xr += c.re[j] * v.x - c.im[j] * v.y;
            xi += c.re[j] * v.y + c.im[j] * v.x;
            lr += c.re[j] * l.x - c.im[j] * l.y;
            li += c.re[j] * l.y + c.im[j] * l.x;
        }
        double2 bi = b[i];
        double2 ri = make_double2(bi.x - lr, bi.y - li);
        x[i] = make_double2(xr, xi);
        r[i] = ri;
        if (r32) r32[i] = make_float2((float)ri.x, (float)ri.y);
        red[0] += ri.x * ri.x + ri.y * ri.y;
    }
    publish_partials<double, 1>(red, partials);
}

// the kernels above for a ring count known only at run time (1 .. kRing)
template <int C = 1>
void launch_gram(int cnt, int G, cudaStream_t st, int n, const RingPtrs& R, const double2* u, const double2* b,
                 double* partials) {
    if constexpr (C < kRing) {
        if (cnt != C) return launch_gram<C + 1>(cnt, G, st, n, R, u, b, partials);
    }
    gram_row<C><<<G, kStream, 0, st>>>(n, R, u, b, partials);
}
template <int C = 1>
void launch_combine(int cnt, int G, cudaStream_t st, int n, const StartCoef& sc, const double2* b, double2* x,
                    double2* r, float2* r32, double* partials) {
    if constexpr (C < kRing) {
        if (cnt != C) return launch_combine<C + 1>(cnt, G, st, n, sc, b, x, r, r32, partials);
    }
    combine_start<C><<<G, kStream, 0, st>>>(n, sc, b, x, r, r32, partials);
}

// K3: x += e (FP32 correction), r = b - L x in FP64, r32 = r, partial |r|^2.
// The residual needs all of x updated, so the correction is added by a separate pass first.
__global__ void add_correction(int n, const float2* __restrict__ e, double2* x) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float2 ei = e[i];
        double2 xi = x[i];
        xi.x += (double)ei.x;
        xi.y += (double)ei.y;
        x[i] = xi;
    }
}

__global__ void residual64(ComplexEll<double> A, const double2* __restrict__ b, const double2* __restrict__ x,
                           double2* r, float2* r32, double* partials) {
    double red[1] = {0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < A.n; i += gridDim.x * blockDim.x) {
        double2 ax = A.row(i, x);
        double2 bi = b[i];
        double2 ri = make_double2(bi.x - ax.x, bi.y - ax.y);
        r[i] = ri;
        if (r32) r32[i] = make_float2((float)ri.x, (float)ri.y);
        red[0] += ri.x * ri.x + ri.y * ri.y;
    }
    publish_partials<double, 1>(red, partials);
}

// K4: partial x^H M x.  K5: x /= sqrt|x^H M x| (scalar read on device), u = x.
__global__ void mnorm_partial(int n, const double* __restrict__ area, const double2* __restrict__ x, double* partials) {
    double red[1] = {0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double2 xi = x[i];
        red[0] += area[i] * (xi.x * xi.x + xi.y * xi.y);
    }
    publish_partials<double, 1>(red, partials);
}

__global__ void normalize_to(int n, const double* __restrict__ scal, const double2* __restrict__ x, double2* u) {
    const double s = sqrt(fabs(scal[0]));
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double2 xi = x[i];
        u[i] = make_double2(xi.x / s, xi.y / s);
    }
}

// Stand-alone SpMV y = L x over the ELL rows (read-only x: gathers through the read-only path),
// one thread per row at full occupancy; used to measure the SpMV against the HBM roofline.
template <typename T>
__global__ void __launch_bounds__(256) spmv_ell(ComplexEll<T> A, const typename V2of<T>::type* __restrict__ x,
                                                typename V2of<T>::type* __restrict__ y) {
    using V2 = typename V2of<T>::type;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.n) return;
    int c[3];
    V2 a[3], xc[3];
#pragma unroll
    for (int j = 0; j < 3; j++) {
        c[j] = __ldg(A.nbr + j * A.n + i);
        a[j] = __ldg(A.val + j * A.n + i);
    }
    const V2 xi = __ldg(x + i);
    const T d = __ldg(A.diag + i);
#pragma unroll
    for (int j = 0; j < 3; j++) xc[j] = __ldg(x + c[j]);
    T re = d * xi.x, im = d * xi.y;
#pragma unroll
    for (int j = 0; j < 3; j++) {
        re += a[j].x * xc[j].x - a[j].y * xc[j].y;
        im += a[j].x * xc[j].y + a[j].y * xc[j].x;
    }
    V2 o;
    o.x = re;
    o.y = im;
    y[i] = o;
}

// Start of a plain solve L x = b: x = 0, r = b, r32 = r, partial |b|^2.
__global__ void start_from_rhs(int n, const double2* __restrict__ b, double2* x, double2* r, float2* r32,
                               double* partials) {
    double red[1] = {0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double2 bi = b[i];
        x[i] = make_double2(0.0, 0.0);
        r[i] = bi;
        if (r32) r32[i] = make_float2((float)bi.x, (float)bi.y);
        red[0] += bi.x * bi.x + bi.y * bi.y;
    }
    publish_partials<double, 1>(red, partials);
}

// ---------------------------------------------------------------- reverse power iteration
// Adjoint of u_{k+1} = x / s, x = L^-1 M u_k, s = sqrt(x^H M x) (the field's inverse power
// iteration), for a loss seeded through the field angle phi_f = arg(c_f) / N of the last iterate
// c.  With the real inner product <a, b> = Re(a^H b):
//   seed       gu = i dphi c / (N |c|^2)                (dl = <gu, dc>)
//   per step   a = <gu, u_{k+1}>, gx = (gu - a M u_{k+1}) / s_{k+1}, d area -= a |u_{k+1}|^2 / 2;
//              L mu = gx (the same Hermitian solve as the forward step);
//              d area_f += Re(conj(mu_f) u_k,f), d theta_fj += N Im(conj(mu_f) L_fj x_g)
//              (dL_fj / dtheta = i N L_fj, x = s u_{k+1}), gu = M mu.
__global__ void adj_seed(int n, int N, const double* __restrict__ dphi, const double2* __restrict__ c, double2* gu) {
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < n; f += gridDim.x * blockDim.x) {
        const double2 cf = c[f];
        const double w = dphi[f] / ((double)N * (cf.x * cf.x + cf.y * cf.y));
        gu[f] = make_double2(-w * cf.y, w * cf.x);
    }
}

// block partials of Re(gu^H u)
__global__ void adj_dot(int n, const double2* __restrict__ gu, const double2* __restrict__ u, double* partials) {
    double v[1] = {0.0};
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < n; f += gridDim.x * blockDim.x) {
        const double2 g = gu[f], w = u[f];
        v[0] += g.x * w.x + g.y * w.y;
    }
    block_sum<double, 1>(v);
    if (threadIdx.x == 0) partials[blockIdx.x] = v[0];
}

// gx = (gu - a area u) / s into b; g_area -= a |u|^2 / 2.  scal[0] = a, s2[0] = s^2.
__global__ void adj_rhs(int n, const double2* __restrict__ gu, const double2* __restrict__ u,
                        const double* __restrict__ area, const double* __restrict__ scal, const double* __restrict__ s2,
                        double2* b, double* g_area) {
    const double a = scal[0], s = sqrt(fabs(s2[0]));
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < n; f += gridDim.x * blockDim.x) {
        const double2 g = gu[f], w = u[f];
        const double m = area[f];
        b[f] = make_double2((g.x - a * m * w.x) / s, (g.y - a * m * w.y) / s);
        g_area[f] -= 0.5 * a * (w.x * w.x + w.y * w.y);
    }
}

// after L mu = gx: the area and transport-angle terms of this step and gu = M mu
__global__ void adj_accumulate(ComplexEll<double> A, int N, const double2* __restrict__ mu, const double2* __restrict__ u,
                               const double2* __restrict__ uprev, const double* __restrict__ s2,
                               const double* __restrict__ area, double* g_area, double* g_theta, double2* gu) {
    const int n = A.n;
    const double s = sqrt(fabs(s2[0]));
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < n; f += gridDim.x * blockDim.x) {
        const double2 m = mu[f], up = uprev[f];
        g_area[f] += m.x * up.x + m.y * up.y;
#pragma unroll
        for (int j = 0; j < 3; j++) {
            const int g = A.nbr[j * n + f];
            if (g == f) continue;   // a boundary side: no transport angle
            const double2 l = A.val[j * n + f], w = u[g];
            const double xr = s * w.x, xi = s * w.y;
            const double lr = l.x * xr - l.y * xi, li = l.x * xi + l.y * xr;   // L_fj x_g
            g_theta[j * n + f] += (double)N * (m.x * li - m.y * lr);            // N Im(conj(mu) L x)
        }
        const double a = area[f];
        gu[f] = make_double2(a * m.x, a * m.y);
    }
}

__global__ void zero_f2(int n, float2* e) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) e[i] = make_float2(0.f, 0.f);
}

}  // namespace mtk

using namespace mtk;

namespace {

// y = G^+ h for a small Hermitian G (cnt x cnt), through the real symmetric embedding
// [[Re G, -Im G], [Im G, Re G]] and cyclic Jacobi rotations; eigenvalues below
// 1e-12 * max are dropped (the warm-start basis becomes nearly dependent as the iterates settle).
void hermitian_pinv_solve(const std::vector<double>& Gr, const std::vector<double>& Gi, const std::vector<double>& hr,
                          const std::vector<double>& hi, int cnt, std::vector<double>& yr, std::vector<double>& yi) {
    const int m = 2 * cnt;
    std::vector<double> A((size_t)m * m), Vm((size_t)m * m, 0.0), rhs(m);
    for (int i = 0; i < cnt; i++)
        for (int j = 0; j < cnt; j++) {
            double a = Gr[i * kRing + j], b = Gi[i * kRing + j];
            A[(size_t)i * m + j] = a;
            A[(size_t)(i + cnt) * m + (j + cnt)] = a;
            A[(size_t)i * m + (j + cnt)] = -b;
            A[(size_t)(i + cnt) * m + j] = b;
        }
    for (int i = 0; i < cnt; i++) { rhs[i] = hr[i]; rhs[i + cnt] = hi[i]; }
    for (int i = 0; i < m; i++) Vm[(size_t)i * m + i] = 1.0;
    for (int sweep = 0; sweep < 60; sweep++) {
        double off = 0;
        for (int p = 0; p < m; p++) for (int q = p + 1; q < m; q++) off += A[(size_t)p * m + q] * A[(size_t)p * m + q];
        if (off < 1e-30) break;
        for (int p = 0; p < m; p++)
            for (int q = p + 1; q < m; q++) {
                double apq = A[(size_t)p * m + q];
                if (std::fabs(apq) < 1e-300) continue;
                double app = A[(size_t)p * m + p], aqq = A[(size_t)q * m + q];
                double theta = (aqq - app) / (2 * apq);
                double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1));
                double c = 1 / std::sqrt(t * t + 1), sn = t * c;
                for (int k = 0; k < m; k++) {
                    double akp = A[(size_t)k * m + p], akq = A[(size_t)k * m + q];
                    A[(size_t)k * m + p] = c * akp - sn * akq;
                    A[(size_t)k * m + q] = sn * akp + c * akq;
                }
                for (int k = 0; k < m; k++) {
                    double apk = A[(size_t)p * m + k], aqk = A[(size_t)q * m + k];
                    A[(size_t)p * m + k] = c * apk - sn * aqk;
                    A[(size_t)q * m + k] = sn * apk + c * aqk;
                }
                for (int k = 0; k < m; k++) {
                    double vkp = Vm[(size_t)k * m + p], vkq = Vm[(size_t)k * m + q];
                    Vm[(size_t)k * m + p] = c * vkp - sn * vkq;
                    Vm[(size_t)k * m + q] = sn * vkp + c * vkq;
                }
            }
    }
    double lmax = 0;
    for (int k = 0; k < m; k++) lmax = std::max(lmax, std::fabs(A[(size_t)k * m + k]));
    std::vector<double> y(m, 0.0);
    for (int k = 0; k < m; k++) {
        double lam = A[(size_t)k * m + k];
        if (!(lam > 1e-12 * lmax)) continue;
        double d = 0;
        for (int i = 0; i < m; i++) d += Vm[(size_t)i * m + k] * rhs[i];
        d /= lam;
        for (int i = 0; i < m; i++) y[i] += d * Vm[(size_t)i * m + k];
    }
    yr.assign(y.begin(), y.begin() + cnt);
    yi.assign(y.begin() + cnt, y.end());
}

struct FieldSolver {
    mtk_ctx* c;
    int n;
    DBuf<int> nbr, nbr_in;
    DBuf<double> theta, area, d64, inv64;
    DBuf<float> d32, inv32, area32;
    DBuf<double2> v64, u, b, Lu, x, r, z64, p64, q64;
    DBuf<double2> ringU[kRing], ringL[kRing];
    DBuf<float2> v32, r32, e32, z32, p32, q32;
    int grid = 0;
    double pcg_ms = 0, pcg_bytes = 0;
    long long pcg_launches = 0, pcg_passes = 0;
    // multigrid hierarchy (host-built, device-resident), both precisions
    struct CsrBufs {
        DBuf<int> ptr, col;
        DBuf<double2> v64;
        DBuf<float2> v32;
        int n = 0, group = 1;
        size_t nnz = 0;
        SellIdx sell;              // SELL-32 copy (mtk_sell.cuh) where sell_worth holds
        DBuf<double2> s64;
        DBuf<float2> s32;
    };
    struct LevelBufs {
        CsrBufs R, S, P;
        DBuf<double2> r64, y64;
        DBuf<float2> r32, y32;
    } lvb[kMaxLevels];
    DBuf<double2> Ainv64, rc64, yc64;
    DBuf<float2> Ainv32, rc32, yc32;
    DevHierarchy<double> H64{};
    DevHierarchy<float> H32{};
    DBuf<unsigned char> hier_dev64, hier_dev32;   // device copies of the hierarchy descriptors
    // level 0 (applied from the ELL rows): rows renumbered by aggregate, perm[new] = old
    std::vector<int> perm;
    DBuf<int> agg0, chunk0;
    DBuf<double2> t064, rb64, pb64, sv64, vv64;
    DBuf<float2> t032, rb32, pb32, sv32, vv32;
    DevLevel0<double> L064{};
    DevLevel0<float> L032{};
    bool amg = false;
    int amg_levels = 0, amg_coarse = 0;
    double vcycle_bytes64 = 0, vcycle_bytes32 = 0;   // algorithmic bytes of one inner cycle (levels >= 1)

    int upload_csr(const HostCsr& M, CsrBufs& B, int group) {
        cudaStream_t st = c->stream;
        B.n = M.n;
        B.group = group;
        B.nnz = M.col.size();
        MTK_TRY(B.ptr.upload(M.ptr.data(), M.ptr.size(), st));
        MTK_TRY(B.col.upload(M.col.data(), M.col.size(), st));
        std::vector<double2> v64(M.val.size());
        std::vector<float2> v32(M.val.size());
        for (size_t i = 0; i < M.val.size(); i++) {
            v64[i] = make_double2(M.val[i].real(), M.val[i].imag());
            v32[i] = make_float2((float)M.val[i].real(), (float)M.val[i].imag());
        }
        MTK_TRY(B.v64.upload(v64.data(), v64.size(), st));
        MTK_TRY(B.v32.upload(v32.data(), v32.size(), st));
        return MTK_OK;
    }

    // Builds the aggregation hierarchy from theta (same off-diagonals as field_assemble) on the
    // original face numbering and sets perm (rows numbered by level-0 aggregate).  Level 0 keeps
    // no matrices; levels >= 1 are uploaded as CSR cycle operators.  Leaves amg false (Jacobi)
    // when the mesh is too small to coarsen.
    int build_amg(const int* nbr_h, const double* theta_h, int N) {
        const double pi = 3.14159265358979323846;
        std::vector<int> nbr3(nbr_h, nbr_h + 3 * (size_t)n);
        std::vector<std::complex<double>> vals(3 * (size_t)n);
#pragma omp parallel for schedule(static)
        for (int f = 0; f < n; f++)
            for (int j = 0; j < 3; j++) {
                double ang = (double)N * (theta_h[3 * f + j] + pi);
                vals[(size_t)j * n + f] = std::complex<double>(-std::cos(ang), -std::sin(ang));
            }
        // the Galerkin products run on the device (CDevBuilder, the same arrays as the host
        // build); the host builds when the device build declines (a row beyond its capacity)
        HostHierarchy HH;
        const auto tb0 = std::chrono::steady_clock::now();
        std::vector<DevCycleOpsC> dops;
        HostLevel dL0;
        bool dev_ok = false;
        if (!getenv("MTK_MG_HOST")) {
            CDevBuilder B(c, c->stream);
            std::vector<std::complex<double>> dAinv;
            int dnc = 0;
            MTK_TRY(B.build(ell_to_csr(n, nbr3, vals, 3.0 + 1e-9), dL0, dops, dnc, dAinv, dev_ok));
            if (dev_ok) { HH.nc = dnc; HH.Ainv = std::move(dAinv); }
        }
        if (!dev_ok) {
            dops.clear();
            if (!build_hierarchy(n, nbr3, vals, 3.0 + 1e-9, HH, 1)) return MTK_OK;   // keep Jacobi
        }
        {
            const char* e = getenv("MTK_DEBUG");
            if (e && e[0] == '1')
                fprintf(stderr, "[field host]   (hierarchy build %.1f ms, %s)\n",
                        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - tb0).count(),
                        dev_ok ? "device Galerkin products" : "host");
        }
        const int nl = dev_ok ? (int)dops.size() : (int)HH.lv.size();
        if (nl == 0) return MTK_OK;
        const HostLevel& L0 = dev_ok ? dL0 : HH.lv[0];
        const int nagg = (int)L0.mptr.size() - 1;
        // chunks of <= 32 rows holding whole aggregates
        std::vector<int> chunk{0};
        for (int a2 = 0; a2 < nagg; a2++) {
            const int sz = L0.mptr[a2 + 1] - L0.mptr[a2];
            if (sz > 32) return MTK_OK;   // a chunk must hold a whole aggregate
            if (L0.mptr[a2 + 1] - chunk.back() > 32) chunk.push_back(L0.mptr[a2]);
        }
        chunk.push_back(n);
        perm = L0.mem;
        cudaStream_t st = c->stream;
        {
            std::vector<int> ag(n);
            std::vector<double2> t64(n);
            std::vector<float2> t32(n);
            for (int a2 = 0; a2 < nagg; a2++)
                for (int k = L0.mptr[a2]; k < L0.mptr[a2 + 1]; k++) {
                    const std::complex<double> tv = L0.T[perm[k]];
                    ag[k] = a2;
                    t64[k] = make_double2(tv.real(), tv.imag());
                    t32[k] = make_float2((float)tv.real(), (float)tv.imag());
                }
            MTK_TRY(agg0.upload(ag.data(), ag.size(), st));
            MTK_TRY(t064.upload(t64.data(), t64.size(), st));
            MTK_TRY(t032.upload(t32.data(), t32.size(), st));
            MTK_TRY(chunk0.upload(chunk.data(), chunk.size(), st));
        }
        const int nchunk = (int)chunk.size() - 1;
        const double dg = 3.0 + 1e-9;
        L064 = DevLevel0<double>{nagg, nchunk, agg0.p, t064.p, chunk0.p, 1.0 / dg, kOmega, kAlpha, L0.wp};
        L032 = DevLevel0<float>{nagg, nchunk, agg0.p, t032.p, chunk0.p, (float)(1.0 / dg), (float)kOmega, (float)kAlpha,
                                (float)L0.wp};
        // lanes per row of a CSR phase: fewest rounds x dependent loads (ptr, then batches of four
        // entries per lane, each a column load and a gather) over the persistent grid
        const double threads = (double)c->num_sms * kBlock;
        auto grp = [&](int rows, double avg) {
            int best = 1;
            double bc = 1e300;
            for (int g = 1; g <= 32; g <<= 1) {
                const double rounds = std::ceil(rows * (double)g / threads);
                const double cost = rounds * (1.0 + 2.0 * std::ceil(avg / (4.0 * g)));
                if (cost < bc - 1e-9) { bc = cost; best = g; }
            }
            return best;
        };
        auto avg = [](const HostCsr& M) { return M.n > 0 ? (double)M.col.size() / M.n : 0.0; };
        auto davg = [](const DevCsrC& M) { return M.n > 0 ? (double)M.nnz / M.n : 0.0; };
        // a matrix for which the cost model picks several lanes per row, with enough rows to fill
        // the grid with one lane per row and short rows, gets a SELL-32 copy and one lane per row
        const bool use_sell = !getenv("MTK_NO_SELL");
        auto worth = [&](int rows, double a) { return use_sell && sell_worth(rows, a); };
        auto sgrp = [&](int rows, double a) { return worth(rows, a) ? 1 : grp(rows, a); };
        bool up_sell = false, r_sell = false;
        // adopt a device CSR (FP64 values) and its FP32 copy
        auto adopt = [&](DevCsrC& D, CsrBufs& B, int group) -> int {
            B.n = D.n;
            B.group = group;
            B.nnz = D.nnz;
            B.ptr = std::move(D.ptr);
            B.col = std::move(D.col);
            B.v64 = std::move(D.val);
            MTK_TRY(B.v32.alloc(std::max<size_t>(D.nnz, 1)));
            if (D.nnz) cgpu::to_f32_vals<<<stream_grid(c), kStream, 0, st>>>(D.nnz, B.v64.p, B.v32.p);
            MTK_CUDA_TRY(cudaGetLastError());
            return MTK_OK;
        };
        const int ni = nl - 1;   // inner (CSR) levels
        std::vector<double> lv_nnz(3 * (size_t)std::max(ni, 1)), lv_n(2 * (size_t)std::max(ni, 1));
        for (int i = 0; i < ni; i++) {
            LevelBufs& B = lvb[i];
            int ln = 0;
            if (dev_ok) {
                DevCycleOpsC& O = dops[i + 1];
                lv_nnz[3 * i] = (double)O.R.nnz; lv_nnz[3 * i + 1] = (double)O.S.nnz; lv_nnz[3 * i + 2] = (double)O.P.nnz;
                lv_n[2 * i] = O.S.n; lv_n[2 * i + 1] = O.R.n;
                up_sell = worth(O.S.n, std::max(davg(O.S), davg(O.P)));
                r_sell = worth(O.R.n, davg(O.R));
                const int up = sgrp(O.S.n, std::max(davg(O.S), davg(O.P)));
                MTK_TRY(adopt(O.R, B.R, sgrp(O.R.n, davg(O.R))));
                MTK_TRY(adopt(O.S, B.S, up));
                MTK_TRY(adopt(O.P, B.P, up));
                ln = B.S.n;
            } else {
                const HostCycleOps& O = HH.ops[i + 1];
                lv_nnz[3 * i] = (double)O.R.col.size(); lv_nnz[3 * i + 1] = (double)O.S.col.size(); lv_nnz[3 * i + 2] = (double)O.P.col.size();
                lv_n[2 * i] = O.S.n; lv_n[2 * i + 1] = O.R.n;
                up_sell = worth(O.S.n, std::max(avg(O.S), avg(O.P)));
                r_sell = worth(O.R.n, avg(O.R));
                MTK_TRY(upload_csr(O.R, B.R, sgrp(O.R.n, avg(O.R))));
                const int up = sgrp(O.S.n, std::max(avg(O.S), avg(O.P)));
                MTK_TRY(upload_csr(O.S, B.S, up));
                MTK_TRY(upload_csr(O.P, B.P, up));
                ln = O.S.n;
            }
            MTK_TRY(B.r64.alloc(ln)); MTK_TRY(B.r32.alloc(ln));
            MTK_TRY(B.y64.alloc(ln)); MTK_TRY(B.y32.alloc(ln));
            for (CsrBufs* C : {&B.R, &B.S, &B.P})
                if (C->n > 0 && (C == &B.R ? r_sell : up_sell)) {
                    MTK_TRY(sell_build_index(c, st, C->n, C->ptr.p, C->col.p, C->sell));
                    MTK_TRY(sell_fill_values<double2>(c, st, C->n, C->ptr.p, C->col.p, C->v64.p, C->sell, C->s64));
                    MTK_TRY(sell_fill_values<float2>(c, st, C->n, C->ptr.p, C->col.p, C->v32.p, C->sell, C->s32));
                }
            auto mk64 = [](const CsrBufs& C) {
                DevCsr<double> M{C.n, C.group, C.ptr.p, C.col.p, C.v64.p};
                if (C.sell.sptr.p) { M.sptr = C.sell.sptr.p; M.scol = C.sell.scol.p; M.sval = C.s64.p; }
                return M;
            };
            auto mk32 = [](const CsrBufs& C) {
                DevCsr<float> M{C.n, C.group, C.ptr.p, C.col.p, C.v32.p};
                if (C.sell.sptr.p) { M.sptr = C.sell.sptr.p; M.scol = C.sell.scol.p; M.sval = C.s32.p; }
                return M;
            };
            H64.L[i] = DevLevel<double>{mk64(B.R), mk64(B.S), mk64(B.P), B.r64.p, B.y64.p};
            H32.L[i] = DevLevel<float>{mk32(B.R), mk32(B.S), mk32(B.P), B.r32.p, B.y32.p};
        }
        std::vector<double2> a64(HH.Ainv.size());
        std::vector<float2> a32(HH.Ainv.size());
        for (size_t i = 0; i < HH.Ainv.size(); i++) {
            a64[i] = make_double2(HH.Ainv[i].real(), HH.Ainv[i].imag());
            a32[i] = make_float2((float)HH.Ainv[i].real(), (float)HH.Ainv[i].imag());
        }
        MTK_TRY(Ainv64.upload(a64.data(), a64.size(), st));
        MTK_TRY(Ainv32.upload(a32.data(), a32.size(), st));
        MTK_TRY(rc64.alloc(HH.nc)); MTK_TRY(yc64.alloc(HH.nc));
        MTK_TRY(rc32.alloc(HH.nc)); MTK_TRY(yc32.alloc(HH.nc));
        H64.nlev = ni; H64.nc = HH.nc; H64.Ainv = Ainv64.p; H64.rc = rc64.p; H64.yc = yc64.p;
        H32.nlev = ni; H32.nc = HH.nc; H32.Ainv = Ainv32.p; H32.rc = rc32.p; H32.yc = yc32.p;
        // inner-cycle traffic: every matrix entry once (value + column) plus row pointers, each
        // level vector read / written once per use, the dense coarsest inverse; plus the level-1
        // right-hand side written by the restriction and read by the level-0 prolongation
        {
            auto cyc = [&](double T) {
                double bt = 0;
                for (int i = 0; i < ni; i++) {
                    const double nnz = lv_nnz[3 * i] + lv_nnz[3 * i + 1] + lv_nnz[3 * i + 2];
                    const double nS = lv_n[2 * i], nR = lv_n[2 * i + 1];
                    bt += nnz * (2 * T + 4) + 4.0 * (nR + 2.0 * nS);
                    bt += 2 * T * (2.0 * nS + 2.0 * nR + nS);
                }
                bt += (double)HH.nc * HH.nc * 2 * T + 4.0 * HH.nc * T;
                bt += 2.0 * nagg * 2 * T;
                return bt;
            };
            vcycle_bytes64 = cyc(8);
            vcycle_bytes32 = cyc(4);
        }
        MTK_TRY(hier_dev64.alloc(sizeof(DevHierarchy<double>)));
        MTK_TRY(hier_dev32.alloc(sizeof(DevHierarchy<float>)));
        amg = true;
        amg_levels = nl;
        amg_coarse = HH.nc;
        return MTK_OK;
    }

    template <typename T> DevHierarchy<T> hier() const;
    ComplexEll<double> A64() const { return {n, nbr.p, v64.p, d64.p}; }
    ComplexEll<float> A32() const { return {n, nbr.p, v32.p, d32.p}; }

    int finalize(int nb, int K) {
        finalize_partials<<<1, kStream, 0, c->stream>>>(c->partials, nb, K, c->scalars);
        c->kernels++;
        MTK_CUDA_TRY(cudaGetLastError());
        return MTK_OK;
    }
    int read_scalars(int K) {
        MTK_CUDA_TRY(cudaMemcpyAsync(c->h_scalars, c->scalars, K * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        MTK_CUDA_TRY(cudaStreamSynchronize(c->stream));
        return MTK_OK;
    }
    // Runs the persistent PCG and returns its status, iterations in *iters.  rb / pb are the
    // second residual and direction buffers of the multigrid kernel.
    template <typename T, typename V2>
    int pcg(ComplexEll<T> A, const T* minv, const V2* bb, V2* xx, V2* rr, V2* zz, V2* pp, V2* qq, V2* rb, V2* pb,
            V2* sb, V2* vb, double tol2, int maxit, long long* iters, double* final_rr) {
        int g = 0;
        MTK_TRY(reset_barrier(c));
        MTK_CUDA_TRY(cudaEventRecord(c->ev_k0, c->stream));
        if (amg) {
            DevHierarchy<T> H = hier<T>();
            DevHierarchy<T>* Hd = reinterpret_cast<DevHierarchy<T>*>(sizeof(T) == 8 ? hier_dev64.p : hier_dev32.p);
            MTK_CUDA_TRY(cudaMemcpyAsync(Hd, &H, sizeof(H), cudaMemcpyHostToDevice, c->stream));
            const DevHierarchy<T>* Hc = Hd;
            const DevLevel0<T> L0 = level0<T>();
            const T dg = (T)(3.0 + 1e-9);
            MTK_TRY(launch_persistent(c, pcg_complex_mg<T>, &g, A, L0, dg, Hc, bb, xx, rr, rb, zz, pp, pb, qq, sb, vb,
                                      reinterpret_cast<T*>(c->partials), barrier_of(c), tol2, maxit, c->dev_int));
        } else {
            MTK_TRY(launch_persistent(c, pcg_complex<T>, &g, A, minv, bb, xx, rr, zz, pp, qq,
                                      reinterpret_cast<T*>(c->partials), barrier_of(c), tol2, maxit, c->dev_int));
        }
        MTK_CUDA_TRY(cudaEventRecord(c->ev_k1, c->stream));
        MTK_CUDA_TRY(cudaMemcpyAsync(c->h_int, c->dev_int, 8 * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
        MTK_CUDA_TRY(cudaStreamSynchronize(c->stream));
        float kms = 0;
        cudaEventElapsedTime(&kms, c->ev_k0, c->ev_k1);
        pcg_ms += kms;
        pcg_launches++;
        // algorithmic bytes per iteration and row.  Jacobi: SpMV 3*(2T+4) + T + 2*2T, x/r/p
        // updates 3*3*2T, z = M^-1 r T + 2T.  Multigrid, level 0 from the ELL rows (3*(2T+4) per
        // pass, five passes): A z, p_old in, p, q out (8T); B r, q, p, x in, x, r, s out (14T);
        // C s in + agg + T_k (2T + 4 + 2T); D agg + T_k, v out (4 + 4T); E r, v in, z out (6T);
        // plus the inner cycle (counted in build_amg)
        const double T_ = (double)sizeof(T);
        const double ell = 3.0 * (2 * T_ + 4);
        const double per_row = amg ? 5 * ell + 8 * T_ + 14 * T_ + (4 + 4 * T_) + (4 + 4 * T_) + 6 * T_
                                   : ell + T_ + 4.0 * T_ + 18.0 * T_ + 3.0 * T_;
        const double cyc = amg ? (sizeof(T) == 8 ? vcycle_bytes64 : vcycle_bytes32) : 0.0;
        pcg_bytes += (per_row * (double)n + cyc) * (double)(c->h_int[1] + 1);
        pcg_passes += c->h_int[1] + 1;
        *iters += c->h_int[1];
        if (final_rr) *final_rr = reinterpret_cast<double*>(c->h_int + 4)[0];
        int st = c->h_int[0];
        if (st == 5) return MTK_ERR_TIMEOUT;
        if (st == 4) return MTK_ERR_BREAKDOWN;
        if (st == 3) return MTK_ERR_NOT_CONVERGED;
        return MTK_OK;
    }
    template <typename T> DevLevel0<T> level0() const;
};

template <> DevLevel0<double> FieldSolver::level0<double>() const { return L064; }
template <> DevLevel0<float> FieldSolver::level0<float>() const { return L032; }
template <> DevHierarchy<double> FieldSolver::hier<double>() const { return H64; }
template <> DevHierarchy<float> FieldSolver::hier<float>() const { return H32; }

}  // namespace

namespace {
// Reverse pass of the power iteration (mtk_field_power_adjoint): dphi[nF] in, per face the
// derivatives with respect to theta (3 nF, [3 f + j] for the halfedge F(f,j) -> F(f,j+1)) and
// to the face area (nF) out.
struct FieldAdjoint {
    const double* dphi;
    double* g_theta;
    double* g_area;
};

// The field solves: with rhs == nullptr the inverse power iteration from x0 (n_iter steps,
// M-normalised), otherwise one solve L x = rhs from x = 0 (x0 and n_iter unused); with adj the
// iterates are kept and the reverse pass follows the forward one.

int field_run(mtk_ctx* c, int32_t nF, int32_t nRosy, const int32_t* nbr_h, const double* theta_h, const double* area_h,
              const double* x0, int32_t n_iter, const mtk_solve_opts* opts_in, double* out, mtk_stats* stats,
              const double* rhs, const FieldAdjoint* adj = nullptr) {
    if (rhs) n_iter = 1;
    if (!c || nF <= 0 || nRosy <= 0 || !nbr_h || !theta_h || !area_h || (!x0 && !rhs) || !out || n_iter < 0)
        return MTK_ERR_BAD_INPUT;
    for (int64_t i = 0; i < 3 * (int64_t)nF; i++)
        if (nbr_h[i] < -1 || nbr_h[i] >= nF || nbr_h[i] == i / 3) {
            mtk_set_last_error("face neighbour out of range (a face index other than its own, or -1 for a boundary side)",
                               __FILE__, __LINE__);
            return MTK_ERR_BAD_INPUT;
        }
    mtk_solve_opts opts;
    mtk_default_opts(&opts);
    if (opts_in) opts = *opts_in;
    MTK_CUDA_TRY(cudaSetDevice(c->device));
    AllocStreamScope alloc_scope(c->stream);
    FieldSolver S;
    S.c = c;
    S.n = nF;
    const int n = nF;
    cudaStream_t st = c->stream;
    MTK_CUDA_TRY(cudaEventRecord(c->ev_a, st));
    const char* dbg_env = getenv("MTK_DEBUG");
    const bool debug = dbg_env && dbg_env[0] == '1';
    {
        auto th0 = std::chrono::steady_clock::now();
        if (!getenv("MTK_NO_AMG")) MTK_TRY(S.build_amg(nbr_h, theta_h, nRosy));
        if (debug)
            fprintf(stderr, "[field host] multigrid set-up %.1f ms (levels %d, coarse %d)\n",
                    std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - th0).count(), S.amg_levels,
                    S.amg_coarse);
    }
    // with the multigrid the solver works on faces numbered by level-0 aggregate
    std::vector<int32_t> nbr_p;
    std::vector<double> theta_p, area_p, x0_p;
    const int32_t* nbr_u = nbr_h;
    const double *theta_u = theta_h, *area_u = area_h, *x0_u = x0;
    if (S.amg) {
        std::vector<int> inv(n);
        for (int k = 0; k < n; k++) inv[S.perm[k]] = k;
        nbr_p.resize(3 * (size_t)n);
        theta_p.resize(3 * (size_t)n);
        area_p.resize(n);
        x0_p.resize(2 * (size_t)n);
#pragma omp parallel for schedule(static)
        for (int k = 0; k < n; k++) {
            const int f = S.perm[k];
            for (int j = 0; j < 3; j++) {
                const int g = nbr_h[3 * (size_t)f + j];
                nbr_p[3 * (size_t)k + j] = g < 0 ? -1 : inv[g];
                theta_p[3 * (size_t)k + j] = theta_h[3 * (size_t)f + j];
            }
            area_p[k] = area_h[f];
            const double* src = rhs ? rhs : x0;   // the vector that enters in face order
            x0_p[2 * (size_t)k] = src[2 * (size_t)f];
            x0_p[2 * (size_t)k + 1] = src[2 * (size_t)f + 1];
        }
        nbr_u = nbr_p.data();
        theta_u = theta_p.data();
        area_u = area_p.data();
        x0_u = x0_p.data();
    } else if (rhs) {
        x0_u = rhs;
    }
    MTK_TRY(S.nbr_in.upload(nbr_u, 3 * (size_t)n, st));
    MTK_TRY(S.theta.upload(theta_u, 3 * (size_t)n, st));
    MTK_TRY(S.area.upload(area_u, n, st));
    const int ring = std::min(kRing, std::max(n_iter, 1));
    for (int j = 0; j < ring; j++) { MTK_TRY(S.ringU[j].alloc(n)); MTK_TRY(S.ringL[j].alloc(n)); }
    if (!rhs) MTK_CUDA_TRY(cudaMemcpyAsync(S.ringU[0].p, x0_u, sizeof(double2) * n, cudaMemcpyHostToDevice, st));
    MTK_TRY(S.nbr.alloc(3 * (size_t)n));
    MTK_TRY(S.v64.alloc(3 * (size_t)n));
    MTK_TRY(S.v32.alloc(3 * (size_t)n));
    MTK_TRY(S.d64.alloc(n)); MTK_TRY(S.inv64.alloc(n)); MTK_TRY(S.d32.alloc(n)); MTK_TRY(S.inv32.alloc(n));
    MTK_TRY(S.area32.alloc(n));
    MTK_TRY(S.b.alloc(n)); MTK_TRY(S.Lu.alloc(n)); MTK_TRY(S.x.alloc(n)); MTK_TRY(S.r.alloc(n));
    if (rhs) MTK_CUDA_TRY(cudaMemcpyAsync(S.b.p, x0_u, sizeof(double2) * n, cudaMemcpyHostToDevice, st));
    const bool mixed = opts.precision == MTK_PREC_MIXED;
    if (mixed) {
        MTK_TRY(S.r32.alloc(n)); MTK_TRY(S.e32.alloc(n)); MTK_TRY(S.z32.alloc(n)); MTK_TRY(S.p32.alloc(n)); MTK_TRY(S.q32.alloc(n));
        if (S.amg) { MTK_TRY(S.rb32.alloc(n)); MTK_TRY(S.pb32.alloc(n)); MTK_TRY(S.sv32.alloc(n)); MTK_TRY(S.vv32.alloc(n)); }
    } else {
        MTK_TRY(S.z64.alloc(n)); MTK_TRY(S.p64.alloc(n)); MTK_TRY(S.q64.alloc(n));
        if (S.amg) { MTK_TRY(S.rb64.alloc(n)); MTK_TRY(S.pb64.alloc(n)); MTK_TRY(S.sv64.alloc(n)); MTK_TRY(S.vv64.alloc(n)); }
    }
    const int G = stream_grid(c);
    field_assemble<<<G, kStream, 0, st>>>(n, nRosy, S.nbr_in.p, S.theta.p, S.area.p, S.nbr.p, S.v64.p, S.v32.p, S.d64.p,
                                         S.d32.p, S.inv64.p, S.inv32.p, S.area32.p);
    c->kernels++;
    MTK_CUDA_TRY(cudaGetLastError());

    long long iters = 0, solves = 0, refines = 0;
    double worst = 0.0;
    std::vector<double> Gr(kRing * kRing, 0.0), Gi(kRing * kRing, 0.0);
    const double tol = opts.tol;
    // Attainable reduction of the FP32 solves, per refinement (first, second, later): the FP64
    // residual after a correction exceeds the FP32 recursive one by the rounding of the FP32
    // operator times the correction, which the near-null modes amplify (in the late power steps
    // the first correction reaches only ~1/50 of its start residual however far FP32 iterates).
    // Measured as sqrt(max(0, rr_fp64 - rr_fp32)) / |r_start| and used to stop the next step's
    // solves at half of it instead of iterating below what FP64 will see.
    double floor_rel[3] = {0.0, 0.0, 0.0};
    DBuf<double2> Uall;   // the iterates u_0 .. u_n (reverse pass only)
    DBuf<double> sall;    // s_k^2 = x_k^H M x_k
    if (adj) {
        MTK_TRY(Uall.alloc((size_t)(n_iter + 1) * n));
        MTK_TRY(sall.alloc((size_t)n_iter + 1));
        MTK_CUDA_TRY(cudaMemcpyAsync(Uall.p, S.ringU[0].p, sizeof(double2) * n, cudaMemcpyDeviceToDevice, st));
    }
    // FP32 refinement cannot converge on a near-singular operator: on a flat or developable open
    // patch a parallel field has zero Dirichlet energy, so L's smallest eigenvalue is the 1e-9
    // shift (condition ~6e9, which FP32 drops from the operator entirely).  A solve whose FP32
    // refinement stops reducing the FP64 residual (or runs out of refinements) continues in
    // FP64 PCG from its current iterate, and the rest of the run stays in FP64.  There the solve
    // stops on the recursive residual; the true residual is bounded by about cond(L) * eps.
    bool fallback64 = false;
    auto alloc64 = [&]() -> int {
        if (S.z64.p) return MTK_OK;
        MTK_TRY(S.z64.alloc(n)); MTK_TRY(S.p64.alloc(n)); MTK_TRY(S.q64.alloc(n));
        if (S.amg) { MTK_TRY(S.rb64.alloc(n)); MTK_TRY(S.pb64.alloc(n)); MTK_TRY(S.sv64.alloc(n)); MTK_TRY(S.vv64.alloc(n)); }
        return MTK_OK;
    };
    // one solve L x = b from the current x / r (S.b, S.x, S.r, and S.r32 when MIXED) to the
    // relative residual tol: FP64 PCG, or FP32 PCG inside FP64 refinement; rr in: the start
    // residual |r|^2, out: the final one
    auto solve_to_goal = [&](double bnorm2, double& rr) -> int {
        const double goal2 = tol * tol * bnorm2;
        solves++;
        refines++;
        if (mixed && !fallback64) {
            int outer = 0;
            bool stalled = false;
            while (rr > goal2) {
                if (outer >= opts.max_refine) { stalled = true; break; }
                outer++;
                // inner FP32 solve L e = r to inner_tol relative (at least the outer goal)
                double itol = opts.inner_tol;
                double need = std::sqrt(goal2 / rr) * 0.5;
                if (need > itol) itol = need;
                const int ki = std::min(outer, 3) - 1;
                const double fl = std::min(0.5 * floor_rel[ki], 0.1);
                if (fl > itol) itol = fl;
                zero_f2<<<G, kStream, 0, st>>>(n, S.e32.p);
                c->kernels++;
                double frr = 0.0;
                const long long it0 = iters;
                int s = S.pcg<float, float2>(S.A32(), S.inv32.p, S.r32.p, S.e32.p, S.z32.p /*r*/, S.p32.p /*z*/,
                                             S.q32.p /*p*/, reinterpret_cast<float2*>(S.Lu.p) /*q*/, S.rb32.p, S.pb32.p,
                                             S.sv32.p, S.vv32.p, itol * itol * rr,
                                             opts.max_iter, &iters, &frr);
                if (debug)
                    fprintf(stderr, "[field pcg] status %d iterations %lld rr %.3e target %.3e (from %.3e)\n", s,
                            iters - it0, frr, itol * itol * rr, rr);
                // an FP32 breakdown (p^H A p <= 0 in single precision) means the inner solve has
                // stagnated: its last iterate is still a valid correction, and the FP64 refinement
                // decides what comes next
                if (s == MTK_ERR_TIMEOUT) return s;
                const double rr_prev = rr;
                add_correction<<<G, kStream, 0, st>>>(n, S.e32.p, S.x.p);
                residual64<<<G, kStream, 0, st>>>(S.A64(), S.b.p, S.x.p, S.r.p, S.r32.p, c->partials);
                c->kernels += 2;
                MTK_TRY(S.finalize(G, 1));
                MTK_TRY(S.read_scalars(1));
                rr = c->h_scalars[0];
                refines++;
                if (!(rr == rr)) return MTK_ERR_BREAKDOWN;
                if (rr > goal2 && rr >= rr_prev) { stalled = true; break; }
                if (s == MTK_OK && rr_prev > 0) floor_rel[ki] = std::sqrt(std::max(rr - frr, 0.0) / rr_prev);
            }
            if (!stalled) return MTK_OK;
            fallback64 = true;
            if (debug) fprintf(stderr, "[field] FP32 refinement stalled at %.3e: FP64 PCG from here on\n", std::sqrt(rr / bnorm2));
            MTK_TRY(alloc64());
        }
        {
            double frr = 0;
            int s = S.pcg<double, double2>(S.A64(), S.inv64.p, S.b.p, S.x.p, S.r.p, S.z64.p, S.p64.p, S.q64.p, S.rb64.p,
                                           S.pb64.p, S.sv64.p, S.vv64.p, goal2,
                                           opts.max_iter, &iters, &frr);
            if (s != MTK_OK) return s;
            // true FP64 residual of the result
            residual64<<<G, kStream, 0, st>>>(S.A64(), S.b.p, S.x.p, S.r.p, nullptr, c->partials);
            c->kernels++;
            MTK_TRY(S.finalize(G, 1));
            MTK_TRY(S.read_scalars(1));
            rr = c->h_scalars[0];
            refines++;
        }
        return MTK_OK;
    };
    for (int k = 0; k < n_iter; k++) {
        double bnorm2 = 0, rr = 0;
        if (rhs) {   // plain solve: x = 0, r = b
            start_from_rhs<<<G, kStream, 0, st>>>(n, S.b.p, S.x.p, S.r.p, mixed ? S.r32.p : nullptr, c->partials);
            c->kernels++;
            MTK_TRY(S.finalize(G, 1));
            MTK_TRY(S.read_scalars(1));
            bnorm2 = rr = c->h_scalars[0];
        } else {
            // b = M u_k, L u_k kept in the ring; Galerkin start on the last `ring` iterates
            const int slot = k % ring;
            const int cnt = std::min(k + 1, ring);
            double2* uk = S.ringU[slot].p;
            power_prepare<<<G, kStream, 0, st>>>(S.A64(), S.area.p, uk, S.b.p, S.ringL[slot].p, c->partials);
            c->kernels++;
            MTK_TRY(S.finalize(G, 3));
            MTK_CUDA_TRY(cudaMemcpyAsync(c->h_scalars, c->scalars, 3 * sizeof(double), cudaMemcpyDeviceToHost, st));
            RingPtrs R{};
            std::vector<int> slots(cnt);
            for (int j = 0; j < cnt; j++) {
                int sj = (slot - j + ring) % ring;
                slots[j] = sj;
                R.V[j] = S.ringU[sj].p;
                R.LV[j] = S.ringL[sj].p;
            }
            R.cnt = cnt;
            launch_gram(cnt, G, st, n, R, uk, S.b.p, c->partials);
            c->kernels++;
            MTK_TRY(S.finalize(G, 4 * cnt));
            MTK_CUDA_TRY(cudaMemcpyAsync(c->h_scalars + 8, c->scalars, 4 * cnt * sizeof(double), cudaMemcpyDeviceToHost, st));
            MTK_CUDA_TRY(cudaStreamSynchronize(st));
            // row / column of the new iterate; older entries stay valid (their vectors are unchanged)
            for (int j = 0; j < cnt; j++) {
                int sj = slots[j];
                double gr = c->h_scalars[8 + 4 * j], gi = c->h_scalars[8 + 4 * j + 1];
                Gr[slot * kRing + sj] = gr;
                Gi[slot * kRing + sj] = gi;
                Gr[sj * kRing + slot] = gr;
                Gi[sj * kRing + slot] = -gi;
                if (sj == slot) Gi[slot * kRing + slot] = 0.0;
            }
            std::vector<double> gr_sub(kRing * kRing), gi_sub(kRing * kRing), hr(cnt), hi(cnt), yr, yi;
            for (int a = 0; a < cnt; a++) {
                for (int b2 = 0; b2 < cnt; b2++) {
                    gr_sub[a * kRing + b2] = Gr[slots[a] * kRing + slots[b2]];
                    gi_sub[a * kRing + b2] = Gi[slots[a] * kRing + slots[b2]];
                }
                hr[a] = c->h_scalars[8 + 4 * a + 2];
                hi[a] = c->h_scalars[8 + 4 * a + 3];
            }
            hermitian_pinv_solve(gr_sub, gi_sub, hr, hi, cnt, yr, yi);
            StartCoef sc{};
            for (int j = 0; j < cnt; j++) { sc.re[j] = yr[j]; sc.im[j] = yi[j]; sc.V[j] = R.V[j]; sc.LV[j] = R.LV[j]; }
            sc.cnt = cnt;
            launch_combine(cnt, G, st, n, sc, S.b.p, S.x.p, S.r.p, mixed ? S.r32.p : nullptr, c->partials);
            c->kernels++;
            MTK_TRY(S.finalize(G, 1));
            MTK_CUDA_TRY(cudaMemcpyAsync(c->h_scalars + 3, c->scalars, sizeof(double), cudaMemcpyDeviceToHost, st));
            MTK_CUDA_TRY(cudaStreamSynchronize(st));
            bnorm2 = c->h_scalars[2];
            rr = c->h_scalars[3];
        }
        if (!(bnorm2 == bnorm2) || !(rr == rr)) {   // a NaN in the inputs reached the right-hand side
            mtk_set_last_error("field solve: NaN in the right-hand side or the start residual", __FILE__, __LINE__);
            return MTK_ERR_BREAKDOWN;
        }
        const double start_rel = bnorm2 > 0 ? std::sqrt(rr / bnorm2) : 0.0;
        if (const int s2 = solve_to_goal(bnorm2, rr); s2 != MTK_OK) {
            if (s2 == MTK_ERR_NOT_CONVERGED)
                mtk_set_last_error("field solve: PCG reached its iteration cap (max_iter)", __FILE__, __LINE__);
            else if (s2 == MTK_ERR_BREAKDOWN)
                mtk_set_last_error("field solve: PCG breakdown (p^H L p <= 0 or NaN)", __FILE__, __LINE__);
            return s2;
        }
        double rel = bnorm2 > 0 ? std::sqrt(rr / bnorm2) : 0.0;
        if (rel > worst) worst = rel;
        if (debug)
            fprintf(stderr, "[field] power step %d: pcg iterations %lld (total), refinements %lld, start residual %.2e, final %.2e\n",
                    k, iters, refines, start_rel, rel);
        if (rhs) break;
        // x /= sqrt|x^H M x|; u = x
        mnorm_partial<<<G, kStream, 0, st>>>(n, S.area.p, S.x.p, c->partials);
        c->kernels++;
        MTK_TRY(S.finalize(G, 1));
        normalize_to<<<G, kStream, 0, st>>>(n, c->scalars, S.x.p, S.ringU[(k + 1) % ring].p);
        c->kernels++;
        MTK_CUDA_TRY(cudaGetLastError());
        if (adj) {   // keep u_{k+1} and s_{k+1}^2 for the reverse pass
            MTK_CUDA_TRY(cudaMemcpyAsync(Uall.p + (size_t)(k + 1) * n, S.ringU[(k + 1) % ring].p, sizeof(double2) * n,
                                         cudaMemcpyDeviceToDevice, st));
            MTK_CUDA_TRY(cudaMemcpyAsync(sall.p + k + 1, c->scalars, sizeof(double), cudaMemcpyDeviceToDevice, st));
        }
    }
    if (adj) {
        // reverse pass over the stored iterates (faces in the solver's order)
        std::vector<double> dphi_p(n);
        for (int k = 0; k < n; k++) dphi_p[k] = adj->dphi[S.amg ? S.perm[k] : k];
        DBuf<double> d_dphi, g_area, g_theta;
        DBuf<double2> gu;
        MTK_TRY(d_dphi.upload(dphi_p.data(), n, st));
        MTK_TRY(g_area.alloc(n)); MTK_TRY(g_area.zero(st));
        MTK_TRY(g_theta.alloc(3 * (size_t)n)); MTK_TRY(g_theta.zero(st));
        MTK_TRY(gu.alloc(n));
        adj_seed<<<G, kStream, 0, st>>>(n, nRosy, d_dphi.p, Uall.p + (size_t)n_iter * n, gu.p);
        c->kernels++;
        for (int k = n_iter; k >= 1; k--) {
            const double2* uk = Uall.p + (size_t)k * n;
            const double2* up = Uall.p + (size_t)(k - 1) * n;
            adj_dot<<<G, kStream, 0, st>>>(n, gu.p, uk, c->partials);
            c->kernels++;
            MTK_TRY(S.finalize(G, 1));
            adj_rhs<<<G, kStream, 0, st>>>(n, gu.p, uk, S.area.p, c->scalars, sall.p + k, S.b.p, g_area.p);
            start_from_rhs<<<G, kStream, 0, st>>>(n, S.b.p, S.x.p, S.r.p, mixed ? S.r32.p : nullptr, c->partials);
            c->kernels += 2;
            MTK_TRY(S.finalize(G, 1));
            MTK_TRY(S.read_scalars(1));
            double rr = c->h_scalars[0];
            if (!(rr == rr)) {
                mtk_set_last_error("field adjoint: NaN in the reverse pass", __FILE__, __LINE__);
                return MTK_ERR_BREAKDOWN;
            }
            const double bnorm2 = rr;
            MTK_TRY(solve_to_goal(bnorm2, rr));
            const double rel = bnorm2 > 0 ? std::sqrt(rr / bnorm2) : 0.0;
            if (rel > worst) worst = rel;
            adj_accumulate<<<G, kStream, 0, st>>>(S.A64(), nRosy, S.x.p, uk, up, sall.p + k, S.area.p, g_area.p,
                                                  g_theta.p, gu.p);
            c->kernels++;
            MTK_CUDA_TRY(cudaGetLastError());
        }
        std::vector<double> ha(n), ht(3 * (size_t)n);
        MTK_CUDA_TRY(cudaMemcpyAsync(ha.data(), g_area.p, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
        MTK_CUDA_TRY(cudaMemcpyAsync(ht.data(), g_theta.p, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, st));
        MTK_CUDA_TRY(cudaStreamSynchronize(st));
        for (int k = 0; k < n; k++) {
            const int f = S.amg ? S.perm[k] : k;
            adj->g_area[f] = ha[k];
            for (int j = 0; j < 3; j++) adj->g_theta[3 * (size_t)f + j] = ht[(size_t)j * n + k];
        }
    }
    std::vector<double> out_p;
    double* out_u = out;
    if (S.amg) {
        out_p.resize(2 * (size_t)n);
        out_u = out_p.data();
    }
    MTK_CUDA_TRY(cudaMemcpyAsync(out_u, rhs ? S.x.p : S.ringU[n_iter % ring].p, sizeof(double2) * n,
                                 cudaMemcpyDeviceToHost, st));
    MTK_CUDA_TRY(cudaEventRecord(c->ev_b, st));
    MTK_CUDA_TRY(cudaStreamSynchronize(st));
    if (S.amg) {
#pragma omp parallel for schedule(static)
        for (int k = 0; k < n; k++) {
            out[2 * (size_t)S.perm[k]] = out_p[2 * (size_t)k];
            out[2 * (size_t)S.perm[k] + 1] = out_p[2 * (size_t)k + 1];
        }
    }
    float ms = 0;
    cudaEventElapsedTime(&ms, c->ev_a, c->ev_b);
    if (stats) {
        stats->pcg_iters += iters;
        stats->solves += solves;
        stats->refinements += refines;
        stats->spmv_calls += iters + refines + n_iter;
        if (worst > stats->max_rel_residual) stats->max_rel_residual = worst;
        stats->ms_field += ms;
        stats->field_pcg_launches += S.pcg_launches;
        stats->field_pcg_passes += S.pcg_passes;
        stats->field_pcg_ms += S.pcg_ms;
        stats->field_pcg_bytes += S.pcg_bytes;
        stats->kernel_launches = c->kernels;
    }
    return MTK_OK;
}
}  // namespace

extern "C" int mtk_field_smoothest(mtk_ctx* c, int32_t nF, int32_t nRosy, const int32_t* nbr_h,
                                   const double* theta_h, const double* area_h, const double* x0,
                                   int32_t n_iter, const mtk_solve_opts* opts_in, double* out, mtk_stats* stats) {
    if (!x0) return MTK_ERR_BAD_INPUT;
    return field_run(c, nF, nRosy, nbr_h, theta_h, area_h, x0, n_iter, opts_in, out, stats, nullptr);
}

extern "C" int mtk_field_power_adjoint(mtk_ctx* c, int32_t nF, int32_t nRosy, const int32_t* nbr_h, const double* theta_h,
                                       const double* area_h, const double* x0, int32_t n_iter, const mtk_solve_opts* opts_in,
                                       const double* dphi, double* out, double* g_theta, double* g_area, mtk_stats* stats) {
    if (!x0 || !dphi || !g_theta || !g_area || n_iter < 1) return MTK_ERR_BAD_INPUT;
    const FieldAdjoint adj{dphi, g_theta, g_area};
    return field_run(c, nF, nRosy, nbr_h, theta_h, area_h, x0, n_iter, opts_in, out, stats, nullptr, &adj);
}

extern "C" int mtk_field_solve(mtk_ctx* c, int32_t nF, int32_t nRosy, const int32_t* nbr_h, const double* theta_h,
                               const double* area_h, const double* rhs, const mtk_solve_opts* opts_in, double* out,
                               mtk_stats* stats) {
    if (!rhs) return MTK_ERR_BAD_INPUT;
    return field_run(c, nF, nRosy, nbr_h, theta_h, area_h, nullptr, 1, opts_in, out, stats, rhs);
}

// SpMV roofline measurement: assembles the field operator and times `reps` stand-alone SpMVs,
// each after an L2 flush (a 256 MiB write), each with its own CUDA-event pair on the stream.
extern "C" int mtk_field_spmv_bench(mtk_ctx* c, int32_t nF, int32_t nRosy, const int32_t* nbr_h, const double* theta_h,
                                    int32_t precision, int32_t reps, double* ms_per_spmv, double* bytes_per_spmv,
                                    double* ms_copy_same_bytes) {
    if (!c || nF <= 0 || !nbr_h || !theta_h || reps <= 0 || !ms_per_spmv || !bytes_per_spmv) return MTK_ERR_BAD_INPUT;
    for (int64_t i = 0; i < 3 * (int64_t)nF; i++)
        if (nbr_h[i] < -1 || nbr_h[i] >= nF || nbr_h[i] == i / 3) return MTK_ERR_BAD_INPUT;
    MTK_CUDA_TRY(cudaSetDevice(c->device));
    AllocStreamScope alloc_scope(c->stream);
    cudaStream_t st = c->stream;
    const int n = nF;
    DBuf<int> nbr_in, nbr;
    DBuf<double> theta, area, d64, inv64;
    DBuf<float> d32, inv32, area32;
    DBuf<double2> v64, x64, y64;
    DBuf<float2> v32, x32, y32;
    DBuf<unsigned char> flush;
    MTK_TRY(nbr_in.upload(nbr_h, 3 * (size_t)n, st));
    MTK_TRY(theta.upload(theta_h, 3 * (size_t)n, st));
    std::vector<double> ones(n, 1.0);
    MTK_TRY(area.upload(ones.data(), n, st));
    MTK_TRY(nbr.alloc(3 * (size_t)n)); MTK_TRY(v64.alloc(3 * (size_t)n)); MTK_TRY(v32.alloc(3 * (size_t)n));
    MTK_TRY(d64.alloc(n)); MTK_TRY(inv64.alloc(n)); MTK_TRY(d32.alloc(n)); MTK_TRY(inv32.alloc(n)); MTK_TRY(area32.alloc(n));
    const int G = stream_grid(c);
    field_assemble<<<G, kStream, 0, st>>>(n, nRosy, nbr_in.p, theta.p, area.p, nbr.p, v64.p, v32.p, d64.p, d32.p,
                                         inv64.p, inv32.p, area32.p);
    const size_t kFlush = 256u << 20;
    MTK_TRY(flush.alloc(kFlush));
    const bool fp64 = precision == MTK_PREC_FP64;
    std::vector<double> xh(2 * (size_t)n);
    for (int i = 0; i < n; i++) { xh[2 * i] = 1.0 / (1 + i % 7); xh[2 * i + 1] = 0.5 / (1 + i % 5); }
    if (fp64) {
        MTK_TRY(x64.upload(reinterpret_cast<const double2*>(xh.data()), n, st));
        MTK_TRY(y64.alloc(n));
    } else {
        std::vector<float2> xf(n);
        for (int i = 0; i < n; i++) xf[i] = make_float2((float)xh[2 * i], (float)xh[2 * i + 1]);
        MTK_TRY(x32.upload(xf.data(), n, st));
        MTK_TRY(y32.alloc(n));
    }
    const int blocks = (n + 255) / 256;
    double total = 0;
    for (int rep = -1; rep < reps; rep++) {   // rep -1: warm-up
        MTK_CUDA_TRY(cudaMemsetAsync(flush.p, rep & 0xff, kFlush, st));
        MTK_CUDA_TRY(cudaEventRecord(c->ev_k0, st));
        if (fp64) spmv_ell<double><<<blocks, 256, 0, st>>>(ComplexEll<double>{n, nbr.p, v64.p, d64.p}, x64.p, y64.p);
        else spmv_ell<float><<<blocks, 256, 0, st>>>(ComplexEll<float>{n, nbr.p, v32.p, d32.p}, x32.p, y32.p);
        MTK_CUDA_TRY(cudaEventRecord(c->ev_k1, st));
        MTK_CUDA_TRY(cudaEventSynchronize(c->ev_k1));
        float ms = 0;
        cudaEventElapsedTime(&ms, c->ev_k0, c->ev_k1);
        if (rep >= 0) total += ms;
        c->kernels++;
    }
    MTK_CUDA_TRY(cudaGetLastError());
    *ms_per_spmv = total / reps;
    // algorithmic bytes per row: 3 x (value + column) + diagonal + own x + y (gathered x not counted)
    *bytes_per_spmv = (double)n * (fp64 ? 3.0 * (16 + 4) + 8 + 16 + 16 : 3.0 * (8 + 4) + 4 + 8 + 8);
    if (ms_copy_same_bytes) {   // a device copy moving the same bytes (read + write), same flush and timing
        const size_t half = ((size_t)(*bytes_per_spmv / 2) + 255) & ~(size_t)255;
        DBuf<unsigned char> src, dst;
        MTK_TRY(src.alloc(half));
        MTK_TRY(dst.alloc(half));
        MTK_CUDA_TRY(cudaMemsetAsync(src.p, 1, half, st));
        double tc = 0;
        for (int rep = -1; rep < reps; rep++) {
            MTK_CUDA_TRY(cudaMemsetAsync(flush.p, rep & 0xff, kFlush, st));
            MTK_CUDA_TRY(cudaEventRecord(c->ev_k0, st));
            MTK_CUDA_TRY(cudaMemcpyAsync(dst.p, src.p, half, cudaMemcpyDeviceToDevice, st));
            MTK_CUDA_TRY(cudaEventRecord(c->ev_k1, st));
            MTK_CUDA_TRY(cudaEventSynchronize(c->ev_k1));
            float ms = 0;
            cudaEventElapsedTime(&ms, c->ev_k0, c->ev_k1);
            if (rep >= 0) tc += ms;
        }
        *ms_copy_same_bytes = tc / reps;
    }
    return MTK_OK;
}
