// Assembled sparse systems on the device: the general linear-solver seam under the field and
// integration solvers (mtk_csr_create / mtk_csr_pcg / mtk_csr_smallest_eig).
//
// The reference solves assembled matrices directly: solveSquare / solveSmallestEig on an SprsC
// (sparse_linear_solver.h:16-54) and the LMSolver's linear-solver template parameter
// (CholeskyWrapper, iter_rounding.h:14-31) on JᵀJ.  A caller that already holds such a matrix
// (symmetric or Hermitian positive definite) hands it over once as CSR; it stays on the device
// in FP64 and FP32, and every solve runs the persistent Jacobi-preconditioned CG kernel below on
// up to kMaxRhs right-hand sides at once (the matrix is read once per iteration for all of them:
// u and v, or the real and imaginary parts, in one launch), in FP64 or as FP32 CG inside FP64
// iterative refinement.  Rows are one thread each, entries walked in order four loads in flight;
// all reductions are fixed-order, so a solve is bit-reproducible.
#include <algorithm>
#include <cmath>
#include <vector>

#include "mtk_ctx.cuh"

struct mtk_csr {
    int n = 0;
    long long nnz = 0;
    int cplx = 0;                       // 1: Hermitian complex values (re, im)
    mtk::DBuf<int> ptr, col;
    mtk::DBuf<double> v64, d64inv;      // values (2 per entry when complex), Jacobi inverse
    mtk::DBuf<float> v32, d32inv;
};

namespace {

using namespace mtk;

constexpr int kMaxRhs = 4;

// value arithmetic: real (T) or complex (two T per entry / vector element)
template <typename T, bool C>
struct Ar;
template <typename T>
struct Ar<T, false> {
    static constexpr int W = 1;
    // acc += a * x
    __device__ static void mac(const T* a, const T* x, T* acc) { acc[0] += a[0] * x[0]; }
    // Re(conj(u) v)
    __device__ static T dot(const T* u, const T* v) { return u[0] * v[0]; }
};
template <typename T>
struct Ar<T, true> {
    static constexpr int W = 2;
    __device__ static void mac(const T* a, const T* x, T* acc) {
        acc[0] += a[0] * x[0] - a[1] * x[1];
        acc[1] += a[0] * x[1] + a[1] * x[0];
    }
    __device__ static T dot(const T* u, const T* v) { return u[0] * v[0] + u[1] * v[1]; }
};

template <typename T>
struct DevMat {
    int n;
    const int* ptr;
    const int* col;
    const T* val;
    const T* dinv;   // real Jacobi inverse (the diagonal of a Hermitian matrix is real)
};

// y_c(row) = (A x_c)(row) for the R columns (vector element c * n * W + row * W + w)
template <typename T, bool C, int R>
__device__ __forceinline__ void row_apply(const DevMat<T>& A, int row, const T* x, T (&y)[R][2]) {
    using A_ = Ar<T, C>;
    constexpr int W = A_::W;
#pragma unroll
    for (int c = 0; c < R; c++) y[c][0] = y[c][1] = T(0);
    const int e = __ldg(A.ptr + row + 1);
    for (int p = __ldg(A.ptr + row); p < e; p += 4) {
        int cc[4];
        T a[4][2];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            cc[u] = p + u < e ? __ldg(A.col + p + u) : -1;
#pragma unroll
            for (int w = 0; w < W; w++) a[u][w] = p + u < e ? __ldg(A.val + (size_t)(p + u) * W + w) : T(0);
        }
#pragma unroll
        for (int u = 0; u < 4; u++) {
            if (cc[u] < 0) continue;
#pragma unroll
            for (int c = 0; c < R; c++) {
                T xv[2];
#pragma unroll
                for (int w = 0; w < W; w++) xv[w] = __ldcg(x + ((size_t)c * A.n + cc[u]) * W + w);
                A_::mac(a[u], xv, y[c]);
            }
        }
    }
}

// Persistent Jacobi PCG on R columns at once: each column runs its own CG (own alpha, beta),
// converged columns are frozen.  out: [0] status, [1] iterations (of the slowest column),
// (double*)(out + 4) the largest final |r|^2 / |b|^2 ratio's |r|^2.  tol2[c] = target |r_c|^2.
template <typename T, bool C, int R>
__global__ void __launch_bounds__(kBlock, 1) csr_pcg(DevMat<T> A, const T* __restrict__ b, T* x, T* r, T* z, T* p,
                                                     T* q, T* partials, GridBarrier bar, const double* __restrict__ tol2,
                                                     int maxit, int* out) {
    using A_ = Ar<T, C>;
    constexpr int W = A_::W;
    const int n = A.n;
    const size_t cs = (size_t)n * W;   // column stride
    const int stride = gridDim.x * blockDim.x;
    const int t0 = blockIdx.x * blockDim.x + threadIdx.x;
    T red[2 * R];
    T rz[R], rr[R];
    bool done[R];
    int status = 3, it = 0;
    // r = b - A x, z = D^-1 r, p = z
#pragma unroll
    for (int k = 0; k < 2 * R; k++) red[k] = T(0);
    for (int i = t0; i < n; i += stride) {
        T ax[R][2];
        row_apply<T, C, R>(A, i, x, ax);
        const T m = A.dinv[i];
#pragma unroll
        for (int c = 0; c < R; c++) {
            T rv[2], zv[2];
#pragma unroll
            for (int w = 0; w < W; w++) {
                const size_t o = c * cs + (size_t)i * W + w;
                rv[w] = b[o] - ax[c][w];
                zv[w] = m * rv[w];
                r[o] = rv[w];
                z[o] = zv[w];
                p[o] = zv[w];
            }
            red[2 * c] += A_::dot(rv, zv);
            red[2 * c + 1] += A_::dot(rv, rv);
        }
    }
    publish_partials<T, 2 * R>(red, partials);
    if (!grid_sync(bar)) { status = 5; goto finish; }
    gather_partials<T, 2 * R>(partials, red);
#pragma unroll
    for (int c = 0; c < R; c++) {
        rz[c] = red[2 * c];
        rr[c] = red[2 * c + 1];
        done[c] = (double)rr[c] <= tol2[c];
    }
    for (;;) {
        bool all = true;
#pragma unroll
        for (int c = 0; c < R; c++) all = all && done[c];
        if (all) { status = 0; break; }
        if (it >= maxit) { status = 3; break; }
        // q = A p, <p, q>
        T pq[R];
#pragma unroll
        for (int c = 0; c < R; c++) pq[c] = T(0);
        for (int i = t0; i < n; i += stride) {
            T ap[R][2];
            row_apply<T, C, R>(A, i, p, ap);
#pragma unroll
            for (int c = 0; c < R; c++) {
                T pv[2];
#pragma unroll
                for (int w = 0; w < W; w++) {
                    const size_t o = c * cs + (size_t)i * W + w;
                    q[o] = ap[c][w];
                    pv[w] = __ldcg(p + o);
                }
                pq[c] += A_::dot(pv, ap[c]);
            }
        }
        publish_partials<T, R>(pq, partials + 2 * R * gridDim.x);
        if (!grid_sync(bar)) { status = 5; break; }
        gather_partials<T, R>(partials + 2 * R * gridDim.x, pq);
        T alpha[R];
        bool bad = false;
#pragma unroll
        for (int c = 0; c < R; c++) {
            if (!done[c] && !(pq[c] > T(0))) bad = true;
            alpha[c] = done[c] ? T(0) : rz[c] / pq[c];
        }
        if (bad) { status = 4; break; }
        // x += alpha p, r -= alpha q, z = D^-1 r
#pragma unroll
        for (int k = 0; k < 2 * R; k++) red[k] = T(0);
        for (int i = t0; i < n; i += stride) {
            const T m = A.dinv[i];
#pragma unroll
            for (int c = 0; c < R; c++) {
                T rv[2], zv[2];
#pragma unroll
                for (int w = 0; w < W; w++) {
                    const size_t o = c * cs + (size_t)i * W + w;
                    x[o] += alpha[c] * __ldcg(p + o);
                    rv[w] = __ldcg(r + o) - alpha[c] * __ldcg(q + o);
                    zv[w] = m * rv[w];
                    r[o] = rv[w];
                    z[o] = zv[w];
                }
                red[2 * c] += A_::dot(rv, zv);
                red[2 * c + 1] += A_::dot(rv, rv);
            }
        }
        publish_partials<T, 2 * R>(red, partials + 3 * R * gridDim.x);
        if (!grid_sync(bar)) { status = 5; break; }
        gather_partials<T, 2 * R>(partials + 3 * R * gridDim.x, red);
        T beta[R];
#pragma unroll
        for (int c = 0; c < R; c++) {
            const T rzn = red[2 * c];
            if (!done[c]) {
                rr[c] = red[2 * c + 1];
                if (rr[c] != rr[c]) bad = true;
                beta[c] = rzn / rz[c];
                rz[c] = rzn;
                done[c] = (double)rr[c] <= tol2[c];
            } else {
                beta[c] = T(0);
            }
        }
        if (bad) { status = 4; break; }
        // p = z + beta p
        for (int i = t0; i < n; i += stride)
#pragma unroll
            for (int c = 0; c < R; c++)
#pragma unroll
                for (int w = 0; w < W; w++) {
                    const size_t o = c * cs + (size_t)i * W + w;
                    p[o] = __ldcg(z + o) + beta[c] * __ldcg(p + o);
                }
        it++;
        if (!grid_sync(bar)) { status = 5; break; }
    }
finish:
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        out[0] = status;
        out[1] = it;
    }
}

// FP64 residual r = b - A x (and its FP32 copy) with per-column |r|^2 partials
template <bool C, int R>
__global__ void csr_residual64(DevMat<double> A, const double* __restrict__ b, const double* __restrict__ x, double* r,
                               float* r32, double* partials) {
    using A_ = Ar<double, C>;
    constexpr int W = A_::W;
    const size_t cs = (size_t)A.n * W;
    double red[R];
#pragma unroll
    for (int c = 0; c < R; c++) red[c] = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < A.n; i += gridDim.x * blockDim.x) {
        double ax[R][2];
        row_apply<double, C, R>(A, i, x, ax);
#pragma unroll
        for (int c = 0; c < R; c++) {
            double rv[2];
#pragma unroll
            for (int w = 0; w < W; w++) {
                const size_t o = c * cs + (size_t)i * W + w;
                rv[w] = b[o] - ax[c][w];
                r[o] = rv[w];
                if (r32) r32[o] = (float)rv[w];
            }
            red[c] += A_::dot(rv, rv);
        }
    }
    block_sum<double, R>(red);
    if (threadIdx.x == 0)
#pragma unroll
        for (int c = 0; c < R; c++) partials[c * gridDim.x + blockIdx.x] = red[c];
}

__global__ void csr_sum_partials(const double* partials, int nb, int K, double* out) {
    for (int k = threadIdx.x; k < K; k += blockDim.x) {
        double s = 0.0;
        for (int b = 0; b < nb; b++) s += partials[k * nb + b];
        out[k] = s;
    }
}

__global__ void add_f32_to_f64(size_t m, const float* __restrict__ e, double* x) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < m; i += (size_t)gridDim.x * blockDim.x) x[i] += e[i];
}

__global__ void jacobi_inverse(int n, int cplx, const int* __restrict__ ptr, const int* __restrict__ col,
                               const double* __restrict__ val, double* d64, float* d32, int* bad) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double d = 0.0;
        for (int p = ptr[i]; p < ptr[i + 1]; p++)
            if (col[p] == i) d += val[(size_t)p * (cplx ? 2 : 1)];
        if (!(d > 0.0)) atomicExch(bad, 1);
        d64[i] = d > 0.0 ? 1.0 / d : 0.0;
        d32[i] = (float)(d > 0.0 ? 1.0 / d : 0.0);
    }
}

__global__ void to_f32(size_t m, const double* __restrict__ a, float* b) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < m; i += (size_t)gridDim.x * blockDim.x) b[i] = (float)a[i];
}

template <typename T>
DevMat<T> dev_mat(const mtk_csr* A);
template <>
DevMat<double> dev_mat<double>(const mtk_csr* A) { return {A->n, A->ptr.p, A->col.p, A->v64.p, A->d64inv.p}; }
template <>
DevMat<float> dev_mat<float>(const mtk_csr* A) { return {A->n, A->ptr.p, A->col.p, A->v32.p, A->d32inv.p}; }

// one persistent PCG launch on R columns; *iters += iterations
template <typename T, bool C, int R>
int launch_pcg(mtk_ctx* c, const mtk_csr* A, const T* b, T* x, T* r, T* z, T* p, T* q, const double* tol2_dev, int maxit,
               long long* iters) {
    int g = 0;
    MTK_TRY(launch_persistent(c, csr_pcg<T, C, R>, &g, dev_mat<T>(A), b, x, r, z, p, q, reinterpret_cast<T*>(c->partials),
                              barrier_of(c), tol2_dev, maxit, c->dev_int));
    MTK_CUDA_TRY(cudaMemcpyAsync(c->h_int, c->dev_int, 2 * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    MTK_CUDA_TRY(cudaStreamSynchronize(c->stream));
    *iters += c->h_int[1];
    const int st = c->h_int[0];
    if (st == 5) return MTK_ERR_TIMEOUT;
    if (st == 4) return MTK_ERR_BREAKDOWN;
    if (st == 3) return MTK_ERR_NOT_CONVERGED;
    return MTK_OK;
}

// FP64 residual of R columns: |r_c|^2 into h[c]
template <bool C, int R>
int residual(mtk_ctx* c, const mtk_csr* A, const double* b, const double* x, double* r, float* r32, std::vector<double>& h) {
    const int G = stream_grid(c);
    csr_residual64<C, R><<<G, kStream, 0, c->stream>>>(dev_mat<double>(A), b, x, r, r32, c->partials);
    csr_sum_partials<<<1, 32, 0, c->stream>>>(c->partials, G, R, c->scalars);
    c->kernels += 2;
    MTK_CUDA_TRY(cudaGetLastError());
    h.assign(R, 0.0);
    MTK_CUDA_TRY(cudaMemcpyAsync(h.data(), c->scalars, sizeof(double) * R, cudaMemcpyDeviceToHost, c->stream));
    MTK_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return MTK_OK;
}

// Solve A X = B for R (<= kMaxRhs) device columns: FP64 PCG, or FP32 PCG inside FP64 refinement.
// On return *worst = the largest relative residual.
template <bool C, int R>
int solve_cols(mtk_ctx* c, const mtk_csr* A, const double* b, double* x, const mtk_solve_opts& o, mtk_stats* st,
               double* worst) {
    const size_t m = (size_t)R * A->n * (C ? 2 : 1);
    cudaStream_t s = c->stream;
    DBuf<double> r, tol2;
    MTK_TRY(r.alloc(m));
    MTK_TRY(tol2.alloc(R));
    std::vector<double> rr, bb;
    const bool mixed = o.precision == MTK_PREC_MIXED;
    DBuf<float> r32;
    if (mixed) MTK_TRY(r32.alloc(m));
    // |b_c|^2 from the residual of x = 0 would need a second vector: use r = b - A x and b's norm
    {
        DBuf<double> zero;
        MTK_TRY(zero.alloc(m));
        MTK_TRY(zero.zero(s));
        MTK_TRY((residual<C, R>(c, A, b, zero.p, r.p, nullptr, bb)));
    }
    MTK_TRY((residual<C, R>(c, A, b, x, r.p, mixed ? r32.p : nullptr, rr)));
    std::vector<double> goal(R);
    for (int k = 0; k < R; k++) goal[k] = o.tol * o.tol * bb[k];
    long long iters = 0;
    int refines = 1;
    auto rel_worst = [&]() {
        double w = 0;
        for (int k = 0; k < R; k++) w = std::max(w, bb[k] > 0 ? std::sqrt(rr[k] / bb[k]) : 0.0);
        return w;
    };
    if (!mixed) {
        DBuf<double> z, p, q;
        MTK_TRY(z.alloc(m)); MTK_TRY(p.alloc(m)); MTK_TRY(q.alloc(m));
        MTK_CUDA_TRY(cudaMemcpyAsync(tol2.p, goal.data(), sizeof(double) * R, cudaMemcpyHostToDevice, s));
        DBuf<double> rw;
        MTK_TRY(rw.alloc(m));
        MTK_TRY((launch_pcg<double, C, R>(c, A, b, x, rw.p, z.p, p.p, q.p, tol2.p, o.max_iter, &iters)));
        MTK_TRY((residual<C, R>(c, A, b, x, r.p, nullptr, rr)));
        refines++;
    } else {
        DBuf<float> e, z, p, q, rw;
        MTK_TRY(e.alloc(m)); MTK_TRY(z.alloc(m)); MTK_TRY(p.alloc(m)); MTK_TRY(q.alloc(m)); MTK_TRY(rw.alloc(m));
        for (int outer = 0;; outer++) {
            bool ok = true;
            for (int k = 0; k < R; k++) ok = ok && rr[k] <= goal[k];
            if (ok) break;
            if (outer >= o.max_refine) return MTK_ERR_NOT_CONVERGED;
            // inner FP32 target: inner_tol of each column's current residual (at least its goal)
            std::vector<double> t2(R);
            for (int k = 0; k < R; k++) {
                double itol = std::max(o.inner_tol, 0.5 * std::sqrt(goal[k] / std::max(rr[k], 1e-300)));
                t2[k] = rr[k] <= goal[k] ? 1e300 : itol * itol * rr[k];
            }
            MTK_CUDA_TRY(cudaMemcpyAsync(tol2.p, t2.data(), sizeof(double) * R, cudaMemcpyHostToDevice, s));
            MTK_TRY(e.zero(s));
            const int ps = launch_pcg<float, C, R>(c, A, r32.p, e.p, rw.p, z.p, p.p, q.p, tol2.p, o.max_iter, &iters);
            if (ps == MTK_ERR_TIMEOUT) return ps;
            add_f32_to_f64<<<stream_grid(c), kStream, 0, s>>>(m, e.p, x);
            c->kernels++;
            const std::vector<double> prev = rr;
            MTK_TRY((residual<C, R>(c, A, b, x, r.p, r32.p, rr)));
            refines++;
            bool progress = false;
            for (int k = 0; k < R; k++) {
                if (!(rr[k] == rr[k])) return MTK_ERR_BREAKDOWN;
                if (rr[k] < prev[k] || rr[k] <= goal[k]) progress = true;
            }
            if (!progress) return MTK_ERR_NOT_CONVERGED;
        }
    }
    *worst = rel_worst();
    if (st) {
        st->pcg_iters += iters;
        st->solves += R;
        st->refinements += refines;
        st->spmv_calls += iters + refines;
        if (*worst > st->max_rel_residual) st->max_rel_residual = *worst;
        st->kernel_launches = c->kernels;
    }
    for (int k = 0; k < R; k++)
        if (rr[k] > goal[k] * 1.0000001) return MTK_ERR_NOT_CONVERGED;
    return MTK_OK;
}

template <bool C>
int solve_any(mtk_ctx* c, const mtk_csr* A, int R, const double* b, double* x, const mtk_solve_opts& o, mtk_stats* st,
              double* worst) {
    switch (R) {
        case 1: return solve_cols<C, 1>(c, A, b, x, o, st, worst);
        case 2: return solve_cols<C, 2>(c, A, b, x, o, st, worst);
        case 3: return solve_cols<C, 3>(c, A, b, x, o, st, worst);
        default: return solve_cols<C, 4>(c, A, b, x, o, st, worst);
    }
}

// M-norm of x (complex, M real-valued or Hermitian CSR): <x, M x>
__global__ void mnorm_csr(DevMat<double> M, const double* __restrict__ x, double* partials) {
    double red[1] = {0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < M.n; i += gridDim.x * blockDim.x) {
        double y[1][2];
        row_apply<double, true, 1>(M, i, x, y);
        red[0] += x[2 * i] * y[0][0] + x[2 * i + 1] * y[0][1];
    }
    block_sum<double, 1>(red);
    if (threadIdx.x == 0) partials[blockIdx.x] = red[0];
}

__global__ void mul_csr(DevMat<double> M, const double* __restrict__ x, double* y) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < M.n; i += gridDim.x * blockDim.x) {
        double v[1][2];
        row_apply<double, true, 1>(M, i, x, v);
        y[2 * i] = v[0][0];
        y[2 * i + 1] = v[0][1];
    }
}

__global__ void scale_by_inv_sqrt(size_t m, const double* __restrict__ s2, double* x) {
    const double s = sqrt(fabs(s2[0]));
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < m; i += (size_t)gridDim.x * blockDim.x) x[i] /= s;
}

}  // namespace

extern "C" int mtk_csr_create(mtk_ctx* c, int32_t n, const int32_t* ptr, const int32_t* col, const double* val,
                              int32_t complex_values, mtk_csr** out) {
    if (!c || !out || n <= 0 || !ptr || !col || !val) return MTK_ERR_BAD_INPUT;
    *out = nullptr;
    if (ptr[0] != 0) return MTK_ERR_BAD_INPUT;
    for (int i = 0; i < n; i++)
        if (ptr[i + 1] < ptr[i]) return MTK_ERR_BAD_INPUT;
    const long long nnz = ptr[n];
    for (long long p = 0; p < nnz; p++)
        if (col[p] < 0 || col[p] >= n) {
            mtk_set_last_error("mtk_csr_create: column index out of range", __FILE__, __LINE__);
            return MTK_ERR_BAD_INPUT;
        }
    MTK_CUDA_TRY(cudaSetDevice(c->device));
    cudaStream_t s = c->stream;
    auto* A = new mtk_csr();
    A->n = n;
    A->nnz = nnz;
    A->cplx = complex_values ? 1 : 0;
    const size_t nv = (size_t)std::max<long long>(nnz, 1) * (A->cplx ? 2 : 1);
    int st = A->ptr.upload(ptr, n + 1, s);
    if (st == MTK_OK) st = A->col.upload(col, std::max<long long>(nnz, 1), s);
    if (st == MTK_OK) st = A->v64.upload(val, nv, s);
    if (st == MTK_OK) st = A->v32.alloc(nv);
    if (st == MTK_OK) st = A->d64inv.alloc(n);
    if (st == MTK_OK) st = A->d32inv.alloc(n);
    DBuf<int> bad;
    if (st == MTK_OK) st = bad.alloc(1);
    if (st == MTK_OK) st = bad.zero(s);
    if (st != MTK_OK) { delete A; return st; }
    const int G = stream_grid(c);
    to_f32<<<G, kStream, 0, s>>>(nv, A->v64.p, A->v32.p);
    jacobi_inverse<<<G, kStream, 0, s>>>(n, A->cplx, A->ptr.p, A->col.p, A->v64.p, A->d64inv.p, A->d32inv.p, bad.p);
    c->kernels += 2;
    int hbad = 0;
    cudaError_t e = cudaMemcpyAsync(&hbad, bad.p, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) { mtk_set_last_error(cudaGetErrorString(e), __FILE__, __LINE__); delete A; return MTK_ERR_CUDA; }
    if (hbad) {
        mtk_set_last_error("mtk_csr_create: a diagonal entry is not positive (the solvers need an SPD / HPD matrix)",
                           __FILE__, __LINE__);
        delete A;
        return MTK_ERR_BAD_INPUT;
    }
    *out = A;
    return MTK_OK;
}

extern "C" int mtk_csr_destroy(mtk_csr* A) {
    delete A;
    return MTK_OK;
}

extern "C" int mtk_csr_pcg(mtk_ctx* c, const mtk_csr* A, int32_t nrhs, const double* b, double* x,
                           const mtk_solve_opts* opts_in, mtk_stats* stats) {
    if (!c || !A || nrhs <= 0 || !b || !x) return MTK_ERR_BAD_INPUT;
    mtk_solve_opts o;
    mtk_default_opts(&o);
    if (opts_in) o = *opts_in;
    MTK_CUDA_TRY(cudaSetDevice(c->device));
    AllocStreamScope alloc_scope(c->stream);
    cudaStream_t s = c->stream;
    const size_t col = (size_t)A->n * (A->cplx ? 2 : 1);
    int status = MTK_OK;
    for (int c0 = 0; c0 < nrhs; c0 += kMaxRhs) {
        const int R = std::min(kMaxRhs, nrhs - c0);
        DBuf<double> db, dx;
        MTK_TRY(db.upload(b + c0 * col, R * col, s));
        MTK_TRY(dx.upload(x + c0 * col, R * col, s));
        double worst = 0;
        const int st = A->cplx ? solve_any<true>(c, A, R, db.p, dx.p, o, stats, &worst)
                               : solve_any<false>(c, A, R, db.p, dx.p, o, stats, &worst);
        MTK_CUDA_TRY(cudaMemcpyAsync(x + c0 * col, dx.p, sizeof(double) * R * col, cudaMemcpyDeviceToHost, s));
        MTK_CUDA_TRY(cudaStreamSynchronize(s));
        if (st != MTK_OK && status == MTK_OK) status = st;
    }
    return status;
}

extern "C" int mtk_csr_smallest_eig(mtk_ctx* c, const mtk_csr* L, const mtk_csr* M, const double* x0, int32_t n_iter,
                                    const mtk_solve_opts* opts_in, double* out, mtk_stats* stats) {
    if (!c || !L || !M || !x0 || !out || n_iter < 0 || !L->cplx || !M->cplx || L->n != M->n) return MTK_ERR_BAD_INPUT;
    mtk_solve_opts o;
    mtk_default_opts(&o);
    if (opts_in) o = *opts_in;
    MTK_CUDA_TRY(cudaSetDevice(c->device));
    AllocStreamScope alloc_scope(c->stream);
    cudaStream_t s = c->stream;
    const int n = L->n;
    const int G = stream_grid(c);
    DBuf<double> u, b, x;
    MTK_TRY(u.upload(x0, 2 * (size_t)n, s));
    MTK_TRY(b.alloc(2 * (size_t)n));
    MTK_TRY(x.alloc(2 * (size_t)n));
    for (int k = 0; k < n_iter; k++) {
        // x = L^-1 M u (from x = u as the start), x /= sqrt|x^H M x|, u = x
        mul_csr<<<G, kStream, 0, s>>>(dev_mat<double>(M), u.p, b.p);
        MTK_CUDA_TRY(cudaMemcpyAsync(x.p, u.p, sizeof(double) * 2 * n, cudaMemcpyDeviceToDevice, s));
        c->kernels++;
        double worst = 0;
        MTK_TRY((solve_cols<true, 1>(c, L, b.p, x.p, o, stats, &worst)));
        mnorm_csr<<<G, kStream, 0, s>>>(dev_mat<double>(M), x.p, c->partials);
        csr_sum_partials<<<1, 32, 0, s>>>(c->partials, G, 1, c->scalars);
        scale_by_inv_sqrt<<<G, kStream, 0, s>>>(2 * (size_t)n, c->scalars, x.p);
        c->kernels += 3;
        MTK_CUDA_TRY(cudaMemcpyAsync(u.p, x.p, sizeof(double) * 2 * n, cudaMemcpyDeviceToDevice, s));
    }
    MTK_CUDA_TRY(cudaMemcpyAsync(out, u.p, sizeof(double) * 2 * n, cudaMemcpyDeviceToHost, s));
    MTK_CUDA_TRY(cudaStreamSynchronize(s));
    return MTK_OK;
}
