// Smoothest N-RoSy field on the device: connection-Laplacian assembly, complex Hermitian
// SpMV, persistent PCG (FP32 or FP64) and the inverse power iteration with FP64 residuals,
// Rayleigh quotient and normalisation.
//
// Replaces (metriko) face_rosy_field.h:43-49 + :72-110 and sparse_linear_solver.h:452-477.
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
#include <cmath>
#include <vector>

#include "mtk_ctx.cuh"

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
// count + 1e-9 (face_rosy_field.h:88-101).  No atomics: every row is written by its owner.
__global__ void field_assemble(int n, int N, const int* __restrict__ nbr_in, const double* __restrict__ theta,
                               const double* __restrict__ area, int* nbr, double2* v64, float2* v32,
                               double* d64, float* d32, double* inv64, float* inv32, float* area32) {
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < n; f += gridDim.x * blockDim.x) {
        int cnt = 0;
        for (int j = 0; j < 3; j++) {
            int g = nbr_in[3 * f + j];
            double s, c;
            sincos((double)N * (theta[3 * f + j] + 3.14159265358979323846), &s, &c);
            double2 a = make_double2(-c, -s);
            nbr[j * n + f] = g;
            v64[j * n + f] = a;
            v32[j * n + f] = make_float2((float)a.x, (float)a.y);
            cnt++;
        }
        double d = (double)cnt + 1e-9;
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
__global__ void __launch_bounds__(kBlock) pcg_complex(ComplexEll<T> A, const T* __restrict__ minv,
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

// K2: x = g u, r = b - g Lu (exact algebra of the Galerkin start), partial |r|^2, r32 = r
// g = scal[1] / scal[0] read on the device (no host round trip).
__global__ void power_start(int n, const double* __restrict__ scal, const double2* __restrict__ u,
                            const double2* __restrict__ b, const double2* __restrict__ Lu, double2* x, double2* r,
                            float2* r32, double* partials) {
    const double g = scal[0] > 0 ? scal[1] / scal[0] : 0.0;
    double red[1] = {0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double2 ui = u[i], bi = b[i], li = Lu[i];
        double2 xi = make_double2(g * ui.x, g * ui.y);
        double2 ri = make_double2(bi.x - g * li.x, bi.y - g * li.y);
        x[i] = xi;
        r[i] = ri;
        if (r32) r32[i] = make_float2((float)ri.x, (float)ri.y);
        red[0] += ri.x * ri.x + ri.y * ri.y;
    }
    publish_partials<double, 1>(red, partials);
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

__global__ void zero_f2(int n, float2* e) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) e[i] = make_float2(0.f, 0.f);
}

}  // namespace mtk

using namespace mtk;

namespace {

struct FieldSolver {
    mtk_ctx* c;
    int n;
    DBuf<int> nbr, nbr_in;
    DBuf<double> theta, area, d64, inv64;
    DBuf<float> d32, inv32, area32;
    DBuf<double2> v64, u, b, Lu, x, r, z64, p64, q64;
    DBuf<float2> v32, r32, e32, z32, p32, q32;
    int grid = 0;
    double pcg_ms = 0, pcg_bytes = 0;
    long long pcg_launches = 0;

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
    // Runs the persistent PCG and returns its status, iterations in *iters.
    template <typename T, typename V2>
    int pcg(ComplexEll<T> A, const T* minv, const V2* bb, V2* xx, V2* rr, V2* zz, V2* pp, V2* qq, double tol2,
            int maxit, long long* iters, double* final_rr) {
        int g = 0;
        MTK_TRY(reset_barrier(c));
        MTK_CUDA_TRY(cudaEventRecord(c->ev_k0, c->stream));
        MTK_TRY(launch_persistent(c, pcg_complex<T>, &g, A, minv, bb, xx, rr, zz, pp, qq,
                                  reinterpret_cast<T*>(c->partials), barrier_of(c), tol2, maxit, c->dev_int));
        MTK_CUDA_TRY(cudaEventRecord(c->ev_k1, c->stream));
        MTK_CUDA_TRY(cudaMemcpyAsync(c->h_int, c->dev_int, 8 * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
        MTK_CUDA_TRY(cudaStreamSynchronize(c->stream));
        float kms = 0;
        cudaEventElapsedTime(&kms, c->ev_k0, c->ev_k1);
        pcg_ms += kms;
        pcg_launches++;
        // algorithmic bytes per iteration and row: SpMV 3*(2T+4) + T + 2*2T, x/r/p updates
        // 3 * 3*2T, z = M^-1 r: T + 2T (the r read is shared with the r update)
        const double per_row = 3.0 * (2 * sizeof(T) + 4) + sizeof(T) + 4.0 * sizeof(T) + 18.0 * sizeof(T) + 3.0 * sizeof(T);
        pcg_bytes += per_row * (double)n * (double)(c->h_int[1] + 1);
        *iters += c->h_int[1];
        if (final_rr) *final_rr = reinterpret_cast<double*>(c->h_int + 4)[0];
        int st = c->h_int[0];
        if (st == 5) return MTK_ERR_TIMEOUT;
        if (st == 4) return MTK_ERR_BREAKDOWN;
        if (st == 3) return MTK_ERR_NOT_CONVERGED;
        return MTK_OK;
    }
};

}  // namespace

extern "C" int mtk_field_smoothest(mtk_ctx* c, int32_t nF, int32_t nRosy, const int32_t* nbr_h,
                                   const double* theta_h, const double* area_h, const double* x0,
                                   int32_t n_iter, const mtk_solve_opts* opts_in, double* out, mtk_stats* stats) {
    if (!c || nF <= 0 || nRosy <= 0 || !nbr_h || !theta_h || !area_h || !x0 || !out || n_iter < 0) return MTK_ERR_BAD_INPUT;
    for (int64_t i = 0; i < 3 * (int64_t)nF; i++)
        if (nbr_h[i] < 0 || nbr_h[i] >= nF) { mtk_set_last_error("face neighbour out of range (closed meshes only)", __FILE__, __LINE__); return MTK_ERR_BAD_INPUT; }
    mtk_solve_opts opts;
    mtk_default_opts(&opts);
    if (opts_in) opts = *opts_in;
    MTK_CUDA_TRY(cudaSetDevice(c->device));
    FieldSolver S;
    S.c = c;
    S.n = nF;
    const int n = nF;
    cudaStream_t st = c->stream;
    MTK_CUDA_TRY(cudaEventRecord(c->ev_a, st));
    MTK_TRY(S.nbr_in.upload(nbr_h, 3 * (size_t)n, st));
    MTK_TRY(S.theta.upload(theta_h, 3 * (size_t)n, st));
    MTK_TRY(S.area.upload(area_h, n, st));
    MTK_TRY(S.u.upload(reinterpret_cast<const double2*>(x0), n, st));
    MTK_TRY(S.nbr.alloc(3 * (size_t)n));
    MTK_TRY(S.v64.alloc(3 * (size_t)n));
    MTK_TRY(S.v32.alloc(3 * (size_t)n));
    MTK_TRY(S.d64.alloc(n)); MTK_TRY(S.inv64.alloc(n)); MTK_TRY(S.d32.alloc(n)); MTK_TRY(S.inv32.alloc(n));
    MTK_TRY(S.area32.alloc(n));
    MTK_TRY(S.b.alloc(n)); MTK_TRY(S.Lu.alloc(n)); MTK_TRY(S.x.alloc(n)); MTK_TRY(S.r.alloc(n));
    const bool mixed = opts.precision == MTK_PREC_MIXED;
    if (mixed) {
        MTK_TRY(S.r32.alloc(n)); MTK_TRY(S.e32.alloc(n)); MTK_TRY(S.z32.alloc(n)); MTK_TRY(S.p32.alloc(n)); MTK_TRY(S.q32.alloc(n));
    } else {
        MTK_TRY(S.z64.alloc(n)); MTK_TRY(S.p64.alloc(n)); MTK_TRY(S.q64.alloc(n));
    }
    const int G = stream_grid(c);
    field_assemble<<<G, kStream, 0, st>>>(n, nRosy, S.nbr_in.p, S.theta.p, S.area.p, S.nbr.p, S.v64.p, S.v32.p, S.d64.p,
                                         S.d32.p, S.inv64.p, S.inv32.p, S.area32.p);
    c->kernels++;
    MTK_CUDA_TRY(cudaGetLastError());

    long long iters = 0, solves = 0, refines = 0;
    double worst = 0.0;
    const double tol = opts.tol;
    for (int k = 0; k < n_iter; k++) {
        // b = M u, Galerkin start x = u (u^H M u)/(u^H L u), r = b - L x
        power_prepare<<<G, kStream, 0, st>>>(S.A64(), S.area.p, S.u.p, S.b.p, S.Lu.p, c->partials);
        c->kernels++;
        MTK_TRY(S.finalize(G, 3));
        power_start<<<G, kStream, 0, st>>>(n, c->scalars, S.u.p, S.b.p, S.Lu.p, S.x.p, S.r.p, mixed ? S.r32.p : nullptr,
                                          c->partials);
        c->kernels++;
        MTK_CUDA_TRY(cudaMemcpyAsync(c->h_scalars, c->scalars, 3 * sizeof(double), cudaMemcpyDeviceToHost, st));
        MTK_TRY(S.finalize(G, 1));
        MTK_CUDA_TRY(cudaMemcpyAsync(c->h_scalars + 3, c->scalars, sizeof(double), cudaMemcpyDeviceToHost, st));
        MTK_CUDA_TRY(cudaStreamSynchronize(st));
        const double bnorm2 = c->h_scalars[2];
        double rr = c->h_scalars[3];
        const double goal2 = tol * tol * bnorm2;
        solves++;
        refines++;
        if (!mixed) {
            double frr = 0;
            int s = S.pcg<double, double2>(S.A64(), S.inv64.p, S.b.p, S.x.p, S.r.p, S.z64.p, S.p64.p, S.q64.p, goal2,
                                           opts.max_iter, &iters, &frr);
            if (s != MTK_OK) return s;
            // true FP64 residual of the result
            residual64<<<G, kStream, 0, st>>>(S.A64(), S.b.p, S.x.p, S.r.p, nullptr, c->partials);
            c->kernels++;
            MTK_TRY(S.finalize(G, 1));
            MTK_TRY(S.read_scalars(1));
            rr = c->h_scalars[0];
            refines++;
        } else {
            int outer = 0;
            while (rr > goal2) {
                if (outer >= opts.max_refine) return MTK_ERR_NOT_CONVERGED;
                outer++;
                // inner FP32 solve L e = r to inner_tol relative (at least the outer goal)
                double itol = opts.inner_tol;
                double need = std::sqrt(goal2 / rr) * 0.5;
                if (need > itol) itol = need;
                zero_f2<<<G, kStream, 0, st>>>(n, S.e32.p);
                c->kernels++;
                int s = S.pcg<float, float2>(S.A32(), S.inv32.p, S.r32.p, S.e32.p, S.z32.p /*r*/, S.p32.p /*z*/,
                                             S.q32.p /*p*/, reinterpret_cast<float2*>(S.Lu.p) /*q*/, itol * itol * rr,
                                             opts.max_iter, &iters, nullptr);
                if (s == MTK_ERR_TIMEOUT || s == MTK_ERR_BREAKDOWN) return s;
                add_correction<<<G, kStream, 0, st>>>(n, S.e32.p, S.x.p);
                residual64<<<G, kStream, 0, st>>>(S.A64(), S.b.p, S.x.p, S.r.p, S.r32.p, c->partials);
                c->kernels += 2;
                MTK_TRY(S.finalize(G, 1));
                MTK_TRY(S.read_scalars(1));
                rr = c->h_scalars[0];
                refines++;
            }
        }
        double rel = bnorm2 > 0 ? std::sqrt(rr / bnorm2) : 0.0;
        if (rel > worst) worst = rel;
        // x /= sqrt|x^H M x|; u = x
        mnorm_partial<<<G, kStream, 0, st>>>(n, S.area.p, S.x.p, c->partials);
        c->kernels++;
        MTK_TRY(S.finalize(G, 1));
        normalize_to<<<G, kStream, 0, st>>>(n, c->scalars, S.x.p, S.u.p);
        c->kernels++;
        MTK_CUDA_TRY(cudaGetLastError());
    }
    MTK_CUDA_TRY(cudaMemcpyAsync(out, S.u.p, sizeof(double2) * n, cudaMemcpyDeviceToHost, st));
    MTK_CUDA_TRY(cudaEventRecord(c->ev_b, st));
    MTK_CUDA_TRY(cudaStreamSynchronize(st));
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
        stats->field_pcg_ms += S.pcg_ms;
        stats->field_pcg_bytes += S.pcg_bytes;
        stats->kernel_launches = c->kernels;
    }
    return MTK_OK;
}
