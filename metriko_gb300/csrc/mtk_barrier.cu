// Local-injectivity pieces of the IGM rounding (the reference's localInjectivity option):
// the per-face barrier of InjectiveBarrier (core/igm/iterative_rounding/injective_barrier.h:10-110)
// and the orientation check of locally_injectivity_check (core/igm/parameterization_integ.ipp:46-63),
// as device kernels behind C-ABI entry points.
#include <cmath>
#include <limits>

#include "mtk_common.cuh"
#include "mtk_ctx.cuh"

using namespace mtk;

namespace {

// One row per (face i, vector j): v0 = field vector j, v1 = vector (j+1) mod N of face i,
// V = |F2_j| |F2_{j+1}| of the intrinsic field, r = cross(v0, v1) / V (volume ratio) and, with
// s = 0.5, the cubic spline bar(r) = (r/s)^3 - 3 (r/s)^2 + 3 r/s, the barrier 1/bar - 1
// (infinite for r <= 0, zero for r >= s), its derivative -bar'(r) / bar^2 (0 where the barrier is
// below 1e-8, infinite where it is infinite) and the row of dr/d(v0.x, v0.y, v1.x, v1.y).
// The cubes and squares are products (the reference calls pow).
__global__ void barrier_rows(int nF, int N, const double* __restrict__ F2, const double* __restrict__ field, int update_j,
                             double* fB, double* dB, double* S) {
    const double s = 0.5;
    const double inf = __longlong_as_double(0x7ff0000000000000LL);
    const int rows = nF * N;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < rows; k += gridDim.x * blockDim.x) {
        const int i = k / N, j = k % N, j1 = (j + 1) % N;
        const size_t o0 = 2 * (size_t)N * i + 2 * j, o1 = 2 * (size_t)N * i + 2 * j1;
        // norms, cross product and S rounded as the reference's expressions (no fused multiply-add)
        const double n0 = __dsqrt_rn(__dadd_rn(__dmul_rn(F2[o0], F2[o0]), __dmul_rn(F2[o0 + 1], F2[o0 + 1])));
        const double n1 = __dsqrt_rn(__dadd_rn(__dmul_rn(F2[o1], F2[o1]), __dmul_rn(F2[o1 + 1], F2[o1 + 1])));
        const double V = __dmul_rn(n0, n1);
        const double v0x = field[o0], v0y = field[o0 + 1], v1x = field[o1], v1y = field[o1 + 1];
        const double r = __ddiv_rn(__dsub_rn(__dmul_rn(v0x, v1y), __dmul_rn(v0y, v1x)), V);
        const double q = r / s;
        const double bar = q * q * q - 3.0 * (q * q) + 3.0 * r / s;
        double bar2 = 1.0 / bar - 1.0;
        if (r <= 0) bar2 = inf;
        if (r >= s) bar2 = 0.0;
        fB[k] = bar2;
        if (!update_j) continue;
        double d = 3.0 * (r * r / (s * s * s)) - 6.0 * (r / (s * s)) + 3.0 / s;
        if (r <= 0) d = inf;
        if (r >= s) d = 0.0;
        double der = -d / (bar * bar);
        if (fabs(bar2) < 10e-9) der = 0.0;
        else if (bar2 == inf) der = inf;
        dB[k] = der;
        S[4 * (size_t)k] = __ddiv_rn(v1y, V);
        S[4 * (size_t)k + 1] = __ddiv_rn(-v1x, V);
        S[4 * (size_t)k + 2] = __ddiv_rn(-v0y, V);
        S[4 * (size_t)k + 3] = __ddiv_rn(v0x, V);
    }
}

// Orientation of every cut face in the parameterization: corners a, b, c (functions 0 and 1 of
// each corner, cfn row layout [corner][function]); flipped where cross(b - a, c - a) < 0.
// out[0] = flipped faces, out[1] = the first flipped face (nF when none).
__global__ void orientation_count(int nF, int N, const double* __restrict__ cfn, int* out) {
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < nF; f += gridDim.x * blockDim.x) {
        const double* c = cfn + 3 * (size_t)N * f;
        const double ax = c[0], ay = c[1];
        const double d1x = __dsub_rn(c[N], ax), d1y = __dsub_rn(c[N + 1], ay);
        const double d2x = __dsub_rn(c[2 * N], ax), d2y = __dsub_rn(c[2 * N + 1], ay);
        if (__dsub_rn(__dmul_rn(d1x, d2y), __dmul_rn(d1y, d2x)) < 0) {   // rounded as the reference's
            atomicAdd(out, 1);
            atomicMin(out + 1, f);
        }
    }
}

}  // namespace

extern "C" int mtk_injective_barrier(mtk_ctx* c, int32_t nF, int32_t N, const double* intrinsic_field,
                                     const double* field, int32_t update_j, double* f_barrier, double* bar_der,
                                     double* s_rows) {
    if (!c || nF < 0 || N < 2 || !intrinsic_field || !field || !f_barrier || (update_j && (!bar_der || !s_rows)))
        return MTK_ERR_BAD_INPUT;
    if (nF == 0) return MTK_OK;
    MTK_CUDA_TRY(cudaSetDevice(c->device));
    AllocStreamScope alloc_scope(c->stream);
    cudaStream_t st = c->stream;
    const size_t nv = 2 * (size_t)N * nF, nr = (size_t)N * nF;
    DBuf<double> dF2, dfield, dfB, ddB, dS;
    MTK_TRY(dF2.upload(intrinsic_field, nv, st));
    MTK_TRY(dfield.upload(field, nv, st));
    MTK_TRY(dfB.alloc(nr));
    MTK_TRY(ddB.alloc(update_j ? nr : 1));
    MTK_TRY(dS.alloc(update_j ? 4 * nr : 1));
    barrier_rows<<<stream_grid(c), kStream, 0, st>>>(nF, N, dF2.p, dfield.p, update_j, dfB.p, ddB.p, dS.p);
    c->kernels++;
    MTK_CUDA_TRY(cudaGetLastError());
    MTK_CUDA_TRY(cudaMemcpyAsync(f_barrier, dfB.p, sizeof(double) * nr, cudaMemcpyDeviceToHost, st));
    if (update_j) {
        MTK_CUDA_TRY(cudaMemcpyAsync(bar_der, ddB.p, sizeof(double) * nr, cudaMemcpyDeviceToHost, st));
        MTK_CUDA_TRY(cudaMemcpyAsync(s_rows, dS.p, sizeof(double) * 4 * nr, cudaMemcpyDeviceToHost, st));
    }
    MTK_CUDA_TRY(cudaStreamSynchronize(st));
    return MTK_OK;
}

extern "C" int mtk_local_injectivity(mtk_ctx* c, int32_t nF, int32_t N, const double* cfn, int32_t* n_flipped,
                                     int32_t* first_flipped) {
    if (!c || nF < 0 || N < 2 || !cfn || !n_flipped) return MTK_ERR_BAD_INPUT;
    *n_flipped = 0;
    if (first_flipped) *first_flipped = nF;
    if (nF == 0) return MTK_OK;
    MTK_CUDA_TRY(cudaSetDevice(c->device));
    AllocStreamScope alloc_scope(c->stream);
    cudaStream_t st = c->stream;
    DBuf<double> dc;
    MTK_TRY(dc.upload(cfn, 3 * (size_t)N * nF, st));
    int h[2] = {0, nF};
    MTK_CUDA_TRY(cudaMemcpyAsync(c->dev_int, h, sizeof(h), cudaMemcpyHostToDevice, st));
    orientation_count<<<stream_grid(c), kStream, 0, st>>>(nF, N, dc.p, c->dev_int);
    c->kernels++;
    MTK_CUDA_TRY(cudaGetLastError());
    MTK_CUDA_TRY(cudaMemcpyAsync(h, c->dev_int, sizeof(h), cudaMemcpyDeviceToHost, st));
    MTK_CUDA_TRY(cudaStreamSynchronize(st));
    *n_flipped = h[0];
    if (first_flipped) *first_flipped = h[1];
    return MTK_OK;
}
