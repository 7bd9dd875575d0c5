// Vertex-position gradient: the assembly backward of the per-face geometry.
//
// The loss's dependence on the vertex positions goes through four per-face quantities, each a
// function of the face's three corners p0, p1, p2 only (the formulas of the Hmesh constructor,
// hmesh.h:461-489, and of the gradient operator G2, parameterization_integ.ipp:11-24):
//   area       A = |(p1 - p0) x (p2 - p0)| / 2
//   farg       of the second and third halfedges (the first is 0): f1 = acos(e1 . e0),
//              f2 = f1 + acos(e2 . e1), e0 = dir(p1 - p0), e1 = dir(p2 - p1), e2 = dir(p0 - p2)
//   G2 entries gx_a, gy_a = (n x (p_{a+2} - p_{a+1}) / 2A) . (bX, bY), bX = e0,
//              bY = dir(-(p1 - p0) x n), n the unit normal
// Given the loss's derivatives with respect to those (dA, df1, df2 from the reverse pass of the
// field, dgx, dgy from the integration), one thread per face evaluates the formulas nine times
// in forward-mode dual numbers (value and derivative along one coordinate of p0, p1, p2) and
// forms the face's nine-coordinate gradient; the vertices then gather their faces' corner
// gradients in ascending face order (deterministic, no atomics).
#include <vector>

#include "mtk_ctx.cuh"

namespace {

using namespace mtk;

struct Dual {
    double v, d;   // value, derivative along the seeded coordinate
};
__device__ __forceinline__ Dual operator+(Dual a, Dual b) { return {a.v + b.v, a.d + b.d}; }
__device__ __forceinline__ Dual operator-(Dual a, Dual b) { return {a.v - b.v, a.d - b.d}; }
__device__ __forceinline__ Dual operator*(Dual a, Dual b) { return {a.v * b.v, a.d * b.v + a.v * b.d}; }
__device__ __forceinline__ Dual operator/(Dual a, Dual b) { return {a.v / b.v, (a.d * b.v - a.v * b.d) / (b.v * b.v)}; }
__device__ __forceinline__ Dual dsqrt(Dual a) {
    const double r = sqrt(a.v);
    return {r, 0.5 * a.d / r};
}
__device__ __forceinline__ Dual dacos(Dual a) { return {acos(a.v), -a.d / sqrt(1.0 - a.v * a.v)}; }

struct Vec3D {
    Dual x, y, z;
};
__device__ __forceinline__ Vec3D operator-(const Vec3D& a, const Vec3D& b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ Vec3D scale(const Vec3D& a, Dual s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ Dual dot(const Vec3D& a, const Vec3D& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ Vec3D cross(const Vec3D& a, const Vec3D& b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ Dual norm(const Vec3D& a) { return dsqrt(dot(a, a)); }
__device__ __forceinline__ Vec3D unit(const Vec3D& a) { return scale(a, Dual{1.0, 0.0} / norm(a)); }

// One face: d loss / d (p0, p1, p2) into g9 (corner-major, x y z).
__device__ void face_backward(const double* P, double gA, double gf1, double gf2, const double* gx, const double* gy,
                              double* g9) {
    for (int q = 0; q < 9; q++) {
        Vec3D p[3];
        for (int c = 0; c < 3; c++) {
            p[c].x = {P[3 * c + 0], q == 3 * c + 0 ? 1.0 : 0.0};
            p[c].y = {P[3 * c + 1], q == 3 * c + 1 ? 1.0 : 0.0};
            p[c].z = {P[3 * c + 2], q == 3 * c + 2 ? 1.0 : 0.0};
        }
        const Vec3D x = p[1] - p[0], t = p[2] - p[0];
        const Vec3D n = cross(x, t);
        const Dual nn = norm(n);
        const Dual A = nn * Dual{0.5, 0.0};
        const Vec3D bX = unit(x);
        const Vec3D nh = scale(n, Dual{1.0, 0.0} / nn);
        const Vec3D bY = unit(scale(cross(x, n), Dual{-1.0, 0.0}));
        const Vec3D e1 = unit(p[2] - p[1]), e2 = unit(p[0] - p[2]);
        const Dual f1 = dacos(dot(e1, bX));
        const Dual f2 = f1 + dacos(dot(e2, e1));
        double d = gA * A.d + gf1 * f1.d + gf2 * f2.d;
        const Dual twoA = A * Dual{2.0, 0.0};
        for (int a = 0; a < 3; a++) {
            const Vec3D g = scale(cross(nh, p[(a + 2) % 3] - p[(a + 1) % 3]), Dual{1.0, 0.0} / twoA);
            d += gx[a] * dot(g, bX).d + gy[a] * dot(g, bY).d;
        }
        g9[q] = d;
    }
}

__global__ void faces_backward(int nF, const double* __restrict__ V, const int* __restrict__ F,
                               const double* __restrict__ gA, const double* __restrict__ gf1,
                               const double* __restrict__ gf2, const double* __restrict__ dgx,
                               const double* __restrict__ dgy, double* g9) {
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < nF; f += gridDim.x * blockDim.x) {
        double P[9];
        for (int c = 0; c < 3; c++)
            for (int k = 0; k < 3; k++) P[3 * c + k] = V[3 * (size_t)F[3 * f + c] + k];
        face_backward(P, gA[f], gf1[f], gf2[f], dgx + 3 * (size_t)f, dgy + 3 * (size_t)f, g9 + 9 * (size_t)f);
    }
}

// per vertex: the sum of its corners' gradients over its faces (entries 3 f + corner, ascending)
__global__ void vertex_gather(int nV, const int* __restrict__ vf_ptr, const int* __restrict__ vf_corner,
                             const double* __restrict__ g9, double* gV) {
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nV; v += gridDim.x * blockDim.x) {
        double s[3] = {0, 0, 0};
        for (int e = vf_ptr[v]; e < vf_ptr[v + 1]; e++) {
            const int fc = vf_corner[e];
            for (int k = 0; k < 3; k++) s[k] += g9[3 * (size_t)fc + k];
        }
        for (int k = 0; k < 3; k++) gV[3 * (size_t)v + k] = s[k];
    }
}

}  // namespace

extern "C" int mtk_face_geometry_backward(mtk_ctx* c, int32_t nV, int32_t nF, const double* V, const int32_t* F,
                                          const double* g_area, const double* g_farg1, const double* g_farg2,
                                          const double* g_gx, const double* g_gy, double* grad_V) {
    if (!c || nV <= 0 || nF <= 0 || !V || !F || !g_area || !g_farg1 || !g_farg2 || !g_gx || !g_gy || !grad_V)
        return MTK_ERR_BAD_INPUT;
    for (int64_t i = 0; i < 3 * (int64_t)nF; i++)
        if (F[i] < 0 || F[i] >= nV) {
            mtk_set_last_error("face corner index out of range", __FILE__, __LINE__);
            return MTK_ERR_BAD_INPUT;
        }
    MTK_CUDA_TRY(cudaSetDevice(c->device));
    AllocStreamScope alloc_scope(c->stream);
    cudaStream_t st = c->stream;
    // vertex -> (face, corner) entries in ascending face order
    std::vector<int> ptr(nV + 1, 0), corner(3 * (size_t)nF);
    for (int64_t i = 0; i < 3 * (int64_t)nF; i++) ptr[F[i] + 1]++;
    for (int v = 0; v < nV; v++) ptr[v + 1] += ptr[v];
    {
        std::vector<int> pos(ptr.begin(), ptr.end() - 1);
        for (int64_t i = 0; i < 3 * (int64_t)nF; i++) corner[pos[F[i]]++] = (int)i;
    }
    DBuf<double> dV, dgA, dg1, dg2, dgx, dgy, g9, gV;
    DBuf<int> dF, dptr, dcorner;
    MTK_TRY(dV.upload(V, 3 * (size_t)nV, st));
    MTK_TRY(dF.upload(F, 3 * (size_t)nF, st));
    MTK_TRY(dgA.upload(g_area, nF, st));
    MTK_TRY(dg1.upload(g_farg1, nF, st));
    MTK_TRY(dg2.upload(g_farg2, nF, st));
    MTK_TRY(dgx.upload(g_gx, 3 * (size_t)nF, st));
    MTK_TRY(dgy.upload(g_gy, 3 * (size_t)nF, st));
    MTK_TRY(dptr.upload(ptr.data(), ptr.size(), st));
    MTK_TRY(dcorner.upload(corner.data(), corner.size(), st));
    MTK_TRY(g9.alloc(9 * (size_t)nF));
    MTK_TRY(gV.alloc(3 * (size_t)nV));
    const int G = stream_grid(c);
    faces_backward<<<G, kStream, 0, st>>>(nF, dV.p, dF.p, dgA.p, dg1.p, dg2.p, dgx.p, dgy.p, g9.p);
    vertex_gather<<<G, kStream, 0, st>>>(nV, dptr.p, dcorner.p, g9.p, gV.p);
    c->kernels += 2;
    MTK_CUDA_TRY(cudaGetLastError());
    MTK_CUDA_TRY(cudaMemcpyAsync(grad_V, gV.p, sizeof(double) * 3 * nV, cudaMemcpyDeviceToHost, st));
    MTK_CUDA_TRY(cudaStreamSynchronize(st));
    return MTK_OK;
}
