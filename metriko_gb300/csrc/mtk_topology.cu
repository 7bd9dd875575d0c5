// Curl matching and singular indices on the device (mtk_curl_matching).
//
// Replaces the host loops of FaceRosyField::computeMatching(MatchingType::Curl):
// computeConnection (face_rosy_field.h:109-117), cMatching (:169-202) and computeSingular
// (:100-107), with one thread per edge and one per vertex, closed meshes.
//  * The face frame of f is rebuilt from its corners as in the Hmesh constructor (hmesh.h:461-474):
//    bX = dir(p1 - p0), bY = dir(-(p1 - p0) x n), n = (p1 - p0) x (p2 - p0).
//  * The field vectors are field(f, i) = e^{i arg(c_f) / N} e^{2 pi i i / N} (face_rosy_field.h:37-43).
//  * Per edge e (halfedge 2e from edge_vert(e,0) to edge_vert(e,1), faces edge_face(e,0/1)):
//    v = dir(edge vector), connection = (v.bX1 + i v.bY1) / (v.bX0 + i v.bY0);
//    matching = the first i of least sum_j (v . (v1_{(i+j)%N} - v0_j))^2 (strict '<');
//    effort = arg(prod_j field(f1, (j + i) % N) / (field(f0, j) connection)).
//  * Per vertex: the ring from vert_half[v] by h <- twin(prev h) (twin h = h ^ 1), each
//    halfedge adding -effort (the edge's canonical halfedge 2e) or +effort (its twin 2e + 1),
//    singular = round((N angleDefect + sum) / 2 pi).
// The arithmetic is the host's, in the same order, up to the last-bit rounding of the device's
// cos/sin/atan2/sqrt; the integer decisions are the host's (tested on every fixture and at the
// 1.3M-face benchmark size).  A ring that does not close within kMaxRing halfedges sets the error
// word and leaves that vertex's index at 0 (the call then fails with MTK_ERR_BAD_INPUT).
#include <cmath>
#include <vector>

#include "mtk_ctx.cuh"

namespace {

using namespace mtk;

constexpr double kTwoPi = 6.28318530717958647692;
constexpr int kMaxRing = 1 << 16;

struct C2 {
    double re, im;
};
__device__ __forceinline__ C2 cmul(C2 a, C2 b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
__device__ __forceinline__ C2 cdiv(C2 a, C2 b) {
    const double d = b.re * b.re + b.im * b.im;
    return {(a.re * b.re + a.im * b.im) / d, (a.im * b.re - a.re * b.im) / d};
}

struct V3 {
    double x, y, z;
};
__device__ __forceinline__ V3 vsub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ double vdot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V3 vcross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
__device__ __forceinline__ V3 vunit(V3 a) {
    const double r = sqrt(vdot(a, a));
    return {a.x / r, a.y / r, a.z / r};
}
__device__ __forceinline__ V3 vload(const double* __restrict__ P, int v) {
    return {P[3 * (size_t)v], P[3 * (size_t)v + 1], P[3 * (size_t)v + 2]};
}

__device__ __forceinline__ void face_frame(const double* __restrict__ P, const int* __restrict__ F, int f, V3& bx, V3& by) {
    const V3 p0 = vload(P, F[3 * (size_t)f]), p1 = vload(P, F[3 * (size_t)f + 1]), p2 = vload(P, F[3 * (size_t)f + 2]);
    const V3 x = vsub(p1, p0), t = vsub(p2, p0);
    const V3 n = vcross(x, t);
    bx = vunit(x);
    const V3 c = vcross(x, n);
    by = vunit(V3{-c.x, -c.y, -c.z});
}

// the N field vectors of face f as complex numbers in its frame
__device__ __forceinline__ void face_field(const double* __restrict__ c, int f, int N, C2* out) {
    const double a = atan2(c[2 * (size_t)f + 1], c[2 * (size_t)f]) / N;
    const C2 root{cos(a), sin(a)};
    for (int i = 0; i < N; i++) {
        const double b = kTwoPi * i / N;
        out[i] = i ? cmul(root, C2{cos(b), sin(b)}) : root;
    }
}

// NT > 0: N fixed at compile time (the arrays stay in registers); NT = 0: N from the argument
template <int NT>
__global__ void curl_matching(int nE, int Nrt, const double* __restrict__ P, const int* __restrict__ F,
                              const int* __restrict__ ev, const int* __restrict__ ef, const double* __restrict__ c,
                              int* __restrict__ matching, double* __restrict__ effort) {
    const int N = NT > 0 ? NT : Nrt;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nE; e += gridDim.x * blockDim.x) {
        const int f0 = ef[2 * (size_t)e], f1 = ef[2 * (size_t)e + 1];
        const V3 v = vunit(vsub(vload(P, ev[2 * (size_t)e + 1]), vload(P, ev[2 * (size_t)e])));
        V3 bx0, by0, bx1, by1;
        face_frame(P, F, f0, bx0, by0);
        face_frame(P, F, f1, bx1, by1);
        C2 g0[NT > 0 ? NT : 8], g1[NT > 0 ? NT : 8];
        face_field(c, f0, N, g0);
        face_field(c, f1, N, g1);
        // v . (bX a + bY b) for each field vector of either face
        double d0[NT > 0 ? NT : 8], d1[NT > 0 ? NT : 8];
        const double x0 = vdot(v, bx0), y0 = vdot(v, by0), x1 = vdot(v, bx1), y1 = vdot(v, by1);
        for (int j = 0; j < N; j++) {
            d0[j] = vdot(v, V3{bx0.x * g0[j].re + by0.x * g0[j].im, bx0.y * g0[j].re + by0.y * g0[j].im,
                               bx0.z * g0[j].re + by0.z * g0[j].im});
            d1[j] = vdot(v, V3{bx1.x * g1[j].re + by1.x * g1[j].im, bx1.y * g1[j].re + by1.y * g1[j].im,
                               bx1.z * g1[j].re + by1.z * g1[j].im});
        }
        int iM = 0;
        double mn = 32767000.;
        for (int i = 0; i < N; i++) {
            double curl = 0;
            for (int j = 0; j < N; j++) {
                const double d = d1[(i + j) % N] - d0[j];
                curl += d * d;
            }
            if (curl < mn) { iM = i; mn = curl; }
        }
        matching[e] = iM;
        const C2 conn = cdiv(C2{x1, y1}, C2{x0, y0});
        C2 coef{1.0, 0.0};
        for (int i = 0; i < N; i++) coef = cmul(coef, cdiv(g1[(i + iM) % N], cmul(g0[i], conn)));
        effort[e] = atan2(coef.im, coef.re);
    }
}

__global__ void singular_index(int nV, int N, const int* __restrict__ vert_half, const int* __restrict__ prev,
                               const double* __restrict__ defect, const double* __restrict__ effort,
                               int* __restrict__ singular, int* err) {
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nV; v += gridDim.x * blockDim.x) {
        double sum = defect[v] * N;
        const int h0 = vert_half[v];
        int h = h0, steps = 0;
        do {
            sum += ((h & 1) ? 1.0 : -1.0) * effort[h >> 1];
            h = prev[h] ^ 1;
        } while (h != h0 && ++steps < kMaxRing);
        if (h != h0) {
            atomicExch(err, 1);
            singular[v] = 0;
            continue;
        }
        singular[v] = (int)round(sum / kTwoPi);   // std::round: halves away from zero
    }
}

}  // namespace

extern "C" int mtk_curl_matching(mtk_ctx* c, int32_t nV, int32_t nF, int32_t nE, int32_t N, const double* V,
                                 const int32_t* F, const int32_t* edge_vert, const int32_t* edge_face,
                                 const int32_t* vert_half, const int32_t* prev_half, const double* angle_defect,
                                 const double* compressed, int32_t* matching, int32_t* singular) {
    if (!c || nV <= 0 || nF <= 0 || nE <= 0 || N < 1 || N > 8 || !V || !F || !edge_vert || !edge_face || !vert_half ||
        !prev_half || !angle_defect || !compressed || !matching || !singular)
        return MTK_ERR_BAD_INPUT;
    const int64_t nH = 2 * (int64_t)nE;
    auto bad = [](const char* what) {
        mtk_set_last_error(what, __FILE__, __LINE__);
        return MTK_ERR_BAD_INPUT;
    };
    for (int64_t i = 0; i < 3 * (int64_t)nF; i++)
        if (F[i] < 0 || F[i] >= nV) return bad("mtk_curl_matching: face corner out of range");
    for (int64_t i = 0; i < nH; i++) {
        if (edge_vert[i] < 0 || edge_vert[i] >= nV) return bad("mtk_curl_matching: edge vertex out of range");
        if (edge_face[i] < 0 || edge_face[i] >= nF) return bad("mtk_curl_matching: edge face out of range (closed meshes only)");
        if (prev_half[i] < 0 || prev_half[i] >= nH) return bad("mtk_curl_matching: prev halfedge out of range");
    }
    for (int i = 0; i < nV; i++)
        if (vert_half[i] < 0 || vert_half[i] >= nH) return bad("mtk_curl_matching: vertex halfedge out of range");
    MTK_CUDA_TRY(cudaSetDevice(c->device));
    AllocStreamScope alloc_scope(c->stream);
    cudaStream_t st = c->stream;
    DBuf<double> dV, dc, ddef, deff;
    DBuf<int> dF, dev, def, dvh, dprev, dm, ds;
    MTK_TRY(dV.upload(V, 3 * (size_t)nV, st));
    MTK_TRY(dF.upload(F, 3 * (size_t)nF, st));
    MTK_TRY(dev.upload(edge_vert, (size_t)nH, st));
    MTK_TRY(def.upload(edge_face, (size_t)nH, st));
    MTK_TRY(dvh.upload(vert_half, nV, st));
    MTK_TRY(dprev.upload(prev_half, (size_t)nH, st));
    MTK_TRY(ddef.upload(angle_defect, nV, st));
    MTK_TRY(dc.upload(compressed, 2 * (size_t)nF, st));
    MTK_TRY(deff.alloc(nE));
    MTK_TRY(dm.alloc(nE));
    MTK_TRY(ds.alloc(nV));
    MTK_CUDA_TRY(cudaMemsetAsync(c->dev_err, 0, sizeof(int), st));
    const int G = stream_grid(c) * 4;
    auto kernel = N == 4 ? curl_matching<4> : curl_matching<0>;
    kernel<<<G, kStream, 0, st>>>(nE, N, dV.p, dF.p, dev.p, def.p, dc.p, dm.p, deff.p);
    singular_index<<<G, kStream, 0, st>>>(nV, N, dvh.p, dprev.p, ddef.p, deff.p, ds.p, c->dev_err);
    c->kernels += 2;
    MTK_CUDA_TRY(cudaGetLastError());
    MTK_CUDA_TRY(cudaMemcpyAsync(matching, dm.p, sizeof(int) * nE, cudaMemcpyDeviceToHost, st));
    MTK_CUDA_TRY(cudaMemcpyAsync(singular, ds.p, sizeof(int) * nV, cudaMemcpyDeviceToHost, st));
    MTK_CUDA_TRY(cudaMemcpyAsync(c->h_int, c->dev_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    MTK_CUDA_TRY(cudaStreamSynchronize(st));
    if (c->h_int[0]) return bad("mtk_curl_matching: a vertex ring does not close");
    return MTK_OK;
}
