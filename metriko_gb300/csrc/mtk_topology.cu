// Curl matching and singular indices on the device (mtk_curl_matching).
//
// Replaces the host loops of FaceRosyField::computeMatching(MatchingType::Curl):
// computeConnection (face_rosy_field.h:109-117), cMatching (:169-202) and computeSingular
// (:100-107), with one thread per edge and one per vertex.  Boundary edges (a face slot of -1)
// keep matching -1 and effort 0 (:121-122, :170); boundary vertices keep the index 1 (:101-102).
//  * The face frame of f is rebuilt from its corners as in the Hmesh constructor (hmesh.h:461-474):
//    bX = dir(p1 - p0), bY = dir(-(p1 - p0) x n), n = (p1 - p0) x (p2 - p0).
//  * The field vectors are field(f, i) = e^{i arg(c_f) / N} e^{2 pi i i / N} (face_rosy_field.h:37-43).
//  * Per edge e (halfedge 2e from edge_vert(e,0) to edge_vert(e,1), faces edge_face(e,0/1)):
//    v = dir(edge vector), connection = (v.bX1 + i v.bY1) / (v.bX0 + i v.bY0);
//    matching = the first i of least sum_j (v . (v1_{(i+j)%N} - v0_j))^2 (strict '<');
//    effort = arg(prod_j field(f1, (j + i) % N) / (field(f0, j) connection)).
//  * Per vertex: the ring from vert_half[v] by h <- twin(prev h), each halfedge adding -effort
//    (the edge's canonical halfedge edge2half[e]) or +effort (its twin),
//    singular = round((N angleDefect + sum) / 2 pi); a ring that meets a boundary halfedge (id
//    >= 3 nF: boundary halfedges are numbered after the interior ones) marks a boundary vertex.
//    A closed mesh may pass no halfedge arrays: its halfedges are 2e and 2e + 1 (twin h = h ^ 1).
// The arithmetic is the host's, in the same order, up to the last-bit rounding of the device's
// cos/sin/atan2/sqrt; the integer decisions are the host's (tested on every fixture and at the
// 1.3M-face benchmark size).  A ring that does not close within kMaxRing halfedges sets the error
// word and leaves that vertex's index at 0 (the call then fails with MTK_ERR_BAD_INPUT).
//
// Field inputs from the raw mesh on the device (mtk_mesh_field_inputs, mtk_field_smoothest_mesh):
// the face across each face side (-1 on a boundary side, with theta 0), theta = heArgOnFace(h) -
// heArgOnFace(twin h) and the face areas of the Hmesh constructor (hmesh.h:313-489) without
// building the halfedge mesh.  The face
// sides are paired through a hash table keyed by their sorted vertex pair; the face frames and
// halfedge angles repeat the host's arithmetic in its order (no contraction into fused
// multiply-adds), so area and the pairing are the host's bit for bit and theta differs from it
// only by the last-bit rounding of acos.  The pipeline entry point starts the field solve from
// these while a host thread builds the halfedge mesh.
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
        if (f0 < 0 || f1 < 0) {   // boundary edge
            matching[e] = -1;
            effort[e] = 0.0;
            continue;
        }
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

// twin/hedge/e2h: the halfedge arrays of a mesh with boundary, or all null for the closed
// numbering (halfedges 2e, 2e + 1); nI = 3 nF, the first boundary halfedge id
__global__ void singular_index(int nV, int N, int nI, const int* __restrict__ vert_half, const int* __restrict__ prev,
                               const int* __restrict__ twin, const int* __restrict__ hedge, const int* __restrict__ e2h,
                               const double* __restrict__ defect, const double* __restrict__ effort,
                               int* __restrict__ singular, int* err) {
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nV; v += gridDim.x * blockDim.x) {
        double sum = defect[v] * N;
        const int h0 = vert_half[v];
        int h = h0, steps = 0;
        bool boundary = false;
        do {
            if (twin) {
                if (h >= nI) boundary = true;
                const int e = hedge[h];
                sum += (e2h[e] == h ? -1.0 : 1.0) * effort[e];
                h = twin[prev[h]];
            } else {
                sum += ((h & 1) ? 1.0 : -1.0) * effort[h >> 1];
                h = prev[h] ^ 1;
            }
        } while (h != h0 && ++steps < kMaxRing);
        if (h != h0) {
            atomicExch(err, 1);
            singular[v] = 0;
            continue;
        }
        singular[v] = boundary ? 1 : (int)round(sum / kTwoPi);   // std::round: halves away from zero
    }
}

// ------------------------------------------------------------------ field inputs from V, F
constexpr unsigned long long kEmpty = ~0ull;

__device__ __forceinline__ unsigned long long mix64(unsigned long long k) {
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdull;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ull;
    k ^= k >> 33;
    return k;
}

// each face side (f, j) from F(f, j) to F(f, j+1) into the table keyed by its sorted vertex pair;
// the first two sides of a key fill its two slots, a third sets err bit 1 (non-manifold edge)
__global__ void sides_insert(int nF, const int* __restrict__ F, unsigned long long mask, unsigned long long* keys,
                             int* s0, int* s1, int* err) {
    const int ns = 3 * nF;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < ns; s += gridDim.x * blockDim.x) {
        const int f = s / 3, j = s - 3 * f;
        const int a = F[3 * (size_t)f + j], b = F[3 * (size_t)f + (j + 1) % 3];
        if (a == b) { atomicOr(err, 8); continue; }
        const unsigned long long key = ((unsigned long long)min(a, b) << 32) | (unsigned long long)max(a, b);
        unsigned long long h = mix64(key) & mask;
        for (unsigned long long probe = 0; probe <= mask; probe++) {
            const unsigned long long prev = atomicCAS(keys + h, kEmpty, key);
            if (prev == kEmpty || prev == key) {
                if (atomicCAS(s0 + h, -1, s) != -1 && atomicCAS(s1 + h, -1, s) != -1) atomicOr(err, 1);
                break;
            }
            h = (h + 1) & mask;
        }
    }
}

// partner side of every side (stays -1 for the one side of a boundary edge); err bit 4: two sides
// running the same way (inconsistent orientation)
__global__ void sides_pair(unsigned long long nslot, const int* __restrict__ F, const unsigned long long* __restrict__ keys,
                           const int* __restrict__ s0, const int* __restrict__ s1, int* partner, int* err) {
    for (unsigned long long h = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; h < nslot;
         h += (unsigned long long)gridDim.x * blockDim.x) {
        if (keys[h] == kEmpty) continue;
        const int a = s0[h], b = s1[h];
        if (b < 0) continue;   // boundary edge
        const int fa = a / 3, ja = a - 3 * fa, fb = b / 3, jb = b - 3 * fb;
        const int ta = F[3 * (size_t)fa + ja], tb = F[3 * (size_t)fb + jb];
        if (ta == tb) atomicOr(err, 4);
        partner[a] = b;
        partner[b] = a;
    }
}

__device__ __forceinline__ double sq_rn(V3 a) {
    return __dadd_rn(__dadd_rn(__dmul_rn(a.x, a.x), __dmul_rn(a.y, a.y)), __dmul_rn(a.z, a.z));
}
__device__ __forceinline__ double dot_rn(V3 a, V3 b) {
    return __dadd_rn(__dadd_rn(__dmul_rn(a.x, b.x), __dmul_rn(a.y, b.y)), __dmul_rn(a.z, b.z));
}
__device__ __forceinline__ V3 sub_rn(V3 a, V3 b) { return {__dsub_rn(a.x, b.x), __dsub_rn(a.y, b.y), __dsub_rn(a.z, b.z)}; }
__device__ __forceinline__ V3 unit_rn(V3 a) {   // Row3d::normalized
    const double n = sq_rn(a);
    if (!(n > 0)) return a;
    const double r = __dsqrt_rn(n);
    return {__ddiv_rn(a.x, r), __ddiv_rn(a.y, r), __ddiv_rn(a.z, r)};
}

// per face: heArgOnFace of its three sides (hmesh.h:480-489) and its area (hmesh.h:461-474)
__global__ void face_angles(int nF, const double* __restrict__ P, const int* __restrict__ F, double* farg, double* area) {
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < nF; f += gridDim.x * blockDim.x) {
        const V3 p0 = vload(P, F[3 * (size_t)f]), p1 = vload(P, F[3 * (size_t)f + 1]), p2 = vload(P, F[3 * (size_t)f + 2]);
        const V3 x = sub_rn(p1, p0);
        const V3 dm = sub_rn(p0, p2);
        const V3 t{__dmul_rn(dm.x, -1.0), __dmul_rn(dm.y, -1.0), __dmul_rn(dm.z, -1.0)};
        const V3 n{__dsub_rn(__dmul_rn(x.y, t.z), __dmul_rn(x.z, t.y)), __dsub_rn(__dmul_rn(x.z, t.x), __dmul_rn(x.x, t.z)),
                   __dsub_rn(__dmul_rn(x.x, t.y), __dmul_rn(x.y, t.x))};
        area[f] = __dmul_rn(__dsqrt_rn(sq_rn(n)), 0.5);
        const V3 bx = unit_rn(x);
        const V3 e[3] = {unit_rn(sub_rn(p1, p0)), unit_rn(sub_rn(p2, p1)), unit_rn(sub_rn(p0, p2))};
        double sum = 0.0;
        for (int j = 0; j < 3; j++) {
            const V3 v1 = e[j], v2 = e[(j + 2) % 3];
            if (__dsqrt_rn(sq_rn(sub_rn(v1, bx))) > 1e-10) sum = __dadd_rn(sum, acos(dot_rn(v1, v2)));
            farg[3 * (size_t)f + j] = sum;
        }
    }
}

__global__ void side_outputs(int nF, const int* __restrict__ partner, const double* __restrict__ farg, int* nbr,
                             double* theta) {
    const int ns = 3 * nF;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < ns; s += gridDim.x * blockDim.x) {
        const int t = partner[s];
        if (t < 0) {   // boundary side: no neighbour (face_rosy_field.h:64)
            nbr[s] = -1;
            theta[s] = 0.0;
            continue;
        }
        nbr[s] = t / 3;
        theta[s] = __dsub_rn(farg[s], farg[t]);
    }
}

// ------------------------------------------------------------------ singularity paths (seams)
// cut_mesh_with_singularities' searches (face_rosy_field.h:287-326, libigl's unit-weight
// dijkstra): for each source in order, a breadth-first search by levels from the source until a
// level holds a vertex of the cut; the path runs from the smallest-id such vertex back along the
// predecessors (each vertex's predecessor: its smallest-id neighbour in the previous level) and
// joins the cut.  One cooperative launch runs every search, one grid barrier per level:
//  * sd[v] = (search << 32) | level marks the vertices reached by the current search (claimed by
//    compare-and-swap, so each vertex enters one level once); pred[v] keeps, per search, the
//    smallest neighbour id of the previous level by a 64-bit atomicMin on
//    ((~search) << 32) | neighbour -- both are independent of the order of the expansion;
//  * a vertex is checked against the cut when it is claimed, and the smallest cut vertex of the
//    new level (atomicMin) ends the search after the barrier;
//  * counts and minima rotate over three slots (level d reads slot d % 3, fills (d + 1) % 3 and
//    clears (d + 2) % 3), so no slot is cleared while another CTA may still read it;
//  * one thread walks the path back, adds its vertices to the cut and flags its edges.
// Every loop is bounded (levels <= nV, path <= nV steps) and every wait is the bounded grid
// barrier; a timeout leaves the error flag set and the call returns MTK_ERR_TIMEOUT.
constexpr int kNone = 0x7fffffff;

__global__ void __launch_bounds__(kBlock, 1) seam_paths(int nV, int ns, const int* __restrict__ vptr,
                                                       const int* __restrict__ vv, const int* __restrict__ ve,
                                                       const int* __restrict__ src, int* in_cut, unsigned long long* sd,
                                                       unsigned long long* pred, int* fr, int* ctl,
                                                       unsigned char* seam_edge, GridBarrier bar) {
    // ctl: [0] vertices on the cut, [1..3] frontier counts, [4..6] smallest cut vertex per slot
    const int stride = gridDim.x * blockDim.x;
    const int t0 = blockIdx.x * blockDim.x + threadIdx.x;
    const bool lead = blockIdx.x == 0 && threadIdx.x == 0;
    for (int si = 0; si < ns; si++) {
        const int s = src[si];
        const unsigned int iter = (unsigned int)si + 1u;
        if (ld_volatile(ctl) == 0) {
            // no cut vertex anywhere: the search would exhaust the mesh, the path is the source
            // alone.  Every CTA reads ctl[0] before the lead changes it (first barrier), so all
            // CTAs take this branch together.
            if (!grid_sync(bar)) return;
            if (lead) { in_cut[s] = 1; ctl[0] = 1; }
            if (!grid_sync(bar)) return;
            continue;
        }
        if (ld_volatile(in_cut + s)) continue;   // found at level 0: the path is the source alone
        if (lead) {
            fr[0] = s;
            ctl[1] = 1; ctl[2] = 0; ctl[3] = 0;
            ctl[4] = kNone; ctl[5] = kNone; ctl[6] = kNone;
            sd[s] = ((unsigned long long)iter << 32);
            pred[s] = ~0ull;
        }
        if (!grid_sync(bar)) return;
        int found = -1;
        for (int d = 0; d < nV; d++) {
            const int p = d % 3, q = (d + 1) % 3, r = (d + 2) % 3;
            const int n = ld_volatile(ctl + 1 + p);
            const int* cur = fr + (size_t)p * nV;
            int* nxt = fr + (size_t)q * nV;
            if (lead) { ctl[1 + r] = 0; ctl[4 + r] = kNone; }
            const unsigned long long lvl = ((unsigned long long)iter << 32) | (unsigned int)(d + 1);
            const unsigned long long pk_hi = (unsigned long long)(~iter) << 32;
            for (int i = t0; i < n; i += stride) {
                const int u = __ldcg(cur + i);
                const unsigned long long pk = pk_hi | (unsigned int)u;
                const int e1 = vptr[u + 1];
                for (int k = vptr[u]; k < e1; k++) {
                    const int w = vv[k];
                    unsigned long long old = atomicAdd(sd + w, 0ull);
                    bool join = false;
                    for (int tries = 0; tries < 64; tries++) {
                        if ((old >> 32) == iter) { join = old == lvl; break; }
                        const unsigned long long prev = atomicCAS(sd + w, old, lvl);
                        if (prev == old) {   // claimed: w enters level d + 1
                            const int idx = atomicAdd(ctl + 1 + q, 1);
                            nxt[idx] = w;
                            if (ld_volatile(in_cut + w)) atomicMin(ctl + 4 + q, w);
                            join = true;
                            break;
                        }
                        old = prev;
                    }
                    if (join) atomicMin(pred + w, pk);
                }
            }
            if (!grid_sync(bar)) return;
            const int f = ld_volatile(ctl + 4 + q);
            if (f != kNone) { found = f; break; }
            if (ld_volatile(ctl + 1 + q) == 0) break;   // the search exhausted its component
        }
        if (lead) {
            int ncut = ctl[0];
            if (found >= 0) {
                int v = found;
                for (int step = 0; v != s && step < nV; step++) {
                    if (!in_cut[v]) { in_cut[v] = 1; ncut++; }
                    const int u = (int)(unsigned int)(pred[v] & 0xffffffffull);
                    for (int k = vptr[v]; k < vptr[v + 1]; k++)
                        if (vv[k] == u) { seam_edge[ve[k]] = 1; break; }
                    v = u;
                }
            }
            if (!in_cut[s]) { in_cut[s] = 1; ncut++; }
            ctl[0] = ncut;
        }
        if (!grid_sync(bar)) return;
    }
}

// ------------------------------------------------------------------ combing turns
// compute_combbed_field's search (face_rosy_field.h:217-242): from face 0 (turn 0), across every
// face side that is neither a seam nor a boundary, the neighbour's turn is (the side's signed
// matching + the face's turn) mod N.  The reference pops a queue; here the faces are reached level
// by level (one grid barrier per level), a face taking the value of whichever neighbour of the
// previous level claims it first.  Every singular vertex lies on the seam, so no loop inside the
// cut disk carries holonomy: the turns do not depend on the path, and any claim gives the
// reference's value (the tests compare with the host search on every fixture).
__global__ void __launch_bounds__(kBlock, 1) comb_turns(int nF, int N, const int* __restrict__ nb,
                                                       const int* __restrict__ nm, int* turns, int* fr, int* ctl,
                                                       GridBarrier bar) {
    // ctl[0..2]: frontier counts per slot (level d reads d % 3, fills (d + 1) % 3, clears (d + 2) % 3)
    const int stride = gridDim.x * blockDim.x;
    const int t0 = blockIdx.x * blockDim.x + threadIdx.x;
    const bool lead = blockIdx.x == 0 && threadIdx.x == 0;
    for (int d = 0; d < nF; d++) {
        const int p = d % 3, q = (d + 1) % 3, r = (d + 2) % 3;
        const int n = ld_volatile(ctl + p);
        if (n == 0) break;
        const int* cur = fr + (size_t)p * nF;
        int* nxt = fr + (size_t)q * nF;
        if (lead) ctl[r] = 0;
        for (int i = t0; i < n; i += stride) {
            const int f = __ldcg(cur + i);
            const int tf = __ldcg(turns + f);
            for (int j = 0; j < 3; j++) {
                const int g = nb[3 * (size_t)f + j];
                if (g < 0) continue;
                const int val = ((nm[3 * (size_t)f + j] + tf) % N + N) % N;
                if (atomicCAS(turns + g, -1, val) == -1) nxt[atomicAdd(ctl + q, 1)] = g;
            }
        }
        if (!grid_sync(bar)) return;
    }
}

}  // namespace

extern "C" int mtk_comb_turns(mtk_ctx* c, int32_t nF, int32_t N, const int32_t* nb, const int32_t* nm, int32_t* turns) {
    if (!c || nF <= 0 || N < 1 || !nb || !nm || !turns) return MTK_ERR_BAD_INPUT;
    for (int64_t i = 0; i < 3 * (int64_t)nF; i++)
        if (nb[i] < -1 || nb[i] >= nF) {
            mtk_set_last_error("mtk_comb_turns: neighbour out of range", __FILE__, __LINE__);
            return MTK_ERR_BAD_INPUT;
        }
    MTK_CUDA_TRY(cudaSetDevice(c->device));
    AllocStreamScope alloc_scope(c->stream);
    cudaStream_t st = c->stream;
    DBuf<int> dnb, dnm, dturn, dfr, dctl;
    MTK_TRY(dnb.upload(nb, 3 * (size_t)nF, st));
    MTK_TRY(dnm.upload(nm, 3 * (size_t)nF, st));
    MTK_TRY(dturn.alloc(nF));
    MTK_TRY(dfr.alloc(3 * (size_t)nF));
    MTK_CUDA_TRY(cudaMemsetAsync(dturn.p, 0xff, sizeof(int) * nF, st));   // -1: not reached
    const int zero = 0;
    MTK_CUDA_TRY(cudaMemcpyAsync(dturn.p, &zero, sizeof(int), cudaMemcpyHostToDevice, st));
    MTK_CUDA_TRY(cudaMemcpyAsync(dfr.p, &zero, sizeof(int), cudaMemcpyHostToDevice, st));
    const int h_ctl[3] = {1, 0, 0};
    MTK_TRY(dctl.upload(h_ctl, 3, st));
    int grid = 0;
    MTK_TRY(launch_persistent(c, comb_turns, &grid, (int)nF, (int)N, (const int*)dnb.p, (const int*)dnm.p, dturn.p, dfr.p,
                              dctl.p, barrier_of(c)));
    MTK_CUDA_TRY(cudaGetLastError());
    MTK_CUDA_TRY(cudaMemcpyAsync(turns, dturn.p, sizeof(int) * nF, cudaMemcpyDeviceToHost, st));
    MTK_CUDA_TRY(cudaMemcpyAsync(c->h_int, c->dev_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    MTK_CUDA_TRY(cudaStreamSynchronize(st));
    if (c->h_int[0]) {
        mtk_set_last_error("mtk_comb_turns: a grid barrier wait ran out", __FILE__, __LINE__);
        return MTK_ERR_TIMEOUT;
    }
    return MTK_OK;
}

extern "C" int mtk_seam_paths(mtk_ctx* c, int32_t nV, int32_t nE, const int32_t* vptr, const int32_t* vv,
                              const int32_t* ve, int32_t n_src, const int32_t* src, uint8_t* in_cut, uint8_t* seam) {
    if (!c || nV <= 0 || nE <= 0 || n_src < 0 || !vptr || !vv || !ve || (n_src > 0 && !src) || !in_cut || !seam)
        return MTK_ERR_BAD_INPUT;
    auto bad = [](const char* what) {
        mtk_set_last_error(what, __FILE__, __LINE__);
        return MTK_ERR_BAD_INPUT;
    };
    if (vptr[0] != 0) return bad("mtk_seam_paths: vptr[0] must be 0");
    for (int v = 0; v < nV; v++)
        if (vptr[v + 1] < vptr[v]) return bad("mtk_seam_paths: vptr must not decrease");
    const int64_t nadj = vptr[nV];
    for (int64_t k = 0; k < nadj; k++) {
        if (vv[k] < 0 || vv[k] >= nV) return bad("mtk_seam_paths: neighbour out of range");
        if (ve[k] < 0 || ve[k] >= nE) return bad("mtk_seam_paths: edge out of range");
    }
    for (int i = 0; i < n_src; i++)
        if (src[i] < 0 || src[i] >= nV) return bad("mtk_seam_paths: source out of range");
    if (n_src == 0) return MTK_OK;
    MTK_CUDA_TRY(cudaSetDevice(c->device));
    AllocStreamScope alloc_scope(c->stream);
    cudaStream_t st = c->stream;
    std::vector<int> cut_i(nV);
    int ncut = 0;
    for (int v = 0; v < nV; v++) { cut_i[v] = in_cut[v] ? 1 : 0; ncut += cut_i[v]; }
    DBuf<int> dptr, dvv, dve, dsrc, dcut, dfr, dctl;
    DBuf<unsigned long long> dsd, dpred;
    DBuf<unsigned char> dseam;
    MTK_TRY(dptr.upload(vptr, (size_t)nV + 1, st));
    MTK_TRY(dvv.upload(vv, (size_t)nadj, st));
    MTK_TRY(dve.upload(ve, (size_t)nadj, st));
    MTK_TRY(dsrc.upload(src, (size_t)n_src, st));
    MTK_TRY(dcut.upload(cut_i.data(), (size_t)nV, st));
    MTK_TRY(dseam.upload(seam, (size_t)nE, st));
    MTK_TRY(dfr.alloc(3 * (size_t)nV));
    MTK_TRY(dsd.alloc(nV));
    MTK_TRY(dpred.alloc(nV));
    int h_ctl[8] = {ncut, 0, 0, 0, kNone, kNone, kNone, 0};
    MTK_TRY(dctl.upload(h_ctl, 8, st));
    MTK_CUDA_TRY(cudaMemsetAsync(dsd.p, 0, sizeof(unsigned long long) * nV, st));      // no search yet
    MTK_CUDA_TRY(cudaMemsetAsync(dpred.p, 0xff, sizeof(unsigned long long) * nV, st));  // above every key
    int grid = 0;
    MTK_TRY(launch_persistent(c, seam_paths, &grid, (int)nV, (int)n_src, (const int*)dptr.p, (const int*)dvv.p,
                              (const int*)dve.p, (const int*)dsrc.p, dcut.p, dsd.p, dpred.p, dfr.p, dctl.p, dseam.p,
                              barrier_of(c)));
    MTK_CUDA_TRY(cudaGetLastError());
    MTK_CUDA_TRY(cudaMemcpyAsync(cut_i.data(), dcut.p, sizeof(int) * nV, cudaMemcpyDeviceToHost, st));
    MTK_CUDA_TRY(cudaMemcpyAsync(seam, dseam.p, (size_t)nE, cudaMemcpyDeviceToHost, st));
    MTK_CUDA_TRY(cudaMemcpyAsync(c->h_int, c->dev_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    MTK_CUDA_TRY(cudaStreamSynchronize(st));
    if (c->h_int[0]) {
        mtk_set_last_error("mtk_seam_paths: a grid barrier wait ran out", __FILE__, __LINE__);
        return MTK_ERR_TIMEOUT;
    }
    for (int v = 0; v < nV; v++) in_cut[v] = (uint8_t)cut_i[v];
    return MTK_OK;
}

extern "C" int mtk_mesh_field_inputs(mtk_ctx* c, int32_t nV, int32_t nF, const double* V, const int32_t* F, int32_t* nbr,
                                     double* theta, double* area) {
    if (!c || nV <= 0 || nF <= 0 || !V || !F || !nbr || !theta || !area) return MTK_ERR_BAD_INPUT;
    if (nF > (1 << 29)) return MTK_ERR_BAD_INPUT;
    for (int64_t i = 0; i < 3 * (int64_t)nF; i++)
        if (F[i] < 0 || F[i] >= nV) {
            mtk_set_last_error("mtk_mesh_field_inputs: face corner out of range", __FILE__, __LINE__);
            return MTK_ERR_BAD_INPUT;
        }
    MTK_CUDA_TRY(cudaSetDevice(c->device));
    AllocStreamScope alloc_scope(c->stream);
    cudaStream_t st = c->stream;
    const size_t ns = 3 * (size_t)nF;
    size_t nslot = 1;
    while (nslot < ns) nslot <<= 1;   // at most half full: a key takes one slot for two sides
    DBuf<double> dV, dfarg, darea, dtheta;
    DBuf<int> dF, ds0, ds1, dpart, dnbr;
    DBuf<unsigned long long> dkeys;
    MTK_TRY(dV.upload(V, 3 * (size_t)nV, st));
    MTK_TRY(dF.upload(F, ns, st));
    MTK_TRY(dkeys.alloc(nslot));
    MTK_TRY(ds0.alloc(nslot));
    MTK_TRY(ds1.alloc(nslot));
    MTK_TRY(dpart.alloc(ns));
    MTK_TRY(dfarg.alloc(ns));
    MTK_TRY(darea.alloc(nF));
    MTK_TRY(dnbr.alloc(ns));
    MTK_TRY(dtheta.alloc(ns));
    MTK_CUDA_TRY(cudaMemsetAsync(dkeys.p, 0xff, sizeof(unsigned long long) * nslot, st));
    MTK_CUDA_TRY(cudaMemsetAsync(ds0.p, 0xff, sizeof(int) * nslot, st));
    MTK_CUDA_TRY(cudaMemsetAsync(ds1.p, 0xff, sizeof(int) * nslot, st));
    MTK_CUDA_TRY(cudaMemsetAsync(dpart.p, 0xff, sizeof(int) * ns, st));
    MTK_CUDA_TRY(cudaMemsetAsync(c->dev_err, 0, sizeof(int), st));
    const int G = stream_grid(c) * 4;
    sides_insert<<<G, kStream, 0, st>>>(nF, dF.p, (unsigned long long)(nslot - 1), dkeys.p, ds0.p, ds1.p, c->dev_err);
    sides_pair<<<G, kStream, 0, st>>>((unsigned long long)nslot, dF.p, dkeys.p, ds0.p, ds1.p, dpart.p, c->dev_err);
    face_angles<<<G, kStream, 0, st>>>(nF, dV.p, dF.p, dfarg.p, darea.p);
    MTK_CUDA_TRY(cudaMemcpyAsync(c->h_int, c->dev_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    MTK_CUDA_TRY(cudaStreamSynchronize(st));
    c->kernels += 3;
    if (const int e = c->h_int[0]) {
        mtk_set_last_error(e & 1   ? "mtk_mesh_field_inputs: non-manifold edge (three or more faces)"
                           : e & 4 ? "mtk_mesh_field_inputs: inconsistently oriented faces"
                                   : "mtk_mesh_field_inputs: degenerate face side",
                           __FILE__, __LINE__);
        return MTK_ERR_BAD_INPUT;
    }
    side_outputs<<<G, kStream, 0, st>>>(nF, dpart.p, dfarg.p, dnbr.p, dtheta.p);
    c->kernels++;
    MTK_CUDA_TRY(cudaGetLastError());
    MTK_CUDA_TRY(cudaMemcpyAsync(nbr, dnbr.p, sizeof(int) * ns, cudaMemcpyDeviceToHost, st));
    MTK_CUDA_TRY(cudaMemcpyAsync(theta, dtheta.p, sizeof(double) * ns, cudaMemcpyDeviceToHost, st));
    MTK_CUDA_TRY(cudaMemcpyAsync(area, darea.p, sizeof(double) * nF, cudaMemcpyDeviceToHost, st));
    MTK_CUDA_TRY(cudaStreamSynchronize(st));
    return MTK_OK;
}

extern "C" int mtk_field_smoothest_mesh(mtk_ctx* c, int32_t nV, int32_t nF, const double* V, const int32_t* F,
                                        int32_t nRosy, const double* x0, int32_t n_iter, const mtk_solve_opts* opts,
                                        double* out, mtk_stats* stats) {
    if (!c || nF <= 0 || !x0 || !out) return MTK_ERR_BAD_INPUT;
    std::vector<int32_t> nbr(3 * (size_t)nF);
    std::vector<double> theta(3 * (size_t)nF), area(nF);
    MTK_TRY(mtk_mesh_field_inputs(c, nV, nF, V, F, nbr.data(), theta.data(), area.data()));
    return mtk_field_smoothest(c, nF, nRosy, nbr.data(), theta.data(), area.data(), x0, n_iter, opts, out, stats);
}

extern "C" int mtk_curl_matching(mtk_ctx* c, int32_t nV, int32_t nF, int32_t nE, int32_t N, const double* V,
                                 const int32_t* F, const int32_t* edge_vert, const int32_t* edge_face,
                                 const int32_t* vert_half, const int32_t* prev_half, const int32_t* twin_half,
                                 const int32_t* half_edge, const int32_t* edge_half, const double* angle_defect,
                                 const double* compressed, int32_t* matching, int32_t* singular) {
    if (!c || nV <= 0 || nF <= 0 || nE <= 0 || N < 1 || N > 8 || !V || !F || !edge_vert || !edge_face || !vert_half ||
        !prev_half || !angle_defect || !compressed || !matching || !singular)
        return MTK_ERR_BAD_INPUT;
    const int64_t nH = 2 * (int64_t)nE;
    auto bad = [](const char* what) {
        mtk_set_last_error(what, __FILE__, __LINE__);
        return MTK_ERR_BAD_INPUT;
    };
    const bool general = twin_half != nullptr;
    if (general != (half_edge != nullptr) || general != (edge_half != nullptr))
        return bad("mtk_curl_matching: twin_half, half_edge and edge_half are given together or not at all");
    if (3 * (int64_t)nF > nH) return bad("mtk_curl_matching: more face corners than halfedges");
    for (int64_t i = 0; i < 3 * (int64_t)nF; i++)
        if (F[i] < 0 || F[i] >= nV) return bad("mtk_curl_matching: face corner out of range");
    for (int64_t i = 0; i < nH; i++) {
        if (edge_vert[i] < 0 || edge_vert[i] >= nV) return bad("mtk_curl_matching: edge vertex out of range");
        if (edge_face[i] < -1 || edge_face[i] >= nF || (!general && edge_face[i] < 0))
            return bad("mtk_curl_matching: edge face out of range (-1 on a boundary edge needs the halfedge arrays)");
        if (prev_half[i] < 0 || prev_half[i] >= nH) return bad("mtk_curl_matching: prev halfedge out of range");
        if (general && (twin_half[i] < 0 || twin_half[i] >= nH || half_edge[i] < 0 || half_edge[i] >= nE))
            return bad("mtk_curl_matching: twin or edge of a halfedge out of range");
    }
    if (general)
        for (int i = 0; i < nE; i++)
            if (edge_half[i] < 0 || edge_half[i] >= nH) return bad("mtk_curl_matching: edge halfedge out of range");
    for (int i = 0; i < nV; i++)
        if (vert_half[i] < 0 || vert_half[i] >= nH) return bad("mtk_curl_matching: vertex halfedge out of range");
    MTK_CUDA_TRY(cudaSetDevice(c->device));
    AllocStreamScope alloc_scope(c->stream);
    cudaStream_t st = c->stream;
    DBuf<double> dV, dc, ddef, deff;
    DBuf<int> dF, dev, def, dvh, dprev, dm, ds, dtwin, dhe, de2h;
    if (general) {
        MTK_TRY(dtwin.upload(twin_half, (size_t)nH, st));
        MTK_TRY(dhe.upload(half_edge, (size_t)nH, st));
        MTK_TRY(de2h.upload(edge_half, (size_t)nE, st));
    }
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
    singular_index<<<G, kStream, 0, st>>>(nV, N, 3 * nF, dvh.p, dprev.p, general ? dtwin.p : nullptr,
                                          general ? dhe.p : nullptr, general ? de2h.p : nullptr, ddef.p, deff.p, ds.p,
                                          c->dev_err);
    c->kernels += 2;
    MTK_CUDA_TRY(cudaGetLastError());
    MTK_CUDA_TRY(cudaMemcpyAsync(matching, dm.p, sizeof(int) * nE, cudaMemcpyDeviceToHost, st));
    MTK_CUDA_TRY(cudaMemcpyAsync(singular, ds.p, sizeof(int) * nV, cudaMemcpyDeviceToHost, st));
    MTK_CUDA_TRY(cudaMemcpyAsync(c->h_int, c->dev_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    MTK_CUDA_TRY(cudaStreamSynchronize(st));
    if (c->h_int[0]) return bad("mtk_curl_matching: a vertex ring does not close");
    return MTK_OK;
}
