//
// Restates parts of metriko (https://github.com/komietty/metriko),
// Copyright (C) 2025 Saki Komikado <komietty@gmail.com>.
// This Source Code Form is subject to the terms of the Mozilla Public License v.2.0
// (https://mozilla.org/MPL/2.0/).
//
// metriko-gb300: seamless parameterization front-end (RosyParameterization).
//
// Replaces metriko include/metriko/core/igm/parameterization.h:11-152,
// parameterization_setup.ipp:3-170 and parameterization_integ.ipp:3-120.
//  * setup() is host code with the reference's control flow: transition ids along the seam,
//    per-halfedge matchings, the vertex+transition -> cut-vertex map (vtrans2cut), the
//    constraints of non-trivial permutation cycles, uncompress (sign symmetry), fixed,
//    integer and singular index sets.
//  * integ() reduces the constraints (matrix_ops.h), builds UFull's kernel block, the target
//    field and the grid length, and runs naive integration + seamless LM + greedy rounding on
//    the GPU (mtk_iterative_rounding), then forms nfn and cfn.  With localInjectivity, the naive
//    integration runs on the GPU and the damped LM path with the injective barrier
//    (li::iterative_rounding, iterative_rounding/local_injectivity.h) runs on the host, its
//    linear solves by the device FP64 PCG (mtk_csr_pcg) and its orientation checks by
//    mtk_local_injectivity.
// The cut mesh is a lightweight CutMesh (positions + faces): integ() only uses its indices and
// per-face geometry, which equals the raw mesh's.
//
#ifndef METRIKO_PARAMETERIZATION_H
#define METRIKO_PARAMETERIZATION_H
#include <chrono>
#include <cmath>
#include <future>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <memory>
#include <set>

#include "metriko/core/hmesh/hmesh.h"
#include "metriko/core/igm/iterative_rounding/iter_rounding.h"
#include "metriko/core/igm/iterative_rounding/local_injectivity.h"
#include "metriko/core/solver/matrix_ops.h"

namespace metriko {
    struct CutMesh {
        int nV = 0, nF = 0;
        MatXd pos;
        MatXi idx;
    };

    // First halfedge in cw order from v.half() on a boundary edge (parameterization.h:82,136), or
    // on a seam edge (:81,137); v.half() when there is none.
    inline int first_cw_half(const Hmesh& m, int v, const std::vector<bool>* seam) {
        const int h0 = m.vert2half[v];
        int h = h0;
        do {
            if (seam ? bool((*seam)[m.edge[h]]) : m.isBE[m.edge[h]] != 0) return h;
            h = m.next[m.twin[h]];
        } while (h != h0);
        return h0;
    }

    // parameterization.h:126-152: duplicate every vertex once per seam sector.  A boundary vertex
    // starts at its first boundary-edge halfedge and skips its boundary halfedge.
    inline std::unique_ptr<CutMesh> compute_cut_mesh(const Hmesh& m, const std::vector<bool>& seam) {
        auto cm = std::make_unique<CutMesh>();
        cm->nF = m.nF;
        cm->idx = MatXi(m.nF, 3, -1);
        // copies are numbered vertex by vertex in ascending order, so the count pass, a prefix
        // sum and an assignment pass (both parallel over vertices) give the serial numbering
        std::vector<int> bgn(m.nV), base(m.nV + 1, 0);
        METRIKO_PARALLEL_FOR
        for (int v = 0; v < m.nV; v++) {
            const int b = first_cw_half(m, v, m.isBV[v] ? nullptr : &seam);
            bgn[v] = b;
            int cnt = 0, h = b;
            do {
                if (m.face[h] >= 0 && (seam[m.edge[h]] || h == b)) cnt++;
                h = m.twin[m.prev[h]];
            } while (h != b);
            base[v + 1] = cnt;
        }
        for (int v = 0; v < m.nV; v++) base[v + 1] += base[v];
        cm->nV = base[m.nV];
        cm->pos = MatXd(cm->nV, 3);
        METRIKO_PARALLEL_FOR
        for (int v = 0; v < m.nV; v++) {
            int c = base[v] - 1, h = bgn[v];
            do {
                if (m.face[h] < 0) { h = m.twin[m.prev[h]]; continue; }
                if (seam[m.edge[h]] || h == bgn[v]) {
                    c++;
                    for (int k = 0; k < 3; k++) cm->pos(c, k) = m.pos(v, k);
                }
                const int f = m.face[h];
                for (int j = 0; j < 3; j++) if (m.idx(f, j) == v) cm->idx(f, j) = c;
                h = m.twin[m.prev[h]];
            } while (h != bgn[v]);
        }
        return cm;
    }

    // Host products of integ() handed to the device (mtk_igm_desc points into these buffers).
    struct IntegSystem {
        SprsD fullx2Nfunc;
        std::vector<int> uniqueJ, full2y, w_ptr, w_idx;
        std::vector<double> F2, w_val, cutV;
        MatXd USmall;
        double length = 0;
        mtk_igm_desc desc{};
    };

    class RosyParameterization {
        const Hmesh& raw;
        const CutMesh& cut;
        const MatXd& ext;
        const VecXi& singlars;
        const VecXi& matching;
        const std::vector<bool>& seam;
        double gridscale;
        int nT = 0;     // transitions
        int nR = 0;     // raw vertices + transitions
        int nS = 0;     // inner singular vertices
    public:
        int N = 4;
        int n = 2;
        SprsD vtrans2cut;
        SprsD constraint;
        SprsD uncompress;
        VecXi he2matching;
        VecXi he2transidx;
        VecXi integerIdcs;
        VecXi singularIdcs;
        VecXi fixedIdcs;
        VecXd fixedVals;
        MatXi lreductor;
        VecXd fullx;
        VecXd naivex;        // naive Poisson solution (ni.x0), for diagnostics
        MatXd nfn;
        MatXd cfn;
        double deviation = 0;   // map_deviation of the result (computed by integ())
        // When set (nF x 3N doubles, row-major), integ() writes the corner values there instead
        // of into cfn, which then stays empty: a caller's output buffer, filled without a copy
        double* cfn_target = nullptr;
        std::vector<int> fixOrder, fixVals;   // greedy rounding order (diagnostics)
        bool verbose = false;
        bool seamless = false;
        bool roundSeams = true;
        bool localInjectivity = false;
        int nJ = 0, nZ = 0;  // constrained block / kernel dimension (diagnostics)

        RosyParameterization(const Hmesh& raw_, const CutMesh& cut_, const MatXd& ext_, const VecXi& sing_,
                             const VecXi& matching_, const std::vector<bool>& seam_, const int degree,
                             const double ratio = 0.02)
            : raw(raw_), cut(cut_), ext(ext_), singlars(sing_), matching(matching_), seam(seam_), gridscale(ratio) {
            N = degree;
            if (N % 2 != 0) throw std::invalid_argument("odd N is not supported (N = 4 and other even N only)");
            n = N / 2;
            lreductor = MatXi(N, n, 0);
            for (int i = 0; i < n; i++) { lreductor(i, i) = 1; lreductor(n + i, i) = -1; }
            fixedVals = VecXd::Zero(n);
            compute_he2transidx();
            compute_he2matching();
            nR = raw.nV + nT;
            nS = 0;
            for (int v = 0; v < raw.nV; v++) nS += is_inside_singular(v);
        }

        int numTransitions() const { return nT; }
        int numSingular() const { return nS; }

        void setup();
        void build_system(IntegSystem& sys);   // host part of integ()
        // The reduced system of the localInjectivity path (li::System: G = G2 fullx2Nfunc UFull,
        // F2, length, the index sets), from build_system's products; host only.
        void li_system(const IntegSystem& sys, li::System& s) const;
        // x (full variables) -> the reduced coordinates [y ; z] of UFull (z by least squares on the
        // constrained block: USmall has full column rank)
        std::vector<double> to_reduced(const IntegSystem& sys, const li::System& s, const VecXd& x) const;
        void build_target(IntegSystem& sys) const;   // F2, length, cutV of build_system
        // Size-field gradient of the naive integration (mtk_size_field_gradient); no counterpart
        // in the reference.  s: log-size per raw vertex; T: per-face loss target (8 per face) or
        // nullptr for the integration target.  Fills fullx with x(s).
        double size_field_gradient(const VecXd& s, const VecXd* T, double mu, VecXd& grad_s);
        // The same loss with the integration target, plus its partial derivatives at fixed x
        // (mtk_size_field_position_partials): per face the G2 entries (dgx, dgy: 3 per face), the
        // field angle (dphi), and the grid length (*dlength, *length_out = the grid length).
        double size_field_position_partials(const VecXd& s, double mu, VecXd& grad_s, std::vector<double>& dgx,
                                            std::vector<double>& dgy, std::vector<double>& dphi, double* dlength,
                                            double* length_out);
        bool integ();

    private:
        // parameterization.h:80-82
        bool is_inside_singular(int v) const { return !raw.isBV[v] && singlars[v] != 0; }
        int first_seam_he(int v) const { return first_cw_half(raw, v, &seam); }
        int first_bndr_he(int v) const { return first_cw_half(raw, v, nullptr); }

        // parameterization_setup.ipp:3-9
        void compute_he2matching() {
            he2matching = VecXi(raw.nH);
            for (int h = 0; h < raw.nH; h++) {
                int m = (raw.edge2half[raw.edge[h]] == h ? -1 : 1) * matching[raw.edge[h]];
                he2matching[h] = m < 0 ? (N + m % N) % N : m % N;
            }
        }

        // parameterization_setup.ipp:11-50
        void compute_he2transidx() {
            he2transidx = VecXi(raw.nH, 32767);
            std::vector<int> valence(raw.nV, 0);
            std::vector<char> claimed(raw.nE, 0);
            for (int e = 0; e < raw.nE; e++)
                if (seam[e]) { valence[raw.edge2vert(e, 0)]++; valence[raw.edge2vert(e, 1)]++; }
            int tid = 1;
            for (int v = 0; v < raw.nV; v++) {
                if ((valence[v] == 2 && !is_inside_singular(v)) || valence[v] == 0) continue;
                int h0 = first_bndr_he(v), cH = h0;
                do {
                    int cE = raw.edge[cH];
                    if (!raw.isBE[cE] && seam[cE] && !claimed[cE]) {
                        he2transidx[cH] = tid;
                        he2transidx[raw.twin[cH]] = -tid;
                        claimed[cE] = 1;
                        int jv = raw.head[cH];
                        // traces the seam until a singular or boundary vertex
                        while (valence[jv] == 2 && !is_inside_singular(jv) && !raw.isBV[jv]) {
                            int nh = -1, g0 = raw.vert2half[jv], g = g0;
                            do {
                                if (seam[raw.edge[g]] && !claimed[raw.edge[g]]) { nh = g; break; }
                                g = raw.twin[raw.prev[g]];
                            } while (g != g0);
                            if (nh < 0) throw std::runtime_error("seam tracing failed");
                            he2transidx[nh] = tid;
                            he2transidx[raw.twin[nh]] = -tid;
                            claimed[raw.edge[nh]] = 1;
                            jv = raw.head[nh];
                        }
                        tid++;
                    }
                    cH = raw.twin[raw.prev[cH]];
                } while (cH != h0);
            }
            nT = tid - 1;
        }
    };

    inline void RosyParameterization::setup() {
        // cyclic permutation group (setup.ipp:55-61)
        std::vector<MatXi> perms(N);
        MatXi unit = MatXi::Zero(N, N);
        for (int i = 0; i < N; i++) unit((i + 1) % N, i) = 1;
        perms[0] = MatXi::Identity(N, N);
        for (int i = 1; i < N; i++) perms[i] = unit * perms[i - 1];
        const MatXi I = MatXi::Identity(N, N);
        std::vector<TripD> vT, cT;
        auto block = [&](std::vector<TripD>& T, const MatXi& mat, int r0, int c0) {
            for (int i = 0; i < mat.rows(); i++)
                for (int j = 0; j < mat.cols(); j++)
                    if (mat(i, j) != 0) T.emplace_back(r0 + i, c0 + j, double(mat(i, j)));
        };
        int currConstraint = 0;
        // vertices away from the seam: one cut copy, identity block, no constraint (found in
        // parallel; their rows of vtrans2cut are written directly below)
        std::vector<int> plainCut(raw.nV, -1);
        METRIKO_PARALLEL_FOR
        for (int v = 0; v < raw.nV; v++) {
            if (raw.isBV[v]) continue;
            const int g0 = raw.vert2half[v];
            int g = g0;
            bool onSeam = false;
            do {
                if (seam[raw.edge[g]]) { onSeam = true; break; }
                g = raw.twin[raw.prev[g]];
            } while (g != g0);
            if (onSeam) continue;
            const int f = raw.face[g0];
            for (int j = 0; j < 3; j++) if (raw.idx(f, j) == v) plainCut[v] = cut.idx(f, j);
        }
        for (int v = 0; v < raw.nV; v++) {       // setup.ipp:66-124, vertices on the seam or boundary
            if (plainCut[v] >= 0) continue;
            const bool bv = raw.isBV[v];
            std::vector<MatXi> pm{I};
            std::vector<int> pidx{v};
            int iVcut = -1;
            const int h0 = bv ? first_bndr_he(v) : first_seam_he(v);
            int h = h0;
            do {
                if (raw.face[h] < 0) break;   // the boundary halfedge ends the fan (setup.ipp:77)
                int f = raw.face[h];
                int jVcut = -1;
                for (int j = 0; j < 3; j++) if (raw.idx(f, j) == v) jVcut = cut.idx(f, j);
                if (jVcut != iVcut) {
                    iVcut = jVcut;
                    for (size_t i = 0; i < pidx.size(); i++) block(vT, pm[i], N * iVcut, N * pidx[i]);
                }
                int hn = raw.twin[raw.prev[h]];
                if (raw.face[hn] >= 0 && seam[raw.edge[hn]]) {
                    const MatXi& p = perms[he2matching[hn]];
                    int t = he2transidx[hn];
                    if (t > 0) {
                        for (auto& mm : pm) mm = p * mm;
                        pm.push_back(I);
                        pidx.push_back(raw.nV + t - 1);
                    } else {
                        pm.push_back(-I);
                        pidx.push_back(raw.nV - t - 1);
                        for (auto& mm : pm) mm = p * mm;
                    }
                }
                h = hn;
            } while (h != h0);
            if (bv) continue;                  // no constraint on a boundary vertex (setup.ipp:105)
            std::set<int> uniq(pidx.begin(), pidx.end());
            std::vector<int> idcs(uniq.begin(), uniq.end());
            std::vector<MatXi> mats(idcs.size());
            bool any = false;
            for (size_t j = 0; j < idcs.size(); j++) {
                mats[j] = MatXi::Zero(N, N);
                for (size_t k = 0; k < pidx.size(); k++) if (idcs[j] == pidx[k]) mats[j] += pm[k];
                if (idcs[j] == v) mats[j] -= I;
                if (!mats[j].isZero()) any = true;
            }
            if (any) {
                for (size_t j = 0; j < mats.size(); j++) block(cT, mats[j], N * currConstraint, N * idcs[j]);
                currConstraint++;
            }
        }
        {   // vtrans2cut: seam rows from their triplets (summed, pruned), the other rows one 1 each
            SprsD seamRows(N * cut.nV, N * nR);
            seamRows.setFromTriplets(vT.begin(), vT.end());
            seamRows.prune(1e-3);
            std::vector<int> plainRow(N * (size_t)cut.nV, -1);   // row -> column of its single 1
            METRIKO_PARALLEL_FOR
            for (int v = 0; v < raw.nV; v++)
                if (plainCut[v] >= 0)
                    for (int i = 0; i < N; i++) plainRow[(size_t)N * plainCut[v] + i] = N * v + i;
            const int rows = N * cut.nV;
            vtrans2cut = SprsD(rows, N * nR);
            std::vector<int>& vp = vtrans2cut.ptr;
            for (int r = 0; r < rows; r++)
                vp[r + 1] = vp[r] + (plainRow[r] >= 0 ? 1 : seamRows.ptr[r + 1] - seamRows.ptr[r]);
            vtrans2cut.idx.resize(vp[rows]);
            vtrans2cut.val.resize(vp[rows]);
            METRIKO_PARALLEL_FOR
            for (int r = 0; r < rows; r++) {
                int o = vp[r];
                if (plainRow[r] >= 0) { vtrans2cut.idx[o] = plainRow[r]; vtrans2cut.val[o] = 1.0; continue; }
                for (int q = seamRows.ptr[r]; q < seamRows.ptr[r + 1]; q++, o++) {
                    vtrans2cut.idx[o] = seamRows.idx[q];
                    vtrans2cut.val[o] = seamRows.val[q];
                }
            }
        }
        constraint = SprsD(N * currConstraint, N * nR);
        constraint.setFromTriplets(cT.begin(), cT.end());
        constraint.prune(1e-3);
        {   // uncompress: block-diagonal copies of lreductor (at most one entry per row)
            uncompress = SprsD(N * nR, n * nR);
            std::vector<int> rc(N), rv(N);
            for (int a = 0; a < N; a++) {
                rc[a] = -1;
                for (int b2 = 0; b2 < n; b2++)
                    if (lreductor(a, b2) != 0) {
                        if (rc[a] >= 0) throw std::runtime_error("lreductor row with two entries");
                        rc[a] = b2;
                        rv[a] = lreductor(a, b2);
                    }
            }
            std::vector<int>& up = uncompress.ptr;
            for (int i = 0; i < N * nR; i++) up[i + 1] = up[i] + (rc[i % N] >= 0 ? 1 : 0);
            uncompress.idx.resize(up[N * nR]);
            uncompress.val.resize(up[N * nR]);
            METRIKO_PARALLEL_FOR
            for (int i = 0; i < N * nR; i++) {
                const int a = i % N;
                if (rc[a] < 0) continue;
                uncompress.idx[up[i]] = (i - a) * n / N + rc[a];
                uncompress.val[up[i]] = double(rv[a]);
            }
        }

        fixedIdcs = VecXi(n);
        if (nS == 0) {
            for (int j = 0; j < n; j++) fixedIdcs[j] = j;
        } else {
            int iV = 0;
            for (iV = 0; iV < raw.nV; iV++) if (is_inside_singular(iV)) break;
            for (int j = 0; j < n; j++) fixedIdcs[j] = n * iV + j;
        }
        integerIdcs = VecXi(nT * n);
        for (int i = 0; i < nT; i++) for (int j = 0; j < n; j++) integerIdcs[n * i + j] = n * (raw.nV + i) + j;
        singularIdcs = VecXi(n * nS);
        int c = 0;
        for (int v = 0; v < raw.nV; v++)
            if (is_inside_singular(v)) for (int j = 0; j < n; j++) singularIdcs[c++] = n * v + j;
    }

    // The check at the end of the reference's integ() (parameterization_integ.ipp:100-117): on
    // every face the 3D gradient of each of the N functions -- the corner hat-function gradients
    // n x (next(h) vector) / (2 area) of G3 (:11-27), corners in the order of the face's
    // halfedges, F(f,0), F(f,1), F(f,2) -- against the extrinsic field; returns the mean over
    // faces and functions of |normalized(ext_k) - normalized(grad_k)|.  cfn: nF x 3N, the value
    // of function k at corner j in column N j + k.  Per-face sums in parallel, their total in
    // face order.
    inline double map_deviation(const MatXd& cutV, const MatXi& cutF, const double* cfn, const MatXd& ext, int N) {
        const int nF = cutF.rows();
        if (nF == 0 || N <= 0) return 0;
        std::vector<double> part(nF);
        METRIKO_PARALLEL_FOR
        for (int f = 0; f < nF; f++) {
            const Row3d p[3] = {row3(cutV, cutF(f, 0)), row3(cutV, cutF(f, 1)), row3(cutV, cutF(f, 2))};
            const Row3d n = (p[1] - p[0]).cross(p[2] - p[0]);
            const double a2 = n.norm();
            const Row3d nu = n.normalized();
            Row3d g[3];
            for (int j = 0; j < 3; j++) g[j] = nu.cross(p[(j + 2) % 3] - p[(j + 1) % 3]) / a2;
            double s = 0;
            for (int k = 0; k < N; k++) {
                const double* c = cfn + 3 * size_t(N) * f;
                Row3d grad = g[0] * c[k];
                grad = grad + g[1] * c[N + k];
                grad = grad + g[2] * c[2 * N + k];
                const Row3d e{ext(f, 3 * k), ext(f, 3 * k + 1), ext(f, 3 * k + 2)};
                s += (e.normalized() - grad.normalized()).norm();
            }
            part[f] = s;
        }
        double sum = 0;
        for (double v : part) sum += v;
        return sum / (double(nF) * N);
    }
    inline double map_deviation(const MatXd& cutV, const MatXi& cutF, const MatXd& cfn, const MatXd& ext, int N) {
        return map_deviation(cutV, cutF, cfn.data(), ext, N);
    }

    inline void RosyParameterization::build_system(IntegSystem& sys) {
        // The target field, the grid length and the cut-vertex copy read only the cut mesh and
        // the extrinsic field: computed on a host thread while the sparse products run.
        auto target = std::async(std::launch::async, [this, &sys] { build_target(sys); });
        SprsD& fullx2Nfunc = sys.fullx2Nfunc;
        fullx2Nfunc = vtrans2cut * uncompress;
        SprsD Cfull = constraint * uncompress;     // structural zeros kept (Eigen product semantics)
        reduce_to_linearly_independent(Cfull);
        const int nFull = n * nR;

        // ---- UFull = permutation * blockdiag(I, kernel(CSmall))  (iter_rounding_init.h:98-154)
        std::vector<int>& uniqueJ = sys.uniqueJ;
        uniqueJ.clear();
        {
            std::vector<char> used(nFull, 0);
            for (int p = 0; p < Cfull.nonZeros(); p++) used[Cfull.idx[p]] = 1;
            for (int i = 0; i < nFull; i++) if (used[i]) uniqueJ.push_back(i);
        }
        std::vector<int>& full2y = sys.full2y;
        full2y.assign(nFull, -1);
        MatXd& USmall = sys.USmall;
        USmall = MatXd();
        if (Cfull.rows() == 0) {
            uniqueJ.clear();
            for (int i = 0; i < nFull; i++) full2y[i] = i;
        } else {
            std::vector<int> slot(nFull, -1);
            for (size_t s = 0; s < uniqueJ.size(); s++) slot[uniqueJ[s]] = int(s);
            MatXd CSmall(Cfull.rows(), int(uniqueJ.size()), 0.0);
            for (int i = 0; i < Cfull.rows(); i++)
                for (int p = Cfull.ptr[i]; p < Cfull.ptr[i + 1]; p++) CSmall(i, slot[Cfull.idx[p]]) = Cfull.val[p];
            USmall = fullpiv_kernel(CSmall);
            int y = 0;
            for (int i = 0; i < nFull; i++) if (slot[i] < 0) full2y[i] = y++;
        }
        nJ = int(uniqueJ.size());
        nZ = USmall.cols();

        // ---- W = rows k < n of fullx2Nfunc (rows k >= n are their negatives)
        std::vector<int>& w_ptr = sys.w_ptr;
        std::vector<int>& w_idx = sys.w_idx;
        std::vector<double>& w_val = sys.w_val;
        w_ptr.assign(n * size_t(cut.nV) + 1, 0);
        w_idx.clear();
        w_val.clear();
        for (int c = 0; c < cut.nV; c++)
            for (int k = 0; k < n; k++) {
                int r = N * c + k;
                for (int p = fullx2Nfunc.ptr[r]; p < fullx2Nfunc.ptr[r + 1]; p++) {
                    if (fullx2Nfunc.val[p] == 0) continue;
                    w_idx.push_back(fullx2Nfunc.idx[p]);
                    w_val.push_back(fullx2Nfunc.val[p]);
                }
                w_ptr[n * c + k + 1] = int(w_idx.size());
            }
        target.get();

        mtk_igm_desc& d = sys.desc;
        d = mtk_igm_desc{};
        d.nF = cut.nF; d.nCut = cut.nV; d.N = N; d.n = n;
        d.cutF = cut.idx.data(); d.cutV = sys.cutV.data();
        d.w_ptr = w_ptr.data(); d.w_idx = w_idx.data(); d.w_val = w_val.data();
        d.nFull = nFull; d.full2y = full2y.data();
        d.nJ = nJ; d.nZ = nZ; d.uniqueJ = uniqueJ.data(); d.USmall = USmall.data();
        d.F2 = sys.F2.data(); d.length = sys.length;
        d.nFixed = fixedIdcs.size(); d.fixedIdcs = fixedIdcs.data(); d.fixedVals = fixedVals.data();
        d.nSingular = singularIdcs.size(); d.singularIdcs = singularIdcs.data();
        d.nInteger = integerIdcs.size(); d.integerIdcs = integerIdcs.data();
        d.seamless = seamless; d.roundSeams = roundSeams;
    }

    inline void RosyParameterization::li_system(const IntegSystem& sys, li::System& s) const {
        s.N = N;
        s.n = n;
        s.nF = cut.nF;
        s.nCut = cut.nV;
        s.nfull = n * nR;
        s.nZ = int(sys.USmall.cols());
        s.nY = 0;
        for (int v : sys.full2y) s.nY = std::max(s.nY, v + 1);
        s.nred = s.nY + s.nZ;
        s.length = sys.length;
        s.F2 = sys.F2;
        s.full2y = sys.full2y;
        s.jslot.assign(s.nfull, -1);
        for (size_t k = 0; k < sys.uniqueJ.size(); k++) s.jslot[sys.uniqueJ[k]] = int(k);
        s.USmall = sys.USmall;
        s.fullx2N = &sys.fullx2Nfunc;
        s.cutF = cut.idx;
        s.fixedIdcs.assign(fixedIdcs.begin(), fixedIdcs.end());
        s.fixedVals.assign(fixedVals.begin(), fixedVals.end());
        s.singularIdcs.assign(singularIdcs.begin(), singularIdcs.end());
        s.integerIdcs.assign(integerIdcs.begin(), integerIdcs.end());
        s.roundSeams = roundSeams;
        li::build_gradients(s, cut.pos, raw.faceNormal, raw.faceBasisX, raw.faceBasisY, raw.faceArea);
    }

    inline std::vector<double> RosyParameterization::to_reduced(const IntegSystem& sys, const li::System& s,
                                                                const VecXd& x) const {
        std::vector<double> xs(s.nred, 0.0);
        for (int i = 0; i < s.nfull; i++) if (s.full2y[i] >= 0) xs[s.full2y[i]] = x[i];
        const int nJ = int(sys.uniqueJ.size()), nZ = s.nZ;
        if (nZ == 0) return xs;
        // normal equations of USmall z = x_J (nZ x nZ, Cholesky)
        MatXd A(nZ, nZ, 0.0);
        std::vector<double> b(nZ, 0.0);
        for (int r = 0; r < nJ; r++) {
            const double xj = x[sys.uniqueJ[r]];
            for (int a = 0; a < nZ; a++) {
                b[a] += sys.USmall(r, a) * xj;
                for (int c = 0; c < nZ; c++) A(a, c) += sys.USmall(r, a) * sys.USmall(r, c);
            }
        }
        for (int j = 0; j < nZ; j++) {
            double d = A(j, j);
            for (int k = 0; k < j; k++) d -= A(j, k) * A(j, k);
            d = std::sqrt(d);
            A(j, j) = d;
            for (int i = j + 1; i < nZ; i++) {
                double v = A(i, j);
                for (int k = 0; k < j; k++) v -= A(i, k) * A(j, k);
                A(i, j) = v / d;
            }
        }
        for (int i = 0; i < nZ; i++) {
            double v = b[i];
            for (int k = 0; k < i; k++) v -= A(i, k) * b[k];
            b[i] = v / A(i, i);
        }
        for (int i = nZ - 1; i >= 0; i--) {
            double v = b[i];
            for (int k = i + 1; k < nZ; k++) v -= A(k, i) * b[k];
            b[i] = v / A(i, i);
        }
        for (int z = 0; z < nZ; z++) xs[s.nY + z] = b[z];
        return xs;
    }

    inline void RosyParameterization::build_target(IntegSystem& sys) const {
        // ---- target field (integ.ipp:30-43) and grid length (:70)
        // the per-vector lengths in parallel, their sum in the serial order
        std::vector<double> vlen(size_t(N) * cut.nF);
        METRIKO_PARALLEL_FOR
        for (int f = 0; f < cut.nF; f++)
            for (int j = 0; j < N; j++) {
                double s = 0;
                for (int k = 0; k < 3; k++) s += ext(f, 3 * j + k) * ext(f, 3 * j + k);
                vlen[size_t(N) * f + j] = std::sqrt(s);
            }
        double norm = 0;
        for (double v : vlen) norm += v;
        norm /= double(N) * cut.nF;
        std::vector<double>& F2 = sys.F2;
        F2.assign(2 * size_t(N) * cut.nF, 0.0);
        METRIKO_PARALLEL_FOR
        for (int f = 0; f < cut.nF; f++)
            for (int i = 0; i < N; i++) {
                double sx = 0, sy = 0;
                for (int k = 0; k < 3; k++) {
                    sx += ext(f, 3 * i + k) * raw.faceBasisX(f, k);
                    sy += ext(f, 3 * i + k) * raw.faceBasisY(f, k);
                }
                F2[2 * N * f + 2 * i] = sx;
                F2[2 * N * f + 2 * i + 1] = sy;
            }
        double mn[3] = {1e300, 1e300, 1e300}, mx[3] = {-1e300, -1e300, -1e300};
        for (int i = 0; i < cut.nV; i++)
            for (int k = 0; k < 3; k++) { mn[k] = std::min(mn[k], cut.pos(i, k)); mx[k] = std::max(mx[k], cut.pos(i, k)); }
        double bb = std::sqrt((mx[0] - mn[0]) * (mx[0] - mn[0]) + (mx[1] - mn[1]) * (mx[1] - mn[1]) + (mx[2] - mn[2]) * (mx[2] - mn[2]));
        const double length = bb * gridscale / norm;
        sys.length = length;
        std::vector<double>& cutV = sys.cutV;
        cutV.assign(3 * size_t(cut.nV), 0.0);
        for (int i = 0; i < cut.nV; i++) for (int k = 0; k < 3; k++) cutV[3 * i + k] = cut.pos(i, k);
    }

    inline double RosyParameterization::size_field_gradient(const VecXd& s, const VecXd* T, double mu, VecXd& grad_s) {
        IntegSystem sys;
        build_system(sys);
        if (s.size() != raw.nV || (T && T->size() != 8 * raw.nF)) throw std::invalid_argument("size field: bad sizes");
        grad_s = VecXd(raw.nV);
        fullx = VecXd(sys.desc.nFull);
        double loss = 0;
        gpu::check(mtk_size_field_gradient(gpu::context(), &sys.desc, &gpu::options().solve, raw.nV, raw.idx.data(),
                                           s.data(), T ? T->data() : nullptr, mu, &loss, grad_s.data(), fullx.data(),
                                           &gpu::stats()),
                   "mtk_size_field_gradient");
        return loss;
    }

    inline double RosyParameterization::size_field_position_partials(const VecXd& s, double mu, VecXd& grad_s,
                                                                     std::vector<double>& dgx, std::vector<double>& dgy,
                                                                     std::vector<double>& dphi, double* dlength,
                                                                     double* length_out) {
        IntegSystem sys;
        build_system(sys);
        if (s.size() != raw.nV) throw std::invalid_argument("size field: bad sizes");
        grad_s = VecXd(raw.nV);
        fullx = VecXd(sys.desc.nFull);
        dgx.assign(3 * size_t(raw.nF), 0.0);
        dgy.assign(3 * size_t(raw.nF), 0.0);
        dphi.assign(raw.nF, 0.0);
        double loss = 0;
        gpu::check(mtk_size_field_position_partials(gpu::context(), &sys.desc, &gpu::options().solve, raw.nV,
                                                    raw.idx.data(), s.data(), mu, &loss, grad_s.data(), fullx.data(),
                                                    dgx.data(), dgy.data(), dphi.data(), dlength, &gpu::stats()),
                   "mtk_size_field_position_partials");
        if (length_out) *length_out = sys.length;
        return loss;
    }

    inline bool RosyParameterization::integ() {
        IntegSystem sys;
        auto t0 = std::chrono::steady_clock::now();
        build_system(sys);
        if (getenv("MTK_DEBUG") && getenv("MTK_DEBUG")[0] == '1')
            fprintf(stderr, "[host] %-22s %8.1f ms\n", "integ build_system",
                    std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count());
        const SprsD& fullx2Nfunc = sys.fullx2Nfunc;
        bool success = true;
        if (!localInjectivity) {
            success = iterative_rounding(sys.desc, fullx, naivex, fixOrder, fixVals);
        } else {
            // the naive integration on the device, then the damped LM path (li::iterative_rounding)
            // with its linear solves on the device (mtk_csr_pcg, FP64) and the orientation check
            // of the map by mtk_local_injectivity
            mtk_igm_desc nd = sys.desc;
            nd.seamless = 0;
            std::vector<int> fo, fv;
            VecXd nx;
            iterative_rounding(nd, naivex, nx, fo, fv);
            li::System ls;
            li_system(sys, ls);
            const std::vector<double> xs0 = to_reduced(sys, ls, naivex);
            // The damped LM systems carry squared weights from 1e-4 to 1e10 and, near the barrier,
            // rows that grow without bound: a PCG whose recurrence reaches 1e-13 can leave a true
            // relative residual of up to ~1e-4 there, where the reference factorizes.  So each
            // solve is refined three times in FP64 (the residual b - S x exact on the host, one
            // more PCG for the correction), which brings it to round-off.  A PCG counts as done when it stopped on its own test: NOT_CONVERGED from the final
            // true-residual check only (the stats are written after the PCG's test passed; an
            // exhausted cap returns before them).  A breakdown (the analogue of a failed
            // factorization) or an exhausted cap fails the first pass and ends the refinement.
            li::Solve solve = [](const SprsD& S, const std::vector<double>& b, std::vector<double>& x) {
                mtk_csr* A = nullptr;
                if (mtk_csr_create(gpu::context(), S.nr, S.ptr.data(), S.idx.data(), S.val.data(), 0, &A) != MTK_OK) return false;
                mtk_solve_opts o = gpu::options().solve;
                o.precision = MTK_PREC_FP64;
                o.tol = 1e-13;
                o.max_iter = std::max(o.max_iter, 20 * S.nr + 1000);
                auto pcg = [&](const std::vector<double>& rhs, std::vector<double>& out) {
                    out.assign(S.nr, 0.0);
                    mtk_stats st{};
                    const int s = mtk_csr_pcg(gpu::context(), A, 1, rhs.data(), out.data(), &o, &st);
                    if (s == MTK_OK) return true;
                    if (s != MTK_ERR_NOT_CONVERGED || st.solves == 0 || st.pcg_iters >= o.max_iter) return false;
                    for (double v : out)
                        if (!std::isfinite(v)) return false;
                    return true;
                };
                bool ok = pcg(b, x);
                if (ok) {
                    std::vector<double> r(S.nr), e;
                    for (int k = 0; k < 3; k++) {
                        METRIKO_PARALLEL_FOR
                        for (int i = 0; i < S.nr; i++) {
                            double t = b[i];
                            for (int q = S.ptr[i]; q < S.ptr[i + 1]; q++) t -= S.val[q] * x[S.idx[q]];
                            r[i] = t;
                        }
                        if (!pcg(r, e)) break;
                        for (int i = 0; i < S.nr; i++) x[i] += e[i];
                    }
                }
                mtk_csr_destroy(A);
                return ok;
            };
            auto injective = [this, &ls, &fullx2Nfunc](const std::vector<double>& xs) {
                const std::vector<double> X = ls.ufull_times(xs);
                const std::vector<double> NF = fullx2Nfunc * X;
                std::vector<double> cfn_(12 * size_t(cut.nF));
                for (int f = 0; f < cut.nF; f++)
                    for (int j = 0; j < 3; j++)
                        for (int k = 0; k < N; k++) cfn_[3 * size_t(N) * f + N * j + k] = NF[N * size_t(cut.idx(f, j)) + k];
                int flipped = 0;
                gpu::check(mtk_local_injectivity(gpu::context(), cut.nF, N, cfn_.data(), &flipped, nullptr),
                           "mtk_local_injectivity");
                return flipped == 0;
            };
            li::Result r = li::iterative_rounding(ls, xs0, seamless, solve, injective);
            success = r.success;
            fullx = VecXd(r.fullx);
            fixOrder = r.fixOrder;
            fixVals = r.fixVals;
        }

        // ---- nfn (cut vertex x N) and cfn (face x 3N)  (integ.ipp:88-98)
        std::vector<double> NF = fullx2Nfunc * fullx.d;
        nfn = MatXd(cut.nV, N);
        METRIKO_PARALLEL_FOR
        for (int i = 0; i < cut.nV; i++) for (int k = 0; k < N; k++) nfn(i, k) = NF[N * size_t(i) + k];
        if (!cfn_target) cfn = MatXd(raw.nF, 3 * N);
        double* cf = cfn_target ? cfn_target : cfn.data();
        METRIKO_PARALLEL_FOR
        for (int f = 0; f < raw.nF; f++)
            for (int j = 0; j < 3; j++)
                for (int k = 0; k < N; k++) cf[3 * size_t(N) * f + N * j + k] = NF[N * size_t(cut.idx(f, j)) + k];
        // ---- how close the map's gradients are to the field (integ.ipp:100-117)
        deviation = map_deviation(cut.pos, cut.idx, cf, ext, N);
        if (verbose || (getenv("MTK_DEBUG") && getenv("MTK_DEBUG")[0] == '1'))
            fprintf(stderr, "Deviation of the recovered tf from the original : %.9g\n", deviation);
        return success;
    }
}

#endif
