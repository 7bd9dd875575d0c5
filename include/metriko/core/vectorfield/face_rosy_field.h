//
// Restates parts of metriko (https://github.com/komietty/metriko),
// Copyright (C) 2025 Saki Komikado <komietty@gmail.com>.
// This Source Code Form is subject to the terms of the Mozilla Public License v.2.0
// (https://mozilla.org/MPL/2.0/).
//
// metriko-gb300: face-based N-RoSy field, matching, singularities, seams, combing.
//
// Replaces metriko include/metriko/core/vectorfield/face_rosy_field.h:16-360.
//  * The smoothest field (connectionLaplacian + galerkinMassMatrix + solveSmallestEig, :43-110)
//    is computed on the GPU by mtk_field_smoothest (assembly, PCG inverse iteration).
//  * Matching, singularities, seams, combing and the extrinsic field are host algorithms with
//    integer outputs; they follow the reference's control flow and tie-breaking exactly.
//  * The seam builder restates libigl v2.5.0 cut_mesh_from_singularities (flood fill from
//    face 0, then leaf retraction scanning faces in order, at most 10001 passes) and
//    dijkstra (unit weights, pops ordered by (distance, vertex id)).
//  * The power iteration starts from mtk_seeded_init(nF, options().seed) instead of
//    VecXc::Random.
//
#ifndef METRIKO_FACE_ROSY_FIELD_H
#define METRIKO_FACE_ROSY_FIELD_H
#include <deque>
#include <functional>
#include <memory>
#include <queue>
#include <set>

#include "base_field.h"
#include "metriko/gpu/device.h"

namespace metriko {
    class FaceRosyField : public BaseVectorField {
    public:
        FaceRosyField(const Hmesh& m, const int nRosy) : BaseVectorField(m, nRosy) {}
        FaceRosyField(const Hmesh& m, const int nRosy, FieldType type, const VecXc* start = nullptr)
            : BaseVectorField(m, nRosy) {
            switch (type) {
                case FieldType::Smoothest: compressed = solveSmoothest(start); break;
                case FieldType::CurvatureAligned: compressed = solveCurvatureAligned(); break;
                default: break;
            }
            if (compressed.size() == m.nF) set_field_from_compressed();
        }

        // face_rosy_field.h:37-43: field(f,i) = pow(polar(1, arg c_f), 1/N) * pow(r, i)
        void set_field_from_compressed() {
            const complex r = std::polar(1., TwoPI / rosyN);
            std::vector<complex> rpow(rosyN);   // pow(r, i), the same factor for every face
            for (int i = 0; i < rosyN; i++) rpow[i] = i ? std::exp(double(i) * std::log(r)) : complex(1, 0);
            field = MatXc(mesh.nF, rosyN);
            METRIKO_PARALLEL_FOR
            for (int f = 0; f < mesh.nF; f++) {
                complex root = std::exp(std::log(std::polar(1., std::arg(compressed[f]))) * (1. / rosyN));
                for (int i = 0; i < rosyN; i++) field(f, i) = root * rpow[i];
            }
        }

        // Inputs of the device assembly: neighbour across each face halfedge and
        // theta = farg(h) - farg(twin h); L(f, nbr) = -(-e^{i theta})^N (face_rosy_field.h:52-75).
        // A boundary side has no neighbour (-1, theta 0) and adds nothing to L (:64).
        void assembly_inputs(std::vector<int>& nbr, std::vector<double>& theta) const {
            nbr.resize(3 * size_t(mesh.nF));
            theta.resize(3 * size_t(mesh.nF));
            METRIKO_PARALLEL_FOR
            for (int f = 0; f < mesh.nF; f++)
                for (int j = 0; j < 3; j++) {
                    int h = mesh.face2half3(f, j), t = mesh.twin[h];
                    nbr[3 * f + j] = mesh.face[t];
                    theta[3 * f + j] = mesh.face[t] < 0 ? 0.0 : mesh.heArgOnFace[h] - mesh.heArgOnFace[t];
                }
        }

        VecXc solveSmoothest(const VecXc* start, int nIter = -1) {
            if (nIter < 0) nIter = gpu::options().n_iter;
            std::vector<int> nbr;
            std::vector<double> theta;
            assembly_inputs(nbr, theta);
            std::vector<double> x0(2 * size_t(mesh.nF));
            if (start) {
                if (start->size() != mesh.nF) throw std::invalid_argument("start vector size");
                for (int f = 0; f < mesh.nF; f++) { x0[2 * f] = (*start)[f].real(); x0[2 * f + 1] = (*start)[f].imag(); }
            } else {
                mtk_seeded_init(mesh.nF, gpu::options().seed, x0.data());
            }
            std::vector<double> out(2 * size_t(mesh.nF));
            gpu::check(mtk_field_smoothest(gpu::context(), mesh.nF, rosyN, nbr.data(), theta.data(), mesh.faceArea.data(),
                                           x0.data(), nIter, &gpu::options().solve, out.data(), &gpu::stats()),
                       "mtk_field_smoothest");
            VecXc c(mesh.nF);
            for (int f = 0; f < mesh.nF; f++) c[f] = complex(out[2 * f], out[2 * f + 1]);
            return c;
        }

        // face_rosy_field.h:86-98: D_f = 1/4 sum over the halfedges h of f of
        // -(e^{i farg(h)} |h|)^2 / |h| * dihedral(h), with the dihedral angle of h
        // atan2(v . (n1 x n2), n1 . n2) (v = h / |h|, n1, n2 the normals of h's and twin(h)'s faces,
        // hmesh.h:508-519).
        VecXc principalCurvatureDir() const {
            VecXc D(mesh.nF);
            METRIKO_PARALLEL_FOR
            for (int f = 0; f < mesh.nF; f++) {
                complex dir(0, 0);
                for (int j = 0; j < 3; j++) {
                    const int h = mesh.face2half3(f, j);
                    const Half hh{{h, &mesh}};
                    const Row3d vec = hh.vec();
                    const double l = vec.norm();
                    const int g = mesh.face[mesh.twin[h]];
                    double darg = 0;   // 0 on a boundary edge (hmesh.h:510-513)
                    if (g >= 0) {
                        const Row3d n1 = row3(mesh.faceNormal, f), n2 = row3(mesh.faceNormal, g);
                        darg = std::atan2((vec / l).dot(n1.cross(n2)), n1.dot(n2));
                    }
                    const complex c = std::polar(1., mesh.heArgOnFace[h]) * l;
                    dir += -c * c / l * darg;
                }
                D[f] = dir * 0.25;
            }
            return D;
        }

        // face_rosy_field.h:25-33 (lambda = 0): D (squared for N = 4), rhs = M D / sqrt|D^H M D|,
        // compressed = L^-1 rhs by one device solve (mtk_field_solve).
        VecXc solveCurvatureAligned() {
            if (rosyN != 2 && rosyN != 4) throw std::invalid_argument("CurvatureAligned needs N = 2 or 4");
            VecXc D = principalCurvatureDir();
            if (rosyN == 4) for (int f = 0; f < mesh.nF; f++) D[f] = D[f] * D[f];
            double dmd = 0;
            for (int f = 0; f < mesh.nF; f++) dmd += mesh.faceArea[f] * std::norm(D[f]);
            const double sc = 1.0 / std::sqrt(std::abs(dmd));
            std::vector<double> rhs(2 * size_t(mesh.nF));
            for (int f = 0; f < mesh.nF; f++) {
                const complex v = mesh.faceArea[f] * D[f] * sc;
                rhs[2 * f] = v.real();
                rhs[2 * f + 1] = v.imag();
            }
            std::vector<int> nbr;
            std::vector<double> theta;
            assembly_inputs(nbr, theta);
            std::vector<double> out(2 * size_t(mesh.nF));
            gpu::check(mtk_field_solve(gpu::context(), mesh.nF, rosyN, nbr.data(), theta.data(), mesh.faceArea.data(),
                                       rhs.data(), &gpu::options().solve, out.data(), &gpu::stats()),
                       "mtk_field_solve");
            VecXc c(mesh.nF);
            for (int f = 0; f < mesh.nF; f++) c[f] = complex(out[2 * f], out[2 * f + 1]);
            return c;
        }

        void computeConnection() {      // face_rosy_field.h:109-117 (interior edges; 0 on the boundary)
            connection = VecXc(mesh.nE, complex(0, 0));
            METRIKO_PARALLEL_FOR
            for (int e = 0; e < mesh.nE; e++) {
                if (mesh.isBE[e]) continue;
                Row3d v = Half{{mesh.edge2half[e], &mesh}}.vec().normalized();
                int f0 = mesh.edge2face(e, 0), f1 = mesh.edge2face(e, 1);
                complex ef(v.dot(row3(mesh.faceBasisX, f0)), v.dot(row3(mesh.faceBasisY, f0)));
                complex eg(v.dot(row3(mesh.faceBasisX, f1)), v.dot(row3(mesh.faceBasisY, f1)));
                connection[e] = eg / ef;
            }
        }

        // face_rosy_field.h:100-107: boundary vertices keep the initial 1
        void computeSingular(const VecXd& effort) {
            singular = VecXi(mesh.nV, 1);
            METRIKO_PARALLEL_FOR
            for (int v = 0; v < mesh.nV; v++) {
                if (mesh.isBV[v]) continue;
                double sum = mesh.angleDefect[v] * rosyN;
                int h0 = mesh.vert2half[v], h = h0;
                do {
                    sum += (mesh.edge2half[mesh.edge[h]] == h ? -1 : 1) * effort[mesh.edge[h]];
                    h = mesh.twin[mesh.prev[h]];
                } while (h != h0);
                singular[v] = static_cast<int>(std::round(sum / TwoPI));
            }
        }

        // face_rosy_field.h:119-135.  Inside a device pipeline call (a context bound to the host
        // thread) the Curl matching and the singular indices come from mtk_curl_matching, one
        // thread per edge and per vertex, with the same integer results; `connection` is then left
        // empty (nothing downstream of the matching reads it).
        void computeMatching(const MatchingType type) {
            if (type == MatchingType::Curl && gpu::bound_context() && rosyN <= 8) {
                matching = VecXi(mesh.nE, -1);
                singular = VecXi(mesh.nV, 0);
                connection = VecXc();
                // a closed mesh's halfedges are 2e / 2e + 1, so the twin and edge arrays stay here
                const bool b = mesh.hasBoundary;
                gpu::check(mtk_curl_matching(gpu::bound_context(), mesh.nV, mesh.nF, mesh.nE, rosyN, mesh.pos.data(),
                                             mesh.idx.data(), mesh.edge2vert.data(), mesh.edge2face.data(),
                                             mesh.vert2half.data(), mesh.prev.data(), b ? mesh.twin.data() : nullptr,
                                             b ? mesh.edge.data() : nullptr, b ? mesh.edge2half.data() : nullptr,
                                             mesh.angleDefect.data(), reinterpret_cast<const double*>(compressed.data()),
                                             matching.data(), singular.data()),
                           "mtk_curl_matching");
                return;
            }
            computeConnection();
            matching = VecXi(mesh.nE, -1);
            VecXd effort = VecXd::Zero(mesh.nE);
            if (type == MatchingType::Principal) pMatching(effort);
            else cMatching(effort);
            computeSingular(effort);
        }

    private:
        void pMatching(VecXd& effort) {    // face_rosy_field.h:138-167 (interior edges)
            METRIKO_PARALLEL_FOR
            for (int e = 0; e < mesh.nE; e++) {
                if (mesh.isBE[e]) continue;
                int f0 = mesh.edge2face(e, 0), f1 = mesh.edge2face(e, 1);
                complex conn = connection[e];
                double minRot = 1000.;
                int offset = 0;
                complex coef(1, 0);
                complex transport0 = conn * field(f0, 0);
                for (int i = 0; i < rosyN; i++) {
                    complex jf = field(f0, i), jg = field(f1, i);
                    coef *= jg / (conn * jf);
                    double r = std::arg(jg / transport0);
                    if (std::abs(r) < std::abs(minRot)) { offset = i; minRot = r; }
                }
                effort[e] = std::arg(coef);
                double residuals = 0;
                for (int i = 0; i < rosyN; i++) residuals += std::arg(field(f1, (i + offset) % rosyN) / (conn * field(f0, i)));
                matching[e] = offset - static_cast<int>(std::round((residuals - effort[e]) / TwoPI));
            }
        }

        void cMatching(VecXd& effort) {    // face_rosy_field.h:169-202 (interior edges)
            METRIKO_PARALLEL_FOR
            for (int e = 0; e < mesh.nE; e++) {
                if (mesh.isBE[e]) continue;
                int iM = 0;
                double mn = 32767000.;
                Row3d v = Half{{mesh.edge2half[e], &mesh}}.vec().normalized();
                int f0 = mesh.edge2face(e, 0), f1 = mesh.edge2face(e, 1);
                Row3d bx0 = row3(mesh.faceBasisX, f0), by0 = row3(mesh.faceBasisY, f0);
                Row3d bx1 = row3(mesh.faceBasisX, f1), by1 = row3(mesh.faceBasisY, f1);
                for (int i = 0; i < rosyN; i++) {
                    double curl = 0;
                    for (int j = 0; j < rosyN; j++) {
                        complex c0 = field(f0, j), c1 = field(f1, (i + j) % rosyN);
                        Row3d v0 = bx0 * c0.real() + by0 * c0.imag();
                        Row3d v1 = bx1 * c1.real() + by1 * c1.imag();
                        double d = v.dot(v1 - v0);
                        curl += d * d;
                    }
                    if (curl < mn) { iM = i; mn = curl; }
                }
                matching[e] = iM;
                complex coef(1, 0);
                for (int i = 0; i < rosyN; i++) coef *= field(f1, (i + iM) % rosyN) / (field(f0, i) * connection[e]);
                effort[e] = std::arg(coef);
            }
        }
    };

    // face_rosy_field.h:207-249 (the search crosses no boundary edge; they keep matching -1)
    inline std::unique_ptr<FaceRosyField> compute_combbed_field(const FaceRosyField& fld, const std::vector<bool>& seam) {
        const Hmesh& m = fld.mesh;
        const int N = fld.rosyN;
        auto F = std::make_unique<FaceRosyField>(m, N);
        F->field = MatXc(m.nF, N, complex(0, 0));
        F->connection = fld.connection;
        F->compressed = fld.compressed;
        F->singular = fld.singular;
        std::vector<int> turns(m.nF, 0);
        std::vector<char> visit(m.nF, 0);
        // per face side: the neighbour across it (-1 across a seam) and the signed matching,
        // gathered in parallel so that the sequential search touches one array
        std::vector<int> nb(3 * size_t(m.nF)), nm(3 * size_t(m.nF));
        METRIKO_PARALLEL_FOR
        for (int i = 0; i < m.nF; i++)
            for (int j = 0; j < 3; j++) {
                const int e = m.edge[m.face2half3(i, j)];
                const bool b = m.edge2face(e, 0) == i;
                nb[3 * size_t(i) + j] = (seam[e] || m.isBE[e]) ? -1 : (b ? m.edge2face(e, 1) : m.edge2face(e, 0));
                nm[3 * size_t(i) + j] = (b ? 1 : -1) * fld.matching[e];
            }
        if (gpu::bound_context()) {
            // inside a device pipeline call: the same turns from the level-by-level search on the
            // device (mtk_comb_turns; the turns do not depend on the path inside the cut disk)
            gpu::check(mtk_comb_turns(gpu::bound_context(), m.nF, N, nb.data(), nm.data(), turns.data()), "mtk_comb_turns");
            METRIKO_PARALLEL_FOR
            for (int i = 0; i < m.nF; i++) {
                visit[i] = turns[i] >= 0;
                if (turns[i] < 0) turns[i] = 0;
            }
        } else {
            std::deque<std::pair<int, int>> q;
            q.emplace_back(0, 0);
            while (!q.empty()) {
                auto [i, mm] = q.front();
                q.pop_front();
                if (visit[i]) continue;
                visit[i] = 1;
                turns[i] = mm;
                for (int j = 0; j < 3; j++) {
                    const int fn = nb[3 * size_t(i) + j];
                    if (fn >= 0 && !visit[fn]) q.emplace_back(fn, (nm[3 * size_t(i) + j] + mm + 1000 * N) % N);
                }
            }
        }
        METRIKO_PARALLEL_FOR
        for (int i = 0; i < m.nF; i++)
            if (visit[i])
                for (int k = 0; k < N; k++) F->field(i, k) = fld.field(i, (k + turns[i]) % N);
        F->matching = VecXi(m.nE, -1);
        METRIKO_PARALLEL_FOR
        for (int e = 0; e < m.nE; e++)
            if (!m.isBE[e])
                F->matching[e] = (turns[m.edge2face(e, 0)] - turns[m.edge2face(e, 1)] + fld.matching[e] + 1000 * N) % N;
        return F;
    }

    // face_rosy_field.h:251-264 (N = 4)
    inline MatXd compute_extrinsic_field(const Hmesh& mesh, const FaceRosyField& fld, int rosyN) {
        MatXd ext(mesh.nF, 3 * rosyN);
        METRIKO_PARALLEL_FOR
        for (int f = 0; f < mesh.nF; f++) {
            Row3d bx = row3(mesh.faceBasisX, f), by = row3(mesh.faceBasisY, f);
            for (int i = 0; i < rosyN; i++) {
                complex c = fld.field(f, i);
                Row3d v = (bx * c.real() + by * c.imag()).normalized();
                for (int k = 0; k < 3; k++) ext(f, 3 * i + k) = v[k];
            }
        }
        return ext;
    }

    namespace detail {
        // TT(f,s): face across edge s = (F(f,s), F(f,s+1)); TTi(f,s): that edge's slot in TT(f,s);
        // both -1 on a boundary side.
        inline void triangle_adjacency(const Hmesh& m, MatXi& TT, MatXi& TTi) {
            TT = MatXi(m.nF, 3);
            TTi = MatXi(m.nF, 3);
            METRIKO_PARALLEL_FOR
            for (int f = 0; f < m.nF; f++)
                for (int s = 0; s < 3; s++) {
                    int t = m.twin[m.face2half3(f, s)];
                    int g = m.face[t];
                    TT(f, s) = g;
                    TTi(f, s) = g < 0 ? -1 : (m.face2half3(g, 0) == t ? 0 : (m.face2half3(g, 1) == t ? 1 : 2));
                }
        }

        // libigl cut_mesh_from_singularities with an all-zero matching (see file header).  A
        // boundary side is never crossed by the flood fill, so it stays a seam, and the retraction
        // counts it once (TT = -1 <= f); boundary loops are cycles and are never retracted.
        inline MatXi spanning_cut(const Hmesh& m, const MatXi& TT, const MatXi& TTi) {
            const MatXi& F = m.idx;
            const int nF = m.nF;
            MatXi seams(nF, 3, 1);
            std::vector<char> visited(nF, 0);
            std::vector<int> queue(nF);   // FIFO: every face enters once
            for (int f0 = 0; f0 < nF; f0++) {
                if (visited[f0]) continue;
                visited[f0] = 1;
                size_t head = 0, tail = 0;
                queue[tail++] = f0;
                while (head < tail) {
                    const int f = queue[head++];
                    for (int s = 0; s < 3; s++) {
                        int g = TT(f, s), j = TTi(f, s);
                        if (g >= 0 && !visited[g]) {
                            visited[g] = 1;
                            seams(f, s) = 0;
                            seams(g, j) = 0;
                            queue[tail++] = g;
                        }
                    }
                }
            }
            // Retract: exact pass-by-pass semantics, event driven.
            std::vector<int> e(m.nV, 0);
            for (int f = 0; f < nF; f++)
                for (int s = 0; s < 3; s++)
                    if (seams(f, s) && TT(f, s) <= f) { e[F(f, s)]++; e[F(f, (s + 1) % 3)]++; }
            std::vector<int> vptr(m.nV + 1, 0);
            for (int f = 0; f < nF; f++)
                for (int s = 0; s < 3; s++)
                    if (seams(f, s)) { vptr[F(f, s) + 1]++; vptr[F(f, (s + 1) % 3) + 1]++; }
            for (int v = 0; v < m.nV; v++) vptr[v + 1] += vptr[v];
            std::vector<int> vpos(vptr[m.nV]);
            {
                std::vector<int> fill(vptr.begin(), vptr.end() - 1);
                for (int f = 0; f < nF; f++)
                    for (int s = 0; s < 3; s++)
                        if (seams(f, s)) { vpos[fill[F(f, s)]++] = 3 * f + s; vpos[fill[F(f, (s + 1) % 3)]++] = 3 * f + s; }
            }
            // Leaf pruning reaches the same fixed point in any order (what is left is the unique
            // subgraph without degree-1 vertices), and the reference's pass loop stops only at that
            // fixed point unless it hits its pass cap (10001 passes).  Every pass removes at least
            // all edges that are leaves when it starts, so the number of passes is at most the
            // depth of simultaneous peeling: when that depth is within the cap the fixed point is
            // the answer, computed here in O(E); otherwise the passes are simulated exactly below.
            {
                std::vector<int> deg(e);
                MatXi pruned = seams;
                std::vector<int> layer, next_layer;
                for (int v = 0; v < m.nV; v++) if (deg[v] == 1) layer.push_back(v);
                int depth = 0;
                while (!layer.empty() && depth <= 10000) {
                    depth++;
                    next_layer.clear();
                    for (int v : layer) {
                        if (deg[v] != 1) continue;
                        for (int k = vptr[v]; k < vptr[v + 1]; k++) {
                            const int qp = vpos[k], f = qp / 3, s2 = qp % 3;
                            if (!pruned(f, s2)) continue;
                            const int a = F(f, s2), b = F(f, (s2 + 1) % 3), w = a == v ? b : a;
                            pruned(f, s2) = 0;
                            if (TT(f, s2) >= 0) pruned(TT(f, s2), TTi(f, s2)) = 0;
                            deg[v]--;
                            deg[w]--;
                            if (deg[w] == 1) next_layer.push_back(w);
                            break;
                        }
                    }
                    layer.swap(next_layer);
                }
                if (layer.empty()) return pruned;
            }
            auto leaf_edge = [&](int p) { int f = p / 3, s = p % 3; return e[F(f, s)] == 1 || e[F(f, (s + 1) % 3)] == 1; };
            std::priority_queue<int, std::vector<int>, std::greater<int>> cur;
            for (int f = 0; f < nF; f++)
                for (int s = 0; s < 3; s++)
                    if (seams(f, s) && leaf_edge(3 * f + s)) cur.push(3 * f + s);
            std::vector<int> nxt;
            int guard = 0;
            while (true) {
                bool removed = false;
                int cursor = -1;
                while (!cur.empty()) {
                    int p = cur.top();
                    cur.pop();
                    if (p <= cursor) continue;
                    cursor = p;
                    int f = p / 3, s = p % 3;
                    if (!seams(f, s)) continue;
                    int a = F(f, s), b = F(f, (s + 1) % 3);
                    if (e[a] == 1 || e[b] == 1) {
                        seams(f, s) = 0;
                        if (TT(f, s) >= 0) seams(TT(f, s), TTi(f, s)) = 0;
                        e[a]--;
                        e[b]--;
                        removed = true;
                        for (int v : {a, b}) {
                            if (e[v] != 1) continue;
                            for (int k = vptr[v]; k < vptr[v + 1]; k++) {
                                int qp = vpos[k];
                                if (!seams(qp / 3, qp % 3)) continue;
                                if (qp > p) cur.push(qp);
                                else nxt.push_back(qp);
                            }
                        }
                    }
                }
                guard++;
                if (!removed || guard > 10000) break;
                std::sort(nxt.begin(), nxt.end());
                nxt.erase(std::unique(nxt.begin(), nxt.end()), nxt.end());
                for (int p : nxt) cur.push(p);
                nxt.clear();
            }
            return seams;
        }
    }

    // The part of cut_mesh_with_singularities that depends on the mesh alone: the triangle
    // adjacency, the spanning cut (libigl's cut with an all-zero matching) and the vertex
    // adjacency that the singularity-path searches walk.  Depends on no field, so a caller may
    // compute it while the field is solved (mtk_pipeline_run does, on a host thread).
    struct SeamBase {
        MatXi TT, TTi, cuts;
        std::vector<int> vptr, vv;   // vertex -> neighbouring vertices (one per outgoing halfedge)
        std::vector<int> ve;         // the edge of each (vertex, neighbour) entry
    };

    inline SeamBase seam_base(const Hmesh& m) {
        SeamBase b;
        detail::triangle_adjacency(m, b.TT, b.TTi);
        b.cuts = detail::spanning_cut(m, b.TT, b.TTi);
        b.vptr.assign(m.nV + 1, 0);
        METRIKO_PARALLEL_FOR
        for (int v = 0; v < m.nV; v++) {
            int cnt = 0, h = m.vert2half[v];
            do { cnt++; h = m.twin[m.prev[h]]; } while (h != m.vert2half[v]);
            b.vptr[v + 1] = cnt;
        }
        for (int v = 0; v < m.nV; v++) b.vptr[v + 1] += b.vptr[v];
        b.vv.resize(b.vptr[m.nV]);
        b.ve.resize(b.vptr[m.nV]);
        METRIKO_PARALLEL_FOR
        for (int v = 0; v < m.nV; v++) {
            int q = b.vptr[v], h = m.vert2half[v];
            do { b.ve[q] = m.edge[h]; b.vv[q++] = m.head[h]; h = m.twin[m.prev[h]]; } while (h != m.vert2half[v]);
        }
        return b;
    }

    // face_rosy_field.h:268-343 (cut_mesh_with_singularities), continuing from seam_base(m)
    inline void cut_mesh_with_singularities(const Hmesh& m, const VecXi& singularities, SeamBase&& base, MatXi& cuts) {
        const MatXi& F = m.idx;
        const MatXi& TT = base.TT;
        const MatXi& TTi = base.TTi;
        const std::vector<int>& vptr = base.vptr;
        const std::vector<int>& vv = base.vv;
        cuts = std::move(base.cuts);
        std::vector<int> in_cut(m.nV, 0);
        for (int f = 0; f < m.nF; f++) for (int j = 0; j < 3; j++) if (cuts(f, j)) in_cut[F(f, j)] = 1;
        std::vector<int> dist(m.nV, -1), prev(m.nV, -1), touched;
        long long ncut = 0;
        for (int v = 0; v < m.nV; v++) ncut += in_cut[v];
        for (int i = 0; i < singularities.size(); i++) {
            const int src = singularities[i];
            if (ncut == 0) {
                // no target at all: the search would exhaust the mesh and return -1, so the path
                // is the singularity alone
                in_cut[src] = 1;
                ncut = 1;
                continue;
            }
            // unit-weight Dijkstra with pops ordered by (distance, id), run as a breadth-first
            // search by levels: a vertex's predecessor is the first popped neighbour that reached
            // it, i.e. its smallest-id neighbour in the previous level, and the search ends at the
            // smallest-id cut vertex of the first level that holds one (the order in which a level
            // is expanded does not matter, so levels are not sorted)
            for (int v : touched) { dist[v] = -1; prev[v] = -1; }
            touched.clear();
            dist[src] = 0;
            touched.push_back(src);
            std::vector<int> level{src}, nlevel;
            int found = -1;
            for (int d = 0; !level.empty() && found < 0; d++) {
                for (int u : level)
                    if (in_cut[u] && (found < 0 || u < found)) found = u;
                if (found >= 0) break;
                nlevel.clear();
                for (int u : level)
                    for (int k = vptr[u]; k < vptr[u + 1]; k++) {
                        const int w = vv[k];
                        if (dist[w] < 0) {
                            dist[w] = d + 1;
                            prev[w] = u;
                            touched.push_back(w);
                            nlevel.push_back(w);
                        } else if (dist[w] == d + 1 && u < prev[w]) {
                            prev[w] = u;
                        }
                    }
                level.swap(nlevel);
            }
            std::vector<int> path;
            if (found == -1) path.push_back(src);
            else for (int v = found; v != -1; v = prev[v]) path.push_back(v);
            for (int v : path) { ncut += !in_cut[v]; in_cut[v] = 1; }
            for (size_t ii = 0; ii + 1 < path.size(); ii++) {
                // the edge v0 v1 is cut on both of its faces
                const int v0 = path[ii], v1 = path[ii + 1];
                int h = m.vert2half[v0];
                while (m.head[h] != v1) h = m.twin[m.prev[h]];
                const int fi = m.face[h];
                int j = -1;
                for (int z = 0; z < 3; z++)
                    if ((F(fi, z) == v0 && F(fi, (z + 1) % 3) == v1) || (F(fi, z) == v1 && F(fi, (z + 1) % 3) == v0)) j = z;
                cuts(fi, j) = 1;
                // never a boundary edge: every boundary vertex is on the cut, and a search stops at
                // the first cut vertex it reaches
                if (TT(fi, j) >= 0) cuts(TT(fi, j), TTi(fi, j)) = 1;
            }
        }
    }

    // face_rosy_field.h:268-343 (cut_mesh_with_singularities)
    inline void cut_mesh_with_singularities(const Hmesh& m, const VecXi& singularities, MatXi& cuts) {
        cut_mesh_with_singularities(m, singularities, seam_base(m), cuts);
    }

    // face_rosy_field.h:345-360, with seam_base(f.mesh) computed beforehand.  Inside a device
    // pipeline call (a context bound to the host thread) the singularity-path searches run on the
    // device (mtk_seam_paths: the same searches, the same paths, one launch for all of them); the
    // seam is the spanning cut's edges plus the paths' edges either way.
    inline std::vector<bool> compute_seam(const FaceRosyField& f, SeamBase&& base) {
        std::vector<bool> seam(f.mesh.nE, false);
        std::vector<int> sv;
        for (int v = 0; v < f.mesh.nV; v++) if (f.singular[v] != 0) sv.push_back(v);
        if (gpu::bound_context() && !base.ve.empty()) {
            const Hmesh& m = f.mesh;
            std::vector<uint8_t> in_cut(m.nV, 0), flag(m.nE, 0);
            for (int iF = 0; iF < m.nF; iF++)
                for (int j = 0; j < 3; j++)
                    if (base.cuts(iF, j)) { in_cut[m.idx(iF, j)] = 1; flag[m.face2edge(iF, j)] = 1; }
            gpu::check(mtk_seam_paths(gpu::bound_context(), m.nV, m.nE, base.vptr.data(), base.vv.data(), base.ve.data(),
                                      int(sv.size()), sv.data(), in_cut.data(), flag.data()),
                       "mtk_seam_paths");
            for (int e = 0; e < m.nE; e++) seam[e] = flag[e] != 0;
            return seam;
        }
        MatXi cuts;
        cut_mesh_with_singularities(f.mesh, VecXi(sv), std::move(base), cuts);
        for (int iF = 0; iF < f.mesh.nF; iF++)
            for (int j = 0; j < 3; j++) if (cuts(iF, j)) seam[f.mesh.face2edge(iF, j)] = true;
        return seam;
    }

    // face_rosy_field.h:345-360
    inline std::vector<bool> compute_seam(const FaceRosyField& f) { return compute_seam(f, seam_base(f.mesh)); }
}

#endif
