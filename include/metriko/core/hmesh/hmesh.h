//
// Restates parts of metriko (https://github.com/komietty/metriko),
// Copyright (C) 2025 Saki Komikado <komietty@gmail.com>.
// This Source Code Form is subject to the terms of the Mozilla Public License v.2.0
// (https://mozilla.org/MPL/2.0/).
//
// metriko-gb300: halfedge mesh (DCEL) with the reference's numbering.
//
// Replaces metriko include/metriko/core/hmesh/hmesh.h:24-569 (struct Hmesh, handles, dcel()).
// Consistently oriented, edge-manifold triangle meshes, closed or with boundary loops, are
// accepted; anything else throws std::invalid_argument.
//
// Numbering follows the reference exactly, because every later integer decision depends on it:
//  * edges: libigl v2.5.0 edge_topology -- entries (min v, max v, face, corner) sorted
//    lexicographically, one edge per distinct (min, max); edge2face(e,0) is the face in which
//    the edge runs min->max, -1 on the side of a boundary edge that has no face (restated from
//    libigl's documented behaviour);
//  * interior halfedges are numbered in edge order, slot 0 (tail edge2vert(e,0), face
//    edge2face(e,0)) before slot 1, skipping a slot without a face (dcel, hmesh.h:254-258): a
//    closed mesh has 2e and its twin 2e+1;
//  * boundary halfedges (face -1) follow from 3 nF on, loop by loop (hmesh.h:393-418): loops in
//    the order of their first interior halfedge without a twin, each walked backwards along the
//    interior halfedges it borders; loop2half[l] is the loop's first boundary halfedge;
//  * vert2half[v] is the last interior halfedge written for v in edge order (hmesh.h:268-279,
//    :377); edge2half[e] is the slot-0 halfedge, or the boundary halfedge when slot 0 has no face
//    (:420-421);
//  * face2half[f] runs F(f,0)->F(f,1) (hmesh.h:379).
//
#ifndef METRIKO_HMESH_H
#define METRIKO_HMESH_H
#include "metriko/core/common/typedef.h"

namespace metriko {
    struct Hmesh;
    struct Half; struct Vert; struct Edge; struct Face; struct Crnr;

    struct Elem {
        int id;
        const Hmesh* m;
        bool operator==(const Elem& rhs) const { return id == rhs.id; }
    };

    template <typename N> struct AdjIter;
    struct AdjVH; struct AdjFH;

    struct Face : Elem {
        Half half() const;
        Row3d basisX() const;
        Row3d basisY() const;
        Row3d normal() const;
        Row3d center() const;
        double area() const;
        AdjIter<AdjFH> adjHalfs(bool ccw = true) const;
        AdjIter<AdjFH> adjHalfs(Half h, bool ccw = true) const;
    };
    struct Edge : Elem {
        Half half() const;
        Vert vert0() const;
        Vert vert1() const;
        Face face0() const;
        Face face1() const;
        double len() const;
        double cot() const;
        bool isBoundary() const;
    };
    struct Vert : Elem {
        Half half() const;
        Row3d pos() const;
        Row3d basisX() const;
        Row3d basisY() const;
        Row3d normal() const;
        double baryArea() const;
        double circArea() const;
        bool isBoundary() const;
        bool isInterior() const;
        AdjIter<AdjVH> adjHalfs(bool ccw = true) const;
        AdjIter<AdjVH> adjHalfs(Half h, bool ccw = true) const;
    };
    // boundary loop (closed meshes have none: Hmesh::loops stays empty)
    struct Loop : Elem {
        Half half() const;
    };
    // corner c of face f sits at F(f, c - 3f); its halfedge is the one opposite that vertex
    struct Crnr : Elem {
        Half half() const;
        Vert vert() const;
        Face face() const;
    };
    struct Half : Elem {
        Half next() const;
        Half prev() const;
        Half twin() const;
        Vert tail() const;
        Vert head() const;
        Edge edge() const;
        Face face() const;
        Crnr crnr() const;
        double farg() const;
        double varg() const;
        double darg() const;
        double cot() const;
        double len() const { return vec().norm(); }
        bool isBoundary() const;
        bool isCanonical() const;
        Row3d vec() const;
    };

    struct Hmesh {
        int nV = 0, nF = 0, nE = 0, nH = 0, nL = 0, nC = 0, nEularChars = 0;
        std::vector<int> vert2half, edge2half, face2half, crnr2half;
        std::vector<int> next, prev, twin, tail, head, edge, face, crnr;
        std::vector<Half> halfs;
        std::vector<Vert> verts;
        std::vector<Edge> edges;
        std::vector<Face> faces;
        MatXd pos;
        MatXi idx;
        MatXi edge2vert;   // nE x 2
        MatXi edge2face;   // nE x 2
        MatXi face2edge;   // nF x 3, edge of (F(f,j), F(f,j+1))
        MatXi face2half3;  // nF x 3, halfedge of face f on face2edge(f,j)
        MatXd faceBasisX, faceBasisY, faceNormal, baryCenter;
        VecXd faceArea, angleDefect, heArgOnFace;   // heArgOnFace: 0 on boundary halfedges
        std::vector<int> loop2half;   // first boundary halfedge of each boundary loop
        std::vector<bool> isBV;       // vertex on a boundary edge
        std::vector<char> isBE;       // edge with one face
        bool hasBoundary = false;
        // filled by finish() (hmesh.h:444-568 of the reference): vertex frames, dual areas,
        // cotangents, dihedral angles, halfedge angles around vertices, corner handles
        MatXd vertBasisX, vertBasisY, vertNormal;
        VecXd baryDualArea, circDualArea, halfCotan, edgeCotan, dihedralArg, heArgOnVert;
        std::vector<Crnr> crnrs;
        std::vector<Loop> loops;

        Hmesh(const MatXd& V, const MatXi& F);
        // Two-phase construction: connectivity, face frames, normals, centres, areas and halfedge
        // angles (all that a smoothest-field solve reads); finish() adds the element lists
        // (halfs, verts, edges, faces, crnrs), the angle defects and the vertex and edge
        // geometry below, which stay empty until then.
        struct Deferred {};
        Hmesh(const MatXd& V, const MatXi& F, Deferred);
        void finish();
        Hmesh(const Hmesh&) = delete;
        Hmesh& operator=(const Hmesh&) = delete;
    };

    struct AdjBase {
        Half h;
        bool bgn;
        bool ccw;
        AdjBase(Half h_, bool c) : h(h_), bgn(false), ccw(c) {}
        Half operator*() const { return h; }
        bool operator!=(const AdjBase& a) const { return !bgn || h.id != a.h.id; }
    };
    struct AdjVH : AdjBase {
        AdjVH(const Hmesh* m, int hid, bool c) : AdjBase(Half{{hid, m}}, c) {}
        AdjVH& operator++() { h = ccw ? h.prev().twin() : h.twin().next(); bgn = true; return *this; }
    };
    struct AdjFH : AdjBase {
        AdjFH(const Hmesh* m, int hid, bool c) : AdjBase(Half{{hid, m}}, c) {}
        AdjFH& operator++() { h = ccw ? h.next() : h.prev(); bgn = true; return *this; }
    };
    template <typename N>
    struct AdjIter {
        AdjIter(const Hmesh* m, int iX, bool ccw) : bgnNav(N(m, iX, ccw)), endNav(N(m, iX, ccw)) {}
        N begin() { return bgnNav; }
        N end() { return endNav; }
        N bgnNav, endNav;
    };

    inline Half Half::next() const { return {{m->next[id], m}}; }
    inline Half Half::prev() const { return {{m->prev[id], m}}; }
    inline Half Half::twin() const { return {{m->twin[id], m}}; }
    inline Vert Half::tail() const { return {{m->tail[id], m}}; }
    inline Vert Half::head() const { return {{m->head[id], m}}; }
    inline Edge Half::edge() const { return {{m->edge[id], m}}; }
    inline Face Half::face() const { return {{m->face[id], m}}; }
    inline Crnr Half::crnr() const { return {{m->crnr[id], m}}; }
    inline double Half::farg() const { return m->heArgOnFace[id]; }
    inline double Half::varg() const { return m->heArgOnVert[id]; }
    inline double Half::darg() const { return m->dihedralArg[id]; }
    inline double Half::cot() const { return m->halfCotan[id]; }
    inline double Edge::len() const { return Half{{m->edge2half[id], m}}.len(); }
    inline double Edge::cot() const { return m->edgeCotan[id]; }
    inline Row3d Vert::basisX() const { return row3(m->vertBasisX, id); }
    inline Row3d Vert::basisY() const { return row3(m->vertBasisY, id); }
    inline Row3d Vert::normal() const { return row3(m->vertNormal, id); }
    inline double Vert::baryArea() const { return m->baryDualArea[id]; }
    inline double Vert::circArea() const { return m->circDualArea[id]; }
    inline Half Loop::half() const { return {{m->loop2half[id], m}}; }
    inline Half Crnr::half() const { return {{m->crnr2half[id], m}}; }
    inline Vert Crnr::vert() const { return half().prev().tail(); }
    inline Face Crnr::face() const { return half().face(); }
    inline bool Half::isCanonical() const { return m->edge2half[m->edge[id]] == id; }
    inline bool Half::isBoundary() const { return m->face[id] == -1; }
    inline bool Edge::isBoundary() const { return m->isBE[id] != 0; }
    inline bool Vert::isBoundary() const { return m->isBV[id]; }
    inline bool Vert::isInterior() const { return !m->isBV[id]; }
    inline Row3d Half::vec() const { return row3(m->pos, m->head[id]) - row3(m->pos, m->tail[id]); }
    inline Half Vert::half() const { return {{m->vert2half[id], m}}; }
    inline Row3d Vert::pos() const { return row3(m->pos, id); }
    inline Half Edge::half() const { return {{m->edge2half[id], m}}; }
    inline Vert Edge::vert0() const { return {{m->edge2vert(id, 0), m}}; }
    inline Vert Edge::vert1() const { return {{m->edge2vert(id, 1), m}}; }
    inline Face Edge::face0() const { return {{m->edge2face(id, 0), m}}; }
    inline Face Edge::face1() const { return {{m->edge2face(id, 1), m}}; }
    inline Half Face::half() const { return {{m->face2half[id], m}}; }
    inline Row3d Face::basisX() const { return row3(m->faceBasisX, id); }
    inline Row3d Face::basisY() const { return row3(m->faceBasisY, id); }
    inline Row3d Face::normal() const { return row3(m->faceNormal, id); }
    inline Row3d Face::center() const { return row3(m->baryCenter, id); }
    inline double Face::area() const { return m->faceArea[id]; }
    inline AdjIter<AdjFH> Face::adjHalfs(bool ccw) const { return {m, m->face2half[id], ccw}; }
    inline AdjIter<AdjFH> Face::adjHalfs(Half h, bool ccw) const { return {m, h.id, ccw}; }
    inline AdjIter<AdjVH> Vert::adjHalfs(bool ccw) const { return {m, m->vert2half[id], ccw}; }
    inline AdjIter<AdjVH> Vert::adjHalfs(Half h, bool ccw) const { return {m, h.id, ccw}; }

    // libigl v2.5.0 edge_topology semantics (see file header).  EV: nE x 2, FE: nF x 3, EF: nE x 2.
    // Built in parallel with the serial definition's result: entries are bucketed by their smaller
    // vertex (atomic slots; each bucket is then sorted by (hi, face, corner), a total order, so the
    // slot order does not matter), edge ids are the running count of distinct (lo, hi) pairs in
    // that order, and the checks report the error the serial pass would meet first (a third face
    // on any edge, else the first edge in order with one face or a repeated face).
    inline void edge_topology(const MatXi& F, int nV, MatXi& EV, MatXi& FE, MatXi& EF) {
        const int nF = F.rows();
        const long long nEnt = 3LL * nF;
        struct Ent { int hi, f, i, a; };
        std::vector<int> cnt(nV + 1, 0);
        int bad = 0;
        METRIKO_PARALLEL_FOR
        for (int f = 0; f < nF; f++)
            for (int i = 0; i < 3; i++) {
                int a = F(f, i), b = F(f, (i + 1) % 3);
                if (a < 0 || a >= nV || b < 0 || b >= nV || a == b) { __atomic_store_n(&bad, 1, __ATOMIC_RELAXED); continue; }
                __atomic_fetch_add(&cnt[std::min(a, b) + 1], 1, __ATOMIC_RELAXED);
            }
        if (bad) throw std::invalid_argument("bad face index");
        for (int v = 0; v < nV; v++) cnt[v + 1] += cnt[v];
        std::vector<Ent> ent(nEnt);
        std::vector<int> fill(cnt.begin(), cnt.end() - 1);
        METRIKO_PARALLEL_FOR
        for (int f = 0; f < nF; f++)
            for (int i = 0; i < 3; i++) {
                int a = F(f, i), b = F(f, (i + 1) % 3);
                ent[__atomic_fetch_add(&fill[std::min(a, b)], 1, __ATOMIC_RELAXED)] = {std::max(a, b), f, i, a};
            }
        std::vector<int> lo_of(nEnt);
        METRIKO_PARALLEL_FOR
        for (int v = 0; v < nV; v++) {
            std::sort(ent.begin() + cnt[v], ent.begin() + cnt[v + 1], [](const Ent& x, const Ent& y) {
                if (x.hi != y.hi) return x.hi < y.hi;
                if (x.f != y.f) return x.f < y.f;
                return x.i < y.i;
            });
            for (int p = cnt[v]; p < cnt[v + 1]; p++) lo_of[p] = v;
        }
        std::vector<int> eid(nEnt);    // 1 where an entry starts a new (lo, hi), then its edge id
        METRIKO_PARALLEL_FOR
        for (long long p = 0; p < nEnt; p++) eid[p] = p == 0 || lo_of[p] != lo_of[p - 1] || ent[p].hi != ent[p - 1].hi;
        int nE = 0;
        for (long long p = 0; p < nEnt; p++) { nE += eid[p]; eid[p] = nE - 1; }
        std::vector<int> first(nE + 1);
        METRIKO_PARALLEL_FOR
        for (long long p = 0; p < nEnt; p++) if (p == 0 || eid[p] != eid[p - 1]) first[eid[p]] = int(p);
        first[nE] = int(nEnt);
        EV = MatXi(nE, 2, -1);
        EF = MatXi(nE, 2, -1);
        FE = MatXi(nF, 3, -1);
        int over = 0;
        std::vector<char> err(nE, 0);  // 1: one face (boundary), 2: the same face twice
        METRIKO_PARALLEL_FOR
        for (int e = 0; e < nE; e++) {
            const int p0 = first[e], c = first[e + 1] - p0;
            EV(e, 0) = lo_of[p0];
            EV(e, 1) = ent[p0].hi;
            EF(e, 0) = ent[p0].f;
            if (c >= 2) EF(e, 1) = ent[p0 + 1].f;
            if (c > 2) __atomic_store_n(&over, 1, __ATOMIC_RELAXED);
            for (int p = p0; p < p0 + c; p++) FE(ent[p].f, ent[p].i) = e;
            if (c > 2) continue;
            // slot 0 holds the face in which the edge runs lo -> hi (-1 when a boundary edge's
            // one face runs hi -> lo)
            if (ent[p0].a != lo_of[p0]) std::swap(EF(e, 0), EF(e, 1));
            if (c == 2 && EF(e, 0) == EF(e, 1)) err[e] = 2;
            else if (c == 2 && ent[p0].a == ent[p0 + 1].a) err[e] = 3;   // both faces run the same way
        }
        if (over) throw std::invalid_argument("mesh is not edge-manifold");
        auto it = std::find_if(err.begin(), err.end(), [](char x) { return x != 0; });
        if (it != err.end())
            throw std::invalid_argument(*it == 2 ? "degenerate edge" : "inconsistently oriented faces");
    }

    inline Hmesh::Hmesh(const MatXd& V, const MatXi& F) : Hmesh(V, F, Deferred{}) { finish(); }

    inline Hmesh::Hmesh(const MatXd& V, const MatXi& F, Deferred) {
        if (V.cols() != 3 || F.cols() != 3) throw std::invalid_argument("V and F must have 3 columns");
        pos = V;
        idx = F;
        nV = V.rows();
        nF = F.rows();
        edge_topology(F, nV, edge2vert, face2edge, edge2face);
        nE = edge2vert.rows();
        nH = 2 * nE;
        nC = 3 * nF;
        nEularChars = nV - nE + nF;
        const int nI = 3 * nF;   // interior halfedges (one per face corner)
        vert2half.assign(nV, -1);
        edge2half.resize(nE);
        face2half.resize(nF);
        crnr2half.assign(nC, -1);
        next.assign(nH, -1); prev.assign(nH, -1); twin.assign(nH, -1); tail.assign(nH, -1);
        head.assign(nH, -1); edge.assign(nH, -1); face.assign(nH, -1); crnr.assign(nH, -1);
        isBE.assign(nE, 0);
        // EH(e, s): the interior halfedge of edge e in slot s (-1 when the slot has no face), the
        // running count of faced slots in (edge, slot) order
        MatXi EH(nE, 2, -1);
        {
            std::vector<int> cnt(nE + 1, 0);
            METRIKO_PARALLEL_FOR
            for (int e = 0; e < nE; e++) {
                const int c = (edge2face(e, 0) >= 0) + (edge2face(e, 1) >= 0);
                cnt[e + 1] = c;
                isBE[e] = c == 1;
            }
            for (int e = 0; e < nE; e++) cnt[e + 1] += cnt[e];
            if (cnt[nE] != nI) throw std::invalid_argument("mesh is not edge-manifold");
            METRIKO_PARALLEL_FOR
            for (int e = 0; e < nE; e++) {
                int h = cnt[e];
                for (int k = 0; k < 2; k++) {
                    if (edge2face(e, k) < 0) continue;
                    EH(e, k) = h;
                    tail[h] = edge2vert(e, k);
                    face[h] = edge2face(e, k);
                    edge[h] = e;
                    h++;
                }
                if (EH(e, 0) >= 0 && EH(e, 1) >= 0) { twin[EH(e, 0)] = EH(e, 1); twin[EH(e, 1)] = EH(e, 0); }
            }
        }
        // last write wins in (edge, slot) order (dcel, hmesh.h:268-279, :377): the survivor is
        // the largest interior halfedge id starting at the vertex
        METRIKO_PARALLEL_FOR
        for (int h = 0; h < nI; h++) {
            int* slot = &vert2half[tail[h]];
            int cur = __atomic_load_n(slot, __ATOMIC_RELAXED);
            while (h > cur && !__atomic_compare_exchange_n(slot, &cur, h, true, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) {
            }
        }
        for (int v = 0; v < nV; v++) if (vert2half[v] < 0) throw std::invalid_argument("isolated vertex");
        face2half3 = MatXi(nF, 3);
        METRIKO_PARALLEL_FOR
        for (int f = 0; f < nF; f++)
            for (int j = 0; j < 3; j++) {
                int e = face2edge(f, j);
                face2half3(f, j) = EH(e, edge2face(e, 0) == f ? 0 : 1);
            }
        METRIKO_PARALLEL_FOR
        for (int f = 0; f < nF; f++) {
            for (int j = 0; j < 3; j++) {
                next[face2half3(f, j)] = face2half3(f, (j + 1) % 3);
                prev[face2half3(f, (j + 1) % 3)] = face2half3(f, j);
            }
            face2half[f] = face2half3(f, 0);
            // corner 3f+it is the halfedge opposite F(f,it) (hmesh.h:429-442)
            for (int it = 0; it < 3; it++) {
                int h = face2half3(f, (it + 1) % 3);
                crnr2half[3 * f + it] = h;
                crnr[h] = 3 * f + it;
            }
        }
        METRIKO_PARALLEL_FOR
        for (int h = 0; h < nI; h++) head[h] = tail[next[h]];
        // boundary loops (hmesh.h:393-418): each interior halfedge without a twin, in id order,
        // starts a new loop unless an earlier loop took it; the loop's boundary halfedges are
        // numbered on from 3 nF, each the reverse of the interior halfedge it borders, walking
        // to the previous interior halfedge without a twin around the shared vertex
        loop2half.clear();
        {
            int iB = nI;
            for (int iH = 0; iH < nI; iH++) {
                if (twin[iH] != -1) continue;
                int jH = iH;
                const int jB = iB;
                bool done = false;
                while (true) {
                    if (iB >= nH) throw std::invalid_argument("mesh is not edge-manifold");
                    tail[iB] = head[jH];
                    head[iB] = tail[jH];
                    edge[iB] = edge[jH];
                    prev[iB] = iB - 1;
                    next[iB] = iB + 1;
                    twin[jH] = iB;
                    twin[iB] = jH;
                    jH = prev[jH];
                    long long guard = 0;
                    while (twin[jH] != -1) {
                        if (jH == iH) { done = true; break; }
                        jH = prev[twin[jH]];
                        if (++guard > nH) throw std::invalid_argument("mesh is not edge-manifold");
                    }
                    if (done) break;
                    iB++;
                }
                prev[jB] = iB;
                next[iB] = jB;
                loop2half.push_back(jB);
                iB++;
            }
            if (iB != nH) throw std::invalid_argument("mesh is not edge-manifold");
        }
        nL = int(loop2half.size());
        hasBoundary = nL > 0;
        isBV.assign(nV, false);
        METRIKO_PARALLEL_FOR
        for (int e = 0; e < nE; e++) edge2half[e] = EH(e, 0) >= 0 ? EH(e, 0) : twin[EH(e, 1)];
        for (int e = 0; e < nE; e++)
            if (isBE[e]) { isBV[edge2vert(e, 0)] = true; isBV[edge2vert(e, 1)] = true; }

        faceBasisX = MatXd(nF, 3); faceBasisY = MatXd(nF, 3); faceNormal = MatXd(nF, 3); baryCenter = MatXd(nF, 3);
        faceArea = VecXd(nF); heArgOnFace = VecXd(nH, 0.0);
        METRIKO_PARALLEL_FOR
        for (int f = 0; f < nF; f++) {
            Row3d p0 = row3(pos, F(f, 0)), p1 = row3(pos, F(f, 1)), p2 = row3(pos, F(f, 2));
            Row3d x = p1 - p0;
            Row3d t = (p0 - p2) * -1;
            Row3d n = x.cross(t);
            set_row3(faceBasisX, f, x.normalized());
            set_row3(faceBasisY, f, (-x.cross(n)).normalized());
            set_row3(faceNormal, f, n.normalized());
            set_row3(baryCenter, f, (p0 + p1 + p2) / 3.0);
            faceArea[f] = n.norm() * 0.5;
        }
        METRIKO_PARALLEL_FOR
        for (int f = 0; f < nF; f++) {     // hmesh.h:480-489
            double sum = 0;
            Row3d bx = row3(faceBasisX, f);
            for (int j = 0; j < 3; j++) {
                Half h{{face2half3(f, j), this}};
                Row3d v1 = h.vec().normalized();
                Row3d v2 = h.prev().vec().normalized();
                if ((v1 - bx).norm() > 1e-10) sum += std::acos(v1.dot(v2));
                heArgOnFace[h.id] = sum;
            }
        }
    }

    inline void Hmesh::finish() {
        faces.resize(nF);
        verts.resize(nV);
        edges.resize(nE);
        halfs.resize(nH);
        crnrs.resize(nC);
        METRIKO_PARALLEL_FOR
        for (int i = 0; i < nH; i++) {
            halfs[i] = Half{{i, this}};
            if (i < nF) faces[i] = Face{{i, this}};
            if (i < nV) verts[i] = Vert{{i, this}};
            if (i < nE) edges[i] = Edge{{i, this}};
            if (i < nC) crnrs[i] = Crnr{{i, this}};
        }
        loops.resize(nL);
        for (int l = 0; l < nL; l++) loops[l] = Loop{{l, this}};
        // halfedge angles around each vertex and the angle defect (hmesh.h:557-568): the angle
        // sum in ring order from vert2half, each halfedge's running sum rescaled to 2 pi; at a
        // boundary vertex the ring includes its boundary halfedge, whose angle is the one between
        // the vertex's two boundary edges, and the defect is pi - sum
        angleDefect = VecXd(nV);
        heArgOnVert = VecXd(nH);
        METRIKO_PARALLEL_FOR
        for (int v = 0; v < nV; v++) {
            double sum = 0;
            for (Half h : verts[v].adjHalfs()) {
                heArgOnVert[h.id] = sum;
                Row3d v1 = h.vec().normalized();
                Row3d v2 = h.prev().twin().vec().normalized();
                sum += std::acos(v1.dot(v2));
            }
            angleDefect[v] = isBV[v] ? PI - sum : TwoPI - sum;
            for (Half h : verts[v].adjHalfs()) heArgOnVert[h.id] *= TwoPI / sum;
        }
        // vertex normals: area-weighted face normals summed in face order (hmesh.h:491-498), so
        // each vertex adds its faces by ascending id; then the vertex frame (:500-506)
        vertNormal = MatXd(nV, 3);
        vertBasisX = MatXd(nV, 3);
        vertBasisY = MatXd(nV, 3);
        METRIKO_PARALLEL_FOR
        for (int v = 0; v < nV; v++) {
            int fs[64], k = 0;
            bool small = true;
            for (Half h : verts[v].adjHalfs()) {
                if (h.face().id < 0) continue;
                if (k == 64) { small = false; break; }
                fs[k++] = h.face().id;
            }
            std::vector<int> big;
            const int* list = fs;
            if (!small) {
                for (Half h : verts[v].adjHalfs()) if (h.face().id >= 0) big.push_back(h.face().id);
                std::sort(big.begin(), big.end());
                list = big.data();
                k = int(big.size());
            } else {
                std::sort(fs, fs + k);
            }
            Row3d n(0, 0, 0);
            for (int q = 0; q < k; q++) {
                const int f = list[q];
                const double a = faceArea[f];
                n = Row3d(n[0] + faceNormal(f, 0) * a, n[1] + faceNormal(f, 1) * a, n[2] + faceNormal(f, 2) * a);
            }
            n = n.normalized();
            set_row3(vertNormal, v, n);
            const Row3d d = row3(pos, head[vert2half[v]]) - row3(pos, v);
            const Row3d x = (d - n * d.dot(n)).normalized();
            set_row3(vertBasisX, v, x);
            set_row3(vertBasisY, v, n.cross(x));
        }
        // dihedral angle and cotangent of each halfedge (hmesh.h:508-533), edge cotangents; the
        // dihedral angle is 0 on both halfedges of a boundary edge, the cotangent 0 on a boundary
        // halfedge
        dihedralArg = VecXd(nH);
        halfCotan = VecXd(nH);
        METRIKO_PARALLEL_FOR
        for (int i = 0; i < nH; i++) {
            const Half h{{i, this}};
            if (isBE[edge[i]]) {
                dihedralArg[i] = 0;
            } else {
                const Row3d n1 = row3(faceNormal, face[i]), n2 = row3(faceNormal, face[twin[i]]);
                const Row3d v = h.vec() / h.len();
                dihedralArg[i] = std::atan2(v.dot(n1.cross(n2)), n1.dot(n2));
            }
            if (face[i] < 0) { halfCotan[i] = 0.; continue; }
            const Row3d vn = h.next().vec();
            const Row3d vp = h.prev().vec() * -1;
            halfCotan[i] = vp.dot(vn) / vp.cross(vn).norm();
        }
        edgeCotan = VecXd(nE);
        METRIKO_PARALLEL_FOR
        for (int e = 0; e < nE; e++) edgeCotan[e] = (halfCotan[edge2half[e]] + halfCotan[twin[edge2half[e]]]) * 0.5;
        // dual areas (hmesh.h:535-546): barycentric and circumcentric, summed in ring order
        baryDualArea = VecXd(nV);
        circDualArea = VecXd(nV);
        METRIKO_PARALLEL_FOR
        for (int v = 0; v < nV; v++) {
            double a1 = 0, a2 = 0;
            for (Half h : verts[v].adjHalfs()) {
                if (h.face().id != -1) a1 += faceArea[h.face().id];
                a2 += h.cot() * h.vec().squaredNorm();
                a2 += h.prev().cot() * h.prev().vec().squaredNorm();
            }
            baryDualArea[v] = a1 / 3.;
            circDualArea[v] = a2 * 0.125;
        }
    }
}

#endif
