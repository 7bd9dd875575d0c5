//
// Restates parts of metriko (https://github.com/komietty/metriko),
// Copyright (C) 2025 Saki Komikado <komietty@gmail.com>.
// This Source Code Form is subject to the terms of the Mozilla Public License v.2.0
// (https://mozilla.org/MPL/2.0/).
//
// metriko-gb300: motorcycle graph on a parameterisation (host only).
//
// Replaces metriko include/metriko/core/tmesh/motorcycle.h:11-291 with the geometric helpers of
// core/common/utilities.h:11-157 and core/hmesh/utilities.h:54-73.  From every singular vertex,
// one trace ("motorcycle") per axis direction of the parameterisation that leaves into one of
// its faces; the traces advance one face per step, in rounds over all traces, turning by the
// matching when they cross an edge, until each one hits a segment already laid by another trace
// (the hit trace's segment is split there: HitL / HitR on its two halves, HitB on the hitting
// one).  The result is the same as the reference's: the same ports in the same order, the same
// segments with the same end points (bit for bit, compiled without floating-point contraction:
// the complex products and lerps are written out as the reference's std::complex expressions
// evaluate), the same crash records.  Differences in form: traces and crashes are indices into
// mcurvs instead of pointers; the search for the first segment a new segment crosses looks only
// at the segments laid in that face (the reference scans every segment of every other trace) and
// breaks exact ties in the reference's scan order (trace, then position along the trace); the
// rounds are bounded (std::runtime_error when the segment count passes max_segments; the
// reference loops until every trace has crashed).
//
// Input: cfn[3 nF] the parameterisation at the face corners (corner j of face f at 3 f + j,
// the value at vertex F(f, j)), matching[nE] (the combed matching), singular[nV] (non-zero at
// the vertices that emit traces).  Closed meshes: a boundary vertex flagged singular would
// start traces through its boundary halfedge, as in the reference, and is rejected.
//
#ifndef METRIKO_MOTORCYCLE_H
#define METRIKO_MOTORCYCLE_H
#include <cmath>
#include <complex>
#include <stdexcept>
#include <vector>

#include "metriko/core/hmesh/hmesh.h"

namespace metriko {
    namespace mc {
        constexpr double kPi = 3.14159265358979323846;
        inline complex quater_rot(int i) {   // get_quater_rot (utilities.h:11-19)
            switch ((i % 4 + 4) % 4) {
                case 0: return {1, 0};
                case 1: return {0, 1};
                case 2: return {-1, 0};
                default: return {0, -1};
            }
        }
        inline double cross(complex a, complex b) { return a.real() * b.imag() - a.imag() * b.real(); }
        inline double dot(complex a, complex b) { return a.real() * b.real() + a.imag() * b.imag(); }
        inline complex sub(complex a, complex b) { return {a.real() - b.real(), a.imag() - b.imag()}; }
        inline complex add(complex a, complex b) { return {a.real() + b.real(), a.imag() + b.imag()}; }
        inline complex mul(complex a, complex b) {
            return {a.real() * b.real() - a.imag() * b.imag(), a.real() * b.imag() + a.imag() * b.real()};
        }
        inline complex lerp(complex a, complex b, double t) {   // a (1 - t) + b t
            const double s = 1.0 - t;
            return {a.real() * s + b.real() * t, a.imag() * s + b.imag() * t};
        }
        inline bool isccw(complex a, complex b, complex c) { return cross(sub(b, a), sub(c, a)) > 0; }
        inline double orientation(complex a, complex b, complex c) { return cross(sub(b, a), sub(c, a)); }
        inline bool points_into(complex d, complex a, complex b, complex c) {
            const complex ad = add(a, d);
            return isccw(a, b, ad) && isccw(a, ad, c);
        }
        inline bool equal(complex a, complex b, double tol = 1e-10) { return std::abs(sub(a, b)) < tol; }
        // find_extended_intersection (utilities.h:127-142): lines a-b and c-d; the 2x2 system
        // solved by the cofactor inverse (determinant m00 m11 - m10 m01, rows m_i0 r0 + m_i1 r1)
        inline bool extended_intersection(complex a, complex b, complex c, complex d, double& r_ab, double& r_cd) {
            const complex ba = sub(b, a);
            const double m00 = d.real() - c.real(), m01 = -ba.real();
            const double m10 = d.imag() - c.imag(), m11 = -ba.imag();
            const double det = m00 * m11 - m10 * m01;
            if (det == 0) return false;
            const double inv = 1.0 / det;
            const double i00 = m11 * inv, i10 = -m10 * inv, i01 = -m01 * inv, i11 = m00 * inv;
            const double r0 = -c.real() + a.real(), r1 = -c.imag() + a.imag();
            r_cd = i00 * r0 + i01 * r1;
            r_ab = i10 * r0 + i11 * r1;
            return true;
        }
        inline bool strict_intersection(complex a, complex b, complex c, complex d, double& r_ab, double& r_cd) {
            return extended_intersection(a, b, c, d, r_ab, r_cd) && r_ab > 0 && r_ab < 1 && r_cd > 0 && r_cd < 1;
        }
    }

    enum MvertType { None, HitL, HitR, HitB };

    struct Mport {
        int id = -1;
        int vert = -1;
        int face = -1;
        complex uv;
        complex dir;
        int next = -1;
        int prev = -1;
    };

    struct Mvert {
        complex uv;
        int crash = -1;            // the trace hit at this point (index into mcurvs), -1 for none
        MvertType type = None;
    };

    struct Msgmt {
        int curv = -1;             // the trace (index into mcurvs)
        int face = -1;
        Mvert fr, to;
        int id = -1, prev_id = -1, next_id = -1;
        complex diff() const { return mc::sub(to.uv, fr.uv); }
        bool operator==(const Msgmt& o) const { return face == o.face && fr.uv == o.fr.uv && to.uv == o.to.uv; }
    };

    struct Mcurv {
        int port = -1;             // index into mports (= the trace's index)
        std::vector<Msgmt> sgmts;
        // trace state (the reference's Cache): the halfedge the last segment left through, the
        // ratio along it, the direction, and whether the trace has crashed
        int half = -1;
        double ratio = 0;
        complex dir;
        bool intersected = false;
    };

    class MotorcycleGraph {
    public:
        std::vector<Mport> mports;
        std::vector<Mcurv> mcurvs;

        MotorcycleGraph(const Hmesh& mesh, const VecXc& cfn, const VecXi& matching, const VecXi& singular,
                        long long max_segments = -1)
            : m(mesh), cfn(cfn) {
            if (cfn.size() != 3 * m.nF || matching.size() != m.nE || singular.size() != m.nV)
                throw std::invalid_argument("MotorcycleGraph: cfn, matching or singular has the wrong size");
            gen_ports(singular);
            mcurvs.resize(mports.size());
            order.resize(mports.size());
            face_segs.assign(m.nF, {});
            for (size_t i = 0; i < mports.size(); i++) mcurvs[i].port = (int)i;
            for (int c = 0; c < (int)mcurvs.size(); c++) add_segment_init(c);
            const long long cap = max_segments > 0 ? max_segments : 64LL * (m.nF + 16);
            auto open = [&] {
                for (const Mcurv& cv : mcurvs) if (!cv.intersected) return true;
                return false;
            };
            while (open()) {
                for (int c = 0; c < (int)mcurvs.size(); c++) add_segment_next(c, matching);
                if ((long long)pool.size() > cap) throw std::runtime_error("MotorcycleGraph: the traces do not close");
            }
            for (int c = 0; c < (int)mcurvs.size(); c++) {   // post_process (motorcycle.h:126-133)
                Mcurv& cv = mcurvs[c];
                cv.sgmts.clear();
                for (int u : order[c]) cv.sgmts.push_back(pool[u]);
                for (int i = 0; i < (int)cv.sgmts.size(); i++) {
                    cv.sgmts[i].id = i;
                    cv.sgmts[i].prev_id = i - 1;
                    cv.sgmts[i].next_id = i + 1 < (int)cv.sgmts.size() ? i + 1 : -1;
                }
            }
        }

    private:
        const Hmesh& m;
        const VecXc& cfn;
        std::vector<Msgmt> pool;                   // every segment, by creation
        std::vector<std::vector<int>> order;       // per trace: its segments (pool ids) in order
        std::vector<std::vector<int>> face_segs;   // per face: the pool ids laid in it

        complex corner(int h) const { return cfn[m.crnr[h]]; }

        // gen_ports (motorcycle.h:166-212)
        void gen_ports(const VecXi& singular) {
            int counter = 0;
            for (int v = 0; v < m.nV; v++) {
                if (singular[v] == 0) continue;
                if (m.isBV[v]) throw std::invalid_argument("MotorcycleGraph: a boundary vertex is flagged singular");
                std::vector<Mport> ports;
                const int h0 = m.vert2half[v];
                int h = h0;
                do {
                    const complex a = corner(m.next[h]), b = corner(m.prev[h]), c = corner(h);
                    if (mc::orientation(a, b, c) < 0) throw std::invalid_argument("Orientation should be ccw order");
                    int r;
                    for (r = 0; r < 4; r++)
                        if (!mc::points_into(mc::quater_rot(r), a, b, c) && r > 0) break;
                    std::vector<Mport> temps;
                    const complex ba = mc::sub(b, a), ca = mc::sub(c, a);
                    for (int i = 0; i < 4; i++) {
                        const complex dir = mc::quater_rot(r - i);
                        if (mc::points_into(dir, a, b, c) || std::arg(dir) == std::arg(ba) || std::arg(dir) == std::arg(ca)) {
                            Mport p;
                            p.vert = v;
                            p.face = m.face[h];
                            p.uv = a;
                            p.dir = dir;
                            temps.push_back(p);
                        }
                    }
                    // by the projection on b - a, largest first; equal projections keep their order
                    for (size_t i = 1; i < temps.size(); i++)
                        for (size_t j = i; j > 0 && mc::dot(temps[j].dir, ba) > mc::dot(temps[j - 1].dir, ba); j--)
                            std::swap(temps[j], temps[j - 1]);
                    for (Mport& p : temps) p.id = counter++;
                    ports.insert(ports.end(), temps.begin(), temps.end());
                    h = m.twin[m.prev[h]];
                } while (h != h0);
                const int s = (int)ports.size();
                for (int i = 0; i < s; i++) {
                    ports[i].prev = ports[(i - 1 + s) % s].id;
                    ports[i].next = ports[(i + 1) % s].id;
                }
                mports.insert(mports.end(), ports.begin(), ports.end());
            }
        }

        int position(int c, int u) const {
            const std::vector<int>& o = order[c];
            for (int i = 0; i < (int)o.size(); i++) if (o[i] == u) return i;
            return -1;
        }

        // Mcurv::split_segment (motorcycle.h:108-124): split segment u of trace c where the new
        // segment `crash` hits it
        void split_segment(int c, int u, const Msgmt& crash, double ratio) {
            Msgmt& s = pool[u];
            const bool ccw = mc::cross(crash.diff(), s.diff()) > 0;
            const complex uv = mc::lerp(s.fr.uv, s.to.uv, ratio);
            Msgmt t;
            t.curv = c;
            t.face = s.face;
            t.fr = Mvert{uv, crash.curv, ccw ? HitL : HitR};
            t.to = s.to;
            s.to = Mvert{uv, crash.curv, ccw ? HitR : HitL};
            const int nu = (int)pool.size();
            const int face = s.face;
            pool.push_back(t);
            std::vector<int>& o = order[c];
            o.insert(o.begin() + position(c, u) + 1, nu);
            face_segs[face].push_back(nu);
        }

        // Mcurv::add_segment (motorcycle.h:250-291)
        void add_segment(int c, complex dir, complex uv0, int h) {
            const complex uv1 = corner(m.prev[h]), uv2 = corner(m.next[h]);
            double r_ab = 0, r_cd = 0;
            if (!mc::extended_intersection(uv0, mc::add(uv0, dir), uv1, uv2, r_ab, r_cd))
                throw std::runtime_error("MotorcycleGraph: a trace runs parallel to the edge it leaves through");
            const complex uv3 = mc::lerp(uv1, uv2, r_cd);
            const int face = m.face[h];
            int best = -1, best_c = -1;
            double best_ab = 0, best_cd = 0;
            for (int u : face_segs[face]) {
                const Msgmt& s = pool[u];
                if (s.curv == c) continue;
                double ab = 0, cd = 0;
                if (!mc::strict_intersection(uv0, uv3, s.fr.uv, s.to.uv, ab, cd)) continue;
                bool take = best < 0 || ab < best_ab;
                if (!take && ab == best_ab)   // the reference keeps the first in (trace, position) order
                    take = s.curv < best_c || (s.curv == best_c && position(s.curv, u) < position(best_c, best));
                if (take) { best = u; best_c = s.curv; best_ab = ab; best_cd = cd; }
            }
            Msgmt seg;
            seg.curv = c;
            seg.face = face;
            seg.fr = Mvert{uv0, -1, None};
            Mcurv& cv = mcurvs[c];
            cv.half = h;
            cv.ratio = r_cd;
            cv.dir = dir;
            if (best < 0) {
                seg.to = Mvert{uv3, -1, None};
                cv.intersected = false;
            } else {
                seg.to = Mvert{mc::lerp(uv0, uv3, best_ab), best_c, HitB};
                cv.intersected = true;
            }
            const int nu = (int)pool.size();
            pool.push_back(seg);
            order[c].push_back(nu);
            face_segs[face].push_back(nu);
            if (best >= 0) split_segment(best_c, best, pool[nu], best_cd);
        }

        // Mcurv::add_segment_init (motorcycle.h:215-227)
        void add_segment_init(int c) {
            const Mport& p = mports[mcurvs[c].port];
            int h = -1;
            const int h0 = m.face2half[p.face];
            for (int k = 0, g = h0; k < 3; k++, g = m.next[g])
                if (m.head[g] != p.vert && m.tail[g] != p.vert) h = g;
            add_segment(c, p.dir, p.uv, h);
        }

        // get_oppsite_half (hmesh/utilities.h:54-73)
        int opposite_half(complex origin, complex dir, int fr) const {
            const int h0 = m.face2half[m.face[fr]];
            for (int k = 0, h = h0; k < 3; k++, h = m.next[h]) {
                if (h == fr) continue;
                const complex a = mc::sub(corner(m.prev[h]), origin), b = mc::sub(corner(m.next[h]), origin);
                if (mc::cross(a, dir) * mc::cross(b, dir) < 0) return h;
            }
            throw std::runtime_error("MotorcycleGraph: a trace leaves its face through a vertex");
        }

        // Mcurv::add_segment_next (motorcycle.h:230-247)
        void add_segment_next(int c, const VecXi& matching) {
            const Mcurv& cv = mcurvs[c];
            if (cv.intersected) return;
            const int h = m.twin[cv.half];
            const int mt = (m.edge2half[m.edge[h]] == h ? 1 : -1) * matching[m.edge[h]];
            const complex uv0 = mc::lerp(corner(m.next[h]), corner(m.prev[h]), cv.ratio);
            const complex dir = mc::mul(std::polar(1., mc::kPi / 2 * mt), cv.dir);
            add_segment(c, dir, uv0, opposite_half(uv0, dir, h));
        }
    };
}

#endif
