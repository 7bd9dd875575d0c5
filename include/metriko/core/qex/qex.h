//
// Restates parts of metriko (https://github.com/komietty/metriko),
// Copyright (C) 2025 Saki Komikado <komietty@gmail.com>.
// This Source Code Form is subject to the terms of the Mozilla Public License v.2.0
// (https://mozilla.org/MPL/2.0/).
//
// metriko-gb300: quad extraction (QEx) from a seamless integer-grid map (host only).
//
// Replaces metriko include/metriko/core/qex/common.h:8-147, sanitization.h:11-56,
// gen_q_vert.h:11-59, gen_q_port.h:11-108, gen_q_edge.h:11-121 and gen_q_face.h:8-40, with
// calc_coefficient / conversion_2d_3d of core/common/utilities.h:109-123 and
// core/hmesh/utilities.h:23-52, called in the order of example/example_qex.cpp:125-205:
//   sanitization            snap each vertex's first corner (to the grid at a singular vertex,
//                           to the precision of its largest coordinate elsewhere) and transport
//                           it around the vertex by the edge transitions
//   generate_q_vert         integer grid points at vertices, on edges and inside faces
//   generate_*_qport        the axis directions leaving each grid point (four at edge and face
//                           points, one per sector at vertices), linked in a ring
//   generate_q_edge         from every port, the grid line across faces (uv mapped by the
//                           transition of each edge it crosses) to the port facing it
//   generate_q_faces        quads: from each q-half-edge, three turns to the previous port
//   quad_soup               the example's output: four corner positions per quad
// Same results as the reference (compiled without floating-point contraction, bit for bit):
// the same expressions (std::round, the 2x2 cofactor inverse, sqrt of the sum of squares),
// the same visiting orders and first-match rules.  Differences in form: q-edges and q-half-edges
// hold port indices where the reference holds references; the port searches run over per-face,
// per-edge and per-vertex buckets in index order (the reference filters the whole list); a grid
// line that does not reach a port within a bounded number of faces, a missing face port and an
// edge point with other than four ports stop with std::runtime_error (the reference loops or
// asserts).  Closed meshes (the reference throws at a boundary crossing).
//
#ifndef METRIKO_QEX_H
#define METRIKO_QEX_H
#include <cmath>
#include <stdexcept>
#include <vector>

#include "metriko/core/tmesh/motorcycle.h"

namespace metriko::qex {
    constexpr double EPS = 1e-9;

    struct Qvert {
        complex uv;
        Row3d pos;
        int sid = -1;   // the vertex, edge or face it lies on
    };

    struct Qport {
        int idx = -1;
        int vid = -1;
        int eid = -1;
        int fid = -1;
        complex uv;
        complex dir;
        Row3d pos;
        bool isConnected = false;
        int next_id = -1;
        int prev_id = -1;
    };

    struct Qedge {
        int port1 = -1, port2 = -1;   // indices into the ports
    };

    struct Qhalf {
        int edge = -1;
        int idx = -1;
        bool cannonical = true;
        int p1 = -1, p2 = -1;
        int port1() const { return p1; }
        int port2() const { return p2; }
    };

    struct Qface {
        std::vector<Qhalf> qhalfs;
    };

    // ---------------------------------------------------------------- common.h
    inline double orientation(complex pa, complex pb, complex pc) {
        const double acx = pa.real() - pc.real(), bcx = pb.real() - pc.real();
        const double acy = pa.imag() - pc.imag(), bcy = pb.imag() - pc.imag();
        return acx * bcy - acy * bcx;
    }
    inline bool is_collinear(complex pa, complex pb, complex pc) { return std::abs(orientation(pa, pb, pc)) < EPS; }
    inline bool is_points_into(complex p1, complex p2, complex p3, complex uv) {
        return orientation(p1, p2, uv) > EPS && orientation(p1, p3, uv) < EPS;
    }
    inline bool is_inside_triangle(complex pa, complex pb, complex pc, complex uv) {
        return orientation(pa, pb, uv) > EPS && orientation(pb, pc, uv) > EPS && orientation(pc, pa, uv) > EPS;
    }
    inline complex nearby_grid(complex a) { return {std::round(a.real()), std::round(a.imag())}; }
    inline double nearby_grid(double x, double dir) {
        if (dir == 0) return x;
        const double f = std::abs(std::fmod(x, 1.));
        if (f < EPS || 1 - f < EPS) x += dir * EPS;
        return dir > 0 ? std::ceil(x) : std::floor(x);
    }
    inline complex nearby_grid(complex uv, complex dir) {
        return {nearby_grid(uv.real(), dir.real()), nearby_grid(uv.imag(), dir.imag())};
    }

    // calc_coefficient + conversion_2d_3d: uv -> the point of the triangle (o, a, b) in 3D
    inline Row3d conversion_2d_3d(complex o2, complex a2, complex b2, const Row3d& o3, const Row3d& a3, const Row3d& b3,
                                  complex uv) {
        const complex v1 = mc::sub(a2, o2), v2 = mc::sub(b2, o2), d = mc::sub(uv, o2);
        const double m00 = v1.real(), m01 = v2.real(), m10 = v1.imag(), m11 = v2.imag();
        const double inv = 1.0 / (m00 * m11 - m10 * m01);
        const double i00 = m11 * inv, i10 = -m10 * inv, i01 = -m01 * inv, i11 = m00 * inv;
        const double c0 = i00 * d.real() + i01 * d.imag(), c1 = i10 * d.real() + i11 * d.imag();
        return o3 + (a3 - o3) * c0 + (b3 - o3) * c1;
    }

    namespace detail {
        inline int cvert(const Hmesh& m, int c) { return m.idx(c / 3, c % 3); }
        inline Row3d vpos(const Hmesh& m, int v) { return Row3d(m.pos(v, 0), m.pos(v, 1), m.pos(v, 2)); }
        inline Row3d conversion_face(const Hmesh& m, const VecXc& cfn, int f, complex uv) {
            const int h = m.face2half[f];
            const int c1 = m.crnr[h], c2 = m.crnr[m.next[h]], c3 = m.crnr[m.prev[h]];
            return conversion_2d_3d(cfn[c1], cfn[c2], cfn[c3], vpos(m, cvert(m, c1)), vpos(m, cvert(m, c2)),
                                    vpos(m, cvert(m, c3)), uv);
        }
        template <typename Fn>
        inline void vert_ring(const Hmesh& m, int v, Fn fn) {
            const int h0 = m.vert2half[v];
            int h = h0;
            do {
                fn(h);
                h = m.twin[m.prev[h]];
            } while (h != h0);
        }
    }

    // compute_trs_matrix (common.h:72-89): per halfedge, the rotation r and integer translation t
    // of the map uv -> r uv + t from its face to its twin's
    inline void compute_trs_matrix(const Hmesh& m, const VecXc& cfn, const VecXi& matching, int rosyN, VecXc& heR,
                                   VecXc& heT) {
        heR = VecXc(m.nH);
        heT = VecXc(m.nH);
        for (int h = 0; h < m.nH; h++) {
            const complex uv1 = cfn[m.crnr[m.next[h]]], uv2 = cfn[m.crnr[m.prev[m.twin[h]]]];
            int mm = (m.edge2half[m.edge[h]] == h ? 1 : -1) * matching[m.edge[h]];
            mm = mm < 0 ? (rosyN + mm % rosyN) % rosyN : mm % rosyN;
            const complex r = mc::quater_rot(mm);
            const complex t = mc::sub(uv2, mc::mul(r, uv1));
            heR[h] = r;
            heT[h] = complex(std::round(t.real()), std::round(t.imag()));
        }
    }

    // sanitization (sanitization.h:11-56)
    inline void sanitization(const Hmesh& m, const VecXi& matching, const VecXi& singular, int rosyN, VecXc& cfn) {
        if (m.nL > 0) throw std::invalid_argument("qex: meshes with boundary are not supported");
        VecXc heR, heT;
        compute_trs_matrix(m, cfn, matching, rosyN, heR, heT);
        for (int v = 0; v < m.nV; v++) {
            double mx = 0;
            detail::vert_ring(m, v, [&](int h) {
                const complex uv = cfn[m.crnr[m.next[h]]];
                mx = std::max(mx, std::abs(uv.real()));
                mx = std::max(mx, std::abs(uv.imag()));
            });
            bool init = false;
            detail::vert_ring(m, v, [&](int h) {
                const int cc = m.crnr[m.next[h]];
                if (!init) {
                    const complex uv = cfn[cc];
                    if (singular[v]) {
                        cfn[cc] = complex(std::round(uv.real()), std::round(uv.imag()));
                    } else {
                        const double delta = std::pow(2.0, std::log2(mx));
                        const complex ds((double)((0 < uv.real()) - (uv.real() < 0)) * delta,
                                         (double)((0 < uv.imag()) - (uv.imag() < 0)) * delta);
                        cfn[cc] = mc::sub(mc::add(cfn[cc], ds), ds);
                    }
                } else {
                    const int tw = m.twin[h];
                    cfn[cc] = mc::add(mc::mul(heR[tw], cfn[m.crnr[m.prev[tw]]]), heT[tw]);
                }
                init = true;
            });
        }
    }

    // generate_q_vert (gen_q_vert.h:11-59)
    inline void generate_q_vert(const Hmesh& m, const VecXc& cfn, std::vector<Qvert>& vqvs, std::vector<Qvert>& eqvs,
                                std::vector<Qvert>& fqvs) {
        for (int v = 0; v < m.nV; v++) {   // checks one corner, as the reference
            const complex uv = cfn[m.crnr[m.next[m.vert2half[v]]]];
            const double x = std::fmod(std::abs(uv.real()), 1.), y = std::fmod(std::abs(uv.imag()), 1.);
            if ((x < EPS || 1 - x < EPS) && (y < EPS || 1 - y < EPS)) vqvs.push_back(Qvert{complex(x, y), detail::vpos(m, v), v});
        }
        for (int e = 0; e < m.nE; e++) {
            const int h = m.edge2half[e];
            const Row3d p1 = detail::vpos(m, m.tail[h]), p2 = detail::vpos(m, m.head[h]);
            const complex uv1 = cfn[m.crnr[m.next[h]]], uv2 = cfn[m.crnr[m.prev[h]]];
            const int x0 = (int)std::floor(std::min(uv1.real(), uv2.real())), y0 = (int)std::floor(std::min(uv1.imag(), uv2.imag()));
            const int x1 = (int)std::ceil(std::max(uv1.real(), uv2.real())), y1 = (int)std::ceil(std::max(uv1.imag(), uv2.imag()));
            for (int x = x0; x <= x1; x++)
                for (int y = y0; y <= y1; y++) {
                    const complex xy(x, y);
                    const double a = std::abs(mc::sub(xy, uv1)) / std::abs(mc::sub(uv2, uv1));
                    if (is_collinear(uv1, uv2, xy) && a > EPS && a < 1 - EPS) eqvs.push_back(Qvert{xy, p1 + (p2 - p1) * a, e});
                }
        }
        for (int f = 0; f < m.nF; f++) {
            const Row3d p1 = detail::vpos(m, m.idx(f, 0)), p2 = detail::vpos(m, m.idx(f, 1)), p3 = detail::vpos(m, m.idx(f, 2));
            const complex uv1 = cfn[3 * f], uv2 = cfn[3 * f + 1], uv3 = cfn[3 * f + 2];
            const int x0 = (int)std::floor(std::min({uv1.real(), uv2.real(), uv3.real()}));
            const int y0 = (int)std::floor(std::min({uv1.imag(), uv2.imag(), uv3.imag()}));
            const int x1 = (int)std::ceil(std::max({uv1.real(), uv2.real(), uv3.real()}));
            const int y1 = (int)std::ceil(std::max({uv1.imag(), uv2.imag(), uv3.imag()}));
            for (int x = x0; x <= x1; x++)
                for (int y = y0; y <= y1; y++) {
                    const complex xy(x, y);
                    if (is_inside_triangle(uv1, uv2, uv3, xy))
                        fqvs.push_back(Qvert{xy, conversion_2d_3d(uv1, uv2, uv3, p1, p2, p3, xy), f});
                }
        }
    }

    namespace detail {
        inline void link_ring(std::vector<Qport>& tmp, std::vector<Qport>& qports) {
            const int s = (int)tmp.size();
            for (int i = 0; i < s; i++) tmp[i].idx = (int)qports.size() + i;
            for (int i = 0; i < s; i++) {
                tmp[i].prev_id = tmp[(i - 1 + s) % s].idx;
                tmp[i].next_id = tmp[(i + 1) % s].idx;
            }
            qports.insert(qports.end(), tmp.begin(), tmp.end());
        }
        inline int first_into(complex uv1, complex uv2, complex uv3) {
            int r;
            for (r = 0; r < 4; r++)
                if (is_points_into(uv1, uv2, uv3, mc::add(uv1, mc::quater_rot(r)))) break;
            return r;
        }
    }

    // generate_vqvert_qport (gen_q_port.h:79-108)
    inline void generate_vqvert_qport(const Hmesh& m, const VecXc& cfn, const std::vector<Qvert>& vqverts,
                                      std::vector<Qport>& qports) {
        for (const Qvert& qv : vqverts) {
            std::vector<Qport> tmp;
            detail::vert_ring(m, qv.sid, [&](int h) {
                const complex uv1 = cfn[m.crnr[m.next[h]]], uv2 = cfn[m.crnr[m.prev[h]]], uv3 = cfn[m.crnr[h]];
                const int r = detail::first_into(uv1, uv2, uv3);
                for (int i = 0; i < 4; i++) {
                    const complex d = mc::quater_rot((r + i + 3) % 4);
                    const bool f1 = is_points_into(uv1, uv2, uv3, mc::add(uv1, d));
                    const bool f2 = is_collinear(uv1, uv2, mc::add(uv1, d));
                    const bool f3 = mc::dot(mc::sub(uv2, uv1), d) > 0;
                    if (f1 || (f2 && f3)) {
                        Qport p;
                        p.vid = qv.sid;
                        p.fid = m.face[h];
                        p.uv = uv1;
                        p.dir = d;
                        p.pos = qv.pos;
                        tmp.push_back(p);
                    }
                }
            });
            detail::link_ring(tmp, qports);
        }
    }

    // generate_eqvert_qport (gen_q_port.h:11-56); the visited directions are shared by every edge
    // point, as in the reference
    inline void generate_eqvert_qport(const Hmesh& m, const VecXc& cfn, const std::vector<Qvert>& eqverts,
                                      std::vector<Qport>& qports) {
        std::vector<Row3d> visit;
        for (const Qvert& qv : eqverts) {
            std::vector<Qport> tmp;
            const int e = qv.sid;
            const int h0 = m.edge2half[e];
            for (const int h : {h0, m.twin[h0]}) {
                const int c1 = m.crnr[m.next[h]], c2 = m.crnr[m.prev[h]];
                const complex uv1 = cfn[c1], uv2 = cfn[c2], uv3 = cfn[m.crnr[h]];
                const Row3d p1 = detail::vpos(m, detail::cvert(m, c1)), p2 = detail::vpos(m, detail::cvert(m, c2));
                const complex uv = mc::lerp(uv1, uv2, (qv.pos - p1).norm() / (p2 - p1).norm());
                const int r = detail::first_into(uv1, uv2, uv3);
                for (int i = 0; i < 4; i++) {
                    const complex dir = mc::quater_rot((r + i + 2) % 4);
                    const bool f1 = orientation(uv1, uv2, mc::add(uv, dir)) >= 0;
                    const Row3d ev = detail::conversion_face(m, cfn, m.face[h], mc::add(uv, dir)).normalized();
                    bool seen = false;
                    for (const Row3d& w : visit)
                        if ((ev - w).norm() < EPS) { seen = true; break; }
                    if (f1 && !seen) {
                        Qport p;
                        p.eid = e;
                        p.fid = m.face[h];
                        p.uv = nearby_grid(uv);
                        p.dir = dir;
                        p.pos = qv.pos;
                        tmp.push_back(p);
                        visit.push_back(ev);
                    }
                }
            }
            if (tmp.size() != 4) throw std::runtime_error("qex: an edge grid point without four ports");
            detail::link_ring(tmp, qports);
        }
    }

    // generate_fqvert_qport (gen_q_port.h:58-77)
    inline void generate_fqvert_qport(const Hmesh& m, const std::vector<Qvert>& fqverts, std::vector<Qport>& qports) {
        (void)m;
        for (const Qvert& qv : fqverts) {
            std::vector<Qport> tmp(4);
            for (int i = 0; i < 4; i++) {
                tmp[i].fid = qv.sid;
                tmp[i].uv = qv.uv;
                tmp[i].dir = mc::quater_rot(i);
                tmp[i].pos = qv.pos;
            }
            detail::link_ring(tmp, qports);
        }
    }

    namespace detail {
        // predict_extrinsic_collinear (gen_q_edge.h:11-27)
        inline bool collinear_pair(const Hmesh& m, const VecXc& cfn, complex ori, complex dir, int face, const Qport& pair) {
            const Row3d pb1 = conversion_face(m, cfn, face, ori);
            const Row3d pb2 = conversion_face(m, cfn, face, mc::add(ori, dir));
            const Row3d pa1 = conversion_face(m, cfn, pair.fid, pair.uv);
            const Row3d pa2 = conversion_face(m, cfn, pair.fid, mc::add(pair.uv, pair.dir));
            const Row3d da = (pa2 - pa1).normalized(), db = (pb2 - pb1).normalized(), dc = (pa1 - pb1).normalized();
            return std::abs(1. - db.dot(dc)) < EPS && std::abs(1. + da.dot(db)) < EPS;
        }
    }

    // generate_q_edge (gen_q_edge.h:45-121)
    inline std::vector<Qedge> generate_q_edge(const Hmesh& m, const VecXc& cfn, const VecXi& matching,
                                              std::vector<Qport>& qports, long long max_steps = -1) {
        std::vector<Qedge> qedges;
        VecXc heR, heT;
        compute_trs_matrix(m, cfn, matching, 4, heR, heT);
        std::vector<std::vector<int>> by_face(m.nF), by_edge(m.nE), by_vert(m.nV);
        for (const Qport& p : qports) {
            by_face[p.fid].push_back(p.idx);
            if (p.eid >= 0) by_edge[p.eid].push_back(p.idx);
            if (p.vid >= 0) by_vert[p.vid].push_back(p.idx);
        }
        const long long cap = max_steps > 0 ? max_steps : 4LL * m.nF + 16;
        for (Qport& pfr : qports) {
            if (pfr.isConnected) continue;
            complex ori = pfr.uv, dir = pfr.dir;
            complex gri = nearby_grid(ori, dir);
            int f = pfr.fid;
            for (long long step = 0;; step++) {
                int hit = -1;
                if (is_inside_triangle(cfn[3 * f], cfn[3 * f + 1], cfn[3 * f + 2], gri)) {   // face port
                    const complex nd = -dir;
                    for (int q : by_face[f]) {
                        const Qport& p = qports[q];
                        if (p.idx == pfr.idx) continue;
                        if (mc::equal(p.dir, nd) && std::abs(mc::sub(p.uv, gri)) < EPS) { hit = q; break; }
                    }
                    if (hit < 0) throw std::runtime_error("qex: face port not found");
                }
                for (int k = 0, h = m.face2half[f]; hit < 0 && k < 3; k++, h = m.next[h])   // edge port
                    for (int q : by_edge[m.edge[h]]) {
                        const Qport& p = qports[q];
                        if (p.isConnected || p.eid == pfr.eid) continue;
                        if (detail::collinear_pair(m, cfn, ori, dir, f, p)) { hit = q; break; }
                    }
                for (int k = 0, h = m.face2half[f]; hit < 0 && k < 3; k++, h = m.next[h])   // vertex port
                    for (int q : by_vert[m.tail[h]]) {
                        const Qport& p = qports[q];
                        if (p.isConnected || p.vid == pfr.vid) continue;
                        if (detail::collinear_pair(m, cfn, ori, dir, f, p)) { hit = q; break; }
                    }
                if (hit >= 0) {
                    pfr.isConnected = true;
                    qports[hit].isConnected = true;
                    qedges.push_back(Qedge{pfr.idx, hit});
                    break;
                }
                // pick_next_half (gen_q_edge.h:29-43): the edge the grid line leaves through
                int nh = -1;
                complex pt;
                for (int k = 0, h = m.face2half[f]; k < 3; k++, h = m.next[h]) {
                    const complex uv1 = cfn[m.crnr[m.next[h]]], uv2 = cfn[m.crnr[m.prev[h]]];
                    double rab = 0, rcd = 0;
                    if (mc::strict_intersection(ori, mc::add(ori, dir * 1e2), uv1, uv2, rab, rcd) && rab > EPS) {
                        nh = h;
                        pt = mc::lerp(uv1, uv2, rcd);
                        break;
                    }
                }
                if (nh < 0) throw std::runtime_error("qex: no next half found");
                f = m.face[m.twin[nh]];
                ori = mc::add(mc::mul(heR[nh], pt), heT[nh]);
                dir = mc::mul(heR[nh], dir);
                gri = nearby_grid(ori, dir);
                if (step + 1 > cap) throw std::runtime_error("qex: a grid line reaches no port");
            }
        }
        return qedges;
    }

    // generate_q_faces (gen_q_face.h:8-40)
    inline std::vector<Qface> generate_q_faces(const std::vector<Qport>& qps, const std::vector<Qedge>& qes) {
        std::vector<Qhalf> qhs;
        for (int i = 0; i < (int)qes.size(); i++) {
            qhs.push_back(Qhalf{i, 2 * i, true, qes[i].port1, qes[i].port2});
            qhs.push_back(Qhalf{i, 2 * i + 1, false, qes[i].port2, qes[i].port1});
        }
        std::vector<int> by_start(qps.size(), -1);   // the first half starting at each port
        for (const Qhalf& qh : qhs)
            if (by_start[qh.p1] < 0) by_start[qh.p1] = qh.idx;
        std::vector<char> visit(qhs.size(), 0);
        std::vector<Qface> qfs;
        for (size_t k0 = 0; k0 < qhs.size(); k0++) {
            if (visit[k0]) continue;
            Qface qf;
            qf.qhalfs.push_back(qhs[k0]);
            visit[k0] = 1;
            int qp = qhs[k0].p2;
            for (int i = 0; i < 3; i++) {
                const int k = by_start[qps[qp].prev_id];
                if (k < 0) break;
                qf.qhalfs.push_back(qhs[k]);
                visit[k] = 1;
                qp = qhs[k].p2;
            }
            if (qf.qhalfs.size() == 4) qfs.push_back(std::move(qf));
        }
        return qfs;
    }

    // example_qex.cpp:231-240: four corner positions per quad (rows 4 i + j), faces (i: 4i..4i+3)
    inline void quad_soup(const std::vector<Qport>& qps, const std::vector<Qface>& qfs, MatXd& pos, MatXi& idx) {
        const int l = (int)qfs.size();
        pos = MatXd(4 * l, 3);
        idx = MatXi(l, 4);
        for (int i = 0; i < l; i++)
            for (int j = 0; j < 4; j++) {
                const Row3d& p = qps[qfs[i].qhalfs[j].port1()].pos;
                for (int k = 0; k < 3; k++) pos(4 * i + j, k) = p[k];
                idx(i, j) = 4 * i + j;
            }
    }
}

#endif
