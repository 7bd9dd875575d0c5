//
// Restates parts of metriko (https://github.com/komietty/metriko),
// Copyright (C) 2025 Saki Komikado <komietty@gmail.com>.
// This Source Code Form is subject to the terms of the Mozilla Public License v.2.0
// (https://mozilla.org/MPL/2.0/).
//
// metriko-gb300: T-mesh of a motorcycle graph (host only).
//
// Replaces metriko include/metriko/core/tmesh/tmesh.h:11-305.  A T-edge runs along one trace
// from a crash point (or the trace's start at its singular vertex) to the next crash point; it
// has two T-half-edges (the canonical one along the trace first).  T-quads are the cycles of
// choose_next_thalf, which at a crash point turns onto the trace that was hit (a side change)
// and otherwise continues along the same trace; each quad's half-edges carry their side 0-3 and
// the list is rotated so that it does not start in the middle of a side.  th2sing marks the
// half-edge at the start of each trace with its singular vertex.  Same tables, same order as
// the reference; T-half-edges and T-edges are values that point back into their Tmesh, which is
// therefore neither copied nor moved.  tedge_lengths gives the uv length of every T-edge (the
// quantity quantization targets, example/example_qgp.cpp:84-94).
//
#ifndef METRIKO_TMESH_H
#define METRIKO_TMESH_H
#include <algorithm>
#include <stdexcept>
#include <utility>
#include <vector>

#include "motorcycle.h"

namespace metriko {
    class Tmesh;

    struct Tedge {
        int id = -1;
        int curv = -1;             // the trace the T-edge runs along
        Msgmt seg_fr, seg_to;      // its first and last segments
        complex uv_fr() const { return seg_fr.fr.uv; }
        complex uv_to() const { return seg_to.to.uv; }
        MvertType type_fr() const { return seg_fr.fr.type; }
        MvertType type_to() const { return seg_to.to.type; }
    };

    struct Thalf {
        const Tmesh* tmesh = nullptr;
        int id = -1;
        int teid = -1;
        int twid = -1;
        bool cannonical = true;

        bool operator==(const Thalf& o) const {
            return id == o.id && twid == o.twid && teid == o.teid && cannonical == o.cannonical;
        }
        const Thalf& twin() const;
        const Thalf& next() const;
        const Thalf& prev() const;
        const Tedge& edge() const;
        complex uv_fr() const { return cannonical ? edge().uv_fr() : edge().uv_to(); }
        complex uv_to() const { return cannonical ? edge().uv_to() : edge().uv_fr(); }
        const Msgmt& sg_fr() const { return cannonical ? edge().seg_fr : edge().seg_to; }
        const Msgmt& sg_to() const { return cannonical ? edge().seg_to : edge().seg_fr; }
        complex dif_fr() const { return sg_fr().diff() * (cannonical ? 1. : -1.); }
        complex dif_to() const { return sg_to().diff() * (cannonical ? 1. : -1.); }
        std::vector<Thalf> adj_thalfs() const;
    };

    struct Tquad {
        int id = -1;
        std::vector<int> thids;
        std::vector<int> sides;

        int find_first_thid(int side) const {
            for (size_t i = 0; i < sides.size(); i++) if (sides[i] == side) return thids[i];
            return -1;
        }
        int find_side(const Thalf& th) const {
            for (size_t i = 0; i < thids.size(); i++) if (thids[i] == th.id) return sides[i];
            return -1;
        }
        std::vector<int> thids_by_side(int side, bool reverse = false) const {
            std::vector<int> r;
            const int n = (int)thids.size();
            for (int i = 0; i < n; i++) {
                const int j = reverse ? n - i - 1 : i;
                if (sides[j] == side) r.push_back(thids[j]);
            }
            return r;
        }
    };

    class Tmesh {
    public:
        std::vector<Tquad> tquads;
        std::vector<Thalf> thalfs;
        std::vector<Tedge> tedges;
        VecXi th2sing;   // the singular vertex a trace starts from, on its first half-edge; else -1
        VecXi th2quad;
        VecXi th2side;
        VecXi th2iter;
        size_t nTQ = 0, nTE = 0, nTH = 0;

        explicit Tmesh(const MotorcycleGraph& g) : graph(&g) {
            const std::vector<Mcurv>& mcurvs = g.mcurvs;
            for (int c = 0; c < (int)mcurvs.size(); c++) {   // tmesh.h:162-173
                const Mcurv& cv = mcurvs[c];
                if (cv.sgmts.empty()) continue;
                Msgmt start = cv.sgmts.front();
                for (const Msgmt& s : cv.sgmts) {
                    if (s.to.type == None) continue;
                    const int k = (int)tedges.size();
                    tedges.push_back(Tedge{k, c, start, s});
                    thalfs.push_back(Thalf{this, 2 * k, k, 2 * k + 1, true});
                    thalfs.push_back(Thalf{this, 2 * k + 1, k, 2 * k, false});
                    if (s.next_id != -1) start = cv.sgmts[s.next_id];
                }
            }
            nTE = tedges.size();
            nTH = thalfs.size();
            std::vector<char> visit(nTH, 0);
            for (size_t first = 0; first < nTH; first++) {   // tmesh.h:175-183
                if (visit[first]) continue;
                Tquad q;
                q.id = (int)tquads.size();
                int side = 0, cur = (int)first;
                size_t guard = 0;
                do {
                    q.thids.push_back(cur);
                    q.sides.push_back(side);
                    const auto [nx, turn] = choose_next_thalf(cur);
                    if (turn) side = (side + 1) % 4;
                    cur = nx;
                    if (++guard > nTH + 4) throw std::runtime_error("Tmesh: a T-quad walk does not close");
                } while (cur != (int)first);
                if (q.sides.front() == q.sides.back()) {   // do not start in the middle of a side
                    const int s0 = q.sides.front();
                    size_t n = 0;
                    while (n < q.sides.size() && q.sides[n] == s0) n++;
                    std::rotate(q.sides.begin(), q.sides.begin() + n, q.sides.end());
                    std::rotate(q.thids.begin(), q.thids.begin() + n, q.thids.end());
                }
                if (q.sides.front() == q.sides.back()) throw std::runtime_error("Tmesh: a T-quad with one side");
                for (int t : q.thids) visit[t] = 1;
                tquads.push_back(std::move(q));
            }
            nTQ = tquads.size();
            th2side = VecXi(nTH, 0);
            th2quad = VecXi(nTH, 0);
            th2iter = VecXi(nTH, 0);
            th2sing = VecXi(nTH, -1);
            for (size_t i = 0; i < nTQ; i++)
                for (size_t j = 0; j < tquads[i].thids.size(); j++) {
                    const int t = tquads[i].thids[j];
                    th2quad[t] = (int)i;
                    th2side[t] = tquads[i].sides[j];
                    th2iter[t] = (int)j;
                }
            for (const Mcurv& cv : mcurvs) {   // tmesh.h:199-204
                if (cv.sgmts.empty()) continue;
                for (const Thalf& th : thalfs)
                    if (th.edge().seg_fr == cv.sgmts.front()) { th2sing[th.id] = g.mports[cv.port].vert; break; }
            }
        }
        Tmesh(const Tmesh&) = delete;
        Tmesh& operator=(const Tmesh&) = delete;

        int next_thid(int cur) const {
            const Tquad& q = tquads[th2quad[cur]];
            return q.thids[(th2iter[cur] + 1) % q.thids.size()];
        }
        int prev_thid(int cur) const {
            const Tquad& q = tquads[th2quad[cur]];
            return q.thids[(th2iter[cur] - 1 + q.thids.size()) % q.thids.size()];
        }

    private:
        const MotorcycleGraph* graph;

        // the first half-edge (by id) with the given orientation whose T-edge starts or ends at ms
        int find_th(const Msgmt& ms, bool cannonical) const {
            for (const Thalf& th : thalfs) {
                const Tedge& te = tedges[th.teid];
                if (th.cannonical == cannonical && (te.seg_fr == ms || te.seg_to == ms)) return th.id;
            }
            throw std::runtime_error("Tmesh: T-half-edge not found");
        }

        // Tquad::choose_next_thalf (tmesh.h:260-305): the next half-edge of the quad and whether
        // the walk turns a corner there
        std::pair<int, bool> choose_next_thalf(int cur) const {
            const std::vector<Mcurv>& mcurvs = graph->mcurvs;
            const Thalf& th = thalfs[cur];
            const Tedge& te = tedges[th.teid];
            if (th.cannonical) {
                if (te.type_to() == HitB) {
                    const complex uv2 = te.seg_to.to.uv;
                    const complex dif = te.seg_to.diff();
                    for (const Msgmt& ms : mcurvs[te.seg_to.to.crash].sgmts) {
                        if (ms.face != te.seg_to.face) continue;
                        if (mc::equal(ms.fr.uv, uv2) && mc::cross(dif, ms.diff()) > 0) return {find_th(ms, true), true};
                        if (mc::equal(ms.to.uv, uv2) && mc::cross(dif, -ms.diff()) > 0) return {find_th(ms, false), true};
                    }
                    throw std::runtime_error("Tmesh: T-half-edge not found");
                }
                if (te.type_to() == HitR) return {find_th(mcurvs[te.seg_to.to.crash].sgmts.back(), false), true};
                return {cur + 2, false};
            }
            const Mcurv& own = mcurvs[te.seg_fr.curv];
            if (te.seg_fr == own.sgmts.front()) {
                const Mcurv& c = mcurvs[graph->mports[own.port].prev];
                return {find_th(c.sgmts.front(), true), true};
            }
            if (te.type_fr() == HitR) return {find_th(mcurvs[te.seg_fr.fr.crash].sgmts.back(), false), true};
            return {cur - 2, false};
        }
    };

    inline const Tedge& Thalf::edge() const { return tmesh->tedges[teid]; }
    inline const Thalf& Thalf::twin() const { return tmesh->thalfs[twid]; }
    inline const Thalf& Thalf::next() const { return tmesh->thalfs[tmesh->next_thid(id)]; }
    inline const Thalf& Thalf::prev() const { return tmesh->thalfs[tmesh->prev_thid(id)]; }

    // Thalf::adj_thalfs (tmesh.h:236-257)
    inline std::vector<Thalf> Thalf::adj_thalfs() const {
        std::vector<Thalf> res;
        const MvertType type = cannonical ? sg_to().to.type : sg_to().fr.type;
        const Thalf& nx = next();
        const Thalf& tw = twin();
        switch (type) {
            case HitR:
                res.push_back(nx);
                res.push_back(nx.twin().next());
                break;
            case HitB:
            case HitL:
                res.push_back(nx);
                res.push_back(tw.prev().twin());
                break;
            default:;
        }
        return res;
    }

    // uv length of every T-edge: the sum of |segment| from its first to its last segment along
    // its trace (example/example_qgp.cpp:84-94)
    inline VecXd tedge_lengths(const MotorcycleGraph& g, const Tmesh& tm) {
        VecXd R = VecXd::Zero(tm.nTE);
        for (size_t i = 0; i < tm.nTE; i++) {
            const Tedge& te = tm.tedges[i];
            bool on = false;
            for (const Msgmt& s : g.mcurvs[te.curv].sgmts) {
                if (s == te.seg_fr) on = true;
                if (on) {
                    R[i] += std::abs(s.diff());
                    if (s == te.seg_to) break;
                }
            }
        }
        return R;
    }
}

#endif
