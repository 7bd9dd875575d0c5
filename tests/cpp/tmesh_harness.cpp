// Runs the header-only motorcycle graph and T-mesh (include/metriko/core/tmesh/) on the CPU and
// prints every port, segment, T-edge, T-quad, th2sing and T-edge length.  Input (binary, argv[1]):
// nV, nF, nE (int32), V (nV x 3 doubles), F (nF x 3 int32), cfn (3 nF complex as (re, im) double
// pairs), matching (nE int32), singular (nV int32).  Output (text, argv[2]), doubles as %.17g:
//   P n / p id vert face uv.re uv.im dir.re dir.im next prev
//   C n / c nseg / s face fr.re fr.im fr.crash fr.type to.re to.im to.crash to.type id prev next
//   E n / e curv seg_fr.id seg_to.id          Q n / q count thid side ...
//   S th2sing...                               R length...
// Exit code 5 (message on stderr) when the graph or the T-mesh throws.
#include <cstdio>
#include <fstream>
#include <memory>
#include <stdexcept>

#include "metriko/core/tmesh/tmesh.h"

using namespace metriko;

int main(int argc, char** argv) {
    if (argc < 3) return 2;
    std::ifstream in(argv[1], std::ios::binary);
    int h[3];
    in.read(reinterpret_cast<char*>(h), sizeof(h));
    MatXd V(h[0], 3);
    MatXi F(h[1], 3);
    std::vector<double> c(6 * size_t(h[1]));
    VecXi matching(h[2]), singular(h[0]);
    in.read(reinterpret_cast<char*>(V.data()), sizeof(double) * 3 * h[0]);
    in.read(reinterpret_cast<char*>(F.data()), sizeof(int) * 3 * h[1]);
    in.read(reinterpret_cast<char*>(c.data()), sizeof(double) * c.size());
    in.read(reinterpret_cast<char*>(matching.data()), sizeof(int) * h[2]);
    in.read(reinterpret_cast<char*>(singular.data()), sizeof(int) * h[0]);
    if (!in) return 3;
    auto mesh = std::make_unique<Hmesh>(V, F);
    if (mesh->nE != h[2]) return 4;
    VecXc cfn(3 * size_t(h[1]));
    for (int i = 0; i < 3 * h[1]; i++) cfn[i] = complex(c[2 * size_t(i)], c[2 * size_t(i) + 1]);
    try {
        MotorcycleGraph g(*mesh, cfn, matching, singular);
        Tmesh tm(g);
        VecXd R = tedge_lengths(g, tm);
        FILE* o = std::fopen(argv[2], "w");
        if (!o) return 6;
        std::fprintf(o, "P %zu\n", g.mports.size());
        for (const Mport& p : g.mports)
            std::fprintf(o, "p %d %d %d %.17g %.17g %.17g %.17g %d %d\n", p.id, p.vert, p.face, p.uv.real(), p.uv.imag(),
                         p.dir.real(), p.dir.imag(), p.next, p.prev);
        std::fprintf(o, "C %zu\n", g.mcurvs.size());
        for (const Mcurv& cv : g.mcurvs) {
            std::fprintf(o, "c %zu\n", cv.sgmts.size());
            for (const Msgmt& s : cv.sgmts)
                std::fprintf(o, "s %d %.17g %.17g %d %d %.17g %.17g %d %d %d %d %d\n", s.face, s.fr.uv.real(), s.fr.uv.imag(),
                             s.fr.crash, (int)s.fr.type, s.to.uv.real(), s.to.uv.imag(), s.to.crash, (int)s.to.type, s.id,
                             s.prev_id, s.next_id);
        }
        std::fprintf(o, "E %zu\n", tm.nTE);
        for (const Tedge& te : tm.tedges) std::fprintf(o, "e %d %d %d\n", te.curv, te.seg_fr.id, te.seg_to.id);
        std::fprintf(o, "Q %zu\n", tm.nTQ);
        for (const Tquad& q : tm.tquads) {
            std::fprintf(o, "q %zu", q.thids.size());
            for (size_t i = 0; i < q.thids.size(); i++) std::fprintf(o, " %d %d", q.thids[i], q.sides[i]);
            std::fprintf(o, "\n");
        }
        std::fprintf(o, "S");
        for (size_t i = 0; i < tm.nTH; i++) std::fprintf(o, " %d", tm.th2sing[i]);
        std::fprintf(o, "\nR");
        for (size_t i = 0; i < tm.nTE; i++) std::fprintf(o, " %.17g", R[i]);
        std::fprintf(o, "\n");
        std::fclose(o);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 5;
    }
    return 0;
}
