// Runs the header-only quad extraction (include/metriko/core/qex/qex.h) on the CPU in the order
// of the reference's example_qex.cpp and prints every stage.  Input (binary, argv[1]): nV, nF, nE
// (int32), V (nV x 3 doubles), F (nF x 3 int32), cfn (3 nF complex as (re, im) pairs), matching
// (nE int32), singular (nV int32).  Output (text, argv[2]), doubles as %.17g:
//   U (3 nF sanitized corner values re im ...)
//   G kind n / g uv.re uv.im pos.x pos.y pos.z sid         (kind v, e, f)
//   P n / p idx vid eid fid uv.re uv.im dir.re dir.im pos.x pos.y pos.z next prev connected
//   E n / e port1 port2             Q n / q port1 port1 port1 port1 (of the four half-edges)
// Exit code 5 (message on stderr) when a stage throws.
#include <cstdio>
#include <fstream>
#include <memory>
#include <stdexcept>

#include "metriko/core/qex/qex.h"

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
        qex::sanitization(*mesh, matching, singular, 4, cfn);
        std::vector<qex::Qvert> vq, eq, fq;
        qex::generate_q_vert(*mesh, cfn, vq, eq, fq);
        std::vector<qex::Qport> ports;
        qex::generate_vqvert_qport(*mesh, cfn, vq, ports);
        qex::generate_eqvert_qport(*mesh, cfn, eq, ports);
        qex::generate_fqvert_qport(*mesh, fq, ports);
        auto edges = qex::generate_q_edge(*mesh, cfn, matching, ports);
        auto faces = qex::generate_q_faces(ports, edges);
        FILE* o = std::fopen(argv[2], "w");
        if (!o) return 6;
        std::fprintf(o, "U");
        for (int i = 0; i < cfn.size(); i++) std::fprintf(o, " %.17g %.17g", cfn[i].real(), cfn[i].imag());
        std::fprintf(o, "\n");
        const std::vector<qex::Qvert>* groups[3] = {&vq, &eq, &fq};
        const char kinds[3] = {'v', 'e', 'f'};
        for (int k = 0; k < 3; k++) {
            std::fprintf(o, "G %c %zu\n", kinds[k], groups[k]->size());
            for (const qex::Qvert& q : *groups[k])
                std::fprintf(o, "g %.17g %.17g %.17g %.17g %.17g %d\n", q.uv.real(), q.uv.imag(), q.pos[0], q.pos[1], q.pos[2], q.sid);
        }
        std::fprintf(o, "P %zu\n", ports.size());
        for (const qex::Qport& p : ports)
            std::fprintf(o, "p %d %d %d %d %.17g %.17g %.17g %.17g %.17g %.17g %.17g %d %d %d\n", p.idx, p.vid, p.eid, p.fid,
                         p.uv.real(), p.uv.imag(), p.dir.real(), p.dir.imag(), p.pos[0], p.pos[1], p.pos[2], p.next_id,
                         p.prev_id, p.isConnected ? 1 : 0);
        std::fprintf(o, "E %zu\n", edges.size());
        for (const qex::Qedge& e : edges) std::fprintf(o, "e %d %d\n", e.port1, e.port2);
        std::fprintf(o, "Q %zu\n", faces.size());
        for (const qex::Qface& f : faces)
            std::fprintf(o, "q %d %d %d %d\n", f.qhalfs[0].port1(), f.qhalfs[1].port1(), f.qhalfs[2].port1(), f.qhalfs[3].port1());
        std::fclose(o);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 5;
    }
    return 0;
}
