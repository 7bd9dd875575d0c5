// A reference-style caller of the header-only host API: the example_igm.cpp sequence
// (Hmesh -> field -> Curl matching -> seam -> cut mesh -> combing -> extrinsic field ->
// RosyParameterization::setup) with the field given as its compressed eigenvector (the
// FaceRosyField constructor that solves for it needs a GPU), plus the element handles and
// iterators.  Reads nV, nF, V (nV x 3 double), F (nF x 3 int32) and the compressed field
// (nF complex) from a binary file; prints one "key value" pair per line.
#include <cstdio>
#include <fstream>
#include <memory>

#include "metriko/core/igm/parameterization.h"
#include "metriko/core/vectorfield/face_rosy_field.h"

using namespace metriko;

int main(int argc, char** argv) {
    if (argc < 2) return 2;
    std::ifstream in(argv[1], std::ios::binary);
    int h[2];
    in.read(reinterpret_cast<char*>(h), sizeof(h));
    MatXd V(h[0], 3);
    MatXi F(h[1], 3);
    std::vector<double> c(2 * size_t(h[1]));
    in.read(reinterpret_cast<char*>(V.data()), sizeof(double) * 3 * h[0]);
    in.read(reinterpret_cast<char*>(F.data()), sizeof(int) * 3 * h[1]);
    in.read(reinterpret_cast<char*>(c.data()), sizeof(double) * c.size());
    if (!in) return 3;

    auto mesh = std::make_unique<Hmesh>(V, F);
    auto rawf = std::make_unique<FaceRosyField>(*mesh, 4);
    rawf->compressed = VecXc(mesh->nF);
    for (int f = 0; f < mesh->nF; f++) rawf->compressed[f] = complex(c[2 * f], c[2 * f + 1]);
    rawf->set_field_from_compressed();
    rawf->computeMatching(MatchingType::Curl);
    auto seam = compute_seam(*rawf);
    auto cutm = compute_cut_mesh(*mesh, seam);
    auto cmbf = compute_combbed_field(*rawf, seam);
    MatXd extf = compute_extrinsic_field(*mesh, *cmbf, 4);
    RosyParameterization rp(*mesh, *cutm, extf, cmbf->singular, cmbf->matching, seam, 4, 0.03);
    rp.seamless = true;
    rp.roundSeams = false;
    rp.setup();

    long long sing = 0, nseam = 0, match = 0;
    for (int v = 0; v < mesh->nV; v++) sing += std::abs(rawf->singular[v]) * (v + 1LL);
    for (bool s : seam) nseam += s;
    for (int e = 0; e < mesh->nE; e++) match += cmbf->matching[e] * (e % 97 + 1LL);
    std::printf("nV %d\nnE %d\nnCut %d\nnT %d\nnS %d\nsingular %lld\nseam %lld\nmatching %lld\n", mesh->nV, mesh->nE,
                cutm->nV, rp.numTransitions(), rp.numSingular(), sing, nseam, match);

    // element handles: every face's halfedge loop, every vertex ring, corners, edges
    long long loops = 0, rings = 0, bad = 0;
    double area = 0, bary = 0;
    for (Face f : mesh->faces) {
        int k = 0;
        for (Half hh : f.adjHalfs()) {
            if (hh.face().id != f.id) bad++;
            k++;
        }
        loops += k;
        area += f.area();
    }
    for (Vert v : mesh->verts) {
        for (Half hh : v.adjHalfs()) {
            if (hh.tail().id != v.id || hh.twin().head().id != v.id) bad++;
            rings++;
        }
        bary += v.baryArea();
    }
    for (Crnr cr : mesh->crnrs) {
        const int f = cr.id / 3, j = cr.id % 3;
        if (cr.face().id != f || cr.vert().id != F(f, j) || cr.half().crnr().id != cr.id) bad++;
    }
    for (Edge e : mesh->edges) {
        if (e.half().edge().id != e.id || !e.half().isCanonical() || e.len() <= 0) bad++;
        if (e.vert0().id != e.half().tail().id || e.face0().id != e.half().face().id) bad++;
    }
    std::printf("loops %lld\nrings %lld\nbad %lld\narea_minus_bary %.3e\n", loops, rings, bad, area - bary);
    return 0;
}
