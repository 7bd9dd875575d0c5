// Runs the localInjectivity rounding path of the header-only host API (li::iterative_rounding)
// on the CPU: the example_igm.cpp sequence up to RosyParameterization::build_system with the
// field given as its compressed eigenvector, the naive integration given as full variables, the
// linear solves by Jacobi-preconditioned CG on the host (the same method as the device
// mtk_csr_pcg the product calls) and the orientation check on the host.
// Input (binary): nV, nF (int32), ratio (double), round_seams (int32), V, F, compressed (nF complex),
// x0 (nFull doubles, preceded by nFull as int32).  Like the product's solves, the CG stops on its
// recurrence (relative residual 1e-13), fails at its iteration cap or on a breakdown, and each
// solve is refined three times on the exact residual.  Output (binary, argv[2]): success, n_fix,
// fix_order[n_fix], fix_vals[n_fix] (int32), nFull (int32), fullx (doubles), x_ni (doubles),
// ni_iterations, resolves (int32).
#include <cmath>
#include <cstdio>
#include <fstream>
#include <memory>

#include "metriko/core/igm/parameterization.h"
#include "metriko/core/vectorfield/face_rosy_field.h"

using namespace metriko;

static bool pcg1(const SprsD& A, const std::vector<double>& b, std::vector<double>& x) {
    const int n = A.nr;
    x.assign(n, 0.0);
    std::vector<double> dinv(n, 0.0), r(b), z(n), p(n), q(n);
    for (int i = 0; i < n; i++)
        for (int k = A.ptr[i]; k < A.ptr[i + 1]; k++)
            if (A.idx[k] == i) dinv[i] = 1.0 / A.val[k];
    double bb = 0, rz = 0;
    for (int i = 0; i < n; i++) { bb += b[i] * b[i]; z[i] = dinv[i] * r[i]; p[i] = z[i]; rz += r[i] * z[i]; }
    if (bb == 0) return true;
    const int max_iter = 20 * n + 1000;   // the product's cap
    for (int it = 0; it < max_iter; it++) {
        double pq = 0;
        for (int i = 0; i < n; i++) {
            double s = 0;
            for (int k = A.ptr[i]; k < A.ptr[i + 1]; k++) s += A.val[k] * p[A.idx[k]];
            q[i] = s;
            pq += p[i] * s;
        }
        if (!(pq > 0)) return false;
        const double alpha = rz / pq;
        double rr = 0, rzn = 0;
        for (int i = 0; i < n; i++) {
            x[i] += alpha * p[i];
            r[i] -= alpha * q[i];
            z[i] = dinv[i] * r[i];
            rr += r[i] * r[i];
            rzn += r[i] * z[i];
        }
        if (rr <= 1e-26 * bb) return true;
        const double beta = rzn / rz;
        rz = rzn;
        for (int i = 0; i < n; i++) p[i] = z[i] + beta * p[i];
    }
    return false;
}

// one pass and three FP64 refinements on the exact residual, as the product's solves
static bool pcg(const SprsD& A, const std::vector<double>& b, std::vector<double>& x) {
    if (!pcg1(A, b, x)) return false;
    std::vector<double> r(A.nr), e;
    for (int k = 0; k < 3; k++) {
        for (int i = 0; i < A.nr; i++) {
            double t = b[i];
            for (int q = A.ptr[i]; q < A.ptr[i + 1]; q++) t -= A.val[q] * x[A.idx[q]];
            r[i] = t;
        }
        if (!pcg1(A, r, e)) break;
        for (int i = 0; i < A.nr; i++) x[i] += e[i];
    }
    return true;
}

int main(int argc, char** argv) {
    if (argc < 3) return 2;
    std::ifstream in(argv[1], std::ios::binary);
    int h[2], rs = 0, nfull = 0;
    double ratio = 0;
    in.read(reinterpret_cast<char*>(h), sizeof(h));
    in.read(reinterpret_cast<char*>(&ratio), sizeof(ratio));
    in.read(reinterpret_cast<char*>(&rs), sizeof(rs));
    MatXd V(h[0], 3);
    MatXi F(h[1], 3);
    std::vector<double> c(2 * size_t(h[1]));
    in.read(reinterpret_cast<char*>(V.data()), sizeof(double) * 3 * h[0]);
    in.read(reinterpret_cast<char*>(F.data()), sizeof(int) * 3 * h[1]);
    in.read(reinterpret_cast<char*>(c.data()), sizeof(double) * c.size());
    in.read(reinterpret_cast<char*>(&nfull), sizeof(nfull));
    VecXd x0(nfull);
    in.read(reinterpret_cast<char*>(x0.data()), sizeof(double) * nfull);
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
    RosyParameterization rp(*mesh, *cutm, extf, cmbf->singular, cmbf->matching, seam, 4, ratio);
    rp.seamless = true;
    rp.roundSeams = rs != 0;
    rp.localInjectivity = true;
    rp.setup();
    IntegSystem sys;
    rp.build_system(sys);
    if (sys.desc.nFull != nfull) return 4;
    li::System ls;
    rp.li_system(sys, ls);
    const std::vector<double> xs0 = rp.to_reduced(sys, ls, x0);
    auto injective = [&](const std::vector<double>& xs) {
        const std::vector<double> X = ls.ufull_times(xs);
        const std::vector<double> NF = sys.fullx2Nfunc * X;
        for (int f = 0; f < cutm->nF; f++) {
            const int a = cutm->idx(f, 0), b = cutm->idx(f, 1), cc = cutm->idx(f, 2);
            const double d1x = NF[4 * size_t(b)] - NF[4 * size_t(a)], d1y = NF[4 * size_t(b) + 1] - NF[4 * size_t(a) + 1];
            const double d2x = NF[4 * size_t(cc)] - NF[4 * size_t(a)], d2y = NF[4 * size_t(cc) + 1] - NF[4 * size_t(a) + 1];
            if (d1x * d2y - d1y * d2x < 0) return false;
        }
        return true;
    };
    li::Result r = li::iterative_rounding(ls, xs0, true, pcg, injective);

    std::ofstream out(argv[2], std::ios::binary);
    int hdr[2] = {r.success ? 1 : 0, int(r.fixOrder.size())};
    out.write(reinterpret_cast<const char*>(hdr), sizeof(hdr));
    out.write(reinterpret_cast<const char*>(r.fixOrder.data()), sizeof(int) * r.fixOrder.size());
    out.write(reinterpret_cast<const char*>(r.fixVals.data()), sizeof(int) * r.fixVals.size());
    const int nf = int(r.fullx.size());
    out.write(reinterpret_cast<const char*>(&nf), sizeof(nf));
    out.write(reinterpret_cast<const char*>(r.fullx.data()), sizeof(double) * nf);
    out.write(reinterpret_cast<const char*>(r.x_ni.data()), sizeof(double) * nf);
    int tail[2] = {r.ni_iterations, r.resolves};
    out.write(reinterpret_cast<const char*>(tail), sizeof(tail));
    return 0;
}
