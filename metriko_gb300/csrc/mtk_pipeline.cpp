// mtk_pipeline_run: the example_igm.cpp:13-31 call sequence through the header-only host API
// (include/metriko/...), with host buffers in and out.  Topology stages run on the host, the
// field and the integration / rounding solves on the GPU.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <future>
#if defined(_OPENMP)
#include <omp.h>
#endif

#include "metriko/core/igm/parameterization.h"
#include "metriko/core/vectorfield/face_rosy_field.h"

void mtk_set_last_error(const char* msg, const char* file, int line);

using namespace metriko;

namespace {
// Host work that runs beside the GPU field solve uses a quarter of the cores for its parallel
// loops, so that the field's own host steps keep most of them (per-thread OpenMP setting).
void side_thread_cores(int share = 4) {
#if defined(_OPENMP)
    omp_set_num_threads(std::max(1, omp_get_num_procs() / share));
#endif
}
}

extern "C" int mtk_pipeline_run(mtk_ctx* ctx, int32_t nV, int32_t nF, const double* Vb, const int32_t* Fb,
                                const mtk_pipeline_opts* popts, const mtk_solve_opts* sopts, int32_t* singular,
                                int32_t* matching, uint8_t* seam_out, double* compressed, double* cfn_out,
                                double* fullx_out, double* x_naive, int32_t fullx_cap, int32_t* n_full,
                                int32_t* fix_order, int32_t* fix_vals, int32_t fix_cap, int32_t* n_fixed,
                                int32_t* counts, mtk_stats* stats) {
    if (!ctx || nV <= 0 || nF <= 0 || !Vb || !Fb || !popts) return MTK_ERR_BAD_INPUT;
    using clk = std::chrono::steady_clock;
    auto t0 = clk::now();
    const bool dbg = getenv("MTK_DEBUG") && getenv("MTK_DEBUG")[0] == '1';
    auto stamp = [&](const char* what, clk::time_point& a) {
        auto b = clk::now();
        if (dbg) fprintf(stderr, "[host] %-22s %8.1f ms\n", what, std::chrono::duration<double, std::milli>(b - a).count());
        a = b;
    };
    auto ts2 = clk::now();
    double host_ms = 0;
    auto lap = [&](clk::time_point& a) {
        auto b = clk::now();
        host_ms += std::chrono::duration<double, std::milli>(b - a).count();
        a = b;
    };
    gpu::bound_context() = ctx;
    struct Unbind { ~Unbind() { gpu::bound_context() = nullptr; } } unbind;
    gpu::stats() = mtk_stats{};
    if (sopts) gpu::options().solve = *sopts;
    else mtk_default_opts(&gpu::options().solve);
    gpu::options().seed = popts->seed;
    gpu::options().n_iter = popts->n_iter > 0 ? popts->n_iter : 50;
    try {
        auto ts = clk::now();
        auto host_mesh_input = [Vb, Fb, nV, nF] {
            std::pair<MatXd, MatXi> vf{MatXd(nV, 3), MatXi(nF, 3)};
            std::memcpy(vf.first.data(), Vb, sizeof(double) * 3 * size_t(nV));
            std::memcpy(vf.second.data(), Fb, sizeof(int32_t) * 3 * size_t(nF));
            return vf;
        };
        const bool seams = popts->stop_after != 1;
        std::unique_ptr<Hmesh> mesh;
        std::unique_ptr<FaceRosyField> rawfp;
        SeamBase base;
        if (popts->field_type != 1) {
            // the smoothest field needs only the face pairing, the halfedge angles and the areas:
            // computed on the device from V and F (mtk_field_smoothest_mesh), so a host thread
            // builds the whole halfedge mesh and the field-independent part of the seam search
            // while the GPU solves
            auto built = std::async(std::launch::async, [&host_mesh_input, seams] {
                side_thread_cores(2);
                const auto [V, F] = host_mesh_input();   // the host copy of V, F beside the solve
                auto m = std::make_unique<Hmesh>(V, F, Hmesh::Deferred{});
                m->finish();
                SeamBase b = seams ? seam_base(*m) : SeamBase{};
                return std::make_pair(std::move(m), std::move(b));
            });
            std::vector<double> x0(2 * size_t(nF)), cfield(2 * size_t(nF));
            mtk_seeded_init(nF, gpu::options().seed, x0.data());
            const int fs = mtk_field_smoothest_mesh(ctx, nV, nF, Vb, Fb, 4, x0.data(), gpu::options().n_iter,
                                                    &gpu::options().solve, cfield.data(), &gpu::stats());
            stamp("field (gpu)", ts2);
            ts = clk::now();
            auto pr = built.get();   // a wait here (the mesh outlasting the field) is host time
            lap(ts);
            stamp("hmesh join", ts2);
            gpu::check(fs, "mtk_field_smoothest_mesh");
            mesh = std::move(pr.first);
            base = std::move(pr.second);
            rawfp = std::make_unique<FaceRosyField>(*mesh, 4);
            rawfp->compressed = VecXc(nF);
            for (int f = 0; f < nF; f++) rawfp->compressed[f] = complex(cfield[2 * f], cfield[2 * f + 1]);
            rawfp->set_field_from_compressed();
            lap(ts);
            stamp("field expansion", ts2);
        } else {
            {
                const auto [V, F] = host_mesh_input();
                mesh = std::make_unique<Hmesh>(V, F, Hmesh::Deferred{});
            }
            lap(ts);
            stamp("hmesh", ts2);
            // while the GPU solves the field, a host thread completes the mesh (element lists,
            // angle defects: neither is read by the field solve) and computes the field-independent
            // part of the seam search
            auto pending = std::async(std::launch::async, [&m = *mesh, seams] {
                side_thread_cores();
                m.finish();
                return seams ? seam_base(m) : SeamBase{};
            });
            rawfp = std::make_unique<FaceRosyField>(*mesh, 4, FieldType::CurvatureAligned);
            stamp("field (gpu)", ts2);
            ts = clk::now();
            base = pending.get();
        }
        FaceRosyField& rawf = *rawfp;
        rawf.computeMatching(MatchingType::Curl);
        stamp("matching+singular", ts2);
        if (compressed)
            for (int f = 0; f < nF; f++) { compressed[2 * f] = rawf.compressed[f].real(); compressed[2 * f + 1] = rawf.compressed[f].imag(); }
        if (singular) std::memcpy(singular, rawf.singular.data(), sizeof(int32_t) * nV);
        if (counts) { counts[0] = mesh->nV; counts[1] = mesh->nE; }
        if (popts->stop_after == 1) {
            if (matching) std::memcpy(matching, rawf.matching.data(), sizeof(int32_t) * mesh->nE);
            lap(ts);
            if (stats) { *stats = gpu::stats(); stats->ms_host = host_ms; stats->ms_total = std::chrono::duration<double, std::milli>(clk::now() - t0).count(); }
            return MTK_OK;
        }
        auto seam = compute_seam(rawf, std::move(base));
        stamp("seam", ts2);
        // the cut mesh and the combing both read only the seam: the cut mesh on a host thread
        auto cut_pending = std::async(std::launch::async, [&m = *mesh, &seam] { return compute_cut_mesh(m, seam); });
        auto cmbf = compute_combbed_field(rawf, seam);
        MatXd extf = compute_extrinsic_field(*mesh, *cmbf, 4);
        auto cutm = cut_pending.get();
        stamp("cut mesh+combing+extr", ts2);
        RosyParameterization rp(*mesh, *cutm, extf, cmbf->singular, cmbf->matching, seam, 4, popts->ratio);
        rp.seamless = popts->seamless != 0;
        rp.localInjectivity = popts->local_injectivity != 0;
        rp.roundSeams = popts->round_seams != 0;
        rp.verbose = false;
        stamp("transitions", ts2);
        rp.setup();
        stamp("setup", ts2);
        lap(ts);
        if (matching) std::memcpy(matching, cmbf->matching.data(), sizeof(int32_t) * mesh->nE);
        if (seam_out) for (int e = 0; e < mesh->nE; e++) seam_out[e] = seam[e] ? 1 : 0;
        if (counts) {
            counts[2] = cutm->nV;
            counts[3] = rp.numTransitions();
            counts[4] = rp.numSingular();
        }
        if (popts->stop_after == 2) {
            if (stats) { *stats = gpu::stats(); stats->ms_host = host_ms; stats->ms_total = std::chrono::duration<double, std::milli>(clk::now() - t0).count(); }
            return MTK_OK;
        }
        rp.cfn_target = cfn_out;   // the corner values straight into the caller's buffer
        bool ok = rp.integ();
        stamp("integ (host+gpu)", ts2);
        const int nFull = rp.fullx.size();
        if (counts) { counts[5] = rp.nJ; counts[6] = rp.nZ; counts[7] = nFull; }
        if (n_full) *n_full = nFull;
        if (fullx_out && fullx_cap >= nFull) std::memcpy(fullx_out, rp.fullx.data(), sizeof(double) * nFull);
        if (x_naive && fullx_cap >= nFull) std::memcpy(x_naive, rp.naivex.data(), sizeof(double) * nFull);
        const int nfix = int(rp.fixOrder.size());
        if (n_fixed) *n_fixed = nfix;
        for (int i = 0; i < nfix && i < fix_cap; i++) {
            if (fix_order) fix_order[i] = rp.fixOrder[i];
            if (fix_vals) fix_vals[i] = rp.fixVals[i];
        }

        if (stats) {
            *stats = gpu::stats();
            stats->ms_total = std::chrono::duration<double, std::milli>(clk::now() - t0).count();
            stats->ms_host = stats->ms_total - stats->ms_field - stats->ms_integrate - stats->ms_rounding;
        }
        return ok ? MTK_OK : MTK_ERR_ROUNDING;
    } catch (const std::invalid_argument& e) {
        mtk_set_last_error(e.what(), __FILE__, __LINE__);
        return MTK_ERR_BAD_INPUT;
    } catch (const metriko::gpu::status_error& e) {
        mtk_set_last_error(e.what(), __FILE__, __LINE__);
        return e.status;
    } catch (const std::exception& e) {
        mtk_set_last_error(e.what(), __FILE__, __LINE__);
        return MTK_ERR_CUDA;
    }
}

extern "C" int mtk_pipeline_size_field_gradient(mtk_ctx* ctx, int32_t nV, int32_t nF, const double* Vb, const int32_t* Fb,
                                                const mtk_pipeline_opts* popts, const mtk_solve_opts* sopts,
                                                const double* s, const double* T, double mu, double* loss,
                                                double* grad_s, double* fullx_out, int32_t fullx_cap, int32_t* n_full,
                                                mtk_stats* stats) {
    if (!ctx || nV <= 0 || nF <= 0 || !Vb || !Fb || !popts || !s || !loss || !grad_s) return MTK_ERR_BAD_INPUT;
    gpu::bound_context() = ctx;
    struct Unbind { ~Unbind() { gpu::bound_context() = nullptr; } } unbind;
    gpu::stats() = mtk_stats{};
    if (sopts) gpu::options().solve = *sopts;
    else mtk_default_opts(&gpu::options().solve);
    gpu::options().seed = popts->seed;
    gpu::options().n_iter = popts->n_iter > 0 ? popts->n_iter : 50;
    try {
        MatXd V(nV, 3);
        MatXi F(nF, 3);
        std::memcpy(V.data(), Vb, sizeof(double) * 3 * size_t(nV));
        std::memcpy(F.data(), Fb, sizeof(int32_t) * 3 * size_t(nF));
        auto mesh = std::make_unique<Hmesh>(V, F, Hmesh::Deferred{});
        auto pending = std::async(std::launch::async, [&m = *mesh] { side_thread_cores(); m.finish(); return seam_base(m); });   // during the field solve
        FaceRosyField rawf(*mesh, 4, popts->field_type == 1 ? FieldType::CurvatureAligned : FieldType::Smoothest);
        SeamBase base = pending.get();
        rawf.computeMatching(MatchingType::Curl);
        auto seam = compute_seam(rawf, std::move(base));
        auto cut_pending = std::async(std::launch::async, [&m = *mesh, &seam] { return compute_cut_mesh(m, seam); });
        auto cmbf = compute_combbed_field(rawf, seam);
        MatXd extf = compute_extrinsic_field(*mesh, *cmbf, 4);
        auto cutm = cut_pending.get();
        RosyParameterization rp(*mesh, *cutm, extf, cmbf->singular, cmbf->matching, seam, 4, popts->ratio);
        rp.seamless = false;
        rp.localInjectivity = false;
        rp.roundSeams = popts->round_seams != 0;
        rp.verbose = false;
        rp.setup();
        VecXd sv(std::vector<double>(s, s + nV)), grad;
        VecXd Tv;
        if (T) Tv = VecXd(std::vector<double>(T, T + 8 * size_t(nF)));
        *loss = rp.size_field_gradient(sv, T ? &Tv : nullptr, mu, grad);
        std::memcpy(grad_s, grad.data(), sizeof(double) * nV);
        const int nFull = rp.fullx.size();
        if (n_full) *n_full = nFull;
        if (fullx_out && fullx_cap >= nFull) std::memcpy(fullx_out, rp.fullx.data(), sizeof(double) * nFull);
        if (stats) *stats = gpu::stats();
        return MTK_OK;
    } catch (const std::invalid_argument& e) {
        mtk_set_last_error(e.what(), __FILE__, __LINE__);
        return MTK_ERR_BAD_INPUT;
    } catch (const metriko::gpu::status_error& e) {
        mtk_set_last_error(e.what(), __FILE__, __LINE__);
        return e.status;
    } catch (const std::exception& e) {
        mtk_set_last_error(e.what(), __FILE__, __LINE__);
        return MTK_ERR_CUDA;
    }
}

extern "C" int mtk_pipeline_position_gradient(mtk_ctx* ctx, int32_t nV, int32_t nF, const double* Vb, const int32_t* Fb,
                                              const mtk_pipeline_opts* popts, const mtk_solve_opts* sopts,
                                              const double* s, double mu, double* loss, double* grad_s, double* grad_V,
                                              double* fullx_out, int32_t fullx_cap, int32_t* n_full, mtk_stats* stats) {
    if (!ctx || nV <= 0 || nF <= 0 || !Vb || !Fb || !popts || !s || !loss || !grad_s || !grad_V || !(mu >= 0))
        return MTK_ERR_BAD_INPUT;
    gpu::bound_context() = ctx;
    struct Unbind { ~Unbind() { gpu::bound_context() = nullptr; } } unbind;
    gpu::stats() = mtk_stats{};
    if (sopts) gpu::options().solve = *sopts;
    else mtk_default_opts(&gpu::options().solve);
    gpu::options().seed = popts->seed;
    gpu::options().n_iter = popts->n_iter > 0 ? popts->n_iter : 50;
    try {
        MatXd V(nV, 3);
        MatXi F(nF, 3);
        std::memcpy(V.data(), Vb, sizeof(double) * 3 * size_t(nV));
        std::memcpy(F.data(), Fb, sizeof(int32_t) * 3 * size_t(nF));
        auto mesh = std::make_unique<Hmesh>(V, F, Hmesh::Deferred{});
        auto pending = std::async(std::launch::async, [&m = *mesh] { side_thread_cores(); m.finish(); return seam_base(m); });
        FaceRosyField rawf(*mesh, 4, FieldType::Smoothest);
        SeamBase base = pending.get();
        rawf.computeMatching(MatchingType::Curl);
        auto seam = compute_seam(rawf, std::move(base));
        auto cut_pending = std::async(std::launch::async, [&m = *mesh, &seam] { return compute_cut_mesh(m, seam); });
        auto cmbf = compute_combbed_field(rawf, seam);
        MatXd extf = compute_extrinsic_field(*mesh, *cmbf, 4);
        auto cutm = cut_pending.get();
        RosyParameterization rp(*mesh, *cutm, extf, cmbf->singular, cmbf->matching, seam, 4, popts->ratio);
        rp.seamless = false;
        rp.localInjectivity = false;
        rp.roundSeams = popts->round_seams != 0;
        rp.verbose = false;
        rp.setup();
        // 1. the loss, its s gradient and its partials at fixed x (G2 entries, field angle, length)
        VecXd sv(std::vector<double>(s, s + nV)), gs;
        std::vector<double> dgx, dgy, dphi;
        double dlength = 0, length = 0;
        *loss = rp.size_field_position_partials(sv, mu, gs, dgx, dgy, dphi, &dlength, &length);
        std::memcpy(grad_s, gs.data(), sizeof(double) * nV);
        // 2. the field angle through the power iteration: derivatives of theta and of the areas
        std::vector<int> nb;
        std::vector<double> th;
        rawf.assembly_inputs(nb, th);
        std::vector<double> x0(2 * size_t(nF)), cfield(2 * size_t(nF)), gth(3 * size_t(nF)), gar(nF);
        mtk_seeded_init(nF, gpu::options().seed, x0.data());
        gpu::check(mtk_field_power_adjoint(ctx, nF, 4, nb.data(), th.data(), mesh->faceArea.data(), x0.data(),
                                           gpu::options().n_iter, &gpu::options().solve, dphi.data(), cfield.data(),
                                           gth.data(), gar.data(), &gpu::stats()),
                   "mtk_field_power_adjoint");
        // theta_fj = farg(h) - farg(twin h) for the halfedge h of f on edge j
        const Hmesh& m = *mesh;
        std::vector<double> gfarg(m.nH, 0.0), gf1(nF), gf2(nF);
        for (int f = 0; f < nF; f++)
            for (int j = 0; j < 3; j++) {
                const int h = m.face2half3(f, j);
                gfarg[h] += gth[3 * size_t(f) + j];
                gfarg[m.twin[h]] -= gth[3 * size_t(f) + j];
            }
        for (int f = 0; f < nF; f++) {
            gf1[f] = gfarg[m.face2half3(f, 1)];
            gf2[f] = gfarg[m.face2half3(f, 2)];
        }
        // 3. per-face geometry backward and the vertex gather
        gpu::check(mtk_face_geometry_backward(ctx, nV, nF, Vb, Fb, gar.data(), gf1.data(), gf2.data(), dgx.data(),
                                              dgy.data(), grad_V),
                   "mtk_face_geometry_backward");
        // 4. length = ratio |D| / norm, D the bounding-box diagonal: its extreme vertices (the
        //    first vertex holding each extreme coordinate)
        double D[3];
        int imax[3] = {0, 0, 0}, imin[3] = {0, 0, 0};
        for (int k = 0; k < 3; k++) {
            for (int v = 1; v < nV; v++) {
                if (Vb[3 * size_t(v) + k] > Vb[3 * size_t(imax[k]) + k]) imax[k] = v;
                if (Vb[3 * size_t(v) + k] < Vb[3 * size_t(imin[k]) + k]) imin[k] = v;
            }
            D[k] = Vb[3 * size_t(imax[k]) + k] - Vb[3 * size_t(imin[k]) + k];
        }
        const double dn = std::sqrt(D[0] * D[0] + D[1] * D[1] + D[2] * D[2]);
        const double norm = popts->ratio * dn / length;
        for (int k = 0; k < 3; k++) {
            const double g = dlength * popts->ratio * D[k] / (dn * norm);
            grad_V[3 * size_t(imax[k]) + k] += g;
            grad_V[3 * size_t(imin[k]) + k] -= g;
        }
        const int nFull = rp.fullx.size();
        if (n_full) *n_full = nFull;
        if (fullx_out && fullx_cap >= nFull) std::memcpy(fullx_out, rp.fullx.data(), sizeof(double) * nFull);
        if (stats) *stats = gpu::stats();
        return MTK_OK;
    } catch (const std::invalid_argument& e) {
        mtk_set_last_error(e.what(), __FILE__, __LINE__);
        return MTK_ERR_BAD_INPUT;
    } catch (const metriko::gpu::status_error& e) {
        mtk_set_last_error(e.what(), __FILE__, __LINE__);
        return e.status;
    } catch (const std::exception& e) {
        mtk_set_last_error(e.what(), __FILE__, __LINE__);
        return MTK_ERR_CUDA;
    }
}

extern "C" int mtk_topology_from_field(int32_t nV, int32_t nF, const double* Vb, const int32_t* Fb,
                                       const double* compressed, double ratio, int32_t round_seams,
                                       int32_t* singular, int32_t* matching, uint8_t* seam_out, int32_t* cutF,
                                       int32_t* counts, double* length) {
    if (nV <= 0 || nF <= 0 || !Vb || !Fb || !compressed) return MTK_ERR_BAD_INPUT;
    using clk = std::chrono::steady_clock;
    const bool dbg = getenv("MTK_DEBUG") && getenv("MTK_DEBUG")[0] == '1';
    auto ts = clk::now();
    auto stamp = [&](const char* what) {
        auto b = clk::now();
        if (dbg) fprintf(stderr, "[host] %-22s %8.1f ms\n", what, std::chrono::duration<double, std::milli>(b - ts).count());
        ts = b;
    };
    try {
        MatXd V(nV, 3);
        MatXi F(nF, 3);
        std::memcpy(V.data(), Vb, sizeof(double) * 3 * size_t(nV));
        std::memcpy(F.data(), Fb, sizeof(int32_t) * 3 * size_t(nF));
        // the same two-thread order as mtk_pipeline_run (the mesh completed and the seam base
        // computed on a host thread while the field is set up)
        auto mesh = std::make_unique<Hmesh>(V, F, Hmesh::Deferred{});
        stamp("hmesh");
        auto pending = std::async(std::launch::async, [&m = *mesh] { side_thread_cores(); m.finish(); return seam_base(m); });
        FaceRosyField rawf(*mesh, 4);
        rawf.compressed = VecXc(nF);
        for (int f = 0; f < nF; f++) rawf.compressed[f] = complex(compressed[2 * f], compressed[2 * f + 1]);
        rawf.set_field_from_compressed();
        SeamBase base = pending.get();
        rawf.computeMatching(MatchingType::Curl);
        stamp("matching+singular");
        if (singular) std::memcpy(singular, rawf.singular.data(), sizeof(int32_t) * nV);
        auto seam = compute_seam(rawf, std::move(base));
        stamp("seam");
        auto cut_pending = std::async(std::launch::async, [&m = *mesh, &seam] { return compute_cut_mesh(m, seam); });
        auto cmbf = compute_combbed_field(rawf, seam);
        MatXd extf = compute_extrinsic_field(*mesh, *cmbf, 4);
        auto cutm = cut_pending.get();
        stamp("cut mesh+combing+extr");
        RosyParameterization rp(*mesh, *cutm, extf, cmbf->singular, cmbf->matching, seam, 4, ratio);
        rp.seamless = true;
        rp.roundSeams = round_seams != 0;
        stamp("transitions");
        rp.setup();
        stamp("setup");
        IntegSystem sys;
        rp.build_system(sys);
        stamp("integ build_system");
        if (matching) std::memcpy(matching, cmbf->matching.data(), sizeof(int32_t) * mesh->nE);
        if (seam_out) for (int e = 0; e < mesh->nE; e++) seam_out[e] = seam[e] ? 1 : 0;
        if (cutF) std::memcpy(cutF, cutm->idx.data(), sizeof(int32_t) * 3 * size_t(nF));
        if (counts) {
            counts[0] = mesh->nV; counts[1] = mesh->nE; counts[2] = cutm->nV; counts[3] = rp.numTransitions();
            counts[4] = rp.numSingular(); counts[5] = rp.nJ; counts[6] = rp.nZ; counts[7] = sys.desc.nFull;
        }
        if (length) *length = sys.length;
        return MTK_OK;
    } catch (const std::invalid_argument& e) {
        mtk_set_last_error(e.what(), __FILE__, __LINE__);
        return MTK_ERR_BAD_INPUT;
    } catch (const metriko::gpu::status_error& e) {
        mtk_set_last_error(e.what(), __FILE__, __LINE__);
        return e.status;
    } catch (const std::exception& e) {
        mtk_set_last_error(e.what(), __FILE__, __LINE__);
        return MTK_ERR_BAD_INPUT;
    }
}

extern "C" int mtk_field_inputs(int32_t nV, int32_t nF, const double* Vb, const int32_t* Fb, int32_t* nbr,
                                double* theta, double* area) {
    if (nV <= 0 || nF <= 0 || !Vb || !Fb || !nbr || !theta) return MTK_ERR_BAD_INPUT;
    try {
        MatXd V(nV, 3);
        MatXi F(nF, 3);
        std::memcpy(V.data(), Vb, sizeof(double) * 3 * size_t(nV));
        std::memcpy(F.data(), Fb, sizeof(int32_t) * 3 * size_t(nF));
        Hmesh mesh(V, F);
        FaceRosyField fld(mesh, 4);
        std::vector<int> nb;
        std::vector<double> th;
        fld.assembly_inputs(nb, th);
        std::memcpy(nbr, nb.data(), sizeof(int32_t) * nb.size());
        std::memcpy(theta, th.data(), sizeof(double) * th.size());
        if (area) std::memcpy(area, mesh.faceArea.data(), sizeof(double) * nF);
        return MTK_OK;
    } catch (const std::exception& e) {
        mtk_set_last_error(e.what(), __FILE__, __LINE__);
        return MTK_ERR_BAD_INPUT;
    }
}

extern "C" int mtk_map_deviation(int32_t nF, int32_t N, int32_t nCut, const int32_t* cutF, const double* cutV,
                                 const double* cfn, const double* ext, double* deviation) {
    if (nF < 0 || N <= 0 || nCut < 0 || !deviation || (nF > 0 && (!cutF || !cutV || !cfn || !ext)))
        return MTK_ERR_BAD_INPUT;
    for (size_t i = 0; i < 3 * size_t(nF); i++)
        if (cutF[i] < 0 || cutF[i] >= nCut) return MTK_ERR_BAD_INPUT;
    MatXd V(nCut, 3), C(nF, 3 * N), E(nF, 3 * N);
    MatXi F(nF, 3);
    std::memcpy(V.data(), cutV, sizeof(double) * 3 * size_t(nCut));
    std::memcpy(F.data(), cutF, sizeof(int32_t) * 3 * size_t(nF));
    std::memcpy(C.data(), cfn, sizeof(double) * 3 * size_t(N) * nF);
    std::memcpy(E.data(), ext, sizeof(double) * 3 * size_t(N) * nF);
    *deviation = map_deviation(V, F, C, E, N);
    return MTK_OK;
}

extern "C" int mtk_mesh_geometry(int32_t nV, int32_t nF, const double* Vb, const int32_t* Fb, double* vert_normal,
                                 double* vert_basis_x, double* vert_basis_y, double* bary_area, double* circ_area,
                                 double* half_cotan, double* edge_cotan, double* dihedral, double* he_arg_on_vert,
                                 double* angle_defect) {
    if (nV <= 0 || nF <= 0 || !Vb || !Fb) return MTK_ERR_BAD_INPUT;
    try {
        MatXd V(nV, 3);
        MatXi F(nF, 3);
        std::memcpy(V.data(), Vb, sizeof(double) * 3 * size_t(nV));
        std::memcpy(F.data(), Fb, sizeof(int32_t) * 3 * size_t(nF));
        Hmesh m(V, F);
        auto put = [](double* dst, const double* src, size_t n) { if (dst) std::memcpy(dst, src, sizeof(double) * n); };
        put(vert_normal, m.vertNormal.data(), 3 * size_t(nV));
        put(vert_basis_x, m.vertBasisX.data(), 3 * size_t(nV));
        put(vert_basis_y, m.vertBasisY.data(), 3 * size_t(nV));
        put(bary_area, m.baryDualArea.data(), nV);
        put(circ_area, m.circDualArea.data(), nV);
        put(half_cotan, m.halfCotan.data(), m.nH);
        put(edge_cotan, m.edgeCotan.data(), m.nE);
        put(dihedral, m.dihedralArg.data(), m.nH);
        put(he_arg_on_vert, m.heArgOnVert.data(), m.nH);
        put(angle_defect, m.angleDefect.data(), nV);
        return MTK_OK;
    } catch (const std::exception& e) {
        mtk_set_last_error(e.what(), __FILE__, __LINE__);
        return MTK_ERR_BAD_INPUT;
    }
}
