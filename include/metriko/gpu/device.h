//
// metriko-gb300: host-side handle on the CUDA library (libmetriko_cuda.so, C ABI in
// include/metriko_cuda.h).  The numerical hot path has no CPU fallback: when no device or
// library is present the first call throws std::runtime_error.
//
#ifndef METRIKO_GPU_DEVICE_H
#define METRIKO_GPU_DEVICE_H
#include <memory>
#include <stdexcept>
#include <string>

#include "metriko_cuda.h"

namespace metriko::gpu {
    // A failed library call: carries the mtk_status, so callers above the C++ API (the C ABI
    // pipeline entry points) can hand the same status on.
    struct status_error : std::runtime_error {
        int status;
        status_error(int s, const std::string& msg) : std::runtime_error(msg), status(s) {}
    };

    inline void check(int status, const char* what) {
        if (status != MTK_OK)
            throw status_error(status, std::string(what) + ": " + mtk_status_string(status) + " " + mtk_last_error());
    }

    // Solver options shared by the header-only entry points (FaceRosyField, integ()).
    struct Options {
        mtk_solve_opts solve{};
        int seed = 0;           // start vector of the power iteration
        int n_iter = 50;        // power iterations (sparse_linear_solver.h:29, nIter = 50)
        int device = 0;
        Options() { mtk_default_opts(&solve); }
    };
    inline Options& options() { static Options o; return o; }

    // One context per process and device, created on first use.
    class Context {
    public:
        static mtk_ctx* get() {
            static std::unique_ptr<mtk_ctx, int (*)(mtk_ctx*)> ctx(nullptr, mtk_ctx_destroy);
            if (!ctx) {
                mtk_ctx* c = nullptr;
                check(mtk_ctx_create(options().device, &c), "mtk_ctx_create");
                ctx.reset(c);
            }
            return ctx.get();
        }
    };

    // Statistics of the last calls (accumulated; reset by the caller).
    inline mtk_stats& stats() { static mtk_stats s{}; return s; }
    // Context override used by mtk_pipeline_run (the caller owns that context).
    inline mtk_ctx*& bound_context() { static thread_local mtk_ctx* c = nullptr; return c; }
    inline mtk_ctx* context() { return bound_context() ? bound_context() : Context::get(); }
}

#endif
