// Context lifetime, status strings and the deterministic start vector.
#include <cstring>
#include <mutex>
#include <string>

#include "mtk_ctx.cuh"

static thread_local std::string g_last_error;

void mtk_set_last_error(const char* msg, const char* file, int line) {
    g_last_error = std::string(msg) + " (" + file + ":" + std::to_string(line) + ")";
}

extern "C" const char* mtk_last_error(void) { return g_last_error.c_str(); }

extern "C" const char* mtk_status_string(int s) {
    switch (s) {
        case MTK_OK: return "ok";
        case MTK_ERR_BAD_INPUT: return "bad input";
        case MTK_ERR_CUDA: return "cuda error";
        case MTK_ERR_NOT_CONVERGED: return "not converged";
        case MTK_ERR_BREAKDOWN: return "pcg breakdown";
        case MTK_ERR_TIMEOUT: return "device wait timed out";
        case MTK_ERR_NO_DEVICE: return "no cuda device";
        case MTK_ERR_ROUNDING: return "rounding integrality check failed";
        default: return "unknown status";
    }
}

extern "C" void mtk_default_opts(mtk_solve_opts* o) {
    o->precision = MTK_PREC_MIXED;
    o->tol = 1e-8;
    o->max_iter = 50000;
    o->max_refine = 12;
    o->inner_tol = 3e-6;   // just above the FP32 floor: fewest FP64 refinement restarts
}

extern "C" int mtk_ctx_create(int device, mtk_ctx** out) {
    if (!out) return MTK_ERR_BAD_INPUT;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        mtk_set_last_error("no CUDA device visible", __FILE__, __LINE__);
        return MTK_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= ndev) return MTK_ERR_BAD_INPUT;
    MTK_CUDA_TRY(cudaSetDevice(device));
    int coop = 0;
    MTK_CUDA_TRY(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device));
    if (!coop) { mtk_set_last_error("device lacks cooperative launch", __FILE__, __LINE__); return MTK_ERR_CUDA; }
    auto* c = new mtk_ctx();
    c->device = device;
    cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
    c->partial_blocks = c->num_sms * 8;
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev_a);
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev_b);
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev_k0);
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev_k1);
    if (e == cudaSuccess) e = cudaMalloc(&c->bar, 4 * sizeof(unsigned int));
    if (e == cudaSuccess) e = cudaMalloc(&c->dev_err, sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&c->partials, sizeof(double) * 16 * c->partial_blocks);
    if (e == cudaSuccess) e = cudaMalloc(&c->scalars, sizeof(double) * 64);
    if (e == cudaSuccess) e = cudaMalloc(&c->dev_int, sizeof(int) * 16);
    if (e == cudaSuccess) e = cudaMallocHost(&c->h_scalars, sizeof(double) * 64);
    if (e == cudaSuccess) e = cudaMallocHost(&c->h_int, sizeof(int) * 16);
    if (e == cudaSuccess) e = cudaMemset(c->bar, 0, 4 * sizeof(unsigned int));
    if (e == cudaSuccess) e = cudaMemset(c->dev_err, 0, sizeof(int));
    // the device's default memory pool serves the stream-ordered buffers of every call; keep
    // what it has allocated between calls (released by mtk_ctx_destroy)
    if (e == cudaSuccess) {
        cudaMemPool_t pool;
        e = cudaDeviceGetDefaultMemPool(&pool, device);
        uint64_t keep = UINT64_MAX;
        if (e == cudaSuccess) e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    if (e != cudaSuccess) {
        mtk_set_last_error(cudaGetErrorString(e), __FILE__, __LINE__);
        mtk_ctx_destroy(c);
        return MTK_ERR_CUDA;
    }
    *out = c;
    return MTK_OK;
}

extern "C" int mtk_ctx_destroy(mtk_ctx* c) {
    if (!c) return MTK_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    {
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, c->device) == cudaSuccess) cudaMemPoolTrimTo(pool, 0);
    }
    if (c->bar) cudaFree(c->bar);
    if (c->dev_err) cudaFree(c->dev_err);
    if (c->partials) cudaFree(c->partials);
    if (c->scalars) cudaFree(c->scalars);
    if (c->dev_int) cudaFree(c->dev_int);
    if (c->h_scalars) cudaFreeHost(c->h_scalars);
    if (c->h_int) cudaFreeHost(c->h_int);
    if (c->ev_a) cudaEventDestroy(c->ev_a);
    if (c->ev_b) cudaEventDestroy(c->ev_b);
    if (c->ev_k0) cudaEventDestroy(c->ev_k0);
    if (c->ev_k1) cudaEventDestroy(c->ev_k1);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return MTK_OK;
}

extern "C" int64_t mtk_ctx_kernel_count(const mtk_ctx* c) { return c ? c->kernels : 0; }

extern "C" int mtk_ctx_set_wait_limit(mtk_ctx* c, int64_t polls) {
    if (!c || polls < 0) return MTK_ERR_BAD_INPUT;
    c->wait_limit = polls > 0 ? (long long)polls : 0;
    return MTK_OK;
}

// splitmix64 over (seed, 2f) and (seed, 2f+1), mapped to [-1, 1).  Replaces the
// std::rand-based VecXc::Random start of solveSmallestEig (sparse_linear_solver.h:32) with a
// reproducible vector that the CPU oracle regenerates bit-for-bit.  Every entry depends only on
// its index, so the host threads split the range.
extern "C" void mtk_seeded_init(int32_t n, int32_t seed, double* out) {
    const uint64_t G = 0x9E3779B97F4A7C15ULL;
#pragma omp parallel for schedule(static) if (n > 65536)
    for (int64_t i = 0; i < 2 * (int64_t)n; i++) {
        uint64_t z = (uint64_t)(uint32_t)seed * G + (uint64_t)(i + 1) * G;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
        z = z ^ (z >> 31);
        double u = (double)(z >> 11) * (1.0 / 9007199254740992.0);
        out[i] = 2.0 * u - 1.0;
    }
}
