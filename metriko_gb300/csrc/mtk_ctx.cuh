// Context object behind the opaque mtk_ctx handle, plus small device-buffer helpers.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "mtk_common.cuh"

struct mtk_ctx {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev_a = nullptr, ev_b = nullptr;
    cudaEvent_t ev_k0 = nullptr, ev_k1 = nullptr;   // around each persistent-kernel launch
    // bounded grid barrier state (3 words) + error flag, and reduction scratch
    unsigned int* bar = nullptr;   // [0] count, [1] generation
    int* dev_err = nullptr;
    double* partials = nullptr;    // reduction partials (>= 8 slots per block)
    double* scalars = nullptr;     // finalized scalars (64 doubles)
    double* h_scalars = nullptr;   // pinned host mirror of scalars
    int* h_int = nullptr;          // pinned host ints
    int* dev_int = nullptr;        // device ints (iteration counts, status)
    int partial_blocks = 0;        // capacity in blocks
    long long kernels = 0;
    long long wait_limit = mtk::kSpinLimit;   // polls of a grid-barrier wait before MTK_ERR_TIMEOUT
};

namespace mtk {

// Stream of the context call running on this host thread (set by AllocStreamScope at the entry
// points): device buffers are then allocated and freed in that stream's order from the device's
// memory pool, whose release threshold the context raises, so a repeated call reuses the pool's
// blocks instead of calling cudaMalloc / cudaFree (and the device-wide synchronisation of
// cudaFree).  Every use of such a buffer is on the same stream.
inline cudaStream_t& alloc_stream() {
    static thread_local cudaStream_t s = nullptr;
    return s;
}
struct AllocStreamScope {
    cudaStream_t prev;
    explicit AllocStreamScope(cudaStream_t s) : prev(alloc_stream()) { alloc_stream() = s; }
    ~AllocStreamScope() { alloc_stream() = prev; }
    AllocStreamScope(const AllocStreamScope&) = delete;
    AllocStreamScope& operator=(const AllocStreamScope&) = delete;
};

// RAII device buffer (allocation happens once per solve set-up, never inside the loops):
// stream-ordered inside a context call, plain cudaMalloc outside one.
template <typename T>
struct DBuf {
    T* p = nullptr;
    size_t n = 0;
    cudaStream_t s = nullptr;   // stream of a stream-ordered allocation
    bool async = false;
    DBuf() = default;
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    DBuf(DBuf&& o) noexcept : p(o.p), n(o.n), s(o.s), async(o.async) { o.p = nullptr; o.n = 0; }
    DBuf& operator=(DBuf&& o) noexcept {
        if (this != &o) {
            release();
            p = o.p;
            n = o.n;
            s = o.s;
            async = o.async;
            o.p = nullptr;
            o.n = 0;
        }
        return *this;
    }
    ~DBuf() { release(); }
    void release() {
        if (p) {
            if (async) cudaFreeAsync(p, s);
            else cudaFree(p);
        }
        p = nullptr;
    }
    int alloc(size_t count) {
        release();
        n = count;
        if (count == 0) return MTK_OK;
        s = alloc_stream();
        async = s != nullptr;
        cudaError_t e = async ? cudaMallocAsync(reinterpret_cast<void**>(&p), count * sizeof(T), s)
                              : cudaMalloc(&p, count * sizeof(T));
        if (e != cudaSuccess) { mtk_set_last_error(cudaGetErrorString(e), __FILE__, __LINE__); p = nullptr; return MTK_ERR_CUDA; }
        return MTK_OK;
    }
    int upload(const T* h, size_t count, cudaStream_t s) {
        MTK_TRY(alloc(count));
        if (count) MTK_CUDA_TRY(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s));
        return MTK_OK;
    }
    int zero(cudaStream_t s) {
        if (n) MTK_CUDA_TRY(cudaMemsetAsync(p, 0, n * sizeof(T), s));
        return MTK_OK;
    }
};

inline GridBarrier barrier_of(mtk_ctx* c) { return GridBarrier{c->bar, c->bar + 1, c->dev_err, c->wait_limit}; }

// Resets the barrier words and the error flag before a cooperative launch.
inline int reset_barrier(mtk_ctx* c) {
    MTK_CUDA_TRY(cudaMemsetAsync(c->bar, 0, 2 * sizeof(unsigned int), c->stream));
    MTK_CUDA_TRY(cudaMemsetAsync(c->dev_err, 0, sizeof(int), c->stream));
    return MTK_OK;
}

// Cooperative launch of a persistent kernel sized to fill every SM.
template <typename K, typename... Args>
int launch_persistent(mtk_ctx* c, K kernel, int* grid_out, Args... args) {
    int per_sm = 0;
    MTK_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kBlock, 0));
    if (per_sm < 1) { mtk_set_last_error("persistent kernel does not fit on an SM", __FILE__, __LINE__); return MTK_ERR_CUDA; }
    per_sm = 1;   // one CTA per SM: fewest barrier arrivals
    int grid = c->num_sms * per_sm;
    if (grid > c->partial_blocks) grid = c->partial_blocks;
    if (grid_out) *grid_out = grid;
    void* params[] = {reinterpret_cast<void*>(&args)...};
    MTK_TRY(reset_barrier(c));
    MTK_CUDA_TRY(cudaLaunchCooperativeKernel(reinterpret_cast<void*>(kernel), dim3(grid), dim3(kBlock), params, 0, c->stream));
    c->kernels++;
    return MTK_OK;
}

inline int stream_grid(mtk_ctx* c) { return c->num_sms * 2; }

}  // namespace mtk
