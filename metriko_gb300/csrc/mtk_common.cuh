// Shared device helpers for the metriko GB300 kernels.
//
// * status codes returned through the C ABI (include/metriko_cuda.h);
// * a bounded software grid barrier for cooperative persistent kernels: every spin has an
//   iteration cap after which the kernel records MTK_ERR_TIMEOUT in a device flag and all
//   blocks leave the solve loop (no trap, no unbounded wait);
// * deterministic reductions: every block writes one partial per slot, and after the grid
//   barrier every block re-reduces all partials in the same fixed order, so each block holds
//   bit-identical scalars without a second barrier.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>

#include "metriko_cuda.h"

#define MTK_CUDA_TRY(expr)                                                           \
    do {                                                                             \
        cudaError_t _e = (expr);                                                     \
        if (_e != cudaSuccess) {                                                     \
            mtk_set_last_error(cudaGetErrorString(_e), __FILE__, __LINE__);          \
            return MTK_ERR_CUDA;                                                     \
        }                                                                            \
    } while (0)

#define MTK_TRY(expr)                          \
    do {                                       \
        int _s = (expr);                       \
        if (_s != MTK_OK) return _s;           \
    } while (0)

void mtk_set_last_error(const char* msg, const char* file, int line);

namespace mtk {

constexpr int kBlock = 1024;              // threads per CTA (persistent solvers: one CTA per SM)
constexpr int kWarps = kBlock / 32;      // upper bound on warps per CTA
constexpr int kStream = 256;              // threads per CTA of the streaming (non-persistent) kernels
constexpr long long kSpinLimit = 1LL << 24;   // bounded spin (about a second with backoff)

struct GridBarrier {
    unsigned int* count;       // arrivals in the current generation
    unsigned int* gen;         // generation counter
    int* err;                  // sticky error flag (MTK_ERR_TIMEOUT)
    long long limit = kSpinLimit;   // polls before a waiting CTA gives up
};

__device__ __forceinline__ unsigned int ld_acquire(const unsigned int* p) {
    unsigned int v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(unsigned int* p, unsigned int v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ int ld_volatile(const int* p) {
    return *reinterpret_cast<const volatile int*>(p);
}

__device__ __forceinline__ unsigned int atom_add_acq_rel(unsigned int* p, unsigned int v) {
    unsigned int old;
    asm volatile("atom.add.acq_rel.gpu.global.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}
__device__ __forceinline__ void st_relaxed(unsigned int* p, unsigned int v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Grid-wide barrier for a cooperative launch (one CTA per SM).  Thread 0 of every CTA
// arrives with an acq_rel atomic; the last arrival resets the counter and publishes the next
// generation with a release store; the others poll it with acquire loads (tight spin first,
// then nanosleep backoff) for at most `limit` polls (kSpinLimit unless the context sets a
// smaller wait limit), after which MTK_ERR_TIMEOUT is
// recorded and every CTA leaves.  Returns false (in every thread) on timeout or a recorded
// error; callers then leave their loop.
__device__ __forceinline__ bool grid_sync(const GridBarrier& b) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = ld_volatile(b.err) == 0;
        if (ok) {
            unsigned int g = ld_acquire(b.gen);
            unsigned int arrived = atom_add_acq_rel(b.count, 1u);
            if (arrived == gridDim.x - 1) {
                st_relaxed(b.count, 0u);
                st_release(b.gen, g + 1);
            } else {
                long long spins = 0;
                while (ld_acquire(b.gen) == g) {
                    if (++spins > b.limit) { atomicExch(b.err, (int)MTK_ERR_TIMEOUT); ok = 0; break; }
                    if ((spins & 255) == 0 && ld_volatile(b.err) != 0) { ok = 0; break; }
                    if (spins > 2048) __nanosleep(100);
                }
            }
        }
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// Fixed-order block reduction of K values per thread; result valid in all threads.
// a * b + c with one rounding (values recomputed by several threads come out bit-identical)
template <typename T> __device__ __forceinline__ T fmaT(T a, T b, T c);
template <> __device__ __forceinline__ float fmaT<float>(float a, float b, float c) { return __fmaf_rn(a, b, c); }
template <> __device__ __forceinline__ double fmaT<double>(double a, double b, double c) { return __fma_rn(a, b, c); }

template <typename T, int K>
__device__ __forceinline__ void block_sum(T (&v)[K]) {
    __shared__ T s_red[K][kWarps];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < K; k++) {
        T x = v[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if (lane == 0) s_red[k][warp] = x;
    }
    __syncthreads();
    const int nw = (int)(blockDim.x >> 5);
#pragma unroll
    for (int k = 0; k < K; k++) {
        T x = T(0);
        for (int w = 0; w < nw; w++) x += s_red[k][w];
        v[k] = x;
    }
    __syncthreads();
}

// Writes the block partials (K values) to partials[k * gridDim.x + blockIdx.x].
template <typename T, int K>
__device__ __forceinline__ void publish_partials(T (&v)[K], T* partials) {
    block_sum<T, K>(v);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < K; k++) partials[k * gridDim.x + blockIdx.x] = v[k];
    }
}

// After a grid barrier: every block reduces all partials in the same order.
template <typename T, int K>
__device__ __forceinline__ void gather_partials(const T* partials, T (&out)[K]) {
    T v[K];
#pragma unroll
    for (int k = 0; k < K; k++) {
        T x = T(0);
        for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) x += __ldcg(partials + k * gridDim.x + b);
        v[k] = x;
    }
    block_sum<T, K>(v);
#pragma unroll
    for (int k = 0; k < K; k++) out[k] = v[k];
}

// ----------------------------------------------------------------- small complex helpers
template <typename T> struct cplx { T re, im; };
template <typename T> __device__ __forceinline__ cplx<T> cmul(cplx<T> a, cplx<T> b) {
    return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
template <typename T> __device__ __forceinline__ cplx<T> cadd(cplx<T> a, cplx<T> b) { return {a.re + b.re, a.im + b.im}; }

}  // namespace mtk
