// SELL-32 copies of the solvers' CSR matrices (sliced ELLPACK, slice height 32, no row sorting).
//
// Rows are taken 32 at a time (a slice); each slice is padded to its longest row and stored
// column-major, so entry k of row r sits at sptr[r / 32] + 32 k + (r % 32).  A warp that owns a
// slice -- lane i on row 32 s + i, the same thread <-> row mapping as the persistent kernels'
// grid-stride row loops -- then reads each entry position with one coalesced request instead of
// 32 scattered ones.  Padding entries have column -1 and value 0 and are skipped, and the
// entries of a row are visited in CSR order, so a row sum comes out bit-identical to the CSR
// one-thread-per-row loop.
//
// Built on the device once per matrix (set-up): slice widths, a host scan of the slice sizes
// (one small copy each way), then a fill pass.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "mtk_ctx.cuh"

namespace mtk {

// When a SELL-32 copy pays (measured on the GB300 with the persistent solvers' phase timers, at
// 1.3M faces): on the phases of levels with at least 100K rows and at most 48 entries per row on
// average -- the restriction of the IGM free block's first level (about 43 entries per row:
// 39.1 -> 28.1 us per application) and the up-phase of the field's first inner level
// (28.4 -> 22.3 us), where one lane per row with coalesced entry loads beats the scattered
// per-thread row walks.  Small levels (fewer rows than the grid has threads) lose lane
// parallelism and keep CSR; so does the finest IGM level's up-phase (about 7 entries per row:
// 63 -> 70 us with SELL), which the caller leaves out.
constexpr double kSellMaxAvg = 48.0;
constexpr int kSellMinRows = 100000;
inline bool sell_worth(int n, double avg) { return n >= kSellMinRows && avg <= kSellMaxAvg; }

namespace sellk {
// w[s] = longest row of slice s
static __global__ void slice_widths(int n, const int* __restrict__ ptr, int* w) {
    const int ns = (n + 31) >> 5;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < ns; s += gridDim.x * blockDim.x) {
        int m = 0;
        const int r1 = min(n, 32 * s + 32);
        for (int r = 32 * s; r < r1; r++) m = max(m, __ldg(ptr + r + 1) - __ldg(ptr + r));
        w[s] = m;
    }
}

// one thread per row slot (32 per slice, padding slots included); scol / val may be null
template <typename V>
static __global__ void fill(int n, const int* __restrict__ ptr, const int* __restrict__ col, const V* __restrict__ val,
                            const int* __restrict__ sptr, int* scol, V* sval) {
    const int ns = (n + 31) >> 5;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < 32LL * ns; q += (long long)gridDim.x * blockDim.x) {
        const int r = (int)q, s = r >> 5, lane = r & 31;
        const int b = sptr[s], w = (sptr[s + 1] - b) >> 5;
        const int p0 = r < n ? ptr[r] : 0, len = r < n ? ptr[r + 1] - p0 : 0;
        for (int k = 0; k < w; k++) {
            const int o = b + 32 * k + lane;
            if (k < len) {
                if (scol) scol[o] = col[p0 + k];
                if (val) sval[o] = val[p0 + k];
            } else {
                if (scol) scol[o] = -1;
                if (val) sval[o] = V{};
            }
        }
    }
}
}  // namespace sellk

// Device SELL-32 arrays of one matrix (column indices shared by the value copies).
struct SellIdx {
    DBuf<int> sptr, scol;
    long long entries = 0;   // padded entries (32 x sum of slice widths)
};

// Slice layout of the n-row CSR (ptr, col) on `st`: sptr (slices + 1) and scol.
inline int sell_build_index(mtk_ctx* c, cudaStream_t st, int n, const int* ptr, const int* col, SellIdx& S) {
    const int ns = (n + 31) >> 5;
    DBuf<int> w;
    MTK_TRY(w.alloc(std::max(ns, 1)));
    if (ns > 0) sellk::slice_widths<<<stream_grid(c), kStream, 0, st>>>(n, ptr, w.p);
    MTK_CUDA_TRY(cudaGetLastError());
    std::vector<int> hw(ns), hp(ns + 1, 0);
    if (ns > 0) MTK_CUDA_TRY(cudaMemcpyAsync(hw.data(), w.p, sizeof(int) * ns, cudaMemcpyDeviceToHost, st));
    MTK_CUDA_TRY(cudaStreamSynchronize(st));
    long long tot = 0;
    for (int s = 0; s < ns; s++) {
        hp[s] = (int)tot;
        tot += 32LL * hw[s];
    }
    if (tot > 2147483647LL) { mtk_set_last_error("SELL-32 matrix beyond 2^31 entries", __FILE__, __LINE__); return MTK_ERR_BAD_INPUT; }
    hp[ns] = (int)tot;
    S.entries = tot;
    MTK_TRY(S.sptr.upload(hp.data(), hp.size(), st));
    MTK_TRY(S.scol.alloc(std::max<long long>(tot, 1)));
    if (ns > 0)
        sellk::fill<int><<<stream_grid(c), kStream, 0, st>>>(n, ptr, col, nullptr, S.sptr.p, S.scol.p, nullptr);
    c->kernels += ns > 0 ? 2 : 0;
    MTK_CUDA_TRY(cudaGetLastError());
    return MTK_OK;
}

// Values of the CSR (ptr, col, val) in the slice layout of S.
template <typename V>
int sell_fill_values(mtk_ctx* c, cudaStream_t st, int n, const int* ptr, const int* col, const V* val, const SellIdx& S,
                     DBuf<V>& sval) {
    const int ns = (n + 31) >> 5;
    MTK_TRY(sval.alloc(std::max<long long>(S.entries, 1)));
    if (ns > 0) {
        sellk::fill<V><<<stream_grid(c), kStream, 0, st>>>(n, ptr, col, val, S.sptr.p, nullptr, sval.p);
        c->kernels++;
    }
    MTK_CUDA_TRY(cudaGetLastError());
    return MTK_OK;
}

}  // namespace mtk
