// Integer-grid-map integration and greedy rounding on the device.
//
// Replaces (metriko) iterative_rounding (iter_rounding.h:33-113), NaiveIntegration
// (iter_rounding_init.h:16-233), SeamlessIntegration (iter_rounding_loop.h:10-125) and the
// per-iteration SimplicialLLT factorisations of LMSolver (levenberg_marquardt.h:140-231).
//
// Structure used instead of assembling X2F^T X2F on the host:
//   X2F = G2 * fullx2Nfunc * UFull, and under sign symmetry (functions k+n = -functions k)
//   X2F^T X2F = UFull^T (2 W^T S W) UFull,
// with S the per-face gradient Gram matrix of the cut mesh (S_ab = sum_f g_a . g_b, a scalar
// stiffness shared by u and v), W the cut-vertex <- full-variable map (rows k < n of
// fullx2Nfunc: +-1 permutations plus seam translations) and UFull = [I ; USmall] in the
// reference's reduced coordinates xs = [y ; z].  The operator is applied matrix-free:
//   B: U = W [y ; USmall z]   (u,v of every cut vertex: two right-hand sides in one pass)
//   C: Q = S U                (SELL-free padded CSR, one thread per cut vertex)
//   D: y' = 2 W_y^T Q,  XJ' = 2 W_J^T Q
//   E: z' = USmall^T XJ'      (replicated per block: nZ is small)
// The kernel coordinates z (and the constraint projector on them) are replicated in every
// block's shared memory, so the constrained block costs no extra grid barrier.
//
// Constraints (the reference's 1e8 / 1e10 penalty rows) are imposed exactly by projection:
// fixed free variables are Dirichlet entries, fixed constrained variables are rows of USmall
// on z, kept orthonormal (Q) so that P_z = I - Q^T Q.  The difference from the penalty
// solution is O(1 / penalty).
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <vector>

#include "mtk_amg_real.cuh"
#include "mtk_amg_real_gpu.cuh"
#include "mtk_ctx.cuh"
#include "mtk_sell.cuh"

namespace mtk {

constexpr int kMaxFaceDeg = 30;   // faces around one cut vertex (stiffness row capacity)

template <typename T>
struct IgmOp {
    int nCut, nY, nZ, nJ;
    const int* w_ptr;   // 2*nCut + 1
    const int* w_tag;   // >= 0: y index, < 0: -1 - J slot
    const T* w_val;
    const int* s_ptr;   // nCut + 1 (padded rows)
    const int* s_col;
    const T* s_val;
    const int* yt_ptr;  // nY + 1: rows r (= 2c + k) referencing y_j
    const int* yt_row;
    const T* yt_val;
    const int* jt_ptr;  // nJ + 1
    const int* jt_row;
    const T* jt_val;
    const T* Us;        // nJ x nZ
    T scale, shift;
    T* U;               // 2*nCut gather buffer
    T* Qc;              // 2*nCut stiffness product
    T* XoJ;             // nJ
    // assembled operator (FP32 inner solves; null: the matrix-free chain above)
    const int* ka_ptr;  // K_yy = 2 W_y^T S W_y, nY rows (CSR)
    const int* ka_col;
    const T* ka_val;
    const int* cy_ptr;  // C_yJ = 2 W_y^T S W_J, nY rows, J columns
    const int* cy_col;
    const T* cy_val;
    const int* cj_ptr;  // C_Jy = C_yJ^T, nJ rows, y columns
    const int* cj_col;
    const T* cj_val;
    const T* BJJ;       // 2 W_J^T S W_J, nJ x nJ (row-major)
    // translation rows (the long lists of W_J^T / C_Jy: every cut copy along a seam segment
    // references its translation) cut into chunks of at most kJChunk entries, one warp each,
    // spread over the grid; chunk c of row jc_row[c] starts at entry jc_beg[c] of that row's list
    // and writes its partial sum to XoJp[c]; row s owns the chunks [jc_first[s], jc_first[s + 1]),
    // which the reader adds in order.  jc_n = 0: one warp per row.
    int jc_n = 0;
    const int* jc_row = nullptr;
    const int* jc_beg = nullptr;
    const int* jc_first = nullptr;
    T* XoJp = nullptr;
};
constexpr int kJChunk = 256;

// chunks of the translation rows given their CSR row pointer (host)
inline void translation_chunks(const std::vector<int>& ptr, std::vector<int>& row, std::vector<int>& beg,
                               std::vector<int>& first) {
    const int nJ = (int)ptr.size() - 1;
    row.clear(); beg.clear(); first.assign(nJ + 1, 0);
    for (int s = 0; s < nJ; s++) {
        first[s] = (int)row.size();
        int e = ptr[s];
        do {
            row.push_back(s);
            beg.push_back(e);
            e += kJChunk;
        } while (e < ptr[s + 1]);
    }
    first[nJ] = (int)row.size();
}
// the end of chunk c: kJChunk entries on, or its row's end
__device__ __forceinline__ int jchunk_end(const int* __restrict__ ptr, const int* __restrict__ jc_row,
                                          const int* __restrict__ jc_beg, int c) {
    const int e = jc_beg[c] + kJChunk;
    const int re = ptr[jc_row[c] + 1];
    return e < re ? e : re;
}

// Shared-memory layout of the replicated z state (cz, wsum: the Schur coarse space).
template <typename T>
struct ZSmem {
    T *xz, *rz, *zz, *pz, *qz, *XJ, *tmpJ, *tz, *cz, *wsum;
    __device__ void bind(T* base, int nZ, int nJ) {
        xz = base; rz = xz + nZ; zz = rz + nZ; pz = zz + nZ; qz = pz + nZ; tz = qz + nZ;
        XJ = tz + nZ; tmpJ = XJ + nJ; cz = tmpJ + nJ; wsum = cz + nZ;
    }
};
constexpr int kPhiSlot = 8;     // partials offset (in blocks) of the coarse-space dots
constexpr int kMaxPhi = 64;     // largest z block that gets the Schur coarse space
// bytes of ZSmem for nZ, nJ (the per-warp coarse-space sums only where the coarse space can be on)
__host__ __device__ inline size_t zsmem_bytes(size_t elem, int nZ, int nJ) {
    return elem * (7 * (size_t)nZ + 2 * (size_t)nJ + (nZ <= kMaxPhi ? (size_t)kWarps * nZ : 0) + 8);
}

template <typename T>
struct ZProj {
    int kq;             // orthonormal constraint rows on z
    const T* Q;         // kq x nZ
    const T* Minv;      // nZ x nZ (dense inverse of the z block) or nullptr
};

// v <- v - Q^T (Q v) on a replicated smem vector (block-wide).  tmp: >= kq scratch.
template <typename T>
__device__ void project_z(const ZProj<T>& P, int nZ, T* v, T* tmp) {
    if (P.kq == 0) return;
    for (int a = threadIdx.x; a < P.kq; a += blockDim.x) {
        T s = T(0);
        for (int j = 0; j < nZ; j++) s += P.Q[(size_t)a * nZ + j] * v[j];
        tmp[a] = s;
    }
    __syncthreads();
    for (int j = threadIdx.x; j < nZ; j += blockDim.x) {
        T s = v[j];
        for (int a = 0; a < P.kq; a++) s -= P.Q[(size_t)a * nZ + j] * tmp[a];
        v[j] = s;
    }
    __syncthreads();
}

// out = Minv * in (dense) or copy; replicated.
template <typename T>
__device__ void precond_z(const ZProj<T>& P, int nZ, const T* in, T* out) {
    for (int j = threadIdx.x; j < nZ; j += blockDim.x) {
        T s = T(0);
        if (P.Minv) {
            for (int k = 0; k < nZ; k++) s += P.Minv[(size_t)j * nZ + k] * in[k];
        } else {
            s = in[j];
        }
        out[j] = s;
    }
    __syncthreads();
}

// Fixed-order block dot of two replicated smem vectors (same value in every block).
template <typename T>
__device__ T smem_dot(const T* a, const T* b, int n) {
    T v[1] = {T(0)};
    for (int j = threadIdx.x; j < n; j += blockDim.x) v[0] += a[j] * b[j];
    block_sum<T, 1>(v);
    return v[0];
}

// Operator K p, with p = [py (global) ; pz (smem)].  Result: qy (global, masked, projected)
// and qz (smem, projected).  Returns partial <py, qy> of this block in *pq_part and false on
// a barrier failure.  Three grid barriers.  With pnew set, the free part of the direction is
// formed on the fly, p_y = zy + beta py (every reader recomputes it with one rounding), and
// written to pnew by the thread that owns the row in phase D.
template <typename T>
__device__ bool igm_apply(const IgmOp<T>& A, const ZProj<T>& P, const unsigned char* __restrict__ fixy,
                          const T* py, const T* pz, T* qy, T* qz, ZSmem<T>& zs, const GridBarrier& bar, T& pq_part,
                          const T* zy = nullptr, T beta = T(0), T* pnew = nullptr) {
    const int stride = gridDim.x * blockDim.x;
    const int t0 = blockIdx.x * blockDim.x + threadIdx.x;
    // A (replicated): XJ = USmall pz
    for (int s = threadIdx.x; s < A.nJ; s += blockDim.x) {
        T acc = T(0);
        const T* row = A.Us + (size_t)s * A.nZ;
        for (int j = 0; j < A.nZ; j++) acc += row[j] * pz[j];
        zs.XJ[s] = acc;
    }
    __syncthreads();
    // B: U = W [py ; XJ]
    for (int r = t0; r < 2 * A.nCut; r += stride) {
        T acc = T(0);
        for (int e = A.w_ptr[r]; e < A.w_ptr[r + 1]; e++) {
            int tag = A.w_tag[e];
            T xv;
            if (tag < 0) xv = zs.XJ[-1 - tag];
            else if (pnew) xv = fmaT<T>(beta, __ldcg(py + tag), __ldcg(zy + tag));
            else xv = __ldcg(py + tag);
            acc += A.w_val[e] * xv;
        }
        A.U[r] = acc;
    }
    if (!grid_sync(bar)) return false;
    // C: Qc = S U  (two right-hand sides per row)
    for (int c = t0; c < A.nCut; c += stride) {
        T a0 = T(0), a1 = T(0);
        for (int e = A.s_ptr[c]; e < A.s_ptr[c + 1]; e++) {
            int b = A.s_col[e];
            T s = A.s_val[e];
            a0 += s * __ldcg(A.U + 2 * b);
            a1 += s * __ldcg(A.U + 2 * b + 1);
        }
        A.Qc[2 * c] = a0;
        A.Qc[2 * c + 1] = a1;
    }
    if (!grid_sync(bar)) return false;
    // D: qy = scale * 2 W_y^T Qc + shift * py (masked);  XoJ = 2 W_J^T Qc
    const T two_scale = T(2) * A.scale;
    T part = T(0);
    for (int j = t0; j < A.nY; j += stride) {
        T acc = T(0);
        for (int e = A.yt_ptr[j]; e < A.yt_ptr[j + 1]; e++) acc += A.yt_val[e] * __ldcg(A.Qc + A.yt_row[e]);
        T pj;
        if (pnew) {
            pj = fmaT<T>(beta, __ldcg(py + j), __ldcg(zy + j));
            pnew[j] = pj;
        } else {
            pj = __ldcg(py + j);
        }
        T qv = fixy[j] ? T(0) : two_scale * acc + A.shift * pj;
        qy[j] = qv;
        part += pj * qv;
    }
    // constrained variables: seam translations are referenced by every cut copy along their
    // seam segment (long lists), so one warp reduces each list (fixed lane order)
    {
        const int lane = threadIdx.x & 31;
        const int nwarps = stride >> 5;
        const int gw = nwarps - 1 - (t0 >> 5);   // last warps of the grid
        if (A.jc_n > 0) {
            for (int ch = gw; ch < A.jc_n; ch += nwarps) {
                T acc = T(0);
                const int e1 = jchunk_end(A.jt_ptr, A.jc_row, A.jc_beg, ch);
                for (int e = A.jc_beg[ch] + lane; e < e1; e += 32) acc += A.jt_val[e] * __ldcg(A.Qc + A.jt_row[e]);
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
                if (lane == 0) A.XoJp[ch] = T(2) * acc;
            }
        } else {
            for (int s = gw; s < A.nJ; s += nwarps) {
                T acc = T(0);
                for (int e = A.jt_ptr[s] + lane; e < A.jt_ptr[s + 1]; e += 32) acc += A.jt_val[e] * __ldcg(A.Qc + A.jt_row[e]);
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
                if (lane == 0) A.XoJ[s] = T(2) * acc;
            }
        }
    }
    pq_part = part;
    return true;
    // (E is done by the caller after the next barrier: igm_apply_z)
}

// The same operator from the assembled blocks, in one phase and one grid barrier (taken by the
// caller): XJ = USmall pz (replicated); per free row q_y = scale (K_yy p + C_yJ XJ) + shift p
// (masked), and per translation XoJ = C_Jy p + BJJ XJ (one warp each, fixed lane order).  The
// direction is formed on the fly as in igm_apply.
template <typename T>
__device__ bool igm_apply_asm(const IgmOp<T>& A, const unsigned char* __restrict__ fixy, const T* py, const T* pz,
                              T* qy, ZSmem<T>& zs, T& pq_part, const T* zy = nullptr, T beta = T(0),
                              T* pnew = nullptr) {
    const int stride = gridDim.x * blockDim.x;
    const int t0 = blockIdx.x * blockDim.x + threadIdx.x;
    for (int s = threadIdx.x; s < A.nJ; s += blockDim.x) {
        T acc = T(0);
        const T* row = A.Us + (size_t)s * A.nZ;
        for (int j = 0; j < A.nZ; j++) acc += row[j] * pz[j];
        zs.XJ[s] = acc;
    }
    __syncthreads();
    T part = T(0);
    for (int j = t0; j < A.nY; j += stride) {
        T pj;
        if (pnew) {
            pj = fmaT<T>(beta, __ldcg(py + j), __ldcg(zy + j));
            pnew[j] = pj;
        } else {
            pj = __ldcg(py + j);
        }
        T acc = T(0);
        const int e1 = __ldg(A.ka_ptr + j + 1);
        for (int e = __ldg(A.ka_ptr + j); e < e1; e += 4) {   // four gathers in flight
            int cc[4];
            T vv[4], pc[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                cc[u] = e + u < e1 ? __ldg(A.ka_col + e + u) : -1;
                vv[u] = e + u < e1 ? __ldg(A.ka_val + e + u) : T(0);
            }
#pragma unroll
            for (int u = 0; u < 4; u++) {
                if (cc[u] < 0) { pc[u] = T(0); continue; }
                pc[u] = pnew ? fmaT<T>(beta, __ldcg(py + cc[u]), __ldcg(zy + cc[u])) : __ldcg(py + cc[u]);
            }
#pragma unroll
            for (int u = 0; u < 4; u++) acc += vv[u] * pc[u];
        }
        for (int e = __ldg(A.cy_ptr + j); e < __ldg(A.cy_ptr + j + 1); e++) acc += __ldg(A.cy_val + e) * zs.XJ[__ldg(A.cy_col + e)];
        const T qv = fixy[j] ? T(0) : A.scale * acc + A.shift * pj;
        qy[j] = qv;
        part += pj * qv;
    }
    {
        const int lane = threadIdx.x & 31;
        const int nwarps = stride >> 5;
        const int gw = nwarps - 1 - (t0 >> 5);   // last warps of the grid
        if (A.jc_n > 0) {
            for (int ch = gw; ch < A.jc_n; ch += nwarps) {
                const int s = A.jc_row[ch];
                T acc = T(0);
                const int e1 = jchunk_end(A.cj_ptr, A.jc_row, A.jc_beg, ch);
                for (int e = A.jc_beg[ch] + lane; e < e1; e += 32) {
                    const int y = A.cj_col[e];
                    const T pv = pnew ? fmaT<T>(beta, __ldcg(py + y), __ldcg(zy + y)) : __ldcg(py + y);
                    acc += A.cj_val[e] * pv;
                }
                if (ch == A.jc_first[s])   // the row's first chunk also takes the dense J block
                    for (int t = lane; t < A.nJ; t += 32) acc += A.BJJ[(size_t)s * A.nJ + t] * zs.XJ[t];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
                if (lane == 0) A.XoJp[ch] = acc;
            }
        } else {
            for (int s = gw; s < A.nJ; s += nwarps) {
                T acc = T(0);
                for (int e = A.cj_ptr[s] + lane; e < A.cj_ptr[s + 1]; e += 32) {
                    const int y = A.cj_col[e];
                    const T pv = pnew ? fmaT<T>(beta, __ldcg(py + y), __ldcg(zy + y)) : __ldcg(py + y);
                    acc += A.cj_val[e] * pv;
                }
                for (int t = lane; t < A.nJ; t += 32) acc += A.BJJ[(size_t)s * A.nJ + t] * zs.XJ[t];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
                if (lane == 0) A.XoJ[s] = acc;
            }
        }
    }
    pq_part = part;
    return true;
}

// Schur coarse space of the z block.  Phi (nY x nZ; the kernels read an FP16 row-major copy) holds approximations of
// -K_yy^-1 K_yz, so the columns of Z = [Phi ; I] are the z directions extended into the free
// block with (nearly) least energy; the preconditioner adds Z W Z^T r to the multigrid of the
// free block, W = P (P G P + ridge)^-1 P with G = Z^T K Z (the P's keep it on the feasible z
// directions; rows of fixed variables are zero in the input and masked in the output).  With
// an exact Phi this is the block factorisation K^-1 = [K_yy^-1 0; 0 0] + Z S^-1 Z^T (S the Schur
// complement of the z block), so the coupled system converges like the free block alone.
//
// Block partials of Phi^T r_y in fixed order: out[k * gridDim.x + blockIdx.x].  Phi is row-major
// FP16 with rows padded to kp = nZ rounded up to 8 (16-byte loads); the columns are taken
// kPhiChunk at a time in one pass over r (each thread keeps one sum per column of the chunk, over
// the same rows in the same order as a pass per column would).
constexpr int kPhiChunk = 16;
template <typename T>
__device__ void phi_dots_publish(const __half* __restrict__ Phi, int nY, int nZ, const T* r, T* out, T* wsum) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int stride = gridDim.x * blockDim.x;
    const int t0 = blockIdx.x * blockDim.x + threadIdx.x;
    const int kp = (nZ + 7) & ~7;
    for (int k0 = 0; k0 < nZ; k0 += kPhiChunk) {
        const int kc = nZ - k0 < kPhiChunk ? nZ - k0 : kPhiChunk;
        T a[kPhiChunk];
#pragma unroll
        for (int u = 0; u < kPhiChunk; u++) a[u] = T(0);
        for (int j = t0; j < nY; j += stride) {
            const T rj = __ldcg(r + j);
#pragma unroll
            for (int g = 0; g < kPhiChunk / 8; g++) {
                if (8 * g >= kc) break;
                const uint4 v = __ldg(reinterpret_cast<const uint4*>(Phi + (size_t)j * kp + k0 + 8 * g));
                const __half2* h2 = reinterpret_cast<const __half2*>(&v);
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const float2 f = __half22float2(h2[q]);
                    a[8 * g + 2 * q] += (T)f.x * rj;
                    a[8 * g + 2 * q + 1] += (T)f.y * rj;
                }
            }
        }
#pragma unroll
        for (int u = 0; u < kPhiChunk; u++) {
            T v = a[u];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0 && u < kc) wsum[warp * nZ + k0 + u] = v;
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < nZ; k += blockDim.x) {
        T v = T(0);
        for (int w = 0; w < nw; w++) v += wsum[w * nZ + k];
        out[k * gridDim.x + blockIdx.x] = v;
    }
    __syncthreads();
}

// After a grid barrier: c = P (Phi^T r_y + r_z), zz = P Minv c (the coarse coefficients y_c).
template <typename T>
__device__ void phi_coarse(const ZProj<T>& P, int nZ, const T* parts, ZSmem<T>& zs) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int k = warp; k < nZ; k += nw) {
        T v = T(0);
        for (int b = lane; b < (int)gridDim.x; b += 32) v += __ldcg(parts + k * gridDim.x + b);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) zs.cz[k] = v + zs.rz[k];
    }
    __syncthreads();
    project_z(P, nZ, zs.cz, zs.tz);
    precond_z(P, nZ, zs.cz, zs.zz);
    project_z(P, nZ, zs.zz, zs.tz);
}

// E (replicated, after a barrier): qz = P_z (scale USmall^T XoJ + shift pz)
template <typename T>
__device__ void igm_apply_z(const IgmOp<T>& A, const ZProj<T>& P, const T* pz, T* qz, ZSmem<T>& zs) {
    for (int s = threadIdx.x; s < A.nJ; s += blockDim.x) {
        if (A.jc_n > 0) {   // the row's chunk partials in chunk order
            T v = T(0);
            for (int ch = A.jc_first[s]; ch < A.jc_first[s + 1]; ch++) v += __ldcg(A.XoJp + ch);
            zs.tmpJ[s] = v;
        } else {
            zs.tmpJ[s] = __ldcg(A.XoJ + s);
        }
    }
    __syncthreads();
    for (int j = threadIdx.x; j < A.nZ; j += blockDim.x) {
        T acc = T(0);
        for (int s = 0; s < A.nJ; s++) acc += A.Us[(size_t)s * A.nZ + j] * zs.tmpJ[s];
        qz[j] = A.scale * acc + A.shift * pz[j];
    }
    __syncthreads();
    project_z(P, A.nZ, qz, zs.tz);
}

// Persistent projected PCG.  mode 0: solve K x = b from a feasible x (x, b: [y ; z] global).
// mode 1: residual only, r = P(b - K x) written to r, |r|^2 in out.
// out[0] status, out[1] iterations, (double*)(out+4): final |r|^2.
// ZG: the replicated z state of each CTA lives in its own slice of zglob (zstride values) instead
// of shared memory, for constraint kernels too large for an SM's shared memory (a mesh with
// many singularities); the arithmetic is the same.
template <typename T, bool ZG>
__global__ void __launch_bounds__(kBlock, 1) igm_pcg(IgmOp<T> A, ZProj<T> P, const unsigned char* __restrict__ fixy,
                                                 const T* __restrict__ minvy, const T* __restrict__ b, T* x, T* r, T* z,
                                                 T* p, T* p2, T* q, T* partials, GridBarrier bar, double tol2,
                                                 int maxit, int mode, int* out,
                                                 const RDevHierarchy<T>* __restrict__ Hp, T mg_scale,
                                                 const __half* __restrict__ Phi, T* zglob, long long zstride) {
    extern __shared__ unsigned char smem_raw[];
    ZSmem<T> zs;
    zs.bind(ZG ? zglob + (size_t)blockIdx.x * (size_t)zstride : reinterpret_cast<T*>(smem_raw), A.nZ, A.nJ);
    const int nY = A.nY, nZ = A.nZ;
    const int stride = gridDim.x * blockDim.x;
    const int t0 = blockIdx.x * blockDim.x + threadIdx.x;
    int status = 3, it = 0;
    T rr = T(0);
    T part[2];
    T pq1[1];
    const bool defl = Phi && Hp && mode == 0 && nZ > 0;   // Schur coarse space on (see phi_coarse)
    T* phi_parts = partials + kPhiSlot * gridDim.x;
    // replicated z state
    for (int j = threadIdx.x; j < nZ; j += blockDim.x) {
        zs.xz[j] = x[nY + j];
        zs.pz[j] = x[nY + j];
    }
    __syncthreads();
    // r = P(b - K x): apply K to x (py = x_y)
    T pqp = T(0);
    if (A.ka_ptr) igm_apply_asm(A, fixy, x, zs.pz, q, zs, pqp);
    else if (!igm_apply(A, P, fixy, x, zs.pz, q, zs.qz, zs, bar, pqp)) { status = 5; goto done; }
    if (!grid_sync(bar)) { status = 5; goto done; }
    igm_apply_z(A, P, zs.pz, zs.qz, zs);
    part[0] = T(0);
    part[1] = T(0);
    for (int j = t0; j < nY; j += stride) {
        T rj = fixy[j] ? T(0) : b[j] - q[j];
        r[j] = rj;
        part[1] += rj * rj;
        if (mode == 0 && !Hp) {
            T zj = minvy[j] * rj;
            z[j] = zj;
            part[0] += rj * zj;
        }
    }
    for (int j = threadIdx.x; j < nZ; j += blockDim.x) zs.rz[j] = __ldg(b + nY + j) - zs.qz[j];
    __syncthreads();
    project_z(P, nZ, zs.rz, zs.tz);
    if (defl) phi_dots_publish(Phi, nY, nZ, r, phi_parts, zs.wsum);
    if (mode == 0 && Hp) {   // multigrid on the free block: z_y = mask (B r_y) / scale (+ Phi y_c)
        if (!grid_sync(bar)) { status = 5; goto done; }
        if (defl) phi_coarse(P, nZ, phi_parts, zs);
        if (!rvcycle(*Hp, mg_scale, fixy, bar, &part[0], defl ? Phi : nullptr, nZ, zs.zz)) { status = 5; goto done; }
    }
    if (mode == 0) {
        if (!defl) {
            precond_z(P, nZ, zs.rz, zs.zz);
            project_z(P, nZ, zs.zz, zs.tz);
        }
        for (int j = threadIdx.x; j < nZ; j += blockDim.x) zs.pz[j] = zs.zz[j];
        __syncthreads();
    }
    publish_partials<T, 2>(part, partials);
    if (!grid_sync(bar)) { status = 5; goto done; }
    gather_partials<T, 2>(partials, part);
    {
        T rz = part[0] + (mode == 0 ? smem_dot(zs.rz, zs.zz, nZ) : T(0));
        rr = part[1] + smem_dot(zs.rz, zs.rz, nZ);
        if (mode == 1) {
            if (blockIdx.x == 0)
                for (int j = threadIdx.x; j < nZ; j += blockDim.x) r[nY + j] = zs.rz[j];
            status = 0;
            goto done;
        }
        T beta = T(0);
        const T* pold = z;   // first direction p = z (beta = 0)
        T* pw = p;
        for (;;) {
            if ((double)rr <= tol2) { status = 0; break; }
            if (it >= maxit) { status = 3; break; }
            // q = K p, p = z + beta p_old formed on the fly and stored in pw
            T pq_part = T(0);
            if (A.ka_ptr) igm_apply_asm(A, fixy, pold, zs.pz, q, zs, pq_part, z, beta, pw);
            else if (!igm_apply(A, P, fixy, pold, zs.pz, q, zs.qz, zs, bar, pq_part, z, beta, pw)) { status = 5; break; }
            pq1[0] = pq_part;
            publish_partials<T, 1>(pq1, partials + 2 * gridDim.x);
            if (!grid_sync(bar)) { status = 5; break; }
            gather_partials<T, 1>(partials + 2 * gridDim.x, pq1);
            igm_apply_z(A, P, zs.pz, zs.qz, zs);
            T pq = pq1[0] + smem_dot(zs.pz, zs.qz, nZ);
            if (!(pq > T(0))) {
                status = 4;
                if (blockIdx.x == 0 && threadIdx.x == 0) {
                    reinterpret_cast<double*>(out + 6)[0] = (double)pq;
                    reinterpret_cast<double*>(out + 8)[0] = (double)rz;
                    reinterpret_cast<double*>(out + 10)[0] = (double)pq1[0];
                }
                break;
            }
            T alpha = rz / pq;
            part[0] = T(0);
            part[1] = T(0);
            for (int j = t0; j < nY; j += stride) {
                T rj = r[j] - alpha * q[j];
                x[j] += alpha * pw[j];
                r[j] = rj;
                if (!Hp) {
                    T zj = minvy[j] * rj;
                    z[j] = zj;
                    part[0] += rj * zj;
                }
                part[1] += rj * rj;
            }
            for (int j = threadIdx.x; j < nZ; j += blockDim.x) {
                zs.xz[j] += alpha * zs.pz[j];
                zs.rz[j] -= alpha * zs.qz[j];
            }
            __syncthreads();
            if (defl) phi_dots_publish(Phi, nY, nZ, r, phi_parts, zs.wsum);
            if (Hp) {
                if (!grid_sync(bar)) { status = 5; break; }
                if (defl) phi_coarse(P, nZ, phi_parts, zs);
                if (!rvcycle(*Hp, mg_scale, fixy, bar, &part[0], defl ? Phi : nullptr, nZ, zs.zz)) { status = 5; break; }
            }
            if (!defl) {
                precond_z(P, nZ, zs.rz, zs.zz);
                project_z(P, nZ, zs.zz, zs.tz);
            }
            publish_partials<T, 2>(part, partials + 3 * gridDim.x);
            if (!grid_sync(bar)) { status = 5; break; }
            gather_partials<T, 2>(partials + 3 * gridDim.x, part);
            T rz_new = part[0] + smem_dot(zs.rz, zs.zz, nZ);
            rr = part[1] + smem_dot(zs.rz, zs.rz, nZ);
            if (rr != rr) { status = 4; break; }
            beta = rz_new / rz;
            rz = rz_new;
            for (int j = threadIdx.x; j < nZ; j += blockDim.x) zs.pz[j] = zs.zz[j] + beta * zs.pz[j];
            __syncthreads();
            pold = pw;
            pw = (pw == p) ? p2 : p;
            it++;
        }
        if (blockIdx.x == 0)
            for (int j = threadIdx.x; j < nZ; j += blockDim.x) x[nY + j] = zs.xz[j];
    }
done:
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        out[0] = status;
        out[1] = it;
        reinterpret_cast<double*>(out + 4)[0] = (double)rr;
    }
}

// ------------------------------------------------------------------------ set-up kernels
// Per-face hat-function gradients in the face frame (parameterization_integ.ipp:11-24):
// g_j = n x (P_{j+2} - P_{j+1}) / (2A); grad[6f + 2j] = g_j . bX, grad[6f + 2j + 1] = g_j . bY.
__global__ void face_gradients(int nF, const int* __restrict__ cutF, const double* __restrict__ V, double* grad) {
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < nF; f += gridDim.x * blockDim.x) {
        double P[3][3];
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 3; k++) P[j][k] = V[3 * cutF[3 * f + j] + k];
        double x[3], t[3], n[3];
        for (int k = 0; k < 3; k++) { x[k] = P[1][k] - P[0][k]; t[k] = -(P[0][k] - P[2][k]); }
        n[0] = x[1] * t[2] - x[2] * t[1];
        n[1] = x[2] * t[0] - x[0] * t[2];
        n[2] = x[0] * t[1] - x[1] * t[0];
        double nn = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
        double xn = sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
        double area = nn * 0.5;
        double un[3] = {n[0] / nn, n[1] / nn, n[2] / nn};
        double bx[3] = {x[0] / xn, x[1] / xn, x[2] / xn};
        double c[3];   // -(x cross n)
        c[0] = -(x[1] * n[2] - x[2] * n[1]);
        c[1] = -(x[2] * n[0] - x[0] * n[2]);
        c[2] = -(x[0] * n[1] - x[1] * n[0]);
        double cn = sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
        double by[3] = {c[0] / cn, c[1] / cn, c[2] / cn};
        for (int j = 0; j < 3; j++) {
            double e[3];
            for (int k = 0; k < 3; k++) e[k] = P[(j + 2) % 3][k] - P[(j + 1) % 3][k];
            double g[3];
            g[0] = (un[1] * e[2] - un[2] * e[1]) / (area * 2);
            g[1] = (un[2] * e[0] - un[0] * e[2]) / (area * 2);
            g[2] = (un[0] * e[1] - un[1] * e[0]) / (area * 2);
            grad[6 * f + 2 * j] = g[0] * bx[0] + g[1] * bx[1] + g[2] * bx[2];
            grad[6 * f + 2 * j + 1] = g[0] * by[0] + g[1] * by[1] + g[2] * by[2];
        }
    }
}

// Stiffness row of cut vertex c gathered from its faces (ascending face ids), entries sorted
// by column and written into the padded CSR row; padding entries are (c, 0).  Deterministic.
__global__ void assemble_stiffness(int nCut, const int* __restrict__ vf_ptr, const int* __restrict__ vf_face,
                                   const int* __restrict__ cutF, const double* __restrict__ grad,
                                   const int* __restrict__ s_ptr, int* s_col, double* s_val, float* s_val32,
                                   double* s_diag) {
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nCut; c += gridDim.x * blockDim.x) {
        int cols[kMaxFaceDeg + 2];
        double vals[kMaxFaceDeg + 2];
        int cnt = 0;
        for (int k = vf_ptr[c]; k < vf_ptr[c + 1]; k++) {
            int f = vf_face[k];
            int a = cutF[3 * f] == c ? 0 : (cutF[3 * f + 1] == c ? 1 : 2);
            double ga0 = grad[6 * f + 2 * a], ga1 = grad[6 * f + 2 * a + 1];
            for (int j = 0; j < 3; j++) {
                int bcol = cutF[3 * f + j];
                double v = ga0 * grad[6 * f + 2 * j] + ga1 * grad[6 * f + 2 * j + 1];
                int pos = -1;
                for (int q = 0; q < cnt; q++) if (cols[q] == bcol) { pos = q; break; }
                if (pos < 0) {
                    if (cnt < kMaxFaceDeg + 2) { cols[cnt] = bcol; vals[cnt] = v; cnt++; }
                } else {
                    vals[pos] += v;
                }
            }
        }
        for (int i = 1; i < cnt; i++) {   // insertion sort by column
            int kc = cols[i];
            double kv = vals[i];
            int j = i - 1;
            while (j >= 0 && cols[j] > kc) { cols[j + 1] = cols[j]; vals[j + 1] = vals[j]; j--; }
            cols[j + 1] = kc;
            vals[j + 1] = kv;
        }
        int base = s_ptr[c], cap = s_ptr[c + 1] - base;
        double dg = 0;
        for (int i = 0; i < cap; i++) {
            int col = i < cnt ? cols[i] : c;
            double v = i < cnt ? vals[i] : 0.0;
            s_col[base + i] = col;
            s_val[base + i] = v;
            s_val32[base + i] = (float)v;
            if (i < cnt && col == c) dg = v;
        }
        s_diag[c] = dg;
    }
}

// Per cut vertex: hb[2c + k] = sum_f g_c . (F[f,k] - F[f,k+n]) for k < n (N = 4, n = 2).
__global__ void cut_loads(int nCut, const int* __restrict__ vf_ptr, const int* __restrict__ vf_face,
                          const int* __restrict__ cutF, const double* __restrict__ grad, const double* __restrict__ Ff,
                          double* hb) {
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nCut; c += gridDim.x * blockDim.x) {
        double h[4] = {0, 0, 0, 0};
        for (int k = vf_ptr[c]; k < vf_ptr[c + 1]; k++) {
            int f = vf_face[k];
            int a = cutF[3 * f] == c ? 0 : (cutF[3 * f + 1] == c ? 1 : 2);
            double gx = grad[6 * f + 2 * a], gy = grad[6 * f + 2 * a + 1];
            for (int fn = 0; fn < 4; fn++) h[fn] += gx * Ff[8 * f + 2 * fn] + gy * Ff[8 * f + 2 * fn + 1];
        }
        hb[2 * c] = h[0] - h[2];
        hb[2 * c + 1] = h[1] - h[3];
    }
}

// Reduced right-hand side, free part: b_y = scale * W_y^T hb + shift * prev_y ; J part -> XbJ.
__global__ void rhs_reduce(int nY, int nJ, const int* __restrict__ yt_ptr, const int* __restrict__ yt_row,
                           const double* __restrict__ yt_val, const int* __restrict__ jt_ptr, const int* __restrict__ jt_row,
                           const double* __restrict__ jt_val, const double* __restrict__ hb, double scale, double shift,
                           const double* __restrict__ prev, const unsigned char* __restrict__ fixy, double* b, double* XbJ) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < nY; j += gridDim.x * blockDim.x) {
        double acc = 0;
        for (int e = yt_ptr[j]; e < yt_ptr[j + 1]; e++) acc += yt_val[e] * hb[yt_row[e]];
        b[j] = fixy && fixy[j] ? 0.0 : scale * acc + (prev ? shift * prev[j] : 0.0);
    }
    {   // one warp per constrained variable (long seam lists)
        const int lane = threadIdx.x & 31;
        const int nwarps = (gridDim.x * blockDim.x) >> 5;
        for (int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < nJ; s += nwarps) {
            double acc = 0;
            for (int e = jt_ptr[s] + lane; e < jt_ptr[s + 1]; e += 32) acc += jt_val[e] * hb[jt_row[e]];
            for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
            if (lane == 0) XbJ[s] = acc;
        }
    }
}

// z part of the right-hand side (one block): b_z = scale * USmall^T XbJ + shift * prev_z
__global__ void rhs_reduce_z(int nY, int nZ, int nJ, const double* __restrict__ Us, const double* __restrict__ XbJ,
                             double scale, double shift, const double* __restrict__ prev, double* b) {
    for (int j = threadIdx.x; j < nZ; j += blockDim.x) {
        double acc = 0;
        for (int s = 0; s < nJ; s++) acc += Us[(size_t)s * nZ + j] * XbJ[s];
        b[nY + j] = scale * acc + (prev ? shift * prev[nY + j] : 0.0);
    }
}

// Jacobi diagonal of the free block: 2 scale sum val^2 S_cc + shift.
__global__ void jacobi_y(int nY, const int* __restrict__ yt_ptr, const int* __restrict__ yt_row,
                         const double* __restrict__ yt_val, const double* __restrict__ s_diag, double scale, double shift,
                         double* minv64, float* minv32) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < nY; j += gridDim.x * blockDim.x) {
        double acc = 0;
        for (int e = yt_ptr[j]; e < yt_ptr[j + 1]; e++) acc += yt_val[e] * yt_val[e] * s_diag[yt_row[e] >> 1];
        double d = 2 * scale * acc + shift;
        double m = d > 0 ? 1.0 / d : 1.0;
        minv64[j] = m;
        minv32[j] = (float)m;
    }
}

// X (full variables) from xs: free -> y, constrained -> USmall z.  Full layout for fullx.
__global__ void expand_full(int nFull, const int* __restrict__ full2y, const int* __restrict__ full2j, int nY, int nZ,
                            const double* __restrict__ Us, const double* __restrict__ xs, double* X) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nFull; i += gridDim.x * blockDim.x) {
        int y = full2y[i];
        double v;
        if (y >= 0) {
            v = xs[y];
        } else {
            int s = full2j[i];
            v = 0;
            for (int j = 0; j < nZ; j++) v += Us[(size_t)s * nZ + j] * xs[nY + j];
        }
        X[i] = v;
    }
}

// Value X of full variable i from the reduced coordinates: a free variable is its y entry, a
// constrained one the USmall row times z (same order of additions as the host).
__device__ __forceinline__ double left_value(int i, const int* __restrict__ full2y, const int* __restrict__ full2j,
                                             int nY, int nZ, const double* __restrict__ Us, const double* __restrict__ xs) {
    int y = full2y[i];
    if (y >= 0) return xs[y];
    int s = full2j[i];
    double X = 0;
    for (int j = 0; j < nZ; j++) X += Us[(size_t)s * nZ + j] * xs[nY + j];
    return X;
}

// X(full) of the fixed variables (the post-rounding check): a free variable's value, or a
// translation's USmall row times the z block (summed in the host's order).
__global__ void fixed_values(int nfix, const int* __restrict__ fixed, const int* __restrict__ full2y,
                             const int* __restrict__ full2j, int nY, int nZ, const double* __restrict__ Us,
                             const double* __restrict__ xs, double* out) {
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nfix; q += gridDim.x * blockDim.x) {
        const int full = fixed[q], y = full2y[full];
        if (y >= 0) { out[q] = xs[y]; continue; }
        const int sl = full2j[full];
        double t = 0.0;
        for (int j = 0; j < nZ; j++) t = __dadd_rn(t, __dmul_rn(Us[(size_t)sl * nZ + j], xs[nY + j]));
        out[q] = t;
    }
}

// Greedy pick of SeamlessIntegration::initFixedIndices (iter_rounding_loop.h:34-38) over the left
// indices, one CTA.  The reference keeps the first position with the smallest |X - round X|
// under a strict '<'.  Here distances within its integrality threshold (1e-6, :73: no re-solve
// follows) count as 0, and candidates within kTieWindow of the smallest distance are taken by
// position: they are equal in exact arithmetic (variables tied by a constraint, already-integral
// values), so round-off and the reference's O(1 / penalty) residuals cannot reorder them.
// out: [0] pick position, [1] its distance, [2] its X, [3] smallest distance outside the tie
// group (1e300 when none), [4] the strict '<' pick position (raw distances), [5] its distance.
constexpr double kTieWindow = 1e-8;

__global__ void round_argmin(int nLeft, const int* __restrict__ left, const int* __restrict__ full2y,
                             const int* __restrict__ full2j, int nY, int nZ, const double* __restrict__ Us,
                             const double* __restrict__ xs, double* out) {
    __shared__ double sd[kStream];
    __shared__ int si[kStream];
    // pass 1: smallest raw distance and the first position holding it (the strict '<' pick)
    double bd = 1e300;
    int bk = 0x7fffffff;
    for (int t = threadIdx.x; t < nLeft; t += blockDim.x) {
        double X = left_value(left[t], full2y, full2j, nY, nZ, Us, xs);
        double d = fabs(X - round(X));
        if (d < bd) { bd = d; bk = t; }
    }
    sd[threadIdx.x] = bd;
    si[threadIdx.x] = bk;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            const double od = sd[threadIdx.x + w];
            const int ok = si[threadIdx.x + w];
            if (od < sd[threadIdx.x] || (od == sd[threadIdx.x] && ok < si[threadIdx.x])) {
                sd[threadIdx.x] = od;
                si[threadIdx.x] = ok;
            }
        }
        __syncthreads();
    }
    const double draw_min = sd[0];
    const int kstrict = si[0];
    const double dmin = draw_min <= 10e-7 ? 0.0 : draw_min;
    __syncthreads();
    // pass 2: first position inside the tie group, and the best distance outside it
    int bi = 0x7fffffff;
    double bX = 0, bdist = 0, other = 1e300;
    for (int t = threadIdx.x; t < nLeft; t += blockDim.x) {
        double X = left_value(left[t], full2y, full2j, nY, nZ, Us, xs);
        double d = fabs(X - round(X));
        if (d <= 10e-7) d = 0.0;
        if (d <= dmin + kTieWindow) {
            if (t < bi) { bi = t; bX = X; bdist = d; }
        } else {
            other = fmin(other, d);
        }
    }
    __shared__ double sX[kStream], sdd[kStream], so[kStream];
    si[threadIdx.x] = bi; sX[threadIdx.x] = bX; sdd[threadIdx.x] = bdist; so[threadIdx.x] = other;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            if (si[threadIdx.x + w] < si[threadIdx.x]) {
                si[threadIdx.x] = si[threadIdx.x + w]; sX[threadIdx.x] = sX[threadIdx.x + w]; sdd[threadIdx.x] = sdd[threadIdx.x + w];
            }
            so[threadIdx.x] = fmin(so[threadIdx.x], so[threadIdx.x + w]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = (double)si[0]; out[1] = sdd[0]; out[2] = sX[0]; out[3] = so[0];
        out[4] = (double)kstrict; out[5] = draw_min;
    }
}

// NI-LM field block (Gauss-Newton with the diagonal field block eliminated exactly):
// f* = (wI^2 length grad(x) + wC^2 F2) / (wI^2 + wC^2), grad over the N functions.
__global__ void lm_field_target(int nF, const int* __restrict__ cutF, const double* __restrict__ grad,
                                const double* __restrict__ U /* 2*nCut */, const double* __restrict__ F2, double length,
                                double wI2, double wC2, double* Fout) {
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < nF; f += gridDim.x * blockDim.x) {
        double g[2][2] = {{0, 0}, {0, 0}};
        for (int a = 0; a < 3; a++) {
            int c = cutF[3 * f + a];
            double gx = grad[6 * f + 2 * a], gy = grad[6 * f + 2 * a + 1];
            for (int k = 0; k < 2; k++) { g[k][0] += gx * U[2 * c + k]; g[k][1] += gy * U[2 * c + k]; }
        }
        for (int k = 0; k < 4; k++) {
            double sgn = k < 2 ? 1.0 : -1.0;
            for (int comp = 0; comp < 2; comp++) {
                double gg = sgn * g[k & 1][comp];
                Fout[8 * f + 2 * k + comp] = (wI2 * length * gg + wC2 * F2[8 * f + 2 * k + comp]) / (wI2 + wC2);
            }
        }
    }
}

// U = W X for FP64 xs (used by lm_field_target).
__global__ void gather_U(int nCut, const int* __restrict__ w_ptr, const int* __restrict__ w_tag,
                         const double* __restrict__ w_val, const double* __restrict__ xs, const double* __restrict__ XJ,
                         double* U) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < 2 * nCut; r += gridDim.x * blockDim.x) {
        double acc = 0;
        for (int e = w_ptr[r]; e < w_ptr[r + 1]; e++) {
            int tag = w_tag[e];
            acc += w_val[e] * (tag >= 0 ? xs[tag] : XJ[-1 - tag]);
        }
        U[r] = acc;
    }
}

__global__ void xj_from_z(int nJ, int nY, int nZ, const double* __restrict__ Us, const double* __restrict__ xs, double* XJ) {
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nJ; s += gridDim.x * blockDim.x) {
        double v = 0;
        for (int j = 0; j < nZ; j++) v += Us[(size_t)s * nZ + j] * xs[nY + j];
        XJ[s] = v;
    }
}

__global__ void to_f32(int n, const double* __restrict__ a, float* b) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) b[i] = (float)a[i];
}
__global__ void add_f32(int n, const float* __restrict__ e, double* x) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) x[i] += (double)e[i];
}

// x_z += P_z e_z with the FP64 projector (one block).  The FP32 solve's own projector leaves
// O(1e-7) components along the constraint rows; the FP64 residual cannot see components in
// the null space of K, so they are removed here before the correction is accumulated.
// scratch: 2 nZ doubles of global memory when they do not fit in shared memory, else null
__global__ void add_z_projected(int nY, int nZ, int kq, const double* __restrict__ Q, const float* __restrict__ e,
                                double* x, double* scratch) {
    extern __shared__ double sz[];
    double* ez = scratch ? scratch : sz;
    double* t = ez + nZ;
    for (int j = threadIdx.x; j < nZ; j += blockDim.x) ez[j] = (double)e[nY + j];
    __syncthreads();
    for (int a = threadIdx.x; a < kq; a += blockDim.x) {
        double v = 0;
        for (int j = 0; j < nZ; j++) v += Q[(size_t)a * nZ + j] * ez[j];
        t[a] = v;
    }
    __syncthreads();
    for (int j = threadIdx.x; j < nZ; j += blockDim.x) {
        double v = ez[j];
        for (int a = 0; a < kq; a++) v -= Q[(size_t)a * nZ + j] * t[a];
        x[nY + j] += v;
    }
}

// Size-field loss, per face (functions k = 0..3 with k >= 2 the negatives of k - 2): the
// gradient g of the parameterization U, r = length g - es_f T_f (8 values), rT_f = r . T_f, and
// the partial sum of |r|^2.
// Partial derivatives of the size-field loss with the integration target (T = F2) at fixed x,
// for the vertex-position gradient (x minimises the loss's first term, so dl/dV is the partial
// at fixed x): per face, with r_fk = length grad(u_k)_f - e_f F2_fk and NF[c, k] the function
// values at the cut corners (sign symmetry: NF[c, k + 2] = -NF[c, k]),
//   dgx[3 f + a] = 2 length sum_k r_fk,x NF[c_a, k],   dgy likewise with the y components,
//   dphi[f] = sum_k (-2 e_f r_fk) . (-F2_fk,y, F2_fk,x)   (F2_fk = (cos, sin) of the field angle),
// and the block partials of dl/dlength = sum_f sum_k 2 r_fk . grad(u_k)_f.
__global__ void face_position_partials(int nF, const int* __restrict__ cutF, const double* __restrict__ grad,
                                       const double* __restrict__ U, double length, const double* __restrict__ es,
                                       const double* __restrict__ F2, double* dgx, double* dgy, double* dphi,
                                       double* partials) {
    double red[1] = {0};
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < nF; f += gridDim.x * blockDim.x) {
        double g[2][2] = {{0, 0}, {0, 0}};
        for (int a = 0; a < 3; a++) {
            const int c = cutF[3 * f + a];
            const double gx = grad[6 * f + 2 * a], gy = grad[6 * f + 2 * a + 1];
            for (int k = 0; k < 2; k++) { g[k][0] += gx * U[2 * c + k]; g[k][1] += gy * U[2 * c + k]; }
        }
        double r[4][2];
        double dl = 0, dp = 0;
        for (int k = 0; k < 4; k++) {
            const double sgn = k < 2 ? 1.0 : -1.0;
            for (int comp = 0; comp < 2; comp++) {
                const double gu = sgn * g[k & 1][comp];
                r[k][comp] = length * gu - es[f] * F2[8 * f + 2 * k + comp];
                dl += 2.0 * r[k][comp] * gu;
            }
            const double tx = F2[8 * f + 2 * k], ty = F2[8 * f + 2 * k + 1];
            dp += -2.0 * es[f] * (r[k][0] * -ty + r[k][1] * tx);
        }
        for (int a = 0; a < 3; a++) {
            const int c = cutF[3 * f + a];
            double sx = 0, sy = 0;
            for (int k = 0; k < 4; k++) {
                const double nf = (k < 2 ? 1.0 : -1.0) * U[2 * c + (k & 1)];
                sx += r[k][0] * nf;
                sy += r[k][1] * nf;
            }
            dgx[3 * f + a] = 2.0 * length * sx;
            dgy[3 * f + a] = 2.0 * length * sy;
        }
        dphi[f] = dp;
        red[0] += dl;
    }
    publish_partials<double, 1>(red, partials);
}

__global__ void face_residual(int nF, const int* __restrict__ cutF, const double* __restrict__ grad,
                              const double* __restrict__ U, double length, const double* __restrict__ es,
                              const double* __restrict__ T, double* r, double* rT, double* partials) {
    double red[1] = {0};
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < nF; f += gridDim.x * blockDim.x) {
        double g[2][2] = {{0, 0}, {0, 0}};
        for (int a = 0; a < 3; a++) {
            const int c = cutF[3 * f + a];
            const double gx = grad[6 * f + 2 * a], gy = grad[6 * f + 2 * a + 1];
            for (int k = 0; k < 2; k++) { g[k][0] += gx * U[2 * c + k]; g[k][1] += gy * U[2 * c + k]; }
        }
        double dot = 0, sq = 0;
        for (int k = 0; k < 4; k++) {
            const double sgn = k < 2 ? 1.0 : -1.0;
            for (int comp = 0; comp < 2; comp++) {
                const double t = T[8 * f + 2 * k + comp];
                const double v = length * sgn * g[k & 1][comp] - es[f] * t;
                r[8 * f + 2 * k + comp] = v;
                dot += v * t;
                sq += v * v;
            }
        }
        rT[f] = dot;
        red[0] += sq;
    }
    publish_partials<double, 1>(red, partials);
}

// Phi rounded to FP16 (the kernels' copy, row-major with rows padded to kp entries, the padding
// zeroed beforehand); the FP32 copy (column-major) keeps the rounded values, so the Galerkin
// block built from it belongs to the basis the kernels apply.
__global__ void phi_round_half(int nY, int nZ, int kp, float* phi, __half* phih) {
    const size_t n = (size_t)nY * nZ;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const size_t j = i % nY, k = i / nY;
        const __half h = __float2half_rn(phi[i]);
        phih[j * kp + k] = h;
        phi[i] = __half2float(h);
    }
}

// Block partials of Phi^T v (FP64 sums): partials[k * gridDim.x + blockIdx.x], k < nZ.
__global__ void phi_tdot(int nY, int nZ, const float* __restrict__ Phi, const float* __restrict__ v, double* partials) {
    for (int k = 0; k < nZ; k++) {
        double a[1] = {0};
        const float* col = Phi + (size_t)k * nY;
        for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < nY; j += gridDim.x * blockDim.x)
            a[0] += (double)col[j] * (double)v[j];
        block_sum<double, 1>(a);
        if (threadIdx.x == 0) partials[k * gridDim.x + blockIdx.x] = a[0];
    }
}

// out[k] = fixed-order sum of partials[k * nb + 0 .. nb), k < K (one block).
__global__ void finalize_k(const double* partials, int nb, int K, double* out) {
    for (int k = 0; k < K; k++) {
        double v[1] = {0};
        for (int i = threadIdx.x; i < nb; i += blockDim.x) v[0] += partials[k * nb + i];
        block_sum<double, 1>(v);
        if (threadIdx.x == 0) out[k] = v[0];
    }
}

// Fixed-order sum of one partial per block (written by publish_partials over nb blocks).
__global__ void finalize1(const double* partials, int nb, double* out) {
    double v[1] = {0};
    for (int i = threadIdx.x; i < nb; i += blockDim.x) v[0] += partials[i];
    block_sum<double, 1>(v);
    if (threadIdx.x == 0) out[0] = v[0];
}

// q_f = (X2F lambda)_f . F2_f: the gradient of the parameterization U(lambda) against the target.
__global__ void face_target_dot(int nF, const int* __restrict__ cutF, const double* __restrict__ grad,
                                const double* __restrict__ U, const double* __restrict__ F2, double* q) {
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < nF; f += gridDim.x * blockDim.x) {
        double g[2][2] = {{0, 0}, {0, 0}};
        for (int a = 0; a < 3; a++) {
            const int c = cutF[3 * f + a];
            const double gx = grad[6 * f + 2 * a], gy = grad[6 * f + 2 * a + 1];
            for (int k = 0; k < 2; k++) { g[k][0] += gx * U[2 * c + k]; g[k][1] += gy * U[2 * c + k]; }
        }
        double dot = 0;
        for (int k = 0; k < 4; k++) {
            const double sgn = k < 2 ? 1.0 : -1.0;
            for (int comp = 0; comp < 2; comp++) dot += sgn * g[k & 1][comp] * F2[8 * f + 2 * k + comp];
        }
        q[f] = dot;
    }
}

}  // namespace mtk

using namespace mtk;

namespace {

// Differentiation of the naive integration with a per-vertex log-size field s: the target of
// face f is exp(mean of s over its corners) * F2_f, and the loss
//   l(s) = sum_f |length X2F_f x(s) - exp(sbar_f) T_f|^2 + mu sum_edges (s_i - s_j)^2
// is differentiated by one adjoint solve K lambda = dl/dx (the forward system, symmetric) and
// the assembly backward of the right-hand side.
struct SizeFieldJob {
    int nV;
    const int32_t* F;   // raw faces (nF x 3)
    const double* s;    // log-size per raw vertex
    const double* T;    // loss target per face (8 values), null: the integration target F2
    double mu;
    double* loss;
    double* grad_s;     // nV
    // position partials (face_position_partials; T must be null), all null when not wanted
    double* dgx = nullptr;      // 3 nF
    double* dgy = nullptr;      // 3 nF
    double* dphi = nullptr;     // nF
    double* dlength = nullptr;  // 1
};

struct Igm {
    mtk_ctx* c = nullptr;
    cudaStream_t st = nullptr;
    int nF = 0, nCut = 0, nY = 0, nZ = 0, nJ = 0, nFull = 0, nRed = 0;
    double length = 0;
    // host copies needed by the loop
    std::vector<int> full2y, full2j;
    std::vector<double> USmall;      // nJ x nZ
    // device topology / operators
    DBuf<int> cutF, vf_ptr, vf_face, s_ptr, s_col, w_ptr, w_tag, yt_ptr, yt_row, jt_ptr, jt_row, d_full2y, d_full2j, left;
    DBuf<double> cutV, grad, s_val, s_diag, w_val, yt_val, jt_val, Us, F2, Fsi, hb, XbJ, U, Qc, XoJ, minvy, Mz, Qz;
    DBuf<float> s_val32, w_val32, yt_val32, jt_val32, Us32, minvy32, Mz32, Qz32, U32, Qc32, XoJ32;
    DBuf<double> xs, bsys, r64, z64, p64, q64, prev, Xfull, XJ64, scratch;
    DBuf<float> r32, e32, z32, p32, q32, pb32;
    // assembled operator of the FP32 inner solves
    bool asm_ok = false;
    DBuf<int> ka_ptr, ka_col, cy_ptr, cy_col, cj_ptr, cj_col;
    // Schur coarse space of the z block (phi_coarse): Phi column-major nY x nZ, G0 = Z^T K0 Z and
    // C0 = Z^T Z for Z = [Phi ; I] and the unscaled operator K0
    bool phi_ok = false;
    DBuf<float> phi, qid32;   // Phi (FP32, its values FP16-representable) while it is built
    DBuf<__half> phih;         // Phi as the kernels read it
    std::vector<double> G0, C0;
    DBuf<float> ka_val32, cy_val32, cj_val32, bjj32;
    // translation-row chunks of the matrix-free (jt) and the assembled (cj) operator
    DBuf<int> jtc_row, jtc_beg, jtc_first, cjc_row, cjc_beg, cjc_first;
    int jtc_n = 0, cjc_n = 0;
    DBuf<double> XoJp;
    DBuf<float> XoJp32;
    DBuf<double> pb64;   // second direction buffers of the PCG (double-buffered p)
    // attainable reduction of the FP32 solves per refinement (first, second, later), measured as
    // sqrt(max(0, rr_fp64 - rr_fp32)) / |r_start|: the next solves stop at half of it
    double floor_rel[3] = {0.0, 0.0, 0.0};
    DBuf<unsigned char> fixy;
    std::vector<unsigned char> h_fixy;
    int kq = 0;
    size_t smem64 = 0, smem32 = 0;
    // z state of the PCG kernel in global memory when it needs more than kZSmemMax bytes
    static constexpr size_t kZSmemMax = 200 * 1024;
    int nZ_ = 0, nJ_ = 0;
    bool z_global_forced = false;
    DBuf<unsigned char> zstate_global;
    DBuf<double> zproj_scratch;
    double pcg_ms = 0, pcg_bytes = 0;
    long long pcg_launches = 0, pcg_passes = 0;
    long long nnzW = 0, nnzS = 0, nnzYT = 0;
    // multigrid on the free block (host-built)
    struct RCsrBufs {
        DBuf<int> ptr, col;
        DBuf<double> v64;
        DBuf<float> v32;
        int n = 0, group = 1;
        size_t nnz = 0;
        SellIdx sell;                 // SELL-32 copy (mtk_sell.cuh) where sell_worth holds
        DBuf<double> s64;
        DBuf<float> s32;
    };
    struct RLevelBufs { RCsrBufs R, S, P; DBuf<double> r64, y64; DBuf<float> r32, y32; } rlv[kRMaxLevels];
    DBuf<double> rAinv64, rrc64, ryc64;
    DBuf<float> rAinv32, rrc32, ryc32;
    DBuf<unsigned char> rh_dev64, rh_dev32;
    RDevHierarchy<double> RH64{};
    RDevHierarchy<float> RH32{};
    bool mg = false;
    int mg_levels = 0;
    double mg_bytes64 = 0, mg_bytes32 = 0;   // algorithmic bytes of one V-cycle
    double cur_scale = 1.0;
    template <typename T> RDevHierarchy<T> rhier() const;

    int upload_rcsr(const RCsr& M, RCsrBufs& B, int group) {
        B.n = M.n;
        B.group = group;
        B.nnz = M.col.size();
        MTK_TRY(B.ptr.upload(M.ptr.data(), M.ptr.size(), st));
        MTK_TRY(B.col.upload(M.col.data(), M.col.size(), st));
        MTK_TRY(B.v64.upload(M.val.data(), M.val.size(), st));
        std::vector<float> v32(M.val.begin(), M.val.end());
        MTK_TRY(B.v32.upload(v32.data(), v32.size(), st));
        return MTK_OK;
    }

    int build_mg(RCsr K, std::vector<int> node, std::vector<int> comp, int nnode, DevCsr64* dK = nullptr) {
        // the Galerkin products run on the device (RDevBuilder, the same arrays as the host
        // build); the host builds when the device build declines (a row beyond its capacity)
        const auto tb0 = std::chrono::steady_clock::now();
        std::vector<DevCycleOps> dops;
        std::vector<double> Ainv;
        int nc = 0;
        bool dev_ok = false;
        if (!getenv("MTK_MG_HOST")) {
            RDevBuilder B(c, st);
            MTK_TRY(B.build(K, node, comp, nnode, dops, nc, Ainv, dev_ok, dK));
        }
        RHierarchy HH;
        if (!dev_ok) {
            dops.clear();
            if (!build_real_hierarchy(std::move(K), std::move(node), std::move(comp), nnode, HH)) return MTK_OK;
            nc = HH.nc;
            Ainv = HH.Ainv;
        }
        if (debug())
            fprintf(stderr, "[igm host]   (hierarchy build %.1f ms, %s)\n",
                    std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - tb0).count(),
                    dev_ok ? "device Galerkin products" : "host");
        const int nl = dev_ok ? (int)dops.size() : (int)HH.lv.size();
        if (nl == 0) return MTK_OK;
        // lanes per row of a CSR phase: fewest rounds x dependent loads (ptr, then batches of four
        // entries per lane, each a column load and a gather) over the persistent grid
        const double threads = (double)c->num_sms * kBlock;
        auto grp = [&](int n, size_t nnz) {
            const double avg = n > 0 ? (double)nnz / n : 0.0;
            int best = 1;
            double bc = 1e300;
            for (int g = 1; g <= 32; g <<= 1) {
                const double cost = std::ceil(n * (double)g / threads) * (1.0 + 2.0 * std::ceil(avg / (4.0 * g)));
                if (cost < bc - 1e-9) { bc = cost; best = g; }
            }
            return best;
        };
        // a matrix for which the cost model picks several lanes per row, with enough rows to fill
        // the grid with one lane per row and short rows, gets a SELL-32 copy and one lane per row
        const bool use_sell = !getenv("MTK_NO_SELL");
        auto sell_rows = [&](int n, double avg) { return use_sell && sell_worth(n, avg); };
        auto avg_of = [](int n, size_t nnz) { return n > 0 ? (double)nnz / n : 0.0; };
        // adopt a device CSR (FP64 values) and its FP32 copy
        auto adopt = [&](DevCsr64& D, RCsrBufs& B, int group) -> int {
            B.n = D.n;
            B.group = group;
            B.nnz = D.nnz;
            B.ptr = std::move(D.ptr);
            B.col = std::move(D.col);
            B.v64 = std::move(D.val);
            MTK_TRY(B.v32.alloc(std::max<size_t>(D.nnz, 1)));
            if (D.nnz)
                rgpu::to_f32_vals<<<stream_grid(c), kStream, 0, st>>>(D.nnz, B.v64.p, B.v32.p);
            MTK_CUDA_TRY(cudaGetLastError());
            return MTK_OK;
        };
        std::vector<double> lvl_nnz(3 * nl), lvl_n(2 * nl);   // R, S, P entries; S rows, R rows
        std::vector<char> up_sell(nl, 0), r_sell(nl, 0);       // phases given SELL-32 copies
        for (int l = 0; l < nl; l++) {
            RLevelBufs& B = rlv[l];
            int nS, nR;
            size_t zR, zS, zP;
            if (dev_ok) {
                DevCycleOps& O = dops[l];
                nS = O.S.n; nR = O.R.n; zR = O.R.nnz; zS = O.S.nnz; zP = O.P.nnz;
                // level 0's up phase writes z with the thread-per-row mapping of the PCG vector
                // loops, which read it with no grid barrier in between: keep it at one lane per row
                // level 0's up phase stays CSR, one lane per row (short rows; see sell_worth)
                up_sell[l] = l > 0 && sell_rows(nS, std::max(avg_of(nS, zS), avg_of(O.P.n, zP)));
                r_sell[l] = sell_rows(nR, avg_of(nR, zR));
                const int up = l == 0 || up_sell[l] ? 1 : std::max(grp(nS, zS), grp(O.P.n, zP));
                MTK_TRY(adopt(O.R, B.R, r_sell[l] ? 1 : grp(nR, zR)));
                if (debug())
                    fprintf(stderr, "[igm host]   level %d: %d rows (S %.1f, P %.1f per row), R %d rows (%.1f per row)%s%s\n",
                            l, nS, avg_of(nS, zS), avg_of(O.P.n, zP), nR, avg_of(nR, zR), up_sell[l] ? ", up SELL" : "",
                            r_sell[l] ? ", R SELL" : "");
                MTK_TRY(adopt(O.S, B.S, up));
                MTK_TRY(adopt(O.P, B.P, up));
            } else {
                const RCycleOps& O = HH.ops[l];
                nS = O.S.n; nR = O.R.n; zR = O.R.col.size(); zS = O.S.col.size(); zP = O.P.col.size();
                up_sell[l] = l > 0 && sell_rows(nS, std::max(avg_of(nS, zS), avg_of(O.P.n, zP)));
                r_sell[l] = sell_rows(nR, avg_of(nR, zR));
                const int up = l == 0 || up_sell[l] ? 1 : std::max(grp(nS, zS), grp(O.P.n, zP));
                MTK_TRY(upload_rcsr(O.R, B.R, r_sell[l] ? 1 : grp(nR, zR)));
                MTK_TRY(upload_rcsr(O.S, B.S, up));
                MTK_TRY(upload_rcsr(O.P, B.P, up));
            }
            lvl_nnz[3 * l] = (double)zR; lvl_nnz[3 * l + 1] = (double)zS; lvl_nnz[3 * l + 2] = (double)zP;
            lvl_n[2 * l] = nS; lvl_n[2 * l + 1] = nR;
            if (l > 0) {
                MTK_TRY(B.r64.alloc(nS)); MTK_TRY(B.y64.alloc(nS));
                MTK_TRY(B.r32.alloc(nS)); MTK_TRY(B.y32.alloc(nS));
            }
            for (RCsrBufs* C : {&B.R, &B.S, &B.P})
                if (C->n > 0 && (C == &B.R ? r_sell[l] : up_sell[l])) {
                    MTK_TRY(sell_build_index(c, st, C->n, C->ptr.p, C->col.p, C->sell));
                    MTK_TRY(sell_fill_values<double>(c, st, C->n, C->ptr.p, C->col.p, C->v64.p, C->sell, C->s64));
                    MTK_TRY(sell_fill_values<float>(c, st, C->n, C->ptr.p, C->col.p, C->v32.p, C->sell, C->s32));
                }
            auto m64 = [](const RCsrBufs& C) {
                RDevCsr<double> M{C.n, C.group, C.ptr.p, C.col.p, C.v64.p};
                if (C.sell.sptr.p) { M.sptr = C.sell.sptr.p; M.scol = C.sell.scol.p; M.sval = C.s64.p; }
                return M;
            };
            auto m32 = [](const RCsrBufs& C) {
                RDevCsr<float> M{C.n, C.group, C.ptr.p, C.col.p, C.v32.p};
                if (C.sell.sptr.p) { M.sptr = C.sell.sptr.p; M.scol = C.sell.scol.p; M.sval = C.s32.p; }
                return M;
            };
            RH64.L[l] = RDevLevel<double>{m64(B.R), m64(B.S), m64(B.P), B.r64.p, B.y64.p};
            RH32.L[l] = RDevLevel<float>{m32(B.R), m32(B.S), m32(B.P), B.r32.p, B.y32.p};
        }
        MTK_TRY(rAinv64.upload(Ainv.data(), Ainv.size(), st));
        std::vector<float> a32(Ainv.begin(), Ainv.end());
        MTK_TRY(rAinv32.upload(a32.data(), a32.size(), st));
        MTK_TRY(rrc64.alloc(nc)); MTK_TRY(ryc64.alloc(nc));
        MTK_TRY(rrc32.alloc(nc)); MTK_TRY(ryc32.alloc(nc));
        RH64.nlev = nl; RH64.nc = nc; RH64.Ainv = rAinv64.p; RH64.rc = rrc64.p; RH64.yc = ryc64.p;
        RH32.nlev = nl; RH32.nc = nc; RH32.Ainv = rAinv32.p; RH32.rc = rrc32.p; RH32.yc = ryc32.p;
        {
            auto cyc = [&](double T) {
                double b = 0;
                for (int l = 0; l < nl; l++) {
                    const double nnz = lvl_nnz[3 * l] + lvl_nnz[3 * l + 1] + lvl_nnz[3 * l + 2];
                    const double nS = lvl_n[2 * l], nR = lvl_n[2 * l + 1];
                    b += nnz * (T + 4) + 4.0 * (nR + 2.0 * nS) + T * (3.0 * nS + 2.0 * nR);
                }
                return b + (double)nc * nc * T + 2.0 * nc * T;
            };
            mg_bytes64 = cyc(8);
            mg_bytes32 = cyc(4);
        }
        MTK_TRY(rh_dev64.alloc(sizeof(RDevHierarchy<double>)));
        MTK_TRY(rh_dev32.alloc(sizeof(RDevHierarchy<float>)));
        mg = true;
        mg_levels = nl;
        return MTK_OK;
    }

    // Algorithmic bytes of one projected-PCG iteration (operator chain + vector updates):
    //   W gather   nnzW (tag 4 + val T + z, p_old 2T) + 2 nCut (ptr 4 + U write T)
    //   S product  nnzS (col 4 + val T) + nCut ptr 4 + U read 2T + Qc write 2T
    //   W^T gather nnzYT (row 4 + val T + Qc T) + nY (ptr 4 + z, p_old read 2T + p, q write 2T)
    //   updates    nY * 6 T  (x, r, p, q read; x, r write); the preconditioner is counted apart
    double iter_bytes(size_t T) const {
        return (double)nnzW * (4 + 3 * T) + 2.0 * nCut * (4 + T) + (double)nnzS * (4 + T) + nCut * (4.0 + 4 * T) +
               (double)nnzYT * (4 + 2 * T) + (double)nY * (4 + 4 * T) + (double)nY * 6 * T;
    }

    IgmOp<double> op64(double scale, double shift) {
        IgmOp<double> A{nCut, nY, nZ, nJ, w_ptr.p, w_tag.p, w_val.p, s_ptr.p, s_col.p, s_val.p, yt_ptr.p, yt_row.p,
                        yt_val.p, jt_ptr.p, jt_row.p, jt_val.p, Us.p, scale, shift, U.p, Qc.p, XoJ.p,
                        nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
        if (jtc_n > 0) { A.jc_n = jtc_n; A.jc_row = jtc_row.p; A.jc_beg = jtc_beg.p; A.jc_first = jtc_first.p; A.XoJp = XoJp.p; }
        return A;
    }
    IgmOp<float> op32(double scale, double shift) {
        const bool a = asm_ok;
        IgmOp<float> A{nCut, nY, nZ, nJ, w_ptr.p, w_tag.p, w_val32.p, s_ptr.p, s_col.p, s_val32.p, yt_ptr.p, yt_row.p,
                       yt_val32.p, jt_ptr.p, jt_row.p, jt_val32.p, Us32.p, (float)scale, (float)shift, U32.p, Qc32.p,
                       XoJ32.p, a ? ka_ptr.p : nullptr, ka_col.p, ka_val32.p, cy_ptr.p, cy_col.p, cy_val32.p, cj_ptr.p,
                       cj_col.p, cj_val32.p, bjj32.p};
        if (a && cjc_n > 0) {
            A.jc_n = cjc_n; A.jc_row = cjc_row.p; A.jc_beg = cjc_beg.p; A.jc_first = cjc_first.p; A.XoJp = XoJp32.p;
        } else if (!a && jtc_n > 0) {
            A.jc_n = jtc_n; A.jc_row = jtc_row.p; A.jc_beg = jtc_beg.p; A.jc_first = jtc_first.p; A.XoJp = XoJp32.p;
        }
        return A;
    }

    // chunk lists of the translation rows of a CSR row pointer held on the host
    int upload_chunks(const std::vector<int>& ptr, DBuf<int>& row, DBuf<int>& beg, DBuf<int>& first, int& n) {
        std::vector<int> r, b, f;
        translation_chunks(ptr, r, b, f);
        n = (int)r.size();
        if (n == 0) return MTK_OK;
        MTK_TRY(row.upload(r.data(), r.size(), st));
        MTK_TRY(beg.upload(b.data(), b.size(), st));
        MTK_TRY(first.upload(f.data(), f.size(), st));
        const size_t need = std::max<size_t>(n, std::max(jtc_n, cjc_n));
        if (XoJp.n < need) { MTK_TRY(XoJp.alloc(need)); MTK_TRY(XoJp32.alloc(need)); }
        return MTK_OK;
    }

    template <typename T>
    int run_pcg(IgmOp<T> A, ZProj<T> P, const T* minv, const T* b, T* x, T* r, T* z, T* p, T* q, double tol2, int maxit,
                int mode, size_t smem, long long* iters, double* rr_out) {
        const __half* phiP = (phi_ok && mg && mode == 0) ? phih.p : nullptr;
        // the replicated z state in shared memory, or (a constraint kernel too large for it, or
        // MTK_Z_GLOBAL=1) in one global slice per CTA
        const bool zg = smem > kZSmemMax || z_global_forced;
        auto kern = zg ? igm_pcg<T, true> : igm_pcg<T, false>;
        if (zg) smem = 0;
        MTK_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        int per_sm = 0;
        MTK_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kBlock, smem));
        if (per_sm < 1) { mtk_set_last_error("IGM solver does not fit on an SM", __FILE__, __LINE__); return MTK_ERR_CUDA; }
        per_sm = 1;   // one CTA per SM
        int grid = std::min(c->num_sms * per_sm, c->partial_blocks);
        T* zglob = nullptr;
        long long zstride = 0;
        if (zg) {
            zstride = (long long)((zsmem_bytes(sizeof(T), nZ_, nJ_) + sizeof(double) - 1) / sizeof(T));
            zstride = (zstride + 31) & ~31LL;   // 256-byte aligned slices (FP64) / 128-byte (FP32)
            const size_t need = (size_t)grid * (size_t)zstride * sizeof(T);
            if (zstate_global.n < need) MTK_TRY(zstate_global.alloc(need));
            zglob = reinterpret_cast<T*>(zstate_global.p);
        }
        const unsigned char* fx = fixy.p;
        T* partials = reinterpret_cast<T*>(c->partials);
        GridBarrier bar = barrier_of(c);
        int* out = c->dev_int;
        const RDevHierarchy<T>* Hp = nullptr;
        T mg_scale = T(0);
        if (mg && mode == 0) {
            RDevHierarchy<T> H = rhier<T>();
            H.L[0].r = r;    // level 0 = the free block of the PCG residual / preconditioned residual
            H.L[0].y = z;
            unsigned char* dst = sizeof(T) == 8 ? rh_dev64.p : rh_dev32.p;
            MTK_CUDA_TRY(cudaMemcpyAsync(dst, &H, sizeof(H), cudaMemcpyHostToDevice, st));
            Hp = reinterpret_cast<const RDevHierarchy<T>*>(dst);
            mg_scale = T(1.0 / cur_scale);
        }
        T* p2 = sizeof(T) == 8 ? reinterpret_cast<T*>(pb64.p) : reinterpret_cast<T*>(pb32.p);
        void* params[] = {&A, &P, (void*)&fx, (void*)&minv, (void*)&b, (void*)&x, (void*)&r, (void*)&z, (void*)&p,
                          (void*)&p2, (void*)&q, (void*)&partials, &bar, &tol2, &maxit, &mode, (void*)&out,
                          (void*)&Hp, (void*)&mg_scale, (void*)&phiP, (void*)&zglob, (void*)&zstride};
        MTK_TRY(reset_barrier(c));
        MTK_CUDA_TRY(cudaEventRecord(c->ev_k0, st));
        MTK_CUDA_TRY(cudaLaunchCooperativeKernel(reinterpret_cast<void*>(kern), dim3(grid), dim3(kBlock), params, smem, st));
        MTK_CUDA_TRY(cudaEventRecord(c->ev_k1, st));
        c->kernels++;
        MTK_CUDA_TRY(cudaMemcpyAsync(c->h_int, c->dev_int, 8 * sizeof(int), cudaMemcpyDeviceToHost, st));
        MTK_CUDA_TRY(cudaStreamSynchronize(st));
        float kms = 0;
        cudaEventElapsedTime(&kms, c->ev_k0, c->ev_k1);
        pcg_ms += kms;
        pcg_launches++;
        pcg_bytes += (iter_bytes(sizeof(T)) + (Hp ? (sizeof(T) == 8 ? mg_bytes64 : mg_bytes32) : 0.0) +
                      (phiP ? 4.0 * nZ * (double)nY : 0.0)) *
                     (double)(c->h_int[1] + 1);
        pcg_passes += c->h_int[1] + 1;
        if (iters) *iters += c->h_int[1];
        if (rr_out) *rr_out = reinterpret_cast<double*>(c->h_int + 4)[0];
        int s = c->h_int[0];
        if (debug())
            fprintf(stderr, "[igm_pcg T=%zu mode=%d] status=%d iters=%d rr=%.3e tol2=%.3e kq=%d%s\n", sizeof(T), mode, s,
                    c->h_int[1], reinterpret_cast<double*>(c->h_int + 4)[0], tol2, kq,
                    s == 4 ? " (breakdown)" : "");
        if (s == 4 && debug())
            fprintf(stderr, "   pq=%.3e rz=%.3e pq_y=%.3e\n", reinterpret_cast<double*>(c->h_int + 6)[0],
                    reinterpret_cast<double*>(c->h_int + 8)[0], reinterpret_cast<double*>(c->h_int + 10)[0]);
        if (s == 5) return MTK_ERR_TIMEOUT;
        if (s == 4) return MTK_ERR_BREAKDOWN;
        if (s == 3) return MTK_ERR_NOT_CONVERGED;
        return MTK_OK;
    }

    static bool debug() {
        static int d = -1;
        if (d < 0) { const char* e = getenv("MTK_DEBUG"); d = (e && *e == '1') ? 1 : 0; }
        return d == 1;
    }

    int grid() const { return stream_grid(c); }

    // b = scale * UFull^T W^T hb(F) + shift * prev   (prev may be null)
    int build_rhs(const double* Fface, double scale, double shift, const double* prevx, double* b) {
        cut_loads<<<grid(), kStream, 0, st>>>(nCut, vf_ptr.p, vf_face.p, cutF.p, grad.p, Fface, hb.p);
        rhs_reduce<<<grid(), kStream, 0, st>>>(nY, nJ, yt_ptr.p, yt_row.p, yt_val.p, jt_ptr.p, jt_row.p, jt_val.p, hb.p, scale,
                                              shift, prevx, fixy.p, b, XbJ.p);
        rhs_reduce_z<<<1, kStream, 0, st>>>(nY, nZ, nJ, Us.p, XbJ.p, scale, shift, prevx, b);
        c->kernels += 3;
        MTK_CUDA_TRY(cudaGetLastError());
        return MTK_OK;
    }

    // Solve K x = b (projected, x feasible on entry) to ||P(b - K x)|| <= tol ||P b||.
    int solve(double scale, double shift, const double* b, double* x, const mtk_solve_opts& o, mtk_stats* stats,
              double* rel_out) {
        cur_scale = scale;
        long long iters = 0, refines = 0;
        double rr = 0, bb = 0;
        // ||P b||^2: residual mode with x = 0 gives P(b)
        MTK_CUDA_TRY(cudaMemsetAsync(scratch.p, 0, sizeof(double) * nRed, st));
        MTK_TRY(run_pcg<double>(op64(scale, shift), ZProj<double>{kq, Qz.p, Mz.p}, minvy.p, b, scratch.p, r64.p, z64.p,
                                p64.p, q64.p, 0.0, 0, 1, smem64, nullptr, &bb));
        const double goal2 = o.tol * o.tol * bb;
        if (o.precision == MTK_PREC_FP64) {
            int s = run_pcg<double>(op64(scale, shift), ZProj<double>{kq, Qz.p, Mz.p}, minvy.p, b, x, r64.p, z64.p, p64.p,
                                    q64.p, goal2, o.max_iter, 0, smem64, &iters, &rr);
            if (s != MTK_OK) return s;
            MTK_TRY(run_pcg<double>(op64(scale, shift), ZProj<double>{kq, Qz.p, Mz.p}, minvy.p, b, x, r64.p, z64.p, p64.p,
                                    q64.p, 0.0, 0, 1, smem64, nullptr, &rr));
            refines++;
        } else {
            MTK_TRY(run_pcg<double>(op64(scale, shift), ZProj<double>{kq, Qz.p, Mz.p}, minvy.p, b, x, r64.p, z64.p, p64.p,
                                    q64.p, 0.0, 0, 1, smem64, nullptr, &rr));
            refines++;
            int outer = 0;
            while (rr > goal2) {
                if (outer >= o.max_refine) return MTK_ERR_NOT_CONVERGED;
                outer++;
                double itol = o.inner_tol;
                double need = std::sqrt(goal2 / rr) * 0.5;
                if (need > itol) itol = need;
                to_f32<<<grid(), kStream, 0, st>>>(nRed, r64.p, r32.p);
                MTK_CUDA_TRY(cudaMemsetAsync(e32.p, 0, sizeof(float) * nRed, st));
                c->kernels++;
                const int ki = std::min(outer, 3) - 1;
                const double fl = std::min(0.5 * floor_rel[ki], 0.1);
                if (fl > itol) itol = fl;
                double frr = 0.0;
                int s = run_pcg<float>(op32(scale, shift), ZProj<float>{kq, Qz32.p, Mz32.p}, minvy32.p, r32.p, e32.p,
                                       z32.p /*r*/, p32.p /*z*/, q32.p /*p*/, reinterpret_cast<float*>(Xfull.p) /*q*/,
                                       itol * itol * rr, o.max_iter, 0, smem32, &iters, &frr);
                // an FP32 breakdown (p^H A p <= 0 in single precision) means the inner solve has
                // stagnated: its last iterate is still a valid correction, and the FP64 refinement
                // decides what comes next (bounded by max_refine, stopped when it makes no progress)
                if (s == MTK_ERR_TIMEOUT) return s;
                const double rr_prev = rr;
                add_f32<<<grid(), kStream, 0, st>>>(nY, e32.p, x);
                if (nZ > 0) {
                    const size_t zb = sizeof(double) * 2 * (size_t)nZ;
                    const bool zgl = zb > 48 * 1024;   // default dynamic shared-memory limit
                    if (zgl && zproj_scratch.n < 2 * (size_t)nZ) MTK_TRY(zproj_scratch.alloc(2 * (size_t)nZ));
                    add_z_projected<<<1, kStream, zgl ? 0 : zb, st>>>(nY, nZ, kq, Qz.p, e32.p, x,
                                                                     zgl ? zproj_scratch.p : nullptr);
                }
                c->kernels += 2;
                MTK_TRY(run_pcg<double>(op64(scale, shift), ZProj<double>{kq, Qz.p, Mz.p}, minvy.p, b, x, r64.p, z64.p,
                                        p64.p, q64.p, 0.0, 0, 1, smem64, nullptr, &rr));
                refines++;
                if (!(rr == rr)) return MTK_ERR_BREAKDOWN;
                if (rr > goal2 && rr >= rr_prev) return MTK_ERR_NOT_CONVERGED;
                if (s == MTK_OK && rr_prev > 0) floor_rel[ki] = std::sqrt(std::max(rr - frr, 0.0) / rr_prev);
            }
        }
        double rel = bb > 0 ? std::sqrt(rr / bb) : 0.0;
        if (rel_out) *rel_out = rel;
        if (stats) {
            stats->pcg_iters += iters;
            stats->solves += 1;
            stats->refinements += refines;
            stats->spmv_calls += iters + refines + 1;
            if (rel > stats->max_rel_residual) stats->max_rel_residual = rel;
        }
        return MTK_OK;
    }

    // Schur coarse space (phi_coarse).  Column k of Phi: FP32 PCG on the free block with the z
    // block frozen at e_k (projector Q = I, right-hand side 0, so the free block solves
    // K_yy phi = -K_yz e_k), to 1e-2 of its start residual (a coarse-space basis needs no more:
    // the Galerkin G below keeps the preconditioner exact on its span).  Then per column one
    // operator application w = -K0 [phi_k ; e_k] (residual mode, no projection) and
    // G0_lk = -(phi_l . w_y + w_z,l), C0_lk = phi_l . phi_k + delta_lk.  Leaves phi_ok false
    // (block Jacobi) when the multigrid is off, the z block is empty or larger than kMaxPhi,
    // or a column solve breaks down.
    int build_phi(long long* iters) {
        phi_ok = false;
        if (!mg || nZ <= 0 || nZ > kMaxPhi) return MTK_OK;
        MTK_TRY(phi.alloc((size_t)nY * nZ));
        MTK_CUDA_TRY(cudaMemsetAsync(phi.p, 0, sizeof(float) * (size_t)nY * nZ, st));
        std::vector<float> eye((size_t)nZ * nZ, 0.f);
        for (int k = 0; k < nZ; k++) eye[(size_t)k * nZ + k] = 1.f;
        MTK_TRY(qid32.upload(eye.data(), eye.size(), st));
        const double save_scale = cur_scale;
        cur_scale = 1.0;
        const ZProj<float> frozen{nZ, qid32.p, Mz32.p};
        const ZProj<float> open{0, qid32.p, Mz32.p};
        float* xk = e32.p;
        float* zero = r32.p;
        float* qf = reinterpret_cast<float*>(Xfull.p);
        MTK_CUDA_TRY(cudaMemsetAsync(zero, 0, sizeof(float) * nRed, st));
        for (int k = 0; k < nZ; k++) {
            MTK_CUDA_TRY(cudaMemsetAsync(xk, 0, sizeof(float) * nRed, st));
            c->h_scalars[0] = 0.0;
            reinterpret_cast<float*>(c->h_scalars)[0] = 1.f;
            MTK_CUDA_TRY(cudaMemcpyAsync(xk + nY + k, c->h_scalars, sizeof(float), cudaMemcpyHostToDevice, st));
            double rr0 = 0;
            MTK_TRY(run_pcg<float>(op32(1.0, 0.0), frozen, minvy32.p, zero, xk, z32.p, p32.p, q32.p, qf, 0.0, 0, 1, smem32,
                                   nullptr, &rr0));
            if (!(rr0 > 0)) continue;   // z_k does not touch the free block: phi_k = 0
            int s = run_pcg<float>(op32(1.0, 0.0), frozen, minvy32.p, zero, xk, z32.p, p32.p, q32.p, qf, 1e-4 * rr0, 200, 0,
                                   smem32, iters, nullptr);
            if (s == MTK_ERR_TIMEOUT) return s;
            if (s != MTK_OK && s != MTK_ERR_NOT_CONVERGED) { cur_scale = save_scale; return MTK_OK; }
            MTK_CUDA_TRY(cudaMemcpyAsync(phi.p + (size_t)k * nY, xk, sizeof(float) * nY, cudaMemcpyDeviceToDevice, st));
        }
        const int kp = (nZ + 7) & ~7;
        MTK_TRY(phih.alloc((size_t)nY * kp));
        MTK_CUDA_TRY(cudaMemsetAsync(phih.p, 0, sizeof(__half) * (size_t)nY * kp, st));
        phi_round_half<<<stream_grid(c), kStream, 0, st>>>(nY, nZ, kp, phi.p, phih.p);
        c->kernels++;
        MTK_CUDA_TRY(cudaGetLastError());
        G0.assign((size_t)nZ * nZ, 0.0);
        C0.assign((size_t)nZ * nZ, 0.0);
        const int nb = stream_grid(c);
        std::vector<float> wz(nZ);
        std::vector<double> dw(nZ), dp(nZ);
        for (int k = 0; k < nZ; k++) {
            MTK_CUDA_TRY(cudaMemsetAsync(xk, 0, sizeof(float) * nRed, st));
            MTK_CUDA_TRY(cudaMemcpyAsync(xk, phi.p + (size_t)k * nY, sizeof(float) * nY, cudaMemcpyDeviceToDevice, st));
            reinterpret_cast<float*>(c->h_scalars)[0] = 1.f;
            MTK_CUDA_TRY(cudaMemcpyAsync(xk + nY + k, c->h_scalars, sizeof(float), cudaMemcpyHostToDevice, st));
            MTK_TRY(run_pcg<float>(op32(1.0, 0.0), open, minvy32.p, zero, xk, z32.p, p32.p, q32.p, qf, 0.0, 0, 1, smem32,
                                   nullptr, nullptr));
            // w = z32 (= -K0 Z_k): G0 column k; Phi^T phi_k: C0 column k
            // (nb * nZ partials and nZ scalars fit the context buffers for nZ <= kMaxPhi)
            phi_tdot<<<nb, kStream, 0, st>>>(nY, nZ, phi.p, z32.p, c->partials);
            finalize_k<<<1, kStream, 0, st>>>(c->partials, nb, nZ, c->scalars);
            MTK_CUDA_TRY(cudaMemcpyAsync(dw.data(), c->scalars, sizeof(double) * nZ, cudaMemcpyDeviceToHost, st));
            phi_tdot<<<nb, kStream, 0, st>>>(nY, nZ, phi.p, phi.p + (size_t)k * nY, c->partials);
            finalize_k<<<1, kStream, 0, st>>>(c->partials, nb, nZ, c->scalars);
            MTK_CUDA_TRY(cudaMemcpyAsync(dp.data(), c->scalars, sizeof(double) * nZ, cudaMemcpyDeviceToHost, st));
            c->kernels += 4;
            MTK_CUDA_TRY(cudaGetLastError());
            MTK_CUDA_TRY(cudaMemcpyAsync(wz.data(), z32.p + nY, sizeof(float) * nZ, cudaMemcpyDeviceToHost, st));
            MTK_CUDA_TRY(cudaStreamSynchronize(st));
            for (int l = 0; l < nZ; l++) {
                G0[(size_t)l * nZ + k] = -(dw[l] + (double)wz[l]);
                C0[(size_t)l * nZ + k] = dp[l] + (l == k ? 1.0 : 0.0);
            }
        }
        for (int a = 0; a < nZ; a++)
            for (int b = 0; b < a; b++) {
                const double g = 0.5 * (G0[(size_t)a * nZ + b] + G0[(size_t)b * nZ + a]);
                G0[(size_t)a * nZ + b] = G0[(size_t)b * nZ + a] = g;
                const double h = 0.5 * (C0[(size_t)a * nZ + b] + C0[(size_t)b * nZ + a]);
                C0[(size_t)a * nZ + b] = C0[(size_t)b * nZ + a] = h;
            }
        cur_scale = save_scale;
        phi_ok = true;
        return MTK_OK;
    }
};

template <> RDevHierarchy<double> Igm::rhier<double>() const { return RH64; }
template <> RDevHierarchy<float> Igm::rhier<float>() const { return RH32; }

// Orthonormal rows (two-pass Gram-Schmidt); returns false if `row` is dependent.
bool add_orthonormal(std::vector<std::vector<double>>& Q, std::vector<double> row) {
    double n0 = 0;
    for (double v : row) n0 += v * v;
    n0 = std::sqrt(n0);
    if (n0 == 0) return false;
    for (int pass = 0; pass < 2; pass++)
        for (auto& q : Q) {
            double d = 0;
            for (size_t j = 0; j < row.size(); j++) d += q[j] * row[j];
            for (size_t j = 0; j < row.size(); j++) row[j] -= d * q[j];
        }
    double n = 0;
    for (double v : row) n += v * v;
    n = std::sqrt(n);
    if (n <= 1e-10 * n0) return false;
    for (double& v : row) v /= n;
    Q.push_back(std::move(row));
    return true;
}

// Dense Cholesky inverse of an SPD matrix (n x n, row-major); returns false if not SPD.
bool spd_inverse(std::vector<double>& A, int n) {
    std::vector<double> L(A);
    for (int j = 0; j < n; j++) {
        double d = L[(size_t)j * n + j];
        for (int k = 0; k < j; k++) d -= L[(size_t)j * n + k] * L[(size_t)j * n + k];
        if (!(d > 0)) return false;
        d = std::sqrt(d);
        L[(size_t)j * n + j] = d;
        for (int i = j + 1; i < n; i++) {
            double s = L[(size_t)i * n + j];
            for (int k = 0; k < j; k++) s -= L[(size_t)i * n + k] * L[(size_t)j * n + k];
            L[(size_t)i * n + j] = s / d;
        }
    }
    // inverse via solving L L^T X = I column by column
    std::vector<double> inv((size_t)n * n, 0.0), y(n);
    for (int col = 0; col < n; col++) {
        for (int i = 0; i < n; i++) {
            double s = i == col ? 1.0 : 0.0;
            for (int k = 0; k < i; k++) s -= L[(size_t)i * n + k] * y[k];
            y[i] = s / L[(size_t)i * n + i];
        }
        for (int i = n - 1; i >= 0; i--) {
            double s = y[i];
            for (int k = i + 1; k < n; k++) s -= L[(size_t)k * n + i] * inv[(size_t)k * n + col];
            inv[(size_t)i * n + col] = s / L[(size_t)i * n + i];
        }
    }
    A.swap(inv);
    return true;
}

}  // namespace

namespace {
int igm_run(mtk_ctx* c, const mtk_igm_desc* d, const mtk_solve_opts* opts_in, double* fullx, int32_t* fix_order,
            int32_t* fix_vals, int32_t* n_fixed, double* x_naive, mtk_stats* stats, const SizeFieldJob* job) {
    if (!c || !d || !fullx) return MTK_ERR_BAD_INPUT;
    if (d->N != 4 || d->n != 2) { mtk_set_last_error("only N = 4 (n = 2) is supported", __FILE__, __LINE__); return MTK_ERR_BAD_INPUT; }
    if (d->nF <= 0 || d->nCut <= 0 || d->nFull <= 0 || !d->cutF || !d->cutV || !d->w_ptr || !d->full2y || !d->F2)
        return MTK_ERR_BAD_INPUT;
    mtk_solve_opts o;
    mtk_default_opts(&o);
    if (opts_in) o = *opts_in;
    MTK_CUDA_TRY(cudaSetDevice(c->device));
    AllocStreamScope alloc_scope(c->stream);
    auto t_start = std::chrono::steady_clock::now();
    Igm S;
    S.c = c;
    S.st = c->stream;
    cudaStream_t st = c->stream;
    const int nF = d->nF, nCut = d->nCut, nFull = d->nFull, nJ = d->nJ, nZ = d->nZ;
    S.nF = nF; S.nCut = nCut; S.nFull = nFull; S.nJ = nJ; S.nZ = nZ; S.length = d->length;
    // ---- index maps
    S.full2y.assign(d->full2y, d->full2y + nFull);
    S.full2j.assign(nFull, -1);
    int nY = 0;
    for (int i = 0; i < nFull; i++) if (S.full2y[i] >= 0) nY = std::max(nY, S.full2y[i] + 1);
    for (int s = 0; s < nJ; s++) {
        int i = d->uniqueJ[s];
        if (i < 0 || i >= nFull || S.full2y[i] >= 0) return MTK_ERR_BAD_INPUT;
        S.full2j[i] = s;
    }
    std::vector<int> y2full(nY, -1);
    for (int i = 0; i < nFull; i++) if (S.full2y[i] >= 0) y2full[S.full2y[i]] = i;
    for (int j = 0; j < nY; j++) if (y2full[j] < 0) return MTK_ERR_BAD_INPUT;
    S.nY = nY;
    S.nRed = nY + nZ;
    S.USmall.assign(d->USmall, d->USmall + (size_t)nJ * nZ);
    for (int i = 0; i < 3 * nF; i++) if (d->cutF[i] < 0 || d->cutF[i] >= nCut) return MTK_ERR_BAD_INPUT;
    // ---- W with tags, and its transpose split into y / J parts
    const int nW = 2 * nCut;
    const int nnzW = d->w_ptr[nW];
    S.nnzW = nnzW;
    std::vector<int> tag(nnzW);
    for (int e = 0; e < nnzW; e++) {
        int i = d->w_idx[e];
        if (i < 0 || i >= nFull) return MTK_ERR_BAD_INPUT;
        tag[e] = S.full2y[i] >= 0 ? S.full2y[i] : -1 - S.full2j[i];
    }
    std::vector<int> yptr(nY + 1, 0), jptr(nJ + 1, 0);
    for (int e = 0; e < nnzW; e++) { if (tag[e] >= 0) yptr[tag[e] + 1]++; else jptr[-tag[e]]++; }
    for (int j = 0; j < nY; j++) yptr[j + 1] += yptr[j];
    for (int s = 0; s < nJ; s++) jptr[s + 1] += jptr[s];
    std::vector<int> yrow(yptr[nY]), jrow(jptr[nJ]);
    S.nnzYT = yptr[nY];
    std::vector<double> yval(yptr[nY]), jval(jptr[nJ]);
    {
        std::vector<int> fy(yptr.begin(), yptr.end() - 1), fj(jptr.begin(), jptr.end() - 1);
        for (int r = 0; r < nW; r++)
            for (int e = d->w_ptr[r]; e < d->w_ptr[r + 1]; e++) {
                if (tag[e] >= 0) { int p = fy[tag[e]]++; yrow[p] = r; yval[p] = d->w_val[e]; }
                else { int s = -1 - tag[e]; int p = fj[s]++; jrow[p] = r; jval[p] = d->w_val[e]; }
            }
    }
    // ---- cut vertex -> faces and padded stiffness rows
    std::vector<int> vptr(nCut + 1, 0);
    for (int i = 0; i < 3 * nF; i++) vptr[d->cutF[i] + 1]++;
    int maxdeg = 0;
    for (int v = 0; v < nCut; v++) maxdeg = std::max(maxdeg, vptr[v + 1]);
    if (maxdeg > kMaxFaceDeg) { mtk_set_last_error("vertex with more than 30 faces", __FILE__, __LINE__); return MTK_ERR_BAD_INPUT; }
    std::vector<int> sptr(nCut + 1, 0);
    for (int v = 0; v < nCut; v++) sptr[v + 1] = sptr[v] + vptr[v + 1] + 2;
    S.nnzS = sptr[nCut];
    for (int v = 0; v < nCut; v++) vptr[v + 1] += vptr[v];
    std::vector<int> vface(vptr[nCut]);
    {
        std::vector<int> fill(vptr.begin(), vptr.end() - 1);
        for (int f = 0; f < nF; f++) for (int j = 0; j < 3; j++) vface[fill[d->cutF[3 * f + j]]++] = f;
    }
    // ---- uploads
    MTK_TRY(S.cutF.upload(d->cutF, 3 * (size_t)nF, st));
    MTK_TRY(S.cutV.upload(d->cutV, 3 * (size_t)nCut, st));
    MTK_TRY(S.vf_ptr.upload(vptr.data(), vptr.size(), st));
    MTK_TRY(S.vf_face.upload(vface.data(), vface.size(), st));
    MTK_TRY(S.s_ptr.upload(sptr.data(), sptr.size(), st));
    MTK_TRY(S.s_col.alloc(sptr[nCut])); MTK_TRY(S.s_val.alloc(sptr[nCut])); MTK_TRY(S.s_val32.alloc(sptr[nCut]));
    MTK_TRY(S.s_diag.alloc(nCut));
    MTK_TRY(S.w_ptr.upload(d->w_ptr, nW + 1, st));
    MTK_TRY(S.w_tag.upload(tag.data(), nnzW, st));
    MTK_TRY(S.w_val.upload(d->w_val, nnzW, st));
    std::vector<float> wv32(d->w_val, d->w_val + nnzW), yv32(yval.begin(), yval.end()), jv32(jval.begin(), jval.end());
    MTK_TRY(S.w_val32.upload(wv32.data(), nnzW, st));
    MTK_TRY(S.yt_ptr.upload(yptr.data(), yptr.size(), st));
    MTK_TRY(S.yt_row.upload(yrow.data(), yrow.size(), st));
    MTK_TRY(S.yt_val.upload(yval.data(), yval.size(), st));
    MTK_TRY(S.yt_val32.upload(yv32.data(), yv32.size(), st));
    MTK_TRY(S.jt_ptr.upload(jptr.data(), jptr.size(), st));
    if (!getenv("MTK_NO_JCHUNK")) MTK_TRY(S.upload_chunks(jptr, S.jtc_row, S.jtc_beg, S.jtc_first, S.jtc_n));
    MTK_TRY(S.jt_row.upload(jrow.data(), jrow.size(), st));
    MTK_TRY(S.jt_val.upload(jval.data(), jval.size(), st));
    MTK_TRY(S.jt_val32.upload(jv32.data(), jv32.size(), st));
    MTK_TRY(S.Us.upload(S.USmall.data(), S.USmall.size(), st));
    std::vector<float> us32(S.USmall.begin(), S.USmall.end());
    MTK_TRY(S.Us32.upload(us32.data(), us32.size(), st));
    MTK_TRY(S.d_full2y.upload(S.full2y.data(), nFull, st));
    MTK_TRY(S.d_full2j.upload(S.full2j.data(), nFull, st));
    MTK_TRY(S.F2.upload(d->F2, 8 * (size_t)nF, st));
    MTK_TRY(S.Fsi.alloc(8 * (size_t)nF));
    MTK_TRY(S.grad.alloc(6 * (size_t)nF));
    MTK_TRY(S.hb.alloc(2 * (size_t)nCut)); MTK_TRY(S.XbJ.alloc(std::max(nJ, 1)));
    MTK_TRY(S.U.alloc(2 * (size_t)nCut)); MTK_TRY(S.Qc.alloc(2 * (size_t)nCut)); MTK_TRY(S.XoJ.alloc(std::max(nJ, 1)));
    MTK_TRY(S.U32.alloc(2 * (size_t)nCut)); MTK_TRY(S.Qc32.alloc(2 * (size_t)nCut)); MTK_TRY(S.XoJ32.alloc(std::max(nJ, 1)));
    MTK_TRY(S.minvy.alloc(std::max(nY, 1))); MTK_TRY(S.minvy32.alloc(std::max(nY, 1)));
    const int nRed = S.nRed;
    MTK_TRY(S.xs.alloc(nRed)); MTK_TRY(S.bsys.alloc(nRed)); MTK_TRY(S.r64.alloc(nRed)); MTK_TRY(S.z64.alloc(nRed));
    MTK_TRY(S.p64.alloc(nRed)); MTK_TRY(S.q64.alloc(nRed)); MTK_TRY(S.prev.alloc(nRed)); MTK_TRY(S.scratch.alloc(nRed));
    MTK_TRY(S.Xfull.alloc(std::max(nFull, nRed)));
    MTK_TRY(S.XJ64.alloc(std::max(nJ, 1)));
    MTK_TRY(S.r32.alloc(nRed)); MTK_TRY(S.e32.alloc(nRed)); MTK_TRY(S.z32.alloc(nRed)); MTK_TRY(S.p32.alloc(nRed));
    MTK_TRY(S.q32.alloc(nRed)); MTK_TRY(S.pb32.alloc(nRed)); MTK_TRY(S.pb64.alloc(nRed));
    S.h_fixy.assign(std::max(nY, 1), 0);
    MTK_TRY(S.fixy.upload(S.h_fixy.data(), S.h_fixy.size(), st));
    const int nLeftCap = std::max(1, d->nSingular + d->nInteger);
    MTK_TRY(S.left.alloc(nLeftCap));
    // shared memory for the replicated z state: 6 nZ + 2 nJ values
    S.smem64 = zsmem_bytes(sizeof(double), nZ, nJ);
    S.smem32 = zsmem_bytes(sizeof(float), nZ, nJ);
    S.nZ_ = nZ;
    S.nJ_ = nJ;
    S.z_global_forced = getenv("MTK_Z_GLOBAL") && getenv("MTK_Z_GLOBAL")[0] == '1';

    const int G = S.grid();
    MTK_CUDA_TRY(cudaEventRecord(c->ev_a, st));
    face_gradients<<<G, kStream, 0, st>>>(nF, S.cutF.p, S.cutV.p, S.grad.p);
    assemble_stiffness<<<G, kStream, 0, st>>>(nCut, S.vf_ptr.p, S.vf_face.p, S.cutF.p, S.grad.p, S.s_ptr.p, S.s_col.p,
                                             S.s_val.p, S.s_val32.p, S.s_diag.p);
    c->kernels += 2;
    MTK_CUDA_TRY(cudaGetLastError());

    // ---- dense z block of the normal matrix (host, FP64) for the block-Jacobi preconditioner:
    //      K_zz = scale * USmall^T (2 W_J^T S W_J) USmall + shift I.  Only faces touching J matter.
    std::vector<double> h_grad(6 * (size_t)nF);
    MTK_CUDA_TRY(cudaMemcpyAsync(h_grad.data(), S.grad.p, sizeof(double) * h_grad.size(), cudaMemcpyDeviceToHost, st));
    MTK_CUDA_TRY(cudaStreamSynchronize(st));
    // ---- multigrid for the free block: K_pre = 2 W_y^T S W_y + delta I, delta = 1e-4 / length^2
    //      (the seamless system is length^2 K_pre exactly; the naive one up to the shift)
    auto th0 = std::chrono::steady_clock::now();
    auto tlap = th0;
    auto lap = [&](const char* what) {   // set-up stage times (MTK_DEBUG=1)
        if (!Igm::debug()) return;
        const auto t = std::chrono::steady_clock::now();
        fprintf(stderr, "[igm host]   %-28s %7.1f ms\n", what, std::chrono::duration<double, std::milli>(t - tlap).count());
        tlap = t;
    };
    if (nY > 0 && !getenv("MTK_NO_AMG")) {
        const double delta = 1e-4 / (d->length * d->length);
        RCsr K;
        DevCsr64 dK;
        bool dev_K = false;
        if (!getenv("MTK_MG_HOST")) {
            // K_yy + delta I, the FP32 operator arrays and C_yJ / C_Jy assembled on the device (the
            // arrays of the host assembly below, same rounding and order); K comes back to the host
            // for the aggregation
            RDevBuilder B(c, st);
            MTK_TRY(B.prepare());
            DevCsr64 Hs, Cy, Cj;
            const rgpu::StiffVisit sv{S.vf_ptr.p, S.vf_face.p, S.cutF.p, S.grad.p};
            MTK_TRY(B.two_pass(nCut, Hs, [&](int* cnt, const int* optr, int* oc, double* ov) {
                rgpu::rows_sorted<<<B.grid(nCut), kStream, 0, st>>>(nCut, sv, cnt, optr, oc, ov, B.err_.p);
            }));
            const rgpu::FreeBlockVisit kv{S.yt_ptr.p, S.yt_row.p, S.yt_val.p, Hs.ptr.p, Hs.col.p, Hs.val.p,
                                          S.w_ptr.p, S.w_tag.p, S.w_val.p, delta, false};
            MTK_TRY(B.two_pass(nY, dK, [&](int* cnt, const int* optr, int* oc, double* ov) {
                rgpu::rows_sorted<<<B.grid(nY), kStream, 0, st>>>(nY, kv, cnt, optr, oc, ov, B.err_.p);
            }));
            if (!getenv("MTK_NO_ASM")) {
                MTK_TRY(S.ka_ptr.alloc(nY + 1));
                MTK_TRY(S.ka_col.alloc(std::max<size_t>(dK.nnz, 1)));
                MTK_TRY(S.ka_val32.alloc(std::max<size_t>(dK.nnz, 1)));
                MTK_CUDA_TRY(cudaMemcpyAsync(S.ka_ptr.p, dK.ptr.p, sizeof(int) * (nY + 1), cudaMemcpyDeviceToDevice, st));
                MTK_CUDA_TRY(cudaMemcpyAsync(S.ka_col.p, dK.col.p, sizeof(int) * dK.nnz, cudaMemcpyDeviceToDevice, st));
                rgpu::free_block_f32<<<B.grid(nY), kStream, 0, st>>>(nY, dK.ptr.p, dK.col.p, dK.val.p, delta, S.ka_val32.p);
                const rgpu::FreeBlockVisit cv{S.yt_ptr.p, S.yt_row.p, S.yt_val.p, Hs.ptr.p, Hs.col.p, Hs.val.p,
                                              S.w_ptr.p, S.w_tag.p, S.w_val.p, 0.0, true};
                MTK_TRY(B.two_pass(nY, Cy, [&](int* cnt, const int* optr, int* oc, double* ov) {
                    rgpu::rows_sorted<<<B.grid(nY), kStream, 0, st>>>(nY, cv, cnt, optr, oc, ov, B.err_.p);
                }));
                MTK_TRY(B.transpose(Cy, std::max(nJ, 1), Cj, 1.0));
                auto to32 = [&](DevCsr64& M, DBuf<int>& ptr, DBuf<int>& col, DBuf<float>& v32) -> int {
                    ptr = std::move(M.ptr);
                    col = std::move(M.col);
                    MTK_TRY(v32.alloc(std::max<size_t>(M.nnz, 1)));
                    if (M.nnz) rgpu::to_f32_vals<<<B.grid((long long)M.nnz), kStream, 0, st>>>(M.nnz, M.val.p, v32.p);
                    else MTK_CUDA_TRY(cudaMemsetAsync(v32.p, 0, sizeof(float), st));
                    return MTK_OK;
                };
                MTK_TRY(to32(Cy, S.cy_ptr, S.cy_col, S.cy_val32));
                MTK_TRY(to32(Cj, S.cj_ptr, S.cj_col, S.cj_val32));
                if (Cy.nnz == 0) {   // empty coupling: one harmless entry so every array exists
                    const int z = 0;
                    MTK_CUDA_TRY(cudaMemcpyAsync(S.cy_col.p, &z, sizeof(int), cudaMemcpyHostToDevice, st));
                    MTK_CUDA_TRY(cudaMemcpyAsync(S.cj_col.p, &z, sizeof(int), cudaMemcpyHostToDevice, st));
                }
            }
            MTK_CUDA_TRY(cudaGetLastError());
            bool over = false;
            MTK_TRY(B.failed(over));
            if (!over) {
                K.n = nY;
                K.ptr.resize(nY + 1);
                K.col.resize(dK.nnz);
                K.val.resize(dK.nnz);
                MTK_CUDA_TRY(cudaMemcpyAsync(K.ptr.data(), dK.ptr.p, sizeof(int) * (nY + 1), cudaMemcpyDeviceToHost, st));
                MTK_CUDA_TRY(cudaMemcpyAsync(K.col.data(), dK.col.p, sizeof(int) * dK.nnz, cudaMemcpyDeviceToHost, st));
                MTK_CUDA_TRY(cudaMemcpyAsync(K.val.data(), dK.val.p, sizeof(double) * dK.nnz, cudaMemcpyDeviceToHost, st));
                MTK_CUDA_TRY(cudaStreamSynchronize(st));
                dev_K = true;
                if (!getenv("MTK_NO_ASM")) S.asm_ok = true;   // BJJ is uploaded once it is built below
                lap("free block K (device) + download");
            }
        }
        if (!dev_K) {
            std::vector<int> hs_ptr, hs_col;
            std::vector<double> hs_val;
            build_rows_parallel<double>(
                nCut, nCut,
                [&](int c2, auto add) {
                    for (int k = vptr[c2]; k < vptr[c2 + 1]; k++) {
                        const int f = vface[k];
                        const int a = d->cutF[3 * f] == c2 ? 0 : (d->cutF[3 * f + 1] == c2 ? 1 : 2);
                        for (int j = 0; j < 3; j++)
                            add(d->cutF[3 * f + j], h_grad[6 * f + 2 * a] * h_grad[6 * f + 2 * j] +
                                                        h_grad[6 * f + 2 * a + 1] * h_grad[6 * f + 2 * j + 1]);
                    }
                },
                hs_ptr, hs_col, hs_val);
            lap("stiffness (cut vertices)");
            K = RCsr();
            K.n = nY;
            build_rows_parallel<double>(
                nY, nY,
                [&](int j, auto add) {
                    for (int e = yptr[j]; e < yptr[j + 1]; e++) {
                        const int r = yrow[e], c2 = r >> 1, kk = r & 1;
                        const double w1 = yval[e];
                        for (int p = hs_ptr[c2]; p < hs_ptr[c2 + 1]; p++) {
                            const int r2 = 2 * hs_col[p] + kk;
                            const double sv = hs_val[p];
                            for (int e2 = d->w_ptr[r2]; e2 < d->w_ptr[r2 + 1]; e2++) {
                                const int y2 = tag[e2];
                                if (y2 >= 0) add(y2, 2.0 * w1 * sv * d->w_val[e2]);
                            }
                        }
                    }
                    add(j, delta);
                },
                K.ptr, K.col, K.val);
            lap("free block K");
            // assembled operator of the FP32 inner solves: K_yy (without the multigrid's delta), the
            // free-to-translation coupling C_yJ and its transpose
            if (!getenv("MTK_NO_ASM")) {
                std::vector<float> kv(K.val.size());
    #pragma omp parallel for schedule(static)
                for (int j = 0; j < nY; j++)
                    for (int q = K.ptr[j]; q < K.ptr[j + 1]; q++)
                        kv[q] = (float)(K.col[q] == j ? K.val[q] - delta : K.val[q]);
                MTK_TRY(S.ka_ptr.upload(K.ptr.data(), K.ptr.size(), st));
                MTK_TRY(S.ka_col.upload(K.col.data(), K.col.size(), st));
                MTK_TRY(S.ka_val32.upload(kv.data(), kv.size(), st));
                std::vector<int> cptr, ccol;
                std::vector<double> cval;
                build_rows_parallel<double>(
                    nY, std::max(nJ, 1),
                    [&](int j, auto add) {
                        for (int e = yptr[j]; e < yptr[j + 1]; e++) {
                            const int r = yrow[e], c2 = r >> 1, kk = r & 1;
                            const double w1 = yval[e];
                            for (int q = hs_ptr[c2]; q < hs_ptr[c2 + 1]; q++) {
                                const int r2 = 2 * hs_col[q] + kk;
                                const double sv = hs_val[q];
                                for (int e2 = d->w_ptr[r2]; e2 < d->w_ptr[r2 + 1]; e2++)
                                    if (tag[e2] < 0) add(-1 - tag[e2], 2.0 * w1 * sv * d->w_val[e2]);
                            }
                        }
                    },
                    cptr, ccol, cval);
                std::vector<float> cv32(cval.begin(), cval.end());
                std::vector<int> tptr(std::max(nJ, 1) + 1, 0), tcol(ccol.size());
                std::vector<float> tval(ccol.size());
                for (int c2 : ccol) tptr[c2 + 1]++;
                for (int a2 = 0; a2 < std::max(nJ, 1); a2++) tptr[a2 + 1] += tptr[a2];
                {
                    std::vector<int> fill(tptr.begin(), tptr.end() - 1);
                    for (int j = 0; j < nY; j++)
                        for (int q = cptr[j]; q < cptr[j + 1]; q++) {
                            const int t = fill[ccol[q]]++;
                            tcol[t] = j;
                            tval[t] = (float)cval[q];
                        }
                }
                if (ccol.empty()) { ccol.push_back(0); cv32.push_back(0.f); tcol.push_back(0); tval.push_back(0.f); }
                MTK_TRY(S.cy_ptr.upload(cptr.data(), cptr.size(), st));
                MTK_TRY(S.cy_col.upload(ccol.data(), ccol.size(), st));
                MTK_TRY(S.cy_val32.upload(cv32.data(), cv32.size(), st));
                MTK_TRY(S.cj_ptr.upload(tptr.data(), tptr.size(), st));
                MTK_TRY(S.cj_col.upload(tcol.data(), tcol.size(), st));
                MTK_TRY(S.cj_val32.upload(tval.data(), tval.size(), st));
                MTK_CUDA_TRY(cudaStreamSynchronize(st));
                S.asm_ok = true;   // BJJ is uploaded once it is built below
                lap("assembled operator + upload");
            }
        }
        std::vector<int> node(nY), comp(nY);
        for (int j = 0; j < nY; j++) { node[j] = y2full[j] / 2; comp[j] = y2full[j] % 2; }
        MTK_TRY(S.build_mg(std::move(K), std::move(node), std::move(comp), nFull / 2, dev_K ? &dK : nullptr));
        lap("hierarchy + upload");
    }
    if (Igm::debug())
        fprintf(stderr, "[igm host] multigrid set-up %.1f ms (levels %d)\n",
                std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - th0).count(), S.mg_levels);
    std::vector<double> BJJ((size_t)nJ * nJ, 0.0);
    if (nJ > 0) {
        std::vector<char> touchJ(nCut, 0);
        for (int r = 0; r < nW; r++)
            for (int e = d->w_ptr[r]; e < d->w_ptr[r + 1]; e++) if (tag[e] < 0) touchJ[r >> 1] = 1;
        for (int f = 0; f < nF; f++) {
            int cv[3] = {d->cutF[3 * f], d->cutF[3 * f + 1], d->cutF[3 * f + 2]};
            if (!touchJ[cv[0]] && !touchJ[cv[1]] && !touchJ[cv[2]]) continue;
            for (int a = 0; a < 3; a++)
                for (int b = 0; b < 3; b++) {
                    double sab = h_grad[6 * f + 2 * a] * h_grad[6 * f + 2 * b] + h_grad[6 * f + 2 * a + 1] * h_grad[6 * f + 2 * b + 1];
                    for (int k = 0; k < 2; k++) {
                        int ra = 2 * cv[a] + k, rb = 2 * cv[b] + k;
                        for (int e1 = d->w_ptr[ra]; e1 < d->w_ptr[ra + 1]; e1++) {
                            if (tag[e1] >= 0) continue;
                            for (int e2 = d->w_ptr[rb]; e2 < d->w_ptr[rb + 1]; e2++) {
                                if (tag[e2] >= 0) continue;
                                BJJ[(size_t)(-1 - tag[e1]) * nJ + (-1 - tag[e2])] += 2.0 * d->w_val[e1] * sab * d->w_val[e2];
                            }
                        }
                    }
                }
        }
    }
    if (S.asm_ok) {
        std::vector<float> b32(BJJ.begin(), BJJ.end());
        if (b32.empty()) b32.push_back(0.f);
        MTK_TRY(S.bjj32.upload(b32.data(), b32.size(), st));
        if (!getenv("MTK_NO_JCHUNK") && nJ > 0) {   // chunks of the translation rows of C_Jy
            std::vector<int> cptr(nJ + 1);
            MTK_CUDA_TRY(cudaMemcpyAsync(cptr.data(), S.cj_ptr.p, sizeof(int) * (nJ + 1), cudaMemcpyDeviceToHost, st));
            MTK_CUDA_TRY(cudaStreamSynchronize(st));
            MTK_TRY(S.upload_chunks(cptr, S.cjc_row, S.cjc_beg, S.cjc_first, S.cjc_n));
        }
    }
    auto build_zblock = [&](double scale, double shift, std::vector<double>& Kzz) {
        Kzz.assign((size_t)nZ * nZ, 0.0);
        if (S.phi_ok) {   // Galerkin block of the Schur coarse space
            for (size_t i = 0; i < Kzz.size(); i++) Kzz[i] = scale * S.G0[i] + shift * S.C0[i];
            return;
        }
        std::vector<double> tmp((size_t)nJ * nZ, 0.0);   // BJJ * USmall
        for (int a = 0; a < nJ; a++)
            for (int b = 0; b < nJ; b++) {
                double v = BJJ[(size_t)a * nJ + b];
                if (v == 0) continue;
                for (int j = 0; j < nZ; j++) tmp[(size_t)a * nZ + j] += v * S.USmall[(size_t)b * nZ + j];
            }
        for (int i = 0; i < nZ; i++)
            for (int j = 0; j < nZ; j++) {
                double s = 0;
                for (int a = 0; a < nJ; a++) s += S.USmall[(size_t)a * nZ + i] * tmp[(size_t)a * nZ + j];
                Kzz[(size_t)i * nZ + j] = scale * s + (i == j ? shift : 0.0);
            }
    };
    // constraint state
    std::vector<std::vector<double>> Qrows;          // orthonormal rows on z
    std::vector<std::vector<double>> Arows;          // raw constraint rows on z
    std::vector<double> Avals;
    auto upload_constraints = [&](double scale, double shift) -> int {
        // projector rows
        S.kq = (int)Qrows.size();
        std::vector<double> q((size_t)std::max(S.kq, 1) * std::max(nZ, 1), 0.0);
        for (int a = 0; a < S.kq; a++) for (int j = 0; j < nZ; j++) q[(size_t)a * nZ + j] = Qrows[a][j];
        MTK_TRY(S.Qz.upload(q.data(), q.size(), st));
        std::vector<float> q32(q.begin(), q.end());
        MTK_TRY(S.Qz32.upload(q32.data(), q32.size(), st));
        // z-block preconditioner: inverse of (P K_zz P + Q^T Q) restricted, i.e. of K_zz on the
        // complement plus identity on the constrained directions
        if (nZ > 0) {
            std::vector<double> Kzz;
            build_zblock(scale, shift, Kzz);
            std::vector<double> PK((size_t)nZ * nZ);
            // P K P + Q^T Q (SPD when K is SPD on range(P))
            std::vector<double> Pm((size_t)nZ * nZ, 0.0);
            for (int i = 0; i < nZ; i++) Pm[(size_t)i * nZ + i] = 1.0;
            for (auto& qr : Qrows)
                for (int i = 0; i < nZ; i++) for (int j = 0; j < nZ; j++) Pm[(size_t)i * nZ + j] -= qr[i] * qr[j];
            std::vector<double> t1((size_t)nZ * nZ, 0.0);
            for (int i = 0; i < nZ; i++) for (int k = 0; k < nZ; k++) {
                double a = Pm[(size_t)i * nZ + k];
                if (a == 0) continue;
                for (int j = 0; j < nZ; j++) t1[(size_t)i * nZ + j] += a * Kzz[(size_t)k * nZ + j];
            }
            for (int i = 0; i < nZ; i++) for (int j = 0; j < nZ; j++) {
                double s = 0;
                for (int k = 0; k < nZ; k++) s += t1[(size_t)i * nZ + k] * Pm[(size_t)k * nZ + j];
                PK[(size_t)i * nZ + j] = s;
            }
            // ridge on the constrained directions, scaled from the unprojected block (the
            // projected block is pure round-off once the constraints pin every z direction)
            double dmax = 0;
            for (int i = 0; i < nZ; i++) dmax = std::max(dmax, Kzz[(size_t)i * nZ + i]);
            if (!(dmax > 0)) dmax = 1;
            for (auto& qr : Qrows) for (int i = 0; i < nZ; i++) for (int j = 0; j < nZ; j++) PK[(size_t)i * nZ + j] += dmax * qr[i] * qr[j];
            std::vector<double> inv = PK;
            if (!spd_inverse(inv, nZ)) {   // fall back to the diagonal
                inv.assign((size_t)nZ * nZ, 0.0);
                for (int i = 0; i < nZ; i++) { double v = PK[(size_t)i * nZ + i]; inv[(size_t)i * nZ + i] = v > 0 ? 1.0 / v : 1.0; }
            }
            MTK_TRY(S.Mz.upload(inv.data(), inv.size(), st));
            std::vector<float> inv32(inv.begin(), inv.end());
            MTK_TRY(S.Mz32.upload(inv32.data(), inv32.size(), st));
        } else {
            double one = 1.0;
            float onef = 1.f;
            MTK_TRY(S.Mz.upload(&one, 1, st));
            MTK_TRY(S.Mz32.upload(&onef, 1, st));
        }
        jacobi_y<<<G, kStream, 0, st>>>(nY, S.yt_ptr.p, S.yt_row.p, S.yt_val.p, S.s_diag.p, scale, shift, S.minvy.p, S.minvy32.p);
        c->kernels++;
        MTK_TRY(S.fixy.upload(S.h_fixy.data(), S.h_fixy.size(), st));
        MTK_CUDA_TRY(cudaGetLastError());
        return MTK_OK;
    };
    // Adds the constraint X[full] = val; moves xs (device) to the nearest feasible point.
    auto add_constraint = [&](int full, double val) -> int {
        int y = S.full2y[full];
        if (y >= 0) {
            S.h_fixy[y] = 1;
            MTK_CUDA_TRY(cudaMemcpyAsync(S.xs.p + y, &val, sizeof(double), cudaMemcpyHostToDevice, st));
            MTK_CUDA_TRY(cudaStreamSynchronize(st));
            return MTK_OK;
        }
        int s = S.full2j[full];
        std::vector<double> row(S.USmall.begin() + (size_t)s * nZ, S.USmall.begin() + (size_t)(s + 1) * nZ);
        // A row in the span of the earlier rows adds no constraint (its value is implied by
        // them; the greedy order only fixes such a variable when it is already integral).
        if (!add_orthonormal(Qrows, row)) return MTK_OK;
        Arows.push_back(row);
        Avals.push_back(val);
        // feasible correction of z: z += A^T (A A^T)^+ (g - A z), via the orthonormal basis:
        // solve in the row space with least squares (Q spans the rows of A).
        std::vector<double> z(nZ);
        MTK_CUDA_TRY(cudaMemcpyAsync(z.data(), S.xs.p + S.nY, sizeof(double) * nZ, cudaMemcpyDeviceToHost, st));
        MTK_CUDA_TRY(cudaStreamSynchronize(st));
        // Gauss-Newton on the small system: minimise |dz| s.t. A (z + dz) = g (a few refinement passes)
        const int m = (int)Arows.size();
        for (int pass = 0; pass < 3; pass++) {
            std::vector<double> res(m);
            double worst = 0;
            for (int a = 0; a < m; a++) {
                double t = Avals[a];
                for (int j = 0; j < nZ; j++) t -= Arows[a][j] * z[j];
                res[a] = t;
                worst = std::max(worst, std::fabs(t));
            }
            if (worst < 1e-13) break;
            // normal equations (A A^T) w = res, dz = A^T w (m small; Cholesky with tiny ridge)
            std::vector<double> AAt((size_t)m * m);
            for (int a = 0; a < m; a++)
                for (int b2 = 0; b2 < m; b2++) {
                    double t = 0;
                    for (int j = 0; j < nZ; j++) t += Arows[a][j] * Arows[b2][j];
                    AAt[(size_t)a * m + b2] = t + (a == b2 ? 1e-14 : 0.0);
                }
            if (!spd_inverse(AAt, m)) break;
            std::vector<double> w(m, 0.0);
            for (int a = 0; a < m; a++) for (int b2 = 0; b2 < m; b2++) w[a] += AAt[(size_t)a * m + b2] * res[b2];
            for (int j = 0; j < nZ; j++) {
                double t = 0;
                for (int a = 0; a < m; a++) t += Arows[a][j] * w[a];
                z[j] += t;
            }
        }
        MTK_CUDA_TRY(cudaMemcpyAsync(S.xs.p + S.nY, z.data(), sizeof(double) * nZ, cudaMemcpyHostToDevice, st));
        MTK_CUDA_TRY(cudaStreamSynchronize(st));
        return MTK_OK;
    };
    DBuf<int> fixd;      // fixed full indices of the post-rounding check
    DBuf<double> fixv;   // their values
    MTK_TRY(fixd.alloc(nLeftCap));
    MTK_TRY(fixv.alloc(nLeftCap));

    mtk_stats local{};
    mtk_stats* stt = stats ? stats : &local;
    // ================= naive integration (iter_rounding_init.h:171-212) =================
    // length X2F^T X2F x = X2F^T F2 with the anchor rows UFull[fixedIdcs] x = fixedVals.
    const double length = d->length;
    MTK_CUDA_TRY(cudaMemsetAsync(S.xs.p, 0, sizeof(double) * nRed, st));
    for (int k = 0; k < d->nFixed; k++) MTK_TRY(add_constraint(d->fixedIdcs[k], d->fixedVals[k]));
    MTK_TRY(upload_constraints(length, 0.0));
    if (!getenv("MTK_NO_PHI")) {
        auto tp0 = std::chrono::steady_clock::now();
        long long phi_iters = 0;
        MTK_TRY(S.build_phi(&phi_iters));
        stt->pcg_iters += phi_iters;
        if (S.phi_ok) MTK_TRY(upload_constraints(length, 0.0));
        if (Igm::debug())
            fprintf(stderr, "[igm host] Schur coarse space %s: %lld PCG iterations, %.1f ms\n", S.phi_ok ? "on" : "off",
                    phi_iters, std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - tp0).count());
    }
    std::vector<double> es;   // size-field job: exp(sbar_f) per face, target es_f * F2_f
    if (job) {
        es.resize(nF);
        std::vector<double> ft(8 * (size_t)nF);
        for (int f = 0; f < nF; f++) {
            es[f] = std::exp((job->s[job->F[3 * f]] + job->s[job->F[3 * f + 1]] + job->s[job->F[3 * f + 2]]) / 3.0);
            for (int k = 0; k < 8; k++) ft[8 * (size_t)f + k] = es[f] * d->F2[8 * (size_t)f + k];
        }
        MTK_CUDA_TRY(cudaMemcpyAsync(S.Fsi.p, ft.data(), sizeof(double) * ft.size(), cudaMemcpyHostToDevice, st));
        MTK_CUDA_TRY(cudaStreamSynchronize(st));
    }
    MTK_TRY(S.build_rhs(job ? S.Fsi.p : S.F2.p, 1.0, 0.0, nullptr, S.bsys.p));
    double rel = 0;
    MTK_TRY(S.solve(length, 0.0, S.bsys.p, S.xs.p, o, stt, &rel));
    if (job) {
        // loss terms per face, dl/dx = 2 length X2F^T r, the adjoint solve, then (X2F lambda) . F2
        DBuf<double> d_es, d_T, r8, rT, q, lam;
        MTK_TRY(d_es.upload(es.data(), nF, st));
        if (job->T) MTK_TRY(d_T.upload(job->T, 8 * (size_t)nF, st));
        MTK_TRY(r8.alloc(8 * (size_t)nF)); MTK_TRY(rT.alloc(nF)); MTK_TRY(q.alloc(nF)); MTK_TRY(lam.alloc(nRed));
        xj_from_z<<<G, kStream, 0, st>>>(nJ, nY, nZ, S.Us.p, S.xs.p, S.XJ64.p);
        gather_U<<<G, kStream, 0, st>>>(nCut, S.w_ptr.p, S.w_tag.p, S.w_val.p, S.xs.p, S.XJ64.p, S.U.p);
        face_residual<<<G, kStream, 0, st>>>(nF, S.cutF.p, S.grad.p, S.U.p, length, d_es.p, job->T ? d_T.p : S.F2.p, r8.p,
                                             rT.p, c->partials);
        finalize1<<<1, kStream, 0, st>>>(c->partials, G, c->scalars);
        c->kernels += 4;
        MTK_CUDA_TRY(cudaGetLastError());
        double lsum = 0;
        MTK_CUDA_TRY(cudaMemcpyAsync(&lsum, c->scalars, sizeof(double), cudaMemcpyDeviceToHost, st));
        if (job->dgx) {   // position partials at the forward x (U still holds W x)
            DBuf<double> pgx, pgy, pph;
            MTK_TRY(pgx.alloc(3 * (size_t)nF)); MTK_TRY(pgy.alloc(3 * (size_t)nF)); MTK_TRY(pph.alloc(nF));
            face_position_partials<<<G, kStream, 0, st>>>(nF, S.cutF.p, S.grad.p, S.U.p, length, d_es.p, S.F2.p, pgx.p,
                                                          pgy.p, pph.p, c->partials);
            finalize1<<<1, kStream, 0, st>>>(c->partials, G, c->scalars + 1);
            c->kernels += 2;
            MTK_CUDA_TRY(cudaGetLastError());
            MTK_CUDA_TRY(cudaMemcpyAsync(job->dgx, pgx.p, sizeof(double) * 3 * nF, cudaMemcpyDeviceToHost, st));
            MTK_CUDA_TRY(cudaMemcpyAsync(job->dgy, pgy.p, sizeof(double) * 3 * nF, cudaMemcpyDeviceToHost, st));
            MTK_CUDA_TRY(cudaMemcpyAsync(job->dphi, pph.p, sizeof(double) * nF, cudaMemcpyDeviceToHost, st));
            MTK_CUDA_TRY(cudaMemcpyAsync(job->dlength, c->scalars + 1, sizeof(double), cudaMemcpyDeviceToHost, st));
            MTK_CUDA_TRY(cudaStreamSynchronize(st));
        }
        MTK_TRY(S.build_rhs(r8.p, 2.0 * length, 0.0, nullptr, S.bsys.p));
        MTK_CUDA_TRY(cudaMemsetAsync(lam.p, 0, sizeof(double) * nRed, st));   // feasible: fixed entries 0
        double rel2 = 0;
        MTK_TRY(S.solve(length, 0.0, S.bsys.p, lam.p, o, stt, &rel2));
        xj_from_z<<<G, kStream, 0, st>>>(nJ, nY, nZ, S.Us.p, lam.p, S.XJ64.p);
        gather_U<<<G, kStream, 0, st>>>(nCut, S.w_ptr.p, S.w_tag.p, S.w_val.p, lam.p, S.XJ64.p, S.U.p);
        face_target_dot<<<G, kStream, 0, st>>>(nF, S.cutF.p, S.grad.p, S.U.p, S.F2.p, q.p);
        c->kernels += 3;
        MTK_CUDA_TRY(cudaGetLastError());
        std::vector<double> h_rT(nF), h_q(nF);
        MTK_CUDA_TRY(cudaMemcpyAsync(h_rT.data(), rT.p, sizeof(double) * nF, cudaMemcpyDeviceToHost, st));
        MTK_CUDA_TRY(cudaMemcpyAsync(h_q.data(), q.p, sizeof(double) * nF, cudaMemcpyDeviceToHost, st));
        MTK_CUDA_TRY(cudaStreamSynchronize(st));
        // assembly backward: dsbar_f / ds_v = 1/3 for the corners of f; smoothness over edges
        // (half of (s_a - s_b)^2 per face side: an interior edge once, a boundary edge at half weight)
        const double* sv = job->s;
        double smooth = 0;
        std::fill(job->grad_s, job->grad_s + job->nV, 0.0);
        for (int f = 0; f < nF; f++) {
            const double gf = es[f] / 3.0 * (h_q[f] - 2.0 * h_rT[f]);
            for (int j = 0; j < 3; j++) {
                const int a = job->F[3 * f + j], b = job->F[3 * f + (j + 1) % 3];
                job->grad_s[a] += gf;
                const double dsv = sv[a] - sv[b];
                smooth += 0.5 * dsv * dsv;
                job->grad_s[a] += job->mu * dsv;
                job->grad_s[b] -= job->mu * dsv;
            }
        }
        *job->loss = lsum + job->mu * smooth;
        MTK_CUDA_TRY(cudaEventRecord(c->ev_b, st));
        MTK_CUDA_TRY(cudaStreamSynchronize(st));
        float msj = 0;
        cudaEventElapsedTime(&msj, c->ev_a, c->ev_b);
        stt->ms_integrate += msj;
        stt->igm_pcg_launches += S.pcg_launches;
        stt->igm_pcg_passes += S.pcg_passes;
        stt->igm_pcg_ms += S.pcg_ms;
        stt->igm_pcg_bytes += S.pcg_bytes;
        expand_full<<<G, kStream, 0, st>>>(nFull, S.d_full2y.p, S.d_full2j.p, nY, nZ, S.Us.p, S.xs.p, S.Xfull.p);
        c->kernels++;
        MTK_CUDA_TRY(cudaMemcpyAsync(fullx, S.Xfull.p, sizeof(double) * nFull, cudaMemcpyDeviceToHost, st));
        MTK_CUDA_TRY(cudaStreamSynchronize(st));
        stt->kernel_launches = c->kernels;
        return MTK_OK;
    }
    if (x_naive) {
        expand_full<<<G, kStream, 0, st>>>(nFull, S.d_full2y.p, S.d_full2j.p, nY, nZ, S.Us.p, S.xs.p, S.Xfull.p);
        c->kernels++;
        MTK_CUDA_TRY(cudaMemcpyAsync(x_naive, S.Xfull.p, sizeof(double) * nFull, cudaMemcpyDeviceToHost, st));
    }
    // x0 of the naive solution, kept for the "nothing rounded" exit (iter_rounding.h:111)
    DBuf<double> x0red;
    MTK_TRY(x0red.alloc(nRed));
    MTK_CUDA_TRY(cudaMemcpyAsync(x0red.p, S.xs.p, sizeof(double) * nRed, cudaMemcpyDeviceToDevice, st));
    MTK_CUDA_TRY(cudaEventRecord(c->ev_b, st));
    MTK_CUDA_TRY(cudaStreamSynchronize(st));
    float ms = 0;
    cudaEventElapsedTime(&ms, c->ev_a, c->ev_b);
    stt->ms_integrate += ms;
    int status = MTK_OK;
    int nfix = 0;
    auto finish = [&](const double* xsrc) -> int {
        stt->igm_pcg_launches += S.pcg_launches;
        stt->igm_pcg_passes += S.pcg_passes;
        stt->igm_pcg_ms += S.pcg_ms;
        stt->igm_pcg_bytes += S.pcg_bytes;
        expand_full<<<G, kStream, 0, st>>>(nFull, S.d_full2y.p, S.d_full2j.p, nY, nZ, S.Us.p, xsrc, S.Xfull.p);
        c->kernels++;
        MTK_CUDA_TRY(cudaMemcpyAsync(fullx, S.Xfull.p, sizeof(double) * nFull, cudaMemcpyDeviceToHost, st));
        MTK_CUDA_TRY(cudaStreamSynchronize(st));
        if (n_fixed) *n_fixed = nfix;
        stt->kernel_launches = c->kernels;
        stt->ms_total += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count();
        return status;
    };
    if (!d->seamless) return finish(S.xs.p);

    // ================= NI Levenberg-Marquardt (lambda = 0), levenberg_marquardt.h:140-231 =======
    // Variables (xs, f); the f block of J^T J is diagonal and is eliminated exactly.  From the
    // naive solution the reduced Gauss-Newton step for xs is zero (same normal equations), so
    // one step gives f* = (wI^2 length grad(x) + wC^2 F2) / (wI^2 + wC^2); the second
    // iteration's direction is zero and the solve stops (direction norm < tolerance).
    MTK_CUDA_TRY(cudaEventRecord(c->ev_a, st));
    {
        const double wI = 10e3, wC = 1.0;
        xj_from_z<<<G, kStream, 0, st>>>(nJ, nY, nZ, S.Us.p, S.xs.p, S.XJ64.p);
        gather_U<<<G, kStream, 0, st>>>(nCut, S.w_ptr.p, S.w_tag.p, S.w_val.p, S.xs.p, S.XJ64.p, S.U.p);
        lm_field_target<<<G, kStream, 0, st>>>(nF, S.cutF.p, S.grad.p, S.U.p, S.F2.p, length, wI * wI, wC * wC, S.Fsi.p);
        c->kernels += 3;
        MTK_CUDA_TRY(cudaGetLastError());
        stt->lm_iterations += 2;
    }
    // ================= seamless rounding loop (iter_rounding.h:99-109) ==========================
    // SI: wInteg = 1, wClose = 0.01, wConst = 1e5; X2F_si = length * G2 * fullx2N * UFull.
    const double scale_si = length * length, shift_si = 0.01 * 0.01;
    // SI constraints start empty (the NI anchor is not an SI constraint)
    Qrows.clear(); Arows.clear(); Avals.clear();
    std::fill(S.h_fixy.begin(), S.h_fixy.end(), 0);
    S.kq = 0;
    std::vector<int> leftv;
    const bool roundSeams = d->roundSeams != 0;
    bool roundedSingulars = false;
    if (roundSeams) leftv.assign(d->integerIdcs, d->integerIdcs + d->nInteger);
    else leftv.assign(d->singularIdcs, d->singularIdcs + d->nSingular);
    bool rounded = false;
    double min_margin = 1e300;
    std::vector<double> h_arg(6);
    bool constraints_dirty = true;
    while (!leftv.empty()) {
        // ---- initFixedIndices: argmin |X - round X| over leftIdcs (FP64 on the device)
        MTK_CUDA_TRY(cudaMemcpyAsync(S.left.p, leftv.data(), sizeof(int) * leftv.size(), cudaMemcpyHostToDevice, st));
        round_argmin<<<1, kStream, 0, st>>>((int)leftv.size(), S.left.p, S.d_full2y.p, S.d_full2j.p, nY, nZ, S.Us.p, S.xs.p,
                                           c->scalars);
        c->kernels++;
        MTK_CUDA_TRY(cudaMemcpyAsync(h_arg.data(), c->scalars, 6 * sizeof(double), cudaMemcpyDeviceToHost, st));
        MTK_CUDA_TRY(cudaStreamSynchronize(st));
        const int k = (int)h_arg[0];
        const double mind = h_arg[1];
        if (Igm::debug()) fprintf(stderr, "[round] left=%zu pick=%d full=%d X=%.9f d=%.3e second=%.3e\n", leftv.size(), k, leftv[k], h_arg[2], mind, h_arg[3]);
        if (h_arg[3] < 1e299) min_margin = std::min(min_margin, h_arg[3] - mind);
        if ((int)h_arg[4] != k) {   // a tie resolved by position, not by the strict '<'
            if (mind > 10e-7) {     // among fractional candidates
                stt->strict_order_differs++;
                stt->strict_order_gap = std::max(stt->strict_order_gap, std::fabs(h_arg[2] - std::round(h_arg[2])) - h_arg[5]);
            } else {                // among already-integral candidates (no re-solve follows)
                stt->integral_order_differs++;
            }
        }
        const int idx = leftv[k];
        const int ival = (int)std::round(h_arg[2]);
        if (fix_order && nfix < nLeftCap) { fix_order[nfix] = idx; if (fix_vals) fix_vals[nfix] = ival; }
        nfix++;
        leftv.erase(leftv.begin() + k);
        if (leftv.empty() && !roundSeams && !roundedSingulars) {
            leftv.assign(d->integerIdcs, d->integerIdcs + d->nInteger);
            roundedSingulars = true;
        }
        // prev = xs (xPrev = xCurr) before the constraint moves xs
        MTK_CUDA_TRY(cudaMemcpyAsync(S.prev.p, S.xs.p, sizeof(double) * nRed, cudaMemcpyDeviceToDevice, st));
        MTK_TRY(add_constraint(idx, (double)ival));
        constraints_dirty = true;
        if (!(mind > 10e-7)) continue;    // already integral: no re-solve
        rounded = true;
        // ---- LM solve of the SI objective: one exact constrained Gauss-Newton step
        MTK_CUDA_TRY(cudaEventRecord(c->ev_a, st));
        if (constraints_dirty) { MTK_TRY(upload_constraints(scale_si, shift_si)); constraints_dirty = false; }
        // b = length UFull^T W^T hb(F_si) + shift * xPrev
        MTK_TRY(S.build_rhs(S.Fsi.p, length, shift_si, S.prev.p, S.bsys.p));
        int s = S.solve(scale_si, shift_si, S.bsys.p, S.xs.p, o, stt, &rel);
        if (s != MTK_OK) { status = s; break; }
        stt->resolves++;
        stt->lm_iterations += 2;
        MTK_CUDA_TRY(cudaEventRecord(c->ev_b, st));
        MTK_CUDA_TRY(cudaStreamSynchronize(st));
        cudaEventElapsedTime(&ms, c->ev_a, c->ev_b);
        stt->ms_rounding += ms;
        // ---- post_checking: every fixed value within 1e-6 of an integer
        double worst = 0;
        const int nchk = fix_order ? std::min(nfix, nLeftCap) : 0;
        if (nchk > 0) {   // all fixed values in one kernel and one copy
            MTK_CUDA_TRY(cudaMemcpyAsync(fixd.p, fix_order, sizeof(int) * nchk, cudaMemcpyHostToDevice, st));
            fixed_values<<<G, kStream, 0, st>>>(nchk, fixd.p, S.d_full2y.p, S.d_full2j.p, nY, nZ, S.Us.p, S.xs.p, fixv.p);
            c->kernels++;
            MTK_CUDA_TRY(cudaGetLastError());
            std::vector<double> hv(nchk);
            MTK_CUDA_TRY(cudaMemcpyAsync(hv.data(), fixv.p, sizeof(double) * nchk, cudaMemcpyDeviceToHost, st));
            MTK_CUDA_TRY(cudaStreamSynchronize(st));
            for (double v : hv) worst = std::max(worst, std::fabs(v - std::round(v)));
        }
        if (worst > 10e-7) { status = MTK_ERR_ROUNDING; break; }
    }
    stt->min_order_margin = std::min(stt->min_order_margin == 0 ? 1e300 : stt->min_order_margin, min_margin);
    if (!rounded) return finish(x0red.p);
    return finish(S.xs.p);
}
}  // namespace

extern "C" int mtk_iterative_rounding(mtk_ctx* c, const mtk_igm_desc* d, const mtk_solve_opts* opts_in, double* fullx,
                                      int32_t* fix_order, int32_t* fix_vals, int32_t* n_fixed, double* x_naive,
                                      mtk_stats* stats) {
    return igm_run(c, d, opts_in, fullx, fix_order, fix_vals, n_fixed, x_naive, stats, nullptr);
}

extern "C" int mtk_size_field_position_partials(mtk_ctx* c, const mtk_igm_desc* d, const mtk_solve_opts* opts,
                                                int32_t nV, const int32_t* F, const double* s, double mu, double* loss,
                                                double* grad_s, double* fullx, double* dgx, double* dgy, double* dphi,
                                                double* dlength, mtk_stats* stats) {
    if (!c || !d || !F || !s || !loss || !grad_s || !fullx || !dgx || !dgy || !dphi || !dlength || nV <= 0 || !(mu >= 0))
        return MTK_ERR_BAD_INPUT;
    for (int64_t i = 0; i < 3 * (int64_t)d->nF; i++)
        if (F[i] < 0 || F[i] >= nV) return MTK_ERR_BAD_INPUT;
    SizeFieldJob job{nV, F, s, nullptr, mu, loss, grad_s, dgx, dgy, dphi, dlength};
    return igm_run(c, d, opts, fullx, nullptr, nullptr, nullptr, nullptr, stats, &job);
}

extern "C" int mtk_size_field_gradient(mtk_ctx* c, const mtk_igm_desc* d, const mtk_solve_opts* opts, int32_t nV,
                                       const int32_t* F, const double* s, const double* T, double mu, double* loss,
                                       double* grad_s, double* fullx, mtk_stats* stats) {
    if (!c || !d || !F || !s || !loss || !grad_s || !fullx || nV <= 0 || !(mu >= 0)) return MTK_ERR_BAD_INPUT;
    for (int64_t i = 0; i < 3 * (int64_t)d->nF; i++)
        if (F[i] < 0 || F[i] >= nV) return MTK_ERR_BAD_INPUT;
    SizeFieldJob job{nV, F, s, T, mu, loss, grad_s};
    return igm_run(c, d, opts, fullx, nullptr, nullptr, nullptr, nullptr, stats, &job);
}
