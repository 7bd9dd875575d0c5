//
// Restates parts of metriko (https://github.com/komietty/metriko),
// Copyright (C) 2025 Saki Komikado <komietty@gmail.com>, and the published algorithm of Eigen's
// FullPivLU::kernel().  This Source Code Form is subject to the terms of the Mozilla Public
// License v.2.0 (https://mozilla.org/MPL/2.0/).
//
// metriko-gb300: small dense helpers of the constraint reduction.
//
// reduce_to_linearly_independent replaces metriko include/metriko/core/solver/matrix_ops.h:12-28.
// The reference keeps the rows picked by Eigen SparseQR<COLAMD>'s column pivoting of C^T; this
// build keeps the first maximal independent subset in row order (greedy two-pass Gram-Schmidt).
// Both span the same row space, so the constraint null space is identical.
//
// fullpiv_kernel restates Eigen FullPivLU::kernel() as used by NaiveIntegration
// (iter_rounding_init.h:129-130): LU with complete pivoting (pivot = first maximum |a_ij| of the
// trailing block in column-major order), rank threshold eps * min(rows, cols) * max pivot,
// kernel basis = identity on the free columns and -U11^-1 U12 on the pivot columns.
//
#ifndef METRIKO_SOLVER_COMMON_H
#define METRIKO_SOLVER_COMMON_H
#include <limits>

#include "metriko/core/common/typedef.h"

namespace metriko {
    // Rows in order, each kept when its part orthogonal to the rows kept before (modified
    // Gram-Schmidt, two passes) keeps more than tol of its norm.  Each basis vector is walked over
    // its nonzero columns only: the skipped terms are exact zeros, so every nonzero value (and
    // every decision) is the one of the dense loops; constraint rows have a handful of nonzeros
    // and the basis vectors stay sparse.
    inline std::vector<int> independent_rows(const MatXd& C, double tol = 1e-9) {
        std::vector<std::vector<double>> basis;
        std::vector<std::vector<int>> support;
        std::vector<int> keep;
        for (int i = 0; i < C.rows(); i++) {
            std::vector<double> r(C.row(i), C.row(i) + C.cols());
            double n0 = 0;
            for (double v : r) n0 += v * v;
            n0 = std::sqrt(n0);
            if (n0 == 0) continue;
            for (int pass = 0; pass < 2; pass++)
                for (size_t b = 0; b < basis.size(); b++) {
                    const std::vector<double>& q = basis[b];
                    const std::vector<int>& nz = support[b];
                    double d = 0;
                    for (int j : nz) d += q[j] * r[j];
                    for (int j : nz) r[j] -= d * q[j];
                }
            double n = 0;
            for (double v : r) n += v * v;
            n = std::sqrt(n);
            if (n > tol * n0) {
                std::vector<int> nz;
                for (size_t j = 0; j < r.size(); j++) {
                    r[j] /= n;
                    if (r[j] != 0) nz.push_back(int(j));
                }
                basis.push_back(std::move(r));
                support.push_back(std::move(nz));
                keep.push_back(i);
            }
        }
        return keep;
    }

    // Structural entries (explicit zeros included, as Eigen keeps them after a product) decide
    // which columns take part; the dense work is done on those columns only.
    inline void reduce_to_linearly_independent(SprsD& mat) {
        if (mat.rows() == 0) return;
        std::vector<int> cols(mat.idx.begin(), mat.idx.end());
        std::sort(cols.begin(), cols.end());
        cols.erase(std::unique(cols.begin(), cols.end()), cols.end());
        MatXd dense(mat.rows(), int(cols.size()), 0.0);
        for (int i = 0; i < mat.rows(); i++)
            for (int p = mat.ptr[i]; p < mat.ptr[i + 1]; p++)
                dense(i, int(std::lower_bound(cols.begin(), cols.end(), mat.idx[p]) - cols.begin())) = mat.val[p];
        std::vector<int> keep = independent_rows(dense);
        std::vector<TripD> T;
        for (size_t j = 0; j < keep.size(); j++)
            for (int p = mat.ptr[keep[j]]; p < mat.ptr[keep[j] + 1]; p++) T.emplace_back(int(j), mat.idx[p], mat.val[p]);
        SprsD out(int(keep.size()), mat.cols());
        out.setFromTriplets(T.begin(), T.end());
        mat = std::move(out);
    }

    inline MatXd fullpiv_kernel(MatXd A) {
        const int rows = A.rows(), cols = A.cols(), size = std::min(rows, cols);
        std::vector<int> colq(cols);
        std::iota(colq.begin(), colq.end(), 0);
        double maxpivot = 0;
        int nzp = size;
        // The pivot is the first maximum of |a_ij| over the trailing block in column-major order,
        // i.e. the maximum with the smallest (column, row).  Rows are scanned in parallel (each
        // thread keeps its best under that order, the bests are merged under it too) and the
        // trailing rows are eliminated in parallel; every entry gets the arithmetic of the serial
        // loops, so the factors do not depend on the thread count.
        struct Piv { double a; int i, j; };
        auto better = [](const Piv& x, const Piv& y) {   // x before y
            if (x.a != y.a) return x.a > y.a;
            if (x.j != y.j) return x.j < y.j;
            return x.i < y.i;
        };
        for (int k = 0; k < size; k++) {
            Piv best{-1.0, k, k};
#if defined(_OPENMP)
            #pragma omp parallel if ((long long)(rows - k) * (cols - k) > 65536)
            {
                Piv mine{-1.0, k, k};
                #pragma omp for schedule(static) nowait
                for (int i = k; i < rows; i++)
                    for (int j = k; j < cols; j++) {
                        const Piv c{std::fabs(A(i, j)), i, j};
                        if (better(c, mine)) mine = c;
                    }
                #pragma omp critical(metriko_fullpiv)
                if (better(mine, best)) best = mine;
            }
#else
            for (int i = k; i < rows; i++)
                for (int j = k; j < cols; j++) {
                    const Piv c{std::fabs(A(i, j)), i, j};
                    if (better(c, best)) best = c;
                }
#endif
            const int pr = best.i, pc = best.j;
            if (best.a == 0.0) { nzp = k; break; }
            maxpivot = std::max(maxpivot, best.a);
            if (pr != k) for (int j = 0; j < cols; j++) std::swap(A(k, j), A(pr, j));
            if (pc != k) { for (int i = 0; i < rows; i++) std::swap(A(i, k), A(i, pc)); std::swap(colq[k], colq[pc]); }
            if (k < rows - 1) for (int i = k + 1; i < rows; i++) A(i, k) /= A(k, k);
            if (k < size - 1) {
                #pragma omp parallel for schedule(static) if ((long long)(rows - k) * (cols - k) > 65536)
                for (int i = k + 1; i < rows; i++) {
                    const double l = A(i, k);
                    for (int j = k + 1; j < cols; j++) A(i, j) -= l * A(k, j);
                }
            }
        }
        const double thr = std::numeric_limits<double>::epsilon() * size * maxpivot;
        std::vector<int> piv;
        for (int i = 0; i < nzp; i++) if (std::fabs(A(i, i)) > thr) piv.push_back(i);
        const int rank = int(piv.size()), dimker = cols - rank;
        MatXd K(cols, dimker, 0.0);
        if (dimker == 0) return K;
        MatXd U(rank, cols, 0.0);
        for (int i = 0; i < rank; i++) for (int j = i; j < cols; j++) U(i, j) = A(piv[i], j);
        for (int i = 0; i < rank; i++) if (piv[i] != i) for (int r = 0; r < rank; r++) std::swap(U(r, i), U(r, piv[i]));
        // back substitution U11 X = U12, stored in the trailing columns of U (columns independent)
        METRIKO_PARALLEL_FOR
        for (int j = 0; j < dimker; j++)
            for (int i = rank - 1; i >= 0; i--) {
                double s = U(i, rank + j);
                for (int k = i + 1; k < rank; k++) s -= U(i, k) * U(k, rank + j);
                U(i, rank + j) = s / U(i, i);
            }
        for (int i = rank - 1; i >= 0; i--) if (piv[i] != i) for (int r = 0; r < rank; r++) std::swap(U(r, i), U(r, piv[i]));
        for (int i = 0; i < rank; i++) for (int j = 0; j < dimker; j++) K(colq[i], j) = -U(i, rank + j);
        for (int k = 0; k < dimker; k++) K(colq[rank + k], k) = 1.0;
        return K;
    }
}

#endif
