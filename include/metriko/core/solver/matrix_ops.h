//
// metriko-gb300: small dense helpers of the constraint reduction.
//
// reduce_to_linearly_independent replaces metriko include/metriko/core/solver/matrix_ops.h:12-28.
// The reference keeps the rows picked by Eigen SparseQR<COLAMD>'s column pivoting of C^T; this
// build keeps the first maximal independent subset in row order (greedy two-pass Gram-Schmidt).
// Both span the same row space, so the constraint null space is identical.
//
// fullpiv_kernel restates Eigen FullPivLU::kernel() as used by NaiveIntegration
// (iter_rounding_init.h:226-228): LU with complete pivoting (pivot = first maximum |a_ij| of the
// trailing block in column-major order), rank threshold eps * min(rows, cols) * max pivot,
// kernel basis = identity on the free columns and -U11^-1 U12 on the pivot columns.
//
#ifndef METRIKO_SOLVER_COMMON_H
#define METRIKO_SOLVER_COMMON_H
#include <limits>

#include "metriko/core/common/typedef.h"

namespace metriko {
    inline std::vector<int> independent_rows(const MatXd& C, double tol = 1e-9) {
        std::vector<std::vector<double>> basis;
        std::vector<int> keep;
        for (int i = 0; i < C.rows(); i++) {
            std::vector<double> r(C.row(i), C.row(i) + C.cols());
            double n0 = 0;
            for (double v : r) n0 += v * v;
            n0 = std::sqrt(n0);
            if (n0 == 0) continue;
            for (int pass = 0; pass < 2; pass++)
                for (auto& q : basis) {
                    double d = 0;
                    for (size_t j = 0; j < r.size(); j++) d += q[j] * r[j];
                    for (size_t j = 0; j < r.size(); j++) r[j] -= d * q[j];
                }
            double n = 0;
            for (double v : r) n += v * v;
            n = std::sqrt(n);
            if (n > tol * n0) {
                for (double& v : r) v /= n;
                basis.push_back(std::move(r));
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
        for (int k = 0; k < size; k++) {
            double best = -1;
            int pr = k, pc = k;
            for (int j = k; j < cols; j++)
                for (int i = k; i < rows; i++) {
                    double a = std::fabs(A(i, j));
                    if (a > best) { best = a; pr = i; pc = j; }
                }
            if (best == 0.0) { nzp = k; break; }
            maxpivot = std::max(maxpivot, best);
            if (pr != k) for (int j = 0; j < cols; j++) std::swap(A(k, j), A(pr, j));
            if (pc != k) { for (int i = 0; i < rows; i++) std::swap(A(i, k), A(i, pc)); std::swap(colq[k], colq[pc]); }
            if (k < rows - 1) for (int i = k + 1; i < rows; i++) A(i, k) /= A(k, k);
            if (k < size - 1)
                for (int i = k + 1; i < rows; i++) {
                    double l = A(i, k);
                    for (int j = k + 1; j < cols; j++) A(i, j) -= l * A(k, j);
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
        // back substitution U11 X = U12, stored in the trailing columns of U
        for (int i = rank - 1; i >= 0; i--)
            for (int j = 0; j < dimker; j++) {
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
