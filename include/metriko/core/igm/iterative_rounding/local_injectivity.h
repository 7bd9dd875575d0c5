//
// Restates parts of metriko (https://github.com/komietty/metriko),
// Copyright (C) 2025 Saki Komikado <komietty@gmail.com>.
// This Source Code Form is subject to the terms of the Mozilla Public License v.2.0
// (https://mozilla.org/MPL/2.0/).
//
// metriko-gb300: iterative rounding with localInjectivity = true.
//
// Replaces, for RosyParameterization::localInjectivity, the damped Levenberg-Marquardt path of
// iterative_rounding (core/igm/iterative_rounding/iter_rounding.h:57-109): NaiveIntegration's
// LM (iter_rounding_init.h:26-72, weights wInteg = wConst = 1e4, wClose = 1) with the barrier
// rows of InjectiveBarrier (injective_barrier.h:18-106, wBarrier = 1e-4, the Jacobian scaled by
// wInteg * wClose as iter_rounding_common.h:77-79 does) and the stop at the first locally
// injective map (post_iteration, parameterization_integ.ipp:46-63); then SeamlessIntegration's
// greedy rounding (iter_rounding_loop.h:29-100, weights 1 / 1e5 / 0.01) with one damped LM per
// rounded variable.  The LM is the reference's LMSolver + DiagonalDamping
// (core/solver/levenberg_marquardt.h:13-231): the normal matrix J^T J + lambda diag(J^T J),
// lambda from 0.01, divided by 10 after a step that lowers the energy (to a finite value),
// multiplied by 10 otherwise.
//
// The penalty formulation is kept (fixed variables are rows of weight wConst, not eliminated),
// because the damping also damps those rows.  The normal equations are formed in the reduced
// coordinates xs = [y ; z] of the constraint kernel (UFull): G = G2 * fullx2Nfunc * UFull maps xs
// to the per-face gradients of the N functions (2 N per face).  In the naive integration the
// face-field unknowns f (2 N per face) are eliminated face by face (an 8 x 8 solve each for N = 4):
// with A_f the (f, f) block of the damped normal matrix,
//   S = sum_f G_f^T W_f G_f + lambda wInteg^2 length^2 diag(G^T G) + wConst^2 (C^T C + lambda diag(C^T C)),
//   W_f = wInteg^2 length^2 A_f^-1 (A_f - wInteg^2 I)      (no cancellation: A_f - wInteg^2 I is formed directly),
// and the face unknowns follow back from their 8 x 8 blocks.  The seamless systems are
// S = sum_f G_f^T W_f G_f + wClose^2 I + wConst^2 C^T C, W_f = length^2 (wInteg^2 I + wBarrier^2 B_f^T B_f),
// damped on their diagonal.  The linear solves go through a caller-supplied solver (the device
// PCG on assembled CSR matrices, mtk_csr_pcg, in the product; the role of the reference's
// CholeskyWrapper).
//
#ifndef METRIKO_LOCAL_INJECTIVITY_H
#define METRIKO_LOCAL_INJECTIVITY_H
#include <algorithm>
#include <cmath>
#include <functional>
#include <limits>
#include <tuple>
#include <stdexcept>
#include <utility>
#include <vector>

#include "metriko/core/common/typedef.h"

namespace metriko {
namespace li {
    constexpr double kInf = std::numeric_limits<double>::infinity();
    constexpr double kNIwInteg = 10e3, kNIwConst = 10e3, kNIwClose = 1.0;   // iter_rounding_init.h:87
    constexpr double kSIwInteg = 1.0, kSIwConst = 10e4, kSIwClose = 0.01;   // iter_rounding_loop.h:109
    constexpr double kwBarrier = 1e-4;
    constexpr double kTieWindow = 1e-8;   // greedy rounding ties (the same rule as mtk_iterative_rounding)

    // Symmetric positive-definite solve S x = b; S holds both triangles.  Returns false when the
    // solve fails (the LM then stops, as on a failed factorisation).
    using Solve = std::function<bool(const SprsD& S, const std::vector<double>& b, std::vector<double>& x)>;

    struct System {
        int N = 4, n = 2, nF = 0, nY = 0, nZ = 0, nred = 0, nfull = 0, nCut = 0;
        double length = 0;
        SprsD G;                          // 2 N nF x nred: per-face function gradients (face frame)
        std::vector<double> F2;           // 2 N nF: the target field, face frame
        std::vector<int> full2y, jslot;   // UFull: free variable -> y, constrained variable -> USmall row
        MatXd USmall;                     // nJ x nZ
        const SprsD* fullx2N = nullptr;   // N nCut x nfull
        MatXi cutF;                       // nF x 3
        std::vector<int> fixedIdcs;       // naive anchor (full variables)
        std::vector<double> fixedVals;
        std::vector<int> singularIdcs, integerIdcs;
        bool roundSeams = false;

        // the row of UFull for full variable i, as (reduced column, value)
        void ufull_row(int i, std::vector<std::pair<int, double>>& out) const {
            out.clear();
            if (full2y[i] >= 0) { out.emplace_back(full2y[i], 1.0); return; }
            const int s = jslot[i];
            for (int z = 0; z < nZ; z++) if (USmall(s, z) != 0) out.emplace_back(nY + z, USmall(s, z));
        }
        std::vector<double> ufull_times(const std::vector<double>& xs) const {
            std::vector<double> X(nfull, 0.0);
            METRIKO_PARALLEL_FOR
            for (int i = 0; i < nfull; i++) {
                if (full2y[i] >= 0) { X[i] = xs[full2y[i]]; continue; }
                double s = 0;
                for (int z = 0; z < nZ; z++) s += USmall(jslot[i], z) * xs[nY + z];
                X[i] = s;
            }
            return X;
        }
        // rows of UFull at the given full variables, n_rows x nred
        SprsD rows_of(const std::vector<int>& idx) const {
            SprsD C(int(idx.size()), nred);
            std::vector<std::pair<int, double>> r;
            for (size_t k = 0; k < idx.size(); k++) {
                ufull_row(idx[k], r);
                std::sort(r.begin(), r.end());
                for (auto& e : r) { C.idx.push_back(e.first); C.val.push_back(e.second); }
                C.ptr[k + 1] = int(C.idx.size());
            }
            return C;
        }
    };

    // G = G2 fullx2Nfunc UFull with G2 of parameterization_integ.ipp:11-24: corner a of cut face f
    // (the tail of its a-th halfedge, F(f, a)) has the gradient g_a = n x (P_{a+2} - P_{a+1}) / (2 A),
    // entries (g_a . bX, g_a . bY) in rows 2 N f + 2 k + {0, 1} for every function k.
    inline void build_gradients(System& s, const MatXd& cutV, const MatXd& faceNormal, const MatXd& faceBasisX,
                                const MatXd& faceBasisY, const VecXd& faceArea) {
        const int N = s.N, nF = s.nF;
        s.G = SprsD(2 * N * nF, s.nred);
        std::vector<std::vector<std::pair<int, double>>> rows(2 * size_t(N) * nF);
        METRIKO_PARALLEL_FOR
        for (int f = 0; f < nF; f++) {
            const Row3d n = row3(faceNormal, f), bx = row3(faceBasisX, f), by = row3(faceBasisY, f);
            const double a2 = faceArea[f] * 2;
            std::vector<std::pair<int, double>> ur;
            for (int a = 0; a < 3; a++) {
                const Row3d p1 = row3(cutV, s.cutF(f, (a + 1) % 3)), p2 = row3(cutV, s.cutF(f, (a + 2) % 3));
                const Row3d g = n.cross(p2 - p1) / a2;
                const double gx = g.dot(bx), gy = g.dot(by);
                const int cv = s.cutF(f, a);
                for (int k = 0; k < N; k++) {
                    const int r0 = N * cv + k;
                    for (int p = s.fullx2N->ptr[r0]; p < s.fullx2N->ptr[r0 + 1]; p++) {
                        const double w = s.fullx2N->val[p];
                        if (w == 0) continue;
                        s.ufull_row(s.fullx2N->idx[p], ur);
                        for (auto& e : ur) {
                            rows[2 * size_t(N) * f + 2 * k].emplace_back(e.first, gx * w * e.second);
                            rows[2 * size_t(N) * f + 2 * k + 1].emplace_back(e.first, gy * w * e.second);
                        }
                    }
                }
            }
        }
        for (size_t r = 0; r < rows.size(); r++) {
            auto& e = rows[r];
            std::sort(e.begin(), e.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
            for (size_t k = 0; k < e.size(); k++) {
                if (k > 0 && e[k].first == e[k - 1].first) { s.G.val.back() += e[k].second; continue; }
                s.G.idx.push_back(e[k].first);
                s.G.val.push_back(e[k].second);
            }
            s.G.ptr[r + 1] = int(s.G.idx.size());
        }
    }

    // InjectiveBarrier (injective_barrier.h:18-106) for the intrinsic field F2: per row k = N i + j
    // (vectors j and (j + 1) mod N of face i) fB = 1 / bar(r) - 1 with r the volume ratio of the
    // two vectors (infinite for r <= 0, 0 for r >= 1/2), der = d fB / d r (0 where |fB| < 1e-8,
    // infinite where fB is), and the row S = d r / d(v0, v1).
    struct Barrier {
        int N = 4, nF = 0;
        std::vector<double> V;
        void init(const std::vector<double>& F2, int N_, int nF_) {
            N = N_;
            nF = nF_;
            V.assign(size_t(N) * nF, 0.0);
            for (int i = 0; i < nF; i++)
                for (int j = 0; j < N; j++) {
                    const double* a = &F2[2 * size_t(N) * i + 2 * j];
                    const double* b = &F2[2 * size_t(N) * i + 2 * ((j + 1) % N)];
                    V[size_t(N) * i + j] = std::sqrt(a[0] * a[0] + a[1] * a[1]) * std::sqrt(b[0] * b[0] + b[1] * b[1]);
                }
        }
        void update(const double* field, bool upd, std::vector<double>& fB, std::vector<double>& der,
                    std::vector<double>& S) const {
            const double s = 0.5;
            const size_t nr = size_t(N) * nF;
            fB.assign(nr, 0.0);
            if (upd) { der.assign(nr, 0.0); S.assign(4 * nr, 0.0); }
            METRIKO_PARALLEL_FOR
            for (int i = 0; i < nF; i++)
                for (int j = 0; j < N; j++) {
                    const size_t k = size_t(N) * i + j;
                    const double* v0 = field + 2 * size_t(N) * i + 2 * j;
                    const double* v1 = field + 2 * size_t(N) * i + 2 * ((j + 1) % N);
                    const double v = V[k];
                    const double r = (v0[0] * v1[1] - v0[1] * v1[0]) / v;
                    const double q = r / s;
                    const double bar = q * q * q - 3 * (q * q) + 3 * r / s;
                    double b2 = 1.0 / bar - 1.0;
                    if (r <= 0) b2 = kInf;
                    if (r >= s) b2 = 0.0;
                    fB[k] = b2;
                    if (!upd) continue;
                    double d = 3.0 * (r * r / (s * s * s)) - 6.0 * (r / (s * s)) + 3.0 / s;
                    if (r <= 0) d = kInf;
                    if (r >= s) d = 0.0;
                    double dd = -d / (bar * bar);
                    if (std::abs(b2) < 10e-9) dd = 0.0;
                    else if (b2 == kInf) dd = kInf;
                    der[k] = dd;
                    S[4 * k] = v1[1] / v;
                    S[4 * k + 1] = -v1[0] / v;
                    S[4 * k + 2] = -v0[1] / v;
                    S[4 * k + 3] = v0[0] / v;
                }
        }
    };

    // column-summed squares of a CSR matrix (diag(A^T A))
    inline std::vector<double> col_sumsq(const SprsD& A) {
        std::vector<double> d(A.nc, 0.0);
        for (int i = 0; i < A.nr; i++) for (int p = A.ptr[i]; p < A.ptr[i + 1]; p++) d[A.idx[p]] += A.val[p] * A.val[p];
        return d;
    }

    // 8 x 8 (M = 2N) symmetric positive-definite solve by Cholesky; false if not positive definite
    template <int M>
    inline bool chol_inplace(double (&A)[M][M]) {
        for (int j = 0; j < M; j++) {
            double d = A[j][j];
            for (int k = 0; k < j; k++) d -= A[j][k] * A[j][k];
            if (!(d > 0)) return false;
            d = std::sqrt(d);
            A[j][j] = d;
            for (int i = j + 1; i < M; i++) {
                double v = A[i][j];
                for (int k = 0; k < j; k++) v -= A[i][k] * A[j][k];
                A[i][j] = v / d;
            }
        }
        return true;
    }
    template <int M>
    inline void chol_solve(const double (&L)[M][M], double* x) {
        for (int i = 0; i < M; i++) {
            double v = x[i];
            for (int k = 0; k < i; k++) v -= L[i][k] * x[k];
            x[i] = v / L[i][i];
        }
        for (int i = M - 1; i >= 0; i--) {
            double v = x[i];
            for (int k = i + 1; k < M; k++) v -= L[k][i] * x[k];
            x[i] = v / L[i][i];
        }
    }

    // Assembles S = sum_f G_f^T W_f G_f + diag, W_f (2N x 2N, row-major per face) given; the rows of G
    // of face f are 2 N f .. 2 N f + 2 N - 1.  Both triangles, columns ascending.
    inline SprsD assemble_gwg(const System& s, const std::vector<double>& W, const std::vector<double>& diag) {
        const int M = 2 * s.N, nred = s.nred;
        // per reduced column: the faces whose rows touch it
        std::vector<std::vector<int>> colf(nred);
        for (int f = 0; f < s.nF; f++)
            for (int r = M * f; r < M * f + M; r++)
                for (int p = s.G.ptr[r]; p < s.G.ptr[r + 1]; p++) {
                    auto& v = colf[s.G.idx[p]];
                    if (v.empty() || v.back() != f) v.push_back(f);
                }
        SprsD S(nred, nred);
        std::vector<std::vector<std::pair<int, double>>> rows(nred);
        METRIKO_PARALLEL_FOR
        for (int a = 0; a < nred; a++) {
            std::vector<std::pair<int, double>> e;
            for (int f : colf[a]) {
                // G_f(:, a) (M values) then (W_f G_f(:, a)) . G_f(:, b) for every b of the face
                double ga[16] = {0};
                for (int r = 0; r < M; r++)
                    for (int p = s.G.ptr[M * f + r]; p < s.G.ptr[M * f + r + 1]; p++)
                        if (s.G.idx[p] == a) ga[r] = s.G.val[p];
                double wg[16] = {0};
                for (int r = 0; r < M; r++) {
                    double v = 0;
                    for (int c = 0; c < M; c++) v += W[size_t(M) * M * f + size_t(M) * r + c] * ga[c];
                    wg[r] = v;
                }
                for (int r = 0; r < M; r++)
                    for (int p = s.G.ptr[M * f + r]; p < s.G.ptr[M * f + r + 1]; p++) e.emplace_back(s.G.idx[p], wg[r] * s.G.val[p]);
            }
            e.emplace_back(a, diag[a]);
            std::sort(e.begin(), e.end(), [](const auto& x, const auto& y) { return x.first < y.first; });
            std::vector<std::pair<int, double>> m;
            for (auto& x : e) {
                if (!m.empty() && m.back().first == x.first) m.back().second += x.second;
                else m.push_back(x);
            }
            rows[a] = std::move(m);
        }
        for (int a = 0; a < nred; a++) {
            for (auto& x : rows[a]) { S.idx.push_back(x.first); S.val.push_back(x.second); }
            S.ptr[a + 1] = int(S.idx.size());
        }
        return S;
    }

    inline void merge_into(SprsD& S, std::vector<std::vector<std::pair<int, double>>>& add);

    inline bool all_finite(const std::vector<double>& v) {
        for (double x : v) if (!std::isfinite(x)) return false;
        return true;
    }

    // The objective of one of the two LM problems: energy, gradient (-J^T E) and damped normal
    // equations; `solve_step` returns the LM direction.
    struct Problem {
        virtual ~Problem() = default;
        virtual double energy(const std::vector<double>& x) = 0;
        // linearise at x: the residuals and Jacobian data for rhs and the normal equations;
        // returns false when the Jacobian is not finite (an infinite barrier derivative)
        virtual bool linearize(const std::vector<double>& x) = 0;
        virtual double foo() const = 0;   // |J^T E|_inf at the linearisation point
        // direction of the damped normal equations at the linearisation point
        virtual bool direction(double lambda, const Solve& solve, std::vector<double>& d) = 0;
        virtual bool post_iteration(const std::vector<double>&) { return false; }
    };

    struct LMResult {
        bool flag = false;
        std::vector<double> x;
        double lambda = 0;
        int iterations = 0;
    };

    // levenberg_marquardt.h:140-231 with DiagonalDamping (levenberg_marquardt.h:13-88).
    inline LMResult lm_solve_damped(Problem& P, std::vector<double> x0, double lam, const Solve& solve, int max_iter,
                                    double func_tol, double foo_tol) {
        LMResult R;
        std::vector<double> prevx = x0, x = x0, d;
        bool finite = P.linearize(prevx);
        int it = 0;
        auto norm = [](const std::vector<double>& v) { double s = 0; for (double a : v) s += a * a; return std::sqrt(s); };
        while (true) {
            if (P.foo() < foo_tol) x = prevx;
            if (!finite || !P.direction(lam, solve, d)) { R.flag = false; R.x = x; R.lambda = lam; R.iterations = it; return R; }
            if (norm(d) < func_tol) { R.flag = true; R.x = prevx; R.lambda = lam; R.iterations = it; return R; }
            std::vector<double> trial(prevx.size());
            for (size_t i = 0; i < trial.size(); i++) trial[i] = prevx[i] + d[i];
            const double e_prev = P.energy(prevx), e_new = P.energy(trial);
            if (e_prev > e_new) {
                x = trial;
                if (std::abs(e_prev - e_new) < func_tol) { R.flag = false; R.x = x; R.lambda = lam; R.iterations = it; return R; }
            } else {
                x = prevx;
            }
            finite = P.linearize(x);
            // DiagonalDamping::update: the energies at prevx and prevx + direction
            lam = (e_prev > e_new && e_new != kInf) ? lam / 10.0 : lam * 10.0;
            if (P.post_iteration(x)) { R.flag = true; R.x = x; R.lambda = lam; R.iterations = it; return R; }
            it++;
            prevx = x;
            if (it > max_iter) { R.flag = false; R.x = x; R.lambda = lam; R.iterations = it; return R; }
        }
    }

    // NaiveIntegration with the barrier (iter_rounding_init.h:26-72, iter_rounding_common.h:60-94):
    // unknowns [xs (nred) ; f (2 N nF)].
    struct Naive : Problem {
        const System& s;
        const Barrier& bar;
        SprsD C;                      // UFull rows of the anchor
        std::vector<double> gg;       // diag(G^T G)
        std::vector<double> cc;       // diag(C^T C)
        std::function<bool(const std::vector<double>&)> injective;   // post_iteration check (null: none)
        // linearisation data
        std::vector<double> EI, EC, EK, EB, der, Srow;
        double foo_ = 0;
        const double wI = kNIwInteg, wC = kNIwClose, wK = kNIwConst, wB = kwBarrier;

        Naive(const System& s_, const Barrier& b_) : s(s_), bar(b_) {
            C = s.rows_of(s.fixedIdcs);
            gg = col_sumsq(s.G);
            cc = col_sumsq(C);
        }
        int nx() const { return s.nred; }
        int nf() const { return 2 * s.N * s.nF; }
        void residuals(const std::vector<double>& x, bool upd) {
            const int n2 = nf();
            std::vector<double> xs(x.begin(), x.begin() + nx());
            const double* f = x.data() + nx();
            const std::vector<double> Gx = s.G * xs;
            EI.assign(n2, 0.0);
            EC.assign(n2, 0.0);
            for (int i = 0; i < n2; i++) {
                EI[i] = (f[i] - s.length * Gx[i]) * wI;
                EC[i] = (f[i] - s.F2[i]) * wC;
            }
            const std::vector<double> Cx = C * xs;
            EK.assign(Cx.size(), 0.0);
            for (size_t i = 0; i < Cx.size(); i++) EK[i] = (Cx[i] - s.fixedVals[i]) * wK;
            std::vector<double> fB;
            bar.update(f, upd, fB, der, Srow);
            EB.assign(fB.size(), 0.0);
            for (size_t i = 0; i < fB.size(); i++) EB[i] = fB[i] * wB;
        }
        double energy(const std::vector<double>& x) override {
            std::vector<double> sEI, sEC, sEK, sEB, sd, sS;
            std::swap(sEI, EI); std::swap(sEC, EC); std::swap(sEK, EK); std::swap(sEB, EB); std::swap(sd, der); std::swap(sS, Srow);
            residuals(x, false);
            double e = 0;
            for (double v : EI) e += v * v;
            for (double v : EC) e += v * v;
            for (double v : EK) e += v * v;
            for (double v : EB) e += v * v;
            std::swap(sEI, EI); std::swap(sEC, EC); std::swap(sEK, EK); std::swap(sEB, EB); std::swap(sd, der); std::swap(sS, Srow);
            return e;
        }
        // the barrier Jacobian row k on the face unknowns: wInteg * wClose * der_k * S_k at the
        // two vectors' four entries (iter_rounding_common.h:77-79 scales it by wInteg)
        bool linearize(const std::vector<double>& x) override {
            residuals(x, true);
            if (!all_finite(der)) return false;
            // rhs = -J^T E: x part wI length G^T EI - wK C^T EK; f part -(wI EI + wC EC + JB^T EB)
            foo_ = 0;
            std::vector<double> rx = gT_times(EI);
            for (auto& v : rx) v *= wI * s.length;
            std::vector<double> ck = ct_times(EK);
            for (int i = 0; i < nx(); i++) rx[i] -= wK * ck[i];
            std::vector<double> rf = rf_vector();
            for (double v : rx) foo_ = std::max(foo_, std::abs(v));
            for (double v : rf) foo_ = std::max(foo_, std::abs(v));
            return std::isfinite(foo_);
        }
        double foo() const override { return foo_; }
        std::vector<double> gT_times(const std::vector<double>& v) const {
            std::vector<double> o(nx(), 0.0);
            for (int r = 0; r < s.G.nr; r++) for (int p = s.G.ptr[r]; p < s.G.ptr[r + 1]; p++) o[s.G.idx[p]] += s.G.val[p] * v[r];
            return o;
        }
        std::vector<double> ct_times(const std::vector<double>& v) const {
            std::vector<double> o(nx(), 0.0);
            for (int r = 0; r < C.nr; r++) for (int p = C.ptr[r]; p < C.ptr[r + 1]; p++) o[C.idx[p]] += C.val[p] * v[r];
            return o;
        }
        // JB_f (N x 2N) of face i
        void jb(int i, double (&J)[8][8]) const {
            const int N = s.N;
            for (int j = 0; j < N; j++) for (int c = 0; c < 2 * N; c++) J[j][c] = 0;
            for (int j = 0; j < N; j++) {
                const size_t k = size_t(N) * i + j;
                const double w = wI * wC * der[k];
                const int c0 = 2 * j, c1 = 2 * ((j + 1) % N);
                J[j][c0] += w * Srow[4 * k];
                J[j][c0 + 1] += w * Srow[4 * k + 1];
                J[j][c1] += w * Srow[4 * k + 2];
                J[j][c1 + 1] += w * Srow[4 * k + 3];
            }
        }
        std::vector<double> rf_vector() const {
            const int N = s.N, M = 2 * N;
            std::vector<double> rf(nf(), 0.0);
            for (int i = 0; i < s.nF; i++) {
                double J[8][8];
                jb(i, J);
                for (int c = 0; c < M; c++) {
                    double v = wI * EI[M * i + c] + wC * EC[M * i + c];
                    for (int j = 0; j < N; j++) v += J[j][c] * EB[size_t(N) * i + j];
                    rf[M * i + c] = -v;
                }
            }
            return rf;
        }
        bool direction(double lam, const Solve& solve, std::vector<double>& d) override {
            const int N = s.N, M = 2 * N, nF = s.nF;
            if (M != 8) throw std::invalid_argument("localInjectivity: N = 4 only");
            const double wI2 = wI * wI, wC2 = wC * wC, L2 = s.length * s.length;
            std::vector<double> W(size_t(M) * M * nF);
            std::vector<double> Ainv_rf(nf());   // A_f^-1 r_f per face
            std::vector<double> Lf(size_t(M) * M * nF);   // Cholesky factors of A_f
            const std::vector<double> rf = rf_vector();
            bool ok = true;
            for (int i = 0; i < nF && ok; i++) {
                double J[8][8];
                jb(i, J);
                double B[8][8];
                for (int a = 0; a < M; a++)
                    for (int b = 0; b < M; b++) {
                        double v = 0;
                        for (int j = 0; j < N; j++) v += J[j][a] * J[j][b];
                        B[a][b] = v;
                    }
                double A[8][8], Am[8][8];   // A_f and A_f - wI^2 I
                for (int a = 0; a < M; a++)
                    for (int b = 0; b < M; b++) {
                        const double damp = a == b ? lam * B[a][a] : 0.0;
                        A[a][b] = B[a][b] + damp + (a == b ? (1 + lam) * (wI2 + wC2) : 0.0);
                        Am[a][b] = B[a][b] + damp + (a == b ? lam * (wI2 + wC2) + wC2 : 0.0);
                    }
                double Lc[8][8];
                for (int a = 0; a < M; a++) for (int b = 0; b < M; b++) Lc[a][b] = A[a][b];
                if (!chol_inplace<8>(Lc)) { ok = false; break; }
                for (int a = 0; a < M; a++) for (int b = 0; b < M; b++) Lf[size_t(M) * M * i + M * a + b] = Lc[a][b];
                // W_f = wI^2 L2 A^-1 Am (columns of Am solved)
                for (int b = 0; b < M; b++) {
                    double col[8];
                    for (int a = 0; a < M; a++) col[a] = Am[a][b];
                    chol_solve<8>(Lc, col);
                    for (int a = 0; a < M; a++) W[size_t(M) * M * i + M * a + b] = wI2 * L2 * col[a];
                }
                // symmetrise (A^-1 Am is symmetric in exact arithmetic)
                for (int a = 0; a < M; a++)
                    for (int b = a + 1; b < M; b++) {
                        double& x1 = W[size_t(M) * M * i + M * a + b];
                        double& x2 = W[size_t(M) * M * i + M * b + a];
                        const double m = 0.5 * (x1 + x2);
                        x1 = m;
                        x2 = m;
                    }
                double v[8];
                for (int a = 0; a < M; a++) v[a] = rf[M * i + a];
                chol_solve<8>(Lc, v);
                for (int a = 0; a < M; a++) Ainv_rf[M * i + a] = v[a];
            }
            if (!ok || !all_finite(W)) return false;
            // diagonal: lambda wI^2 L2 diag(G^T G) + wK^2 (1 + lambda) diag(C^T C) (C^T C's off-diagonals below)
            std::vector<double> dg(nx());
            for (int a = 0; a < nx(); a++) dg[a] = lam * wI2 * L2 * gg[a];
            SprsD S = assemble_gwg(s, W, dg);
            // + wK^2 (C^T C + lambda diag(C^T C))
            add_ctc(S, wK * wK, lam);
            // rhs_x = r_x + wI^2 length G^T A^-1 r_f
            std::vector<double> rx = gT_times(EI);
            for (auto& q : rx) q *= wI * s.length;
            const std::vector<double> ck = ct_times(EK);
            const std::vector<double> ga = gT_times(Ainv_rf);
            std::vector<double> rhs(nx());
            for (int a = 0; a < nx(); a++) rhs[a] = rx[a] - wK * ck[a] + wI2 * s.length * ga[a];
            std::vector<double> dx;
            if (!solve(S, rhs, dx)) return false;
            // d_f = A_f^-1 (r_f + wI^2 length G_f dx)
            const std::vector<double> Gdx = s.G * dx;
            d.assign(nx() + nf(), 0.0);
            for (int a = 0; a < nx(); a++) d[a] = dx[a];
            for (int i = 0; i < nF; i++) {
                double Lc[8][8], v[8];
                for (int a = 0; a < M; a++) for (int b = 0; b < M; b++) Lc[a][b] = Lf[size_t(M) * M * i + M * a + b];
                for (int a = 0; a < M; a++) v[a] = rf[M * i + a] + wI2 * s.length * Gdx[M * i + a];
                chol_solve<8>(Lc, v);
                for (int a = 0; a < M; a++) d[nx() + M * i + a] = v[a];
            }
            return true;
        }
        // S += w (C^T C + lambda diag(C^T C)), entries merged into S's pattern (new ones inserted)
        void add_ctc(SprsD& S, double w, double lam) const {
            std::vector<std::vector<std::pair<int, double>>> add(nx());
            for (int r = 0; r < C.nr; r++)
                for (int p = C.ptr[r]; p < C.ptr[r + 1]; p++)
                    for (int q = C.ptr[r]; q < C.ptr[r + 1]; q++) add[C.idx[p]].emplace_back(C.idx[q], w * C.val[p] * C.val[q]);
            for (int a = 0; a < nx(); a++) if (cc[a] != 0) add[a].emplace_back(a, w * lam * cc[a]);
            merge_into(S, add);
        }
        bool post_iteration(const std::vector<double>& x) override {
            if (!injective) return false;
            return injective(std::vector<double>(x.begin(), x.begin() + nx()));
        }
    };

    // merges extra entries (per row, any order, duplicates summed) into a CSR matrix
    inline void merge_into(SprsD& S, std::vector<std::vector<std::pair<int, double>>>& add) {
        SprsD O(S.nr, S.nc);
        for (int a = 0; a < S.nr; a++) {
            auto& e = add[a];
            for (int p = S.ptr[a]; p < S.ptr[a + 1]; p++) e.emplace_back(S.idx[p], S.val[p]);
            std::sort(e.begin(), e.end(), [](const auto& x, const auto& y) { return x.first < y.first; });
            for (size_t k = 0; k < e.size(); k++) {
                if (k > 0 && e[k].first == e[k - 1].first) { O.val.back() += e[k].second; continue; }
                O.idx.push_back(e[k].first);
                O.val.push_back(e[k].second);
            }
            O.ptr[a + 1] = int(O.idx.size());
        }
        S = std::move(O);
    }

    // SeamlessIntegration with the barrier (iter_rounding_loop.h:29-100, iter_rounding_common.h:60-94)
    struct Seamless : Problem {
        const System& s;
        const Barrier& bar;
        std::vector<double> F2t;     // target: the naive LM's face field
        std::vector<double> xPrev, xCurr, xInit;
        std::vector<int> leftIdcs, fixedIdcs, fixedVals;
        bool roundedSingulars = false;
        SprsD C;
        std::vector<double> EI, EC, EK, EB, der, Srow, field;
        double foo_ = 0;
        const double wI = kSIwInteg, wC = kSIwClose, wK = kSIwConst, wB = kwBarrier;
        int strict_differs = 0;

        Seamless(const System& s_, const Barrier& b_, std::vector<double> xinit, std::vector<double> F2_)
            : s(s_), bar(b_), F2t(std::move(F2_)), xPrev(xinit), xCurr(xinit), xInit(xinit) {
            leftIdcs = s.roundSeams ? s.integerIdcs : s.singularIdcs;
        }
        int nx() const { return s.nred; }
        // iter_rounding_loop.h:29-74 with the tie rule of mtk_iterative_rounding: distances within
        // 1e-6 count as 0 and the first candidate within kTieWindow of the smallest is taken
        bool init_fixed_indices() {
            xPrev = xCurr;
            const std::vector<double> X = s.ufull_times(xCurr);
            double dmin = kInf;
            std::vector<double> dist(leftIdcs.size());
            for (size_t i = 0; i < leftIdcs.size(); i++) {
                const double v = X[leftIdcs[i]];
                double dd = std::fabs(v - std::round(v));
                if (dd <= 10e-7) dd = 0;
                dist[i] = dd;
                dmin = std::min(dmin, dd);
            }
            size_t k = 0;
            while (k < dist.size() && !(dist[k] <= dmin + kTieWindow)) k++;
            const int idx = leftIdcs[k];
            fixedIdcs.push_back(idx);
            fixedVals.push_back(int(std::round(X[idx])));
            leftIdcs.erase(leftIdcs.begin() + k);
            if (leftIdcs.empty() && !s.roundSeams && !roundedSingulars) {
                leftIdcs = s.integerIdcs;
                roundedSingulars = true;
            }
            C = s.rows_of(fixedIdcs);
            return dist[k] > 10e-7;
        }
        void residuals(const std::vector<double>& xs, bool upd) {
            const int n2 = 2 * s.N * s.nF;
            field = s.G * xs;
            for (auto& v : field) v *= s.length;
            EI.assign(n2, 0.0);
            for (int i = 0; i < n2; i++) EI[i] = (field[i] - F2t[i]) * wI;
            EC.assign(nx(), 0.0);
            for (int i = 0; i < nx(); i++) EC[i] = (xs[i] - xPrev[i]) * wC;
            const std::vector<double> Cx = C * xs;
            EK.assign(Cx.size(), 0.0);
            for (size_t i = 0; i < Cx.size(); i++) EK[i] = (Cx[i] - fixedVals[i]) * wK;
            std::vector<double> fB;
            bar.update(field.data(), upd, fB, der, Srow);
            EB.assign(fB.size(), 0.0);
            for (size_t i = 0; i < fB.size(); i++) EB[i] = fB[i] * wB;
        }
        double energy(const std::vector<double>& x) override {
            auto keep = std::make_tuple(EI, EC, EK, EB, der, Srow, field);
            residuals(x, false);
            double e = 0;
            for (double v : EI) e += v * v;
            for (double v : EC) e += v * v;
            for (double v : EK) e += v * v;
            for (double v : EB) e += v * v;
            std::tie(EI, EC, EK, EB, der, Srow, field) = keep;
            return e;
        }
        // the barrier Jacobian of face i on its field entries: wBarrier der_k S_k (then length G)
        void jb(int i, double (&J)[8][8]) const {
            const int N = s.N;
            for (int j = 0; j < N; j++) for (int c = 0; c < 2 * N; c++) J[j][c] = 0;
            for (int j = 0; j < N; j++) {
                const size_t k = size_t(N) * i + j;
                const double w = wB * der[k];
                const int c0 = 2 * j, c1 = 2 * ((j + 1) % N);
                J[j][c0] += w * Srow[4 * k];
                J[j][c0 + 1] += w * Srow[4 * k + 1];
                J[j][c1] += w * Srow[4 * k + 2];
                J[j][c1 + 1] += w * Srow[4 * k + 3];
            }
        }
        // -J^T E
        std::vector<double> rhs() const {
            const int N = s.N, M = 2 * N;
            std::vector<double> v(2 * size_t(N) * s.nF, 0.0);   // field-space part: wI EI + JB^T EB
            for (int i = 0; i < s.nF; i++) {
                double J[8][8];
                jb(i, J);
                for (int c = 0; c < M; c++) {
                    double a = wI * EI[M * i + c];
                    for (int j = 0; j < N; j++) a += J[j][c] * EB[size_t(N) * i + j];
                    v[M * i + c] = a;
                }
            }
            std::vector<double> r(nx(), 0.0);
            for (int row = 0; row < s.G.nr; row++)
                for (int p = s.G.ptr[row]; p < s.G.ptr[row + 1]; p++) r[s.G.idx[p]] += s.G.val[p] * v[row];
            for (int a = 0; a < nx(); a++) r[a] = -(s.length * r[a] + wC * EC[a]);
            for (int row = 0; row < C.nr; row++)
                for (int p = C.ptr[row]; p < C.ptr[row + 1]; p++) r[C.idx[p]] -= wK * C.val[p] * EK[row];
            return r;
        }
        bool linearize(const std::vector<double>& x) override {
            residuals(x, true);
            if (!all_finite(der)) return false;
            foo_ = 0;
            for (double v : rhs()) foo_ = std::max(foo_, std::abs(v));
            return std::isfinite(foo_);
        }
        double foo() const override { return foo_; }
        bool direction(double lam, const Solve& solve, std::vector<double>& d) override {
            const int N = s.N, M = 2 * N, nF = s.nF;
            const double L2 = s.length * s.length;
            std::vector<double> W(size_t(M) * M * nF);
            for (int i = 0; i < nF; i++) {
                double J[8][8];
                jb(i, J);
                for (int a = 0; a < M; a++)
                    for (int b = 0; b < M; b++) {
                        double v = 0;
                        for (int j = 0; j < N; j++) v += J[j][a] * J[j][b];
                        W[size_t(M) * M * i + M * a + b] = L2 * (v + (a == b ? wI * wI : 0.0));
                    }
            }
            if (!all_finite(W)) return false;
            std::vector<double> dg(nx(), wC * wC);
            SprsD S = assemble_gwg(s, W, dg);
            {   // + wK^2 C^T C
                std::vector<std::vector<std::pair<int, double>>> add(nx());
                for (int r = 0; r < C.nr; r++)
                    for (int p = C.ptr[r]; p < C.ptr[r + 1]; p++)
                        for (int q = C.ptr[r]; q < C.ptr[r + 1]; q++) add[C.idx[p]].emplace_back(C.idx[q], wK * wK * C.val[p] * C.val[q]);
                merge_into(S, add);
            }
            // + lambda diag(S) (DiagonalDamping: lambda times the diagonal of J^T J)
            for (int a = 0; a < S.nr; a++)
                for (int p = S.ptr[a]; p < S.ptr[a + 1]; p++)
                    if (S.idx[p] == a) S.val[p] *= (1.0 + lam);
            if (!all_finite(S.val)) return false;
            return solve(S, rhs(), d);
        }
        bool post_checking(const std::vector<double>& x) {
            const std::vector<double> X = s.ufull_times(x);
            double mx = -1;
            for (int i : fixedIdcs) mx = std::max(mx, std::abs(X[i] - std::round(X[i])));
            xCurr = x;
            xInit = x;
            xPrev = x;
            return mx <= 10e-7;
        }
    };

    struct Result {
        bool success = false;
        std::vector<double> fullx, x_ni;
        std::vector<int> fixOrder, fixVals;
        int ni_iterations = 0, resolves = 0;
    };

    // iter_rounding.h:57-111 with localInjectivity = true.  xs_naive: the naive integration in
    // reduced coordinates; injective(xs): the locally-injective check of the map UFull xs.
    inline Result iterative_rounding(const System& s, const std::vector<double>& xs_naive, bool seamless,
                                     const Solve& solve, const std::function<bool(const std::vector<double>&)>& injective) {
        Result R;
        Barrier bar;
        bar.init(s.F2, s.N, s.nF);
        Naive ni(s, bar);
        ni.injective = injective;
        std::vector<double> x0(xs_naive);
        x0.insert(x0.end(), s.F2.begin(), s.F2.end());
        LMResult lm = lm_solve_damped(ni, x0, 0.01, solve, 100, 10e-10, 10e-10);
        R.ni_iterations = lm.iterations;
        std::vector<double> X_(lm.x.begin(), lm.x.begin() + s.nred);
        std::vector<double> F2_(lm.x.begin() + s.nred, lm.x.end());
        R.x_ni = s.ufull_times(X_);
        if (!seamless) { R.success = true; R.fullx = R.x_ni; return R; }
        Seamless si(s, bar, X_, F2_);
        bool rounded = false;
        R.success = true;
        std::vector<double> xs;
        while (!si.leftIdcs.empty()) {
            if (!si.init_fixed_indices()) continue;
            rounded = true;
            LMResult r = lm_solve_damped(si, si.xInit, 0.01, solve, 100, 1e-7, 1e-7);
            xs = r.x;
            R.resolves++;
            if (!si.post_checking(xs)) { R.success = false; break; }
        }
        R.fullx = rounded ? s.ufull_times(xs) : s.ufull_times(xs_naive);
        R.fixOrder = si.fixedIdcs;
        R.fixVals = si.fixedVals;
        return R;
    }
}   // namespace li
}   // namespace metriko

#endif
