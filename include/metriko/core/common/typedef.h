//
// metriko-gb300: minimal dense/sparse containers behind the reference's type names.
//
// The reference spells its host API with Eigen types (include/metriko/core/common/typedef.h:13-40
// in metriko): complex, Row3d, VecXi/VecXd/VecXc, MatXi/MatXd/MatXc, SprsD/SprsC, TripD/TripC.
// Eigen is not a dependency of this library, so the same names are provided here with only the
// operations the field + integration + IGM path needs.  Dense matrices are row-major.
//
#ifndef METRIKO_TYPEDEF_H
#define METRIKO_TYPEDEF_H
#include <algorithm>
#include <cassert>
#include <cmath>
#include <complex>
#include <cstdint>
#include <numeric>
#include <stdexcept>
#include <vector>

// Element-parallel host loops (each iteration writes only its own outputs, so results do not
// depend on the thread count).
#if defined(_OPENMP)
#define METRIKO_PARALLEL_FOR _Pragma("omp parallel for schedule(static)")
#else
#define METRIKO_PARALLEL_FOR
#endif

namespace metriko {
    constexpr double PI = 3.14159265358979323846;
    constexpr double TwoPI = 2 * PI;
    constexpr double EPS = 1e-9;
    using complex = std::complex<double>;

    // ------------------------------------------------------------------ fixed-size rows
    struct Row3d {
        double v[3] = {0, 0, 0};
        Row3d() = default;
        Row3d(double a, double b, double c) : v{a, b, c} {}
        double x() const { return v[0]; }
        double y() const { return v[1]; }
        double z() const { return v[2]; }
        double& operator[](int i) { return v[i]; }
        double operator[](int i) const { return v[i]; }
        Row3d operator+(const Row3d& o) const { return {v[0] + o.v[0], v[1] + o.v[1], v[2] + o.v[2]}; }
        Row3d operator-(const Row3d& o) const { return {v[0] - o.v[0], v[1] - o.v[1], v[2] - o.v[2]}; }
        Row3d operator-() const { return {-v[0], -v[1], -v[2]}; }
        Row3d operator*(double s) const { return {v[0] * s, v[1] * s, v[2] * s}; }
        Row3d operator/(double s) const { return {v[0] / s, v[1] / s, v[2] / s}; }
        Row3d& operator+=(const Row3d& o) { v[0] += o.v[0]; v[1] += o.v[1]; v[2] += o.v[2]; return *this; }
        double dot(const Row3d& o) const { return v[0] * o.v[0] + v[1] * o.v[1] + v[2] * o.v[2]; }
        Row3d cross(const Row3d& o) const {
            return {v[1] * o.v[2] - v[2] * o.v[1], v[2] * o.v[0] - v[0] * o.v[2], v[0] * o.v[1] - v[1] * o.v[0]};
        }
        double squaredNorm() const { return v[0] * v[0] + v[1] * v[1] + v[2] * v[2]; }
        double norm() const { return std::sqrt(squaredNorm()); }
        Row3d normalized() const { double n = squaredNorm(); return n > 0 ? *this / std::sqrt(n) : *this; }
    };
    inline Row3d operator*(double s, const Row3d& r) { return r * s; }
    using Vec3d = Row3d;

    // ------------------------------------------------------------------ dense vector
    template <typename T>
    struct VecX {
        std::vector<T> d;
        VecX() = default;
        explicit VecX(size_t n, T val = T()) : d(n, val) {}
        VecX(std::vector<T> v) : d(std::move(v)) {}
        static VecX Zero(size_t n) { return VecX(n, T(0)); }
        static VecX Constant(size_t n, T c) { return VecX(n, c); }
        int size() const { return static_cast<int>(d.size()); }
        int rows() const { return size(); }
        void resize(size_t n) { d.resize(n); }
        void setConstant(T c) { std::fill(d.begin(), d.end(), c); }
        void setZero() { setConstant(T(0)); }
        T& operator[](size_t i) { return d[i]; }
        const T& operator[](size_t i) const { return d[i]; }
        T& operator()(size_t i) { return d[i]; }
        const T& operator()(size_t i) const { return d[i]; }
        T* data() { return d.data(); }
        const T* data() const { return d.data(); }
        auto begin() { return d.begin(); }
        auto end() { return d.end(); }
        auto begin() const { return d.begin(); }
        auto end() const { return d.end(); }
    };
    using VecXi = VecX<int>;
    using VecXd = VecX<double>;
    using VecXc = VecX<complex>;
    using VecXb = VecX<bool>;

    // ------------------------------------------------------------------ dense matrix (row-major)
    template <typename T>
    struct MatX {
        int r = 0, c = 0;
        std::vector<T> d;
        MatX() = default;
        MatX(int rows, int cols, T val = T()) : r(rows), c(cols), d(size_t(rows) * cols, val) {}
        static MatX Zero(int rows, int cols) { return MatX(rows, cols, T(0)); }
        static MatX Constant(int rows, int cols, T v) { return MatX(rows, cols, v); }
        static MatX Identity(int n, int m) { MatX a(n, m, T(0)); for (int i = 0; i < std::min(n, m); i++) a(i, i) = T(1); return a; }
        int rows() const { return r; }
        int cols() const { return c; }
        void resize(int rows, int cols) { r = rows; c = cols; d.assign(size_t(rows) * cols, T()); }
        T& operator()(int i, int j) { return d[size_t(i) * c + j]; }
        const T& operator()(int i, int j) const { return d[size_t(i) * c + j]; }
        T* row(int i) { return d.data() + size_t(i) * c; }
        const T* row(int i) const { return d.data() + size_t(i) * c; }
        T* data() { return d.data(); }
        const T* data() const { return d.data(); }
        MatX operator*(const MatX& o) const {
            MatX out(r, o.c, T(0));
            for (int i = 0; i < r; i++)
                for (int k = 0; k < c; k++) {
                    T a = (*this)(i, k);
                    if (a == T(0)) continue;
                    for (int j = 0; j < o.c; j++) out(i, j) += a * o(k, j);
                }
            return out;
        }
        MatX operator-() const { MatX o(*this); for (auto& x : o.d) x = -x; return o; }
        MatX& operator+=(const MatX& o) { for (size_t i = 0; i < d.size(); i++) d[i] += o.d[i]; return *this; }
        MatX& operator-=(const MatX& o) { for (size_t i = 0; i < d.size(); i++) d[i] -= o.d[i]; return *this; }
        bool isZero() const { for (auto& x : d) if (x != T(0)) return false; return true; }
    };
    using MatXi = MatX<int>;
    using MatXd = MatX<double>;
    using MatXc = MatX<complex>;

    inline Row3d row3(const MatXd& m, int i) { return {m(i, 0), m(i, 1), m(i, 2)}; }
    inline void set_row3(MatXd& m, int i, const Row3d& v) { m(i, 0) = v[0]; m(i, 1) = v[1]; m(i, 2) = v[2]; }

    // ------------------------------------------------------------------ sparse (CSR)
    template <typename T>
    struct Triplet {
        int r, c;
        T v;
        Triplet(int r_, int c_, T v_) : r(r_), c(c_), v(v_) {}
        int row() const { return r; }
        int col() const { return c; }
        T value() const { return v; }
    };
    using TripI = Triplet<int>;
    using TripD = Triplet<double>;
    using TripC = Triplet<complex>;

    // Compressed sparse rows with sorted, unique column indices.
    template <typename T>
    struct Sprs {
        int nr = 0, nc = 0;
        std::vector<int> ptr{0}, idx;
        std::vector<T> val;
        Sprs() = default;
        Sprs(int rows, int cols) : nr(rows), nc(cols), ptr(rows + 1, 0) {}
        int rows() const { return nr; }
        int cols() const { return nc; }
        int nonZeros() const { return static_cast<int>(idx.size()); }
        void resize(int rows, int cols) { nr = rows; nc = cols; ptr.assign(rows + 1, 0); idx.clear(); val.clear(); }

        // Duplicates are summed in input order (Eigen setFromTriplets semantics).  Stable scatter
        // by row, then every row is sorted by column (stable) and merged in parallel.
        template <typename It>
        void setFromTriplets(It b, It e) {
            std::vector<int> cnt(nr + 1, 0);
            size_t n = 0;
            for (It it = b; it != e; ++it) { cnt[it->r + 1]++; n++; }
            for (int i = 0; i < nr; i++) cnt[i + 1] += cnt[i];
            std::vector<int> ci(n);
            std::vector<T> cv(n);
            {
                std::vector<int> fill(cnt.begin(), cnt.end() - 1);
                for (It it = b; it != e; ++it) { int p = fill[it->r]++; ci[p] = it->c; cv[p] = it->v; }
            }
            std::vector<int> ucnt(nr + 1, 0);
            METRIKO_PARALLEL_FOR
            for (int i = 0; i < nr; i++) {
                const int b0 = cnt[i], e0 = cnt[i + 1], k = e0 - b0;
                if (k > 32) {
                    std::vector<std::pair<int, T>> rb(k);
                    for (int q = 0; q < k; q++) rb[q] = {ci[b0 + q], cv[b0 + q]};
                    std::stable_sort(rb.begin(), rb.end(), [](const auto& x, const auto& y) { return x.first < y.first; });
                    for (int q = 0; q < k; q++) { ci[b0 + q] = rb[q].first; cv[b0 + q] = rb[q].second; }
                } else {
                    for (int q = b0 + 1; q < e0; q++) {   // insertion sort (stable)
                        const int c = ci[q];
                        const T v = cv[q];
                        int r = q - 1;
                        while (r >= b0 && ci[r] > c) { ci[r + 1] = ci[r]; cv[r + 1] = cv[r]; r--; }
                        ci[r + 1] = c;
                        cv[r + 1] = v;
                    }
                }
                int u = 0;
                for (int q = b0; q < e0; q++) if (q == b0 || ci[q] != ci[q - 1]) u++;
                ucnt[i + 1] = u;
            }
            for (int i = 0; i < nr; i++) ucnt[i + 1] += ucnt[i];
            idx.assign(ucnt[nr], 0);
            val.assign(ucnt[nr], T(0));
            METRIKO_PARALLEL_FOR
            for (int i = 0; i < nr; i++) {
                int o = ucnt[i] - 1;
                for (int q = cnt[i]; q < cnt[i + 1]; q++) {
                    if (q == cnt[i] || ci[q] != ci[q - 1]) { o++; idx[o] = ci[q]; val[o] = cv[q]; }
                    else val[o] += cv[q];
                }
            }
            ptr = std::move(ucnt);
        }
        // Removes entries with |v| <= |reference| * epsilon (Eigen prune semantics).
        void prune(double reference, double epsilon = 1e-12) {
            std::vector<int> np(nr + 1, 0), ni;
            std::vector<T> nv;
            for (int i = 0; i < nr; i++) {
                for (int p = ptr[i]; p < ptr[i + 1]; p++)
                    if (std::abs(val[p]) > std::abs(reference) * epsilon) { ni.push_back(idx[p]); nv.push_back(val[p]); }
                np[i + 1] = static_cast<int>(ni.size());
            }
            ptr = std::move(np); idx = std::move(ni); val = std::move(nv);
        }
        std::vector<T> operator*(const std::vector<T>& x) const {
            std::vector<T> y(nr, T(0));
            METRIKO_PARALLEL_FOR
            for (int i = 0; i < nr; i++) {
                T s(0);
                for (int p = ptr[i]; p < ptr[i + 1]; p++) s += val[p] * x[idx[p]];
                y[i] = s;
            }
            return y;
        }
        VecX<T> operator*(const VecX<T>& x) const { return VecX<T>((*this) * x.d); }
        Sprs transpose() const {
            std::vector<Triplet<T>> t;
            t.reserve(idx.size());
            for (int i = 0; i < nr; i++) for (int p = ptr[i]; p < ptr[i + 1]; p++) t.emplace_back(idx[p], i, val[p]);
            Sprs o(nc, nr);
            o.setFromTriplets(t.begin(), t.end());
            return o;
        }
        // Rows formed independently (a count pass, then a fill pass): each entry is 0 plus its
        // products in visit order, columns ascending -- the same arrays for any thread count.
        Sprs operator*(const Sprs& B) const {
            if (nc != B.nr) throw std::invalid_argument("sparse product: size mismatch");
            Sprs C(nr, B.nc);
            auto row = [&](int i, std::vector<std::pair<int, T>>& e) {
                e.clear();
                for (int p = ptr[i]; p < ptr[i + 1]; p++) {
                    const int k = idx[p];
                    for (int q = B.ptr[k]; q < B.ptr[k + 1]; q++) e.emplace_back(B.idx[q], val[p] * B.val[q]);
                }
                for (size_t k = 1; k < e.size(); k++) {   // stable insertion sort (rows are short)
                    const auto x = e[k];
                    size_t j = k;
                    while (j > 0 && e[j - 1].first > x.first) { e[j] = e[j - 1]; j--; }
                    e[j] = x;
                }
            };
#pragma omp parallel
            {
                std::vector<std::pair<int, T>> e;
#pragma omp for schedule(static)
                for (int i = 0; i < nr; i++) {
                    row(i, e);
                    int cnt = 0;
                    for (size_t k = 0; k < e.size(); k++) cnt += (k == 0 || e[k].first != e[k - 1].first) ? 1 : 0;
                    C.ptr[i + 1] = cnt;
                }
            }
            for (int i = 0; i < nr; i++) C.ptr[i + 1] += C.ptr[i];
            C.idx.resize(C.ptr[nr]);
            C.val.resize(C.ptr[nr]);
#pragma omp parallel
            {
                std::vector<std::pair<int, T>> e;
#pragma omp for schedule(static)
                for (int i = 0; i < nr; i++) {
                    row(i, e);
                    int o = C.ptr[i] - 1;
                    for (size_t k = 0; k < e.size(); k++) {
                        if (k == 0 || e[k].first != e[k - 1].first) { o++; C.idx[o] = e[k].first; C.val[o] = T(0); }
                        C.val[o] += e[k].second;
                    }
                }
            }
            return C;
        }
    };
    using SprsI = Sprs<int>;
    using SprsD = Sprs<double>;
    using SprsC = Sprs<complex>;
}

#endif
