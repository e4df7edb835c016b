// Minimal fixed-size stand-in for the parts of Eigen that the reference's
// distance-type, distance and ACCD routines use (Library/Math/Distance/
// DISTANCE_TYPE.h, DISTANCE_UNCLASSIFIED.h, POINT_*.h, EDGE_EDGE.h, CCD.h), so
// those routines can be compiled from their own source for the oracle's checks.
// Test infrastructure only.
//
// Eigen is not available here.  What Eigen decides internally is restated in
// this file and is part of the stated arithmetic policy of the compiled
// reference:
//   * 3-term reductions (dot, squaredNorm, the coefficients of small matrix
//     products) are summed left to right, ((p0 + p1) + p2);
//   * cross products are (a1 b2 - a2 b1, a2 b0 - a0 b2, a0 b1 - a1 b0);
//   * the 2x2 LDL^T is Eigen's pivoted LDL^T (pivot = larger |diagonal|, the
//     first on ties; L21 = A21 / D0; D1 = A11 - L21 (D0 L21); solve through the
//     transposition, L, D^-1 with |D| <= DBL_MIN pseudo-inverted to 0, L^T).
// Whether products fuse into those sums is left to the compiler's contraction
// (the reference builds with -mfma, so GCC's default contraction applies).
#pragma once
#include <algorithm>
#include <cmath>
#include <limits>
#include <vector>

namespace Eigen {

template <class T, int R, int C>
struct Matrix;

template <class T, int R, int C>
struct RowRef {
    Matrix<T, R, C>& m;
    int i;
    template <int R2, int C2>
    RowRef& operator=(const Matrix<T, R2, C2>& v)
    {
        static_assert(R2 * C2 == C, "row size");
        for (int j = 0; j < C; ++j) m(i, j) = v.a[j];
        return *this;
    }
    RowRef& operator=(const RowRef& o)
    {
        for (int j = 0; j < C; ++j) m(i, j) = o.m(o.i, j);
        return *this;
    }
    T operator()(int j) const { return m(i, j); }
    Matrix<T, 1, C> eval() const
    {
        Matrix<T, 1, C> r;
        for (int j = 0; j < C; ++j) r.a[j] = m(i, j);
        return r;
    }
    Matrix<T, 1, C> cross(const RowRef& o) const;
    template <int R2, int C2>
    Matrix<T, 1, C> cross(const Matrix<T, R2, C2>& o) const;
};

template <class T, int R, int C>
struct ColRef {
    Matrix<T, R, C>& m;
    int j;
    template <int R2, int C2>
    ColRef& operator=(const Matrix<T, R2, C2>& v)
    {
        static_assert(R2 * C2 == R, "column size");
        for (int i = 0; i < R; ++i) m(i, j) = v.a[i];
        return *this;
    }
};

template <class T, int N>
struct LDLT;

template <class T, int R, int C>
struct Matrix {
    T a[R * C];  // column-major
    Matrix() = default;
    template <int R2, int C2>
    Matrix(const Matrix<T, R2, C2>& o)  // vector transposition on assignment, as Eigen allows
    {
        static_assert(R2 * C2 == R * C && (R == 1 || C == 1), "vector conversion only");
        for (int k = 0; k < R * C; ++k) a[k] = o.a[k];
    }
    Matrix(const RowRef<T, 2, 3>& r) : Matrix(r.eval()) {}
    T& operator()(int i, int j) { return a[j * R + i]; }
    T operator()(int i, int j) const { return a[j * R + i]; }
    T& operator()(int k) { return a[k]; }
    T operator()(int k) const { return a[k]; }
    T& operator[](int k) { return a[k]; }
    T operator[](int k) const { return a[k]; }
    RowRef<T, R, C> row(int i) { return RowRef<T, R, C>{*this, i}; }
    ColRef<T, R, C> col(int j) { return ColRef<T, R, C>{*this, j}; }
    Matrix<T, C, R> transpose() const
    {
        Matrix<T, C, R> t;
        for (int i = 0; i < R; ++i)
            for (int j = 0; j < C; ++j) t(j, i) = (*this)(i, j);
        return t;
    }
    Matrix operator+(const Matrix& o) const
    {
        Matrix r;
        for (int k = 0; k < R * C; ++k) r.a[k] = a[k] + o.a[k];
        return r;
    }
    Matrix operator-(const Matrix& o) const
    {
        Matrix r;
        for (int k = 0; k < R * C; ++k) r.a[k] = a[k] - o.a[k];
        return r;
    }
    Matrix operator-() const
    {
        Matrix r;
        for (int k = 0; k < R * C; ++k) r.a[k] = -a[k];
        return r;
    }
    Matrix operator/(T s) const
    {
        Matrix r;
        for (int k = 0; k < R * C; ++k) r.a[k] = a[k] / s;
        return r;
    }
    Matrix& operator+=(const Matrix& o)
    {
        for (int k = 0; k < R * C; ++k) a[k] = a[k] + o.a[k];
        return *this;
    }
    Matrix& operator-=(const Matrix& o)
    {
        for (int k = 0; k < R * C; ++k) a[k] = a[k] - o.a[k];
        return *this;
    }
    template <int R2, int C2>
    T dot(const Matrix<T, R2, C2>& o) const
    {
        static_assert(R2 * C2 == R * C, "dot size");
        T s = a[0] * o.a[0];
        for (int k = 1; k < R * C; ++k) s = s + a[k] * o.a[k];
        return s;
    }
    T squaredNorm() const { return dot(*this); }
    T norm() const { return std::sqrt(squaredNorm()); }
    template <int R2, int C2>
    Matrix cross(const Matrix<T, R2, C2>& b) const
    {
        static_assert(R * C == 3 && R2 * C2 == 3, "cross of 3-vectors");
        Matrix r;
        r.a[0] = a[1] * b.a[2] - a[2] * b.a[1];
        r.a[1] = a[2] * b.a[0] - a[0] * b.a[2];
        r.a[2] = a[0] * b.a[1] - a[1] * b.a[0];
        return r;
    }
    LDLT<T, R> ldlt() const;
};

template <class T, int R, int C>
Matrix<T, 1, C> RowRef<T, R, C>::cross(const RowRef& o) const
{
    return eval().cross(o.eval());
}
template <class T, int R, int C>
template <int R2, int C2>
Matrix<T, 1, C> RowRef<T, R, C>::cross(const Matrix<T, R2, C2>& o) const
{
    return eval().cross(o);
}

template <class T, int R, int C>
Matrix<T, R, C> operator*(T s, const Matrix<T, R, C>& m)
{
    Matrix<T, R, C> r;
    for (int k = 0; k < R * C; ++k) r.a[k] = s * m.a[k];
    return r;
}

// small matrix product, each coefficient a left-to-right reduction
template <class T, int R, int K, int C>
Matrix<T, R, C> operator*(const Matrix<T, R, K>& x, const Matrix<T, K, C>& y)
{
    Matrix<T, R, C> r;
    for (int i = 0; i < R; ++i)
        for (int j = 0; j < C; ++j) {
            T s = x(i, 0) * y(0, j);
            for (int k = 1; k < K; ++k) s = s + x(i, k) * y(k, j);
            r(i, j) = s;
        }
    return r;
}

template <class T>
struct LDLT<T, 2> {
    T d0 = 0, d1 = 0, l10 = 0;
    bool swapped = false;
    template <class M>
    explicit LDLT(const M& A)
    {
        T a00 = A(0, 0), a10 = A(1, 0), a11 = A(1, 1);
        swapped = std::abs(a11) > std::abs(a00);
        if (swapped) std::swap(a00, a11);
        d0 = a00;
        if (d0 == T(0)) {
            l10 = 0;
            d1 = a11;
            zero = true;
            return;
        }
        l10 = a10 / d0;
        const T t = d0 * l10;
        d1 = a11 - l10 * t;
    }
    bool zero = false;
    Matrix<T, 2, 1> solve(const Matrix<T, 2, 1>& b) const
    {
        Matrix<T, 2, 1> y;
        if (zero) {  // all-zero diagonal: nothing is factorised and the solve gives zeros
            y.a[0] = 0;
            y.a[1] = 0;
            return y;
        }
        T z0 = swapped ? b.a[1] : b.a[0];
        T z1 = swapped ? b.a[0] : b.a[1];
        z1 = z1 - l10 * z0;
        const T tol = std::numeric_limits<T>::min();
        z0 = (std::abs(d0) > tol) ? z0 / d0 : T(0);
        z1 = (std::abs(d1) > tol) ? z1 / d1 : T(0);
        z0 = z0 - l10 * z1;
        y.a[0] = swapped ? z1 : z0;
        y.a[1] = swapped ? z0 : z1;
        return y;
    }
};

template <class T, int R, int C>
LDLT<T, R> Matrix<T, R, C>::ldlt() const
{
    return LDLT<T, R>(*this);
}

using Vector3d = Matrix<double, 3, 1>;
using RowVector3d = Matrix<double, 1, 3>;

}  // namespace Eigen
