// Test infrastructure: nested forward-mode dual numbers for the CPU oracle.
// Dn<Dn<double, N>, N> carries a value, its gradient and its Hessian in N
// variables (seed() marks variable k); used by the oracle's element restatements
// so that their derivatives come from the energy alone.
#pragma once
#include <cmath>

namespace orc_dual {

template <typename T, int N>
struct Dn {
    T v;
    T d[N];
};

template <typename T>
struct Const {
    static T make(double c) { return c; }
};
template <typename T, int N>
struct Const<Dn<T, N>> {
    static Dn<T, N> make(double c)
    {
        Dn<T, N> r;
        r.v = Const<T>::make(c);
        for (int k = 0; k < N; ++k) r.d[k] = Const<T>::make(0.0);
        return r;
    }
};
template <typename T>
T C(double c)
{
    return Const<T>::make(c);
}

template <typename T, int N>
Dn<T, N> operator+(const Dn<T, N>& a, const Dn<T, N>& b)
{
    Dn<T, N> r;
    r.v = a.v + b.v;
    for (int k = 0; k < N; ++k) r.d[k] = a.d[k] + b.d[k];
    return r;
}
template <typename T, int N>
Dn<T, N> operator-(const Dn<T, N>& a, const Dn<T, N>& b)
{
    Dn<T, N> r;
    r.v = a.v - b.v;
    for (int k = 0; k < N; ++k) r.d[k] = a.d[k] - b.d[k];
    return r;
}
template <typename T, int N>
Dn<T, N> operator*(const Dn<T, N>& a, const Dn<T, N>& b)
{
    Dn<T, N> r;
    r.v = a.v * b.v;
    for (int k = 0; k < N; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
    return r;
}
template <typename T, int N>
Dn<T, N> operator/(const Dn<T, N>& a, const Dn<T, N>& b)
{
    Dn<T, N> r;
    r.v = a.v / b.v;
    for (int k = 0; k < N; ++k) r.d[k] = (a.d[k] * b.v - a.v * b.d[k]) / (b.v * b.v);
    return r;
}
inline double sq_root(double a) { return std::sqrt(a); }
template <typename T, int N>
Dn<T, N> sq_root(const Dn<T, N>& a)
{
    Dn<T, N> r;
    r.v = sq_root(a.v);
    for (int k = 0; k < N; ++k) r.d[k] = a.d[k] / (r.v + r.v);
    return r;
}
inline double ln(double a) { return std::log(a); }
template <typename T, int N>
Dn<T, N> ln(const Dn<T, N>& a)
{
    Dn<T, N> r;
    r.v = ln(a.v);
    for (int k = 0; k < N; ++k) r.d[k] = a.d[k] / a.v;
    return r;
}

inline double value(double a) { return a; }
template <typename T, int N>
double value(const Dn<T, N>& a)
{
    return value(a.v);
}

template <int N>
using D2 = Dn<Dn<double, N>, N>;

// variable k of N seeded for value, gradient and Hessian
template <int N>
D2<N> seed(double x, int k)
{
    D2<N> r = C<D2<N>>(x);
    r.v.d[k] = 1.0;
    r.d[k].v = 1.0;
    return r;
}

}  // namespace orc_dual
