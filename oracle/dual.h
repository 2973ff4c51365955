// dual.h — forward-mode dual numbers for the FP64 oracle (test infrastructure only).
//
// Dual<N> carries a value and N partial derivatives and propagates them through +, -, *, /,
// sqrt and pow by the chain rule, the operator-overloading forward mode of ForwardDiff.jl
// (which the reference's own tests use, test/general/smoothing_kernels.jl:121).  Comparisons and
// branches see the value only, so a dual run takes exactly the branches and the neighbour sets
// of the plain FP64 run, and its value part equals that run's result.
#pragma once

#include <cmath>

namespace orc {

template <int N>
struct Dual {
    double v = 0.0;
    double d[N] = {};
    Dual() = default;
    Dual(double x) : v(x) {}  // NOLINT: constants promote implicitly, as in ForwardDiff
};

template <int N>
inline Dual<N> operator+(const Dual<N>& a, const Dual<N>& b) {
    Dual<N> r(a.v + b.v);
    for (int k = 0; k < N; ++k) r.d[k] = a.d[k] + b.d[k];
    return r;
}
template <int N>
inline Dual<N> operator-(const Dual<N>& a, const Dual<N>& b) {
    Dual<N> r(a.v - b.v);
    for (int k = 0; k < N; ++k) r.d[k] = a.d[k] - b.d[k];
    return r;
}
template <int N>
inline Dual<N> operator-(const Dual<N>& a) {
    Dual<N> r(-a.v);
    for (int k = 0; k < N; ++k) r.d[k] = -a.d[k];
    return r;
}
template <int N>
inline Dual<N> operator*(const Dual<N>& a, const Dual<N>& b) {
    Dual<N> r(a.v * b.v);
    for (int k = 0; k < N; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
    return r;
}
template <int N>
inline Dual<N> operator/(const Dual<N>& a, const Dual<N>& b) {
    Dual<N> r(a.v / b.v);
    const double ib = 1.0 / b.v;
    for (int k = 0; k < N; ++k) r.d[k] = (a.d[k] - r.v * b.d[k]) * ib;
    return r;
}
template <int N>
inline Dual<N>& operator+=(Dual<N>& a, const Dual<N>& b) {
    a = a + b;
    return a;
}
template <int N> inline Dual<N> operator+(const Dual<N>& a, double b) { return a + Dual<N>(b); }
template <int N> inline Dual<N> operator+(double a, const Dual<N>& b) { return Dual<N>(a) + b; }
template <int N> inline Dual<N> operator-(const Dual<N>& a, double b) { return a - Dual<N>(b); }
template <int N> inline Dual<N> operator-(double a, const Dual<N>& b) { return Dual<N>(a) - b; }
template <int N> inline Dual<N> operator*(const Dual<N>& a, double b) { return a * Dual<N>(b); }
template <int N> inline Dual<N> operator*(double a, const Dual<N>& b) { return Dual<N>(a) * b; }
template <int N> inline Dual<N> operator/(const Dual<N>& a, double b) { return a / Dual<N>(b); }
template <int N> inline Dual<N> operator/(double a, const Dual<N>& b) { return Dual<N>(a) / b; }
template <int N> inline bool operator<(const Dual<N>& a, const Dual<N>& b) { return a.v < b.v; }
template <int N> inline bool operator<(const Dual<N>& a, double b) { return a.v < b; }
template <int N> inline bool operator>(const Dual<N>& a, double b) { return a.v > b; }
template <int N> inline bool operator<=(const Dual<N>& a, double b) { return a.v <= b; }

template <int N>
inline Dual<N> sqrt(const Dual<N>& a) {
    Dual<N> r(std::sqrt(a.v));
    const double s = 0.5 / r.v;
    for (int k = 0; k < N; ++k) r.d[k] = a.d[k] * s;
    return r;
}
// x^p for a constant exponent p
template <int N>
inline Dual<N> pow(const Dual<N>& a, double p) {
    Dual<N> r(std::pow(a.v, p));
    const double s = p * std::pow(a.v, p - 1.0);
    for (int k = 0; k < N; ++k) r.d[k] = a.d[k] * s;
    return r;
}
// fused multiply-add a * b + c (the CK2N54 update's @muladd); derivative of the product form
template <int N>
inline Dual<N> fma(const Dual<N>& a, const Dual<N>& b, const Dual<N>& c) {
    Dual<N> r(std::fma(a.v, b.v, c.v));
    for (int k = 0; k < N; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k] + c.d[k];
    return r;
}
template <int N> inline bool isnan(const Dual<N>& a) { return std::isnan(a.v); }

// value of a scalar (plain double or dual), for branches and cell indices
inline double val(double x) { return x; }
template <int N> inline double val(const Dual<N>& a) { return a.v; }

}  // namespace orc
