// Forward-mode dual numbers (FP64) for the CPU oracle.
//
// TEST INFRASTRUCTURE ONLY (see mirk_oracle.hpp). The reference differentiates its
// collocation residual with ForwardDiff dual numbers through sparse colouring
// (lib/BoundaryValueDiffEqMIRK/src/mirk.jl:824-838); the oracle gets the same exact
// derivatives by pushing N tangent directions through the user's f and bc.
#pragma once
#include <cmath>
#include <type_traits>

namespace oracle {

template <int N>
struct Dual {
    double v;
    double d[N];
    Dual() : v(0) { for (int k = 0; k < N; ++k) d[k] = 0; }
    Dual(double x) : v(x) { for (int k = 0; k < N; ++k) d[k] = 0; }  // NOLINT: implicit by design
    Dual& operator+=(const Dual& o) { v += o.v; for (int k = 0; k < N; ++k) d[k] += o.d[k]; return *this; }
    Dual& operator-=(const Dual& o) { v -= o.v; for (int k = 0; k < N; ++k) d[k] -= o.d[k]; return *this; }
    Dual& operator*=(const Dual& o) { *this = *this * o; return *this; }
    Dual& operator/=(const Dual& o) { *this = *this / o; return *this; }
    friend Dual operator-(const Dual& a) { Dual r; r.v = -a.v; for (int k = 0; k < N; ++k) r.d[k] = -a.d[k]; return r; }
    friend Dual operator+(const Dual& a) { return a; }
    friend Dual operator+(const Dual& a, const Dual& b) { Dual r; r.v = a.v + b.v; for (int k = 0; k < N; ++k) r.d[k] = a.d[k] + b.d[k]; return r; }
    friend Dual operator-(const Dual& a, const Dual& b) { Dual r; r.v = a.v - b.v; for (int k = 0; k < N; ++k) r.d[k] = a.d[k] - b.d[k]; return r; }
    friend Dual operator*(const Dual& a, const Dual& b) { Dual r; r.v = a.v * b.v; for (int k = 0; k < N; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k]; return r; }
    friend Dual operator/(const Dual& a, const Dual& b) {
        Dual r; r.v = a.v / b.v; const double ib = 1.0 / b.v;
        for (int k = 0; k < N; ++k) r.d[k] = (a.d[k] - r.v * b.d[k]) * ib;
        return r;
    }
    template <class S, class = std::enable_if_t<std::is_arithmetic<S>::value>>
    friend Dual operator+(const Dual& a, S b) { Dual r = a; r.v += double(b); return r; }
    template <class S, class = std::enable_if_t<std::is_arithmetic<S>::value>>
    friend Dual operator+(S b, const Dual& a) { Dual r = a; r.v += double(b); return r; }
    template <class S, class = std::enable_if_t<std::is_arithmetic<S>::value>>
    friend Dual operator-(const Dual& a, S b) { Dual r = a; r.v -= double(b); return r; }
    template <class S, class = std::enable_if_t<std::is_arithmetic<S>::value>>
    friend Dual operator-(S b, const Dual& a) { Dual r = -a; r.v += double(b); return r; }
    template <class S, class = std::enable_if_t<std::is_arithmetic<S>::value>>
    friend Dual operator*(const Dual& a, S b) { Dual r; r.v = a.v * double(b); for (int k = 0; k < N; ++k) r.d[k] = a.d[k] * double(b); return r; }
    template <class S, class = std::enable_if_t<std::is_arithmetic<S>::value>>
    friend Dual operator*(S b, const Dual& a) { return a * b; }
    template <class S, class = std::enable_if_t<std::is_arithmetic<S>::value>>
    friend Dual operator/(const Dual& a, S b) { return a * (1.0 / double(b)); }
    template <class S, class = std::enable_if_t<std::is_arithmetic<S>::value>>
    friend Dual operator/(S b, const Dual& a) { return Dual(double(b)) / a; }
    friend bool operator<(const Dual& a, const Dual& b) { return a.v < b.v; }
    friend bool operator>(const Dual& a, const Dual& b) { return a.v > b.v; }
    friend bool operator<=(const Dual& a, const Dual& b) { return a.v <= b.v; }
    friend bool operator>=(const Dual& a, const Dual& b) { return a.v >= b.v; }
    template <class S, class = std::enable_if_t<std::is_arithmetic<S>::value>>
    friend bool operator<(const Dual& a, S b) { return a.v < b; }
    template <class S, class = std::enable_if_t<std::is_arithmetic<S>::value>>
    friend bool operator>(const Dual& a, S b) { return a.v > b; }
};

// chain rule helper: value fv, derivative scale dfv
template <int N>
inline Dual<N> chain(const Dual<N>& a, double fv, double dfv) {
    Dual<N> r; r.v = fv;
    for (int k = 0; k < N; ++k) r.d[k] = dfv * a.d[k];
    return r;
}
template <int N> inline Dual<N> sin(const Dual<N>& a) { return chain(a, std::sin(a.v), std::cos(a.v)); }
template <int N> inline Dual<N> cos(const Dual<N>& a) { return chain(a, std::cos(a.v), -std::sin(a.v)); }
template <int N> inline Dual<N> tan(const Dual<N>& a) { const double t = std::tan(a.v); return chain(a, t, 1.0 + t * t); }
template <int N> inline Dual<N> exp(const Dual<N>& a) { const double e = std::exp(a.v); return chain(a, e, e); }
template <int N> inline Dual<N> log(const Dual<N>& a) { return chain(a, std::log(a.v), 1.0 / a.v); }
template <int N> inline Dual<N> sqrt(const Dual<N>& a) { const double s = std::sqrt(a.v); return chain(a, s, 0.5 / s); }
template <int N> inline Dual<N> tanh(const Dual<N>& a) { const double t = std::tanh(a.v); return chain(a, t, 1.0 - t * t); }
template <int N> inline Dual<N> sinh(const Dual<N>& a) { return chain(a, std::sinh(a.v), std::cosh(a.v)); }
template <int N> inline Dual<N> cosh(const Dual<N>& a) { return chain(a, std::cosh(a.v), std::sinh(a.v)); }
template <int N> inline Dual<N> atan(const Dual<N>& a) { return chain(a, std::atan(a.v), 1.0 / (1.0 + a.v * a.v)); }
template <int N> inline Dual<N> fabs(const Dual<N>& a) { return a.v < 0 ? -a : a; }
template <int N> inline Dual<N> abs(const Dual<N>& a) { return a.v < 0 ? -a : a; }
template <int N> inline Dual<N> pow(const Dual<N>& a, double e) {
    const double pv = std::pow(a.v, e);
    return chain(a, pv, e * std::pow(a.v, e - 1.0));
}

inline double value_of(double x) { return x; }
template <int N> inline double value_of(const Dual<N>& x) { return x.v; }

}  // namespace oracle
