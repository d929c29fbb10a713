// Device prelude for the JIT-compiled MIRK kernels: problem-source macros, forward-mode
// dual numbers and scalar math overloads. Compiled by NVRTC for sm_103a ahead of the
// user's problem source (BVP_F / BVP_BC / BVP_BCA / BVP_BCB bodies).
//
// The reference differentiates f and bc with ForwardDiff dual numbers
// (lib/BoundaryValueDiffEqMIRK/src/mirk.jl:824-838, Core/src/types.jl:93-114); the GPU
// Jacobian kernel does the same in registers with Dual<float, 2M>.
#pragma once

#define BVP_DEV __device__ __forceinline__

#define BVP_F \
    template <class T, class P> BVP_DEV void bvp_f(T* du, const T* u, const P* p, P t)
#define BVP_BC \
    template <class T, class P> BVP_DEV void bvp_bc(T* res, const T* const* ua, const P* p)
#define BVP_BCA \
    template <class T, class P> BVP_DEV void bvp_bca(T* res, const T* ua, const P* p)
#define BVP_BCB \
    template <class T, class P> BVP_DEV void bvp_bcb(T* res, const T* ub, const P* p)
// optional: S u for the singular term S y / t of y' = S y / t + f(t, y) (a source that
// defines BVP_SING is compiled with BVP_SINGULAR=1)
#define BVP_SING \
    template <class T, class P> BVP_DEV void bvp_sing(T* su, const T* u, const P* p)

namespace bvp {

template <class X> struct is_arith { static constexpr bool value = false; };
template <> struct is_arith<float> { static constexpr bool value = true; };
template <> struct is_arith<double> { static constexpr bool value = true; };
template <> struct is_arith<int> { static constexpr bool value = true; };
template <> struct is_arith<long> { static constexpr bool value = true; };
template <> struct is_arith<long long> { static constexpr bool value = true; };
template <> struct is_arith<unsigned> { static constexpr bool value = true; };
template <bool B, class X = void> struct enable_if {};
template <class X> struct enable_if<true, X> { using type = X; };
#define BVP_IF_ARITH(S) class = typename ::bvp::enable_if<::bvp::is_arith<S>::value>::type

// the dual overloads below must not hide the scalar ones inside this namespace
using ::fabs; using ::sin; using ::cos; using ::tan; using ::exp; using ::log; using ::sqrt;
using ::tanh; using ::sinh; using ::cosh; using ::atan; using ::pow;

// scalar math in the scalar's own precision
BVP_DEV float m_sin(float x) { return sinf(x); }
BVP_DEV double m_sin(double x) { return sin(x); }
BVP_DEV float m_cos(float x) { return cosf(x); }
BVP_DEV double m_cos(double x) { return cos(x); }
BVP_DEV void m_sincos(float x, float* s, float* c) { sincosf(x, s, c); }
BVP_DEV void m_sincos(double x, double* s, double* c) { sincos(x, s, c); }
BVP_DEV float m_tan(float x) { return tanf(x); }
BVP_DEV double m_tan(double x) { return tan(x); }
BVP_DEV float m_exp(float x) { return expf(x); }
BVP_DEV double m_exp(double x) { return exp(x); }
BVP_DEV float m_log(float x) { return logf(x); }
BVP_DEV double m_log(double x) { return log(x); }
BVP_DEV float m_sqrt(float x) { return sqrtf(x); }
BVP_DEV double m_sqrt(double x) { return sqrt(x); }
BVP_DEV float m_tanh(float x) { return tanhf(x); }
BVP_DEV double m_tanh(double x) { return tanh(x); }
BVP_DEV float m_sinh(float x) { return sinhf(x); }
BVP_DEV double m_sinh(double x) { return sinh(x); }
BVP_DEV float m_cosh(float x) { return coshf(x); }
BVP_DEV double m_cosh(double x) { return cosh(x); }
BVP_DEV float m_atan(float x) { return atanf(x); }
BVP_DEV double m_atan(double x) { return atan(x); }
BVP_DEV float m_pow(float x, float e) { return powf(x, e); }
BVP_DEV double m_pow(double x, double e) { return pow(x, e); }

template <class R, int N>
struct Dual {
    R v;
    R d[N];
    BVP_DEV Dual() : v(R(0)) {
#pragma unroll
        for (int k = 0; k < N; ++k) d[k] = R(0);
    }
    template <class S, BVP_IF_ARITH(S)>
    BVP_DEV Dual(S x) : v(R(x)) {  // NOLINT: implicit by design
#pragma unroll
        for (int k = 0; k < N; ++k) d[k] = R(0);
    }
    BVP_DEV Dual& operator+=(const Dual& o) { v += o.v; for (int k = 0; k < N; ++k) d[k] += o.d[k]; return *this; }
    BVP_DEV Dual& operator-=(const Dual& o) { v -= o.v; for (int k = 0; k < N; ++k) d[k] -= o.d[k]; return *this; }
};

template <class R, int N> BVP_DEV Dual<R, N> operator-(const Dual<R, N>& a) {
    Dual<R, N> r; r.v = -a.v;
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = -a.d[k];
    return r;
}
template <class R, int N> BVP_DEV Dual<R, N> operator+(const Dual<R, N>& a) { return a; }
template <class R, int N> BVP_DEV Dual<R, N> operator+(const Dual<R, N>& a, const Dual<R, N>& b) {
    Dual<R, N> r; r.v = a.v + b.v;
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = a.d[k] + b.d[k];
    return r;
}
template <class R, int N> BVP_DEV Dual<R, N> operator-(const Dual<R, N>& a, const Dual<R, N>& b) {
    Dual<R, N> r; r.v = a.v - b.v;
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = a.d[k] - b.d[k];
    return r;
}
template <class R, int N> BVP_DEV Dual<R, N> operator*(const Dual<R, N>& a, const Dual<R, N>& b) {
    Dual<R, N> r; r.v = a.v * b.v;
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
    return r;
}
template <class R, int N> BVP_DEV Dual<R, N> operator/(const Dual<R, N>& a, const Dual<R, N>& b) {
    Dual<R, N> r; r.v = a.v / b.v;
    const R ib = R(1) / b.v;
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = (a.d[k] - r.v * b.d[k]) * ib;
    return r;
}
template <class R, int N, class S, BVP_IF_ARITH(S)>
BVP_DEV Dual<R, N> operator+(const Dual<R, N>& a, S b) { Dual<R, N> r = a; r.v += R(b); return r; }
template <class R, int N, class S, BVP_IF_ARITH(S)>
BVP_DEV Dual<R, N> operator+(S b, const Dual<R, N>& a) { Dual<R, N> r = a; r.v += R(b); return r; }
template <class R, int N, class S, BVP_IF_ARITH(S)>
BVP_DEV Dual<R, N> operator-(const Dual<R, N>& a, S b) { Dual<R, N> r = a; r.v -= R(b); return r; }
template <class R, int N, class S, BVP_IF_ARITH(S)>
BVP_DEV Dual<R, N> operator-(S b, const Dual<R, N>& a) { Dual<R, N> r = -a; r.v += R(b); return r; }
template <class R, int N, class S, BVP_IF_ARITH(S)>
BVP_DEV Dual<R, N> operator*(const Dual<R, N>& a, S b) {
    Dual<R, N> r; const R bb = R(b); r.v = a.v * bb;
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = a.d[k] * bb;
    return r;
}
template <class R, int N, class S, BVP_IF_ARITH(S)>
BVP_DEV Dual<R, N> operator*(S b, const Dual<R, N>& a) { return a * b; }
template <class R, int N, class S, BVP_IF_ARITH(S)>
BVP_DEV Dual<R, N> operator/(const Dual<R, N>& a, S b) { return a * (R(1) / R(b)); }
template <class R, int N, class S, BVP_IF_ARITH(S)>
BVP_DEV Dual<R, N> operator/(S b, const Dual<R, N>& a) { return Dual<R, N>(R(b)) / a; }
template <class R, int N> BVP_DEV bool operator<(const Dual<R, N>& a, const Dual<R, N>& b) { return a.v < b.v; }
template <class R, int N> BVP_DEV bool operator>(const Dual<R, N>& a, const Dual<R, N>& b) { return a.v > b.v; }
template <class R, int N, class S, BVP_IF_ARITH(S)> BVP_DEV bool operator<(const Dual<R, N>& a, S b) { return a.v < R(b); }
template <class R, int N, class S, BVP_IF_ARITH(S)> BVP_DEV bool operator>(const Dual<R, N>& a, S b) { return a.v > R(b); }

template <class R, int N>
BVP_DEV Dual<R, N> d_chain(const Dual<R, N>& a, R fv, R dfv) {
    Dual<R, N> r; r.v = fv;
#pragma unroll
    for (int k = 0; k < N; ++k) r.d[k] = dfv * a.d[k];
    return r;
}
template <class R, int N> BVP_DEV Dual<R, N> sin(const Dual<R, N>& a) { R s, c; m_sincos(a.v, &s, &c); return d_chain(a, s, c); }
template <class R, int N> BVP_DEV Dual<R, N> cos(const Dual<R, N>& a) { R s, c; m_sincos(a.v, &s, &c); return d_chain(a, c, -s); }
template <class R, int N> BVP_DEV Dual<R, N> tan(const Dual<R, N>& a) { const R t = m_tan(a.v); return d_chain(a, t, R(1) + t * t); }
template <class R, int N> BVP_DEV Dual<R, N> exp(const Dual<R, N>& a) { const R e = m_exp(a.v); return d_chain(a, e, e); }
template <class R, int N> BVP_DEV Dual<R, N> log(const Dual<R, N>& a) { return d_chain(a, m_log(a.v), R(1) / a.v); }
template <class R, int N> BVP_DEV Dual<R, N> sqrt(const Dual<R, N>& a) { const R s = m_sqrt(a.v); return d_chain(a, s, R(0.5) / s); }
template <class R, int N> BVP_DEV Dual<R, N> tanh(const Dual<R, N>& a) { const R t = m_tanh(a.v); return d_chain(a, t, R(1) - t * t); }
template <class R, int N> BVP_DEV Dual<R, N> sinh(const Dual<R, N>& a) { return d_chain(a, m_sinh(a.v), m_cosh(a.v)); }
template <class R, int N> BVP_DEV Dual<R, N> cosh(const Dual<R, N>& a) { return d_chain(a, m_cosh(a.v), m_sinh(a.v)); }
template <class R, int N> BVP_DEV Dual<R, N> atan(const Dual<R, N>& a) { return d_chain(a, m_atan(a.v), R(1) / (R(1) + a.v * a.v)); }
template <class R, int N> BVP_DEV Dual<R, N> fabs(const Dual<R, N>& a) { return a.v < R(0) ? -a : a; }
template <class R, int N> BVP_DEV Dual<R, N> abs(const Dual<R, N>& a) { return a.v < R(0) ? -a : a; }
template <class R, int N, class S, BVP_IF_ARITH(S)>
BVP_DEV Dual<R, N> pow(const Dual<R, N>& a, S e) {
    const R ee = R(e);
    return d_chain(a, m_pow(a.v, ee), ee * m_pow(a.v, ee - R(1)));
}

}  // namespace bvp
