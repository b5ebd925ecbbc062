// ss_dual1.cuh — a one-direction forward-mode dual number D1<S> (value and
// one tangent) over a scalar S (double or float), so the
// templated potential code (ss_device.cuh) differentiates along one parameter
// direction per thread: the progenitor's orbit sensitivities use one lane per
// parameter, and the release's dependence on the potential parameters uses one
// evaluation per parameter.
#pragma once

#include "ss_common.cuh"

namespace ssg {

template <class S>
struct D1 {
    S v, d;
    __host__ __device__ constexpr D1() : v(0), d(0) {}
    __host__ __device__ constexpr D1(const S& a, const S& b) : v(a), d(b) {}
    __host__ __device__ constexpr D1(int a) : v(a), d(0) {}  // NOLINT
    __host__ __device__ D1(float a) : v(a), d(0) {}          // NOLINT
    __host__ __device__ D1(double a) : v(S(a)), d(0) {}      // NOLINT
};

template <class S> __device__ __forceinline__ D1<S> operator+(const D1<S>& a, const D1<S>& b) { return D1<S>(a.v + b.v, a.d + b.d); }
template <class S> __device__ __forceinline__ D1<S> operator-(const D1<S>& a, const D1<S>& b) { return D1<S>(a.v - b.v, a.d - b.d); }
template <class S> __device__ __forceinline__ D1<S> operator-(const D1<S>& a) { return D1<S>(-a.v, -a.d); }
template <class S> __device__ __forceinline__ D1<S> operator*(const D1<S>& a, const D1<S>& b) {
    return D1<S>(a.v * b.v, a.d * b.v + a.v * b.d);
}
template <class S> __device__ __forceinline__ D1<S> operator*(float a, const D1<S>& b) { return D1<S>(a * b.v, a * b.d); }
template <class S> __device__ __forceinline__ D1<S> operator*(const D1<S>& a, float b) { return D1<S>(b * a.v, b * a.d); }
template <class S> __device__ __forceinline__ D1<S> operator+(const D1<S>& a, float b) { return D1<S>(a.v + S(b), a.d); }
template <class S> __device__ __forceinline__ D1<S> operator+(float a, const D1<S>& b) { return D1<S>(S(a) + b.v, b.d); }
template <class S> __device__ __forceinline__ D1<S> operator-(const D1<S>& a, float b) { return D1<S>(a.v - S(b), a.d); }
template <class S> __device__ __forceinline__ D1<S> operator-(float a, const D1<S>& b) { return D1<S>(S(a) - b.v, -b.d); }
template <class S> __device__ __forceinline__ D1<S>& operator+=(D1<S>& a, const D1<S>& b) {
    a = a + b;
    return a;
}

template <class S> __device__ __forceinline__ D1<S> s_rsqrt(const D1<S>& x) {
    S y = s_rsqrt(x.v);
    return D1<S>(y, (-0.5f * (y * y * y)) * x.d);
}
template <class S> __device__ __forceinline__ D1<S> s_rcp(const D1<S>& x) {
    S r = s_rcp(x.v);
    return D1<S>(r, -(r * r) * x.d);
}
template <class S> __device__ __forceinline__ D1<S> s_log1p(const D1<S>& x) {
    return D1<S>(s_log1p(x.v), x.d * s_rcp(S(1) + x.v));
}
template <class S> __device__ __forceinline__ D1<S> s_log(const D1<S>& x) {
    return D1<S>(s_log(x.v), x.d * s_rcp(x.v));
}
template <class S> __device__ __forceinline__ double sval(const D1<S>& x) { return (double)x.v; }
template <class S> __device__ __forceinline__ D1<S> s_sqrt(const D1<S>& x) {
    S r = s_sqrt(x.v);
    return D1<S>(r, (0.5f * s_rcp(r)) * x.d);
}

template <class S> __device__ __forceinline__ D1<S> gammainc_p(S a, S lg, const D1<S>& x) {
    return D1<S>(gammainc_p(a, lg, x.v), gammainc_dp(a, lg, x.v) * x.d);
}
template <class S> __device__ __forceinline__ D1<S> gammainc_dp(S a, S lg, const D1<S>& x) {
    const S dp = gammainc_dp(a, lg, x.v);
    return D1<S>(dp, (dp * ((a - S(1)) * s_rcp(x.v) - S(1))) * x.d);
}

template <class S> __device__ __forceinline__ S from_double(double c);
template <> __device__ __forceinline__ double from_double<double>(double c) { return c; }
template <> __device__ __forceinline__ float from_double<float>(double c) { return (float)c; }

// One fixed Dopri5 step of the Hamiltonian flow with T = D1<S> state and
// parameters (static composition C, no center track).
template <class C, class S>
__device__ __forceinline__ void dopri5_step_dual(const PotDev<D1<S>>& P, const D1<S>& h, D1<S> y[6]) {
    typedef D1<S> T;
    auto K = [](double c) { return T(from_double<S>(c), S(0)); };
    const T a21 = K(SS_A21), a31 = K(SS_A31), a32 = K(SS_A32), a41 = K(SS_A41), a42 = K(SS_A42), a43 = K(SS_A43);
    const T a51 = K(SS_A51), a52 = K(SS_A52), a53 = K(SS_A53), a54 = K(SS_A54);
    const T a61 = K(SS_A61), a62 = K(SS_A62), a63 = K(SS_A63), a64 = K(SS_A64), a65 = K(SS_A65);
    const T b1 = K(SS_B1), b3 = K(SS_B3), b4 = K(SS_B4), b5 = K(SS_B5), b6 = K(SS_B6);
    T k1[6], k2[6], k3[6], k4[6], k5[6], k6[6], ys[6];
    auto f = [&](const T* s, T* k) {
        T g[3];
        C::template grad<T, T, false>(P, s, s, g, nullptr);
        k[0] = s[3]; k[1] = s[4]; k[2] = s[5];
        k[3] = -g[0]; k[4] = -g[1]; k[5] = -g[2];
    };
    f(y, k1);
#pragma unroll
    for (int i = 0; i < 6; ++i) ys[i] = y[i] + h * (a21 * k1[i]);
    f(ys, k2);
#pragma unroll
    for (int i = 0; i < 6; ++i) ys[i] = y[i] + h * (a31 * k1[i] + a32 * k2[i]);
    f(ys, k3);
#pragma unroll
    for (int i = 0; i < 6; ++i) ys[i] = y[i] + h * (a41 * k1[i] + a42 * k2[i] + a43 * k3[i]);
    f(ys, k4);
#pragma unroll
    for (int i = 0; i < 6; ++i) ys[i] = y[i] + h * (a51 * k1[i] + a52 * k2[i] + a53 * k3[i] + a54 * k4[i]);
    f(ys, k5);
#pragma unroll
    for (int i = 0; i < 6; ++i)
        ys[i] = y[i] + h * (a61 * k1[i] + a62 * k2[i] + a63 * k3[i] + a64 * k4[i] + a65 * k5[i]);
    f(ys, k6);
#pragma unroll
    for (int i = 0; i < 6; ++i) y[i] = y[i] + h * (b1 * k1[i] + b3 * k3[i] + b4 * k4[i] + b5 * k5[i] + b6 * k6[i]);
}

// Tangent of the prepared parameters q of one component with respect to its
// raw parameter p[j] (the host preparation in prepare_potential):
// returns dq[0..5].
__host__ __device__ inline void prepared_param_tangent(int kind, const double* p, int j, double G, double dq[6]) {
    for (int i = 0; i < 6; ++i) dq[i] = 0.0;
    switch (kind) {
        case SS_NFW:  // q = {G m, rs, 1/rs, soft}
            if (j == 0) dq[0] = G;
            if (j == 1) { dq[1] = 1.0; dq[2] = -1.0 / (p[1] * p[1]); }
            if (j == 2) dq[3] = 1.0;
            break;
        case SS_TRIAXIAL_NFW:  // q = {G m, rs, 1/q1, 1/q2, 1/q3, 1/rs}
            if (j == 0) dq[0] = G;
            if (j == 1) { dq[1] = 1.0; dq[5] = -1.0 / (p[1] * p[1]); }
            if (j >= 2 && j <= 4) dq[j] = -1.0 / (p[j] * p[j]);
            break;
        case SS_MIYAMOTO_NAGAI:  // q = {G m, a, b^2}
            if (j == 0) dq[0] = G;
            if (j == 1) dq[1] = 1.0;
            if (j == 2) dq[2] = 2.0 * p[2];
            break;
        case SS_HERNQUIST:  // q = {G m, rs, soft}
            if (j == 0) dq[0] = G;
            if (j == 1) dq[1] = 1.0;
            if (j == 2) dq[2] = 1.0;
            break;
        case SS_PLUMMER:  // q = {G m, rs^2}
            if (j == 0) dq[0] = G;
            if (j == 1) dq[1] = 2.0 * p[1];
            break;
        case SS_ISOCHRONE:  // q = {G m, a, a^2}
            if (j == 0) dq[0] = G;
            if (j == 1) { dq[1] = 1.0; dq[2] = 2.0 * p[1]; }
            break;
        case SS_SH_EXPANSION:  // q = {scale}
            if (j == 0) dq[0] = 1.0;
            break;
        default:
            break;
    }
}

}  // namespace ssg
