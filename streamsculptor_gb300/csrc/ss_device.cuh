// ss_device.cuh — device-side potential model shared by every kernel.
//
// The reference computes forces as jax.grad of scalar potentials
// (main.py:37-40) and tidal tensors / r-hat^T H r-hat as nested jacfwd
// (main.py:59-85).  Here every component has a hand-derived analytic gradient
// and Hessian, templated on the scalar type so the same source serves FP64,
// FP32 and the forward-mode dual numbers used for release Jacobians.
//
// Spherical components are written as grad Phi = g(r) x and
// Hessian = g I + h x x^T with h = g'(r)/r.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <type_traits>
#include <utility>

#include "../../include/streamsculptor_gb300.h"

namespace ssg {

// ------------------------------------------------------------ dual numbers
// Forward-mode dual with N tangent directions (release Jacobians).
template <int N>
struct Dual {
    double v;
    double d[N];
    __host__ __device__ Dual() : v(0.0) {
#pragma unroll
        for (int i = 0; i < N; ++i) d[i] = 0.0;
    }
    __host__ __device__ Dual(double c) : v(c) {  // NOLINT
#pragma unroll
        for (int i = 0; i < N; ++i) d[i] = 0.0;
    }
};
template <int N>
__host__ __device__ inline Dual<N> operator+(const Dual<N>& a, const Dual<N>& b) {
    Dual<N> r;
    r.v = a.v + b.v;
#pragma unroll
    for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i];
    return r;
}
template <int N>
__host__ __device__ inline Dual<N> operator-(const Dual<N>& a, const Dual<N>& b) {
    Dual<N> r;
    r.v = a.v - b.v;
#pragma unroll
    for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i];
    return r;
}
template <int N>
__host__ __device__ inline Dual<N> operator-(const Dual<N>& a) {
    Dual<N> r;
    r.v = -a.v;
#pragma unroll
    for (int i = 0; i < N; ++i) r.d[i] = -a.d[i];
    return r;
}
template <int N>
__host__ __device__ inline Dual<N> operator*(const Dual<N>& a, const Dual<N>& b) {
    Dual<N> r;
    r.v = a.v * b.v;
#pragma unroll
    for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
    return r;
}
template <int N>
__host__ __device__ inline Dual<N> operator/(const Dual<N>& a, const Dual<N>& b) {
    Dual<N> r;
    double inv = 1.0 / b.v;
    r.v = a.v * inv;
#pragma unroll
    for (int i = 0; i < N; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) * inv;
    return r;
}
template <int N>
__host__ __device__ inline Dual<N>& operator+=(Dual<N>& a, const Dual<N>& b) {
    a = a + b;
    return a;
}
template <int N>
__host__ __device__ inline Dual<N>& operator-=(Dual<N>& a, const Dual<N>& b) {
    a = a - b;
    return a;
}
template <int N>
__host__ __device__ inline Dual<N> operator*(const Dual<N>& a, double b) {
    Dual<N> r;
    r.v = a.v * b;
#pragma unroll
    for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b;
    return r;
}
template <int N> __host__ __device__ inline Dual<N> operator*(double a, const Dual<N>& b) { return b * a; }
template <int N> __host__ __device__ inline Dual<N> operator+(const Dual<N>& a, double b) { Dual<N> r = a; r.v += b; return r; }
template <int N> __host__ __device__ inline Dual<N> operator+(double a, const Dual<N>& b) { Dual<N> r = b; r.v += a; return r; }
template <int N> __host__ __device__ inline Dual<N> operator-(const Dual<N>& a, double b) { Dual<N> r = a; r.v -= b; return r; }
template <int N> __host__ __device__ inline Dual<N> operator-(double a, const Dual<N>& b) { return Dual<N>(a) - b; }
template <int N> __host__ __device__ inline Dual<N> operator/(const Dual<N>& a, double b) { return a * (1.0 / b); }
template <int N> __host__ __device__ inline Dual<N> operator/(double a, const Dual<N>& b) { return Dual<N>(a) / b; }

template <int N>
__device__ inline Dual<N> chain(const Dual<N>& x, double fv, double dfv) {
    Dual<N> r;
    r.v = fv;
#pragma unroll
    for (int i = 0; i < N; ++i) r.d[i] = dfv * x.d[i];
    return r;
}

// Scalar helpers overloaded for float / double / Dual.
// FP32: hardware reciprocal (square root) estimates refined by one Newton
// step (no IEEE special-case paths; arguments are positive and finite).
// FP64: the hardware estimates of rcp.approx.ftz.f64 / rsqrt.approx.ftz.f64
// refined by one third-order step: with e = 1 - x y (reciprocal) or
// e = 1 - x y^2 (reciprocal square root), 1/x = y / (1 - e) and x^(-1/2) =
// y (1 - e)^(-1/2) are expanded to e^2, which leaves an error of order e^3
// below the final rounding; no IEEE special-case paths (arguments are
// positive and finite).  GB300 issues FP64 at 1/64 of the FP32 rate, so the
// force evaluations are written in as few FP64 instructions as their
// accuracy allows.
#include "ss_log_table.inc"

__device__ __forceinline__ float  s_sqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double s_sqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float s_rsqrt(float x) {
    // hardware estimate + one Newton step: y (3 - x y^2) / 2
    float y = rsqrtf(x);
    float e = fmaf(-x * y, y, 1.0f);
    return fmaf(0.5f * y, e, y);
}
__device__ __forceinline__ double rsqrt_estimate(double x) {
    double y;
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    return y;
}
__device__ __forceinline__ double rcp_estimate(double x) {
    double y;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    return y;
}
__device__ __forceinline__ double s_rsqrt(double x) {
    const double y = rsqrt_estimate(x);
    const double e = fma(-x * y, y, 1.0);
    return fma(y * e, fma(e, 0.375, 0.5), y);  // y (1 + e/2 + 3 e^2 / 8)
}
__device__ __forceinline__ float  s_log1p(float x) { return log1pf(x); }
// ln(1 + u), u >= 0 (NFW's ln(1 + r / r_s)), table-driven after Tang (ACM
// TOMS 16, 1990): w = 1 + u is rounded and its rounding error c kept
// (ln(1 + u) = ln w + c / w to first order in c); w = 2^k m with m in
// [1, 2) and j the nearest breakpoint F_j = 1 + j / 128; with G_j = 1 / F_j
// rounded and L_j = -ln G_j from the table, ln m = L_j + ln(1 + r) exactly,
// r = m G_j - 1 from one FMA, |r| < 2^-8; ln(1 + r) by its Taylor series
// through r^7 (the next term is below 2^-59 r).
__device__ __forceinline__ double s_log1p(double u) {
    const double w = 1.0 + u;
    const double bb = w - 1.0;
    const double c = (1.0 - (w - bb)) + (u - bb);  // the rounding error of 1 + u, exactly (TwoSum)
    const double rw0 = rcp_estimate(w);
    const double rw = fma(rw0, fma(-w, rw0, 1.0), rw0);  // 1 / w to ~2^-44: c / w is the whole result for tiny u
    const int hi = __double2hiint(w), lo = __double2loint(w);
    const int k = (hi >> 20) - 1023;
    const int j = ((hi & 0x000fffff) + 0x1000) >> 13;  // nearest of 128 breakpoints: 0 .. 128
    const double m = __hiloint2double((hi & 0x000fffff) | 0x3ff00000, lo);
    const double2 t = __ldg(&g_ln_tab[j]);
    const double r = fma(m, t.x, -1.0);
    double q = fma(r, -1.0 / 7.0, 1.0 / 6.0);
    q = fma(r, q, -0.2);
    q = fma(r, q, 0.25);
    q = fma(r, q, -1.0 / 3.0);
    q = fma(r, q, 0.5);
    const double p = fma(-r * r, q, r);  // ln(1 + r)
    const double kd = (double)k;
    return fma(kd, SS_LN2_HI, t.y) + (p + fma(kd, SS_LN2_LO, c * rw));
}
__device__ __forceinline__ float s_rcp(float x) {
    // hardware estimate + one Newton step: r (2 - x r)
    float r = __fdividef(1.0f, x);
    return fmaf(r, fmaf(-x, r, 1.0f), r);
}
__device__ __forceinline__ double s_rcp(double x) {
    const double y = rcp_estimate(x);
    const double e = fma(-x, y, 1.0);
    return fma(y, fma(e, e, e), y);  // y (1 + e + e^2)
}
__device__ __forceinline__ double s_cbrt(double x) { return cbrt(x); }
template <int N> __device__ inline Dual<N> s_sqrt(const Dual<N>& x) { double s = sqrt(x.v); return chain(x, s, 0.5 / s); }
template <int N> __device__ inline Dual<N> s_rsqrt(const Dual<N>& x) { double s = 1.0 / sqrt(x.v); return chain(x, s, -0.5 * s / x.v); }
template <int N> __device__ inline Dual<N> s_log1p(const Dual<N>& x) { return chain(x, log1p(x.v), 1.0 / (1.0 + x.v)); }
template <int N> __device__ inline Dual<N> s_rcp(const Dual<N>& x) { double r = 1.0 / x.v; return chain(x, r, -r * r); }
template <int N> __device__ inline Dual<N> s_cbrt(const Dual<N>& x) { double c = cbrt(x.v); return chain(x, c, c / (3.0 * x.v)); }
__device__ __forceinline__ float  s_log(float x) { return logf(x); }
__device__ __forceinline__ double s_log(double x) { return log(x); }
template <int N> __device__ inline Dual<N> s_log(const Dual<N>& x) { return chain(x, log(x.v), 1.0 / x.v); }
// value part of a scalar or dual number
__device__ __forceinline__ double sval(float x) { return (double)x; }
__device__ __forceinline__ double sval(double x) { return x; }
template <int N> __device__ __forceinline__ double sval(const Dual<N>& x) { return x.v; }

// ---------------------------------------------------- prepared potential
// Parameters are pre-combined on the host (G*m, 1/r_s, b^2 ...).
template <class R>
struct CompDev {
    int32_t kind;
    int32_t center;
    R q[6];
};

// Spherical-harmonic expansion table (SS_SH_EXPANSION).  tab64 is the
// caller's [nk][nt][2] (value, d/du) table; tab32, when set, is the FP32
// per-interval copy {f_k, du f'_k, f_k+1, du f'_k+1} [nk-1][nt] that the
// FP32 stream builds in its workspace.
struct ExpDev {
    const double* tab64;
    const float4* tab32;
    double u0, du, inv_du;
    int32_t nk, lmax;
};

struct TrackDev {
    const double* knots;
    const double* slopes;
    double t0;
    double dt;
    int64_t n;
    int32_t linear;  // 1: piecewise-linear through the knots (slopes unused)
};

struct ShDev {
    int32_t kind;
    int32_t n;
    const double* m;
    const double* a;
    const double* x0;
    const double* v;
    const double* t0;
    double t_window;
    double G;
    // SS_SH_GRID: [n][ng][2] (value, d/du) spline tables in u = ln r
    const double* grid;
    const double* gu0;
    const double* gdu;
    int32_t ng;
};

template <class R>
struct PotDev {
    int32_t n;
    int32_t has_track;
    CompDev<R> c[SS_MAX_COMPONENTS];
    TrackDev track;
    ShDev sh;
    ExpDev ex;
    // time-dependent parts: the pattern speed shared by the rotating
    // components, and the frame-velocity track of SS_UNIFORM_ACCEL
    double omega;
    int32_t has_rot;
    int32_t has_facc;
    TrackDev fvel;
    // SS_GROWS: bit k set when component k is multiplied by g(t), column 0
    // of the growth track
    int32_t grow_mask;
    TrackDev growth;
};

// What the time-dependent components need at one evaluation time: the
// rotation (c, s) = (cos, sin)(omega t) of the rotating components' frame
// and the gradient ga = dv_frame/dt of SS_UNIFORM_ACCEL.  FP64 callers form
// it from t (time_dep), the FP32 stream reads it per stage from a table.
template <class T>
struct TimeDep {
    T c, s;
    T ga[3];
    T amp;  // growth factor g(t) of the SS_GROWS components
    __host__ __device__ TimeDep() : c(T(1)), s(T(0)), amp(T(1)) { ga[0] = ga[1] = ga[2] = T(0); }
};

// --------------------------------------------------------------- track
// C1 cubic Hermite through knots at t0 + k dt (the progenitor spline).
__device__ inline void track_eval(const TrackDev& tr, double t, double c[3]) {
    double u = (t - tr.t0) / tr.dt;
    double fk = floor(u);
    int64_t k = (int64_t)fk;
    if (k < 0) k = 0;
    if (k > tr.n - 2) k = tr.n - 2;
    double s = u - (double)k;
    if (tr.linear) {
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            double p0 = __ldg(tr.knots + 3 * k + i), p1 = __ldg(tr.knots + 3 * (k + 1) + i);
            c[i] = p0 + s * (p1 - p0);
        }
        return;
    }
    double s2 = s * s, s3 = s2 * s;
    double h00 = 2.0 * s3 - 3.0 * s2 + 1.0;
    double h10 = s3 - 2.0 * s2 + s;
    double h01 = -2.0 * s3 + 3.0 * s2;
    double h11 = s3 - s2;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        double p0 = __ldg(tr.knots + 3 * k + i), p1 = __ldg(tr.knots + 3 * (k + 1) + i);
        double m0 = __ldg(tr.slopes + 3 * k + i), m1 = __ldg(tr.slopes + 3 * (k + 1) + i);
        c[i] = h00 * p0 + h10 * tr.dt * m0 + h01 * p1 + h11 * tr.dt * m1;
    }
}

// d/dt of the piecewise-linear frame-velocity track at t: the slope of the
// segment holding t (the end segments continue outside the knots), the
// derivative of a linear RegularGridInterpolator.
// A cubic track gives the derivative of its Hermite segment.
__device__ inline void track_slope(const TrackDev& tr, double t, double d[3]) {
    double u = (t - tr.t0) / tr.dt;
    int64_t k = (int64_t)floor(u);
    if (k < 0) k = 0;
    if (k > tr.n - 2) k = tr.n - 2;
    const double s = u - (double)k;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const double p0 = __ldg(tr.knots + 3 * k + i), p1 = __ldg(tr.knots + 3 * (k + 1) + i);
        if (tr.linear) {
            d[i] = (p1 - p0) / tr.dt;
        } else {
            const double m0 = __ldg(tr.slopes + 3 * k + i), m1 = __ldg(tr.slopes + 3 * (k + 1) + i);
            d[i] = ((6.0 * s * s - 6.0 * s) * (p0 - p1)) / tr.dt + (3.0 * s * s - 4.0 * s + 1.0) * m0 +
                   (3.0 * s * s - 2.0 * s) * m1;
        }
    }
}

template <class R>
__device__ inline TimeDep<double> time_dep(const PotDev<R>& P, double t) {
    TimeDep<double> td;
    if (P.has_rot) sincos(P.omega * t, &td.s, &td.c);
    if (P.has_facc) track_slope(P.fvel, t, td.ga);
    if (P.grow_mask) {
        double gv[3];
        track_eval(P.growth, t, gv);
        td.amp = gv[0];
    }
    return td;
}

template <class T, class S>
__device__ __forceinline__ TimeDep<T> time_dep_as(const TimeDep<S>& a) {
    TimeDep<T> r;
    r.c = T(a.c);
    r.s = T(a.s);
    r.ga[0] = T(a.ga[0]);
    r.ga[1] = T(a.ga[1]);
    r.ga[2] = T(a.ga[2]);
    r.amp = T(a.amp);
    return r;
}

// ------------------------------------------------- spherical profiles
// g(r) with grad Phi = g x, and (optionally) h = g'(r)/r.  `r2` is the
// (softened) squared radius.
// F(u) / u^3 with F(u) = ln(1+u) - u/(1+u), the NFW enclosed-mass shape,
// evaluated without cancellation in FP32: for u < 2, with s = u/(2+u),
// ln(1+u) = 2 atanh(s) and u/(1+u) = 2s/(1+s) give
// F = 2 s^2/(1+s) + 2 s^3 sum_k s^(2k)/(2k+3), all terms positive
// (12 terms reach float precision for s < 1/2); for u >= 2 the direct
// difference loses at most a factor 2.5.
__device__ __forceinline__ float nfw_F_over_u3(float u, float inv_u) {
    float F;
    if (u < 2.0f) {
        float s = u * s_rcp(2.0f + u);
        float w = s * s;
        float P = 1.0f / 27.0f;
        P = fmaf(P, w, 1.0f / 25.0f);
        P = fmaf(P, w, 1.0f / 23.0f);
        P = fmaf(P, w, 1.0f / 21.0f);
        P = fmaf(P, w, 1.0f / 19.0f);
        P = fmaf(P, w, 1.0f / 17.0f);
        P = fmaf(P, w, 1.0f / 15.0f);
        P = fmaf(P, w, 1.0f / 13.0f);
        P = fmaf(P, w, 1.0f / 11.0f);
        P = fmaf(P, w, 1.0f / 9.0f);
        P = fmaf(P, w, 1.0f / 7.0f);
        P = fmaf(P, w, 1.0f / 5.0f);
        P = fmaf(P, w, 1.0f / 3.0f);
        F = 2.0f * w * (s_rcp(1.0f + s) + s * P);
    } else {
        F = log1pf(u) - u * s_rcp(1.0f + u);
    }
    return F * (inv_u * inv_u * inv_u);
}

template <class T, class R, bool HESS>
__device__ __forceinline__ void nfw_gh(const R* q, const T& r2, T& g, T& h) {
    // Phi = -GM ln(1 + r/rs)/r  (NFWPotential, potential.py:80-84)
    if constexpr (std::is_same<T, float>::value && !HESS) {
        // g = GM F(u) / r^3 = (GM / rs^3) F(u) / u^3, u = r / rs
        T inv_r = s_rsqrt(r2);
        T u = r2 * inv_r * q[2];
        g = (q[0] * q[2] * q[2] * q[2]) * nfw_F_over_u3(u, q[1] * inv_r);
        return;
    }
    T inv_r = s_rsqrt(r2);
    T r = r2 * inv_r;
    T L = s_log1p(r * q[2]);
    T inv_rrs = s_rcp(r + q[1]);
    T inv_r2 = inv_r * inv_r;
    g = q[0] * inv_r2 * (L * inv_r - inv_rrs);
    if (HESS) {
        // g'(r) = GM [ -3 L / r^4 + (4 r + 3 rs) / (r^3 (r + rs)^2) ]
        T inv_r4 = inv_r2 * inv_r2;
        T gp = q[0] * (-3.0f * L * inv_r4 + (4.0f * r + 3.0f * q[1]) * inv_r2 * inv_r * inv_rrs * inv_rrs);
        h = gp * inv_r;
    }
}

template <class T, class R, bool HESS>
__device__ __forceinline__ void hernquist_gh(const R* q, const T& r2, T& g, T& h) {
    // Phi = -GM/(r + rs)  (HernquistPotential, potential.py:135-138)
    T inv_r = s_rsqrt(r2);
    T r = r2 * inv_r;
    T inv_rrs = s_rcp(r + q[1]);
    g = q[0] * inv_r * inv_rrs * inv_rrs;
    if (HESS) {
        T gp = -q[0] * (3.0f * r + q[1]) * inv_r * inv_r * inv_rrs * inv_rrs * inv_rrs;
        h = gp * inv_r;
    }
}

template <class T, class R, bool HESS>
__device__ __forceinline__ void plummer_gh(const R* q, const T& r2, T& g, T& h) {
    // Phi = -GM/sqrt(r^2 + b^2)  (PlummerPotential, potential.py:127-130)
    T id = s_rsqrt(r2 + q[1]);
    T id2 = id * id;
    g = q[0] * id2 * id;
    if (HESS) h = -3.0f * g * id2;
}

template <class T, class R, bool HESS>
__device__ __forceinline__ void isochrone_gh(const R* q, const T& r2, T& g, T& h) {
    // Phi = -GM/(a + sqrt(r^2 + a^2))  (Isochrone, potential.py:119-122)
    T s2 = r2 + q[2];
    T inv_s = s_rsqrt(s2);
    T s = s2 * inv_s;
    T inv_as = s_rcp(q[1] + s);
    g = q[0] * inv_s * inv_as * inv_as;
    if (HESS) h = -q[0] * (3.0f * s + q[1]) * inv_s * inv_s * inv_s * inv_as * inv_as * inv_as;
}

// Regularised lower incomplete gamma function P(a, x) = gamma(a, x) /
// Gamma(a), a > 0, x >= 0, given lg = ln Gamma(a) (PowerLawCutoffPotential,
// potential.py:357-388, evaluates it with jax.scipy.special.gammainc).  With
// e = x^a e^-x / Gamma(a): for x < a + 1 the power series
//   P = e sum_{n>=0} x^n / (a (a+1) ... (a+n)),
// else P = 1 - e F with the continued fraction
//   F = 1 / (x + 1 - a - 1 (1 - a) / (x + 3 - a - 2 (2 - a) / (x + 5 - a - ...)))
// (Abramowitz & Stegun 6.5.29 and 6.5.31), evaluated by the modified Lentz
// method; both stop once a term moves the result by less than the
// precision of S (bounded at 500 terms).
template <class S>
__device__ __forceinline__ S gammainc_p_s(S a, S lg, S x) {
    constexpr bool dbl = sizeof(S) == 8;
    const S eps = dbl ? S(1e-16) : S(6e-8);
    const S tiny = dbl ? S(1e-300) : S(1e-30);
    if (!(x > S(0))) return S(0);
    const S e = exp(a * log(x) - x - lg);
    if (x < a + S(1)) {
        S term = S(1) / a, sum = term;
        for (int n = 1; n < 500; ++n) {
            term *= x / (a + S(n));
            sum += term;
            if (fabs(term) < fabs(sum) * eps) break;
        }
        return sum * e;
    }
    S b = x + S(1) - a, c = S(1) / tiny, d = S(1) / b, h = d;
    for (int i = 1; i < 500; ++i) {
        const S an = -S(i) * (S(i) - a);
        b += S(2);
        d = an * d + b;
        if (fabs(d) < tiny) d = tiny;
        c = b + an / c;
        if (fabs(c) < tiny) c = tiny;
        d = S(1) / d;
        const S del = d * c;
        h *= del;
        if (fabs(del - S(1)) < eps) break;
    }
    return S(1) - e * h;
}
// dP/dx = x^(a-1) e^-x / Gamma(a)
template <class S>
__device__ __forceinline__ S gammainc_dp_s(S a, S lg, S x) {
    return x > S(0) ? exp((a - S(1)) * log(x) - x - lg) : S(0);
}
__device__ __forceinline__ float gammainc_p(float a, float lg, float x) { return gammainc_p_s<float>(a, lg, x); }
__device__ __forceinline__ double gammainc_p(double a, double lg, double x) { return gammainc_p_s<double>(a, lg, x); }
__device__ __forceinline__ float gammainc_dp(float a, float lg, float x) { return gammainc_dp_s<float>(a, lg, x); }
__device__ __forceinline__ double gammainc_dp(double a, double lg, double x) { return gammainc_dp_s<double>(a, lg, x); }
template <int N>
__device__ inline Dual<N> gammainc_p(double a, double lg, const Dual<N>& x) {
    return chain(x, gammainc_p(a, lg, x.v), gammainc_dp(a, lg, x.v));
}
template <int N>
__device__ inline Dual<N> gammainc_dp(double a, double lg, const Dual<N>& x) {
    const double dp = gammainc_dp(a, lg, x.v);
    return chain(x, dp, dp * ((a - 1.0) / x.v - 1.0));
}

template <class T, class R, bool HESS>
__device__ __forceinline__ void powerlaw_cutoff_gh(const R* q, const T& r2, T& g, T& h) {
    // dPhi/dr = G m P(a, r^2 / r_c^2) / r^2, a = (3 - alpha) / 2
    // (PowerLawCutoffPotential.gradient_func, potential.py:380-388);
    // q = {G m, a, 1 / r_c^2, ln Gamma(a), ...}
    const T x = r2 * q[2];
    const T P = gammainc_p(q[1], q[3], x);
    const T inv_r = s_rsqrt(r2);
    const T inv_r3 = inv_r * inv_r * inv_r;
    g = q[0] * P * inv_r3;
    if (HESS) {
        // g'(r) / r = G m (2 P'(x) / r_c^2 - 3 P / r^2) / r^3
        const T dP = gammainc_dp(q[1], q[3], x);
        h = q[0] * (2.0f * q[2] * dP - 3.0f * P * inv_r * inv_r) * inv_r3;
    }
}

// Regularised incomplete beta function I_z(a, b) = B(z; a, b) / B(a, b),
// a, b > 0, for ZhaoPotential (potential.py:282-355, which evaluates it with
// jax.scipy.special.betainc).  lb = ln B(a, b); zc = 1 - z is passed
// separately so that callers can form it without cancellation.  With
// f = z^a zc^b / B(a, b), for z < (a + 1) / (a + b + 2)
//   I = f / a * 1 / (1 + d1 / (1 + d2 / (1 + ...))),
//   d_{2m+1} = -(a + m)(a + b + m) z / ((a + 2m)(a + 2m + 1)),
//   d_{2m}   = m (b - m) z / ((a + 2m - 1)(a + 2m))
// (Abramowitz & Stegun 26.5.8), else I = 1 - I_zc(b, a); the fraction is
// evaluated by the modified Lentz method and stops once a pair of terms
// moves it by less than the precision of S (bounded at 300 pairs).
template <class S>
__device__ __forceinline__ S betainc_cf(S a, S b, S z) {
    constexpr bool dbl = sizeof(S) == 8;
    const S eps = dbl ? S(1e-16) : S(6e-8);
    const S tiny = dbl ? S(1e-300) : S(1e-30);
    S c = S(1), d = S(1) - (a + b) * z / (a + S(1));
    if (fabs(d) < tiny) d = tiny;
    d = S(1) / d;
    S h = d;
    for (int m = 1; m < 300; ++m) {
        const S m2 = S(2 * m);
        S an = S(m) * (b - S(m)) * z / ((a + m2 - S(1)) * (a + m2));
        d = S(1) + an * d;
        if (fabs(d) < tiny) d = tiny;
        c = S(1) + an / c;
        if (fabs(c) < tiny) c = tiny;
        d = S(1) / d;
        h *= d * c;
        an = -(a + S(m)) * (a + b + S(m)) * z / ((a + m2) * (a + m2 + S(1)));
        d = S(1) + an * d;
        if (fabs(d) < tiny) d = tiny;
        c = S(1) + an / c;
        if (fabs(c) < tiny) c = tiny;
        d = S(1) / d;
        const S del = d * c;
        h *= del;
        if (fabs(del - S(1)) < eps) break;
    }
    return h;
}
template <class S>
__device__ __forceinline__ S betainc_s(S a, S b, S lb, S z, S zc) {
    if (!(z > S(0))) return S(0);
    if (!(zc > S(0))) return S(1);
    const S f = exp(a * log(z) + b * log(zc) - lb);
    if (z < (a + S(1)) / (a + b + S(2))) return f * betainc_cf(a, b, z) / a;
    return S(1) - f * betainc_cf(b, a, zc) / b;
}
// dI_z/dz = z^(a-1) zc^(b-1) / B(a, b)
template <class S>
__device__ __forceinline__ S betainc_dz_s(S a, S b, S lb, S z, S zc) {
    return (z > S(0) && zc > S(0)) ? exp((a - S(1)) * log(z) + (b - S(1)) * log(zc) - lb) : S(0);
}
__device__ __forceinline__ float betainc(float a, float b, float lb, float z, float zc) {
    return betainc_s<float>(a, b, lb, z, zc);
}
__device__ __forceinline__ double betainc(double a, double b, double lb, double z, double zc) {
    return betainc_s<double>(a, b, lb, z, zc);
}
__device__ __forceinline__ float betainc_dz(float a, float b, float lb, float z, float zc) {
    return betainc_dz_s<float>(a, b, lb, z, zc);
}
__device__ __forceinline__ double betainc_dz(double a, double b, double lb, double z, double zc) {
    return betainc_dz_s<double>(a, b, lb, z, zc);
}
// z and zc = 1 - z carry the same derivative with opposite signs; the
// duals follow z
template <int N>
__device__ inline Dual<N> betainc(double a, double b, double lb, const Dual<N>& z, const Dual<N>& zc) {
    return chain(z, betainc(a, b, lb, z.v, zc.v), betainc_dz(a, b, lb, z.v, zc.v));
}
template <int N>
__device__ inline Dual<N> betainc_dz(double a, double b, double lb, const Dual<N>& z, const Dual<N>& zc) {
    const double dz = betainc_dz(a, b, lb, z.v, zc.v);
    return chain(z, dz, dz * ((a - 1.0) / z.v - (b - 1.0) / zc.v));
}
// x^p for x > 0
__device__ __forceinline__ float s_pow(float x, float p) { return exp2f(p * log2f(x)); }
__device__ __forceinline__ double s_pow(double x, double p) { return exp(p * log(x)); }
template <int N>
__device__ inline Dual<N> s_pow(const Dual<N>& x, double p) {
    const double v = s_pow(x.v, p);
    return chain(x, v, p * v / x.v);
}

// ZhaoPotential (potential.py:282-355).  Its gradient in the reference is
// the forward difference (Phi(r + dr) - Phi(r)) / dr, dr = 1e-5 r + 1e-8, of
// its potential (potential.py:347-354); here it is the exact derivative
// dPhi/dr = G m I_z(a1, b1) / r^2 (the enclosed mass, a1 = alpha (3 - gamma),
// b1 = alpha (beta - 3), z = y / (1 + y), y = (r / r_s)^(1/alpha)) taken at
// the difference's midpoint r_m = r + dr / 2, which equals the forward
// difference to O(dr^2) (relative ~1e-11) without its cancellation, and
// whose r-derivative is the reference's autodiff Hessian of the difference
// to the same order.  q = {G m, 1 / r_s, 1 / alpha, a1, b1, ln B(a1, b1)}.
template <class T, class R, bool HESS>
__device__ __forceinline__ void zhao_gh(const R* q, const T& r2, T& g, T& h) {
    const T r = s_sqrt(r2);
    const T rm = r + (r * 5e-6f + 5e-9f);  // the FP32 constants only round the small term
    const T y = s_pow(rm * q[1], q[2]);
    const T zc = s_rcp(1.0f + y);
    const T z = y * zc;
    const T I = betainc(q[3], q[4], q[5], z, zc);
    const T irm = s_rcp(rm);
    const T gr = q[0] * I * irm * irm;  // dPhi/dr at r_m
    const T ir = s_rcp(r);
    g = gr * ir;
    if (HESS) {
        // dz/dr_m = z zc / (alpha r_m); dr_m/dr = 1 + 5e-6
        const T dI = betainc_dz(q[3], q[4], q[5], z, zc) * z * zc * q[2] * irm;
        T dgr = q[0] * (dI - 2.0f * I * irm) * irm * irm;
        dgr = dgr + dgr * 5e-6f;
        h = (dgr - g) * ir * ir;
    }
}

// Adds grad Phi of one component of compile-time kind KIND at x (already
// shifted to its center) to grad[3]; when HESS, adds its Hessian
// (xx, yy, zz, xy, xz, yz) to H[6].
template <int KIND, class T, class R, bool HESS>
__device__ __forceinline__ void kind_grad(const R* q, const T x[3], T grad[3], T H[6]) {
    if constexpr (KIND == SS_NFW || KIND == SS_HERNQUIST || KIND == SS_PLUMMER || KIND == SS_ISOCHRONE ||
                  KIND == SS_POWERLAW_CUTOFF || KIND == SS_ZHAO) {
        T r2 = x[0] * x[0] + x[1] * x[1] + x[2] * x[2];
        T g, h;
        if constexpr (KIND == SS_NFW) {
            nfw_gh<T, R, HESS>(q, r2 + q[3], g, h);
        } else if constexpr (KIND == SS_HERNQUIST) {
            hernquist_gh<T, R, HESS>(q, r2 + q[2], g, h);
        } else if constexpr (KIND == SS_PLUMMER) {
            plummer_gh<T, R, HESS>(q, r2, g, h);
        } else if constexpr (KIND == SS_POWERLAW_CUTOFF) {
            powerlaw_cutoff_gh<T, R, HESS>(q, r2, g, h);
        } else if constexpr (KIND == SS_ZHAO) {
            zhao_gh<T, R, HESS>(q, r2, g, h);
        } else {
            isochrone_gh<T, R, HESS>(q, r2, g, h);
        }
        grad[0] += g * x[0];
        grad[1] += g * x[1];
        grad[2] += g * x[2];
        if constexpr (HESS) {
            H[0] += g + h * x[0] * x[0];
            H[1] += g + h * x[1] * x[1];
            H[2] += g + h * x[2] * x[2];
            H[3] += h * x[0] * x[1];
            H[4] += h * x[0] * x[2];
            H[5] += h * x[1] * x[2];
        }
    } else if constexpr (KIND == SS_TRIAXIAL_NFW) {
        // Phi(x) = NFW(xi), xi_i = x_i / q_i  (potential.py:92-97)
        T xi[3] = {x[0] * q[2], x[1] * q[3], x[2] * q[4]};
        T r2 = xi[0] * xi[0] + xi[1] * xi[1] + xi[2] * xi[2];
        R qq[4] = {q[0], q[1], q[5], R(0)};
        T g, h;
        nfw_gh<T, R, HESS>(qq, r2, g, h);
        grad[0] += g * xi[0] * q[2];
        grad[1] += g * xi[1] * q[3];
        grad[2] += g * xi[2] * q[4];
        if constexpr (HESS) {
            H[0] += (g + h * xi[0] * xi[0]) * (q[2] * q[2]);
            H[1] += (g + h * xi[1] * xi[1]) * (q[3] * q[3]);
            H[2] += (g + h * xi[2] * xi[2]) * (q[4] * q[4]);
            H[3] += h * xi[0] * xi[1] * (q[2] * q[3]);
            H[4] += h * xi[0] * xi[2] * (q[2] * q[4]);
            H[5] += h * xi[1] * xi[2] * (q[3] * q[4]);
        }
    } else if constexpr (KIND == SS_MIYAMOTO_NAGAI) {
        // Phi = -GM / sqrt(R^2 + (a + sqrt(z^2 + b^2))^2)  (potential.py:69-72)
        T zb2 = x[2] * x[2] + q[2];
        T izeta = s_rsqrt(zb2);
        T zeta = zb2 * izeta;
        T az = zeta + q[1];
        T S2 = x[0] * x[0] + x[1] * x[1] + az * az;
        T iS = s_rsqrt(S2);
        T iS2 = iS * iS;
        T gm_iS3 = q[0] * iS2 * iS;
        T fz = az * izeta;  // (a + zeta) / zeta
        grad[0] += gm_iS3 * x[0];
        grad[1] += gm_iS3 * x[1];
        grad[2] += gm_iS3 * x[2] * fz;
        if constexpr (HESS) {
            T k3 = -3.0f * gm_iS3 * iS2;  // -3 GM / S^5
            H[0] += gm_iS3 + k3 * x[0] * x[0];
            H[1] += gm_iS3 + k3 * x[1] * x[1];
            H[3] += k3 * x[0] * x[1];
            H[4] += k3 * x[0] * x[2] * fz;
            H[5] += k3 * x[1] * x[2] * fz;
            T z2 = x[2] * x[2];
            H[2] += gm_iS3 * (fz - q[1] * z2 * izeta * izeta * izeta) + k3 * z2 * fz * fz;
        }
    }
}

// Rotating bars, evaluated in the frame turning with pattern speed omega:
// x' = (c x + s y, -s x + c y, z) with (c, s) = (cos, sin)(omega t), so
// grad = R^T grad' and H = R^T H' R (BarPotential, potential.py:178-198:
// the simulation-frame point rotated by -omega t).
//
// SS_BAR, Long & Murali (1992) eq. 8a: Phi' = K [g(X - a) - g(X + a)],
// K = G m / 2a, g(w) = ln(w + T), T = sqrt(w^2 + Y^2 + B^2),
// B = b + sqrt(c^2 + z^2); q = {K, a, b, c^2}.  With Q = 1 / (T (w + T)):
// dg/dw = 1/T, dg/dY = Y Q, dg/dz = B B' Q, and the second derivatives below.
template <class T, class R, bool HESS>
__device__ __forceinline__ void bar_lm_grad(const R* q, const T xp[3], T g[3], T H[6]) {
    const T X = xp[0], Y = xp[1], z = xp[2];
    const T S = s_sqrt(T(q[3]) + z * z);
    const T B = T(q[2]) + S;
    const T Bp = z * s_rcp(S);  // dB/dz
    const T rho2 = Y * Y + B * B;
    T acc[6] = {T(0), T(0), T(0), T(0), T(0), T(0)};  // d2 xx yy zz xy xz yz
#pragma unroll
    for (int side = 0; side < 2; ++side) {
        const T w = side == 0 ? X - T(q[1]) : X + T(q[1]);
        const R sg = side == 0 ? R(1) : R(-1);
        const T Tn = s_sqrt(w * w + rho2);
        const T iT = s_rcp(Tn);
        const T Q = iT * s_rcp(w + Tn);
        g[0] += T(q[0]) * sg * iT;
        g[1] += T(q[0]) * sg * Y * Q;
        g[2] += T(q[0]) * sg * B * Bp * Q;
        if constexpr (HESS) {
            const T iT3 = iT * iT * iT;
            const T E = Q * (iT * iT + Q);  // -dQ/dY / Y
            const T Bpp = T(q[3]) * s_rcp(S * S * S);
            acc[0] += sg * (-w * iT3);
            acc[3] += sg * (-Y * iT3);
            acc[4] += sg * (-B * Bp * iT3);
            acc[1] += sg * (Q - Y * Y * E);
            acc[5] += sg * (-Y * B * Bp * E);
            acc[2] += sg * ((Bp * Bp + B * Bpp) * Q - B * B * Bp * Bp * E);
        }
    }
    if constexpr (HESS) {
#pragma unroll
        for (int i = 0; i < 6; ++i) H[i] = T(q[0]) * acc[i];
    }
}

// SS_DEHNEN_BAR (DehnenBarPotential, potential.py:200-222) in its corotating
// frame: Phi' = A W(r) P2, P2 = (x'^2 - y'^2) cos 2phi_b + 2 x'y' sin 2phi_b,
// W = U(r)/r^2: -Rb^3 r^-5 for r >= Rb, r/Rb^3 - 2/r^2 inside;
// q = {A, Rb, cos 2phi_b, sin 2phi_b}, A = alpha v0^2/3 (R0/Rb)^3.
template <class T, class R, bool HESS>
__device__ __forceinline__ void bar_dehnen_grad(const R* q, const T xp[3], T g[3], T H[6]) {
    const T x = xp[0], y = xp[1], z = xp[2];
    const T r2 = x * x + y * y + z * z;
    const T r = s_sqrt(r2), ir = s_rcp(r);
    const R Rb = q[1], Rb3 = q[1] * q[1] * q[1];
    T W, W1, W2;  // W, dW/dr, d2W/dr2
    if (sval(r) >= (double)Rb) {
        const T ir2 = ir * ir, ir5 = ir2 * ir2 * ir;
        W = T(-Rb3) * ir5;
        W1 = T(R(5) * Rb3) * ir5 * ir;
        W2 = T(R(-30) * Rb3) * ir5 * ir2;
    } else {
        const T ir2 = ir * ir;
        W = r * T(R(1) / Rb3) - T(R(2)) * ir2;
        W1 = T(R(1) / Rb3) + T(R(4)) * ir2 * ir;
        W2 = T(R(-12)) * ir2 * ir2;
    }
    const T C2 = T(q[2]), S2 = T(q[3]);
    const T P2 = (x * x - y * y) * C2 + T(R(2)) * x * y * S2;
    const T dP[3] = {T(R(2)) * (x * C2 + y * S2), T(R(2)) * (x * S2 - y * C2), T(0)};
    const T u[3] = {x * ir, y * ir, z * ir};
    const T A = T(q[0]);
#pragma unroll
    for (int i = 0; i < 3; ++i) g[i] += A * (W1 * u[i] * P2 + W * dP[i]);
    if constexpr (HESS) {
        // A [W'' u u^T P2 + W' (I - u u^T)/r P2 + W' (u dP^T + dP u^T) + W d2P]
        const int ia[6] = {0, 1, 2, 0, 0, 1}, ib[6] = {0, 1, 2, 1, 2, 2};
        const T d2P[6] = {T(R(2)) * C2, T(R(-2)) * C2, T(0), T(R(2)) * S2, T(0), T(0)};
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            const int i = ia[k], j = ib[k];
            const T uu = u[i] * u[j];
            const T id = i == j ? T(1) : T(0);
            H[k] = A * (W2 * uu * P2 + W1 * (id - uu) * ir * P2 + W1 * (u[i] * dP[j] + dP[i] * u[j]) + W * d2P[k]);
        }
    }
}

// A rotating component at x (simulation frame), added to grad / H.
template <int KIND, class T, class R, bool HESS>
__device__ __forceinline__ void rot_grad(const R* q, const T x[3], const TimeDep<T>& td, T grad[3], T H[6]) {
    const T xp[3] = {td.c * x[0] + td.s * x[1], td.c * x[1] - td.s * x[0], x[2]};
    T gp[3] = {T(0), T(0), T(0)}, Hp[6];
    if constexpr (KIND == SS_BAR)
        bar_lm_grad<T, R, HESS>(q, xp, gp, Hp);
    else
        bar_dehnen_grad<T, R, HESS>(q, xp, gp, Hp);
    grad[0] += td.c * gp[0] - td.s * gp[1];
    grad[1] += td.s * gp[0] + td.c * gp[1];
    grad[2] += gp[2];
    if constexpr (HESS) {
        // H = R^T H' R, R = [[c, s, 0], [-s, c, 0], [0, 0, 1]]
        const T c = td.c, s = td.s;
        const T a = Hp[0], b = Hp[1], e = Hp[3], f = Hp[4], h = Hp[5];
        H[0] += c * c * a - T(R(2)) * c * s * e + s * s * b;
        H[1] += s * s * a + T(R(2)) * c * s * e + c * c * b;
        H[2] += Hp[2];
        H[3] += c * s * (a - b) + (c * c - s * s) * e;
        H[4] += c * f - s * h;
        H[5] += s * f + c * h;
    }
}

// Runtime-kind dispatch (the generic path for any composition).
template <class T, class R, bool HESS>
__device__ __forceinline__ void comp_grad(const CompDev<R>& c, const T x[3], T grad[3], T H[6],
                                          const TimeDep<T>& td = TimeDep<T>()) {
    switch (c.kind) {
        case SS_BAR: rot_grad<SS_BAR, T, R, HESS>(c.q, x, td, grad, H); break;
        case SS_DEHNEN_BAR: rot_grad<SS_DEHNEN_BAR, T, R, HESS>(c.q, x, td, grad, H); break;
        case SS_UNIFORM_ACCEL:
            grad[0] += td.ga[0];
            grad[1] += td.ga[1];
            grad[2] += td.ga[2];
            break;
        case SS_NFW: kind_grad<SS_NFW, T, R, HESS>(c.q, x, grad, H); break;
        case SS_TRIAXIAL_NFW: kind_grad<SS_TRIAXIAL_NFW, T, R, HESS>(c.q, x, grad, H); break;
        case SS_MIYAMOTO_NAGAI: kind_grad<SS_MIYAMOTO_NAGAI, T, R, HESS>(c.q, x, grad, H); break;
        case SS_HERNQUIST: kind_grad<SS_HERNQUIST, T, R, HESS>(c.q, x, grad, H); break;
        case SS_PLUMMER: kind_grad<SS_PLUMMER, T, R, HESS>(c.q, x, grad, H); break;
        case SS_ISOCHRONE: kind_grad<SS_ISOCHRONE, T, R, HESS>(c.q, x, grad, H); break;
        case SS_POWERLAW_CUTOFF: kind_grad<SS_POWERLAW_CUTOFF, T, R, HESS>(c.q, x, grad, H); break;
        case SS_ZHAO: kind_grad<SS_ZHAO, T, R, HESS>(c.q, x, grad, H); break;
        default: break;
    }
}

// ------------------------------------------- spherical-harmonic expansion
// Phi = scale * sum_lm f_lm(r) Y_lm(n), n = x / r, real Schmidt harmonics
// (the layout is documented with ss_expansion in the C header).  The
// angular parts come from the regular solid harmonics at the unit vector,
//   R_l^m = r^l P_l^m(cos theta) e^{i m phi} / (l+m)!,
//   R_m^m = (x + i y)/(2m) R_{m-1}^{m-1},  R_{m+1}^m = z R_m^m,
//   R_l^m = ((2l-1) z R_{l-1}^m - r^2 R_{l-2}^m) / ((l-m)(l+m)),
// so Y_lm = N_lm {Re, Im} R_l^m(n) with N_l0 = l!, N_lm = sqrt(2 (l-m)!(l+m)!).
// Their derivatives are lower-degree harmonics (R_l^{-m} = (-1)^m conj R_l^m):
//   d/dx R_l^m = (R_{l-1}^{m-1} - R_{l-1}^{m+1}) / 2,
//   d/dy R_l^m = i (R_{l-1}^{m+1} + R_{l-1}^{m-1}) / 2,   d/dz R_l^m = R_{l-1}^m,
// which gives gradients and Hessians without differentiating the recurrence.
// With K = Y_lm(n), a0 = f, a1 = f', a2 = f'' (in r), homogeneity gives
//   grad = sum [G1 K n + (a0/r) (grad K)(n)],           G1 = a1 - l a0 / r,
//   H    = sum [G2 K n n^T + (G1/r) K (I - n n^T) + (G1/r)(n gK^T + gK n^T)
//               + (a0/r^2) (hess K)(n)],               G2 = a2 - 2 l a1/r + l(l+1) a0/r^2.
static __constant__ double c_shnorm[SS_SHEXP_LMAX + 1][SS_SHEXP_LMAX + 1] = {
    {1.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0},
    {1.0, 2.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0},
    {2.0, 3.4641016151377544, 6.928203230275509, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0},
    {6.0, 9.797958971132712, 15.491933384829668, 37.94733192202055, 0.0, 0.0, 0.0, 0.0, 0.0},
    {24.0, 37.94733192202055, 53.665631459994955, 100.39920318408906, 283.9718295887816, 0.0, 0.0, 0.0, 0.0},
    {120.0, 185.903200617956, 245.92681838303037, 401.59681273635624, 851.9154887663448, 2693.9933184772376, 0.0,
     0.0, 0.0},
    {720.0, 1099.8181667894016, 1391.172167634186, 2086.758251451279, 3809.8818879330106, 8934.965025113417,
     30951.626774694734, 0.0, 0.0},
    {5040.0, 7619.763775866021, 9332.266605707318, 13197.818001472819, 21886.105181141756, 43772.21036228351,
     111597.67739518596, 417560.27397251286, 0.0},
    {40320.0, 60480.0, 72287.42629254413, 97877.63789548662, 151631.38461413587, 273357.36609793414,
     590519.4025601529, 1617203.9871333486, 6468815.948533394}};
// the same table as a compile-time function (immediates in unrolled code)
__host__ __device__ constexpr double shnorm_ct(int l, int m) {
    const double t[SS_SHEXP_LMAX + 1][SS_SHEXP_LMAX + 1] = {
    {1.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0},
    {1.0, 2.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0},
    {2.0, 3.4641016151377544, 6.928203230275509, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0},
    {6.0, 9.797958971132712, 15.491933384829668, 37.94733192202055, 0.0, 0.0, 0.0, 0.0, 0.0},
    {24.0, 37.94733192202055, 53.665631459994955, 100.39920318408906, 283.9718295887816, 0.0, 0.0, 0.0, 0.0},
    {120.0, 185.903200617956, 245.92681838303037, 401.59681273635624, 851.9154887663448, 2693.9933184772376, 0.0,
     0.0, 0.0},
    {720.0, 1099.8181667894016, 1391.172167634186, 2086.758251451279, 3809.8818879330106, 8934.965025113417,
     30951.626774694734, 0.0, 0.0},
    {5040.0, 7619.763775866021, 9332.266605707318, 13197.818001472819, 21886.105181141756, 43772.21036228351,
     111597.67739518596, 417560.27397251286, 0.0},
    {40320.0, 60480.0, 72287.42629254413, 97877.63789548662, 151631.38461413587, 273357.36609793414,
     590519.4025601529, 1617203.9871333486, 6468815.948533394}};
    return t[l][m];
}

template <class T>
struct SolidH {
    T C[SS_SHEXP_LMAX + 1][SS_SHEXP_LMAX + 1];
    T S[SS_SHEXP_LMAX + 1][SS_SHEXP_LMAX + 1];
    // real and imaginary parts of R_l^m for any integer l, m (zero outside)
    __device__ __forceinline__ T c(int l, int m) const {
        if (l < 0 || m > l || -m > l) return T(0);
        if (m >= 0) return C[l][m];
        return (m & 1) ? T(0) - C[l][-m] : C[l][-m];
    }
    __device__ __forceinline__ T s(int l, int m) const {
        if (l < 0 || m > l || -m > l) return T(0);
        if (m >= 0) return S[l][m];
        return (m & 1) ? S[l][-m] : T(0) - S[l][-m];
    }
};

// Straight-line code for float/double; rolled loops for the dual-number
// types (their unrolled form only adds spills and compile time).
template <class T>
struct ShUnroll {
    static constexpr int n = std::is_floating_point<T>::value ? 32 : 1;
};

template <class T>
__device__ __forceinline__ void solid_harmonics(const T n[3], SolidH<T>& R) {
    constexpr int LM = SS_SHEXP_LMAX;
    constexpr int UR = ShUnroll<T>::n;
    R.C[0][0] = T(1);
    R.S[0][0] = T(0);
#pragma unroll UR
    for (int m = 1; m <= LM; ++m) {
        const T f = T(1.0 / (2.0 * m));
        R.C[m][m] = (n[0] * R.C[m - 1][m - 1] - n[1] * R.S[m - 1][m - 1]) * f;
        R.S[m][m] = (n[0] * R.S[m - 1][m - 1] + n[1] * R.C[m - 1][m - 1]) * f;
    }
#pragma unroll UR
    for (int m = 0; m < LM; ++m) {
        R.C[m + 1][m] = n[2] * R.C[m][m];
        R.S[m + 1][m] = n[2] * R.S[m][m];
    }
#pragma unroll UR
    for (int m = 0; m <= LM; ++m) {
#pragma unroll UR
        for (int l = m + 2; l <= LM; ++l) {
            const T a = T((2.0 * l - 1.0) / ((double)(l - m) * (l + m)));
            const T b = T(1.0 / ((double)(l - m) * (l + m)));
            R.C[l][m] = a * n[2] * R.C[l - 1][m] - b * R.C[l - 2][m];
            R.S[l][m] = a * n[2] * R.S[l - 1][m] - b * R.S[l - 2][m];
        }
    }
}

// Radial spline of every term at u = ln r: Hermite basis weights and the
// knot interval.  e is the distance (in knot spacings) beyond the end knot
// where the spline continues linearly.
template <class T>
struct RadialBasis {
    int k;
    T h[4], hs[4], hss[4], e;
};

template <class T>
__device__ __forceinline__ void radial_basis(const ExpDev& E, const T& u, RadialBasis<T>& B) {
    const double us = (sval(u) - E.u0) * E.inv_du;
    int k = (int)floor(us);
    k = k < 0 ? 0 : (k > E.nk - 2 ? E.nk - 2 : k);
    B.k = k;
    T s = (u - T(E.u0 + (double)k * E.du)) * T(E.inv_du);
    T sc = s;
    if (sval(s) < 0.0) sc = T(0);
    if (sval(s) > 1.0) sc = T(1);
    B.e = s - sc;
    const T one(1), two(2), three(3), six(6);
    T om = one - sc;
    B.h[0] = (one + two * sc) * om * om;
    B.h[1] = sc * om * om;
    B.h[2] = sc * sc * (three - two * sc);
    B.h[3] = sc * sc * (sc - one);
    B.hs[0] = six * sc * (sc - one);
    B.hs[1] = om * (one - three * sc);
    B.hs[2] = six * sc * om;
    B.hs[3] = sc * (three * sc - two);
    const bool inside = sval(B.e) == 0.0;
    B.hss[0] = inside ? T(12) * sc - six : T(0);
    B.hss[1] = inside ? six * sc - T(4) : T(0);
    B.hss[2] = inside ? six - T(12) * sc : T(0);
    B.hss[3] = inside ? six * sc - two : T(0);
}

// Phi_0(u) and dPhi_0/du of a cubic Hermite spline in u through n knots at
// u0 + k du, knot k holding (value, d/du) at tab[2k], tab[2k + 1], continued
// linearly in u outside the knots: the form of an expansion's radial
// functions (radial_basis, radial_term), used for the exact spherical part
// of the learned surrogate (ss_mlp.base).
template <class T, class V>
__device__ __forceinline__ void base_spline(const V* tab, int n, T u0, T du, T inv_du, T u, T& f, T& fu) {
    int k = (int)floor((u - u0) * inv_du);
    k = k < 0 ? 0 : (k > n - 2 ? n - 2 : k);
    const T s = (u - (u0 + T(k) * du)) * inv_du;
    const T sc = s < T(0) ? T(0) : (s > T(1) ? T(1) : s);
    const T e = s - sc, om = T(1) - sc;
    const T c0 = T(tab[2 * k]), c1 = T(tab[2 * k + 1]) * du, c2 = T(tab[2 * k + 2]), c3 = T(tab[2 * k + 3]) * du;
    const T fs = T(6) * sc * (sc - T(1)) * c0 + om * (T(1) - T(3) * sc) * c1 + T(6) * sc * om * c2 +
                 sc * (T(3) * sc - T(2)) * c3;
    f = (T(1) + T(2) * sc) * om * om * c0 + sc * om * om * c1 + sc * sc * (T(3) - T(2) * sc) * c2 +
        sc * sc * (sc - T(1)) * c3 + e * fs;
    fu = fs * inv_du;
}

// f, df/ds, d2f/ds2 of term j (s in knot spacings).
template <class T>
__device__ __forceinline__ void radial_term(const ExpDev& E, const RadialBasis<T>& B, int nt, int j, T& f, T& fs,
                                            T& fss) {
    T c0, c1, c2, c3;
    if constexpr (std::is_same<T, float>::value) {
        if (E.tab32) {
            const float4 t = __ldg(E.tab32 + (size_t)B.k * nt + j);
            c0 = t.x; c1 = t.y; c2 = t.z; c3 = t.w;
        } else {
            const double* a = E.tab64 + ((size_t)B.k * nt + j) * 2;
            const double* b = a + (size_t)nt * 2;
            c0 = (float)__ldg(a); c1 = (float)(__ldg(a + 1) * E.du);
            c2 = (float)__ldg(b); c3 = (float)(__ldg(b + 1) * E.du);
        }
    } else {
        const double* a = E.tab64 + ((size_t)B.k * nt + j) * 2;
        const double* b = a + (size_t)nt * 2;
        c0 = T(__ldg(a)); c1 = T(__ldg(a + 1) * E.du);
        c2 = T(__ldg(b)); c3 = T(__ldg(b + 1) * E.du);
    }
    fs = B.hs[0] * c0 + B.hs[1] * c1 + B.hs[2] * c2 + B.hs[3] * c3;
    f = B.h[0] * c0 + B.h[1] * c1 + B.h[2] * c2 + B.h[3] * c3 + B.e * fs;
    fss = B.hss[0] * c0 + B.hss[1] * c1 + B.hss[2] * c2 + B.hss[3] * c3;
}

// Rows of R_l^m (m = 0..l): the gradient of a degree-l term needs degree
// l-1 and its Hessian degree l-2, so the recurrence runs degree by degree
// keeping three rows (the live set stays small).
template <class T>
struct ShRow {
    T c[SS_SHEXP_LMAX + 1], s[SS_SHEXP_LMAX + 1];
};

// {Re, Im} R_l^m of a row of degree l for any m (R_l^{-m} = (-1)^m conj R_l^m)
template <class T>
__device__ __forceinline__ T row_c(const ShRow<T>& R, int l, int m) {
    if (l < 0 || m > l || -m > l) return T(0);
    if (m >= 0) return R.c[m];
    return (m & 1) ? T(0) - R.c[-m] : R.c[-m];
}
template <class T>
__device__ __forceinline__ T row_s(const ShRow<T>& R, int l, int m) {
    if (l < 0 || m > l || -m > l) return T(0);
    if (m >= 0) return R.s[m];
    return (m & 1) ? R.s[-m] : T(0) - R.s[-m];
}

template <class T, class R, bool HESS>
__device__ __forceinline__ void shexp_grad_impl(const ExpDev& E, const R scale, const T x[3], T grad[3], T H[6]) {
    constexpr int LM = SS_SHEXP_LMAX;
    constexpr int UR = ShUnroll<T>::n;
    const int L = E.lmax;
    const int nt = (L + 1) * (L + 1);
    T r2 = x[0] * x[0] + x[1] * x[1] + x[2] * x[2];
    T ir = s_rsqrt(r2);
    T r = r2 * ir;
    T n[3] = {x[0] * ir, x[1] * ir, x[2] * ir};
    RadialBasis<T> B;
    radial_basis<T>(E, s_log(r), B);
    const T idu = T(E.inv_du);
    ShRow<T> R0, R1, R2;  // degrees l, l-1, l-2 (at the unit vector, r = 1)
#pragma unroll UR
    for (int m = 0; m <= LM; ++m) {
        R0.c[m] = R0.s[m] = R1.c[m] = R1.s[m] = R2.c[m] = R2.s[m] = T(0);
    }
    R0.c[0] = T(1);
    T S1(0), S2(0), V[3] = {T(0), T(0), T(0)}, W[3] = {T(0), T(0), T(0)};
    T M[6] = {T(0), T(0), T(0), T(0), T(0), T(0)};
#pragma unroll UR
    for (int l = 0; l <= LM; ++l) {
        if (l > L) break;
        if (l > 0) {
#pragma unroll UR
            for (int m = 0; m < l; ++m) {
                R2.c[m] = R1.c[m];
                R2.s[m] = R1.s[m];
                R1.c[m] = R0.c[m];
                R1.s[m] = R0.s[m];
            }
#pragma unroll UR
            for (int m = 0; m + 2 <= l; ++m) {
                const T a = T((2.0 * l - 1.0) / ((double)(l - m) * (l + m)));
                const T b = T(1.0 / ((double)(l - m) * (l + m)));
                R0.c[m] = a * n[2] * R1.c[m] - b * R2.c[m];
                R0.s[m] = a * n[2] * R1.s[m] - b * R2.s[m];
            }
            R0.c[l - 1] = n[2] * R1.c[l - 1];
            R0.s[l - 1] = n[2] * R1.s[l - 1];
            const T f = T(1.0 / (2.0 * l));
            R0.c[l] = (n[0] * R1.c[l - 1] - n[1] * R1.s[l - 1]) * f;
            R0.s[l] = (n[0] * R1.s[l - 1] + n[1] * R1.c[l - 1]) * f;
        }
        const T fl = T((double)l);
#pragma unroll UR
        for (int mm = -l; mm <= l; ++mm) {
            const int m = mm < 0 ? -mm : mm;
            const bool cs = mm >= 0;  // cos part (Re) or sin part (Im)
            const T N = T(c_shnorm[l][m]);
            T f, fs, fss;
            radial_term<T>(E, B, nt, l * l + l + mm, f, fs, fss);
            // radial derivatives in r: a1 = f_u / r, a2 = (f_uu - f_u) / r^2
            const T fu = fs * idu;
            const T a0 = f * N;
            const T a1 = fu * ir * N;
            const T G1 = a1 - fl * a0 * ir;
            const T K = cs ? R0.c[m] : R0.s[m];
            S1 += G1 * K;
            // grad of {Re, Im} R_l^m at n, from degree l-1
            T gk[3];
            if (cs) {
                gk[0] = T(0.5) * (row_c(R1, l - 1, m - 1) - row_c(R1, l - 1, m + 1));
                gk[1] = T(0) - T(0.5) * (row_s(R1, l - 1, m + 1) + row_s(R1, l - 1, m - 1));
                gk[2] = row_c(R1, l - 1, m);
            } else {
                gk[0] = T(0.5) * (row_s(R1, l - 1, m - 1) - row_s(R1, l - 1, m + 1));
                gk[1] = T(0.5) * (row_c(R1, l - 1, m + 1) + row_c(R1, l - 1, m - 1));
                gk[2] = row_s(R1, l - 1, m);
            }
            V[0] += a0 * gk[0];
            V[1] += a0 * gk[1];
            V[2] += a0 * gk[2];
            if constexpr (HESS) {
                const T fuu = fss * idu * idu;
                const T a2 = (fuu - fu) * ir * ir * N;
                const T G2 = a2 - T(2.0) * fl * a1 * ir + fl * (fl + T(1)) * a0 * ir * ir;
                S2 += G2 * K;
                W[0] += G1 * gk[0];
                W[1] += G1 * gk[1];
                W[2] += G1 * gk[2];
                // Hessian of R_l^m from degree l-2: xx (Q_{m-2} - 2Q_m + Q_{m+2})/4,
                // yy -(Q_{m+2} + 2Q_m + Q_{m-2})/4, zz Q_m, xy i(Q_{m-2} - Q_{m+2})/4,
                // xz (Q_{m-1} - Q_{m+1})/2, yz i(Q_{m+1} + Q_{m-1})/2
                const int k2 = l - 2;
                T hk[6];
                if (cs) {
                    hk[0] = T(0.25) * (row_c(R2, k2, m - 2) - T(2) * row_c(R2, k2, m) + row_c(R2, k2, m + 2));
                    hk[1] = T(0) - T(0.25) * (row_c(R2, k2, m + 2) + T(2) * row_c(R2, k2, m) + row_c(R2, k2, m - 2));
                    hk[2] = row_c(R2, k2, m);
                    hk[3] = T(0) - T(0.25) * (row_s(R2, k2, m - 2) - row_s(R2, k2, m + 2));
                    hk[4] = T(0.5) * (row_c(R2, k2, m - 1) - row_c(R2, k2, m + 1));
                    hk[5] = T(0) - T(0.5) * (row_s(R2, k2, m + 1) + row_s(R2, k2, m - 1));
                } else {
                    hk[0] = T(0.25) * (row_s(R2, k2, m - 2) - T(2) * row_s(R2, k2, m) + row_s(R2, k2, m + 2));
                    hk[1] = T(0) - T(0.25) * (row_s(R2, k2, m + 2) + T(2) * row_s(R2, k2, m) + row_s(R2, k2, m - 2));
                    hk[2] = row_s(R2, k2, m);
                    hk[3] = T(0.25) * (row_c(R2, k2, m - 2) - row_c(R2, k2, m + 2));
                    hk[4] = T(0.5) * (row_s(R2, k2, m - 1) - row_s(R2, k2, m + 1));
                    hk[5] = T(0.5) * (row_c(R2, k2, m + 1) + row_c(R2, k2, m - 1));
                }
#pragma unroll
                for (int i = 0; i < 6; ++i) M[i] += a0 * hk[i];
            }
        }
    }
    const T sc = T(scale);
    grad[0] += sc * (S1 * n[0] + V[0] * ir);
    grad[1] += sc * (S1 * n[1] + V[1] * ir);
    grad[2] += sc * (S1 * n[2] + V[2] * ir);
    if constexpr (HESS) {
        const int ia[6] = {0, 1, 2, 0, 0, 1}, ib[6] = {0, 1, 2, 1, 2, 2};
        const T Sr = S1 * ir, ir2 = ir * ir;
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            const int a = ia[q], b = ib[q];
            T v = S2 * n[a] * n[b] - Sr * n[a] * n[b] + (n[a] * W[b] + W[a] * n[b]) * ir + M[q] * ir2;
            if (a == b) v += Sr;
            H[q] += sc * v;
        }
    }
}

// Out-of-line entry points: the expansion is ~2000 instructions, so the
// stage loops call it instead of inlining it six times.  The gradient-only
// forms pass the position by value so that it stays in registers.
template <class S>
struct Vec3 {
    S x, y, z;
};

template <class S>
__device__ __noinline__ Vec3<S> shexp_grad_value(const ExpDev E, S scale, S x0, S x1, S x2) {
    const S x[3] = {x0, x1, x2};
    S g[3] = {S(0), S(0), S(0)};
    shexp_grad_impl<S, S, false>(E, scale, x, g, nullptr);
    return Vec3<S>{g[0], g[1], g[2]};
}

// ------------------------------------ expansion gradient for FP32 streams
// The stream integrator calls this form: each thread keeps its solid
// harmonics R_l^m(n) in a column of shared memory (slot 2q, 2q+1 = Re, Im
// of q = l(l+1)/2 + m; slot 90 = 0) and one rolled loop runs over the terms,
// reading each term's slots and coefficients (normalisation and the
// derivative rules folded in) from constant memory.  Small code, no
// dynamically indexed registers.  Term j: K = cK R[sK],
// grad K = (cx1 R[sx1] + cx2 R[sx2], cy1 R[sy1] + cy2 R[sy2], cz R[sz]).
static __constant__ short4 c_shterm_i[81][2] = {
    {{0, 90, 90, 90}, {90, 90, 0, 0}},
    {{5, 1, 90, 90}, {0, 90, 1, 0}},
    {{2, 90, 90, 90}, {90, 0, 1, 0}},
    {{4, 0, 90, 90}, {1, 90, 1, 0}},
    {{11, 5, 90, 90}, {4, 90, 2, 0}},
    {{9, 3, 90, 90}, {2, 5, 2, 0}},
    {{6, 4, 4, 5}, {5, 2, 2, 0}},
    {{8, 2, 90, 90}, {3, 4, 2, 0}},
    {{10, 4, 90, 90}, {5, 90, 2, 0}},
    {{19, 11, 90, 90}, {10, 90, 3, 0}},
    {{17, 9, 90, 90}, {8, 11, 3, 0}},
    {{15, 7, 11, 10}, {6, 9, 3, 0}},
    {{12, 8, 8, 9}, {9, 6, 3, 0}},
    {{14, 6, 10, 11}, {7, 8, 3, 0}},
    {{16, 8, 90, 90}, {9, 10, 3, 0}},
    {{18, 10, 90, 90}, {11, 90, 3, 0}},
    {{29, 19, 90, 90}, {18, 90, 4, 0}},
    {{27, 17, 90, 90}, {16, 19, 4, 0}},
    {{25, 15, 19, 18}, {14, 17, 4, 0}},
    {{23, 13, 17, 16}, {12, 15, 4, 0}},
    {{20, 14, 14, 15}, {15, 12, 4, 0}},
    {{22, 12, 16, 17}, {13, 14, 4, 0}},
    {{24, 14, 18, 19}, {15, 16, 4, 0}},
    {{26, 16, 90, 90}, {17, 18, 4, 0}},
    {{28, 18, 90, 90}, {19, 90, 4, 0}},
    {{41, 29, 90, 90}, {28, 90, 5, 0}},
    {{39, 27, 90, 90}, {26, 29, 5, 0}},
    {{37, 25, 29, 28}, {24, 27, 5, 0}},
    {{35, 23, 27, 26}, {22, 25, 5, 0}},
    {{33, 21, 25, 24}, {20, 23, 5, 0}},
    {{30, 22, 22, 23}, {23, 20, 5, 0}},
    {{32, 20, 24, 25}, {21, 22, 5, 0}},
    {{34, 22, 26, 27}, {23, 24, 5, 0}},
    {{36, 24, 28, 29}, {25, 26, 5, 0}},
    {{38, 26, 90, 90}, {27, 28, 5, 0}},
    {{40, 28, 90, 90}, {29, 90, 5, 0}},
    {{55, 41, 90, 90}, {40, 90, 6, 0}},
    {{53, 39, 90, 90}, {38, 41, 6, 0}},
    {{51, 37, 41, 40}, {36, 39, 6, 0}},
    {{49, 35, 39, 38}, {34, 37, 6, 0}},
    {{47, 33, 37, 36}, {32, 35, 6, 0}},
    {{45, 31, 35, 34}, {30, 33, 6, 0}},
    {{42, 32, 32, 33}, {33, 30, 6, 0}},
    {{44, 30, 34, 35}, {31, 32, 6, 0}},
    {{46, 32, 36, 37}, {33, 34, 6, 0}},
    {{48, 34, 38, 39}, {35, 36, 6, 0}},
    {{50, 36, 40, 41}, {37, 38, 6, 0}},
    {{52, 38, 90, 90}, {39, 40, 6, 0}},
    {{54, 40, 90, 90}, {41, 90, 6, 0}},
    {{71, 55, 90, 90}, {54, 90, 7, 0}},
    {{69, 53, 90, 90}, {52, 55, 7, 0}},
    {{67, 51, 55, 54}, {50, 53, 7, 0}},
    {{65, 49, 53, 52}, {48, 51, 7, 0}},
    {{63, 47, 51, 50}, {46, 49, 7, 0}},
    {{61, 45, 49, 48}, {44, 47, 7, 0}},
    {{59, 43, 47, 46}, {42, 45, 7, 0}},
    {{56, 44, 44, 45}, {45, 42, 7, 0}},
    {{58, 42, 46, 47}, {43, 44, 7, 0}},
    {{60, 44, 48, 49}, {45, 46, 7, 0}},
    {{62, 46, 50, 51}, {47, 48, 7, 0}},
    {{64, 48, 52, 53}, {49, 50, 7, 0}},
    {{66, 50, 54, 55}, {51, 52, 7, 0}},
    {{68, 52, 90, 90}, {53, 54, 7, 0}},
    {{70, 54, 90, 90}, {55, 90, 7, 0}},
    {{89, 71, 90, 90}, {70, 90, 8, 0}},
    {{87, 69, 90, 90}, {68, 71, 8, 0}},
    {{85, 67, 71, 70}, {66, 69, 8, 0}},
    {{83, 65, 69, 68}, {64, 67, 8, 0}},
    {{81, 63, 67, 66}, {62, 65, 8, 0}},
    {{79, 61, 65, 64}, {60, 63, 8, 0}},
    {{77, 59, 63, 62}, {58, 61, 8, 0}},
    {{75, 57, 61, 60}, {56, 59, 8, 0}},
    {{72, 58, 58, 59}, {59, 56, 8, 0}},
    {{74, 56, 60, 61}, {57, 58, 8, 0}},
    {{76, 58, 62, 63}, {59, 60, 8, 0}},
    {{78, 60, 64, 65}, {61, 62, 8, 0}},
    {{80, 62, 66, 67}, {63, 64, 8, 0}},
    {{82, 64, 68, 69}, {65, 66, 8, 0}},
    {{84, 66, 70, 71}, {67, 68, 8, 0}},
    {{86, 68, 90, 90}, {69, 70, 8, 0}},
    {{88, 70, 90, 90}, {71, 90, 8, 0}}};
static __constant__ float c_shterm_f[81][6] = {
    {1.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f},
    {2.000000000e+00f, 1.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f, 1.000000000e+00f, 0.000000000e+00f},
    {1.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f, 1.000000000e+00f},
    {2.000000000e+00f, 1.000000000e+00f, 0.000000000e+00f, 0.000000000e+00f, -1.000000000e+00f, 0.000000000e+00f},
    {6.928203230e+00f, 3.464101615e+00f, 0.000000000e+00f, 0.000000000e+00f, 3.464101615e+00f, 0.000000000e+00f},
    {3.464101615e+00f, 1.732050808e+00f, 0.000000000e+00f, 0.000000000e+00f, 1.732050808e+00f, 3.464101615e+00f},
    {2.000000000e+00f, -1.000000000e+00f, -1.000000000e+00f, -1.000000000e+00f, -1.000000000e+00f, 2.000000000e+00f},
    {3.464101615e+00f, 1.732050808e+00f, 0.000000000e+00f, 0.000000000e+00f, -1.732050808e+00f, 3.464101615e+00f},
    {6.928203230e+00f, 3.464101615e+00f, 0.000000000e+00f, 0.000000000e+00f, -3.464101615e+00f, 0.000000000e+00f},
    {3.794733192e+01f, 1.897366596e+01f, 0.000000000e+00f, 0.000000000e+00f, 1.897366596e+01f, 0.000000000e+00f},
    {1.549193338e+01f, 7.745966692e+00f, 0.000000000e+00f, 0.000000000e+00f, 7.745966692e+00f, 1.549193338e+01f},
    {9.797958971e+00f, 4.898979486e+00f, -4.898979486e+00f, 4.898979486e+00f, 4.898979486e+00f, 9.797958971e+00f},
    {6.000000000e+00f, -3.000000000e+00f, -3.000000000e+00f, -3.000000000e+00f, -3.000000000e+00f, 6.000000000e+00f},
    {9.797958971e+00f, 4.898979486e+00f, -4.898979486e+00f, -4.898979486e+00f, -4.898979486e+00f, 9.797958971e+00f},
    {1.549193338e+01f, 7.745966692e+00f, 0.000000000e+00f, 0.000000000e+00f, -7.745966692e+00f, 1.549193338e+01f},
    {3.794733192e+01f, 1.897366596e+01f, 0.000000000e+00f, 0.000000000e+00f, -1.897366596e+01f, 0.000000000e+00f},
    {2.839718296e+02f, 1.419859148e+02f, 0.000000000e+00f, 0.000000000e+00f, 1.419859148e+02f, 0.000000000e+00f},
    {1.003992032e+02f, 5.019960159e+01f, 0.000000000e+00f, 0.000000000e+00f, 5.019960159e+01f, 1.003992032e+02f},
    {5.366563146e+01f, 2.683281573e+01f, -2.683281573e+01f, 2.683281573e+01f, 2.683281573e+01f, 5.366563146e+01f},
    {3.794733192e+01f, 1.897366596e+01f, -1.897366596e+01f, 1.897366596e+01f, 1.897366596e+01f, 3.794733192e+01f},
    {2.400000000e+01f, -1.200000000e+01f, -1.200000000e+01f, -1.200000000e+01f, -1.200000000e+01f, 2.400000000e+01f},
    {3.794733192e+01f, 1.897366596e+01f, -1.897366596e+01f, -1.897366596e+01f, -1.897366596e+01f, 3.794733192e+01f},
    {5.366563146e+01f, 2.683281573e+01f, -2.683281573e+01f, -2.683281573e+01f, -2.683281573e+01f, 5.366563146e+01f},
    {1.003992032e+02f, 5.019960159e+01f, 0.000000000e+00f, 0.000000000e+00f, -5.019960159e+01f, 1.003992032e+02f},
    {2.839718296e+02f, 1.419859148e+02f, 0.000000000e+00f, 0.000000000e+00f, -1.419859148e+02f, 0.000000000e+00f},
    {2.693993318e+03f, 1.346996659e+03f, 0.000000000e+00f, 0.000000000e+00f, 1.346996659e+03f, 0.000000000e+00f},
    {8.519154888e+02f, 4.259577444e+02f, 0.000000000e+00f, 0.000000000e+00f, 4.259577444e+02f, 8.519154888e+02f},
    {4.015968127e+02f, 2.007984064e+02f, -2.007984064e+02f, 2.007984064e+02f, 2.007984064e+02f, 4.015968127e+02f},
    {2.459268184e+02f, 1.229634092e+02f, -1.229634092e+02f, 1.229634092e+02f, 1.229634092e+02f, 2.459268184e+02f},
    {1.859032006e+02f, 9.295160031e+01f, -9.295160031e+01f, 9.295160031e+01f, 9.295160031e+01f, 1.859032006e+02f},
    {1.200000000e+02f, -6.000000000e+01f, -6.000000000e+01f, -6.000000000e+01f, -6.000000000e+01f, 1.200000000e+02f},
    {1.859032006e+02f, 9.295160031e+01f, -9.295160031e+01f, -9.295160031e+01f, -9.295160031e+01f, 1.859032006e+02f},
    {2.459268184e+02f, 1.229634092e+02f, -1.229634092e+02f, -1.229634092e+02f, -1.229634092e+02f, 2.459268184e+02f},
    {4.015968127e+02f, 2.007984064e+02f, -2.007984064e+02f, -2.007984064e+02f, -2.007984064e+02f, 4.015968127e+02f},
    {8.519154888e+02f, 4.259577444e+02f, 0.000000000e+00f, 0.000000000e+00f, -4.259577444e+02f, 8.519154888e+02f},
    {2.693993318e+03f, 1.346996659e+03f, 0.000000000e+00f, 0.000000000e+00f, -1.346996659e+03f, 0.000000000e+00f},
    {3.095162677e+04f, 1.547581339e+04f, 0.000000000e+00f, 0.000000000e+00f, 1.547581339e+04f, 0.000000000e+00f},
    {8.934965025e+03f, 4.467482513e+03f, 0.000000000e+00f, 0.000000000e+00f, 4.467482513e+03f, 8.934965025e+03f},
    {3.809881888e+03f, 1.904940944e+03f, -1.904940944e+03f, 1.904940944e+03f, 1.904940944e+03f, 3.809881888e+03f},
    {2.086758251e+03f, 1.043379126e+03f, -1.043379126e+03f, 1.043379126e+03f, 1.043379126e+03f, 2.086758251e+03f},
    {1.391172168e+03f, 6.955860838e+02f, -6.955860838e+02f, 6.955860838e+02f, 6.955860838e+02f, 1.391172168e+03f},
    {1.099818167e+03f, 5.499090834e+02f, -5.499090834e+02f, 5.499090834e+02f, 5.499090834e+02f, 1.099818167e+03f},
    {7.200000000e+02f, -3.600000000e+02f, -3.600000000e+02f, -3.600000000e+02f, -3.600000000e+02f, 7.200000000e+02f},
    {1.099818167e+03f, 5.499090834e+02f, -5.499090834e+02f, -5.499090834e+02f, -5.499090834e+02f, 1.099818167e+03f},
    {1.391172168e+03f, 6.955860838e+02f, -6.955860838e+02f, -6.955860838e+02f, -6.955860838e+02f, 1.391172168e+03f},
    {2.086758251e+03f, 1.043379126e+03f, -1.043379126e+03f, -1.043379126e+03f, -1.043379126e+03f, 2.086758251e+03f},
    {3.809881888e+03f, 1.904940944e+03f, -1.904940944e+03f, -1.904940944e+03f, -1.904940944e+03f, 3.809881888e+03f},
    {8.934965025e+03f, 4.467482513e+03f, 0.000000000e+00f, 0.000000000e+00f, -4.467482513e+03f, 8.934965025e+03f},
    {3.095162677e+04f, 1.547581339e+04f, 0.000000000e+00f, 0.000000000e+00f, -1.547581339e+04f, 0.000000000e+00f},
    {4.175602740e+05f, 2.087801370e+05f, 0.000000000e+00f, 0.000000000e+00f, 2.087801370e+05f, 0.000000000e+00f},
    {1.115976774e+05f, 5.579883870e+04f, 0.000000000e+00f, 0.000000000e+00f, 5.579883870e+04f, 1.115976774e+05f},
    {4.377221036e+04f, 2.188610518e+04f, -2.188610518e+04f, 2.188610518e+04f, 2.188610518e+04f, 4.377221036e+04f},
    {2.188610518e+04f, 1.094305259e+04f, -1.094305259e+04f, 1.094305259e+04f, 1.094305259e+04f, 2.188610518e+04f},
    {1.319781800e+04f, 6.598909001e+03f, -6.598909001e+03f, 6.598909001e+03f, 6.598909001e+03f, 1.319781800e+04f},
    {9.332266606e+03f, 4.666133303e+03f, -4.666133303e+03f, 4.666133303e+03f, 4.666133303e+03f, 9.332266606e+03f},
    {7.619763776e+03f, 3.809881888e+03f, -3.809881888e+03f, 3.809881888e+03f, 3.809881888e+03f, 7.619763776e+03f},
    {5.040000000e+03f, -2.520000000e+03f, -2.520000000e+03f, -2.520000000e+03f, -2.520000000e+03f, 5.040000000e+03f},
    {7.619763776e+03f, 3.809881888e+03f, -3.809881888e+03f, -3.809881888e+03f, -3.809881888e+03f, 7.619763776e+03f},
    {9.332266606e+03f, 4.666133303e+03f, -4.666133303e+03f, -4.666133303e+03f, -4.666133303e+03f, 9.332266606e+03f},
    {1.319781800e+04f, 6.598909001e+03f, -6.598909001e+03f, -6.598909001e+03f, -6.598909001e+03f, 1.319781800e+04f},
    {2.188610518e+04f, 1.094305259e+04f, -1.094305259e+04f, -1.094305259e+04f, -1.094305259e+04f, 2.188610518e+04f},
    {4.377221036e+04f, 2.188610518e+04f, -2.188610518e+04f, -2.188610518e+04f, -2.188610518e+04f, 4.377221036e+04f},
    {1.115976774e+05f, 5.579883870e+04f, 0.000000000e+00f, 0.000000000e+00f, -5.579883870e+04f, 1.115976774e+05f},
    {4.175602740e+05f, 2.087801370e+05f, 0.000000000e+00f, 0.000000000e+00f, -2.087801370e+05f, 0.000000000e+00f},
    {6.468815949e+06f, 3.234407974e+06f, 0.000000000e+00f, 0.000000000e+00f, 3.234407974e+06f, 0.000000000e+00f},
    {1.617203987e+06f, 8.086019936e+05f, 0.000000000e+00f, 0.000000000e+00f, 8.086019936e+05f, 1.617203987e+06f},
    {5.905194026e+05f, 2.952597013e+05f, -2.952597013e+05f, 2.952597013e+05f, 2.952597013e+05f, 5.905194026e+05f},
    {2.733573661e+05f, 1.366786830e+05f, -1.366786830e+05f, 1.366786830e+05f, 1.366786830e+05f, 2.733573661e+05f},
    {1.516313846e+05f, 7.581569231e+04f, -7.581569231e+04f, 7.581569231e+04f, 7.581569231e+04f, 1.516313846e+05f},
    {9.787763790e+04f, 4.893881895e+04f, -4.893881895e+04f, 4.893881895e+04f, 4.893881895e+04f, 9.787763790e+04f},
    {7.228742629e+04f, 3.614371315e+04f, -3.614371315e+04f, 3.614371315e+04f, 3.614371315e+04f, 7.228742629e+04f},
    {6.048000000e+04f, 3.024000000e+04f, -3.024000000e+04f, 3.024000000e+04f, 3.024000000e+04f, 6.048000000e+04f},
    {4.032000000e+04f, -2.016000000e+04f, -2.016000000e+04f, -2.016000000e+04f, -2.016000000e+04f, 4.032000000e+04f},
    {6.048000000e+04f, 3.024000000e+04f, -3.024000000e+04f, -3.024000000e+04f, -3.024000000e+04f, 6.048000000e+04f},
    {7.228742629e+04f, 3.614371315e+04f, -3.614371315e+04f, -3.614371315e+04f, -3.614371315e+04f, 7.228742629e+04f},
    {9.787763790e+04f, 4.893881895e+04f, -4.893881895e+04f, -4.893881895e+04f, -4.893881895e+04f, 9.787763790e+04f},
    {1.516313846e+05f, 7.581569231e+04f, -7.581569231e+04f, -7.581569231e+04f, -7.581569231e+04f, 1.516313846e+05f},
    {2.733573661e+05f, 1.366786830e+05f, -1.366786830e+05f, -1.366786830e+05f, -1.366786830e+05f, 2.733573661e+05f},
    {5.905194026e+05f, 2.952597013e+05f, -2.952597013e+05f, -2.952597013e+05f, -2.952597013e+05f, 5.905194026e+05f},
    {1.617203987e+06f, 8.086019936e+05f, 0.000000000e+00f, 0.000000000e+00f, -8.086019936e+05f, 1.617203987e+06f},
    {6.468815949e+06f, 3.234407974e+06f, 0.000000000e+00f, 0.000000000e+00f, -3.234407974e+06f, 0.000000000e+00f}};
static __constant__ float c_shrec[9][9][2] = {
    {{0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}},
    {{0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}},
    {{7.500000000e-01f, 2.500000000e-01f}, {0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}},
    {{5.555555556e-01f, 1.111111111e-01f}, {6.250000000e-01f, 1.250000000e-01f}, {0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}},
    {{4.375000000e-01f, 6.250000000e-02f}, {4.666666667e-01f, 6.666666667e-02f}, {5.833333333e-01f, 8.333333333e-02f}, {0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}},
    {{3.600000000e-01f, 4.000000000e-02f}, {3.750000000e-01f, 4.166666667e-02f}, {4.285714286e-01f, 4.761904762e-02f}, {5.625000000e-01f, 6.250000000e-02f}, {0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}},
    {{3.055555556e-01f, 2.777777778e-02f}, {3.142857143e-01f, 2.857142857e-02f}, {3.437500000e-01f, 3.125000000e-02f}, {4.074074074e-01f, 3.703703704e-02f}, {5.500000000e-01f, 5.000000000e-02f}, {0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}},
    {{2.653061224e-01f, 2.040816327e-02f}, {2.708333333e-01f, 2.083333333e-02f}, {2.888888889e-01f, 2.222222222e-02f}, {3.250000000e-01f, 2.500000000e-02f}, {3.939393939e-01f, 3.030303030e-02f}, {5.416666667e-01f, 4.166666667e-02f}, {0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}},
    {{2.343750000e-01f, 1.562500000e-02f}, {2.380952381e-01f, 1.587301587e-02f}, {2.500000000e-01f, 1.666666667e-02f}, {2.727272727e-01f, 1.818181818e-02f}, {3.125000000e-01f, 2.083333333e-02f}, {3.846153846e-01f, 2.564102564e-02f}, {5.357142857e-01f, 3.571428571e-02f}, {0.0f, 0.0f}, {0.0f, 0.0f}}};
static __constant__ float c_shinv2l[9] = {0.0f, 5.000000000e-01f, 2.500000000e-01f, 1.666666667e-01f, 1.250000000e-01f, 1.000000000e-01f, 8.333333333e-02f, 7.142857143e-02f, 6.250000000e-02f};
static constexpr int SH_COLS = 128, SH_SLOTS = 91;

static __device__ __noinline__ Vec3<float> shexp_grad_smem(const ExpDev E, float scale, float x0, float x1, float x2) {
    __shared__ float shcol[SH_SLOTS * SH_COLS];
    float* col = shcol + threadIdx.x;
#define SH_(s) col[(s) * SH_COLS]
    const int L = E.lmax;
    const int nt = (L + 1) * (L + 1);
    const float r2 = x0 * x0 + x1 * x1 + x2 * x2;
    const float ir = s_rsqrt(r2);
    const float r = r2 * ir;
    const float n0 = x0 * ir, n1 = x1 * ir, n2 = x2 * ir;
    SH_(90) = 0.0f;
    SH_(0) = 1.0f;
    SH_(1) = 0.0f;
#pragma unroll 1
    for (int l = 1; l <= L; ++l) {
        const int qp = (l - 1) * l / 2, q0 = l * (l + 1) / 2;  // rows l-1 and l
        const float cpp = SH_(2 * (qp + l - 1)), spp = SH_(2 * (qp + l - 1) + 1);
        const float f = c_shinv2l[l];
        SH_(2 * (q0 + l)) = (n0 * cpp - n1 * spp) * f;
        SH_(2 * (q0 + l) + 1) = (n0 * spp + n1 * cpp) * f;
        SH_(2 * (q0 + l - 1)) = n2 * cpp;
        SH_(2 * (q0 + l - 1) + 1) = n2 * spp;
        const int qpp = (l - 2) * (l - 1) / 2;  // row l-2
#pragma unroll 1
        for (int m = 0; m + 2 <= l; ++m) {
            const float a = c_shrec[l][m][0] * n2, b = c_shrec[l][m][1];
            SH_(2 * (q0 + m)) = a * SH_(2 * (qp + m)) - b * SH_(2 * (qpp + m));
            SH_(2 * (q0 + m) + 1) = a * SH_(2 * (qp + m) + 1) - b * SH_(2 * (qpp + m) + 1);
        }
    }
    RadialBasis<float> B;
    radial_basis<float>(E, s_log(r), B);
    const float idu = (float)E.inv_du;
    float S1 = 0.0f, V0 = 0.0f, V1 = 0.0f, V2 = 0.0f;
#pragma unroll 2
    for (int j = 0; j < nt; ++j) {
        const short4 i0 = c_shterm_i[j][0], i1 = c_shterm_i[j][1];
        float f, fs, fss;
        radial_term<float>(E, B, nt, j, f, fs, fss);
        const float a1 = fs * idu * ir;
        const float G1 = a1 - (float)i1.z * f * ir;
        S1 = fmaf(G1, c_shterm_f[j][0] * SH_(i0.x), S1);
        const float gx = c_shterm_f[j][1] * SH_(i0.y) + c_shterm_f[j][2] * SH_(i0.z);
        const float gy = c_shterm_f[j][3] * SH_(i0.w) + c_shterm_f[j][4] * SH_(i1.x);
        const float gz = c_shterm_f[j][5] * SH_(i1.y);
        V0 = fmaf(f, gx, V0);
        V1 = fmaf(f, gy, V1);
        V2 = fmaf(f, gz, V2);
    }
#undef SH_
    return Vec3<float>{scale * (S1 * n0 + V0 * ir), scale * (S1 * n1 + V1 * ir), scale * (S1 * n2 + V2 * ir)};
}

// Straight-line FP32 form for a compile-time degree L (the stream's common
// case, l_max = 8, with the FP32 interval table): every harmonic and term
// index is a compile-time constant, so the rows live in registers and each
// term is one float4 load plus ~30 FP32 operations.
template <int L>
static __device__ __noinline__ Vec3<float> shexp_grad_fixed(const ExpDev E, float scale, float x0, float x1, float x2) {
    constexpr int nt = (L + 1) * (L + 1);
    const float r2 = x0 * x0 + x1 * x1 + x2 * x2;
    const float ir = s_rsqrt(r2);
    const float r = r2 * ir;
    const float n[3] = {x0 * ir, x1 * ir, x2 * ir};
    RadialBasis<float> B;
    radial_basis<float>(E, s_log(r), B);
    const float4* tab = E.tab32 + (size_t)B.k * nt;
    const float idu = (float)E.inv_du;
    float R0c[L + 1], R0s[L + 1], R1c[L + 1], R1s[L + 1], R2c[L + 1], R2s[L + 1];
#pragma unroll
    for (int m = 0; m <= L; ++m) R0c[m] = R0s[m] = R1c[m] = R1s[m] = R2c[m] = R2s[m] = 0.0f;
    R0c[0] = 1.0f;
    float S1 = 0.0f, V0 = 0.0f, V1 = 0.0f, V2 = 0.0f;
#pragma unroll
    for (int l = 0; l <= L; ++l) {
        if (l > 0) {
#pragma unroll
            for (int m = 0; m < l; ++m) {
                R2c[m] = R1c[m];
                R2s[m] = R1s[m];
                R1c[m] = R0c[m];
                R1s[m] = R0s[m];
            }
#pragma unroll
            for (int m = 0; m + 2 <= l; ++m) {
                const float a = (float)((2.0 * l - 1.0) / ((double)(l - m) * (l + m)));
                const float b = (float)(1.0 / ((double)(l - m) * (l + m)));
                R0c[m] = a * n[2] * R1c[m] - b * R2c[m];
                R0s[m] = a * n[2] * R1s[m] - b * R2s[m];
            }
            R0c[l - 1] = n[2] * R1c[l - 1];
            R0s[l - 1] = n[2] * R1s[l - 1];
            const float f = (float)(1.0 / (2.0 * l));
            R0c[l] = (n[0] * R1c[l - 1] - n[1] * R1s[l - 1]) * f;
            R0s[l] = (n[0] * R1s[l - 1] + n[1] * R1c[l - 1]) * f;
        }
        // {Re, Im} of the degree-(l-1) row at any m (R^{-m} = (-1)^m conj R^m)
        auto c1 = [&](int m) -> float {
            if (m > l - 1 || -m > l - 1) return 0.0f;
            return m >= 0 ? R1c[m] : ((m & 1) ? -R1c[-m] : R1c[-m]);
        };
        auto s1 = [&](int m) -> float {
            if (m > l - 1 || -m > l - 1) return 0.0f;
            return m >= 0 ? R1s[m] : ((m & 1) ? R1s[-m] : -R1s[-m]);
        };
        const float fl = (float)l;
#pragma unroll
        for (int mm = -l; mm <= l; ++mm) {
            const int m = mm < 0 ? -mm : mm;
            const float N = (float)shnorm_ct(l, m);
            const float4 t = __ldg(tab + (l * l + l + mm));
            const float fs = B.hs[0] * t.x + B.hs[1] * t.y + B.hs[2] * t.z + B.hs[3] * t.w;
            const float f = B.h[0] * t.x + B.h[1] * t.y + B.h[2] * t.z + B.h[3] * t.w + B.e * fs;
            const float G1 = (fs * idu - fl * f) * ir;
            float K, g0, g1, g2;
            if (mm >= 0) {
                K = R0c[m];
                g0 = 0.5f * (c1(m - 1) - c1(m + 1));
                g1 = -0.5f * (s1(m + 1) + s1(m - 1));
                g2 = c1(m);
            } else {
                K = R0s[m];
                g0 = 0.5f * (s1(m - 1) - s1(m + 1));
                g1 = 0.5f * (c1(m + 1) + c1(m - 1));
                g2 = s1(m);
            }
            const float fN = f * N;
            S1 = fmaf(G1 * N, K, S1);
            V0 = fmaf(fN, g0, V0);
            V1 = fmaf(fN, g1, V1);
            V2 = fmaf(fN, g2, V2);
        }
    }
    return Vec3<float>{scale * (S1 * n[0] + V0 * ir), scale * (S1 * n[1] + V1 * ir), scale * (S1 * n[2] + V2 * ir)};
}

template <class T, class R, bool HESS>
__device__ __noinline__ void shexp_grad_ref(const ExpDev& E, const R scale, const T x[3], T grad[3], T H[6]) {
    shexp_grad_impl<T, R, HESS>(E, scale, x, grad, H);
}

template <class T, class R, bool HESS>
__device__ __forceinline__ void shexp_grad(const ExpDev& E, const R scale, const T x[3], T grad[3], T H[6]) {
    if constexpr (std::is_same<T, float>::value && std::is_same<T, R>::value && !HESS) {
        if (E.lmax == SS_SHEXP_LMAX && E.tab32 != nullptr) {
            const Vec3<float> g = shexp_grad_fixed<SS_SHEXP_LMAX>(E, scale, x[0], x[1], x[2]);
            grad[0] += g.x;
            grad[1] += g.y;
            grad[2] += g.z;
        } else if (blockDim.x <= SH_COLS) {
            const Vec3<float> g = shexp_grad_smem(E, scale, x[0], x[1], x[2]);
            grad[0] += g.x;
            grad[1] += g.y;
            grad[2] += g.z;
        } else {
            shexp_grad_ref<T, R, HESS>(E, scale, x, grad, H);
        }
    } else if constexpr (std::is_floating_point<T>::value && std::is_same<T, R>::value && !HESS) {
        const Vec3<T> g = shexp_grad_value<T>(E, scale, x[0], x[1], x[2]);
        grad[0] += g.x;
        grad[1] += g.y;
        grad[2] += g.z;
    } else {
        shexp_grad_ref<T, R, HESS>(E, scale, x, grad, H);
    }
}

// Phi of the expansion (FP64; potential evaluation only).
__device__ inline double shexp_phi(const ExpDev& E, double scale, const double x[3]) {
    double r2 = x[0] * x[0] + x[1] * x[1] + x[2] * x[2];
    double ir = rsqrt(r2);
    double r = r2 * ir;
    double n[3] = {x[0] * ir, x[1] * ir, x[2] * ir};
    SolidH<double> Q;
    solid_harmonics<double>(n, Q);
    RadialBasis<double> B;
    radial_basis<double>(E, log(r), B);
    const int nt = (E.lmax + 1) * (E.lmax + 1);
    double phi = 0.0;
#pragma unroll
    for (int l = 0; l <= SS_SHEXP_LMAX; ++l) {
        if (l > E.lmax) break;
#pragma unroll
        for (int mm = -l; mm <= l; ++mm) {
            const int m = mm < 0 ? -mm : mm;
            double f, fs, fss;
            radial_term<double>(E, B, nt, l * l + l + mm, f, fs, fss);
            phi += f * c_shnorm[l][m] * (mm >= 0 ? Q.c(l, m) : Q.s(l, m));
        }
    }
    return scale * phi;
}

// Subhalo line potential (potential.py:802-904): grad Phi_s and, for the
// response kernel, grad of dPhi_s/da.  rel = x - (x0 + v (t - t0)).
// Plummer: Phi = -Gm/sqrt(r^2+a^2);  dPhi/da = Gm a / D^3.
// Hernquist: Phi = -Gm/(r + a);       dPhi/da = Gm / (r + a)^2.
template <class T, bool STRUCT>
__device__ __forceinline__ void subhalo_grad(int kind, T Gm, T a, const T rel[3], T gphi[3], T gdphi[3]) {
    T r2 = rel[0] * rel[0] + rel[1] * rel[1] + rel[2] * rel[2];
    T g, gs = T(0);
    if (kind == SS_SH_PLUMMER) {
        T id = s_rsqrt(r2 + a * a);
        T id2 = id * id;
        T id3 = id2 * id;
        g = Gm * id3;
        if (STRUCT) gs = -3.0f * Gm * a * id3 * id2;  // grad(Gm a D^-3) = -3 Gm a D^-5 rel
    } else {
        T r = s_sqrt(r2);
        T inv_r = s_rcp(r);
        T inv_ra = s_rcp(r + a);
        g = Gm * inv_r * inv_ra * inv_ra;
        if (STRUCT) gs = -2.0f * Gm * inv_r * inv_ra * inv_ra * inv_ra;  // grad(Gm (r+a)^-2)
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        gphi[i] = g * rel[i];
        if (STRUCT) gdphi[i] = gs * rel[i];
    }
}

// Composite gradient (and Hessian), components summed in list order
// (Potential_Combine.gradient_func, potential.py:1291-1296).  `x` is the
// position; `xs` the same position relative to the center track at this
// time (used by SS_CENTER_TRACK components; callers that can form it more
// accurately than x - c pass it directly).
template <class T, class R, bool HESS>
__device__ __forceinline__ void pot_grad(const PotDev<R>& P, const T x[3], const T xs[3], T grad[3], T H[6],
                                         const TimeDep<T>& td = TimeDep<T>()) {
    grad[0] = grad[1] = grad[2] = T(0);
    if (HESS) {
#pragma unroll
        for (int i = 0; i < 6; ++i) H[i] = T(0);
    }
#pragma unroll 1
    for (int k = 0; k < P.n; ++k) {
        const CompDev<R>& c = P.c[k];
        const T* xc = c.center == SS_CENTER_TRACK ? xs : x;
        if ((P.grow_mask >> k) & 1) {
            // GrowingPotential: this component times g(t)
            T g2[3] = {T(0), T(0), T(0)}, H2[6] = {T(0), T(0), T(0), T(0), T(0), T(0)};
            if (c.kind == SS_SH_EXPANSION)
                shexp_grad<T, R, HESS>(P.ex, c.q[0], xc, g2, H2);
            else
                comp_grad<T, R, HESS>(c, xc, g2, H2, td);
#pragma unroll
            for (int i = 0; i < 3; ++i) grad[i] += td.amp * g2[i];
            if (HESS) {
#pragma unroll
                for (int i = 0; i < 6; ++i) H[i] += td.amp * H2[i];
            }
        } else if (c.kind == SS_SH_EXPANSION) {
            shexp_grad<T, R, HESS>(P.ex, c.q[0], xc, grad, H);
        } else {
            comp_grad<T, R, HESS>(c, xc, grad, H, td);
        }
    }
}

// A composition known at compile time: each KC = kind | (center << 4).  The
// hot kernels are instantiated for the common Galactic models so the force
// is straight-line code (no runtime loop or kind switch).
template <int KIND, int CENTER>
struct KC_ {
    static constexpr int value = KIND | (CENTER << 4);
};

template <int... KCS>
struct Comp {
    static constexpr int n = sizeof...(KCS);
    // whether a component sits on the center track, known at compile time
    template <class R>
    static __device__ __forceinline__ constexpr bool uses_track(const PotDev<R>&) {
        return ((KCS >> 4) | ... | 0) != 0;
    }
    template <class T, class R, bool HESS, int... I>
    static __device__ __forceinline__ void add(const PotDev<R>& P, const T x[3], const T xs[3], T grad[3], T H[6],
                                               const TimeDep<T>& td, std::integer_sequence<int, I...>) {
        (one<(KCS & 15), T, R, HESS>(P, I, (KCS >> 4) ? xs : x, grad, H, td), ...);
    }
    template <int KIND, class T, class R, bool HESS>
    static __device__ __forceinline__ void one(const PotDev<R>& P, int i, const T x[3], T grad[3], T H[6],
                                               const TimeDep<T>& td) {
        if constexpr (KIND == SS_SH_EXPANSION)
            shexp_grad<T, R, HESS>(P.ex, P.c[i].q[0], x, grad, H);
        else if constexpr (KIND == SS_BAR || KIND == SS_DEHNEN_BAR)
            rot_grad<KIND, T, R, HESS>(P.c[i].q, x, td, grad, H);
        else if constexpr (KIND == SS_UNIFORM_ACCEL) {
            grad[0] += td.ga[0];
            grad[1] += td.ga[1];
            grad[2] += td.ga[2];
        } else
            kind_grad<KIND, T, R, HESS>(P.c[i].q, x, grad, H);
    }
    template <class T, class R, bool HESS>
    static __device__ __forceinline__ void grad(const PotDev<R>& P, const T x[3], const T xs[3], T g[3], T H[6],
                                                const TimeDep<T>& td = TimeDep<T>()) {
        g[0] = g[1] = g[2] = T(0);
        if (HESS) {
#pragma unroll
            for (int i = 0; i < 6; ++i) H[i] = T(0);
        }
        add<T, R, HESS>(P, x, xs, g, H, td, std::make_integer_sequence<int, n>{});
    }
    // component k alone (k uniform across the warp), added to g
    template <class T, class R, bool HESS, int... I>
    static __device__ __forceinline__ void add_only(const PotDev<R>& P, int k, const T x[3], const T xs[3], T g[3],
                                                    T H[6], const TimeDep<T>& td, std::integer_sequence<int, I...>) {
        ((k == I ? one<(KCS & 15), T, R, HESS>(P, I, (KCS >> 4) ? xs : x, g, H, td) : void()), ...);
    }
    template <class T, class R, bool HESS>
    static __device__ __forceinline__ void grad_only(const PotDev<R>& P, int k, const T x[3], const T xs[3], T g[3],
                                                     T H[6], const TimeDep<T>& td = TimeDep<T>()) {
        g[0] = g[1] = g[2] = T(0);
        add_only<T, R, HESS>(P, k, x, xs, g, H, td, std::make_integer_sequence<int, n>{});
    }
    template <class R>
    static bool matches(const PotDev<R>& P) {
        const int kc[] = {KCS...};
        if (P.n != n) return false;
        for (int i = 0; i < n; ++i)
            if ((P.c[i].kind | (P.c[i].center << 4)) != kc[i]) return false;
        return true;
    }
};

struct GenericComp {
    template <class R>
    static __device__ __forceinline__ bool uses_track(const PotDev<R>& P) {
        return P.has_track != 0;
    }
    template <class T, class R, bool HESS>
    static __device__ __forceinline__ void grad(const PotDev<R>& P, const T x[3], const T xs[3], T g[3], T H[6],
                                                const TimeDep<T>& td = TimeDep<T>()) {
        pot_grad<T, R, HESS>(P, x, xs, g, H, td);
    }
};

#define SS_T_ (SS_CENTER_TRACK << 4)
// NFW + MN + Hernquist (the stream workloads), the same with the moving
// progenitor, the Gala Milky Way (MN, bulge, nucleus, NFW) with and without
// it, the triaxial-halo model, and single NFW / Plummer.
using CompMW3 = Comp<SS_NFW, SS_MIYAMOTO_NAGAI, SS_HERNQUIST>;
using CompMW3P = Comp<SS_NFW, SS_MIYAMOTO_NAGAI, SS_HERNQUIST, SS_PLUMMER | SS_T_>;
using CompGala = Comp<SS_MIYAMOTO_NAGAI, SS_HERNQUIST, SS_HERNQUIST, SS_NFW>;
using CompGalaP = Comp<SS_MIYAMOTO_NAGAI, SS_HERNQUIST, SS_HERNQUIST, SS_NFW, SS_PLUMMER | SS_T_>;
using CompTri3 = Comp<SS_TRIAXIAL_NFW, SS_MIYAMOTO_NAGAI, SS_HERNQUIST>;
using CompTri3P = Comp<SS_TRIAXIAL_NFW, SS_MIYAMOTO_NAGAI, SS_HERNQUIST, SS_PLUMMER | SS_T_>;
using CompNFW = Comp<SS_NFW>;
using CompPlummer = Comp<SS_PLUMMER>;
using CompSHExp = Comp<SS_SH_EXPANSION>;

// Calls f(Comp{}) for the matching compiled composition, else f(GenericComp{}).
template <class R, class F>
inline auto dispatch_comp(const PotDev<R>& P, F&& f) {
    if (P.grow_mask) return f(GenericComp{});  // growing components: the generic loop scales them
    if (CompMW3::matches(P)) return f(CompMW3{});
    if (CompMW3P::matches(P)) return f(CompMW3P{});
    if (CompGala::matches(P)) return f(CompGala{});
    if (CompGalaP::matches(P)) return f(CompGalaP{});
    if (CompTri3::matches(P)) return f(CompTri3{});
    if (CompTri3P::matches(P)) return f(CompTri3P{});
    if (CompNFW::matches(P)) return f(CompNFW{});
    if (CompPlummer::matches(P)) return f(CompPlummer{});
    if (CompSHExp::matches(P)) return f(CompSHExp{});
    return f(GenericComp{});
}

// A tabulated spherical subhalo (SS_SH_GRID) at squared distance r2: the
// cubic Hermite spline Phi(u), u = ln r, of its row s (linear in u outside
// the knots).  grad Phi = g rel and, with HESS, H = g I + gr rel rel^T:
// g = Phi_u / r^2, gr = (Phi_uu - 2 Phi_u) / r^4.  phi (optional) = Phi.
template <class T, bool HESS>
__device__ __forceinline__ void grid_subhalo_gh(const ShDev& sh, int s, T r2, T& g, T& gr, T* phi = nullptr) {
    const double* tab = sh.grid + (size_t)s * sh.ng * 2;
    const double u0 = __ldg(sh.gu0 + s), du = __ldg(sh.gdu + s);
    const T ir2 = s_rcp(r2);
    const T u = T(0.5) * s_log(r2);
    const double uu = (sval(u) - u0) / du;
    T fu, fuu;
    if (uu < 0.0 || uu > (double)(sh.ng - 1)) {
        const int k = uu < 0.0 ? 0 : sh.ng - 1;
        fu = T(__ldg(tab + 2 * k + 1));
        fuu = T(0);
        if (phi) *phi = T(__ldg(tab + 2 * k)) + fu * (u - T(u0 + du * k));
    } else {
        int k = (int)floor(uu);
        if (k > sh.ng - 2) k = sh.ng - 2;
        const T x = (u - T(u0 + du * k)) * T(1.0 / du);
        const T f0 = T(__ldg(tab + 2 * k)), d0 = T(du * __ldg(tab + 2 * k + 1));
        const T f1 = T(__ldg(tab + 2 * k + 2)), d1 = T(du * __ldg(tab + 2 * k + 3));
        const T x2 = x * x;
        // d/dx of the Hermite basis h00, h10, h01, h11, then d2/dx2
        const T a00 = T(6) * x2 - T(6) * x, a10 = T(3) * x2 - T(4) * x + T(1);
        const T a11 = T(3) * x2 - T(2) * x;
        fu = (a00 * (f0 - f1) + a10 * d0 + a11 * d1) * T(1.0 / du);
        fuu = ((T(12) * x - T(6)) * (f0 - f1) + (T(6) * x - T(4)) * d0 + (T(6) * x - T(2)) * d1) * T(1.0 / (du * du));
        if (phi) {
            const T x3 = x2 * x;
            *phi = (T(2) * x3 - T(3) * x2 + T(1)) * f0 + (x3 - T(2) * x2 + x) * d0 + (T(3) * x2 - T(2) * x3) * f1 +
                   (x3 - x2) * d1;
        }
    }
    g = fu * ir2;
    if (HESS) gr = (fuu - T(2) * fu) * ir2 * ir2;
}

// Subhalo sum in the potential (nonlinear perturbed streams), FP64 table.
template <class T>
__device__ __forceinline__ void subhalo_sum_grad(const ShDev& sh, const T x[3], double t, T grad[3]) {
#pragma unroll 1
    for (int j = 0; j < sh.n; ++j) {
        double t0 = __ldg(sh.t0 + j);
        double tau = t - t0;
        if (!(fabs(tau) < sh.t_window)) continue;
        T rel[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) rel[i] = x[i] - T(__ldg(sh.x0 + 3 * j + i) + __ldg(sh.v + 3 * j + i) * tau);
        T gphi[3], dummy[3];
        if (sh.kind == SS_SH_GRID) {
            T g, gr;
            grid_subhalo_gh<T, false>(sh, j, rel[0] * rel[0] + rel[1] * rel[1] + rel[2] * rel[2], g, gr);
            gphi[0] = g * rel[0];
            gphi[1] = g * rel[1];
            gphi[2] = g * rel[2];
        } else {
            subhalo_grad<T, false>(sh.kind, T(sh.G * __ldg(sh.m + j)), T(__ldg(sh.a + j)), rel, gphi, dummy);
        }
        grad[0] += gphi[0];
        grad[1] += gphi[1];
        grad[2] += gphi[2];
    }
}

}  // namespace ssg
