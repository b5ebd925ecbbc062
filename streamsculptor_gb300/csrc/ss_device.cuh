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
// FP64: rsqrt (<= 1 ulp) saves the separate square root and division.
__device__ __forceinline__ float  s_sqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double s_sqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float s_rsqrt(float x) {
    // hardware estimate + one Newton step: y (3 - x y^2) / 2
    float y = rsqrtf(x);
    float e = fmaf(-x * y, y, 1.0f);
    return fmaf(0.5f * y, e, y);
}
__device__ __forceinline__ double s_rsqrt(double x) { return rsqrt(x); }
__device__ __forceinline__ float  s_log1p(float x) { return log1pf(x); }
__device__ __forceinline__ double s_log1p(double x) { return log1p(x); }
__device__ __forceinline__ float s_rcp(float x) {
    // hardware estimate + one Newton step: r (2 - x r)
    float r = __fdividef(1.0f, x);
    return fmaf(r, fmaf(-x, r, 1.0f), r);
}
__device__ __forceinline__ double s_rcp(double x) { return 1.0 / x; }
__device__ __forceinline__ double s_cbrt(double x) { return cbrt(x); }
template <int N> __device__ inline Dual<N> s_sqrt(const Dual<N>& x) { double s = sqrt(x.v); return chain(x, s, 0.5 / s); }
template <int N> __device__ inline Dual<N> s_rsqrt(const Dual<N>& x) { double s = 1.0 / sqrt(x.v); return chain(x, s, -0.5 * s / x.v); }
template <int N> __device__ inline Dual<N> s_log1p(const Dual<N>& x) { return chain(x, log1p(x.v), 1.0 / (1.0 + x.v)); }
template <int N> __device__ inline Dual<N> s_rcp(const Dual<N>& x) { double r = 1.0 / x.v; return chain(x, r, -r * r); }
template <int N> __device__ inline Dual<N> s_cbrt(const Dual<N>& x) { double c = cbrt(x.v); return chain(x, c, c / (3.0 * x.v)); }

// ---------------------------------------------------- prepared potential
// Parameters are pre-combined on the host (G*m, 1/r_s, b^2 ...).
template <class R>
struct CompDev {
    int32_t kind;
    int32_t center;
    R q[6];
};

struct TrackDev {
    const double* knots;
    const double* slopes;
    double t0;
    double dt;
    int64_t n;
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
};

template <class R>
struct PotDev {
    int32_t n;
    int32_t has_track;
    CompDev<R> c[SS_MAX_COMPONENTS];
    TrackDev track;
    ShDev sh;
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

// Adds grad Phi of one component of compile-time kind KIND at x (already
// shifted to its center) to grad[3]; when HESS, adds its Hessian
// (xx, yy, zz, xy, xz, yz) to H[6].
template <int KIND, class T, class R, bool HESS>
__device__ __forceinline__ void kind_grad(const R* q, const T x[3], T grad[3], T H[6]) {
    if constexpr (KIND == SS_NFW || KIND == SS_HERNQUIST || KIND == SS_PLUMMER || KIND == SS_ISOCHRONE) {
        T r2 = x[0] * x[0] + x[1] * x[1] + x[2] * x[2];
        T g, h;
        if constexpr (KIND == SS_NFW) {
            nfw_gh<T, R, HESS>(q, r2 + q[3], g, h);
        } else if constexpr (KIND == SS_HERNQUIST) {
            hernquist_gh<T, R, HESS>(q, r2 + q[2], g, h);
        } else if constexpr (KIND == SS_PLUMMER) {
            plummer_gh<T, R, HESS>(q, r2, g, h);
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

// Runtime-kind dispatch (the generic path for any composition).
template <class T, class R, bool HESS>
__device__ __forceinline__ void comp_grad(const CompDev<R>& c, const T x[3], T grad[3], T H[6]) {
    switch (c.kind) {
        case SS_NFW: kind_grad<SS_NFW, T, R, HESS>(c.q, x, grad, H); break;
        case SS_TRIAXIAL_NFW: kind_grad<SS_TRIAXIAL_NFW, T, R, HESS>(c.q, x, grad, H); break;
        case SS_MIYAMOTO_NAGAI: kind_grad<SS_MIYAMOTO_NAGAI, T, R, HESS>(c.q, x, grad, H); break;
        case SS_HERNQUIST: kind_grad<SS_HERNQUIST, T, R, HESS>(c.q, x, grad, H); break;
        case SS_PLUMMER: kind_grad<SS_PLUMMER, T, R, HESS>(c.q, x, grad, H); break;
        case SS_ISOCHRONE: kind_grad<SS_ISOCHRONE, T, R, HESS>(c.q, x, grad, H); break;
        default: break;
    }
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
__device__ __forceinline__ void pot_grad(const PotDev<R>& P, const T x[3], const T xs[3], T grad[3], T H[6]) {
    grad[0] = grad[1] = grad[2] = T(0);
    if (HESS) {
#pragma unroll
        for (int i = 0; i < 6; ++i) H[i] = T(0);
    }
#pragma unroll 1
    for (int k = 0; k < P.n; ++k) {
        const CompDev<R>& c = P.c[k];
        comp_grad<T, R, HESS>(c, c.center == SS_CENTER_TRACK ? xs : x, grad, H);
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
    template <class T, class R, bool HESS, int... I>
    static __device__ __forceinline__ void add(const PotDev<R>& P, const T x[3], const T xs[3], T grad[3], T H[6],
                                               std::integer_sequence<int, I...>) {
        (kind_grad<(KCS & 15), T, R, HESS>(P.c[I].q, (KCS >> 4) ? xs : x, grad, H), ...);
    }
    template <class T, class R, bool HESS>
    static __device__ __forceinline__ void grad(const PotDev<R>& P, const T x[3], const T xs[3], T g[3], T H[6]) {
        g[0] = g[1] = g[2] = T(0);
        if (HESS) {
#pragma unroll
            for (int i = 0; i < 6; ++i) H[i] = T(0);
        }
        add<T, R, HESS>(P, x, xs, g, H, std::make_integer_sequence<int, n>{});
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
    template <class T, class R, bool HESS>
    static __device__ __forceinline__ void grad(const PotDev<R>& P, const T x[3], const T xs[3], T g[3], T H[6]) {
        pot_grad<T, R, HESS>(P, x, xs, g, H);
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

// Calls f(Comp{}) for the matching compiled composition, else f(GenericComp{}).
template <class R, class F>
inline auto dispatch_comp(const PotDev<R>& P, F&& f) {
    if (CompMW3::matches(P)) return f(CompMW3{});
    if (CompMW3P::matches(P)) return f(CompMW3P{});
    if (CompGala::matches(P)) return f(CompGala{});
    if (CompGalaP::matches(P)) return f(CompGalaP{});
    if (CompTri3::matches(P)) return f(CompTri3{});
    if (CompTri3P::matches(P)) return f(CompTri3P{});
    if (CompNFW::matches(P)) return f(CompNFW{});
    if (CompPlummer::matches(P)) return f(CompPlummer{});
    return f(GenericComp{});
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
        subhalo_grad<T, false>(sh.kind, T(sh.G * __ldg(sh.m + j)), T(__ldg(sh.a + j)), rel, gphi, dummy);
        grad[0] += gphi[0];
        grad[1] += gphi[1];
        grad[2] += gphi[2];
    }
}

}  // namespace ssg
