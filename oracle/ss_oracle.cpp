// ss_oracle.cpp — CPU FP64 oracle for the streamsculptor_gb300 hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker: the parity tests, the
// smoke check and the CPU-baseline leg of the benchmark call it; the product
// (streamsculptor_gb300/) never links, imports or runs it.
//
// It restates the reference (jnibauer/streamsculptor, pure Python/JAX) on the
// CPU in double precision, the way the reference computes it:
//   * every potential is a scalar formula; forces, Hessians and third
//     derivatives come from forward-mode automatic differentiation of that
//     formula (nested dual numbers), as the reference takes jax.grad /
//     jax.jacfwd of Potential.potential (main.py:37-40, 59-65, 76-85);
//   * time stepping is the classical fixed-step Dormand-Prince 5(4) tableau
//     (Dormand & Prince 1980).  The reference delegates stepping to the
//     third-party diffrax==0.7.0 (Dopri5/Dopri8 with a PID controller,
//     main.py:139-162); with dtmin = dtmax = dt and force_dtmin the accepted
//     steps are these fixed steps, and the 5th-order solution is
//     y + h * sum_i b_i k_i with the published weights;
//   * the progenitor-track spline is restated from the published definition
//     of interpax==0.3.4 Interpolator1D(method='cubic') (C1 cubic Hermite,
//     knot slopes = mean of adjacent secants, one-sided at the ends).
// The product kernels use hand-derived analytic gradients and Hessians, so
// the two are independent restatements of the same mathematics.
//
// Build: oracle/build_oracle.py (g++ -O3 -fopenmp -shared).

#include "../include/streamsculptor_gb300.h"

#include <cmath>
#include <cstring>
#include <limits>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

// ------------------------------------------------------------------ duals
template <class T, int N>
struct Dual {
    T v;
    T d[N];
    Dual() : v(0.0) {
        for (int i = 0; i < N; ++i) d[i] = T(0.0);
    }
    Dual(double c) : v(c) {  // NOLINT: implicit constant
        for (int i = 0; i < N; ++i) d[i] = T(0.0);
    }
    static Dual cst(const T& c) {
        Dual r;
        r.v = c;
        return r;
    }
    static Dual var(const T& c, int k) {
        Dual r;
        r.v = c;
        r.d[k] = T(1.0);
        return r;
    }
};

template <class T, int N>
Dual<T, N> operator+(const Dual<T, N>& a, const Dual<T, N>& b) {
    Dual<T, N> r;
    r.v = a.v + b.v;
    for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i];
    return r;
}
template <class T, int N>
Dual<T, N> operator-(const Dual<T, N>& a, const Dual<T, N>& b) {
    Dual<T, N> r;
    r.v = a.v - b.v;
    for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i];
    return r;
}
template <class T, int N>
Dual<T, N> operator-(const Dual<T, N>& a) {
    Dual<T, N> r;
    r.v = -a.v;
    for (int i = 0; i < N; ++i) r.d[i] = -a.d[i];
    return r;
}
template <class T, int N>
Dual<T, N> operator*(const Dual<T, N>& a, const Dual<T, N>& b) {
    Dual<T, N> r;
    r.v = a.v * b.v;
    for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
    return r;
}
template <class T, int N>
Dual<T, N> operator/(const Dual<T, N>& a, const Dual<T, N>& b) {
    Dual<T, N> r;
    T inv = T(1.0) / b.v;
    r.v = a.v * inv;
    for (int i = 0; i < N; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) * inv;
    return r;
}
template <class T, int N> Dual<T, N> operator+(const Dual<T, N>& a, double b) { return a + Dual<T, N>(b); }
template <class T, int N> Dual<T, N> operator+(double a, const Dual<T, N>& b) { return Dual<T, N>(a) + b; }
template <class T, int N> Dual<T, N> operator-(const Dual<T, N>& a, double b) { return a - Dual<T, N>(b); }
template <class T, int N> Dual<T, N> operator-(double a, const Dual<T, N>& b) { return Dual<T, N>(a) - b; }
template <class T, int N>
Dual<T, N> operator*(const Dual<T, N>& a, double b) {
    Dual<T, N> r;
    r.v = a.v * b;
    for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b;
    return r;
}
template <class T, int N> Dual<T, N> operator*(double a, const Dual<T, N>& b) { return b * a; }
template <class T, int N> Dual<T, N> operator/(const Dual<T, N>& a, double b) { return a * (1.0 / b); }
template <class T, int N> Dual<T, N> operator/(double a, const Dual<T, N>& b) { return Dual<T, N>(a) / b; }

// chain rule helper: f(x) with value fv and derivative dfv (both of type T)
template <class T, int N>
Dual<T, N> chain(const Dual<T, N>& x, const T& fv, const T& dfv) {
    Dual<T, N> r;
    r.v = fv;
    for (int i = 0; i < N; ++i) r.d[i] = dfv * x.d[i];
    return r;
}

inline double sqrt_(double x) { return std::sqrt(x); }
inline double log_(double x) { return std::log(x); }
inline double pow_(double x, double p) { return std::pow(x, p); }
inline double value(double x) { return x; }

template <class T, int N>
Dual<T, N> sqrt_(const Dual<T, N>& x) {
    T s = sqrt_(x.v);
    return chain(x, s, T(0.5) / s);
}
template <class T, int N>
Dual<T, N> log_(const Dual<T, N>& x) {
    return chain(x, log_(x.v), T(1.0) / x.v);
}
template <class T, int N>
Dual<T, N> pow_(const Dual<T, N>& x, double p) {
    return chain(x, pow_(x.v, p), p * pow_(x.v, p - 1.0));
}
inline double exp_(double x) { return std::exp(x); }
template <class T, int N>
Dual<T, N> exp_(const Dual<T, N>& x) {
    T e = exp_(x.v);
    return chain(x, e, e);
}

// Regularised lower incomplete gamma P(a, x) (what jax.scipy.special.gammainc
// computes; PowerLawCutoffPotential, potential.py:357-388): the power series
// x^a e^-x / Gamma(a) sum_n x^n / (a (a+1) ... (a+n)) below x = a + 1, else
// one minus the Legendre continued fraction of the upper function
// (Abramowitz & Stegun 6.5.29, 6.5.31), to double precision.  Pinned
// against scipy.special.gammainc by the oracle tests.
inline double gammainc_(double a, double x) {
    if (!(x > 0.0)) return 0.0;
    const double e = std::exp(a * std::log(x) - x - std::lgamma(a));
    if (x < a + 1.0) {
        double term = 1.0 / a, sum = term;
        for (int n = 1; n < 1000 && std::fabs(term) >= std::fabs(sum) * 1e-17; ++n) {
            term *= x / (a + n);
            sum += term;
        }
        return sum * e;
    }
    // F = 1 / (b0 - a1 / (b1 - a2 / (b2 - ...))), b_i = x + 2 i + 1 - a, a_i = i (i - a),
    // by forward recurrence of the convergents A_i / B_i (rescaled to stay finite)
    double A0 = 1.0, B0 = 0.0, A1 = 0.0, B1 = 1.0;  // convergents of the fraction 1 / (...)
    double f = 0.0, prev = -1.0;
    for (int i = 0; i < 2000; ++i) {
        const double bi = x + 2.0 * i + 1.0 - a;
        const double ai = i == 0 ? 1.0 : -(double)i * ((double)i - a);
        const double A2 = bi * A1 + ai * A0, B2 = bi * B1 + ai * B0;
        A0 = A1; B0 = B1; A1 = A2; B1 = B2;
        const double sc = 1.0 / B1;  // keep the convergents bounded
        A0 *= sc; B0 *= sc; A1 *= sc; B1 = 1.0;
        f = A1;
        if (i > 2 && std::fabs(f - prev) <= 4e-16 * std::fabs(f)) break;
        prev = f;
    }
    return 1.0 - e * f;
}
inline double dgammainc_(double a, double x) { return x > 0.0 ? std::exp((a - 1.0) * std::log(x) - x - std::lgamma(a)) : 0.0; }
template <class T, int N>
T dgammainc_t(double a, const T& x) {
    return exp_((a - 1.0) * log_(x) - x - std::lgamma(a));
}
inline double dgammainc_t(double a, double x) { return dgammainc_(a, x); }
template <class T, int N>
Dual<T, N> gammainc_(double a, const Dual<T, N>& x) {
    return chain(x, gammainc_(a, x.v), dgammainc_t<T, N>(a, x.v));
}

inline double log1p_(double x) { return std::log1p(x); }
template <class T, int N>
Dual<T, N> log1p_(const Dual<T, N>& x) {
    return chain(x, log1p_(x.v), T(1.0) / (1.0 + x.v));
}

// Regularised incomplete beta function I_z(a, b) (what
// jax.scipy.special.betainc computes; ZhaoPotential, potential.py:282-355):
// the hypergeometric series
//   I_z(a, b) = z^a (1 - z)^b / (a B(a, b)) sum_n (a + b)_n / (a + 1)_n z^n
// (Abramowitz & Stegun 26.5.23 with 15.1.1) for z < (a + 1) / (a + b + 2),
// where its term ratio stays below one, else 1 - I_{1-z}(b, a); to double
// precision.  (The product kernels evaluate the continued fraction instead.)
// Pinned against scipy.special.betainc by the oracle tests.
inline double lbeta_(double a, double b) { return std::lgamma(a) + std::lgamma(b) - std::lgamma(a + b); }
inline double betainc_(double a, double b, double z) {
    if (!(z > 0.0)) return 0.0;
    if (!(z < 1.0)) return 1.0;
    if (z >= (a + 1.0) / (a + b + 2.0)) return 1.0 - betainc_(b, a, 1.0 - z);
    double term = 1.0, sum = 1.0;
    for (int n = 0; n < 100000; ++n) {
        term *= (a + b + n) * z / (a + 1.0 + n);
        sum += term;
        if (std::fabs(term) < 1e-17 * sum) break;
    }
    return std::exp(a * std::log(z) + b * std::log1p(-z) - lbeta_(a, b)) * sum / a;
}
// dI_z/dz = z^(a-1) (1 - z)^(b-1) / B(a, b)
template <class T, int N>
T dbetainc_t(double a, double b, const T& z) {
    return exp_((a - 1.0) * log_(z) + (b - 1.0) * log_(1.0 - z) - lbeta_(a, b));
}
inline double dbetainc_t(double a, double b, double z) {
    return std::exp((a - 1.0) * std::log(z) + (b - 1.0) * std::log1p(-z) - lbeta_(a, b));
}
template <class T, int N>
Dual<T, N> betainc_(double a, double b, const Dual<T, N>& z) {
    return chain(z, betainc_(a, b, z.v), dbetainc_t<T, N>(a, b, z.v));
}

inline double cos_(double x) { return std::cos(x); }
inline double sin_(double x) { return std::sin(x); }
inline double atan2_(double y, double x) { return std::atan2(y, x); }
template <class T, int N>
Dual<T, N> cos_(const Dual<T, N>& x) {
    return chain(x, cos_(x.v), -sin_(x.v));
}
template <class T, int N>
Dual<T, N> sin_(const Dual<T, N>& x) {
    return chain(x, sin_(x.v), cos_(x.v));
}
// atan2 with d/dy = x / (x^2 + y^2), d/dx = -y / (x^2 + y^2)
template <class T, int N>
Dual<T, N> atan2_(const Dual<T, N>& y, const Dual<T, N>& x) {
    Dual<T, N> r;
    r.v = atan2_(y.v, x.v);
    T den = x.v * x.v + y.v * y.v;
    T a = x.v / den, b = -y.v / den;
    for (int i = 0; i < N; ++i) r.d[i] = a * y.d[i] + b * x.d[i];
    return r;
}
template <class T, int N>
double value(const Dual<T, N>& x) {
    return value(x.v);
}

// ---------------------------------------------------------------- spline
// interpax 'cubic' (C1 local cubic Hermite) restated: slopes are the mean of
// the two adjacent secants, one-sided secant at the ends.
static void track_slopes(const double* knots, int64_t n, double dt, double* slopes) {
    for (int64_t k = 0; k < n; ++k) {
        for (int c = 0; c < 3; ++c) {
            double s;
            if (n < 2) {
                s = 0.0;
            } else if (k == 0) {
                s = (knots[3 * 1 + c] - knots[c]) / dt;
            } else if (k == n - 1) {
                s = (knots[3 * k + c] - knots[3 * (k - 1) + c]) / dt;
            } else {
                double sl = (knots[3 * k + c] - knots[3 * (k - 1) + c]) / dt;
                double sr = (knots[3 * (k + 1) + c] - knots[3 * k + c]) / dt;
                s = 0.5 * (sl + sr);
            }
            slopes[3 * k + c] = s;
        }
    }
}

static void track_eval(const ss_track& tr, double t, double c[3]) {
    double u = (t - tr.t0) / tr.dt;
    int64_t k = (int64_t)std::floor(u);
    if (k < 0) k = 0;
    if (k > tr.n_knots - 2) k = tr.n_knots - 2;
    double s = u - (double)k;
    if (tr.linear) {  // RegularGridInterpolator(method='linear', fill_value=None)
        for (int i = 0; i < 3; ++i) c[i] = tr.knots[3 * k + i] + s * (tr.knots[3 * (k + 1) + i] - tr.knots[3 * k + i]);
        return;
    }
    double s2 = s * s, s3 = s2 * s;
    double h00 = 2 * s3 - 3 * s2 + 1;
    double h10 = s3 - 2 * s2 + s;
    double h01 = -2 * s3 + 3 * s2;
    double h11 = s3 - s2;
    for (int i = 0; i < 3; ++i) {
        double p0 = tr.knots[3 * k + i], p1 = tr.knots[3 * (k + 1) + i];
        double m0 = tr.slopes[3 * k + i], m1 = tr.slopes[3 * (k + 1) + i];
        c[i] = h00 * p0 + h10 * tr.dt * m0 + h01 * p1 + h11 * tr.dt * m1;
    }
}

// d/dt of a track by central differences of track_eval inside the segment
// holding t (exact for the linear form; the cubic form's derivative to
// round-off of the difference), jax.jacfwd of the velocity spline in
// UniformAcceleration.gradient (potential.py:497-499).
static void track_deriv(const ss_track& tr, double t, double d[3]) {
    double u = (t - tr.t0) / tr.dt;
    int64_t k = (int64_t)std::floor(u);
    if (k < 0) k = 0;
    if (k > tr.n_knots - 2) k = tr.n_knots - 2;
    if (tr.linear) {
        for (int i = 0; i < 3; ++i) d[i] = (tr.knots[3 * (k + 1) + i] - tr.knots[3 * k + i]) / tr.dt;
        return;
    }
    double s = u - (double)k;
    for (int i = 0; i < 3; ++i) {
        double p0 = tr.knots[3 * k + i], p1 = tr.knots[3 * (k + 1) + i];
        double m0 = tr.slopes[3 * k + i], m1 = tr.slopes[3 * (k + 1) + i];
        // derivative of the Hermite basis, chain factor 1/dt
        d[i] = ((6 * s * s - 6 * s) * p0 + (3 * s * s - 4 * s + 1) * tr.dt * m0 + (-6 * s * s + 6 * s) * p1 +
                (3 * s * s - 2 * s) * tr.dt * m1) / tr.dt;
    }
}

// ------------------------------------------------------------ potentials
// ZhaoPotential._potential (potential.py:314-331) as written, at radius r:
// p = {m, r_s, alpha, beta, gamma}, rho0 from _rho0 (:308-312), and the
// reference's replacement of p0 = alpha (2 - gamma) <= 0 by sqrt(eps).
template <class S>
S zhao_phi_r(const double* p, double G, const S& r) {
    const double m = p[0], r_s = p[1], al = p[2], be = p[3], ga = p[4];
    const double rho0 = m / (4.0 * M_PI * al * std::exp(lbeta_(al * (3.0 - ga), al * (be - 3.0))));
    const S xa = pow_(r / r_s, 1.0 / al);
    const S z = xa / (1.0 + xa);
    const double p0 = al * (2.0 - ga), q0 = al * (be - 3.0), c0 = al * (be - ga);
    const S term_l = std::exp(lbeta_(c0 - q0, q0)) * betainc_(c0 - q0, q0, z);
    const double p0s = p0 <= 0.0 ? std::sqrt(std::numeric_limits<double>::epsilon()) : p0;
    const double logB = lbeta_(p0s, c0 - p0);
    const S log1mI = log1p_(-betainc_(p0s, c0 - p0, z));
    const S term_r = exp_(logB + log1mI);
    return -4.0 * M_PI * G * rho0 * al * (term_l / r + term_r / r_s);
}

// ZhaoPotential.gradient_func (potential.py:347-354) as written: the forward
// difference of the potential over [r, r + dr], dr = 1e-5 r + 1e-8, along
// x / r; adds scale times it to g.
template <class S>
void zhao_grad_add(const double* p, double G, const S x[3], double scale, S g[3]) {
    const S r = sqrt_(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
    const S dr = 1e-5 * r + 1e-8;
    const S dphi_dr = (zhao_phi_r(p, G, r + dr) - zhao_phi_r(p, G, r)) / dr;
    for (int i = 0; i < 3; ++i) g[i] = g[i] + scale * (dphi_dr * x[i] / r);
}

// Each follows the scalar formula of the reference class named beside it.
template <class S>
S phi_component(const ss_component& c, double G, const S x[3]) {
    const double* p = c.p;
    switch (c.kind) {
        case SS_NFW: {  // NFWPotential.potential, potential.py:80-84
            double v_h2 = -G * p[0] / p[1];
            S m = sqrt_(x[0] * x[0] + x[1] * x[1] + x[2] * x[2] + p[2]) / p[1];
            return v_h2 * log_(1.0 + m) / m;
        }
        case SS_TRIAXIAL_NFW: {  // TriaxialNFWPotential.potential, potential.py:92-97
            S xs[3] = {x[0] / p[2], x[1] / p[3], x[2] / p[4]};
            double v_h2 = -G * p[0] / p[1];
            S m = sqrt_(xs[0] * xs[0] + xs[1] * xs[1] + xs[2] * xs[2]) / p[1];
            return v_h2 * log_(1.0 + m) / m;
        }
        case SS_MIYAMOTO_NAGAI: {  // MiyamotoNagaiDisk.potential, potential.py:69-72
            S R2 = x[0] * x[0] + x[1] * x[1];
            S q = sqrt_(x[2] * x[2] + p[2] * p[2]) + p[1];
            return -G * p[0] / sqrt_(R2 + q * q);
        }
        case SS_HERNQUIST: {  // HernquistPotential.potential, potential.py:135-138
            S r = sqrt_(x[0] * x[0] + x[1] * x[1] + x[2] * x[2] + p[2]);
            return -G * p[0] / (r + p[1]);
        }
        case SS_PLUMMER: {  // PlummerPotential.potential, potential.py:127-130
            S r2 = x[0] * x[0] + x[1] * x[1] + x[2] * x[2];
            return -G * p[0] / sqrt_(r2 + p[1] * p[1]);
        }
        case SS_ISOCHRONE: {  // Isochrone.potential, potential.py:119-122
            S r = sqrt_(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
            return -G * p[0] / (p[1] + sqrt_(r * r + p[1] * p[1]));
        }
        case SS_POWERLAW_CUTOFF: {  // PowerLawCutoffPotential.potential, potential.py:365-378, as written
            const double t0 = 0.5 * p[1], t1 = -t0, t2 = t1 + 1.5;
            S t3 = x[0] * x[0] + x[1] * x[1] + x[2] * x[2];
            S t4 = t3 / (p[2] * p[2]);
            const double t5 = G * p[0];
            S t6 = t5 * gammainc_(t2, t4) * std::tgamma(t2) / (sqrt_(t3) * std::tgamma(t1 + 2.5));
            return t0 * t6 - 1.5 * t6 + t5 * gammainc_(t1 + 1.0, t4) * std::tgamma(t1 + 1.0) / (p[2] * std::tgamma(t2));
        }
        case SS_ZHAO:  // ZhaoPotential.potential, potential.py:333-336
            return zhao_phi_r(p, G, sqrt_(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]));
        default:
            return S(std::numeric_limits<double>::quiet_NaN());
    }
}

// Time-dependent components.
template <class S>
S phi_component_t(const ss_component& c, double G, const S x[3], double t, const ss_track& fvel) {
    const double* p = c.p;
    switch (c.kind) {
        case SS_BAR: {  // BarPotential.potential, potential.py:185-198: rotate by ang = -Omega t
            double ang = -p[4] * t;
            double R00 = std::cos(ang), R01 = -std::sin(ang), R10 = std::sin(ang), R11 = std::cos(ang);
            S xc = R00 * x[0] + R01 * x[1], yc = R10 * x[0] + R11 * x[1], zc = x[2];
            S bz = p[2] + sqrt_(p[3] * p[3] + zc * zc);
            S Tp = sqrt_((p[1] + xc) * (p[1] + xc) + yc * yc + bz * bz);
            S Tm = sqrt_((p[1] - xc) * (p[1] - xc) + yc * yc + bz * bz);
            return (G * p[0] / (2.0 * p[1])) * log_((xc - p[1] + Tm) / (xc + p[1] + Tp));
        }
        case SS_DEHNEN_BAR: {  // DehnenBarPotential.potential, potential.py:205-222
            S phi = atan2_(x[1], x[0]);
            S R2 = x[0] * x[0] + x[1] * x[1];
            S r2 = R2 + x[2] * x[2];
            S r = sqrt_(r2);
            S U = value(r) >= p[3] ? -pow_(r / p[3], -3.0) : pow_(r / p[3], 3.0) - 2.0;
            double pref = p[0] * (p[1] * p[1] / 3.0) * std::pow(p[2] / p[3], 3.0);
            return pref * (R2 / r2) * U * cos_(2.0 * (phi - p[4] - p[5] * t));
        }
        case SS_UNIFORM_ACCEL: {  // gradient dv/dt (potential.py:497-499): Phi = (dv/dt) . x
            double d[3];
            track_deriv(fvel, t, d);
            return d[0] * x[0] + d[1] * x[1] + d[2] * x[2];
        }
        default:
            return phi_component(c, G, x);
    }
}

// One subhalo on a line, SubhaloLinePotential.potential_per_SH,
// potential.py:832-850 (Plummer) — the Hernquist form follows
// SubhaloLinePotential_Custom with a HernquistPotential.  Zero outside the
// window |t - t0| < t_window.  `S2` lets the caller differentiate in the
// scale radius a as well (SubhaloLinePotential_dRadius, potential.py:861-866).
// A tabulated subhalo (SS_SH_GRID): the cubic Hermite spline of row j in
// u = ln r through its knots (value, d/du), continued linearly outside —
// interpax.Interpolator1D(method='cubic') over the log-radius grid of
// TNFWSubhaloLinePotential.single_subhalo_potential (potential.py:1068-1072),
// whose knot derivatives the caller supplies.
template <class S>
S phi_grid_row(const ss_subhalos& sh, int64_t j, const S& r2) {
    const double* tab = sh.grid + (size_t)j * sh.n_grid * 2;
    const double u0 = sh.grid_u0[j], du = sh.grid_du[j];
    const int64_t n = sh.n_grid;
    S u = 0.5 * log_(r2);
    double uu = (value(u) - u0) / du;
    if (uu < 0.0) return tab[0] + tab[1] * (u - u0);
    if (uu > (double)(n - 1)) return tab[2 * (n - 1)] + tab[2 * (n - 1) + 1] * (u - (u0 + du * (n - 1)));
    int64_t k = (int64_t)std::floor(uu);
    if (k > n - 2) k = n - 2;
    S x = (u - (u0 + du * k)) / du;
    S x2 = x * x, x3 = x2 * x;
    return (2.0 * x3 - 3.0 * x2 + 1.0) * tab[2 * k] + (x3 - 2.0 * x2 + x) * (du * tab[2 * k + 1]) +
           (3.0 * x2 - 2.0 * x3) * tab[2 * k + 2] + (x3 - x2) * (du * tab[2 * k + 3]);
}

template <class S>
S phi_subhalo(int kind, double G, double m, const S& a, const double x0[3], const double v[3],
              double t0, double t_window, const S x[3], double t, const ss_subhalos* tab = nullptr, int64_t j = 0) {
    if (!(std::fabs(t - t0) < t_window)) return S(0.0);
    S rel[3];
    for (int i = 0; i < 3; ++i) rel[i] = x[i] - (x0[i] + v[i] * (t - t0));
    S r2 = rel[0] * rel[0] + rel[1] * rel[1] + rel[2] * rel[2];
    if (kind == SS_SH_GRID) return phi_grid_row(*tab, j, r2);
    if (kind == SS_SH_PLUMMER) return -G * m / sqrt_(r2 + a * a);
    return -G * m / (sqrt_(r2) + a);
}

// Spherical-harmonic expansion (SS_SH_EXPANSION): restated from the
// definition in the C header with spherical angles and the textbook
// associated-Legendre recurrence in cos(theta) (no Condon-Shortley phase),
//   P_m^m = (2m-1)!! sin^m(theta),  P_{m+1}^m = (2m+1) cos(theta) P_m^m,
//   (l-m) P_l^m = (2l-1) cos(theta) P_{l-1}^m - (l+m-1) P_{l-2}^m,
// cos(m phi), sin(m phi) by the angle-addition recurrence, Schmidt factors
// sqrt(2 (l-m)!/(l+m)!), and the radial cubic Hermite spline in ln r with
// linear continuation outside the knots.  (The product kernels use Cartesian
// solid harmonics and analytic derivatives instead.)
template <class S>
S phi_expansion(const ss_expansion& E, double scale, const S x[3]) {
    const int L = E.l_max, nt = (L + 1) * (L + 1);
    S rho2 = x[0] * x[0] + x[1] * x[1];
    S r = sqrt_(rho2 + x[2] * x[2]);
    S rho = sqrt_(rho2);
    S ct = x[2] / r, st = rho / r, cp = x[0] / rho, sp = x[1] / rho;
    // radial spline
    S u = log_(r);
    double us = (value(u) - E.log_r0) / E.dlog_r;
    int k = (int)std::floor(us);
    if (k < 0) k = 0;
    if (k > E.n_knots - 2) k = E.n_knots - 2;
    S s = (u - (E.log_r0 + k * E.dlog_r)) / E.dlog_r;
    S sc = s;
    if (value(s) < 0.0) sc = S(0.0);
    if (value(s) > 1.0) sc = S(1.0);
    S ext = s - sc;
    S h00 = (1.0 + 2.0 * sc) * (1.0 - sc) * (1.0 - sc), h10 = sc * (1.0 - sc) * (1.0 - sc);
    S h01 = sc * sc * (3.0 - 2.0 * sc), h11 = sc * sc * (sc - 1.0);
    S d00 = 6.0 * sc * (sc - 1.0), d10 = (1.0 - sc) * (1.0 - 3.0 * sc), d01 = 6.0 * sc * (1.0 - sc),
      d11 = sc * (3.0 * sc - 2.0);
    auto radial = [&](int j) {
        const double* a = E.coef + ((size_t)k * nt + j) * 2;
        const double* b = a + 2 * nt;
        double f0 = a[0], g0 = a[1] * E.dlog_r, f1 = b[0], g1 = b[1] * E.dlog_r;
        S fs = d00 * f0 + d10 * g0 + d01 * f1 + d11 * g1;
        return h00 * f0 + h10 * g0 + h01 * f1 + h11 * g1 + ext * fs;
    };
    // associated Legendre functions P[l][m] and cos/sin(m phi)
    S P[SS_SHEXP_LMAX + 1][SS_SHEXP_LMAX + 1];
    S cm[SS_SHEXP_LMAX + 1], sm[SS_SHEXP_LMAX + 1];
    cm[0] = S(1.0);
    sm[0] = S(0.0);
    for (int m = 1; m <= L; ++m) {
        cm[m] = cm[m - 1] * cp - sm[m - 1] * sp;
        sm[m] = sm[m - 1] * cp + cm[m - 1] * sp;
    }
    P[0][0] = S(1.0);
    for (int m = 1; m <= L; ++m) P[m][m] = (2.0 * m - 1.0) * st * P[m - 1][m - 1];
    for (int m = 0; m < L; ++m) P[m + 1][m] = (2.0 * m + 1.0) * ct * P[m][m];
    for (int m = 0; m <= L; ++m)
        for (int l = m + 2; l <= L; ++l)
            P[l][m] = ((2.0 * l - 1.0) * ct * P[l - 1][m] - (l + m - 1.0) * P[l - 2][m]) / (double)(l - m);
    S phi(0.0);
    for (int l = 0; l <= L; ++l) {
        phi = phi + radial(l * l + l) * P[l][0];
        for (int m = 1; m <= l; ++m) {
            double norm = std::sqrt(2.0 * std::tgamma(l - m + 1.0) / std::tgamma(l + m + 1.0));
            phi = phi + norm * P[l][m] * (radial(l * l + l + m) * cm[m] + radial(l * l + l - m) * sm[m]);
        }
    }
    return scale * phi;
}

// Components whose reference gradient is not the derivative of their
// potential: ZhaoPotential (a forward difference of it).
inline bool fd_kind(int kind) { return kind == SS_ZHAO; }

// skip_fd: leave out the fd_kind components (their gradients are added by
// fd_grad_add instead of differentiating this sum).
template <class S>
S phi_total(const ss_potential& P, const S x[3], double t, bool skip_fd = false) {
    S acc(0.0);
    double c[3] = {0, 0, 0};
    bool have_c = false;
    for (int k = 0; k < P.n_components; ++k) {
        const ss_component& comp = P.comp[k];
        if (skip_fd && fd_kind(comp.kind)) continue;
        // GrowingPotential.potential, potential.py:474-477: the wrapped
        // potential times growth_func(t) (column 0 of the growth track)
        double gk = 1.0;
        if (comp.center & SS_GROWS) {
            double gv[3];
            track_eval(P.growth, t, gv);
            gk = gv[0];
        }
        if (comp.center & SS_CENTER_TRACK) {
            if (!have_c) {
                track_eval(P.track, t, c);
                have_c = true;
            }
            S xs[3] = {x[0] - c[0], x[1] - c[1], x[2] - c[2]};
            acc = acc + gk * (comp.kind == SS_SH_EXPANSION ? phi_expansion(P.expansion, comp.p[0], xs)
                                                           : phi_component_t(comp, P.G, xs, t, P.frame_velocity));
        } else {
            acc = acc + gk * (comp.kind == SS_SH_EXPANSION ? phi_expansion(P.expansion, comp.p[0], x)
                                                           : phi_component_t(comp, P.G, x, t, P.frame_velocity));
        }
    }
    const ss_subhalos& sh = P.subhalos;
    if (sh.n > 0) {
        S s(0.0);
        for (int64_t j = 0; j < sh.n; ++j)
            s = s + phi_subhalo<S>(sh.kind, P.G, sh.m[j], S(sh.a[j]), sh.x0 + 3 * j, sh.v + 3 * j,
                                   sh.t0[j], sh.t_window, x, t, &sh, j);
        acc = acc + s;
    }
    return acc;
}

typedef Dual<double, 3> D3;
typedef Dual<D3, 3> DD3;

// The gradients of the fd_kind components at x, added to g, with the
// center and growth handling of phi_total.
template <class S>
void fd_grad_add(const ss_potential& P, const S x[3], double t, S g[3]) {
    double c[3] = {0, 0, 0};
    bool have_c = false;
    for (int k = 0; k < P.n_components; ++k) {
        const ss_component& comp = P.comp[k];
        if (!fd_kind(comp.kind)) continue;
        double gk = 1.0;
        if (comp.center & SS_GROWS) {
            double gv[3];
            track_eval(P.growth, t, gv);
            gk = gv[0];
        }
        if (comp.center & SS_CENTER_TRACK) {
            if (!have_c) {
                track_eval(P.track, t, c);
                have_c = true;
            }
            S xs[3] = {x[0] - c[0], x[1] - c[1], x[2] - c[2]};
            zhao_grad_add(comp.p, P.G, xs, gk, g);
        } else {
            zhao_grad_add(comp.p, P.G, x, gk, g);
        }
    }
}
inline bool has_fd(const ss_potential& P) {
    for (int k = 0; k < P.n_components; ++k)
        if (fd_kind(P.comp[k].kind)) return true;
    return false;
}

// gradient by forward-mode AD of the scalar potential (main.py:37-40), plus
// the fd_kind components' own gradients
template <class S>
void grad_total(const ss_potential& P, const S x[3], double t, S g[3]) {
    Dual<S, 3> xd[3];
    for (int i = 0; i < 3; ++i) xd[i] = Dual<S, 3>::var(x[i], i);
    Dual<S, 3> f = phi_total(P, xd, t, true);
    for (int i = 0; i < 3; ++i) g[i] = f.d[i];
    if (has_fd(P)) fd_grad_add(P, x, t, g);
}

// Hessian by nested forward-mode AD (jacfwd of the gradient, main.py:59-65)
template <class S>
void hess_total(const ss_potential& P, const S x[3], double t, S* phi, S g[3], S H[3][3]) {
    typedef Dual<S, 3> I;
    typedef Dual<I, 3> O;
    O xd[3];
    for (int i = 0; i < 3; ++i) {
        I inner = I::var(x[i], i);
        xd[i] = O::var(inner, i);
    }
    const bool fd = has_fd(P);
    O f = phi_total(P, xd, t, true);
    if (phi) *phi = fd ? phi_total(P, x, t) : f.v.v;
    for (int i = 0; i < 3; ++i) {
        g[i] = f.d[i].v;
        for (int j = 0; j < 3; ++j) H[i][j] = f.d[i].d[j];
    }
    if (fd) {
        // the fd_kind gradients and their Jacobian (jacfwd of the gradient)
        I xi[3], gi[3] = {I(0.0), I(0.0), I(0.0)};
        for (int i = 0; i < 3; ++i) xi[i] = I::var(x[i], i);
        fd_grad_add(P, xi, t, gi);
        for (int i = 0; i < 3; ++i) {
            g[i] = g[i] + gi[i].v;
            for (int j = 0; j < 3; ++j) H[i][j] = H[i][j] + gi[i].d[j];
        }
    }
}

// ------------------------------------------------------------ Dopri5
// Dormand & Prince (1980) RK5(4)7M tableau; the 5th-order solution uses b.
static const double C2 = 1.0 / 5.0, C3 = 3.0 / 10.0, C4 = 4.0 / 5.0, C5 = 8.0 / 9.0;
static const double A21 = 1.0 / 5.0;
static const double A31 = 3.0 / 40.0, A32 = 9.0 / 40.0;
static const double A41 = 44.0 / 45.0, A42 = -56.0 / 15.0, A43 = 32.0 / 9.0;
static const double A51 = 19372.0 / 6561.0, A52 = -25360.0 / 2187.0, A53 = 64448.0 / 6561.0,
                    A54 = -212.0 / 729.0;
static const double A61 = 9017.0 / 3168.0, A62 = -355.0 / 33.0, A63 = 46732.0 / 5247.0,
                    A64 = 49.0 / 176.0, A65 = -5103.0 / 18656.0;
static const double B1 = 35.0 / 384.0, B3 = 500.0 / 1113.0, B4 = 125.0 / 192.0,
                    B5 = -2187.0 / 6784.0, B6 = 11.0 / 84.0;

// One fixed step of size h from time t.  f(t, y, dydt) fills dydt.
template <class F>
void dopri5_step(F& f, double t, double h, double* y, int n, std::vector<double>& w) {
    w.resize((size_t)7 * n);
    double* k1 = w.data();
    double* k2 = k1 + n;
    double* k3 = k2 + n;
    double* k4 = k3 + n;
    double* k5 = k4 + n;
    double* k6 = k5 + n;
    double* ys = k6 + n;
    f(t, y, k1);
    for (int i = 0; i < n; ++i) ys[i] = y[i] + h * (A21 * k1[i]);
    f(t + C2 * h, ys, k2);
    for (int i = 0; i < n; ++i) ys[i] = y[i] + h * (A31 * k1[i] + A32 * k2[i]);
    f(t + C3 * h, ys, k3);
    for (int i = 0; i < n; ++i) ys[i] = y[i] + h * (A41 * k1[i] + A42 * k2[i] + A43 * k3[i]);
    f(t + C4 * h, ys, k4);
    for (int i = 0; i < n; ++i)
        ys[i] = y[i] + h * (A51 * k1[i] + A52 * k2[i] + A53 * k3[i] + A54 * k4[i]);
    f(t + C5 * h, ys, k5);
    for (int i = 0; i < n; ++i)
        ys[i] = y[i] + h * (A61 * k1[i] + A62 * k2[i] + A63 * k3[i] + A64 * k4[i] + A65 * k5[i]);
    f(t + h, ys, k6);
    for (int i = 0; i < n; ++i)
        y[i] = y[i] + h * (B1 * k1[i] + B3 * k3[i] + B4 * k4[i] + B5 * k5[i] + B6 * k6[i]);
}

// Hamiltonian vector field (x, v) -> (v, -grad Phi): velocity_acceleration,
// main.py:116-120.
struct HamRHS {
    const ss_potential* P;
    void operator()(double t, const double* y, double* dy) const {
        double g[3];
        grad_total<double>(*P, y, t, g);
        dy[0] = y[3];
        dy[1] = y[4];
        dy[2] = y[5];
        dy[3] = -g[0];
        dy[4] = -g[1];
        dy[5] = -g[2];
    }
};

// ------------------------------------------------------------ release
// Potential.omega, main.py:88-96
template <class S>
S omega(const S x[3], const S v[3]) {
    S rad = sqrt_(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
    S L0 = x[1] * v[2] - x[2] * v[1];
    S L1 = x[2] * v[0] - x[0] * v[2];
    S L2 = x[0] * v[1] - x[1] * v[0];
    S r2 = rad * rad;
    S o0 = L0 / r2, o1 = L1 / r2, o2 = L2 / r2;
    return sqrt_(o0 * o0 + o1 * o1 + o2 * o2);
}

// Potential.d2phidr2, main.py:76-85: r_hat^T (Hessian) r_hat
template <class S>
S d2phidr2(const ss_potential& P, const S x[3], double t) {
    S rad = sqrt_(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
    S rh[3] = {x[0] / rad, x[1] / rad, x[2] / rad};
    S g[3], H[3][3];
    hess_total<S>(P, x, t, nullptr, g, H);
    S acc(0.0);
    for (int i = 0; i < 3; ++i) {
        S row(0.0);
        for (int j = 0; j < 3; ++j) row = row + H[i][j] * rh[j];
        acc = acc + row * rh[i];
    }
    return acc;
}

// Potential.tidalr, main.py:98-104
template <class S>
S tidalr(const ss_potential& P, const S x[3], const S v[3], double Msat, double t) {
    S om = omega(x, v);
    return pow_(P.G * Msat / (om * om - d2phidr2(P, x, t)), 1.0 / 3.0);
}

// Potential.release_model, main.py:209-280, with the four Gaussian draws
// (main.py:263-266) supplied as z[0..3].
template <class S>
void release_fardal(const ss_potential& P, const S x[3], const S v[3], double Msat, double t,
                    const double* z, const double* kv, S out[2][6]) {
    double kr_bar = kv[0], kvphi_bar = kv[1], kz_bar = kv[2], kvz_bar = kv[3];
    double s_kr = kv[4], s_kvphi = kv[5], s_kz = kv[6], s_kvz = kv[7];
    S om = omega(x, v);
    S r = sqrt_(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
    S rh[3] = {x[0] / r, x[1] / r, x[2] / r};
    S r_t = tidalr(P, x, v, Msat, t);
    S v_circ = om * r_t;
    S L[3] = {x[1] * v[2] - x[2] * v[1], x[2] * v[0] - x[0] * v[2], x[0] * v[1] - x[1] * v[0]};
    S Ln = sqrt_(L[0] * L[0] + L[1] * L[1] + L[2] * L[2]);
    S zh[3] = {L[0] / Ln, L[1] / Ln, L[2] / Ln};
    S vr = v[0] * rh[0] + v[1] * rh[1] + v[2] * rh[2];
    S pv[3] = {v[0] - vr * rh[0], v[1] - vr * rh[1], v[2] - vr * rh[2]};
    S pn = sqrt_(pv[0] * pv[0] + pv[1] * pv[1] + pv[2] * pv[2]);
    S ph[3] = {pv[0] / pn, pv[1] / pn, pv[2] / pn};
    double kr = kr_bar + z[0] * s_kr;
    double kvphi = kr * (kvphi_bar + z[1] * s_kvphi);
    double kz = kz_bar + z[2] * s_kz;
    double kvz = kvz_bar + z[3] * s_kvz;
    for (int i = 0; i < 3; ++i) {
        // trailing arm (main.py:269-272)
        S pt = x[i] + kr * rh[i] * r_t;
        pt = pt + zh[i] * kz * r_t;
        S vt = v[i] + kvphi * v_circ * ph[i];
        vt = vt + kvz * v_circ * zh[i];
        // leading arm (main.py:275-278)
        S pl = x[i] + kr * rh[i] * (-r_t);
        pl = pl + zh[i] * kz * (-r_t);
        S vl = v[i] + kvphi * v_circ * (-1.0) * ph[i];
        vl = vl + kvz * v_circ * (-1.0) * zh[i];
        out[0][i] = pl;
        out[0][3 + i] = vl;
        out[1][i] = pt;
        out[1][3 + i] = vt;
    }
}

// release_model_Chen25, streamhelpers.py:352-432, with the multivariate
// normal draw given as posvel = mean + L z.
template <class S>
void release_chen25(const ss_potential& P, const S x[3], const S v[3], double Msat, double t,
                    const double* z, const double* mean, const double* Lc, S out[2][6]) {
    S r_t = tidalr(P, x, v, Msat, t);
    double pvs[6];
    for (int i = 0; i < 6; ++i) {
        double s = mean[i];
        for (int j = 0; j < 6; ++j) s += Lc[6 * i + j] * z[j];
        pvs[i] = s;
    }
    S r = sqrt_(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
    S xh[3] = {x[0] / r, x[1] / r, x[2] / r};
    S L[3] = {x[1] * v[2] - x[2] * v[1], x[2] * v[0] - x[0] * v[2], x[0] * v[1] - x[1] * v[0]};
    S Ln = sqrt_(L[0] * L[0] + L[1] * L[1] + L[2] * L[2]);
    S zh[3] = {L[0] / Ln, L[1] / Ln, L[2] / Ln};
    S vr = v[0] * xh[0] + v[1] * xh[1] + v[2] * xh[2];
    S pv[3] = {v[0] - vr * xh[0], v[1] - vr * xh[1], v[2] - vr * xh[2]};
    S pn = sqrt_(pv[0] * pv[0] + pv[1] * pv[1] + pv[2] * pv[2]);
    S yh[3] = {pv[0] / pn, pv[1] / pn, pv[2] / pn};
    S Dr = pvs[0] * r_t;
    S v_esc = sqrt_(2.0 * P.G * Msat / Dr);
    S Dv = pvs[3] * v_esc;
    const double deg = 0.017453292519943295;
    double phi = pvs[1] * deg, theta = pvs[2] * deg, alpha = pvs[4] * deg, beta = pvs[5] * deg;
    double ct = std::cos(theta), st = std::sin(theta), cp = std::cos(phi), sp = std::sin(phi);
    double ca = std::cos(alpha), sa = std::sin(alpha), cb = std::cos(beta), sb = std::sin(beta);
    for (int i = 0; i < 3; ++i) {
        S ax = (Dr * ct * cp) * xh[i], ay = (Dr * ct * sp) * yh[i], az = (Dr * st) * zh[i];
        S bx = (Dv * cb * ca) * xh[i], by = (Dv * cb * sa) * yh[i], bz = (Dv * sb) * zh[i];
        out[1][i] = x[i] + ax + ay + az;
        out[1][3 + i] = v[i] + bx + by + bz;
        out[0][i] = x[i] - ax - ay + az;
        out[0][3 + i] = v[i] - bx - by + bz;
    }
}

// ------------------------------------------------------ perturbation term
// MassRadiusPerturbation_OTF.term, fields.py:174-206.  State layout:
// y[0:6] = base (x0, v0); then per subhalo s, ncol columns:
// [dx/deps (3), dv/deps (3), d2x/deps dr (3), d2v/deps dr (3)].
struct PertRHS {
    const ss_potential* P;  // base potential (no subhalos)
    const ss_subhalos* sh;
    int ncol;
    void operator()(double t, const double* y, double* dy) const {
        const double* x0 = y;
        double phi, g[3], H[3][3];
        hess_total<double>(*P, x0, t, &phi, g, H);
        dy[0] = y[3];
        dy[1] = y[4];
        dy[2] = y[5];
        dy[3] = -g[0];
        dy[4] = -g[1];
        dy[5] = -g[2];
        // tidal tensor d2H/dq2 = -Hessian (fields.py:190)
        double T[3][3];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) T[i][j] = -H[i][j];
        // second order (MassRadiusPerturbation_OTF_SecondOrder, fields.py:260-320):
        // d2a_dx2[i][j][k] = d^2 a_i / dx_j dx_k = -d^3 Phi, by AD of the Hessian
        double d2a[3][3][3] = {};
        if (ncol == 18) {
            typedef Dual<double, 3> D3;
            D3 xd[3], ph, gg[3], HH[3][3];
            for (int i = 0; i < 3; ++i) xd[i] = D3::var(x0[i], i);
            hess_total<D3>(*P, xd, t, &ph, gg, HH);
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j)
                    for (int k = 0; k < 3; ++k) d2a[i][j][k] = -HH[i][j].d[k];
        }
        for (int64_t s = 0; s < sh->n; ++s) {
            // -jacfwd(potential_per_SH) and -jacfwd(structural potential_per_SH)
            // for subhalo s (perturbative.py:40-41): gradient in x of Phi_s and
            // of dPhi_s/da, by AD in x (outer) and a (inner).
            typedef Dual<double, 1> Da;
            typedef Dual<Da, 3> Dx;
            Dx xd[3];
            for (int i = 0; i < 3; ++i) xd[i] = Dx::var(Da(x0[i]), i);
            Da a = Da::var(sh->a[s], 0);
            Dx f = phi_subhalo<Dx>(sh->kind, P->G, sh->m[s], Dx::cst(a), sh->x0 + 3 * s,
                                   sh->v + 3 * s, sh->t0[s], sh->t_window, xd, t, sh, s);
            double a1[3], a1r[3];
            for (int i = 0; i < 3; ++i) {
                a1[i] = -f.d[i].v;
                a1r[i] = -f.d[i].d[0];
            }
            const double* u = y + 6 + (size_t)s * ncol;
            double* du = dy + 6 + (size_t)s * ncol;
            for (int i = 0; i < 3; ++i) {
                du[i] = u[3 + i];
                double acc = a1[i];
                for (int j = 0; j < 3; ++j) acc += T[i][j] * u[j];
                du[3 + i] = acc;
            }
            if (ncol >= 12) {
                for (int i = 0; i < 3; ++i) {
                    du[6 + i] = u[9 + i];
                    double acc = a1r[i];
                    for (int j = 0; j < 3; ++j) acc += T[i][j] * u[6 + j];
                    du[9 + i] = acc;
                }
            }
            if (ncol == 18) {
                // dapert_dx = -(Hessian of Phi_s), by nested AD in x
                typedef Dual<double, 3> I3;
                typedef Dual<I3, 3> O3;
                O3 xs2[3];
                for (int i = 0; i < 3; ++i) xs2[i] = O3::var(I3::var(x0[i], i), i);
                O3 fs = phi_subhalo<O3>(sh->kind, P->G, sh->m[s], O3(sh->a[s]), sh->x0 + 3 * s, sh->v + 3 * s,
                                        sh->t0[s], sh->t_window, xs2, t, sh, s);
                // d2a = T x2 + einsum('ikj,nk->nij') contracted with x1 + dapert_dx x1
                for (int i = 0; i < 3; ++i) {
                    du[12 + i] = u[15 + i];
                    double acc = 0.0;
                    for (int j = 0; j < 3; ++j) acc += T[i][j] * u[12 + j];
                    for (int k = 0; k < 3; ++k)
                        for (int j = 0; j < 3; ++j) acc += d2a[i][k][j] * u[k] * u[j];
                    for (int j = 0; j < 3; ++j) acc += -fs.d[i].d[j] * u[j];
                    du[15 + i] = acc;
                }
            }
        }
    }
};

}  // namespace orc

using namespace orc;

extern "C" {

int or_abi_version(void) { return SS_ABI_VERSION; }

int64_t or_abi_sizeof(int which) {
    switch (which) {
        case 0: return (int64_t)sizeof(ss_potential);
        case 1: return (int64_t)sizeof(ss_stream_cfg);
        case 2: return (int64_t)sizeof(ss_release_cfg);
        case 3: return (int64_t)sizeof(ss_pert_cfg);
        case 4: return (int64_t)sizeof(ss_component);
        case 5: return (int64_t)sizeof(ss_track);
        case 6: return (int64_t)sizeof(ss_subhalos);
        case 7: return (int64_t)sizeof(ss_expansion);
        case 8: return (int64_t)sizeof(ss_mlp);
        default: return -1;
    }
}

void or_track_slopes(const double* knots, int64_t n, double dt, double* slopes) {
    track_slopes(knots, n, dt, slopes);
}

void or_track_eval(const ss_potential* P, const double* t, int64_t n, double* out) {
    for (int64_t i = 0; i < n; ++i) track_eval(P->track, t[i], out + 3 * i);
}

// Phi, grad, Hessian at n points (any output may be NULL).
void or_potential_eval(const ss_potential* P, const double* xyz, int64_t n, const double* t,
                       double t_scalar, double* phi, double* grad, double* hess) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        double ti = t ? t[i] : t_scalar;
        const double* x = xyz + 3 * i;
        double f, g[3], H[3][3];
        hess_total<double>(*P, x, ti, &f, g, H);
        if (phi) phi[i] = f;
        if (grad)
            for (int k = 0; k < 3; ++k) grad[3 * i + k] = g[k];
        if (hess)
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) hess[9 * i + 3 * a + b] = H[a][b];
    }
}

// Gradient only (first-order AD), as the integrators use it.
void or_gradient(const ss_potential* P, const double* xyz, int64_t n, double t, double* grad) {
    for (int64_t i = 0; i < n; ++i) grad_total<double>(*P, xyz + 3 * i, t, grad + 3 * i);
}

// Fixed-step Dopri5 orbits: out [n_orbits, n_steps/save_every + 1, 6].
void or_orbit(const ss_potential* P, const double* w0, int64_t n_orbits, double t0, double dt,
              int64_t n_steps, int64_t save_every, double* out) {
    int64_t n_save = n_steps / save_every + 1;
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t o = 0; o < n_orbits; ++o) {
        HamRHS f{P};
        std::vector<double> w;
        double y[6];
        for (int i = 0; i < 6; ++i) y[i] = w0[6 * o + i];
        double* base = out + (size_t)o * n_save * 6;
        for (int i = 0; i < 6; ++i) base[i] = y[i];
        for (int64_t n = 0; n < n_steps; ++n) {
            dopri5_step(f, t0 + (double)n * dt, dt, y, 6, w);
            if ((n + 1) % save_every == 0)
                for (int i = 0; i < 6; ++i) base[6 * ((n + 1) / save_every) + i] = y[i];
        }
    }
}

// Release model; jac (nullable) = d(ics)/d(prog_w) by forward-mode AD with
// third derivatives of the potential (BaseStreamModel.release_func_jacobian,
// perturbative.py:280-296).
void or_release(const ss_potential* P, const ss_release_cfg* cfg, const double* prog_w,
                const double* t_rel, const double* msat, const double* normals, double* ics,
                double* jac) {
    const int nz = cfg->model == SS_RELEASE_CHEN25 ? 6 : 4;
    const int64_t total = cfg->n_release * cfg->n_draw;
#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t q = 0; q < total; ++q) {
        int64_t r = q / cfg->n_draw;
        const double* w = prog_w + 6 * r;
        const double* z = normals + (size_t)q * nz;
        double x[3] = {w[0], w[1], w[2]}, v[3] = {w[3], w[4], w[5]};
        double out[2][6];
        if (cfg->model == SS_RELEASE_CHEN25)
            release_chen25<double>(*P, x, v, msat[r], t_rel[r], z, cfg->chen_mean, cfg->chen_L, out);
        else
            release_fardal<double>(*P, x, v, msat[r], t_rel[r], z, cfg->kvals, out);
        for (int a = 0; a < 2; ++a)
            for (int i = 0; i < 6; ++i) ics[(size_t)q * 12 + 6 * a + i] = out[a][i];
        if (jac) {
            typedef Dual<double, 6> D6;
            D6 xd[3], vd[3];
            for (int i = 0; i < 3; ++i) {
                xd[i] = D6::var(w[i], i);
                vd[i] = D6::var(w[3 + i], 3 + i);
            }
            D6 od[2][6];
            if (cfg->model == SS_RELEASE_CHEN25)
                release_chen25<D6>(*P, xd, vd, msat[r], t_rel[r], z, cfg->chen_mean, cfg->chen_L, od);
            else
                release_fardal<D6>(*P, xd, vd, msat[r], t_rel[r], z, cfg->kvals, od);
            for (int a = 0; a < 2; ++a)
                for (int i = 0; i < 6; ++i)
                    for (int j = 0; j < 6; ++j) jac[(size_t)q * 72 + 36 * a + 6 * i + j] = od[a][i].d[j];
        }
    }
}

// Stream integration (gen_stream_vmapped, main.py:343-368): particle p starts
// at global step (p / ppr) * spr and takes fixed Dopri5 steps to n_steps.
void or_stream(const ss_potential* P, const ss_stream_cfg* cfg, const double* ics, double* final_w,
               float* snaps, int32_t* status, int n_threads) {
#ifdef _OPENMP
    if (n_threads > 0) omp_set_num_threads(n_threads);
#endif
    const int64_t N = cfg->n_particles;
    const int64_t n_snap = cfg->snap_stride > 0 ? cfg->n_steps / cfg->snap_stride : 0;
    const float fnan = std::numeric_limits<float>::quiet_NaN();
#pragma omp parallel for schedule(dynamic, 8)
    for (int64_t p = 0; p < N; ++p) {
        // ensembles: particle p is particle p % stream_particles of stream
        // p / stream_particles, which feels its own subhalo rows
        const int64_t grp = cfg->stream_particles;
        const int64_t pg = p + cfg->first_particle;  // global index (sub-range runs)
        const int64_t pl = grp > 0 ? pg % grp : pg;
        ss_potential Pl = *P;
        if (cfg->subhalos_per_stream > 0) {
            const int64_t k = cfg->subhalos_per_stream, o = (pg / grp) * k;
            Pl.subhalos.n = k;
            Pl.subhalos.m += o;
            Pl.subhalos.a += o;
            Pl.subhalos.x0 += 3 * o;
            Pl.subhalos.v += 3 * o;
            Pl.subhalos.t0 += o;
        }
        HamRHS f{&Pl};
        std::vector<double> w;
        int64_t start = (pl / cfg->particles_per_release) * (int64_t)cfg->steps_per_release;
        double y[6];
        for (int i = 0; i < 6; ++i) y[i] = ics[6 * p + i];
        if (snaps) {
            for (int64_t k = 0; k < n_snap; ++k) {
                int64_t step = (k + 1) * cfg->snap_stride;
                if (step < start)
                    for (int i = 0; i < 6; ++i) snaps[((size_t)k * N + p) * 6 + i] = fnan;
                else if (step == start)
                    for (int i = 0; i < 6; ++i) snaps[((size_t)k * N + p) * 6 + i] = (float)y[i];
            }
        }
        for (int64_t n = start; n < cfg->n_steps; ++n) {
            dopri5_step(f, cfg->t0 + (double)n * cfg->dt, cfg->dt, y, 6, w);
            if (snaps && n_snap > 0 && (n + 1) % cfg->snap_stride == 0) {
                int64_t k = (n + 1) / cfg->snap_stride - 1;
                for (int i = 0; i < 6; ++i) snaps[((size_t)k * N + p) * 6 + i] = (float)y[i];
            }
        }
        bool ok = true;
        for (int i = 0; i < 6; ++i) ok = ok && std::isfinite(y[i]);
        if (status) status[p] = ok ? 0 : 1;
        if (final_w)
            for (int i = 0; i < 6; ++i) final_w[6 * p + i] = y[i];
    }
}

// Subhalo potentials and their derivatives at points (tests):
// phi [n, n_sh], grad [n, n_sh, 3], dphi_da [n, n_sh], grad_dphi_da [n, n_sh, 3].
void or_subhalo_eval(const ss_subhalos* sh, double G, const double* xyz, int64_t n, double t,
                     double* phi, double* grad, double* dphi_da, double* grad_dphi_da) {
    typedef Dual<double, 1> Da;
    typedef Dual<Da, 3> Dx;
    for (int64_t i = 0; i < n; ++i) {
        Dx xd[3];
        for (int k = 0; k < 3; ++k) xd[k] = Dx::var(Da(xyz[3 * i + k]), k);
        for (int64_t s = 0; s < sh->n; ++s) {
            Da a = Da::var(sh->a[s], 0);
            Dx f = phi_subhalo<Dx>(sh->kind, G, sh->m[s], Dx::cst(a), sh->x0 + 3 * s, sh->v + 3 * s,
                                   sh->t0[s], sh->t_window, xd, t, sh, s);
            size_t o = (size_t)i * sh->n + s;
            if (phi) phi[o] = f.v.v;
            if (dphi_da) dphi_da[o] = f.v.d[0];
            for (int k = 0; k < 3; ++k) {
                if (grad) grad[3 * o + k] = f.d[k].v;
                if (grad_dphi_da) grad_dphi_da[3 * o + k] = f.d[k].d[0];
            }
        }
    }
}

// The perturbation vector field itself (fields.py:174-206), for pinning
// against the reference notebook's printed term.
void or_pert_term(const ss_potential* P, const ss_subhalos* sh, int ncol, double t, const double* y,
                  double* dy) {
    PertRHS f{P, sh, ncol};
    f(t, y, dy);
}

// First-order response integration (compute_perturbation_OTF,
// perturbative.py:100-135): the coupled pytree [6 + n_sh*ncol] per particle.
void or_pert_response(const ss_potential* P, const ss_subhalos* sh, const ss_pert_cfg* cfg,
                      const double* base_ics, const double* pert_ics, double* base_out,
                      double* pert_out) {
    const int64_t N = cfg->n_particles;
    const int64_t nsh = sh->n;
    const int ncol = cfg->ncol;
    const int64_t per = nsh * ncol;
    const int64_t n_saves = cfg->save_stride > 0 ? cfg->n_steps / cfg->save_stride + 1 : 1;
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t p = 0; p < N; ++p) {
        PertRHS f{P, sh, ncol};
        std::vector<double> w, y((size_t)(6 + per));
        for (int i = 0; i < 6; ++i) y[i] = base_ics[6 * p + i];
        for (int64_t k = 0; k < per; ++k) y[6 + k] = pert_ics ? pert_ics[(size_t)p * per + k] : 0.0;
        int64_t start = (p / cfg->particles_per_release) * (int64_t)cfg->steps_per_release;
        auto save = [&](int64_t slot) {
            double* o = pert_out + ((size_t)slot * N + p) * per;
            for (int64_t k = 0; k < per; ++k) o[k] = y[6 + k];
        };
        if (cfg->save_stride > 0) {
            // saves before the particle's start hold its initial response
            for (int64_t k = 0; k < n_saves; ++k)
                if (k * cfg->save_stride <= start) save(k);
        }
        for (int64_t n = start; n < cfg->n_steps; ++n) {
            dopri5_step(f, cfg->t0 + (double)n * cfg->dt, cfg->dt, y.data(), (int)(6 + per), w);
            if (cfg->save_stride > 0 && (n + 1) % cfg->save_stride == 0) save((n + 1) / cfg->save_stride);
        }
        if (cfg->save_stride == 0) save(0);
        if (base_out)
            for (int i = 0; i < 6; ++i) base_out[6 * p + i] = y[i];
    }
}

// Binned sums (computed_binned_track, streamhelpers.py:201-228):
// bin(i) = #edges <= key[i] (numpy.digitize, right=False); items with
// bin in [0, n_edges-2] are summed per component, NaN values skipped.
void or_binned_sums(const double* values, const double* key, int64_t n, int32_t ncomp,
                    const double* edges, int32_t n_edges, double* sums, double* counts) {
    int32_t nb = n_edges - 1;
    for (int64_t i = 0; i < (int64_t)nb * ncomp; ++i) {
        sums[i] = 0.0;
        counts[i] = 0.0;
    }
    for (int64_t i = 0; i < n; ++i) {
        double k = key[i];
        int32_t b = 0;
        while (b < n_edges && edges[b] <= k) ++b;
        if (b >= nb) continue;
        for (int c = 0; c < ncomp; ++c) {
            double v = values[(size_t)i * ncomp + c];
            if (std::isnan(v)) continue;
            sums[(size_t)b * ncomp + c] += v;
            counts[(size_t)b * ncomp + c] += 1.0;
        }
    }
}

}  // extern "C"
