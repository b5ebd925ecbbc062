// ss_api.cu — C ABI entry points for potential evaluation, FP64 orbits,
// the progenitor track, the release model, binned sums and the FMA peak probe.
// The stream kernels live in ss_stream.cu, the response kernels in ss_pert.cu.

#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <atomic>
#include <algorithm>
#include <cmath>

#include "ss_release.cuh"

namespace ssg {

static thread_local char g_err[512] = "";
static std::atomic<long long> g_launches{0};

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

int set_error(int code, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}

const char* last_error() { return g_err; }

// (v - R(v)) / R(v) in R: the relative rounding error of storing v as R
// (0 when R is double).
template <class R>
static R rel_residual(double v) {
    if constexpr (std::is_same<R, double>::value) {
        return R(0);
    } else {
        const double r = (double)R(v);
        return r != 0.0 ? R((v - r) / r) : R(0);
    }
}

template <class R>
int prepare_potential(const ss_potential* in, PotDev<R>* out, bool allow_subhalos) {
    SS_CHECK_ARG(in != nullptr, "potential is NULL");
    SS_CHECK_ARG(in->n_components >= 0 && in->n_components <= SS_MAX_COMPONENTS,
                 "n_components=%d outside [0, %d]", in->n_components, SS_MAX_COMPONENTS);
    SS_CHECK_ARG(std::isfinite(in->G) && in->G > 0.0, "G must be finite and > 0");
    memset(out, 0, sizeof(*out));
    out->n = in->n_components;
    bool need_track = false;
    bool need_expansion = false;
    const double G = in->G;
    for (int k = 0; k < in->n_components; ++k) {
        const ss_component& c = in->comp[k];
        const double* p = c.p;
        CompDev<R>& d = out->c[k];
        d.kind = c.kind;
        SS_CHECK_ARG((c.center & ~(SS_CENTER_TRACK | SS_GROWS)) == 0, "component %d: center=%d invalid", k, c.center);
        d.center = c.center & SS_CENTER_TRACK;
        need_track |= (d.center == SS_CENTER_TRACK);
        if (c.center & SS_GROWS) out->grow_mask |= 1 << k;
        for (int i = 0; i < 6; ++i) SS_CHECK_ARG(std::isfinite(p[i]), "component %d: non-finite parameter p[%d]", k, i);
        // FP32 only: slot 5 of the spherical and disk kinds holds the relative
        // rounding of q[0] = G m, (G m - q[0]) / q[0], and slot 4 of NFW that
        // of q[2] = 1 / r_s, so that a kernel can restore them to FP64
        // accuracy with one FMA each (a fixed relative error in a
        // component's mass biases every orbit the same way); zero in FP64
        if (c.kind == SS_NFW || c.kind == SS_MIYAMOTO_NAGAI || c.kind == SS_HERNQUIST || c.kind == SS_PLUMMER ||
            c.kind == SS_ISOCHRONE)
            d.q[5] = rel_residual<R>(G * p[0]);
        switch (c.kind) {
            case SS_NFW:
                SS_CHECK_ARG(p[1] > 0.0 && p[2] >= 0.0, "component %d (NFW): need r_s > 0, soft >= 0", k);
                d.q[0] = R(G * p[0]); d.q[1] = R(p[1]); d.q[2] = R(1.0 / p[1]); d.q[3] = R(p[2]);
                d.q[4] = rel_residual<R>(1.0 / p[1]);
                break;
            case SS_TRIAXIAL_NFW:
                SS_CHECK_ARG(p[1] > 0.0 && p[2] > 0.0 && p[3] > 0.0 && p[4] > 0.0,
                             "component %d (TriaxialNFW): need r_s, q1, q2, q3 > 0", k);
                d.q[0] = R(G * p[0]); d.q[1] = R(p[1]); d.q[2] = R(1.0 / p[2]); d.q[3] = R(1.0 / p[3]);
                d.q[4] = R(1.0 / p[4]); d.q[5] = R(1.0 / p[1]);
                break;
            case SS_MIYAMOTO_NAGAI:
                SS_CHECK_ARG(p[1] >= 0.0 && p[2] > 0.0, "component %d (MiyamotoNagai): need a >= 0, b > 0", k);
                d.q[0] = R(G * p[0]); d.q[1] = R(p[1]); d.q[2] = R(p[2] * p[2]);
                break;
            case SS_HERNQUIST:
                SS_CHECK_ARG(p[1] >= 0.0 && p[2] >= 0.0, "component %d (Hernquist): need r_s >= 0, soft >= 0", k);
                d.q[0] = R(G * p[0]); d.q[1] = R(p[1]); d.q[2] = R(p[2]);
                break;
            case SS_PLUMMER:
                SS_CHECK_ARG(p[1] >= 0.0, "component %d (Plummer): need r_s >= 0", k);
                d.q[0] = R(G * p[0]); d.q[1] = R(p[1] * p[1]);
                break;
            case SS_ISOCHRONE:
                SS_CHECK_ARG(p[1] > 0.0, "component %d (Isochrone): need a > 0", k);
                d.q[0] = R(G * p[0]); d.q[1] = R(p[1]); d.q[2] = R(p[1] * p[1]);
                break;
            case SS_POWERLAW_CUTOFF: {
                // q = {G m, a = (3 - alpha) / 2, 1 / r_c^2, ln Gamma(a), ln Gamma(a - 1/2) (NaN for
                // a <= 1/2: no potential value), 1 / r_c}
                SS_CHECK_ARG(p[1] < 3.0 && p[2] > 0.0, "component %d (PowerLawCutoff): need alpha < 3, r_c > 0", k);
                const double a = 0.5 * (3.0 - p[1]);
                d.q[0] = R(G * p[0]); d.q[1] = R(a); d.q[2] = R(1.0 / (p[2] * p[2])); d.q[3] = R(std::lgamma(a));
                d.q[4] = R(a > 0.5 ? std::lgamma(a - 0.5) : std::nan("")); d.q[5] = R(1.0 / p[2]);
                break;
            }
            case SS_ZHAO: {
                // q = {G m, 1 / r_s, 1 / alpha, a1 = alpha (3 - gamma), b1 = alpha (beta - 3), ln B(a1, b1)};
                // gamma < 2 keeps the potential's second incomplete beta function proper (the reference
                // replaces alpha (2 - gamma) <= 0 by sqrt(eps), a different potential)
                SS_CHECK_ARG(p[1] > 0.0 && p[2] > 0.0 && p[3] > 3.0 && p[4] >= 0.0 && p[4] < 2.0,
                             "component %d (Zhao): need r_s > 0, alpha > 0, beta > 3, 0 <= gamma < 2", k);
                const double a1 = p[2] * (3.0 - p[4]), b1 = p[2] * (p[3] - 3.0);
                d.q[0] = R(G * p[0]); d.q[1] = R(1.0 / p[1]); d.q[2] = R(1.0 / p[2]); d.q[3] = R(a1);
                d.q[4] = R(b1); d.q[5] = R(std::lgamma(a1) + std::lgamma(b1) - std::lgamma(a1 + b1));
                break;
            }
            case SS_SH_EXPANSION: {
                const ss_expansion& e = in->expansion;
                SS_CHECK_ARG(!need_expansion, "component %d: only one SS_SH_EXPANSION component per potential", k);
                SS_CHECK_ARG(e.coef != nullptr, "component %d (expansion): coefficient table is NULL", k);
                SS_CHECK_ARG(e.l_max >= 0 && e.l_max <= SS_SHEXP_LMAX, "component %d (expansion): l_max=%d outside [0, %d]",
                             k, e.l_max, SS_SHEXP_LMAX);
                SS_CHECK_ARG(e.n_knots >= 2 && e.n_knots <= (1 << 20), "component %d (expansion): need >= 2 knots", k);
                SS_CHECK_ARG(std::isfinite(e.log_r0) && std::isfinite(e.dlog_r) && e.dlog_r > 0.0,
                             "component %d (expansion): need finite log_r0 and dlog_r > 0", k);
                need_expansion = true;
                d.q[0] = R(p[0]);
                out->ex.tab64 = e.coef;
                out->ex.tab32 = nullptr;
                out->ex.u0 = e.log_r0;
                out->ex.du = e.dlog_r;
                out->ex.inv_du = 1.0 / e.dlog_r;
                out->ex.nk = e.n_knots;
                out->ex.lmax = e.l_max;
                break;
            }
            case SS_BAR:
            case SS_DEHNEN_BAR: {
                const double om = c.kind == SS_BAR ? p[4] : p[5];
                SS_CHECK_ARG(!out->has_rot || out->omega == om,
                             "component %d: the rotating components of one potential need one pattern speed", k);
                out->has_rot = 1;
                out->omega = om;
                if (c.kind == SS_BAR) {
                    SS_CHECK_ARG(p[1] > 0.0 && p[2] >= 0.0 && p[3] >= 0.0, "component %d (Bar): need a > 0, b, c >= 0",
                                 k);
                    d.q[0] = R(G * p[0] / (2.0 * p[1])); d.q[1] = R(p[1]); d.q[2] = R(p[2]); d.q[3] = R(p[3] * p[3]);
                } else {
                    SS_CHECK_ARG(p[3] > 0.0, "component %d (DehnenBar): need Rb > 0", k);
                    const double rr = p[2] / p[3];
                    d.q[0] = R(p[0] * p[1] * p[1] / 3.0 * rr * rr * rr); d.q[1] = R(p[3]);
                    d.q[2] = R(cos(2.0 * p[4])); d.q[3] = R(sin(2.0 * p[4]));
                }
                break;
            }
            case SS_UNIFORM_ACCEL: {
                const ss_track& fv = in->frame_velocity;
                SS_CHECK_ARG(fv.knots != nullptr && fv.n_knots >= 2 && std::isfinite(fv.dt) && fv.dt > 0.0 &&
                                 std::isfinite(fv.t0) && (fv.linear || fv.slopes != nullptr),
                             "component %d (UniformAcceleration): frame_velocity track needs >= 2 knots, dt > 0", k);
                out->has_facc = 1;
                out->fvel.knots = fv.knots;
                out->fvel.slopes = fv.slopes;
                out->fvel.t0 = fv.t0;
                out->fvel.dt = fv.dt;
                out->fvel.n = fv.n_knots;
                out->fvel.linear = fv.linear ? 1 : 0;
                break;
            }
            default:
                return set_error(SS_ERR_INVALID_ARGUMENT, "component %d: unknown kind %d", k, c.kind);
        }
    }
    if (out->grow_mask) {
        const ss_track& gr = in->growth;
        SS_CHECK_ARG(gr.knots != nullptr && gr.n_knots >= 2 && std::isfinite(gr.dt) && gr.dt > 0.0 &&
                         std::isfinite(gr.t0) && (gr.linear || gr.slopes != nullptr),
                     "SS_GROWS components need a growth track with >= 2 knots, dt > 0");
        out->growth.knots = gr.knots;
        out->growth.slopes = gr.slopes;
        out->growth.t0 = gr.t0;
        out->growth.dt = gr.dt;
        out->growth.n = gr.n_knots;
        out->growth.linear = gr.linear ? 1 : 0;
    }
    out->has_track = need_track ? 1 : 0;
    if (need_track) {
        const ss_track& tr = in->track;
        SS_CHECK_ARG(tr.knots != nullptr && (tr.linear || tr.slopes != nullptr), "center track: knots/slopes NULL");
        SS_CHECK_ARG(tr.n_knots >= 2, "center track: need >= 2 knots");
        SS_CHECK_ARG(std::isfinite(tr.dt) && tr.dt > 0.0 && std::isfinite(tr.t0), "center track: need dt > 0");
        out->track.knots = tr.knots;
        out->track.slopes = tr.slopes;
        out->track.t0 = tr.t0;
        out->track.dt = tr.dt;
        out->track.n = tr.n_knots;
        out->track.linear = tr.linear ? 1 : 0;
    }
    const ss_subhalos& sh = in->subhalos;
    SS_CHECK_ARG(sh.n >= 0 && sh.n <= (int64_t)1 << 30, "subhalos: bad n");
    if (sh.n > 0) {
        SS_CHECK_ARG(allow_subhalos, "this entry point takes the subhalos separately; potential.subhalos must be empty");
        SS_CHECK_ARG(sh.kind == SS_SH_PLUMMER || sh.kind == SS_SH_HERNQUIST || sh.kind == SS_SH_GRID,
                     "subhalos: unknown kind %d", sh.kind);
        SS_CHECK_ARG(sh.m && sh.a && sh.x0 && sh.v && sh.t0, "subhalos: NULL table pointer");
        SS_CHECK_ARG(!(sh.t_window < 0.0), "subhalos: t_window < 0");
        SS_CHECK_ARG(sh.kind != SS_SH_GRID ||
                         (sh.grid && sh.grid_u0 && sh.grid_du && sh.n_grid >= 2 && sh.n_grid <= (1 << 20)),
                     "subhalos: SS_SH_GRID needs grid tables with >= 2 knots");
        out->sh.grid = sh.grid;
        out->sh.gu0 = sh.grid_u0;
        out->sh.gdu = sh.grid_du;
        out->sh.ng = (int32_t)sh.n_grid;
        out->sh.kind = sh.kind;
        out->sh.n = (int32_t)sh.n;
        out->sh.m = sh.m;
        out->sh.a = sh.a;
        out->sh.x0 = sh.x0;
        out->sh.v = sh.v;
        out->sh.t0 = sh.t0;
        out->sh.t_window = sh.t_window;
        out->sh.G = G;
    }
    return SS_OK;
}

template int prepare_potential<double>(const ss_potential*, PotDev<double>*, bool);
template int prepare_potential<float>(const ss_potential*, PotDev<float>*, bool);

// ------------------------------------------------------------- Phi (FP64)
__device__ double comp_phi(const PotDev<double>& P, const CompDev<double>& c, const double xin[3],
                           const TimeDep<double>& td = TimeDep<double>()) {
    const double* q = c.q;
    // rotating components: their corotating-frame position
    const bool rot = c.kind == SS_BAR || c.kind == SS_DEHNEN_BAR;
    const double x[3] = {rot ? td.c * xin[0] + td.s * xin[1] : xin[0], rot ? td.c * xin[1] - td.s * xin[0] : xin[1],
                         xin[2]};
    double r2 = x[0] * x[0] + x[1] * x[1] + x[2] * x[2];
    switch (c.kind) {
        case SS_BAR: {
            const double B = q[2] + sqrt(q[3] + x[2] * x[2]);
            const double rho2 = x[1] * x[1] + B * B;
            const double wm = x[0] - q[1], wp = x[0] + q[1];
            return q[0] * log((wm + sqrt(wm * wm + rho2)) / (wp + sqrt(wp * wp + rho2)));
        }
        case SS_DEHNEN_BAR: {
            const double r = sqrt(r2), Rb = q[1];
            const double W = r >= Rb ? -Rb * Rb * Rb / (r2 * r2 * r) : r / (Rb * Rb * Rb) - 2.0 / r2;
            return q[0] * W * ((x[0] * x[0] - x[1] * x[1]) * q[2] + 2.0 * x[0] * x[1] * q[3]);
        }
        case SS_UNIFORM_ACCEL:
            return 0.0;  // a force without a potential (UniformAcceleration.potential raises)
        case SS_SH_EXPANSION:
            return shexp_phi(P.ex, q[0], x);
        case SS_NFW: {
            double r = sqrt(r2 + q[3]);
            return -q[0] * log1p(r * q[2]) / r;
        }
        case SS_TRIAXIAL_NFW: {
            double a = x[0] * q[2], b = x[1] * q[3], d = x[2] * q[4];
            double r = sqrt(a * a + b * b + d * d);
            return -q[0] * log1p(r * q[5]) / r;
        }
        case SS_MIYAMOTO_NAGAI: {
            double az = sqrt(x[2] * x[2] + q[2]) + q[1];
            return -q[0] / sqrt(x[0] * x[0] + x[1] * x[1] + az * az);
        }
        case SS_HERNQUIST:
            return -q[0] / (sqrt(r2 + q[2]) + q[1]);
        case SS_PLUMMER:
            return -q[0] / sqrt(r2 + q[1]);
        case SS_ISOCHRONE:
            return -q[0] / (q[1] + sqrt(r2 + q[2]));
        case SS_POWERLAW_CUTOFF: {
            // Phi = -G m P(a, x) / r + G m Gamma(a - 1/2) P(a - 1/2, x) / (Gamma(a) r_c), x = r^2 / r_c^2
            // (PowerLawCutoffPotential.potential, potential.py:365-378, with Gamma(a + 1) = a Gamma(a))
            if (!(q[1] > 0.5)) return nan("");
            const double xx = r2 * q[2];
            return -q[0] * gammainc_p(q[1], q[3], xx) / sqrt(r2) +
                   q[0] * exp(q[4] - q[3]) * q[5] * gammainc_p(q[1] - 0.5, q[4], xx);
        }
        case SS_ZHAO: {
            // Phi = -G m (I_z(a1, b1) / r + B(p0, c0 - p0) / B(a1, b1) I_zc(c0 - p0, p0) / r_s),
            // p0 = alpha (2 - gamma) = a1 - alpha, c0 - p0 = alpha (beta - 2) = b1 + alpha, zc = 1 - z
            // (ZhaoPotential._potential, potential.py:314-331, with 4 pi G rho0 alpha = G m / B(a1, b1)
            // and 1 - I_z(p, q) = I_zc(q, p))
            const double r = sqrt(r2), al = 1.0 / q[2];
            const double y = s_pow(r * q[1], q[2]), zc = 1.0 / (1.0 + y), z = y * zc;
            const double p0 = q[3] - al, p1 = q[4] + al;
            const double lb2 = lgamma(p0) + lgamma(p1) - lgamma(p0 + p1);
            return -q[0] * (betainc(q[3], q[4], q[5], z, zc) / r + exp(lb2 - q[5]) * betainc(p1, p0, lb2, zc, z) * q[1]);
        }
        default:
            return nan("");
    }
}

__global__ void potential_eval_kernel(PotDev<double> P, const double* __restrict__ xyz, int64_t n,
                                      const double* __restrict__ tarr, double t_scalar, double* phi,
                                      double* grad, double* hess) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double t = tarr ? tarr[i] : t_scalar;
    double x[3] = {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
    double c[3] = {0.0, 0.0, 0.0};
    if (P.has_track) track_eval(P.track, t, c);
    const TimeDep<double> td = time_dep(P, t);
    if (phi) {
        double f = 0.0;
        for (int k = 0; k < P.n; ++k) {
            const double gk = ((P.grow_mask >> k) & 1) ? td.amp : 1.0;  // GrowingPotential
            if (P.c[k].center == SS_CENTER_TRACK) {
                double xs[3] = {x[0] - c[0], x[1] - c[1], x[2] - c[2]};
                f += gk * comp_phi(P, P.c[k], xs, td);
            } else {
                f += gk * comp_phi(P, P.c[k], x, td);
            }
        }
        for (int j = 0; j < P.sh.n; ++j) {
            double tau = t - P.sh.t0[j];
            if (!(fabs(tau) < P.sh.t_window)) continue;
            double rel[3];
            for (int k = 0; k < 3; ++k) rel[k] = x[k] - (P.sh.x0[3 * j + k] + P.sh.v[3 * j + k] * tau);
            double r2 = rel[0] * rel[0] + rel[1] * rel[1] + rel[2] * rel[2];
            double Gm = P.sh.G * P.sh.m[j], a = P.sh.a[j];
            if (P.sh.kind == SS_SH_GRID) {
                double g, gr, ph;
                grid_subhalo_gh<double, false>(P.sh, j, r2, g, gr, &ph);
                f += ph;
            } else {
                f += P.sh.kind == SS_SH_PLUMMER ? -Gm / sqrt(r2 + a * a) : -Gm / (sqrt(r2) + a);
            }
        }
        phi[i] = f;
    }
    if (grad || hess) {
        double g[3], H[6];
        const double xs[3] = {x[0] - c[0], x[1] - c[1], x[2] - c[2]};
        pot_grad<double, double, true>(P, x, xs, g, H, td);
        if (P.sh.n > 0) subhalo_sum_grad<double>(P.sh, x, t, g);
        if (grad)
            for (int k = 0; k < 3; ++k) grad[3 * i + k] = g[k];
        if (hess) {
            double* o = hess + 9 * i;
            o[0] = H[0]; o[1] = H[3]; o[2] = H[4];
            o[3] = H[3]; o[4] = H[1]; o[5] = H[5];
            o[6] = H[4]; o[7] = H[5]; o[8] = H[2];
        }
    }
}

// ------------------------------------------------------------- orbits
template <class C>
__global__ void __launch_bounds__(64) orbit_f64_kernel(PotDev<double> P, const double* __restrict__ w0,
                                                       int64_t n_orbits, double t0, double dt, int64_t n_steps,
                                                       int64_t save_every, double* __restrict__ out) {
    int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= n_orbits) return;
    const int64_t n_save = n_steps / save_every + 1;
    double y[6];
    for (int i = 0; i < 6; ++i) y[i] = w0[6 * o + i];
    double* base = out + o * n_save * 6;
    for (int i = 0; i < 6; ++i) base[i] = y[i];
    for (int64_t n = 0; n < n_steps; ++n) {
        dopri5_step_f64<C>(P, t0 + (double)n * dt, dt, y);
        if ((n + 1) % save_every == 0) {
            double* b = base + 6 * ((n + 1) / save_every);
            for (int i = 0; i < 6; ++i) b[i] = y[i];
        }
    }
}

// Orbit o with its own step (dts[o], or dt_all) and, for k > 0, its own
// subhalo rows [o k, (o + 1) k).
template <class C>
__global__ void __launch_bounds__(64) orbit_ensemble_kernel(PotDev<double> P, const double* __restrict__ w0,
                                                            int64_t n_orbits, double t0, const double* __restrict__ dts,
                                                            double dt_all, int64_t n_steps, int64_t save_every,
                                                            int32_t k, double* __restrict__ out) {
    int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= n_orbits) return;
    const double dt = dts ? dts[o] : dt_all;
    const ShDev sh = subhalo_slice(P.sh, o, k);
    const int64_t n_save = n_steps / save_every + 1;
    double y[6];
    for (int i = 0; i < 6; ++i) y[i] = w0[6 * o + i];
    double* base = out + o * n_save * 6;
    for (int i = 0; i < 6; ++i) base[i] = y[i];
    for (int64_t n = 0; n < n_steps; ++n) {
        dopri5_step_f64<C>(P, sh, t0 + (double)n * dt, dt, y);
        if ((n + 1) % save_every == 0) {
            double* b = base + 6 * ((n + 1) / save_every);
            for (int i = 0; i < 6; ++i) b[i] = y[i];
        }
    }
}

// ------------------------------------------------------------- track
// Knot slopes as interpax 'cubic' defines them: mean of the adjacent
// secants, one-sided at the ends.
__global__ void track_slopes_kernel(const double* __restrict__ knots, int64_t n, double dt, double* slopes) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 3 * n) return;
    int64_t k = i / 3;
    int c = (int)(i % 3);
    double s;
    if (n < 2) {
        s = 0.0;
    } else if (k == 0) {
        s = (knots[3 + c] - knots[c]) / dt;
    } else if (k == n - 1) {
        s = (knots[3 * k + c] - knots[3 * (k - 1) + c]) / dt;
    } else {
        double sl = (knots[3 * k + c] - knots[3 * (k - 1) + c]) / dt;
        double sr = (knots[3 * (k + 1) + c] - knots[3 * k + c]) / dt;
        s = 0.5 * (sl + sr);
    }
    slopes[i] = s;
}

template <bool JAC>
__global__ void release_kernel(PotDev<double> P, double G, ss_release_cfg cfg, const double* __restrict__ prog_w,
                               const double* __restrict__ t_rel, const double* __restrict__ msat,
                               const double* __restrict__ normals, double* __restrict__ ics,
                               double* __restrict__ jac) {
    int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t total = cfg.n_release * cfg.n_draw;
    if (q >= total) return;
    int64_t r = q / cfg.n_draw;
    const int nz = cfg.model == SS_RELEASE_CHEN25 ? 6 : 4;
    const double* z = normals + q * nz;
    const double* w = prog_w + 6 * r;
    if (!JAC) {
        double x[3] = {w[0], w[1], w[2]}, v[3] = {w[3], w[4], w[5]};
        double out[2][6];
        release_one<double>(P, G, cfg, x, v, msat[r], t_rel[r], z, out);
        for (int a = 0; a < 2; ++a)
            for (int i = 0; i < 6; ++i) ics[q * 12 + 6 * a + i] = out[a][i];
    } else {
        typedef Dual<6> D6;
        D6 x[3], v[3];
        for (int i = 0; i < 3; ++i) {
            x[i] = D6(w[i]);
            x[i].d[i] = 1.0;
            v[i] = D6(w[3 + i]);
            v[i].d[3 + i] = 1.0;
        }
        D6 out[2][6];
        release_one<D6>(P, G, cfg, x, v, msat[r], t_rel[r], z, out);
        for (int a = 0; a < 2; ++a)
            for (int i = 0; i < 6; ++i) {
                ics[q * 12 + 6 * a + i] = out[a][i].v;
                for (int j = 0; j < 6; ++j) jac[q * 72 + 36 * a + 6 * i + j] = out[a][i].d[j];
            }
    }
}

// ------------------------------------------------------------- binned sums
__global__ void binned_sums_kernel(const double* __restrict__ values, const double* __restrict__ key, int64_t n,
                                   int ncomp, const double* __restrict__ edges, int n_edges, double* sums,
                                   double* counts) {
    extern __shared__ double sm[];
    const int nb = n_edges - 1;
    const int nslots = nb * ncomp;
    double* s_sum = sm;
    double* s_cnt = sm + nslots;
    for (int i = threadIdx.x; i < 2 * nslots; i += blockDim.x) sm[i] = 0.0;
    __syncthreads();
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double k = key[i];
        // number of edges <= k (upper bound); NaN keys compare false -> bin 0
        int lo = 0, hi = n_edges;
        while (lo < hi) {
            int mid = (lo + hi) >> 1;
            if (edges[mid] <= k) lo = mid + 1; else hi = mid;
        }
        int b = lo;
        if (b >= nb) continue;
        for (int c = 0; c < ncomp; ++c) {
            double v = values[i * ncomp + c];
            if (isnan(v)) continue;
            atomicAdd(s_sum + b * ncomp + c, v);
            atomicAdd(s_cnt + b * ncomp + c, 1.0);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nslots; i += blockDim.x) {
        if (s_cnt[i] != 0.0) {
            atomicAdd(sums + i, s_sum[i]);
            atomicAdd(counts + i, s_cnt[i]);
        }
    }
}

// ------------------------------------------------------------- FMA peak
template <class T>
__global__ void __launch_bounds__(256) peak_fma_kernel(int64_t iters, T* sink) {
    T a0 = T(threadIdx.x) * T(1e-3), a1 = a0 + T(1), a2 = a0 + T(2), a3 = a0 + T(3);
    T a4 = a0 + T(4), a5 = a0 + T(5), a6 = a0 + T(6), a7 = a0 + T(7);
    const T b = T(0.999999), c = T(1e-6);
    for (int64_t i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            a0 = fma(a0, b, c); a1 = fma(a1, b, c); a2 = fma(a2, b, c); a3 = fma(a3, b, c);
            a4 = fma(a4, b, c); a5 = fma(a5, b, c); a6 = fma(a6, b, c); a7 = fma(a7, b, c);
        }
    }
    T s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
    if (s == T(-12345.678)) sink[threadIdx.x] = s;
}

// The same chains in the packed form of the paired stream kernel: each
// fma.rn.f32x2 instruction is two FP32 FMAs, one per lane.
__global__ void __launch_bounds__(256) peak_fma2_kernel(int64_t iters, float* sink) {
    const float x = (float)threadIdx.x * 1e-3f;
    float2 a0 = make_float2(x, x + 0.5f), a1 = make_float2(x + 1, x + 1.5f), a2 = make_float2(x + 2, x + 2.5f),
           a3 = make_float2(x + 3, x + 3.5f), a4 = make_float2(x + 4, x + 4.5f), a5 = make_float2(x + 5, x + 5.5f),
           a6 = make_float2(x + 6, x + 6.5f), a7 = make_float2(x + 7, x + 7.5f);
    const float2 b = make_float2(0.999999f, 0.999999f), c = make_float2(1e-6f, 1e-6f);
    for (int64_t i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            a0 = __ffma2_rn(a0, b, c); a1 = __ffma2_rn(a1, b, c); a2 = __ffma2_rn(a2, b, c);
            a3 = __ffma2_rn(a3, b, c); a4 = __ffma2_rn(a4, b, c); a5 = __ffma2_rn(a5, b, c);
            a6 = __ffma2_rn(a6, b, c); a7 = __ffma2_rn(a7, b, c);
        }
    }
    const float s = a0.x + a0.y + a1.x + a1.y + a2.x + a2.y + a3.x + a3.y + a4.x + a4.y + a5.x + a5.y + a6.x +
                    a6.y + a7.x + a7.y;
    if (s == -12345.678f) sink[threadIdx.x] = s;
}

__global__ void math_f64_kernel(int fn, const double* __restrict__ x, int64_t n, double* out, double* ref) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double v = x[i];
    if (fn == 0) {
        out[i] = s_rcp(v);
        if (ref) ref[i] = 1.0 / v;
    } else if (fn == 1) {
        out[i] = s_rsqrt(v);
        if (ref) ref[i] = rsqrt(v);
    } else {
        out[i] = s_log1p(v);
        if (ref) ref[i] = log1p(v);
    }
}

}  // namespace ssg

using namespace ssg;

static inline unsigned grid_for(int64_t n, int block) { return (unsigned)((n + block - 1) / block); }

// Device -> pinned host copy by SM stores.  Pinned host memory is
// addressable from kernels under unified addressing (on Grace-Blackwell
// over the coherent chip-to-chip link), so a kernel can move a strided row
// block with plain loads and stores, without the copy engine.  Units of 16,
// 4 or 1 bytes, the widest that every address, the width and the pitch
// allow; a grid-stride loop over the rows x units of the block.
template <class U>
__global__ void __launch_bounds__(256) copy_rows_kernel(char* __restrict__ dst, const char* __restrict__ src,
                                                        int64_t rows, int64_t pitch, int64_t off, int64_t units) {
    const int64_t total = rows * units;
    for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < total;
         u += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = u / units, c = u - r * units;
        const int64_t b = r * pitch + off + c * (int64_t)sizeof(U);
        *reinterpret_cast<U*>(dst + b) = __ldcs(reinterpret_cast<const U*>(src + b));
    }
}

static int copy_rows_sm(void* dst, const void* src, int64_t rows, int64_t pitch, int64_t off, int64_t width,
                        cudaStream_t s) {
    cudaPointerAttributes ad{}, as{};
    if (cudaPointerGetAttributes(&ad, dst) != cudaSuccess || cudaPointerGetAttributes(&as, src) != cudaSuccess) {
        cudaGetLastError();  // not sticky: clear it so that later launch checks do not see it
        return set_error(SS_ERR_INVALID_ARGUMENT, "kind 3: cannot query the buffers' memory types");
    }
    SS_CHECK_ARG(ad.type == cudaMemoryTypeHost && ad.devicePointer != nullptr,
                 "kind 3: dst must be pinned host memory addressable from the device");
    SS_CHECK_ARG(as.type == cudaMemoryTypeDevice || as.type == cudaMemoryTypeManaged,
                 "kind 3: src must be device memory");
    char* d = static_cast<char*>(ad.devicePointer);
    const char* sp = static_cast<const char*>(src);
    auto al = [&](int64_t a) {
        return ((uintptr_t)d % a) == 0 && ((uintptr_t)sp % a) == 0 && off % a == 0 && width % a == 0 && pitch % a == 0;
    };
    int dev = 0, n_sm = 0;
    SS_CUDA_TRY(cudaGetDevice(&dev));
    SS_CUDA_TRY(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev));
    const int64_t ub = al(16) ? 16 : al(4) ? 4 : 1;
    const int64_t units = width / ub, total = rows * units;
    const unsigned grid = (unsigned)std::min<int64_t>((total + 255) / 256, 4 * (int64_t)n_sm);
    if (ub == 16)
        copy_rows_kernel<uint4><<<grid, 256, 0, s>>>(d, sp, rows, pitch, off, units);
    else if (ub == 4)
        copy_rows_kernel<uint32_t><<<grid, 256, 0, s>>>(d, sp, rows, pitch, off, units);
    else
        copy_rows_kernel<unsigned char><<<grid, 256, 0, s>>>(d, sp, rows, pitch, off, units);
    SS_LAUNCH_CHECK();
    return SS_OK;
}

extern "C" {

int ss_abi_version(void) { return SS_ABI_VERSION; }

int64_t ss_kernel_launches(void) { return (int64_t)g_launches.load(std::memory_order_relaxed); }

const char* ss_last_error(void) { return ssg::last_error(); }

int ss_copy_rows_async(void* dst, const void* src, int64_t rows, int64_t pitch_bytes, int64_t offset_bytes,
                       int64_t width_bytes, int kind, void* stream) {
    SS_CHECK_ARG(dst != nullptr && src != nullptr, "NULL buffer");
    SS_CHECK_ARG(rows >= 0 && width_bytes >= 0 && offset_bytes >= 0 && offset_bytes + width_bytes <= pitch_bytes,
                 "bad rows/pitch/offset/width");
    SS_CHECK_ARG(kind >= 0 && kind <= 3, "kind must be 0 (D2H), 1 (H2D), 2 (D2D) or 3 (D2H by SM stores)");
    if (rows == 0 || width_bytes == 0) return SS_OK;
    if (kind == 3) return copy_rows_sm(dst, src, rows, pitch_bytes, offset_bytes, width_bytes, (cudaStream_t)stream);
    const cudaMemcpyKind k = kind == 0 ? cudaMemcpyDeviceToHost : kind == 1 ? cudaMemcpyHostToDevice
                                                                             : cudaMemcpyDeviceToDevice;
    SS_CUDA_TRY(cudaMemcpy2DAsync((char*)dst + offset_bytes, (size_t)pitch_bytes, (const char*)src + offset_bytes,
                                  (size_t)pitch_bytes, (size_t)width_bytes, (size_t)rows, k, (cudaStream_t)stream));
    return SS_OK;
}

int64_t ss_abi_sizeof(int which) {
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

int ss_potential_eval(const ss_potential* pot, const double* xyz, int64_t n, const double* t, double t_scalar,
                      double* phi, double* grad, double* hess, void* stream) {
    PotDev<double> P;
    int rc = prepare_potential<double>(pot, &P, true);
    if (rc) return rc;
    SS_CHECK_ARG(n >= 0, "n < 0");
    if (n == 0) return SS_OK;
    SS_CHECK_ARG(xyz != nullptr, "xyz is NULL");
    potential_eval_kernel<<<grid_for(n, 128), 128, 0, (cudaStream_t)stream>>>(P, xyz, n, t, t_scalar, phi, grad,
                                                                              hess);
    SS_LAUNCH_CHECK();
    return SS_OK;
}

// Threads per block of the one-thread-per-orbit kernels.  An SM's warps
// share its FP64 pipe, so while the orbits fit one warp per SM they are
// spread that way (32-thread blocks); larger batches use 64.
static int orbit_block(int64_t n_orbits) {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                  cudaSuccess)
        return 64;
    return n_orbits <= 32 * (int64_t)sms ? 32 : 64;
}

int ss_orbit_f64(const ss_potential* pot, const double* w0, int64_t n_orbits, double t0, double dt,
                 int64_t n_steps, int64_t save_every, double* out, void* stream) {
    PotDev<double> P;
    int rc = prepare_potential<double>(pot, &P, true);
    if (rc) return rc;
    SS_CHECK_ARG(n_orbits >= 0 && n_steps >= 0, "negative size");
    SS_CHECK_ARG(save_every >= 1, "save_every must be >= 1");
    SS_CHECK_ARG(std::isfinite(dt) && dt != 0.0 && std::isfinite(t0), "dt must be finite and non-zero");
    if (n_orbits == 0) return SS_OK;
    SS_CHECK_ARG(w0 && out, "NULL buffer");
    dispatch_comp(P, [&](auto comp) {
        const int bs = orbit_block(n_orbits);
        orbit_f64_kernel<decltype(comp)><<<grid_for(n_orbits, bs), bs, 0, (cudaStream_t)stream>>>(
            P, w0, n_orbits, t0, dt, n_steps, save_every, out);
        return 0;
    });
    SS_LAUNCH_CHECK();
    return SS_OK;
}

int ss_orbit_ensemble_f64(const ss_potential* pot, const double* w0, int64_t n_orbits, double t0, const double* dt,
                          double dt_all, int64_t n_steps, int64_t save_every, int32_t subhalos_per_orbit, double* out,
                          void* stream) {
    PotDev<double> P;
    int rc = prepare_potential<double>(pot, &P, true);
    if (rc) return rc;
    SS_CHECK_ARG(n_orbits >= 0 && n_steps >= 0, "negative size");
    SS_CHECK_ARG(save_every >= 1, "save_every must be >= 1");
    SS_CHECK_ARG(std::isfinite(t0), "t0 must be finite");
    SS_CHECK_ARG(dt != nullptr || (std::isfinite(dt_all) && dt_all != 0.0), "dt_all must be finite and non-zero");
    SS_CHECK_ARG(subhalos_per_orbit >= 0, "subhalos_per_orbit < 0");
    SS_CHECK_ARG(subhalos_per_orbit == 0 || pot->subhalos.n >= n_orbits * (int64_t)subhalos_per_orbit,
                 "the subhalo table needs subhalos_per_orbit rows for each of the %lld orbits", (long long)n_orbits);
    if (n_orbits == 0) return SS_OK;
    SS_CHECK_ARG(w0 && out, "NULL buffer");
    dispatch_comp(P, [&](auto comp) {
        const int bs = orbit_block(n_orbits);
        orbit_ensemble_kernel<decltype(comp)><<<grid_for(n_orbits, bs), bs, 0, (cudaStream_t)stream>>>(
            P, w0, n_orbits, t0, dt, dt_all, n_steps, save_every, subhalos_per_orbit, out);
        return 0;
    });
    SS_LAUNCH_CHECK();
    return SS_OK;
}

int ss_track_slopes(const double* knots, int64_t n_knots, double dt, double* slopes, void* stream) {
    SS_CHECK_ARG(knots && slopes, "NULL buffer");
    SS_CHECK_ARG(n_knots >= 2, "need >= 2 knots");
    SS_CHECK_ARG(std::isfinite(dt) && dt > 0.0, "dt must be > 0");
    track_slopes_kernel<<<grid_for(3 * n_knots, 256), 256, 0, (cudaStream_t)stream>>>(knots, n_knots, dt, slopes);
    SS_LAUNCH_CHECK();
    return SS_OK;
}

int ss_release_f64(const ss_potential* pot, const ss_release_cfg* cfg, const double* prog_w, const double* t_rel,
                   const double* msat, const double* normals, double* ics, double* jac, void* stream) {
    PotDev<double> P;
    int rc = prepare_potential<double>(pot, &P, true);
    if (rc) return rc;
    SS_CHECK_ARG(cfg != nullptr, "cfg is NULL");
    SS_CHECK_ARG(cfg->n_release >= 0 && cfg->n_draw >= 1, "n_release >= 0 and n_draw >= 1 required");
    SS_CHECK_ARG(cfg->model == SS_RELEASE_FARDAL || cfg->model == SS_RELEASE_CHEN25, "unknown release model %d",
                 cfg->model);
    int64_t total = cfg->n_release * cfg->n_draw;
    if (total == 0) return SS_OK;
    SS_CHECK_ARG(prog_w && t_rel && msat && normals && ics, "NULL buffer");
    cudaStream_t s = (cudaStream_t)stream;
    if (jac)
        release_kernel<true><<<grid_for(total, 64), 64, 0, s>>>(P, pot->G, *cfg, prog_w, t_rel, msat, normals, ics, jac);
    else
        release_kernel<false><<<grid_for(total, 128), 128, 0, s>>>(P, pot->G, *cfg, prog_w, t_rel, msat, normals, ics,
                                                                   nullptr);
    SS_LAUNCH_CHECK();
    return SS_OK;
}

int ss_binned_sums(const double* values, const double* key, int64_t n, int32_t ncomp, const double* edges,
                   int32_t n_edges, double* sums, double* counts, void* stream) {
    SS_CHECK_ARG(ncomp >= 1 && ncomp <= 64, "ncomp must be in [1, 64]");
    SS_CHECK_ARG(n_edges >= 2, "need >= 2 edges");
    SS_CHECK_ARG(n >= 0, "n < 0");
    SS_CHECK_ARG(edges && sums && counts, "NULL buffer");
    int64_t nslots = (int64_t)(n_edges - 1) * ncomp;
    SS_CHECK_ARG(2 * nslots * (int64_t)sizeof(double) <= 96 * 1024, "too many bins x components for one block");
    cudaStream_t s = (cudaStream_t)stream;
    SS_CUDA_TRY(cudaMemsetAsync(sums, 0, nslots * sizeof(double), s));
    SS_CUDA_TRY(cudaMemsetAsync(counts, 0, nslots * sizeof(double), s));
    if (n == 0) return SS_OK;
    SS_CHECK_ARG(values && key, "NULL buffer");
    size_t smem = 2 * nslots * sizeof(double);
    if (smem > 48 * 1024)
        SS_CUDA_TRY(cudaFuncSetAttribute(binned_sums_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int64_t blocks = grid_for(n, 256);
    if (blocks > 4 * 152) blocks = 4 * 152;
    binned_sums_kernel<<<(unsigned)blocks, 256, smem, s>>>(values, key, n, ncomp, edges, n_edges, sums, counts);
    SS_LAUNCH_CHECK();
    return SS_OK;
}

int ss_math_f64(int fn, const double* x, int64_t n, double* out, double* ref, void* stream) {
    SS_CHECK_ARG(fn >= 0 && fn <= 2, "fn must be 0 (reciprocal), 1 (rsqrt) or 2 (log1p)");
    SS_CHECK_ARG(n >= 0, "n < 0");
    if (n == 0) return SS_OK;
    SS_CHECK_ARG(x != nullptr && out != nullptr, "NULL buffer");
    math_f64_kernel<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(fn, x, n, out, ref);
    SS_LAUNCH_CHECK();
    return SS_OK;
}

int ss_peak_fma(int precision, int64_t iters, double* out_flops, float* sink, void* stream) {
    SS_CHECK_ARG(precision == 32 || precision == 64 || precision == 2, "precision must be 32, 64 or 2 (f32x2)");
    SS_CHECK_ARG(iters >= 1 && sink != nullptr, "iters >= 1 and a sink buffer of >= 256 floats required");
    int dev = 0, sms = 0;
    SS_CUDA_TRY(cudaGetDevice(&dev));
    SS_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    unsigned blocks = (unsigned)sms * 8u;
    cudaStream_t s = (cudaStream_t)stream;
    if (precision == 32)
        peak_fma_kernel<float><<<blocks, 256, 0, s>>>(iters, sink);
    else if (precision == 2)
        peak_fma2_kernel<<<blocks, 256, 0, s>>>(iters, sink);
    else
        peak_fma_kernel<double><<<blocks, 256, 0, s>>>(iters, reinterpret_cast<double*>(sink));  // sink >= 512 floats
    SS_LAUNCH_CHECK();
    if (out_flops) *out_flops = (precision == 2 ? 2.0 : 1.0) * 2.0 * 32.0 * (double)iters * 256.0 * (double)blocks;
    return SS_OK;
}

}  // extern "C"
