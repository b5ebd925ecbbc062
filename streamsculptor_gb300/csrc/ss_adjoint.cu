// ss_adjoint.cu — gradients of a loss on the final stream with respect to the
// potential's parameters and the progenitor's present-day phase-space point.
//
// The reference differentiates streams with forward-mode jax.jacfwd through
// diffrax (adjoint=ForwardMode(), main.py:160; tests.ipynb:2959, 3182).  Here
// the gradient is assembled from three pieces, each a kernel:
//   * stream_adjoint_kernel: the discrete adjoint of every particle's FP32
//     Dopri5 steps.  The forward FP32-compensated pass stores the state every
//     K steps; backwards, each K-step segment is recomputed from its
//     checkpoint into a per-thread tape, then stepped back with the
//     transposed stage Jacobians (Hessian-vector products of Phi) while the
//     parameter gradient accumulates (d grad Phi / d theta)^T kappa;
//   * release_vjp_kernel: the release map's vector-Jacobian product, with
//     respect to the progenitor state (forward-mode duals, third derivatives
//     of Phi) and to the potential parameters (through the tidal radius,
//     d(r_hat^T H r_hat)/d theta by one-direction duals);
//   * the progenitor's sensitivities come from ss_prog_tangents_f64
//     (ss_shoot.cu): forward-mode tangents of the parallel-in-time orbit.
// Parameter slots: slot 6 c + j is raw parameter p[j] of component c.

#include <cuda_runtime.h>

#include <cmath>

#include "ss_dual1.cuh"
#include "ss_release.cuh"
#include "ss_stream.cuh"

namespace ssg {

// ------------------------------------------------------- force VJPs (FP32)
// For one component at x (relative to its center): hk += H kv (Hessian of
// Phi times kv) and gp[j] += kv . d(grad Phi)/d p[j] for its raw parameters.
template <int KIND>
__device__ __forceinline__ void kind_vjp(const float* q, float G, const float x[3], const float kv[3], float hk[3],
                                         float* gp) {
    if constexpr (KIND == SS_NFW || KIND == SS_HERNQUIST || KIND == SS_PLUMMER || KIND == SS_ISOCHRONE) {
        float r2 = x[0] * x[0] + x[1] * x[1] + x[2] * x[2];
        float g, h;
        if constexpr (KIND == SS_NFW) {
            r2 += q[3];
            nfw_gh<float, float, true>(q, r2, g, h);
        } else if constexpr (KIND == SS_HERNQUIST) {
            r2 += q[2];
            hernquist_gh<float, float, true>(q, r2, g, h);
        } else if constexpr (KIND == SS_PLUMMER) {
            plummer_gh<float, float, true>(q, r2, g, h);
        } else {
            isochrone_gh<float, float, true>(q, r2, g, h);
        }
        const float s = x[0] * kv[0] + x[1] * kv[1] + x[2] * kv[2];
#pragma unroll
        for (int i = 0; i < 3; ++i) hk[i] += g * kv[i] + h * s * x[i];
        const float dg_dm = g * G * s_rcp(q[0]);
        float dg_dp1;
        if constexpr (KIND == SS_NFW) {
            const float inv_r = s_rsqrt(r2);
            const float irrs = s_rcp(r2 * inv_r + q[1]);
            dg_dp1 = -q[0] * inv_r * q[2] * irrs * irrs;  // d g / d rs
        } else if constexpr (KIND == SS_HERNQUIST) {
            const float inv_r = s_rsqrt(r2);
            const float irrs = s_rcp(r2 * inv_r + q[1]);
            dg_dp1 = -2.0f * q[0] * inv_r * irrs * irrs * irrs;  // d g / d rs
        } else if constexpr (KIND == SS_PLUMMER) {
            const float id = s_rsqrt(r2 + q[1]);
            dg_dp1 = -3.0f * g * sqrtf(q[1]) * id * id;  // d g / d b
        } else {
            const float inv_s = s_rsqrt(r2 + q[2]);
            const float a_s = q[1] * inv_s;
            const float inv_as = s_rcp(q[1] + (r2 + q[2]) * inv_s);
            dg_dp1 = g * (-a_s * inv_s - 2.0f * inv_as * (1.0f + a_s));  // d g / d a
        }
        gp[0] += dg_dm * s;
        gp[1] += dg_dp1 * s;
    } else if constexpr (KIND == SS_TRIAXIAL_NFW) {
        const float qi[3] = {q[2], q[3], q[4]};
        const float xi[3] = {x[0] * qi[0], x[1] * qi[1], x[2] * qi[2]};
        const float r2 = xi[0] * xi[0] + xi[1] * xi[1] + xi[2] * xi[2];
        const float qq[4] = {q[0], q[1], q[5], 0.0f};
        float g, h;
        nfw_gh<float, float, true>(qq, r2, g, h);
        const float S = xi[0] * qi[0] * kv[0] + xi[1] * qi[1] * kv[1] + xi[2] * qi[2] * kv[2];
#pragma unroll
        for (int i = 0; i < 3; ++i) hk[i] += qi[i] * (g * kv[i] * qi[i] + h * xi[i] * S);
        const float inv_r = s_rsqrt(r2);
        const float irrs = s_rcp(r2 * inv_r + q[1]);
        gp[0] += g * G * s_rcp(q[0]) * S;
        gp[1] += -q[0] * inv_r * q[5] * irrs * irrs * S;
#pragma unroll
        for (int k = 0; k < 3; ++k) gp[2 + k] += -h * xi[k] * xi[k] * qi[k] * S - 2.0f * g * kv[k] * xi[k] * qi[k] * qi[k];
    } else if constexpr (KIND == SS_MIYAMOTO_NAGAI) {
        const float zb2 = x[2] * x[2] + q[2];
        const float izeta = s_rsqrt(zb2);
        const float zeta = zb2 * izeta;
        const float A = zeta + q[1];
        const float iS = s_rsqrt(x[0] * x[0] + x[1] * x[1] + A * A);
        const float iS2 = iS * iS;
        const float iS3 = iS2 * iS;
        const float fz = A * izeta;
        // Hessian (as in kind_grad) times kv
        const float gm3 = q[0] * iS3;
        const float k3 = -3.0f * gm3 * iS2;
        const float z2 = x[2] * x[2];
        const float Hxx = gm3 + k3 * x[0] * x[0], Hyy = gm3 + k3 * x[1] * x[1];
        const float Hxy = k3 * x[0] * x[1], Hxz = k3 * x[0] * x[2] * fz, Hyz = k3 * x[1] * x[2] * fz;
        const float Hzz = gm3 * (fz - q[1] * z2 * izeta * izeta * izeta) + k3 * z2 * fz * fz;
        hk[0] += Hxx * kv[0] + Hxy * kv[1] + Hxz * kv[2];
        hk[1] += Hxy * kv[0] + Hyy * kv[1] + Hyz * kv[2];
        hk[2] += Hxz * kv[0] + Hyz * kv[1] + Hzz * kv[2];
        const float w = x[0] * kv[0] + x[1] * kv[1] + x[2] * fz * kv[2];
        const float b = sqrtf(q[2]);
        gp[0] += G * iS3 * w;                                                          // d/dm
        gp[1] += q[0] * (-3.0f * A * iS3 * iS2 * w + iS3 * x[2] * kv[2] * izeta);       // d/da
        gp[2] += q[0] * (-3.0f * A * b * izeta * iS3 * iS2 * w -
                         iS3 * x[2] * kv[2] * q[1] * b * izeta * izeta * izeta);          // d/db
    }
}

template <int... KCS>
struct CompVJP {
    template <int... I>
    static __device__ __forceinline__ void add(const PotDev<float>& P, float G, const float x[3], const float kv[3],
                                               float hk[3], float* gp, std::integer_sequence<int, I...>) {
        (kind_vjp<(KCS & 15)>(P.c[I].q, G, x, kv, hk, gp + 6 * I), ...);
    }
    static __device__ __forceinline__ void vjp(const PotDev<float>& P, float G, const float x[3], const float kv[3],
                                               float hk[3], float* gp) {
        add(P, G, x, kv, hk, gp, std::make_integer_sequence<int, sizeof...(KCS)>{});
    }
};

template <class C>
struct VJPOf;
template <int... KCS>
struct VJPOf<Comp<KCS...>> {
    using type = CompVJP<KCS...>;
    static constexpr int n = sizeof...(KCS);
};

// ------------------------------------------------------- stream adjoint
struct AdjArgs {
    StreamArgs s;         // h_hi/h_lo, N, ppr, spr, n_steps (no track, no subhalos)
    const float4* ckpt;   // [n_seg, N, 3]
    const double* lam_final;  // [N, 6]
    double* lam_ic;       // [N, 6]
    double* g_theta;      // [6 * n_comp] (accumulated)
    float G;
};

template <class C, int K>
__global__ void __launch_bounds__(128) stream_adjoint_kernel(PotDev<float> P, AdjArgs a) {
    using V = typename VJPOf<C>::type;
    constexpr int NS = 6 * VJPOf<C>::n;
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = p < a.s.N;
    float gth[NS];
#pragma unroll
    for (int i = 0; i < NS; ++i) gth[i] = 0.0f;
    if (valid) {
        const int start = (int)((p / a.s.ppr) * (int64_t)a.s.spr);
        const int L = a.s.n_steps - start;
        float lx[3], lv[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            lx[i] = (float)a.lam_final[6 * p + i];
            lv[i] = (float)a.lam_final[6 * p + 3 + i];
        }
        const float h = a.s.h_hi;
        float tape[K][6];
        const int nseg = (L + K - 1) / K;
        for (int seg = nseg - 1; seg >= 0; --seg) {
            const float4* c = a.ckpt + ((int64_t)seg * a.s.N + p) * 3;
            const float4 c0 = c[0], c1 = c[1], c2 = c[2];
            float xh[3] = {c0.x, c0.y, c0.z}, vh[3] = {c0.w, c1.x, c1.y};
            float xl[3] = {c1.z, c1.w, c2.x}, vl[3] = {c2.y, c2.z, c2.w};
            const int n0 = start + seg * K;
            const int n1 = min(n0 + K, a.s.n_steps);
            for (int n = n0; n < n1; ++n) {
                float* tp = tape[n - n0];
                tp[0] = xh[0]; tp[1] = xh[1]; tp[2] = xh[2];
                tp[3] = vh[0]; tp[4] = vh[1]; tp[5] = vh[2];
                step_f32k<C, SUB_NONE>(P, a.s, n, xh, xl, vh, vl);
            }
            for (int n = n1 - 1; n >= n0; --n) {
                const float* tp = tape[n - n0];
                // stage states of the plain FP32 step from the taped state
                float Yx[6][3], kx[6][3], kvv[6][3];
                const float A[6][5] = {{0, 0, 0, 0, 0},
                                       {(float)SS_A21, 0, 0, 0, 0},
                                       {(float)SS_A31, (float)SS_A32, 0, 0, 0},
                                       {(float)SS_A41, (float)SS_A42, (float)SS_A43, 0, 0},
                                       {(float)SS_A51, (float)SS_A52, (float)SS_A53, (float)SS_A54, 0},
                                       {(float)SS_A61, (float)SS_A62, (float)SS_A63, (float)SS_A64, (float)SS_A65}};
                const float B[6] = {(float)SS_B1, 0.0f, (float)SS_B3, (float)SS_B4, (float)SS_B5, (float)SS_B6};
#pragma unroll
                for (int st = 0; st < 6; ++st) {
                    float Yv[3];
#pragma unroll
                    for (int i = 0; i < 3; ++i) {
                        float sx = 0.0f, sv = 0.0f;
#pragma unroll
                        for (int j = 0; j < st; ++j) {
                            sx += A[st][j] * kx[j][i];
                            sv += A[st][j] * kvv[j][i];
                        }
                        Yx[st][i] = tp[i] + h * sx;
                        Yv[i] = tp[3 + i] + h * sv;
                    }
                    float g[3];
                    C::template grad<float, float, false>(P, Yx[st], Yx[st], g, nullptr);
#pragma unroll
                    for (int i = 0; i < 3; ++i) {
                        kx[st][i] = Yv[i];
                        kvv[st][i] = -g[i];
                    }
                }
                // transposed stages, last to first
                float mux[6][3], muv[6][3];
#pragma unroll
                for (int st = 5; st >= 0; --st) {
                    float kapx[3], kapv[3];
#pragma unroll
                    for (int i = 0; i < 3; ++i) {
                        float ax = B[st] * lx[i], av = B[st] * lv[i];
#pragma unroll
                        for (int j = st + 1; j < 6; ++j) {
                            ax += A[j][st] * mux[j][i];
                            av += A[j][st] * muv[j][i];
                        }
                        kapx[i] = h * ax;
                        kapv[i] = h * av;
                    }
                    // mu = J^T kappa = (-H kappa_v, kappa_x); theta += (d a/d theta)^T kappa_v
                    const float nk[3] = {-kapv[0], -kapv[1], -kapv[2]};
                    float hk[3] = {0.0f, 0.0f, 0.0f};
                    V::vjp(P, a.G, Yx[st], nk, hk, gth);
#pragma unroll
                    for (int i = 0; i < 3; ++i) {
                        mux[st][i] = hk[i];
                        muv[st][i] = kapx[i];
                    }
                }
#pragma unroll
                for (int i = 0; i < 3; ++i) {
                    float sx = 0.0f, sv = 0.0f;
#pragma unroll
                    for (int st = 0; st < 6; ++st) {
                        sx += mux[st][i];
                        sv += muv[st][i];
                    }
                    lx[i] += sx;
                    lv[i] += sv;
                }
            }
        }
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            a.lam_ic[6 * p + i] = lx[i];
            a.lam_ic[6 * p + 3 + i] = lv[i];
        }
    }
    // warp reduction of the parameter gradient, one atomic per warp and slot
#pragma unroll
    for (int i = 0; i < NS; ++i) {
        float v = gth[i];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0 && v != 0.0f) atomicAdd(a.g_theta + i, (double)v);
    }
}

// ------------------------------------------------------- release VJP (FP64)
struct RelVJPArgs {
    ss_release_cfg cfg;
    const double* prog_w;
    const double* t_rel;
    const double* msat;
    const double* normals;
    const double* lam_ics;  // [n_release, n_draw, 2, 6]
    double* g_prog;         // [n_release, 6] (accumulated)
    double* g_theta;        // [6 * n_comp] (accumulated)
    const double* raw;      // [n_comp, 6] raw parameters
    double G;
};

// d(ics)/d(r_t) of one draw for the release models (main.py:263-278;
// streamhelpers.py:380-430): every offset is linear in r_t except the
// Chen25 escape-velocity scale Dv ~ r_t^-1/2.
__device__ void release_drt(const ss_release_cfg& cfg, double G, double Msat, const double rh[3], const double zh[3],
                            const double ph[3], double om, double rt, const double* z, double out[2][6]) {
    if (cfg.model == SS_RELEASE_CHEN25) {
        double pvs[6];
        for (int i = 0; i < 6; ++i) {
            double s = cfg.chen_mean[i];
            for (int j = 0; j < 6; ++j) s += cfg.chen_L[6 * i + j] * z[j];
            pvs[i] = s;
        }
        const double deg = 0.017453292519943295;
        double phi = pvs[1] * deg, theta = pvs[2] * deg, alpha = pvs[4] * deg, beta = pvs[5] * deg;
        double ct = cos(theta), st = sin(theta), cp = cos(phi), sp = sin(phi);
        double ca = cos(alpha), sa = sin(alpha), cb = cos(beta), sb = sin(beta);
        double Dr = pvs[0] * rt;
        double Dv = pvs[3] * sqrt(2.0 * G * Msat / Dr);
        double dDr = pvs[0], dDv = -0.5 * Dv / rt;
        for (int i = 0; i < 3; ++i) {
            double ax = dDr * ct * cp * rh[i], ay = dDr * ct * sp * ph[i], az = dDr * st * zh[i];
            double bx = dDv * cb * ca * rh[i], by = dDv * cb * sa * ph[i], bz = dDv * sb * zh[i];
            out[1][i] = ax + ay + az;
            out[1][3 + i] = bx + by + bz;
            out[0][i] = -ax - ay + az;
            out[0][3 + i] = -bx - by + bz;
        }
    } else {
        const double* kv = cfg.kvals;
        double kr = kv[0] + z[0] * kv[4];
        double kvphi = kr * (kv[1] + z[1] * kv[5]);
        double kz = kv[2] + z[2] * kv[6];
        double kvz = kv[3] + z[3] * kv[7];
        for (int i = 0; i < 3; ++i) {
            double dp = kr * rh[i] + kz * zh[i];
            double dv = (kvphi * ph[i] + kvz * zh[i]) * om;
            out[1][i] = dp;
            out[1][3 + i] = dv;
            out[0][i] = -dp;
            out[0][3 + i] = -dv;
        }
    }
}

__global__ void release_vjp_kernel(PotDev<double> P, RelVJPArgs a) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t total = a.cfg.n_release * a.cfg.n_draw;
    if (q >= total) return;
    const int64_t r = q / a.cfg.n_draw;
    const int nz = a.cfg.model == SS_RELEASE_CHEN25 ? 6 : 4;
    const double* z = a.normals + q * nz;
    const double* w = a.prog_w + 6 * r;
    const double* lam = a.lam_ics + q * 12;
    const double Msat = a.msat[r], t = a.t_rel[r];
    // 1. progenitor state: forward-mode duals through the whole release
    {
        typedef Dual<6> D6;
        D6 x[3], v[3];
        for (int i = 0; i < 3; ++i) {
            x[i] = D6(w[i]);
            x[i].d[i] = 1.0;
            v[i] = D6(w[3 + i]);
            v[i].d[3 + i] = 1.0;
        }
        D6 out[2][6];
        release_one<D6>(P, a.G, a.cfg, x, v, Msat, t, z, out);
        for (int j = 0; j < 6; ++j) {
            double s = 0.0;
            for (int arm = 0; arm < 2; ++arm)
                for (int i = 0; i < 6; ++i) s += lam[6 * arm + i] * out[arm][i].d[j];
            atomicAdd(a.g_prog + 6 * r + j, s);
        }
    }
    // 2. potential parameters, through r_t = (G Msat / (Omega^2 - r^T H r))^(1/3)
    double x[3] = {w[0], w[1], w[2]}, v[3] = {w[3], w[4], w[5]};
    double rh[3], zh[3], ph[3], om;
    const double rt = release_tidal_radius<double>(P, x, v, a.G * Msat, t, rh, zh, ph, om);
    double dic[2][6];
    release_drt(a.cfg, a.G, Msat, rh, zh, ph, om, rt, z, dic);
    double lam_drt = 0.0;
    for (int arm = 0; arm < 2; ++arm)
        for (int i = 0; i < 6; ++i) lam_drt += lam[6 * arm + i] * dic[arm][i];
    // r^T H r and its parameter derivatives
    double c3[3] = {0.0, 0.0, 0.0};
    if (P.has_track) track_eval(P.track, t, c3);
    const double xs[3] = {x[0] - c3[0], x[1] - c3[1], x[2] - c3[2]};
    double g[3], H[6];
    pot_grad<double, double, true>(P, x, xs, g, H);
    const double d2 = H[0] * rh[0] * rh[0] + H[1] * rh[1] * rh[1] + H[2] * rh[2] * rh[2] +
                      2.0 * (H[3] * rh[0] * rh[1] + H[4] * rh[0] * rh[2] + H[5] * rh[1] * rh[2]);
    const double drt_dd2 = rt / (3.0 * (om * om - d2));
    typedef D1<double> DD;
    for (int c = 0; c < P.n; ++c) {
        for (int j = 0; j < 6; ++j) {
            double dq[6];
            prepared_param_tangent(P.c[c].kind, a.raw + 6 * c, j, a.G, dq);
            bool any = false;
            for (int i = 0; i < 6; ++i) any |= dq[i] != 0.0;
            if (!any) continue;
            // Hessian of component c alone, differentiated along p[j]
            DD qd[6];
            for (int i = 0; i < 6; ++i) qd[i] = DD(P.c[c].q[i], dq[i]);
            const double* xc = P.c[c].center == SS_CENTER_TRACK ? xs : x;
            DD xd[3] = {DD(xc[0], 0.0), DD(xc[1], 0.0), DD(xc[2], 0.0)};
            DD gd[3] = {DD(0), DD(0), DD(0)}, Hd[6] = {DD(0), DD(0), DD(0), DD(0), DD(0), DD(0)};
            switch (P.c[c].kind) {
                case SS_NFW: kind_grad<SS_NFW, DD, DD, true>(qd, xd, gd, Hd); break;
                case SS_TRIAXIAL_NFW: kind_grad<SS_TRIAXIAL_NFW, DD, DD, true>(qd, xd, gd, Hd); break;
                case SS_MIYAMOTO_NAGAI: kind_grad<SS_MIYAMOTO_NAGAI, DD, DD, true>(qd, xd, gd, Hd); break;
                case SS_HERNQUIST: kind_grad<SS_HERNQUIST, DD, DD, true>(qd, xd, gd, Hd); break;
                case SS_PLUMMER: kind_grad<SS_PLUMMER, DD, DD, true>(qd, xd, gd, Hd); break;
                case SS_ISOCHRONE: kind_grad<SS_ISOCHRONE, DD, DD, true>(qd, xd, gd, Hd); break;
                default: break;
            }
            const double dd2 = Hd[0].d * rh[0] * rh[0] + Hd[1].d * rh[1] * rh[1] + Hd[2].d * rh[2] * rh[2] +
                               2.0 * (Hd[3].d * rh[0] * rh[1] + Hd[4].d * rh[0] * rh[2] + Hd[5].d * rh[1] * rh[2]);
            atomicAdd(a.g_theta + 6 * c + j, lam_drt * drt_dd2 * dd2);
        }
    }
}

}  // namespace ssg

using namespace ssg;

extern "C" {

int ss_stream_f32k_ckpt(const ss_potential* pot, const ss_stream_cfg* cfg, const double* ics, double* final_w,
                        int32_t* status, float* ckpt, int32_t ckpt_stride, void* stream) {
    PotDev<float> P;
    int rc = prepare_potential<float>(pot, &P, false);
    if (rc) return rc;
    SS_CHECK_ARG(cfg != nullptr && cfg->first_particle == 0 && cfg->snap_pitch == 0 && cfg->stream_particles == 0,
                 "the adjoint path runs whole single streams (first_particle = snap_pitch = stream_particles = 0)");
    SS_CHECK_ARG(!P.has_track && !P.has_rot && !P.has_facc && !P.grow_mask,
                 "the adjoint supports static potentials (no center track, rotation or frame acceleration) only");
    SS_CHECK_ARG(cfg && cfg->n_particles >= 0 && cfg->n_steps >= 0 && cfg->n_steps < (1LL << 30), "bad cfg");
    SS_CHECK_ARG(cfg->particles_per_release >= 1 && cfg->steps_per_release >= 0, "bad release layout");
    SS_CHECK_ARG(std::isfinite(cfg->dt) && cfg->dt > 0.0, "dt must be > 0");
    SS_CHECK_ARG(ckpt_stride == 64, "ckpt_stride must be 64");
    if (cfg->n_particles == 0) return SS_OK;
    SS_CHECK_ARG(ics && ckpt, "NULL buffer");
    StreamArgs a;
    memset(&a, 0, sizeof(a));
    a.ics = ics;
    a.final_w = final_w;
    a.status = status;
    a.N = cfg->n_particles;
    a.ppr = cfg->particles_per_release;
    a.spr = cfg->steps_per_release;
    a.n_steps = (int32_t)cfg->n_steps;
    a.stride = 1;
    a.t0 = cfg->t0;
    a.dt = cfg->dt;
    a.h_hi = (float)cfg->dt;
    a.h_lo = (float)(cfg->dt - (double)a.h_hi);
    a.ckpt = reinterpret_cast<float4*>(ckpt);
    a.ckpt_stride = ckpt_stride;
    const int block = 128;
    unsigned grid = (unsigned)((cfg->n_particles + block - 1) / block);
    dispatch_comp(P, [&](auto comp) {
        stream_f32k_kernel<decltype(comp), SUB_NONE, true><<<grid, block, 0, (cudaStream_t)stream>>>(P, a);
        return 0;
    });
    SS_LAUNCH_CHECK();
    return SS_OK;
}

int ss_stream_adjoint_f32(const ss_potential* pot, const ss_stream_cfg* cfg, const float* ckpt, int32_t ckpt_stride,
                          const double* lam_final, double* lam_ic, double* g_theta, void* stream) {
    PotDev<float> P;
    int rc = prepare_potential<float>(pot, &P, false);
    if (rc) return rc;
    SS_CHECK_ARG(cfg != nullptr && cfg->first_particle == 0 && cfg->snap_pitch == 0 && cfg->stream_particles == 0,
                 "the adjoint path runs whole single streams (first_particle = snap_pitch = stream_particles = 0)");
    for (int k = 0; k < P.n; ++k)
        SS_CHECK_ARG(P.c[k].kind != SS_SH_EXPANSION && P.c[k].kind != SS_POWERLAW_CUTOFF && P.c[k].kind != SS_ZHAO,
                     "component %d: kind %d has no adjoint", k, P.c[k].kind);
    SS_CHECK_ARG(!P.has_track && !P.has_rot && !P.has_facc && !P.grow_mask,
                 "the adjoint supports static potentials (no center track, rotation or frame acceleration) only");
    SS_CHECK_ARG(cfg && cfg->n_particles >= 0 && cfg->n_steps >= 0 && cfg->n_steps < (1LL << 30), "bad cfg");
    SS_CHECK_ARG(cfg->particles_per_release >= 1 && cfg->steps_per_release >= 0, "bad release layout");
    SS_CHECK_ARG(std::isfinite(cfg->dt) && cfg->dt > 0.0, "dt must be > 0");
    SS_CHECK_ARG(ckpt_stride == 64, "ckpt_stride must be 64");
    if (cfg->n_particles == 0) return SS_OK;
    SS_CHECK_ARG(ckpt && lam_final && lam_ic && g_theta, "NULL buffer");
    AdjArgs a;
    memset(&a, 0, sizeof(a));
    a.s.N = cfg->n_particles;
    a.s.ppr = cfg->particles_per_release;
    a.s.spr = cfg->steps_per_release;
    a.s.n_steps = (int32_t)cfg->n_steps;
    a.s.stride = 1;
    a.s.t0 = cfg->t0;
    a.s.dt = cfg->dt;
    a.s.h_hi = (float)cfg->dt;
    a.s.h_lo = (float)(cfg->dt - (double)a.s.h_hi);
    a.ckpt = reinterpret_cast<const float4*>(ckpt);
    a.lam_final = lam_final;
    a.lam_ic = lam_ic;
    a.g_theta = g_theta;
    a.G = (float)pot->G;
    const int block = 128;
    unsigned grid = (unsigned)((cfg->n_particles + block - 1) / block);
    int launched = 0;
    dispatch_comp(P, [&](auto comp) {
        using C = decltype(comp);
        if constexpr (!std::is_same<C, GenericComp>::value) {
            stream_adjoint_kernel<C, 64><<<grid, block, 0, (cudaStream_t)stream>>>(P, a);
            launched = 1;
        }
        return 0;
    });
    if (!launched)
        return set_error(SS_ERR_UNSUPPORTED, "the adjoint is compiled for the built-in potential compositions only");
    SS_LAUNCH_CHECK();
    return SS_OK;
}

int ss_release_vjp(const ss_potential* pot, const ss_release_cfg* cfg, const double* prog_w, const double* t_rel,
                   const double* msat, const double* normals, const double* lam_ics, const double* raw_params,
                   double* g_prog, double* g_theta, void* stream) {
    PotDev<double> P;
    int rc = prepare_potential<double>(pot, &P, false);
    if (rc) return rc;
    for (int k = 0; k < P.n; ++k)
        SS_CHECK_ARG(P.c[k].kind != SS_SH_EXPANSION && P.c[k].kind != SS_POWERLAW_CUTOFF && P.c[k].kind != SS_ZHAO,
                     "component %d: kind %d has no adjoint", k, P.c[k].kind);
    SS_CHECK_ARG(!P.has_rot && !P.has_facc && !P.grow_mask, "the release adjoint supports static potentials only");
    SS_CHECK_ARG(cfg && cfg->n_release >= 0 && cfg->n_draw >= 1, "bad cfg");
    int64_t total = cfg->n_release * cfg->n_draw;
    if (total == 0) return SS_OK;
    SS_CHECK_ARG(prog_w && t_rel && msat && normals && lam_ics && raw_params && g_prog && g_theta, "NULL buffer");
    RelVJPArgs a;
    a.cfg = *cfg;
    a.prog_w = prog_w;
    a.t_rel = t_rel;
    a.msat = msat;
    a.normals = normals;
    a.lam_ics = lam_ics;
    a.g_prog = g_prog;
    a.g_theta = g_theta;
    a.raw = raw_params;
    a.G = pot->G;
    release_vjp_kernel<<<(unsigned)((total + 63) / 64), 64, 0, (cudaStream_t)stream>>>(P, a);
    SS_LAUNCH_CHECK();
    return SS_OK;
}

}  // extern "C"
