// ss_release.cuh — the release model (particle spray) on the device,
// templated on double and forward-mode duals: shared by the release kernel
// (ss_api.cu) and the release vector-Jacobian product (ss_adjoint.cu).
#pragma once

#include "ss_common.cuh"

namespace ssg {

// ------------------------------------------------------------- release
// tidal radius pieces, templated on double / Dual<6>:
// omega (main.py:88-96), d2phidr2 (main.py:76-85), tidalr (main.py:98-104).
template <class T>
__device__ inline T release_tidal_radius(const PotDev<double>& P, const T x[3], const T v[3], double GMsat, double t,
                                  T rh[3], T zh[3], T ph[3], T& om) {
    T r2 = x[0] * x[0] + x[1] * x[1] + x[2] * x[2];
    T r = s_sqrt(r2);
    T ir = s_rcp(r);
    rh[0] = x[0] * ir; rh[1] = x[1] * ir; rh[2] = x[2] * ir;
    T L[3] = {x[1] * v[2] - x[2] * v[1], x[2] * v[0] - x[0] * v[2], x[0] * v[1] - x[1] * v[0]};
    T L2 = L[0] * L[0] + L[1] * L[1] + L[2] * L[2];
    T Ln = s_sqrt(L2);
    om = Ln * s_rcp(r2);
    T iLn = s_rcp(Ln);
    zh[0] = L[0] * iLn; zh[1] = L[1] * iLn; zh[2] = L[2] * iLn;
    T vr = v[0] * rh[0] + v[1] * rh[1] + v[2] * rh[2];
    T pv[3] = {v[0] - vr * rh[0], v[1] - vr * rh[1], v[2] - vr * rh[2]};
    T ipn = s_rsqrt(pv[0] * pv[0] + pv[1] * pv[1] + pv[2] * pv[2]);
    ph[0] = pv[0] * ipn; ph[1] = pv[1] * ipn; ph[2] = pv[2] * ipn;
    double c[3] = {0.0, 0.0, 0.0};
    if (P.has_track) track_eval(P.track, t, c);
    T xs[3] = {x[0] - c[0], x[1] - c[1], x[2] - c[2]};
    T g[3], H[6];
    pot_grad<T, double, true>(P, x, xs, g, H, time_dep_as<T>(time_dep(P, t)));
    // r_hat^T H r_hat
    T d2 = H[0] * rh[0] * rh[0] + H[1] * rh[1] * rh[1] + H[2] * rh[2] * rh[2] +
           2.0 * (H[3] * rh[0] * rh[1] + H[4] * rh[0] * rh[2] + H[5] * rh[1] * rh[2]);
    return s_cbrt(GMsat * s_rcp(om * om - d2));
}

template <class T>
__device__ inline void release_one(const PotDev<double>& P, double G, const ss_release_cfg& cfg, const T x[3],
                            const T v[3], double Msat, double t, const double* z, T out[2][6]) {
    T rh[3], zh[3], ph[3], om;
    T rt = release_tidal_radius<T>(P, x, v, G * Msat, t, rh, zh, ph, om);
    if (cfg.model == SS_RELEASE_CHEN25) {
        // release_model_Chen25, streamhelpers.py:352-432
        double pvs[6];
        for (int i = 0; i < 6; ++i) {
            double s = cfg.chen_mean[i];
            for (int j = 0; j < 6; ++j) s += cfg.chen_L[6 * i + j] * z[j];
            pvs[i] = s;
        }
        T Dr = pvs[0] * rt;
        T vesc = s_sqrt(2.0 * G * Msat * s_rcp(Dr));
        T Dv = pvs[3] * vesc;
        const double deg = 0.017453292519943295;
        double phi = pvs[1] * deg, theta = pvs[2] * deg, alpha = pvs[4] * deg, beta = pvs[5] * deg;
        double ct = cos(theta), st = sin(theta), cp = cos(phi), sp = sin(phi);
        double ca = cos(alpha), sa = sin(alpha), cb = cos(beta), sb = sin(beta);
        for (int i = 0; i < 3; ++i) {
            T ax = (Dr * (ct * cp)) * rh[i], ay = (Dr * (ct * sp)) * ph[i], az = (Dr * st) * zh[i];
            T bx = (Dv * (cb * ca)) * rh[i], by = (Dv * (cb * sa)) * ph[i], bz = (Dv * sb) * zh[i];
            out[1][i] = x[i] + ax + ay + az;
            out[1][3 + i] = v[i] + bx + by + bz;
            out[0][i] = x[i] - ax - ay + az;
            out[0][3 + i] = v[i] - bx - by + bz;
        }
    } else {
        // Potential.release_model, main.py:209-280
        const double* kv = cfg.kvals;
        double kr = kv[0] + z[0] * kv[4];
        double kvphi = kr * (kv[1] + z[1] * kv[5]);
        double kz = kv[2] + z[2] * kv[6];
        double kvz = kv[3] + z[3] * kv[7];
        T vc = om * rt;
        for (int i = 0; i < 3; ++i) {
            T dpos = (kr * rt) * rh[i] + (kz * rt) * zh[i];
            T dvel = (kvphi * vc) * ph[i] + (kvz * vc) * zh[i];
            out[1][i] = x[i] + dpos;      // trailing: nudged out
            out[1][3 + i] = v[i] + dvel;
            out[0][i] = x[i] - dpos;      // leading: nudged in
            out[0][3 + i] = v[i] - dvel;
        }
    }
}

}  // namespace ssg
