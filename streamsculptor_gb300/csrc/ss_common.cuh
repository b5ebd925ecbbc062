// ss_common.cuh — host-side helpers shared by the translation units:
// error reporting, potential preparation (raw reference parameters ->
// pre-combined device parameters), the Dormand-Prince tableau and the FP64
// step used by the orbit / stream / release / response kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>

#include <cmath>

#include "ss_device.cuh"

namespace ssg {

// ------------------------------------------------------------- errors
int set_error(int code, const char* fmt, ...);
const char* last_error();

#define SS_CHECK_ARG(cond, ...)                                          \
    do {                                                                 \
        if (!(cond)) return ::ssg::set_error(SS_ERR_INVALID_ARGUMENT, __VA_ARGS__); \
    } while (0)

#define SS_CUDA_TRY(expr)                                                              \
    do {                                                                               \
        cudaError_t _e = (expr);                                                       \
        if (_e != cudaSuccess)                                                         \
            return ::ssg::set_error(SS_ERR_CUDA, "%s: %s", #expr, cudaGetErrorString(_e)); \
    } while (0)

// Every kernel launch is followed by SS_LAUNCH_CHECK, which also counts it
// (ss_kernel_launches).
void count_launch();

#define SS_LAUNCH_CHECK()                                                                    \
    do {                                                                                     \
        ::ssg::count_launch();                                                               \
        cudaError_t _e = cudaGetLastError();                                                 \
        if (_e != cudaSuccess)                                                               \
            return ::ssg::set_error(SS_ERR_CUDA, "kernel launch: %s", cudaGetErrorString(_e)); \
    } while (0)

// Raw parameters (reference units) -> PotDev<R>.  Validates kinds, counts,
// positivity and the center track.  `allow_subhalos` = false rejects a
// potential that carries a subhalo table.
template <class R>
int prepare_potential(const ss_potential* in, PotDev<R>* out, bool allow_subhalos);

// ------------------------------------------------------ Dopri5 tableau
// Dormand & Prince (1980) RK5(4)7M; 5th-order weights b (b2 = b7 = 0).
#define SS_C2 (1.0 / 5.0)
#define SS_C3 (3.0 / 10.0)
#define SS_C4 (4.0 / 5.0)
#define SS_C5 (8.0 / 9.0)
#define SS_A21 (1.0 / 5.0)
#define SS_A31 (3.0 / 40.0)
#define SS_A32 (9.0 / 40.0)
#define SS_A41 (44.0 / 45.0)
#define SS_A42 (-56.0 / 15.0)
#define SS_A43 (32.0 / 9.0)
#define SS_A51 (19372.0 / 6561.0)
#define SS_A52 (-25360.0 / 2187.0)
#define SS_A53 (64448.0 / 6561.0)
#define SS_A54 (-212.0 / 729.0)
#define SS_A61 (9017.0 / 3168.0)
#define SS_A62 (-355.0 / 33.0)
#define SS_A63 (46732.0 / 5247.0)
#define SS_A64 (49.0 / 176.0)
#define SS_A65 (-5103.0 / 18656.0)
#define SS_B1 (35.0 / 384.0)
#define SS_B3 (500.0 / 1113.0)
#define SS_B4 (125.0 / 192.0)
#define SS_B5 (-2187.0 / 6784.0)
#define SS_B6 (11.0 / 84.0)
// Nystrom coefficients of the tableau for second-order systems x'' = A(x, t):
// stage positions x + c_s h v + h^2 sum_k abar_sk A_k with abar = a a, and
// the 5th-order position update x + h v + h^2 sum_k bbar_k A_k, bbar = b a.
constexpr double SS_N31 = SS_A32 * SS_A21;
constexpr double SS_N41 = SS_A42 * SS_A21 + SS_A43 * SS_A31;
constexpr double SS_N42 = SS_A43 * SS_A32;
constexpr double SS_N51 = SS_A52 * SS_A21 + SS_A53 * SS_A31 + SS_A54 * SS_A41;
constexpr double SS_N52 = SS_A53 * SS_A32 + SS_A54 * SS_A42;
constexpr double SS_N53 = SS_A54 * SS_A43;
constexpr double SS_N61 = SS_A62 * SS_A21 + SS_A63 * SS_A31 + SS_A64 * SS_A41 + SS_A65 * SS_A51;
constexpr double SS_N62 = SS_A63 * SS_A32 + SS_A64 * SS_A42 + SS_A65 * SS_A52;
constexpr double SS_N63 = SS_A64 * SS_A43 + SS_A65 * SS_A53;
constexpr double SS_N64 = SS_A65 * SS_A54;
constexpr double SS_NB1 = SS_B3 * SS_A31 + SS_B4 * SS_A41 + SS_B5 * SS_A51 + SS_B6 * SS_A61;
constexpr double SS_NB2 = SS_B3 * SS_A32 + SS_B4 * SS_A42 + SS_B5 * SS_A52 + SS_B6 * SS_A62;
constexpr double SS_NB3 = SS_B4 * SS_A43 + SS_B5 * SS_A53 + SS_B6 * SS_A63;
constexpr double SS_NB4 = SS_B5 * SS_A54 + SS_B6 * SS_A64;
constexpr double SS_NB5 = SS_B6 * SS_A65;

// FP64 acceleration of the full potential (components + track + subhalos)
// at time t: velocity_acceleration, main.py:116-120.
// C: the composition (Comp<...> or GenericComp); sh: the subhalo rows this
// particle feels (P.sh, or one stream's slice of it in an ensemble run).
// cen: the center track's position at t when the caller has it (the stream
// kernel tabulates it per stage time), else NULL.
template <class C>
__device__ __forceinline__ void accel_f64(const PotDev<double>& P, const ShDev& sh, const double x[3], double t,
                                          double a[3], const double* cen = nullptr) {
    double c[3] = {0.0, 0.0, 0.0};
    if (cen) {
        c[0] = cen[0];
        c[1] = cen[1];
        c[2] = cen[2];
    } else if (P.has_track) {
        track_eval(P.track, t, c);
    }
    const double xs[3] = {x[0] - c[0], x[1] - c[1], x[2] - c[2]};
    double g[3];
    C::template grad<double, double, false>(P, x, xs, g, nullptr, time_dep(P, t));
    if (sh.n > 0) subhalo_sum_grad<double>(sh, x, t, g);
    a[0] = -g[0];
    a[1] = -g[1];
    a[2] = -g[2];
}

// One fixed Dopri5 step of the Hamiltonian flow (x, v) in FP64.  cen: the
// center track at the six stage times t + c_s h (c = 0, 1/5, 3/10, 4/5, 8/9,
// 1), or NULL to evaluate it per stage.
template <class C>
__device__ __forceinline__ void dopri5_step_f64(const PotDev<double>& P, const ShDev& sh, double t, double h,
                                                double y[6], const double (*cen)[3] = nullptr) {
    double k1[6], k2[6], k3[6], k4[6], k5[6], k6[6], ys[6];
    // stage 1
    k1[0] = y[3]; k1[1] = y[4]; k1[2] = y[5];
    accel_f64<C>(P, sh, y, t, k1 + 3, cen ? cen[0] : nullptr);
#pragma unroll
    for (int i = 0; i < 6; ++i) ys[i] = y[i] + h * (SS_A21 * k1[i]);
    k2[0] = ys[3]; k2[1] = ys[4]; k2[2] = ys[5];
    accel_f64<C>(P, sh, ys, t + SS_C2 * h, k2 + 3, cen ? cen[1] : nullptr);
#pragma unroll
    for (int i = 0; i < 6; ++i) ys[i] = y[i] + h * (SS_A31 * k1[i] + SS_A32 * k2[i]);
    k3[0] = ys[3]; k3[1] = ys[4]; k3[2] = ys[5];
    accel_f64<C>(P, sh, ys, t + SS_C3 * h, k3 + 3, cen ? cen[2] : nullptr);
#pragma unroll
    for (int i = 0; i < 6; ++i) ys[i] = y[i] + h * (SS_A41 * k1[i] + SS_A42 * k2[i] + SS_A43 * k3[i]);
    k4[0] = ys[3]; k4[1] = ys[4]; k4[2] = ys[5];
    accel_f64<C>(P, sh, ys, t + SS_C4 * h, k4 + 3, cen ? cen[3] : nullptr);
#pragma unroll
    for (int i = 0; i < 6; ++i)
        ys[i] = y[i] + h * (SS_A51 * k1[i] + SS_A52 * k2[i] + SS_A53 * k3[i] + SS_A54 * k4[i]);
    k5[0] = ys[3]; k5[1] = ys[4]; k5[2] = ys[5];
    accel_f64<C>(P, sh, ys, t + SS_C5 * h, k5 + 3, cen ? cen[4] : nullptr);
#pragma unroll
    for (int i = 0; i < 6; ++i)
        ys[i] = y[i] + h * (SS_A61 * k1[i] + SS_A62 * k2[i] + SS_A63 * k3[i] + SS_A64 * k4[i] + SS_A65 * k5[i]);
    k6[0] = ys[3]; k6[1] = ys[4]; k6[2] = ys[5];
    accel_f64<C>(P, sh, ys, t + h, k6 + 3, cen ? cen[5] : nullptr);
#pragma unroll
    for (int i = 0; i < 6; ++i)
        y[i] = y[i] + h * (SS_B1 * k1[i] + SS_B3 * k3[i] + SS_B4 * k4[i] + SS_B5 * k5[i] + SS_B6 * k6[i]);
}

template <class C>
__device__ __forceinline__ void dopri5_step_f64(const PotDev<double>& P, double t, double h, double y[6]) {
    dopri5_step_f64<C>(P, P.sh, t, h, y);
}

// The subhalo rows [g k, (g + 1) k) of sh (one stream or orbit of an
// ensemble); k <= 0 keeps the whole table.
__device__ __forceinline__ ShDev subhalo_slice(const ShDev& sh, int64_t g, int32_t k) {
    ShDev s = sh;
    if (k > 0 && sh.n > 0) {
        const int64_t o = g * (int64_t)k;
        s.m += o;
        s.a += o;
        s.x0 += 3 * o;
        s.v += 3 * o;
        s.t0 += o;
        s.n = k;
    }
    return s;
}

}  // namespace ssg
