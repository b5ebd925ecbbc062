// ss_shoot.cu — the progenitor's FP64 orbit, parallel in time.
//
// One orbit is one long dependency chain, and on GB300 a dependent FP64
// chain is slow (FP64 FMA ~64 cycles, rsqrt ~420, log1p ~2100, measured)
// while FP64 throughput is plentiful: 10^4 orbits take as long as one.  So
// the orbit is solved by multiple shooting with Newton's method:
//   * split the n_steps fixed Dopri5 steps into S slices of M steps;
//   * guess the slice starts U_n with a cheap FP32 integration (coarse steps);
//   * iterate: integrate every slice in parallel in FP64 from U_n (its end
//     F_n = F(U_n), and the saved states of its steps), and its 6x6 Jacobian
//     J_n in FP32 (six forward-mode tangent lanes per slice); then the Newton
//     update of the joins, e_{n+1} = J_n e_n + (F_n - U_{n+1}) with e_0 = 0,
//     U_{n+1} += e_{n+1}, an affine recurrence solved as a parallel prefix
//     scan over the slices (composition (A2,b2) o (A1,b1) = (A2 A1, A2 b1 + b2));
//   * an FP32 Jacobian makes the iteration converge linearly with a factor
//     ~1e-6 instead of quadratically, which still reaches the FP64 round-off
//     floor in a few iterations; the iteration stops when the largest relative
//     update is below `tol` or stops shrinking below 1e-12 (the round-off floor);
//   * the last slice pass wrote the saved states (its starts differ from the
//     final ones by less than the last update).
// The result is the serial fixed-step FP64 Dopri5 orbit (the same step map
// composed n_steps times) up to round-off in the slice joins.  Static
// potentials (no center track, no subhalos) only; the entry point falls back
// to the serial kernel otherwise.

#include <cuda_runtime.h>

#include <cmath>

#include "ss_dual1.cuh"

namespace ssg {

static constexpr int SHOOT_M = 8;   // FP64 steps per slice
static constexpr int SHOOT_C = 8;   // FP64 steps per coarse FP32 guess step
static constexpr int SHOOT_ITERS = 8;

struct ShootArgs {
    const double* w0;
    double dt;
    int32_t n_steps;
    int32_t S;        // slices
    int32_t save_every;
    int32_t n_save;
    double* U;        // [S + 1, 6] slice starts
    double* F;        // [S, 6] slice ends
    double* J;        // [S, 36] floats dF_i/dU_j at [i * 6 + j] (space for 36 S doubles)
    int32_t* flag;    // [0] converged, [1] Newton sweeps done, [2] last update (float bits)
    double tol;
    double* out;      // [n_save, 6]
};

__device__ __forceinline__ int slice_len(const ShootArgs& a, int n) {
    return n < a.S - 1 ? SHOOT_M : a.n_steps - SHOOT_M * (a.S - 1);
}

// Plain FP32 Dopri5 step (initial guess only).
template <class C>
__device__ __forceinline__ void dopri5_step_f32(const PotDev<float>& P, float h, float y[6]) {
    float k[6][6], ys[6];
    const float A[6][5] = {{0, 0, 0, 0, 0},
                           {(float)SS_A21, 0, 0, 0, 0},
                           {(float)SS_A31, (float)SS_A32, 0, 0, 0},
                           {(float)SS_A41, (float)SS_A42, (float)SS_A43, 0, 0},
                           {(float)SS_A51, (float)SS_A52, (float)SS_A53, (float)SS_A54, 0},
                           {(float)SS_A61, (float)SS_A62, (float)SS_A63, (float)SS_A64, (float)SS_A65}};
    const float B[6] = {(float)SS_B1, 0.0f, (float)SS_B3, (float)SS_B4, (float)SS_B5, (float)SS_B6};
#pragma unroll
    for (int s = 0; s < 6; ++s) {
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            float acc = 0.0f;
#pragma unroll
            for (int j = 0; j < s; ++j) acc += A[s][j] * k[j][c];
            ys[c] = y[c] + h * acc;
        }
        float g[3];
        C::template grad<float, float, false>(P, ys, ys, g, nullptr);
        k[s][0] = ys[3]; k[s][1] = ys[4]; k[s][2] = ys[5];
        k[s][3] = -g[0]; k[s][4] = -g[1]; k[s][5] = -g[2];
    }
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        float acc = 0.0f;
#pragma unroll
        for (int s = 0; s < 6; ++s) acc += B[s] * k[s][c];
        y[c] += h * acc;
    }
}

// Serial FP32 guess of the slice starts with coarse steps.
template <class C>
__global__ void shoot_guess_kernel(PotDev<float> P, ShootArgs a) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    float y[6];
    for (int i = 0; i < 6; ++i) {
        y[i] = (float)a.w0[i];
        a.U[i] = a.w0[i];
    }
    for (int n = 0; n < a.S; ++n) {
        const int len = slice_len(a, n);
        const int nc = (len + SHOOT_C - 1) / SHOOT_C;
        const float h = (float)(a.dt * (double)len / (double)nc);
        for (int j = 0; j < nc; ++j) dopri5_step_f32<C>(P, h, y);
        for (int i = 0; i < 6; ++i) a.U[6 * (n + 1) + i] = (double)y[i];
    }
}

// Every slice from its start in FP64: its end F_n and (when saving) the
// states of its steps.
template <class C>
__global__ void __launch_bounds__(64) shoot_f64_kernel(PotDev<double> P, ShootArgs a) {
    if (a.flag[0]) return;
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= a.S) return;
    double y[6];
#pragma unroll
    for (int j = 0; j < 6; ++j) y[j] = a.U[6 * n + j];
    if (a.out && n == 0)
        for (int j = 0; j < 6; ++j) a.out[j] = y[j];
    const int len = slice_len(a, n);
    for (int s = 0; s < len; ++s) {
        dopri5_step_f64<C>(P, 0.0, a.dt, y);
        const int g = n * SHOOT_M + s + 1;
        if (a.out && g % a.save_every == 0 && g / a.save_every < a.n_save)
            for (int j = 0; j < 6; ++j) a.out[6 * (g / a.save_every) + j] = y[j];
    }
#pragma unroll
    for (int j = 0; j < 6; ++j) a.F[6 * n + j] = y[j];
}

// The slices' Jacobians in FP32: lane 6 n + i carries the tangent along
// U_j = e_i; J_n is stored as floats [S, 36] at a.J.
template <class C>
__global__ void __launch_bounds__(96) shoot_jac_kernel(PotDev<float> P32, ShootArgs a) {
    if (a.flag[0]) return;
    const int lane = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = lane / 6, i = lane % 6;
    if (n >= a.S) return;
    typedef D1<float> T;
    PotDev<T> Q;
    Q.n = P32.n;
    Q.has_track = 0;
    Q.grow_mask = 0;
    Q.ex = P32.ex;
#pragma unroll
    for (int c = 0; c < C::n; ++c) {
        Q.c[c].kind = P32.c[c].kind;
        Q.c[c].center = P32.c[c].center;
#pragma unroll
        for (int j = 0; j < 6; ++j) Q.c[c].q[j] = T(P32.c[c].q[j], 0.0f);
    }
    T y[6];
#pragma unroll
    for (int j = 0; j < 6; ++j) y[j] = T((float)a.U[6 * n + j], j == i ? 1.0f : 0.0f);
    const T h((float)a.dt, 0.0f);
    const int len = slice_len(a, n);
    for (int s = 0; s < len; ++s) dopri5_step_dual<C, float>(Q, h, y);
    float* J = reinterpret_cast<float*>(a.J);
#pragma unroll
    for (int j = 0; j < 6; ++j) J[36 * n + 6 * j + i] = y[j].d;
}

// Newton update of the joins as a parallel prefix scan of the affine maps
// e -> J_n e + r_n (r_n = F_n - U_{n+1}, FP32; e_0 = 0): each thread composes
// a contiguous segment, a Hillis-Steele scan combines the segments, each
// thread replays its segment from its entry value and adds e to U (FP64).
static constexpr int SCAN_T = 256;

__device__ __forceinline__ void mat6_mul(const float A[36], const float B[36], float C_[36]) {
#pragma unroll
    for (int r = 0; r < 6; ++r)
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            float s = 0.0f;
#pragma unroll
            for (int k = 0; k < 6; ++k) s = fmaf(A[6 * r + k], B[6 * k + c], s);
            C_[6 * r + c] = s;
        }
}

__global__ void __launch_bounds__(SCAN_T) shoot_scan_kernel(ShootArgs a) {
    if (a.flag[0]) return;
    __shared__ float sA[SCAN_T * 36];
    __shared__ float sb[SCAN_T * 6];
    __shared__ float sw[SCAN_T];
    const int t = threadIdx.x, S = a.S;
    const int seg = (S + SCAN_T - 1) / SCAN_T;
    const int n0 = min(S, t * seg), n1 = min(S, n0 + seg);
    const float* J = reinterpret_cast<const float*>(a.J);
    // segment composition
    float A[36], b[6];
#pragma unroll
    for (int k = 0; k < 36; ++k) A[k] = (k % 7 == 0) ? 1.0f : 0.0f;
#pragma unroll
    for (int k = 0; k < 6; ++k) b[k] = 0.0f;
    for (int n = n0; n < n1; ++n) {
        float Jn[36], r[6], T2[36], b2[6];
#pragma unroll
        for (int k = 0; k < 36; ++k) Jn[k] = J[36 * n + k];
#pragma unroll
        for (int k = 0; k < 6; ++k) r[k] = (float)(a.F[6 * n + k] - a.U[6 * (n + 1) + k]);
        mat6_mul(Jn, A, T2);
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            float s = r[q];
#pragma unroll
            for (int k = 0; k < 6; ++k) s = fmaf(Jn[6 * q + k], b[k], s);
            b2[q] = s;
        }
#pragma unroll
        for (int k = 0; k < 36; ++k) A[k] = T2[k];
#pragma unroll
        for (int k = 0; k < 6; ++k) b[k] = b2[k];
    }
#pragma unroll
    for (int k = 0; k < 36; ++k) sA[36 * t + k] = A[k];
#pragma unroll
    for (int k = 0; k < 6; ++k) sb[6 * t + k] = b[k];
    __syncthreads();
    // inclusive scan over the segments: (A_t, b_t) <- (A_t, b_t) o (A_{t-s}, b_{t-s})
    for (int st = 1; st < SCAN_T; st <<= 1) {
        float Ap[36], bp[6];
        const bool take = t >= st;
        if (take) {
#pragma unroll
            for (int k = 0; k < 36; ++k) Ap[k] = sA[36 * (t - st) + k];
#pragma unroll
            for (int k = 0; k < 6; ++k) bp[k] = sb[6 * (t - st) + k];
        }
        __syncthreads();
        if (take) {
            float T2[36], b2[6];
            mat6_mul(A, Ap, T2);
#pragma unroll
            for (int q = 0; q < 6; ++q) {
                float s = b[q];
#pragma unroll
                for (int k = 0; k < 6; ++k) s = fmaf(A[6 * q + k], bp[k], s);
                b2[q] = s;
            }
#pragma unroll
            for (int k = 0; k < 36; ++k) A[k] = T2[k];
#pragma unroll
            for (int k = 0; k < 6; ++k) b[k] = b2[k];
#pragma unroll
            for (int k = 0; k < 36; ++k) sA[36 * t + k] = A[k];
#pragma unroll
            for (int k = 0; k < 6; ++k) sb[6 * t + k] = b[k];
        }
        __syncthreads();
    }
    // replay the segment from its entry value e (the previous prefix's b)
    float e[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) e[k] = t > 0 ? sb[6 * (t - 1) + k] : 0.0f;
    float worst = 0.0f;
    for (int n = n0; n < n1; ++n) {
        float e2[6];
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            float s = (float)(a.F[6 * n + q] - a.U[6 * (n + 1) + q]);
#pragma unroll
            for (int k = 0; k < 6; ++k) s = fmaf(J[36 * n + 6 * q + k], e[k], s);
            e2[q] = s;
        }
        float ex = 0.0f, ev = 0.0f, nx = 0.0f, nv = 0.0f;
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            e[q] = e2[q];
            const double u = a.U[6 * (n + 1) + q] + (double)e2[q];
            a.U[6 * (n + 1) + q] = u;
            const float uf = (float)u;
            if (q < 3) {
                ex = fmaf(e2[q], e2[q], ex);
                nx = fmaf(uf, uf, nx);
            } else {
                ev = fmaf(e2[q], e2[q], ev);
                nv = fmaf(uf, uf, nv);
            }
        }
        worst = fmaxf(worst, fmaxf(ex / fmaxf(nx, 1e-30f), ev / fmaxf(nv, 1e-30f)));
    }
    sw[t] = worst;
    __syncthreads();
    for (int st = SCAN_T / 2; st > 0; st >>= 1) {
        if (t < st) sw[t] = fmaxf(sw[t], sw[t + st]);
        __syncthreads();
    }
    if (t == 0) {
        const float w = sqrtf(sw[0]);  // largest relative update
        const float prev = __int_as_float(a.flag[2]);
        a.flag[1] += 1;
        const bool floor_reached = a.flag[1] > 1 && w < 1e-12f && w > 0.5f * prev;
        if (w < (float)a.tol || floor_reached) a.flag[0] = 1;
        a.flag[2] = __float_as_int(w);
    }
}

// Guess + Newton iterations of one orbit (slice starts in a.U); returns
// the number of kernels launched.  With a.out set, the last slice pass
// writes the saved states.
template <class C>
static int launch_shoot(const PotDev<double>& P, const PotDev<float>& P32, const ShootArgs& a, cudaStream_t st) {
    shoot_guess_kernel<C><<<1, 32, 0, st>>>(P32, a);
    for (int it = 0; it < SHOOT_ITERS; ++it) {
        shoot_f64_kernel<C><<<(unsigned)((a.S + 63) / 64), 64, 0, st>>>(P, a);
        shoot_jac_kernel<C><<<(unsigned)((6 * a.S + 95) / 96), 96, 0, st>>>(P32, a);
        shoot_scan_kernel<<<1, SCAN_T, 0, st>>>(a);
    }
    return 1 + 3 * SHOOT_ITERS;
}

// ------------------------------------------------------------ sensitivities
// Progenitor sensitivities to every raw parameter (slot 6 c + j) and every
// component of the present-day state, on the release grid of the forward
// leg.  Direction d < NS is parameter slot d; d >= NS is state component
// d - NS.

struct TanArgs {
    const double* raw;   // [n_comp, 6]
    double G;
    int32_t S;
    int32_t NS;          // 6 n_comp
    int32_t n_dir;       // NS + 6
    int32_t n_steps;
    int32_t save_every;
    int32_t n_save;
    double dt;
    const double* Ub;    // back leg slice starts [S + 1, 6]
    const double* Uf;    // forward leg slice starts [S + 1, 6]
    double* Mb;          // [S, 6, 6 + NS]: [J | dF/dtheta] per back slice
    double* Mf;          // [S, 6, 6 + NS] per forward slice
    double* W;           // [S + 1, n_dir, 6] forward-leg start tangents
    double* states;      // [n_save, 6]
    double* tangents;    // [n_save, n_dir, 6]
};

template <class S_>
__device__ __forceinline__ void seed_params(const PotDev<double>& P, const TanArgs& a, int slot, PotDev<D1<S_>>& Q) {
    Q.n = P.n;
    Q.has_track = 0;
    Q.grow_mask = 0;
    Q.ex = P.ex;
    for (int c = 0; c < P.n; ++c) {
        double dq[6] = {0, 0, 0, 0, 0, 0};
        if (slot >= 0 && slot / 6 == c) prepared_param_tangent(P.c[c].kind, a.raw + 6 * c, slot % 6, a.G, dq);
        Q.c[c].kind = P.c[c].kind;
        Q.c[c].center = P.c[c].center;
        for (int j = 0; j < 6; ++j) Q.c[c].q[j] = D1<S_>(P.c[c].q[j], dq[j]);
    }
}

// lane (n, col): col < 6 state direction e_col, col >= 6 parameter slot col - 6
template <class C>
__global__ void __launch_bounds__(64) shoot_sens_kernel(PotDev<double> P, TanArgs a, int back) {
    const int ncol = 6 + a.NS;
    const int lane = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = lane / ncol, col = lane % ncol;
    if (n >= a.S) return;
    typedef D1<double> T;
    PotDev<T> Q;
    seed_params<double>(P, a, col >= 6 ? col - 6 : -1, Q);
    const double* U = back ? a.Ub : a.Uf;
    T y[6];
    for (int j = 0; j < 6; ++j) y[j] = T(U[6 * n + j], j == col ? 1.0 : 0.0);
    const T h(back ? -a.dt : a.dt, 0.0);
    const int len = n < a.S - 1 ? SHOOT_M : a.n_steps - SHOOT_M * (a.S - 1);
    for (int s = 0; s < len; ++s) dopri5_step_dual<C, double>(Q, h, y);
    double* M = (back ? a.Mb : a.Mf) + (int64_t)n * 6 * ncol;
    for (int j = 0; j < 6; ++j) M[j * ncol + col] = y[j].d;
}

// One thread per direction: chain the slice sensitivities through the back
// leg and then the forward leg.
__global__ void shoot_recur_kernel(TanArgs a) {
    const int d = threadIdx.x;
    if (d >= a.n_dir) return;
    const int ncol = 6 + a.NS;
    double v[6];
    for (int j = 0; j < 6; ++j) v[j] = (d >= a.NS && d - a.NS == j) ? 1.0 : 0.0;
    for (int leg = 0; leg < 2; ++leg) {
        const double* Mleg = leg == 0 ? a.Mb : a.Mf;
        for (int n = 0; n < a.S; ++n) {
            if (leg == 1)
                for (int j = 0; j < 6; ++j) a.W[((int64_t)n * a.n_dir + d) * 6 + j] = v[j];
            const double* M = Mleg + (int64_t)n * 6 * ncol;
            double w[6];
            for (int r = 0; r < 6; ++r) {
                double s = d < a.NS ? M[r * ncol + 6 + d] : 0.0;
                for (int c = 0; c < 6; ++c) s += M[r * ncol + c] * v[c];
                w[r] = s;
            }
            for (int j = 0; j < 6; ++j) v[j] = w[j];
        }
    }
    for (int j = 0; j < 6; ++j) a.W[((int64_t)a.S * a.n_dir + d) * 6 + j] = v[j];
}

// lane (n, d): forward slice n from (Uf[n], W[n, d]) with parameter seeds,
// writing states and tangents at the save points.
template <class C>
__global__ void __launch_bounds__(64) shoot_tan_save_kernel(PotDev<double> P, TanArgs a) {
    const int lane = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = lane / a.n_dir, d = lane % a.n_dir;
    if (n >= a.S) return;
    typedef D1<double> T;
    PotDev<T> Q;
    seed_params<double>(P, a, d < a.NS ? d : -1, Q);
    T y[6];
    for (int j = 0; j < 6; ++j) y[j] = T(a.Uf[6 * n + j], a.W[((int64_t)n * a.n_dir + d) * 6 + j]);
    auto save = [&](int k) {
        if (d == 0)
            for (int j = 0; j < 6; ++j) a.states[6 * k + j] = y[j].v;
        for (int j = 0; j < 6; ++j) a.tangents[((int64_t)k * a.n_dir + d) * 6 + j] = y[j].d;
    };
    if (n == 0) save(0);
    const T h(a.dt, 0.0);
    const int len = n < a.S - 1 ? SHOOT_M : a.n_steps - SHOOT_M * (a.S - 1);
    for (int s = 0; s < len; ++s) {
        dopri5_step_dual<C, double>(Q, h, y);
        const int g = n * SHOOT_M + s + 1;
        if (g % a.save_every == 0 && g / a.save_every < a.n_save) save(g / a.save_every);
    }
}

}  // namespace ssg

using namespace ssg;

extern "C" {

int64_t ss_orbit_shoot_slices(int64_t n_steps) {
    if (n_steps < 0) return set_error(SS_ERR_INVALID_ARGUMENT, "n_steps < 0");
    return (n_steps + SHOOT_M - 1) / SHOOT_M;
}

int64_t ss_orbit_shoot_workspace_bytes(int64_t n_steps) {
    if (n_steps < 0) return set_error(SS_ERR_INVALID_ARGUMENT, "n_steps < 0");
    const int64_t S = (n_steps + SHOOT_M - 1) / SHOOT_M;
    return (6 * (S + 1) + 6 * S + 36 * S) * (int64_t)sizeof(double) + 4 * (int64_t)sizeof(int32_t) + 256;
}

int ss_orbit_shoot_f64(const ss_potential* pot, const double* w0, double t0, double dt, int64_t n_steps,
                       int64_t save_every, double* out, void* workspace, int64_t workspace_bytes, double tol,
                       void* stream) {
    PotDev<double> P;
    int rc = prepare_potential<double>(pot, &P, true);
    if (rc) return rc;
    SS_CHECK_ARG(n_steps >= 0 && n_steps < (1LL << 30), "n_steps outside [0, 2^30)");
    SS_CHECK_ARG(save_every >= 1, "save_every must be >= 1");
    SS_CHECK_ARG(std::isfinite(dt) && dt != 0.0 && std::isfinite(t0), "dt must be finite and non-zero");
    SS_CHECK_ARG(w0 && out, "NULL buffer");
    SS_CHECK_ARG(tol > 0.0 && tol < 1e-6, "tol must be in (0, 1e-6)");
    cudaStream_t st = (cudaStream_t)stream;
    const bool is_static = !P.has_track && P.sh.n == 0 && !P.has_rot && !P.has_facc && !P.grow_mask;
    const int64_t S = (n_steps + SHOOT_M - 1) / SHOOT_M;
    bool handled = false;
    if (is_static && S >= 2) {
        SS_CHECK_ARG(workspace != nullptr && workspace_bytes >= ss_orbit_shoot_workspace_bytes(n_steps),
                     "workspace of %lld bytes needed", (long long)ss_orbit_shoot_workspace_bytes(n_steps));
        SS_CHECK_ARG(((uintptr_t)workspace % 8) == 0, "workspace must be 8-byte aligned");
        PotDev<float> P32;
        rc = prepare_potential<float>(pot, &P32, true);
        if (rc) return rc;
        ShootArgs a;
        a.w0 = w0;
        a.dt = dt;
        a.n_steps = (int32_t)n_steps;
        a.S = (int32_t)S;
        a.save_every = (int32_t)save_every;
        a.n_save = (int32_t)(n_steps / save_every + 1);
        a.U = (double*)workspace;
        a.F = a.U + 6 * (S + 1);
        a.J = a.F + 6 * S;
        a.flag = (int32_t*)(a.J + 36 * S);
        a.tol = tol;
        a.out = out;
        SS_CUDA_TRY(cudaMemsetAsync(a.flag, 0, 4 * sizeof(int32_t), st));
        int launched = 0;
        dispatch_comp(P, [&](auto comp) {
            using C = decltype(comp);
            if constexpr (!std::is_same<C, GenericComp>::value) launched = launch_shoot<C>(P, P32, a, st);
            return 0;
        });
        for (int i = 1; i < launched; ++i) count_launch();
        if (launched) {
            SS_LAUNCH_CHECK();
            handled = true;
        }
    }
    if (!handled) return ss_orbit_f64(pot, w0, 1, t0, dt, n_steps, save_every, out, stream);
    return SS_OK;
}

int64_t ss_prog_tangents_workspace_bytes(int64_t n_steps, int32_t n_comp) {
    if (n_steps < 0 || n_comp < 1) return set_error(SS_ERR_INVALID_ARGUMENT, "bad arguments");
    const int64_t S = (n_steps + SHOOT_M - 1) / SHOOT_M;
    const int64_t NS = 6 * n_comp, nd = NS + 6;
    const int64_t leg = 6 * (S + 1) + 6 * S + 36 * S + 2;  // U, F, J, flags (two doubles)
    return (2 * leg + 2 * S * 6 * (6 + NS) + (S + 1) * nd * 6) * (int64_t)sizeof(double) + 256;
}

int ss_prog_tangents_f64(const ss_potential* pot, const double* raw_params, const double* w0, double dt,
                         int32_t n_steps, int32_t save_every, double* states, double* tangents,
                         const double* starts_back, const double* starts_fwd, void* workspace,
                         int64_t workspace_bytes, void* stream) {
    PotDev<double> P;
    int rc = prepare_potential<double>(pot, &P, false);
    if (rc) return rc;
    SS_CHECK_ARG(!P.has_track && !P.has_rot && !P.has_facc && !P.grow_mask, "progenitor tangents need a static potential");
    SS_CHECK_ARG(P.n >= 1 && P.n <= 4, "progenitor tangents support 1 to 4 components (one warp of directions)");
    SS_CHECK_ARG(std::isfinite(dt) && dt > 0.0 && n_steps >= 2 * SHOOT_M && save_every >= 1, "bad steps");
    SS_CHECK_ARG(raw_params && w0 && states && tangents, "NULL buffer");
    const int64_t need = ss_prog_tangents_workspace_bytes(n_steps, P.n);
    SS_CHECK_ARG(workspace && workspace_bytes >= need && ((uintptr_t)workspace % 8) == 0,
                 "workspace of %lld bytes (8-byte aligned) needed", (long long)need);
    PotDev<float> P32;
    rc = prepare_potential<float>(pot, &P32, false);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const int S = (n_steps + SHOOT_M - 1) / SHOOT_M;
    const int NS = 6 * P.n, nd = NS + 6;
    double* ws = (double*)workspace;
    const int64_t leg = 6 * (S + 1) + 6 * S + 36 * S + 2;
    auto leg_args = [&](double* base, const double* start, double h) {
        ShootArgs a;
        a.w0 = start;
        a.dt = h;
        a.n_steps = n_steps;
        a.S = S;
        a.save_every = 1;
        a.n_save = 0;
        a.U = base;
        a.F = a.U + 6 * (S + 1);
        a.J = a.F + 6 * S;
        a.flag = (int32_t*)(a.J + 36 * S);
        a.tol = 1e-14;
        a.out = nullptr;
        return a;
    };
    ShootArgs ab = leg_args(ws, w0, -dt);
    ShootArgs af = leg_args(ws + leg, ws + 6 * S, dt);  // forward leg starts at the back leg's end
    TanArgs t;
    t.raw = raw_params;
    t.G = pot->G;
    t.S = S;
    t.NS = NS;
    t.n_dir = nd;
    t.n_steps = n_steps;
    t.save_every = save_every;
    t.n_save = n_steps / save_every + 1;
    t.dt = dt;
    t.Ub = ab.U;
    t.Uf = af.U;
    t.Mb = ws + 2 * leg;
    t.Mf = t.Mb + (int64_t)S * 6 * (6 + NS);
    t.W = t.Mf + (int64_t)S * 6 * (6 + NS);
    t.states = states;
    t.tangents = tangents;
    SS_CUDA_TRY(cudaMemsetAsync(ab.flag, 0, 4 * sizeof(int32_t), st));
    SS_CUDA_TRY(cudaMemsetAsync(af.flag, 0, 4 * sizeof(int32_t), st));
    SS_CHECK_ARG((starts_back == nullptr) == (starts_fwd == nullptr), "give both leg starts or neither");
    const bool reuse = starts_back != nullptr;
    if (reuse) {
        SS_CUDA_TRY(cudaMemcpyAsync(ab.U, starts_back, 6 * (size_t)(S + 1) * sizeof(double), cudaMemcpyDeviceToDevice,
                                    st));
        SS_CUDA_TRY(cudaMemcpyAsync(af.U, starts_fwd, 6 * (size_t)(S + 1) * sizeof(double), cudaMemcpyDeviceToDevice,
                                    st));
    }
    int launched = 0;
    dispatch_comp(P, [&](auto comp) {
        using C = decltype(comp);
        if constexpr (!std::is_same<C, GenericComp>::value) {
            if (!reuse) {
                launched += launch_shoot<C>(P, P32, ab, st);
                launched += launch_shoot<C>(P, P32, af, st);
            }
            const int lanes = S * (6 + NS);
            shoot_sens_kernel<C><<<(unsigned)((lanes + 63) / 64), 64, 0, st>>>(P, t, 1);
            shoot_sens_kernel<C><<<(unsigned)((lanes + 63) / 64), 64, 0, st>>>(P, t, 0);
            shoot_recur_kernel<<<1, 32, 0, st>>>(t);
            shoot_tan_save_kernel<C><<<(unsigned)((S * nd + 63) / 64), 64, 0, st>>>(P, t);
            launched += 4;
        }
        return 0;
    });
    if (!launched)
        return set_error(SS_ERR_UNSUPPORTED, "progenitor tangents are compiled for the built-in compositions only");
    for (int i = 1; i < launched; ++i) count_launch();
    SS_LAUNCH_CHECK();
    return SS_OK;
}

}  // extern "C"
