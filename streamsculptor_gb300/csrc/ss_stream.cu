// ss_stream.cu — the hot path: every released star integrated from its
// release step to the end with fixed-step Dormand-Prince 5(4), force fused
// into the stage loop, state and stages in registers.
//
// Reference: Potential.gen_stream_vmapped / gen_stream_scan (main.py:312-368)
// integrate particle i (lead and trail) from ts[i] to ts[-1] through
// integrate_orbit (main.py:125-163); gen_stream_vmapped_Chen25
// (streamhelpers.py:491-543) adds the moving progenitor (a
// TimeDepTranslatingPotential on a cubic spline of the progenitor orbit);
// gen_stream_vmapped_with_pert (streamhelpers.py:89-146) adds subhalos.
//
// Layout: one thread per particle; particles are ordered by release (release
// r owns particles [r*ppr, (r+1)*ppr)), so the earliest (longest) particles
// sit in the lowest blocks and are scheduled first.  A warp runs in global
// lock-step from its earliest start step: lanes released later idle until
// their release step, so every active lane evaluates the same stage time and
// the track / subhalo table reads are warp-uniform broadcasts.
//
// Two precisions:
//   ss_stream_f64   FP64 state, stages and force (parity path).
//   ss_stream_f32k  FP32 stages and force; position and velocity kept as
//                   compensated hi+lo float pairs; the increments are formed
//                   as h*v_hi (exact two-product) plus small corrections, so
//                   float rounding of the tableau touches only second-order
//                   terms.  Time and release bookkeeping are integer/FP64 and
//                   happen outside the step loop; the progenitor track and
//                   subhalo lines are pre-tabulated in FP32 (workspace).

#include <cuda_runtime.h>

#include <cmath>

#include "ss_common.cuh"

namespace ssg {

struct StreamArgs {
    const double* ics;
    double* final_w;
    float* snaps;
    int32_t* status;
    int64_t N;
    int32_t ppr;
    int32_t spr;
    int32_t n_steps;
    int32_t stride;
    double t0;
    double dt;
    // f32k only
    float h_hi;
    float h_lo;
    const float4* ctab;   // [(n_steps*5+1) x 2] track positions (hi, lo) at stage times
    const float4* shtab;  // [n_sh*3] subhalo lines
    int32_t n_sh;
    int32_t sh_kind;
};

// Write the snapshot k for lane state y (or NaN when not yet released).
template <class T>
__device__ __forceinline__ void write_snap(float* snaps, int64_t N, int64_t k, int64_t p, bool exists, const T y[6]) {
    float2* o = reinterpret_cast<float2*>(snaps + (k * N + p) * 6);
    const float nanf_ = __int_as_float(0x7fc00000);
    if (exists) {
        o[0] = make_float2((float)y[0], (float)y[1]);
        o[1] = make_float2((float)y[2], (float)y[3]);
        o[2] = make_float2((float)y[4], (float)y[5]);
    } else {
        o[0] = make_float2(nanf_, nanf_);
        o[1] = make_float2(nanf_, nanf_);
        o[2] = make_float2(nanf_, nanf_);
    }
}

// ------------------------------------------------------------------ FP64
__global__ void __launch_bounds__(64) stream_f64_kernel(PotDev<double> P, StreamArgs a) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = p < a.N;
    const int start = valid ? (int)((p / a.ppr) * (int64_t)a.spr) : a.n_steps;
    const int wstart = (int)__reduce_min_sync(0xffffffffu, (unsigned)start);
    double y[6];
    if (valid) {
#pragma unroll
        for (int i = 0; i < 6; ++i) y[i] = a.ics[6 * p + i];
    } else {
#pragma unroll
        for (int i = 0; i < 6; ++i) y[i] = 0.0;
    }
    if (a.snaps && valid) {
        for (int64_t k = 0; (k + 1) * (int64_t)a.stride <= wstart; ++k) {
            int64_t step = (k + 1) * (int64_t)a.stride;
            write_snap<double>(a.snaps, a.N, k, p, step >= start, y);
        }
    }
    for (int n = wstart; n < a.n_steps; ++n) {
        if (valid && n >= start) dopri5_step_f64(P, a.t0 + (double)n * a.dt, a.dt, y);
        if (a.snaps && (n + 1) % a.stride == 0 && valid)
            write_snap<double>(a.snaps, a.N, (n + 1) / a.stride - 1, p, n + 1 >= start, y);
    }
    if (!valid) return;
    bool ok = true;
#pragma unroll
    for (int i = 0; i < 6; ++i) ok = ok && isfinite(y[i]);
    if (a.status) a.status[p] = ok ? 0 : 1;
    if (a.final_w) {
#pragma unroll
        for (int i = 0; i < 6; ++i) a.final_w[6 * p + i] = y[i];
    }
}

// ------------------------------------------------------------------ FP32-K
#define F_C2 0.2f
#define F_C3 0.3f
#define F_C4 0.8f
#define F_C5 ((float)(8.0 / 9.0))
#define F_(x) ((float)(x))

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// Acceleration at the stage position xh + d (xh: the particle's hi part,
// d: the small remainder of the stage offset).  Components on the center
// track use (xh - c_hi) + (d - c_lo): xh and c_hi are close, so the
// difference is exact and the separation keeps its relative precision.
__device__ __forceinline__ void accel_f32(const PotDev<float>& P, const StreamArgs& a, const float xh[3],
                                          const float d[3], int slot, float trel, float A[3]) {
    const float X[3] = {xh[0] + d[0], xh[1] + d[1], xh[2] + d[2]};
    float xs[3] = {X[0], X[1], X[2]};
    if (P.has_track) {
        const float4 ch = __ldg(a.ctab + 2 * slot);
        const float4 cl = __ldg(a.ctab + 2 * slot + 1);
        xs[0] = (xh[0] - ch.x) + (d[0] - cl.x);
        xs[1] = (xh[1] - ch.y) + (d[1] - cl.y);
        xs[2] = (xh[2] - ch.z) + (d[2] - cl.z);
    }
    float g[3];
    pot_grad<float, float, false>(P, X, xs, g, nullptr);
#pragma unroll 1
    for (int j = 0; j < a.n_sh; ++j) {
        float4 s0 = __ldg(a.shtab + 3 * j);
        float4 s1 = __ldg(a.shtab + 3 * j + 1);
        float4 s2 = __ldg(a.shtab + 3 * j + 2);
        float tau = trel - s2.x;
        if (!(fabsf(tau) < s2.y)) continue;
        float rel[3] = {X[0] - (s0.x + s1.x * trel), X[1] - (s0.y + s1.y * trel), X[2] - (s0.z + s1.z * trel)};
        float gp[3], dummy[3];
        subhalo_grad<float, false>(a.sh_kind, s0.w, s1.w, rel, gp, dummy);
        g[0] += gp[0];
        g[1] += gp[1];
        g[2] += gp[2];
    }
    A[0] = -g[0];
    A[1] = -g[1];
    A[2] = -g[2];
}

// One compensated step.  V_i = vh + d_i and sum_j a_ij = c_i, sum_i b_i = 1
// are used exactly, so only the small parts d_i and A_i - A_1 see the
// rounded tableau.
__device__ __forceinline__ void step_f32k(const PotDev<float>& P, const StreamArgs& a, int n, float xh[3],
                                          float xl[3], float vh[3], float vl[3]) {
    const float h = a.h_hi;
    const float tn = (float)n * h;  // time since global step 0 (subhalo lines)
    const int s0 = 5 * n;
    float A1[3], A2[3], A3[3], A4[3], A5[3], A6[3];
    float d1[3], d2[3], d3[3], d4[3], d5[3], d6[3];
    float D[3];  // stage position offset from xh (small)
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        D[i] = xl[i];
        d1[i] = vl[i];
    }
    accel_f32(P, a, xh, D, s0, tn, A1);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        d2[i] = vl[i] + h * (F_(SS_A21) * A1[i]);
        D[i] = xl[i] + h * (F_C2 * vh[i] + F_(SS_A21) * d1[i]);
    }
    accel_f32(P, a, xh, D, s0 + 1, tn + F_C2 * h, A2);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        d3[i] = vl[i] + h * (F_(SS_A31) * A1[i] + F_(SS_A32) * A2[i]);
        D[i] = xl[i] + h * (F_C3 * vh[i] + F_(SS_A31) * d1[i] + F_(SS_A32) * d2[i]);
    }
    accel_f32(P, a, xh, D, s0 + 2, tn + F_C3 * h, A3);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        d4[i] = vl[i] + h * (F_(SS_A41) * A1[i] + F_(SS_A42) * A2[i] + F_(SS_A43) * A3[i]);
        D[i] = xl[i] + h * (F_C4 * vh[i] + F_(SS_A41) * d1[i] + F_(SS_A42) * d2[i] + F_(SS_A43) * d3[i]);
    }
    accel_f32(P, a, xh, D, s0 + 3, tn + F_C4 * h, A4);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        d5[i] = vl[i] + h * (F_(SS_A51) * A1[i] + F_(SS_A52) * A2[i] + F_(SS_A53) * A3[i] + F_(SS_A54) * A4[i]);
        D[i] = xl[i] + h * (F_C5 * vh[i] + F_(SS_A51) * d1[i] + F_(SS_A52) * d2[i] + F_(SS_A53) * d3[i] +
                            F_(SS_A54) * d4[i]);
    }
    accel_f32(P, a, xh, D, s0 + 4, tn + F_C5 * h, A5);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        d6[i] = vl[i] + h * (F_(SS_A61) * A1[i] + F_(SS_A62) * A2[i] + F_(SS_A63) * A3[i] + F_(SS_A64) * A4[i] +
                             F_(SS_A65) * A5[i]);
        D[i] = xl[i] + h * (vh[i] + F_(SS_A61) * d1[i] + F_(SS_A62) * d2[i] + F_(SS_A63) * d3[i] +
                            F_(SS_A64) * d4[i] + F_(SS_A65) * d5[i]);
    }
    accel_f32(P, a, xh, D, s0 + 5, tn + h, A6);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        // position: h * (vh + Db), Db = sum b_i d_i
        float Db = F_(SS_B1) * d1[i] + F_(SS_B3) * d3[i] + F_(SS_B4) * d4[i] + F_(SS_B5) * d5[i] + F_(SS_B6) * d6[i];
        float pp = h * vh[i];
        float pe = fmaf(h, vh[i], -pp);
        float lo = pe + (a.h_lo * vh[i] + h * Db);
        float s, e;
        two_sum(xh[i], pp, s, e);
        float l2 = xl[i] + (e + lo);
        xh[i] = s + l2;
        xl[i] = l2 - (xh[i] - s);
        // velocity: h * (A1 + sum_{i>=3} b_i (A_i - A1))
        float Sv = A1[i] + (F_(SS_B3) * (A3[i] - A1[i]) + F_(SS_B4) * (A4[i] - A1[i]) + F_(SS_B5) * (A5[i] - A1[i]) +
                            F_(SS_B6) * (A6[i] - A1[i]));
        float qp = h * Sv;
        float qe = fmaf(h, Sv, -qp) + a.h_lo * Sv;
        two_sum(vh[i], qp, s, e);
        l2 = vl[i] + (e + qe);
        vh[i] = s + l2;
        vl[i] = l2 - (vh[i] - s);
    }
}

__global__ void __launch_bounds__(128) stream_f32k_kernel(PotDev<float> P, StreamArgs a) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = p < a.N;
    const int start = valid ? (int)((p / a.ppr) * (int64_t)a.spr) : a.n_steps;
    const int wstart = (int)__reduce_min_sync(0xffffffffu, (unsigned)start);
    float xh[3], xl[3], vh[3], vl[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        double xd = valid ? a.ics[6 * p + i] : 0.0;
        double vd = valid ? a.ics[6 * p + 3 + i] : 0.0;
        xh[i] = (float)xd;
        xl[i] = (float)(xd - (double)xh[i]);
        vh[i] = (float)vd;
        vl[i] = (float)(vd - (double)vh[i]);
    }
    if (a.snaps && valid) {
        float y[6] = {xh[0], xh[1], xh[2], vh[0], vh[1], vh[2]};
        for (int64_t k = 0; (k + 1) * (int64_t)a.stride <= wstart; ++k) {
            int64_t step = (k + 1) * (int64_t)a.stride;
            write_snap<float>(a.snaps, a.N, k, p, step >= start, y);
        }
    }
    for (int n = wstart; n < a.n_steps; ++n) {
        if (valid && n >= start) step_f32k(P, a, n, xh, xl, vh, vl);
        if (a.snaps && (n + 1) % a.stride == 0 && valid) {
            float y[6] = {xh[0], xh[1], xh[2], vh[0], vh[1], vh[2]};
            write_snap<float>(a.snaps, a.N, (n + 1) / a.stride - 1, p, n + 1 >= start, y);
        }
    }
    if (!valid) return;
    bool ok = true;
#pragma unroll
    for (int i = 0; i < 3; ++i) ok = ok && isfinite(xh[i]) && isfinite(vh[i]) && isfinite(xl[i]) && isfinite(vl[i]);
    if (a.status) a.status[p] = ok ? 0 : 1;
    if (a.final_w) {
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            a.final_w[6 * p + i] = (double)xh[i] + (double)xl[i];
            a.final_w[6 * p + 3 + i] = (double)vh[i] + (double)vl[i];
        }
    }
}

// Track positions at every stage time of the run, FP64 Hermite -> a hi/lo
// float pair (two float4).  Slot 5n + s holds c(t0 + (n + c_s) dt) for
// c = {0, 1/5, 3/10, 4/5, 8/9}; slot 5 n_steps holds c(t0 + n_steps dt).
__global__ void track_table_kernel(TrackDev tr, double t0, double dt, int32_t n_steps, float4* tab) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t total = 5 * (int64_t)n_steps + 1;
    if (i >= total) return;
    int64_t n = i / 5;
    int s = (int)(i % 5);
    const double cs[5] = {0.0, SS_C2, SS_C3, SS_C4, SS_C5};
    double t = t0 + ((double)n + cs[s]) * dt;
    double c[3];
    track_eval(tr, t, c);
    float hx = (float)c[0], hy = (float)c[1], hz = (float)c[2];
    tab[2 * i] = make_float4(hx, hy, hz, 0.f);
    tab[2 * i + 1] = make_float4((float)(c[0] - (double)hx), (float)(c[1] - (double)hy), (float)(c[2] - (double)hz), 0.f);
}

// Subhalo lines relative to the run start t0: position at t0, velocity,
// (t0_s - t0, window).
__global__ void subhalo_table_kernel(ShDev sh, double t0, float4* tab) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= sh.n) return;
    double tau = t0 - sh.t0[j];
    tab[3 * j] = make_float4((float)(sh.x0[3 * j] + sh.v[3 * j] * tau), (float)(sh.x0[3 * j + 1] + sh.v[3 * j + 1] * tau),
                             (float)(sh.x0[3 * j + 2] + sh.v[3 * j + 2] * tau), (float)(sh.G * sh.m[j]));
    tab[3 * j + 1] = make_float4((float)sh.v[3 * j], (float)sh.v[3 * j + 1], (float)sh.v[3 * j + 2], (float)sh.a[j]);
    float win = isinf(sh.t_window) ? __int_as_float(0x7f800000) : (float)sh.t_window;
    tab[3 * j + 2] = make_float4((float)(sh.t0[j] - t0), win, 0.f, 0.f);
}

static int check_stream_cfg(const ss_stream_cfg* cfg) {
    SS_CHECK_ARG(cfg != nullptr, "cfg is NULL");
    SS_CHECK_ARG(cfg->n_particles >= 0, "n_particles < 0");
    SS_CHECK_ARG(cfg->n_steps >= 0 && cfg->n_steps < (1LL << 30), "n_steps outside [0, 2^30)");
    SS_CHECK_ARG(cfg->particles_per_release >= 1 && cfg->steps_per_release >= 0, "bad release layout");
    SS_CHECK_ARG(std::isfinite(cfg->dt) && cfg->dt > 0.0 && std::isfinite(cfg->t0), "dt must be finite and > 0");
    SS_CHECK_ARG(cfg->snap_stride >= 0, "snap_stride < 0");
    int64_t n_rel = (cfg->n_particles + cfg->particles_per_release - 1) / cfg->particles_per_release;
    SS_CHECK_ARG(n_rel == 0 || (n_rel - 1) * (int64_t)cfg->steps_per_release <= cfg->n_steps,
                 "last release starts after n_steps");
    return SS_OK;
}

static StreamArgs make_args(const ss_stream_cfg* cfg, const double* ics, double* final_w, float* snaps,
                            int32_t* status) {
    StreamArgs a;
    memset(&a, 0, sizeof(a));
    a.ics = ics;
    a.final_w = final_w;
    a.snaps = cfg->snap_stride > 0 && cfg->n_steps >= cfg->snap_stride ? snaps : nullptr;
    a.status = status;
    a.N = cfg->n_particles;
    a.ppr = cfg->particles_per_release;
    a.spr = cfg->steps_per_release;
    a.n_steps = (int32_t)cfg->n_steps;
    a.stride = cfg->snap_stride > 0 ? cfg->snap_stride : 1;
    a.t0 = cfg->t0;
    a.dt = cfg->dt;
    a.h_hi = (float)cfg->dt;
    a.h_lo = (float)(cfg->dt - (double)a.h_hi);
    return a;
}

static int64_t f32k_workspace(const ss_potential* pot, const ss_stream_cfg* cfg) {
    int64_t bytes = 0;
    bool track = false;
    for (int k = 0; k < pot->n_components && k < SS_MAX_COMPONENTS; ++k) track |= pot->comp[k].center == SS_CENTER_TRACK;
    if (track) bytes += (5 * cfg->n_steps + 1) * 2 * (int64_t)sizeof(float4);
    bytes = (bytes + 255) / 256 * 256;
    if (pot->subhalos.n > 0) bytes += 3 * pot->subhalos.n * (int64_t)sizeof(float4);
    return bytes;
}

}  // namespace ssg

using namespace ssg;

extern "C" {

int ss_stream_f64(const ss_potential* pot, const ss_stream_cfg* cfg, const double* ics, double* final_w, float* snaps,
                  int32_t* status, void* stream) {
    PotDev<double> P;
    int rc = prepare_potential<double>(pot, &P, true);
    if (rc) return rc;
    rc = check_stream_cfg(cfg);
    if (rc) return rc;
    if (cfg->n_particles == 0) return SS_OK;
    SS_CHECK_ARG(ics != nullptr, "ics is NULL");
    StreamArgs a = make_args(cfg, ics, final_w, snaps, status);
    const int block = 64;
    unsigned grid = (unsigned)((cfg->n_particles + block - 1) / block);
    stream_f64_kernel<<<grid, block, 0, (cudaStream_t)stream>>>(P, a);
    SS_LAUNCH_CHECK();
    return SS_OK;
}

int64_t ss_stream_workspace_bytes(const ss_potential* pot, const ss_stream_cfg* cfg) {
    if (!pot || !cfg) return set_error(SS_ERR_INVALID_ARGUMENT, "NULL argument");
    return f32k_workspace(pot, cfg);
}

int ss_stream_f32k(const ss_potential* pot, const ss_stream_cfg* cfg, const double* ics, double* final_w,
                   float* snaps, int32_t* status, void* workspace, int64_t workspace_bytes, void* stream) {
    PotDev<float> P;
    int rc = prepare_potential<float>(pot, &P, true);
    if (rc) return rc;
    rc = check_stream_cfg(cfg);
    if (rc) return rc;
    if (cfg->n_particles == 0) return SS_OK;
    SS_CHECK_ARG(ics != nullptr, "ics is NULL");
    int64_t need = f32k_workspace(pot, cfg);
    if (need > 0 && (workspace == nullptr || workspace_bytes < need))
        return set_error(SS_ERR_WORKSPACE, "workspace of %lld bytes needed, %lld given", (long long)need,
                         (long long)workspace_bytes);
    SS_CHECK_ARG(need == 0 || ((uintptr_t)workspace % 256) == 0, "workspace must be 256-byte aligned");
    cudaStream_t s = (cudaStream_t)stream;
    StreamArgs a = make_args(cfg, ics, final_w, snaps, status);
    char* ws = (char*)workspace;
    if (P.has_track) {
        float4* tab = (float4*)ws;
        int64_t total = 5 * cfg->n_steps + 1;
        track_table_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(P.track, cfg->t0, cfg->dt,
                                                                            (int32_t)cfg->n_steps, tab);
        SS_LAUNCH_CHECK();
        a.ctab = tab;
        ws += (total * 2 * (int64_t)sizeof(float4) + 255) / 256 * 256;
    }
    if (pot->subhalos.n > 0) {
        PotDev<double> Pd;
        rc = prepare_potential<double>(pot, &Pd, true);
        if (rc) return rc;
        float4* tab = (float4*)ws;
        subhalo_table_kernel<<<(unsigned)((Pd.sh.n + 127) / 128), 128, 0, s>>>(Pd.sh, cfg->t0, tab);
        SS_LAUNCH_CHECK();
        a.shtab = tab;
        a.n_sh = Pd.sh.n;
        a.sh_kind = Pd.sh.kind;
    }
    const int block = 128;
    unsigned grid = (unsigned)((cfg->n_particles + block - 1) / block);
    stream_f32k_kernel<<<grid, block, 0, s>>>(P, a);
    SS_LAUNCH_CHECK();
    return SS_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// No-allocation variant of ss_stream_f32k.
//
// Some callers cannot allocate device memory at all: language bindings that
// reach this library through a bare C FFI and hold no device allocator, host
// code that must not make a call that may synchronize the device (cudaMalloc
// and cudaFree can), and applications whose device memory is owned entirely
// by another allocator.  For them the FP32 stream's scratch (the progenitor
// track and subhalo tables) lives in this fixed file-scope array instead of
// a caller workspace.  Every GPU that loads the library holds the array until
// the process exits.
#define SS_NOALLOC_SCRATCH_BYTES (4LL << 20)

static __device__ __align__(256) unsigned char g_noalloc_scratch[SS_NOALLOC_SCRATCH_BYTES];

#include <mutex>

namespace {
std::mutex g_noalloc_mu;
void* g_noalloc_ptr[64] = {nullptr};
}  // namespace

// Device address of g_noalloc_scratch on the current device, looked up once
// per device (host code cannot use the symbol's host-side name as a device
// pointer).
static int noalloc_scratch(void** out) {
    int dev = 0;
    SS_CUDA_TRY(cudaGetDevice(&dev));
    SS_CHECK_ARG(dev >= 0 && dev < 64, "device ordinal %d out of range", dev);
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (g_noalloc_ptr[dev] == nullptr) {
        void* p = nullptr;
        SS_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        g_noalloc_ptr[dev] = p;
    }
    *out = g_noalloc_ptr[dev];
    return SS_OK;
}

extern "C" int ss_stream_f32k_noalloc(const ss_potential* pot, const ss_stream_cfg* cfg, const double* ics,
                                      double* final_w, float* snaps, int32_t* status, void* stream) {
    if (!pot || !cfg) return set_error(SS_ERR_INVALID_ARGUMENT, "NULL argument");
    const int64_t need = f32k_workspace(pot, cfg);
    if (need > SS_NOALLOC_SCRATCH_BYTES)
        return set_error(SS_ERR_WORKSPACE,
                         "ss_stream_f32k_noalloc: this run needs %lld bytes of scratch but the fixed scratch holds "
                         "%lld (about 26000 steps with a moving progenitor); use ss_stream_f32k with a workspace",
                         (long long)need, (long long)SS_NOALLOC_SCRATCH_BYTES);
    void* scratch = nullptr;
    int rc = noalloc_scratch(&scratch);
    if (rc) return rc;
    return ss_stream_f32k(pot, cfg, ics, final_w, snaps, status, scratch, SS_NOALLOC_SCRATCH_BYTES, stream);
}
