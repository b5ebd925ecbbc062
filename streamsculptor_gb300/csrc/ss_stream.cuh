// ss_stream.cuh — device code of the stream integrators shared by the
// stream kernels (ss_stream.cu) and the adjoint (ss_adjoint.cu): launch
// arguments, snapshot writes, the FP64 and FP32-compensated kernels and the
// compensated FP32 Dopri5 step.
#pragma once

#include <cuda_runtime.h>

#include "ss_common.cuh"

namespace ssg {

enum { SUB_NONE = 0, SUB_LINES = 1, SUB_GRID = 2 };

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
    const float4* ttab;   // [(n_steps*5+1) x 2] (cos, sin, ga.x, ga.y), (ga.z, g, -, -) at stage times
    int32_t n_sh;
    int32_t sh_kind;
    ShDev shg;  // SS_SH_GRID: the FP64 spline tables of the subhalos
    // optional checkpoints of the compensated state every ckpt_stride local
    // steps: [n_seg, N, 3] float4 = (xh, vh.x), (vh.yz, xl.xy), (xl.z, vl)
    float4* ckpt;
    int32_t ckpt_stride;
    // sub-range runs: global index of local particle 0, snapshot row pitch
    int64_t p_off;
    int64_t snap_pitch;
    // ensembles: particles per stream (0 = one stream) and subhalo rows per
    // stream (0 = every particle feels the whole table)
    int64_t grp;
    int32_t sh_per_grp;
};

// The FP32 per-interval copy of a potential's expansion table (ss_stream.cu):
// its size in bytes (0 without an expansion), and its construction into
// `ws` (16-byte aligned) on stream s, which sets P.ex.tab32.
int64_t expansion_table32_bytes(const ss_potential* pot);
int expansion_table32(PotDev<float>& P, void* ws, cudaStream_t s);

// Release step of global particle q (its index within its stream picks the
// release when the run is an ensemble of streams).
__device__ __forceinline__ int stream_start(const StreamArgs& a, int64_t q) {
    const int64_t ql = a.grp > 0 ? q % a.grp : q;
    return (int)((ql / a.ppr) * (int64_t)a.spr);
}

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
// Steps per chunk of the FP64 kernel's shared stage-time track table.
constexpr int F64_CHUNK = 32;
constexpr int F64_BLOCK = 64;

// The block steps in chunks of F64_CHUNK steps from its earliest start.
// With a center track (the moving progenitor) the block first tabulates
// the track at the chunk's 6 F64_CHUNK stage times in shared memory (each
// thread evaluates a few), so a stage reads its center instead of
// evaluating the FP64 Hermite segment: the evaluations are the same
// (same times, same arithmetic), one per block instead of one per thread.
template <class C>
__device__ __forceinline__ void stream_f64_body(const PotDev<double>& P, const StreamArgs& a) {
    __shared__ double ctab[6 * F64_CHUNK][3];
    __shared__ int s_start;
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = p < a.N;
    const int start = valid ? stream_start(a, p + a.p_off) : a.n_steps;
    const int wstart = (int)__reduce_min_sync(0xffffffffu, (unsigned)start);
    if (threadIdx.x == 0) s_start = a.n_steps;
    __syncthreads();
    if ((threadIdx.x & 31) == 0) atomicMin(&s_start, wstart);
    __syncthreads();
    const int bstart = s_start;
    const bool tab = P.has_track;
    const ShDev sh = a.sh_per_grp > 0 ? subhalo_slice(P.sh, (p + a.p_off) / a.grp, a.sh_per_grp) : P.sh;
    double y[6];
    if (valid) {
#pragma unroll
        for (int i = 0; i < 6; ++i) y[i] = a.ics[6 * p + i];
    } else {
#pragma unroll
        for (int i = 0; i < 6; ++i) y[i] = 0.0;
    }
    if (a.snaps && valid) {
        for (int64_t k = 0; (k + 1) * (int64_t)a.stride <= bstart; ++k) {
            int64_t step = (k + 1) * (int64_t)a.stride;
            write_snap<double>(a.snaps, a.snap_pitch, k, p + a.p_off, step >= start, y);
        }
    }
    for (int n0 = bstart; n0 < a.n_steps; n0 += F64_CHUNK) {
        const int cnt = min(F64_CHUNK, a.n_steps - n0);
        if (tab) {
            __syncthreads();  // the previous chunk's table has been read
            for (int i = threadIdx.x; i < 6 * cnt; i += blockDim.x) {
                const int j = i / 6, s = i - 6 * j;
                // the stage times of dopri5_step_f64: t_n + c_s h
                const double t = a.t0 + (double)(n0 + j) * a.dt;
                const double c = s == 1 ? SS_C2 : s == 2 ? SS_C3 : s == 3 ? SS_C4 : SS_C5;
                track_eval(P.track, s == 0 ? t : s == 5 ? t + a.dt : t + c * a.dt, ctab[i]);
            }
            __syncthreads();
        }
        for (int j = 0; j < cnt; ++j) {
            const int n = n0 + j;
            if (valid && n >= start)
                dopri5_step_f64<C>(P, sh, a.t0 + (double)n * a.dt, a.dt, y, tab ? &ctab[6 * j] : nullptr);
            if (a.snaps && (n + 1) % a.stride == 0 && valid)
                write_snap<double>(a.snaps, a.snap_pitch, (n + 1) / a.stride - 1, p + a.p_off, n + 1 >= start, y);
        }
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

// ------------------------------------------------- FP64, component-split
// Small runs (fewer warps than the GPU has schedulers) leave most of the FP64
// units idle, and each warp's FP64 instructions are issued one after another
// by its scheduler's FP64 unit: the run lasts as long as the longest tracks'
// warps take to issue their instructions, whatever the number of active
// lanes.  This form spreads each particle over the C::n (>= 3) warps of one
// block: warp w evaluates component w of the force, and warps 0-2 each own
// one coordinate pair (x_w, v_w) of the state and do its share of the Dopri5
// arithmetic.  Per stage the owners publish their stage position through
// shared memory, every warp evaluates its component there, and each owner
// sums its coordinate of the component gradients in component order: the
// same operations per coordinate as dopri5_step_f64, with two barriers per
// stage.  A lane whose particle is not yet released steps with h = 0 (its
// state is unchanged), so that every thread reaches every barrier.
// Compiled compositions without subhalos only.

// Component w's gradient at the stage position in xsh (time t, center cen
// or the track), into gsh[w][lane].
template <class C>
__device__ __forceinline__ void split_component(const PotDev<double>& P, double t, const double* cen,
                                                const double (*xsh)[32], double (*gsh)[32][3], int w, int lane) {
    const double x[3] = {xsh[0][lane], xsh[1][lane], xsh[2][lane]};
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
    C::template grad_only<double, double, false>(P, w, x, xs, g, nullptr, time_dep(P, t));
    gsh[w][lane][0] = g[0];
    gsh[w][lane][1] = g[1];
    gsh[w][lane][2] = g[2];
}

// One Dopri5 step (stage times from the global step dt, increments from h)
// of the coordinate pair (yp, yv) = (x_w, v_w) owned by warps w < 3.
template <class C>
__device__ __forceinline__ void split_step_f64(const PotDev<double>& P, double t, double dt, double h, double& yp,
                                               double& yv, const double (*cen)[3], double (*xsh)[32],
                                               double (*gsh)[32][3], int w, int lane) {
    const bool own = w < 3;
    double kp[6], kv[6];  // per stage: the coordinate's velocity and acceleration
    const double cs[6] = {0.0, SS_C2, SS_C3, SS_C4, SS_C5, 1.0};
#pragma unroll
    for (int s = 0; s < 6; ++s) {
        double xp = yp, xv = yv;  // warps w >= 3 own no coordinate
        if (own && s == 1) { xp = yp + h * (SS_A21 * kp[0]); xv = yv + h * (SS_A21 * kv[0]); }
        if (own && s == 2) {
            xp = yp + h * (SS_A31 * kp[0] + SS_A32 * kp[1]);
            xv = yv + h * (SS_A31 * kv[0] + SS_A32 * kv[1]);
        }
        if (own && s == 3) {
            xp = yp + h * (SS_A41 * kp[0] + SS_A42 * kp[1] + SS_A43 * kp[2]);
            xv = yv + h * (SS_A41 * kv[0] + SS_A42 * kv[1] + SS_A43 * kv[2]);
        }
        if (own && s == 4) {
            xp = yp + h * (SS_A51 * kp[0] + SS_A52 * kp[1] + SS_A53 * kp[2] + SS_A54 * kp[3]);
            xv = yv + h * (SS_A51 * kv[0] + SS_A52 * kv[1] + SS_A53 * kv[2] + SS_A54 * kv[3]);
        }
        if (own && s == 5) {
            xp = yp + h * (SS_A61 * kp[0] + SS_A62 * kp[1] + SS_A63 * kp[2] + SS_A64 * kp[3] + SS_A65 * kp[4]);
            xv = yv + h * (SS_A61 * kv[0] + SS_A62 * kv[1] + SS_A63 * kv[2] + SS_A64 * kv[3] + SS_A65 * kv[4]);
        }
        if (own) xsh[w][lane] = xp;
        __syncthreads();  // the stage position is complete
        split_component<C>(P, t + cs[s] * dt, cen ? cen[s] : nullptr, xsh, gsh, w, lane);
        __syncthreads();  // every component's gradient is in
        if (own) {
            double g = gsh[0][lane][w];
#pragma unroll
            for (int k = 1; k < C::n; ++k) g += gsh[k][lane][w];
            kp[s] = xv;
            kv[s] = -g;
        }
    }
    if (own) {
        yp = yp + h * (SS_B1 * kp[0] + SS_B3 * kp[2] + SS_B4 * kp[3] + SS_B5 * kp[4] + SS_B6 * kp[5]);
        yv = yv + h * (SS_B1 * kv[0] + SS_B3 * kv[2] + SS_B4 * kv[3] + SS_B5 * kv[4] + SS_B6 * kv[5]);
    }
}

// Block of 32 C::n threads for 32 particles; the outputs go through a
// shared copy of the state (warp 0 writes them).
template <class C>
__device__ __forceinline__ void stream_f64_split_body(const PotDev<double>& P, const StreamArgs& a) {
    static_assert(C::n >= 3, "the split form needs a warp per coordinate");
    __shared__ double xsh[3][32];
    __shared__ double gsh[C::n][32][3];
    __shared__ double ysh[6][32];
    __shared__ double ctab[6 * F64_CHUNK][3];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const bool own = w < 3;
    const int64_t p = (int64_t)blockIdx.x * 32 + lane;
    const bool valid = p < a.N;
    const int64_t q = valid ? p : a.N - 1;  // lanes past the end follow the last particle (never written)
    const int start = stream_start(a, q + a.p_off);
    const int bstart = (int)__reduce_min_sync(0xffffffffu, (unsigned)start);  // the same in every warp
    const bool tab = P.has_track;
    double yp = 0.0, yv = 0.0;
    if (own) {
        yp = a.ics[6 * q + w];
        yv = a.ics[6 * q + 3 + w];
    }
    const bool out = w == 0 && valid;
    if (a.snaps && out) {
        double y0[6];
#pragma unroll
        for (int i = 0; i < 6; ++i) y0[i] = a.ics[6 * q + i];
        for (int64_t k = 0; (k + 1) * (int64_t)a.stride <= bstart; ++k) {
            const int64_t step = (k + 1) * (int64_t)a.stride;
            write_snap<double>(a.snaps, a.snap_pitch, k, p + a.p_off, step >= start, y0);
        }
    }
    for (int n0 = bstart; n0 < a.n_steps; n0 += F64_CHUNK) {
        const int cnt = min(F64_CHUNK, a.n_steps - n0);
        if (tab) {
            __syncthreads();  // the previous chunk's table has been read
            for (int i = threadIdx.x; i < 6 * cnt; i += blockDim.x) {
                const int j = i / 6, s = i - 6 * j;
                const double t = a.t0 + (double)(n0 + j) * a.dt;
                const double c = s == 1 ? SS_C2 : s == 2 ? SS_C3 : s == 3 ? SS_C4 : SS_C5;
                track_eval(P.track, s == 0 ? t : s == 5 ? t + a.dt : t + c * a.dt, ctab[i]);
            }
            __syncthreads();
        }
        for (int j = 0; j < cnt; ++j) {
            const int n = n0 + j;
            split_step_f64<C>(P, a.t0 + (double)n * a.dt, a.dt, n >= start ? a.dt : 0.0, yp, yv,
                              tab ? &ctab[6 * j] : nullptr, xsh, gsh, w, lane);
            if (a.snaps && (n + 1) % a.stride == 0) {  // block-uniform
                if (own) {
                    ysh[w][lane] = yp;
                    ysh[3 + w][lane] = yv;
                }
                __syncthreads();
                if (out) {
                    double y[6];
#pragma unroll
                    for (int i = 0; i < 6; ++i) y[i] = ysh[i][lane];
                    write_snap<double>(a.snaps, a.snap_pitch, (n + 1) / a.stride - 1, p + a.p_off, n + 1 >= start, y);
                }
                __syncthreads();  // read before the next gather
            }
        }
    }
    if (own) {
        ysh[w][lane] = yp;
        ysh[3 + w][lane] = yv;
    }
    __syncthreads();
    if (!out) return;
    double y[6];
    bool ok = true;
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        y[i] = ysh[i][lane];
        ok = ok && isfinite(y[i]);
    }
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
// SUB: the run's subhalos — SUB_NONE, SUB_LINES (Plummer / Hernquist) or
// SUB_GRID (tabulated).  The kernels are instantiated per case, so a run
// carries only the subhalo code it uses: the six force evaluations of a
// step are inlined, and a compact step issues measurably fewer instructions.
template <class C, int SUB = SUB_LINES>
__device__ __forceinline__ void accel_f32(const PotDev<float>& P, const StreamArgs& a, const float xh[3],
                                          const float d[3], int slot, float trel, float A[3], int shb, int she) {
    const float X[3] = {xh[0] + d[0], xh[1] + d[1], xh[2] + d[2]};
    float xs[3] = {X[0], X[1], X[2]};
    if (C::uses_track(P)) {
        const float4 ch = __ldg(a.ctab + 2 * slot);
        const float4 cl = __ldg(a.ctab + 2 * slot + 1);
        xs[0] = (xh[0] - ch.x) + (d[0] - cl.x);
        xs[1] = (xh[1] - ch.y) + (d[1] - cl.y);
        xs[2] = (xh[2] - ch.z) + (d[2] - cl.z);
    }
    float g[3];
    TimeDep<float> td;  // read by rotating / frame-accelerated components only
    if (a.ttab) {
        const float4 t0 = __ldg(a.ttab + 2 * slot);
        const float4 t1 = __ldg(a.ttab + 2 * slot + 1);
        td.c = t0.x;
        td.s = t0.y;
        td.ga[0] = t0.z;
        td.ga[1] = t0.w;
        td.ga[2] = t1.x;
        td.amp = t1.y;
    }
    C::template grad<float, float, false>(P, X, xs, g, nullptr, td);
    if constexpr (SUB != SUB_NONE) {
#pragma unroll 1
    for (int j = shb; j < she; ++j) {
        float4 s0 = __ldg(a.shtab + 3 * j);
        float4 s1 = __ldg(a.shtab + 3 * j + 1);
        float4 s2 = __ldg(a.shtab + 3 * j + 2);
        float tau = trel - s2.x;
        if (!(fabsf(tau) < s2.y)) continue;
        float rel[3] = {X[0] - (s0.x + s1.x * trel), X[1] - (s0.y + s1.y * trel), X[2] - (s0.z + s1.z * trel)};
        float gp[3], dummy[3];
        if constexpr (SUB == SUB_GRID) {
            float g, gr;
            grid_subhalo_gh<float, false>(a.shg, j, rel[0] * rel[0] + rel[1] * rel[1] + rel[2] * rel[2], g, gr);
            gp[0] = g * rel[0];
            gp[1] = g * rel[1];
            gp[2] = g * rel[2];
        } else {
            subhalo_grad<float, false>(a.sh_kind, s0.w, s1.w, rel, gp, dummy);
        }
        g[0] += gp[0];
        g[1] += gp[1];
        g[2] += gp[2];
    }
    }
    A[0] = -g[0];
    A[1] = -g[1];
    A[2] = -g[2];
}

// One compensated step.  V_i = vh + d_i and sum_j a_ij = c_i, sum_i b_i = 1
// are used exactly, so only the small parts d_i and A_i - A_1 see the
// rounded tableau.
// shb, she: the subhalo rows [shb, she) of the table this particle feels
// (she < 0: all of them).
template <class C, int SUB = SUB_LINES>
__device__ __forceinline__ void step_f32k(const PotDev<float>& P, const StreamArgs& a, int n, float xh[3],
                                          float xl[3], float vh[3], float vl[3], int shb = 0, int she = -1) {
    if (she < 0) she = a.n_sh;
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
    accel_f32<C, SUB>(P, a, xh, D, s0, tn, A1, shb, she);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        d2[i] = vl[i] + h * (F_(SS_A21) * A1[i]);
        D[i] = xl[i] + h * (F_C2 * vh[i] + F_(SS_A21) * d1[i]);
    }
    accel_f32<C, SUB>(P, a, xh, D, s0 + 1, tn + F_C2 * h, A2, shb, she);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        d3[i] = vl[i] + h * (F_(SS_A31) * A1[i] + F_(SS_A32) * A2[i]);
        D[i] = xl[i] + h * (F_C3 * vh[i] + F_(SS_A31) * d1[i] + F_(SS_A32) * d2[i]);
    }
    accel_f32<C, SUB>(P, a, xh, D, s0 + 2, tn + F_C3 * h, A3, shb, she);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        d4[i] = vl[i] + h * (F_(SS_A41) * A1[i] + F_(SS_A42) * A2[i] + F_(SS_A43) * A3[i]);
        D[i] = xl[i] + h * (F_C4 * vh[i] + F_(SS_A41) * d1[i] + F_(SS_A42) * d2[i] + F_(SS_A43) * d3[i]);
    }
    accel_f32<C, SUB>(P, a, xh, D, s0 + 3, tn + F_C4 * h, A4, shb, she);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        d5[i] = vl[i] + h * (F_(SS_A51) * A1[i] + F_(SS_A52) * A2[i] + F_(SS_A53) * A3[i] + F_(SS_A54) * A4[i]);
        D[i] = xl[i] + h * (F_C5 * vh[i] + F_(SS_A51) * d1[i] + F_(SS_A52) * d2[i] + F_(SS_A53) * d3[i] +
                            F_(SS_A54) * d4[i]);
    }
    accel_f32<C, SUB>(P, a, xh, D, s0 + 4, tn + F_C5 * h, A5, shb, she);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        d6[i] = vl[i] + h * (F_(SS_A61) * A1[i] + F_(SS_A62) * A2[i] + F_(SS_A63) * A3[i] + F_(SS_A64) * A4[i] +
                             F_(SS_A65) * A5[i]);
        D[i] = xl[i] + h * (vh[i] + F_(SS_A61) * d1[i] + F_(SS_A62) * d2[i] + F_(SS_A63) * d3[i] +
                            F_(SS_A64) * d4[i] + F_(SS_A65) * d5[i]);
    }
    accel_f32<C, SUB>(P, a, xh, D, s0 + 5, tn + h, A6, shb, she);
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

// CKPT: the run records checkpoints (the adjoint's forward pass).
template <class C, int SUB, bool CKPT = false>
__global__ void __launch_bounds__(128) stream_f32k_kernel(PotDev<float> P, StreamArgs a) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = p < a.N;
    const int start = valid ? stream_start(a, p + a.p_off) : a.n_steps;
    const int wstart = (int)__reduce_min_sync(0xffffffffu, (unsigned)start);
    const int shb = a.sh_per_grp > 0 ? (int)((p + a.p_off) / a.grp) * a.sh_per_grp : 0;
    const int she = a.sh_per_grp > 0 ? shb + a.sh_per_grp : a.n_sh;
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
            write_snap<float>(a.snaps, a.snap_pitch, k, p + a.p_off, step >= start, y);
        }
    }
    int next_snap = (wstart / a.stride + 1) * a.stride;  // first snapshot step after wstart
    for (int n = wstart; n < a.n_steps; ++n) {
        if (valid && n >= start) {
            if (CKPT && (n - start) % a.ckpt_stride == 0) {
                float4* c = a.ckpt + ((int64_t)((n - start) / a.ckpt_stride) * a.N + p) * 3;
                c[0] = make_float4(xh[0], xh[1], xh[2], vh[0]);
                c[1] = make_float4(vh[1], vh[2], xl[0], xl[1]);
                c[2] = make_float4(xl[2], vl[0], vl[1], vl[2]);
            }
            step_f32k<C, SUB>(P, a, n, xh, xl, vh, vl, shb, she);
        }
        if (n + 1 == next_snap) {  // snapshot rows follow every a.stride global steps
            next_snap += a.stride;
            if (a.snaps && valid) {
                float y[6] = {xh[0], xh[1], xh[2], vh[0], vh[1], vh[2]};
                write_snap<float>(a.snaps, a.snap_pitch, (n + 1) / a.stride - 1, p + a.p_off, n + 1 >= start, y);
            }
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

}  // namespace ssg
