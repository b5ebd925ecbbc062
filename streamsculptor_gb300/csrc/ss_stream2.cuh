// ss_stream2.cuh — the FP32-compensated stream kernel with two particles per
// thread.  Lane .x of every float2 holds particle 2t, lane .y particle 2t+1,
// and every FP32 add, multiply and FMA of the step acts on both through the
// packed f32x2 instructions of sm_100 and later: one issue slot for two
// operations.  The scalar kernel spends about three quarters of its issue
// slots on FP32 adds, multiplies and FMAs; pairing them leaves the FMA pipe,
// not instruction issue, as the bound.  Reciprocal and square-root estimates
// stay per lane (the special-function unit has no packed form); their Newton
// refinements are packed.
//
// The packed instructions round each lane to nearest like their scalar
// forms, and the negated accelerations below only flip signs, which is
// exact.  The step is the compensated step of the scalar kernel (step_f32k)
// in Nystrom form (below), and the forces restore the components' masses
// (and NFW's 1 / r_s) from their FP32 rounding residuals.  Both matter at
// the 1e-7 level: in the stage-velocity form the rounded tableau biases the
// position update by about as much as the FP32 masses bias the force, and on
// the static workloads the two biases happen to cancel in part; the Nystrom
// form rounds only the combined coefficients, so the corrected masses are
// what bring its error below the scalar kernel's.
//
// Used for runs without subhalos or with analytic subhalo lines (Plummer,
// Hernquist) whose composition is compiled (Comp<...>) from the kinds below;
// the others keep the scalar kernel.
#pragma once

#include "ss_f2.cuh"
#include "ss_stream.cuh"

namespace ssg {


// F(u) = ln(1+u) - u/(1+u) for both lanes (nfw_F_over_u3 without the
// 1/u^3).  For lanes with u < 2, with s = u / (2+u) and w = s^2 (<= 1/4):
// ln(1+u) = 2 atanh(s) = 2 s sum_k w^k / (2k+1), so
//   F = s (u / (1+u) + w P(w)),  P(w) = 2 sum_k w^k / (2k+3),
// with one reciprocal R = 1 / ((2+u)(1+u)) for both s = u (1+u) R and
// u / (1+u) = u (2+u) R, and P fitted over [0, 1/4] by a polynomial of
// degree 6 (least squares in relative error; 3e-8 with its coefficients
// rounded to FP32, where the Taylor series needs degree 12; gen_nfw_poly.py
// makes and checks them).  No term cancels, so F keeps
// its relative accuracy as u -> 0 (F ~ u^2 / 2).  Lanes with u >= 2 take
// the direct difference (each branch runs only when a lane needs it).
// lanes with u >= 2: out of line, so that log1pf's registers do not count
// against the step loop's (the branch is rare on bound orbits)
static __device__ __noinline__ f2 nfw_F2_far(f2 u) {
    const f2 L = make_float2(log1pf(u.x), log1pf(u.y));
    return fma2(neg2(u), rcp2(add2(bc(1.0f), u)), L);
}

__device__ __forceinline__ f2 nfw_F2(f2 u) {
    const bool sx = u.x < 2.0f, sy = u.y < 2.0f;
    f2 F = make_float2(0.0f, 0.0f);
    if (sx || sy) {
        const f2 A = add2(bc(2.0f), u), B = add2(bc(1.0f), u);
        const f2 uR = mul2(u, rcp2(mul2(A, B)));
        const f2 s = mul2(uR, B), t = mul2(uR, A);  // u / (2+u), u / (1+u)
        const f2 w = mul2(s, s);
        f2 P = fma2(bc(0.312188774f), w, bc(0.0821260512f));
        P = fma2(P, w, bc(0.194957018f));
        P = fma2(P, w, bc(0.221027091f));
        P = fma2(P, w, bc(0.285765111f));
        P = fma2(P, w, bc(0.399999201f));
        P = fma2(P, w, bc(0.666666687f));
        F = mul2(s, fma2(w, P, t));
    }
    if (!(sx && sy)) {
        const f2 Fl = nfw_F2_far(u);
        if (!sx) F.x = Fl.x;
        if (!sy) F.y = Fl.y;
    }
    return F;
}

// Snapshot rows of the paired kernel: one warp holds 64 consecutive
// particles (particles 2l and 2l + 1 in lane l), 12 floats per lane and
// 1536 contiguous bytes per row.  Written per lane as 8-byte pieces, each
// store instruction covers a third of every 128-byte line it touches; the
// warp instead stages its row in shared memory (each lane's 48 bytes as
// three float4, conflict-free at that stride) and writes it back as three
// stores of 512 contiguous bytes, whole lines, which matters most when the
// snapshots go straight into pinned host memory.
#ifndef SS_SNAP_COALESCED
#define SS_SNAP_COALESCED 1
#endif
constexpr int F2_WARPS = 4;  // warps per block of the paired kernel (128 threads)

__device__ __forceinline__ void write_snap_warp(float4* out, float4* stage, float4 f0, float4 f1, float4 f2) {
    const int l = threadIdx.x & 31;
    stage[3 * l] = f0;
    stage[3 * l + 1] = f1;
    stage[3 * l + 2] = f2;
    __syncwarp();
#pragma unroll
    for (int j = 0; j < 3; ++j) out[32 * j + l] = stage[32 * j + l];
    __syncwarp();
}

// Snapshot row k of one warp's particles (every lane calls it; the callers
// are warp-uniform): lane l holds particles p0 = 2t and p1 = 2t + 1 (v0, v1:
// they exist; ex0, ex1: released by the row's step).  A warp of 32 full
// pairs at a 16-byte aligned address writes the row in three coalesced
// stores (write_snap_warp), any other warp per particle.
__device__ __forceinline__ void snap_row2(const StreamArgs& a, float4* stage, int64_t k, int64_t p0, int64_t p1,
                                          bool v0, bool v1, bool ex0, bool ex1, const f2 xh[3], const f2 vh[3]) {
#if SS_SNAP_COALESCED
    float* row = a.snaps + (k * a.snap_pitch + (p0 - 2 * (int64_t)(threadIdx.x & 31)) + a.p_off) * 6;
    const bool full = blockDim.x <= 32 * F2_WARPS && __all_sync(0xffffffffu, v1) &&
                      (reinterpret_cast<uintptr_t>(row) & 15) == 0;
    if (full) {
        const float q = __int_as_float(0x7fc00000);  // NaN: not yet released
        write_snap_warp(reinterpret_cast<float4*>(row), stage,
                        ex0 ? make_float4(xh[0].x, xh[1].x, xh[2].x, vh[0].x) : make_float4(q, q, q, q),
                        make_float4(ex0 ? vh[1].x : q, ex0 ? vh[2].x : q, ex1 ? xh[0].y : q, ex1 ? xh[1].y : q),
                        ex1 ? make_float4(xh[2].y, vh[0].y, vh[1].y, vh[2].y) : make_float4(q, q, q, q));
        return;
    }
#endif
    if (v0) {
        const float y0[6] = {xh[0].x, xh[1].x, xh[2].x, vh[0].x, vh[1].x, vh[2].x};
        write_snap<float>(a.snaps, a.snap_pitch, k, p0 + a.p_off, ex0, y0);
        if (v1) {
            const float y1[6] = {xh[0].y, xh[1].y, xh[2].y, vh[0].y, vh[1].y, vh[2].y};
            write_snap<float>(a.snaps, a.snap_pitch, k, p1 + a.p_off, ex1, y1);
        }
    }
}

// The same out of line, for the rows before a warp's first release (run
// once per row before the step loop, so the loop keeps its registers).
static __device__ __noinline__ void snap_row2_cold(const StreamArgs& a, float4* stage, int64_t k, int64_t p0, int64_t p1,
                                            bool v0, bool v1, bool ex0, bool ex1, const f2 xh[3], const f2 vh[3]) {
    snap_row2(a, stage, k, p0, p1, v0, v1, ex0, ex1, xh, vh);
}

// grad Phi of one component of kind KIND at x (shifted to its center), added
// to g: the FP32 forms of kind_grad without the Hessian, with the masses
// (and NFW's 1 / r_s) restored to FP64 accuracy from their stored FP32
// rounding residuals.  The triaxial halo has no free parameter slot and keeps
// its FP32 parameters.
template <int KIND>
struct PairKind {
    static constexpr bool ok = KIND == SS_NFW || KIND == SS_TRIAXIAL_NFW || KIND == SS_MIYAMOTO_NAGAI ||
                               KIND == SS_HERNQUIST || KIND == SS_PLUMMER || KIND == SS_ISOCHRONE;
};

template <int KIND>
__device__ __forceinline__ void kind_grad2(const float* q, const f2 x[3], f2 g[3]) {
    if constexpr (KIND == SS_NFW) {
        // g = G m F(u) / r^3, u = r / r_s (nfw_gh); G m and 1 / r_s carry
        // their FP32 rounding residuals (q[5], q[4])
        const f2 r2 = add2(norm2sq(x), bc(q[3]));
        const f2 inv_r = rsqrt2(r2);
        f2 u = mul2(mul2(r2, inv_r), bc(q[2]));
        u = fma2(u, bc(q[4]), u);
        f2 gg = mul2(bc(q[0]), mul2(nfw_F2(u), mul2(mul2(inv_r, inv_r), inv_r)));
        gg = fma2(gg, bc(q[5]), gg);
#pragma unroll
        for (int i = 0; i < 3; ++i) g[i] = fma2(gg, x[i], g[i]);
    } else if constexpr (KIND == SS_TRIAXIAL_NFW) {
        const f2 xi[3] = {mul2(x[0], bc(q[2])), mul2(x[1], bc(q[3])), mul2(x[2], bc(q[4]))};
        const f2 r2 = norm2sq(xi);
        const f2 inv_r = rsqrt2(r2);
        const f2 u = mul2(mul2(r2, inv_r), bc(q[5]));
        const f2 gg = mul2(bc(q[0]), mul2(nfw_F2(u), mul2(mul2(inv_r, inv_r), inv_r)));
#pragma unroll
        for (int i = 0; i < 3; ++i) g[i] = fma2(mul2(gg, xi[i]), bc(q[2 + i]), g[i]);
    } else if constexpr (KIND == SS_MIYAMOTO_NAGAI) {
        const f2 zb2 = fma2(x[2], x[2], bc(q[2]));
        const f2 izeta = rsqrt2(zb2);
        const f2 zeta = mul2(zb2, izeta);
        const f2 az = add2(zeta, bc(q[1]));
        const f2 S2 = fma2(az, az, fma2(x[1], x[1], mul2(x[0], x[0])));
        const f2 iS = rsqrt2(S2);
        f2 gm = mul2(mul2(bc(q[0]), mul2(iS, iS)), iS);
        gm = fma2(gm, bc(q[5]), gm);
        const f2 fz = mul2(az, izeta);
        g[0] = fma2(gm, x[0], g[0]);
        g[1] = fma2(gm, x[1], g[1]);
        g[2] = fma2(mul2(gm, x[2]), fz, g[2]);
    } else {
        const f2 r2 = norm2sq(x);
        f2 gg;
        if constexpr (KIND == SS_HERNQUIST) {
            const f2 r2s = add2(r2, bc(q[2]));
            const f2 inv_r = rsqrt2(r2s);
            const f2 irr = rcp2(add2(mul2(r2s, inv_r), bc(q[1])));
            gg = mul2(mul2(mul2(bc(q[0]), inv_r), irr), irr);
        } else if constexpr (KIND == SS_PLUMMER) {
            const f2 id = rsqrt2(add2(r2, bc(q[1])));
            gg = mul2(mul2(bc(q[0]), mul2(id, id)), id);
        } else {  // SS_ISOCHRONE
            const f2 s2 = add2(r2, bc(q[2]));
            const f2 inv_s = rsqrt2(s2);
            const f2 inv_as = rcp2(add2(bc(q[1]), mul2(s2, inv_s)));
            gg = mul2(mul2(mul2(bc(q[0]), inv_s), inv_as), inv_as);
        }
        gg = fma2(gg, bc(q[5]), gg);
#pragma unroll
        for (int i = 0; i < 3; ++i) g[i] = fma2(gg, x[i], g[i]);
    }
}

// The packed force of a compiled composition; ok is false when a component
// has no packed form (the run then takes the scalar kernel).
template <class C>
struct PairComp {
    static constexpr bool ok = false;
};

template <int... KCS>
struct PairComp<Comp<KCS...>> {
    static constexpr bool ok = (PairKind<(KCS & 15)>::ok && ...);
    template <int... I>
    static __device__ __forceinline__ void add(const PotDev<float>& P, const f2 x[3], const f2 xs[3], f2 g[3],
                                               std::integer_sequence<int, I...>) {
        (kind_grad2<(KCS & 15)>(P.c[I].q, (KCS >> 4) ? xs : x, g), ...);
    }
    static __device__ __forceinline__ void grad(const PotDev<float>& P, const f2 x[3], const f2 xs[3], f2 g[3]) {
        g[0] = g[1] = g[2] = make_float2(0.0f, 0.0f);
        add(P, x, xs, g, std::make_integer_sequence<int, sizeof...(KCS)>{});
    }
};

// grad Phi of the subhalo lines [shb, she) at stage time trel (time since
// global step 0), added to g: the Plummer and Hernquist forms of
// subhalo_grad.  Both lanes feel the same rows (the launch guarantees that a
// pair never straddles two streams of an ensemble), so the table loads and
// the time-window test are uniform across the pair.
__device__ __forceinline__ void subhalo_lines2(const StreamArgs& a, const f2 X[3], float trel, int shb, int she,
                                               f2 g[3]) {
#pragma unroll 1
    for (int j = shb; j < she; ++j) {
        const float4 s0 = __ldg(a.shtab + 3 * j);
        const float4 s1 = __ldg(a.shtab + 3 * j + 1);
        const float4 s2 = __ldg(a.shtab + 3 * j + 2);
        const float tau = trel - s2.x;
        if (!(fabsf(tau) < s2.y)) continue;
        const f2 rel[3] = {sub2(X[0], bc(s0.x + s1.x * trel)), sub2(X[1], bc(s0.y + s1.y * trel)),
                           sub2(X[2], bc(s0.z + s1.z * trel))};
        const f2 r2 = norm2sq(rel);
        f2 gg;
        if (a.sh_kind == SS_SH_PLUMMER) {
            // G m / (r^2 + a^2)^(3/2)
            const f2 id = rsqrt2(add2(r2, bc(s1.w * s1.w)));
            gg = mul2(mul2(bc(s0.w), mul2(id, id)), id);
        } else {
            // Hernquist: G m / (r (r + a)^2)
            const f2 r = make_float2(s_sqrt(r2.x), s_sqrt(r2.y));
            const f2 ira = rcp2(add2(r, bc(s1.w)));
            gg = mul2(mul2(mul2(bc(s0.w), rcp2(r)), ira), ira);
        }
#pragma unroll
        for (int i = 0; i < 3; ++i) g[i] = fma2(gg, rel[i], g[i]);
    }
}

// grad Phi (not the acceleration) at the stage position xh + d; see
// accel_f32 for the center-track difference.  SUB_LINES adds the subhalo
// lines [shb, she) at stage time trel.
template <class C, int SUB>
__device__ __forceinline__ void grad2_at(const PotDev<float>& P, const StreamArgs& a, const f2 xh[3], const f2 d[3],
                                         int slot, float trel, int shb, int she, f2 g[3]) {
    const f2 X[3] = {add2(xh[0], d[0]), add2(xh[1], d[1]), add2(xh[2], d[2])};
    f2 xs[3] = {X[0], X[1], X[2]};
    if (C::uses_track(P)) {
        const float4 ch = __ldg(a.ctab + 2 * slot);
        const float4 cl = __ldg(a.ctab + 2 * slot + 1);
        xs[0] = add2(sub2(xh[0], bc(ch.x)), sub2(d[0], bc(cl.x)));
        xs[1] = add2(sub2(xh[1], bc(ch.y)), sub2(d[1], bc(cl.y)));
        xs[2] = add2(sub2(xh[2], bc(ch.z)), sub2(d[2], bc(cl.z)));
    }
    PairComp<C>::grad(P, X, xs, g);
    if constexpr (SUB == SUB_LINES) subhalo_lines2(a, X, trel, shb, she, g);
}

__device__ __forceinline__ void two_sum2(f2 a, f2 b, f2& s, f2& e) {
    s = add2(a, b);
    const f2 bb = sub2(s, a);
    e = add2(sub2(a, sub2(s, bb)), sub2(b, bb));
}

// Nystrom form of the Dormand-Prince stages.  With V_j = v + h sum_k a_jk A_k
// the stage positions x + h sum_j a_sj V_j are x + c_s h v + h^2 sum_k
// abar_sk A_k, abar = a a, and the 5th-order position update is
// x + h v + h^2 sum_k bbar_k A_k, bbar = b a (SS_N.., ss_common.cuh): the
// same numbers without the stage velocities, so a step keeps five fewer
// vectors and does a third less stage arithmetic.

// One compensated step of both lanes: the arithmetic of step_f32k in
// Nystrom form.  H, HLO: each lane's step (hi, lo); a lane whose particle is
// not yet released gets 0, which leaves its normalised state unchanged.
// G_i = grad Phi = -A_i, NH = -H.  The stage position offset from xh is
// D_s = xl + h (c_s vh + T_s), T_s = c_s vl + h sum_k abar_sk A_k (small).
// SUB_LINES: the pair feels the subhalo rows [shb, she) at the stage times
// of step_f32k.
template <class C, int SUB>
__device__ __forceinline__ void step2_f32k(const PotDev<float>& P, const StreamArgs& a, int n, f2 H, f2 HLO,
                                           f2 xh[3], f2 xl[3], f2 vh[3], f2 vl[3], int shb, int she) {
    const f2 NH = neg2(H);
    const int s0 = 5 * n;
    const float h = a.h_hi;
    const float tn = (float)n * h;  // time since global step 0 (subhalo lines)
    f2 G1[3], G2[3], G3[3], G4[3], G[3], D[3];
    f2 Sv[3], Sb[3];  // sum_{i>=3} b_i (G_i - G1) and sum_k bbar_k G_k
    grad2_at<C, SUB>(P, a, xh, xl, s0, tn, shb, she, G1);
#pragma unroll
    for (int i = 0; i < 3; ++i) D[i] = fma2(H, fma2(bc(F_C2), vh[i], mul2(bc(F_C2), vl[i])), xl[i]);
    grad2_at<C, SUB>(P, a, xh, D, s0 + 1, tn + F_C2 * h, shb, she, G2);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const f2 T = fma2(NH, mul2(bc(F_(SS_N31)), G1[i]), mul2(bc(F_C3), vl[i]));
        D[i] = fma2(H, fma2(bc(F_C3), vh[i], T), xl[i]);
    }
    grad2_at<C, SUB>(P, a, xh, D, s0 + 2, tn + F_C3 * h, shb, she, G3);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        Sv[i] = mul2(bc(F_(SS_B3)), sub2(G3[i], G1[i]));
        const f2 S = fma2(bc(F_(SS_N42)), G2[i], mul2(bc(F_(SS_N41)), G1[i]));
        const f2 T = fma2(NH, S, mul2(bc(F_C4), vl[i]));
        D[i] = fma2(H, fma2(bc(F_C4), vh[i], T), xl[i]);
    }
    grad2_at<C, SUB>(P, a, xh, D, s0 + 3, tn + F_C4 * h, shb, she, G4);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        Sv[i] = fma2(bc(F_(SS_B4)), sub2(G4[i], G1[i]), Sv[i]);
        const f2 S = fma2(bc(F_(SS_N53)), G3[i], fma2(bc(F_(SS_N52)), G2[i], mul2(bc(F_(SS_N51)), G1[i])));
        const f2 T = fma2(NH, S, mul2(bc(F_C5), vl[i]));
        D[i] = fma2(H, fma2(bc(F_C5), vh[i], T), xl[i]);
    }
    grad2_at<C, SUB>(P, a, xh, D, s0 + 4, tn + F_C5 * h, shb, she, G);  // G5
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        Sv[i] = fma2(bc(F_(SS_B5)), sub2(G[i], G1[i]), Sv[i]);
        Sb[i] = fma2(bc(F_(SS_NB5)), G[i],
                     fma2(bc(F_(SS_NB4)), G4[i],
                          fma2(bc(F_(SS_NB3)), G3[i], fma2(bc(F_(SS_NB2)), G2[i], mul2(bc(F_(SS_NB1)), G1[i])))));
        const f2 S = fma2(bc(F_(SS_N64)), G4[i],
                          fma2(bc(F_(SS_N63)), G3[i], fma2(bc(F_(SS_N62)), G2[i], mul2(bc(F_(SS_N61)), G1[i]))));
        const f2 T = fma2(NH, S, vl[i]);  // c_6 = 1
        D[i] = fma2(H, add2(vh[i], T), xl[i]);
    }
    grad2_at<C, SUB>(P, a, xh, D, s0 + 5, tn + h, shb, she, G);  // G6
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        // position: h (vh + Db), Db = vl + h sum_k bbar_k A_k
        const f2 Db = fma2(NH, Sb[i], vl[i]);
        const f2 pp = mul2(H, vh[i]);
        const f2 pen = fma2(NH, vh[i], pp);  // minus the rounding error of h vh
        const f2 lo = sub2(fma2(H, Db, mul2(HLO, vh[i])), pen);
        f2 s, e;
        two_sum2(xh[i], pp, s, e);
        f2 l2 = add2(xl[i], add2(e, lo));
        xh[i] = add2(s, l2);
        xl[i] = sub2(l2, sub2(xh[i], s));
        // velocity: -h (G1 + sum_{i>=3} b_i (G_i - G1)) = h (A1 + ...)
        const f2 Sg = add2(G1[i], fma2(bc(F_(SS_B6)), sub2(G[i], G1[i]), Sv[i]));
        const f2 qp = mul2(NH, Sg);
        const f2 qen = fma2(HLO, Sg, fma2(H, Sg, qp));  // minus the low part of h Sv
        two_sum2(vh[i], qp, s, e);
        l2 = add2(vl[i], sub2(e, qen));
        vh[i] = add2(s, l2);
        vl[i] = sub2(l2, sub2(vh[i], s));
    }
}

// SUB: SUB_NONE or SUB_LINES (analytic subhalo lines).  With subhalo rows
// per stream (ensembles), the launch takes this kernel only when a pair
// never straddles two streams: an even stream length and an even first
// particle.
template <class C, int SUB = SUB_NONE>
__global__ void __launch_bounds__(128, 4) stream_f32k2_kernel(PotDev<float> P, StreamArgs a) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t p0 = 2 * t, p1 = 2 * t + 1;
    const bool v0 = p0 < a.N, v1 = p1 < a.N;
    // subhalo rows of lane x's stream (lane y's is the same); read only by
    // threads whose lane x is a particle
    const int shb = a.sh_per_grp > 0 ? (int)((p0 + a.p_off) / a.grp) * a.sh_per_grp : 0;
    const int she = a.sh_per_grp > 0 ? shb + a.sh_per_grp : a.n_sh;
    const int st0 = v0 ? stream_start(a, p0 + a.p_off) : a.n_steps;
    const int st1 = v1 ? stream_start(a, p1 + a.p_off) : a.n_steps;
    const int tstart = st0 < st1 ? st0 : st1;
    const int wstart = (int)__reduce_min_sync(0xffffffffu, (unsigned)tstart);
    f2 xh[3], xl[3], vh[3], vl[3];
    {
        // lane y of a thread past the end repeats lane x (it never steps)
        const int64_t q0 = v0 ? p0 : 0, q1 = v1 ? p1 : q0;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            const double x0 = v0 ? a.ics[6 * q0 + i] : 0.0, x1 = v0 ? a.ics[6 * q1 + i] : 0.0;
            const double u0 = v0 ? a.ics[6 * q0 + 3 + i] : 0.0, u1 = v0 ? a.ics[6 * q1 + 3 + i] : 0.0;
            xh[i] = make_float2((float)x0, (float)x1);
            xl[i] = make_float2((float)(x0 - (double)xh[i].x), (float)(x1 - (double)xh[i].y));
            vh[i] = make_float2((float)u0, (float)u1);
            vl[i] = make_float2((float)(u0 - (double)vh[i].x), (float)(u1 - (double)vh[i].y));
        }
    }
    __shared__ float4 snap_stage[F2_WARPS][96];  // one 1536-byte snapshot row per warp
    // the rows before the warp's first release (NaN, or the initial state at
    // a particle's own release step)
    if (a.snaps) {
        for (int64_t k = 0; (k + 1) * (int64_t)a.stride <= wstart; ++k) {
            const int64_t step = (k + 1) * (int64_t)a.stride;
            snap_row2_cold(a, snap_stage[threadIdx.x >> 5], k, p0, p1, v0, v1, step >= st0, step >= st1, xh, vh);
        }
    }
    int next_snap = (wstart / a.stride + 1) * a.stride;
    for (int n = wstart; n < a.n_steps; ++n) {
        if (v0 && n >= tstart) {
            const f2 H = make_float2(n >= st0 ? a.h_hi : 0.0f, n >= st1 ? a.h_hi : 0.0f);
            const f2 HLO = make_float2(n >= st0 ? a.h_lo : 0.0f, n >= st1 ? a.h_lo : 0.0f);
            step2_f32k<C, SUB>(P, a, n, H, HLO, xh, xl, vh, vl, shb, she);
        }
        if (n + 1 == next_snap) {  // warp-uniform: every lane steps from wstart
            next_snap += a.stride;
            if (a.snaps)
                snap_row2(a, snap_stage[threadIdx.x >> 5], (n + 1) / a.stride - 1, p0, p1, v0, v1, n + 1 >= st0,
                          n + 1 >= st1, xh, vh);
        }
    }
    if (!v0) return;
#pragma unroll
    for (int lane = 0; lane < 2; ++lane) {
        if (lane == 1 && !v1) break;
        const int64_t p = lane ? p1 : p0;
        float X[3], XL[3], V[3], VL[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            X[i] = lane ? xh[i].y : xh[i].x;
            XL[i] = lane ? xl[i].y : xl[i].x;
            V[i] = lane ? vh[i].y : vh[i].x;
            VL[i] = lane ? vl[i].y : vl[i].x;
        }
        bool ok = true;
#pragma unroll
        for (int i = 0; i < 3; ++i) ok = ok && isfinite(X[i]) && isfinite(V[i]) && isfinite(XL[i]) && isfinite(VL[i]);
        if (a.status) a.status[p] = ok ? 0 : 1;
        if (a.final_w) {
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                a.final_w[6 * p + i] = (double)X[i] + (double)XL[i];
                a.final_w[6 * p + 3 + i] = (double)V[i] + (double)VL[i];
            }
        }
    }
}

// Launches stream_f32k2_kernel<C, SUB_LINES> (instantiated in
// ss_stream2.cu, a translation unit of its own so that it compiles in
// parallel with the other stream kernels).
template <class C>
void launch_f32k2_lines(const PotDev<float>& P, const StreamArgs& a, unsigned grid, int block, cudaStream_t s);

}  // namespace ssg
