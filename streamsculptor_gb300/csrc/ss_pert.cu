// ss_pert.cu — response of stream tracks to many subhalos.
//
// Reference: MassRadiusPerturbation_OTF.term (fields.py:174-206) integrated
// per particle by GenerateMassRadiusPerturbation.compute_perturbation_OTF
// (perturbative.py:100-135).  The reference's state per particle is the
// pytree [x0v0 (6), (N_sh, 12)]; every stage evaluates the base force, the
// tidal tensor T = -Hessian(Phi_base)(x0) and, per subhalo s,
//   d/dt (x1, v1)   = (v1,  -grad Phi_s(x0)        + T x1)
//   d/dt (x1r, v1r) = (v1r, -grad dPhi_s/da_s(x0)  + T x1r)
// With 18 columns the second-order mass response of
// MassRadiusPerturbation_OTF_SecondOrder (fields.py:260-320) follows:
//   d/dt (x2, v2)   = (v2,  T x2 + x1^T (d2a/dx2) x1 - Hessian(Phi_s) x1),
// which needs the third derivatives of Phi_base on the base track.
//
// The base track does not depend on the subhalos, so it is computed once per
// particle instead of once per (particle, subhalo):
//   phase 1  one thread per particle integrates x0v0 in FP64 with the same
//            Dopri5 steps and writes, for every step, the six stage
//            positions x0 and tidal tensors T (a 56-value record) to the
//            caller's workspace;
//   phase 2  one thread per (particle, subhalo) system integrates the linear
//            response with the identical tableau, reading the particle's
//            records (all threads of a block share a particle, so the reads
//            are broadcasts).
// Integrating the coupled system and integrating the base first give the
// same stage values: the base stages never read the response.
// Particles are processed in chunks whose records fit the workspace.

#include <cuda_runtime.h>

#include <cmath>

#include "ss_common.cuh"
#include "ss_f2.cuh"
#include "ss_pert.cuh"

namespace ssg {

// ------------------------------------------------------------- phase 2
// derivative of one ncol-state at a stage: K = (v1, a1 + T x1 [, v1r, a1r + T x1r])
// one stage record (x0[3], T[6]) from the 16-byte aligned shared-memory copy
__device__ __forceinline__ void load_stage(const float* p, float r[9]) {
    const float4 a = *reinterpret_cast<const float4*>(p);
    const float4 b = *reinterpret_cast<const float4*>(p + 4);
    r[0] = a.x; r[1] = a.y; r[2] = a.z; r[3] = a.w;
    r[4] = b.x; r[5] = b.y; r[6] = b.z; r[7] = b.w;
    r[8] = p[8];
}
__device__ __forceinline__ void load_stage(const double* p, double r[9]) {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const double2 v = *reinterpret_cast<const double2*>(p + 2 * i);
        r[2 * i] = v.x;
        r[2 * i + 1] = v.y;
    }
    r[8] = p[8];
}

// Hessian of one subhalo's potential at rel (xx yy zz xy xz yz)
template <class R>
__device__ __forceinline__ void subhalo_hess(int kind, R Gm, R a, const R rel[3], R Hs[6]) {
    const R r2 = rel[0] * rel[0] + rel[1] * rel[1] + rel[2] * rel[2];
    R g, gr;  // grad = g rel, H = g I + gr rel rel^T
    if (kind == SS_SH_PLUMMER) {
        const R id = s_rsqrt(r2 + a * a);
        const R id2 = id * id, id3 = id2 * id;
        g = Gm * id3;
        gr = R(-3) * Gm * id3 * id2;
    } else {
        const R r = s_sqrt(r2);
        const R ir = s_rcp(r), ira = s_rcp(r + a);
        g = Gm * ir * ira * ira;
        gr = -Gm * (R(3) * r + a) * ir * ir * ir * ira * ira * ira;
    }
    Hs[0] = g + gr * rel[0] * rel[0];
    Hs[1] = g + gr * rel[1] * rel[1];
    Hs[2] = g + gr * rel[2] * rel[2];
    Hs[3] = gr * rel[0] * rel[1];
    Hs[4] = gr * rel[0] * rel[2];
    Hs[5] = gr * rel[1] * rel[2];
}

// SHK: the subhalo kind, known at compile time (SS_SH_PLUMMER,
// SS_SH_HERNQUIST, or SS_SH_GRID for tabulated subhalos, mass response
// only); the kernels are instantiated per kind so each carries only the
// subhalo code it uses.
template <class R, int NCOL, int SHK>
__device__ __forceinline__ void pert_rhs(const R* recp, const R U[NCOL], int, R Gm, R a, const R P0[3],
                                         const R V[3], R trel, R tau0, R window, R K[NCOL], const ShDev& sh, int sidx) {
    R rec[9];
    load_stage(recp, rec);
    R rel[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) rel[i] = rec[i] - (P0[i] + V[i] * trel);
    R gphi[3], gdphi[3];
    R gg = R(0), ggr = R(0);  // SS_SH_GRID: grad = gg rel, Hessian = gg I + ggr rel rel^T
    if constexpr (SHK == SS_SH_GRID) {
        grid_subhalo_gh<R, NCOL == 18>(sh, sidx, rel[0] * rel[0] + rel[1] * rel[1] + rel[2] * rel[2], gg, ggr);
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            gphi[i] = gg * rel[i];
            gdphi[i] = R(0);
        }
    } else {
        subhalo_grad<R, NCOL >= 12>(SHK, Gm, a, rel, gphi, gdphi);
    }
    // window: |t - t0_s| < t_window
    R on = fabs(trel - tau0) < window ? R(1) : R(0);
    const R* T = rec + 3;
    if constexpr (NCOL == 18) {
        // second order in the subhalo mass (fields.py:260-320):
        //   d(x2)/dt = v2,  d(v2)/dt = T x2 + x1^T (d2a/dx2) x1 - H_s x1
        const R* D = recp + 9;  // d2a: xxx xxy xxz xyy xyz xzz yyy yyz yzz zzz
        const R* x1 = U;
        const R* x2 = U + 12;
        R Hs[6];
        if constexpr (SHK == SS_SH_GRID) {
            Hs[0] = gg + ggr * rel[0] * rel[0];
            Hs[1] = gg + ggr * rel[1] * rel[1];
            Hs[2] = gg + ggr * rel[2] * rel[2];
            Hs[3] = ggr * rel[0] * rel[1];
            Hs[4] = ggr * rel[0] * rel[2];
            Hs[5] = ggr * rel[1] * rel[2];
        } else {
            subhalo_hess<R>(SHK, Gm, a, rel, Hs);
        }
        const R x0s = x1[0] * x1[0], x1s = x1[1] * x1[1], x2s = x1[2] * x1[2];
        const R x01 = x1[0] * x1[1], x02 = x1[0] * x1[2], x12 = x1[1] * x1[2];
        // Q_i = sum_jk d2a_ijk x1_j x1_k with d2a symmetric
        const R Qx = D[0] * x0s + D[3] * x1s + D[5] * x2s + R(2) * (D[1] * x01 + D[2] * x02 + D[4] * x12);
        const R Qy = D[1] * x0s + D[6] * x1s + D[8] * x2s + R(2) * (D[3] * x01 + D[4] * x02 + D[7] * x12);
        const R Qz = D[2] * x0s + D[7] * x1s + D[9] * x2s + R(2) * (D[4] * x01 + D[5] * x02 + D[8] * x12);
        K[12] = U[15];
        K[13] = U[16];
        K[14] = U[17];
        K[15] = Qx + (T[0] * x2[0] + T[3] * x2[1] + T[4] * x2[2]) - on * (Hs[0] * x1[0] + Hs[3] * x1[1] + Hs[4] * x1[2]);
        K[16] = Qy + (T[3] * x2[0] + T[1] * x2[1] + T[5] * x2[2]) - on * (Hs[3] * x1[0] + Hs[1] * x1[1] + Hs[5] * x1[2]);
        K[17] = Qz + (T[4] * x2[0] + T[5] * x2[1] + T[2] * x2[2]) - on * (Hs[4] * x1[0] + Hs[5] * x1[1] + Hs[2] * x1[2]);
    }
    // T: xx yy zz xy xz yz
#pragma unroll
    for (int b = 0; b < (NCOL == 18 ? 2 : NCOL / 6); ++b) {
        const R* x1 = U + 6 * b;
        K[6 * b + 0] = U[6 * b + 3];
        K[6 * b + 1] = U[6 * b + 4];
        K[6 * b + 2] = U[6 * b + 5];
        const R* gs = b == 0 ? gphi : gdphi;
        K[6 * b + 3] = -on * gs[0] + (T[0] * x1[0] + T[3] * x1[1] + T[4] * x1[2]);
        K[6 * b + 4] = -on * gs[1] + (T[3] * x1[0] + T[1] * x1[1] + T[5] * x1[2]);
        K[6 * b + 5] = -on * gs[2] + (T[4] * x1[0] + T[5] * x1[1] + T[2] * x1[2]);
    }
}

// The block's threads share one particle, so its base-track records are
// staged in shared memory PERT_STEPS_STAGED steps at a time (coalesced global loads,
// stage records padded to 12 values for vector loads); threads past the last
// subhalo run on subhalo 0 and discard their result so that every thread
// reaches the block barriers.
static constexpr int PERT_STEPS_STAGED = 16;

template <class R, int NCOL, int SHK>
__global__ void __launch_bounds__(128) pert_response_kernel(ShDev sh, PertArgs a, int sblocks) {
    constexpr int ORD = NCOL == 18 ? 2 : 1;
    constexpr int RL = rec_len(ORD), SL = stage_len(ORD), SW = ORD == 2 ? 20 : 12;
    __shared__ __align__(16) R srec[PERT_STEPS_STAGED][6][SW];
    const int64_t i = blockIdx.x / sblocks;          // particle within the chunk
    const int sb = blockIdx.x - (int)(i * sblocks);
    const int s_raw = sb * blockDim.x + threadIdx.x;  // subhalo
    if (i >= a.np) return;                           // whole block
    const bool active = s_raw < sh.n;
    const int s = active ? s_raw : 0;
    const int64_t p = a.p0 + i;
    const int start = (int)pert_start(p, a.ppr, a.spr);
    const R* rec = reinterpret_cast<const R*>(a.table) +
                   (pert_offset(p, a.ppr, a.spr, a.n_steps) - pert_offset(a.p0, a.ppr, a.spr, a.n_steps)) * RL;
    // subhalo line relative to the run start t0: P0 + V (t - t0)
    const double tau = a.t0 - sh.t0[s];
    const R P0[3] = {(R)(sh.x0[3 * s] + sh.v[3 * s] * tau), (R)(sh.x0[3 * s + 1] + sh.v[3 * s + 1] * tau),
                     (R)(sh.x0[3 * s + 2] + sh.v[3 * s + 2] * tau)};
    const R V[3] = {(R)sh.v[3 * s], (R)sh.v[3 * s + 1], (R)sh.v[3 * s + 2]};
    const R Gm = (R)(sh.G * sh.m[s]);
    const R am = (R)sh.a[s];
    const R tau0 = (R)(sh.t0[s] - a.t0);
    const R window = (R)sh.t_window;
    const int64_t nsh = sh.n;

    R u[NCOL];
    const R* ic = reinterpret_cast<const R*>(a.pert_ics);
#pragma unroll
    for (int c = 0; c < NCOL; ++c) u[c] = ic ? ic[(p * nsh + s) * NCOL + c] : R(0);
    R* out = reinterpret_cast<R*>(a.pert_out);
    auto save = [&](int slot) {
        if (!active) return;
        R* o = out + (((int64_t)slot * a.N + p) * nsh + s) * NCOL;
#pragma unroll
        for (int c = 0; c < NCOL; ++c) o[c] = u[c];
    };
    if (a.save_stride > 0) {
        for (int k = 0; k < a.n_saves && (int64_t)k * a.save_stride <= start; ++k) save(k);
    }
    const R h = (R)a.dt;
    const R cs[6] = {R(0), R(SS_C2), R(SS_C3), R(SS_C4), R(SS_C5), R(1)};
    for (int n0 = start; n0 < a.n_steps; n0 += PERT_STEPS_STAGED, rec += PERT_STEPS_STAGED * RL) {
      const int cnt = min(PERT_STEPS_STAGED, a.n_steps - n0);
      __syncthreads();  // the previous chunk has been consumed
      for (int e = threadIdx.x; e < cnt * 6 * SL; e += blockDim.x) {
          const int j = e / (6 * SL), r = e - 6 * SL * j, st = r / SL, q = r - SL * st;
          srec[j][st][q] = rec[(int64_t)j * RL + r];
      }
      __syncthreads();
      for (int j = 0; j < cnt; ++j) {
        const int n = n0 + j;
        const R tn = (R)n * h;
        R k[6][NCOL];
        R U[NCOL];
#pragma unroll
        for (int st = 0; st < 6; ++st) {
#pragma unroll
            for (int c = 0; c < NCOL; ++c) {
                R acc = R(0);
                if (st == 1) acc = R(SS_A21) * k[0][c];
                if (st == 2) acc = R(SS_A31) * k[0][c] + R(SS_A32) * k[1][c];
                if (st == 3) acc = R(SS_A41) * k[0][c] + R(SS_A42) * k[1][c] + R(SS_A43) * k[2][c];
                if (st == 4) acc = R(SS_A51) * k[0][c] + R(SS_A52) * k[1][c] + R(SS_A53) * k[2][c] + R(SS_A54) * k[3][c];
                if (st == 5)
                    acc = R(SS_A61) * k[0][c] + R(SS_A62) * k[1][c] + R(SS_A63) * k[2][c] + R(SS_A64) * k[3][c] +
                          R(SS_A65) * k[4][c];
                U[c] = st == 0 ? u[c] : u[c] + h * acc;
            }
            pert_rhs<R, NCOL, SHK>(&srec[j][st][0], U, sh.kind, Gm, am, P0, V, tn + cs[st] * h, tau0, window, k[st],
                                   sh, s);
        }
#pragma unroll
        for (int c = 0; c < NCOL; ++c)
            u[c] = u[c] + h * (R(SS_B1) * k[0][c] + R(SS_B3) * k[2][c] + R(SS_B4) * k[3][c] + R(SS_B5) * k[4][c] +
                               R(SS_B6) * k[5][c]);
        if (a.save_stride > 0 && (n + 1) % a.save_stride == 0) save((n + 1) / a.save_stride);
      }
    }
    if (a.save_stride == 0) save(0);
}

// The FP32 response with two subhalos per thread (s0 = 2q, s1 = 2q + 1 of
// the block's 256) in packed f32x2 lanes, for Plummer and Hernquist subhalo
// lines (ncol 6 and 12), in Nystrom form.  Each response column block is a
// second-order system x1'' = T(t) x1 - grad(Phi_s or dPhi_s/da_s)(x0(t))
// (the acceleration does not depend on v1), so the Dormand-Prince stages
// need only each stage's acceleration: stage positions
// x1 + c_s h v1 + h^2 sum_k abar_sk A_k, and the update x1 + h v1 +
// h^2 sum_k bbar_k A_k, v1 + h sum_k b_k A_k — the same step as
// pert_response_kernel's first-order form with half the stage storage and a
// third less stage arithmetic.  Each add, multiply and FMA is one packed
// instruction for both systems, and each base-track record is read from
// shared memory once for the pair.
template <int NB, int SHK>
__device__ __forceinline__ void pert_acc2(const float* recp, const f2 X[NB][3], f2 Gm, f2 am, const f2 P0[3],
                                          const f2 V[3], float trel, f2 tau0, float window, f2 A[NB][3]) {
    float rec[9];
    load_stage(recp, rec);
    const f2 tr = bc(trel);
    f2 rel[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) rel[i] = sub2(bc(rec[i]), fma2(V[i], tr, P0[i]));
    const f2 r2 = norm2sq(rel);
    f2 g, gs = bc(0.0f);
    if constexpr (SHK == SS_SH_PLUMMER) {
        const f2 id = rsqrt2(fma2(am, am, r2));
        const f2 id2 = mul2(id, id);
        g = mul2(Gm, mul2(id2, id));
        if constexpr (NB == 2) gs = mul2(mul2(bc(-3.0f), mul2(g, am)), id2);  // grad(Gm a D^-3) = -3 Gm a D^-5 rel
    } else {
        const f2 r = make_float2(s_sqrt(r2.x), s_sqrt(r2.y));
        const f2 inv_r = rcp2(r);
        const f2 inv_ra = rcp2(add2(r, am));
        g = mul2(mul2(mul2(Gm, inv_r), inv_ra), inv_ra);
        if constexpr (NB == 2) gs = mul2(mul2(bc(-2.0f), g), inv_ra);  // grad(Gm (r+a)^-2)
    }
    // window: |t - t0_s| < t_window, per lane
    const f2 on = make_float2(fabsf(trel - tau0.x) < window ? 1.0f : 0.0f, fabsf(trel - tau0.y) < window ? 1.0f : 0.0f);
    // T: xx yy zz xy xz yz
    const f2 T0 = bc(rec[3]), T1 = bc(rec[4]), T2 = bc(rec[5]), T3 = bc(rec[6]), T4 = bc(rec[7]), T5 = bc(rec[8]);
#pragma unroll
    for (int b = 0; b < NB; ++b) {
        const f2 ng = neg2(mul2(on, b == 0 ? g : gs));
        A[b][0] = fma2(ng, rel[0], fma2(T4, X[b][2], fma2(T3, X[b][1], mul2(T0, X[b][0]))));
        A[b][1] = fma2(ng, rel[1], fma2(T5, X[b][2], fma2(T1, X[b][1], mul2(T3, X[b][0]))));
        A[b][2] = fma2(ng, rel[2], fma2(T2, X[b][2], fma2(T5, X[b][1], mul2(T4, X[b][0]))));
    }
}

// Mass columns only (ncol 6): 5 blocks of 128 per SM (96 registers: no
// spills for Plummer subhalos, 16 bytes for Hernquist; 1 % faster than the
// unbounded 116 registers on the Plummer workload).
template <int NCOL, int SHK>
__global__ void __launch_bounds__(128, NCOL == 6 ? 5 : 1) pert_response2_kernel(ShDev sh, PertArgs a, int sblocks) {
    constexpr int RL = rec_len(1), SL = stage_len(1), SW = 12, NB = NCOL / 6;
    __shared__ __align__(16) float srec[PERT_STEPS_STAGED][6][SW];
    const int64_t i = blockIdx.x / sblocks;          // particle within the chunk
    const int sb = blockIdx.x - (int)(i * sblocks);
    const int64_t q = (int64_t)sb * blockDim.x + threadIdx.x;  // subhalo pair
    if (i >= a.np) return;                           // whole block
    const bool act0 = 2 * q < sh.n, act1 = 2 * q + 1 < sh.n;
    const int s0 = act0 ? (int)(2 * q) : 0, s1 = act1 ? (int)(2 * q + 1) : s0;
    const int64_t p = a.p0 + i;
    const int start = (int)pert_start(p, a.ppr, a.spr);
    const float* rec = reinterpret_cast<const float*>(a.table) +
                       (pert_offset(p, a.ppr, a.spr, a.n_steps) - pert_offset(a.p0, a.ppr, a.spr, a.n_steps)) * RL;
    // subhalo lines relative to the run start t0: P0 + V (t - t0)
    const double tau_0 = a.t0 - sh.t0[s0], tau_1 = a.t0 - sh.t0[s1];
    f2 P0[3], V[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        P0[d] = make_float2((float)(sh.x0[3 * s0 + d] + sh.v[3 * s0 + d] * tau_0),
                            (float)(sh.x0[3 * s1 + d] + sh.v[3 * s1 + d] * tau_1));
        V[d] = make_float2((float)sh.v[3 * s0 + d], (float)sh.v[3 * s1 + d]);
    }
    const f2 Gm = make_float2((float)(sh.G * sh.m[s0]), (float)(sh.G * sh.m[s1]));
    const f2 am = make_float2((float)sh.a[s0], (float)sh.a[s1]);
    const f2 tau0 = make_float2((float)(sh.t0[s0] - a.t0), (float)(sh.t0[s1] - a.t0));
    const float window = (float)sh.t_window;
    const int64_t nsh = sh.n;

    f2 u[NCOL];
    const float* ic = reinterpret_cast<const float*>(a.pert_ics);
#pragma unroll
    for (int c = 0; c < NCOL; ++c)
        u[c] = ic ? make_float2(ic[(p * nsh + s0) * NCOL + c], ic[(p * nsh + s1) * NCOL + c]) : bc(0.0f);
    float* out = reinterpret_cast<float*>(a.pert_out);
    auto save = [&](int slot) {
        float* o = out + (((int64_t)slot * a.N + p) * nsh + s0) * NCOL;  // s1 = s0 + 1 follows
        if (act0) {
#pragma unroll
            for (int c = 0; c < NCOL; ++c) o[c] = u[c].x;
        }
        if (act1) {
#pragma unroll
            for (int c = 0; c < NCOL; ++c) o[NCOL + c] = u[c].y;
        }
    };
    if (a.save_stride > 0) {
        for (int k = 0; k < a.n_saves && (int64_t)k * a.save_stride <= start; ++k) save(k);
    }
    const float h = (float)a.dt;
    const f2 H = bc(h);
    const float cs[6] = {0.0f, (float)SS_C2, (float)SS_C3, (float)SS_C4, (float)SS_C5, 1.0f};
    for (int n0 = start; n0 < a.n_steps; n0 += PERT_STEPS_STAGED, rec += PERT_STEPS_STAGED * RL) {
        const int cnt = min(PERT_STEPS_STAGED, a.n_steps - n0);
        __syncthreads();  // the previous chunk has been consumed
        for (int e = threadIdx.x; e < cnt * 6 * SL; e += blockDim.x) {
            const int j = e / (6 * SL), r = e - 6 * SL * j, st = r / SL, qq = r - SL * st;
            srec[j][st][qq] = rec[(int64_t)j * RL + r];
        }
        __syncthreads();
        for (int j = 0; j < cnt; ++j) {
            const int n = n0 + j;
            const float tn = (float)n * h;
            f2 A[6][NB][3];  // stage accelerations of each column block
#pragma unroll
            for (int st = 0; st < 6; ++st) {
                f2 X[NB][3];
#pragma unroll
                for (int bl = 0; bl < NB; ++bl) {
#pragma unroll
                    for (int d = 0; d < 3; ++d) {
                        // h sum_k abar_sk A_k (stage 2 has none)
                        f2 acc = bc(0.0f);
                        if (st == 2) acc = mul2(bc((float)SS_N31), A[0][bl][d]);
                        if (st == 3) acc = fma2(bc((float)SS_N42), A[1][bl][d], mul2(bc((float)SS_N41), A[0][bl][d]));
                        if (st == 4)
                            acc = fma2(bc((float)SS_N53), A[2][bl][d],
                                       fma2(bc((float)SS_N52), A[1][bl][d], mul2(bc((float)SS_N51), A[0][bl][d])));
                        if (st == 5)
                            acc = fma2(bc((float)SS_N64), A[3][bl][d],
                                       fma2(bc((float)SS_N63), A[2][bl][d],
                                            fma2(bc((float)SS_N62), A[1][bl][d],
                                                 mul2(bc((float)SS_N61), A[0][bl][d]))));
                        const f2 x = u[6 * bl + d], v = u[6 * bl + 3 + d];
                        X[bl][d] = st == 0 ? x : fma2(H, fma2(bc(cs[st]), v, mul2(H, acc)), x);
                    }
                }
                pert_acc2<NB, SHK>(&srec[j][st][0], X, Gm, am, P0, V, tn + cs[st] * h, tau0, window, A[st]);
            }
#pragma unroll
            for (int bl = 0; bl < NB; ++bl) {
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    f2 sx = mul2(bc((float)SS_NB1), A[0][bl][d]);
                    sx = fma2(bc((float)SS_NB2), A[1][bl][d], sx);
                    sx = fma2(bc((float)SS_NB3), A[2][bl][d], sx);
                    sx = fma2(bc((float)SS_NB4), A[3][bl][d], sx);
                    sx = fma2(bc((float)SS_NB5), A[4][bl][d], sx);
                    f2 sv = mul2(bc((float)SS_B1), A[0][bl][d]);
                    sv = fma2(bc((float)SS_B3), A[2][bl][d], sv);
                    sv = fma2(bc((float)SS_B4), A[3][bl][d], sv);
                    sv = fma2(bc((float)SS_B5), A[4][bl][d], sv);
                    sv = fma2(bc((float)SS_B6), A[5][bl][d], sv);
                    f2& x = u[6 * bl + d];
                    f2& v = u[6 * bl + 3 + d];
                    x = fma2(H, fma2(H, sx, v), x);  // x + h (v + h sum bbar_k A_k)
                    v = fma2(H, sv, v);
                }
            }
            if (a.save_stride > 0 && (n + 1) % a.save_stride == 0) save((n + 1) / a.save_stride);
        }
    }
    if (a.save_stride == 0) save(0);
}

// Per-subhalo potentials and derivatives at points (the perturbation
// generator's jacfwd(potential_per_SH), perturbative.py:40-41).
__global__ void subhalo_eval_kernel(ShDev sh, const double* __restrict__ xyz, int64_t n, double t, double* phi,
                                    double* grad, double* dphi_da, double* grad_dphi_da) {
    int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= n * sh.n) return;
    int64_t i = idx / sh.n;
    int s = (int)(idx % sh.n);
    double tau = t - sh.t0[s];
    bool on = fabs(tau) < sh.t_window;
    double rel[3];
    for (int k = 0; k < 3; ++k) rel[k] = xyz[3 * i + k] - (sh.x0[3 * s + k] + sh.v[3 * s + k] * tau);
    double Gm = sh.G * sh.m[s], a = sh.a[s];
    double r2 = rel[0] * rel[0] + rel[1] * rel[1] + rel[2] * rel[2];
    double gphi[3], gd[3];
    double phv;
    if (sh.kind == SS_SH_GRID) {
        // tabulated profile: no scale radius, so d/da is zero
        double g, gr;
        grid_subhalo_gh<double, false>(sh, s, r2, g, gr, &phv);
        for (int k = 0; k < 3; ++k) {
            gphi[k] = g * rel[k];
            gd[k] = 0.0;
        }
    } else {
        subhalo_grad<double, true>(sh.kind, Gm, a, rel, gphi, gd);
        phv = sh.kind == SS_SH_PLUMMER ? -Gm / sqrt(r2 + a * a) : -Gm / (sqrt(r2) + a);
    }
    if (phi) phi[idx] = on ? phv : 0.0;
    if (dphi_da) {
        double v = sh.kind == SS_SH_GRID      ? 0.0
                   : sh.kind == SS_SH_PLUMMER ? Gm * a / ((r2 + a * a) * sqrt(r2 + a * a))
                                              : Gm / ((sqrt(r2) + a) * (sqrt(r2) + a));
        dphi_da[idx] = on ? v : 0.0;
    }
    for (int k = 0; k < 3; ++k) {
        if (grad) grad[3 * idx + k] = on ? gphi[k] : 0.0;
        if (grad_dphi_da) grad_dphi_da[3 * idx + k] = on ? gd[k] : 0.0;
    }
}

// The field itself at one point (MassRadiusPerturbation_OTF.term,
// fields.py:174-206, and MassRadiusPerturbation_OTF_SecondOrder.term,
// fields.py:284-320): y = [x0v0 (6), n_sh x ncol], dy the same layout.
// One thread per subhalo evaluates the stage record at x0 and the same
// pert_rhs as the response kernels; thread 0 writes the base derivative.
template <int NCOL>
__global__ void __launch_bounds__(128) pert_term_kernel(PotDev<double> P, ShDev sh, double t,
                                                        const double* __restrict__ y, double* __restrict__ dy) {
    constexpr int ORD = NCOL == 18 ? 2 : 1;
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= sh.n) return;
    __align__(16) double r[20];
    double g[3];
    base_stage<GenericComp, ORD>(P, y, t, g, r);
    if (s == 0) {
        dy[0] = y[3];
        dy[1] = y[4];
        dy[2] = y[5];
        dy[3] = -g[0];
        dy[4] = -g[1];
        dy[5] = -g[2];
    }
    // subhalo line relative to t: P0 + V (t' - t), evaluated at t' = t
    const double tau = t - sh.t0[s];
    const double P0[3] = {sh.x0[3 * s] + sh.v[3 * s] * tau, sh.x0[3 * s + 1] + sh.v[3 * s + 1] * tau,
                          sh.x0[3 * s + 2] + sh.v[3 * s + 2] * tau};
    const double V[3] = {sh.v[3 * s], sh.v[3 * s + 1], sh.v[3 * s + 2]};
    double U[NCOL], K[NCOL];
#pragma unroll
    for (int c = 0; c < NCOL; ++c) U[c] = y[6 + s * NCOL + c];
    const double Gm = sh.kind == SS_SH_GRID ? 0.0 : sh.G * sh.m[s];
    if (sh.kind == SS_SH_GRID)
        pert_rhs<double, NCOL, SS_SH_GRID>(r, U, sh.kind, Gm, sh.a[s], P0, V, 0.0, sh.t0[s] - t, sh.t_window, K, sh,
                                           (int)s);
    else if (sh.kind == SS_SH_PLUMMER)
        pert_rhs<double, NCOL, SS_SH_PLUMMER>(r, U, sh.kind, Gm, sh.a[s], P0, V, 0.0, sh.t0[s] - t, sh.t_window, K,
                                              sh, (int)s);
    else
        pert_rhs<double, NCOL, SS_SH_HERNQUIST>(r, U, sh.kind, Gm, sh.a[s], P0, V, 0.0, sh.t0[s] - t, sh.t_window, K,
                                                sh, (int)s);
#pragma unroll
    for (int c = 0; c < NCOL; ++c) dy[6 + s * NCOL + c] = K[c];
}

static int prepare_subhalos(const ss_subhalos* in, double G, ShDev* out, int ncol = 6) {
    SS_CHECK_ARG(in != nullptr, "subhalos is NULL");
    SS_CHECK_ARG(in->n >= 1 && in->n <= (1 << 30), "subhalos: n must be in [1, 2^30]");
    SS_CHECK_ARG(in->kind == SS_SH_PLUMMER || in->kind == SS_SH_HERNQUIST || in->kind == SS_SH_GRID,
                 "subhalos: unknown kind %d", in->kind);
    SS_CHECK_ARG(in->m && in->a && in->x0 && in->v && in->t0, "subhalos: NULL table pointer");
    SS_CHECK_ARG(!(in->t_window < 0.0), "subhalos: t_window < 0");
    if (in->kind == SS_SH_GRID) {
        SS_CHECK_ARG(in->grid && in->grid_u0 && in->grid_du && in->n_grid >= 2 && in->n_grid <= (1 << 20),
                     "subhalos: SS_SH_GRID needs grid tables with >= 2 knots");
        SS_CHECK_ARG(ncol == 6, "tabulated subhalos have no scale-radius response: ncol must be 6");
    }
    out->grid = in->grid;
    out->gu0 = in->grid_u0;
    out->gdu = in->grid_du;
    out->ng = (int32_t)in->n_grid;
    out->kind = in->kind;
    out->n = (int32_t)in->n;
    out->m = in->m;
    out->a = in->a;
    out->x0 = in->x0;
    out->v = in->v;
    out->t0 = in->t0;
    out->t_window = in->t_window;
    out->G = G;
    return SS_OK;
}

}  // namespace ssg

using namespace ssg;

extern "C" {

int ss_subhalo_eval(const ss_subhalos* sh, double G, const double* xyz, int64_t n, double t, double* phi,
                    double* grad, double* dphi_da, double* grad_dphi_da, void* stream) {
    ShDev S;
    int rc = prepare_subhalos(sh, G, &S);
    if (rc) return rc;
    SS_CHECK_ARG(n >= 0, "n < 0");
    if (n == 0) return SS_OK;
    SS_CHECK_ARG(xyz != nullptr, "xyz is NULL");
    int64_t total = n * S.n;
    subhalo_eval_kernel<<<(unsigned)((total + 127) / 128), 128, 0, (cudaStream_t)stream>>>(S, xyz, n, t, phi, grad,
                                                                                          dphi_da, grad_dphi_da);
    SS_LAUNCH_CHECK();
    return SS_OK;
}

int64_t ss_pert_workspace_bytes(const ss_pert_cfg* cfg, int precision, int64_t particles_per_chunk) {
    if (!cfg || (precision != 32 && precision != 64) || particles_per_chunk < 1 || cfg->n_steps < 0)
        return set_error(SS_ERR_INVALID_ARGUMENT, "bad arguments");
    // the first particles are the longest: n_steps records each
    return particles_per_chunk * cfg->n_steps * rec_len(cfg->ncol == 18 ? 2 : 1) * (precision == 64 ? 8 : 4);
}

static int pert_args(const ss_pert_cfg* cfg, int precision, PertArgs* a) {
    SS_CHECK_ARG(cfg != nullptr, "cfg is NULL");
    SS_CHECK_ARG(precision == 32 || precision == 64, "precision must be 32 or 64");
    SS_CHECK_ARG(cfg->ncol == 6 || cfg->ncol == 12 || cfg->ncol == 18, "ncol must be 6, 12 or 18");
    SS_CHECK_ARG(cfg->n_particles >= 0 && cfg->n_steps >= 0 && cfg->n_steps < (1LL << 30), "bad sizes");
    SS_CHECK_ARG(cfg->particles_per_release >= 1 && cfg->steps_per_release >= 0, "bad release layout");
    SS_CHECK_ARG(std::isfinite(cfg->dt) && cfg->dt != 0.0 && std::isfinite(cfg->t0), "dt must be finite, non-zero");
    SS_CHECK_ARG(cfg->save_stride >= 0, "save_stride < 0");
    const int64_t n_rel = (cfg->n_particles + cfg->particles_per_release - 1) / cfg->particles_per_release;
    SS_CHECK_ARG(n_rel == 0 || (n_rel - 1) * (int64_t)cfg->steps_per_release <= cfg->n_steps,
                 "last release starts after n_steps");
    memset(a, 0, sizeof(*a));
    a->N = cfg->n_particles;
    a->ppr = cfg->particles_per_release;
    a->spr = cfg->steps_per_release;
    a->n_steps = (int32_t)cfg->n_steps;
    a->ncol = cfg->ncol;
    a->save_stride = cfg->save_stride;
    a->n_saves = cfg->save_stride > 0 ? (int32_t)(cfg->n_steps / cfg->save_stride + 1) : 1;
    a->t0 = cfg->t0;
    a->dt = cfg->dt;
    return SS_OK;
}

// response kernels over [0, N) in grid-sized chunks; a.table = the records of particle 0
// response kernel for the run's precision and column count
extern "C++" {
template <class R, int SHK>
static void launch_response_kind(const ShDev& S, const PertArgs& a, unsigned g2, int sblock, int sblocks,
                                 cudaStream_t st) {
    if constexpr (SHK == SS_SH_GRID) {
        pert_response_kernel<R, 6, SHK><<<g2, sblock, 0, st>>>(S, a, sblocks);  // mass response only
    } else if (std::is_same<R, float>::value && (a.ncol == 6 || a.ncol == 12)) {
        // two subhalos per thread (packed f32x2): blocks of 128 pairs
        const int sblocks2 = (int)((S.n + 2 * sblock - 1) / (2 * sblock));
        const unsigned g = (unsigned)(a.np * sblocks2);
        if (a.ncol == 12) pert_response2_kernel<12, SHK><<<g, sblock, 0, st>>>(S, a, sblocks2);
        else pert_response2_kernel<6, SHK><<<g, sblock, 0, st>>>(S, a, sblocks2);
    } else {
        if (a.ncol == 18) pert_response_kernel<R, 18, SHK><<<g2, sblock, 0, st>>>(S, a, sblocks);
        else if (a.ncol == 12) pert_response_kernel<R, 12, SHK><<<g2, sblock, 0, st>>>(S, a, sblocks);
        else pert_response_kernel<R, 6, SHK><<<g2, sblock, 0, st>>>(S, a, sblocks);
    }
}

template <class R>
static void launch_response_r(const ShDev& S, const PertArgs& a, unsigned g2, int sblock, int sblocks,
                              cudaStream_t st) {
    if (S.kind == SS_SH_GRID) launch_response_kind<R, SS_SH_GRID>(S, a, g2, sblock, sblocks, st);
    else if (S.kind == SS_SH_PLUMMER) launch_response_kind<R, SS_SH_PLUMMER>(S, a, g2, sblock, sblocks, st);
    else launch_response_kind<R, SS_SH_HERNQUIST>(S, a, g2, sblock, sblocks, st);
}
}  // extern "C++"

static void launch_response(const ShDev& S, const PertArgs& a, int precision, unsigned g2, int sblock, int sblocks,
                            cudaStream_t st) {
    if (precision == 64) launch_response_r<double>(S, a, g2, sblock, sblocks, st);
    else launch_response_r<float>(S, a, g2, sblock, sblocks, st);
}

static int pert_response_launch(const ShDev& S, PertArgs a, int precision, cudaStream_t st) {
    const int sblock = 128;
    const int sblocks = (int)((S.n + sblock - 1) / sblock);
    const int64_t max_np = ((1LL << 31) - 1) / sblocks;
    const int64_t esz = precision == 64 ? 8 : 4;
    char* table0 = (char*)a.table;
    for (int64_t p0 = 0; p0 < a.N; p0 += max_np) {
        a.p0 = p0;
        a.np = a.N - p0 < max_np ? a.N - p0 : max_np;
        a.table = table0 + pert_offset(p0, a.ppr, a.spr, a.n_steps) * rec_len(a.ncol == 18 ? 2 : 1) * esz;
        launch_response(S, a, precision, (unsigned)(a.np * sblocks), sblock, sblocks, st);
        SS_LAUNCH_CHECK();
    }
    return SS_OK;
}

int ss_pert_response(const ss_potential* base, const ss_subhalos* sh, const ss_pert_cfg* cfg, int precision,
                     const double* base_ics, const void* pert_ics, double* base_out, void* pert_out, void* workspace,
                     int64_t workspace_bytes, void* stream) {
    PotDev<double> P;
    int rc = prepare_potential<double>(base, &P, false);
    if (rc) return rc;
    ShDev S;
    rc = prepare_subhalos(sh, base->G, &S, cfg ? cfg->ncol : 6);
    if (rc) return rc;
    SS_CHECK_ARG(cfg != nullptr, "cfg is NULL");
    SS_CHECK_ARG(precision == 32 || precision == 64, "precision must be 32 or 64");
    SS_CHECK_ARG(cfg->ncol == 6 || cfg->ncol == 12 || cfg->ncol == 18, "ncol must be 6, 12 or 18");
    SS_CHECK_ARG(cfg->n_particles >= 0 && cfg->n_steps >= 0 && cfg->n_steps < (1LL << 30), "bad sizes");
    SS_CHECK_ARG(cfg->particles_per_release >= 1 && cfg->steps_per_release >= 0, "bad release layout");
    SS_CHECK_ARG(std::isfinite(cfg->dt) && cfg->dt != 0.0 && std::isfinite(cfg->t0), "dt must be finite, non-zero");
    SS_CHECK_ARG(cfg->save_stride >= 0, "save_stride < 0");
    if (cfg->n_particles == 0) return SS_OK;
    SS_CHECK_ARG(base_ics && pert_out, "NULL buffer");
    int64_t n_rel = (cfg->n_particles + cfg->particles_per_release - 1) / cfg->particles_per_release;
    SS_CHECK_ARG((n_rel - 1) * (int64_t)cfg->steps_per_release <= cfg->n_steps, "last release starts after n_steps");
    const int64_t esz = precision == 64 ? 8 : 4;
    const int64_t rec_bytes = rec_len(cfg->ncol == 18 ? 2 : 1) * esz;
    const int64_t cap_records = workspace ? workspace_bytes / rec_bytes : 0;
    if (cfg->n_steps > 0 && cap_records < cfg->n_steps)
        return set_error(SS_ERR_WORKSPACE, "workspace of >= %lld bytes needed (one particle), %lld given",
                         (long long)(cfg->n_steps * rec_bytes), (long long)workspace_bytes);
    SS_CHECK_ARG(workspace == nullptr || ((uintptr_t)workspace % 16) == 0, "workspace must be 16-byte aligned");

    PertArgs a;
    memset(&a, 0, sizeof(a));
    a.N = cfg->n_particles;
    a.ppr = cfg->particles_per_release;
    a.spr = cfg->steps_per_release;
    a.n_steps = (int32_t)cfg->n_steps;
    a.ncol = cfg->ncol;
    a.save_stride = cfg->save_stride;
    a.n_saves = cfg->save_stride > 0 ? (int32_t)(cfg->n_steps / cfg->save_stride + 1) : 1;
    a.t0 = cfg->t0;
    a.dt = cfg->dt;
    a.base_ics = base_ics;
    a.base_out = base_out;
    a.pert_ics = pert_ics;
    a.pert_out = pert_out;
    a.table = workspace;
    cudaStream_t st = (cudaStream_t)stream;
    const int sblock = 128;
    const int sblocks = (int)((S.n + sblock - 1) / sblock);
    int64_t p0 = 0;
    while (p0 < a.N) {
        // largest chunk [p0, p1) whose records fit the workspace
        int64_t lo = p0 + 1, hi = a.N;
        const int64_t base_off = pert_offset(p0, a.ppr, a.spr, a.n_steps);
        while (lo < hi) {
            int64_t mid = (lo + hi + 1) / 2;
            if (pert_offset(mid, a.ppr, a.spr, a.n_steps) - base_off <= cap_records) lo = mid; else hi = mid - 1;
        }
        int64_t p1 = lo;
        // keep the grid within limits
        const int64_t max_np = ((1LL << 31) - 1) / sblocks;
        if (p1 - p0 > max_np) p1 = p0 + max_np;
        a.p0 = p0;
        a.np = p1 - p0;
        unsigned g1 = (unsigned)((a.np + 63) / 64);
        unsigned g2 = (unsigned)(a.np * sblocks);
        launch_base(P, a, precision, g1, st);
        SS_LAUNCH_CHECK();
        launch_response(S, a, precision, g2, sblock, sblocks, st);
        SS_LAUNCH_CHECK();
        p0 = p1;
    }
    return SS_OK;
}

int64_t ss_pert_track_bytes(const ss_pert_cfg* cfg, int precision) {
    PertArgs a;
    int rc = pert_args(cfg, precision, &a);
    if (rc) return rc;
    return pert_offset(a.N, a.ppr, a.spr, a.n_steps) * rec_len(a.ncol == 18 ? 2 : 1) * (precision == 64 ? 8 : 4);
}

int ss_pert_base_track(const ss_potential* base, const ss_pert_cfg* cfg, int precision, const double* base_ics,
                       double* base_out, void* track, int64_t track_bytes, void* stream) {
    PotDev<double> P;
    int rc = prepare_potential<double>(base, &P, false);
    if (rc) return rc;
    PertArgs a;
    rc = pert_args(cfg, precision, &a);
    if (rc) return rc;
    if (a.N == 0) return SS_OK;
    SS_CHECK_ARG(base_ics != nullptr, "base_ics is NULL");
    const int64_t need = ss_pert_track_bytes(cfg, precision);
    SS_CHECK_ARG(track != nullptr && track_bytes >= need && ((uintptr_t)track % 16) == 0,
                 "track of %lld bytes (16-byte aligned) needed", (long long)need);
    a.base_ics = base_ics;
    a.base_out = base_out;
    a.table = track;
    a.p0 = 0;
    a.np = a.N;
    cudaStream_t st = (cudaStream_t)stream;
    const unsigned g1 = (unsigned)((a.N + 63) / 64);
    launch_base(P, a, precision, g1, st);
    SS_LAUNCH_CHECK();
    return SS_OK;
}

int ss_pert_response_track(const ss_subhalos* sh, double G, const ss_pert_cfg* cfg, int precision,
                           const void* track, const void* pert_ics, void* pert_out, void* stream) {
    ShDev S;
    SS_CHECK_ARG(std::isfinite(G) && G > 0.0, "G must be finite and > 0");
    int rc = prepare_subhalos(sh, G, &S, cfg ? cfg->ncol : 6);
    if (rc) return rc;
    PertArgs a;
    rc = pert_args(cfg, precision, &a);
    if (rc) return rc;
    if (a.N == 0) return SS_OK;
    SS_CHECK_ARG(track != nullptr && pert_out != nullptr, "NULL buffer");
    SS_CHECK_ARG(((uintptr_t)track % 16) == 0, "track must be 16-byte aligned");
    a.pert_ics = pert_ics;
    a.pert_out = pert_out;
    a.table = const_cast<void*>(track);
    return pert_response_launch(S, a, precision, (cudaStream_t)stream);
}

int ss_pert_term(const ss_potential* base, const ss_subhalos* sh, int ncol, double t, const double* y, double* dy,
                 void* stream) {
    PotDev<double> P;
    int rc = prepare_potential<double>(base, &P, false);
    if (rc) return rc;
    ShDev S;
    rc = prepare_subhalos(sh, base->G, &S, ncol);
    if (rc) return rc;
    SS_CHECK_ARG(ncol == 6 || ncol == 12 || ncol == 18, "ncol must be 6, 12 or 18");
    SS_CHECK_ARG(std::isfinite(t), "t must be finite");
    SS_CHECK_ARG(y != nullptr && dy != nullptr, "NULL buffer");
    cudaStream_t st = (cudaStream_t)stream;
    const unsigned g = (unsigned)((S.n + 127) / 128);
    if (ncol == 18) pert_term_kernel<18><<<g, 128, 0, st>>>(P, S, t, y, dy);
    else if (ncol == 12) pert_term_kernel<12><<<g, 128, 0, st>>>(P, S, t, y, dy);
    else pert_term_kernel<6><<<g, 128, 0, st>>>(P, S, t, y, dy);
    SS_LAUNCH_CHECK();
    return SS_OK;
}

}  // extern "C"
